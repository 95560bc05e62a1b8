// Field post-processing on the device:
//   * h_from_e — H = (i/ω)·Pμ⁻¹·(Cₑ e + jₘ)        (src/model/model.jl:276-279,
//     Pμ = I): the forward-difference curl E→H of the operator, one pass;
//   * e_from_h — E = (−i/ω)·Pε⁻¹·(Cₘ h − jₑ)       (model.jl:281-284) for a
//     diagonal Pε: the backward-difference curl H→E of the operator (ghost
//     H(−1) mirrors H(0) on a symmetry wall, Bloch axes wrap with the phase),
//     divided by ε at each E sample, one pass;
//   * corner means — the create_Mcs interpolation (model.jl:287-306):
//     Mcₑ averages E_w backward along w onto the primal voxel corners with
//     weights s∆lₘ and 1/s∆lₑ (isfwdₑ = boundft .!= EE = false);
//     Mcₘ averages H_w forward along w onto the dual corners with weights
//     s∆lₑ and 1/s∆lₘ (isfwdₘ = boundft .!= HH = true):
//         Ec_w[j] = (s∆lₘ[j−1]·E_w[j−1] + s∆lₘ[j]·E_w[j]) / (2·s∆lₑ[j])
//         Hc_w[j] = (s∆lₑ[j]·H_w[j] + s∆lₑ[j+1]·H_w[j+1]) / (2·s∆lₘ[j]).
//     Ghosts: E_w[−1] mirrors E_w[0] (weight s∆lₘ[0]) on a symmetry wall,
//     H_w[N] = 0 there (normal H on the PEC plane); Bloch axes wrap with the
//     phase e^{∓ikL}.  These are the same two-point means the ε tensor's
//     off-diagonal averaging uses.
// All kernels are grid-stride loops over cells, x fastest (coalesced).
#include <cuda_runtime.h>

#include "operator_common.cuh"

namespace fdfd {

__global__ void k_h_from_e(OpArgs<double> a, Extra<double> ex, const double2 *__restrict__ e,
                           const double2 *__restrict__ jm, double2 *__restrict__ hout, double2 iow) {
  const long long nc = a.ncell;
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < nc;
       cell += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(cell % a.N[0]), j = (int)((cell / a.N[0]) % a.N[1]), k = (int)(cell / ((long long)a.N[0] * a.N[1]));
    const double2 cmx = a.cm[0][i], cmy = a.cm[1][j], cmz = a.cm[2][k];
    const double2 ex0 = load_e<double, false>(e, a, ex, i, j, k, 0);
    const double2 ey0 = load_e<double, false>(e, a, ex, i, j, k, 1);
    const double2 ez0 = load_e<double, false>(e, a, ex, i, j, k, 2);
    const double2 exy = load_e<double, false>(e, a, ex, i, j + 1, k, 0);
    const double2 exz = load_e<double, false>(e, a, ex, i, j, k + 1, 0);
    const double2 eyx = load_e<double, false>(e, a, ex, i + 1, j, k, 1);
    const double2 eyz = load_e<double, false>(e, a, ex, i, j, k + 1, 1);
    const double2 ezx = load_e<double, false>(e, a, ex, i + 1, j, k, 2);
    const double2 ezy = load_e<double, false>(e, a, ex, i, j + 1, k, 2);
    double2 h[3];
    h[0] = csub(cmul(cmy, csub(ezy, ez0)), cmul(cmz, csub(eyz, ey0)));
    h[1] = csub(cmul(cmz, csub(exz, ex0)), cmul(cmx, csub(ezx, ez0)));
    h[2] = csub(cmul(cmx, csub(eyx, ey0)), cmul(cmy, csub(exy, ex0)));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (jm) h[c] = cadd(h[c], jm[3 * cell + c]);
      hout[3 * cell + c] = cmul(iow, h[c]);
    }
  }
}

// H_c at the cell one step back along w from `cell` (t: the cell's index
// along w, stride: the cell stride along w).
__device__ __forceinline__ double2 h_back(const double2 *__restrict__ hin, const OpArgs<double> &a,
                                          const Extra<double> &ex, long long cell, int t, int w, long long stride,
                                          int c) {
  if (t > 0) return hin[3 * (cell - stride) + c];
  if (a.bloch[w]) return cmul(hin[3 * (cell + (long long)(a.N[w] - 1) * stride) + c], ex.phinv[w]);
  return hin[3 * cell + c];  // mirror: H(−1) = H(0)
}

__global__ void k_e_from_h(OpArgs<double> a, Extra<double> ex, const double2 *__restrict__ hin,
                           const double2 *__restrict__ je, double2 *__restrict__ eout, double2 miow) {
  const long long nc = a.ncell;
  const long long sy = a.N[0], sz = (long long)a.N[0] * a.N[1];
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < nc;
       cell += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(cell % a.N[0]), j = (int)((cell / a.N[0]) % a.N[1]), k = (int)(cell / sz);
    const double2 cex = a.ce[0][i], cey = a.ce[1][j], cez = a.ce[2][k];
    const double2 hx = hin[3 * cell], hy = hin[3 * cell + 1], hz = hin[3 * cell + 2];
    const double2 hzj = h_back(hin, a, ex, cell, j, 1, sy, 2), hyk = h_back(hin, a, ex, cell, k, 2, sz, 1);
    const double2 hxk = h_back(hin, a, ex, cell, k, 2, sz, 0), hzi = h_back(hin, a, ex, cell, i, 0, 1, 2);
    const double2 hyi = h_back(hin, a, ex, cell, i, 0, 1, 1), hxj = h_back(hin, a, ex, cell, j, 1, sy, 0);
    double2 e[3];
    e[0] = csub(cmul(cey, csub(hz, hzj)), cmul(cez, csub(hy, hyk)));
    e[1] = csub(cmul(cez, csub(hx, hxk)), cmul(cex, csub(hz, hzi)));
    e[2] = csub(cmul(cex, csub(hy, hyi)), cmul(cey, csub(hx, hxj)));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (je) e[c] = csub(e[c], je[3 * cell + c]);
      eout[3 * cell + c] = cscale(cmul(miow, e[c]), 1.0 / a.eps[c * nc + cell]);
    }
  }
}

__global__ void k_corner_mean(OpArgs<double> a, Extra<double> ex, int hfield, const double2 *__restrict__ in,
                              double2 *__restrict__ out) {
  const long long nc = a.ncell;
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < nc;
       cell += (long long)gridDim.x * blockDim.x) {
    const int g[3] = {(int)(cell % a.N[0]), (int)((cell / a.N[0]) % a.N[1]), (int)(cell / ((long long)a.N[0] * a.N[1]))};
#pragma unroll
    for (int w = 0; w < 3; ++w) {
      const long long stride = (w == 0) ? 1 : (w == 1) ? a.N[0] : (long long)a.N[0] * a.N[1];
      const int n = a.N[w], t = g[w];
      const double2 self = in[3 * cell + w];
      double2 r;
      if (!hfield) {
        // backward mean of E_w onto the primal corner t
        double2 nb, wnb;
        if (t > 0) {
          nb = in[3 * (cell - stride) + w];
          wnb = ex.sdlm[w][t - 1];
        } else if (a.bloch[w]) {
          nb = cmul(in[3 * (cell + (long long)(n - 1) * stride) + w], ex.phinv[w]);
          wnb = ex.sdlm[w][n - 1];
        } else {
          nb = self;
          wnb = ex.sdlm[w][0];
        }
        r = cadd(cmul(wnb, nb), cmul(ex.sdlm[w][t], self));
        r = cmul(r, cinv(cscale(ex.sdle[w][t], 2.0)));
      } else {
        // forward mean of H_w onto the dual corner t
        double2 nb = czero<double2>(), wnb = czero<double2>();
        if (t + 1 < n) {
          nb = in[3 * (cell + stride) + w];
          wnb = ex.sdle[w][t + 1];
        } else if (a.bloch[w]) {
          nb = cmul(in[3 * (cell - (long long)(n - 1) * stride) + w], ex.ph[w]);
          wnb = ex.sdle[w][0];
        }
        r = cadd(cmul(ex.sdle[w][t], self), cmul(wnb, nb));
        r = cmul(r, cinv(cscale(ex.sdlm[w][t], 2.0)));
      }
      out[3 * cell + w] = r;
    }
  }
}

// 2D slices (TE/TM): host vectors carry only the components in `mask`
// (bit c = component c), component-fastest per cell.
__global__ void k_unpack(const double2 *__restrict__ src, double2 *__restrict__ dst, int mask, long long ncell) {
  const int nc = __popc(mask);
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < ncell;
       cell += (long long)gridDim.x * blockDim.x) {
    int q = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double2 v = make_double2(0.0, 0.0);
      if (mask & (1 << c)) v = src[nc * cell + q++];
      dst[3 * cell + c] = v;
    }
  }
}

__global__ void k_pack(const double2 *__restrict__ src, double2 *__restrict__ dst, int mask, long long ncell) {
  const int nc = __popc(mask);
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < ncell;
       cell += (long long)gridDim.x * blockDim.x) {
    int q = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      if (mask & (1 << c)) dst[nc * cell + q++] = src[3 * cell + c];
  }
}

__global__ void k_pack_real(const double *__restrict__ src, double *__restrict__ dst, int mask, long long ncell) {
  const int nc = __popc(mask);
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < ncell;
       cell += (long long)gridDim.x * blockDim.x) {
    int q = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      if (mask & (1 << c)) dst[nc * cell + q++] = src[3 * cell + c];
  }
}

int field_mask(const fdfd_handle *h, bool hfield) {
  if (h->slice2d == FDFD_SLICE_TE) return hfield ? 4 : 3;
  if (h->slice2d == FDFD_SLICE_TM) return hfield ? 3 : 4;
  return 7;
}

static int ensure_stage(fdfd_handle *h) {
  if (h->stage64) return FDFD_OK;
  if (dev_malloc(&h->stage64, 3 * (size_t)h->ncell * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    h->stage64 = nullptr;
    return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(2D staging) failed");
  }
  return FDFD_OK;
}

int h2d_field(fdfd_handle *h, const double *src, double2 *dst, int mask) {
  const long long nc = h->ncell;
  if (mask == 7)
    return cuda_check(h, cudaMemcpyAsync(dst, src, 3 * nc * sizeof(double2), cudaMemcpyHostToDevice, h->stream),
                      "H2D field");
  int rc = ensure_stage(h);
  if (rc) return rc;
  const int n = __builtin_popcount(mask);
  if ((rc = cuda_check(h, cudaMemcpyAsync(h->stage64, src, n * nc * sizeof(double2), cudaMemcpyHostToDevice, h->stream),
                       "H2D field")))
    return rc;
  k_unpack<<<152 * 4, 256, 0, h->stream>>>(h->stage64, dst, mask, nc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_unpack");
}

int d2h_field(fdfd_handle *h, const double2 *src, double *dst, int mask) {
  const long long nc = h->ncell;
  if (mask == 7)
    return cuda_check(h, cudaMemcpyAsync(dst, src, 3 * nc * sizeof(double2), cudaMemcpyDeviceToHost, h->stream),
                      "D2H field");
  int rc = ensure_stage(h);
  if (rc) return rc;
  const int n = __builtin_popcount(mask);
  k_pack<<<152 * 4, 256, 0, h->stream>>>(src, h->stage64, mask, nc);
  h->launches++;
  if ((rc = cuda_check(h, cudaGetLastError(), "k_pack"))) return rc;
  return cuda_check(h, cudaMemcpyAsync(dst, h->stage64, n * nc * sizeof(double2), cudaMemcpyDeviceToHost, h->stream),
                    "D2H field");
}

int d2h_real(fdfd_handle *h, const double *src, double *dst, int mask) {
  const long long nc = h->ncell;
  if (mask == 7)
    return cuda_check(h, cudaMemcpyAsync(dst, src, 3 * nc * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
                      "D2H values");
  int rc = ensure_stage(h);
  if (rc) return rc;
  const int n = __builtin_popcount(mask);
  double *st = reinterpret_cast<double *>(h->stage64);
  k_pack_real<<<152 * 4, 256, 0, h->stream>>>(src, st, mask, nc);
  h->launches++;
  if ((rc = cuda_check(h, cudaGetLastError(), "k_pack_real"))) return rc;
  return cuda_check(h, cudaMemcpyAsync(dst, st, n * nc * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
                    "D2H values");
}

int h_from_e_dev_impl(fdfd_handle *h, const double2 *e, const double2 *jm, double2 *hout) {
  const OpArgs<double> a = op_args<double>(h);
  const Extra<double> ex = make_extra<double>(h);
  // i/ω for complex ω
  const double wr = h->omega[0], wi = h->omega[1], d = wr * wr + wi * wi;
  if (!(d > 0.0)) return set_error(h, FDFD_ERR_ARG, "h_from_e needs ω ≠ 0");
  const double2 iow = make_double2(wi / d, wr / d);
  k_h_from_e<<<152 * 8, 256, 0, h->stream>>>(a, ex, e, jm, hout, iow);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_h_from_e");
}

int e_from_h_dev_impl(fdfd_handle *h, const double2 *hin, const double2 *je, double2 *eout) {
  if (h->has_off)
    return set_error(h, FDFD_ERR_UNSUPPORTED, "e_from_h needs a diagonal ε (Pε \\ …), as in the reference");
  const OpArgs<double> a = op_args<double>(h);
  const Extra<double> ex = make_extra<double>(h);
  // −i/ω for complex ω
  const double wr = h->omega[0], wi = h->omega[1], d = wr * wr + wi * wi;
  if (!(d > 0.0)) return set_error(h, FDFD_ERR_ARG, "e_from_h needs ω ≠ 0");
  const double2 miow = make_double2(-wi / d, -wr / d);
  k_e_from_h<<<152 * 8, 256, 0, h->stream>>>(a, ex, hin, je, eout, miow);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_e_from_h");
}

int corner_mean_dev_impl(fdfd_handle *h, int hfield, const double2 *in, double2 *out) {
  const OpArgs<double> a = op_args<double>(h);
  const Extra<double> ex = make_extra<double>(h);
  k_corner_mean<<<152 * 8, 256, 0, h->stream>>>(a, ex, hfield, in, out);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_corner_mean");
}

}  // namespace fdfd
