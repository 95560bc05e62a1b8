// fdfd_residual_dev_noalloc: the FP64 residual r = b − A x and ‖r‖₂² of
// fdfd_residual_dev, for callers that cannot allocate device memory.
//
// Who cannot allocate: a caller whose GPU memory is owned by another
// allocator — a framework's caching pool (CUDA.jl's, PyTorch's) that has
// reserved the device, so a fresh cudaMalloc fails or steals from its
// budget — or a caller in the middle of a pipelined stream that must not
// pay the implicit device synchronisation a cudaMalloc/cudaFree can cause.
// fdfd_residual_dev may grow the handle's reduction buffer on first use;
// this variant never allocates: the operator kernel's per-block partial
// sums, its arrival counter and its result slot live in one file-scope
// __device__ array of fixed size, present on every GPU that loads the
// library until the process exits.
//
// Limits and rules (also stated in include/fdfd_gb300.h):
//   * at most NOALLOC_MAX_BLOCKS thread-block partials (16384): the z-chunk
//     is lengthened until the grid fits, so only an x-y tiling of more than
//     16384 tiles of 32×8 cells (about 2048×2048 cells per plane) is
//     rejected with FDFD_ERR_ARG;
//   * E formulation only; synchronous (returns with ‖r‖² on the host);
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (a host-side name is not a device address); make
//     that first call before any stream capture;
//   * every call shares the array and the counter is cleared at the start of
//     each call: calls that overlap on the GPU (other streams, other
//     handles) race — serialise them.
#include <cstddef>
#include <mutex>

#include "krylov_fin.cuh"

namespace fdfd {

int launch_residual_ext(fdfd_handle *h, const double2 *x, double2 *r, const double2 *b, RedBuf red, int max_blocks,
                        KScalars *sc);

constexpr int NOALLOC_MAX_BLOCKS = 16384;
constexpr size_t NOALLOC_PART_BYTES = sizeof(double2) * 2 * NOALLOC_MAX_BLOCKS;  // 512 KiB
constexpr size_t NOALLOC_COUNT_OFF = NOALLOC_PART_BYTES;
constexpr size_t NOALLOC_SC_OFF = NOALLOC_PART_BYTES + 256;
constexpr size_t NOALLOC_BYTES = NOALLOC_SC_OFF + ((sizeof(KScalars) + 255) / 256) * 256;

// partials [0, 512 KiB) | arrival counter (+256 B) | finalisation scalars
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

static unsigned char *s_scratch[MAX_DEVICES] = {nullptr};
static std::mutex s_mutex;

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
static int scratch_for(fdfd_handle *h, unsigned char **out) {
  if (h->dev < 0 || h->dev >= MAX_DEVICES) return set_error(h, FDFD_ERR_ARG, "device ordinal too large");
  std::lock_guard<std::mutex> lock(s_mutex);
  if (!s_scratch[h->dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_check(h, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    s_scratch[h->dev] = (unsigned char *)p;
  }
  *out = s_scratch[h->dev];
  return FDFD_OK;
}

}  // namespace fdfd

using namespace fdfd;

extern "C" int fdfd_residual_dev_noalloc(fdfd_handle *h, const void *x, const void *b, void *r, double *rnorm2) {
  if (!h || !x || !b || !r || !rnorm2) return set_error(h, FDFD_ERR_ARG, "null argument");
  if (h->ft != FDFD_EE) return set_error(h, FDFD_ERR_UNSUPPORTED, "the allocation-free residual is for the E formulation");
  int rc = cuda_check(h, cudaSetDevice(h->dev), "cudaSetDevice");
  if (rc) return rc;
  unsigned char *base = nullptr;
  if ((rc = scratch_for(h, &base))) return rc;
  RedBuf red;
  red.part = reinterpret_cast<double2 *>(base);
  red.count = reinterpret_cast<unsigned int *>(base + NOALLOC_COUNT_OFF);
  KScalars *sc = reinterpret_cast<KScalars *>(base + NOALLOC_SC_OFF);
  // the counter and the gate flag (sc->done) must start at zero
  rc = cuda_check(h, cudaMemsetAsync(base + NOALLOC_COUNT_OFF, 0, NOALLOC_BYTES - NOALLOC_COUNT_OFF, h->stream),
                  "clear scratch");
  if (rc) return rc;
  rc = launch_residual_ext(h, (const double2 *)x, (double2 *)r, (const double2 *)b, red, NOALLOC_MAX_BLOCKS, sc);
  if (rc) return rc;
  double v = 0.0;
  rc = cuda_check(h, cudaMemcpyAsync(&v, reinterpret_cast<unsigned char *>(sc) + offsetof(KScalars, dot0), sizeof(double),
                                     cudaMemcpyDeviceToHost, h->stream),
                  "D2H residual");
  if (rc) return rc;
  rc = cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
  if (rc) return rc;
  *rnorm2 = v;
  return FDFD_OK;
}
