// On-device material assignment and Kottke smoothing (placeholder until the
// kernels land).
#include "fdfd_internal.cuh"

namespace fdfd {
int smooth_objects_impl(fdfd_handle *h, const double *const lprim[3], const fdfd_object *objs, int nobj,
                        double eps_bg, const fdfd_design *design) {
  (void)lprim; (void)objs; (void)nobj; (void)eps_bg; (void)design;
  return set_error(h, FDFD_ERR_UNSUPPORTED, "fdfd_smooth_objects is not available yet");
}
}  // namespace fdfd
