// LBP reference-adjoint instantiations for the stereo variant (any Lv <= 16).
#include "lbp_backward.cuh"

namespace bpl {
int lbp_backward_stereo(const BwdArgs& a, cudaStream_t s) {
  if (a.Lv == 6) return lbp_backward_stereo_lv6(a, s);
  if (a.Lv == 8) return lbp_backward_stereo_lv8(a, s);
  return dispatch_bwd<BPL_LBP_STEREO, 16>(a, s);
}
}  // namespace bpl
