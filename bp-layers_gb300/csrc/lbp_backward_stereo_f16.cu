// LBP reference-adjoint instantiations for the stereo variant, FP16 messages
// (6 or 8 jump taps; other tap counts use the generic tap loop).
#include "lbp_backward.cuh"

namespace bpl {
int lbp_backward_stereo_f16_lv6(const BwdArgs& a, cudaStream_t s);
int lbp_backward_stereo_f16_lv8(const BwdArgs& a, cudaStream_t s);

int lbp_backward_stereo_f16(const BwdArgs& a, cudaStream_t s) {
  if (a.Lv == 6) return lbp_backward_stereo_f16_lv6(a, s);
  if (a.Lv == 8) return lbp_backward_stereo_f16_lv8(a, s);
  return dispatch_bwd<BPL_LBP_STEREO, 16, __half>(a, s);
}
}  // namespace bpl
