// LBP reference-adjoint instantiations for the stereo variant, FP16 messages, 8 jump taps.
#include "lbp_backward.cuh"

namespace bpl {
int lbp_backward_stereo_f16_lv8(const BwdArgs& a, cudaStream_t s) { return dispatch_bwd<BPL_LBP_STEREO, 8, __half>(a, s); }
}  // namespace bpl
