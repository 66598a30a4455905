// LBP reference-adjoint instantiations for the stereo variant with 8 jump taps.
#include "lbp_backward.cuh"

namespace bpl {
int lbp_backward_stereo_lv8(const BwdArgs& a, cudaStream_t s) { return dispatch_bwd<BPL_LBP_STEREO, 8>(a, s); }
}  // namespace bpl
