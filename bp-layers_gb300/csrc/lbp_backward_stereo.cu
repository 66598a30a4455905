// LBP reference-adjoint instantiations for the stereo pairwise variant.
#include "lbp_backward.cuh"

namespace bpl {
int lbp_backward_stereo(const BwdArgs& a, cudaStream_t s) { return dispatch_bwd<BPL_LBP_STEREO>(a, s); }
}  // namespace bpl
