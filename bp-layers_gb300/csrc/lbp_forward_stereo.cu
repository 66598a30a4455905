// LBP forward instantiations for the stereo pairwise variant.
#include "lbp_forward.cuh"

namespace bpl {
int lbp_forward_stereo(const FwdArgs& a, cudaStream_t s) { return dispatch_k<BPL_LBP_STEREO>(a, s); }
}  // namespace bpl
