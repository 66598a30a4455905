// LBP forward instantiations for the stereo pairwise variant, FP16 storage.
#include "lbp_forward.cuh"

namespace bpl {
int lbp_forward_stereo_f16(const FwdArgs& a, cudaStream_t s) { return dispatch_k<BPL_LBP_STEREO, __half>(a, s); }
}  // namespace bpl
