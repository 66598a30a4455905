// LBP forward instantiations for the stereo pairwise variant, FP16 storage:
// the lean kernel (lbp_forward_f16.cuh) for up to 256 labels, the general
// kernel for wider rows.
#include "lbp_forward_f16.cuh"

namespace bpl {
int lbp_forward_stereo_f16(const FwdArgs& a, cudaStream_t s) {
  if (a.L <= 256) return dispatch_f16(a, s);
  return dispatch_k<BPL_LBP_STEREO, __half>(a, s);
}
}  // namespace bpl
