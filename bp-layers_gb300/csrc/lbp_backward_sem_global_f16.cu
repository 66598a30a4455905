// LBP reference-adjoint instantiations for the sem_global pairwise variant, FP16 messages.
#include "lbp_backward.cuh"

namespace bpl {
int lbp_backward_sem_global_f16(const BwdArgs& a, cudaStream_t s) { return dispatch_bwd<BPL_LBP_SEM_GLOBAL, 0, __half>(a, s); }
}  // namespace bpl
