// LBP reference-adjoint instantiations for the sem_global pairwise variant.
#include "lbp_backward.cuh"

namespace bpl {
int lbp_backward_sem_global(const BwdArgs& a, cudaStream_t s) { return dispatch_bwd<BPL_LBP_SEM_GLOBAL, 0>(a, s); }
}  // namespace bpl
