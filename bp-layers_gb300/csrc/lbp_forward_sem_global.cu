// LBP forward instantiations for the sem_global pairwise variant.
#include "lbp_forward.cuh"

namespace bpl {
int lbp_forward_sem_global(const FwdArgs& a, cudaStream_t s) { return dispatch_k<BPL_LBP_SEM_GLOBAL>(a, s); }
}  // namespace bpl
