// LBP forward instantiations for the sem_global pairwise variant, FP16 storage.
#include "lbp_forward.cuh"

namespace bpl {
int lbp_forward_sem_global_f16(const FwdArgs& a, cudaStream_t s) { return dispatch_k<BPL_LBP_SEM_GLOBAL, __half>(a, s); }
}  // namespace bpl
