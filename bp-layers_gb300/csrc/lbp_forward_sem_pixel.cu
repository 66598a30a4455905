// LBP forward instantiations for the sem_pixel pairwise variant.
#include "lbp_forward.cuh"

namespace bpl {
int lbp_forward_sem_pixel(const FwdArgs& a, cudaStream_t s) { return dispatch_k<BPL_LBP_SEM_PIXEL>(a, s); }
}  // namespace bpl
