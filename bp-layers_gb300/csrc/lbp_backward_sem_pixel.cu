// LBP reference-adjoint instantiations for the sem_pixel pairwise variant.
#include "lbp_backward.cuh"

namespace bpl {
int lbp_backward_sem_pixel(const BwdArgs& a, cudaStream_t s) { return dispatch_bwd<BPL_LBP_SEM_PIXEL, 0>(a, s); }
}  // namespace bpl
