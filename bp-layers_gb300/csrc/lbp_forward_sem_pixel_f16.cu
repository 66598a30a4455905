// LBP forward instantiations for the sem_pixel pairwise variant, FP16 storage.
#include "lbp_forward.cuh"

namespace bpl {
int lbp_forward_sem_pixel_f16(const FwdArgs& a, cudaStream_t s) { return dispatch_k<BPL_LBP_SEM_PIXEL, __half>(a, s); }
}  // namespace bpl
