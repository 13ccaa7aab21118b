// cpa_cc_reenc.cu — instantiates the IND-CPA kernel for form kCudaCore, op kReenc
// (template in cpa_impl.cuh; one translation unit per pair so that they
// compile in parallel).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_cc_reenc(const CpaArgs &a, cudaStream_t s) { return launch_op<kCudaCore, kReenc>(a, s); }
}  // namespace tmvp
