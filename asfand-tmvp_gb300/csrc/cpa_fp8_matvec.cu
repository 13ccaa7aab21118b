// cpa_fp8_matvec.cu — instantiates the IND-CPA kernel for form kFp8TC, op kMatvec
// (template in cpa_impl.cuh; one translation unit per pair so that they
// compile in parallel).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_fp8_matvec(const CpaArgs &a, cudaStream_t s) { return launch_op<kFp8TC, kMatvec>(a, s); }
}  // namespace tmvp
