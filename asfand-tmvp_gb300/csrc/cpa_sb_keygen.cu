// cpa_sb_keygen.cu — instantiates the IND-CPA kernel for form kSchoolbook, op kKeygen
// (template in cpa_impl.cuh; one translation unit per pair so that they
// compile in parallel).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_sb_keygen(const CpaArgs &a, cudaStream_t s) { return launch_op<kSchoolbook, kKeygen>(a, s); }
}  // namespace tmvp
