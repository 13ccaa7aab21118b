// cpa_sb_reenc.cu — instantiates the IND-CPA kernel for form kSchoolbook, op kReenc
// (template in cpa_impl.cuh; one translation unit per pair so that they
// compile in parallel).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_sb_reenc(const CpaArgs &a, cudaStream_t s) { return launch_op<kSchoolbook, kReenc>(a, s); }
}  // namespace tmvp
