// cpa_f8u_reenc.cu — instantiates the IND-CPA kernel for form kFp8Tcgen05
// (tcgen05 tensor cores), op kReenc (template in cpa_impl.cuh / cpa_tc_kernel.cuh;
// one translation unit per pair so that they compile in parallel).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_f8u_reenc(const CpaArgs &a, cudaStream_t s) { return launch_op<kFp8Tcgen05, kReenc>(a, s); }
}  // namespace tmvp
