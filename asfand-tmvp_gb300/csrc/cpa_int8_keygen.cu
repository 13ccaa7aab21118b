// cpa_int8_keygen.cu — instantiates the IND-CPA kernel for form kInt8TC, op kKeygen
// (template in cpa_impl.cuh; one translation unit per pair so that they
// compile in parallel).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_int8_keygen(const CpaArgs &a, cudaStream_t s) { return launch_op<kInt8TC, kKeygen>(a, s); }
}  // namespace tmvp
