// cpa_fp8_decrypt.cu — instantiates the IND-CPA kernel for form kFp8TC, op kDecrypt
// (template in cpa_impl.cuh; one translation unit per pair so that they
// compile in parallel).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_fp8_decrypt(const CpaArgs &a, cudaStream_t s) { return launch_op<kFp8TC, kDecrypt>(a, s); }
}  // namespace tmvp
