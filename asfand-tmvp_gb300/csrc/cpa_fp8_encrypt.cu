// cpa_fp8_encrypt.cu — instantiates the IND-CPA kernel for form kFp8TC, op kEncrypt
// (template in cpa_impl.cuh; one translation unit per pair so that they
// compile in parallel).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_fp8_encrypt(const CpaArgs &a, cudaStream_t s) { return launch_op<kFp8TC, kEncrypt>(a, s); }
}  // namespace tmvp
