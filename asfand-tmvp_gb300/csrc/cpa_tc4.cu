// cpa_tc4.cu — instantiates the IND-CPA kernels of form kToomCook (Toom-Cook 4-way on CUDA cores)
// for the five ops (template in cpa_impl.cuh).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_tc4_decrypt(const CpaArgs &a, cudaStream_t s) { return launch_op<kToomCook, kDecrypt>(a, s); }
int cpa_launch_tc4_encrypt(const CpaArgs &a, cudaStream_t s) { return launch_op<kToomCook, kEncrypt>(a, s); }
int cpa_launch_tc4_reenc(const CpaArgs &a, cudaStream_t s) { return launch_op<kToomCook, kReenc>(a, s); }
int cpa_launch_tc4_keygen(const CpaArgs &a, cudaStream_t s) { return launch_op<kToomCook, kKeygen>(a, s); }
int cpa_launch_tc4_matvec(const CpaArgs &a, cudaStream_t s) { return launch_op<kToomCook, kMatvec>(a, s); }
}  // namespace tmvp
