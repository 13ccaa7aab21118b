// cpa_dp2a.cu — instantiates the IND-CPA kernels of form kDp2a (TMVP with dp2a on CUDA cores)
// for the five ops (template in cpa_impl.cuh).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_dp2a_decrypt(const CpaArgs &a, cudaStream_t s) { return launch_op<kDp2a, kDecrypt>(a, s); }
int cpa_launch_dp2a_encrypt(const CpaArgs &a, cudaStream_t s) { return launch_op<kDp2a, kEncrypt>(a, s); }
int cpa_launch_dp2a_reenc(const CpaArgs &a, cudaStream_t s) { return launch_op<kDp2a, kReenc>(a, s); }
int cpa_launch_dp2a_keygen(const CpaArgs &a, cudaStream_t s) { return launch_op<kDp2a, kKeygen>(a, s); }
int cpa_launch_dp2a_matvec(const CpaArgs &a, cudaStream_t s) { return launch_op<kDp2a, kMatvec>(a, s); }
}  // namespace tmvp
