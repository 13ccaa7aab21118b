// cpa_fp8.cu — instantiates the IND-CPA kernels for form kFp8TC (see cpa_impl.cuh).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_fp8(int op, const CpaArgs &a, cudaStream_t s) { return launch_form<kFp8TC>(op, a, s); }
size_t cpa_smem_fp8(int op, const KemParams &P) { return smem_form<kFp8TC>(op, P); }
}  // namespace tmvp
