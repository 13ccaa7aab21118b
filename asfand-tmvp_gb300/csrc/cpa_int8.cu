// cpa_int8.cu — instantiates the IND-CPA kernels for form kInt8TC (see cpa_impl.cuh).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_int8(int op, const CpaArgs &a, cudaStream_t s) { return launch_form<kInt8TC>(op, a, s); }
size_t cpa_smem_int8(int op, const KemParams &P) { return smem_form<kInt8TC>(op, P); }
}  // namespace tmvp
