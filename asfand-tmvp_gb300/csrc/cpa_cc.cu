// cpa_cc.cu — instantiates the IND-CPA kernels for form kCudaCore (see cpa_impl.cuh).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_cc(int op, const CpaArgs &a, cudaStream_t s) { return launch_form<kCudaCore>(op, a, s); }
size_t cpa_smem_cc(int op, const KemParams &P) { return smem_form<kCudaCore>(op, P); }
}  // namespace tmvp
