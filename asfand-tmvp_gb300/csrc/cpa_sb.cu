// cpa_sb.cu — instantiates the IND-CPA kernels for form kSchoolbook (see cpa_impl.cuh).
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_sb(int op, const CpaArgs &a, cudaStream_t s) { return launch_form<kSchoolbook>(op, a, s); }
size_t cpa_smem_sb(int op, const KemParams &P) { return smem_form<kSchoolbook>(op, P); }
}  // namespace tmvp
