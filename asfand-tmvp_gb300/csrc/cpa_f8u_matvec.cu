// cpa_f8u_matvec.cu — op kMatvec on the tcgen05 tensor cores, in one of two launch
// shapes picked per (op, parameter set) by the autotuner: one CTA per
// instance (cpa_tc_kernel.cuh), or the persistent pipelined kernel
// (cpa_persist.cuh), which also runs mixed tables of groups.  One translation
// unit per op so that they compile in parallel.
#include "cpa_impl.cuh"
#include "cpa_persist.cuh"

namespace tmvp {
int cpa_launch_f8u_matvec(const CpaArgs &a, cudaStream_t s) {
  const int mode = persist_ctas_per_sm(kMatvec, a.P.set);
  if (mode < 0) return launch_op<kFp8Tcgen05, kMatvec>(a, s);  // one CTA per instance
  return launch_persist<kMatvec>(&a, 1, nullptr, s, mode);
}
int cpa_launch_mixed_matvec(const CpaArgs *g, int ng, const MixTable *dev_tab, cudaStream_t s, int ctas_per_sm) {
  if (ng < 1 || ng > kMaxGroups) return (int)cudaErrorInvalidValue;
  return launch_persist<kMatvec>(g, ng, dev_tab, s, ctas_per_sm < 0 ? 0 : ctas_per_sm);
}
}  // namespace tmvp
