// cpa_f8u_reenc.cu — op kReenc on the tcgen05 tensor cores, in one of two launch
// shapes picked per (op, parameter set) by the autotuner: one CTA per
// instance (cpa5i.cuh, specialised per parameter set), or the persistent pipelined kernel
// (cpa_persist.cuh), which also runs mixed tables of groups.  One translation
// unit per op so that they compile in parallel.
#include "cpa5i.cuh"
#include "cpa_persist.cuh"

namespace tmvp {
int cpa_launch_f8u_reenc(const CpaArgs &a, cudaStream_t s) {
  const int mode = persist_ctas_per_sm(kReenc, a.P.set);
  // one CTA per instance (always for a shared key, which only that kernel reads)
  if (mode < 0 || a.key_shared) return launch_cpa5i_set<kReenc>(a, s);
  return launch_persist<kReenc>(&a, 1, nullptr, s, mode);
}
int cpa_launch_mixed_reenc(const CpaArgs *g, int ng, const MixTable *dev_tab, cudaStream_t s, int ctas_per_sm) {
  if (ng < 1 || ng > kMaxGroups) return (int)cudaErrorInvalidValue;
  if (ctas_per_sm < 0) return launch_cpa5m<kReenc>(g, ng, dev_tab, s);  // one CTA per instance
  return launch_persist<kReenc>(g, ng, dev_tab, s, ctas_per_sm);
}
}  // namespace tmvp
