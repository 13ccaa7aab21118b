// cpa_f8u_matvec.cu — op kMatvec on the tcgen05 tensor cores, in one of two launch
// shapes picked per (op, parameter set) by the autotuner: one CTA per
// instance (cpa5i.cuh, specialised for l = 2 / 3 / 4 with 13-bit digit
// columns, which serve every eq <= 13), or the persistent pipelined kernel
// (cpa_persist.cuh), which also runs mixed tables of groups.  One translation
// unit per op so that they compile in parallel.
#include "cpa5i.cuh"
#include "cpa_impl.cuh"

namespace tmvp {
int cpa_launch_f8u_matvec(const CpaArgs &a, cudaStream_t s) {
  const int mode = persist_ctas_per_sm(kMatvec, a.P.set);
  if (mode < 0) {  // one CTA per instance, the set of Saber's family with this l
    switch (a.P.l) {
      case 2: return launch_cpa5i<kMatvec, 0>(a, s);
      case 3: return launch_cpa5i<kMatvec, 1>(a, s);
      case 4: return launch_cpa5i<kMatvec, 2>(a, s);
    }
    return (int)cudaErrorInvalidValue;
  }
  return launch_persist<kMatvec>(&a, 1, nullptr, s, mode);
}
int cpa_launch_mixed_matvec(const CpaArgs *g, int ng, const MixTable *dev_tab, cudaStream_t s, int ctas_per_sm) {
  if (ng < 1 || ng > kMaxGroups) return (int)cudaErrorInvalidValue;
  return launch_persist<kMatvec>(g, ng, dev_tab, s, ctas_per_sm < 0 ? 0 : ctas_per_sm);
}
}  // namespace tmvp
