// cpa_f8u_decrypt.cu — op kDecrypt on the tcgen05 tensor cores, in one of two launch
// shapes picked per (op, parameter set) by the autotuner: one CTA per
// instance (cpa5i.cuh, specialised per parameter set), or the persistent pipelined kernel
// (cpa_persist.cuh), which also runs mixed tables of groups.  One translation
// unit per op so that they compile in parallel.
#include "cpa5i.cuh"
#include "cpa_persist.cuh"

#include <cstring>

namespace tmvp {
int cpa_launch_f8u_decrypt(const CpaArgs &a, cudaStream_t s) {
  const int mode = persist_ctas_per_sm(kDecrypt, a.P.set);
  // one CTA per instance (always for a shared key, which only that kernel reads)
  if (mode < 0 || a.key_shared) return launch_cpa5i_set<kDecrypt>(a, s);
  return launch_persist<kDecrypt>(&a, 1, nullptr, s, mode);
}
int cpa_launch_mixed_decrypt(const CpaArgs *g, int ng, const MixTable *dev_tab, cudaStream_t s, int ctas_per_sm) {
  if (ng < 1 || ng > kMaxGroups) return (int)cudaErrorInvalidValue;
  if (ctas_per_sm < 0) return launch_cpa5m<kDecrypt>(g, ng, dev_tab, s);  // one CTA per instance
  return launch_persist<kDecrypt>(g, ng, dev_tab, s, ctas_per_sm);
}

int cpa_launch_decrypt_onekey(const CpaArgs &a, void *s) {
  return launch_cpa5i_set<kDecryptK>(a, (cudaStream_t)s);
}

size_t mix_table_bytes() { return sizeof(MixTable); }

void mix_table_build(void *host_dst, const CpaArgs *g, int ng) {
  MixTable *T = static_cast<MixTable *>(host_dst);
  std::memset(T, 0, sizeof(MixTable));
  T->first[0] = 0;
  for (int i = 0; i < ng && i < kMaxGroups; i++) {
    T->g[i] = g[i];
    T->first[i + 1] = T->first[i] + g[i].n;
  }
}
static_assert(kMaxGroups == kMixMaxGroups, "one group limit");
}  // namespace tmvp
