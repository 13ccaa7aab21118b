// cpa_dispatch.cu — runtime dispatch of the IND-CPA kernels over (form, op).
#include <cuda_runtime.h>

#include <atomic>

#include "cpa_kernels.cuh"

namespace tmvp {

#define TMVP_DECL_FORM(f)                                          \
  int cpa_launch_##f##_decrypt(const CpaArgs &, cudaStream_t);     \
  int cpa_launch_##f##_encrypt(const CpaArgs &, cudaStream_t);     \
  int cpa_launch_##f##_reenc(const CpaArgs &, cudaStream_t);       \
  int cpa_launch_##f##_keygen(const CpaArgs &, cudaStream_t);      \
  int cpa_launch_##f##_matvec(const CpaArgs &, cudaStream_t);
TMVP_DECL_FORM(fp8)
TMVP_DECL_FORM(int8)
TMVP_DECL_FORM(cc)
TMVP_DECL_FORM(sb)
TMVP_DECL_FORM(f8u)
TMVP_DECL_FORM(dp2a)
TMVP_DECL_FORM(tc4)
#undef TMVP_DECL_FORM
int cpa_launch_mixed_decrypt(const CpaArgs *, int, const MixTable *, cudaStream_t, int);
int cpa_launch_mixed_encrypt(const CpaArgs *, int, const MixTable *, cudaStream_t, int);
int cpa_launch_mixed_reenc(const CpaArgs *, int, const MixTable *, cudaStream_t, int);
int cpa_launch_mixed_keygen(const CpaArgs *, int, const MixTable *, cudaStream_t, int);
int cpa_launch_mixed_matvec(const CpaArgs *, int, const MixTable *, cudaStream_t, int);

typedef int (*cpa_fn)(const CpaArgs &, cudaStream_t);

int cpa_launch(int form, int op, const CpaArgs &a, void *stream) {
  static const cpa_fn tab[8][5] = {
      {cpa_launch_cc_decrypt, cpa_launch_cc_encrypt, cpa_launch_cc_reenc, cpa_launch_cc_keygen,
       cpa_launch_cc_matvec},
      {cpa_launch_int8_decrypt, cpa_launch_int8_encrypt, cpa_launch_int8_reenc,
       cpa_launch_int8_keygen, cpa_launch_int8_matvec},
      {cpa_launch_fp8_decrypt, cpa_launch_fp8_encrypt, cpa_launch_fp8_reenc, cpa_launch_fp8_keygen,
       cpa_launch_fp8_matvec},
      {nullptr, nullptr, nullptr, nullptr, nullptr},
      {cpa_launch_sb_decrypt, cpa_launch_sb_encrypt, cpa_launch_sb_reenc, cpa_launch_sb_keygen,
       cpa_launch_sb_matvec},
      {cpa_launch_f8u_decrypt, cpa_launch_f8u_encrypt, cpa_launch_f8u_reenc, cpa_launch_f8u_keygen,
       cpa_launch_f8u_matvec},
      {cpa_launch_dp2a_decrypt, cpa_launch_dp2a_encrypt, cpa_launch_dp2a_reenc, cpa_launch_dp2a_keygen,
       cpa_launch_dp2a_matvec},
      {cpa_launch_tc4_decrypt, cpa_launch_tc4_encrypt, cpa_launch_tc4_reenc, cpa_launch_tc4_keygen,
       cpa_launch_tc4_matvec},
  };
  if (form < 0 || form > 7 || op < 0 || op > 4 || !tab[form][op]) return (int)cudaErrorInvalidValue;
  return tab[form][op](a, (cudaStream_t)stream);
}

int cpa_launch_mixed(int op, const CpaArgs *g, int ng, const MixTable *dev_tab, void *stream, int ctas_per_sm) {
  typedef int (*mix_fn)(const CpaArgs *, int, const MixTable *, cudaStream_t, int);
  static const mix_fn tab[5] = {cpa_launch_mixed_decrypt, cpa_launch_mixed_encrypt, cpa_launch_mixed_reenc,
                                cpa_launch_mixed_keygen, cpa_launch_mixed_matvec};
  if (op < 0 || op > 4) return (int)cudaErrorInvalidValue;
  return tab[op](g, ng, dev_tab, (cudaStream_t)stream, ctas_per_sm);
}

namespace {
struct TuneTable {
  std::atomic<int> v[5][6];
  TuneTable() {
    for (auto &row : v)
      for (auto &x : row) x.store(-1);
  }
};
TuneTable g_tune;
}

int persist_ctas_per_sm(int op, int set) {
  if (op < 0 || op > 4 || set < 0 || set > 5) return -1;
  return g_tune.v[op][set].load(std::memory_order_relaxed);
}

void persist_set_ctas_per_sm(int op, int set, int ctas) {
  if (op < 0 || op > 4 || set < 0 || set > 5) return;
  g_tune.v[op][set].store(ctas < -1 ? -1 : ctas, std::memory_order_relaxed);
}

}  // namespace tmvp
