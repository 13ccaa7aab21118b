// cpa_dispatch.cu — runtime dispatch of the IND-CPA kernels over (form, op).
#include <cuda_runtime.h>

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
#undef TMVP_DECL_FORM

typedef int (*cpa_fn)(const CpaArgs &, cudaStream_t);

int cpa_launch(int form, int op, const CpaArgs &a, void *stream) {
  static const cpa_fn tab[6][5] = {
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
  };
  if (form < 0 || form > 5 || op < 0 || op > 4 || !tab[form][op]) return (int)cudaErrorInvalidValue;
  return tab[form][op](a, (cudaStream_t)stream);
}

}  // namespace tmvp
