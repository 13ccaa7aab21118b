// cpa_kernels.cuh — IND-CPA kernels of the batched KEM (one CTA per instance).
//
// Ops (reference launch sequences they replace):
//   kDecrypt  indcpa_kem_dec   SABER cuda_kernel.cu:341-370 / SABLE_indcpa.cu:428-461
//   kEncrypt  indcpa_kem_enc   SABER cuda_kernel.cu:124-178 / SABLE_indcpa.cu:149-224
//   kReenc    the re-encryption + compare of decapsulation
//                              SABER cuda_kernel.cu:383-445 / SABLE_indcpa.cu:473-551
//   kKeygen   indcpa_kem_keypair (Saber round 3; not in the reference)
//   kMatvec   MatrixVectorMul alone (SABER poly.cu:269-376, :1396-1453)
#pragma once
#include <cstddef>
#include <cstdint>

#include "kem_common.cuh"

namespace tmvp {

enum CpaOp : int { kDecrypt = 0, kEncrypt = 1, kReenc = 2, kKeygen = 3, kMatvec = 4 };
// Decryption of several ciphertexts under one key per CTA (tcgen05 form
// only; not in the per-op dispatch tables): the key's secret is staged once
// and the ciphertexts' b' digit columns share every MMA.
constexpr int kDecryptK = 5;

struct CpaArgs {
  KemParams P;
  int n;
  // kEncrypt / kReenc / kKeygen: raw SHAKE streams
  const uint8_t *a_stream;  // [n][gm_bytes]
  const uint8_t *s_stream;  // [n][gs_bytes]
  // public vector b (pk's packed part): pk + i*pk_stride + pk_off
  const uint8_t *pk;
  size_t pk_stride, pk_off;
  // message (32 bytes): msg + i*msg_stride
  const uint8_t *msg;
  size_t msg_stride;
  const uint8_t *ct;  // [n][ct_bytes] (kDecrypt input, kReenc compare)
  const uint8_t *sk;  // [n][sk_bytes] (kDecrypt)
  uint8_t *ct_out;    // kEncrypt
  uint8_t *fail;      // kReenc: 1 where the re-encryption differs
  uint8_t *m_out;     // kDecrypt: [n][64] = m' || H(pk) (H(pk) only if sk has one)
  size_t m_out_stride;
  int copy_hpk;       // kDecrypt: copy sk's H(pk) into m_out[32:64]
  uint8_t *pk_out, *sk_out;  // kKeygen (sk_out: indcpa part || pk; stride sk_stride)
  size_t sk_stride;
  // kMatvec
  const uint16_t *mv_A;
  const int8_t *mv_s;
  uint16_t *mv_out;
  int mv_eq, mv_transpose;
  int *err;           // set when a secret coefficient is outside the form's range
  // tcgen05 per-instance kernel only, for tmvp_selftest_bounded_wait: the
  // input barrier expects 16 bytes more than the copies bring, so its
  // bounded wait runs out (nothing else changes; the copies all land)
  int stall_inputs;
  // tcgen05 per-instance kernel only: sk (decryption) and a_stream
  // (re-encryption) hold one key for every instance (stride 0)
  int key_shared;
};

// Launch over a.n instances on `stream`.  Returns a CUDA error code (0 on
// success).
int cpa_launch(int form, int op, const CpaArgs &a, void *stream);

// kDecryptK over a.n ciphertexts, all under the key at a.sk (a.key_shared
// is implied): ceil(n / per-CTA count) CTAs.
int cpa_launch_decrypt_onekey(const CpaArgs &a, void *stream);

// tcgen05 form only: one persistent launch over `ngroups` (<= kMixMaxGroups)
// groups of instances, each with its own parameter set and buffers.  groups:
// host copies; dev_tab: the same groups as a device table (mix_table_build
// into mix_table_bytes() of device memory; unused when ngroups == 1).
// ctas_per_sm >= 0: the persistent kernel with that many CTAs per SM (0 = as
// many as fit); -1: one CTA per instance over all groups (not for matvec).
constexpr int kMixMaxGroups = 64;
struct MixTable;
size_t mix_table_bytes();
void mix_table_build(void *host_dst, const CpaArgs *groups, int ngroups);
int cpa_launch_mixed(int op, const CpaArgs *groups, int ngroups, const MixTable *dev_tab, void *stream,
                     int ctas_per_sm);

// Launch shape of the tcgen05 kernels per (op, parameter set): -1 = one CTA
// per instance; n >= 0 = the persistent kernel with n CTAs per SM (0 = as many
// as fit).  Default -1; written by the autotuner.
int persist_ctas_per_sm(int op, int set);
void persist_set_ctas_per_sm(int op, int set, int ctas);

}  // namespace tmvp
