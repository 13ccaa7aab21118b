// hash_kernels.cuh — declarations of the Keccak-stage kernels.
#pragma once
#include <cstddef>
#include <cstdint>

#include "kem_common.cuh"

namespace tmvp {

// One SHAKE-128 expansion per instance: 32-byte seed at
// src + i*src_stride + src_off (8-byte aligned), out_bytes (multiple of 8)
// written to out + i*out_stride.  prehash: the seed is first replaced by
// SHAKE-128(seed)[0:32] and, if seed_out is set, stored there.
struct ShakeJob {
  const uint8_t *src;
  size_t src_stride, src_off;
  uint8_t *out;
  size_t out_stride;
  int out_bytes;
  int prehash;
  uint8_t *seed_out;
  size_t seed_out_stride, seed_out_off;
};

// The form of a Keccak launch.  One thread per sponge (this file's kernels)
// keeps a warp's share of the integer pipe busy: ~4.7 us per permutation
// however idle the GPU is, and the best rate once the pipe is full.  One warp
// per sponge (the _w kernels): ~2.1 us per permutation until its shuffles
// fill the SMs (~1 K GenMatrix sponges).  Two threads per sponge (the _p
// kernels): ~3.3 us per permutation up to ~10 K sponges, the thread form's
// integer work per sponge with twice its warps.  Launches of short sponges
// (G, the final key, the key-generation tail: 1-10 permutations) count four
// times against the warp form's limit and twice against the pair form's:
// beside the other stages of a pass they lose there sooner (at batch 32768,
// G and the final key in the pair form: 0.662 against 0.650 ms per pass,
// while a GenMatrix + H(c) front of 32768 sponges gains: 0.352 against 0.369
// ms at batch 16384).  kWarpHashDefault / kPairHashDefault are the limits a
// context starts with (tmvp_ctx_set_warp_hash / _pair_hash).
constexpr size_t kWarpHashDefault = 1024, kPairHashDefault = 32768;
enum HashForm { kHashThread, kHashWarp, kHashPair };
inline HashForm hash_form_for(size_t sponges, bool short_sponges, size_t warp_max, size_t pair_max) {
  if ((short_sponges ? 4 * sponges : sponges) <= warp_max) return kHashWarp;
  if ((short_sponges ? 2 * sponges : sponges) <= pair_max) return kHashPair;
  return kHashThread;
}

// Kernels with two sponge roles over n instances start the second role at
// thread warp_round(n), so that no warp runs both roles: their loops differ
// in length, and a warp holding both would run one after the other.  Their
// grids cover warp_round(n) + n threads.
__host__ __device__ inline size_t warp_round(size_t n) { return (n + 31) & ~(size_t)31; }

__global__ void k_shake_jobs(ShakeJob j0, ShakeJob j1, int n);
__global__ void k_enc_front(KemParams P, const uint8_t *pk, const uint8_t *coins, uint8_t *mbuf,
                            uint8_t *kr, uint8_t *s_stream, uint8_t *a_stream, int n);
__global__ void k_dec_g(KemParams P, const uint8_t *mbuf, uint8_t *kr, uint8_t *s_stream, int n);
__global__ void k_genmatrix(KemParams P, const uint8_t *pk, size_t pk_stride, uint8_t *a_stream, int n);
__global__ void k_replicate16(uint4 *dst, const uint4 *src, int words, size_t n);
__global__ void k_final_key(KemParams P, const uint8_t *ct, const uint8_t *hc, const uint8_t *kr,
                            const uint8_t *fail, const uint8_t *sk, size_t sk_stride, uint8_t *ss, int n);
__global__ void k_dec_front(KemParams P, const uint8_t *sk, const uint8_t *ct, uint8_t *a_stream,
                            uint8_t *hc, int n, int part);
__global__ void k_dec_front_strided(KemParams P, const uint8_t *sk, const uint8_t *ct, uint8_t *a_stream,
                                    uint8_t *hc, int n);
__global__ void k_kp_final(KemParams P, const uint8_t *pk, uint8_t *sk, const uint8_t *coins,
                           int n);
__global__ void k_sha3_256_batch(const uint8_t *in, int inbytes, uint8_t *out, int n);

// The same stages with one warp per sponge (hash_warp.cu): sponge w of a
// launch is block w of kWarpHashBlock threads, warp_blocks(sponges) blocks.
constexpr unsigned kWarpHashBlock = 32;
inline unsigned warp_blocks(size_t sponges) { return (unsigned)sponges; }
__global__ void k_dec_front_w(KemParams P, const uint8_t *sk, const uint8_t *ct, uint8_t *a_stream, uint8_t *hc,
                              int n, int part);
__global__ void k_dec_g_w(KemParams P, const uint8_t *mbuf, uint8_t *kr, uint8_t *s_stream, int n);
__global__ void k_final_key_w(KemParams P, const uint8_t *ct, const uint8_t *hc, const uint8_t *kr,
                              const uint8_t *fail, const uint8_t *sk, size_t sk_stride, uint8_t *ss, int n);
__global__ void k_enc_front_w(KemParams P, const uint8_t *pk, const uint8_t *coins, uint8_t *mbuf, uint8_t *kr,
                              uint8_t *s_stream, uint8_t *a_stream, int n, int with_gm);
__global__ void k_genmatrix_w(KemParams P, const uint8_t *pk, size_t pk_stride, uint8_t *a_stream, int n);
__global__ void k_shake_jobs_w(ShakeJob j0, ShakeJob j1, int n);
__global__ void k_kp_final_w(KemParams P, const uint8_t *pk, uint8_t *sk, const uint8_t *coins, int n);

// The same stages with two threads per sponge (hash_pair.cu): thread t holds
// half t & 1 of sponge t >> 1; kernels with two roles start the second at
// thread warp_round(2n).  Grids of pair_blocks(threads) blocks of
// kPairHashBlock.
constexpr unsigned kPairHashBlock = 128;
inline unsigned pair_blocks(size_t threads) { return (unsigned)((threads + kPairHashBlock - 1) / kPairHashBlock); }
__global__ void k_dec_front_p(KemParams P, const uint8_t *sk, const uint8_t *ct, uint8_t *a_stream, uint8_t *hc,
                              int n, int part);
__global__ void k_dec_g_p(KemParams P, const uint8_t *mbuf, uint8_t *kr, uint8_t *s_stream, int n);
__global__ void k_final_key_p(KemParams P, const uint8_t *ct, const uint8_t *hc, const uint8_t *kr,
                              const uint8_t *fail, const uint8_t *sk, size_t sk_stride, uint8_t *ss, int n);
__global__ void k_enc_front_p(KemParams P, const uint8_t *pk, const uint8_t *coins, uint8_t *mbuf, uint8_t *kr,
                              uint8_t *s_stream, uint8_t *a_stream, int n, int with_gm);
__global__ void k_genmatrix_p(KemParams P, const uint8_t *pk, size_t pk_stride, uint8_t *a_stream, int n);
__global__ void k_shake_jobs_p(ShakeJob j0, ShakeJob j1, int n);
__global__ void k_kp_final_p(KemParams P, const uint8_t *pk, uint8_t *sk, const uint8_t *coins, int n);

// Mixed-parameter decapsulation: group g covers global instances
// [first, first + n) with its own parameters and buffers (device table).
struct HashGroup {
  KemParams P;
  int first, n;
  const uint8_t *sk, *ct;
  uint8_t *a_stream, *s_stream, *mbuf, *kr, *fail, *hc, *ss;
};
// part 1: GenMatrix; part 2: H(c)
__global__ void k_mix_front(const HashGroup *T, int ng, int total, int part);
__global__ void k_mix_g(const HashGroup *T, int ng, int total);
__global__ void k_mix_final(const HashGroup *T, int ng, int total);

}  // namespace tmvp
