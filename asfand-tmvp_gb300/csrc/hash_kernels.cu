// hash_kernels.cu — the Keccak stages of the batched KEM: one thread per
// sponge, register-resident state, 8-byte global accesses.
//
// Replaces the reference's single-block hash kernels and its 25-lane
// shake128_gpu (TMVP-Saber/SABER-GPU/src/poly.cu:918-1114,
// TMVP_SABLE/src/fips202.cu:409-668), which cap the batch at 1024 and rely
// on implicit warp synchrony.  Every kernel here covers any batch size with a
// 1-D grid and has no inter-thread communication.
#include "hash_kernels.cuh"
#include "keccak.cuh"

namespace tmvp {

__device__ __forceinline__ void load_words(uint64_t *dst, const uint8_t *src, int nw) {
  const uint64_t *s = reinterpret_cast<const uint64_t *>(src);
#pragma unroll 4
  for (int i = 0; i < nw; i++) dst[i] = s[i];
}

__device__ __forceinline__ void run_shake_job(const ShakeJob &J, size_t i) {
  uint64_t seed[4];
  load_words(seed, J.src + i * J.src_stride + J.src_off, 4);
  if (J.prehash) {
    // seed_A <- SHAKE-128(seed_A)[0:32] (Saber round-3 key generation)
    uint64_t h[4];
    shake128_32(h, 32, seed);
#pragma unroll
    for (int k = 0; k < 4; k++) seed[k] = h[k];
    if (J.seed_out) {
      uint64_t *so = reinterpret_cast<uint64_t *>(J.seed_out + i * J.seed_out_stride + J.seed_out_off);
#pragma unroll
      for (int k = 0; k < 4; k++) so[k] = seed[k];
    }
  }
  shake128_32(reinterpret_cast<uint64_t *>(J.out + i * J.out_stride), J.out_bytes, seed);
}

__global__ void __launch_bounds__(128) k_shake_jobs(ShakeJob j0, ShakeJob j1, int n) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nal = warp_round((size_t)n);
  if (t < (size_t)n) {
    run_shake_job(j0, t);
  } else if (j1.out && t >= nal && t < nal + n) {
    run_shake_job(j1, t - nal);
  }
}

// Encapsulation front (saber_enc, cuda_kernel.cu:116-127): thread i < n runs
// m = H(coins), H(pk), kr = G(m || H(pk)) and the GenSecret stream
// SHAKE-128(kr[32:64]); threads warp_round(n) + i expand GenMatrix from pk's
// seed.
__global__ void __launch_bounds__(128) k_enc_front(KemParams P, const uint8_t *pk,
                                                    const uint8_t *coins, uint8_t *mbuf,
                                                    uint8_t *kr, uint8_t *s_stream,
                                                    uint8_t *a_stream, int n) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nal = warp_round((size_t)n);
  if (t < (size_t)n) {
    uint64_t c[4], buf[8], g[8];
    load_words(c, coins + t * 32, 4);
    sha3_256_32(buf, c);  // m
    sha3_256_words(buf + 4, reinterpret_cast<const uint64_t *>(pk + t * P.pk_bytes), P.pk_bytes);
    sha3_512_64(g, buf);
    uint64_t *mo = reinterpret_cast<uint64_t *>(mbuf + t * 64);
    uint64_t *ko = reinterpret_cast<uint64_t *>(kr + t * 64);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      mo[k] = buf[k];
      ko[k] = g[k];
    }
    uint64_t seed[4] = {g[4], g[5], g[6], g[7]};
    shake128_32(reinterpret_cast<uint64_t *>(s_stream + t * P.gs_bytes), P.gs_bytes, seed);
  } else if (t >= nal && t < nal + n) {
    const size_t i = t - nal;
    uint64_t seed[4];
    load_words(seed, pk + i * P.pk_bytes + (size_t)P.l * P.polycompbytes, 4);
    shake128_32(reinterpret_cast<uint64_t *>(a_stream + i * P.gm_bytes), P.gm_bytes, seed);
  }
}

// Decapsulation step after decryption (saber_dec, cuda_kernel.cu:378-385):
// kr = G(m' || H(pk)) and the GenSecret stream SHAKE-128(kr[32:64]).
__device__ __forceinline__ void dec_g_one(const KemParams &P, const uint8_t *mbuf, uint8_t *kr,
                                          uint8_t *s_stream, size_t t) {
  uint64_t buf[8], g[8];
  load_words(buf, mbuf + t * 64, 8);
  sha3_512_64(g, buf);
  uint64_t *ko = reinterpret_cast<uint64_t *>(kr + t * 64);
#pragma unroll
  for (int k = 0; k < 8; k++) ko[k] = g[k];
  uint64_t seed[4] = {g[4], g[5], g[6], g[7]};
  shake128_32(reinterpret_cast<uint64_t *>(s_stream + t * P.gs_bytes), P.gs_bytes, seed);
}

__global__ void __launch_bounds__(128) k_dec_g(KemParams P, const uint8_t *mbuf, uint8_t *kr,
                                                uint8_t *s_stream, int n) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (size_t)n) dec_g_one(P, mbuf, kr, s_stream, t);
}

// GenMatrix stream of public key t (seed_A at the end of pk + t * pk_stride),
// for callers that keep one expanded A per key (GenMatrix, saber_enc
// cuda_kernel.cu:116-127).
__global__ void __launch_bounds__(128) k_genmatrix(KemParams P, const uint8_t *pk, size_t pk_stride,
                                                    uint8_t *a_stream, int n) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)n) return;
  uint64_t seed[4];
  load_words(seed, pk + t * pk_stride + (size_t)P.l * P.polycompbytes, 4);
  shake128_32(reinterpret_cast<uint64_t *>(a_stream + t * P.gm_bytes), P.gm_bytes, seed);
}

// GenMatrix of instance t from the seed of the pk embedded in sk.
__device__ __forceinline__ void dec_genmatrix_one(const KemParams &P, const uint8_t *sk, uint8_t *a_stream,
                                                  size_t t) {
  uint64_t seed[4];
  load_words(seed, sk + t * P.sk_bytes + P.indcpa_sk_bytes + (size_t)P.l * P.polycompbytes, 4);
  shake128_32(reinterpret_cast<uint64_t *>(a_stream + t * P.gm_bytes), P.gm_bytes, seed);
}

// H(c) of instance i.
__device__ __forceinline__ void dec_hash_ct_one(const KemParams &P, const uint8_t *ct, uint8_t *hc, size_t i) {
  uint64_t h[4];
  sha3_256_words(h, reinterpret_cast<const uint64_t *>(ct + i * P.ct_bytes), P.ct_bytes);
  uint64_t *o = reinterpret_cast<uint64_t *>(hc + i * 32);
#pragma unroll
  for (int w = 0; w < 4; w++) o[w] = h[w];
}

// Decapsulation front, independent of the decryption: GenMatrix from the seed
// of the pk embedded in sk, and the ciphertext hash H(c) (saber_dec,
// cuda_kernel.cu:383-384 and :447).  part 0: threads i < n expand GenMatrix,
// threads warp_round(n) + i hash; part 1: GenMatrix only; part 2: H(c) only
// (n threads each).
__global__ void __launch_bounds__(128) k_dec_front(KemParams P, const uint8_t *sk,
                                                    const uint8_t *ct, uint8_t *a_stream,
                                                    uint8_t *hc, int n, int part) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nal = warp_round((size_t)n);
  if (part != 0) {
    if (t < (size_t)n) {
      if (part == 1) dec_genmatrix_one(P, sk, a_stream, t);
      else dec_hash_ct_one(P, ct, hc, t);
    }
    return;
  }
  if (t < (size_t)n)
    dec_genmatrix_one(P, sk, a_stream, t);
  else if (t >= nal && t < nal + n)
    dec_hash_ct_one(P, ct, hc, t - nal);
}

// The same 2n sponges (GenMatrix, then H(c)) from a capped grid that leaves
// room on every SM for the decryption beside it: threads stride over the
// sponges, GenMatrix ones (the longer) first.  The stride is a multiple of
// the block, so a warp's threads keep one role.
__global__ void __launch_bounds__(128) k_dec_front_strided(KemParams P, const uint8_t *sk,
                                                            const uint8_t *ct, uint8_t *a_stream,
                                                            uint8_t *hc, int n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x, nal = warp_round((size_t)n);
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nal + n; t += stride) {
    if (t < (size_t)n)
      dec_genmatrix_one(P, sk, a_stream, t);
    else if (t >= nal)
      dec_hash_ct_one(P, ct, hc, t - nal);
  }
}

// Final key derivation.  Encapsulation (cuda_kernel.cu:185-186):
// K = H(kr[0:32] || H(c)); hc, when given, holds H(c) already.  Decapsulation (cuda_kernel.cu:445-450, with the
// FO selection done as specified): K = H((fail ? z : kr[0:32]) || H(c)), the
// selection made with a mask so that it does not branch on `fail`.  sk of
// instance t at sk + t * sk_stride (0: one key for every instance).
__device__ __forceinline__ void final_key_one(const KemParams &P, const uint8_t *ct, const uint8_t *hc,
                                              const uint8_t *kr, const uint8_t *fail, const uint8_t *sk,
                                              size_t sk_stride, uint8_t *ss, size_t t) {
  uint64_t buf[8], k[4];
  load_words(buf, kr + t * 64, 4);
  if (fail) {
    uint64_t mask = 0ull - (uint64_t)(fail[t] != 0);
    uint64_t z[4];
    load_words(z, sk + t * sk_stride + P.sk_bytes - 32, 4);
#pragma unroll
    for (int w = 0; w < 4; w++) buf[w] ^= mask & (buf[w] ^ z[w]);
  }
  if (hc)
    load_words(buf + 4, hc + t * 32, 4);
  else
    sha3_256_words(buf + 4, reinterpret_cast<const uint64_t *>(ct + t * P.ct_bytes), P.ct_bytes);
  sha3_256_64(k, buf);
  uint64_t *o = reinterpret_cast<uint64_t *>(ss + t * 32);
#pragma unroll
  for (int w = 0; w < 4; w++) o[w] = k[w];
}

__global__ void __launch_bounds__(128) k_final_key(KemParams P, const uint8_t *ct,
                                                    const uint8_t *hc, const uint8_t *kr,
                                                    const uint8_t *fail, const uint8_t *sk,
                                                    size_t sk_stride, uint8_t *ss, int n) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (size_t)n) final_key_one(P, ct, hc, kr, fail, sk, sk_stride, ss, t);
}

// ---- mixed-parameter decapsulation: one launch per stage over a group table

__device__ __forceinline__ int hash_group(const HashGroup *T, int ng, int gi) {
  int lo = 0, hi = ng - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (gi >= T[mid].first) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// part 1: GenMatrix of every instance; part 2: H(c); part 0: both, threads
// warp_round(total) + i hashing.
__global__ void __launch_bounds__(128) k_mix_front(const HashGroup *T, int ng, int total, int part) {
  int gi = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  bool gen = part == 1;
  if (part == 0) {
    const int tal = (int)warp_round((size_t)total);
    gen = gi < total;
    if (!gen && (gi < tal || gi >= tal + total)) return;
    if (!gen) gi -= tal;
  } else if (gi >= total) {
    return;
  }
  const HashGroup &G = T[hash_group(T, ng, gi)];
  const size_t i = (size_t)(gi - G.first);
  if (gen) dec_genmatrix_one(G.P, G.sk, G.a_stream, i);
  else dec_hash_ct_one(G.P, G.ct, G.hc, i);
}

__global__ void __launch_bounds__(128) k_mix_g(const HashGroup *T, int ng, int total) {
  const int gi = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (gi >= total) return;
  const HashGroup &G = T[hash_group(T, ng, gi)];
  dec_g_one(G.P, G.mbuf, G.kr, G.s_stream, (size_t)(gi - G.first));
}

__global__ void __launch_bounds__(128) k_mix_final(const HashGroup *T, int ng, int total) {
  const int gi = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (gi >= total) return;
  const HashGroup &G = T[hash_group(T, ng, gi)];
  final_key_one(G.P, G.ct, G.hc, G.kr, G.fail, G.sk, (size_t)G.P.sk_bytes, G.ss, (size_t)(gi - G.first));
}

// Key-generation tail: sk[SK-64 : SK-32] = H(pk), sk[SK-32 : SK] = z.
__global__ void __launch_bounds__(128) k_kp_final(KemParams P, const uint8_t *pk, uint8_t *sk,
                                                   const uint8_t *coins, int n) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)n) return;
  uint64_t h[4], z[4];
  sha3_256_words(h, reinterpret_cast<const uint64_t *>(pk + t * P.pk_bytes), P.pk_bytes);
  load_words(z, coins + t * 96 + 64, 4);
  uint64_t *o = reinterpret_cast<uint64_t *>(sk + t * P.sk_bytes + P.sk_bytes - 64);
#pragma unroll
  for (int w = 0; w < 4; w++) {
    o[w] = h[w];
    o[4 + w] = z[w];
  }
}

// Standalone SHA3-256 / SHA3-512 / SHAKE-128 over a batch (used by tests and
// by the single-instance API).
__global__ void k_sha3_256_batch(const uint8_t *in, int inbytes, uint8_t *out, int n) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)n) return;
  uint64_t h[4];
  sha3_256_words(h, reinterpret_cast<const uint64_t *>(in + t * inbytes), inbytes);
  uint64_t *o = reinterpret_cast<uint64_t *>(out + t * 32);
#pragma unroll
  for (int w = 0; w < 4; w++) o[w] = h[w];
}

// dst[i * words + w] = src[w] for i < n (16-byte words): one key's bytes and
// its expanded A repeated per instance, for the one-key decapsulation.  Blocks
// take instances, threads the words of one (coalesced stores; the source
// stays in L1).
__global__ void __launch_bounds__(256) k_replicate16(uint4 *dst, const uint4 *src, int words, size_t n) {
  for (size_t i = blockIdx.x; i < n; i += gridDim.x) {
    uint4 *d = dst + i * (size_t)words;
    for (int w = threadIdx.x; w < words; w += blockDim.x) d[w] = src[w];
  }
}

}  // namespace tmvp
