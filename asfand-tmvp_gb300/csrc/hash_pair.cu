// hash_pair.cu — the Keccak stages of the batched KEM with two threads per
// sponge (keccak_pair.cuh): the form the host picks for launches too large
// for one warp per sponge and too small to fill the integer pipe with one
// thread per sponge.  Each kernel has the same roles, inputs and outputs as
// its thread-per-sponge counterpart in hash_kernels.cu.
//
// Thread t serves half t & 1 of sponge t >> 1 of its role.  A kernel with two
// roles starts the second at thread warp_round(2n), so every warp holds one
// role (their loops differ in length).  No thread leaves before the
// shuffles: threads past the last sponge of their role work on that sponge
// again and store nothing.
#include "hash_kernels.cuh"
#include "keccak_pair.cuh"

namespace tmvp {

namespace {

struct PairCtx {
  int me;       // 0: low halves, 1: high halves
  int role;     // 0 or 1
  size_t i;     // sponge index within the role (clamped)
  bool live;    // this thread's stores count
};

// n sponges per role; two_roles: the second role's threads follow at
// warp_round(2n).
__device__ __forceinline__ PairCtx pair_ctx(int n, bool two_roles) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nal = warp_round(2 * (size_t)n);
  PairCtx c;
  c.me = (int)(t & 1);
  size_t local = t;
  c.role = 0;
  if (two_roles && t >= nal) {
    c.role = 1;
    local = t - nal;
  }
  c.live = local < 2 * (size_t)n;
  c.i = c.live ? local >> 1 : (size_t)n - 1;
  return c;
}

__device__ __forceinline__ void load_halves(uint32_t *dst, const uint8_t *src, int me, int nw) {
  const uint32_t *s = reinterpret_cast<const uint32_t *>(src) + me;
#pragma unroll
  for (int k = 0; k < nw; k++) dst[k] = s[2 * k];
}

__device__ __forceinline__ void store_halves(uint8_t *dst, const uint32_t *src, int me, int nw, bool live) {
  if (!live) return;
  uint32_t *d = reinterpret_cast<uint32_t *>(dst) + me;
#pragma unroll
  for (int k = 0; k < nw; k++) d[2 * k] = src[k];
}

// SHAKE-128 squeeze of nbytes from a 32-byte seed (halves s[0..3]); only a
// live thread stores.
__device__ __forceinline__ void p_shake128_seed(const PairCtx &c, const uint32_t (&s)[4], uint8_t *out,
                                                int nbytes) {
  uint32_t w[25];
  pair_zero(w);
#pragma unroll
  for (int k = 0; k < 4; k++) w[k] = s[k];
  w[4] ^= pair_half(0x1Full, c.me);
  w[20] ^= pair_half(0x8000000000000000ull, c.me);
  uint32_t *o32 = reinterpret_cast<uint32_t *>(out) + c.me;
  int nw = nbytes >> 3;
  while (nw > 0) {
    pair_keccak_f1600(w, c.me);
    const int k = nw < 21 ? nw : 21;
    if (c.live) {
#pragma unroll
      for (int q = 0; q < 21; q++)
        if (q < k) o32[2 * q] = w[q];
    }
    o32 += 2 * 21;
    nw -= k;
  }
}

__device__ __forceinline__ void p_dec_genmatrix(const PairCtx &c, const KemParams &P, const uint8_t *sk,
                                                uint8_t *a_stream) {
  uint32_t s[4];
  load_halves(s, sk + c.i * P.sk_bytes + P.indcpa_sk_bytes + (size_t)P.l * P.polycompbytes, c.me, 4);
  p_shake128_seed(c, s, a_stream + c.i * P.gm_bytes, P.gm_bytes);
}

__device__ __forceinline__ void p_dec_hash_ct(const PairCtx &c, const KemParams &P, const uint8_t *ct,
                                              uint8_t *hc) {
  uint32_t h[4];
  pair_sha3_256_mem(c.me, ct + c.i * P.ct_bytes, P.ct_bytes, h);
  store_halves(hc + c.i * 32, h, c.me, 4, c.live);
}

}  // namespace

// Decapsulation front (k_dec_front): part 0: GenMatrix sponges, then the H(c)
// sponges from thread warp_round(2n); part 1: GenMatrix only; part 2: H(c)
// only.
__global__ void __launch_bounds__(128) k_dec_front_p(KemParams P, const uint8_t *sk, const uint8_t *ct,
                                                     uint8_t *a_stream, uint8_t *hc, int n, int part) {
  const PairCtx c = pair_ctx(n, part == 0);
  if (part == 2 || c.role == 1)
    p_dec_hash_ct(c, P, ct, hc);
  else
    p_dec_genmatrix(c, P, sk, a_stream);
}

// kr = G(m' || H(pk)) and the GenSecret stream SHAKE-128(kr[32:64]) (k_dec_g).
__global__ void __launch_bounds__(128) k_dec_g_p(KemParams P, const uint8_t *mbuf, uint8_t *kr, uint8_t *s_stream,
                                                 int n) {
  const PairCtx c = pair_ctx(n, false);
  uint32_t m[8], g[8];
  load_halves(m, mbuf + c.i * 64, c.me, 8);
  pair_sha3_lanes<9>(c.me, m, 8, g, 8);
  store_halves(kr + c.i * 64, g, c.me, 8, c.live);
  const uint32_t s[4] = {g[4], g[5], g[6], g[7]};
  p_shake128_seed(c, s, s_stream + c.i * P.gs_bytes, P.gs_bytes);
}

// K = H((fail ? z : kr[0:32]) || H(c)) (k_final_key), the selection by mask.
__global__ void __launch_bounds__(128) k_final_key_p(KemParams P, const uint8_t *ct, const uint8_t *hc,
                                                     const uint8_t *kr, const uint8_t *fail, const uint8_t *sk,
                                                     size_t sk_stride, uint8_t *ss, int n) {
  const PairCtx c = pair_ctx(n, false);
  uint32_t m[8];
  load_halves(m, kr + c.i * 64, c.me, 4);
  if (fail) {
    const uint32_t mask = 0u - (uint32_t)(fail[c.i] != 0);
    uint32_t z[4];
    load_halves(z, sk + c.i * sk_stride + P.sk_bytes - 32, c.me, 4);
#pragma unroll
    for (int k = 0; k < 4; k++) m[k] ^= mask & (m[k] ^ z[k]);
  }
  if (hc) {
    load_halves(m + 4, hc + c.i * 32, c.me, 4);
  } else {
    uint32_t h[4];
    pair_sha3_256_mem(c.me, ct + c.i * P.ct_bytes, P.ct_bytes, h);
#pragma unroll
    for (int k = 0; k < 4; k++) m[4 + k] = h[k];
  }
  uint32_t k4[4];
  pair_sha3_lanes<17>(c.me, m, 8, k4, 4);
  store_halves(ss + c.i * 32, k4, c.me, 4, c.live);
}

// Encapsulation front (k_enc_front): role 0 runs m = H(coins), H(pk),
// kr = G(m || H(pk)) and the GenSecret stream; with_gm: role 1 expands
// GenMatrix from pk's seed.
__global__ void __launch_bounds__(128) k_enc_front_p(KemParams P, const uint8_t *pk, const uint8_t *coins,
                                                     uint8_t *mbuf, uint8_t *kr, uint8_t *s_stream,
                                                     uint8_t *a_stream, int n, int with_gm) {
  const PairCtx c = pair_ctx(n, with_gm != 0);
  if (c.role == 0) {
    uint32_t co[4], buf[8], g[8], h[4];
    load_halves(co, coins + c.i * 32, c.me, 4);
    pair_sha3_lanes<17>(c.me, co, 4, buf, 4);  // m
    pair_sha3_256_mem(c.me, pk + c.i * P.pk_bytes, P.pk_bytes, h);
#pragma unroll
    for (int k = 0; k < 4; k++) buf[4 + k] = h[k];
    store_halves(mbuf + c.i * 64, buf, c.me, 8, c.live);
    pair_sha3_lanes<9>(c.me, buf, 8, g, 8);
    store_halves(kr + c.i * 64, g, c.me, 8, c.live);
    const uint32_t s[4] = {g[4], g[5], g[6], g[7]};
    p_shake128_seed(c, s, s_stream + c.i * P.gs_bytes, P.gs_bytes);
  } else {
    uint32_t s[4];
    load_halves(s, pk + c.i * P.pk_bytes + (size_t)P.l * P.polycompbytes, c.me, 4);
    p_shake128_seed(c, s, a_stream + c.i * P.gm_bytes, P.gm_bytes);
  }
}

// GenMatrix stream of public key i (k_genmatrix).
__global__ void __launch_bounds__(128) k_genmatrix_p(KemParams P, const uint8_t *pk, size_t pk_stride,
                                                     uint8_t *a_stream, int n) {
  const PairCtx c = pair_ctx(n, false);
  uint32_t s[4];
  load_halves(s, pk + c.i * pk_stride + (size_t)P.l * P.polycompbytes, c.me, 4);
  p_shake128_seed(c, s, a_stream + c.i * P.gm_bytes, P.gm_bytes);
}

// Two SHAKE-128 jobs over n instances (k_shake_jobs): role 0 runs j0, role 1
// (from thread warp_round(2n)) runs j1 when it is set.
__global__ void __launch_bounds__(128) k_shake_jobs_p(ShakeJob j0, ShakeJob j1, int n) {
  const PairCtx c = pair_ctx(n, j1.out != nullptr);
  const ShakeJob J = c.role == 0 ? j0 : j1;
  uint32_t s[4];
  load_halves(s, J.src + c.i * J.src_stride + J.src_off, c.me, 4);
  if (J.prehash) {
    // seed_A <- SHAKE-128(seed_A)[0:32]
    uint32_t w[25];
    pair_zero(w);
#pragma unroll
    for (int k = 0; k < 4; k++) w[k] = s[k];
    w[4] ^= pair_half(0x1Full, c.me);
    w[20] ^= pair_half(0x8000000000000000ull, c.me);
    pair_keccak_f1600(w, c.me);
#pragma unroll
    for (int k = 0; k < 4; k++) s[k] = w[k];
    if (J.seed_out) store_halves(J.seed_out + c.i * J.seed_out_stride + J.seed_out_off, s, c.me, 4, c.live);
  }
  p_shake128_seed(c, s, J.out + c.i * J.out_stride, J.out_bytes);
}

// Key-generation tail (k_kp_final): sk[SK-64 : SK-32] = H(pk), sk[SK-32 : SK] = z.
__global__ void __launch_bounds__(128) k_kp_final_p(KemParams P, const uint8_t *pk, uint8_t *sk,
                                                    const uint8_t *coins, int n) {
  const PairCtx c = pair_ctx(n, false);
  uint32_t h[4], t[8];
  pair_sha3_256_mem(c.me, pk + c.i * P.pk_bytes, P.pk_bytes, h);
#pragma unroll
  for (int k = 0; k < 4; k++) t[k] = h[k];
  load_halves(t + 4, coins + c.i * 96 + 64, c.me, 4);
  store_halves(sk + c.i * P.sk_bytes + P.sk_bytes - 64, t, c.me, 8, c.live);
}

}  // namespace tmvp
