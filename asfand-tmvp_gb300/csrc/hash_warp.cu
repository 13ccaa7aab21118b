// hash_warp.cu — the Keccak stages of the batched KEM with one warp per
// sponge (keccak_warp.cuh): the forms the host picks when a launch has few
// sponges, so that the GPU is far from full and a sponge's chain of
// permutations sets the time.  Each kernel has the same roles, inputs and
// outputs as its thread-per-sponge counterpart in hash_kernels.cu.  Blocks
// are one warp and sponge w of a launch is block w: the guards and role
// branches then depend on blockIdx alone, which the compiler knows to be
// uniform (a guard on a warp index derived from threadIdx made it guard every
// shuffle, 40% slower).
#include "hash_kernels.cuh"
#include "keccak_warp.cuh"

namespace tmvp {

namespace {

struct WarpCtx {
  int lane;
  size_t w;
  WarpKeccakLane L;
};

__device__ __forceinline__ WarpCtx warp_ctx() {
  WarpCtx c;
  c.lane = (int)threadIdx.x;
  c.w = blockIdx.x;
  c.L = warp_keccak_lane(c.lane);
  return c;
}

__device__ __forceinline__ uint64_t lane_load(const uint8_t *p, int lane, int nw) {
  return lane < nw ? reinterpret_cast<const uint64_t *>(p)[lane] : 0ull;
}

__device__ __forceinline__ void lane_store(uint8_t *p, int lane, int nw, uint64_t v) {
  if (lane < nw) reinterpret_cast<uint64_t *>(p)[lane] = v;
}

// lane k takes the word of lane (k + from) mod 32
__device__ __forceinline__ uint64_t lanes_down(uint64_t v, int lane, int from) {
  const uint32_t lo = __shfl_sync(0xFFFFFFFFu, (uint32_t)v, (lane + from) & 31);
  const uint32_t hi = __shfl_sync(0xFFFFFFFFu, (uint32_t)(v >> 32), (lane + from) & 31);
  return ((uint64_t)hi << 32) | lo;
}

// SHAKE-128 of a 32-byte seed held in lanes 0..3 (one word each), squeezed
// to out (nbytes, a multiple of 8).
__device__ __forceinline__ void w_shake128_seed(const WarpCtx &c, uint64_t seed, uint64_t *out, int nbytes) {
  uint32_t lo, hi;
  warp_absorb_lanes<21>(lo, hi, c.lane, seed, 4, 0x1F);
  warp_shake128_squeeze(lo, hi, c.L, c.lane, out, nbytes);
}

// SHA3-256 of nbytes (multiple of 8) at in: the digest in lanes 0..3.
__device__ __forceinline__ uint64_t w_sha3_256_mem(const WarpCtx &c, const uint8_t *in, int nbytes) {
  uint32_t lo, hi;
  warp_absorb_words<17>(lo, hi, c.L, c.lane, reinterpret_cast<const uint64_t *>(in), nbytes, 0x06);
  warp_keccak_f1600(lo, hi, c.L);
  return warp_lane_word(lo, hi);
}

// SHA3-256 of a message of nw words held in lanes 0..nw-1 (nw < 17).
__device__ __forceinline__ uint64_t w_sha3_256_lanes(const WarpCtx &c, uint64_t m, int nw) {
  uint32_t lo, hi;
  warp_absorb_lanes<17>(lo, hi, c.lane, m, nw, 0x06);
  warp_keccak_f1600(lo, hi, c.L);
  return warp_lane_word(lo, hi);
}

// SHA3-512 of a 64-byte message held in lanes 0..7.
__device__ __forceinline__ uint64_t w_sha3_512_64(const WarpCtx &c, uint64_t m) {
  uint32_t lo, hi;
  warp_absorb_lanes<9>(lo, hi, c.lane, m, 8, 0x06);
  warp_keccak_f1600(lo, hi, c.L);
  return warp_lane_word(lo, hi);
}

__device__ __forceinline__ void w_dec_genmatrix(const WarpCtx &c, const KemParams &P, const uint8_t *sk,
                                                uint8_t *a_stream, size_t t) {
  const uint64_t seed =
      lane_load(sk + t * P.sk_bytes + P.indcpa_sk_bytes + (size_t)P.l * P.polycompbytes, c.lane, 4);
  w_shake128_seed(c, seed, reinterpret_cast<uint64_t *>(a_stream + t * P.gm_bytes), P.gm_bytes);
}

__device__ __forceinline__ void w_dec_hash_ct(const WarpCtx &c, const KemParams &P, const uint8_t *ct, uint8_t *hc,
                                              size_t i) {
  const uint64_t h = w_sha3_256_mem(c, ct + i * P.ct_bytes, P.ct_bytes);
  lane_store(hc + i * 32, c.lane, 4, h);
}

}  // namespace

// Decapsulation front (k_dec_front): part 0: warps w < n expand GenMatrix,
// warps n..2n-1 hash the ciphertexts; part 1: GenMatrix only; part 2: H(c)
// only.
__global__ void __launch_bounds__(32) k_dec_front_w(KemParams P, const uint8_t *sk, const uint8_t *ct,
                                                     uint8_t *a_stream, uint8_t *hc, int n, int part) {
  const WarpCtx c = warp_ctx();
  if (part == 2) {
    if (c.w < (size_t)n) w_dec_hash_ct(c, P, ct, hc, c.w);
  } else if (c.w < (size_t)n) {
    w_dec_genmatrix(c, P, sk, a_stream, c.w);
  } else if (part == 0 && c.w < 2 * (size_t)n) {
    w_dec_hash_ct(c, P, ct, hc, c.w - n);
  }
}

// kr = G(m' || H(pk)) and the GenSecret stream SHAKE-128(kr[32:64]) (k_dec_g).
__global__ void __launch_bounds__(32) k_dec_g_w(KemParams P, const uint8_t *mbuf, uint8_t *kr, uint8_t *s_stream,
                                                 int n) {
  const WarpCtx c = warp_ctx();
  if (c.w >= (size_t)n) return;
  const uint64_t g = w_sha3_512_64(c, lane_load(mbuf + c.w * 64, c.lane, 8));
  lane_store(kr + c.w * 64, c.lane, 8, g);
  w_shake128_seed(c, lanes_down(g, c.lane, 4), reinterpret_cast<uint64_t *>(s_stream + c.w * P.gs_bytes),
                  P.gs_bytes);
}

// K = H((fail ? z : kr[0:32]) || H(c)) (k_final_key), the selection by mask.
__global__ void __launch_bounds__(32) k_final_key_w(KemParams P, const uint8_t *ct, const uint8_t *hc,
                                                     const uint8_t *kr, const uint8_t *fail, const uint8_t *sk,
                                                     size_t sk_stride, uint8_t *ss, int n) {
  const WarpCtx c = warp_ctx();
  if (c.w >= (size_t)n) return;
  const size_t t = c.w;
  uint64_t m = lane_load(kr + t * 64, c.lane, 4);
  if (fail) {
    const uint64_t mask = 0ull - (uint64_t)(fail[t] != 0);
    const uint64_t z = lane_load(sk + t * sk_stride + P.sk_bytes - 32, c.lane, 4);
    m ^= mask & (m ^ z);
  }
  // H(c) to lanes 4..7
  const uint64_t h = hc ? lane_load(hc + t * 32, c.lane, 4) : w_sha3_256_mem(c, ct + t * P.ct_bytes, P.ct_bytes);
  const uint64_t hup = lanes_down(h, c.lane, 28);  // lane k takes lane k - 4
  if (c.lane >= 4 && c.lane < 8) m = hup;
  const uint64_t k = w_sha3_256_lanes(c, m, 8);
  lane_store(ss + t * 32, c.lane, 4, k);
}

// Encapsulation front (k_enc_front): warps w < n run m = H(coins), H(pk),
// kr = G(m || H(pk)) and the GenSecret stream; with_gm: warps n..2n-1 expand
// GenMatrix from pk's seed.
__global__ void __launch_bounds__(32) k_enc_front_w(KemParams P, const uint8_t *pk, const uint8_t *coins,
                                                     uint8_t *mbuf, uint8_t *kr, uint8_t *s_stream,
                                                     uint8_t *a_stream, int n, int with_gm) {
  const WarpCtx c = warp_ctx();
  if (c.w < (size_t)n) {
    const size_t t = c.w;
    const uint64_t mh = w_sha3_256_lanes(c, lane_load(coins + t * 32, c.lane, 4), 4);
    const uint64_t hpk = w_sha3_256_mem(c, pk + t * P.pk_bytes, P.pk_bytes);
    const uint64_t hup = lanes_down(hpk, c.lane, 28);
    const uint64_t buf = c.lane < 4 ? mh : hup;  // m || H(pk) in lanes 0..7
    lane_store(mbuf + t * 64, c.lane, 8, buf);
    const uint64_t g = w_sha3_512_64(c, buf);
    lane_store(kr + t * 64, c.lane, 8, g);
    w_shake128_seed(c, lanes_down(g, c.lane, 4), reinterpret_cast<uint64_t *>(s_stream + t * P.gs_bytes),
                    P.gs_bytes);
  } else if (with_gm && c.w < 2 * (size_t)n) {
    const size_t i = c.w - n;
    const uint64_t seed = lane_load(pk + i * P.pk_bytes + (size_t)P.l * P.polycompbytes, c.lane, 4);
    w_shake128_seed(c, seed, reinterpret_cast<uint64_t *>(a_stream + i * P.gm_bytes), P.gm_bytes);
  }
}

// GenMatrix stream of public key t (k_genmatrix).
__global__ void __launch_bounds__(32) k_genmatrix_w(KemParams P, const uint8_t *pk, size_t pk_stride,
                                                     uint8_t *a_stream, int n) {
  const WarpCtx c = warp_ctx();
  if (c.w >= (size_t)n) return;
  const uint64_t seed = lane_load(pk + c.w * pk_stride + (size_t)P.l * P.polycompbytes, c.lane, 4);
  w_shake128_seed(c, seed, reinterpret_cast<uint64_t *>(a_stream + c.w * P.gm_bytes), P.gm_bytes);
}

namespace {
__device__ __forceinline__ void w_shake_job(const WarpCtx &c, const ShakeJob &J, size_t i) {
  uint64_t seed = lane_load(J.src + i * J.src_stride + J.src_off, c.lane, 4);
  if (J.prehash) {
    // seed_A <- SHAKE-128(seed_A)[0:32]
    uint32_t lo, hi;
    warp_absorb_lanes<21>(lo, hi, c.lane, seed, 4, 0x1F);
    warp_keccak_f1600(lo, hi, c.L);
    seed = c.lane < 4 ? warp_lane_word(lo, hi) : 0ull;
    if (J.seed_out) lane_store(J.seed_out + i * J.seed_out_stride + J.seed_out_off, c.lane, 4, seed);
  }
  w_shake128_seed(c, seed, reinterpret_cast<uint64_t *>(J.out + i * J.out_stride), J.out_bytes);
}
}  // namespace

// Two SHAKE-128 jobs over n instances (k_shake_jobs): warps w < n run j0,
// warps n..2n-1 run j1 when it is set.
__global__ void __launch_bounds__(32) k_shake_jobs_w(ShakeJob j0, ShakeJob j1, int n) {
  const WarpCtx c = warp_ctx();
  if (c.w < (size_t)n) w_shake_job(c, j0, c.w);
  else if (j1.out && c.w < 2 * (size_t)n) w_shake_job(c, j1, c.w - n);
}

// Key-generation tail (k_kp_final): sk[SK-64 : SK-32] = H(pk), sk[SK-32 : SK] = z.
__global__ void __launch_bounds__(32) k_kp_final_w(KemParams P, const uint8_t *pk, uint8_t *sk,
                                                    const uint8_t *coins, int n) {
  const WarpCtx c = warp_ctx();
  if (c.w >= (size_t)n) return;
  const size_t t = c.w;
  const uint64_t h = w_sha3_256_mem(c, pk + t * P.pk_bytes, P.pk_bytes);
  const uint64_t z = lanes_down(lane_load(coins + t * 96 + 64, c.lane, 4), c.lane, 28);
  lane_store(sk + t * P.sk_bytes + P.sk_bytes - 64, c.lane, 8, c.lane < 4 ? h : z);
}

}  // namespace tmvp
