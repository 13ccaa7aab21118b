// cpa5i.cuh — the tcgen05 IND-CPA kernel specialised per parameter set: one
// CTA of 256 threads per instance, with every width, count and offset a
// compile-time constant.
//
// Per instance:
//   1. the packed inputs arrive by TMA bulk copies (cp.async.bulk) issued by
//      one thread, counted on an mbarrier;
//   2. secrets (CBD or unpacked) straight into s_ext, radix-16 digit columns
//      (r16_digits, raw e4m3 bytes worth digit * 2^-9) with K reversed, then
//      the Hankel core matrices (cpa_umma.cuh);
//   3. one thread issues the 8 l tcgen05.mma (M = 128, N = 16 / 32, K = 32;
//      each window of the Hankel sequence serves both M halves through the
//      negacyclic wrap) into tensor memory and commits them to an mbarrier;
//   4. accumulators -> registers (tcgen05.ld: every digit column of one
//      coefficient per thread) -> the compare / decode / output epilogue
//      (encryption and key generation: rounded 16-bit values, then packed
//      eight coefficients at a time).
// Same results as the runtime-shaped kernels (cpa_tc_kernel.cuh,
// cpa_persist.cuh); the arithmetic per instance is the same.
#pragma once
#include <cstdint>
#include <type_traits>

#include "cpa_persist.cuh"

namespace tmvp {

// l, log2 q, log2 p, log2 T, mu, Sable (same table as make_params)
constexpr int kSetTab[6][6] = {{2, 13, 10, 3, 10, 0}, {3, 13, 10, 4, 8, 0}, {4, 13, 10, 6, 6, 0},
                               {2, 11, 9, 3, 2, 1},   {3, 11, 9, 5, 2, 1},  {4, 11, 10, 3, 2, 1}};

template <int SET>
struct SetC {
  static constexpr int L = kSetTab[SET][0], EQ = kSetTab[SET][1], EP = kSetTab[SET][2], ET = kSetTab[SET][3];
  static constexpr int MU = kSetTab[SET][4], SABLE = kSetTab[SET][5];
  static constexpr int POLYBYTES = EQ * 32, POLYCOMP = EP * 32, SCALE = ET * 32, COIN = MU * 32;
  static constexpr int PK = L * POLYCOMP + 32, INDCPA_SK = SABLE ? L * 64 : L * POLYBYTES;
  static constexpr int SK = INDCPA_SK + PK + 64, CT = L * POLYCOMP + SCALE;
  static constexpr int GM = L * L * POLYBYTES, GS = L * COIN;
  static constexpr int H1 = 1 << (EQ - EP - 1);
  static constexpr int H2 = (1 << (EP - 2)) - (1 << (EP - ET - 1)) + (1 << (EQ - EP - 1));
};

template <int OP, int SET>
struct ShapeC {
  using C = SetC<SET>;
  static constexpr int L = C::L;
  // kDecryptK: R ciphertexts per CTA, as many as fill 16 digit columns
  static constexpr int R = OP == kDecrypt    ? 1
                           : OP == kDecryptK ? 16 / r16_digits(C::EP)
                                             : (OP == kKeygen || OP == kMatvec ? L : L + 1);
  static constexpr int RA = (OP == kDecrypt || OP == kDecryptK) ? 0 : L;
  static constexpr int WA = C::EQ, WB = C::EP;
  static constexpr int DA = r16_digits(WA), DB = r16_digits(WB);
  static constexpr int NCOLS = RA * DA + (R - RA) * DB;
  static_assert(NCOLS <= 16, "at most two 8-column groups per K step");
  static constexpr int G = NCOLS <= 8 ? 1 : 2;     // 8-column groups per K step
  static constexpr int NU = 16 * G;                // N of every MMA (two K steps side by side)
  static constexpr int TMEM_COLS = 32 * G;         // two accumulator regions of NU columns
  static constexpr int col_base(int p) { return p < RA ? p * DA : RA * DA + (p - RA) * DB; }
  static constexpr int digits(int p) { return p < RA ? DA : DB; }
};

constexpr int al16c(int x) { return (x + 15) & ~15; }

// Threads per CTA (one instance): eight warps shorten every staging phase of
// an instance; tensor memory is read by warps w and w + 4 (two M halves).
constexpr int kI5Threads = 256;

// Hankel core matrices per secret polynomial: windows 0..7 (core 4w) over
// row groups 0..15 and two K chunks reach core 4 * 7 + 15 + 2 = 45.
constexpr int kHankelCores5 = 46;
constexpr int kHankelBytes5 = kHankelCores5 * 128;

// Shared-memory layout of one CTA (byte offsets).  The operand region ENG
// holds the Hankel core matrices H (l x kHankelBytes5), the digit columns B
// and s_ext; the packed GenMatrix / GenSecret / b streams and the packed
// secret key are only read before H is written, so they land inside H.
//
// Digit columns of one j: K step t (32 K rows, K reversed) has G groups of 8
// columns and sits in block t & 3, at group slots 0..G-1 for t >= 4 and
// G..2G-1 for t < 4, so one N = 16 G descriptor on block r reads step r + 4
// (columns 0..8G-1) beside step r (columns 8G..16G-1).  Within a block the
// second K chunk of every slot lies LB = 2G * 128 + 16 bytes after the
// first (the pad spreads one column's chunks over the banks).
template <int OP, int SET>
struct LayoutC {
  using C = SetC<SET>;
  using S = ShapeC<OP, SET>;
  static constexpr bool HAS_AS = OP == kEncrypt || OP == kReenc || OP == kKeygen;
  static constexpr bool HAS_B = OP == kEncrypt || OP == kReenc;
  static constexpr bool HAS_CT = OP == kReenc || OP == kDecrypt || OP == kDecryptK;
  static constexpr bool HAS_SK = OP == kDecrypt || OP == kDecryptK;
  // ciphertexts per CTA and their stride in shared memory (16 bytes of
  // slack after each for the field readers)
  static constexpr int NCT = OP == kDecryptK ? S::R : 1;
  static constexpr int CTS = al16c(C::CT + 16);
  // matvec: A as 16-bit coefficients (l x l x 512 bytes) inside H, int8 secrets after it
  static constexpr bool HAS_MV = OP == kMatvec;
  static constexpr int MV_A = C::L * C::L * 512, MV_S = C::L * 256;
  static constexpr int G = S::G;
  static constexpr int LB = 2 * G * 128 + 16;  // second K chunk of a block
  static constexpr int RB = 2 * LB;            // one block
  static constexpr int BJ = 4 * RB;            // digit columns of one j
  // byte offset of K chunk a (16 K rows, K reversed) within one j
  __host__ __device__ static constexpr int chunk_off(int a) {
    return ((a >> 1) & 3) * RB + (a < 8 ? G * 128 : 0) + (a & 1) * LB;
  }
  static constexpr int ENG = 0;
  static constexpr int H = ENG;
  static constexpr int A = H;                                    // streams inside H
  static constexpr int SS = HAS_AS ? al16c(A + C::GM + 16) : (HAS_MV ? al16c(A + MV_A) : A);
  static constexpr int B = HAS_AS ? al16c(SS + C::GS + 16) : SS;
  static constexpr int SKO = H;
  static constexpr int BM = H + C::L * kHankelBytes5;
  static constexpr int EXT = BM + C::L * BJ;
  static constexpr int ENG_END_OPS = EXT + C::L * 512;
  static constexpr int ENG_BYTES = ENG_END_OPS;  // also holds the epilogue's 16-bit values (R x 512 bytes)
  static_assert(S::R * 512 <= ENG_END_OPS, "epilogue values fit the operand region");
  static constexpr int CTO = al16c(ENG + ENG_BYTES);
  static constexpr int MSG = HAS_CT ? al16c(CTO + NCT * CTS) : CTO;
  static constexpr int SEC8 = HAS_B ? al16c(MSG + 32 + 16) : MSG;
  static constexpr int OUT = OP == kKeygen ? al16c(SEC8 + C::L * 256) : SEC8;
  static constexpr int OUT_BYTES = OP == kEncrypt ? C::CT + 16
                                   : (OP == kKeygen ? C::L * C::POLYCOMP + C::INDCPA_SK + 16 : 0);
  static constexpr int BAR = al16c(OUT + OUT_BYTES);  // mbarriers in, mma; TMEM base
  static constexpr int TOTAL = BAR + 32;
  static constexpr int IN_BYTES = (HAS_AS ? C::GM + C::GS : 0) + (HAS_B ? C::L * C::POLYCOMP + 32 : 0) +
                                  (HAS_CT ? C::CT : 0) + (HAS_SK ? C::INDCPA_SK : 0) + (HAS_MV ? MV_A + MV_S : 0);
  static_assert(!HAS_AS || B + (HAS_B ? C::L * C::POLYCOMP + 16 : 0) <= BM, "streams fit inside H");
  static_assert(!HAS_SK || C::INDCPA_SK + 16 <= C::L * kHankelBytes5, "secret key fits inside H");
  static_assert(!HAS_MV || SS + MV_S + 16 <= BM, "matvec inputs fit inside H");
};

// Eight W-bit little-endian fields from byte `byte0` (16 bytes of slack after
// the stream), as four words of two 16-bit lanes.
template <int W>
__device__ __forceinline__ void unpack8c(const uint8_t *base, int byte0, uint32_t (&X)[4]) {
  const uint32_t wp = smem_u32(base) + (uint32_t)(byte0 & ~3);
  const int sh = 8 * (byte0 & 3);
  uint32_t q[5];
#pragma unroll
  for (int i = 0; i < 5; i++) q[i] = lds32(wp + 4 * i);
  uint32_t a[4];
#pragma unroll
  for (int i = 0; i < 4; i++) a[i] = __funnelshift_r(q[i], q[i + 1], sh);
  constexpr uint32_t m = (1u << W) - 1u;
#pragma unroll
  for (int k = 0; k < 8; k += 2) {
    const int b0 = k * W, b1 = (k + 1) * W;
    const uint32_t v0 = __funnelshift_r(a[b0 >> 5], a[(b0 >> 5) + 1 < 4 ? (b0 >> 5) + 1 : 3], b0 & 31) & m;
    const uint32_t v1 = __funnelshift_r(a[b1 >> 5], a[(b1 >> 5) + 1 < 4 ? (b1 >> 5) + 1 : 3], b1 & 31) & m;
    X[k >> 1] = __byte_perm(v0, v1, 0x5410);
  }
}

// Four signed 5-bit top digits t (one per byte) as raw e4m3 bytes: t for
// t < 16, else 0x80 | (32 - t), the number t - 32 (magnitudes up to 16).
__device__ __forceinline__ uint32_t raw_sdigits4(uint32_t t) {
  const uint32_t m = ((t >> 4) & 0x01010101u) * 0xFFu;  // bytes with t >= 16
  return (m & ((0x20202020u - t) | 0x80808080u)) | (~m & t);
}

// Radix-16 digit d (r16_digits) of eight W-bit coefficients X (four words of
// two 16-bit lanes, coefficient 2i in the low lane of X[i]) as raw bytes in
// K-reversed order: .x = coefficients 7, 6, 5, 4 and .y = 3, 2, 1, 0.  The
// e4m3 byte b in 0..16 is the number b * 2^-9 (0..7 subnormal, 8..15 the
// lowest normal binade, 16 = 2^-5), so every digit is its own encoding and
// the accumulators carry the factor 2^-9.
template <int W>
__device__ __forceinline__ uint2 raw_digits8(const uint32_t (&X)[4], int d) {
  const int lo = 4 * d;
  const int wd = W - lo < 4 ? W - lo : (W - lo == 5 ? 5 : 4);
  const uint32_t mask = ((1u << wd) - 1u) * 0x01010101u;
  uint32_t a, b;
  if (lo + wd <= 8) {  // inside the low byte of each lane
    a = __byte_perm(X[2], X[3], 0x0246) >> lo;
    b = __byte_perm(X[0], X[1], 0x0246) >> lo;
  } else if (lo >= 8) {  // inside the high byte
    a = __byte_perm(X[2], X[3], 0x1357) >> (lo - 8);
    b = __byte_perm(X[0], X[1], 0x1357) >> (lo - 8);
  } else {  // across both
    a = __byte_perm(X[2] >> lo, X[3] >> lo, 0x0246);
    b = __byte_perm(X[0] >> lo, X[1] >> lo, 0x0246);
  }
  a &= mask;
  b &= mask;
  if (wd == 5) {
    a = raw_sdigits4(a);
    b = raw_sdigits4(b);
  }
  return make_uint2(a, b);
}

// Digit columns of 32 coefficients of one W-bit packed polynomial: lane m
// (0..7) of an 8-lane group takes coefficients 32m .. 32m + 31, exactly W
// aligned words of the stream at src, so that four groups (a warp) reading
// four polynomials load conflict-free, one 32-bit word per lane per load.
// Coefficient groups 4m .. 4m + 3 of 8 (K rows 8 kq .. 8 kq + 7, kq = 31 - g,
// K reversed) fill the two 16-byte K chunks a = 15 - 2m and 14 - 2m of each
// digit column, one 128-bit store each.  colbase: the digit columns of this
// j (LO::BM + j * LO::BJ as a shared-window address); cb: first column.
template <int W, class LO>
__device__ __forceinline__ void stage_digits32(const uint8_t *sm, int src, uint32_t colbase, int cb, int m) {
  const uint32_t wp = smem_u32(sm) + (uint32_t)(src + 4 * W * m);
  uint32_t w[W];
#pragma unroll
  for (int i = 0; i < W; i++) w[i] = lds32(wp + 4 * i);
  constexpr uint32_t mask = (1u << W) - 1u;
  uint32_t X[16];  // coefficients 2k, 2k + 1 as the low / high 16-bit lanes of X[k]
#pragma unroll
  for (int k = 0; k < 16; k++) {
    uint32_t v[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int bit = W * (2 * k + h), i = bit >> 5, sh = bit & 31;
      v[h] = ((sh + W <= 32) ? (w[i] >> sh) : __funnelshift_r(w[i], w[i + 1], sh)) & mask;
    }
    X[k] = __byte_perm(v[0], v[1], 0x5410);
  }
  const int a1 = 14 - 2 * m;  // and a0 = a1 + 1, LB bytes after it
  const uint32_t c1 = colbase + (uint32_t)LO::chunk_off(a1);
#pragma unroll
  for (int d = 0; d < r16_digits(W); d++) {
    uint2 v[4];
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const uint32_t Xt[4] = {X[4 * t], X[4 * t + 1], X[4 * t + 2], X[4 * t + 3]};
      v[t] = raw_digits8<W>(Xt, d);
    }
    const int n = cb + d;
    const uint32_t col = c1 + (uint32_t)((n >> 3) * 128 + (n & 7) * 16);
    sts128(col + LO::LB, v[1].x, v[1].y, v[0].x, v[0].y);  // chunk a0: kq 30 - 4m, then 31 - 4m
    sts128(col, v[3].x, v[3].y, v[2].x, v[2].y);           // chunk a1: kq 28 - 4m, then 29 - 4m
  }
}

// One instance (CTA of kI5Threads threads; sm: its dynamic shared memory).
template <int OP, int SET>
__device__ __forceinline__ void cpa5i_body(const CpaArgs &a, const unsigned inst, uint8_t *sm) {
  using C = SetC<SET>;
  using S = ShapeC<OP, SET>;
  using LO = LayoutC<OP, SET>;
  constexpr int L = C::L, NU = S::NU, NT = kI5Threads;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mbar_in = smem_u32(sm + LO::BAR), mbar_mma = mbar_in + 8;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + LO::BAR + 16);
  // kDecryptK: this CTA's ciphertexts inst0 .. inst0 + nvalid - 1 (one key)
  constexpr bool DECK = OP == kDecryptK, IS_DEC = OP == kDecrypt || DECK;
  const size_t inst0 = DECK ? (size_t)inst * LO::NCT : (size_t)inst;
  const int nvalid = DECK ? min(LO::NCT, a.n - (int)inst0) : 1;

  // 0. tensor memory, barriers, and the input copies (one thread)
  if (warp == 0) tmem_alloc(smem_u32(tmem_slot), S::TMEM_COLS);
  if (tid == 0) {
    mbar_init(mbar_in, 1);
    mbar_init(mbar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const uint32_t d = smem_u32(sm);
    const uint32_t in_bytes = DECK ? (uint32_t)(C::INDCPA_SK + nvalid * C::CT) : (uint32_t)LO::IN_BYTES;
    mbar_expect_tx(mbar_in, in_bytes + (a.stall_inputs ? 16 : 0));
    if (LO::HAS_AS) {
      bulk_g2s(d + LO::A, a.a_stream + (a.key_shared ? 0 : (size_t)inst * C::GM), C::GM, mbar_in);
      bulk_g2s(d + LO::SS, a.s_stream + (size_t)inst * C::GS, C::GS, mbar_in);
    }
    if (LO::HAS_B) {
      bulk_g2s(d + LO::B, a.pk + (size_t)inst * a.pk_stride + a.pk_off, C::L * C::POLYCOMP, mbar_in);
      bulk_g2s(d + LO::MSG, a.msg + (size_t)inst * a.msg_stride, 32, mbar_in);
    }
    if (DECK) {
      for (int r = 0; r < nvalid; r++) bulk_g2s(d + LO::CTO + r * LO::CTS, a.ct + (inst0 + r) * C::CT, C::CT, mbar_in);
    } else if (LO::HAS_CT) {
      bulk_g2s(d + LO::CTO, a.ct + (size_t)inst * C::CT, C::CT, mbar_in);
    }
    if (LO::HAS_SK)
      bulk_g2s(d + LO::SKO, a.sk + ((a.key_shared || DECK) ? 0 : (size_t)inst * C::SK), C::INDCPA_SK, mbar_in);
    if (LO::HAS_MV) {
      bulk_g2s(d + LO::A, reinterpret_cast<const uint8_t *>(a.mv_A) + (size_t)inst * LO::MV_A, LO::MV_A, mbar_in);
      bulk_g2s(d + LO::SS, reinterpret_cast<const uint8_t *>(a.mv_s) + (size_t)inst * LO::MV_S, LO::MV_S, mbar_in);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(tmem_slot);
  bool ready = true;
  if (warp == 0) ready = mbar_wait_bounded(mbar_in, 0);
  ready = __syncthreads_and(ready) != 0;

  uint32_t *sec8w = reinterpret_cast<uint32_t *>(sm + LO::SEC8);
  uint8_t *H = sm + LO::H, *Bm = sm + LO::BM;
  const uint32_t ext32 = smem_u32(sm + LO::EXT);
  bool ok = true, done = false;
  if (ready) {
    // 1. secrets, straight into s_ext (s_ext[d] = -s[d + 1] for d < 255,
    // s[d - 255] for 255 <= d <= 510, 0 at 511; 128 words per j).  Warp
    // j < L makes polynomial j: lane g encodes the words 2g, 2g + 1
    // (coefficients 8g..8g+7) and takes word 2g + 2 from the next lane
    // (word 0 for lane 31).
    // the secrets of j go to a warp that makes no digit columns where one is free
    const int sj = S::R == 1 ? warp - L : (warp - S::R + 8) % 8;
    if (sj >= 0 && sj < L) {
      const int j = sj, g = lane;
      uint32_t sb[2];
      if (IS_DEC && !C::SABLE) {
        // 13-bit two's complement (SABER pack.cu:53-84)
        constexpr uint32_t m = ((1u << C::EQ) - 1u) * 0x10001u;
        uint32_t X[4];
        unpack8c<C::EQ>(sm + LO::SKO, (32 * j + g) * C::EQ, X);
        uint32_t bad = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) bad |= ((X[i] + 0x00800080u) & m) & 0xFF00FF00u;
        ok = bad == 0u;
        sb[0] = __byte_perm(X[0], X[1], 0x6420);
        sb[1] = __byte_perm(X[2], X[3], 0x6420);
      } else {
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int w = 64 * j + 2 * g + h;
          if (OP == kMatvec) {
            sb[h] = lds32(smem_u32(sm + LO::SS) + 4 * w);  // four int8 coefficients
          } else if (IS_DEC) {
            // 2-bit two's complement (SABLE pack.cu:371-376): one byte = 4 coefficients
            const uint32_t x = sm[LO::SKO + w];
            const uint32_t spread = (x & 3u) | ((x & 0xcu) << 6) | ((x & 0x30u) << 12) | ((x & 0xc0u) << 18);
            sb[h] = spread | (((spread >> 1) & 0x01010101u) * 0xfcu);
          } else if (C::MU == 8) {
            // CBD mu = 8 (SABER poly.cu:864-887)
            const uint32_t x = lds32(smem_u32(sm + LO::SS) + 4 * w);
            uint32_t n = x - ((x >> 1) & 0x55555555u);
            n = (n & 0x33333333u) + ((n >> 2) & 0x33333333u);
            sb[h] = __vsub4(n & 0x0f0f0f0fu, (n >> 4) & 0x0f0f0f0fu);
          } else if (C::MU == 2) {
            // CBD mu = 2 (SABLE fips202.cu:625-651)
            const uint32_t x = sm[LO::SS + w];
            const uint32_t spread = (x & 3u) | ((x & 0xcu) << 6) | ((x & 0x30u) << 12) | ((x & 0xc0u) << 18);
            sb[h] = __vsub4(spread & 0x01010101u, (spread >> 1) & 0x01010101u);
          } else {
            // CBD mu = 6, 10: fields of mu bits, popcount halves
            uint32_t r = 0;
#pragma unroll
            for (int b = 0; b < 4; b++) {
              const uint32_t x = get_bits(sm + LO::SS, (4 * w + b) * C::MU, C::MU);
              const int v = __popc(x & ((1u << (C::MU / 2)) - 1u)) - __popc(x >> (C::MU / 2));
              r |= ((uint32_t)v & 0xffu) << (8 * b);
            }
            sb[h] = r;
          }
        }
      }
      ok = ok && small4(sb[0]) && small4(sb[1]);
      if (OP == kKeygen) {
        sec8w[64 * j + 2 * g] = sb[0];
        sec8w[64 * j + 2 * g + 1] = sb[1];
      }
      const uint32_t e0 = enc4<kFp8Tcgen05>(sb[0]), e1 = enc4<kFp8Tcgen05>(sb[1]);
      const uint32_t nx = __shfl_sync(0xffffffffu, e0, (lane + 1) & 31);
      const uint32_t p0 = __byte_perm(e0, e1, 0x4321), p1 = __byte_perm(e1, nx, 0x4321);
      // word 63: s_ext[255] = s[0] keeps its sign; word 127: s_ext[511] = 0
      const uint32_t n1 = p1 ^ (g == 31 ? 0x00808080u : 0x80808080u);
      const uint32_t q1 = g == 31 ? __byte_perm(e1, 0u, 0x4321) : p1;
      sts64(ext32 + 512 * j + 8 * g, p0 ^ 0x80808080u, n1);
      sts64(ext32 + 512 * j + 256 + 8 * g, p0, q1);
    }
    // 2. digit columns (K reversed, core-matrix order): lane g converts
    // coefficients 8g..8g+7 (K rows k' = 8kq+7..8kq, kq = 31 - g) of one
    // polynomial per item.  Warp p < R makes polynomial p of every j (one
    // item per j); with R == 1 (decryption) warp j makes j.  The columns past
    // NCOLS of each stored group are left as they are: they only feed
    // accumulator columns that are never read.
    const int kq = 31 - lane;
    const uint32_t bl = smem_u32(Bm) + LO::chunk_off(kq >> 1) + 8 * (kq & 1);
    auto item = [&](auto wc, uint32_t src, int cb, int j) {
      constexpr int W = decltype(wc)::value;
      uint32_t X[4];
      unpack8c<W>(sm + src, lane * W, X);
#pragma unroll
      for (int d = 0; d < r16_digits(W); d++) {
        const uint2 v = raw_digits8<W>(X, d);
        const int n = cb + d;
        sts64(bl + j * LO::BJ + (n >> 3) * 128 + (n & 7) * 16, v.x, v.y);
      }
    };
    if constexpr (OP == kMatvec) {
      // coefficients already in 16-bit lanes: digit d of the low 13 bits
      // (the result is needed mod 2^eq, eq <= 13)
      if (warp < L) {
        const int p = warp;
#pragma unroll
        for (int j = 0; j < L; j++) {
          const int ij = a.mv_transpose ? (j * L + p) : (p * L + j);
          const uint32_t src = smem_u32(sm + LO::A) + (uint32_t)(512 * ij + 16 * lane);
          uint32_t X[4];
#pragma unroll
          for (int i = 0; i < 4; i++) X[i] = lds32(src + 4 * i);
#pragma unroll
          for (int d = 0; d < S::DA; d++) {
            const uint2 v = raw_digits8<S::WA>(X, d);
            const int n = p * S::DA + d;
            sts64(bl + j * LO::BJ + (n >> 3) * 128 + (n & 7) * 16, v.x, v.y);
          }
        }
      }
    } else if constexpr (DECK) {
      // warp r makes ciphertext r's b'_j for every j (zero columns past the batch)
      if (warp < S::R) {
#pragma unroll
        for (int j = 0; j < L; j++) {
          if (warp < nvalid) {
            item(std::integral_constant<int, S::WB>{}, LO::CTO + warp * LO::CTS + 32 * j * S::WB, warp * S::DB, j);
          } else {
#pragma unroll
            for (int d0 = 0; d0 < S::DB; d0++) {
              const int n = warp * S::DB + d0;
              sts64(bl + j * LO::BJ + (n >> 3) * 128 + (n & 7) * 16, 0u, 0u);
            }
          }
        }
      }
    } else if constexpr (S::R == 1) {
      if (warp < L) item(std::integral_constant<int, S::WB>{}, LO::CTO + 32 * warp * S::WB, 0, warp);
    } else {
      // public matrix A (RA x L polynomials), then b (encryption, re-encryption):
      // four polynomials per warp, eight lanes each
      constexpr int NA = S::RA * L, NB = (S::R - S::RA) * L;
      constexpr int WA_WARPS = (NA + 3) / 4, WB_WARPS = (NB + 3) / 4;
      static_assert(WA_WARPS + WB_WARPS <= 8, "digit polynomials fit the CTA's warps");
      const uint32_t bm32 = smem_u32(Bm);
      if (warp < WA_WARPS) {
        const int t = 4 * warp + (lane >> 3);
        if (t < NA) {
          const int p = t / L, j = t % L;
          const int ij = (OP == kKeygen) ? (j * L + p) : (p * L + j);
          stage_digits32<S::WA, LO>(sm, LO::A + 32 * ij * S::WA, bm32 + (uint32_t)(j * LO::BJ), p * S::DA, lane & 7);
        }
      } else if (warp < WA_WARPS + WB_WARPS) {
        const int t = 4 * (warp - WA_WARPS) + (lane >> 3);
        if (t < NB) {
          const int pb = t / L, j = t % L;
          stage_digits32<S::WB, LO>(sm, LO::B + 32 * j * S::WB, bm32 + (uint32_t)(j * LO::BJ),
                                    S::RA * S::DA + pb * S::DB, lane & 7);
        }
      }
    }
  }
  __syncthreads();  // s_ext complete, and the streams inside H read, before H is written
  if (ready) stage_hankel_ct<L, NT, kHankelCores5>(smem_u32(H), ext32, tid);
  fence_async_smem();  // generic-proxy writes -> visible to the tensor core
  ok = __syncthreads_and(ok) != 0;
  if (!ok && tid == 0 && a.err) atomicOr(a.err, 1);

  // 3. the MMAs (one thread).  Window w of the Hankel sequence (core 4w)
  // holds rows r of s_ext[r + 32w + e]; rows 128 + r of K step t equal
  // window t + 4 for t < 4, and -(window t - 4) for t >= 4 (s_ext[d + 256] =
  // -s_ext[d] for d < 255).  The descriptor on block r reads steps r + 4 and
  // r, so window r + 4 gives (top, step r + 4 | bottom, step r) in region 0
  // and window r gives (-bottom, step r + 4 | top, step r) in region 1:
  // 8 MMAs per j, top = region0[0] + region1[1], bottom = region0[1] - region1[0].
  if (ready && tid == 0) {
    constexpr uint32_t idesc = umma_idesc_e4m3(NU);
    const uint64_t ad0 = umma_desc(smem_u32(H), 256, 128);
    const uint32_t b0 = smem_u32(Bm);
#pragma unroll
    for (int j = 0; j < L; j++) {
      const uint64_t hj = ad0 + (uint64_t)((j * kHankelBytes5) >> 4);
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const uint64_t bd = umma_desc(b0 + j * LO::BJ + r * LO::RB, LO::LB, 128);
        umma_f8(tmem, hj + (uint64_t)((4 * (r + 4) * 128) >> 4), bd, idesc, (j | r) != 0);
        umma_f8(tmem + NU, hj + (uint64_t)((4 * r * 128) >> 4), bd, idesc, (j | r) != 0);
      }
    }
    umma_commit(mbar_mma);
  }
  // 4. accumulators (one warp polls the MMA barrier, the others wait in the barrier)
  if (ready) {
    bool fin = true;
    if (warp == 0) fin = mbar_wait_bounded(mbar_mma, 0);
    done = __syncthreads_and(fin) != 0;
  }
  tc_fence_after();
  // warp w reads TMEM lanes 32 (w % 4) .. +31 for coefficient
  // k = 128 hsel + 32 q4 + lane (hsel = w / 4): every digit column of k,
  // top = region0[0] + region1[1], bottom = region0[1] - region1[0]
  const int q4 = warp & 3, hsel = warp >> 2;
  const int k = 128 * hsel + 32 * q4 + lane;
  constexpr int G8 = 8 * LO::G;
  float xacc[G8];  // digit column c of coefficient k, times 2^-9 (exact)
  if (done) {
    const uint32_t t0 = tmem + ((uint32_t)(32 * q4) << 16);
    uint32_t f[G8], g[G8];
    if constexpr (G8 == 8) {
      tmem_ld8(t0 + (hsel ? 8 : 0), f);
      tmem_ld8(t0 + (hsel ? 16 : 24), g);
    } else {
      tmem_ld16(t0 + (hsel ? 16 : 0), f);
      tmem_ld16(t0 + (hsel ? 32 : 48), g);
    }
    if (hsel) {
#pragma unroll
      for (int c = 0; c < S::NCOLS; c++) xacc[c] = __uint_as_float(f[c]) - __uint_as_float(g[c]);
    } else {
#pragma unroll
      for (int c = 0; c < S::NCOLS; c++) xacc[c] = __uint_as_float(f[c]) + __uint_as_float(g[c]);
    }
    if constexpr (OP == kEncrypt || OP == kKeygen) {
      // coefficient k of every output polynomial, rounded (b, b') or encoded
      // with the message bit (c_m), as 16-bit values for the packing pass;
      // the MMAs are done, so the operand region is free
      constexpr uint32_t qm = (1u << C::EQ) - 1u, pm = (1u << C::EP) - 1u;
      uint16_t *vals = reinterpret_cast<uint16_t *>(sm + LO::ENG);
#pragma unroll
      for (int p = 0; p < S::R; p++) {
        uint32_t v = 0, off = 0;
#pragma unroll
        for (int d = 0; d < 4; d++) {
          if (d < S::digits(p)) {
            v += (1u << (4 * d)) * __float_as_uint(xacc[S::col_base(p) + d] + 24576.0f);
            off += (1u << (4 * d)) * 0x46C00000u;
          }
        }
        v -= off;
        if (p < L) {
          vals[256 * p + k] = (uint16_t)(((v + C::H1) & qm) >> (C::EQ - C::EP));
        } else {
          const uint32_t mk = (sm[LO::MSG + (k >> 3)] >> (k & 7)) & 1u;
          vals[256 * p + k] = (uint16_t)(((v + C::H1 - (mk << (C::EP - 1))) & pm) >> (C::EP - C::ET));
        }
      }
    }
  } else {
    // an input copy or the tensor core did not complete in time: report, and
    // give what is still in flight a second bounded wait before releasing
    if (tid == 0 && a.err) atomicOr(a.err, 2);
    if (warp == 0) {
      if (!ready) mbar_wait_bounded(mbar_in, 0);
      else mbar_wait_bounded(mbar_mma, 0);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, S::TMEM_COLS);
  if (!done) return;

  // 5. epilogues
  constexpr uint32_t qmask = (1u << C::EQ) - 1u, pmask = (1u << C::EP) - 1u;
  // sum_d 16^d acc_d of the digit columns c0..: each f32
  // accumulator holds x * 2^-9 for an exact integer |x| < 2^22, so adding
  // 1.5 * 2^14 leaves x + 0x46C00000 in its bit pattern; the offsets are
  // removed at the end
  auto combine1 = [&](int c0, int D) -> uint32_t {
    uint32_t v = 0, off = 0;
#pragma unroll
    for (int d = 0; d < 4; d++) {
      if (d < D) {
        v += (1u << (4 * d)) * __float_as_uint(xacc[c0 + d] + 24576.0f);
        off += (1u << (4 * d)) * 0x46C00000u;
      }
    }
    return v - off;
  };
  // W-bit field at bit `bit` of a 4-byte-aligned shared-memory stream
  auto field = [&](int byte_off, int bit, int W) -> uint32_t {
    const uint32_t *w = reinterpret_cast<const uint32_t *>(sm + byte_off) + (bit >> 5);
    return __funnelshift_r(w[0], w[1], bit & 31) & ((1u << W) - 1u);
  };

  if constexpr (OP == kDecrypt) {
    // m'_k = ((v_k + h2 - (c_m,k << (ep-et))) mod p) >> (ep-1): one bit per
    // thread, gathered into bytes by a ballot per warp
    const uint32_t v = combine1(0, S::DB);
    const uint32_t cm = field(LO::CTO + L * C::POLYCOMP, k * C::ET, C::ET);
    const uint32_t t = (v + C::H2 - (cm << (C::EP - C::ET))) & pmask;
    const uint32_t bits = __ballot_sync(0xffffffffu, ((t >> (C::EP - 1)) & 1u) != 0u);
    uint8_t *mo = a.m_out + (size_t)inst * a.m_out_stride;
    if (lane < 4) mo[4 * (4 * hsel + q4) + lane] = (uint8_t)(bits >> (8 * lane));
    if (a.copy_hpk && warp == 0) mo[32 + lane] = a.sk[(a.key_shared ? 0 : (size_t)inst * C::SK) + C::SK - 64 + lane];
  } else if constexpr (DECK) {
    // ciphertext r of the CTA: decode as above from its own columns and c_m
#pragma unroll
    for (int r = 0; r < S::R; r++) {
      if (r >= nvalid) break;
      const uint32_t v = combine1(r * S::DB, S::DB);
      const uint32_t cm = field(LO::CTO + r * LO::CTS + L * C::POLYCOMP, k * C::ET, C::ET);
      const uint32_t t = (v + C::H2 - (cm << (C::EP - C::ET))) & pmask;
      const uint32_t bits = __ballot_sync(0xffffffffu, ((t >> (C::EP - 1)) & 1u) != 0u);
      uint8_t *mo = a.m_out + (inst0 + r) * a.m_out_stride;
      if (lane < 4) mo[4 * (4 * hsel + q4) + lane] = (uint8_t)(bits >> (8 * lane));
      if (a.copy_hpk && warp == 0) mo[32 + lane] = a.sk[C::SK - 64 + lane];
    }
  } else if constexpr (OP == kReenc) {
    // round coefficient k of b' and encode that of v', compare with the ciphertext
    const uint32_t mk = (sm[LO::MSG + (k >> 3)] >> (k & 7)) & 1u;
    uint32_t diff = 0;
#pragma unroll
    for (int p = 0; p < S::R; p++) {
      const uint32_t v = combine1(S::col_base(p), S::digits(p));
      if (p < L) {
        const uint32_t w = ((v + C::H1) & qmask) >> (C::EQ - C::EP);
        diff |= w ^ field(LO::CTO + p * C::POLYCOMP, k * C::EP, C::EP);
      } else {
        const uint32_t w = ((v + C::H1 - (mk << (C::EP - 1))) & pmask) >> (C::EP - C::ET);
        diff |= w ^ field(LO::CTO + L * C::POLYCOMP, k * C::ET, C::ET);
      }
    }
    const int any = __syncthreads_or(diff != 0u);
    if (tid == 0) a.fail[inst] = (uint8_t)(any != 0);
  } else if constexpr (OP == kMatvec) {
    // coefficient k of every output polynomial, mod 2^eq
    const uint32_t m = (1u << a.mv_eq) - 1u;
    uint16_t *o = a.mv_out + (size_t)inst * (L * 256) + k;
#pragma unroll
    for (int p = 0; p < L; p++) o[256 * p] = (uint16_t)(combine1(S::col_base(p), S::DA) & m);
  } else if (OP == kEncrypt) {
    // pack the 16-bit values eight at a time: b' at EP bits, c_m at ET bits
    const uint16_t *vals = reinterpret_cast<const uint16_t *>(sm + LO::ENG);
    for (int idx = tid; idx < S::R * 32; idx += NT) {
      const int p = idx >> 5, grp = idx & 31;
      const uint4 q = *reinterpret_cast<const uint4 *>(vals + 256 * p + 8 * grp);
      const uint32_t W[4] = {q.x, q.y, q.z, q.w};
      if (p < L) pack8(sm + LO::OUT + (32 * p + grp) * C::EP, W, C::EP);
      else pack8(sm + LO::OUT + L * C::POLYCOMP + grp * C::ET, W, C::ET);
    }
    __syncthreads();
    copy16(a.ct_out + (size_t)inst * C::CT, sm + LO::OUT, C::CT);
  } else if (OP == kKeygen) {
    constexpr int bbytes = L * C::POLYCOMP;
    uint8_t *outb = sm + LO::OUT;
    const uint16_t *vals = reinterpret_cast<const uint16_t *>(sm + LO::ENG);
    for (int idx = tid; idx < L * 32; idx += NT) {
      const int p = idx >> 5, grp = idx & 31;
      const uint4 q = *reinterpret_cast<const uint4 *>(vals + 256 * p + 8 * grp);
      const uint32_t W[4] = {q.x, q.y, q.z, q.w};
      pack8(outb + (32 * p + grp) * C::EP, W, C::EP);
    }
    // secret key: 13-bit two's complement (Saber) or 2-bit (Sable) of sec8
    constexpr int sw = C::SABLE ? 2 : C::EQ;
    const int8_t *s8 = reinterpret_cast<const int8_t *>(sm + LO::SEC8);
    for (int grp = tid; grp < L * 32; grp += NT) {
      uint32_t Sv[4];
#pragma unroll
      for (int i = 0; i < 4; i++)
        Sv[i] = ((uint32_t)(int)s8[8 * grp + 2 * i] & 0xffffu) | ((uint32_t)(int)s8[8 * grp + 2 * i + 1] << 16);
      pack8(outb + bbytes + grp * sw, Sv, sw);
    }
    __syncthreads();
    uint8_t *pko = a.pk_out + (size_t)inst * C::PK;
    uint8_t *sko = a.sk_out + (size_t)inst * a.sk_stride;
    for (int i = tid; i < bbytes; i += NT) {
      pko[i] = outb[i];
      sko[C::INDCPA_SK + i] = outb[i];
    }
    if (tid < 32) sko[C::INDCPA_SK + bbytes + tid] = pko[bbytes + tid];  // seed_A
    for (int i = tid; i < C::INDCPA_SK; i += NT) sko[i] = outb[bbytes + i];
  }
}

template <int OP, int SET>
__global__ void __launch_bounds__(kI5Threads, 2) k_cpa5i(CpaArgs a) {
  extern __shared__ __align__(16) uint8_t sm[];
  cpa5i_body<OP, SET>(a, blockIdx.x, sm);
}

// Mixed launch: CTA gi runs instance gi of the group table R (one CTA per
// instance over all groups, whatever their parameter sets).
template <int OP>
__global__ void __launch_bounds__(kI5Threads, 2) k_cpa5m(const __grid_constant__ MixRef R) {
  extern __shared__ __align__(16) uint8_t sm[];
  const int gi = blockIdx.x;
  const int g = find_group(R, gi);
  const CpaArgs &a = group_args(R, g);
  const unsigned inst = (unsigned)(gi - group_first(R, g));
  switch (a.P.set) {
    case 0: cpa5i_body<OP, 0>(a, inst, sm); break;
    case 1: cpa5i_body<OP, 1>(a, inst, sm); break;
    case 2: cpa5i_body<OP, 2>(a, inst, sm); break;
    case 3: cpa5i_body<OP, 3>(a, inst, sm); break;
    case 4: cpa5i_body<OP, 4>(a, inst, sm); break;
    case 5: cpa5i_body<OP, 5>(a, inst, sm); break;
  }
}

// Mixed launch whose groups all have parameter set SET (the per-set launches
// of a mixed pass): the group table travels as a kernel parameter (constant
// bank), so a CTA finds its group and reads its arguments without a global
// round trip; then the same body as k_cpa5i, with the same registers and
// occupancy.  CTA gi runs instance gi of the table.
struct MixParam {
  int ngroups, total;
  int first[kMaxGroups + 1];
  CpaArgs g[kMaxGroups];
};
static_assert(sizeof(MixParam) < 32000, "the group table fits the kernel-parameter space");

template <int OP, int SET>
__global__ void __launch_bounds__(kI5Threads, 2) k_cpa5ms(const __grid_constant__ MixParam T) {
  extern __shared__ __align__(16) uint8_t sm[];
  const int gi = blockIdx.x;
  int lo = 0, hi = T.ngroups - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (gi >= T.first[mid]) lo = mid;
    else hi = mid - 1;
  }
  cpa5i_body<OP, SET>(T.g[lo], (unsigned)(gi - T.first[lo]), sm);
}

template <int OP>
inline void layout5_of(int set, int &total, int &cols) {
  switch (set) {
#define TMVP_L5(S)                                 \
  case S:                                          \
    total = LayoutC<OP, S>::TOTAL;                 \
    cols = ShapeC<OP, S>::TMEM_COLS;               \
    break;
    TMVP_L5(0) TMVP_L5(1) TMVP_L5(2) TMVP_L5(3) TMVP_L5(4) TMVP_L5(5)
#undef TMVP_L5
    default: total = 0; cols = 32;
  }
}

// Pads `smem` until at most 512 / cols CTAs of fn fit on an SM, so that every
// resident CTA's tensor-memory allocation succeeds at once.
template <class F>
inline int cap_tmem_residency(F fn, int &smem, int cols) {
  const int cap = 512 / cols;
  cudaError_t e;
  for (int it = 0; it < 64; it++) {
    if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
      return (int)e;
    int nb = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kI5Threads, smem)) != cudaSuccess) return (int)e;
    if (nb <= cap) return 0;
    smem += 2048;
  }
  return 0;
}

template <int OP, int SET>
inline int launch_cpa5ms(const CpaArgs *groups, int ng, cudaStream_t s) {
  using LO = LayoutC<OP, SET>;
  using S = ShapeC<OP, SET>;
  if (ng < 1 || ng > kMaxGroups) return (int)cudaErrorInvalidValue;
  MixParam T;
  T.ngroups = ng;
  T.first[0] = 0;
  for (int g = 0; g < ng; g++) {
    T.g[g] = groups[g];
    T.first[g + 1] = T.first[g] + groups[g].n;
  }
  T.total = T.first[ng];
  for (int g = ng; g < kMaxGroups; g++) T.first[g + 1] = T.total;
  if (T.total <= 0) return 0;
  auto fn = k_cpa5ms<OP, SET>;
  int smem = LO::TOTAL;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return (int)e;
  int rc = cap_tmem_residency(fn, smem, S::TMEM_COLS);
  if (rc) return rc;
  fn<<<T.total, kI5Threads, smem, s>>>(T);
  return (int)cudaGetLastError();
}

template <int OP>
inline int launch_cpa5m(const CpaArgs *groups, int ng, const MixTable *dev_tab, cudaStream_t s) {
  MixRef R{};
  R.ngroups = ng;
  R.total = 0;
  int smem = 0, cols = 32;
  for (int g = 0; g < ng; g++) {
    R.total += groups[g].n;
    int t, c;
    layout5_of<OP>(groups[g].P.set, t, c);
    smem = std::max(smem, t);
    cols = std::max(cols, c);
  }
  if (R.total <= 0) return 0;
  if (ng == 1) {
    R.one = groups[0];
  } else {
    if (!dev_tab) return (int)cudaErrorInvalidValue;
    R.tab = dev_tab;
  }
  bool one_set = true;
  for (int g = 1; g < ng; g++) one_set = one_set && groups[g].P.set == groups[0].P.set;
  if (one_set) {
    switch (groups[0].P.set) {
      case 0: return launch_cpa5ms<OP, 0>(groups, ng, s);
      case 1: return launch_cpa5ms<OP, 1>(groups, ng, s);
      case 2: return launch_cpa5ms<OP, 2>(groups, ng, s);
      case 3: return launch_cpa5ms<OP, 3>(groups, ng, s);
      case 4: return launch_cpa5ms<OP, 4>(groups, ng, s);
      case 5: return launch_cpa5ms<OP, 5>(groups, ng, s);
    }
  }
  auto fn = k_cpa5m<OP>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return (int)e;
  int rc = cap_tmem_residency(fn, smem, cols);
  if (rc) return rc;
  fn<<<R.total, kI5Threads, smem, s>>>(R);
  return (int)cudaGetLastError();
}

template <int OP, int SET>
inline int launch_cpa5i(const CpaArgs &a, cudaStream_t s) {
  using LO = LayoutC<OP, SET>;
  using S = ShapeC<OP, SET>;
  auto fn = k_cpa5i<OP, SET>;
  int smem = LO::TOTAL;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return (int)e;
  // at most 512 / TMEM_COLS resident CTAs per SM, so every CTA's tensor
  // memory allocation succeeds at once: pad the shared memory until no more fit
  const int cap = 512 / S::TMEM_COLS;
  for (int it = 0; it < 64; it++) {
    if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
      return (int)e;
    int nb = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kI5Threads, smem)) != cudaSuccess) return (int)e;
    if (nb <= cap) break;
    smem += 2048;
  }
  fn<<<OP == kDecryptK ? (a.n + S::R - 1) / S::R : a.n, kI5Threads, smem, s>>>(a);
  return (int)cudaGetLastError();
}

// Dispatch over the six parameter sets (matvec is not set-shaped).
template <int OP>
inline int launch_cpa5i_set(const CpaArgs &a, cudaStream_t s) {
  switch (a.P.set) {
    case 0: return launch_cpa5i<OP, 0>(a, s);
    case 1: return launch_cpa5i<OP, 1>(a, s);
    case 2: return launch_cpa5i<OP, 2>(a, s);
    case 3: return launch_cpa5i<OP, 3>(a, s);
    case 4: return launch_cpa5i<OP, 4>(a, s);
    case 5: return launch_cpa5i<OP, 5>(a, s);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace tmvp
