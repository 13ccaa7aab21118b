// cpa_tc_kernel.cuh — the mma.sync tensor-core IND-CPA kernel (FP8_TC and
// INT8_TC forms, one CTA per instance; the tcgen05 form has its own kernels,
// cpa5i.cuh and cpa_persist.cuh).
//
// Same shape and results as the generic k_cpa template (cpa_impl.cuh), tuned
// for the tensor-core forms, where the integer work around the MMAs dominates:
//   * secrets are sampled / unpacked four coefficients per 32-bit word (SWAR
//     CBD for mu = 8 and mu = 2, SABER poly.cu:864-887 and SABLE
//     fips202.cu:625-651) straight into the 8-bit operand encoding;
//   * Toeplitz copy 0 (srev) is the encoded secret with its words and bytes
//     reversed, the second half negated: s_ext[d] = -s_ext[d + 256];
//   * digit columns come from unpack8 / digit8 (cpa_tc.cuh);
//   * the digit recombination is fused into vectorised epilogues that round,
//     encode, pack and compare eight coefficients at a time without division.
#pragma once
#include <cstdint>

#include "cpa_kernels.cuh"
#include "cpa_tc.cuh"

namespace tmvp {

// Byte offsets of one CTA's shared memory (computed on the host).
struct TcLayout {
  int raw_a, raw_s, raw_b, raw_msg, raw_ct, raw_sk;
  int sec8;   // int8 [l][256]   secret values
  int senc;   // u32  [l][64]    encoded secret words (e4m3 or s8)
  int eng;    // digit columns [l][Q*8][272] then Toeplitz copies [l][4][136] words;
              // int32 accumulators [Q*8][256] alias it after the MMAs
  int out;    // packed output staging (ct / pk part) for encrypt / keygen
  int total;
};

template <int FORM, int OP, int L, int Q>
struct TcCfg {
  static constexpr int R = OP == kDecrypt ? 1 : ((OP == kEncrypt || OP == kReenc) ? L + 1 : L);
  static constexpr int RA = OP == kDecrypt ? 0 : L;
  static constexpr int NT = 128;
};

inline int tc_align(int x) { return (x + 15) & ~15; }

template <int FORM, int OP, int L, int Q>
inline TcLayout tc_layout(const KemParams &P) {
  TcLayout o;
  int off = 0;
  auto take = [&](int bytes) { int r = off; off = tc_align(off + bytes + 16); return r; };
  o.raw_a = o.raw_s = o.raw_b = o.raw_msg = o.raw_ct = o.raw_sk = o.out = -1;
  if (OP == kEncrypt || OP == kReenc || OP == kKeygen) {
    o.raw_a = take(P.gm_bytes);
    o.raw_s = take(P.gs_bytes);
  }
  if (OP == kEncrypt || OP == kReenc) {
    o.raw_b = take(L * P.polycompbytes);
    o.raw_msg = take(32);
  }
  if (OP == kReenc || OP == kDecrypt) o.raw_ct = take(P.ct_bytes);
  if (OP == kDecrypt) o.raw_sk = take(P.indcpa_sk_bytes);
  o.sec8 = take(L * 256);
  o.senc = take(L * 256);
  int eng = L * Q * 8 * kColStride + L * kTzBytesPerPoly;
  if (Q * 8 * 256 * 4 > eng) eng = Q * 8 * 256 * 4;
  o.eng = take(eng);
  if (OP == kEncrypt) o.out = take(P.ct_bytes);
  if (OP == kKeygen) o.out = take(L * P.polycompbytes + P.indcpa_sk_bytes);
  o.total = off;
  return o;
}

// e4m3 magnitudes of 0..7 as a byte-permute table.
constexpr uint32_t kE4m3Lo = 0x44403800u;  // 3, 2, 1, 0
constexpr uint32_t kE4m3Hi = 0x4E4C4A48u;  // 7, 6, 5, 4

// Four signed bytes (|v| <= 7) to the 8-bit operand encoding.
template <int FORM>
__device__ __forceinline__ uint32_t enc4(uint32_t sbytes) {
  if (FORM == kInt8TC) return sbytes;
  uint32_t neg = sbytes & 0x80808080u;
  uint32_t mag = __vabsss4(sbytes);  // per-byte |v|
  uint32_t sel = (mag & 0x7u) | ((mag >> 4) & 0x70u) | ((mag >> 8) & 0x700u) | ((mag >> 12) & 0x7000u);
  return __byte_perm(kE4m3Lo, kE4m3Hi, sel) | neg;
}

// Negation of four encoded bytes.
template <int FORM>
__device__ __forceinline__ uint32_t neg4(uint32_t e) {
  return FORM == kInt8TC ? __vneg4(e) : (e ^ 0x80808080u);
}

// Range check of four signed bytes: every |v| <= 7.
__device__ __forceinline__ bool small4(uint32_t sbytes) {
  return (__vcmpgtu4(__vabsss4(sbytes), 0x07070707u)) == 0u;
}

// Eight w-bit values (16-bit lanes in V) packed into w bytes at dst.
__device__ __forceinline__ void pack8(uint8_t *dst, const uint32_t (&V)[4], int w) {
  uint32_t o[4] = {0u, 0u, 0u, 0u};
  const uint32_t m = (1u << w) - 1u;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    uint32_t v = ((k & 1) ? (V[k >> 1] >> 16) : V[k >> 1]) & m;
    int b = k * w, wi = b >> 5, sh = b & 31;
    o[wi] |= v << sh;
    if (sh + w > 32 && wi < 3) o[wi + 1] |= v >> (32 - sh);
  }
  for (int i = 0; i < w; i++) dst[i] = (uint8_t)(o[i >> 2] >> (8 * (i & 3)));
}

template <int FORM, int OP, int L, int Q>
__global__ void __launch_bounds__(128, (Q >= 4 ? 3 : 4)) k_cpa_tc(CpaArgs a, TcLayout lo) {
  using C = TcCfg<FORM, OP, L, Q>;
  extern __shared__ __align__(16) uint8_t sm[];
  const KemParams &P = a.P;
  const unsigned inst = blockIdx.x;
  const int tid = threadIdx.x;
  static_assert(FORM == kFp8TC || FORM == kInt8TC, "mma.sync forms");

  // 1. packed inputs to shared memory
  if (lo.raw_a >= 0) copy16(sm + lo.raw_a, a.a_stream + (size_t)inst * P.gm_bytes, P.gm_bytes);
  if (lo.raw_s >= 0) copy16(sm + lo.raw_s, a.s_stream + (size_t)inst * P.gs_bytes, P.gs_bytes);
  if (lo.raw_b >= 0)
    copy16(sm + lo.raw_b, a.pk + (size_t)inst * a.pk_stride + a.pk_off, L * P.polycompbytes);
  if (lo.raw_msg >= 0) copy16(sm + lo.raw_msg, a.msg + (size_t)inst * a.msg_stride, 32);
  if (lo.raw_ct >= 0) copy16(sm + lo.raw_ct, a.ct + (size_t)inst * P.ct_bytes, P.ct_bytes);
  if (lo.raw_sk >= 0) copy16(sm + lo.raw_sk, a.sk + (size_t)inst * P.sk_bytes, P.indcpa_sk_bytes);
  __syncthreads();

  // 2. secrets: int8 values (sec8) and their operand encoding (senc), 4 per word
  uint32_t *sec8w = reinterpret_cast<uint32_t *>(sm + lo.sec8);
  uint32_t *sencw = reinterpret_cast<uint32_t *>(sm + lo.senc);
  {
    bool ok = true;
    const bool packed13 = OP == kDecrypt && !P.sable;  // 13-bit two's complement (SABER pack.cu:53-84)
    if (packed13) {
      const uint32_t m = ((1u << P.eq) - 1u) * 0x10001u;
      for (int g8 = tid; g8 < L * 32; g8 += C::NT) {
        uint32_t X[4];
        unpack8(sm + lo.raw_sk, g8 * P.eq, P.eq, X);
        // in range when (v + 128) mod 2^eq < 256; the low byte is then the value
        uint32_t bad = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) bad |= ((X[i] + 0x00800080u) & m) & 0xFF00FF00u;
        const uint32_t s0 = __byte_perm(X[0], X[1], 0x6420), s1 = __byte_perm(X[2], X[3], 0x6420);
        ok = ok && bad == 0u && small4(s0) && small4(s1);
        sec8w[2 * g8] = s0;
        sec8w[2 * g8 + 1] = s1;
        sencw[2 * g8] = enc4<FORM>(s0);
        sencw[2 * g8 + 1] = enc4<FORM>(s1);
      }
    }
    for (int w = packed13 ? L * 64 : tid; w < L * 64; w += C::NT) {
      uint32_t sb;  // four signed bytes
      if (OP == kMatvec) {
        sb = *reinterpret_cast<const uint32_t *>(a.mv_s + (size_t)inst * (L * 256) + 4 * w);
      } else if (OP == kDecrypt) {
        if (P.sable) {
          // 2-bit two's complement (SABLE pack.cu:371-376): one byte = 4 coefficients
          uint32_t x = sm[lo.raw_sk + w];
          uint32_t spread = (x & 3u) | ((x & 0xcu) << 6) | ((x & 0x30u) << 12) | ((x & 0xc0u) << 18);
          uint32_t sgn = (spread >> 1) & 0x01010101u;
          sb = spread | (sgn * 0xfcu);  // sign-extend bit 1 of each byte
        } else {
          uint32_t v0 = get_bits(sm + lo.raw_sk, (4 * w) * P.eq, P.eq);
          uint32_t v1 = get_bits(sm + lo.raw_sk, (4 * w + 1) * P.eq, P.eq);
          uint32_t v2 = get_bits(sm + lo.raw_sk, (4 * w + 2) * P.eq, P.eq);
          uint32_t v3 = get_bits(sm + lo.raw_sk, (4 * w + 3) * P.eq, P.eq);
          // values mod 2^eq of small secrets: the low byte is the int8 value
          // when the value is in range; out-of-range values are flagged
          uint32_t top = (1u << P.eq) - 128u;
          ok = ok && (v0 < 128u || v0 >= top) && (v1 < 128u || v1 >= top) &&
               (v2 < 128u || v2 >= top) && (v3 < 128u || v3 >= top);
          sb = (v0 & 0xffu) | ((v1 & 0xffu) << 8) | ((v2 & 0xffu) << 16) | ((v3 & 0xffu) << 24);
        }
      } else if (P.mu == 8) {
        // CBD mu = 8: coefficient = popcount(low nibble) - popcount(high nibble)
        uint32_t x = *reinterpret_cast<const uint32_t *>(sm + lo.raw_s + 4 * w);
        uint32_t n = x - ((x >> 1) & 0x55555555u);
        n = (n & 0x33333333u) + ((n >> 2) & 0x33333333u);
        sb = __vsub4(n & 0x0f0f0f0fu, (n >> 4) & 0x0f0f0f0fu);
      } else if (P.mu == 2) {
        // CBD mu = 2: one byte = 4 coefficients of (bit 2i) - (bit 2i+1)
        uint32_t x = sm[lo.raw_s + w];
        uint32_t spread = (x & 3u) | ((x & 0xcu) << 6) | ((x & 0x30u) << 12) | ((x & 0xc0u) << 18);
        sb = __vsub4(spread & 0x01010101u, (spread >> 1) & 0x01010101u);
      } else {
        uint32_t r = 0;
        const int h = P.mu >> 1;
#pragma unroll
        for (int b = 0; b < 4; b++) {
          uint32_t x = get_bits(sm + lo.raw_s, (4 * w + b) * P.mu, P.mu);
          int v = __popc(x & ((1u << h) - 1u)) - __popc(x >> h);
          r |= ((uint32_t)v & 0xffu) << (8 * b);
        }
        sb = r;
      }
      ok = ok && small4(sb);
      sec8w[w] = sb;
      sencw[w] = enc4<FORM>(sb);
    }
    if (!ok && a.err) atomicOr(a.err, 1);
  }

  // 3. public digit columns [l][Q*8 columns][kColStride bytes], then the
  //    Toeplitz copies
  uint32_t *colw = reinterpret_cast<uint32_t *>(sm + lo.eng);
  uint32_t *tz = colw + L * Q * 8 * (kColStride / 4);
  const int wa = OP == kMatvec ? a.mv_eq : P.eq, wb = P.ep;
  const int Da = tc_digits<FORM>(wa), Db = tc_digits<FORM>(wb);
  const int c0 = FORM == kFp8TC ? 1 : 0;
  const int ncols = c0 + C::RA * Da + (C::R - C::RA) * Db;
  for (int idx = tid; idx < C::R * L * 32; idx += C::NT) {
    const int grp = idx & 31, j = (idx >> 5) % L, p = idx / (32 * L);
    uint32_t X[4];
    if (OP == kMatvec) {
      int ij = a.mv_transpose ? (j * L + p) : (p * L + j);
      uint4 u = *reinterpret_cast<const uint4 *>(a.mv_A + (size_t)inst * (L * L * 256) + ij * 256 + 8 * grp);
      const uint32_t m = ((1u << wa) - 1u) * 0x10001u;
      X[0] = u.x & m; X[1] = u.y & m; X[2] = u.z & m; X[3] = u.w & m;
    } else if (OP == kDecrypt) {
      unpack8(sm + lo.raw_ct, (32 * j + grp) * wb, wb, X);
    } else if (p < C::RA) {
      int ij = (OP == kKeygen) ? (j * L + p) : (p * L + j);
      unpack8(sm + lo.raw_a, (32 * ij + grp) * wa, wa, X);
    } else {
      unpack8(sm + lo.raw_b, (32 * j + grp) * wb, wb, X);
    }
    const int D = p < C::RA ? Da : Db;
    const int cb = c0 + (p < C::RA ? p * Da : C::RA * Da + (p - C::RA) * Db);
    uint2 *dst = reinterpret_cast<uint2 *>(colw + (j * Q * 8 + cb) * (kColStride / 4) + 2 * grp);
    for (int d = 0; d < D; d++) dst[d * (kColStride / 8)] = digit8<FORM>(X, d);
  }
  __syncthreads();

  // 4. Toeplitz copy 0: srev word u = byte-reversed encoded word 63-u; the
  //    second half is its negation
  for (int idx = tid; idx < L * 130; idx += C::NT) {
    const int j = idx / 130, w = idx % 130;
    uint32_t v = 0;
    if (w < 128) {
      v = __byte_perm(sencw[j * 64 + 63 - (w & 63)], 0, 0x0123);
      if (w >= 64) v = neg4<FORM>(v);
    }
    tz[j * 4 * kTzCopyWords + w] = v;
  }
  __syncthreads();
  for (int idx = tid; idx < L * 3 * 128; idx += C::NT) {
    const int j = idx / 384, r = idx % 384, c = 1 + r / 128, w = r % 128;
    const uint32_t *c0w = tz + j * 4 * kTzCopyWords;
    uint32_t sel = (uint32_t)(c | ((c + 1) << 4) | ((c + 2) << 8) | ((c + 3) << 12));
    tz[j * 4 * kTzCopyWords + c * kTzCopyWords + w] = __byte_perm(c0w[w], c0w[w + 1], sel);
  }
  __syncthreads();

  // 5. MMAs -> int32 accumulators (aliasing the operands)
  tc_engine_v2<FORM, Q, 4>(tz, colw, L, ncols, reinterpret_cast<int *>(sm + lo.eng));
  __syncthreads();
  const int *acc = reinterpret_cast<const int *>(sm + lo.eng);

  // 6. epilogues on groups of eight coefficients
  constexpr int WS = FORM == kFp8TC ? 3 : 8;  // digit weight 2^WS
  // sum_d 2^(WS d) acc_d (- FP8 bias) for coefficients 8*grp .. 8*grp+7 of poly p
  auto combine8 = [&](int p, int grp, uint32_t (&V)[4]) {
    const int D = p < C::RA ? Da : Db;
    const int cb = c0 + (p < C::RA ? p * Da : C::RA * Da + (p - C::RA) * Db);
    uint32_t v[8];
    const int4 *base = reinterpret_cast<const int4 *>(acc + 8 * grp);
    {
      int4 x0 = base[(cb * 256) / 4], x1 = base[(cb * 256) / 4 + 1];
      v[0] = x0.x; v[1] = x0.y; v[2] = x0.z; v[3] = x0.w;
      v[4] = x1.x; v[5] = x1.y; v[6] = x1.z; v[7] = x1.w;
    }
    uint32_t wgt = 1u << WS, wsum = 1u;
    for (int d = 1; d < D; d++) {
      int4 x0 = base[((cb + d) * 256) / 4], x1 = base[((cb + d) * 256) / 4 + 1];
      v[0] += wgt * (uint32_t)x0.x; v[1] += wgt * (uint32_t)x0.y;
      v[2] += wgt * (uint32_t)x0.z; v[3] += wgt * (uint32_t)x0.w;
      v[4] += wgt * (uint32_t)x1.x; v[5] += wgt * (uint32_t)x1.y;
      v[6] += wgt * (uint32_t)x1.z; v[7] += wgt * (uint32_t)x1.w;
      wsum += wgt;
      wgt <<= WS;
    }
    if (FORM == kFp8TC) {
      const uint32_t cf = 8u * wsum;
      int4 r0 = base[0], r1 = base[1];  // column 0: Toeplitz row sums
      v[0] -= cf * (uint32_t)r0.x; v[1] -= cf * (uint32_t)r0.y;
      v[2] -= cf * (uint32_t)r0.z; v[3] -= cf * (uint32_t)r0.w;
      v[4] -= cf * (uint32_t)r1.x; v[5] -= cf * (uint32_t)r1.y;
      v[6] -= cf * (uint32_t)r1.z; v[7] -= cf * (uint32_t)r1.w;
    }
#pragma unroll
    for (int i = 0; i < 4; i++) V[i] = (v[2 * i] & 0xffffu) | (v[2 * i + 1] << 16);
  };

  const uint32_t qmask = (1u << P.eq) - 1u, pmask = (1u << P.ep) - 1u;
  // round(x) = ((x + h1) mod q) >> (eq - ep), applied to two 16-bit lanes
  auto round_lanes = [&](uint32_t x) -> uint32_t {
    uint32_t lo16 = (((x & 0xffffu) + P.h1) & qmask) >> (P.eq - P.ep);
    uint32_t hi16 = (((x >> 16) + P.h1) & qmask) >> (P.eq - P.ep);
    return lo16 | (hi16 << 16);
  };
  // c_m(x, m) = ((x + h1 - (m << (ep-1))) mod p) >> (ep - et)
  auto encode_lanes = [&](uint32_t x, uint32_t mlo, uint32_t mhi) -> uint32_t {
    uint32_t lo16 = (((x & 0xffffu) + P.h1 - (mlo << (P.ep - 1))) & pmask) >> (P.ep - P.et);
    uint32_t hi16 = (((x >> 16) + P.h1 - (mhi << (P.ep - 1))) & pmask) >> (P.ep - P.et);
    return lo16 | (hi16 << 16);
  };

  if (OP == kDecrypt) {
    // m'_k = ((v + h2 - (c_m << (ep-et))) mod p) >> (ep-1), one byte per group
    if (tid < 32) {
      uint32_t V[4], CM[4];
      combine8(0, tid, V);
      unpack8(sm + lo.raw_ct + L * P.polycompbytes, tid * P.et, P.et, CM);
      uint32_t byte = 0;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        uint32_t v = (k & 1) ? (V[k >> 1] >> 16) : (V[k >> 1] & 0xffffu);
        uint32_t cm = (k & 1) ? (CM[k >> 1] >> 16) : (CM[k >> 1] & 0xffffu);
        uint32_t t = (v + P.h2 - (cm << (P.ep - P.et))) & pmask;
        byte |= ((t >> (P.ep - 1)) & 1u) << k;
      }
      uint8_t *mo = a.m_out + (size_t)inst * a.m_out_stride;
      mo[tid] = (uint8_t)byte;
      if (a.copy_hpk) mo[32 + tid] = a.sk[(size_t)inst * P.sk_bytes + P.sk_bytes - 64 + tid];
    }
  } else if (OP == kEncrypt || OP == kReenc) {
    const uint8_t *msg = sm + lo.raw_msg;
    int diff = 0;
    for (int idx = tid; idx < C::R * 32; idx += C::NT) {
      const int p = idx >> 5, grp = idx & 31;
      uint32_t V[4], W[4];
      combine8(p, grp, V);
      int w, byte0;
      if (p < L) {
#pragma unroll
        for (int i = 0; i < 4; i++) W[i] = round_lanes(V[i]);
        w = P.ep;
        byte0 = (32 * p + grp) * P.ep;
      } else {
        uint32_t mb = msg[grp];
#pragma unroll
        for (int i = 0; i < 4; i++) W[i] = encode_lanes(V[i], (mb >> (2 * i)) & 1u, (mb >> (2 * i + 1)) & 1u);
        w = P.et;
        byte0 = L * P.polycompbytes + grp * P.et;
      }
      if (OP == kReenc) {
        uint32_t Cv[4];
        unpack8(sm + lo.raw_ct, byte0, w, Cv);
        diff |= (Cv[0] ^ W[0]) | (Cv[1] ^ W[1]) | (Cv[2] ^ W[2]) | (Cv[3] ^ W[3]);
      } else {
        pack8(sm + lo.out + byte0, W, w);
      }
    }
    if (OP == kReenc) {
      int any = __syncthreads_or(diff != 0);
      if (tid == 0) a.fail[inst] = (uint8_t)(any != 0);
    } else {
      __syncthreads();
      copy16(a.ct_out + (size_t)inst * P.ct_bytes, sm + lo.out, P.ct_bytes);
    }
  } else if (OP == kKeygen) {
    const int bbytes = L * P.polycompbytes;
    uint8_t *outb = sm + lo.out;
    for (int idx = tid; idx < L * 32; idx += C::NT) {
      const int p = idx >> 5, grp = idx & 31;
      uint32_t V[4], W[4];
      combine8(p, grp, V);
#pragma unroll
      for (int i = 0; i < 4; i++) W[i] = round_lanes(V[i]);
      pack8(outb + (32 * p + grp) * P.ep, W, P.ep);
    }
    // secret key: 13-bit two's complement (Saber) or 2-bit (Sable) of sec8
    const int sw = P.sable ? 2 : P.eq;
    const int8_t *s8 = reinterpret_cast<const int8_t *>(sm + lo.sec8);
    for (int grp = tid; grp < L * 32; grp += C::NT) {
      uint32_t S[4];
#pragma unroll
      for (int i = 0; i < 4; i++)
        S[i] = ((uint32_t)(int)s8[8 * grp + 2 * i] & 0xffffu) | ((uint32_t)(int)s8[8 * grp + 2 * i + 1] << 16);
      pack8(outb + bbytes + grp * sw, S, sw);
    }
    __syncthreads();
    uint8_t *pko = a.pk_out + (size_t)inst * P.pk_bytes;
    uint8_t *sko = a.sk_out + (size_t)inst * a.sk_stride;
    for (int i = tid; i < bbytes; i += C::NT) {
      pko[i] = outb[i];
      sko[P.indcpa_sk_bytes + i] = outb[i];
    }
    if (tid < 32) sko[P.indcpa_sk_bytes + bbytes + tid] = pko[bbytes + tid];  // seed_A
    for (int i = tid; i < P.indcpa_sk_bytes; i += C::NT) sko[i] = outb[bbytes + i];
  } else {  // kMatvec
    const uint32_t m = ((1u << a.mv_eq) - 1u) * 0x10001u;
    for (int idx = tid; idx < L * 32; idx += C::NT) {
      const int p = idx >> 5, grp = idx & 31;
      uint32_t V[4];
      combine8(p, grp, V);
      *reinterpret_cast<uint4 *>(a.mv_out + (size_t)inst * (L * 256) + p * 256 + 8 * grp) =
          make_uint4(V[0] & m, V[1] & m, V[2] & m, V[3] & m);
    }
  }
}

template <int FORM, int OP, int L, int Q>
inline int launch_tc(const CpaArgs &a, cudaStream_t s) {
  const TcLayout lo = tc_layout<FORM, OP, L, Q>(a.P);
  auto fn = k_cpa_tc<FORM, OP, L, Q>;
  int smem = lo.total;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return (int)e;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return (int)e;
  fn<<<a.n, 128, smem, s>>>(a, lo);
  return (int)cudaGetLastError();
}

}  // namespace tmvp
