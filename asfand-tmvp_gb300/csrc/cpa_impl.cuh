// cpa_impl.cuh — the IND-CPA kernel template (one CTA per instance) of the
// mma.sync and CUDA-core forms, instantiated per (form, op) in the
// translation units cpa_fp8_*.cu, cpa_int8_*.cu, cpa_cc_*.cu, cpa_sb_*.cu,
// cpa_dp2a.cu and cpa_tc4.cu.
//
// Per instance:
//   1. 16-byte copies of the packed inputs into shared memory;
//   2. secrets unpacked (sk: 13-bit SABER pack.cu:34-46 / 2-bit SABLE
//      pack.cu:366-377) or sampled (CBD of the GenSecret stream,
//      SABER poly.cu:836-916 / SABLE fips202.cu:625-651);
//   3. public polynomials unpacked (13/11-bit A, SABER poly.cu:799-816;
//      10/9-bit b, b', SABER pack.cu:7-17) straight into the engine's layout;
//   4. the engine (cpa_engine.cuh) computes res[r] = sum_j P[r][j] * s_j;
//   5. the op's epilogue: rounding (post_process, SABER poly.cu:381-389),
//      message encoding (post_process2, :391-395), decoding (post_process3,
//      :398-403), bit packing, and the full ciphertext compare.
#pragma once
#include <cstddef>
#include <cstdint>

#include "cpa_engine.cuh"
#include "cpa_kernels.cuh"
#include "cpa_tc.cuh"
#include "cpa_tc_kernel.cuh"

namespace tmvp {

template <int FORM, int OP, int L, int Q_ = 1>
struct CpaCfg {
  static constexpr int R = OP == kDecrypt ? 1 : ((OP == kEncrypt || OP == kReenc) ? L + 1 : L);
  // public polys of width eq (A, or the matvec input); the rest are p-bit (b, b')
  static constexpr int RA = OP == kDecrypt ? 0 : L;
  static constexpr bool TC = FORM == kInt8TC || FORM == kFp8TC;
  static constexpr int Q = Q_;
  static constexpr int WARPS = 4;
  static constexpr int RP = R <= 4 ? 4 : 8;
  static constexpr bool TMVP = FORM == kCudaCore;
  static constexpr bool DP2A = FORM == kDp2a;
  static constexpr bool TOOM = FORM == kToomCook;
  static constexpr int NPROD = TMVP ? 3 : 1;
  static constexpr int NCOL = TMVP ? 128 : 256;
  static constexpr int NT = (TC || TOOM) ? 32 * WARPS : ((TMVP || DP2A) ? 96 : 64);
  // largest |secret| the form multiplies exactly (larger ones set a.err)
  static constexpr int SMAX = TC ? 7 : (DP2A ? 63 : 128);
};

struct CpaLayout {
  int raw_a, raw_s, raw_b, raw_msg, raw_ct, raw_sk;  // byte offsets (-1: absent)
  int sec, eng, res, total;
};

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

// Shared-memory layout of one CTA.  eng holds the engine operands (TC: digit
// columns then Toeplitz copies; CC: Toeplitz sequences, vectors, products).
template <int FORM, int OP, int L, int Q = 1>
__host__ __device__ inline CpaLayout cpa_layout(const KemParams &P) {
  using C = CpaCfg<FORM, OP, L, Q>;
  CpaLayout o;
  int off = 0;
  auto take = [&](int bytes) { int r = off; off = align16(off + bytes + 16); return r; };
  o.raw_a = o.raw_s = o.raw_b = o.raw_msg = o.raw_ct = o.raw_sk = -1;
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
  o.sec = take(L * 256 * 2);
  int eng;
  if (C::TC) {
    eng = L * C::Q * 8 * kColStride + L * kTzBytesPerPoly;
    if (C::Q * 8 * 256 * 4 > eng) eng = C::Q * 8 * 256 * 4;  // int32 accumulators alias it
  } else if (C::DP2A) {
    eng = L * 3 * 64 * 16 + L * 3 * 64 * C::RP * 4 + 3 * C::RP * 128 * 4;
  } else if (C::TOOM) {
    eng = L * 7 * kToomSStride * 4 + C::R * L * 7 * kToomPStride * 4;
    if (C::R * 7 * 128 * 4 > eng) eng = C::R * 7 * 128 * 4;  // products alias the evaluations
  } else {
    eng = L * C::NPROD * 512 * 2 + L * C::NPROD * C::NCOL * C::RP * 2 +
          (C::TMVP ? 3 * C::RP * 128 * 4 : 0);
  }
  o.eng = take(eng);
  o.res = take(C::R * 256 * 2);
  o.total = off;
  return o;
}

// Byte `ob` of the little-endian w-bit stream of values f(k).
template <class F>
__device__ __forceinline__ uint8_t pack_byte(int ob, int w, F f) {
  int bit0 = 8 * ob;
  int k0 = bit0 / w, k1 = (bit0 + 7) / w;
  uint32_t acc = 0;
  for (int k = k0; k <= k1; k++) {
    int sh = k * w - bit0;
    uint32_t v = f(k) & ((1u << w) - 1u);
    acc |= sh >= 0 ? (v << sh) : (v >> (-sh));
  }
  return (uint8_t)acc;
}

template <int FORM, int OP, int L, int Q>
__global__ void __launch_bounds__(CpaCfg<FORM, OP, L, Q>::NT) k_cpa(CpaArgs a) {
  using C = CpaCfg<FORM, OP, L, Q>;
  extern __shared__ __align__(16) uint8_t sm[];
  const KemParams &P = a.P;
  const size_t inst = blockIdx.x;
  const CpaLayout lo = cpa_layout<FORM, OP, L, Q>(P);
  const int tid = threadIdx.x;

  // 1. packed inputs to shared memory
  if (lo.raw_a >= 0) copy16(sm + lo.raw_a, a.a_stream + inst * P.gm_bytes, P.gm_bytes);
  if (lo.raw_s >= 0) copy16(sm + lo.raw_s, a.s_stream + inst * P.gs_bytes, P.gs_bytes);
  if (lo.raw_b >= 0) copy16(sm + lo.raw_b, a.pk + inst * a.pk_stride + a.pk_off, L * P.polycompbytes);
  if (lo.raw_msg >= 0) copy16(sm + lo.raw_msg, a.msg + inst * a.msg_stride, 32);
  if (lo.raw_ct >= 0) copy16(sm + lo.raw_ct, a.ct + inst * P.ct_bytes, P.ct_bytes);
  if (lo.raw_sk >= 0) copy16(sm + lo.raw_sk, a.sk + inst * P.sk_bytes, P.indcpa_sk_bytes);
  __syncthreads();

  // 2. secrets, int16 [L][256]
  int16_t *sec = reinterpret_cast<int16_t *>(sm + lo.sec);
  {
    bool bad = false;
    for (int idx = tid; idx < L * 256; idx += C::NT) {
      int v;
      if (OP == kDecrypt) {
        const uint8_t *rs = sm + lo.raw_sk;
        if (P.sable) {
          uint32_t x = get_bits(rs, idx * 2, 2);
          v = (int)(x ^ 2u) - 2;  // SABLE pack.cu:371-376
        } else {
          uint32_t x = get_bits(rs, idx * P.eq, P.eq);
          v = (int)x - (int)((x >> (P.eq - 1)) << P.eq);
        }
      } else if (OP == kMatvec) {
        v = a.mv_s[inst * (L * 256) + idx];
      } else {
        uint32_t x = get_bits(sm + lo.raw_s, idx * P.mu, P.mu);
        int h = P.mu >> 1;
        v = __popc(x & ((1u << h) - 1u)) - __popc(x >> h);
      }
      if (C::SMAX < 128 && (v > C::SMAX || v < -C::SMAX)) bad = true;
      sec[idx] = (int16_t)v;
    }
    if (bad && a.err) atomicOr(a.err, 1);
  }

  // public coefficient (r, j, k) and its bit width
  auto pub = [&](int r, int j, int k, int &w) -> uint32_t {
    if (OP == kDecrypt) {
      w = P.ep;
      return get_bits(sm + lo.raw_ct, (j * 256 + k) * P.ep, P.ep);
    } else if (OP == kMatvec) {
      w = a.mv_eq;
      size_t base = inst * (size_t)(L * L * 256);
      int ij = a.mv_transpose ? (j * L + r) : (r * L + j);
      return a.mv_A[base + ij * 256 + k] & ((1u << a.mv_eq) - 1u);
    } else if (r == L) {
      w = P.ep;
      return get_bits(sm + lo.raw_b, (j * 256 + k) * P.ep, P.ep);
    } else {
      w = P.eq;
      int ij = (OP == kKeygen) ? (j * L + r) : (r * L + j);
      return get_bits(sm + lo.raw_a, (ij * 256 + k) * P.eq, P.eq);
    }
  };

  uint16_t *res = reinterpret_cast<uint16_t *>(sm + lo.res);
  if (C::TC) {
    uint32_t *colw = reinterpret_cast<uint32_t *>(sm + lo.eng);
    uint32_t *tz = colw + L * C::Q * 8 * (kColStride / 4);
    const int wa = OP == kMatvec ? a.mv_eq : P.eq, wb = P.ep;
    const int Da = tc_digits<FORM>(wa), Db = tc_digits<FORM>(wb);
    const int c0 = FORM == kFp8TC ? 1 : 0;
    const int ncols = tc_cols<FORM>(C::R, C::RA, wa, wb);
    // digit columns: one work item = 8 coefficients of poly p, module index j
    for (int idx = tid; idx < C::R * L * 32; idx += C::NT) {
      const int grp = idx & 31, j = (idx >> 5) % L, p = idx / (32 * L);
      uint32_t X[4];
      if (OP == kMatvec) {
        int ij = a.mv_transpose ? (j * L + p) : (p * L + j);
        uint4 u = *reinterpret_cast<const uint4 *>(a.mv_A + inst * (size_t)(L * L * 256) + ij * 256 + 8 * grp);
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
      uint2 *dst = reinterpret_cast<uint2 *>(colw + (size_t)(j * C::Q * 8 + cb) * (kColStride / 4) + 2 * grp);
      for (int d = 0; d < D; d++) dst[d * (kColStride / 8)] = digit8<FORM>(X, d);
    }
    __syncthreads();  // sec complete
    for (int j = 0; j < L; j++) stage_toeplitz_v2<FORM>(tz + j * 4 * kTzCopyWords, sec + j * 256, C::NT);
    __syncthreads();
    int *accs = reinterpret_cast<int *>(sm + lo.eng);
    tc_engine_v2<FORM, C::Q, C::WARPS>(tz, colw, L, ncols, accs);
    __syncthreads();
    // combine digit columns: res = sum_d w^d acc_d (- FP8 bias correction)
    for (int idx = tid; idx < C::R * 256; idx += C::NT) {
      const int p = idx >> 8, row = idx & 255;
      const int D = p < C::RA ? Da : Db;
      const int cb = c0 + (p < C::RA ? p * Da : C::RA * Da + (p - C::RA) * Db);
      uint32_t v = 0, wgt = 1, wsum = 0;
      for (int d = 0; d < D; d++) {
        v += wgt * (uint32_t)accs[(cb + d) * 256 + row];
        wsum += wgt;
        wgt <<= (FORM == kFp8TC ? 3 : 8);
      }
      if (FORM == kFp8TC) v -= 8u * wsum * (uint32_t)accs[row];
      res[p * 256 + row] = (uint16_t)v;
    }
  } else if (C::DP2A) {
    uint4 *tb = reinterpret_cast<uint4 *>(sm + lo.eng);
    uint32_t *wp = reinterpret_cast<uint32_t *>(tb + L * 3 * 64);
    int *pp = reinterpret_cast<int *>(wp + L * 3 * 64 * C::RP);
    // public pairs: products 0, 1, 2 take v0 + v1, v1, v0 (v0 = coefficients
    // 0..127, v1 = 128..255)
    for (int idx = tid; idx < L * 64 * C::RP; idx += C::NT) {
      const int r = idx % C::RP, cp = (idx / C::RP) & 63, j = idx / (C::RP * 64);
      uint32_t va = 0, vb = 0;  // (v0[c], v0[c+1]) and (v1[c], v1[c+1]), c = 2 cp
      if (r < C::R) {
        if constexpr (OP == kMatvec) {
          const int ij = a.mv_transpose ? (j * L + r) : (r * L + j);
          const uint32_t *A32 = reinterpret_cast<const uint32_t *>(a.mv_A + inst * (size_t)(L * L * 256) + ij * 256);
          const uint32_t m = ((1u << a.mv_eq) - 1u) * 0x10001u;
          va = A32[cp] & m;
          vb = A32[64 + cp] & m;
        } else {
          int w;
          va = pub(r, j, 2 * cp, w) | (pub(r, j, 2 * cp + 1, w) << 16);
          vb = pub(r, j, 2 * cp + 128, w) | (pub(r, j, 2 * cp + 129, w) << 16);
        }
      }
      // halves below 2^14: the sum of the packed words adds them lane by lane
      wp[((j * 3 + 0) * 64 + cp) * C::RP + r] = va + vb;
      wp[((j * 3 + 1) * 64 + cp) * C::RP + r] = vb;
      wp[((j * 3 + 2) * 64 + cp) * C::RP + r] = va;
    }
    __syncthreads();  // sec complete
    auto se = [&](int j, int i) -> int {
      return i >= 255 ? (int)sec[j * 256 + i - 255] : -(int)sec[j * 256 + i + 1];
    };
    // u[k] = t_p[127 - k]: t_0 = T00, t_1 = T01 - T00, t_2 = T00 - T10
    auto u = [&](int j, int p, int k) -> uint32_t {
      if (k > 254) return 0u;
      const int x = 127 - k;
      const int v = p == 0 ? se(j, x + 255)
                           : (p == 1 ? se(j, x + 127) - se(j, x + 255) : se(j, x + 255) - se(j, x + 383));
      return (uint32_t)v & 0xffu;
    };
    // every byte u[k] once (k < 260, in the recombination scratch, free until
    // the engine's end), then the four byte-shifted copies of word w by
    // funnel shifts of words w and w + 1
    constexpr int UB = 260;
    uint8_t *ub = reinterpret_cast<uint8_t *>(pp);
    static_assert(L * 3 * UB <= 3 * C::RP * 128 * 4, "byte sequences fit the recombination scratch");
    for (int idx = tid; idx < L * 3 * UB; idx += C::NT) {
      const int k = idx % UB, jp = idx / UB;
      ub[idx] = (uint8_t)u(jp / 3, jp % 3, k);
    }
    __syncthreads();
    for (int idx = tid; idx < L * 3 * 64; idx += C::NT) {
      const int w = idx & 63, jp = idx >> 6;
      const uint32_t *u32 = reinterpret_cast<const uint32_t *>(ub + jp * UB);
      const uint32_t lo = u32[w], hi = u32[w + 1];
      tb[idx] = make_uint4(lo, __funnelshift_r(lo, hi, 8), __funnelshift_r(lo, hi, 16), __funnelshift_r(lo, hi, 24));
    }
    __syncthreads();
    dp2a_engine<C::RP>(tb, wp, L, C::R, pp, res);
  } else if (C::TOOM) {
    uint32_t *sv = reinterpret_cast<uint32_t *>(sm + lo.eng);
    uint32_t *pv = sv + L * 7 * kToomSStride;
    // public evaluations
    for (int idx = tid; idx < C::R * L * 64; idx += C::NT) {
      const int i = idx & 63, j = (idx >> 6) % L, r = idx / (64 * L);
      int w;
      uint32_t e[7];
      toom4_eval(pub(r, j, i, w), pub(r, j, i + 64, w), pub(r, j, i + 128, w), pub(r, j, i + 192, w), e);
#pragma unroll
      for (int pt = 0; pt < 7; pt++) pv[((r * L + j) * 7 + pt) * kToomPStride + i] = e[pt];
    }
    // zero margins of the secret evaluations
    for (int idx = tid; idx < L * 7 * 128; idx += C::NT) {
      const int x = idx & 127, jp = idx >> 7;
      sv[jp * kToomSStride + (x < 64 ? x : x + 64)] = 0u;
    }
    __syncthreads();  // sec complete
    for (int idx = tid; idx < L * 64; idx += C::NT) {
      const int i = idx & 63, j = idx >> 6;
      const int16_t *sj = sec + j * 256;
      uint32_t e[7];
      toom4_eval((uint32_t)(int)sj[i], (uint32_t)(int)sj[i + 64], (uint32_t)(int)sj[i + 128],
                 (uint32_t)(int)sj[i + 192], e);
#pragma unroll
      for (int pt = 0; pt < 7; pt++) sv[(j * 7 + pt) * kToomSStride + 64 + i] = e[pt];
    }
    __syncthreads();
    toom4_engine<C::R>(sv, pv, L, sv, res);
  } else {
    int16_t *tseq = reinterpret_cast<int16_t *>(sm + lo.eng);
    uint16_t *wv = reinterpret_cast<uint16_t *>(tseq + L * C::NPROD * 512);
    int *pp = reinterpret_cast<int *>(wv + L * C::NPROD * C::NCOL * C::RP);
    // vectors
    for (int idx = tid; idx < L * C::NCOL * C::RP; idx += C::NT) {
      int r = idx % C::RP, c = (idx / C::RP) % C::NCOL, j = idx / (C::RP * C::NCOL);
      uint16_t v0 = 0, v1 = 0;
      if (r < C::R) {
        int w;
        v0 = (uint16_t)pub(r, j, c, w);
        if (C::TMVP) v1 = (uint16_t)pub(r, j, c + 128, w);
      }
      if (C::TMVP) {
        wv[((j * 3 + 0) * C::NCOL + c) * C::RP + r] = (uint16_t)(v0 + v1);
        wv[((j * 3 + 1) * C::NCOL + c) * C::RP + r] = v1;
        wv[((j * 3 + 2) * C::NCOL + c) * C::RP + r] = v0;
      } else {
        wv[(j * C::NCOL + c) * C::RP + r] = v0;
      }
    }
    __syncthreads();  // sec complete
    // Toeplitz defining sequences; se(i) = s_ext[i]
    auto se = [&](int j, int i) -> int {
      return i >= 255 ? (int)sec[j * 256 + i - 255] : -(int)sec[j * 256 + i + 1];
    };
    for (int idx = tid; idx < L * C::NPROD * 512; idx += C::NT) {
      int e = idx & 511, p = (idx >> 9) % C::NPROD, j = idx / (512 * C::NPROD);
      int v = 0;
      if (C::TMVP) {
        int x = e - 128;
        if (x >= -127 && x <= 127) {
          if (p == 0) v = se(j, x + 255);
          else if (p == 1) v = se(j, x + 127) - se(j, x + 255);
          else v = se(j, x + 255) - se(j, x + 383);
        }
      } else {
        int x = e - 256;
        if (x >= -255) v = se(j, x + 255);
      }
      tseq[idx] = (int16_t)v;
    }
    __syncthreads();
    cc_engine<C::TMVP, C::RP>(tseq, wv, L, C::R, pp, res);
  }
  __syncthreads();

  // 5. epilogues
  const uint32_t qmask = (1u << P.eq) - 1u, pmask = (1u << P.ep) - 1u;
  if (OP == kDecrypt) {
    // decode: m'_k = ((v + h2 - (c_m << (ep-et))) mod p) >> (ep-1)
    const uint8_t *cmb = sm + lo.raw_ct + L * P.polycompbytes;
    if (tid < 32) {
      uint32_t byte = 0;
#pragma unroll
      for (int b = 0; b < 8; b++) {
        int k = 8 * tid + b;
        uint32_t cm = get_bits(cmb, k * P.et, P.et);
        uint32_t t = ((uint32_t)res[k] + P.h2 - (cm << (P.ep - P.et))) & pmask;
        byte |= ((t >> (P.ep - 1)) & 1u) << b;
      }
      uint8_t *mo = a.m_out + inst * a.m_out_stride;
      mo[tid] = (uint8_t)byte;
      if (a.copy_hpk) mo[32 + tid] = a.sk[inst * P.sk_bytes + P.sk_bytes - 64 + tid];
    }
  } else if (OP == kEncrypt || OP == kReenc) {
    const uint8_t *msg = sm + lo.raw_msg;
    const int bbytes = L * P.polycompbytes;
    auto bval = [&](int k) -> uint32_t {  // rounded b'
      return ((res[k] + P.h1) & qmask) >> (P.eq - P.ep);
    };
    auto cval = [&](int k) -> uint32_t {  // encoded message
      uint32_t mb = (msg[k >> 3] >> (k & 7)) & 1u;
      return (((uint32_t)res[L * 256 + k] + P.h1 - (mb << (P.ep - 1))) & pmask) >> (P.ep - P.et);
    };
    int diff = 0;
    for (int ob = tid; ob < P.ct_bytes; ob += C::NT) {
      uint8_t v = ob < bbytes ? pack_byte(ob, P.ep, bval) : pack_byte(ob - bbytes, P.et, cval);
      if (OP == kEncrypt) a.ct_out[inst * P.ct_bytes + ob] = v;
      else diff |= (v != sm[lo.raw_ct + ob]);
    }
    if (OP == kReenc) {
      int any = __syncthreads_or(diff);
      if (tid == 0) a.fail[inst] = (uint8_t)(any != 0);
    }
  } else if (OP == kKeygen) {
    const int bbytes = L * P.polycompbytes;
    uint8_t *pko = a.pk_out + inst * P.pk_bytes;
    uint8_t *sko = a.sk_out + inst * a.sk_stride;
    auto bval = [&](int k) -> uint32_t { return ((res[k] + P.h1) & qmask) >> (P.eq - P.ep); };
    for (int ob = tid; ob < bbytes; ob += C::NT) {
      uint8_t v = pack_byte(ob, P.ep, bval);
      pko[ob] = v;
      sko[P.indcpa_sk_bytes + ob] = v;
    }
    if (tid < 32) sko[P.indcpa_sk_bytes + bbytes + tid] = pko[bbytes + tid];  // seed_A
    auto sval = [&](int k) -> uint32_t { return (uint32_t)(int)sec[k]; };
    const int sw = P.sable ? 2 : P.eq;
    for (int ob = tid; ob < P.indcpa_sk_bytes; ob += C::NT) sko[ob] = pack_byte(ob, sw, sval);
  } else {  // kMatvec
    const uint32_t m = (1u << a.mv_eq) - 1u;
    uint16_t *o = a.mv_out + inst * (size_t)(L * 256);
    for (int idx = tid; idx < L * 256; idx += C::NT) o[idx] = (uint16_t)(res[idx] & m);
  }
}

template <int FORM, int OP, int L, int Q>
inline int launch_one(const CpaArgs &a, cudaStream_t s) {
  if (a.key_shared) return (int)cudaErrorInvalidValue;  // per-instance keys only in these forms
  if constexpr (FORM == kFp8TC || FORM == kInt8TC) {
    return launch_tc<FORM, OP, L, Q>(a, s);
  } else {
    using C = CpaCfg<FORM, OP, L, Q>;
    const CpaLayout lo = cpa_layout<FORM, OP, L, Q>(a.P);
    cudaError_t e = cudaFuncSetAttribute(k_cpa<FORM, OP, L, Q>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, lo.total);
    if (e != cudaSuccess) return (int)e;
    k_cpa<FORM, OP, L, Q><<<a.n, C::NT, lo.total, s>>>(a);
    return (int)cudaGetLastError();
  }
}

// n-tiles the tensor-core forms need for (op, l) with the widths of P.
template <int FORM, int OP, int L>
inline int tc_q(const CpaArgs &a) {
  using C = CpaCfg<FORM, OP, L>;
  int wa = OP == kMatvec ? a.mv_eq : a.P.eq;
  return (tc_cols<FORM>(C::R, C::RA, wa, a.P.ep) + 7) / 8;
}

template <int FORM, int OP, int L>
inline int launch_q(const CpaArgs &a, cudaStream_t s) {
  if constexpr (FORM == kCudaCore || FORM == kSchoolbook || FORM == kDp2a || FORM == kToomCook) {
    return launch_one<FORM, OP, L, 1>(a, s);
  } else {
    switch (tc_q<FORM, OP, L>(a)) {
      case 1: return launch_one<FORM, OP, L, 1>(a, s);
      case 2: return launch_one<FORM, OP, L, 2>(a, s);
      case 3: if constexpr (FORM == kFp8TC) return launch_one<FORM, OP, L, 3>(a, s); break;
      case 4:
        if constexpr (FORM == kFp8TC) return launch_one<FORM, OP, L, 4>(a, s);
        break;
    }
    return (int)cudaErrorInvalidValue;
  }
}

template <int FORM, int OP>
inline int launch_op(const CpaArgs &a, cudaStream_t s) {
  switch (a.P.l) {
    case 2: return launch_q<FORM, OP, 2>(a, s);
    case 3: return launch_q<FORM, OP, 3>(a, s);
    case 4: return launch_q<FORM, OP, 4>(a, s);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace tmvp
