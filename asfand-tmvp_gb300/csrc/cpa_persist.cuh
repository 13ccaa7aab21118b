// cpa_persist.cuh — the persistent, pipelined tcgen05 IND-CPA kernel.
//
// One kernel launch covers up to kMaxGroups groups of instances, each group
// with its own parameter set (LightSaber / Saber / FireSaber / Sable l=2,3,4)
// and its own buffers, so a mixed batch runs as one launch.  A grid of
// `ctas_per_sm` x #SM CTAs of 256 threads walks the instances in a static
// stride; every CTA keeps a three-stage pipeline:
//
//   iteration it:  wait raw[it%3]      (TMA bulk copies issued two iterations ago)
//                  stage ops[it&1]     (secrets, radix-16 digit columns, Hankel
//                                       core matrices; cpa_umma.cuh)
//                  issue the MMAs      (tcgen05.mma into TMEM buffer it&1,
//                                       commit -> mma barrier it&1)
//                  epilogue of it-1    (wait its barrier, tcgen05.ld -> int32
//                                       columns, round / pack / compare / decode)
//                  prefetch it+2       (cp.async.bulk of its packed inputs into
//                                       raw[(it+2)%3], which held it-1)
//
// so the tensor core works on instance it while the CTA finishes it-1 and the
// copy engine fetches it+2.  Results are identical to the per-instance
// kernels (cpa_tc_kernel.cuh); the algorithm per instance is the same.
//
// Every wait is bounded: an mbarrier that does not complete within about two
// seconds sets bit 2 of the group's error word and the CTA stops after
// releasing its tensor memory.
#pragma once
#include <cstdint>

#include <algorithm>

#include "cpa_tc_kernel.cuh"

namespace tmvp {

constexpr int kMaxGroups = 64;
constexpr int kWorkers = 256;                    // warps 0-7: staging and epilogues
constexpr int kPersistThreads = kWorkers + 32;   // warp 8: issues the MMAs

// Barrier 1 over the worker warps only (the MMA warp keeps running).
__device__ __forceinline__ void wsync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
__device__ __forceinline__ bool wsync_and(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred a, b;\n\tsetp.ne.u32 a, %1, 0;\n\t"
      "bar.red.and.pred b, 1, 256, a;\n\tselp.u32 %0, 1, 0, b;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)p)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ bool wsync_or(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred a, b;\n\tsetp.ne.u32 a, %1, 0;\n\t"
      "bar.red.or.pred b, 1, 256, a;\n\tselp.u32 %0, 1, 0, b;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)p)
      : "memory");
  return r != 0;
}

// The groups of a mixed launch, in device memory: group g covers global
// instance indices [first[g], first[g+1]) with its own arguments.
struct MixTable {
  int first[kMaxGroups + 1];
  CpaArgs g[kMaxGroups];
};

// Kernel parameter: either one group carried by value (tab == nullptr), or a
// device table of ngroups groups.
struct MixRef {
  int ngroups, total;
  const MixTable *tab;
  CpaArgs one;
};

// Byte offsets of the packed inputs of one instance inside a raw buffer
// (-1: absent for this op).
struct RawOff {
  int a, s, b, msg, ct, sk, bytes;
};

__host__ __device__ inline int al16p(int x) { return (x + 15) & ~15; }

template <int OP>
__host__ __device__ inline RawOff raw_off(const KemParams &P) {
  RawOff r{-1, -1, -1, -1, -1, -1, 0};
  const int L = P.l;
  int off = 0;
  // every piece gets 16 bytes of slack for the unaligned field readers
  if (OP == kMatvec) {
    r.a = off; off = al16p(off + L * L * 512 + 16);
    r.s = off; off = al16p(off + L * 256 + 16);
  }
  if (OP == kEncrypt || OP == kReenc || OP == kKeygen) {
    r.a = off; off = al16p(off + P.gm_bytes + 16);
    r.s = off; off = al16p(off + P.gs_bytes + 16);
  }
  if (OP == kEncrypt || OP == kReenc) {
    r.b = off; off = al16p(off + L * P.polycompbytes + 16);
    r.msg = off; off = al16p(off + 32 + 16);
  }
  if (OP == kReenc || OP == kDecrypt) {
    r.ct = off; off = al16p(off + P.ct_bytes + 16);
  }
  if (OP == kDecrypt) {
    r.sk = off; off = al16p(off + P.indcpa_sk_bytes + 16);
  }
  r.bytes = off;
  return r;
}

// Shape of one instance's products: R public polynomials per module index
// (the first RA of width wa), digit counts, columns and the MMA N.
struct Shape5 {
  int L, R, RA, wa, wb, Da, Db, ncols, NU;
};

template <int OP>
__host__ __device__ inline Shape5 shape5(const CpaArgs &a) {
  Shape5 s;
  s.L = a.P.l;
  s.R = OP == kDecrypt ? 1 : ((OP == kEncrypt || OP == kReenc) ? s.L + 1 : s.L);
  s.RA = OP == kDecrypt ? 0 : s.L;
  s.wa = OP == kMatvec ? a.mv_eq : a.P.eq;
  s.wb = a.P.ep;
  s.Da = r16_digits(s.wa);
  s.Db = r16_digits(s.wb);
  s.ncols = s.RA * s.Da + (s.R - s.RA) * s.Db;
  s.NU = s.ncols <= 16 ? 16 : 32;
  return s;
}

// Per-launch shared-memory layout (host-computed maxima over the groups).
struct PLayout {
  int raw[3];     // packed inputs, three buffers
  int sec8[2];    // int8 secrets [l][256], two buffers (keygen epilogue)
  int senc;       // encoded secret words [l][64]
  int ops[2];     // Hankel [l][kHankelBytes] | digit columns [l][256 x N] | s_ext [l][512]
  int out;        // packed output staging (encrypt / keygen)
  int bar;        // mbarriers raw_full[3], ops_full[2], acc_full[2], tmem_free[2]; TMEM base
  int total;
  int tmem_cols;  // per CTA: two buffers of two M halves of N f32 columns
  int nu_max;
};

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared on the copy engine; completion is counted on
// `mbar` (bytes).  Source, destination and size are multiples of 16 bytes.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

// Group of global instance gi (binary search over the prefix table).
__device__ __forceinline__ int find_group(const MixRef &R, int gi) {
  if (!R.tab) return 0;
  int lo = 0, hi = R.ngroups - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (gi >= R.tab->first[mid]) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
__device__ __forceinline__ const CpaArgs &group_args(const MixRef &R, int g) {
  return R.tab ? R.tab->g[g] : R.one;
}
__device__ __forceinline__ int group_first(const MixRef &R, int g) { return R.tab ? R.tab->first[g] : 0; }

// Issues the bulk copies of instance `inst` of group `a` into raw buffer `dst`.
template <int OP>
__device__ __forceinline__ void prefetch5(const CpaArgs &a, int inst, uint8_t *dst, uint32_t mbar) {
  const KemParams &P = a.P;
  const RawOff ro = raw_off<OP>(P);
  const int L = P.l;
  const uint32_t d = smem_u32(dst);
  uint32_t bytes = 0;
  if (OP == kMatvec) bytes = L * L * 512 + L * 256;
  if (OP == kEncrypt || OP == kReenc || OP == kKeygen) bytes = P.gm_bytes + P.gs_bytes;
  if (OP == kEncrypt || OP == kReenc) bytes += L * P.polycompbytes + 32;
  if (OP == kReenc || OP == kDecrypt) bytes += P.ct_bytes;
  if (OP == kDecrypt) bytes += P.indcpa_sk_bytes;
  mbar_expect_tx(mbar, bytes);
  if (OP == kMatvec) {
    bulk_g2s(d + ro.a, a.mv_A + (size_t)inst * (L * L * 256), L * L * 512, mbar);
    bulk_g2s(d + ro.s, a.mv_s + (size_t)inst * (L * 256), L * 256, mbar);
  }
  if (OP == kEncrypt || OP == kReenc || OP == kKeygen) {
    bulk_g2s(d + ro.a, a.a_stream + (size_t)inst * P.gm_bytes, P.gm_bytes, mbar);
    bulk_g2s(d + ro.s, a.s_stream + (size_t)inst * P.gs_bytes, P.gs_bytes, mbar);
  }
  if (OP == kEncrypt || OP == kReenc) {
    bulk_g2s(d + ro.b, a.pk + (size_t)inst * a.pk_stride + a.pk_off, L * P.polycompbytes, mbar);
    bulk_g2s(d + ro.msg, a.msg + (size_t)inst * a.msg_stride, 32, mbar);
  }
  if (OP == kReenc || OP == kDecrypt) bulk_g2s(d + ro.ct, a.ct + (size_t)inst * P.ct_bytes, P.ct_bytes, mbar);
  if (OP == kDecrypt) bulk_g2s(d + ro.sk, a.sk + (size_t)inst * P.sk_bytes, P.indcpa_sk_bytes, mbar);
}


// Stages one instance from its raw buffer (worker warps): int8 secrets (sec8),
// their e4m3 words (senc), the digit columns and the Hankel core matrices
// (ops).  Ends with the proxy fence and a worker barrier, so the MMAs may read
// ops.  Returns false (in every worker) when a secret coefficient is outside
// |s| <= 7.
template <int OP>
__device__ __forceinline__ bool stage5(const CpaArgs &a, const Shape5 &S, const uint8_t *raw,
                                       const RawOff &ro, uint32_t *sec8w, uint32_t *sencw,
                                       uint8_t *ops) {
  const KemParams &P = a.P;
  const int tid = threadIdx.x, nt = kWorkers;
  const int L = S.L, NU = S.NU;
  uint8_t *H = ops, *B = ops + L * kHankelBytes;
  uint32_t *ext = reinterpret_cast<uint32_t *>(B + L * 256 * NU);
  // 1. secrets, four coefficients per word
  bool ok = true;
  const bool packed13 = OP == kDecrypt && !P.sable;  // 13-bit two's complement (SABER pack.cu:53-84)
  if (packed13) {
    const uint32_t m = ((1u << P.eq) - 1u) * 0x10001u;
    for (int g8 = tid; g8 < L * 32; g8 += nt) {
      uint32_t X[4];
      unpack8(raw + ro.sk, g8 * P.eq, P.eq, X);
      // in range when (v + 128) mod 2^eq < 256; the low byte is then the value
      uint32_t bad = 0;
#pragma unroll
      for (int i = 0; i < 4; i++) bad |= ((X[i] + 0x00800080u) & m) & 0xFF00FF00u;
      const uint32_t s0 = __byte_perm(X[0], X[1], 0x6420), s1 = __byte_perm(X[2], X[3], 0x6420);
      ok = ok && bad == 0u && small4(s0) && small4(s1);
      sec8w[2 * g8] = s0;
      sec8w[2 * g8 + 1] = s1;
      sencw[2 * g8] = enc4<kFp8Tcgen05>(s0);
      sencw[2 * g8 + 1] = enc4<kFp8Tcgen05>(s1);
    }
  }
  for (int w = packed13 ? L * 64 : tid; w < L * 64; w += nt) {
    uint32_t sb;
    if (OP == kMatvec) {
      sb = *reinterpret_cast<const uint32_t *>(raw + ro.s + 4 * w);
    } else if (OP == kDecrypt) {
      if (P.sable) {
        // 2-bit two's complement (SABLE pack.cu:371-376): one byte = 4 coefficients
        uint32_t x = raw[ro.sk + w];
        uint32_t spread = (x & 3u) | ((x & 0xcu) << 6) | ((x & 0x30u) << 12) | ((x & 0xc0u) << 18);
        uint32_t sgn = (spread >> 1) & 0x01010101u;
        sb = spread | (sgn * 0xfcu);
      } else {
        // 13-bit two's complement (SABER pack.cu:53-84)
        uint32_t v0 = get_bits(raw + ro.sk, (4 * w) * P.eq, P.eq);
        uint32_t v1 = get_bits(raw + ro.sk, (4 * w + 1) * P.eq, P.eq);
        uint32_t v2 = get_bits(raw + ro.sk, (4 * w + 2) * P.eq, P.eq);
        uint32_t v3 = get_bits(raw + ro.sk, (4 * w + 3) * P.eq, P.eq);
        uint32_t top = (1u << P.eq) - 128u;
        ok = ok && (v0 < 128u || v0 >= top) && (v1 < 128u || v1 >= top) && (v2 < 128u || v2 >= top) &&
             (v3 < 128u || v3 >= top);
        sb = (v0 & 0xffu) | ((v1 & 0xffu) << 8) | ((v2 & 0xffu) << 16) | ((v3 & 0xffu) << 24);
      }
    } else if (P.mu == 8) {
      // CBD mu = 8 (SABER poly.cu:864-887): popcount(low nibble) - popcount(high nibble)
      uint32_t x = *reinterpret_cast<const uint32_t *>(raw + ro.s + 4 * w);
      uint32_t n = x - ((x >> 1) & 0x55555555u);
      n = (n & 0x33333333u) + ((n >> 2) & 0x33333333u);
      sb = __vsub4(n & 0x0f0f0f0fu, (n >> 4) & 0x0f0f0f0fu);
    } else if (P.mu == 2) {
      // CBD mu = 2 (SABLE fips202.cu:625-651): bit 2i - bit 2i+1
      uint32_t x = raw[ro.s + w];
      uint32_t spread = (x & 3u) | ((x & 0xcu) << 6) | ((x & 0x30u) << 12) | ((x & 0xc0u) << 18);
      sb = __vsub4(spread & 0x01010101u, (spread >> 1) & 0x01010101u);
    } else {
      uint32_t r = 0;
      const int h = P.mu >> 1;
#pragma unroll
      for (int b = 0; b < 4; b++) {
        uint32_t x = get_bits(raw + ro.s, (4 * w + b) * P.mu, P.mu);
        int v = __popc(x & ((1u << h) - 1u)) - __popc(x >> h);
        r |= ((uint32_t)v & 0xffu) << (8 * b);
      }
      sb = r;
    }
    ok = ok && small4(sb);
    sec8w[w] = sb;
    sencw[w] = enc4<kFp8Tcgen05>(sb);
  }
  // 2. digit columns (K reversed, core-matrix order) and zero padding columns
  const int padc = NU - S.ncols;
  for (int idx = tid; idx < L * padc * 16; idx += nt) {
    const int j = idx / (padc * 16), r = idx % (padc * 16), n = S.ncols + r % padc, ac = r / padc;
    *reinterpret_cast<uint4 *>(B + j * 256 * NU + ac * 16 * NU + (n >> 3) * 128 + (n & 7) * 16) =
        make_uint4(0u, 0u, 0u, 0u);
  }
  for (int idx = tid; idx < S.R * L * 32; idx += nt) {
    const int grp = idx & 31, j = (idx >> 5) % L, p = idx / (32 * L);
    uint32_t X[4];
    if (OP == kMatvec) {
      const int ij = a.mv_transpose ? (j * L + p) : (p * L + j);
      uint4 u = *reinterpret_cast<const uint4 *>(raw + ro.a + ij * 512 + 16 * grp);
      const uint32_t m = ((1u << S.wa) - 1u) * 0x10001u;
      X[0] = u.x & m; X[1] = u.y & m; X[2] = u.z & m; X[3] = u.w & m;
    } else if (OP == kDecrypt) {
      unpack8(raw + ro.ct, (32 * j + grp) * S.wb, S.wb, X);
    } else if (p < S.RA) {
      const int ij = (OP == kKeygen) ? (j * L + p) : (p * L + j);
      unpack8(raw + ro.a, (32 * ij + grp) * S.wa, S.wa, X);
    } else {
      unpack8(raw + ro.b, (32 * j + grp) * S.wb, S.wb, X);
    }
    const int D = p < S.RA ? S.Da : S.Db;
    const int cb = p < S.RA ? p * S.Da : S.RA * S.Da + (p - S.RA) * S.Db;
    const int kq = 31 - grp;  // coefficients 8grp..8grp+7 are rows k' = 8kq+7..8kq
    uint8_t *base = B + j * 256 * NU + (kq >> 1) * 16 * NU + 8 * (kq & 1);
    for (int d = 0; d < D; d++) {
      const int n = cb + d;
      const uint2 v = digit8<kFp8Tcgen05>(X, d, p < S.RA ? S.wa : S.wb);
      *reinterpret_cast<uint2 *>(base + (n >> 3) * 128 + (n & 7) * 16) =
          make_uint2(__byte_perm(v.y, 0, 0x0123), __byte_perm(v.x, 0, 0x0123));
    }
  }
  wsync();  // secret words complete before s_ext reads them
  // 3. s_ext, then the Hankel core matrices
  stage_ext(ext, sencw, L, tid, nt, [](uint32_t v) { return v ^ 0x80808080u; });
  wsync();
  stage_hankel(H, ext, L, tid, nt);
  fence_async_smem();  // generic-proxy writes -> visible to the tensor core
  return wsync_and(ok);
}

// The 16 L MMAs of one instance (one thread): D[hh] (TMEM columns
// tmem + hh * NU) = sum_j H_j[rows 128hh..] x B_j.
__device__ __forceinline__ void issue5(const Shape5 &S, const uint8_t *ops, uint32_t tmem, uint32_t mbar) {
  const int L = S.L, NU = S.NU;
  const uint32_t idesc = umma_idesc_e4m3(NU);
  const uint32_t h0 = smem_u32(ops), b0 = h0 + L * kHankelBytes;
  tc_fence_after();
#pragma unroll 1
  for (int j = 0; j < L; j++) {
    // descriptors differ only in the start address field (16-byte units)
    const uint64_t ad0 = umma_desc(h0 + j * kHankelBytes, 256, 128);
    const uint64_t bd0 = umma_desc(b0 + j * 256 * NU, 16 * NU, 128);
    const uint32_t bstep = (uint32_t)(2 * 16 * NU) >> 4;
#pragma unroll
    for (int ks = 0; ks < 8; ks++) {
      const uint64_t bd = bd0 + (uint64_t)(ks * bstep);
#pragma unroll
      for (int hh = 0; hh < 2; hh++) {
        const uint64_t ad = ad0 + (uint64_t)(((16 * hh + 4 * ks) * 128) >> 4);
        umma_f8(tmem + hh * NU, ad, bd, idesc, (j | ks) != 0);
      }
    }
  }
  umma_commit(mbar);
}

// Accumulators of one instance -> int32 columns acc[col][256] in shared
// memory.  Warps 0-3 read M half 0 (rows 0..127), warps 4-7 half 1; warp w
// reads TMEM lanes 32 (w % 4) .. +31.
__device__ __forceinline__ void drain5(const Shape5 &S, uint32_t tmem, int *acc) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int hh = warp >> 2, q = warp & 3;
  const int row = 128 * hh + 32 * q + lane;
  for (int cc = 0; cc < S.NU; cc += 16) {
    uint32_t r[16];
    tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + hh * S.NU + cc, r);
#pragma unroll
    for (int c = 0; c < 16; c++) acc[(cc + c) * 256 + row] = __float2int_rn(__uint_as_float(r[c]));
  }
}

// Epilogue of one instance (worker warps; contains worker barriers): recombines
// the radix-16 digit columns of acc and rounds / encodes / packs / compares /
// decodes eight coefficients at a time (the same arithmetic as the
// per-instance kernel, SABER poly.cu:15-16, pack.cu:7-212, the compare of
// verify_gpu at pack.cu:225-241).
template <int OP>
__device__ __forceinline__ void epi5(const CpaArgs &a, const Shape5 &S, int inst, const uint8_t *raw,
                                     const RawOff &ro, const int *acc, const int8_t *s8, uint8_t *outb) {
  const KemParams &P = a.P;
  const int tid = threadIdx.x, nt = kWorkers;
  const int L = S.L;
  auto combine8 = [&](int p, int grp, uint32_t (&V)[4]) {
    const int D = p < S.RA ? S.Da : S.Db;
    const int cb = p < S.RA ? p * S.Da : S.RA * S.Da + (p - S.RA) * S.Db;
    const int4 *base = reinterpret_cast<const int4 *>(acc + 8 * grp);
    uint32_t v[8];
    {
      int4 x0 = base[cb * 64], x1 = base[cb * 64 + 1];
      v[0] = x0.x; v[1] = x0.y; v[2] = x0.z; v[3] = x0.w;
      v[4] = x1.x; v[5] = x1.y; v[6] = x1.z; v[7] = x1.w;
    }
    for (int d = 1; d < D; d++) {
      const uint32_t wgt = 1u << (4 * d);
      int4 x0 = base[(cb + d) * 64], x1 = base[(cb + d) * 64 + 1];
      v[0] += wgt * (uint32_t)x0.x; v[1] += wgt * (uint32_t)x0.y;
      v[2] += wgt * (uint32_t)x0.z; v[3] += wgt * (uint32_t)x0.w;
      v[4] += wgt * (uint32_t)x1.x; v[5] += wgt * (uint32_t)x1.y;
      v[6] += wgt * (uint32_t)x1.z; v[7] += wgt * (uint32_t)x1.w;
    }
#pragma unroll
    for (int i = 0; i < 4; i++) V[i] = (v[2 * i] & 0xffffu) | (v[2 * i + 1] << 16);
  };
  const uint32_t qmask = (1u << P.eq) - 1u, pmask = (1u << P.ep) - 1u;
  auto round_lanes = [&](uint32_t x) -> uint32_t {
    uint32_t lo16 = (((x & 0xffffu) + P.h1) & qmask) >> (P.eq - P.ep);
    uint32_t hi16 = (((x >> 16) + P.h1) & qmask) >> (P.eq - P.ep);
    return lo16 | (hi16 << 16);
  };
  auto encode_lanes = [&](uint32_t x, uint32_t mlo, uint32_t mhi) -> uint32_t {
    uint32_t lo16 = (((x & 0xffffu) + P.h1 - (mlo << (P.ep - 1))) & pmask) >> (P.ep - P.et);
    uint32_t hi16 = (((x >> 16) + P.h1 - (mhi << (P.ep - 1))) & pmask) >> (P.ep - P.et);
    return lo16 | (hi16 << 16);
  };

  if (OP == kDecrypt) {
    if (tid < 32) {
      uint32_t V[4], CM[4];
      combine8(0, tid, V);
      unpack8(raw + ro.ct + L * P.polycompbytes, tid * P.et, P.et, CM);
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
    wsync();
  } else if (OP == kEncrypt || OP == kReenc) {
    const uint8_t *msg = raw + ro.msg;
    int diff = 0;
    for (int idx = tid; idx < S.R * 32; idx += nt) {
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
        unpack8(raw + ro.ct, byte0, w, Cv);
        diff |= (Cv[0] ^ W[0]) | (Cv[1] ^ W[1]) | (Cv[2] ^ W[2]) | (Cv[3] ^ W[3]);
      } else {
        pack8(outb + byte0, W, w);
      }
    }
    if (OP == kReenc) {
      int any = wsync_or(diff != 0);
      if (tid == 0) a.fail[inst] = (uint8_t)(any != 0);
    } else {
      wsync();
      const uint4 *src = reinterpret_cast<const uint4 *>(outb);
      uint4 *dst = reinterpret_cast<uint4 *>(a.ct_out + (size_t)inst * P.ct_bytes);
      for (int i = tid; i < (P.ct_bytes >> 4); i += nt) dst[i] = src[i];
      wsync();
    }
  } else if (OP == kKeygen) {
    const int bbytes = L * P.polycompbytes;
    for (int idx = tid; idx < L * 32; idx += nt) {
      const int p = idx >> 5, grp = idx & 31;
      uint32_t V[4], W[4];
      combine8(p, grp, V);
#pragma unroll
      for (int i = 0; i < 4; i++) W[i] = round_lanes(V[i]);
      pack8(outb + (32 * p + grp) * P.ep, W, P.ep);
    }
    // secret key: 13-bit two's complement (Saber) or 2-bit (Sable) of sec8
    const int sw = P.sable ? 2 : P.eq;
    for (int grp = tid; grp < L * 32; grp += nt) {
      uint32_t Sv[4];
#pragma unroll
      for (int i = 0; i < 4; i++)
        Sv[i] = ((uint32_t)(int)s8[8 * grp + 2 * i] & 0xffffu) | ((uint32_t)(int)s8[8 * grp + 2 * i + 1] << 16);
      pack8(outb + bbytes + grp * sw, Sv, sw);
    }
    wsync();
    uint8_t *pko = a.pk_out + (size_t)inst * P.pk_bytes;
    uint8_t *sko = a.sk_out + (size_t)inst * a.sk_stride;
    for (int i = tid; i < bbytes; i += nt) {
      pko[i] = outb[i];
      sko[P.indcpa_sk_bytes + i] = outb[i];
    }
    wsync();
    if (tid < 32) sko[P.indcpa_sk_bytes + bbytes + tid] = pko[bbytes + tid];  // seed_A
    for (int i = tid; i < P.indcpa_sk_bytes; i += nt) sko[i] = outb[bbytes + i];
    wsync();
  } else {  // kMatvec
    const uint32_t m = ((1u << a.mv_eq) - 1u) * 0x10001u;
    for (int idx = tid; idx < L * 32; idx += nt) {
      const int p = idx >> 5, grp = idx & 31;
      uint32_t V[4];
      combine8(p, grp, V);
      *reinterpret_cast<uint4 *>(a.mv_out + (size_t)inst * (L * 256) + p * 256 + 8 * grp) =
          make_uint4(V[0] & m, V[1] & m, V[2] & m, V[3] & m);
    }
    wsync();
  }
}

// The persistent kernel (see the top of this file).  The group table is a
// kernel parameter (read from the constant bank), so a captured graph carries
// it by value.  Warps 0-7 stage and finish instances; warp 8 issues the MMAs.
// mbarriers (all with one arrival per phase):
//   raw_full[3]   TMA bytes of the instance in raw[k % 3] have landed
//   ops_full[2]   ops[k & 1] holds instance k's operands (workers -> MMA warp)
//   acc_full[2]   instance k's MMAs are complete (tcgen05.commit -> workers)
//   tmem_free[2]  TMEM buffer k & 1 has been read out (workers -> MMA warp)
// Instance k uses phase parity (k / 3) & 1 of raw_full and (k >> 1) & 1 of the
// others.
static_assert(sizeof(MixRef) <= 4000, "the launch reference must fit the kernel parameter space");

template <int OP>
__global__ void __launch_bounds__(kPersistThreads, 1) k_cpa5p(const __grid_constant__ MixRef T, PLayout lo) {
  extern __shared__ __align__(16) uint8_t sm[];
  const int tid = threadIdx.x;
  const uint32_t bar0 = smem_u32(sm + lo.bar);
  auto raw_full = [&](int k) { return bar0 + 8u * (uint32_t)(k % 3); };
  auto ops_full = [&](int k) { return bar0 + 24u + 8u * (uint32_t)(k & 1); };
  auto acc_full = [&](int k) { return bar0 + 40u + 8u * (uint32_t)(k & 1); };
  auto tmem_free = [&](int k) { return bar0 + 56u + 8u * (uint32_t)(k & 1); };
  auto par3 = [](int k) { return (uint32_t)((k / 3) & 1); };
  auto par2 = [](int k) { return (uint32_t)((k >> 1) & 1); };
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + lo.bar + 72);
  __shared__ volatile int s_abort;

  if (tid < 32) tmem_alloc(smem_u32(tmem_slot), (uint32_t)lo.tmem_cols);
  if (tid == 32) {
    for (int i = 0; i < 9; i++) mbar_init(bar0 + 8u * i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(tmem_slot);
  auto tmem_buf = [&](int k) { return tmem + (uint32_t)((k & 1) * 2 * lo.nu_max); };

  const int total = T.total, stride = gridDim.x;
  const int cnt = (int)blockIdx.x < total ? (total - 1 - (int)blockIdx.x) / stride + 1 : 0;
  auto locate = [&](int k, int &g, int &inst) {
    const int gi = (int)blockIdx.x + k * stride;
    g = find_group(T, gi);
    inst = gi - group_first(T, g);
  };
  // a bounded wait that also gives up once another role has given up
  auto wait = [&](uint32_t mbar, uint32_t parity) {
    const uint64_t t0 = global_ns();
    for (uint32_t i = 0;; i++) {
      if (mbar_try_wait(mbar, parity)) return true;
      if ((i & 63u) == 63u && (s_abort || global_ns() - t0 > 2000000000ull)) {
        s_abort = 1;
        return false;
      }
    }
  };
  // outstanding asynchronous work, for a bounded drain if a wait gives up
  int raw_lo = 0, raw_hi = 0;  // prefetched, not yet waited
  int mma_hi = 0;              // instances whose MMAs were issued

  if (tid >= kWorkers) {
    // ---- MMA warp
    for (int k = 0; k < cnt; k++) {
      if (!wait(ops_full(k), par2(k))) break;
      if (k >= 2 && !wait(tmem_free(k), par2(k - 2))) break;
      if (tid == kWorkers) {
        int g, inst;
        locate(k, g, inst);
        issue5(shape5<OP>(group_args(T, g)), sm + lo.ops[k & 1], tmem_buf(k), acc_full(k));
      }
      __syncwarp();
      mma_hi = k + 1;
    }
    if (s_abort) {
      // at most the last two issued instances can still be running
      for (int k = mma_hi - 2 < 0 ? 0 : mma_hi - 2; k < mma_hi; k++) mbar_wait_bounded(acc_full(k), par2(k));
    }
  } else {
    // ---- worker warps
    auto prefetch = [&](int k) {  // thread 0: inputs of instance k into raw[k % 3]
      int g, inst;
      locate(k, g, inst);
      prefetch5<OP>(group_args(T, g), inst, sm + lo.raw[k % 3], raw_full(k));
    };
    if (tid == 0) {
      if (cnt > 0) prefetch(0);
      if (cnt > 1) prefetch(1);
    }
    raw_hi = cnt < 2 ? cnt : 2;
    for (int it = 0; it <= cnt; it++) {
      if (it < cnt) {
        int g, inst;
        locate(it, g, inst);
        const CpaArgs &a = group_args(T, g);
        const Shape5 S = shape5<OP>(a);
        const RawOff ro = raw_off<OP>(a.P);
        const bool got = wait(raw_full(it), par3(it));
        if (wsync_or(!got)) break;
        raw_lo = it + 1;
        // ops[it & 1] and sec8[it & 1] were last used by instance it-2, finished below
        const bool ok = stage5<OP>(a, S, sm + lo.raw[it % 3], ro, reinterpret_cast<uint32_t *>(sm + lo.sec8[it & 1]),
                                   reinterpret_cast<uint32_t *>(sm + lo.senc), sm + lo.ops[it & 1]);
        if (tid == 0) {
          if (!ok && a.err) atomicOr(a.err, 1);
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(ops_full(it)) : "memory");
        }
      }
      if (it > 0) {
        // instance k = it - 1: accumulators -> int32 columns, then its epilogue
        const int k = it - 1;
        int g, inst;
        locate(k, g, inst);
        const CpaArgs &a = group_args(T, g);
        const Shape5 S = shape5<OP>(a);
        const RawOff ro = raw_off<OP>(a.P);
        const bool done = wait(acc_full(k), par2(k));
        tc_fence_after();
        int *acc = reinterpret_cast<int *>(sm + lo.ops[k & 1]);
        if (__all_sync(0xffffffffu, done)) drain5(S, tmem_buf(k), acc);
        tc_fence_before();
        if (wsync_or(!done)) break;
        if (tid == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tmem_free(k)) : "memory");
        epi5<OP>(a, S, inst, sm + lo.raw[k % 3], ro, acc, reinterpret_cast<const int8_t *>(sm + lo.sec8[k & 1]),
                 sm + lo.out);
      }
      // raw[(it + 2) % 3] held instance it - 1, finished above (epi5 ends with a worker barrier)
      if (it + 2 < cnt) {
        if (tid == 0) prefetch(it + 2);
        raw_hi = it + 3;
      }
    }
    if (s_abort) {
      for (int k = raw_lo; k < raw_hi; k++) mbar_wait_bounded(raw_full(k), par3(k));
    }
  }
  __syncthreads();
  if (s_abort && tid == 0) {
    for (int g = 0; g < T.ngroups; g++)
      if (group_args(T, g).err) atomicOr(group_args(T, g).err, 2);
  }
  tc_fence_before();
  __syncthreads();
  if (tid < 32) tmem_dealloc(tmem, (uint32_t)lo.tmem_cols);
}

}  // namespace tmvp

namespace tmvp {

// Host side: the layout for groups g[0..ng), the launch shape, the launch.
template <int OP>
inline PLayout persist_layout(const CpaArgs *groups, int ng) {
  int raw = 0, lmax = 2, nu = 16, ops = 0, out = 16;
  for (int g = 0; g < ng; g++) {
    const CpaArgs &a = groups[g];
    const Shape5 S = shape5<OP>(a);
    const RawOff ro = raw_off<OP>(a.P);
    raw = std::max(raw, ro.bytes);
    lmax = std::max(lmax, S.L);
    nu = std::max(nu, S.NU);
    ops = std::max(ops, std::max(S.L * (kHankelBytes + 256 * S.NU + 512), S.NU * 1024));
    if (OP == kEncrypt) out = std::max(out, a.P.ct_bytes + 16);
    if (OP == kKeygen) out = std::max(out, S.L * a.P.polycompbytes + a.P.indcpa_sk_bytes + 16);
  }
  PLayout lo;
  int off = 0;
  auto take = [&](int bytes) { int r = off; off = (off + bytes + 127) & ~127; return r; };
  for (int i = 0; i < 2; i++) lo.ops[i] = take(ops);
  for (int i = 0; i < 3; i++) lo.raw[i] = take(raw);
  for (int i = 0; i < 2; i++) lo.sec8[i] = take(lmax * 256);
  lo.senc = take(lmax * 256);
  lo.out = take(out);
  lo.bar = take(96);
  lo.total = off;
  lo.nu_max = nu;
  lo.tmem_cols = 4 * nu;  // 2 buffers x 2 M halves x N
  return lo;
}

// Launches groups[0..ng) (host copies; dev_tab holds the same groups in device
// memory when ng > 1) on `s` with `ctas_per_sm` CTAs per SM (0: as many as
// fit).  Returns a CUDA error code.
template <int OP>
inline int launch_persist(const CpaArgs *groups, int ng, const MixTable *dev_tab, cudaStream_t s,
                          int ctas_per_sm) {
  MixRef R{};
  R.ngroups = ng;
  R.total = 0;
  for (int g = 0; g < ng; g++) R.total += groups[g].n;
  if (R.total <= 0) return 0;
  if (ng == 1) {
    R.tab = nullptr;
    R.one = groups[0];
  } else {
    if (!dev_tab) return (int)cudaErrorInvalidValue;
    R.tab = dev_tab;
  }
  const PLayout lo = persist_layout<OP>(groups, ng);
  auto fn = k_cpa5p<OP>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, lo.total);
  if (e != cudaSuccess) return (int)e;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return (int)e;
  int dev = 0, nsm = 0, fit = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
  if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return (int)e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, fn, kPersistThreads, lo.total)) != cudaSuccess)
    return (int)e;
  fit = std::min(fit, 512 / lo.tmem_cols);  // every CTA's tensor memory fits at once
  if (fit < 1) return (int)cudaErrorInvalidConfiguration;
  const int per = ctas_per_sm > 0 ? std::min(ctas_per_sm, fit) : fit;
  const int grid = std::min(R.total, per * nsm);
  fn<<<grid, kPersistThreads, lo.total, s>>>(R, lo);
  return (int)cudaGetLastError();
}

}  // namespace tmvp
