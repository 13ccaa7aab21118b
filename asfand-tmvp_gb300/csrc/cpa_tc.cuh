// cpa_tc.cuh — operand staging and the mma.sync engine of the tensor-core
// IND-CPA forms.
//
// The mma.sync forms multiply the negacyclic Toeplitz matrix of a small
// secret (A operand, m16 x k32) by digit columns of the public polynomials (B
// operand, k32 x n8):
//   FP8  (mma.sync m16n8k32 e4m3 x e4m3 -> f32): the public coefficient is
//        split into unsigned radix-8 digits d (3 bits each); a column holds
//        the e4m3 encoding of 8 + d, which is the byte 0x50 | d, so a digit
//        column costs one OR per four coefficients.  Column 0 holds 1.0 and
//        yields the row sums of the Toeplitz matrix, which remove the +8 bias:
//            res = sum_d 8^d (acc_d - 8 * rowsum).
//        |acc| <= 768 * 8 * 15 < 2^24, so the f32 accumulator is exact.
//   INT8 (mma.sync m16n8k32 s8 x u8 -> s32): two 8-bit limbs per coefficient.
// The Toeplitz fragments are 4-byte windows of srev[k] = s_ext[510 - k],
// read from four byte-shifted copies so that every window is an aligned word.
// The tcgen05 form (cpa_umma.cuh) uses radix-16 digits (r16_digits), each
// exact in e4m3, and no bias column.
#pragma once
#include <cstdint>

#include "cpa_engine.cuh"
#include "cpa_umma.cuh"
#include "kem_common.cuh"

namespace tmvp {

// 16-byte copy of nbytes (a multiple of 16) by the whole CTA.
__device__ __forceinline__ void copy16(uint8_t *dst, const uint8_t *src, int nbytes) {
  const uint4 *s = reinterpret_cast<const uint4 *>(src);
  uint4 *d = reinterpret_cast<uint4 *>(dst);
  for (int i = threadIdx.x; i < (nbytes >> 4); i += blockDim.x) d[i] = s[i];
}

// Digit columns of a w-bit public coefficient.
template <int FORM>
__host__ __device__ __forceinline__ int tc_digits(int w) {
  return FORM == kFp8TC ? (w + 2) / 3 : (FORM == kFp8Tcgen05 ? r16_digits(w) : 2);
}

// Number of B columns for R public polys whose first RA have width wa and the
// rest width wb (FP8 adds the ones column in front).
template <int FORM>
__host__ __device__ __forceinline__ int tc_cols(int R, int RA, int wa, int wb) {
  int c = RA * tc_digits<FORM>(wa) + (R - RA) * tc_digits<FORM>(wb);
  return FORM == kFp8TC ? c + 1 : c;
}

// Eight w-bit little-endian fields starting at byte `byte0` of a shared-memory
// stream, as four words of two 16-bit lanes (coefficient 2i in the low lane).
// The stream buffer has 16 bytes of slack after its end.
__device__ __forceinline__ void unpack8(const uint8_t *base, int byte0, int w, uint32_t (&X)[4]) {
  const uint32_t *wp = reinterpret_cast<const uint32_t *>(base + (byte0 & ~3));
  const int sh = 8 * (byte0 & 3);
  uint32_t q[5];
#pragma unroll
  for (int i = 0; i < 5; i++) q[i] = wp[i];
  uint32_t a[4];
#pragma unroll
  for (int i = 0; i < 4; i++) a[i] = __funnelshift_r(q[i], q[i + 1], sh);
  const uint32_t m = (1u << w) - 1u;
#pragma unroll
  for (int k = 0; k < 8; k += 2) {
    int b0 = k * w, b1 = (k + 1) * w;
    uint32_t v0 = __funnelshift_r(a[b0 >> 5], a[(b0 >> 5) + 1 < 4 ? (b0 >> 5) + 1 : 3], b0 & 31) & m;
    uint32_t v1 = __funnelshift_r(a[b1 >> 5], a[(b1 >> 5) + 1 < 4 ? (b1 >> 5) + 1 : 3], b1 & 31) & m;
    X[k >> 1] = __byte_perm(v0, v1, 0x5410);
  }
}

// Digit column words for eight coefficients held as 16-bit lanes.
// FP8: bytes 0x50 | ((x >> 3d) & 7).  INT8: limb d = (x >> 8d) & 0xff.
// tcgen05 FP8: e4m3 of (x >> 4d) & 15, or of the signed 5-bit top digit of a
// w-bit coefficient (r16_digits).
template <int FORM>
__device__ __forceinline__ uint2 digit8(const uint32_t (&X)[4], int d, int w = 16) {
  uint32_t t[4];
  if (FORM == kFp8Tcgen05) {
    if (w - 4 * d == 5) {
#pragma unroll
      for (int i = 0; i < 4; i++) t[i] = (X[i] >> (4 * d)) & 0x001F001Fu;
      return make_uint2(e4m3_sdigits4(__byte_perm(t[0], t[1], 0x6420)),
                        e4m3_sdigits4(__byte_perm(t[2], t[3], 0x6420)));
    }
#pragma unroll
    for (int i = 0; i < 4; i++) t[i] = (X[i] >> (4 * d)) & 0x000F000Fu;
    return make_uint2(e4m3_digits4(__byte_perm(t[0], t[1], 0x6420)),
                      e4m3_digits4(__byte_perm(t[2], t[3], 0x6420)));
  } else if (FORM == kFp8TC) {
#pragma unroll
    for (int i = 0; i < 4; i++) t[i] = ((X[i] >> (3 * d)) & 0x00070007u) | 0x00500050u;
    return make_uint2(__byte_perm(t[0], t[1], 0x6420), __byte_perm(t[2], t[3], 0x6420));
  } else {
    const uint32_t sel = d == 0 ? 0x6420 : 0x7531;
    return make_uint2(__byte_perm(X[0], X[1], sel), __byte_perm(X[2], X[3], sel));
  }
}

// 8-bit operand encoding of a small secret coefficient.
template <int FORM>
__device__ __forceinline__ uint32_t enc_small(int v) {
  if (FORM == kFp8TC) {
    uint16_t r;
    asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;" : "=h"(r) : "f"(0.f), "f"((float)v));
    return r & 0xffu;
  }
  return (uint32_t)v & 0xffu;
}

// Toeplitz copies of one secret polynomial (sec: int16 [256]).  Copy 0 is
// srev itself; copy c, word w = srev bytes [4w + c, 4w + c + 4).
template <int FORM>
__device__ __forceinline__ void stage_toeplitz_v2(uint32_t *tz, const int16_t *sec, int nthreads) {
  uint32_t *c0 = tz;
  for (int w = threadIdx.x; w < 130; w += nthreads) {
    uint32_t word = 0;
#pragma unroll
    for (int b = 0; b < 4; b++) {
      int k = 4 * w + b;
      int v = k <= 255 ? (int)sec[255 - k] : (k <= 510 ? -(int)sec[511 - k] : 0);
      word |= enc_small<FORM>(v) << (8 * b);
    }
    c0[w] = word;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 3 * 128; idx += nthreads) {
    int c = 1 + idx / 128, w = idx % 128;
    uint32_t sel = (uint32_t)(c | ((c + 1) << 4) | ((c + 2) << 8) | ((c + 3) << 12));
    tz[c * kTzCopyWords + w] = __byte_perm(c0[w], c0[w + 1], sel);
  }
}

// The mma loop.  WARPS warps, MT = 16/WARPS m-tiles each; Q n-tiles.  colw:
// [l][Q*8 columns][kColStride bytes] (only stored columns are read; colflag
// per thread and tile says whether its column is stored (1), the FP8 ones
// column (2) or padding (0)).  Accumulators are written as int32 to
// acc_out[col][256] after a barrier (the region may alias colw/tz).
template <int FORM, int Q, int WARPS>
__device__ __forceinline__ void tc_engine_v2(const uint32_t *tz, const uint32_t *colw, int l,
                                             int ncols, int *acc_out) {
  constexpr int MT = 16 / WARPS;
  typedef typename AccT<FORM>::type acc_t;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int mt0 = warp * MT;
  const int copy = (3 - g) & 3;
  const int wbase = 63 - (g >> 2) + t - 4 * mt0;
  int kind[Q];  // 0: padding, 1: stored column, 2: ones column
#pragma unroll
  for (int q = 0; q < Q; q++) {
    int col = 8 * q + g;
    kind[q] = col >= ncols ? 0 : ((FORM == kFp8TC && col == 0) ? 2 : 1);
  }
  acc_t acc[MT][Q][4];
#pragma unroll
  for (int i = 0; i < MT; i++)
#pragma unroll
    for (int q = 0; q < Q; q++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[i][q][e] = 0;

  for (int j = 0; j < l; j++) {
    const uint32_t *T = tz + (j * 4 + copy) * kTzCopyWords;
    const uint32_t *B = colw + (size_t)(j * Q * 8 + g) * (kColStride / 4) + t;
    uint32_t a[MT][4];
#pragma unroll 1
    for (int kt = 0; kt < 8; kt++) {
      uint32_t b[Q][2];
#pragma unroll
      for (int q = 0; q < Q; q++) {
        if (kind[q] == 1) {
          b[q][0] = B[q * 8 * (kColStride / 4) + 8 * kt];
          b[q][1] = B[q * 8 * (kColStride / 4) + 8 * kt + 4];
        } else {
          uint32_t v = kind[q] == 2 ? 0x38383838u : 0u;  // e4m3 1.0
          b[q][0] = v;
          b[q][1] = v;
        }
      }
      if (kt > 0) {
#pragma unroll
        for (int i = MT - 1; i >= 2; i--)
#pragma unroll
          for (int e = 0; e < 4; e++) a[i][e] = a[i - 2][e];
      }
#pragma unroll
      for (int i = 0; i < MT; i++) {
        if (kt == 0 || i < 2) {
          int w0 = wbase - 4 * i + 8 * kt;
          a[i][0] = T[w0];
          a[i][1] = T[w0 - 2];
          a[i][2] = T[w0 + 4];
          a[i][3] = T[w0 + 2];
        }
      }
#pragma unroll
      for (int i = 0; i < MT; i++)
#pragma unroll
        for (int q = 0; q < Q; q++) {
          if (FORM == kFp8TC)
            mma_m16n8k32<FORM>(*reinterpret_cast<float(*)[4]>(&acc[i][q][0]), a[i], b[q]);
          else
            mma_m16n8k32_s8u8(*reinterpret_cast<int(*)[4]>(&acc[i][q][0]), a[i], b[q]);
        }
    }
  }
  __syncthreads();  // all warps done reading tz / colw before acc_out (aliased) is written
#pragma unroll
  for (int i = 0; i < MT; i++) {
    const int r0 = 16 * (mt0 + i) + g;
#pragma unroll
    for (int q = 0; q < Q; q++) {
      int c0 = 8 * q + 2 * t;
      if (c0 < ncols) {
        acc_out[c0 * 256 + r0] = acc_to_int(acc[i][q][0]);
        acc_out[c0 * 256 + r0 + 8] = acc_to_int(acc[i][q][2]);
      }
      if (c0 + 1 < ncols) {
        acc_out[(c0 + 1) * 256 + r0] = acc_to_int(acc[i][q][1]);
        acc_out[(c0 + 1) * 256 + r0 + 8] = acc_to_int(acc[i][q][3]);
      }
    }
  }
}

}  // namespace tmvp
