// cpa_engine.cuh — the polynomial engines of the IND-CPA kernels.
//
// Every CPA step of the KEM is one shape: for R public polynomials per
// module index j and l small secrets s_j,
//     res[r] = sum_j P[r][j] * s_j     in Z_{2^16}[x]/(x^256+1).
// MatrixVectorMul (SABER poly.cu:269-376) is R = l with P = A (A^T for key
// generation); InnerProd (poly.cu:227-248) is R = 1; encryption runs both at
// once (R = l+1), because the Toeplitz matrix of s'_j multiplies A[0..l-1][j]
// and b_j alike.
//
// The product s * v is the negacyclic Toeplitz matrix T(s) times v, with
// T(s)[r][c] = s_ext[r - c + 255], s_ext[255 + d] = s[d] (d >= 0) and
// -s[d + 256] (d < 0), as in convertnegacyclictest (poly.cu:1116-1129).
// Nothing here materialises T(s): the mma.sync engines read each 4-byte
// fragment word straight out of the reversed sequence srev[k] =
// s_ext[510 - k] (four byte-shifted copies keep every word aligned), and the
// CUDA-core engine slides a register window along the same sequence.
//
// The engines here:
//   * the mma.sync instructions of the FP8_TC and INT8_TC forms (the engine
//     itself is tc_engine_v2 in cpa_tc.cuh: e4m3 secrets against radix-8
//     public digits biased by 8, with a column of ones for the bias
//     correction; or s8 secrets against u8 limbs);
//   * cc_engine: one-level 2-way TMVP on CUDA cores (the reference's
//     submatrix_cuda / matvecp_cuda / matvecout_cuda split,
//     poly.cu:1295-1392): P1 = T00 (v0+v1), P2 = (T01-T00) v1,
//     P3 = (T00-T10) v0, r_lo = P1+P2, r_hi = P1-P3; or, for the schoolbook
//     form, the full 256x256 product;
//   * dp2a_engine and toom4_engine: the DP2A and Toom-Cook 4-way CUDA-core
//     forms.
#pragma once
#include <cstdint>

#include "kem_common.cuh"

namespace tmvp {

// ---------------------------------------------------------------------------
// Tensor-core (mma.sync) operand strides and instructions, used by the
// FP8_TC / INT8_TC kernels (cpa_tc.cuh, cpa_tc_kernel.cuh)
// ---------------------------------------------------------------------------
// Byte strides of the staged tensor-core operands.
constexpr int kColStride = 272;          // one digit column: 256 bytes + 16 pad
constexpr int kTzCopyWords = 136;        // one shifted copy of srev: 128 words + 8 pad
constexpr int kTzBytesPerPoly = 4 * kTzCopyWords * 4;

template <int FORM>
__device__ __forceinline__ void mma_m16n8k32(float (&d)[4], const uint32_t (&a)[4],
                                             const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k32.row.col.f32.e4m3.e4m3.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void mma_m16n8k32_s8u8(int (&d)[4], const uint32_t (&a)[4],
                                                  const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k32.row.col.s32.s8.u8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+r"(d[0]), "+r"(d[1]), "+r"(d[2]), "+r"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int FORM>
struct AccT { typedef float type; };
template <>
struct AccT<kInt8TC> { typedef int type; };

__device__ __forceinline__ int acc_to_int(float v) { return __float2int_rn(v); }
__device__ __forceinline__ int acc_to_int(int v) { return v; }

// ---------------------------------------------------------------------------
// CUDA-core engine
// ---------------------------------------------------------------------------
// TMVP form: tseq[j][p][x + 128] (int32, x in [-127,127]) are the defining
// sequences of T00, T01-T00, T00-T10; wv[j][p][c][RP] (u16) the vectors
// v0+v1, v1, v0.  Warp p computes product p; lane owns rows 4*lane..4*lane+3.
// Schoolbook form: tseq[j][0][x + 256] for x in [-255, 255], wv[j][0][c][RP]
// = v; 64 threads own 4 rows each.  Entry x = -128 (-256) is a zero pad that
// the last window slide reads.  Accumulation is unsigned (wraps mod 2^32);
// only the low 16 bits are used.
// TMVP recombination: product p of rows row0..row0+3 (acc[i][r]) to shared
// memory, then r_lo = P1 + P2, r_hi = P1 - P3 (SABER poly.cu:1383-1392).
template <int RP, class A>
__device__ __forceinline__ void tmvp_recombine(const A (&acc)[4][RP], bool active, int p, int row0, int R,
                                               int *pp, uint16_t *res) {
  if (active) {
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int r = 0; r < RP; r++)
        if (r < R) pp[(p * RP + r) * 128 + row0 + i] = (int)acc[i][r];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < R * 128; idx += blockDim.x) {
    int r = idx >> 7, k = idx & 127;
    uint32_t p1 = (uint32_t)pp[(0 * RP + r) * 128 + k], p2 = (uint32_t)pp[(1 * RP + r) * 128 + k],
             p3 = (uint32_t)pp[(2 * RP + r) * 128 + k];
    res[r * 256 + k] = (uint16_t)(p1 + p2);
    res[r * 256 + 128 + k] = (uint16_t)(p1 - p3);
  }
}

template <bool TMVP, int RP>
__device__ __forceinline__ void cc_engine(const int16_t *tseq, const uint16_t *wv, int l, int R,
                                          int *pp, uint16_t *res) {
  constexpr int NPROD = TMVP ? 3 : 1;
  constexpr int NCOL = TMVP ? 128 : 256;
  constexpr int XOFF = TMVP ? 128 : 256;  // ts[x] for x in [-XOFF, XOFF); x = -XOFF unused
  const int p = threadIdx.x / (NCOL / 4);
  const int row0 = 4 * (threadIdx.x % (NCOL / 4));
  const bool active = p < NPROD;
  uint32_t acc[4][RP];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int r = 0; r < RP; r++) acc[i][r] = 0;
  if (active) {
    for (int j = 0; j < l; j++) {
      const int16_t *ts = tseq + (j * NPROD + p) * 512 + XOFF;
      const uint16_t *w = wv + (size_t)(j * NPROD + p) * NCOL * RP;
      int win[4];
#pragma unroll
      for (int i = 0; i < 4; i++) win[i] = ts[row0 + i];
#pragma unroll 4
      for (int c = 0; c < NCOL; c++) {
        uint16_t wr[RP];
        if (RP == 4) {
          uint2 u = *reinterpret_cast<const uint2 *>(w + c * RP);
          wr[0] = u.x & 0xffff; wr[1] = u.x >> 16; wr[2] = u.y & 0xffff; wr[3] = u.y >> 16;
        } else {
#pragma unroll
          for (int r = 0; r < RP; r += 4) {
            uint2 u = *reinterpret_cast<const uint2 *>(w + c * RP + r);
            wr[r] = u.x & 0xffff; wr[r + 1] = u.x >> 16; wr[r + 2] = u.y & 0xffff; wr[r + 3] = u.y >> 16;
          }
        }
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int r = 0; r < RP; r++) acc[i][r] += (uint32_t)win[i] * (uint32_t)wr[r];
        // slide: rows row0+i need ts[row0 + i - (c+1)]
#pragma unroll
        for (int i = 3; i >= 1; i--) win[i] = win[i - 1];
        win[0] = ts[row0 - c - 1];
      }
    }
  }
  if (TMVP) {
    tmvp_recombine<RP>(acc, active, p, row0, R, pp, res);
  } else {
    if (active) {
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int r = 0; r < RP; r++)
          if (r < R) res[r * 256 + row0 + i] = (uint16_t)acc[i][r];
    }
  }
}

// ---------------------------------------------------------------------------
// DP2A engine (the DPSaber form; the reference's unused DoDP4Av7 kernels,
// SABER poly.cu:32-224, pair 16-bit public coefficients with 8-bit secrets the
// same way)
// ---------------------------------------------------------------------------
// The one-level TMVP split of cc_engine, with every dp2a instruction doing two
// multiply-adds: a word of two 16-bit public values (v[c], v[c+1]) times two
// signed bytes of a Toeplitz row (T[row][c], T[row][c+1]); dp2a.hi takes the
// next pair (c+2, c+3) against bytes 2 and 3 of the same word.
//   tb[j][p][w] (uint4): component cp = bytes u[4w+cp .. 4w+cp+3] of
//       u[k] = t_p[127 - k] (t_p the defining sequence of product p, t_p[x]
//       for |x| <= 127; 0 past k = 254), so that byte m of row `row`'s word
//       at column c is T_p[row][c+m] = u[127 - row + c + m].
//   wp[j][p][c/2][RP] (u32): v_r[c] | v_r[c+1] << 16 for public poly r.
// Warp p computes product p; lane owns rows 4 lane .. 4 lane + 3, whose four
// words for columns 4cb..4cb+3 are the four components of tb word
// 31 - lane + cb (row 4 lane + i in component 3 - i).  Products stay exact
// while |t_p| <= 127, i.e. |s| <= 63.
template <int RP>
__device__ __forceinline__ void dp2a_engine(const uint4 *tb, const uint32_t *wp, int l, int R, int *pp,
                                            uint16_t *res) {
  const int p = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = 4 * lane;
  const bool active = p < 3;
  int acc[4][RP];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int r = 0; r < RP; r++) acc[i][r] = 0;
  if (active) {
    for (int j = 0; j < l; j++) {
      const uint4 *T = tb + (j * 3 + p) * 64 + 31 - lane;
      const uint4 *W = reinterpret_cast<const uint4 *>(wp + (size_t)(j * 3 + p) * 64 * RP);
#pragma unroll 2
      for (int cb = 0; cb < 32; cb++) {
        const uint4 t = T[cb];
        const int tr[4] = {(int)t.w, (int)t.z, (int)t.y, (int)t.x};
        int va[RP], vb[RP];
#pragma unroll
        for (int q = 0; q < RP / 4; q++) {
          uint4 u = W[(2 * cb) * (RP / 4) + q], v = W[(2 * cb + 1) * (RP / 4) + q];
          va[4 * q] = (int)u.x; va[4 * q + 1] = (int)u.y; va[4 * q + 2] = (int)u.z; va[4 * q + 3] = (int)u.w;
          vb[4 * q] = (int)v.x; vb[4 * q + 1] = (int)v.y; vb[4 * q + 2] = (int)v.z; vb[4 * q + 3] = (int)v.w;
        }
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int r = 0; r < RP; r++) acc[i][r] = __dp2a_hi(vb[r], tr[i], __dp2a_lo(va[r], tr[i], acc[i][r]));
      }
    }
  }
  tmvp_recombine<RP>(acc, active, p, row0, R, pp, res);
}

// ---------------------------------------------------------------------------
// Toom-Cook 4-way engine (the reference's pol_mul, TMVP_SABLE pack.cu:505-732)
// ---------------------------------------------------------------------------
// Each operand's four 64-coefficient quarters are evaluated at the seven
// points 0, 1, -1, 1/2, -1/2, 2, infinity (half points scaled by 8).  The
// products at each point are 64x64 polynomial products; they are linear in
// the operands, so they are summed over the module index j in the evaluation
// domain and each output polynomial is interpolated once.  All arithmetic is
// mod 2^32: the interpolation's exact divisions by 2 and 4 are shifts, those
// by 3, 9 and 15 products with inverses mod 2^32, and every coefficient comes
// out correct mod 2^29.
//   sv[j][pt][kToomSStride] (u32): s_j's evaluation at point pt, at offset 64,
//       zero over the 64 words either side;
//   pv[r][j][pt][kToomPStride] (u32): public poly (r, j)'s evaluation.
// Product phase: warp w takes output blocks cb = w and 7 - w (16 coefficients
// each); lane (pt = lane / 4 < 7, sb = lane % 4) owns coefficients
// 16 cb + 4 sb .. +3 of point pt for all R public polys.  Every lane of a warp
// runs the same i range, the union of its 16 outputs' ranges.
constexpr int kToomSStride = 196;  // 192 words + 4: the seven points' windows fall in distinct bank groups
constexpr int kToomPStride = 68;   // 64 words + 4

__device__ __forceinline__ void toom4_eval(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t (&e)[7]) {
  e[0] = a0;
  e[1] = a0 + a1 + a2 + a3;
  e[2] = a0 - a1 + a2 - a3;
  e[3] = 8 * a0 + 4 * a1 + 2 * a2 + a3;
  e[4] = 8 * a0 - 4 * a1 + 2 * a2 - a3;
  e[5] = a0 + 2 * a1 + 4 * a2 + 8 * a3;
  e[6] = a3;
}

// w[k]: the product at point k -> c[k], coefficient of y^k (y = x^64).
//   E1 = (w1+w2)/2 = c0+c2+c4+c6        O1 = (w1-w2)/2 = c1+c3+c5
//   Eh = (w3+w4)/2 = 64c0+16c2+4c4+c6   V = (w3-w4)/4 = 16c1+4c3+c5
//   S = E1-c0-c6 = c2+c4                T = (Eh-64c0-c6)/4 = 4c2+c4
//   c2 = (T-S)/3, c4 = S-c2;  U = (w5-c0-4c2-16c4-64c6)/2 = c1+4c3+16c5
//   D = (V-U)/15 = c1-c5;  Sm = (V+U-8 O1)/9 = c1+c5
//   c1 = (Sm+D)/2, c5 = Sm-c1, c3 = O1-Sm
__device__ __forceinline__ void toom4_interp(uint32_t (&w)[7]) {
  const uint32_t inv3 = 0xAAAAAAABu, inv9 = 0x38E38E39u, inv15 = 0xEEEEEEEFu;
  const uint32_t c0 = w[0], c6 = w[6];
  const uint32_t e1 = (w[1] + w[2]) >> 1, o1 = (w[1] - w[2]) >> 1;
  const uint32_t eh = (w[3] + w[4]) >> 1, v = (w[3] - w[4]) >> 2;
  const uint32_t sv = e1 - c0 - c6, t = (eh - 64 * c0 - c6) >> 2;
  const uint32_t c2 = (t - sv) * inv3, c4 = sv - c2;
  const uint32_t u = (w[5] - c0 - 4 * c2 - 16 * c4 - 64 * c6) >> 1;
  const uint32_t d = (v - u) * inv15, sm = (v + u - 8 * o1) * inv9;
  const uint32_t c1 = (sm + d) >> 1;
  w[1] = c1; w[2] = c2; w[3] = o1 - sm; w[4] = c4; w[5] = sm - c1;
}

// sv, pv as above; wk: R x 7 x 128 words (may alias sv / pv).  Writes
// res[r][256] for r < R.
template <int R>
__device__ __forceinline__ void toom4_engine(const uint32_t *sv, const uint32_t *pv, int l, uint32_t *wk,
                                             uint16_t *res) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pt = lane >> 2, sb = lane & 3;
  const bool active = pt < 7 && warp < 4;
  uint32_t out[2][4][R];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int cb = h == 0 ? warp : 7 - warp;
    const int c0 = 16 * cb + 4 * sb;
    const int ib_lo = max(0, 16 * cb - 63) >> 2, ib_hi = min(63, 16 * cb + 15) >> 2;
    uint32_t acc[4][R];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int r = 0; r < R; r++) acc[q][r] = 0;
    if (active) {
      for (int j = 0; j < l; j++) {
        const uint32_t *S = sv + (j * 7 + pt) * kToomSStride + 64;
        // window w[0..7] = S[c0 - 4 ib - 4 .. c0 - 4 ib + 3]
        uint4 hi = *reinterpret_cast<const uint4 *>(S + c0 - 4 * ib_lo);
        uint4 lo = *reinterpret_cast<const uint4 *>(S + c0 - 4 * ib_lo - 4);
        for (int ib = ib_lo; ib <= ib_hi; ib++) {
          const uint32_t w[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
          for (int r = 0; r < R; r++) {
            const uint4 pq = *reinterpret_cast<const uint4 *>(pv + ((r * l + j) * 7 + pt) * kToomPStride + 4 * ib);
            const uint32_t pm[4] = {pq.x, pq.y, pq.z, pq.w};
#pragma unroll
            for (int q = 0; q < 4; q++)
#pragma unroll
              for (int m = 0; m < 4; m++) acc[q][r] += pm[m] * w[4 + q - m];
          }
          hi = lo;
          if (ib < ib_hi) lo = *reinterpret_cast<const uint4 *>(S + c0 - 4 * ib - 8);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int r = 0; r < R; r++) out[h][q][r] = acc[q][r];
  }
  __syncthreads();  // every lane is done with sv / pv
  if (active) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int c0 = 16 * (h == 0 ? warp : 7 - warp) + 4 * sb;
#pragma unroll
      for (int r = 0; r < R; r++)
        *reinterpret_cast<uint4 *>(wk + (r * 7 + pt) * 128 + c0) =
            make_uint4(out[h][0][r], out[h][1][r], out[h][2][r], out[h][3][r]);
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < R * 128; idx += blockDim.x) {
    const int r = idx >> 7, c = idx & 127;
    uint32_t w[7];
#pragma unroll
    for (int k = 0; k < 7; k++) w[k] = wk[(r * 7 + k) * 128 + c];
    toom4_interp(w);
#pragma unroll
    for (int k = 0; k < 7; k++) wk[(r * 7 + k) * 128 + c] = w[k];
  }
  __syncthreads();
  // negacyclic fold: coefficient m of the 511-term product is the sum of
  // c_k[m - 64k]; res[m] = full[m] - full[m + 256]
  for (int idx = threadIdx.x; idx < R * 256; idx += blockDim.x) {
    const int r = idx >> 8, m = idx & 255, kk = m >> 6, cc = m & 63;
    const uint32_t *C = wk + r * 7 * 128;
    uint32_t v = C[kk * 128 + cc] - C[(kk + 3) * 128 + cc + 64];
    if (kk >= 1) v += C[(kk - 1) * 128 + cc + 64];
    if (kk <= 2) v -= C[(kk + 4) * 128 + cc];
    res[r * 256 + m] = (uint16_t)v;
  }
}

}  // namespace tmvp
