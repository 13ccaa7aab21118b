// keccak_warp.cuh — Keccak-f[1600] and FIPS 202 sponges with one warp per
// sponge: lane i < 25 of the warp holds state lane i = x + 5y as two 32-bit
// halves, and the round exchanges lanes by warp shuffles.
//
// This is the latency form.  One thread per sponge (keccak.cuh) issues ~180
// integer instructions per round through its warp's share of the integer
// pipe, ~4.7 us per permutation however few sponges run; here a round is 18
// shuffles and ~16 integer instructions per lane, ~2.1 us per permutation
// while the GPU is far from full.  It issues ~5x the instructions per
// permutation, so larger launches take two threads per sponge
// (keccak_pair.cuh) or one.
//
// The round is the same theta / rho / pi / chi / iota as keccak_round (FIPS
// 202 Algorithms 1-6; the reference's KeccakF1600_StatePermute,
// TMVP_SABLE/src/fips202.cu:68-334), regrouped for lanes: theta's column
// parities by shuffles down the column, rho as a per-lane funnel-shift pair
// (the halves swapped at the source when the offset is 32 or more), and pi
// folded into chi: each lane fetches its three chi inputs straight from the
// lanes that pi moves there.  Lanes 25-31 shadow lanes 0-6 so every shuffle
// source is a live lane; their results are never stored.
#pragma once
#include <cstdint>

#include "keccak.cuh"

namespace tmvp {

struct WarpKeccakLane {
  int col[4];        // the other four lanes of this lane's column
  int left, right;   // lanes (x-1, y) and (x+1, y)
  int chi[3];        // pi sources of (x, y), (x+1, y), (x+2, y)
  int rot;           // rho offset mod 32
  bool swap;         // rho offset >= 32
  uint32_t iota;     // all ones on lane 0
};

__device__ __forceinline__ WarpKeccakLane warp_keccak_lane(int lane) {
  constexpr KeccakTables T = make_keccak_tables();
  const int i = lane < 25 ? lane : lane - 25;
  const int x = i % 5, y = i / 5;
  WarpKeccakLane L;
#pragma unroll
  for (int k = 1; k <= 4; k++) L.col[k - 1] = x + 5 * ((y + k) % 5);
  L.left = (x + 4) % 5 + 5 * y;
  L.right = (x + 1) % 5 + 5 * y;
  // pi: B[X + 5Y] = rot(A[x + 5y]) with X = y, Y = 2x + 3y, so position
  // (X, Y) takes lane ((3Y + X) mod 5) + 5X
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int X = (x + k) % 5;
    L.chi[k] = (3 * y + X) % 5 + 5 * X;
  }
  int r = 0;
#pragma unroll
  for (int j = 0; j < 25; j++)
    if (j == i) r = T.rho[j];
  L.rot = r & 31;
  L.swap = r >= 32;
  L.iota = lane == 0 ? 0xFFFFFFFFu : 0u;
  return L;
}

__device__ __forceinline__ uint32_t lop3_xor3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

// One round; rc is the round constant, applied on lane 0 only.
__device__ __forceinline__ void warp_keccak_round(uint32_t &lo, uint32_t &hi, const WarpKeccakLane &L,
                                                  uint64_t rc) {
  constexpr unsigned F = 0xFFFFFFFFu;
  // theta: column parity C[x], then D = C[x-1] ^ rot(C[x+1], 1)
  uint32_t c0 = __shfl_sync(F, lo, L.col[0]), c1 = __shfl_sync(F, lo, L.col[1]);
  uint32_t c2 = __shfl_sync(F, lo, L.col[2]), c3 = __shfl_sync(F, lo, L.col[3]);
  uint32_t d0 = __shfl_sync(F, hi, L.col[0]), d1 = __shfl_sync(F, hi, L.col[1]);
  uint32_t d2 = __shfl_sync(F, hi, L.col[2]), d3 = __shfl_sync(F, hi, L.col[3]);
  const uint32_t cl = lop3_xor3(lop3_xor3(lo, c0, c1), c2, c3);
  const uint32_t ch = lop3_xor3(lop3_xor3(hi, d0, d1), d2, d3);
  const uint32_t ml = __shfl_sync(F, cl, L.left), mh = __shfl_sync(F, ch, L.left);
  const uint32_t pl = __shfl_sync(F, cl, L.right), ph = __shfl_sync(F, ch, L.right);
  const uint32_t el = __funnelshift_l(ph, pl, 1), eh = __funnelshift_l(pl, ph, 1);
  const uint32_t al = lop3_xor3(lo, ml, el), ah = lop3_xor3(hi, mh, eh);
  // rho: P = high word, Q = low word of rot(a, offset mod 32); offsets of 32
  // or more swap them
  const uint32_t P = __funnelshift_l(al, ah, L.rot), Q = __funnelshift_l(ah, al, L.rot);
  const uint32_t bl = L.swap ? P : Q, bh = L.swap ? Q : P;
  // pi + chi: A[x, y] = B[x, y] ^ (~B[x+1, y] & B[x+2, y])
  const uint32_t b0l = __shfl_sync(F, bl, L.chi[0]), b0h = __shfl_sync(F, bh, L.chi[0]);
  const uint32_t b1l = __shfl_sync(F, bl, L.chi[1]), b1h = __shfl_sync(F, bh, L.chi[1]);
  const uint32_t b2l = __shfl_sync(F, bl, L.chi[2]), b2h = __shfl_sync(F, bh, L.chi[2]);
  lo = (b0l ^ (~b1l & b2l)) ^ ((uint32_t)rc & L.iota);
  hi = (b0h ^ (~b1h & b2h)) ^ ((uint32_t)(rc >> 32) & L.iota);
}

__device__ __forceinline__ void warp_keccak_f1600(uint32_t &lo, uint32_t &hi, const WarpKeccakLane &L) {
  constexpr KeccakTables T = make_keccak_tables();
#pragma unroll
  for (int ir = 0; ir < 24; ir++) warp_keccak_round(lo, hi, L, T.rc[ir]);
}

// Sponge helpers.  `lane` is the caller's lane in the warp; the state lives
// in (lo, hi) of lanes 0..24.  All lanes of the warp call them together.

__device__ __forceinline__ uint64_t warp_lane_word(uint32_t lo, uint32_t hi) {
  return ((uint64_t)hi << 32) | lo;
}

__device__ __forceinline__ void warp_xor_word(uint32_t &lo, uint32_t &hi, uint64_t w) {
  lo ^= (uint32_t)w;
  hi ^= (uint32_t)(w >> 32);
}

// Absorb nbytes (a multiple of 8) from 8-byte-aligned global memory at rate
// RATE_W words with the given domain byte, then pad10*1; the state starts at
// zero and is left ready for the first squeeze permutation.
template <int RATE_W>
__device__ __forceinline__ void warp_absorb_words(uint32_t &lo, uint32_t &hi, const WarpKeccakLane &L, int lane,
                                                  const uint64_t *in, int nbytes, uint64_t domain) {
  lo = hi = 0;
  int nw = nbytes >> 3;
  while (nw >= RATE_W) {
    if (lane < RATE_W) warp_xor_word(lo, hi, in[lane]);
    warp_keccak_f1600(lo, hi, L);
    in += RATE_W;
    nw -= RATE_W;
  }
  if (lane < nw) warp_xor_word(lo, hi, in[lane]);
  if (lane == nw) warp_xor_word(lo, hi, domain);
  if (lane == RATE_W - 1) hi ^= 0x80000000u;
}

// Absorb a short message of nw < RATE_W words held one per lane (lane k < nw
// holds word k in w), with the domain byte and padding.
template <int RATE_W>
__device__ __forceinline__ void warp_absorb_lanes(uint32_t &lo, uint32_t &hi, int lane, uint64_t w, int nw,
                                                  uint64_t domain) {
  lo = hi = 0;
  if (lane < nw) warp_xor_word(lo, hi, w);
  if (lane == nw) warp_xor_word(lo, hi, domain);
  if (lane == RATE_W - 1) hi ^= 0x80000000u;
}

// Squeeze nbytes (a multiple of 8) of SHAKE-128 (rate 21 words) to
// 8-byte-aligned global memory, the state already absorbed and padded.
__device__ __forceinline__ void warp_shake128_squeeze(uint32_t &lo, uint32_t &hi, const WarpKeccakLane &L,
                                                      int lane, uint64_t *out, int nbytes) {
  int nw = nbytes >> 3;
  while (nw > 0) {
    warp_keccak_f1600(lo, hi, L);
    const int k = nw < 21 ? nw : 21;
    if (lane < k) out[lane] = warp_lane_word(lo, hi);
    out += 21;
    nw -= k;
  }
}

}  // namespace tmvp
