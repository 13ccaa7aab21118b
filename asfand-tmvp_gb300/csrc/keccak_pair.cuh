// keccak_pair.cuh — Keccak-f[1600] and FIPS 202 sponges with two threads per
// sponge: thread `me` = lane & 1 of an adjacent pair holds the low (0) or
// high (1) 32-bit halves of all 25 state lanes.
//
// The round is keccak_round (keccak.cuh) on halves.  Theta's parities, its
// application and chi are bitwise, so each thread does them on its own
// halves; a 64-bit rotation needs the partner's half of the same lane (one
// shfl.xor) and one funnel shift, and the expression is the same in both
// threads: for an offset r < 32 the new half is the top word of
// (own : partner) << r, for r >= 32 of (partner : own) << (r - 32).  A
// thread issues ~90 integer instructions and 29 shuffles a round, so a pair
// costs the integer pipe what one thread-per-sponge state does, while a warp
// carries 16 sponges instead of 32: twice the warps for a batch, and each
// sponge's permutation about 1.45x faster when the warps do not fill the
// pipe.  Inputs and outputs stay in their byte order (a thread loads and
// stores the 4-byte halves of each 8-byte word).
//
// Round constants and rotation offsets follow FIPS 202 (make_keccak_tables);
// the round is the reference's KeccakF1600_StatePermute
// (TMVP_SABLE/src/fips202.cu:68-334) regrouped for halves.
#pragma once
#include <cstdint>

#include "keccak.cuh"

namespace tmvp {

struct KeccakHalves {
  uint32_t rc[24][2];  // [round][0: low half, 1: high half]
};

__host__ __device__ constexpr KeccakHalves make_keccak_halves() {
  KeccakHalves h{};
  const KeccakTables t = make_keccak_tables();
  for (int i = 0; i < 24; i++) {
    h.rc[i][0] = (uint32_t)t.rc[i];
    h.rc[i][1] = (uint32_t)(t.rc[i] >> 32);
  }
  return h;
}

__constant__ KeccakHalves kKeccakHalves = make_keccak_halves();

__device__ __forceinline__ uint32_t pair_xor3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

// One round on this thread's halves; rc_half is this thread's half of the
// round constant.  Every lane of the warp calls it together.
__device__ __forceinline__ void pair_keccak_round(uint32_t (&w)[25], uint32_t rc_half) {
  constexpr KeccakTables T = make_keccak_tables();
  constexpr unsigned F = 0xFFFFFFFFu;
  uint32_t C[5], E[5], B[25];
#pragma unroll
  for (int x = 0; x < 5; x++) C[x] = pair_xor3(pair_xor3(w[x], w[x + 5], w[x + 10]), w[x + 15], w[x + 20]);
#pragma unroll
  for (int x = 0; x < 5; x++) {
    const uint32_t own = C[(x + 1) % 5], par = __shfl_xor_sync(F, own, 1);
    E[x] = __funnelshift_l(par, own, 1);  // rot(C[x+1], 1)
  }
#pragma unroll
  for (int x = 0; x < 5; x++)
#pragma unroll
    for (int y = 0; y < 5; y++) {
      const int i = x + 5 * y, r = T.rho[i];
      const uint32_t a = pair_xor3(w[i], C[(x + 4) % 5], E[x]);
      uint32_t b = a;
      if (r != 0) {
        const uint32_t par = __shfl_xor_sync(F, a, 1);
        b = r < 32 ? __funnelshift_l(par, a, r) : __funnelshift_l(a, par, r - 32);
      }
      B[y + 5 * ((2 * x + 3 * y) % 5)] = b;
    }
#pragma unroll
  for (int y = 0; y < 5; y++)
#pragma unroll
    for (int x = 0; x < 5; x++)
      w[x + 5 * y] = B[x + 5 * y] ^ (~B[(x + 1) % 5 + 5 * y] & B[(x + 2) % 5 + 5 * y]);
  w[0] ^= rc_half;
}

// The 24-round permutation, two rounds per loop iteration (as keccak_f1600).
__device__ __forceinline__ void pair_keccak_f1600(uint32_t (&w)[25], int me) {
#pragma unroll 1
  for (int ir = 0; ir < 24; ir += 2) {
    pair_keccak_round(w, kKeccakHalves.rc[ir][me]);
    pair_keccak_round(w, kKeccakHalves.rc[ir + 1][me]);
  }
}

__device__ __forceinline__ void pair_zero(uint32_t (&w)[25]) {
#pragma unroll
  for (int i = 0; i < 25; i++) w[i] = 0;
}

// This thread's half of a 64-bit constant (domain bytes, padding).
__device__ __forceinline__ uint32_t pair_half(uint64_t v, int me) { return me ? (uint32_t)(v >> 32) : (uint32_t)v; }

// Absorb nbytes (a multiple of 8) of 8-byte-aligned input at rate RATE_W
// words with the domain byte, then pad10*1; the state is left ready for the
// first squeeze permutation.
template <int RATE_W>
__device__ __forceinline__ void pair_absorb_words(uint32_t (&w)[25], int me, const uint8_t *in, int nbytes,
                                                  uint64_t domain) {
  const uint32_t *in32 = reinterpret_cast<const uint32_t *>(in) + me;
  pair_zero(w);
  int nw = nbytes >> 3;
  while (nw >= RATE_W) {
#pragma unroll
    for (int i = 0; i < RATE_W; i++) w[i] ^= in32[2 * i];
    pair_keccak_f1600(w, me);
    in32 += 2 * RATE_W;
    nw -= RATE_W;
  }
  const uint32_t dom = pair_half(domain, me);
#pragma unroll
  for (int i = 0; i < RATE_W; i++) {
    if (i < nw) w[i] ^= in32[2 * i];
    if (i == nw) w[i] ^= dom;
  }
  w[RATE_W - 1] ^= pair_half(0x8000000000000000ull, me);
}

// SHA3-256 / SHA3-512 of a message of nw < rate words whose halves this
// thread holds (m[0..nw-1]): the first `outw` output words' halves.
template <int RATE_W>
__device__ __forceinline__ void pair_sha3_lanes(int me, const uint32_t *m, int nw, uint32_t *out, int outw) {
  uint32_t w[25];
  pair_zero(w);
#pragma unroll
  for (int i = 0; i < RATE_W; i++)
    if (i < nw) w[i] = m[i];
  const uint32_t dom = pair_half(0x06ull, me);
#pragma unroll
  for (int i = 0; i < RATE_W; i++)
    if (i == nw) w[i] ^= dom;
  w[RATE_W - 1] ^= pair_half(0x8000000000000000ull, me);
  pair_keccak_f1600(w, me);
#pragma unroll
  for (int i = 0; i < 8; i++)
    if (i < outw) out[i] = w[i];
}

// SHA3-256 of nbytes (a multiple of 8) at in: this thread's halves of the
// four digest words.
__device__ __forceinline__ void pair_sha3_256_mem(int me, const uint8_t *in, int nbytes, uint32_t (&h)[4]) {
  uint32_t w[25];
  pair_absorb_words<17>(w, me, in, nbytes, 0x06);
  pair_keccak_f1600(w, me);
#pragma unroll
  for (int i = 0; i < 4; i++) h[i] = w[i];
}

}  // namespace tmvp
