// keccak.cuh — Keccak-f[1600] and the FIPS 202 sponges used by the KEM,
// one thread per sponge with the 25-lane state in registers.
//
// Behaviour follows the reference's serial Keccak
// (TMVP_SABLE/src/fips202.cu:68-405 and :535-578, identical to
// TMVP-Saber/SABER-GPU/src/poly.cu:457-797 and :1076-1114).  The reference
// keeps the state in local memory and runs its hash kernels as a single
// block; here every round is unrolled over registers and one thread serves
// one instance of a batch.  Round constants and rotation offsets are derived
// at compile time from the FIPS 202 definitions (rc LFSR, rho walk).
#pragma once
#include <cstdint>

namespace tmvp {

struct KeccakTables {
  uint64_t rc[24];
  int rho[25];
};

__host__ __device__ constexpr KeccakTables make_keccak_tables() {
  KeccakTables t{};
  // FIPS 202 Algorithm 5 (rc) and Algorithm 6 (iota).
  for (int ir = 0; ir < 24; ir++) {
    uint64_t rc = 0;
    for (int j = 0; j <= 6; j++) {
      int tt = (j + 7 * ir) % 255;
      unsigned r = 1;
      for (int i = 1; i <= tt; i++) {
        r <<= 1;
        if (r & 0x100) r ^= 0x171;
      }
      if (r & 1) rc |= (uint64_t)1 << ((1 << j) - 1);
    }
    t.rc[ir] = rc;
  }
  // FIPS 202 Algorithm 2 (rho).
  t.rho[0] = 0;
  int x = 1, y = 0;
  for (int k = 0; k < 24; k++) {
    t.rho[x + 5 * y] = ((k + 1) * (k + 2) / 2) % 64;
    int nx = y, ny = (2 * x + 3 * y) % 5;
    x = nx;
    y = ny;
  }
  return t;
}

__device__ __forceinline__ uint64_t rotl64(uint64_t v, int n) {
  return n == 0 ? v : ((v << n) | (v >> (64 - n)));
}

// Round constants in the constant bank (the round loop is not unrolled, so
// the constant is indexed by the round counter).
__constant__ KeccakTables kKeccak = make_keccak_tables();

// a ^ b ^ c on both 32-bit halves, one three-input LOP3 each.  Theta applies
// C[x-1] ^ rot(C[x+1], 1) to a lane this way instead of first forming that
// term per column and then XORing it into five lanes (one XOR per column
// half fewer per round).
__device__ __forceinline__ uint64_t xor3_64(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("{\n\t.reg .b32 al, ah, bl, bh, cl, ch, dl, dh;\n\t"
      "mov.b64 {al, ah}, %1;\n\tmov.b64 {bl, bh}, %2;\n\tmov.b64 {cl, ch}, %3;\n\t"
      "lop3.b32 dl, al, bl, cl, 0x96;\n\tlop3.b32 dh, ah, bh, ch, 0x96;\n\t"
      "mov.b64 %0, {dl, dh};\n\t}"
      : "=l"(d)
      : "l"(a), "l"(b), "l"(c));
  return d;
}

// One round over a register-resident state (theta, rho+pi, chi, iota).
__device__ __forceinline__ void keccak_round(uint64_t (&A)[25], uint64_t rc) {
  constexpr KeccakTables T = make_keccak_tables();
  uint64_t C[5], E[5], B[25];
#pragma unroll
  for (int x = 0; x < 5; x++) C[x] = A[x] ^ A[x + 5] ^ A[x + 10] ^ A[x + 15] ^ A[x + 20];
#pragma unroll
  for (int x = 0; x < 5; x++) E[x] = rotl64(C[(x + 1) % 5], 1);
#pragma unroll
  for (int x = 0; x < 5; x++)
#pragma unroll
    for (int y = 0; y < 5; y++)
      B[y + 5 * ((2 * x + 3 * y) % 5)] = rotl64(xor3_64(A[x + 5 * y], C[(x + 4) % 5], E[x]), T.rho[x + 5 * y]);
#pragma unroll
  for (int y = 0; y < 5; y++)
#pragma unroll
    for (int x = 0; x < 5; x++)
      A[x + 5 * y] = B[x + 5 * y] ^ (~B[(x + 1) % 5 + 5 * y] & B[(x + 2) % 5 + 5 * y]);
  A[0] ^= rc;
}

// The 24-round permutation.  The loop body is two rounds: a fully unrolled
// permutation (~5k instructions) does not fit the instruction cache and
// stalls every warp on instruction fetch.
__device__ __forceinline__ void keccak_f1600(uint64_t (&A)[25]) {
#pragma unroll 1
  for (int ir = 0; ir < 24; ir += 2) {
    keccak_round(A, kKeccak.rc[ir]);
    keccak_round(A, kKeccak.rc[ir + 1]);
  }
}

__device__ __forceinline__ void keccak_zero(uint64_t (&A)[25]) {
#pragma unroll
  for (int i = 0; i < 25; i++) A[i] = 0;
}

// Absorb `nbytes` (a multiple of 8) of 8-byte-aligned input with rate
// `rate_w` words and the given domain byte, then pad (FIPS 202 pad10*1).
// Leaves the state ready for the first squeeze permutation.
template <int RATE_W>
__device__ __forceinline__ void keccak_absorb_words(uint64_t (&A)[25], const uint64_t *in,
                                                    int nbytes, uint64_t domain) {
  keccak_zero(A);
  int nw = nbytes >> 3;
  while (nw >= RATE_W) {
#pragma unroll
    for (int i = 0; i < RATE_W; i++) A[i] ^= in[i];
    keccak_f1600(A);
    in += RATE_W;
    nw -= RATE_W;
  }
  // tail of nw < RATE_W whole words, then the domain byte in word nw
#pragma unroll
  for (int i = 0; i < RATE_W; i++) {
    if (i < nw) A[i] ^= in[i];
    if (i == nw) A[i] ^= domain;
  }
  A[RATE_W - 1] ^= 0x8000000000000000ull;
}

// SHA3-256 (rate 136 B = 17 words) of nbytes 8-aligned bytes.
__device__ __forceinline__ void sha3_256_words(uint64_t out[4], const uint64_t *in, int nbytes) {
  uint64_t A[25];
  keccak_absorb_words<17>(A, in, nbytes, 0x06);
  keccak_f1600(A);
#pragma unroll
  for (int i = 0; i < 4; i++) out[i] = A[i];
}

// SHA3-512 (rate 72 B = 9 words) of a 64-byte input held in registers.
__device__ __forceinline__ void sha3_512_64(uint64_t out[8], const uint64_t in[8]) {
  uint64_t A[25];
  keccak_zero(A);
#pragma unroll
  for (int i = 0; i < 8; i++) A[i] = in[i];
  A[8] = 0x06ull | 0x8000000000000000ull;
  keccak_f1600(A);
#pragma unroll
  for (int i = 0; i < 8; i++) out[i] = A[i];
}

// SHA3-256 of a 64-byte input held in registers.
__device__ __forceinline__ void sha3_256_64(uint64_t out[4], const uint64_t in[8]) {
  uint64_t A[25];
  keccak_zero(A);
#pragma unroll
  for (int i = 0; i < 8; i++) A[i] = in[i];
  A[8] = 0x06ull;
  A[16] = 0x8000000000000000ull;
  keccak_f1600(A);
#pragma unroll
  for (int i = 0; i < 4; i++) out[i] = A[i];
}

// SHA3-256 of a 32-byte input held in registers.
__device__ __forceinline__ void sha3_256_32(uint64_t out[4], const uint64_t in[4]) {
  uint64_t A[25];
  keccak_zero(A);
#pragma unroll
  for (int i = 0; i < 4; i++) A[i] = in[i];
  A[4] = 0x06ull;
  A[16] = 0x8000000000000000ull;
  keccak_f1600(A);
#pragma unroll
  for (int i = 0; i < 4; i++) out[i] = A[i];
}

// SHAKE-128 (rate 168 B = 21 words) of a 32-byte seed held in registers,
// squeezing `nbytes` (a multiple of 8) to 8-aligned memory `out`.
__device__ __forceinline__ void shake128_32(uint64_t *out, int nbytes, const uint64_t seed[4]) {
  uint64_t A[25];
  keccak_zero(A);
#pragma unroll
  for (int i = 0; i < 4; i++) A[i] = seed[i];
  A[4] = 0x1Full;
  A[20] = 0x8000000000000000ull;
  int nw = nbytes >> 3;
  while (nw > 0) {
    keccak_f1600(A);
    int k = nw < 21 ? nw : 21;
#pragma unroll
    for (int i = 0; i < 21; i++)
      if (i < k) out[i] = A[i];
    out += 21;
    nw -= k;
  }
}

}  // namespace tmvp
