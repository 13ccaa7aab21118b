// cpa_umma.cuh — the tcgen05 (5th-generation tensor core) engine of the
// FP8 IND-CPA form.
//
// One CTA computes, for its instance, D[256][N] = sum_j H_j x B_j where
//   * H_j is the 256 x 256 matrix of the secret polynomial s_j with the K
//     index reversed: H_j[r][k'] = s_ext[r + k'] (a Hankel matrix), which is
//     the negacyclic Toeplitz matrix T(s_j)[r][c] = s_ext[r - c + 255] with
//     c = 255 - k';
//   * B_j holds N digit columns of the public polynomials of module index j,
//     coefficient c at row k' = 255 - c;
// with tcgen05.mma kind::f8f6f4 (e4m3 x e4m3 -> f32), M = 128 (two halves),
// N = 16 or 32, K = 32 per instruction, A and B read from shared memory and D
// accumulated in tensor memory (TMEM).
//
// Operand layout (K-major, no swizzle): the MMA reads "core matrices" of 8
// rows x 16 bytes, stored as 128 contiguous bytes; the shared-memory
// descriptor gives the byte distance between core matrices adjacent in K
// (leading byte offset, LBO) and in M/N (stride byte offset, SBO).
//   * H_j: the core matrix at 8-row group b and 16-byte K chunk a holds
//     s_ext[8b + 16a + i + e] (row i, byte e), which depends on m = b + 2a
//     only.  So H_j is stored as distinct core matrices at m * 128 bytes and
//     described with SBO = 128 and LBO = 256: the MMA's core matrix (b, a)
//     lands on m = b + 2a.  The per-instance kernel (cpa5i.cuh) reads eight
//     windows of the sequence and needs 46 of them, m = 0..45 (5.75 KB per
//     secret polynomial, kHankelCores5); the persistent kernel
//     (cpa_persist.cuh) keeps the earlier layout of 62 (7.75 KB,
//     kHankelCores) -- either instead of the 64 KB of the dense matrix.
//   * B_j: dense, core (8-column group c, K chunk a) at a * (16 N) + c * 128.
//
// Every product of an e4m3 digit (0..15) and an e4m3 secret (|s| <= 7) is an
// integer of magnitude <= 105, and every sum the MMA forms is an integer of
// magnitude <= 4 * 256 * 105 < 2^17, exact in f32.
#pragma once
#include <cstdint>

#include "kem_common.cuh"

namespace tmvp {

constexpr int kHankelCores = 62;                  // distinct core matrices of H_j
constexpr int kHankelBytes = kHankelCores * 128;  // per secret polynomial (7936 bytes)
constexpr int kUmmaM = 128;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, LBO and SBO in
// 16-byte units, descriptor version 1 (bits 46-48 = 0b001), no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor for kind::f8f6f4: D f32, A and B e4m3, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t umma_idesc_e4m3(int n) {
  return (1u << 4)                      // D format f32
         | (0u << 7) | (0u << 10)       // A, B format e4m3
         | ((uint32_t)(n >> 3) << 17)   // N / 8
         | ((uint32_t)(kUmmaM >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void umma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                        uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// try_wait with a suspend-time hint: the thread sleeps until the phase
// completes or about `ns` nanoseconds pass, instead of spinning.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint32_t mbar, uint32_t parity, uint32_t ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity), "r"(ns)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of an mbarrier: sleeps in 20 us slices and
// gives up after about two seconds (or 2^22 polls), returning false.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  for (uint32_t it = 0; it < (1u << 22); it++) {
    if (mbar_try_wait_sleep(mbar, parity, 20000u)) return true;
    if ((it & 15u) == 15u && global_ns() - t0 > 2000000000ull) return false;
  }
  return false;
}

// 16 consecutive f32 columns of this warp's 32 TMEM lanes.  The load and its
// completion wait are one asm statement, so no use of r[] can be scheduled
// between them.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

// 8 consecutive f32 columns of this warp's 32 TMEM lanes (load and wait in
// one asm statement, as tmem_ld16).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
}

// Byte-wise e4m3 encoding of four digits 0..15 (one per byte).
constexpr uint32_t kE4m3Lo8 = 0x44403800u;  // 3, 2, 1, 0
constexpr uint32_t kE4m3Hi8 = 0x4E4C4A48u;  // 7, 6, 5, 4
__device__ __forceinline__ uint32_t e4m3_digits4(uint32_t d) {
  const uint32_t lo7 = d & 0x07070707u;
  const uint32_t hi = (d >> 3) & 0x01010101u;  // 1 where the digit is 8..15
  // PRMT selector nibbles from the low three bits of each byte
  const uint32_t u = (lo7 | (lo7 >> 4)) & 0x00FF00FFu;
  const uint32_t sel = (u | (u >> 8)) & 0xFFFFu;
  const uint32_t lut = __byte_perm(kE4m3Lo8, kE4m3Hi8, sel);  // e4m3 of 0..7
  const uint32_t big = lo7 | 0x50505050u;                      // e4m3 of 8..15
  const uint32_t m = hi * 0xFFu;
  return (big & m) | (lut & ~m);
}

// Radix-16 digits of a w-bit public coefficient x (results are needed mod
// 2^w): unsigned nibbles, except that a 5-bit top digit t = x >> (w - 5) is
// used as t - 32 when t >= 16.  That changes the product by a multiple of
// 2^w only, and keeps every digit within e4m3's exact integers (|d| <= 16):
// 13-bit coefficients need 3 digits instead of 4, 9-bit ones 2 instead of 3.
__host__ __device__ constexpr int r16_digits(int w) { return w <= 5 ? 1 : 1 + (w - 5 + 3) / 4; }

// e4m3 of four 5-bit top digits t (one per byte), each as the signed value
// t (t < 16) or t - 32 (t >= 16); magnitude 16 encodes as 0x58.
__device__ __forceinline__ uint32_t e4m3_sdigits4(uint32_t t) {
  const uint32_t m = ((t >> 4) & 0x01010101u) * 0xFFu;           // bytes with t >= 16
  const uint32_t mag = (m & (0x20202020u - t)) | (~m & t);       // 32 - t there (1..16), else t
  const uint32_t is16 = (mag >> 4) & 0x01010101u;
  return e4m3_digits4(mag & 0x0F0F0F0Fu) | (is16 * 0x58u) | (m & 0x80808080u);
}

// The encoded sequence s_ext[0..511] of each secret polynomial j < L, from
// its encoded words S (64 per polynomial, byte e of word u = coefficient
// 4u + e): s_ext[d] = -s[d + 1] for d < 255, s[d - 255] for 255 <= d <= 510,
// 0 at 511.  ext: 128 words per polynomial.  NEG negates four encoded bytes.
template <class NEG>
__device__ __forceinline__ void stage_ext(uint32_t *ext, const uint32_t *S, int L, int tid,
                                          int nthreads, NEG neg4f) {
  for (int idx = tid; idx < L * 128; idx += nthreads) {
    const int j = idx >> 7, w = idx & 127;
    const uint32_t *s = S + 64 * j;
    uint32_t v;
    if (w < 63) {
      v = neg4f(__byte_perm(s[w], s[w + 1], 0x4321));
    } else if (w == 63) {
      v = (neg4f(s[63]) >> 8) | (s[0] << 24);
    } else if (w < 127) {
      v = __byte_perm(s[w - 64], s[w - 63], 0x4321);
    } else {
      v = s[63] >> 8;
    }
    ext[idx] = v;
  }
}

// Shared-memory accesses through 32-bit shared-window addresses.
__device__ __forceinline__ uint32_t lds32(uint32_t a) {
  uint32_t v;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ void lds128(uint32_t a, uint32_t &x, uint32_t &y, uint32_t &z, uint32_t &w) {
  asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];" : "=r"(x), "=r"(y), "=r"(z), "=r"(w) : "r"(a));
}
__device__ __forceinline__ void sts64(uint32_t a, uint32_t x, uint32_t y) {
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(a), "r"(x), "r"(y) : "memory");
}
__device__ __forceinline__ void sts128(uint32_t a, uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(x), "r"(y), "r"(z), "r"(w) : "memory");
}

// stage_hankel with compile-time sizes and 32-bit shared addresses (H, ext:
// shared-window byte addresses): the same thread groups, each thread's rows
// unrolled from one load of the ext words they span.  A thread's window
// starts at word q = 2 u0 + par with u0 even, so it loads the 16-byte-aligned
// words from q - par with 128-bit loads (the eight lanes of a row pair share
// them, so a warp's load is one 64-byte wavefront) and takes word i + par by
// a funnel shift.
template <int L, int NT, int CORES>
__device__ __forceinline__ void stage_hankel_ct(uint32_t H, uint32_t ext, int tid) {
  constexpr int PAIRS = NT >> 3;
  constexpr int RUN = (CORES + PAIRS - 1) / PAIRS;  // rows per thread and polynomial
  constexpr int NW = (2 * RUN + 4 + 3) & ~3;         // the 2 RUN + 3 window words, plus one for par
  static_assert(RUN % 2 == 0, "every thread's window starts on a 16-byte boundary");
  static_assert(2 * (CORES - 1) + NW <= 128, "the loads stay inside one polynomial's 512-byte s_ext");
  const int sh = tid & 3, par = (tid >> 2) & 1, u0 = (tid >> 3) * RUN;
  if (u0 >= CORES) return;
  const uint32_t sel = 0x3210u + 0x1111u * (uint32_t)sh;
  const int b = 2 * u0;  // q - par, a multiple of 4
  const int q = b + par;
#pragma unroll
  for (int j = 0; j < L; j++) {
    uint32_t a[NW];
#pragma unroll
    for (int i = 0; i < NW; i += 4) lds128(ext + 512 * j + 4 * (b + i), a[i], a[i + 1], a[i + 2], a[i + 3]);
    uint32_t w[2 * RUN + 3];
#pragma unroll
    for (int i = 0; i < 2 * RUN + 3; i++) w[i] = __funnelshift_rc(a[i], a[i + 1], 32u * (uint32_t)par);
    const uint32_t h = H + (uint32_t)(j * CORES * 128) + 16 * (4 * q + sh);
#pragma unroll
    for (int r = 0; r < RUN; r++)
      if (CORES % PAIRS == 0 || u0 + r < CORES)
        sts128(h + 128 * r, __byte_perm(w[2 * r], w[2 * r + 1], sel), __byte_perm(w[2 * r + 1], w[2 * r + 2], sel),
               __byte_perm(w[2 * r + 2], w[2 * r + 3], sel), __byte_perm(w[2 * r + 3], w[2 * r + 4], sel));
  }
}

// The first `cores` Hankel core matrices of every j < L (H: cores * 128 bytes
// per polynomial):
// row i of core m is s_ext[8m + i .. 8m + i + 15], so row x = 8m + i sits at
// byte 16x.  Rows x = 4q + sh (q < 2 cores) with the same byte shift sh are
// windows of consecutive words.  Thread group g (four threads, sh = 0..3)
// makes the rows q = 2u + (g & 1) for a run of u, from a window of ext words
// that slides by two words per row; the eight threads of two neighbouring
// groups store eight consecutive rows (128 contiguous bytes) at a time.
__device__ __forceinline__ void stage_hankel(uint8_t *H, const uint32_t *ext, int L, int tid,
                                             int nthreads, int cores = kHankelCores) {
  const int pairs = nthreads >> 3;                 // group pairs
  const int run = (cores + pairs - 1) / pairs;      // rows per thread and polynomial
  const int sh = tid & 3, par = (tid >> 2) & 1, u0 = (tid >> 3) * run;
  const uint32_t sel = (uint32_t)(sh | ((sh + 1) << 4) | ((sh + 2) << 8) | ((sh + 3) << 12));
  if (u0 >= cores) return;
  for (int j = 0; j < L; j++) {
    const uint32_t *e = ext + 128 * j;
    uint8_t *hj = H + (size_t)j * cores * 128;
    int q = 2 * u0 + par;
    uint32_t w0 = e[q], w1 = e[q + 1], w2 = e[q + 2], w3 = e[q + 3], w4 = e[q + 4];
    for (int u = u0; u < u0 + run && u < cores; u++, q += 2) {
      *reinterpret_cast<uint4 *>(hj + 16 * (4 * q + sh)) =
          make_uint4(__byte_perm(w0, w1, sel), __byte_perm(w1, w2, sel), __byte_perm(w2, w3, sel),
                     __byte_perm(w3, w4, sel));
      if (u + 1 < u0 + run && u + 1 < cores) {
        w0 = w2; w1 = w3; w2 = w4;
        w3 = e[q + 5];
        w4 = e[q + 6];
      }
    }
  }
}

}  // namespace tmvp
