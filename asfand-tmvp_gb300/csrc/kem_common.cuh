// kem_common.cuh — parameter descriptors and small helpers shared by the
// host API and the kernels of libtmvpkem.
//
// Parameter sets follow TMVP-Saber/SABER-GPU/include/params.h:1-50 (Saber
// family, L = 2/3/4) and TMVP_SABLE/include/SABLE_params.h:1-73 (Sable family,
// Saber_type 1/2/3).
#pragma once
#include <cstddef>
#include <cstdint>

namespace tmvp {

constexpr int kN = 256;  // ring degree
constexpr int kSeedBytes = 32;
constexpr int kKeyBytes = 32;

// Descriptor passed by value to every kernel (lives in the kernel parameter
// constant bank).
struct KemParams {
  int set;
  int l;             // module rank
  int eq, ep, et;    // log2 q, log2 p, log2 T
  int mu;            // CBD parameter
  int sable;         // 1: 2-bit secret-key packing, GenSecret masks mod q
  int polybytes;     // eq * 32
  int polycompbytes; // ep * 32
  int scalebytes;    // et * 32
  int coinbytes;     // mu * 32 (one polynomial)
  int pk_bytes;      // l * polycompbytes + 32
  int indcpa_sk_bytes;
  int sk_bytes;
  int ct_bytes;
  int h1, h2;
  int gm_bytes;      // GenMatrix stream: l * l * polybytes
  int gs_bytes;      // GenSecret stream: l * coinbytes
};

inline bool make_params(int set, KemParams *p) {
  static const int tab[6][6] = {
      {2, 13, 10, 3, 10, 0},  // LightSaber
      {3, 13, 10, 4, 8, 0},   // Saber
      {4, 13, 10, 6, 6, 0},   // FireSaber
      {2, 11, 9, 3, 2, 1},    // Sable, Saber_type 1
      {3, 11, 9, 5, 2, 1},    // Sable, Saber_type 2
      {4, 11, 10, 3, 2, 1},   // Sable, Saber_type 3
  };
  if (set < 0 || set > 5) return false;
  KemParams q{};
  q.set = set;
  q.l = tab[set][0];
  q.eq = tab[set][1];
  q.ep = tab[set][2];
  q.et = tab[set][3];
  q.mu = tab[set][4];
  q.sable = tab[set][5];
  q.polybytes = q.eq * 32;
  q.polycompbytes = q.ep * 32;
  q.scalebytes = q.et * 32;
  q.coinbytes = q.mu * 32;
  q.pk_bytes = q.l * q.polycompbytes + kSeedBytes;
  q.indcpa_sk_bytes = q.sable ? q.l * 64 : q.l * q.polybytes;
  q.sk_bytes = q.indcpa_sk_bytes + q.pk_bytes + 32 + 32;
  q.ct_bytes = q.l * q.polycompbytes + q.scalebytes;
  // SABER poly.cu:15-16, SABLE pack.cu:15-16
  q.h1 = 1 << (q.eq - q.ep - 1);
  q.h2 = (1 << (q.ep - 2)) - (1 << (q.ep - q.et - 1)) + (1 << (q.eq - q.ep - 1));
  q.gm_bytes = q.l * q.l * q.polybytes;
  q.gs_bytes = q.l * q.coinbytes;
  *p = q;
  return true;
}

// Polynomial-multiplication forms (same numbering as tmvp_form).
enum Form : int {
  kCudaCore = 0,
  kInt8TC = 1,
  kFp8TC = 2,
  kAuto = 3,
  kSchoolbook = 4,
  kFp8Tcgen05 = 5,
  kDp2a = 6,
  kToomCook = 7
};

// A form a kernel exists for (kAuto is resolved before launch).
__host__ __device__ constexpr bool form_valid(int f) {
  return f == kCudaCore || f == kInt8TC || f == kFp8TC || f == kSchoolbook || f == kFp8Tcgen05 ||
         f == kDp2a || f == kToomCook;
}

// Little-endian bit-stream field read from a byte array: bits
// [bit, bit + w), w <= 16.  Reads up to 4 bytes starting at bit / 8; callers
// keep 3 bytes of slack after the stream.
__host__ __device__ __forceinline__ uint32_t get_bits(const uint8_t *p, int bit, int w) {
  const uint8_t *q = p + (bit >> 3);
  uint32_t v = (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16);
  return (v >> (bit & 7)) & ((1u << w) - 1u);
}

}  // namespace tmvp
