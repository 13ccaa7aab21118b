/*
 * tmvp_oracle.h — CPU oracle for the batched Saber/Sable KEM path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * serial algorithms (Keccak/SHA3/SHAKE-128, CBD, GenMatrix, bit packing,
 * rounding, negacyclic multiplication, IND-CPA and FO KEM).  Only the tests,
 * the smoke check and the CPU-baseline leg of the benchmark may load it, and
 * only as the checker.  The product path (the CUDA library) never calls it.
 *
 * Parity pin: the restatement is checked against the reference's own test
 * vectors (TMVP-Saber/SABER-GPU/include/tv.h, TMVP_SABLE/include/tv.h) and
 * against a host build of the reference's own kernels (oracle/ref_build).
 */
#ifndef TMVP_ORACLE_H
#define TMVP_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parameter set ids; identical numbering to the CUDA library's tmvp_param_set. */
enum {
  ORC_LIGHTSABER = 0,
  ORC_SABER = 1,
  ORC_FIRESABER = 2,
  ORC_LIGHTSABLE = 3,
  ORC_SABLE = 4,
  ORC_FIRESABLE = 5,
  ORC_NSETS = 6
};

typedef struct {
  int l;            /* module rank                                  */
  int eq, ep, et;   /* log2 of q, p, T                              */
  int mu;           /* CBD parameter                                */
  int sable;        /* 1: 2-bit secret packing, secrets masked mod q */
  int polybytes;    /* eq*256/8                                     */
  int polyvecbytes; /* l*polybytes                                  */
  int polycompbytes;/* ep*256/8                                     */
  int scalebytes;   /* et*256/8                                     */
  int coinbytes;    /* mu*256/8 (per polynomial)                    */
  int pk_bytes;     /* l*polycompbytes + 32                         */
  int indcpa_sk_bytes;
  int sk_bytes;     /* indcpa_sk + pk + 32 + 32                     */
  int ct_bytes;     /* l*polycompbytes + scalebytes                 */
  int h1, h2;
} orc_params;

/* Returns 0 and fills *p for a valid set id, -1 otherwise. */
int orc_get_params(int set, orc_params *p);

/* Hashes (FIPS 202). */
void orc_sha3_256(uint8_t out[32], const uint8_t *in, size_t inlen);
void orc_sha3_512(uint8_t out[64], const uint8_t *in, size_t inlen);
void orc_shake128(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen);
void orc_keccakf1600(uint64_t st[25]);

/* Sampling / expansion. Coefficients are returned as uint16 mod 2^16. */
void orc_gen_matrix(int set, uint16_t *A /*[l][l][256]*/, const uint8_t seed[32]);
void orc_gen_secret(int set, uint16_t *s /*[l][256]*/, const uint8_t seed[32]);
void orc_cbd(int mu, uint16_t s[256], const uint8_t *buf);

/* Little-endian bit-stream packing of n w-bit values (w <= 16). */
void orc_pack_bits(uint8_t *out, const uint16_t *in, int n, int w);
void orc_unpack_bits(uint16_t *out, const uint8_t *in, int n, int w);

/* Negacyclic products in Z_{2^16}[x]/(x^256+1). */
void orc_polmul_schoolbook(uint16_t r[256], const uint16_t a[256], const uint16_t b[256]);
void orc_polmul_tmvp2(uint16_t r[256], const uint16_t a[256], const uint16_t b[256]);
void orc_polmul_toom4(uint16_t r[256], const uint16_t a[256], const uint16_t b[256]);
/* toom4k: Toom-Cook 4-way over 16-bit Karatsuba products; right mod 2^13 only. */
void orc_polmul_toom4k(uint16_t r[256], const uint16_t a[256], const uint16_t b[256]);

/* Multiplication used by the IND-CPA / KEM functions (default schoolbook).
 * Returns 0, or -1 for an unknown id.  Not thread-safe: set it before a batch. */
enum { ORC_POLMUL_SCHOOLBOOK = 0, ORC_POLMUL_TOOM4K = 1 };
int orc_set_polmul(int which);

/* Raw matrix-vector product: out[i] = sum_j A[i][j]*s[j] (transpose=0) or
 * sum_j A[j][i]*s[j] (transpose=1), reduced mod 2^eq.  s is int8 per
 * coefficient (CBD secrets).  n instances, contiguous. */
void orc_matvec_batch(size_t n, int l, int eq, int transpose, uint16_t *out,
                      const uint16_t *A, const int8_t *s, int nthreads);

/* IND-CPA. */
void orc_indcpa_keypair(int set, uint8_t *pk, uint8_t *sk_indcpa,
                        const uint8_t seed_a[32], const uint8_t seed_s[32]);
void orc_indcpa_enc(int set, uint8_t *ct, const uint8_t m[32],
                    const uint8_t noiseseed[32], const uint8_t *pk);
void orc_indcpa_dec(int set, uint8_t m[32], const uint8_t *sk_indcpa,
                    const uint8_t *ct);

/* FO KEM, derandomised.  keypair coins: seed_A(32) | seed_s(32) | z(32).
 * enc coins: 32 bytes (hashed into m).  dec returns 0 if the re-encryption
 * matched and 1 if implicit rejection was taken. */
void orc_kem_keypair(int set, uint8_t *pk, uint8_t *sk, const uint8_t coins[96]);
void orc_kem_enc(int set, uint8_t *ct, uint8_t ss[32], const uint8_t *pk,
                 const uint8_t coins[32]);
int orc_kem_dec(int set, uint8_t ss[32], const uint8_t *ct, const uint8_t *sk);

/* Batched versions over contiguous [n][bytes] arrays, split over nthreads
 * POSIX threads (nthreads <= 0: one thread). */
void orc_kem_keypair_batch(int set, size_t n, uint8_t *pk, uint8_t *sk,
                           const uint8_t *coins, int nthreads);
void orc_kem_enc_batch(int set, size_t n, uint8_t *ct, uint8_t *ss,
                       const uint8_t *pk, const uint8_t *coins, int nthreads);
void orc_kem_dec_batch(int set, size_t n, uint8_t *ss, const uint8_t *ct,
                       const uint8_t *sk, uint8_t *fail, int nthreads);

/* Single-instance latency: `iters` calls of keypair (op 0), encapsulation
 * (1) or decapsulation (2) on one thread, ns[i] = call i's wall time.
 * Returns 0; -1 for a bad argument; -2 if a decapsulation did not match. */
int orc_kem_latency(int set, int op, int iters, double *ns);

#ifdef __cplusplus
}
#endif
#endif
