// diag_keccak.cu — the Keccak-f[1600] permutation rate of this GPU at full
// occupancy: the integer-pipe ceiling of the hash stages.  Every thread keeps
// one register-resident state (the same keccak_f1600 the hash kernels run),
// applies `perms` permutations back to back and stores one word so that the
// work is kept.  As many 64-thread blocks as fit run on every SM at once.
#include <cuda_runtime.h>

#include "keccak.cuh"

namespace tmvp {

__global__ void __launch_bounds__(64) k_diag_keccak(int perms, uint64_t *out) {
  uint64_t A[25];
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
  for (int i = 0; i < 25; i++) A[i] = t * 0x9E3779B97F4A7C15ull + (uint64_t)i;
  for (int p = 0; p < perms; p++) keccak_f1600(A);
  uint64_t x = 0;
#pragma unroll
  for (int i = 0; i < 25; i++) x ^= A[i];
  out[t] = x;
}

// out[0] = permutations per second over the whole GPU, out[1] = resident
// blocks per SM.  `out_words` is caller-provided device scratch of at least
// (SMs x resident blocks x 64) words; the needed count is returned in
// out[2] when it is too small (nothing runs then).
int diag_keccak_rate(int perms, uint64_t *scratch, size_t scratch_words, double *out, cudaStream_t s) {
  if (perms < 1 || perms > (1 << 16) || !out) return (int)cudaErrorInvalidValue;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_diag_keccak, 64, 0)) != cudaSuccess)
    return (int)e;
  const size_t grid = (size_t)nsm * per_sm;
  out[1] = per_sm;
  out[2] = (double)(grid * 64);
  if (!scratch || scratch_words < grid * 64) return (int)cudaErrorInvalidValue;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_diag_keccak<<<(unsigned)grid, 64, 0, s>>>(1, scratch);  // warm-up (module load, clocks)
  cudaEventRecord(a, s);
  k_diag_keccak<<<(unsigned)grid, 64, 0, s>>>(perms, scratch);
  cudaEventRecord(b, s);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return (int)e;
  out[0] = (double)grid * 64 * perms / (ms * 1e-3);
  return 0;
}

}  // namespace tmvp
