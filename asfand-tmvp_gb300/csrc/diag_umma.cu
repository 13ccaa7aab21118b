// diag_umma.cu — tensor-core issue cost of the two exact kinds the IND-CPA
// kernels could use: tcgen05.mma kind::f8f6f4 (e4m3 x e4m3, K = 32) and
// kind::f16 (f16 x f16, K = 16).  Both read 32-byte K rows, so the same
// shared-memory descriptors serve them; one instruction of either kind does
// 128 x N x K multiply-adds.  Each CTA issues `iters` MMAs back to back into
// its own tensor memory (M = 128, operands zero), commits them to an
// mbarrier and times issue-to-completion with clock64; ctas_per_sm CTAs run
// on every SM at once.  Waits are bounded.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "cpa_umma.cuh"

namespace tmvp {

__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// A: 16 row groups x 2 K cores (LBO = 2048 between the K cores, SBO = 128
// between row groups); B: N / 8 row groups, the same way.
constexpr int kDiagA = 4096, kDiagBMax = 256 * 32;

__global__ void __launch_bounds__(128) k_diag_umma(int kind, int n, int iters, long long *cycles, int *err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int bbytes = n * 32;
  uint32_t *w = reinterpret_cast<uint32_t *>(sm);
  for (int i = tid; i < (kDiagA + bbytes) / 4; i += blockDim.x) w[i] = 0u;
  const uint32_t mbar = smem_u32(sm + kDiagA + kDiagBMax);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kDiagA + kDiagBMax + 16);
  const uint32_t ncols = n < 32 ? 32u : (uint32_t)n;
  if (warp == 0) tmem_alloc(smem_u32(tmem_slot), ncols);
  if (tid == 0) {
    mbar_init(mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(tmem_slot);
  bool ok = true;
  if (tid == 0) {
    const uint64_t ad = umma_desc(smem_u32(sm), 2048, 128);
    const uint64_t bd = umma_desc(smem_u32(sm + kDiagA), (uint32_t)(n / 8) * 128, 128);
    // D f32, A and B format 0 (e4m3 for kind::f8f6f4, f16 for kind::f16), K-major
    const uint32_t idesc = (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    const long long t0 = clock64();
    if (kind == 0)
      for (int i = 0; i < iters; i++) umma_f8(tmem, ad, bd, idesc, i > 0);
    else
      for (int i = 0; i < iters; i++) umma_f16(tmem, ad, bd, idesc, i > 0);
    umma_commit(mbar);
    ok = mbar_wait_bounded(mbar, 0);
    const long long t1 = clock64();
    cycles[blockIdx.x] = ok ? t1 - t0 : -1;
    if (!ok && err) atomicOr(err, 2);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

// Median cycles from first issue to completion per MMA over all CTAs
// (out[0]), and that divided by ctas_per_sm, the SM's cycles per MMA when
// that many CTAs issue at once (out[1]).
int diag_umma_rate(int kind, int n, int ctas_per_sm, int iters, int *err, double *out, cudaStream_t s) {
  if ((kind != 0 && kind != 1) || n < 16 || n > 256 || (n & (n - 1)) || ctas_per_sm < 1 ||
      ctas_per_sm * std::max(32, n) > 512 || iters < 1 || iters > (1 << 20) || !out)
    return (int)cudaErrorInvalidValue;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int grid = nsm * ctas_per_sm;
  const int smem = kDiagA + kDiagBMax + 32;
  cudaError_t e = cudaFuncSetAttribute(k_diag_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return (int)e;
  long long *d = nullptr;
  if ((e = cudaMalloc(&d, grid * sizeof(long long))) != cudaSuccess) {
    cudaGetLastError();
    return (int)e;
  }
  k_diag_umma<<<grid, 128, smem, s>>>(kind, n, iters, d, err);
  std::vector<long long> h(grid);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d, grid * sizeof(long long), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d);
  if (e != cudaSuccess) return (int)e;
  std::sort(h.begin(), h.end());
  if (h.front() < 0) return (int)cudaErrorLaunchTimeout;
  out[0] = (double)h[grid / 2] / iters;
  out[1] = out[0] / ctas_per_sm;
  return 0;
}

}  // namespace tmvp
