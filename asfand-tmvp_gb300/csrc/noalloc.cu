// noalloc.cu — batched decapsulation that allocates nothing.
//
// Callers that cannot allocate device memory use this entry point. Examples
// are a host application whose GPU memory is carved up by its own pool
// allocator, and a serving process that forbids allocation after start-up so
// its latency stays flat.  Instead of a context workspace it uses one
// fixed array in device global memory, declared below, which every GPU that
// loads the library holds until the process exits.
//
// Limits and behaviour:
//   * at most TMVP_NOALLOC_MAX_BATCH (1024) instances per call; larger n is
//     rejected with TMVP_EINVAL and nothing is launched;
//   * ct, sk and ss must be device memory of the current GPU, 16-byte aligned;
//   * errors found on the GPU (a secret outside a tensor-core form's exact
//     range, a bounded device wait that gave up) cannot be returned by an
//     asynchronous call: the call writes its result code into the caller's
//     `status` word when the stream reaches the call's end;
//   * the first call on a device (and the first after that device's context
//     was replaced, e.g. by cudaDeviceReset) looks up the array's device
//     address with cudaGetSymbolAddress, with that device current; make that
//     first call before any stream capture;
//   * every call uses the same array and the array keeps the previous call's
//     contents, so calls that overlap on the GPU (different streams, or
//     several host threads) race; serialise them on one stream;
//   * the call is asynchronous on `stream` and runs all stages there;
//   * it calls no cudaMalloc, cudaFree or allocating library routine.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/tmvp_kem.h"
#include "cpa_kernels.cuh"
#include "hash_kernels.cuh"
#include "kem_common.cuh"

static_assert(TMVP_NOALLOC_MAX_BATCH == 1024, "scratch sizing below assumes 1024 instances");

namespace {

using namespace tmvp;

constexpr size_t kMaxBatch = TMVP_NOALLOC_MAX_BATCH;
constexpr size_t kAlignNA = 256;
constexpr size_t upna(size_t x) { return (x + kAlignNA - 1) & ~(kAlignNA - 1); }

// Scratch of one call, laid out for the largest parameter set: GenMatrix
// stream 16 * 416 bytes (FireSaber), GenSecret stream 768 bytes (Saber,
// FireSaber).  7.4 MiB for TMVP_NOALLOC_MAX_BATCH = 1024.
constexpr size_t kGmMax = 16 * 416;
constexpr size_t kGsMax = 3 * 256;  // largest GenSecret stream (Saber, FireSaber: 768 bytes)
constexpr size_t kOffErr = 0;
constexpr size_t kOffA = kAlignNA;
constexpr size_t kOffS = kOffA + upna(kMaxBatch * kGmMax);
constexpr size_t kOffM = kOffS + upna(kMaxBatch * kGsMax);
constexpr size_t kOffKr = kOffM + upna(kMaxBatch * 64);
constexpr size_t kOffFail = kOffKr + upna(kMaxBatch * 64);
constexpr size_t kOffHc = kOffFail + upna(kMaxBatch);
constexpr size_t kScratchBytes = kOffHc + upna(kMaxBatch * 32);

}  // namespace

// The scratch array.  In host code this name is only a host-side stand-in;
// kernels receive the device address that scratch_ptr() looks up.
static __device__ __align__(256) uint8_t g_noalloc_scratch[kScratchBytes];

namespace {

// Turns the stages' error bits (1: a secret outside the exact range of a
// tensor-core form, 2: a bounded wait gave up) into a TMVP code for the
// caller, and clears them for the next call.
__global__ void k_noalloc_status(int *bits, int *status) {
  const int w = *bits;
  if (status) *status = (w & 2) ? TMVP_ETIMEOUT : (w ? TMVP_EINVAL : TMVP_OK);
  *bits = 0;
}

constexpr int kMaxDevices = 64;
std::mutex g_na_mu;
uint8_t *g_na_ptr[kMaxDevices] = {};
CUcontext g_na_ctx[kMaxDevices] = {};

typedef CUresult (*ctx_get_current_fn)(CUcontext *);

// The context current on this thread (the device's primary context for
// runtime-API callers), or nullptr when the driver entry point is missing.
CUcontext current_context() {
  static ctx_get_current_fn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    return reinterpret_cast<ctx_get_current_fn>(p);
  }();
  CUcontext c = nullptr;
  if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
  return c;
}

// Device address of g_noalloc_scratch on the current device.  Looked up once
// per device with that device current, and again when the device's context
// changed since (an address from a destroyed context is no longer valid).
// nullptr on failure.
uint8_t *scratch_ptr(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return nullptr;
  const CUcontext ctx = current_context();
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev] || !ctx || ctx != g_na_ctx[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) {
      cudaGetLastError();
      g_na_ptr[dev] = nullptr;
      return nullptr;
    }
    g_na_ptr[dev] = static_cast<uint8_t *>(p);
    g_na_ctx[dev] = ctx;
  }
  return g_na_ptr[dev];
}

bool device_buffer(const void *p, int dev) {
  if (!p || ((uintptr_t)p & 15)) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev;
}

// The device-side address of the caller's status word: device or managed
// memory of `dev`, or host memory mapped into the device's address space.
// nullptr if the GPU cannot write it.
int *status_address(int *status, int dev) {
  if (((uintptr_t)status & 3)) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, status) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if ((at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev)
    return status;
  if (at.type == cudaMemoryTypeHost && at.devicePointer) return static_cast<int *>(at.devicePointer);
  return nullptr;
}

inline unsigned nblocks(size_t threads) { return (unsigned)((threads + 127) / 128); }

}  // namespace

extern "C" int tmvp_kem_dec_batch_noalloc(tmvp_param_set set, size_t n, uint8_t *ss,
                                          const uint8_t *ct, const uint8_t *sk, tmvp_form form,
                                          int *status, void *stream) {
  KemParams P;
  if (!make_params(set, &P)) return TMVP_EINVAL;
  if (n > kMaxBatch) return TMVP_EINVAL;  // beyond the fixed scratch array
  int f = form == TMVP_FORM_AUTO ? kFp8Tcgen05 : (int)form;
  if (!form_valid(f)) return TMVP_EINVAL;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TMVP_ENOTSUP;
  int *status_d = nullptr;
  if (status && !(status_d = status_address(status, dev))) return TMVP_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) {
    if (status_d && cudaMemsetAsync(status_d, 0, sizeof(int), s) != cudaSuccess) return TMVP_EDEVICE;
    return TMVP_OK;
  }
  if (!device_buffer(ss, dev) || !device_buffer(ct, dev) || !device_buffer(sk, dev))
    return TMVP_EINVAL;
  uint8_t *base = scratch_ptr(dev);
  if (!base) return TMVP_EDEVICE;
  int *err = reinterpret_cast<int *>(base + kOffErr);
  uint8_t *a_stream = base + kOffA, *s_stream = base + kOffS, *mbuf = base + kOffM,
          *kr = base + kOffKr, *fail = base + kOffFail, *hc = base + kOffHc;
  // the error bits must start at zero; every other buffer is fully rewritten
  if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) return TMVP_EDEVICE;
  // the Keccak stages take the form a context would give them by default
  const HashForm ff = hash_form_for(2 * n, false, kWarpHashDefault, kPairHashDefault);
  const HashForm fs = hash_form_for(n, true, kWarpHashDefault, kPairHashDefault);
  if (ff == kHashWarp)
    k_dec_front_w<<<warp_blocks(2 * n), kWarpHashBlock, 0, s>>>(P, sk, ct, a_stream, hc, (int)n, 0);
  else if (ff == kHashPair)
    k_dec_front_p<<<pair_blocks(warp_round(2 * n) + 2 * n), kPairHashBlock, 0, s>>>(P, sk, ct, a_stream, hc,
                                                                                    (int)n, 0);
  else
    k_dec_front<<<nblocks(warp_round(n) + n), 128, 0, s>>>(P, sk, ct, a_stream, hc, (int)n, 0);
  CpaArgs a{};
  a.P = P;
  a.n = (int)n;
  a.ct = ct;
  a.sk = sk;
  a.m_out = mbuf;
  a.m_out_stride = 64;
  a.copy_hpk = 1;
  a.err = err;
  if (cpa_launch(f, kDecrypt, a, s) != 0) return TMVP_EDEVICE;
  if (fs == kHashWarp)
    k_dec_g_w<<<warp_blocks(n), kWarpHashBlock, 0, s>>>(P, mbuf, kr, s_stream, (int)n);
  else if (fs == kHashPair)
    k_dec_g_p<<<pair_blocks(2 * n), kPairHashBlock, 0, s>>>(P, mbuf, kr, s_stream, (int)n);
  else
    k_dec_g<<<nblocks(n), 128, 0, s>>>(P, mbuf, kr, s_stream, (int)n);
  CpaArgs b{};
  b.P = P;
  b.n = (int)n;
  b.a_stream = a_stream;
  b.s_stream = s_stream;
  b.pk = sk;
  b.pk_stride = P.sk_bytes;
  b.pk_off = P.indcpa_sk_bytes;
  b.msg = mbuf;
  b.msg_stride = 64;
  b.ct = ct;
  b.fail = fail;
  b.err = err;
  if (cpa_launch(f, kReenc, b, s) != 0) return TMVP_EDEVICE;
  if (fs == kHashWarp)
    k_final_key_w<<<warp_blocks(n), kWarpHashBlock, 0, s>>>(P, ct, hc, kr, fail, sk, (size_t)P.sk_bytes, ss, (int)n);
  else if (fs == kHashPair)
    k_final_key_p<<<pair_blocks(2 * n), kPairHashBlock, 0, s>>>(P, ct, hc, kr, fail, sk, (size_t)P.sk_bytes, ss,
                                                                (int)n);
  else
    k_final_key<<<nblocks(n), 128, 0, s>>>(P, ct, hc, kr, fail, sk, (size_t)P.sk_bytes, ss, (int)n);
  k_noalloc_status<<<1, 1, 0, s>>>(err, status_d);
  return cudaGetLastError() == cudaSuccess ? TMVP_OK : TMVP_EDEVICE;
}
