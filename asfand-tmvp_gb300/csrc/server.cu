// server.cu — request-serving loop: device-resident keys, continuous
// batching over several in-flight batch slots, memory admission, latency
// statistics, and a seeded Poisson load generator.  No counterpart in the
// reference, whose host API runs one fixed batch per call
// (cuda_kernel.cu:25-479).
//
// Threads:
//   * callers submit requests (zero-copy: the request keeps the caller's in /
//     out pointers) into one FIFO per (parameter set, op);
//   * the scheduler turns the queue whose head waited longest into a batch as
//     soon as a slot is free AND the device arena has room: the batch takes
//     as many requests (up to max_batch) as its block of the arena can hold,
//     for its own parameter set and operation; the block carries the batch's
//     inputs, outputs, gathered keys and matrices and the KEM workspace.  It
//     gathers the inputs into the slot's pinned buffer, copies them to the
//     device, gathers the keys from the device key table by index, launches
//     the batched KEM on the slot's stream, queues the copy of the outputs back
//     and records an event;
//   * the completer waits for slot events in launch order, scatters the
//     outputs to the callers' buffers, records latencies, returns the block to
//     the arena and frees the slot.
// While one slot's batch runs, requests that arrive meanwhile are batched into
// the next free slot, so batches overlap on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_set>
#include <vector>

#include "../../include/tmvp_kem.h"
#include "kem_common.cuh"

namespace tmvp {
size_t kem_ws_bytes(int op, const KemParams &P, size_t n);
int ctx_attach_workspace(tmvp_ctx *c, uint8_t *ws, size_t bytes);
}  // namespace tmvp

namespace {

using Clock = std::chrono::steady_clock;
using tmvp::KemParams;

constexpr int kSets = 6;
constexpr int kMaxCt = 1472, kMaxSk = 3040, kMaxPk = 1312, kMaxGm = 16 * 416;

__global__ void k_gather16(const uint8_t *table, int stride, const uint32_t *idx, uint8_t *out,
                           int n) {
  const int words = stride >> 4;
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)n * words) return;
  int i = (int)(t / words), w = (int)(t % words);
  reinterpret_cast<uint4 *>(out + (size_t)i * stride)[w] =
      reinterpret_cast<const uint4 *>(table + (size_t)idx[i] * stride)[w];
}

struct Req {
  uint64_t ticket;
  int op, set;
  uint32_t idx;
  const uint8_t *in;
  uint8_t *out;
  Clock::time_point t0;
};

struct Slot {
  tmvp_ctx *ctx = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  uint8_t *h_in = nullptr, *h_out = nullptr;
  uint32_t *h_idx = nullptr;
  size_t blk_off = 0, blk_bytes = 0;  // the batch's block of the device arena
  std::vector<Req> batch;
  int set = 0, op = 0, err = 0;
  bool busy = false;      // holds a batch (from scheduling until completion)
  bool launched = false;  // the batch's work and event are queued on the stream
  uint64_t seq = 0;
};

// First-fit allocator over the device arena, 256-byte granules; free blocks
// are kept by offset and merged with their neighbours when returned.
struct ArenaMap {
  size_t bytes = 0, in_use = 0, peak = 0;
  std::map<size_t, size_t> free_blocks;  // offset -> size
  void reset(size_t b) {
    bytes = b;
    in_use = peak = 0;
    free_blocks.clear();
    if (b) free_blocks[0] = b;
  }
  size_t largest() const {
    size_t m = 0;
    for (auto &f : free_blocks) m = std::max(m, f.second);
    return m;
  }
  bool take(size_t n, size_t *off) {
    for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
      if (it->second < n) continue;
      *off = it->first;
      const size_t rest = it->second - n;
      const size_t roff = it->first + n;
      free_blocks.erase(it);
      if (rest) free_blocks[roff] = rest;
      in_use += n;
      peak = std::max(peak, in_use);
      return true;
    }
    return false;
  }
  void give(size_t off, size_t n) {
    in_use -= n;
    auto it = free_blocks.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_blocks.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_blocks.erase(nx);
    }
    if (it != free_blocks.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_blocks.erase(it);
      }
    }
  }
};

struct KeyTable {
  uint8_t *pk = nullptr, *sk = nullptr;  // device
  uint8_t *a = nullptr;                  // device: each key's GenMatrix stream (expanded once)
  size_t n = 0, cap = 0;
  std::vector<uint8_t> h_pk;             // host copy (for the load generator)
};

int sizes_of(int set, KemParams *P) { return tmvp::make_params(set, P) ? 0 : TMVP_EINVAL; }

}  // namespace

struct tmvp_server {
  tmvp_server_config cfg{};
  int device = 0;
  std::vector<Slot> slots;
  KeyTable keys[kSets];
  std::deque<Req> q[kSets][2];
  std::mutex mu;
  std::condition_variable cv_sched, cv_done, cv_comp;
  std::thread sched, comp;
  bool stop = false;
  uint64_t next_ticket = 1, launch_seq = 0, done_seq = 0;
  std::unordered_set<uint64_t> outstanding;
  size_t pending = 0;
  // device arena shared by the batches in flight (memory admission)
  uint8_t *arena = nullptr;
  ArenaMap amap;
  // request buffers of load-generator runs that timed out, kept until destroy
  std::vector<std::unique_ptr<std::vector<uint8_t>>> orphans;
  // statistics
  std::vector<float> lat_us;
  uint64_t submitted = 0, completed = 0, batches = 0, batched_reqs = 0, failed = 0;
  uint64_t admission_waits = 0, admission_splits = 0, checked = 0, mismatched = 0;
  std::atomic<uint64_t> one_key_batches{0};  // counted by launch_batch, outside the lock
  Clock::time_point t_reset = Clock::now();
};

namespace {

void free_slot(Slot &s) {
  if (s.ctx) tmvp_ctx_destroy(s.ctx);
  if (s.st) cudaStreamDestroy(s.st);
  if (s.ev) cudaEventDestroy(s.ev);
  if (s.h_in) cudaFreeHost(s.h_in);
  if (s.h_out) cudaFreeHost(s.h_out);
  if (s.h_idx) cudaFreeHost(s.h_idx);
  s = Slot();
}

constexpr size_t kGran = 256;
inline size_t upg(size_t x) { return (x + kGran - 1) & ~(kGran - 1); }

// Device bytes of one batch of n requests of (set, op): inputs, outputs,
// gathered keys and indices, gathered expanded matrices, KEM workspace.
size_t batch_bytes(int set, int op, size_t n) {
  KemParams P;
  tmvp::make_params(set, &P);
  const bool dec = op == TMVP_OP_DECAPS;
  const size_t inb = dec ? P.ct_bytes : 32, outb = dec ? 32 : P.ct_bytes + 32;
  const size_t kb = dec ? P.sk_bytes : P.pk_bytes;
  const size_t ws = std::max(tmvp::kem_ws_bytes(dec ? 1 : 0, P, n), dec ? tmvp::kem_ws_bytes(2, P, n) : 0);
  return upg(n * inb) + upg(n * outb) + upg(n * kb) + upg(n * 4) + upg(n * P.gm_bytes) + upg(ws);
}

// The most requests of (set, op) whose batch fits `room` bytes (<= cap).
size_t fit_requests(int set, int op, size_t room, size_t cap) {
  size_t lo = 0, hi = cap;
  while (lo < hi) {
    const size_t mid = (lo + hi + 1) / 2;
    if (batch_bytes(set, op, mid) <= room) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// The largest batch of max_batch requests of any set and operation.
size_t max_batch_bytes(int mb) {
  size_t m = 0;
  for (int set = 0; set < kSets; set++)
    for (int op = 0; op < 2; op++) m = std::max(m, batch_bytes(set, op, (size_t)mb));
  return m;
}

int alloc_slot(Slot &s, int device, int mb) {
  if (tmvp_ctx_create(device, 0, &s.ctx) != TMVP_OK) return TMVP_EDEVICE;
  if (cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaMallocHost(&s.h_in, (size_t)mb * kMaxCt) != cudaSuccess ||
      cudaMallocHost(&s.h_out, (size_t)mb * (kMaxCt + 32)) != cudaSuccess ||
      cudaMallocHost(&s.h_idx, (size_t)mb * 4) != cudaSuccess) {
    cudaGetLastError();  // reported here, not by a later call's error check
    return TMVP_ENOMEM;
  }
  s.batch.reserve(mb);
  return TMVP_OK;
}

// Prepares and launches the slot's batch (outside the server lock), in the
// arena block the scheduler reserved for it.
void launch_batch(tmvp_server *S, Slot &s) {
  KemParams P;
  sizes_of(s.set, &P);
  const int n = (int)s.batch.size();
  const bool dec = s.op == TMVP_OP_DECAPS;
  const int inb = dec ? P.ct_bytes : 32, outb = dec ? 32 : P.ct_bytes + 32;
  const int kb = dec ? P.sk_bytes : P.pk_bytes;
  // carve the block in the order batch_bytes counts it
  uint8_t *p = S->arena + s.blk_off;
  uint8_t *d_in = p;
  p += upg((size_t)n * inb);
  uint8_t *d_out = p;
  p += upg((size_t)n * outb);
  uint8_t *d_key = p;
  p += upg((size_t)n * kb);
  uint32_t *d_idx = reinterpret_cast<uint32_t *>(p);
  p += upg((size_t)n * 4);
  uint8_t *d_a = p;
  p += upg((size_t)n * P.gm_bytes);
  const size_t ws_bytes = s.blk_bytes - (size_t)(p - (S->arena + s.blk_off));
  for (int i = 0; i < n; i++) {
    memcpy(s.h_in + (size_t)i * inb, s.batch[i].in, inb);
    s.h_idx[i] = s.batch[i].idx;
  }
  int e = tmvp::ctx_attach_workspace(s.ctx, p, ws_bytes) != TMVP_OK;
  e |= cudaMemcpyAsync(d_in, s.h_in, (size_t)n * inb, cudaMemcpyHostToDevice, s.st);
  const KeyTable &K = S->keys[s.set];
  // a decapsulation batch under one key (a server's long-term key) reads
  // that key in place and shares its secret across ciphertexts
  // (the one-key path shares the key in place on the tcgen05 form only; the
  // block is sized for that case)
  const int f = S->cfg.form;
  bool one_key = dec && n > 1 && (f == TMVP_FORM_AUTO || f == TMVP_FORM_FP8_TCGEN05);
  for (int i = 1; one_key && i < n; i++) one_key = s.h_idx[i] == s.h_idx[0];
  if (one_key) {
    const int rc = tmvp_kem_dec_batch_onekey(s.ctx, (tmvp_param_set)s.set, n, d_out, d_in,
                                             K.sk + (size_t)s.h_idx[0] * P.sk_bytes, (tmvp_form)S->cfg.form, s.st);
    e |= cudaMemcpyAsync(s.h_out, d_out, (size_t)n * 32, cudaMemcpyDeviceToHost, s.st);
    e |= cudaEventRecord(s.ev, s.st);
    s.err = (rc != TMVP_OK || e != 0) ? 1 : 0;
    S->one_key_batches.fetch_add(1, std::memory_order_relaxed);
    return;
  }
  e |= cudaMemcpyAsync(d_idx, s.h_idx, (size_t)n * 4, cudaMemcpyHostToDevice, s.st);
  size_t words = (size_t)n * (kb >> 4);
  k_gather16<<<(unsigned)((words + 255) / 256), 256, 0, s.st>>>(dec ? K.sk : K.pk, kb, d_idx, d_key, n);
  // each key's A was expanded when the key was added: gather it instead of
  // running GenMatrix (23 of a Saber decapsulation's 39 Keccak-f) per request
  const size_t awords = (size_t)n * (P.gm_bytes >> 4);
  k_gather16<<<(unsigned)((awords + 255) / 256), 256, 0, s.st>>>(K.a, P.gm_bytes, d_idx, d_a, n);
  int rc;
  if (dec) {
    rc = tmvp_kem_dec_batch_a(s.ctx, (tmvp_param_set)s.set, n, d_out, d_in, d_key, d_a,
                              (tmvp_form)S->cfg.form, s.st);
  } else {
    rc = tmvp_kem_enc_batch_a(s.ctx, (tmvp_param_set)s.set, n, d_out, d_out + (size_t)n * P.ct_bytes, d_key,
                              d_in, d_a, (tmvp_form)S->cfg.form, s.st);
  }
  e |= cudaMemcpyAsync(s.h_out, d_out, (size_t)n * outb, cudaMemcpyDeviceToHost, s.st);
  e |= cudaEventRecord(s.ev, s.st);
  s.err = (rc != TMVP_OK || e != 0) ? 1 : 0;
}

// The queue whose head has waited longest (false if none).
bool oldest_queue(tmvp_server *S, int *bs, int *bo) {
  *bs = -1;
  Clock::time_point best{};
  for (int st = 0; st < kSets; st++)
    for (int op = 0; op < 2; op++)
      if (!S->q[st][op].empty() && (*bs < 0 || S->q[st][op].front().t0 < best)) {
        best = S->q[st][op].front().t0;
        *bs = st;
        *bo = op;
      }
  return *bs >= 0;
}

void scheduler(tmvp_server *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  bool blocked = false;  // the last wait was for arena memory
  for (;;) {
    Slot *slot = nullptr;
    int bs = -1, bo = -1;
    size_t take = 0;
    S->cv_sched.wait(lk, [&] {
      if (S->stop) return true;
      if (S->pending == 0) return false;
      slot = nullptr;
      for (auto &s : S->slots)
        if (!s.busy) {
          slot = &s;
          break;
        }
      if (!slot) return false;
      oldest_queue(S, &bs, &bo);
      // memory admission: as many of the queue's requests as the largest
      // free block of the arena holds
      const size_t want = std::min<size_t>(S->q[bs][bo].size(), (size_t)S->cfg.max_batch);
      take = fit_requests(bs, bo, S->amap.largest(), want);
      if (take == 0) {
        blocked = true;  // wait for a batch in flight to return its block
        return false;
      }
      if (take < want) S->admission_splits++;
      return true;
    });
    if (S->stop) break;
    if (blocked) {
      S->admission_waits++;
      blocked = false;
    }
    auto &Q = S->q[bs][bo];
    size_t off = 0;
    const size_t bytes = batch_bytes(bs, bo, take);
    if (!S->amap.take(bytes, &off)) continue;  // cannot happen: take was sized to the largest block
    slot->blk_off = off;
    slot->blk_bytes = bytes;
    slot->batch.assign(Q.begin(), Q.begin() + take);
    Q.erase(Q.begin(), Q.begin() + take);
    S->pending -= take;
    slot->set = bs;
    slot->op = bo;
    slot->busy = true;
    slot->seq = S->launch_seq++;
    lk.unlock();
    launch_batch(S, *slot);
    lk.lock();
    slot->launched = true;
    S->batches++;
    S->batched_reqs += take;
    S->cv_comp.notify_one();
  }
}

void completer(tmvp_server *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    Slot *slot = nullptr;
    S->cv_comp.wait(lk, [&] {
      for (auto &s : S->slots)
        if (s.busy && s.launched && s.seq == S->done_seq) {
          slot = &s;
          return true;
        }
      return S->stop && S->launch_seq == S->done_seq;
    });
    if (!slot) break;
    lk.unlock();
    cudaEventSynchronize(slot->ev);
    KemParams P;
    sizes_of(slot->set, &P);
    const int outb = slot->op == TMVP_OP_DECAPS ? 32 : P.ct_bytes + 32;
    const int n = (int)slot->batch.size();
    const auto now = Clock::now();
    std::vector<float> lat(n);
    const bool ok = slot->err == 0 && cudaEventQuery(slot->ev) == cudaSuccess;
    for (int i = 0; i < n && ok; i++) {
      const Req &r = slot->batch[i];
      if (slot->op == TMVP_OP_DECAPS) {
        memcpy(r.out, slot->h_out + (size_t)i * 32, 32);
      } else {  // ct || ss from the two output areas
        memcpy(r.out, slot->h_out + (size_t)i * P.ct_bytes, P.ct_bytes);
        memcpy(r.out + P.ct_bytes, slot->h_out + (size_t)n * P.ct_bytes + (size_t)i * 32, 32);
      }
    }
    for (int i = 0; i < n; i++)
      lat[i] = std::chrono::duration<float, std::micro>(now - slot->batch[i].t0).count();
    (void)outb;
    lk.lock();
    for (int i = 0; i < n; i++) S->outstanding.erase(slot->batch[i].ticket);
    S->lat_us.insert(S->lat_us.end(), lat.begin(), lat.end());
    S->completed += n;
    if (!ok) S->failed += n;
    slot->batch.clear();
    S->amap.give(slot->blk_off, slot->blk_bytes);
    slot->blk_bytes = 0;
    slot->busy = false;
    slot->launched = false;
    S->done_seq++;
    S->cv_done.notify_all();
    S->cv_sched.notify_one();
  }
}

uint64_t splitmix(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int tmvp_server_create(const tmvp_server_config *cfg, tmvp_server **out) {
  if (!cfg || !out) return TMVP_EINVAL;
  *out = nullptr;
  tmvp_server_config c = *cfg;
  if (c.max_batch <= 0) c.max_batch = 4096;
  if (c.max_batch > 65536) return TMVP_EINVAL;
  if (c.slots <= 0) c.slots = 4;
  if (c.form != TMVP_FORM_AUTO && !tmvp::form_valid(c.form)) return TMVP_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return TMVP_ENOTSUP;
  }
  if (c.device < 0 || c.device >= ndev) return TMVP_EINVAL;
  // memory admission: one device arena holds the blocks of every batch in
  // flight; by default as much as `slots` batches of max_batch requests of the
  // largest set need, else mem_budget, which must hold one request of every set
  const size_t arena_bytes = c.mem_budget ? upg(c.mem_budget) : (size_t)c.slots * max_batch_bytes(c.max_batch);
  if (arena_bytes < max_batch_bytes(1)) return TMVP_ENOMEM;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c.device);
  tmvp_server *S = new tmvp_server();
  S->cfg = c;
  S->device = c.device;
  if (cudaMalloc(&S->arena, arena_bytes) != cudaSuccess) {
    cudaGetLastError();
    delete S;
    cudaSetDevice(prev);
    return TMVP_ENOMEM;
  }
  S->amap.reset(arena_bytes);
  S->slots.resize(c.slots);
  for (auto &s : S->slots) {
    int rc = alloc_slot(s, c.device, c.max_batch);
    if (rc != TMVP_OK) {
      for (auto &t : S->slots) free_slot(t);
      cudaFree(S->arena);
      delete S;
      cudaSetDevice(prev);
      return rc;
    }
  }
  S->lat_us.reserve(1 << 20);
  S->sched = std::thread(scheduler, S);
  S->comp = std::thread(completer, S);
  cudaSetDevice(prev);
  *out = S;
  return TMVP_OK;
}

void tmvp_server_destroy(tmvp_server *S) {
  if (!S) return;
  tmvp_server_drain(S, 60000);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_sched.notify_all();
  S->cv_comp.notify_all();
  S->sched.join();
  S->comp.join();
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(S->device);
  for (auto &s : S->slots) free_slot(s);
  if (S->arena) cudaFree(S->arena);
  for (auto &k : S->keys) {
    if (k.pk) cudaFree(k.pk);
    if (k.sk) cudaFree(k.sk);
    if (k.a) cudaFree(k.a);
  }
  cudaSetDevice(prev);
  delete S;
}

int tmvp_server_add_keys(tmvp_server *S, tmvp_param_set set, size_t n, const uint8_t *pk,
                         const uint8_t *sk, uint32_t *key_ids) {
  KemParams P;
  if (!S || sizes_of(set, &P) || !pk || !sk || !key_ids) return TMVP_EINVAL;
  if (n == 0) return TMVP_OK;
  // the key table may move: wait until no batch is in flight
  if (tmvp_server_drain(S, 60000) != TMVP_OK) return TMVP_ETIMEOUT;
  std::lock_guard<std::mutex> lk(S->mu);
  KeyTable &K = S->keys[set];
  if (K.n + n > (1u << 29)) return TMVP_EINVAL;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(S->device);
  if (K.n + n > K.cap) {
    size_t cap = std::max(K.n + n, K.cap * 2);
    uint8_t *npk = nullptr, *nsk = nullptr, *na = nullptr;
    if (cudaMalloc(&npk, cap * P.pk_bytes) != cudaSuccess || cudaMalloc(&nsk, cap * P.sk_bytes) != cudaSuccess ||
        cudaMalloc(&na, cap * P.gm_bytes) != cudaSuccess) {
      if (npk) cudaFree(npk);
      if (nsk) cudaFree(nsk);
      cudaGetLastError();  // reported here, not by a later call's error check
      cudaSetDevice(prev);
      return TMVP_ENOMEM;
    }
    if (K.n) {
      cudaMemcpy(npk, K.pk, K.n * P.pk_bytes, cudaMemcpyDeviceToDevice);
      cudaMemcpy(nsk, K.sk, K.n * P.sk_bytes, cudaMemcpyDeviceToDevice);
      cudaMemcpy(na, K.a, K.n * P.gm_bytes, cudaMemcpyDeviceToDevice);
      cudaFree(K.pk);
      cudaFree(K.sk);
      cudaFree(K.a);
    }
    K.pk = npk;
    K.sk = nsk;
    K.a = na;
    K.cap = cap;
  }
  int e = 0;
  e |= cudaMemcpy(K.pk + K.n * P.pk_bytes, pk, n * P.pk_bytes, cudaMemcpyDefault);
  e |= cudaMemcpy(K.sk + K.n * P.sk_bytes, sk, n * P.sk_bytes, cudaMemcpyDefault);
  // expand each new key's A once (device pk rows -> GenMatrix streams)
  if (!e) {
    Slot &s0 = S->slots[0];
    if (tmvp_genmatrix_batch(s0.ctx, set, n, K.a + K.n * P.gm_bytes, K.pk + K.n * P.pk_bytes, P.pk_bytes, s0.st) !=
            TMVP_OK ||
        cudaStreamSynchronize(s0.st) != cudaSuccess)
      e = 1;
  }
  K.h_pk.resize((K.n + n) * P.pk_bytes);
  cudaMemcpy(K.h_pk.data() + K.n * P.pk_bytes, pk, n * P.pk_bytes, cudaMemcpyDefault);
  for (size_t i = 0; i < n; i++) key_ids[i] = ((uint32_t)set << 29) | (uint32_t)(K.n + i);
  K.n += n;
  cudaSetDevice(prev);
  return e ? TMVP_EDEVICE : TMVP_OK;
}

int tmvp_server_submit(tmvp_server *S, int op, uint32_t key_id, const uint8_t *in, uint8_t *out,
                       uint64_t *ticket) {
  if (!S || !in || !out || (op != TMVP_OP_ENCAPS && op != TMVP_OP_DECAPS)) return TMVP_EINVAL;
  const int set = (int)(key_id >> 29);
  const uint32_t idx = key_id & ((1u << 29) - 1);
  if (set >= kSets) return TMVP_EINVAL;
  Req r{0, op, set, idx, in, out, Clock::now()};
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (idx >= S->keys[set].n) return TMVP_EINVAL;
    r.ticket = S->next_ticket++;
    S->q[set][op].push_back(r);
    S->outstanding.insert(r.ticket);
    S->pending++;
    S->submitted++;
  }
  S->cv_sched.notify_one();
  if (ticket) *ticket = r.ticket;
  return TMVP_OK;
}

int tmvp_server_wait(tmvp_server *S, uint64_t ticket, int timeout_ms) {
  if (!S) return TMVP_EINVAL;
  std::unique_lock<std::mutex> lk(S->mu);
  bool ok = S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                [&] { return S->outstanding.count(ticket) == 0; });
  return ok ? TMVP_OK : TMVP_ETIMEOUT;
}

int tmvp_server_drain(tmvp_server *S, int timeout_ms) {
  if (!S) return TMVP_EINVAL;
  std::unique_lock<std::mutex> lk(S->mu);
  bool ok = S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                [&] { return S->outstanding.empty(); });
  return ok ? TMVP_OK : TMVP_ETIMEOUT;
}

int tmvp_server_get_stats(tmvp_server *S, tmvp_server_stats *o) {
  if (!S || !o) return TMVP_EINVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  memset(o, 0, sizeof *o);
  o->submitted = S->submitted;
  o->completed = S->completed;
  o->batches = S->batches;
  o->mean_batch = S->batches ? (double)S->batched_reqs / S->batches : 0.0;
  o->slots = (int)S->slots.size();
  o->failed = S->failed;
  o->one_key_batches = S->one_key_batches.load(std::memory_order_relaxed);
  o->arena_bytes = S->amap.bytes;
  o->peak_arena_bytes = S->amap.peak;
  o->admission_waits = S->admission_waits;
  o->admission_splits = S->admission_splits;
  o->checked = S->checked;
  o->mismatched = S->mismatched;
  o->elapsed_s = std::chrono::duration<double>(Clock::now() - S->t_reset).count();
  o->throughput = o->elapsed_s > 0 ? S->completed / o->elapsed_s : 0.0;
  if (!S->lat_us.empty()) {
    std::vector<float> v = S->lat_us;
    auto pct = [&](double p) {
      size_t k = (size_t)std::min<double>(v.size() - 1, std::floor(p * (v.size() - 1)));
      std::nth_element(v.begin(), v.begin() + k, v.end());
      return (double)v[k];
    };
    o->p50_us = pct(0.50);
    o->p99_us = pct(0.99);
    o->max_us = *std::max_element(v.begin(), v.end());
  }
  return TMVP_OK;
}

void tmvp_server_reset_stats(tmvp_server *S) {
  if (!S) return;
  std::lock_guard<std::mutex> lk(S->mu);
  S->lat_us.clear();
  S->submitted = S->completed = S->batches = S->batched_reqs = S->failed = 0;
  S->admission_waits = S->admission_splits = S->checked = S->mismatched = 0;
  S->amap.peak = S->amap.in_use;
  S->one_key_batches.store(0, std::memory_order_relaxed);
  S->t_reset = Clock::now();
}

int tmvp_server_loadgen(tmvp_server *S, double rate, double seconds, uint64_t seed,
                        const uint32_t *key_ids, size_t nkeys, double decaps_fraction,
                        uint64_t *submitted) {
  if (!S || !key_ids || nkeys == 0 || rate <= 0 || seconds <= 0) return TMVP_EINVAL;
  // one ciphertext per key (made with the server's own encapsulation path);
  // cts[i] = ct || ss, so a decapsulation of it must give ss back
  std::vector<size_t> ct_off(nkeys);
  std::vector<int> ct_len(nkeys);
  size_t total = 0;
  for (size_t i = 0; i < nkeys; i++) {
    KemParams P;
    int set = (int)(key_ids[i] >> 29);
    if (set >= kSets || sizes_of(set, &P)) return TMVP_EINVAL;
    ct_len[i] = P.ct_bytes;
    ct_off[i] = total;
    total += P.ct_bytes + 32;
  }
  auto cts = std::make_unique<std::vector<uint8_t>>(total);
  auto coins0 = std::make_unique<std::vector<uint8_t>>(32 * nkeys);
  uint64_t st = seed;
  for (auto &c : *coins0) c = (uint8_t)splitmix(st);
  auto orphan = [&](std::unique_ptr<std::vector<uint8_t>> &b) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->orphans.push_back(std::move(b));
  };
  for (size_t i = 0; i < nkeys; i++) {
    uint64_t tk;
    int rc = tmvp_server_submit(S, TMVP_OP_ENCAPS, key_ids[i], coins0->data() + 32 * i,
                                cts->data() + ct_off[i], &tk);
    if (rc) {
      nkeys = i;  // the ones submitted so far still run: drain below
      if (tmvp_server_drain(S, 60000)) {
        orphan(cts);
        orphan(coins0);
        return TMVP_ETIMEOUT;
      }
      return rc;
    }
  }
  if (tmvp_server_drain(S, 60000)) {
    orphan(cts);
    orphan(coins0);
    return TMVP_ETIMEOUT;
  }
  tmvp_server_reset_stats(S);
  // request stream over a ring of output buffers; a ring entry is reused only
  // after its previous request completed (and, for a decapsulation, was
  // checked against the encapsulated key)
  const size_t ring = 1 << 16, ob = kMaxCt + 32;
  auto out = std::make_unique<std::vector<uint8_t>>(ring * ob);
  auto coins = std::make_unique<std::vector<uint8_t>>(ring * 32);
  for (auto &c : *coins) c = (uint8_t)splitmix(st);
  std::vector<uint64_t> ticket(ring, 0);
  std::vector<int64_t> dec_key(ring, -1);  // key index of a decapsulation in the entry
  uint64_t checked = 0, mismatched = 0;
  auto check = [&](size_t e) {
    if (dec_key[e] >= 0) {
      const size_t key = (size_t)dec_key[e];
      checked++;
      mismatched += memcmp(out->data() + e * ob, cts->data() + ct_off[key] + ct_len[key], 32) != 0;
      dec_key[e] = -1;
    }
  };
  const auto t_start = Clock::now();
  double t_next = 0.0;
  uint64_t k = 0;
  int result = TMVP_OK;
  for (;;) {
    double u = ((splitmix(st) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    t_next += -std::log(u) / rate;
    if (t_next > seconds) break;
    for (;;) {  // wait for the arrival time
      double now = std::chrono::duration<double>(Clock::now() - t_start).count();
      if (now >= t_next) break;
      if (t_next - now > 200e-6) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    size_t key = (size_t)(splitmix(st) % nkeys);
    bool dec = ((splitmix(st) >> 11) * (1.0 / 9007199254740992.0)) < decaps_fraction;
    size_t e = k % ring;
    if (ticket[e]) {
      if (tmvp_server_wait(S, ticket[e], 60000) != TMVP_OK) {
        result = TMVP_ETIMEOUT;
        break;
      }
      check(e);
    }
    int rc = dec ? tmvp_server_submit(S, TMVP_OP_DECAPS, key_ids[key], cts->data() + ct_off[key],
                                      out->data() + e * ob, &ticket[e])
                 : tmvp_server_submit(S, TMVP_OP_ENCAPS, key_ids[key], coins->data() + e * 32,
                                      out->data() + e * ob, &ticket[e]);
    if (rc) {
      ticket[e] = 0;
      result = rc;
      break;
    }
    dec_key[e] = dec ? (int64_t)key : -1;
    k++;
  }
  // the request buffers must outlive every request: a bounded wait, and on
  // timeout the buffers are handed to the server (freed at destroy)
  if (tmvp_server_drain(S, 120000) != TMVP_OK) {
    orphan(out);
    orphan(coins);
    orphan(cts);
    return TMVP_ETIMEOUT;
  }
  for (size_t e = 0; e < ring; e++) check(e);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->checked += checked;
    S->mismatched += mismatched;
  }
  if (submitted) *submitted = k;
  return result;
}

}  // extern "C"
