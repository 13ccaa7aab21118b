// server.cu — request-serving loop: device-resident keys, continuous
// batching over several in-flight batch slots, latency statistics, and a
// seeded Poisson load generator.  No counterpart in the reference, whose host
// API runs one fixed batch per call (cuda_kernel.cu:25-479).
//
// Threads:
//   * callers submit requests (zero-copy: the request keeps the caller's in /
//     out pointers) into one FIFO per (parameter set, op);
//   * the scheduler turns the queue whose head waited longest into a batch
//     (up to max_batch) as soon as a slot is free: it gathers the inputs into
//     the slot's pinned buffer, copies them to the device, gathers the keys
//     from the device key table by index, launches the batched KEM on the
//     slot's stream, queues the copy of the outputs back and records an event;
//   * the completer waits for slot events in launch order, scatters the
//     outputs to the callers' buffers, records latencies and frees the slot.
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
#include <mutex>
#include <thread>
#include <unordered_set>
#include <vector>

#include "../../include/tmvp_kem.h"
#include "kem_common.cuh"

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
  uint8_t *d_in = nullptr, *d_out = nullptr, *d_key = nullptr, *d_a = nullptr;
  uint32_t *d_idx = nullptr;
  std::vector<Req> batch;
  int set = 0, op = 0, err = 0;
  bool busy = false;      // holds a batch (from scheduling until completion)
  bool launched = false;  // the batch's work and event are queued on the stream
  uint64_t seq = 0;
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
  // statistics
  std::vector<float> lat_us;
  uint64_t submitted = 0, completed = 0, batches = 0, batched_reqs = 0, failed = 0;
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
  if (s.d_in) cudaFree(s.d_in);
  if (s.d_out) cudaFree(s.d_out);
  if (s.d_key) cudaFree(s.d_key);
  if (s.d_a) cudaFree(s.d_a);
  if (s.d_idx) cudaFree(s.d_idx);
  s = Slot();
}

// Device bytes one slot holds for max_batch requests of the largest set.
size_t slot_bytes(int mb) {
  size_t per = (size_t)kMaxCt + (kMaxCt + 32) + kMaxSk + 4 +  // in, out, keys, idx
               kMaxGm +                                       // the batch's expanded matrices
               16 * 416 + 768 + 64 + 64 + 1 + 32;             // KEM workspace (FireSaber)
  return per * (size_t)mb + 64 * 256;
}

int alloc_slot(Slot &s, int device, int mb) {
  if (tmvp_ctx_create(device, 0, &s.ctx) != TMVP_OK) return TMVP_EDEVICE;
  size_t ws = (size_t)mb * (16 * 416 + 768 + 64 + 64 + 1 + 32) + 8 * 256;
  if (tmvp_ctx_reserve(s.ctx, ws) != TMVP_OK) return TMVP_ENOMEM;
  if (cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaMallocHost(&s.h_in, (size_t)mb * kMaxCt) != cudaSuccess ||
      cudaMallocHost(&s.h_out, (size_t)mb * (kMaxCt + 32)) != cudaSuccess ||
      cudaMallocHost(&s.h_idx, (size_t)mb * 4) != cudaSuccess ||
      cudaMalloc(&s.d_in, (size_t)mb * kMaxCt) != cudaSuccess ||
      cudaMalloc(&s.d_out, (size_t)mb * (kMaxCt + 32)) != cudaSuccess ||
      cudaMalloc(&s.d_key, (size_t)mb * kMaxSk) != cudaSuccess ||
      cudaMalloc(&s.d_idx, (size_t)mb * 4) != cudaSuccess ||
      cudaMalloc(&s.d_a, (size_t)mb * kMaxGm) != cudaSuccess) {
    cudaGetLastError();  // reported here, not by a later call's error check
    return TMVP_ENOMEM;
  }
  s.batch.reserve(mb);
  return TMVP_OK;
}

// Prepares and launches the slot's batch (outside the server lock).
void launch_batch(tmvp_server *S, Slot &s) {
  KemParams P;
  sizes_of(s.set, &P);
  const int n = (int)s.batch.size();
  const int inb = s.op == TMVP_OP_DECAPS ? P.ct_bytes : 32;
  for (int i = 0; i < n; i++) {
    memcpy(s.h_in + (size_t)i * inb, s.batch[i].in, inb);
    s.h_idx[i] = s.batch[i].idx;
  }
  int e = 0;
  e |= cudaMemcpyAsync(s.d_in, s.h_in, (size_t)n * inb, cudaMemcpyHostToDevice, s.st);
  const KeyTable &K = S->keys[s.set];
  // a decapsulation batch under one key (a server's long-term key) reads
  // that key in place and shares its secret across ciphertexts
  bool one_key = s.op == TMVP_OP_DECAPS && n > 1;
  for (int i = 1; one_key && i < n; i++) one_key = s.h_idx[i] == s.h_idx[0];
  if (one_key) {
    const int rc = tmvp_kem_dec_batch_onekey(s.ctx, (tmvp_param_set)s.set, n, s.d_out, s.d_in,
                                             K.sk + (size_t)s.h_idx[0] * P.sk_bytes, (tmvp_form)S->cfg.form, s.st);
    e |= cudaMemcpyAsync(s.h_out, s.d_out, (size_t)n * 32, cudaMemcpyDeviceToHost, s.st);
    e |= cudaEventRecord(s.ev, s.st);
    s.err = (rc != TMVP_OK || e != 0) ? 1 : 0;
    S->one_key_batches.fetch_add(1, std::memory_order_relaxed);
    return;
  }
  e |= cudaMemcpyAsync(s.d_idx, s.h_idx, (size_t)n * 4, cudaMemcpyHostToDevice, s.st);
  const int kb = s.op == TMVP_OP_DECAPS ? P.sk_bytes : P.pk_bytes;
  size_t words = (size_t)n * (kb >> 4);
  k_gather16<<<(unsigned)((words + 255) / 256), 256, 0, s.st>>>(
      s.op == TMVP_OP_DECAPS ? K.sk : K.pk, kb, s.d_idx, s.d_key, n);
  // each key's A was expanded when the key was added: gather it instead of
  // running GenMatrix (23 of a Saber decapsulation's 39 Keccak-f) per request
  const size_t awords = (size_t)n * (P.gm_bytes >> 4);
  k_gather16<<<(unsigned)((awords + 255) / 256), 256, 0, s.st>>>(K.a, P.gm_bytes, s.d_idx, s.d_a, n);
  int rc;
  if (s.op == TMVP_OP_DECAPS) {
    rc = tmvp_kem_dec_batch_a(s.ctx, (tmvp_param_set)s.set, n, s.d_out, s.d_in, s.d_key, s.d_a,
                              (tmvp_form)S->cfg.form, s.st);
  } else {
    rc = tmvp_kem_enc_batch_a(s.ctx, (tmvp_param_set)s.set, n, s.d_out,
                              s.d_out + (size_t)n * P.ct_bytes, s.d_key, s.d_in, s.d_a,
                              (tmvp_form)S->cfg.form, s.st);
  }
  const int outb = s.op == TMVP_OP_DECAPS ? 32 : P.ct_bytes + 32;
  e |= cudaMemcpyAsync(s.h_out, s.d_out, (size_t)n * outb, cudaMemcpyDeviceToHost, s.st);
  e |= cudaEventRecord(s.ev, s.st);
  s.err = (rc != TMVP_OK || e != 0) ? 1 : 0;
}

void scheduler(tmvp_server *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_sched.wait(lk, [&] {
      if (S->stop) return true;
      if (S->pending == 0) return false;
      for (auto &s : S->slots)
        if (!s.busy) return true;
      return false;
    });
    if (S->stop) break;
    Slot *slot = nullptr;
    for (auto &s : S->slots)
      if (!s.busy) {
        slot = &s;
        break;
      }
    // the queue whose head has waited longest
    int bs = -1, bo = -1;
    Clock::time_point best{};
    for (int st = 0; st < kSets; st++)
      for (int op = 0; op < 2; op++)
        if (!S->q[st][op].empty() && (bs < 0 || S->q[st][op].front().t0 < best)) {
          best = S->q[st][op].front().t0;
          bs = st;
          bo = op;
        }
    auto &Q = S->q[bs][bo];
    const size_t take = std::min<size_t>(Q.size(), (size_t)S->cfg.max_batch);
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
  // memory-based admission: as many slots as the budget holds
  if (c.mem_budget) {
    size_t fit = c.mem_budget / slot_bytes(c.max_batch);
    if (fit == 0) return TMVP_ENOMEM;
    c.slots = (int)std::min<size_t>((size_t)c.slots, fit);
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c.device);
  tmvp_server *S = new tmvp_server();
  S->cfg = c;
  S->device = c.device;
  S->slots.resize(c.slots);
  for (auto &s : S->slots) {
    int rc = alloc_slot(s, c.device, c.max_batch);
    if (rc != TMVP_OK) {
      for (auto &t : S->slots) free_slot(t);
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
  S->one_key_batches.store(0, std::memory_order_relaxed);
  S->t_reset = Clock::now();
}

int tmvp_server_loadgen(tmvp_server *S, double rate, double seconds, uint64_t seed,
                        const uint32_t *key_ids, size_t nkeys, double decaps_fraction,
                        uint64_t *submitted) {
  if (!S || !key_ids || nkeys == 0 || rate <= 0 || seconds <= 0) return TMVP_EINVAL;
  // one ciphertext per key (made with the server's own encapsulation path)
  std::vector<std::vector<uint8_t>> cts(nkeys);
  std::vector<uint8_t> coins0(32 * nkeys);
  uint64_t st = seed;
  for (auto &c : coins0) c = (uint8_t)splitmix(st);
  for (size_t i = 0; i < nkeys; i++) {
    KemParams P;
    int set = (int)(key_ids[i] >> 29);
    if (sizes_of(set, &P)) return TMVP_EINVAL;
    cts[i].resize(P.ct_bytes + 32);
    uint64_t tk;
    int rc = tmvp_server_submit(S, TMVP_OP_ENCAPS, key_ids[i], coins0.data() + 32 * i,
                                cts[i].data(), &tk);
    if (rc) return rc;
  }
  if (tmvp_server_drain(S, 60000)) return TMVP_ETIMEOUT;
  tmvp_server_reset_stats(S);
  // request stream
  const size_t ring = 1 << 16;
  std::vector<uint8_t> out(ring * (kMaxCt + 32)), coins(ring * 32);
  for (auto &c : coins) c = (uint8_t)splitmix(st);
  const auto t_start = Clock::now();
  double t_next = 0.0;
  uint64_t k = 0;
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
    size_t slot = k % ring;
    int rc = dec ? tmvp_server_submit(S, TMVP_OP_DECAPS, key_ids[key], cts[key].data(),
                                      out.data() + slot * (kMaxCt + 32), nullptr)
                 : tmvp_server_submit(S, TMVP_OP_ENCAPS, key_ids[key], coins.data() + slot * 32,
                                      out.data() + slot * (kMaxCt + 32), nullptr);
    if (rc) return rc;
    k++;
  }
  // the request buffers live in this frame: wait until every request is done
  while (tmvp_server_drain(S, 60000) != TMVP_OK) {
  }
  if (submitted) *submitted = k;
  return TMVP_OK;
}

}  // extern "C"
