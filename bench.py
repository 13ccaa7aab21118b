#!/usr/bin/env python3
"""Saber decapsulations per second at batch 65536, bit-exact; p50/p99 latency.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: 65536 independent Saber (l=3) instances, each with its own key
pair, decapsulating its own ciphertext (keys and ciphertexts are generated on
the GPU from SplitMix64 seeds before timing; every decapsulated key is then
checked against the encapsulated one, and a sample against the CPU oracle).

One step = one tmvp_kem_dec_batch call over the whole batch with device-
resident inputs (inputs are 222 MB, larger than the 129 MB L2, so no flush is
needed between steps).  `value` is decaps/s of the FP8 tensor-core form;
`forms` adds the other forms timed the same way: the mma.sync FP8 and INT8
tensor-core forms, and the CUDA-core forms (TMVP with IMAD, TMVP with dp2a,
Toom-Cook 4-way).  `e2e` is the same metric through the public C ABI with
pinned HOST buffers (host-to-device copies of ct and sk and the copy of the
keys back are inside the timed region), at the library's default host chunk
and ramp; `e2e_sweep` times the other settings.  `roofline` is the dominant
kernel of the step (the largest share of the step's per-stage device time),
timed live with CUDA events on its own stream, with the other large kernels
in `roofline.others`.  `latency` holds per-call p50/p99: the CPU oracle at
batch 1 (keypair, encapsulation, decapsulation) and this library through the
C ABI with host buffers at batch 1 ... 65536.  `cpu_baseline` is the CPU
oracle with the reference's multiplication (Toom-Cook 4-way over Karatsuba)
timed on a sample over all host threads.  Clocks are sampled through NVML
every millisecond inside the timed region.

--impl reference times the reference's CPU path for this workload (the CPU
oracle port of the reference's serial code with its Toom-Cook / Karatsuba
multiplication; the reference itself has no CPU implementation) on all 65536
decapsulations per step, on all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "asfand-tmvp_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "Saber decaps/sec at batch 64K (INT8-TC vs CUDA-core), bit-exact; p50/p99 latency"
UNIT = "decaps/s"
BATCH = 65536
SABER = 1
CT_BYTES, SK_BYTES, PK_BYTES = 1088, 2304, 992
# schoolbook-equivalent work of one negacyclic 256 x 256 product
POLY_OPS = 2 * 256 * 256
# SM cycles per tcgen05.mma kind::f8f6f4 with M = 128, N = 32, K = 32 when 4 CTAs per SM issue
# back to back (measured on GB300 by the mma_rates workload); N = 256 takes 128
MMA_CYCLES = 39.8
MMA_CYCLES_N16 = 38.8
# tcgen05.mma per Saber re-encryption: 3 secret polynomials x 8 Hankel windows,
# each N = 32 over two K steps (the negacyclic wrap serves both M halves)
REENC_MMAS = 24
DEC_MMAS = 24
# the library's default host-buffer chunk and ramp (tmvp_ctx_set_host_chunk / _ramp)
DEFAULT_HOST_CHUNK, DEFAULT_HOST_RAMP = 16384, 1


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    return 6800.0, 1900.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 25 ms, each sample
    stamped with the host clock, so that the ones taken inside the timed
    region can be told apart."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.rows, self.proc = [], None
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "25"]
        if gpu_id:
            cmd += ["-i", gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append((time.perf_counter(), parts))

    def wait_started(self, timeout: float = 3.0):
        """Block until the first sample arrived (nvidia-smi takes a while to start)."""
        t_end = time.perf_counter() + timeout
        while self.proc and not self.rows and time.perf_counter() < t_end:
            time.sleep(0.01)

    def stop(self, t0: float | None = None, t1: float | None = None):
        """Stats over the samples stamped in [t0, t1] (all samples if none fell there)."""
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if not self.rows:
            return None
        inside = [r for t, r in self.rows if t0 is not None and t0 <= t <= t1]
        rows = inside or [r for _, r in self.rows]
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "samples_in_timed_region": len(inside),
                "samples_total": len(self.rows)}


class NvmlSampler:
    """SM clock, power and clock-event reasons read through NVML (libnvidia-ml,
    read-only queries) every `period` seconds on a thread, each sample stamped
    with the host clock.  Falls back to nothing when NVML is missing."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, uuid: str | None, period: float = 0.001):
        import ctypes
        self.rows, self.ok, self.max_mhz = [], False, None
        self._stop = threading.Event()
        try:
            L = ctypes.CDLL("libnvidia-ml.so.1")
            if L.nvmlInit_v2() != 0:
                return
            h = ctypes.c_void_p()
            if not uuid or L.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(h)) != 0:
                return
            self.L, self.h, self.ct = L, h, ctypes
            mx = ctypes.c_uint()
            if L.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:
                self.max_mhz = float(mx.value)
            self._reasons = getattr(L, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(L, "nvmlDeviceGetCurrentClocksThrottleReasons")
            self.ok = True
        except (OSError, AttributeError):
            return
        self.period = period
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def _run(self):
        ct, L, h = self.ct, self.L, self.h
        clk, rs, pw = ct.c_uint(), ct.c_ulonglong(), ct.c_uint()
        while not self._stop.is_set():
            if L.nvmlDeviceGetClockInfo(h, 1, ct.byref(clk)) == 0:
                r = rs.value if self._reasons(h, ct.byref(rs)) == 0 else 0
                p = pw.value / 1e3 if L.nvmlDeviceGetPowerUsage(h, ct.byref(pw)) == 0 else None
                self.rows.append((time.perf_counter(), float(clk.value), int(r), p))
            time.sleep(self.period)

    def stop(self, t0: float, t1: float):
        if not self.ok:
            return None
        self._stop.set()
        self.t.join(timeout=2)
        inside = [r for r in self.rows if t0 <= r[0] <= t1]
        if not inside:
            return None
        reasons = sorted({n for _, _, r, _ in inside for bit, n in self.REASONS.items() if r & bit})
        pw = [p for *_, p in inside if p is not None]
        return {"sm_mhz": statistics.median(r[1] for r in inside), "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples_in_timed_region": len(inside),
                "power_w_max": max(pw) if pw else None, "source": "NVML, 1 ms period"}


def cpu_decaps_rate(n: int, nthreads: int, seed: int = 99):
    """Oracle decapsulations per second over all host threads on n instances,
    with the reference's multiplication (Toom-Cook 4-way over Karatsuba)."""
    from oracle import pyoracle as O
    import tmvpkem as T
    O.build()
    coins = T.splitmix_bytes(seed, n * 96).reshape(n, 96)
    pk, sk = O.kem_keypair_batch(SABER, coins, nthreads)
    ct, ss = O.kem_enc_batch(SABER, pk, T.splitmix_bytes(seed + 1, n * 32).reshape(n, 32), nthreads)
    O.set_polmul(O.POLMUL_TOOM4K)
    try:
        t0 = time.perf_counter()
        ss2, fail = O.kem_dec_batch(SABER, ct, sk, nthreads)
        dt = time.perf_counter() - t0
    finally:
        O.set_polmul(O.POLMUL_SCHOOLBOOK)
    assert np.array_equal(ss, ss2) and not fail.any()
    return n / dt, (ct, sk, ss)


def cpu_latency_batch1(iters: int = 1000):
    """Config 1: Saber keypair / encapsulation / decapsulation at batch 1 on
    one host thread (the oracle with the reference's multiplication), per-call
    p50 / p99 over `iters` calls each, timed in C."""
    from oracle import pyoracle as O
    O.build()
    out = {}
    O.set_polmul(O.POLMUL_TOOM4K)
    try:
        for op, name in (("keypair", "keypair"), ("enc", "encaps"), ("dec", "decaps")):
            ns = O.kem_latency_ns(SABER, op, iters)
            out[name] = {"p50_us": float(np.percentile(ns, 50)) / 1e3,
                         "p99_us": float(np.percentile(ns, 99)) / 1e3,
                         "mean_us": float(ns.mean()) / 1e3, "calls": iters}
    finally:
        O.set_polmul(O.POLMUL_SCHOOLBOOK)
    out["note"] = ("CPU oracle (C restatement of the reference's serial code, Toom-Cook 4-way over "
                   "Karatsuba as the reference's pol_mul), one host thread, gcc -O3")
    return out


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from oracle import pyoracle as O
    import tmvpkem as T
    nthreads = os.cpu_count() or 1
    n = args.batch
    O.build()
    coins = T.splitmix_bytes(7, n * 96).reshape(n, 96)
    pk, sk = O.kem_keypair_batch(SABER, coins, nthreads)
    ct, ss = O.kem_enc_batch(SABER, pk, T.splitmix_bytes(8, n * 32).reshape(n, 32), nthreads)
    O.set_polmul(O.POLMUL_TOOM4K)
    try:
        for _ in range(args.warmup):
            O.kem_dec_batch(SABER, ct, sk, nthreads)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            ss2, fail = O.kem_dec_batch(SABER, ct, sk, nthreads)
            times.append(time.perf_counter() - t0)
            assert np.array_equal(ss, ss2) and not fail.any()
    finally:
        O.set_polmul(O.POLMUL_SCHOOLBOOK)
    step = statistics.mean(times)
    value = n / step
    desc = (f"CPU oracle (C restatement of the reference's serial Keccak/CBD/pack code, Toom-Cook 4-way "
            f"over Karatsuba multiplication as the reference's pol_mul, gcc -O3), all {n} decapsulations "
            f"per step on {nthreads} threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16",
            "data": "synthetic: SplitMix64-seeded keys and ciphertexts",
            "config": {"workload": "Saber l=3 decapsulation, batch 65536, per-instance keys",
                       "batch": n},
            "latency_ms": {"p50": float(np.percentile(times, 50)) * 1e3,
                           "p99": float(np.percentile(times, 99)) * 1e3, "batch": n},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    import tmvpkem as T

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    T.build.build()
    ctx = T.Context(local)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    n = args.batch

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- inputs (untimed): per-instance keys and ciphertexts, on the GPU
    seed = 1_000_003 * (rank + 1)
    coins = torch.from_numpy(T.splitmix_bytes(seed, n * 96).reshape(n, 96)).to(dev)
    ecoins = torch.from_numpy(T.splitmix_bytes(seed + 1, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, PK_BYTES), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, SK_BYTES), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, CT_BYTES), dtype=torch.uint8, device=dev)
    ss_ref = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(SABER, n, pk, sk, coins, T.FORM_AUTO, sp)
    ctx.kem_enc_ptr(SABER, n, ct, ss_ref, pk, ecoins, T.FORM_AUTO, sp)
    torch.cuda.synchronize()

    # launch shapes for this workload, picked by the library's autotuner
    tuned = {}
    if not args.no_tune:
        tuned = {"saber_launch_shapes": ctx.autotune(SABER, n), "saber_pass": T.tune_pass_get(SABER, n),
                 "note": "tmvp_autotune on its own synthetic batch of this size, before any timing"}

    window = [None, None]  # host clock around the timed region

    def timed(form, steps, stage_timing=False):
        for _ in range(args.warmup):
            ctx.kem_dec_ptr(SABER, n, ss, ct, sk, form, sp)
        if stage_timing:
            ctx.set_timing(True)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        l0 = ctx.launches
        barrier()
        torch.cuda.synchronize()
        window[0] = time.perf_counter()
        ev[0].record(stream)
        for k in range(steps):
            ctx.kem_dec_ptr(SABER, n, ss, ct, sk, form, sp)
            ev[k + 1].record(stream)
        torch.cuda.synchronize()
        window[1] = time.perf_counter()
        barrier()
        launches = ctx.launches - l0
        per = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
        total = ev[0].elapsed_time(ev[steps])
        stages = ctx.stage_stats() if stage_timing else {}
        busy = ctx.stage_busy() if stage_timing else {}
        if stage_timing:
            ctx.set_timing(False)
        ok = bool(torch.equal(ss, ss_ref))
        return total, per, launches, (stages, busy), ok

    gpu_id = None
    try:
        gpu_id = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    sampler = ClockSampler(gpu_id)
    sampler.wait_started()
    nvml = NvmlSampler(gpu_id)
    total_ms, per_ms, launches, (stages, stages_busy), exact_main = timed(T.FORM_AUTO, args.steps,
                                                                         stage_timing=True)
    clocks_nvml = nvml.stop(window[0], window[1])
    clocks_smi = sampler.stop(window[0], window[1])
    clocks = clocks_nvml or clocks_smi
    if clocks_nvml and clocks_smi:
        clocks = dict(clocks_nvml, nvidia_smi=clocks_smi)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = ws * n * args.steps / (total_ms / 1e3)

    # ---- other forms, same workload
    form_rates, form_exact = {}, {}
    kf = max(3, args.steps // 4)
    others = [f for f in args.forms.split(",") if f and f != "none"]
    for name in others:
        form = {v: k for k, v in T.FORM_NAMES.items()}[name]
        tm, _, _, _, ok = timed(form, kf)
        form_rates[name] = n * kf / (tm / 1e3)
        form_exact[name] = ok
    form_rates["auto"] = value / ws

    # ---- end to end through the C ABI with pinned host buffers
    if args.no_e2e:
        e2e_ms, e2e_exact, e2e_value, e2e_chunk = [float("nan")], True, None, (None, {}, False)
    else:
        e2e_ms, e2e_exact, e2e_value, e2e_chunk = _e2e(ctx, T, n, ct, sk, ss_ref, sp, stream, args, ws, local)
    # ---- the same decapsulations with each key's A expanded once beforehand (the
    # serving loop's device-resident keys): GenMatrix leaves the per-call work
    cached = None
    if hasattr(ctx, "kem_dec_a_ptr") and not args.no_extra:
        a_keys = torch.empty((n, T.genmatrix_bytes(SABER)), dtype=torch.uint8, device=dev)
        ctx.genmatrix_ptr(SABER, n, a_keys, pk, None, sp)
        ss_a = torch.empty_like(ss)
        ms_a = _event_ms(stream, lambda: ctx.kem_dec_a_ptr(SABER, n, ss_a, ct, sk, a_keys, T.FORM_AUTO, sp),
                         args.steps)
        cached = {"decaps_per_s": n / (ms_a / 1e3), "ms": ms_a, "bit_exact": bool(torch.equal(ss_a, ss_ref)),
                  "note": "Saber decapsulation at batch 65536 with each key's GenMatrix stream expanded once "
                          "(tmvp_genmatrix_batch), as the serving loop keeps it per key"}
        del a_keys
    # ---- 65536 ciphertexts under ONE key (a server's long-term key): GenMatrix once
    one_key = None
    if hasattr(ctx, "kem_dec_onekey_ptr") and not args.no_extra:
        pk1 = pk[:1].expand(n, -1).contiguous()
        ct1 = torch.empty_like(ct)
        ss1 = torch.empty_like(ss)
        ctx.kem_enc_ptr(SABER, n, ct1, ss1, pk1, ecoins, T.FORM_AUTO, sp)
        sk1 = sk[0].contiguous()
        ss_o = torch.empty_like(ss)
        ms_o = _event_ms(stream, lambda: ctx.kem_dec_onekey_ptr(SABER, n, ss_o, ct1, sk1, T.FORM_AUTO, sp),
                         args.steps)
        one_key = {"decaps_per_s": n / (ms_o / 1e3), "ms": ms_o, "bit_exact": bool(torch.equal(ss_o, ss1)),
                   "note": "65536 Saber ciphertexts decapsulated under one secret key "
                           "(tmvp_kem_dec_batch_onekey): the key's GenMatrix once, then the cached-A chain"}
        # the same from pinned host ciphertexts to host keys (copies inside the timed region)
        ct1_h = ct1.cpu().pin_memory()
        ss_h1 = torch.empty((n, 32), dtype=torch.uint8).pin_memory()
        ms_oh = _event_ms(stream, lambda: ctx.kem_dec_onekey_ptr(SABER, n, ss_h1, ct1_h, sk1, T.FORM_AUTO, sp),
                          max(3, args.steps // 2))
        one_key["e2e"] = {"decaps_per_s": n / (ms_oh / 1e3), "ms": ms_oh,
                          "bit_exact": bool(torch.equal(ss_h1, ss1.cpu())),
                          "h2d_bytes_per_step": n * CT_BYTES, "d2h_bytes_per_step": n * 32}
        del pk1, ct1, ss1, ct1_h, ss_h1
    # ---- bit-exactness against the CPU oracle on a sample
    oracle_ok = None
    if not args.no_oracle:
        from oracle import pyoracle as O
        O.build()
        idx = np.random.default_rng(5).choice(n, 256, replace=False)
        oss, fail = O.kem_dec_batch(SABER, ct.cpu().numpy()[idx], sk.cpu().numpy()[idx],
                                    os.cpu_count() or 1)
        oracle_ok = bool(np.array_equal(oss, ss.cpu().numpy()[idx]) and not fail.any())

    # ---- roofline: the dominant kernel of the step and the other large kernels beside it.
    # In the pass the stages overlap (the Keccak front on a side stream beside the decryption,
    # two chunk chains on two lanes), so a stage's events there also count the time it shares
    # the GPU.  A second run with every stage alone on one stream (tmvp_ctx_set_serial) gives
    # each kernel's own duration, CUDA events on the stream it runs on; the dominant kernel is
    # the one with the largest share of that serialised step.
    hbm, bf16, peak_src = _peaks()
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    diag = _diag_peaks(ctx, props.multi_processor_count, sm_mhz) if not args.no_diag else {}
    ks = max(10, args.steps // 10)
    ctx.set_serial(True)
    try:
        _, _, _, (stages_iso, _), exact_iso = timed(T.FORM_AUTO, ks, stage_timing=True)
    finally:
        ctx.set_serial(False)
    exact_main = exact_main and exact_iso
    roof_all = _roofline_entries(stages_iso, n * ks, hbm, bf16, peak_src, diag,
                                 props.multi_processor_count, sm_mhz)
    for k, v in roof_all.items():  # the same kernel inside the pipelined pass
        if k in stages and stages[k][0]:
            v["avg_launch_ms_in_pass"] = stages[k][1] / stages[k][0]
            v["instances_per_launch_in_pass"] = n * args.steps / stages[k][0]
            # the chunk chains' launches of a stage overlap in the pass: the union of their
            # intervals is the time the stage held the GPU in each step
            busy = stages_busy.get(k)
            if busy:
                v["busy_ms_per_step_in_pass"] = busy / args.steps
                if "mma_instruction_floor_ms" in v:
                    floor_step = v["mma_instruction_floor_ms"] * n / v["instances_per_launch"]
                    v["frac_of_mma_floor_in_pass"] = floor_step / (busy / args.steps)
                if "keccak" in v:
                    key = next(x for x in _STAGE_WORK if k.startswith(x))
                    rate = n * args.steps * _STAGE_WORK[key][2] / (busy / 1e3)
                    pk = v["keccak"].get("peak_perm_per_s")
                    v["keccak"]["perm_per_s_in_pass"] = rate
                    v["keccak"]["frac_in_pass"] = rate / pk if pk else None
                    v["keccak"]["in_pass_note"] = ("permutations of the step over the stage's busy time in the "
                                                   "pass (union of its launches' intervals; it shares the SMs "
                                                   "with the decryption there)")
    lead = max(roof_all, key=lambda k: roof_all[k]["share_of_stage_time"]) if roof_all else None
    roof = dict(roof_all[lead]) if lead else {}
    if lead:
        roof["dominant_by"] = ("largest share of the serialised step (every stage alone on one stream, "
                               f"{ks} steps, CUDA events on that stream)")
        roof["others"] = {k: v for k, v in roof_all.items() if k != lead}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "e4m3 x e4m3 -> f32 (tcgen05), exact integer sums; results u16 mod 2^13",
        "data": "synthetic: 65536 SplitMix64-seeded key pairs and encapsulations per GPU",
        "config": {"workload": "Saber l=3 decapsulation, batch 65536, per-instance keys",
                   "batch": n, "param_set": "Saber", "form": "auto = fp8_tcgen05",
                   "l2": "inputs (222 MB) larger than L2; no flush", "parallelism": f"replicas x{ws}"},
        "forms": form_rates,
        "launch_shapes": tuned,
        "tc_over_cuda_core": (value / ws / form_rates["cuda_core"]) if "cuda_core" in form_rates else None,
        "latency_ms": {"p50": float(np.percentile(per_ms, 50)), "p99": float(np.percentile(per_ms, 99)),
                       "batch": n},
        "bit_exact": {"all_keys_match": exact_main and all(form_exact.values()) and e2e_exact,
                      "checked": n, "oracle_sample": 256, "oracle_match": oracle_ok},
        "roofline": roof,
        "stages_ms_per_launch_in_pass": {k: v[1] / max(v[0], 1) for k, v in stages.items()},
        "stages_busy_ms_per_step_in_pass": {k: b / args.steps for k, b in stages_busy.items()},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * (CT_BYTES + SK_BYTES),
                "d2h_bytes_per_step": n * 32, "ms_per_step": statistics.mean(e2e_ms),
                "p50_ms": float(np.percentile(e2e_ms, 50)), "p99_ms": float(np.percentile(e2e_ms, 99)),
                "host_chunk_ramp": e2e_chunk[0],
                "setting": ("host chunk / ramp chosen by tmvp_autotune for this batch" if e2e_chunk[2]
                            else "the library's built-in host chunk / ramp")},
        "e2e_sweep": {"ms_by_host_chunk_ramp": e2e_chunk[1],
                      "note": "the other host chunk / ramp settings, timed after the reported default"},
        "cached_genmatrix": cached,
        "one_key": one_key,
        "oracle_sample_note": "256 random instances decapsulated by the CPU oracle and compared",
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if not args.no_extra:
        line["workloads"] = _workloads(ctx, T, dev, sp, stream, args)
    if not args.no_latency:
        line["latency"] = {"gpu_by_batch": _gpu_latency(ctx, T, dev, sp, args)}
        if rank == 0 and not args.no_cpu:
            line["latency"]["cpu_batch1"] = cpu_latency_batch1()
    if rank == 0 and not args.no_cpu:
        rate, _ = cpu_decaps_rate(args.cpu_sample, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"{args.cpu_sample} Saber decapsulations (oracle C restatement of "
                                          f"the reference's serial code with its Toom-Cook 4-way / Karatsuba "
                                          f"multiplication, gcc -O3), all host threads"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def _e2e(ctx, T, n, ct, sk, ss_ref, sp, stream, args, ws, device):
    """Host-buffer decapsulation through the C ABI with the library's own
    host chunk / ramp (the autotuner's choice for this batch, else the
    built-in default): the reported figure.  Then, on a second context, the
    other settings (a separate sweep, not used for the reported figure)."""
    import torch
    ct_h = ct.cpu().pin_memory()
    sk_h = sk.cpu().pin_memory()
    ss_h = torch.empty((n, 32), dtype=torch.uint8).pin_memory()
    ke = max(3, args.steps // 2)

    def run(c, steps):
        for _ in range(min(2, args.warmup)):
            c.kem_dec_ptr(SABER, n, ss_h, ct_h, sk_h, T.FORM_AUTO, sp)
        ms = []
        for _ in range(steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            c.kem_dec_ptr(SABER, n, ss_h, ct_h, sk_h, T.FORM_AUTO, sp)
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        return ms, bool(torch.equal(ss_h, ss_ref.cpu()))

    tuned = T.tune_pass_get(SABER, n)
    used = (tuned["host_chunk"], tuned["host_ramp"]) if tuned else (DEFAULT_HOST_CHUNK, DEFAULT_HOST_RAMP)
    e2e_ms, e2e_exact = run(ctx, ke)
    sweep = {}
    if not args.no_sweep:
        c2 = T.Context(device)
        try:
            for chunk, ramp in ((8192, 0), (8192, 1), (16384, 0), (16384, 1), (16384, 2), (16384, 3),
                                (32768, 2), (32768, 3), (32768, 4), (0, 0)):
                c2.set_host_chunk(chunk)
                c2.set_host_ramp(ramp)
                ms, ok = run(c2, max(3, ke // 2))
                e2e_exact = e2e_exact and ok
                sweep[f"{chunk}/{ramp}"] = statistics.mean(ms)
        finally:
            c2.close()
    setting = f"{used[0]}/{used[1]}"
    return e2e_ms, e2e_exact, ws * n / (statistics.mean(e2e_ms) / 1e3), (setting, sweep, bool(tuned))


def _gpu_latency(ctx, T, dev, sp, args):
    """Per-call latency through the C ABI with pinned host buffers (copies in
    and out inside the call): host wall time of tmvp_kem_dec_batch at batch
    1 ... 65536, and of key generation and encapsulation at batch 1."""
    import torch
    out = {}
    nmax = max(args.latency_batches)
    coins = torch.from_numpy(T.splitmix_bytes(4711, nmax * 96).reshape(nmax, 96))
    ec = torch.from_numpy(T.splitmix_bytes(4712, nmax * 32).reshape(nmax, 32))
    pk_d = torch.empty((nmax, PK_BYTES), dtype=torch.uint8, device=dev)
    sk_d = torch.empty((nmax, SK_BYTES), dtype=torch.uint8, device=dev)
    ct_d = torch.empty((nmax, CT_BYTES), dtype=torch.uint8, device=dev)
    ss_d = torch.empty((nmax, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(SABER, nmax, pk_d, sk_d, coins.to(dev), T.FORM_AUTO, sp)
    ctx.kem_enc_ptr(SABER, nmax, ct_d, ss_d, pk_d, ec.to(dev), T.FORM_AUTO, sp)
    torch.cuda.synchronize()
    ct_h, sk_h, ss_ref = ct_d.cpu().pin_memory(), sk_d.cpu().pin_memory(), ss_d.cpu()
    pk_h = pk_d.cpu().pin_memory()
    coins_h, ec_h = coins.pin_memory(), ec.pin_memory()
    out_h = torch.empty((nmax, 32), dtype=torch.uint8).pin_memory()

    def percentiles(fn, calls):
        for _ in range(3):
            fn()
        t = []
        for _ in range(calls):
            t0 = time.perf_counter()
            fn()
            t.append(time.perf_counter() - t0)
        t = np.array(t) * 1e3
        return {"p50_ms": float(np.percentile(t, 50)), "p99_ms": float(np.percentile(t, 99)),
                "mean_ms": float(t.mean()), "calls": calls}

    for b in args.latency_batches:
        calls = 1000 if b <= 256 else (200 if b <= 4096 else 50)
        r = percentiles(lambda b=b: ctx.kem_dec_ptr(SABER, b, out_h, ct_h, sk_h, T.FORM_AUTO, sp), calls)
        r["bit_exact"] = bool(torch.equal(out_h[:b], ss_ref[:b]))
        r["decaps_per_s"] = b / (r["mean_ms"] / 1e3)
        out[f"decaps_{b}"] = r
    pk1 = torch.empty((1, PK_BYTES), dtype=torch.uint8).pin_memory()
    sk1 = torch.empty((1, SK_BYTES), dtype=torch.uint8).pin_memory()
    ct1 = torch.empty((1, CT_BYTES), dtype=torch.uint8).pin_memory()
    ss1 = torch.empty((1, 32), dtype=torch.uint8).pin_memory()
    out["keypair_1"] = percentiles(lambda: ctx.kem_keypair_ptr(SABER, 1, pk1, sk1, coins_h[:1], T.FORM_AUTO, sp), 1000)
    out["encaps_1"] = percentiles(lambda: ctx.kem_enc_ptr(SABER, 1, ct1, ss1, pk_h[:1], ec_h[:1], T.FORM_AUTO, sp), 1000)
    out["encaps_1"]["bit_exact"] = bool(torch.equal(ct1[0], ct_h[0]) and torch.equal(ss1[0], ss_ref[0]))
    out["note"] = ("host wall time per synchronous C-ABI call with pinned host buffers (host-to-device "
                   "copies of the inputs and the device-to-host copy of the outputs inside the call)")
    return out


def _diag_peaks(ctx, nsm, sm_mhz):
    """Live ceilings measured with the library's own diagnostic kernels: the
    Keccak-f[1600] rate at full occupancy (integer pipe) and the dense e4m3
    tcgen05 rate (kind::f8f6f4, M = 128, N = 256, K = 32)."""
    out = {}
    try:
        rate, blocks = ctx.keccak_rate(64)
        out["keccak_perm_per_s"] = rate
        out["keccak_blocks_per_sm"] = blocks
    except Exception:
        pass
    try:
        _, cyc = ctx.umma_rate(0, 256, ctas_per_sm=2, iters=4096)
        out["e4m3_tflops"] = 2 * 128 * 256 * 32 / cyc * nsm * sm_mhz * 1e6 / 1e12
        out["e4m3_cycles_per_mma_n256"] = cyc
    except Exception:
        pass
    return out


# Per Saber instance: (stage prefix, products, algorithmic bytes, Keccak-f, note)
_STAGE_WORK = {
    "dec_front": (0, 1088 + 32 + 3744 + 32, 32,
                  "GenMatrix (23 Keccak-f) + H(c) (9): reads ct 1088 + seed 32, writes the GenMatrix "
                  "stream 3744 + H(c) 32 bytes"),
    "dec_g": (0, 64 + 64 + 768, 6, "G (1 Keccak-f) + GenSecret (5): reads m'||H(pk) 64, writes kr 64 + "
                                   "GenSecret stream 768 bytes"),
    "cpa_reenc": (12, 6593, 0, "12 products x 2*256^2 ops; 6593 bytes"),
    "cpa_decrypt": (3, 1088 + 1248 + 64, 0, "3 products x 2*256^2 ops; reads ct 1088 + secret 1248, "
                                            "writes m' || H(pk) 64 bytes"),
    "final_key": (0, 64 + 32 + 1 + 32 + 32, 1, "1 Keccak-f; reads kr, H(c), fail, z, writes K"),
}


def _roofline_entries(stages, instances, hbm, bf16, peak_src, diag, nsm, sm_mhz):
    """One roofline record per large stage: the Keccak stages against HBM
    (bound 'hbm': their algorithmic bytes) with their permutation rate against
    the measured Keccak ceiling, the tensor-core stages against the measured
    e4m3 rate (or the bf16 figure as a stand-in) and their MMA-issue floor."""
    total = sum(v[1] for v in stages.values()) or 1.0
    out = {}
    for name, (cnt, ms) in stages.items():
        key = next((k for k in _STAGE_WORK if name.startswith(k)), None)
        if key is None or cnt == 0:
            continue
        prods, nbytes, perms, note = _STAGE_WORK[key]
        avg_s = ms / cnt / 1e3
        per_launch = instances / cnt
        rec = {"kernel": name, "avg_launch_ms": avg_s * 1e3, "launches": cnt,
               "share_of_stage_time": ms / total, "instances_per_launch": per_launch,
               "algorithmic": note}
        traffic = _ncu_traffic(name)
        rec["traffic"] = traffic * per_launch / BATCH if traffic is not None else None
        if prods:
            ops = per_launch * prods * POLY_OPS
            ach = ops / avg_s / 1e12
            peak = diag.get("e4m3_tflops")
            rec.update({"bound": "tensor", "achieved": ach, "unit": "TFLOP/s"})
            if peak:
                rec.update({"peak": peak, "frac": ach / peak,
                            "peak_source": "measured live: dense e4m3 tcgen05 rate from the library's "
                                           "issue-rate diagnostic (kind::f8f6f4 M=128 N=256 K=32) at the "
                                           "sampled SM clock; achieved = schoolbook-equivalent integer ops"})
            else:
                rec.update({"peak": bf16, "frac": ach / bf16,
                            "peak_source": f"{peak_src} bf16 dense as a stand-in for e4m3"})
            mmas, cyc, ncol = (REENC_MMAS, MMA_CYCLES, 32) if key == "cpa_reenc" else (DEC_MMAS, MMA_CYCLES_N16, 16)
            floor_s = per_launch * mmas * cyc / (nsm * sm_mhz * 1e6)
            rec["mma_instruction_floor_ms"] = floor_s * 1e3
            rec["frac_of_mma_floor"] = floor_s / avg_s
            rec["mma_floor_note"] = f"{mmas} tcgen05.mma (M=128, N={ncol}, K=32) per instance at {cyc} SM cycles each"
        else:
            gbs = per_launch * nbytes / avg_s / 1e9
            rec.update({"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                        "peak_source": f"{peak_src} HBM copy bandwidth"})
            if perms:
                rate = per_launch * perms / avg_s
                rec["keccak"] = {"perm_per_s": rate, "peak_perm_per_s": diag.get("keccak_perm_per_s"),
                                 "frac": rate / diag["keccak_perm_per_s"] if diag.get("keccak_perm_per_s") else None,
                                 "bound": "integer ALU pipe (LOP3 / funnel shifts)",
                                 "peak_source": "measured live: the library's Keccak-rate diagnostic at full "
                                                "occupancy"}
        out[name] = rec
    return out


def _event_ms(stream, fn, steps, warmup=2):
    """Mean ms per call of fn over `steps` calls, after `warmup` untimed ones."""
    import torch
    for _ in range(warmup):
        fn()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def _workloads(ctx, T, dev, sp, stream, args):
    """The other workloads of this path, timed the same way (device-resident
    inputs, CUDA events): raw TMVP matrix-vector products, the Sable KEM at
    batch 65536, and the serving loop under Poisson load."""
    import torch
    out = {}
    W = set(args.workloads.split(","))
    forms = [("fp8_tc", T.FORM_FP8_TC), ("int8_tc", T.FORM_INT8_TC), ("cuda_core", T.FORM_CUDA_CORE)]
    if hasattr(T, "FORM_FP8_TCGEN05"):
        forms.insert(0, ("fp8_tcgen05", T.FORM_FP8_TCGEN05))
    # raw matrix-vector: 16384 instances of a 3x3 matrix (uniform mod 2^13) times CBD(mu=8) secrets
    if "matvec" in W:
        n, l = 16384, 3
        g = torch.Generator(device="cpu").manual_seed(1234)
        A = torch.randint(0, 1 << 13, (n, l, l, 256), generator=g, dtype=torch.int32).to(torch.int16).to(dev)
        r = torch.randint(0, 256, (n, l, 256), generator=g, dtype=torch.int32)
        pc = torch.tensor([bin(i).count("1") for i in range(16)], dtype=torch.int32)
        s8 = (pc[r & 15] - pc[r >> 4]).to(torch.int8).to(dev)
        mv = {}
        ref = None
        for name, f in forms + [("dp2a", T.FORM_DP2A), ("toom_cook", T.FORM_TOOM_COOK)]:
            o = torch.empty((n, l, 256), dtype=torch.int16, device=dev)
            fn = lambda o=o, f=f: ctx.matvec_ptr(n, l, 13, False, o, A, s8, f, sp)
            for _ in range(3):
                fn()
            ms = _event_ms(stream, fn, 10)
            if ref is None:
                ref = o.clone()
            mv[name] = {"instances_per_s": n / (ms / 1e3), "ms": ms, "matches_first_form": bool(torch.equal(o, ref))}
        if "cuda_core" in mv:
            for name in mv:
                mv[name]["over_cuda_core"] = mv[name]["instances_per_s"] / mv["cuda_core"]["instances_per_s"]
        out["matvec_16384_l3"] = mv
    # Sable l=3 full KEM at batch 65536
    if "sable" in W:
        SABLE = 4
        z = T.sizes(SABLE)
        nb = 65536
        coins = torch.from_numpy(T.splitmix_bytes(77, nb * 96).reshape(nb, 96)).to(dev)
        ecoins = torch.from_numpy(T.splitmix_bytes(78, nb * 32).reshape(nb, 32)).to(dev)
        pk = torch.empty((nb, z.pk_bytes), dtype=torch.uint8, device=dev)
        sk = torch.empty((nb, z.sk_bytes), dtype=torch.uint8, device=dev)
        ct = torch.empty((nb, z.ct_bytes), dtype=torch.uint8, device=dev)
        ss1 = torch.empty((nb, 32), dtype=torch.uint8, device=dev)
        ss2 = torch.empty((nb, 32), dtype=torch.uint8, device=dev)
        sab = {}
        for name, f in forms:
            kp = lambda f=f: ctx.kem_keypair_ptr(SABLE, nb, pk, sk, coins, f, sp)
            en = lambda f=f: ctx.kem_enc_ptr(SABLE, nb, ct, ss1, pk, ecoins, f, sp)
            de = lambda f=f: ctx.kem_dec_ptr(SABLE, nb, ss2, ct, sk, f, sp)
            for fn in (kp, en, de):
                fn()
            t_kp, t_en, t_de = (_event_ms(stream, fn, 3) for fn in (kp, en, de))
            sab[name] = {"keypairs_per_s": nb / (t_kp / 1e3), "encaps_per_s": nb / (t_en / 1e3),
                         "decaps_per_s": nb / (t_de / 1e3),
                         "round_trips_per_s": nb / ((t_kp + t_en + t_de) / 1e3),
                         "bit_exact_round_trip": bool(torch.equal(ss1, ss2))}
        out["sable_l3_kem_65536"] = sab
    # mixed batch: requests of LightSaber, Saber, FireSaber and Sable interleaved, each with a
    if "mixed" in W:
        # count drawn uniformly from 1..8192, decapsulated by one CUDA-graph replay
        rng = np.random.default_rng(4242)
        sets = [0, 1, 2, 4]
        reqs = [(sets[i % 4], int(rng.integers(1, 8193))) for i in range(24)]
        made, outs = [], []
        for i, (sid, cnt) in enumerate(reqs):
            z = T.sizes(sid)
            cc = torch.from_numpy(T.splitmix_bytes(9000 + i, cnt * 96).reshape(cnt, 96)).to(dev)
            ee = torch.from_numpy(T.splitmix_bytes(9500 + i, cnt * 32).reshape(cnt, 32)).to(dev)
            pk_i = torch.empty((cnt, z.pk_bytes), dtype=torch.uint8, device=dev)
            sk_i = torch.empty((cnt, z.sk_bytes), dtype=torch.uint8, device=dev)
            ct_i = torch.empty((cnt, z.ct_bytes), dtype=torch.uint8, device=dev)
            ss_i = torch.empty((cnt, 32), dtype=torch.uint8, device=dev)
            ctx.kem_keypair_ptr(sid, cnt, pk_i, sk_i, cc, T.FORM_AUTO, sp)
            ctx.kem_enc_ptr(sid, cnt, ct_i, ss_i, pk_i, ee, T.FORM_AUTO, sp)
            made.append((sid, cnt, sk_i, ct_i, ss_i))
            outs.append(torch.zeros_like(ss_i))
        total = sum(c for _, c in reqs)
        plan = T.MixedPlan(ctx, [(sid, outs[i], ct_i, sk_i) for i, (sid, _, sk_i, ct_i, _) in enumerate(made)])
        try:
            ms_graph = _event_ms(stream, lambda: plan.launch(sp), 5)
        finally:
            plan.close()
        exact = all(torch.equal(outs[i], made[i][4]) for i in range(len(made)))

        sep_out = [torch.empty_like(o) for o in outs]

        def per_request():
            for i, (sid, cnt, sk_i, ct_i, _) in enumerate(made):
                ctx.kem_dec_ptr(sid, cnt, sep_out[i], ct_i, sk_i, T.FORM_AUTO, sp)
        ms_sep = _event_ms(stream, per_request, 3)
        out["mixed_graph"] = {"requests": len(reqs), "instances": total, "sets": "LightSaber, Saber, FireSaber, Sable",
                              "decaps_per_s": total / (ms_graph / 1e3), "ms": ms_graph,
                              "per_request_calls_decaps_per_s": total / (ms_sep / 1e3),
                              "bit_exact": bool(exact),
                              "launch": "one CUDA graph: the Keccak stages one launch over all 24 requests, "
                                        "decryption and re-encryption one launch per parameter set"}
    # every parameter set: decapsulations per second at batch 65536 (AUTO form)
    if "sets" in W:
        names = ["LightSaber", "Saber", "FireSaber", "LightSable", "Sable", "FireSable"]
        nb = 65536
        per_set = {}
        for sid, name in enumerate(names):
            z = T.sizes(sid)
            coins = torch.from_numpy(T.splitmix_bytes(500 + sid, nb * 96).reshape(nb, 96)).to(dev)
            ecoins = torch.from_numpy(T.splitmix_bytes(600 + sid, nb * 32).reshape(nb, 32)).to(dev)
            pk = torch.empty((nb, z.pk_bytes), dtype=torch.uint8, device=dev)
            sk = torch.empty((nb, z.sk_bytes), dtype=torch.uint8, device=dev)
            ct = torch.empty((nb, z.ct_bytes), dtype=torch.uint8, device=dev)
            ss1 = torch.empty((nb, 32), dtype=torch.uint8, device=dev)
            ss2 = torch.empty((nb, 32), dtype=torch.uint8, device=dev)
            ctx.kem_keypair_ptr(sid, nb, pk, sk, coins, T.FORM_AUTO, sp)
            ctx.kem_enc_ptr(sid, nb, ct, ss1, pk, ecoins, T.FORM_AUTO, sp)
            ms = _event_ms(stream, lambda: ctx.kem_dec_ptr(sid, nb, ss2, ct, sk, T.FORM_AUTO, sp), 10)
            per_set[name] = {"decaps_per_s": nb / (ms / 1e3), "ms": ms, "bit_exact": bool(torch.equal(ss1, ss2))}
            del pk, sk, ct, ss1, ss2, coins, ecoins
        out["decaps_65536_by_set"] = per_set
    # tensor-core issue cost of the two exact kinds the IND-CPA kernels could use
    if "mma_rates" in W:
        rates = {}
        for kind, name in ((0, "f8f6f4_e4m3_K32"), (1, "f16_K16")):
            rates[name] = {}
            for ncol in (16, 32, 64, 128, 256):
                ctas = max(1, min(4, 512 // max(32, ncol)))
                cta, per_sm = ctx.umma_rate(kind, ncol, ctas_per_sm=ctas, iters=4096)
                rates[name][str(ncol)] = {"sm_cycles_per_mma": per_sm, "ctas_per_sm": ctas,
                                          "k_elements": 32 if kind == 0 else 16}
        out["tcgen05_mma_cycles"] = rates
    # serving loop: Poisson arrivals over LightSaber, Saber, FireSaber and Sable (the configured
    # 200 K req/s), then a sweep of offered loads up to saturation
    if "serving" in W:
        rate, secs = 200_000.0, 2.0
        srv = T.Server(device=dev.index or 0, max_batch=4096, slots=4, form=T.FORM_AUTO)
        try:
            ids = []
            for k, sid in enumerate((0, 1, 2, 4)):
                kpk, ksk = ctx.kem_keypair(sid, T.splitmix_bytes(500 + k, 256 * 96).reshape(256, 96))
                ids.append(srv.add_keys(sid, kpk, ksk))
            ids = np.concatenate(ids)
            # warm-up at the same load (module loading, first-touch of the arena), then the measured run
            srv.loadgen(rate=rate, seconds=0.25, seed=20, key_ids=ids, decaps_fraction=0.5)
            srv.reset_stats()
            nreq = srv.loadgen(rate=rate, seconds=secs, seed=21, key_ids=ids, decaps_fraction=0.5)
            st = srv.stats()
            out["serving"] = {"offered_req_per_s": rate, "seconds": secs, "requests": nreq,
                              "throughput_req_per_s": st["throughput"], "p50_us": st["p50_us"],
                              "p99_us": st["p99_us"], "max_us": st["max_us"], "mean_batch": st["mean_batch"],
                              "batches": st["batches"], "slots": st["slots"], "failed": st["failed"],
                              "decaps_checked": st["checked"], "decaps_mismatched": st["mismatched"],
                              "arena_bytes": st["arena_bytes"], "peak_arena_bytes": st["peak_arena_bytes"],
                              "mix": "encaps/decaps 50/50 over LightSaber, Saber, FireSaber, Sable; 256 keys each",
                              "warmup_s": 0.25}
            sweep = []
            for r in args.serving_rates:
                srv.reset_stats()
                nq = srv.loadgen(rate=r, seconds=args.serving_seconds, seed=int(r) % 1000 + 31, key_ids=ids,
                                 decaps_fraction=0.5)
                st = srv.stats()
                sweep.append({"offered_req_per_s": r, "requests": nq, "throughput_req_per_s": st["throughput"],
                              "p50_us": st["p50_us"], "p99_us": st["p99_us"], "mean_batch": st["mean_batch"],
                              "failed": st["failed"], "decaps_mismatched": st["mismatched"]})
            out["serving_sweep"] = {"points": sweep, "seconds_per_point": args.serving_seconds,
                                    "note": "same server, keys and mix; throughput = completed requests / "
                                            "elapsed since the point's start (the generator's own pace "
                                            "caps the highest offered loads)"}
        finally:
            srv.close()
        # memory admission under pressure: an arena of 1/32 of one batch of the largest set (room
        # for ~128 requests) at 1.6 M requests/s
        probe = T.Server(device=dev.index or 0, max_batch=4096, slots=1, form=T.FORM_AUTO)
        one_batch = probe.stats()["arena_bytes"]
        probe.close()
        srv = T.Server(device=dev.index or 0, max_batch=4096, slots=4, form=T.FORM_AUTO,
                       mem_budget=one_batch // 32)
        try:
            ids = []
            for k, sid in enumerate((0, 1, 2, 4)):
                kpk, ksk = ctx.kem_keypair(sid, T.splitmix_bytes(700 + k, 64 * 96).reshape(64, 96))
                ids.append(srv.add_keys(sid, kpk, ksk))
            srv.reset_stats()
            nq = srv.loadgen(rate=1_600_000.0, seconds=0.5, seed=77, key_ids=np.concatenate(ids),
                             decaps_fraction=0.5)
            st = srv.stats()
            out["serving_small_arena"] = {
                "offered_req_per_s": 1_600_000.0, "requests": nq, "throughput_req_per_s": st["throughput"],
                "p50_us": st["p50_us"], "p99_us": st["p99_us"], "mean_batch": st["mean_batch"],
                "arena_bytes": st["arena_bytes"], "peak_arena_bytes": st["peak_arena_bytes"],
                "admission_waits": st["admission_waits"], "admission_splits": st["admission_splits"],
                "failed": st["failed"], "decaps_mismatched": st["mismatched"]}
        finally:
            srv.close()
    return out


def _ncu_traffic(kernel: str):
    """DRAM bytes per launch for `kernel` from the committed ncu summary, scaled
    to the benchmark batch (profiles/dram_traffic.txt: '<stage> <bytes per
    instance>' lines)."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        parts = ln.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1]) * BATCH
            except ValueError:
                return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--cpu-sample", type=int, default=16384)
    ap.add_argument("--no-latency", action="store_true", help="skip the per-call latency measurements")
    ap.add_argument("--no-sweep", action="store_true", help="skip the host chunk / ramp sweep")
    ap.add_argument("--no-diag", action="store_true", help="skip the Keccak / tensor-core ceiling diagnostics")
    ap.add_argument("--serving-rates", default="100000,200000,400000,800000,1600000,3200000,6400000",
                    help="offered loads of the serving sweep, requests/s (comma list)")
    ap.add_argument("--serving-seconds", type=float, default=0.5)
    ap.add_argument("--latency-batches", default="1,16,256,1024,4096,16384,65536",
                    help="batches of the per-call latency curve (comma list)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer (e2e) leg")
    ap.add_argument("--no-oracle", action="store_true", help="skip the oracle sample check")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the matrix-vector, Sable and serving workloads")
    ap.add_argument("--workloads", default="matvec,sable,sets,mixed,mma_rates,serving",
                    help="extra workloads to run (comma list of matvec, sable, sets, mixed, mma_rates, serving)")
    ap.add_argument("--forms", default="fp8_tc,int8_tc,cuda_core,dp2a,toom_cook",
                    help="forms to time besides the headline (AUTO) form (comma list, or 'none')")
    args = ap.parse_args()
    args.latency_batches = [int(x) for x in args.latency_batches.split(",") if x]
    args.serving_rates = [float(x) for x in args.serving_rates.split(",") if x]
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
