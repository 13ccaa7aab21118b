"""Python mirror of libtmvpkem's C ABI (include/tmvp_kem.h).

The library is the product: hand-written sm_103a CUDA kernels behind a C ABI.
This module only loads it with ctypes and wraps its entry points for numpy
arrays (host buffers) and CUDA tensors / raw device pointers (device
buffers).  There is no CPU fallback: if the shared library is missing the
loader raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

LIGHTSABER, SABER, FIRESABER, LIGHTSABLE, SABLE, FIRESABLE = range(6)
SET_NAMES = {LIGHTSABER: "LightSaber", SABER: "Saber", FIRESABER: "FireSaber",
             LIGHTSABLE: "LightSable", SABLE: "Sable", FIRESABLE: "FireSable"}
(FORM_CUDA_CORE, FORM_INT8_TC, FORM_FP8_TC, FORM_AUTO, FORM_SCHOOLBOOK, FORM_FP8_TCGEN05, FORM_DP2A,
 FORM_TOOM_COOK) = range(8)
FORM_NAMES = {FORM_CUDA_CORE: "cuda_core", FORM_INT8_TC: "int8_tc", FORM_FP8_TC: "fp8_tc",
              FORM_AUTO: "auto", FORM_SCHOOLBOOK: "schoolbook", FORM_FP8_TCGEN05: "fp8_tcgen05",
              FORM_DP2A: "dp2a", FORM_TOOM_COOK: "toom_cook"}

OK, EINVAL, ENOMEM, EDEVICE, ETIMEOUT, ENOTSUP = 0, -1, -2, -3, -4, -5

LIB_PATH = _build.LIB
HEADER = os.path.join(_build.REPO, "include", "tmvp_kem.h")
_lib = None


class TmvpError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        msg = lib().tmvp_strerror(code).decode() if _lib is not None else str(code)
        super().__init__(f"{what}: {msg} ({code})" if what else f"{msg} ({code})")


class Sizes(ctypes.Structure):
    _fields_ = [("l", ctypes.c_int), ("eq", ctypes.c_int), ("ep", ctypes.c_int),
                ("et", ctypes.c_int), ("mu", ctypes.c_int), ("pk_bytes", ctypes.c_size_t),
                ("sk_bytes", ctypes.c_size_t), ("ct_bytes", ctypes.c_size_t),
                ("ss_bytes", ctypes.c_size_t), ("indcpa_pk_bytes", ctypes.c_size_t),
                ("indcpa_sk_bytes", ctypes.c_size_t)]


def exported_symbols() -> list[str]:
    """Function names declared in include/tmvp_kem.h."""
    import re
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt)
    skip = {"typedef", "if", "defined", "sizeof", "void"}
    out = []
    for nm in names:
        if nm in skip or nm.isupper() or nm == "tmvp_randombytes_fn":
            continue
        if nm not in out:
            out.append(nm)
    return out


def lib(build_if_missing: bool = False):
    """Load libtmvpkem.so (in-tree build).  Raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"{LIB_PATH} is not built; run tmvpkem.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    P, S, I = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    L.tmvp_strerror.restype = ctypes.c_char_p
    L.tmvp_strerror.argtypes = [I]
    L.tmvp_param_sizes.argtypes = [I, ctypes.POINTER(Sizes)]
    L.tmvp_ctx_create.argtypes = [I, S, ctypes.POINTER(P)]
    L.tmvp_ctx_destroy.argtypes = [P]
    L.tmvp_ctx_destroy.restype = None
    L.tmvp_ctx_workspace_bytes.argtypes = [P]
    L.tmvp_ctx_workspace_bytes.restype = S
    L.tmvp_ctx_launch_count.argtypes = [P]
    L.tmvp_ctx_launch_count.restype = ctypes.c_uint64
    L.tmvp_ctx_set_timing.argtypes = [P, I]
    L.tmvp_ctx_stage_stats.argtypes = [P, I, ctypes.c_char_p, S, ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.POINTER(ctypes.c_double)]
    L.tmvp_kem_keypair_batch.argtypes = [P, I, S, P, P, P, I, P]
    L.tmvp_kem_enc_batch.argtypes = [P, I, S, P, P, P, P, I, P]
    L.tmvp_kem_dec_batch.argtypes = [P, I, S, P, P, P, I, P]
    L.tmvp_genmatrix_bytes.argtypes = [I]
    L.tmvp_genmatrix_bytes.restype = S
    L.tmvp_genmatrix_batch.argtypes = [P, I, S, P, P, S, P]
    L.tmvp_kem_enc_batch_a.argtypes = [P, I, S, P, P, P, P, P, I, P]
    L.tmvp_kem_dec_batch_a.argtypes = [P, I, S, P, P, P, P, I, P]
    L.tmvp_kem_dec_batch_onekey.argtypes = [P, I, S, P, P, P, I, P]
    L.tmvp_indcpa_keypair_batch.argtypes = [P, I, S, P, P, P, I, P]
    L.tmvp_indcpa_enc_batch.argtypes = [P, I, S, P, P, P, P, I, P]
    L.tmvp_indcpa_dec_batch.argtypes = [P, I, S, P, P, P, I, P]
    L.tmvp_matvec_batch.argtypes = [P, S, I, I, I, P, P, P, I, P]
    for nm in ("crypto_kem_keypair", "indcpa_kem_keypair"):
        getattr(L, nm).argtypes = [P, P]
    L.crypto_kem_enc.argtypes = [P, P, P]
    L.crypto_kem_dec.argtypes = [P, P, P]
    L.indcpa_kem_enc.argtypes = [P, P, P, P]
    L.indcpa_kem_dec.argtypes = [P, P, P]
    L.tmvp_set_randombytes.argtypes = [P]
    L.tmvp_set_randombytes.restype = None
    L.tmvp_set_default_param_set.argtypes = [I]
    L.saber_enc.argtypes = [ctypes.c_uint8, P, P, P]
    L.saber_dec.argtypes = [ctypes.c_uint8, P, P, P, P]
    L.SABLE_enc.argtypes = [P, P, P, I]
    L.SABLE_dec.argtypes = [P, P, P, P, I]
    for nm in ("saber_enc", "saber_dec", "SABLE_enc", "SABLE_dec"):
        getattr(L, nm).restype = None
    L.tmvp_ctx_reserve.argtypes = [P, S]
    L.tmvp_ctx_set_host_chunk.argtypes = [P, S]
    L.tmvp_ctx_set_host_ramp.argtypes = [P, ctypes.c_int]
    L.tmvp_selftest_bounded_wait.argtypes = [P, P]
    L.tmvp_diag_umma_rate.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
    L.tmvp_diag_keccak_rate.argtypes = [P, ctypes.c_int, P]
    L.tmvp_ctx_set_dev_chunk.argtypes = [P, S]
    L.tmvp_ctx_set_serial.argtypes = [P, ctypes.c_int]
    L.tmvp_ctx_set_front_cap.argtypes = [P, ctypes.c_int]
    L.tmvp_ctx_set_warp_hash.argtypes = [P, S]
    L.tmvp_ctx_set_pair_hash.argtypes = [P, S]
    L.tmvp_ctx_stage_busy.argtypes = [P, I, ctypes.POINTER(ctypes.c_double)]
    L.tmvp_kem_dec_batch_noalloc.argtypes = [I, S, P, P, P, I, P, P]
    L.tmvp_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(P)]
    L.tmvp_server_destroy.argtypes = [P]
    L.tmvp_server_destroy.restype = None
    L.tmvp_server_add_keys.argtypes = [P, I, S, P, P, P]
    L.tmvp_server_submit.argtypes = [P, I, ctypes.c_uint32, P, P, ctypes.POINTER(ctypes.c_uint64)]
    L.tmvp_server_wait.argtypes = [P, ctypes.c_uint64, I]
    L.tmvp_server_drain.argtypes = [P, I]
    L.tmvp_server_get_stats.argtypes = [P, ctypes.POINTER(ServerStats)]
    L.tmvp_server_reset_stats.argtypes = [P]
    L.tmvp_server_reset_stats.restype = None
    L.tmvp_server_loadgen.argtypes = [P, ctypes.c_double, ctypes.c_double, ctypes.c_uint64, P, S,
                                      ctypes.c_double, ctypes.POINTER(ctypes.c_uint64)]
    L.tmvp_tune_set.argtypes = [I, I, I]
    L.tmvp_tune_get.argtypes = [I, I]
    L.tmvp_autotune.argtypes = [P, I, S, ctypes.POINTER(ctypes.c_int)]
    L.tmvp_tune_pass_set.argtypes = [I, S, ctypes.POINTER(ctypes.c_int)]
    L.tmvp_tune_pass_get.argtypes = [I, S, ctypes.POINTER(ctypes.c_int)]
    L.tmvp_tune_clear.argtypes = []
    L.tmvp_tune_clear.restype = None
    L.tmvp_tune_save.argtypes = [ctypes.c_char_p]
    L.tmvp_tune_load.argtypes = [ctypes.c_char_p]
    L.tmvp_ctx_sync_status.argtypes = [P, P]
    L.tmvp_kem_dec_mixed.argtypes = [P, S, ctypes.POINTER(DecGroup), P]
    L.tmvp_mixed_plan_create.argtypes = [P, S, ctypes.POINTER(DecGroup), ctypes.POINTER(P)]
    L.tmvp_mixed_plan_launch.argtypes = [P, P]
    L.tmvp_mixed_plan_destroy.argtypes = [P]
    L.tmvp_mixed_plan_destroy.restype = None
    L.tmvp_ref_set_batch.argtypes = [I, S]
    L.tmvp_ref_batch.argtypes = [I]
    L.tmvp_ref_batch.restype = S
    _lib = L
    return L


class DecGroup(ctypes.Structure):
    _fields_ = [("set", ctypes.c_int), ("n", ctypes.c_size_t), ("ss", ctypes.c_void_p),
                ("ct", ctypes.c_void_p), ("sk", ctypes.c_void_p)]


STEP_DECRYPT, STEP_ENCRYPT, STEP_REENC, STEP_KEYGEN, STEP_MATVEC = range(5)


def tune_set(step: int, set_id: int, shape: int):
    """Launch shape of a tcgen05 IND-CPA step: -1 one CTA per instance, n >= 0
    the persistent kernel with n CTAs per SM (0 = as many as fit)."""
    _check(lib().tmvp_tune_set(step, set_id, shape), "tmvp_tune_set")


def tune_get(step: int, set_id: int) -> int:
    return lib().tmvp_tune_get(step, set_id)


PASS_FIELDS = ("dev_chunk", "front_cap", "host_chunk", "host_ramp")


def tune_pass_set(set_id: int, n: int, dev_chunk: int, front_cap: int, host_chunk: int, host_ramp: int):
    arr = (ctypes.c_int * 4)(dev_chunk, front_cap, host_chunk, host_ramp)
    _check(lib().tmvp_tune_pass_set(set_id, n, arr), "tmvp_tune_pass_set")


def tune_pass_get(set_id: int, n: int):
    """The autotuner's pass settings for (set, n's batch bucket), or None."""
    arr = (ctypes.c_int * 4)()
    rc = lib().tmvp_tune_pass_get(set_id, n, arr)
    if rc < 0:
        raise TmvpError(rc, "tmvp_tune_pass_get")
    return dict(zip(PASS_FIELDS, list(arr))) if rc == 1 else None


def tune_clear():
    lib().tmvp_tune_clear()


def tune_save(path: str):
    _check(lib().tmvp_tune_save(path.encode()), "tmvp_tune_save")


def tune_load(path: str):
    _check(lib().tmvp_tune_load(path.encode()), "tmvp_tune_load")


def _groups(groups):
    arr = (DecGroup * len(groups))()
    for i, (set_id, ss, ct, sk) in enumerate(groups):
        arr[i] = DecGroup(set_id, ss.shape[0], _ptr(ss), _ptr(ct), _ptr(sk))
    return arr


class MixedPlan:
    """A mixed-parameter decapsulation pass captured into a CUDA graph for
    fixed device buffers (tmvp_mixed_plan)."""

    def __init__(self, ctx, groups):
        self._keep = groups
        h = ctypes.c_void_p()
        arr = _groups(groups)
        _check(lib().tmvp_mixed_plan_create(ctx.h, len(groups), arr, ctypes.byref(h)), "tmvp_mixed_plan_create")
        self.h = h

    def launch(self, stream=None):
        _check(lib().tmvp_mixed_plan_launch(self.h, stream), "tmvp_mixed_plan_launch")

    def close(self):
        if self.h:
            lib().tmvp_mixed_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("mem_budget", ctypes.c_size_t), ("max_batch", ctypes.c_int),
                ("slots", ctypes.c_int), ("form", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("mean_batch", ctypes.c_double),
                ("p50_us", ctypes.c_double), ("p99_us", ctypes.c_double), ("max_us", ctypes.c_double),
                ("elapsed_s", ctypes.c_double), ("throughput", ctypes.c_double), ("slots", ctypes.c_int),
                ("failed", ctypes.c_uint64), ("one_key_batches", ctypes.c_uint64),
                ("arena_bytes", ctypes.c_uint64), ("peak_arena_bytes", ctypes.c_uint64),
                ("admission_waits", ctypes.c_uint64), ("admission_splits", ctypes.c_uint64),
                ("checked", ctypes.c_uint64), ("mismatched", ctypes.c_uint64)]


OP_ENCAPS, OP_DECAPS = 0, 1


def genmatrix_bytes(set_id: int) -> int:
    """Bytes of one key's GenMatrix stream (tmvp_genmatrix_bytes)."""
    return int(lib().tmvp_genmatrix_bytes(set_id))


def sizes(set_id: int) -> Sizes:
    s = Sizes()
    rc = lib().tmvp_param_sizes(set_id, ctypes.byref(s))
    if rc:
        raise TmvpError(rc, "tmvp_param_sizes")
    return s


RANDOMBYTES_FN = ctypes.CFUNCTYPE(None, ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t)


def _ptr(x):
    """Address of a numpy array, a CUDA tensor, or an int device pointer."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        assert x.flags["C_CONTIGUOUS"]
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        assert x.is_contiguous()
        return x.data_ptr()
    raise TypeError(type(x))


def _check(rc: int, what: str):
    if rc != OK:
        raise TmvpError(rc, what)


def _u8(x, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(np.frombuffer(bytes(x), np.uint8) if isinstance(x, (bytes, bytearray))
                             else x)
    if shape is not None:
        a = a.reshape(shape)
    return a


class Context:
    """A libtmvpkem context on one GPU (tmvp_ctx)."""

    def __init__(self, device: int = 0, mem_budget: int = 0):
        h = ctypes.c_void_p()
        _check(lib().tmvp_ctx_create(device, mem_budget, ctypes.byref(h)), "tmvp_ctx_create")
        self.h = h

    def close(self):
        if self.h:
            lib().tmvp_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def workspace_bytes(self) -> int:
        return lib().tmvp_ctx_workspace_bytes(self.h)

    @property
    def launches(self) -> int:
        return lib().tmvp_ctx_launch_count(self.h)

    def set_timing(self, enable: bool):
        _check(lib().tmvp_ctx_set_timing(self.h, int(enable)), "tmvp_ctx_set_timing")

    def stage_stats(self) -> dict:
        """{kernel name: (launches, total device ms)} since timing was enabled."""
        L = lib()
        n = L.tmvp_ctx_stage_stats(self.h, -1, None, 0, None, None)
        out = {}
        for i in range(n):
            name = ctypes.create_string_buffer(64)
            la = ctypes.c_uint64()
            ms = ctypes.c_double()
            _check(L.tmvp_ctx_stage_stats(self.h, i, name, 64, ctypes.byref(la), ctypes.byref(ms)),
                   "tmvp_ctx_stage_stats")
            out[name.value.decode()] = (la.value, ms.value)
        return out

    def stage_busy(self) -> dict:
        """{kernel name: busy device ms} since timing was enabled: the union of
        the stage's launch intervals (overlapping launches counted once)."""
        L = lib()
        n = L.tmvp_ctx_stage_stats(self.h, -1, None, 0, None, None)
        out = {}
        for i in range(n):
            name = ctypes.create_string_buffer(64)
            busy = ctypes.c_double()
            _check(L.tmvp_ctx_stage_stats(self.h, i, name, 64, None, None), "tmvp_ctx_stage_stats")
            _check(L.tmvp_ctx_stage_busy(self.h, i, ctypes.byref(busy)), "tmvp_ctx_stage_busy")
            out[name.value.decode()] = busy.value
        return out

    # --- pointer-level calls (host or device buffers, caller-owned) --------
    def kem_keypair_ptr(self, set_id, n, pk, sk, coins, form=FORM_AUTO, stream=None):
        _check(lib().tmvp_kem_keypair_batch(self.h, set_id, n, _ptr(pk), _ptr(sk), _ptr(coins),
                                            form, stream), "tmvp_kem_keypair_batch")

    def kem_enc_ptr(self, set_id, n, ct, ss, pk, coins, form=FORM_AUTO, stream=None):
        _check(lib().tmvp_kem_enc_batch(self.h, set_id, n, _ptr(ct), _ptr(ss), _ptr(pk),
                                        _ptr(coins), form, stream), "tmvp_kem_enc_batch")

    def kem_dec_ptr(self, set_id, n, ss, ct, sk, form=FORM_AUTO, stream=None):
        _check(lib().tmvp_kem_dec_batch(self.h, set_id, n, _ptr(ss), _ptr(ct), _ptr(sk), form,
                                        stream), "tmvp_kem_dec_batch")

    def genmatrix_ptr(self, set_id, n, a_stream, pk, pk_stride=None, stream=None):
        """a_stream[i] = SHAKE-128(seed_A of pk row i): each key's expanded A (device buffers)."""
        stride = sizes(set_id).pk_bytes if pk_stride is None else pk_stride
        _check(lib().tmvp_genmatrix_batch(self.h, set_id, n, _ptr(a_stream), _ptr(pk), stride, stream),
               "tmvp_genmatrix_batch")

    def kem_enc_a_ptr(self, set_id, n, ct, ss, pk, coins, a_stream, form=FORM_AUTO, stream=None):
        _check(lib().tmvp_kem_enc_batch_a(self.h, set_id, n, _ptr(ct), _ptr(ss), _ptr(pk), _ptr(coins),
                                          _ptr(a_stream), form, stream), "tmvp_kem_enc_batch_a")

    def kem_dec_a_ptr(self, set_id, n, ss, ct, sk, a_stream, form=FORM_AUTO, stream=None):
        _check(lib().tmvp_kem_dec_batch_a(self.h, set_id, n, _ptr(ss), _ptr(ct), _ptr(sk), _ptr(a_stream),
                                          form, stream), "tmvp_kem_dec_batch_a")

    def kem_dec_onekey_ptr(self, set_id, n, ss, ct, sk_one, form=FORM_AUTO, stream=None):
        """n ciphertexts decapsulated under one secret key sk_one (sk_bytes)."""
        _check(lib().tmvp_kem_dec_batch_onekey(self.h, set_id, n, _ptr(ss), _ptr(ct), _ptr(sk_one), form,
                                               stream), "tmvp_kem_dec_batch_onekey")

    def matvec_ptr(self, n, l, eq, transpose, out, A, s, form=FORM_AUTO, stream=None):
        _check(lib().tmvp_matvec_batch(self.h, n, l, eq, int(transpose), _ptr(out), _ptr(A),
                                       _ptr(s), form, stream), "tmvp_matvec_batch")

    def kem_dec_mixed(self, groups, stream=None):
        """groups: [(set_id, ss, ct, sk)] of device tensors; one pass."""
        arr = _groups(groups)
        _check(lib().tmvp_kem_dec_mixed(self.h, len(groups), arr, stream), "tmvp_kem_dec_mixed")

    def set_host_chunk(self, n: int):
        _check(lib().tmvp_ctx_set_host_chunk(self.h, n), "tmvp_ctx_set_host_chunk")

    def umma_rate(self, kind: int, n: int, ctas_per_sm: int = 4, iters: int = 4096):
        """(cycles per MMA of one CTA, of the SM) for tcgen05 kind 0 = f8f6f4, 1 = f16."""
        out = (ctypes.c_double * 2)()
        _check(lib().tmvp_diag_umma_rate(self.h, kind, n, ctas_per_sm, iters, out), "tmvp_diag_umma_rate")
        return out[0], out[1]

    def set_serial(self, on: bool):
        """Run every decapsulation stage alone on the caller's stream (measurement)."""
        _check(lib().tmvp_ctx_set_serial(self.h, int(bool(on))), "tmvp_ctx_set_serial")

    def set_front_cap(self, blocks_per_sm: int):
        """Keccak-front blocks per SM in decapsulation (0 = one thread per sponge)."""
        _check(lib().tmvp_ctx_set_front_cap(self.h, blocks_per_sm), "tmvp_ctx_set_front_cap")

    def set_warp_hash(self, max_sponges: int):
        """Keccak launches of at most max_sponges sponges run one warp per sponge (0: never)."""
        _check(lib().tmvp_ctx_set_warp_hash(self.h, max_sponges), "tmvp_ctx_set_warp_hash")

    def set_pair_hash(self, max_sponges: int):
        """Keccak launches too large for the warp form and of at most max_sponges
        sponges run two threads per sponge (0: never)."""
        _check(lib().tmvp_ctx_set_pair_hash(self.h, max_sponges), "tmvp_ctx_set_pair_hash")

    def keccak_rate(self, perms: int = 64):
        """(Keccak-f[1600] permutations per second at full occupancy, blocks per SM)."""
        out = (ctypes.c_double * 2)()
        _check(lib().tmvp_diag_keccak_rate(self.h, perms, out), "tmvp_diag_keccak_rate")
        return out[0], out[1]

    def set_host_ramp(self, steps: int):
        """First chunks of a host-buffer decapsulation: host_chunk >> steps, ..."""
        _check(lib().tmvp_ctx_set_host_ramp(self.h, steps), "tmvp_ctx_set_host_ramp")

    def set_dev_chunk(self, n: int):
        """Chunk size of device-buffer decapsulation chains (0: one chain)."""
        _check(lib().tmvp_ctx_set_dev_chunk(self.h, n), "tmvp_ctx_set_dev_chunk")

    def sync_status(self, stream=None):
        _check(lib().tmvp_ctx_sync_status(self.h, stream), "tmvp_ctx_sync_status")

    def autotune(self, set_id, n=16384) -> list:
        shapes = (ctypes.c_int * 5)()
        _check(lib().tmvp_autotune(self.h, set_id, n, shapes), "tmvp_autotune")
        return list(shapes)

    # --- numpy conveniences (host buffers) ---------------------------------
    def kem_keypair(self, set_id, coins, form=FORM_AUTO):
        z = sizes(set_id)
        coins = _u8(coins).reshape(-1, 96)
        n = coins.shape[0]
        pk = np.zeros((n, z.pk_bytes), np.uint8)
        sk = np.zeros((n, z.sk_bytes), np.uint8)
        self.kem_keypair_ptr(set_id, n, pk, sk, coins, form)
        return pk, sk

    def kem_enc(self, set_id, pk, coins, form=FORM_AUTO):
        z = sizes(set_id)
        pk = _u8(pk).reshape(-1, z.pk_bytes)
        coins = _u8(coins).reshape(-1, 32)
        n = pk.shape[0]
        ct = np.zeros((n, z.ct_bytes), np.uint8)
        ss = np.zeros((n, 32), np.uint8)
        self.kem_enc_ptr(set_id, n, ct, ss, pk, coins, form)
        return ct, ss

    def kem_dec(self, set_id, ct, sk, form=FORM_AUTO):
        z = sizes(set_id)
        ct = _u8(ct).reshape(-1, z.ct_bytes)
        sk = _u8(sk).reshape(-1, z.sk_bytes)
        n = ct.shape[0]
        ss = np.zeros((n, 32), np.uint8)
        self.kem_dec_ptr(set_id, n, ss, ct, sk, form)
        return ss

    def kem_dec_onekey(self, set_id, ct, sk_one, form=FORM_AUTO):
        z = sizes(set_id)
        ct = _u8(ct).reshape(-1, z.ct_bytes)
        sk_one = _u8(sk_one).reshape(z.sk_bytes)
        n = ct.shape[0]
        ss = np.zeros((n, 32), np.uint8)
        self.kem_dec_onekey_ptr(set_id, n, ss, ct, sk_one, form)
        return ss

    def indcpa_keypair(self, set_id, seeds, form=FORM_AUTO):
        z = sizes(set_id)
        seeds = _u8(seeds).reshape(-1, 64)
        n = seeds.shape[0]
        pk = np.zeros((n, z.pk_bytes), np.uint8)
        sk = np.zeros((n, z.indcpa_sk_bytes), np.uint8)
        _check(lib().tmvp_indcpa_keypair_batch(self.h, set_id, n, _ptr(pk), _ptr(sk), _ptr(seeds),
                                               form, None), "tmvp_indcpa_keypair_batch")
        return pk, sk

    def indcpa_enc(self, set_id, m, noiseseed, pk, form=FORM_AUTO):
        z = sizes(set_id)
        m = _u8(m).reshape(-1, 32)
        ns = _u8(noiseseed).reshape(-1, 32)
        pk = _u8(pk).reshape(-1, z.pk_bytes)
        n = m.shape[0]
        ct = np.zeros((n, z.ct_bytes), np.uint8)
        _check(lib().tmvp_indcpa_enc_batch(self.h, set_id, n, _ptr(ct), _ptr(m), _ptr(ns), _ptr(pk),
                                           form, None), "tmvp_indcpa_enc_batch")
        return ct

    def indcpa_dec(self, set_id, sk, ct, form=FORM_AUTO):
        z = sizes(set_id)
        sk = _u8(sk).reshape(-1, z.indcpa_sk_bytes)
        ct = _u8(ct).reshape(-1, z.ct_bytes)
        n = ct.shape[0]
        m = np.zeros((n, 32), np.uint8)
        _check(lib().tmvp_indcpa_dec_batch(self.h, set_id, n, _ptr(m), _ptr(sk), _ptr(ct), form,
                                           None), "tmvp_indcpa_dec_batch")
        return m

    def matvec(self, A, s, eq=13, transpose=False, form=FORM_AUTO):
        A = np.ascontiguousarray(A, dtype=np.uint16)
        s = np.ascontiguousarray(s, dtype=np.int8)
        n, l = A.shape[0], A.shape[1]
        out = np.zeros((n, l, 256), np.uint16)
        self.matvec_ptr(n, l, eq, transpose, out, A, s, form)
        return out


class Server:
    """The request-serving loop (tmvp_server): device-resident keys,
    continuous batching over several in-flight batch slots."""

    def __init__(self, device=0, mem_budget=0, max_batch=4096, slots=4, form=FORM_AUTO):
        cfg = ServerConfig(device, mem_budget, max_batch, slots, form)
        h = ctypes.c_void_p()
        _check(lib().tmvp_server_create(ctypes.byref(cfg), ctypes.byref(h)), "tmvp_server_create")
        self.h = h

    def close(self):
        if self.h:
            lib().tmvp_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_keys(self, set_id, pk, sk) -> np.ndarray:
        z = sizes(set_id)
        pk = _u8(pk).reshape(-1, z.pk_bytes)
        sk = _u8(sk).reshape(-1, z.sk_bytes)
        ids = np.zeros(pk.shape[0], np.uint32)
        _check(lib().tmvp_server_add_keys(self.h, set_id, pk.shape[0], _ptr(pk), _ptr(sk), _ptr(ids)),
               "tmvp_server_add_keys")
        return ids

    def submit(self, op, key_id, inp: np.ndarray, out: np.ndarray) -> int:
        """inp / out must stay alive until the request completes."""
        t = ctypes.c_uint64()
        _check(lib().tmvp_server_submit(self.h, op, int(key_id), _ptr(inp), _ptr(out), ctypes.byref(t)),
               "tmvp_server_submit")
        return t.value

    def wait(self, ticket, timeout_ms=60000):
        _check(lib().tmvp_server_wait(self.h, ticket, timeout_ms), "tmvp_server_wait")

    def drain(self, timeout_ms=120000):
        _check(lib().tmvp_server_drain(self.h, timeout_ms), "tmvp_server_drain")

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().tmvp_server_get_stats(self.h, ctypes.byref(st)), "tmvp_server_get_stats")
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def reset_stats(self):
        lib().tmvp_server_reset_stats(self.h)

    def loadgen(self, rate, seconds, seed, key_ids, decaps_fraction=0.5) -> int:
        ids = np.ascontiguousarray(key_ids, np.uint32)
        n = ctypes.c_uint64()
        _check(lib().tmvp_server_loadgen(self.h, rate, seconds, seed, _ptr(ids), ids.size,
                                         decaps_fraction, ctypes.byref(n)), "tmvp_server_loadgen")
        return n.value


def splitmix_bytes(seed: int, n: int) -> np.ndarray:
    """Deterministic seed bytes: SplitMix64 stream, little-endian words."""
    nw = (n + 7) // 8
    x = (np.uint64(seed & 0xFFFFFFFFFFFFFFFF) +
         np.arange(1, nw + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15))
    with np.errstate(over="ignore"):
        z = x
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z.astype("<u8").view(np.uint8)[:n].copy()
