"""ctypes binding of the CPU oracle (oracle/tmvp_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the tests, by ``__graft_entry__.smoke``
and by the CPU-baseline leg of ``bench.py`` as the checker.  The product
(the CUDA library and its Python mirror) never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libtmvp_oracle.so")
_lib = None

LIGHTSABER, SABER, FIRESABER, LIGHTSABLE, SABLE, FIRESABLE = range(6)
SET_NAMES = ["LightSaber", "Saber", "FireSaber", "LightSable", "Sable", "FireSable"]


class Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "l", "eq", "ep", "et", "mu", "sable", "polybytes", "polyvecbytes",
        "polycompbytes", "scalebytes", "coinbytes", "pk_bytes", "indcpa_sk_bytes",
        "sk_bytes", "ct_bytes", "h1", "h2")]


def build() -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        L.orc_get_params.argtypes = [ctypes.c_int, ctypes.POINTER(Params)]
        for name in ("orc_sha3_256", "orc_sha3_512"):
            getattr(L, name).argtypes = [P, P, ctypes.c_size_t]
        L.orc_shake128.argtypes = [P, ctypes.c_size_t, P, ctypes.c_size_t]
        L.orc_gen_matrix.argtypes = [ctypes.c_int, P, P]
        L.orc_gen_secret.argtypes = [ctypes.c_int, P, P]
        L.orc_pack_bits.argtypes = [P, P, ctypes.c_int, ctypes.c_int]
        L.orc_unpack_bits.argtypes = [P, P, ctypes.c_int, ctypes.c_int]
        L.orc_polmul_schoolbook.argtypes = [P, P, P]
        L.orc_polmul_tmvp2.argtypes = [P, P, P]
        L.orc_polmul_toom4.argtypes = [P, P, P]
        L.orc_polmul_toom4k.argtypes = [P, P, P]
        L.orc_set_polmul.argtypes = [ctypes.c_int]
        L.orc_kem_latency.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        L.orc_matvec_batch.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       P, P, P, ctypes.c_int]
        L.orc_indcpa_keypair.argtypes = [ctypes.c_int, P, P, P, P]
        L.orc_indcpa_enc.argtypes = [ctypes.c_int, P, P, P, P]
        L.orc_indcpa_dec.argtypes = [ctypes.c_int, P, P, P]
        L.orc_kem_keypair.argtypes = [ctypes.c_int, P, P, P]
        L.orc_kem_enc.argtypes = [ctypes.c_int, P, P, P, P]
        L.orc_kem_dec.argtypes = [ctypes.c_int, P, P, P]
        L.orc_kem_dec.restype = ctypes.c_int
        L.orc_kem_keypair_batch.argtypes = [ctypes.c_int, ctypes.c_size_t, P, P, P, ctypes.c_int]
        L.orc_kem_enc_batch.argtypes = [ctypes.c_int, ctypes.c_size_t, P, P, P, P, ctypes.c_int]
        L.orc_kem_dec_batch.argtypes = [ctypes.c_int, ctypes.c_size_t, P, P, P, P, ctypes.c_int]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def params(set_id: int) -> Params:
    p = Params()
    if lib().orc_get_params(set_id, ctypes.byref(p)) != 0:
        raise ValueError(f"bad parameter set {set_id}")
    return p


def _u8(b) -> np.ndarray:
    return np.ascontiguousarray(np.frombuffer(bytes(b), dtype=np.uint8)) if not isinstance(
        b, np.ndarray) else np.ascontiguousarray(b, dtype=np.uint8)


def sha3_256(data) -> bytes:
    d = _u8(data)
    out = np.zeros(32, np.uint8)
    lib().orc_sha3_256(_p(out), _p(d), d.size)
    return out.tobytes()


def sha3_512(data) -> bytes:
    d = _u8(data)
    out = np.zeros(64, np.uint8)
    lib().orc_sha3_512(_p(out), _p(d), d.size)
    return out.tobytes()


def shake128(data, outlen: int) -> bytes:
    d = _u8(data)
    out = np.zeros(outlen, np.uint8)
    lib().orc_shake128(_p(out), outlen, _p(d), d.size)
    return out.tobytes()


def gen_matrix(set_id: int, seed) -> np.ndarray:
    p = params(set_id)
    A = np.zeros((p.l, p.l, 256), np.uint16)
    lib().orc_gen_matrix(set_id, _p(A), _p(_u8(seed)))
    return A


def gen_secret(set_id: int, seed) -> np.ndarray:
    p = params(set_id)
    s = np.zeros((p.l, 256), np.uint16)
    lib().orc_gen_secret(set_id, _p(s), _p(_u8(seed)))
    return s


def pack_bits(vals: np.ndarray, w: int) -> bytes:
    v = np.ascontiguousarray(vals, dtype=np.uint16)
    out = np.zeros((v.size * w + 7) // 8, np.uint8)
    lib().orc_pack_bits(_p(out), _p(v), v.size, w)
    return out.tobytes()


def unpack_bits(data, n: int, w: int) -> np.ndarray:
    d = _u8(data)
    out = np.zeros(n, np.uint16)
    lib().orc_unpack_bits(_p(out), _p(d), n, w)
    return out


def polmul(a: np.ndarray, b: np.ndarray, method: str = "schoolbook") -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint16)
    b = np.ascontiguousarray(b, dtype=np.uint16)
    r = np.zeros(256, np.uint16)
    fn = {"schoolbook": lib().orc_polmul_schoolbook, "tmvp2": lib().orc_polmul_tmvp2,
          "toom4": lib().orc_polmul_toom4, "toom4k": lib().orc_polmul_toom4k}[method]
    fn(_p(r), _p(a), _p(b))
    return r


POLMUL_SCHOOLBOOK, POLMUL_TOOM4K = 0, 1


def set_polmul(which: int) -> None:
    """Multiplication of the IND-CPA / KEM functions: POLMUL_SCHOOLBOOK (the
    default, used for parity) or POLMUL_TOOM4K (Toom-Cook 4-way with two
    Karatsuba levels, the reference's serial pol_mul; the CPU baseline)."""
    if lib().orc_set_polmul(which) != 0:
        raise ValueError(f"unknown multiplication {which}")


def kem_latency_ns(set_id: int, op: str, iters: int) -> np.ndarray:
    """Per-call wall time in ns of `iters` single-instance keypair / enc / dec
    calls on the calling thread (timed in C with CLOCK_MONOTONIC)."""
    ns = np.zeros(iters, np.float64)
    rc = lib().orc_kem_latency(set_id, {"keypair": 0, "enc": 1, "dec": 2}[op], iters, _p(ns))
    if rc != 0:
        raise RuntimeError(f"orc_kem_latency failed ({rc})")
    return ns


def matvec(A: np.ndarray, s: np.ndarray, eq: int = 13, transpose: bool = False,
           nthreads: int = 1) -> np.ndarray:
    """A: uint16 [n][l][l][256], s: int8 [n][l][256] -> uint16 [n][l][256] mod 2^eq."""
    A = np.ascontiguousarray(A, dtype=np.uint16)
    s = np.ascontiguousarray(s, dtype=np.int8)
    n, l = A.shape[0], A.shape[1]
    out = np.zeros((n, l, 256), np.uint16)
    lib().orc_matvec_batch(n, l, eq, int(transpose), _p(out), _p(A), _p(s), nthreads)
    return out


def indcpa_keypair(set_id: int, seed_a, seed_s):
    p = params(set_id)
    pk = np.zeros(p.pk_bytes, np.uint8)
    sk = np.zeros(p.indcpa_sk_bytes, np.uint8)
    lib().orc_indcpa_keypair(set_id, _p(pk), _p(sk), _p(_u8(seed_a)), _p(_u8(seed_s)))
    return pk.tobytes(), sk.tobytes()


def indcpa_enc(set_id: int, m, noiseseed, pk) -> bytes:
    p = params(set_id)
    ct = np.zeros(p.ct_bytes, np.uint8)
    lib().orc_indcpa_enc(set_id, _p(ct), _p(_u8(m)), _p(_u8(noiseseed)), _p(_u8(pk)))
    return ct.tobytes()


def indcpa_dec(set_id: int, sk_indcpa, ct) -> bytes:
    m = np.zeros(32, np.uint8)
    lib().orc_indcpa_dec(set_id, _p(m), _p(_u8(sk_indcpa)), _p(_u8(ct)))
    return m.tobytes()


def kem_keypair(set_id: int, coins):
    p = params(set_id)
    pk = np.zeros(p.pk_bytes, np.uint8)
    sk = np.zeros(p.sk_bytes, np.uint8)
    lib().orc_kem_keypair(set_id, _p(pk), _p(sk), _p(_u8(coins)))
    return pk.tobytes(), sk.tobytes()


def kem_enc(set_id: int, pk, coins):
    p = params(set_id)
    ct = np.zeros(p.ct_bytes, np.uint8)
    ss = np.zeros(32, np.uint8)
    lib().orc_kem_enc(set_id, _p(ct), _p(ss), _p(_u8(pk)), _p(_u8(coins)))
    return ct.tobytes(), ss.tobytes()


def kem_dec(set_id: int, ct, sk):
    ss = np.zeros(32, np.uint8)
    fail = lib().orc_kem_dec(set_id, _p(ss), _p(_u8(ct)), _p(_u8(sk)))
    return ss.tobytes(), int(fail)


def kem_keypair_batch(set_id: int, coins: np.ndarray, nthreads: int = 1):
    p = params(set_id)
    n = coins.shape[0]
    pk = np.zeros((n, p.pk_bytes), np.uint8)
    sk = np.zeros((n, p.sk_bytes), np.uint8)
    lib().orc_kem_keypair_batch(set_id, n, _p(pk), _p(sk), _p(np.ascontiguousarray(coins)), nthreads)
    return pk, sk


def kem_enc_batch(set_id: int, pk: np.ndarray, coins: np.ndarray, nthreads: int = 1):
    p = params(set_id)
    n = pk.shape[0]
    ct = np.zeros((n, p.ct_bytes), np.uint8)
    ss = np.zeros((n, 32), np.uint8)
    lib().orc_kem_enc_batch(set_id, n, _p(ct), _p(ss), _p(np.ascontiguousarray(pk)),
                            _p(np.ascontiguousarray(coins)), nthreads)
    return ct, ss


def kem_dec_batch(set_id: int, ct: np.ndarray, sk: np.ndarray, nthreads: int = 1):
    n = ct.shape[0]
    ss = np.zeros((n, 32), np.uint8)
    fail = np.zeros(n, np.uint8)
    lib().orc_kem_dec_batch(set_id, n, _p(ss), _p(np.ascontiguousarray(ct)),
                            _p(np.ascontiguousarray(sk)), _p(fail), nthreads)
    return ss, fail
