"""ctypes binding of the host build of the reference's own kernels.

TEST INFRASTRUCTURE ONLY.  ``oracle/ref_build/Makefile`` compiles the
reference's Saber (l=3) and Sable (l=3) kernel sources as host C++ into
``oracle/_ref/``; the drivers replay the reference's launch sequences one
instance at a time.  The libraries exist only where the reference sources were
available at build time; ``available()`` says whether they do.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REF_DIR = os.path.join(_HERE, "_ref")
_libs: dict = {}

SCHEMES = {"saber": "libref_saber.so", "sable": "libref_sable.so"}


def reference_root() -> str:
    """Where the reference sources are read from: $TMVP_REFERENCE_ROOT, else
    the recipe's own default (``make -C oracle/ref_build print-ref``)."""
    env = os.environ.get("TMVP_REFERENCE_ROOT")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", os.path.join(_HERE, "ref_build"), "print-ref"],
                       capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def build(ref_root: str | None = None) -> bool:
    """Compile the reference kernels from ``ref_root`` (default:
    reference_root()); False if the sources are absent."""
    ref_root = ref_root or reference_root()
    if not ref_root or not os.path.isdir(ref_root):
        return False
    subprocess.run(["make", "-s", "-C", os.path.join(_HERE, "ref_build"), f"REF={ref_root}"],
                   check=True)
    return True


def available(scheme: str = "saber") -> bool:
    return os.path.exists(os.path.join(_REF_DIR, SCHEMES[scheme]))


def lib(scheme: str):
    if scheme not in _libs:
        L = ctypes.CDLL(os.path.join(_REF_DIR, SCHEMES[scheme]))
        P = ctypes.c_void_p
        pre = f"ref_{scheme}_"
        getattr(L, pre + "sha3_256").argtypes = [P, P, ctypes.c_size_t]
        getattr(L, pre + "sha3_512").argtypes = [P, P]
        getattr(L, pre + "shake128").argtypes = [P, ctypes.c_size_t, P, ctypes.c_size_t]
        getattr(L, pre + "genmatrix").argtypes = [P, P]
        getattr(L, pre + "gensecret").argtypes = [P, P]
        getattr(L, pre + "matvec").argtypes = [ctypes.c_int, P, P, P]
        getattr(L, pre + "enc").argtypes = [ctypes.c_int, P, P, P, P]
        getattr(L, pre + "dec").argtypes = [ctypes.c_int, P, P, P, P]
        getattr(L, pre + "dec").restype = ctypes.c_int
        if scheme == "sable":
            L.ref_sable_polmul.argtypes = [P, P, P, ctypes.c_uint16]
        _libs[scheme] = L
    return _libs[scheme]


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _u8(b) -> np.ndarray:
    return np.ascontiguousarray(np.frombuffer(bytes(b), dtype=np.uint8))


SIZES = {"saber": dict(l=3, pk=992, sk=2304, ct=1088),
         "sable": dict(l=3, pk=896, sk=1152, ct=1024)}


def genmatrix(scheme: str, seed) -> np.ndarray:
    l = SIZES[scheme]["l"]
    A = np.zeros((l, l, 256), np.uint16)
    getattr(lib(scheme), f"ref_{scheme}_genmatrix")(_p(A), _p(_u8(seed)))
    return A


def gensecret(scheme: str, seed) -> np.ndarray:
    l = SIZES[scheme]["l"]
    s = np.zeros((l, 256), np.uint16)
    getattr(lib(scheme), f"ref_{scheme}_gensecret")(_p(s), _p(_u8(seed)))
    return s


def matvec(scheme: str, mode: int, A: np.ndarray, s: np.ndarray) -> np.ndarray:
    """Raw A*s over Z_2^16 with the reference's mode-1 TMVP or mode-2 schoolbook kernels."""
    A = np.ascontiguousarray(A, dtype=np.uint16)
    s = np.ascontiguousarray(s, dtype=np.uint16)
    out = np.zeros((A.shape[0], 256), np.uint16)
    getattr(lib(scheme), f"ref_{scheme}_matvec")(mode, _p(out), _p(A), _p(s))
    return out


def enc(scheme: str, mode: int, pk, coins):
    z = SIZES[scheme]
    ct = np.zeros(z["ct"], np.uint8)
    k = np.zeros(32, np.uint8)
    getattr(lib(scheme), f"ref_{scheme}_enc")(mode, _p(ct), _p(k), _p(_u8(pk)), _p(_u8(coins)))
    return ct.tobytes(), k.tobytes()


def dec(scheme: str, mode: int, ct, sk):
    z = SIZES[scheme]
    k = np.zeros(32, np.uint8)
    cmp = np.zeros(z["ct"], np.uint8)
    diff = getattr(lib(scheme), f"ref_{scheme}_dec")(mode, _p(k), _p(cmp), _p(_u8(ct)),
                                                      _p(_u8(sk)))
    return k.tobytes(), cmp.tobytes(), int(diff)
