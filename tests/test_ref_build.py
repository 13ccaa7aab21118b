"""The oracle against a host build of the reference's own kernels (only where
the reference sources are available to build it)."""
import os

import numpy as np
import pytest

from oracle import pyref

REF = pyref.reference_root()

pytestmark = pytest.mark.skipif(
    not (pyref.available("saber") or (REF and os.path.isdir(REF))),
    reason="reference sources not present; golden fixtures cover this case")


@pytest.fixture(scope="module")
def ref():
    if not (pyref.available("saber") and pyref.available("sable")):
        pyref.build(REF)
    return pyref


@pytest.mark.parametrize("scheme,set_id", [("saber", 1), ("sable", 4)])
def test_kem_vs_reference_kernels(oracle, ref, scheme, set_id):
    rng = np.random.default_rng(7 + set_id)
    for mode in (1, 2):
        pk, sk = oracle.kem_keypair(set_id, rng.integers(0, 256, 96, dtype=np.uint8))
        coins = rng.integers(0, 256, 32, dtype=np.uint8).tobytes()
        ct, k = ref.enc(scheme, mode, pk, coins)
        assert (ct, k) == oracle.kem_enc(set_id, pk, coins)
        kd, cmp, diff = ref.dec(scheme, mode, ct, sk)
        assert kd == k and cmp == ct and diff == 0
        assert oracle.kem_dec(set_id, ct, sk) == (k, 0)


@pytest.mark.parametrize("scheme,set_id,eq", [("saber", 1, 13), ("sable", 4, 11)])
def test_matvec_and_sampling_vs_reference(oracle, ref, scheme, set_id, eq):
    rng = np.random.default_rng(eq)
    seed = rng.integers(0, 256, 32, dtype=np.uint8)
    assert np.array_equal(ref.genmatrix(scheme, seed), oracle.gen_matrix(set_id, seed))
    assert np.array_equal(ref.gensecret(scheme, seed), oracle.gen_secret(set_id, seed))
    A = rng.integers(0, 1 << eq, (3, 3, 256), dtype=np.uint16)
    s = rng.integers(-4, 5, (3, 256)).astype(np.int8)
    want = oracle.matvec(A[None], s[None], eq=eq)[0]
    for mode in (1, 2):
        got = ref.matvec(scheme, mode, A, s.astype(np.int16).astype(np.uint16)) & ((1 << eq) - 1)
        assert np.array_equal(got, want)
