"""The CPU oracle against independent hashes and the reference's own test vectors."""
import hashlib
import os

import numpy as np
import pytest

from conftest import golden

SETS = range(6)


@pytest.mark.parametrize("n", [0, 1, 7, 8, 31, 32, 71, 72, 135, 136, 137, 167, 168, 169, 1088, 3000])
def test_hashes_match_hashlib(oracle, n):
    d = np.random.default_rng(n).integers(0, 256, n, dtype=np.uint8).tobytes()
    assert oracle.sha3_256(d) == hashlib.sha3_256(d).digest()
    assert oracle.sha3_512(d) == hashlib.sha3_512(d).digest()
    for ol in (1, 32, 168, 169, 3744):
        assert oracle.shake128(d, ol) == hashlib.shake_128(d).digest(ol)


def test_saber_test_vectors(oracle):
    g = golden("saber_l3.npz")
    pk, sk, buf = g["tv_pk"].tobytes(), g["tv_sk"].tobytes(), g["tv_buf"].tobytes()
    # tv.h:4 A = GenMatrix(seed_A)
    A = oracle.gen_matrix(oracle.SABER, pk[-32:])
    assert np.array_equal(A.reshape(-1), g["tv_A"])
    # tv.h:9 m_tv = SHA3-256(buf[0:32])
    assert oracle.sha3_256(buf[:32]) == g["tv_m"].tobytes()
    # sk = s || pk || H(pk) || z
    p = oracle.params(oracle.SABER)
    assert sk[p.indcpa_sk_bytes:p.indcpa_sk_bytes + p.pk_bytes] == pk
    assert sk[-64:-32] == oracle.sha3_256(pk)
    # encapsulation/decapsulation of the test vectors equal the reference kernels' output
    ct, ss = oracle.kem_enc(oracle.SABER, pk, buf[:32])
    assert ct == g["tv_ct"].tobytes() and ss == g["tv_ss"].tobytes()
    ss2, fail = oracle.kem_dec(oracle.SABER, ct, sk)
    assert ss2 == ss and fail == 0


def test_sable_test_vectors(oracle):
    g = golden("sable_l3.npz")
    pk, sk, buf = g["tv_pk"].tobytes(), g["tv_sk"].tobytes(), g["tv_buf"].tobytes()
    m = oracle.sha3_256(buf[:32])
    assert m == g["tv_m"].tobytes()
    # tv.h:17 kr = G(H(buf) || H(pk))
    assert oracle.sha3_512(m + oracle.sha3_256(pk)) == g["tv_kr"].tobytes()
    ct, ss = oracle.kem_enc(oracle.SABLE, pk, buf[:32])
    assert ct == g["tv_ct"].tobytes() and ss == g["tv_ss"].tobytes()
    assert oracle.kem_dec(oracle.SABLE, ct, sk) == (ss, 0)


@pytest.mark.parametrize("name,set_id", [("saber_l3.npz", 1), ("sable_l3.npz", 4)])
def test_test_keys_are_transposed_matvec(oracle, name, set_id):
    """pk = pack_p(round(A^T s)) for the reference's test keys (keypair convention)."""
    g = golden(name)
    pk, sk = g["tv_pk"].tobytes(), g["tv_sk"].tobytes()
    p = oracle.params(set_id)
    A = oracle.gen_matrix(set_id, pk[-32:])
    if p.sable:
        s = [((oracle.unpack_bits(sk[64 * j:64 * j + 64], 256, 2) ^ 2) - 2).astype(np.uint16) for j in range(p.l)]
    else:
        s = [oracle.unpack_bits(sk[p.polybytes * j:p.polybytes * (j + 1)], 256, p.eq) for j in range(p.l)]
    for transpose, expect in ((True, True), (False, False)):
        out = []
        for i in range(p.l):
            acc = np.zeros(256, np.uint16)
            for j in range(p.l):
                acc = (acc + oracle.polmul(A[j][i] if transpose else A[i][j], s[j])).astype(np.uint16)
            b = (((acc.astype(np.int64) + p.h1) & ((1 << p.eq) - 1)) >> (p.eq - p.ep)).astype(np.uint16)
            out.append(oracle.pack_bits(b, p.ep))
        assert (b"".join(out) == pk[:-32]) == expect


@pytest.mark.parametrize("name,set_id", [("saber_l3.npz", 1), ("sable_l3.npz", 4)])
def test_reference_kernel_outputs(oracle, name, set_id):
    """Seeded instances produced by the reference's own kernels decapsulate identically."""
    g = golden(name)
    for i in range(g["rnd_ct"].shape[0]):
        ct, ss = oracle.kem_enc(set_id, g["rnd_pk"][i], g["rnd_coins"][i])
        assert ct == g["rnd_ct"][i].tobytes() and ss == g["rnd_ss"][i].tobytes()
        assert oracle.kem_dec(set_id, ct, g["rnd_sk"][i]) == (ss, 0)
    ss, fail = oracle.kem_dec(set_id, g["rej_ct"], g["rnd_sk"][0])
    assert fail == 1 and ss == g["rej_ss"].tobytes()


def test_matvec_golden(oracle):
    g = golden("matvec.npz")
    for scheme, eq in (("saber", 13), ("sable", 11)):
        out = oracle.matvec(g[f"{scheme}_A"], g[f"{scheme}_s"], eq=eq)
        assert np.array_equal(out, g[f"{scheme}_out"])


def test_tmvp2_equals_schoolbook(oracle):
    rng = np.random.default_rng(3)
    for _ in range(10):
        a = rng.integers(0, 65536, 256, dtype=np.uint16)
        b = rng.integers(0, 65536, 256, dtype=np.uint16)
        assert np.array_equal(oracle.polmul(a, b), oracle.polmul(a, b, "tmvp2"))
    # negacyclic identity: x^255 * x = -1
    x = np.zeros(256, np.uint16); x[1] = 1
    y = np.zeros(256, np.uint16); y[255] = 1
    r = oracle.polmul(x, y)
    assert r[0] == 65535 and not r[1:].any()


def test_toom4_equals_schoolbook(oracle):
    """The Toom-Cook 4-way restatement (mod 2^32 evaluation and interpolation)
    gives the schoolbook product mod 2^16 for any 16-bit operands, including
    the extremes that maximise every evaluation."""
    rng = np.random.default_rng(4)
    cases = [(rng.integers(0, 65536, 256, dtype=np.uint16), rng.integers(0, 65536, 256, dtype=np.uint16))
             for _ in range(10)]
    cases.append((np.full(256, 65535, np.uint16), np.full(256, 65535, np.uint16)))
    cases.append((np.full(256, 8191, np.uint16), (-rng.integers(0, 6, 256)).astype(np.uint16)))
    for a, b in cases:
        assert np.array_equal(oracle.polmul(a, b), oracle.polmul(a, b, "toom4"))
        # 16-bit products (as in the reference's pol_mul): right mod 2^13
        assert np.array_equal(oracle.polmul(a, b) & 8191, oracle.polmul(a, b, "toom4k") & 8191)


@pytest.mark.parametrize("set_id", SETS)
def test_toom4k_kem_equals_schoolbook_kem(oracle, set_id):
    """The CPU baseline's multiplication (Toom-Cook 4-way with Karatsuba, the
    reference's serial pol_mul) gives the schoolbook KEM's bytes: keys,
    ciphertexts, shared secrets and implicit rejection."""
    rng = np.random.default_rng(300 + set_id)
    coins = rng.integers(0, 256, (6, 96), dtype=np.uint8)
    ec = rng.integers(0, 256, (6, 32), dtype=np.uint8)
    pk, sk = oracle.kem_keypair_batch(set_id, coins)
    ct, ss = oracle.kem_enc_batch(set_id, pk, ec)
    ct[2, 5] ^= 1
    ss_d, fail = oracle.kem_dec_batch(set_id, ct, sk)
    try:
        oracle.set_polmul(oracle.POLMUL_TOOM4K)
        pk2, sk2 = oracle.kem_keypair_batch(set_id, coins, 2)
        ct2, ss2 = oracle.kem_enc_batch(set_id, pk2, ec, 2)
        ct2[2, 5] ^= 1
        ss_d2, fail2 = oracle.kem_dec_batch(set_id, ct2, sk2, 2)
    finally:
        oracle.set_polmul(oracle.POLMUL_SCHOOLBOOK)
    assert np.array_equal(pk, pk2) and np.array_equal(sk, sk2)
    assert np.array_equal(ct, ct2) and np.array_equal(ss, ss2)
    assert np.array_equal(ss_d, ss_d2) and np.array_equal(fail, fail2) and fail.tolist() == [0, 0, 1, 0, 0, 0]


def test_single_instance_latency_timer(oracle):
    """orc_kem_latency times single calls (the batch-1 CPU configuration) and
    checks each decapsulation against its encapsulation."""
    for op in ("keypair", "enc", "dec"):
        ns = oracle.kem_latency_ns(oracle.SABER, op, 5)
        assert ns.shape == (5,) and (ns > 0).all()


@pytest.mark.parametrize("w", [1, 2, 3, 4, 5, 6, 9, 10, 11, 13])
def test_pack_roundtrip(oracle, w):
    v = np.random.default_rng(w).integers(0, 1 << w, 256, dtype=np.uint16)
    assert np.array_equal(oracle.unpack_bits(oracle.pack_bits(v, w), 256, w), v)


@pytest.mark.parametrize("set_id", SETS)
def test_kem_roundtrip_and_rejection(oracle, set_id):
    rng = np.random.default_rng(100 + set_id)
    for _ in range(3):
        pk, sk = oracle.kem_keypair(set_id, rng.integers(0, 256, 96, dtype=np.uint8))
        ct, ss = oracle.kem_enc(set_id, pk, rng.integers(0, 256, 32, dtype=np.uint8))
        assert oracle.kem_dec(set_id, ct, sk) == (ss, 0)
        bad = bytearray(ct)
        bad[-1] ^= 0x80
        ss2, fail = oracle.kem_dec(set_id, bytes(bad), sk)
        assert fail == 1 and ss2 != ss


@pytest.mark.parametrize("set_id", SETS)
def test_secret_ranges(oracle, set_id):
    p = oracle.params(set_id)
    s = oracle.gen_secret(set_id, bytes(range(32))).astype(np.int64)
    if p.sable:
        s = np.where(s >= (1 << (p.eq - 1)), s - (1 << p.eq), s)
    else:
        s = np.where(s >= 32768, s - 65536, s)
    assert np.abs(s).max() <= p.mu // 2


def test_batch_threads_match_serial(oracle):
    coins = np.random.default_rng(9).integers(0, 256, (12, 96), dtype=np.uint8)
    pk1, sk1 = oracle.kem_keypair_batch(oracle.SABER, coins, nthreads=1)
    pk4, sk4 = oracle.kem_keypair_batch(oracle.SABER, coins, nthreads=4)
    assert np.array_equal(pk1, pk4) and np.array_equal(sk1, sk4)
    ec = np.random.default_rng(10).integers(0, 256, (12, 32), dtype=np.uint8)
    ct, ss = oracle.kem_enc_batch(oracle.SABER, pk1, ec, nthreads=3)
    ss2, fail = oracle.kem_dec_batch(oracle.SABER, ct, sk1, nthreads=4)
    assert np.array_equal(ss, ss2) and not fail.any()
