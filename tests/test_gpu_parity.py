"""CUDA library vs the oracle, bit-exact, through the C ABI (needs a GB300)."""
import ctypes

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

ALL_FORMS = [0, 1, 2, 4, 5, 6, 7]  # cuda_core, int8_tc, fp8_tc, schoolbook, fp8_tcgen05, dp2a, toom_cook
SETS = range(6)


def _coins(seed, n, w):
    import tmvpkem
    return tmvpkem.splitmix_bytes(seed, n * w).reshape(n, w)


@pytest.mark.parametrize("form", ALL_FORMS)
@pytest.mark.parametrize("l,eq,transpose", [(2, 13, 0), (3, 13, 0), (3, 13, 1), (4, 13, 0),
                                             (3, 11, 0), (4, 11, 1), (2, 10, 0)])
def test_matvec_random(kem, oracle, form, l, eq, transpose):
    T, ctx = kem
    rng = np.random.default_rng(l * 100 + eq + transpose)
    n = 40
    A = rng.integers(0, 1 << eq, (n, l, l, 256), dtype=np.uint16)
    s = rng.integers(-5, 6, (n, l, 256)).astype(np.int8)
    got = ctx.matvec(A, s, eq=eq, transpose=bool(transpose), form=form)
    want = oracle.matvec(A, s, eq=eq, transpose=bool(transpose), nthreads=4)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("form", ALL_FORMS)
def test_matvec_extremes(kem, oracle, form):
    """Largest exact inputs: |s| = 7 everywhere (the tensor-core forms' limit)
    and public values at the digit boundaries, so every accumulator reaches
    its bound."""
    T, ctx = kem
    n, l, eq = 12, 4, 13
    vals = np.array([0, 1, 7, 8, 15, 16, 17, 31, 32, 511, 512, 4095, 4096, 4097, 8176, 8191], np.uint16)
    rng = np.random.default_rng(5)
    A = vals[rng.integers(0, len(vals), (n, l, l, 256))]
    s = np.where(rng.integers(0, 2, (n, l, 256)) == 1, 7, -7).astype(np.int8)
    A[0] = 4096
    s[0] = -7
    A[1] = 8191
    s[1] = 7
    got = ctx.matvec(A, s, eq=eq, form=form)
    assert np.array_equal(got, oracle.matvec(A, s, eq=eq, nthreads=4))


@pytest.mark.parametrize("form", [0, 4, 7])
def test_matvec_wide_secrets_cuda_core(kem, oracle, form):
    """The IMAD CUDA-core forms (TMVP, schoolbook, Toom-Cook) take any int8
    secret."""
    T, ctx = kem
    rng = np.random.default_rng(6)
    A = rng.integers(0, 1 << 13, (8, 3, 3, 256), dtype=np.uint16)
    s = rng.integers(-128, 128, (8, 3, 256)).astype(np.int8)
    assert np.array_equal(ctx.matvec(A, s, eq=13, form=form), oracle.matvec(A, s, eq=13, nthreads=4))


def test_matvec_dp2a_limits(kem, oracle):
    """dp2a multiplies signed bytes of the TMVP operands (differences of two
    secret coefficients), exact for |s| <= 63: the largest secrets with the
    largest public values of every width."""
    T, ctx = kem
    rng = np.random.default_rng(7)
    for eq in (13, 11, 10):
        A = rng.integers(0, 1 << eq, (10, 4, 4, 256), dtype=np.uint16)
        A[:4] = (1 << eq) - 1
        s = np.where(rng.integers(0, 2, (10, 4, 256)) == 1, 63, -63).astype(np.int8)
        s[5:] = rng.integers(-63, 64, (5, 4, 256))
        got = ctx.matvec(A, s, eq=eq, form=T.FORM_DP2A)
        assert np.array_equal(got, oracle.matvec(A, s, eq=eq, nthreads=4))


@pytest.mark.parametrize("form", ALL_FORMS)
def test_matvec_golden(kem, form):
    T, ctx = kem
    g = golden("matvec.npz")
    for scheme, eq in (("saber", 13), ("sable", 11)):
        out = ctx.matvec(g[f"{scheme}_A"], g[f"{scheme}_s"], eq=eq, form=form)
        assert np.array_equal(out, g[f"{scheme}_out"])


@pytest.mark.parametrize("form", ALL_FORMS)
@pytest.mark.parametrize("set_id", SETS)
def test_kem_parity(kem, oracle, set_id, form):
    T, ctx = kem
    n = 24
    kc = _coins(1000 + set_id, n, 96)
    pk, sk = ctx.kem_keypair(set_id, kc, form=form)
    opk, osk = oracle.kem_keypair_batch(set_id, kc, nthreads=4)
    assert np.array_equal(pk, opk) and np.array_equal(sk, osk)
    ec = _coins(2000 + set_id, n, 32)
    ct, ss = ctx.kem_enc(set_id, pk, ec, form=form)
    oct_, oss = oracle.kem_enc_batch(set_id, opk, ec, nthreads=4)
    assert np.array_equal(ct, oct_) and np.array_equal(ss, oss)
    ss2 = ctx.kem_dec(set_id, ct, sk, form=form)
    assert np.array_equal(ss2, ss)
    # tampered ciphertexts: implicit rejection, same key as the oracle
    bad = ct.copy()
    rng = np.random.default_rng(set_id)
    for i in range(n):
        if i % 2 == 0:
            bad[i, rng.integers(0, bad.shape[1])] ^= np.uint8(1 << rng.integers(0, 8))
    ss3 = ctx.kem_dec(set_id, bad, sk, form=form)
    oss3, fail = oracle.kem_dec_batch(set_id, bad, osk, nthreads=4)
    assert np.array_equal(ss3, oss3)
    assert fail[::2].all() and not fail[1::2].any()
    assert (ss3[::2] != ss[::2]).any(axis=1).all()


@pytest.mark.parametrize("form", ALL_FORMS)
@pytest.mark.parametrize("name,set_id", [("saber_l3.npz", 1), ("sable_l3.npz", 4)])
def test_reference_golden(kem, name, set_id, form):
    """Test vectors and seeded instances produced by the reference's own kernels."""
    T, ctx = kem
    g = golden(name)
    ct, ss = ctx.kem_enc(set_id, g["tv_pk"], g["tv_buf"][:32], form=form)
    assert ct[0].tobytes() == g["tv_ct"].tobytes() and ss[0].tobytes() == g["tv_ss"].tobytes()
    assert ctx.kem_dec(set_id, ct, g["tv_sk"], form=form)[0].tobytes() == g["tv_ss"].tobytes()
    ct, ss = ctx.kem_enc(set_id, g["rnd_pk"], g["rnd_coins"], form=form)
    assert np.array_equal(ct, g["rnd_ct"]) and np.array_equal(ss, g["rnd_ss"])
    assert np.array_equal(ctx.kem_dec(set_id, g["rnd_ct"], g["rnd_sk"], form=form), g["rnd_ss"])
    rej = ctx.kem_dec(set_id, g["rej_ct"], g["rnd_sk"][0], form=form)
    assert rej[0].tobytes() == g["rej_ss"].tobytes()


@pytest.mark.parametrize("form", [0, 2, 5, 6, 7])
@pytest.mark.parametrize("set_id", [1, 4])
def test_indcpa_parity(kem, oracle, set_id, form):
    T, ctx = kem
    n = 8
    seeds = _coins(77, n, 64)
    pk, sk = ctx.indcpa_keypair(set_id, seeds, form=form)
    for i in range(n):
        opk, osk = oracle.indcpa_keypair(set_id, seeds[i, :32], seeds[i, 32:])
        assert pk[i].tobytes() == opk and sk[i].tobytes() == osk
    m = _coins(78, n, 32)
    ns = _coins(79, n, 32)
    ct = ctx.indcpa_enc(set_id, m, ns, pk, form=form)
    for i in range(n):
        assert ct[i].tobytes() == oracle.indcpa_enc(set_id, m[i], ns[i], pk[i])
    m2 = ctx.indcpa_dec(set_id, sk, ct, form=form)
    assert np.array_equal(m2, m)


def test_nist_api_and_randombytes_hook(kem, oracle):
    T, ctx = kem
    L = T.lib()
    z = T.sizes(T.SABER)
    state = {"ctr": 0}

    @T.RANDOMBYTES_FN
    def rb(buf, n):
        data = T.splitmix_bytes(4242 + state["ctr"], n)
        state["ctr"] += 1
        ctypes.memmove(buf, data.ctypes.data, n)

    L.tmvp_set_randombytes(ctypes.cast(rb, ctypes.c_void_p))
    try:
        pk = np.zeros(z.pk_bytes, np.uint8)
        sk = np.zeros(z.sk_bytes, np.uint8)
        assert L.crypto_kem_keypair(pk.ctypes.data, sk.ctypes.data) == 0
        opk, osk = oracle.kem_keypair(T.SABER, T.splitmix_bytes(4242, 96))
        assert pk.tobytes() == opk and sk.tobytes() == osk
        ct = np.zeros(z.ct_bytes, np.uint8)
        ss = np.zeros(32, np.uint8)
        assert L.crypto_kem_enc(ct.ctypes.data, ss.ctypes.data, pk.ctypes.data) == 0
        oct_, oss = oracle.kem_enc(T.SABER, opk, T.splitmix_bytes(4243, 32))
        assert ct.tobytes() == oct_ and ss.tobytes() == oss
        ss2 = np.zeros(32, np.uint8)
        assert L.crypto_kem_dec(ss2.ctypes.data, ct.ctypes.data, sk.ctypes.data) == 0
        assert ss2.tobytes() == oss
        # indcpa single-instance API
        ipk = np.zeros(z.pk_bytes, np.uint8)
        isk = np.zeros(z.indcpa_sk_bytes, np.uint8)
        assert L.indcpa_kem_keypair(ipk.ctypes.data, isk.ctypes.data) == 0
        m = T.splitmix_bytes(1, 32)
        seed = T.splitmix_bytes(2, 32)
        c = np.zeros(z.ct_bytes, np.uint8)
        assert L.indcpa_kem_enc(m.ctypes.data, seed.ctypes.data, ipk.ctypes.data, c.ctypes.data) == 0
        m2 = np.zeros(32, np.uint8)
        assert L.indcpa_kem_dec(isk.ctypes.data, c.ctypes.data, m2.ctypes.data) == 0
        assert np.array_equal(m, m2)
    finally:
        L.tmvp_set_randombytes(None)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_reference_shims(kem, oracle, mode):
    """saber_enc/saber_dec and SABLE_enc/SABLE_dec with the reference's calling convention."""
    T, ctx = kem
    L = T.lib()
    for scheme, set_id, B in ((0, T.SABER, 3), (1, T.SABLE, 5)):
        assert L.tmvp_ref_set_batch(scheme, B) == 0
        z = T.sizes(set_id)
        pk, sk = ctx.kem_keypair(set_id, _coins(9 + scheme, B, 96))
        h_c = np.zeros((B, z.ct_bytes), np.uint8)
        h_k = np.zeros((B, 32), np.uint8)
        h_k2 = np.zeros((B, 32), np.uint8)
        if scheme == 0:
            L.saber_enc(mode, h_k.ctypes.data, pk.ctypes.data, h_c.ctypes.data)
            assert L.tmvp_last_error() == 0
            L.saber_dec(mode, h_c.ctypes.data, pk.ctypes.data, sk.ctypes.data, h_k2.ctypes.data)
        else:
            L.SABLE_enc(h_k.ctypes.data, pk.ctypes.data, h_c.ctypes.data, mode)
            assert L.tmvp_last_error() == 0
            L.SABLE_dec(h_c.ctypes.data, pk.ctypes.data, sk.ctypes.data, h_k2.ctypes.data, mode)
        assert L.tmvp_last_error() == 0
        assert np.array_equal(h_k, h_k2) and h_k.any()
        oss, fail = oracle.kem_dec_batch(set_id, h_c, sk)
        assert np.array_equal(oss, h_k) and not fail.any()
    L.tmvp_ref_set_batch(0, 1)
    L.tmvp_ref_set_batch(1, 512)


def test_empty_and_unaligned_buffers(kem, oracle):
    T, ctx = kem
    z = T.sizes(T.SABER)
    # n = 0 is a no-op
    ctx.kem_dec_ptr(T.SABER, 0, None, None, None)
    # host buffers at odd offsets are staged, not read misaligned
    n = 5
    pk, sk = ctx.kem_keypair(T.SABER, _coins(31, n, 96))
    raw = np.zeros(n * z.ct_bytes + 3, np.uint8)
    ct_view = raw[3:]
    ssb = np.zeros(n * 32 + 1, np.uint8)
    ctx.kem_enc_ptr(T.SABER, n, ct_view, ssb[1:], pk, _coins(32, n, 32))
    oct_, oss = oracle.kem_enc_batch(T.SABER, pk, _coins(32, n, 32))
    assert np.array_equal(ct_view.reshape(n, -1), oct_) and np.array_equal(ssb[1:].reshape(n, -1), oss)


def test_out_of_range_secret_is_reported(kem):
    """The tensor-core forms refuse secrets outside their exact range."""
    T, ctx = kem
    A = np.zeros((2, 3, 3, 256), np.uint16)
    s = np.zeros((2, 3, 256), np.int8)
    s[1, 0, 7] = 100
    for form in (T.FORM_FP8_TC, T.FORM_INT8_TC, T.FORM_FP8_TCGEN05, T.FORM_DP2A):
        with pytest.raises(T.TmvpError) as e:
            ctx.matvec(A, s, eq=13, form=form)
        assert e.value.code == T.EINVAL
    s[1, 0, 7] = -64
    with pytest.raises(T.TmvpError):
        ctx.matvec(A, s, eq=13, form=T.FORM_DP2A)
    # the IMAD CUDA-core forms compute it exactly
    for form in (T.FORM_CUDA_CORE, T.FORM_TOOM_COOK):
        out = ctx.matvec(A, s, eq=13, form=form)
        assert not out.any()


@pytest.mark.parametrize("set_id", [0, 1, 2, 3, 4, 5])
def test_cached_genmatrix_matches_plain_calls(kem, set_id):
    """Encapsulation and decapsulation with each key's A expanded once
    (tmvp_genmatrix_batch + the _a entry points) give the plain calls' bytes,
    including the implicit rejection of a tampered ciphertext."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    n = 333
    z = T.sizes(set_id)
    coins = torch.from_numpy(T.splitmix_bytes(900 + set_id, n * 96).reshape(n, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(910 + set_id, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(set_id, n, pk, sk, coins)
    a = torch.empty((n, T.genmatrix_bytes(set_id)), dtype=torch.uint8, device=dev)
    ctx.genmatrix_ptr(set_id, n, a, pk)
    ct1 = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss1 = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ct2, ss2 = torch.empty_like(ct1), torch.empty_like(ss1)
    ctx.kem_enc_ptr(set_id, n, ct1, ss1, pk, ec)
    ctx.kem_enc_a_ptr(set_id, n, ct2, ss2, pk, ec, a)
    torch.cuda.synchronize()
    assert torch.equal(ct1, ct2) and torch.equal(ss1, ss2)
    ct1[7, 11] ^= 0x10
    d1, d2 = torch.zeros_like(ss1), torch.zeros_like(ss1)
    ctx.kem_dec_ptr(set_id, n, d1, ct1, sk)
    ctx.kem_dec_a_ptr(set_id, n, d2, ct1, sk, a)
    torch.cuda.synchronize()
    assert torch.equal(d1, d2)
    good = torch.ones(n, dtype=torch.bool, device=dev)
    good[7] = False
    assert torch.equal(d2[good], ss1[good]) and not torch.equal(d2[7], ss1[7])


def test_failed_workspace_allocation_leaves_context_usable(kem, oracle):
    """A workspace request the GPU cannot hold (2 TiB, refused by cudaMalloc
    without allocating anything) returns ENOMEM, and the next calls on the
    same context succeed and match the oracle: the failed allocation is
    reported once, not again by a later call."""
    import ctypes
    T, ctx = kem
    rc = T.lib().tmvp_ctx_reserve(ctx.h, ctypes.c_size_t(1 << 41))
    assert rc == T.ENOMEM
    n = 4
    coins = _coins(91, n, 96)
    pk, sk = ctx.kem_keypair(T.SABER, coins)
    opk, osk = oracle.kem_keypair_batch(T.SABER, coins)
    assert np.array_equal(pk, opk) and np.array_equal(sk, osk)
    ct, ss = ctx.kem_enc(T.SABER, pk, _coins(92, n, 32))
    assert np.array_equal(ctx.kem_dec(T.SABER, ct, sk), ss)


def test_bounded_wait_reports_timeout(kem, oracle):
    """Failure detection without a fault: the self-test launch's input wait
    can never complete, so the kernel's bounded wait gives up after about two
    seconds (and a second bounded wait for anything in flight), frees its
    tensor memory and reports TMVP_ETIMEOUT; the context and the GPU stay
    usable for the next call."""
    import time
    T, ctx = kem
    t0 = time.perf_counter()
    rc = T.lib().tmvp_selftest_bounded_wait(ctx.h, None)
    dt = time.perf_counter() - t0
    assert rc == T.ETIMEOUT
    assert 1.5 < dt < 60, dt
    rng = np.random.default_rng(11)
    A = rng.integers(0, 1 << 13, (16, 3, 3, 256), dtype=np.uint16)
    s = rng.integers(-5, 6, (16, 3, 256)).astype(np.int8)
    got = ctx.matvec(A, s, eq=13, form=T.FORM_FP8_TCGEN05)
    assert np.array_equal(got, oracle.matvec(A, s, eq=13, nthreads=4))


@pytest.mark.parametrize("set_id", [0, 1, 2, 3, 4, 5])
def test_onekey_decapsulation(kem, oracle, set_id):
    """Ciphertexts under one secret key (tmvp_kem_dec_batch_onekey): the same
    keys as the per-instance call with sk repeated, the encapsulated keys, the
    oracle's on a sample, and implicit rejection of a tampered ciphertext."""
    T, ctx = kem
    n = 1500
    pk, sk = ctx.kem_keypair(set_id, _coins(61 + set_id, 1, 96))
    ct, ss = ctx.kem_enc(set_id, np.repeat(pk, n, axis=0), _coins(71 + set_id, n, 32))
    ct[9, 11] ^= 2
    got = ctx.kem_dec_onekey(set_id, ct, sk[0])
    assert np.array_equal(got, ctx.kem_dec(set_id, ct, np.repeat(sk, n, axis=0)))
    good = np.ones(n, bool)
    good[9] = False
    assert np.array_equal(got[good], ss[good]) and not np.array_equal(got[9], ss[9])
    oss, fail = oracle.kem_dec_batch(set_id, ct[:12], np.repeat(sk, 12, axis=0), nthreads=4)
    assert np.array_equal(got[:12], oss) and fail[9] and not fail[:9].any()


@pytest.mark.parametrize("form", [0, 1, 2, 6])
def test_onekey_decapsulation_other_forms(kem, form):
    """The forms other than tcgen05 run the one-key call on the key repeated
    per instance, with the same bytes."""
    T, ctx = kem
    n = 700
    pk, sk = ctx.kem_keypair(T.SABER, _coins(81, 1, 96))
    ct, ss = ctx.kem_enc(T.SABER, np.repeat(pk, n, axis=0), _coins(82, n, 32))
    ct[3, 0] ^= 1
    got = ctx.kem_dec_onekey(T.SABER, ct, sk[0], form=form)
    assert np.array_equal(got, ctx.kem_dec_onekey(T.SABER, ct, sk[0]))
    assert np.array_equal(got[4:], ss[4:]) and not np.array_equal(got[3], ss[3])


@pytest.mark.parametrize("set_id,n", [(1, 1), (1, 7), (1, 1501), (4, 9), (4, 1503), (2, 11), (3, 6)])
def test_onekey_decapsulation_ragged(kem, set_id, n):
    """Batches that leave the last CTA of the one-key decryption partly
    empty (5 ciphertexts per CTA for 10-bit b', 8 for 9-bit) give the
    per-instance call's bytes."""
    T, ctx = kem
    pk, sk = ctx.kem_keypair(set_id, _coins(91 + n, 1, 96))
    ct, ss = ctx.kem_enc(set_id, np.repeat(pk, n, axis=0), _coins(92 + n, n, 32))
    ct[n - 1, 1] ^= 4
    got = ctx.kem_dec_onekey(set_id, ct, sk[0])
    assert np.array_equal(got, ctx.kem_dec(set_id, ct, np.repeat(sk, n, axis=0)))
    assert np.array_equal(got[:n - 1], ss[:n - 1]) and not np.array_equal(got[n - 1], ss[n - 1])
