"""The Keccak stages in their three forms: one thread per sponge, one warp per
sponge (the state spread over the warp's lanes) and two threads per sponge
(each holding half of every lane), chosen per launch by size
(tmvp_ctx_set_warp_hash / tmvp_ctx_set_pair_hash).  Every output must be the
same bytes in every form and the oracle's (FIPS 202 through the reference's
sponges, TMVP_SABLE/src/fips202.cu:409-668)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALWAYS = 1 << 40
FORMS = {"warp": (ALWAYS, 0), "pair": (0, ALWAYS), "thread": (0, 0)}


def _ctx(T, form):
    c = T.Context(0)
    warp, pair = FORMS[form]
    c.set_warp_hash(warp)
    c.set_pair_hash(pair)
    return c


def _ctxs(T):
    return [_ctx(T, f) for f in FORMS]


@pytest.mark.parametrize("set_id", range(6))
def test_kem_every_form_matches_oracle(kem, oracle, set_id):
    T, _ = kem
    cs = _ctxs(T)
    try:
        for n in (1, 5, 37):
            kc = T.splitmix_bytes(3100 + 10 * set_id + n, n * 96).reshape(n, 96)
            ec = T.splitmix_bytes(3200 + 10 * set_id + n, n * 32).reshape(n, 32)
            keys = [c.kem_keypair(set_id, kc) for c in cs]
            pk, sk = keys[0]
            for pk2, sk2 in keys[1:]:
                assert np.array_equal(pk, pk2) and np.array_equal(sk, sk2)
            encs = [c.kem_enc(set_id, pk, ec) for c in cs]
            ct, ss = encs[0]
            for ct2, ss2 in encs[1:]:
                assert np.array_equal(ct, ct2) and np.array_equal(ss, ss2)
            bad = ct.copy()
            bad[::2, (7 * n) % bad.shape[1]] ^= 0x24  # every other ciphertext tampered
            decs = [c.kem_dec(set_id, bad, sk) for c in cs]
            for d in decs[1:]:
                assert np.array_equal(decs[0], d)
            assert np.array_equal(decs[0][1::2], ss[1::2])
            if n == 5:
                opk, osk = oracle.kem_keypair_batch(set_id, kc)
                assert np.array_equal(pk, opk) and np.array_equal(sk, osk)
                oct_, oss = oracle.kem_enc_batch(set_id, opk, ec)
                assert np.array_equal(ct, oct_) and np.array_equal(ss, oss)
                oss2, fail = oracle.kem_dec_batch(set_id, bad, osk)
                assert np.array_equal(decs[0], oss2) and fail[::2].all() and not fail[1::2].any()
    finally:
        for c in cs:
            c.close()


@pytest.mark.parametrize("set_id", [0, 1, 4])
def test_indcpa_cached_and_onekey_paths_every_form(kem, set_id):
    """IND-CPA key generation and encryption (two SHAKE jobs per instance),
    per-key GenMatrix with the cached-A calls, and the one-key decapsulation
    (one GenMatrix sponge) give the same bytes in every form."""
    import torch
    T, _ = kem
    dev = torch.device("cuda", 0)
    cs = _ctxs(T)
    cw = cs[0]
    try:
        n = 19
        seeds = T.splitmix_bytes(3300 + set_id, n * 64).reshape(n, 64)
        m = T.splitmix_bytes(3310 + set_id, n * 32).reshape(n, 32)
        ns = T.splitmix_bytes(3320 + set_id, n * 32).reshape(n, 32)
        out = []
        for c in cs:
            pk, sk = c.indcpa_keypair(set_id, seeds)
            out.append((pk, sk, c.indcpa_enc(set_id, m, ns, pk)))
        for o in out[1:]:
            for a, b in zip(out[0], o):
                assert np.array_equal(a, b)
        assert np.array_equal(cw.indcpa_dec(set_id, out[0][1], out[0][2]), m)

        z = T.sizes(set_id)
        kc = torch.from_numpy(T.splitmix_bytes(3330 + set_id, n * 96).reshape(n, 96)).to(dev)
        ec = torch.from_numpy(T.splitmix_bytes(3340 + set_id, n * 32).reshape(n, 32)).to(dev)
        pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
        sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
        cw.kem_keypair_ptr(set_id, n, pk, sk, kc)
        res = []
        for c in cs:
            a = torch.empty((n, T.genmatrix_bytes(set_id)), dtype=torch.uint8, device=dev)
            c.genmatrix_ptr(set_id, n, a, pk)
            ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
            ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
            c.kem_enc_a_ptr(set_id, n, ct, ss, pk, ec, a)
            d = torch.zeros_like(ss)
            c.kem_dec_a_ptr(set_id, n, d, ct, sk, a)
            torch.cuda.synchronize()
            assert torch.equal(d, ss)
            res.append((a.cpu(), ct.cpu(), ss.cpu()))
        for r in res[1:]:
            for x, y in zip(res[0], r):
                assert torch.equal(x, y)

        # one key, many ciphertexts
        ct1, ss1 = cw.kem_enc(set_id, np.repeat(pk[:1].cpu().numpy(), n, 0), ec.cpu().numpy())
        for c in cs:
            assert np.array_equal(c.kem_dec_onekey(set_id, ct1, sk[0].cpu().numpy()), ss1)
    finally:
        for c in cs:
            c.close()


def test_default_threshold_boundaries(kem):
    """Around the default limits (warp form: 1024 sponges, pair form: 32768;
    the decapsulation front has 2n sponges, G and the final key count four
    times against the first and twice against the second) the default
    context and each single form agree."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    S = T.SABER
    z = T.sizes(S)
    N = 16385
    kc = torch.from_numpy(T.splitmix_bytes(3400, N * 96).reshape(N, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(3401, N * 32).reshape(N, 32)).to(dev)
    pk = torch.empty((N, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((N, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((N, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((N, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(S, N, pk, sk, kc)
    ctx.kem_enc_ptr(S, N, ct, ss, pk, ec)
    ct[3::4, 100] ^= 0x01
    cs = _ctxs(T)
    try:
        for n in (255, 256, 257, 511, 512, 513, 8191, 8192, 8193, 16384, 16385):
            outs = []
            for c in [ctx] + cs:
                d = torch.zeros((n, 32), dtype=torch.uint8, device=dev)
                c.kem_dec_ptr(S, n, d, ct, sk)
                torch.cuda.synchronize()
                outs.append(d)
            for o in outs[1:]:
                assert torch.equal(outs[0], o), f"n={n}"
            good = torch.ones(n, dtype=torch.bool, device=dev)
            good[3::4] = False
            assert torch.equal(outs[0][good], ss[:n][good])
            assert not (outs[0][~good] == ss[:n][~good]).all(dim=1).any()
    finally:
        for c in cs:
            c.close()
