"""The Keccak stages in both forms: one thread per sponge, and one warp per
sponge (the state spread over the warp's lanes, the form small launches take;
tmvp_ctx_set_warp_hash).  Every output must be the same bytes in both forms
and the oracle's (FIPS 202 through the reference's sponges,
TMVP_SABLE/src/fips202.cu:409-668)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALWAYS = 1 << 40  # every launch one warp per sponge


def _ctx(T, warp_hash):
    c = T.Context(0)
    c.set_warp_hash(warp_hash)
    return c


@pytest.mark.parametrize("set_id", range(6))
def test_kem_both_forms_match_oracle(kem, oracle, set_id):
    T, _ = kem
    cw, ct_ = _ctx(T, ALWAYS), _ctx(T, 0)
    try:
        for n in (1, 5, 37):
            kc = T.splitmix_bytes(3100 + 10 * set_id + n, n * 96).reshape(n, 96)
            ec = T.splitmix_bytes(3200 + 10 * set_id + n, n * 32).reshape(n, 32)
            pk_w, sk_w = cw.kem_keypair(set_id, kc)
            pk_t, sk_t = ct_.kem_keypair(set_id, kc)
            assert np.array_equal(pk_w, pk_t) and np.array_equal(sk_w, sk_t)
            c_w, s_w = cw.kem_enc(set_id, pk_w, ec)
            c_t, s_t = ct_.kem_enc(set_id, pk_w, ec)
            assert np.array_equal(c_w, c_t) and np.array_equal(s_w, s_t)
            bad = c_w.copy()
            bad[::2, (7 * n) % bad.shape[1]] ^= 0x24  # every other ciphertext tampered
            d_w = cw.kem_dec(set_id, bad, sk_w)
            d_t = ct_.kem_dec(set_id, bad, sk_w)
            assert np.array_equal(d_w, d_t)
            assert np.array_equal(d_w[1::2], s_w[1::2])
            if n == 5:
                opk, osk = oracle.kem_keypair_batch(set_id, kc)
                assert np.array_equal(pk_w, opk) and np.array_equal(sk_w, osk)
                oct_, oss = oracle.kem_enc_batch(set_id, opk, ec)
                assert np.array_equal(c_w, oct_) and np.array_equal(s_w, oss)
                oss2, fail = oracle.kem_dec_batch(set_id, bad, osk)
                assert np.array_equal(d_w, oss2) and fail[::2].all() and not fail[1::2].any()
    finally:
        cw.close()
        ct_.close()


@pytest.mark.parametrize("set_id", [0, 1, 4])
def test_indcpa_cached_and_onekey_paths_both_forms(kem, set_id):
    """IND-CPA key generation and encryption (two SHAKE jobs per instance),
    per-key GenMatrix with the cached-A calls, and the one-key decapsulation
    (one GenMatrix sponge) give the same bytes in both forms."""
    import torch
    T, _ = kem
    dev = torch.device("cuda", 0)
    cw, ct_ = _ctx(T, ALWAYS), _ctx(T, 0)
    try:
        n = 19
        seeds = T.splitmix_bytes(3300 + set_id, n * 64).reshape(n, 64)
        m = T.splitmix_bytes(3310 + set_id, n * 32).reshape(n, 32)
        ns = T.splitmix_bytes(3320 + set_id, n * 32).reshape(n, 32)
        out = []
        for c in (cw, ct_):
            pk, sk = c.indcpa_keypair(set_id, seeds)
            out.append((pk, sk, c.indcpa_enc(set_id, m, ns, pk)))
        for a, b in zip(out[0], out[1]):
            assert np.array_equal(a, b)
        assert np.array_equal(cw.indcpa_dec(set_id, out[0][1], out[0][2]), m)

        z = T.sizes(set_id)
        kc = torch.from_numpy(T.splitmix_bytes(3330 + set_id, n * 96).reshape(n, 96)).to(dev)
        ec = torch.from_numpy(T.splitmix_bytes(3340 + set_id, n * 32).reshape(n, 32)).to(dev)
        pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
        sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
        cw.kem_keypair_ptr(set_id, n, pk, sk, kc)
        res = []
        for c in (cw, ct_):
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
        for x, y in zip(res[0], res[1]):
            assert torch.equal(x, y)

        # one key, many ciphertexts
        ct1, ss1 = cw.kem_enc(set_id, np.repeat(pk[:1].cpu().numpy(), n, 0), ec.cpu().numpy())
        for c in (cw, ct_):
            assert np.array_equal(c.kem_dec_onekey(set_id, ct1, sk[0].cpu().numpy()), ss1)
    finally:
        cw.close()
        ct_.close()


def test_default_threshold_boundaries(kem):
    """Around the default 2048-sponge threshold (decapsulation front: 2n
    sponges; G and the final key count four times) the default context, the
    thread form and the warp form agree."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    S = T.SABER
    z = T.sizes(S)
    N = 1025
    kc = torch.from_numpy(T.splitmix_bytes(3400, N * 96).reshape(N, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(3401, N * 32).reshape(N, 32)).to(dev)
    pk = torch.empty((N, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((N, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((N, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((N, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(S, N, pk, sk, kc)
    ctx.kem_enc_ptr(S, N, ct, ss, pk, ec)
    ct[3::4, 100] ^= 0x01
    cw, ct_ = _ctx(T, ALWAYS), _ctx(T, 0)
    try:
        for n in (511, 512, 513, 1023, 1024, 1025):
            outs = []
            for c in (ctx, cw, ct_):
                d = torch.zeros((n, 32), dtype=torch.uint8, device=dev)
                c.kem_dec_ptr(S, n, d, ct, sk)
                torch.cuda.synchronize()
                outs.append(d)
            assert torch.equal(outs[0], outs[1]) and torch.equal(outs[0], outs[2]), f"n={n}"
            good = torch.ones(n, dtype=torch.bool, device=dev)
            good[3::4] = False
            assert torch.equal(outs[0][good], ss[:n][good])
            assert not (outs[0][~good] == ss[:n][~good]).all(dim=1).any()
    finally:
        cw.close()
        ct_.close()
