"""The tensor-core issue-cost diagnostic (tmvp_diag_umma_rate) on both exact
kinds: it completes within its bounded wait, reports consistent per-CTA and
per-SM figures, and refuses shapes tensor memory cannot hold."""
import pytest

pytestmark = pytest.mark.gpu


def test_umma_rate_both_kinds(kem):
    T, ctx = kem
    for kind in (0, 1):  # kind::f8f6f4 (e4m3, K = 32), kind::f16 (K = 16)
        for n, ctas in ((16, 4), (64, 4), (256, 2)):
            cta, sm = ctx.umma_rate(kind, n, ctas_per_sm=ctas, iters=1024)
            assert 1.0 < sm < 10000.0
            assert abs(cta - ctas * sm) <= 1e-9 * cta


def test_umma_rate_refuses_bad_shapes(kem):
    T, ctx = kem
    for kind, n, ctas in ((2, 32, 1), (0, 48, 1), (0, 8, 1), (1, 256, 3), (0, 64, 0)):
        with pytest.raises(T.TmvpError) as e:
            ctx.umma_rate(kind, n, ctas_per_sm=ctas, iters=16)
        assert e.value.code == T.EINVAL


def test_keccak_rate(kem):
    """The permutation-rate diagnostic runs at full occupancy and refuses a
    bad permutation count."""
    T, ctx = kem
    rate, blocks = ctx.keccak_rate(16)
    assert blocks >= 1 and 1e8 < rate < 1e11
    with pytest.raises(T.TmvpError) as e:
        ctx.keccak_rate(0)
    assert e.value.code == T.EINVAL


def test_stage_busy_time(kem):
    """Per-stage busy time (union of a stage's launch intervals): never above
    the summed launch times, equal to them when every stage runs alone, and
    below them where the chunk chains' Keccak fronts overlap."""
    import torch
    T, _ = kem
    dev = torch.device("cuda", 0)
    S = T.SABER
    z = T.sizes(S)
    n = 65536
    kc = torch.from_numpy(T.splitmix_bytes(3500, n * 96).reshape(n, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(3501, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    c = T.Context(0)
    try:
        c.kem_keypair_ptr(S, n, pk, sk, kc)
        c.kem_enc_ptr(S, n, ct, ss, pk, ec)
        d = torch.empty_like(ss)
        for serial in (True, False):
            c.set_serial(serial)
            c.set_dev_chunk(16384)  # four chunk chains on four lanes
            c.set_timing(True)
            for _ in range(3):
                c.kem_dec_ptr(S, n, d, ct, sk)
            stats, busy = c.stage_stats(), c.stage_busy()
            c.set_timing(False)
            torch.cuda.synchronize()
            assert torch.equal(d, ss)
            assert set(stats) == set(busy) and "dec_front" in busy
            for k, (cnt, tot) in stats.items():
                assert 0 < busy[k] <= tot * (1 + 1e-6) + 1e-6, k
                if serial:
                    assert busy[k] >= tot * 0.999 - 1e-6, k
            if not serial:
                assert stats["dec_front"][0] == 12
                assert busy["dec_front"] < stats["dec_front"][1]
    finally:
        c.close()
