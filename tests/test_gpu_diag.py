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
