"""Mixed-parameter decapsulation and launch shapes: a pass over groups of
different parameter sets (Keccak stages one launch over all groups, each
IND-CPA step one launch per set present), and its CUDA-graph plan, give the
same keys as per-set batches (which the parity tests pin to the oracle);
every launch shape, and the autotuner's choice, stay bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _kem_set(T, ctx, set_id, n, seed):
    import torch
    dev = torch.device("cuda", 0)
    z = T.sizes(set_id)
    coins = torch.from_numpy(T.splitmix_bytes(seed, n * 96).reshape(n, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(seed + 1, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(set_id, n, pk, sk, coins)
    ctx.kem_enc_ptr(set_id, n, ct, ss, pk, ec)
    return pk, sk, ct, ss


GROUPS = [(0, 777), (1, 4096), (2, 333), (4, 2500), (3, 17), (5, 1024), (1, 1)]


def test_mixed_matches_batches(kem):
    import torch
    T, ctx = kem
    made = [_kem_set(T, ctx, s, n, 1000 + 7 * i) for i, (s, n) in enumerate(GROUPS)]
    # tamper one ciphertext of the Saber group: implicit rejection as in the batch API
    made[1][2][5, 3] ^= 1
    outs = [torch.zeros_like(m[3]) for m in made]
    ctx.kem_dec_mixed([(s, outs[i], made[i][2], made[i][1]) for i, (s, _) in enumerate(GROUPS)])
    ctx.sync_status()
    for i, (s, n) in enumerate(GROUPS):
        ref = torch.zeros_like(outs[i])
        ctx.kem_dec_ptr(s, n, ref, made[i][2], made[i][1], T.FORM_FP8_TCGEN05)
        torch.cuda.synchronize()
        assert torch.equal(outs[i], ref), f"group {i} (set {s})"
        good = torch.ones(n, dtype=torch.bool, device=outs[i].device)
        if i == 1:
            good[5] = False
        assert torch.equal(outs[i][good], made[i][3][good])
    assert not torch.equal(outs[1][5], made[1][3][5])


def test_mixed_plan_graph_replays(kem):
    import torch
    T, ctx = kem
    groups = [(1, 3000), (4, 1500), (2, 600), (0, 100)]
    made = [_kem_set(T, ctx, s, n, 2000 + i) for i, (s, n) in enumerate(groups)]
    outs = [torch.zeros_like(m[3]) for m in made]
    plan = T.MixedPlan(ctx, [(s, outs[i], made[i][2], made[i][1]) for i, (s, _) in enumerate(groups)])
    try:
        plan.launch()
        ctx.sync_status()
        for i in range(len(groups)):
            assert torch.equal(outs[i], made[i][3])
        # new ciphertexts in the same buffers, replay the same graph
        for i, (s, n) in enumerate(groups):
            ec = torch.from_numpy(T.splitmix_bytes(5000 + i, n * 32).reshape(n, 32)).to(outs[i].device)
            ss_new = torch.empty_like(made[i][3])
            ctx.kem_enc_ptr(s, n, made[i][2], ss_new, made[i][0], ec)
            made[i] = (made[i][0], made[i][1], made[i][2], ss_new)
        torch.cuda.synchronize()
        plan.launch()
        ctx.sync_status()
        for i in range(len(groups)):
            assert torch.equal(outs[i], made[i][3])
    finally:
        plan.close()


@pytest.mark.parametrize("set_id", [1, 2, 4])
def test_every_launch_shape_is_exact(kem, oracle, set_id):
    import torch
    T, ctx = kem
    n = 700
    dev = torch.device("cuda", 0)
    coins = T.splitmix_bytes(77 + set_id, n * 96).reshape(n, 96)
    ec = T.splitmix_bytes(78 + set_id, n * 32).reshape(n, 32)
    opk, osk = oracle.kem_keypair_batch(set_id, coins[:8], 4)
    oct_, oss = oracle.kem_enc_batch(set_id, opk, ec[:8], 4)
    try:
        for shape in (-1, 0, 1, 2):
            for step in range(5):
                T.tune_set(step, set_id, shape)
            pk, sk = ctx.kem_keypair(set_id, coins, form=T.FORM_FP8_TCGEN05)
            ct, ss = ctx.kem_enc(set_id, pk, ec, form=T.FORM_FP8_TCGEN05)
            assert np.array_equal(pk[:8], opk) and np.array_equal(sk[:8], osk), shape
            assert np.array_equal(ct[:8], oct_) and np.array_equal(ss[:8], oss), shape
            assert np.array_equal(ctx.kem_dec(set_id, ct, sk, form=T.FORM_FP8_TCGEN05), ss), shape
            z = T.sizes(set_id)
            A = np.random.default_rng(shape + 9).integers(0, 1 << 13, (64, z.l, z.l, 256)).astype(np.uint16)
            s8 = np.random.default_rng(shape + 10).integers(-5, 6, (64, z.l, 256)).astype(np.int8)
            assert np.array_equal(ctx.matvec(A, s8, 13, form=T.FORM_FP8_TCGEN05),
                                  oracle.matvec(A, s8, eq=13, nthreads=4)), shape
    finally:
        for step in range(5):
            T.tune_set(step, set_id, -1)
    del dev


def test_autotune_choice_is_exact(kem):
    """The autotuner's launch shapes and its pass settings for the batch
    bucket (device chunk, Keccak-front cap, host chunk and ramp) are among
    the candidates, and decapsulation under them stays exact, from device and
    from host buffers."""
    T, ctx = kem
    try:
        shapes = ctx.autotune(1, 4096)
        assert len(shapes) == 5 and all(s in (-1, 0, 1, 2) for s in shapes)
        assert [T.tune_get(step, 1) for step in range(5)] == shapes
        pc = T.tune_pass_get(1, 4096)
        assert pc is not None and pc["dev_chunk"] == 0 and pc["front_cap"] in (0, 8)
        assert (pc["host_chunk"], pc["host_ramp"]) in ((0, 0), (0, 1), (0, 2))  # chunks >= n are skipped
        assert T.tune_pass_get(1, 2500) == pc and T.tune_pass_get(1, 8192) is None
        n = 3000
        coins = T.splitmix_bytes(99, n * 96).reshape(n, 96)
        pk, sk = ctx.kem_keypair(1, coins)
        ct, ss = ctx.kem_enc(1, pk, T.splitmix_bytes(98, n * 32).reshape(n, 32))
        assert np.array_equal(ctx.kem_dec(1, ct, sk), ss)
        # a bucket with chunking: every candidate was checked against the keys
        shapes = ctx.autotune(1, 40000)
        pc = T.tune_pass_get(1, 40000)
        assert pc["dev_chunk"] in (0, 16384, 32768) and pc["host_chunk"] in (0, 8192, 16384, 32768)
    finally:
        T.tune_clear()
