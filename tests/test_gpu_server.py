"""The request-serving loop: results are the same alone and in a concurrent
mix of parameter sets and operations, and match the oracle; batches form and
overlap under load; memory admission cuts and holds batches to fit the batch
arena."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SETS = (0, 1, 2, 4)  # LightSaber, Saber, FireSaber, Sable


def _keys(T, ctx, set_id, n, seed):
    return ctx.kem_keypair(set_id, T.splitmix_bytes(seed, n * 96).reshape(n, 96))


def test_alone_and_in_the_mix(kem, oracle):
    T, ctx = kem
    srv = T.Server(max_batch=512, slots=3)
    try:
        keys, ids = {}, {}
        for s in SETS:
            pk, sk = _keys(T, ctx, s, 8, 100 + s)
            keys[s] = (pk, sk)
            ids[s] = srv.add_keys(s, pk, sk)
        # one encapsulation and one decapsulation alone
        s0 = 1
        z = T.sizes(s0)
        coins = T.splitmix_bytes(42, 32)
        out_alone = np.zeros(z.ct_bytes + 32, np.uint8)
        srv.wait(srv.submit(T.OP_ENCAPS, ids[s0][3], coins, out_alone))
        oct_, oss = oracle.kem_enc(s0, keys[s0][0][3], coins)
        assert out_alone[:z.ct_bytes].tobytes() == oct_ and out_alone[z.ct_bytes:].tobytes() == oss
        ct = out_alone[:z.ct_bytes].copy()
        dec_alone = np.zeros(32, np.uint8)
        srv.wait(srv.submit(T.OP_DECAPS, ids[s0][3], ct, dec_alone))
        assert dec_alone.tobytes() == oss
        # the same two requests inside a mixed concurrent stream
        rng = np.random.default_rng(7)
        reqs = []
        for i in range(3000):
            s = SETS[rng.integers(0, len(SETS))]
            k = int(rng.integers(0, 8))
            zz = T.sizes(s)
            if rng.random() < 0.5:
                inp = T.splitmix_bytes(10_000 + i, 32)
                reqs.append(("enc", s, k, inp, np.zeros(zz.ct_bytes + 32, np.uint8)))
            else:
                c, _ = ctx.kem_enc(s, keys[s][0][k], T.splitmix_bytes(20_000 + i, 32))
                reqs.append(("dec", s, k, c[0], np.zeros(32, np.uint8)))
        mid = len(reqs) // 2
        reqs.insert(mid, ("enc", s0, 3, coins, np.zeros(z.ct_bytes + 32, np.uint8)))
        reqs.insert(mid + 1, ("dec", s0, 3, ct, np.zeros(32, np.uint8)))
        srv.reset_stats()

        def producer(part):
            for op, s, k, inp, out in part:
                srv.submit(T.OP_ENCAPS if op == "enc" else T.OP_DECAPS, ids[s][k], inp, out)

        ths = [threading.Thread(target=producer, args=(reqs[i::2],)) for i in range(2)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        srv.drain()
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["batches"] < len(reqs)  # requests were batched together
        # the two repeated requests give the same bytes as alone
        assert np.array_equal(reqs[mid][4], out_alone)
        assert np.array_equal(reqs[mid + 1][4], dec_alone)
        # everything against the oracle
        for op, s, k, inp, out in reqs:
            zz = T.sizes(s)
            if op == "enc":
                c, kk = oracle.kem_enc(s, keys[s][0][k], inp)
                assert out[:zz.ct_bytes].tobytes() == c and out[zz.ct_bytes:].tobytes() == kk
            else:
                kk, fail = oracle.kem_dec(s, inp, keys[s][1][k])
                assert out.tobytes() == kk and fail == 0
    finally:
        srv.close()


def test_memory_admission_and_loadgen(kem):
    """A batch arena far smaller than the slots could fill: batches are cut to
    what the largest free block holds and wait for blocks to come back, the
    arena is never exceeded, and every decapsulation of the load generator
    gives the encapsulated key."""
    T, ctx = kem
    probe = T.Server(max_batch=256, slots=4)
    try:
        full = probe.stats()["arena_bytes"]  # 4 batches of 256 requests of the largest set
    finally:
        probe.close()
    budget = full // 6  # two thirds of one such batch
    srv = T.Server(max_batch=256, slots=4, mem_budget=budget)
    try:
        st0 = srv.stats()
        assert st0["slots"] == 4 and budget <= st0["arena_bytes"] < budget + 256
        ids = []
        for s in SETS:
            pk, sk = _keys(T, ctx, s, 16, 300 + s)
            ids.append(srv.add_keys(s, pk, sk))
        n = srv.loadgen(rate=20000.0, seconds=0.5, seed=9, key_ids=np.concatenate(ids),
                        decaps_fraction=0.5)
        st = srv.stats()
        assert n > 5000 and st["completed"] == n and st["failed"] == 0
        assert st["checked"] > 1000 and st["mismatched"] == 0
        assert st["p99_us"] >= st["p50_us"] > 0
        assert 0 < st["peak_arena_bytes"] <= st["arena_bytes"]
    finally:
        srv.close()


def test_admission_refuses_then_admits(kem):
    """With room for a third of one FireSaber batch, a dense burst of requests
    is admitted piecewise: batches are cut to what fits, further batches wait
    until memory returns, the arena is never exceeded, and every
    decapsulation gives the encapsulated key."""
    T, ctx = kem
    probe = T.Server(max_batch=512, slots=1)
    try:
        one_batch = probe.stats()["arena_bytes"]  # one batch of 512 requests of the largest set
    finally:
        probe.close()
    srv = T.Server(max_batch=512, slots=3, mem_budget=one_batch // 3)
    try:
        pk, sk = _keys(T, ctx, 2, 8, 777)  # FireSaber
        ids = srv.add_keys(2, pk, sk)
        n = srv.loadgen(rate=1_000_000.0, seconds=0.1, seed=5, key_ids=ids, decaps_fraction=1.0)
        st = srv.stats()
        assert st["completed"] == n and st["failed"] == 0
        assert st["checked"] == n and st["mismatched"] == 0
        # batches were cut to the free blocks (whether a free slot also had to
        # wait depends on how the blocks fragment; the next case forces it)
        assert st["admission_splits"] >= 1
        assert 0 < st["peak_arena_bytes"] <= st["arena_bytes"]
    finally:
        srv.close()
    # an arena for exactly one request of the largest kind: every batch is one
    # request, and a free slot waits while it runs
    probe = T.Server(max_batch=1, slots=1)
    try:
        one_request = probe.stats()["arena_bytes"]
    finally:
        probe.close()
    srv = T.Server(max_batch=512, slots=3, mem_budget=one_request)
    try:
        pk, sk = _keys(T, ctx, 2, 4, 778)
        ids = srv.add_keys(2, pk, sk)
        n = srv.loadgen(rate=1_000_000.0, seconds=0.002, seed=6, key_ids=ids, decaps_fraction=1.0)
        st = srv.stats()
        assert n > 100 and st["completed"] == n and st["failed"] == 0 and st["mismatched"] == 0
        assert st["admission_waits"] >= 1 and st["admission_splits"] >= 1
        assert st["batches"] == n and st["peak_arena_bytes"] <= st["arena_bytes"]
    finally:
        srv.close()


def test_budget_below_one_request_is_refused(kem):
    T, ctx = kem
    with pytest.raises(T.TmvpError) as e:
        T.Server(max_batch=64, slots=2, mem_budget=4096)
    assert e.value.code == T.ENOMEM


def test_one_key_batches(kem, oracle):
    """A server with one key per set: decapsulation batches whose requests all
    use that key take the one-key path, with the same bytes as the
    encapsulations and the oracle; a tampered ciphertext is rejected."""
    T, ctx = kem
    srv = T.Server(max_batch=256, slots=2)
    try:
        keys, ids = {}, {}
        for s in (1, 4):
            pk, sk = _keys(T, ctx, s, 1, 300 + s)
            keys[s] = (pk, sk)
            ids[s] = srv.add_keys(s, pk, sk)
        reqs = []
        for i in range(1200):
            s = (1, 4)[i % 2]
            c, kk = ctx.kem_enc(s, keys[s][0][0], T.splitmix_bytes(40_000 + i, 32))
            c = c[0].copy()
            if i == 601:
                c[5] ^= 1
            reqs.append((s, c, kk[0], np.zeros(32, np.uint8)))
        srv.reset_stats()
        for s, c, _, out in reqs:
            srv.submit(T.OP_DECAPS, ids[s][0], c, out)
        srv.drain()
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["one_key_batches"] >= 1
        for i, (s, c, kk, out) in enumerate(reqs):
            if i == 601:
                okk, fail = oracle.kem_dec(s, c, keys[s][1][0])
                assert fail and out.tobytes() == okk and not np.array_equal(out, kk)
            else:
                assert np.array_equal(out, kk)
    finally:
        srv.close()
