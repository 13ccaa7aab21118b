"""Batch-scale properties on the GPU: 10^6 seeded Saber round trips are
bit-exact, and the raw TMVP matvec at its benchmark size (16384 instances)
agrees with the oracle on a sample and is linear in the secret."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_million_round_trips(kem, oracle):
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    n, chunks = 65536, 16  # 16 * 65536 = 1,048,576 round trips
    z = T.sizes(T.SABER)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ss2 = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    rng = np.random.default_rng(0)
    total = 0
    for c in range(chunks):
        coins = torch.from_numpy(T.splitmix_bytes(7_000_000 + c, n * 96).reshape(n, 96)).to(dev)
        ec = torch.from_numpy(T.splitmix_bytes(8_000_000 + c, n * 32).reshape(n, 32)).to(dev)
        ctx.kem_keypair_ptr(T.SABER, n, pk, sk, coins)
        ctx.kem_enc_ptr(T.SABER, n, ct, ss, pk, ec)
        form = [T.FORM_FP8_TCGEN05, T.FORM_FP8_TC, T.FORM_INT8_TC, T.FORM_CUDA_CORE][c % 4]
        ctx.kem_dec_ptr(T.SABER, n, ss2, ct, sk, form)
        torch.cuda.synchronize()
        assert torch.equal(ss, ss2), f"chunk {c}: decapsulated keys differ"
        total += n
        # every stage of a random sample against the oracle
        idx = rng.choice(n, 16, replace=False)
        c_np = coins.cpu().numpy()[idx]
        opk, osk = oracle.kem_keypair_batch(T.SABER, c_np, 4)
        assert np.array_equal(pk.cpu().numpy()[idx], opk) and np.array_equal(sk.cpu().numpy()[idx], osk)
        oct_, oss = oracle.kem_enc_batch(T.SABER, opk, ec.cpu().numpy()[idx], 4)
        assert np.array_equal(ct.cpu().numpy()[idx], oct_) and np.array_equal(ss.cpu().numpy()[idx], oss)
    assert total >= 1_000_000


@pytest.mark.parametrize("form", [0, 1, 2, 5, 6, 7])
def test_matvec_benchmark_size(kem, oracle, form):
    """16384 instances of a 3x3 matrix (uniform mod 2^13) times CBD(mu=8) secrets."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    n, l = 16384, 3
    rng = np.random.default_rng(11)
    A = rng.integers(0, 1 << 13, (n, l, l, 256), dtype=np.uint16)
    # CBD(mu=8): popcount difference of two nibbles
    b = rng.integers(0, 256, (n, l, 256), dtype=np.uint8)
    pc = np.vectorize(lambda x: bin(int(x)).count("1"), otypes=[np.int8])
    s = (pc(b & 15) - pc(b >> 4)).astype(np.int8)
    At = torch.from_numpy(A.view(np.int16)).to(dev)
    st = torch.from_numpy(s).to(dev)
    out = torch.empty((n, l, 256), dtype=torch.int16, device=dev)
    ctx.matvec_ptr(n, l, 13, 0, out, At, st, form)
    got = out.cpu().numpy().view(np.uint16)
    idx = rng.choice(n, 64, replace=False)
    want = oracle.matvec(A[idx], s[idx], eq=13, nthreads=4)
    assert np.array_equal(got[idx], want)
    # linearity in the secret: A(s1 + s2) = A s1 + A s2 (mod 2^13)
    s1 = np.clip(s, -3, 3).astype(np.int8)
    s2 = (s - s1).astype(np.int8)
    o1 = torch.empty_like(out)
    o2 = torch.empty_like(out)
    ctx.matvec_ptr(n, l, 13, 0, o1, At, torch.from_numpy(s1).to(dev), form)
    ctx.matvec_ptr(n, l, 13, 0, o2, At, torch.from_numpy(s2).to(dev), form)
    summ = (o1.cpu().numpy().view(np.uint16).astype(np.uint32) +
            o2.cpu().numpy().view(np.uint16).astype(np.uint32)) & 8191
    assert np.array_equal(summ.astype(np.uint16), got)


def test_mixed_residency_host_decapsulation(kem):
    """Host inputs larger than one chunk (16384) go through the overlapped
    copy / compute path; the keys equal the device-buffer path's, including a
    ragged last chunk, host outputs, and mixed residency (host ciphertexts
    with device keys and a device output)."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    n = 40000
    z = T.sizes(T.SABER)
    coins = torch.from_numpy(T.splitmix_bytes(31, n * 96).reshape(n, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(32, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(T.SABER, n, pk, sk, coins)
    ctx.kem_enc_ptr(T.SABER, n, ct, ss, pk, ec)
    ct[n - 3, 7] ^= 1  # one rejection in the last chunk
    torch.cuda.synchronize()
    want = torch.empty_like(ss)
    ctx.kem_dec_ptr(T.SABER, n, want, ct, sk)
    torch.cuda.synchronize()
    ct_h, sk_h = ct.cpu().pin_memory(), sk.cpu().pin_memory()
    out_h = torch.zeros((n, 32), dtype=torch.uint8).pin_memory()
    ctx.kem_dec_ptr(T.SABER, n, out_h, ct_h, sk_h)   # host in, host out
    assert torch.equal(out_h, want.cpu())
    out_d = torch.zeros_like(ss)
    ctx.kem_dec_ptr(T.SABER, n, out_d, ct_h, sk)     # host ct, device sk and out
    torch.cuda.synchronize()
    assert torch.equal(out_d, want)
    assert not torch.equal(want[n - 3], ss[n - 3]) and torch.equal(want[:n - 3], ss[:n - 3])


@pytest.mark.parametrize("chunk", [0, 8192, 12000])
def test_chunked_device_decapsulation(kem, chunk):
    """Device buffers larger than the device chunk run as chains on four
    streams (the caller's and three lanes); every chunk size, including a
    ragged last chunk and more chunks than lanes, gives the keys of the
    encapsulation and rejects a tampered ciphertext in the last chunk."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    n = 40000
    z = T.sizes(T.SABER)
    coins = torch.from_numpy(T.splitmix_bytes(41, n * 96).reshape(n, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(42, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(T.SABER, n, pk, sk, coins)
    ctx.kem_enc_ptr(T.SABER, n, ct, ss, pk, ec)
    ct[n - 5, 100] ^= 4
    torch.cuda.synchronize()
    try:
        ctx.set_dev_chunk(chunk)
        out = torch.zeros_like(ss)
        ctx.kem_dec_ptr(T.SABER, n, out, ct, sk)
        torch.cuda.synchronize()
    finally:
        ctx.set_dev_chunk(32768)
    assert torch.equal(out[:n - 5], ss[:n - 5]) and torch.equal(out[n - 4:], ss[n - 4:])
    assert not torch.equal(out[n - 5], ss[n - 5])


@pytest.mark.parametrize("cap", [1, 3, 8])
def test_capped_keccak_front_gives_same_keys(kem, cap):
    """A Keccak front capped at `cap` blocks per SM (threads striding over the
    GenMatrix and H(c) sponges) gives the same keys, rejection included."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    n = 20000
    z = T.sizes(T.SABER)
    coins = torch.from_numpy(T.splitmix_bytes(61, n * 96).reshape(n, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(62, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(T.SABER, n, pk, sk, coins)
    ctx.kem_enc_ptr(T.SABER, n, ct, ss, pk, ec)
    ct[n - 1, 3] ^= 16
    out = torch.zeros_like(ss)
    try:
        ctx.set_front_cap(cap)
        ctx.kem_dec_ptr(T.SABER, n, out, ct, sk)
        torch.cuda.synchronize()
    finally:
        ctx.set_front_cap(0)
    assert torch.equal(out[:n - 1], ss[:n - 1]) and not torch.equal(out[n - 1], ss[n - 1])


def test_serial_stages_give_same_keys(kem):
    """The measurement mode that runs every decapsulation stage alone on the
    caller's stream gives the pipelined pass's keys, rejection included."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    n = 40000
    z = T.sizes(T.SABER)
    coins = torch.from_numpy(T.splitmix_bytes(51, n * 96).reshape(n, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(52, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(T.SABER, n, pk, sk, coins)
    ctx.kem_enc_ptr(T.SABER, n, ct, ss, pk, ec)
    ct[7, 9] ^= 2
    want = torch.empty_like(ss)
    ctx.kem_dec_ptr(T.SABER, n, want, ct, sk)
    out = torch.zeros_like(ss)
    try:
        ctx.set_serial(True)
        ctx.set_timing(True)
        ctx.kem_dec_ptr(T.SABER, n, out, ct, sk)
        torch.cuda.synchronize()
        stages = ctx.stage_stats()
    finally:
        ctx.set_timing(False)
        ctx.set_serial(False)
    assert torch.equal(out, want)
    assert not torch.equal(out[7], ss[7]) and torch.equal(out[8:], ss[8:])
    # one unchunked chain: each stage launched once
    assert all(v[0] == 1 for v in stages.values()) and "dec_front" in stages


@pytest.mark.parametrize("chunk,ramp,pinned", [(1024, 4, True), (4096, 2, True), (16384, 0, True),
                                               (16384, 3, True), (0, 0, True), (4096, 2, False)])
def test_chunked_host_decapsulation(kem, chunk, ramp, pinned):
    """Host buffers run as copy-ahead chunks (ramped first chunks, five input
    slots, four lanes; with pinned buffers GenMatrix of the whole batch runs
    first from the seeds read in place, with pageable ones each chunk expands
    its own); every schedule, including more chunks than slots and a ragged
    last chunk, gives the encapsulation's keys and rejects a tampered
    ciphertext in the last chunk."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    n = 40000
    z = T.sizes(T.SABER)
    coins = torch.from_numpy(T.splitmix_bytes(43, n * 96).reshape(n, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(44, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(T.SABER, n, pk, sk, coins)
    ctx.kem_enc_ptr(T.SABER, n, ct, ss, pk, ec)
    ct[n - 3, 7] ^= 1
    torch.cuda.synchronize()
    ct_h, sk_h = ct.cpu(), sk.cpu()
    out = torch.zeros((n, 32), dtype=torch.uint8)
    if pinned:
        ct_h, sk_h, out = ct_h.pin_memory(), sk_h.pin_memory(), out.pin_memory()
    try:
        ctx.set_host_chunk(chunk)
        ctx.set_host_ramp(ramp)
        ctx.kem_dec_ptr(T.SABER, n, out, ct_h, sk_h)
        torch.cuda.synchronize()
    finally:
        ctx.set_host_chunk(16384)
        ctx.set_host_ramp(1)
    ss_h = ss.cpu()
    assert torch.equal(out[:n - 3], ss_h[:n - 3]) and torch.equal(out[n - 2:], ss_h[n - 2:])
    assert not torch.equal(out[n - 3], ss_h[n - 3])


@pytest.mark.parametrize("chunk,ramp,pinned", [(4096, 2, True), (16384, 1, True), (8192, 0, False)])
def test_chunked_host_onekey_decapsulation(kem, chunk, ramp, pinned):
    """Host ciphertexts under one key run as copy-ahead chunks; the keys equal
    the device-buffer call's, with a tampered ciphertext in the last chunk
    rejected."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    n = 40000
    z = T.sizes(T.SABER)
    coins = torch.from_numpy(T.splitmix_bytes(45, 96).reshape(1, 96)).to(dev)
    pk = torch.empty((1, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((1, z.sk_bytes), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(T.SABER, 1, pk, sk, coins)
    ec = torch.from_numpy(T.splitmix_bytes(46, n * 32).reshape(n, 32)).to(dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ctx.kem_enc_ptr(T.SABER, n, ct, ss, pk.expand(n, -1).contiguous(), ec)
    ct[n - 2, 3] ^= 8
    ref = torch.empty_like(ss)
    ctx.kem_dec_onekey_ptr(T.SABER, n, ref, ct, sk[0])
    torch.cuda.synchronize()
    ct_h, out = ct.cpu(), torch.zeros((n, 32), dtype=torch.uint8)
    if pinned:
        ct_h, out = ct_h.pin_memory(), out.pin_memory()
    try:
        ctx.set_host_chunk(chunk)
        ctx.set_host_ramp(ramp)
        ctx.kem_dec_onekey_ptr(T.SABER, n, out, ct_h, sk[0])
        torch.cuda.synchronize()
    finally:
        ctx.set_host_chunk(16384)
        ctx.set_host_ramp(1)
    assert torch.equal(out, ref.cpu())
    ss_h = ss.cpu()
    assert torch.equal(out[:n - 2], ss_h[:n - 2]) and not torch.equal(out[n - 2], ss_h[n - 2])


@pytest.mark.parametrize("set_id", [1, 2, 4])
def test_one_chain_host_decapsulation_genmatrix_from_mapped_seeds(kem, set_id):
    """Host inputs in one chain (up to the host chunk): with pinned sk the
    GenMatrix launch reads each key's seed in place while ct and sk are
    copied (in its warp, pair or thread form by size); with pageable sk the
    chain expands it after the copy.  Both give the device path's keys,
    tampered ciphertexts rejected."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    z = T.sizes(set_id)
    N = 5000
    coins = torch.from_numpy(T.splitmix_bytes(61 + set_id, N * 96).reshape(N, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(71 + set_id, N * 32).reshape(N, 32)).to(dev)
    pk = torch.empty((N, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((N, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((N, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((N, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(set_id, N, pk, sk, coins)
    ctx.kem_enc_ptr(set_id, N, ct, ss, pk, ec)
    ct[5::9, 11] ^= 0x40
    torch.cuda.synchronize()
    want = torch.empty_like(ss)
    ctx.kem_dec_ptr(set_id, N, want, ct, sk)
    torch.cuda.synchronize()
    want_h = want.cpu()
    assert not (want[5::9] == ss[5::9]).all(dim=1).any()
    for pinned in (True, False):
        ct_h, sk_h, out = ct.cpu(), sk.cpu(), torch.zeros((N, 32), dtype=torch.uint8)
        if pinned:
            ct_h, sk_h, out = ct_h.pin_memory(), sk_h.pin_memory(), out.pin_memory()
        for n in (1, 300, 2048, 5000):
            out.zero_()
            ctx.kem_dec_ptr(set_id, n, out, ct_h, sk_h)
            torch.cuda.synchronize()
            assert torch.equal(out[:n], want_h[:n]), f"pinned={pinned} n={n}"


def test_one_chain_host_decapsulation_within_a_tight_budget(kem):
    """With a workspace budget too small for the early GenMatrix streams (and
    large enough for the chain without them) a pinned-host decapsulation
    still runs, expanding GenMatrix after the copies."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    S = T.SABER
    z = T.sizes(S)
    n = 4096  # ~33 MB of workspace without the early A, ~48 MB with it
    coins = torch.from_numpy(T.splitmix_bytes(81, n * 96).reshape(n, 96)).to(dev)
    ec = torch.from_numpy(T.splitmix_bytes(82, n * 32).reshape(n, 32)).to(dev)
    pk = torch.empty((n, z.pk_bytes), dtype=torch.uint8, device=dev)
    sk = torch.empty((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ct = torch.empty((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    ss = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    ctx.kem_keypair_ptr(S, n, pk, sk, coins)
    ctx.kem_enc_ptr(S, n, ct, ss, pk, ec)
    torch.cuda.synchronize()
    ct_h, sk_h = ct.cpu().pin_memory(), sk.cpu().pin_memory()
    out = torch.zeros((n, 32), dtype=torch.uint8).pin_memory()
    c = T.Context(0, mem_budget=40 << 20)
    try:
        c.kem_dec_ptr(S, n, out, ct_h, sk_h)
        torch.cuda.synchronize()
        assert c.workspace_bytes <= 40 << 20
    finally:
        c.close()
    assert torch.equal(out, ss.cpu())
