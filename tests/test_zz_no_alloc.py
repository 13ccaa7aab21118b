"""The decapsulation entry point that allocates nothing (tmvp_kem_dec_batch_noalloc).

Callers that cannot allocate device memory -- a host whose GPU memory belongs
to its own pool allocator, a serving process that forbids allocation after
start-up so its latency stays flat -- use this entry point; it works out of
a fixed array in device global memory instead of a context workspace.

The tests call it through the C ABI and check, bit for bit, against the
allocating entry point (tmvp_kem_dec_batch):
  * calls in a row on Saber and FireSaber at the 1024-instance maximum
    (FireSaber's GenMatrix stream is the largest the array is sized for) and
    on Sable with the INT8 tensor-core form, tampered ciphertexts included;
  * the status word the GPU fills: TMVP_OK for good keys, TMVP_EINVAL for a
    secret outside the tensor-core range (and TMVP_OK again on the next call);
  * that free device memory does not change across calls, including calls
    with the persistent tcgen05 launch shape chosen;
  * that a batch above the documented maximum is refused.
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_BATCH = 1024  # TMVP_NOALLOC_MAX_BATCH


def _dev(t):
    return ctypes.c_void_p(t.data_ptr())


def _keys(T, ctx, set_id, n, seed):
    coins = T.splitmix_bytes(seed, n * 96).reshape(n, 96)
    pk, sk = ctx.kem_keypair(set_id, coins)
    ct, ss_enc = ctx.kem_enc(set_id, pk, T.splitmix_bytes(seed + 1, n * 32).reshape(n, 32))
    return sk, ct, ss_enc


def _noalloc(T, set_id, ct_d, sk_d, form, status_d, stream):
    import torch
    n = ct_d.shape[0]
    ss_d = torch.full((n, 32), 0xAA, dtype=torch.uint8, device=ct_d.device)
    rc = T.lib().tmvp_kem_dec_batch_noalloc(set_id, n, _dev(ss_d), _dev(ct_d), _dev(sk_d), form,
                                            _dev(status_d), ctypes.c_void_p(stream.cuda_stream))
    assert rc == T.OK
    return ss_d


def test_noalloc_decaps_matches_allocating_path(kem):
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    status = torch.full((1,), 12345, dtype=torch.int32, device=dev)
    cases = [(T.SABER, MAX_BATCH, T.FORM_AUTO), (T.FIRESABER, MAX_BATCH, T.FORM_AUTO),
             (T.SABLE, 333, T.FORM_INT8_TC)]
    for call, (set_id, n, form) in enumerate(cases):
        sk, ct, ss_enc = _keys(T, ctx, set_id, n, 555 + 10 * call)
        # tamper with every fifth ciphertext: implicit rejection must agree too
        ct[::5, 3] ^= 0x41
        want = ctx.kem_dec(set_id, ct, sk, form=form)  # allocating entry point
        ct_d = torch.from_numpy(ct).to(dev)
        sk_d = torch.from_numpy(sk).to(dev)
        torch.cuda.synchronize()
        for rep in range(2):  # two calls in a row share the array
            status.fill_(12345)
            ss_d = _noalloc(T, set_id, ct_d, sk_d, form, status, stream)
            torch.cuda.synchronize()
            assert int(status.item()) == T.OK
            got = ss_d.cpu().numpy()
            assert np.array_equal(got, want), f"case {call} call {rep}: keys differ from tmvp_kem_dec_batch"
        keep = np.ones(n, bool)
        keep[::5] = False
        assert np.array_equal(got[keep], ss_enc[keep])


def test_noalloc_reports_out_of_range_secret(kem):
    """A secret coefficient outside the tensor-core forms' exact range is
    reported through the status word, as the allocating path reports it."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    n = 64
    sk, ct, ss_enc = _keys(T, ctx, T.SABER, n, 901)
    bad = sk.copy()
    bad[5, 0] = 100          # coefficient 0 of instance 5's first secret polynomial := 100
    bad[5, 1] &= 0xE0        # (13-bit packing: bits 8..12 sit in byte 1)
    with pytest.raises(T.TmvpError) as e:
        ctx.kem_dec(T.SABER, ct, bad, form=T.FORM_FP8_TCGEN05)
    assert e.value.code == T.EINVAL
    status = torch.full((1,), 12345, dtype=torch.int32, device=dev)
    ct_d = torch.from_numpy(ct).to(dev)
    _noalloc(T, T.SABER, ct_d, torch.from_numpy(bad).to(dev), T.FORM_FP8_TCGEN05, status, stream)
    torch.cuda.synchronize()
    assert int(status.item()) == T.EINVAL
    # the error bits do not leak into the next call
    ss_d = _noalloc(T, T.SABER, ct_d, torch.from_numpy(sk).to(dev), T.FORM_FP8_TCGEN05, status, stream)
    torch.cuda.synchronize()
    assert int(status.item()) == T.OK
    assert np.array_equal(ss_d.cpu().numpy(), ss_enc)


def test_noalloc_allocates_nothing(kem):
    """Free device memory is the same before and after a run of calls, with
    one CTA per instance and with the persistent tcgen05 launch shape."""
    import torch
    T, ctx = kem
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    n = 512
    sk, ct, ss_enc = _keys(T, ctx, T.SABER, n, 1201)
    ct_d = torch.from_numpy(ct).to(dev)
    sk_d = torch.from_numpy(sk).to(dev)
    status = torch.zeros((1,), dtype=torch.int32, device=dev)
    outs = [torch.empty((n, 32), dtype=torch.uint8, device=dev) for _ in range(4)]
    L = T.lib()
    sidx = ctypes.c_void_p(stream.cuda_stream)

    def call(out):
        assert L.tmvp_kem_dec_batch_noalloc(T.SABER, n, _dev(out), _dev(ct_d), _dev(sk_d), T.FORM_AUTO,
                                            _dev(status), sidx) == T.OK

    try:
        for shape in (-1, 0):  # one CTA per instance; persistent kernel, as many CTAs as fit
            for step in (0, 2):  # decryption, re-encryption
                T.tune_set(step, T.SABER, shape)
            call(outs[0])  # warm-up: loads the kernels of this shape
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info(dev)[0]
            for out in outs:
                call(out)
            torch.cuda.synchronize()
            free1 = torch.cuda.mem_get_info(dev)[0]
            assert free1 == free0, f"shape {shape}: free memory changed by {free0 - free1} bytes"
            assert int(status.item()) == T.OK
            for out in outs:
                assert np.array_equal(out.cpu().numpy(), ss_enc), f"shape {shape}"
    finally:
        for step in (0, 2):
            T.tune_set(step, T.SABER, -1)


def test_noalloc_rejects_oversize_batch(kem):
    import torch
    T, ctx = kem
    n = MAX_BATCH + 1
    z = T.sizes(T.SABER)
    dev = torch.device("cuda", 0)
    ct = torch.zeros((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    sk = torch.zeros((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ss = torch.zeros((n, 32), dtype=torch.uint8, device=dev)
    assert T.lib().tmvp_kem_dec_batch_noalloc(T.SABER, n, _dev(ss), _dev(ct), _dev(sk), T.FORM_AUTO,
                                              None, None) == T.EINVAL
