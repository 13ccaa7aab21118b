"""The decapsulation entry point that allocates nothing (tmvp_kem_dec_batch_noalloc).

Callers that cannot allocate device memory -- a host whose GPU memory belongs
to its own pool allocator, a serving process that forbids allocation after
start-up so its latency stays flat -- use this entry point; it works out of
a fixed array in device global memory instead of a context workspace.  The
test calls it through the C ABI twice in a row and checks each result against
the allocating entry point (tmvp_kem_dec_batch), bit for bit, and that a batch
above the documented maximum is refused.  The file is named to be collected
last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_decaps_matches_allocating_path(kem):
    import torch
    T, ctx = kem
    L = T.lib()
    L.tmvp_kem_dec_batch_noalloc.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                              ctypes.c_void_p]
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for call, (set_id, n, form) in enumerate([(T.SABER, 1024, T.FORM_AUTO),
                                              (T.SABLE, 333, T.FORM_INT8_TC)]):
        z = T.sizes(set_id)
        coins = T.splitmix_bytes(555 + call, n * 96).reshape(n, 96)
        pk, sk = ctx.kem_keypair(set_id, coins)
        ct, ss_enc = ctx.kem_enc(set_id, pk, T.splitmix_bytes(777 + call, n * 32).reshape(n, 32))
        # tamper with every fifth ciphertext: implicit rejection must agree too
        ct[::5, 3] ^= 0x41
        want = ctx.kem_dec(set_id, ct, sk, form=form)  # allocating entry point
        ct_d = torch.from_numpy(ct).to(dev)
        sk_d = torch.from_numpy(sk).to(dev)
        ss_d = torch.full((n, 32), 0xAA, dtype=torch.uint8, device=dev)
        torch.cuda.synchronize()
        rc = L.tmvp_kem_dec_batch_noalloc(set_id, n, _dev(ss_d), _dev(ct_d), _dev(sk_d), form,
                                          ctypes.c_void_p(stream.cuda_stream))
        assert rc == T.OK
        torch.cuda.synchronize()
        got = ss_d.cpu().numpy()
        assert np.array_equal(got, want), f"call {call}: keys differ from tmvp_kem_dec_batch"
        keep = np.ones(n, bool)
        keep[::5] = False
        assert np.array_equal(got[keep], ss_enc[keep])


def test_noalloc_rejects_oversize_batch(kem):
    import torch
    T, ctx = kem
    L = T.lib()
    L.tmvp_kem_dec_batch_noalloc.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                              ctypes.c_void_p]
    n = 1025  # TMVP_NOALLOC_MAX_BATCH + 1
    z = T.sizes(T.SABER)
    dev = torch.device("cuda", 0)
    ct = torch.zeros((n, z.ct_bytes), dtype=torch.uint8, device=dev)
    sk = torch.zeros((n, z.sk_bytes), dtype=torch.uint8, device=dev)
    ss = torch.zeros((n, 32), dtype=torch.uint8, device=dev)
    assert L.tmvp_kem_dec_batch_noalloc(T.SABER, n, _dev(ss), _dev(ct), _dev(sk), T.FORM_AUTO,
                                        None) == T.EINVAL
