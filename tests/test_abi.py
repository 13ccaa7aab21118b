"""C ABI checks that need no GPU: the library loads, exports every entry point
include/tmvp_kem.h declares, and agrees with the oracle on sizes."""
import ctypes
import subprocess

import pytest


@pytest.fixture(scope="module")
def T():
    import tmvpkem
    tmvpkem.build.build()
    return tmvpkem


def test_exports_every_declared_symbol(T):
    names = T.exported_symbols()
    assert len(names) >= 25
    L = T.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", T.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(names) <= exported


def test_param_sizes_match_oracle(T, oracle):
    for s in range(6):
        z, p = T.sizes(s), oracle.params(s)
        assert (z.l, z.eq, z.ep, z.et, z.mu) == (p.l, p.eq, p.ep, p.et, p.mu)
        assert (z.pk_bytes, z.sk_bytes, z.ct_bytes, z.indcpa_sk_bytes) == (
            p.pk_bytes, p.sk_bytes, p.ct_bytes, p.indcpa_sk_bytes)
    # Saber l=3 byte layout of the reference (params.h:32-48)
    z = T.sizes(T.SABER)
    assert (z.pk_bytes, z.sk_bytes, z.ct_bytes) == (992, 2304, 1088)
    z = T.sizes(T.SABLE)
    assert (z.pk_bytes, z.sk_bytes, z.ct_bytes) == (896, 1152, 1024)


def test_invalid_arguments(T):
    s = T.Sizes()
    assert T.lib().tmvp_param_sizes(17, ctypes.byref(s)) == T.EINVAL
    assert T.lib().tmvp_kem_dec_batch(None, 1, 1, None, None, None, 0, None) == T.EINVAL
    assert T.lib().tmvp_strerror(T.ENOMEM).decode().startswith("device workspace")
    assert T.lib().tmvp_ref_batch(0) == 1 and T.lib().tmvp_ref_batch(1) == 512
    # context settings and the self-test refuse a null context before any CUDA call
    assert T.lib().tmvp_ctx_set_host_ramp(None, 1) == T.EINVAL
    assert T.lib().tmvp_ctx_set_host_chunk(None, 16384) == T.EINVAL
    assert T.lib().tmvp_ctx_set_dev_chunk(None, 32768) == T.EINVAL
    assert T.lib().tmvp_ctx_set_warp_hash(None, 2048) == T.EINVAL
    assert T.lib().tmvp_ctx_set_pair_hash(None, 16384) == T.EINVAL
    busy = ctypes.c_double()
    assert T.lib().tmvp_ctx_stage_busy(None, 0, ctypes.byref(busy)) == T.EINVAL
    assert T.lib().tmvp_selftest_bounded_wait(None, None) == T.EINVAL


def test_context_without_gpu_is_refused(T):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert T.lib().tmvp_ctx_create(0, 0, ctypes.byref(h)) == T.ENOTSUP
    assert T.lib().crypto_kem_keypair(None, None) == T.ENOTSUP


def test_genmatrix_bytes(T, oracle):
    """One key's GenMatrix stream is the l x l 13-bit (Saber) or 11-bit (Sable)
    polynomials GenMatrix unpacks: l * l * eq * 32 bytes; unknown sets give 0."""
    for s in range(6):
        p = oracle.params(s)
        assert T.genmatrix_bytes(s) == p.l * p.l * p.eq * 32
    assert T.genmatrix_bytes(T.SABER) == 3744
    assert T.lib().tmvp_genmatrix_bytes(17) == 0


def test_tune_table_and_cache_file(T, tmp_path):
    """The autotuner's per-batch-bucket pass settings and launch shapes round
    trip through the cache file; buckets are ceil(log2 n); malformed lines and
    out-of-range values are refused (no GPU needed)."""
    T.tune_clear()
    try:
        assert T.tune_pass_get(T.SABER, 65536) is None
        T.tune_pass_set(T.SABER, 65536, 16384, 8, 8192, 2)
        T.tune_pass_set(T.SABLE, 3000, 0, 0, 0, 0)
        assert T.tune_pass_get(T.SABER, 40000) == {"dev_chunk": 16384, "front_cap": 8, "host_chunk": 8192,
                                                    "host_ramp": 2}          # same bucket (2^16)
        assert T.tune_pass_get(T.SABER, 32768) is None                       # bucket 2^15
        assert T.tune_pass_get(T.SABLE, 4096)["dev_chunk"] == 0              # 3000 and 4096: bucket 2^12
        assert T.lib().tmvp_tune_set(T.TMVP_STEP_REENC if hasattr(T, "TMVP_STEP_REENC") else 2, T.SABER, 1) == T.OK
        for bad in ((100, 0, 0, 0), (0, 65, 0, 0), (0, 0, 512, 0), (0, 0, 0, 5), (-1, 0, 0, 0)):
            with pytest.raises(T.TmvpError):
                T.tune_pass_set(T.SABER, 1024, *bad)
        path = str(tmp_path / "tune.txt")
        T.tune_save(path)
        T.tune_clear()
        assert T.tune_pass_get(T.SABER, 65536) is None and T.tune_get(2, T.SABER) == -1
        T.tune_load(path)
        assert T.tune_pass_get(T.SABER, 65536)["front_cap"] == 8
        assert T.tune_pass_get(T.SABLE, 4000)["host_chunk"] == 0
        assert T.tune_get(2, T.SABER) == 1
        with open(path, "a") as f:
            f.write("pass 1 16 100 0 0 0\nnonsense\n")
        with pytest.raises(T.TmvpError):
            T.tune_load(path)  # the good lines still load
        assert T.tune_pass_get(T.SABER, 65536)["dev_chunk"] == 16384
        with pytest.raises(T.TmvpError):
            T.tune_load(str(tmp_path / "missing.txt"))
    finally:
        T.tune_clear()
