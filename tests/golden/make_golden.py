"""Generates the golden fixtures in this directory.

Sources, all from the reference repository (path given by --ref):
  * the test vectors in TMVP-Saber/SABER-GPU/include/tv.h and
    TMVP_SABLE/include/tv.h, read as text;
  * outputs of the reference's own Saber/Sable kernels, compiled for the host
    by oracle/ref_build (launch sequences of saber_enc/saber_dec and
    SABLE_enc/SABLE_dec replayed one instance at a time).

Run from the repository root:  python tests/golden/make_golden.py --ref <reference root>
Writes tests/golden/saber_l3.npz, tests/golden/sable_l3.npz and
tests/golden/matvec.npz.
"""
import argparse
import os
import re
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import pyoracle as O  # noqa: E402
from oracle import pyref as R  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_tv(path):
    """Arrays declared as `[static] <type> <name>[...] = { ... };` in a tv.h."""
    txt = open(path).read()
    out = {}
    for m in re.finditer(r'(?:static\s+)?(\w+)\s+(\w+)\s*\[[^\]]*\]\s*=\s*\{([^}]*)\}', txt):
        typ, name, body = m.groups()
        vals = [int(v, 0) for v in body.replace("\n", " ").split(",") if v.strip()]
        out[name] = np.array(vals, dtype=np.uint16 if typ == "uint16_t" else np.uint8)
    return out


def splitmix_bytes(seed: int, n: int) -> np.ndarray:
    """SplitMix64 stream as bytes (the seed generator the tests use)."""
    out = np.empty(n, np.uint8)
    x = seed & 0xFFFFFFFFFFFFFFFF
    for i in range(0, n, 8):
        x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        z ^= z >> 31
        out[i:i + 8] = np.frombuffer(int(z).to_bytes(8, "little"), np.uint8)[:min(8, n - i)]
    return out


def scheme_fixture(scheme, set_id, tv, pk_name, n_random=6):
    pk = tv[pk_name].astype(np.uint8).tobytes()
    sk = tv["sk_tv"].tobytes()
    buf = tv["buf_tv"].tobytes()
    d = {"tv_pk": np.frombuffer(pk, np.uint8), "tv_sk": np.frombuffer(sk, np.uint8),
         "tv_buf": np.frombuffer(buf, np.uint8),
         "tv_m": tv["m_tv"].astype(np.uint8)}
    if "A" in tv:
        d["tv_A"] = tv["A"]
    if "kr_tv" in tv:
        d["tv_kr"] = tv["kr_tv"]
    # reference kernels on the test vectors (mode 1 = TMVP on CUDA cores)
    ct, k = R.enc(scheme, 1, pk, buf[:32])
    kd, cmp, diff = R.dec(scheme, 1, ct, sk)
    assert kd == k and diff == 0
    d["tv_ct"] = np.frombuffer(ct, np.uint8)
    d["tv_ss"] = np.frombuffer(k, np.uint8)
    # seeded instances: keypair by the oracle (the reference has no keypair),
    # encaps and decaps by the reference kernels; plus one tampered ciphertext
    p = O.params(set_id)
    cts, sss, pks, sks, coins = [], [], [], [], []
    for i in range(n_random):
        kc = splitmix_bytes(1000 + 17 * i + set_id, 96)
        pki, ski = O.kem_keypair(set_id, kc)
        ec = splitmix_bytes(5000 + 31 * i + set_id, 32)
        cti, ki = R.enc(scheme, 1 + (i & 1), pki, ec.tobytes())
        kdi, _, di = R.dec(scheme, 2 - (i & 1), cti, ski)
        assert kdi == ki and di == 0
        pks.append(np.frombuffer(pki, np.uint8)); sks.append(np.frombuffer(ski, np.uint8))
        cts.append(np.frombuffer(cti, np.uint8)); sss.append(np.frombuffer(ki, np.uint8))
        coins.append(ec)
    d.update(rnd_pk=np.stack(pks), rnd_sk=np.stack(sks), rnd_ct=np.stack(cts),
             rnd_ss=np.stack(sss), rnd_coins=np.stack(coins))
    # implicit rejection: the spec key for a tampered ciphertext (oracle; the
    # reference's cmov is a no-op, so its key differs by design)
    bad = bytearray(cts[0].tobytes()); bad[7] ^= 0x20
    kb, fail = O.kem_dec(set_id, bytes(bad), sks[0].tobytes())
    assert fail == 1
    d.update(rej_ct=np.frombuffer(bytes(bad), np.uint8), rej_ss=np.frombuffer(kb, np.uint8))
    assert d["rnd_ct"].shape[1] == p.ct_bytes
    return d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True)
    a = ap.parse_args()
    O.build()
    if not R.build(a.ref):
        sys.exit("reference tree not found")
    sab = parse_tv(os.path.join(a.ref, "TMVP-Saber/SABER-GPU/include/tv.h"))
    sbl = parse_tv(os.path.join(a.ref, "TMVP_SABLE/include/tv.h"))
    np.savez_compressed(os.path.join(HERE, "saber_l3.npz"), **scheme_fixture("saber", O.SABER, sab, "pk"))
    np.savez_compressed(os.path.join(HERE, "sable_l3.npz"), **scheme_fixture("sable", O.SABLE, sbl, "pk_tv"))
    # raw matrix-vector products through the reference's TMVP (mode 1) kernels
    mv = {}
    for scheme, eq in (("saber", 13), ("sable", 11)):
        rs = splitmix_bytes(77 + eq, 2 * 9 * 256 * 4)
        A = (np.frombuffer(rs.tobytes(), np.uint16)[:4 * 9 * 256].reshape(4, 3, 3, 256) & ((1 << eq) - 1))
        sb = splitmix_bytes(99 + eq, 4 * 768)
        s = np.stack([O.gen_secret(O.SABER, sb[32 * i:32 * i + 32]) for i in range(4)]).astype(np.int16)
        s = s.astype(np.int8)
        out = np.stack([R.matvec(scheme, 1, A[i], s[i].astype(np.int16).astype(np.uint16))
                        for i in range(4)]) & ((1 << eq) - 1)
        mv[f"{scheme}_A"] = A.astype(np.uint16)
        mv[f"{scheme}_s"] = s
        mv[f"{scheme}_out"] = out.astype(np.uint16)
    np.savez_compressed(os.path.join(HERE, "matvec.npz"), **mv)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
