"""PRST-compatible proofs on the GPU: the Fermat test with proof points, the products, the
certificate and its verification through libkite_gb300.so, file for file against what the
reference's kite-prst wrote for the same numbers (tests/golden/prst.json)."""
import ctypes as C
import hashlib
import json
import os

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "prst.json")) as f:
    CASES = json.load(f)


def _md5s(d, prefix):
    out = {}
    for f in sorted(os.listdir(d)):
        if f.startswith(prefix + "."):
            with open(os.path.join(d, f), "rb") as fh:
                out[f[len(prefix) + 1:]] = hashlib.md5(fh.read()).hexdigest()
    return out


@pytest.mark.parametrize("c", CASES, ids=[f"{c['k']}_{c['n']}_a{c['base']}_c{c['count']}" for c in CASES])
def test_proof_files_identical_to_reference(lib, tmp_path, c):
    from ahnum_gb300 import prst
    k, n, a, count = c["k"], c["n"], c["base"], c["count"]
    r = prst.save(k, n, a, count, str(tmp_path), keep=True)
    assert format(r.res64, "016X") == c["res64"] and r.is_prp == c["is_prp"]
    assert format(r.raw_cert_res64, "016X") == c["raw_cert_res64"]
    assert format(prst.build(k, n, a, count, str(tmp_path), keep=True), "016X") == c["cert_res64"]
    assert _md5s(str(tmp_path), c["prefix"]) == c["files_md5"]
    res, M = prst.verify(k, n, os.path.join(str(tmp_path), c["prefix"] + ".cert"))
    assert format(res, "016X") == c["verify_res64"]
    assert M == n >> (count.bit_length() - 1)


def test_products_resume_and_cleanup(lib, tmp_path):
    """Products already on disk are reused; a stop between points returns PP_ABORTED and leaves
    the finished products; without keep the intermediate points and then the products go."""
    from ahnum_gb300 import native, prst
    from ahnum_gb300.kite import KiteError
    c = CASES[1]
    k, n, a, count = c["k"], c["n"], c["base"], c["count"]
    d = str(tmp_path)
    prst.save(k, n, a, count, d, keep=True)
    pre = os.path.join(d, c["prefix"])
    want = _md5s(d, c["prefix"])
    # drop the last product: the rerun recomputes it from the first ones
    os.remove(pre + ".prod.2")
    os.remove(pre + ".prod.2.md5")
    assert format(prst.save_products(k, n, a, count, d, keep=True), "016X") == c["raw_cert_res64"]
    assert _md5s(d, c["prefix"]) == want
    # a stop request before the first missing level
    for j in range(3):
        os.remove(pre + f".prod.{j}")
        os.remove(pre + f".prod.{j}.md5")
    flag = C.c_int(1)
    with pytest.raises(KiteError, match=str(native.PP_ABORTED)):
        prst.save_products(k, n, a, count, d, keep=True, abort=flag)
    # without keep: points 1..count-1 removed by the save step, the rest by the build step
    prst.save_products(k, n, a, count, d, keep=False)
    left = _md5s(d, c["prefix"])
    assert set(left) == {"proof.0", "proof.0.md5", f"proof.{count}", f"proof.{count}.md5"} | \
        {f"prod.{j}{s}" for j in range(3) for s in ("", ".md5")}
    assert format(prst.build(k, n, a, count, d, keep=False), "016X") == c["cert_res64"]
    assert set(_md5s(d, c["prefix"])) == {"cert", "cert.md5"}


def test_corrupt_point_is_refused(lib, tmp_path):
    """A point whose bytes no longer match its .md5 sidecar stops the product step."""
    from ahnum_gb300 import prst
    from ahnum_gb300.kite import KiteError
    c = CASES[3]
    k, n, a, count = c["k"], c["n"], c["base"], c["count"]
    d = str(tmp_path)
    prst.save(k, n, a, count, d, keep=True)
    p = os.path.join(d, c["prefix"] + ".proof.1")
    b = bytearray(open(p, "rb").read())
    b[-1] ^= 1
    open(p, "wb").write(bytes(b))
    for j in range(1):
        os.remove(os.path.join(d, c["prefix"] + f".prod.{j}"))
    with pytest.raises(KiteError):
        prst.save_products(k, n, a, count, d, keep=True)
