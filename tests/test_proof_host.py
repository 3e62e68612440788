"""Host-side parts of the PRST-compatible proof API (include/kite_proof.h), without a GPU:
fingerprints, point positions, the state-file writer and reader and their .md5 sidecars, against
files the reference's kite-prst wrote (tests/golden/prst.json, made by make_prst_golden.py)."""
import base64
import ctypes as C
import hashlib
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "prst.json")) as f:
    CASES = json.load(f)


def _words(b: bytes, off: int, n: int):
    return [int.from_bytes(b[off + 4 * i: off + 4 * i + 4], "little") for i in range(n)]


def _py_fingerprint(k, n):
    p = 3417905339
    return (k * pow(2, n, p) - 1) % p


def _py_unique(fp, ident: str):
    d = hashlib.md5(fp.to_bytes(4, "little") + ident.encode()).digest()
    return int.from_bytes(d[:4], "little")


@pytest.mark.parametrize("c", CASES, ids=[f"{c['k']}_{c['n']}" for c in CASES])
def test_fingerprints(lib, c):
    fp = lib.pp_fingerprint(c["k"], c["n"])
    assert fp == _py_fingerprint(c["k"], c["n"])
    assert c["prefix"] == f"prst_{fp}"
    assert lib.pp_unique_fingerprint(fp, b"3.20000") == _py_unique(fp, "3.20000")
    assert lib.pp_proof_fingerprint(c["k"], c["n"], c["base"]) == _py_unique(fp, f"{c['base']}.{c['n']}")


def test_points_match_the_files_iterations(lib):
    c = CASES[0]
    from ahnum_gb300 import native
    count = c["count"]
    pos = (C.c_uint32 * (count + 1))()
    lib.pp_points(c["n"], count, pos)
    assert pos[0] == 0 and pos[count] == c["n"]
    assert list(pos) == sorted(pos)
    fpP = lib.pp_proof_fingerprint(c["k"], c["n"], c["base"])
    for key in ("proof.0", "proof.8", "proof.16"):
        b = base64.b64decode(c["files_b64"][key])
        magic, app, fp, it = _words(b, 0, 4)
        assert magic == 0x9F2B3CD4 and app == 4 | native.PP_TYPE_VALUE << 16 and fp == fpP
        assert it == pos[int(key.split(".")[1])]


@pytest.mark.parametrize("c", CASES, ids=[f"{c['k']}_{c['n']}" for c in CASES])
def test_points_match_the_reference(lib, c):
    """pp_points gives the iterations the reference stored in its point files (odd n included)."""
    count = c["count"]
    pos = (C.c_uint32 * (count + 1))()
    lib.pp_points(c["n"], count, pos)
    assert list(pos) == c["point_iterations"]


@pytest.mark.parametrize("key", ["proof.0", "proof.16", "prod.0", "cert"])
def test_write_reproduces_the_reference_file(lib, tmp_path, key):
    """Reading a file the reference wrote and writing its values back gives the same bytes and
    the same .md5 sidecar."""
    from ahnum_gb300 import native
    c = CASES[0]
    raw = base64.b64decode(c["files_b64"][key])
    src = tmp_path / "in"
    src.write_bytes(raw)
    ptype = {"proof": native.PP_TYPE_VALUE, "prod": native.PP_TYPE_PRODUCT, "cert": native.PP_TYPE_CERT}[key.split(".")[0]]
    fp = lib.pp_fingerprint(c["k"], c["n"]) if ptype == native.PP_TYPE_CERT else \
        lib.pp_proof_fingerprint(c["k"], c["n"], c["base"])
    g = (native.PpGiant * 3)()
    it = C.c_int32(0)
    ng = 3 if ptype == native.PP_TYPE_CERT else 1
    assert lib.pp_read(str(src).encode(), ptype, fp, C.byref(it), g, ng) == 0
    dst = tmp_path / "out"
    assert lib.pp_write(str(dst).encode(), ptype, fp, it.value, g, ng) == 0
    assert dst.read_bytes() == raw
    assert hashlib.md5(raw).hexdigest() == c["files_md5"][key]
    assert (tmp_path / "out.md5").read_text() == c["files_md5"][key]
    if g[0].len >= 2:
        lo = g[0].w[0] | g[0].w[1] << 32
        assert lib.pp_res64(C.byref(g[0])) == lo
    for i in range(ng):
        lib.pp_giant_free(C.byref(g[i]))


def test_read_rejects_bad_files(lib, tmp_path):
    from ahnum_gb300 import native
    c = CASES[0]
    raw = base64.b64decode(c["files_b64"]["proof.16"])
    fpP = lib.pp_proof_fingerprint(c["k"], c["n"], c["base"])
    g = (native.PpGiant * 1)()
    it = C.c_int32(0)
    p = tmp_path / "f"
    p.write_bytes(raw)
    assert lib.pp_read(str(p).encode(), native.PP_TYPE_VALUE, fpP, C.byref(it), g, 1) == 0
    lib.pp_giant_free(C.byref(g[0]))
    # wrong fingerprint, wrong type
    assert lib.pp_read(str(p).encode(), native.PP_TYPE_VALUE, fpP ^ 1, C.byref(it), g, 1) != 0
    assert lib.pp_read(str(p).encode(), native.PP_TYPE_PRODUCT, fpP, C.byref(it), g, 1) != 0
    # a present sidecar must match; an absent one is not required
    (tmp_path / "f.md5").write_text("0" * 32)
    assert lib.pp_read(str(p).encode(), native.PP_TYPE_VALUE, fpP, C.byref(it), g, 1) != 0
    (tmp_path / "f.md5").write_text(hashlib.md5(raw).hexdigest())
    assert lib.pp_read(str(p).encode(), native.PP_TYPE_VALUE, fpP, C.byref(it), g, 1) == 0
    lib.pp_giant_free(C.byref(g[0]))
    # truncated value
    p.write_bytes(raw[:-4])
    os.remove(tmp_path / "f.md5")
    assert lib.pp_read(str(p).encode(), native.PP_TYPE_VALUE, fpP, C.byref(it), g, 1) != 0
    assert lib.pp_read(str(tmp_path / "missing").encode(), native.PP_TYPE_VALUE, fpP, C.byref(it), g, 1) != 0


def _reference_points(iterations, count):
    """PRST's point positions as the reference's loop computes them (src/prstproof.c:191-207),
    restated here as the checker of the library's closed form"""
    pos = [0] * (count + 1)
    M = 0
    for i in range(1, count):
        M = iterations
        j = count // 2
        while j > 0 and (i & (j * 2 - 1)) != 0:
            M //= 2
            if i & j:
                pos[i] += M
            if iterations & (count // j // 2):
                pos[i] += 1
            j //= 2
    pos[count] = iterations
    return pos, M


def test_points_closed_form_matches_the_reference_loop(lib):
    import random
    rng = random.Random(3)
    for _ in range(300):
        count = 1 << rng.randrange(1, 11)
        iterations = rng.choice([rng.randrange(count, 5000), rng.randrange(10**5, 2**31 - 1)])
        pos = (C.c_uint32 * (count + 1))()
        M = lib.pp_points(iterations, count, pos)
        want, wM = _reference_points(iterations, count)
        assert list(pos) == want and M == wM, (iterations, count)
