"""Generates tests/golden/prst.json: PRST-format proof files made by the reference's own
`kite-prst` (tools/kite_prst.c with src/prstproof.c, built from the reference sources by
`make -C oracle ref` into oracle/_ref/kite-prst).

For each case it runs, in a scratch directory,
    kite-prst K*2^N-1 -fermat a A -proof save C keep     (test + points + products)
    kite-prst K*2^N-1 -fermat a A -proof build C keep    (certificate)
    kite-prst K*2^N-1 -proof cert prst_<fp>.cert         (verification)
and records the RES64 lines it prints, the iteration stored in every point file, and the MD5 of
every file it leaves (points
prst_<fp>.proof.i, products prst_<fp>.prod.j, certificate prst_<fp>.cert, and their .md5
sidecars).  For the first case it also keeps the bytes of a few files (base64), so that the
file reader and writer can be checked without a GPU.

Usage:  python tests/golden/make_prst_golden.py     (needs oracle/_ref/kite-prst; ~1 min)
"""
from __future__ import annotations

import base64
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
PRST = os.path.join(REPO, "oracle", "_ref", "kite-prst")

# (k, n, base, point count): an even n, an odd n (odd spacings at every level), a probable
# prime, and base 5
CASES = [
    (9357, 20000, 3, 16),
    (1203, 30011, 3, 8),
    (3, 18123, 3, 4),
    (4705, 16001, 5, 2),
]
KEEP_BYTES = ("proof.0", "proof.8", "proof.16", "prod.0", "cert")


def _run(args, cwd):
    p = subprocess.run([PRST] + args, cwd=cwd, capture_output=True, text=True, timeout=600)
    if p.returncode != 0:
        raise RuntimeError(f"kite-prst {' '.join(args)} failed: {p.stdout}{p.stderr}")
    return p.stdout


def _res(pattern, text):
    m = re.search(pattern, text)
    return m.group(1) if m else None


def make_case(k, n, a, count, keep_bytes):
    expr = f"{k}*2^{n}-1"
    with tempfile.TemporaryDirectory() as d:
        out1 = _run([expr, "-fermat", "a", str(a), "-proof", "save", str(count), "keep"], d)
        out2 = _run([expr, "-fermat", "a", str(a), "-proof", "build", str(count), "keep"], d)
        cert = [f for f in os.listdir(d) if f.endswith(".cert")]
        out3 = _run([expr, "-proof", "cert", cert[0]], d)
        files, raw, iters = {}, {}, {}
        prefix = cert[0][:-len(".cert")]
        for f in sorted(os.listdir(d)):
            if not f.startswith(prefix):
                continue
            with open(os.path.join(d, f), "rb") as fh:
                b = fh.read()
            key = f[len(prefix) + 1:]
            files[key] = hashlib.md5(b).hexdigest()
            if key.startswith("proof.") and not key.endswith(".md5"):
                # the iteration word of the header (magic, app id, fingerprint, iteration)
                iters[int(key.split(".")[1])] = int.from_bytes(b[12:16], "little")
            if keep_bytes and key in KEEP_BYTES:
                raw[key] = base64.b64encode(b).decode()
        case = {
            "k": k, "n": n, "base": a, "count": count, "prefix": prefix,
            "is_prp": "probable prime" in out1,
            # a probable prime prints no RES64 line: its residue a^(N-1) mod N is 1
            "res64": _res(r"is not prime\. RES64: ([0-9A-F]{16})", out1) or "0000000000000001",
            "raw_cert_res64": _res(r"raw certificate RES64: ([0-9A-F]{16})", out1),
            "cert_res64": _res(r"certificate RES64: ([0-9A-F]{16})", out2),
            "verify_res64": _res(r"certificate RES64: ([0-9A-F]{16})", out3),
            "point_iterations": [iters[i] for i in range(count + 1)],
            "files_md5": files,
        }
        if raw:
            case["files_b64"] = raw
        return case


def main():
    if not os.path.exists(PRST):
        sys.exit(f"{PRST} is missing: run `make -C oracle ref` first")
    cases = [make_case(k, n, a, c, i == 0) for i, (k, n, a, c) in enumerate(CASES)]
    with open(os.path.join(HERE, "prst.json"), "w") as f:
        json.dump(cases, f, indent=1)
        f.write("\n")
    for c in cases:
        print(c["k"], c["n"], c["base"], c["count"], c["res64"], c["cert_res64"], len(c["files_md5"]))


if __name__ == "__main__":
    main()
