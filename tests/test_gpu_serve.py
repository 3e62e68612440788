"""The served request loop: requests arriving while others run are admitted into the same
GPU batch (continuous batching); every verdict must equal the same test run alone through the
single-test API (kite_prp / kite_llr), and checkpoints in the reference's formats are written
for tests that pass the checkpoint interval."""
import os

import pytest

pytestmark = pytest.mark.gpu


def test_served_verdicts_equal_alone_runs(lib, tmp_path):
    from ahnum_gb300 import serve
    from ahnum_gb300.kite import llr, prp
    reqs = serve.poisson_requests(seed=11, rate_per_s=40.0, duration_s=0.5,
                                  n_range=(12_000, 90_000))
    assert len(reqs) >= 10 and any(r.kind == serve.LLR for r in reqs)
    srv = serve.Server(gerbicz_block=200, checkpoint_dir=str(tmp_path), checkpoint_every=20_000)
    try:
        verdicts, stats = srv.serve(reqs)
    finally:
        srv.close()
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert stats["peak_active"] >= 4          # the tests overlapped on the device
    assert stats["checkpoints"] > 0 and os.listdir(tmp_path)
    for v in verdicts:
        if v.kind == serve.FERMAT:
            a = prp(v.k, v.n)
            assert a.rc == 0 and (a.res64, a.is_prp) == (v.res64, v.is_prime), v
        else:
            a = llr(v.k, v.n)
            assert a.rc == 0 and a.is_prime == v.is_prime, v
            if not a.is_prime and not a.factor:
                assert a.res64 == v.res64, v
        assert v.maxerr < 0.4


def test_checkpoint_files_are_reference_format(lib, tmp_path):
    """a checkpoint written by the batch is read back by kite_prp_checkpoint_iter"""
    import ctypes as C
    from ahnum_gb300.kite import Batch
    with Batch(gerbicz_block=200, gerbicz_blocks=4) as b:
        s = b.add_fermat(9357, 60000)
        for _ in range(6):
            b.step(1)
        path = str(tmp_path / "f.ckpt")
        assert lib.kc_batch_checkpoint(b.h, s, path.encode()) == 0
        it = C.c_uint64()
        assert lib.kite_prp_checkpoint_iter(path.encode(), 9357, 60000, 3, C.byref(it)) == 0
        assert it.value == 800   # verified at the check after 4 blocks of 200
