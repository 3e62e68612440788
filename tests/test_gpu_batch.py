"""The batched engine: tests of different k, n and FFT lengths run together to completion; each
verdict must equal the reference's golden residue and the same test run alone (kite_prp /
kite_llr on its own context), bit for bit."""
import pytest

pytestmark = pytest.mark.gpu

FERMAT = [
    (9357, 20000, 0x79291CD2F47CE48C),
    (8191, 25000, 0xD45538E6F07266C6),
    (3, 26459, 0x1),
    (5, 30000, 0xB7980452FDBC4183),
    (7, 40001, 0xEB4ADF0EC94C09E6),
    (1, 44497, 0x1),
    (1365, 45678, 0xEF89209BAE5FF19A),
    (9999, 60000, 0x1C248905164FFD34),
]
LLR = [
    (3, 26459, None),
    (9357, 20000, 0xDC52061161A0DE1C),
    (9357, 25000, 0x54A27E03D75F2447),
]


@pytest.mark.parametrize("form", ["default", "persistent", "two_parts", "one_stream"])
def test_batch_mixed_fermat_and_llr(lib, monkeypatch, form):
    """Every form of a block gives the golden verdicts: one launch per pass with the slots in
    three parts on three streams (the default), in two parts, on one stream, and the persistent
    kernel over one queue."""
    from ahnum_gb300.kite import Batch, prp
    monkeypatch.delenv("KITE_GB300_BATCH_PERSISTENT", raising=False)
    monkeypatch.delenv("KITE_GB300_BATCH_SPLIT", raising=False)
    if form == "persistent":
        monkeypatch.setenv("KITE_GB300_BATCH_PERSISTENT", "1")
    elif form != "default":
        monkeypatch.setenv("KITE_GB300_BATCH_SPLIT", "2" if form == "two_parts" else "1")
    with Batch(gerbicz_block=200, gerbicz_blocks=20) as b:
        slots = {}
        for k, n, res in FERMAT:
            s = b.add_fermat(k, n)
            assert s >= 0
            slots[s] = ("F", k, n, res)
        for k, n, res in LLR:
            s = b.add_llr(k, n)
            assert s >= 0
            slots[s] = ("L", k, n, res)
        b.run()
        lengths = set()
        for s, (kind, k, n, res) in slots.items():
            st, r = b.result(s)
            assert st == 1, (kind, k, n, r.rc)
            assert r.rc == 0 and r.maxerr < 0.4
            lengths.add(r.fft_len)
            if kind == "F":
                assert r.res64 == res, f"{k}*2^{n}-1 {r.res64:016X}"
                assert bool(r.is_prp) == (res == 1)
                assert r.gerbicz_errors == 0
            else:
                if res is None:
                    assert r.is_prp  # V == 0: prime
                else:
                    assert not r.is_prp and r.res64 == res
        assert len(lengths) >= 4  # genuinely mixed lengths in one launch
    # alone vs in the mix: the same test through the single-test API
    r1 = prp(1365, 45678)
    assert r1.res64 == 0xEF89209BAE5FF19A


def test_batch_admission_budget(lib):
    from ahnum_gb300.kite import Batch
    with Batch(mem_budget=8 << 20) as b:
        ids = [b.add_fermat(9357, 369717, fft_len=28672) for _ in range(8)]
        assert ids[0] >= 0
        assert -2 in ids  # the budget refuses further admissions
        b.release(ids[0])
        assert b.add_fermat(9357, 369717, fft_len=28672) >= 0
