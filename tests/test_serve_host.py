"""Host side of the served request loop (ahnum_gb300/serve.py): the seeded arrival process and
the FFT-length step a confirmation run takes; no GPU."""


def test_served_arrivals_follow_the_workload():
    """The served workload's Poisson arrivals: k odd in [3, 10^4], n log-uniform in
    [10^5, 4 10^6], 80 % Fermat, arrival times increasing within the window, seeded."""
    from ahnum_gb300 import serve
    reqs = serve.poisson_requests(seed=7, rate_per_s=50.0, duration_s=60.0)
    assert len(reqs) > 2000
    assert all(r.k % 2 == 1 and 3 <= r.k <= 10_000 for r in reqs)
    assert all(100_000 <= r.n <= 4_000_000 for r in reqs)
    assert all(0 < a.arrival < b.arrival <= 60.0 for a, b in zip(reqs, reqs[1:]))
    share = sum(r.kind == serve.FERMAT for r in reqs) / len(reqs)
    assert 0.75 < share < 0.85
    assert [(r.k, r.n) for r in serve.poisson_requests(7, 50.0, 1.0)] == \
           [(r.k, r.n) for r in serve.poisson_requests(7, 50.0, 1.0)]
    assert serve.next_fft_len(16384) == 17280 and serve.next_fft_len(20160) == 20480
