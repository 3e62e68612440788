"""CPU oracle (test infrastructure only): a C restatement of the reference's arithmetic and,
where the reference sources are present, the reference's own portable backends.  Only the
tests, the smoke check and the benchmark's CPU-baseline leg use it, as the checker."""
