"""The bench's workload: seeded lengths with the configuration's mix, and the
profiling categories that split it (5-smooth, prime, raw)."""
import numpy as np

import bench


def _smooth(n):
    for p in (2, 3, 5):
        while n % p == 0:
            n //= p
    return n == 1


def test_workload_is_the_seeded_mix():
    ns = bench.workload_sizes()
    assert len(ns) == bench.COUNT
    assert int(ns.sum()) == 33382845
    assert ns.min() >= 16 and ns.max() <= 65537 + 100


def test_categories_partition_the_workload():
    parts = {c: bench.workload_sizes(category=c) for c in ("smooth", "prime", "raw")}
    assert sum(len(v) for v in parts.values()) == bench.COUNT
    assert sum(int(v.sum()) for v in parts.values()) == int(bench.workload_sizes().sum())
    assert all(_smooth(int(n)) for n in parts["smooth"])
    assert all(bench.is_prime(int(n)) for n in parts["prime"])
    # each category keeps the workload's order
    full = list(bench.workload_sizes())
    it = iter(full)
    assert all(any(n == m for m in it) for n in parts["raw"])


def test_lengths_spec():
    assert list(bench.parse_lengths("4096*2,30011")) == [4096, 4096, 30011]
    assert np.asarray(bench.parse_lengths("7*3")).dtype == np.int64
