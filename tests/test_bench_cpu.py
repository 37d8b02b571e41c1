"""bench.py's host-link bound on an end-to-end step (pure arithmetic, no GPU)."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_link_bound_overlaps_the_smaller_transfer(bench):
    # 33.5 MB in, 83.9 MB out at 191 / 208 GB/s alone and 166 GB/s each way together
    t = bench.link_bound_s(33554432, 83886080, 191.0, 208.0, 166.0)
    assert t == pytest.approx(33554432 / 166e9 + (83886080 - 33554432) / 191e9)
    # never faster than the larger transfer alone, never slower than both in series
    assert t >= 83886080 / 191e9
    assert t <= 33554432 / 208e9 + 83886080 / 191e9


def test_link_bound_symmetric_cases(bench):
    # more in than out: the remainder runs at the host-to-device rate
    t = bench.link_bound_s(100e6, 40e6, 190.0, 210.0, 160.0)
    assert t == pytest.approx(40e6 / 160e9 + 60e6 / 210e9)
    # equal transfers: all at the concurrent rate
    assert bench.link_bound_s(50e6, 50e6, 190.0, 210.0, 160.0) == pytest.approx(50e6 / 160e9)
