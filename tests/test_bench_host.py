"""Host-side helpers of bench.py (no GPU): the synthetic inputs, the profiled DRAM traffic
read from the committed ncu summaries, and the roofline peak lookup."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_kets_are_seeded_normalised_and_column_major(bench):
    X = bench.make_kets(300, 7, dtype=np.complex64)
    assert X.flags.f_contiguous and X.dtype == np.complex64 and X.shape == (300, 7)
    assert np.allclose(np.linalg.norm(X.astype(np.complex128), axis=0), 1.0, atol=1e-6)
    assert np.array_equal(X, bench.make_kets(300, 7, dtype=np.complex64))
    # another rank draws other kets
    assert not np.array_equal(X, bench.make_kets(300, 7, rank=1, dtype=np.complex64))


def test_profiled_traffic_of_the_streaming_kernel(bench):
    """The bench's roofline `traffic` is the committed ncu figure of the full launch."""
    t = bench.profile_traffic("cheb_stream_c32_256x256.md")
    assert t is not None and 2.0e9 < t < 4.0e9  # about 1.7 reads + 0.9 writes of a 1.07 GB block
    assert bench.profile_traffic("no_such_summary.md") is None


def test_peak_lookup(bench):
    peak, kind = bench.measured_peak_hbm()
    assert peak > 1000.0 and kind in ("measured", "fallback")


def test_every_profile_names_a_committed_command():
    """Each ncu summary gives the command that made it, and that command runs committed files
    only (bench.py, not a scratch script)."""
    pdir = os.path.join(ROOT, "profiles")
    for name in os.listdir(pdir):
        text = open(os.path.join(pdir, name)).read()
        assert "python bench.py" in text, name
        assert "_work/" not in text, name
