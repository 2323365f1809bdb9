"""Host-side helpers of bench.py (no GPU): the synthetic inputs, the profiled DRAM traffic
read from the committed ncu record, and the roofline peak lookup."""
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


def test_profiled_traffic_of_the_streaming_kernel(bench, tmp_path, monkeypatch):
    """The bench's roofline `traffic` comes from a committed ncu record that names the kernel's
    sources and their sha256; a record whose sources changed is refused."""
    import json
    t, units, rec = bench.profile_traffic()
    if t is None:  # the kernel changed since the capture: the record must say so, not be used
        assert rec.startswith("stale") or rec == "no ncu record"
    else:
        per_unit = t / units  # bytes per site-ket of one launch
        assert 8 * 1.5 < per_unit < 8 * 4.0, per_unit  # between 1.5 and 4 passes over a c32 block
    assert bench.profile_traffic("no_such_record.json") == (None, None, "no ncu record")
    # a record whose hash does not match its sources
    src = json.loads((bench.ROOT / "profiles" / bench.TRAFFIC_RECORD).read_text())
    src["source_sha256"] = "0" * 64
    fake = tmp_path / "profiles"
    fake.mkdir()
    (fake / "x.json").write_text(json.dumps(src))
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    for rel in src["sources"]:
        (tmp_path / rel).parent.mkdir(parents=True, exist_ok=True)
        (tmp_path / rel).write_text("changed kernel")
    t, _, why = bench.profile_traffic("x.json")
    assert t is None and why.startswith("stale")


def test_peak_lookup(bench):
    peak, kind = bench.measured_peak_hbm()
    assert peak > 1000.0 and kind in ("measured", "fallback")


def test_every_profile_names_a_committed_command():
    """Each ncu summary gives the command that made it, and that command runs committed files
    only (bench.py, not a scratch script)."""
    pdir = os.path.join(ROOT, "profiles")
    for name in os.listdir(pdir):
        text = open(os.path.join(pdir, name)).read()
        if name.endswith(".json"):
            import json
            text = json.loads(text)["command"]
        assert "python bench.py" in text, name
        assert "_work/" not in text, name
