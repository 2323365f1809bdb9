"""TimeSequence host logic (src/timesequence.jl) against the reference's own doctest values."""
import numpy as np
import pytest

from lmgpu.timesequence import TimeSequence, differentiate, integrate


def test_constructors_and_lookup():
    ts = TimeSequence(np.arange(0, 1.01, 0.1), np.arange(0, 1.01, 0.1) ** 2)
    assert len(ts) == 11
    assert ts[0.3] == pytest.approx(0.09)
    assert ts[0.3 + 1e-9] == ts[0.3]          # atol sqrt(eps) lookup
    assert ts.get(0.35, "missing") == "missing"
    with pytest.raises(KeyError):
        ts[0.35]
    with pytest.raises(ValueError):
        TimeSequence([0.0, 1.0], [1.0])
    assert len(TimeSequence()) == 0


def test_setindex_keeps_order_and_delete():
    ts = TimeSequence([0.0, 1.0], ["a", "c"])
    ts[0.5] = "b"
    ts[1.0] = "C"
    assert ts.times == [0.0, 0.5, 1.0] and ts.values == ["a", "b", "C"]
    ts.delete(0.5)
    assert ts.times == [0.0, 1.0]
    assert list(ts) == [(0.0, "a"), (1.0, "C")]


def test_differentiate_doctest():
    # src/timesequence.jl:161-191: f(t) = t on 0:0.1:10 -> 1.0 at the midpoints 0.05, 0.15, ...
    t = np.arange(0, 101) * 0.1
    d = differentiate(TimeSequence(t, list(t)))
    assert len(d) == 100
    np.testing.assert_allclose(d.times[:4], [0.05, 0.15, 0.25, 0.35], atol=1e-12)
    np.testing.assert_allclose(d.values, 1.0, atol=1e-9)


def test_integrate_doctest():
    # src/timesequence.jl:220-250: f(t) = t -> t^2/2: 0.0, 0.005, 0.02, 0.045, 0.08, ...
    t = np.arange(0, 101) * 0.1
    F = integrate(TimeSequence(t, list(t)))
    assert len(F) == 101
    np.testing.assert_allclose(F.values[:5], [0.0, 0.005, 0.02, 0.045, 0.08], atol=1e-12)
    np.testing.assert_allclose(F.values, t ** 2 / 2, atol=1e-9)


def test_map_copy_equality():
    ts = TimeSequence([0.0, 1.0], [np.ones(3), np.zeros(3)])
    c = ts.copy()
    assert c == ts
    c.values[0][0] = 5.0
    assert c != ts
    assert ts.map(lambda v: v + 1).values[1].tolist() == [1.0, 1.0, 1.0]
