"""Gauge fields (src/zoo/magneticfields.jl, src/operators/magneticfield.jl).

Each field is a list of components the device assembly kernel evaluates: a kind, a fixed
point and a time-dependent amplitude.  The line integrals themselves are evaluated on the
device exactly as the reference writes them.
"""
from __future__ import annotations

import math
import warnings

from . import _lib


class AbstractField:
    def components(self):
        """[(kind, px, py)] -- the fixed part, one entry per term."""
        raise NotImplementedError

    def amplitudes(self):
        """[float] -- the time-dependent part, aligned with components()."""
        raise NotImplementedError

    def __add__(self, other):
        return FieldSum(_terms(self) + _terms(other))

    def __eq__(self, other):
        return type(self) is type(other) and self.components() == other.components() \
            and self.amplitudes() == other.amplitudes()

    def __hash__(self):
        return hash((type(self).__name__, tuple(self.components()), tuple(self.amplitudes())))


def _terms(f):
    return list(f.fields) if isinstance(f, FieldSum) else [f]


class NoField(AbstractField):
    """Zero magnetic field (src/operators/magneticfield.jl:43-44)."""

    def components(self):
        return []

    def amplitudes(self):
        return []

    def __repr__(self):
        return "NoField()"


class LandauGauge(AbstractField):
    """LI = (x1+x2)(y2-y1) B/2 (src/zoo/magneticfields.jl:11-15)."""

    def __init__(self, B: float):
        self.B = float(B)

    def components(self):
        return [(_lib.LM_FIELD_LANDAU, 0.0, 0.0)]

    def amplitudes(self):
        return [self.B]

    def __repr__(self):
        return f"LandauGauge({self.B})"


class SymmetricGauge(AbstractField):
    """LI = (x1 y2 - x2 y1)/2 B (src/zoo/magneticfields.jl:27-31)."""

    def __init__(self, B: float):
        self.B = float(B)

    def components(self):
        return [(_lib.LM_FIELD_SYMMETRIC, 0.0, 0.0)]

    def amplitudes(self):
        return [self.B]

    def __repr__(self):
        return f"SymmetricGauge({self.B})"


class PointFlux(AbstractField):
    """Point flux through ``point`` in the axial or singular gauge (src/zoo/magneticfields.jl:46-104)."""

    def __init__(self, flux: float, point=(0.0, 0.0), gauge: str = "axial"):
        if gauge not in ("axial", "singular"):
            raise ValueError(f"Invalid gauge: {gauge}; expected one of ('axial', 'singular')")
        self.flux = float(flux)
        self.point = (float(point[0]), float(point[1]))
        if not all(math.isfinite(v) for v in self.point):
            raise ValueError("flux point must be finite")
        self.gauge = gauge

    def components(self):
        kind = _lib.LM_FIELD_POINTFLUX_AXIAL if self.gauge == "axial" else _lib.LM_FIELD_POINTFLUX_SINGULAR
        return [(kind, self.point[0], self.point[1])]

    def amplitudes(self):
        return [self.flux]

    def __repr__(self):
        return f"PointFlux({self.flux}, {self.point}; gauge=:{self.gauge})"


class PointFluxes(AbstractField):
    """Several point fluxes of one gauge (src/zoo/magneticfields.jl:119-187)."""

    def __init__(self, fluxes, points, gauge: str = "axial"):
        if gauge not in ("axial", "singular"):
            raise ValueError(f"Invalid gauge: {gauge}")
        if not hasattr(fluxes, "__len__"):
            fluxes = [float(fluxes)] * len(points)
        if len(fluxes) != len(points):
            raise ValueError("Length of fluxes and points should be the same")
        self.fields = [PointFlux(f, p, gauge) for f, p in zip(fluxes, points)]
        self.gauge = gauge

    def components(self):
        return [c for f in self.fields for c in f.components()]

    def amplitudes(self):
        return [a for f in self.fields for a in f.amplitudes()]


class FieldSum(AbstractField):
    """Sum of fields (src/operators/magneticfield.jl:100-121)."""

    def __init__(self, fields):
        self.fields = list(fields)

    def components(self):
        return [c for f in self.fields for c in f.components()]

    def amplitudes(self):
        return [a for f in self.fields for a in f.amplitudes()]

    def __repr__(self):
        return " + ".join(repr(f) for f in self.fields)


def pbc_warning(field, lattice):
    """adapt_field's warning for a non-singular point flux on a lattice with boundaries."""
    if lattice.has_boundaries():
        for kind, _, _ in field.components():
            if kind == _lib.LM_FIELD_POINTFLUX_AXIAL:
                warnings.warn("Setting flux gauge to singular for a lattice with periodic boundary conditions")
                return
