"""TimeSequence (src/timesequence.jl) and the device readout ring behind it.

``TimeSequence(f, ev(times))`` applies ``f`` to every moment of the evolution
(src/timesequence.jl:41-43).  When ``f`` is ``moment_density`` or ``moment_currents`` the
readouts go through a ``ReadoutRing``: each moment's local densities / bond currents are
computed on the device into a ring slot and downloaded asynchronously into pinned memory, and
the host collects an entry only when its slot is about to be reused (or at the end).  The
evolution loop therefore never waits for a step to finish before it launches the next one.
Any other ``f`` is called on each moment as it is yielded, as in the reference.
"""
from __future__ import annotations

import ctypes as C
import math
import weakref

import numpy as np

from .device import default_context
from .lattice import LatticeValue

_ATOL = math.sqrt(np.finfo(float).eps)  # `≈(t, atol=√eps())` of the reference's get/setindex!


class ReadoutRing:
    """``nslots`` device slots of ``length`` doubles with pinned host copies (lm_ring_*)."""

    def __init__(self, length: int, nslots: int = 8, ctx=None):
        self.ctx = ctx or default_context()
        p = C.c_void_p()
        self.ctx.check(self.ctx.lib.lm_ring_create(self.ctx.handle, int(nslots), int(length), C.byref(p)))
        self.handle = p
        self.nslots = int(nslots)
        self.length = int(length)
        weakref.finalize(self, self.ctx.lib.lm_ring_destroy, p)

    def push_density(self, state, t: float) -> int:
        seq = C.c_int64()
        self.ctx.check(self.ctx.lib.lm_ring_push_localdensity(self.handle, state.handle, float(t), C.byref(seq)))
        return seq.value

    def push_currents(self, H, state, t: float) -> int:
        dh = H.device(self.ctx)
        seq = C.c_int64()
        self.ctx.check(self.ctx.lib.lm_ring_push_currents(self.handle, dh.handle, state.handle, float(t),
                                                          C.byref(seq)))
        return seq.value

    def push_op_currents(self, H, state, t: float, op=None) -> int:
        """DensityCurrents (op None) or LocalOperatorCurrents of a SparseHamiltonian: the value
        of every stored entry, in CSC order."""
        from . import _lib
        from .sparse import _local_op
        dh = H.device(self.ctx)
        buf = _local_op(H, op)
        seq = C.c_int64()
        self.ctx.check(self.ctx.lib.lm_ring_push_op_currents(
            self.handle, dh.handle, state.handle, int(H.lattice.internal), None if buf is None else _lib.dptr(buf),
            float(t), C.byref(seq)))
        return seq.value

    def ready(self, seq: int) -> bool:
        r = C.c_int()
        self.ctx.check(self.ctx.lib.lm_ring_ready(self.handle, int(seq), C.byref(r)))
        return bool(r.value)

    def wait(self, seq: int):
        """(t, values) of entry ``seq`` (a fresh array)."""
        n = C.c_int64()
        t = C.c_double()
        view = C.POINTER(C.c_double)()
        self.ctx.check(self.ctx.lib.lm_ring_wait(self.handle, int(seq), None, C.byref(view), C.byref(n),
                                                 C.byref(t)))
        out = np.ctypeslib.as_array(view, shape=(n.value,)).copy() if n.value else np.empty(0)
        return t.value, out

    @property
    def head(self) -> int:
        h = C.c_int64()
        self.ctx.check(self.ctx.lib.lm_ring_head(self.handle, C.byref(h)))
        return h.value


_rings: dict = {}


def _ring_for(ctx, length: int, nslots: int, index: int = 0) -> ReadoutRing:
    """A ring reused across TimeSequence calls (its pinned slots are allocated once)."""
    key = (id(ctx), int(length), int(nslots), int(index))
    r = _rings.get(key)
    if r is None:
        if len(_rings) >= 8:
            _rings.pop(next(iter(_rings)))
        r = _rings[key] = ReadoutRing(length, nslots, ctx)
    return r


def moment_density(moment):
    """f(moment) = localdensity(moment.state) (src/operators/latticeutils.jl:41-45)."""
    from .observables import localdensity
    return localdensity(moment.state)


def moment_currents(moment):
    """f(moment) = bond values of DensityCurrents(moment.H, moment.state) (src/zoo/currents.jl:92-102);
    for a SparseHamiltonian the value of every stored entry (SiteCurrents.entry_values)."""
    from .observables import DensityCurrents
    return DensityCurrents(moment.H, moment.state).bond_values()


moment_density._lm_readout = "density"
moment_currents._lm_readout = "currents"


def _collect_rings(pairs, it, nslots):
    """Feeds every moment of ``it`` to the ring readouts of ``pairs`` [(f, TimeSequence)]: each
    readout is pushed into its own ring, and an entry is collected only when its slot is about
    to be reused (or at the end), so the loop never waits for a step."""
    from .observables import _site_sum
    from .sparse import SparseHamiltonian
    slots = [None] * len(pairs)  # per readout: (ring, pending sequence numbers, wrap)
    for moment in it:
        st = moment.state
        general = isinstance(moment.H, SparseHamiltonian)
        for i, (f, ts) in enumerate(pairs):
            kind = f._lm_readout
            if slots[i] is None:
                if kind == "density":
                    length = st.n
                elif general:
                    length = max(len(moment.H.rowval), 1)
                else:
                    length = max(st.lattice.nbonds(), 1)
                wrap = ((lambda v, lat=st.lattice: LatticeValue(lat, _site_sum(lat, v))) if kind == "density"
                        else (lambda v: v))
                # two readouts of the same kind and length would share a ring: give each its own
                same = sum(1 for j in range(i) if slots[j] is not None and slots[j][0].length == length)
                slots[i] = (_ring_for(st.ctx, length, nslots, same), [], wrap)
            ring, pending, wrap = slots[i]
            if len(pending) == ring.nslots:  # the oldest slot is about to be reused
                _take(ts, ring, pending.pop(0), wrap)
            if kind == "density":
                pending.append(ring.push_density(st, moment.t))
            elif general:
                pending.append(ring.push_op_currents(moment.H, st, moment.t))
            else:
                pending.append(ring.push_currents(moment.H, st, moment.t))
    for (f, ts), sl in zip(pairs, slots):
        if sl is None:
            continue
        ring, pending, wrap = sl
        for seq in pending:
            _take(ts, ring, seq, wrap)


def _take(ts, ring, seq, wrap):
    t, v = ring.wait(seq)
    ts.times.append(t)
    ts.values.append(wrap(v))


def timesequences(fs, it, nslots: int = 8):
    """One ``TimeSequence`` per readout in ``fs``, all filled from a single pass over the
    evolution iterator ``it``: the loop of the reference's README example, which computes
    ``localdensity(P)`` and ``DensityCurrents(H, P)`` at every moment of ``ev(times)``.

    ``moment_density`` and ``moment_currents`` go through device readout rings (asynchronous
    downloads); any other callable is applied to each moment as it is yielded."""
    out = [TimeSequence() for _ in fs]
    ring_pairs = [(f, ts) for f, ts in zip(fs, out) if getattr(f, "_lm_readout", None) is not None]
    plain = [(f, ts) for f, ts in zip(fs, out) if getattr(f, "_lm_readout", None) is None]
    if plain:
        def tee(src):
            for moment in src:
                for f, ts in plain:
                    ts.times.append(float(moment.t))
                    ts.values.append(f(moment))
                yield moment
        it = tee(it)
    if ring_pairs:
        _collect_rings(ring_pairs, it, nslots)
    else:
        for _ in it:
            pass
    return out


class TimeSequence:
    """A time-ordered sequence of values (src/timesequence.jl:1-13).

    ``TimeSequence()``, ``TimeSequence(times, values)``, ``TimeSequence(f, ev_iter)`` or
    ``TimeSequence(f, ev, times)``; ``nslots`` sizes the readout ring of the device path.
    """

    def __init__(self, *args, nslots: int = 8):
        self.times: list = []
        self.values: list = []
        if not args:
            return
        if callable(args[0]):
            f = args[0]
            it = args[1](args[2]) if len(args) == 3 else args[1]
            self._collect(f, it, nslots)
            return
        ts, vs = args
        ts, vs = list(ts), list(vs)
        if len(ts) != len(vs):
            raise ValueError(f"Keys/values length mismatch:\n{len(ts)} timestamps, {len(vs)} snapshots")
        self.times = [float(t) for t in ts]
        self.values = vs

    def _collect(self, f, it, nslots):
        if getattr(f, "_lm_readout", None) is None:
            for moment in it:
                self.times.append(float(moment.t))
                self.values.append(f(moment))
            return
        _collect_rings([(f, self)], it, nslots)

    # --- AbstractDict{Float64, ET} surface of the reference --------------------------------
    def timestamps(self):
        return self.times

    def __len__(self):
        return len(self.times)

    def __iter__(self):
        return iter(zip(self.times, self.values))

    def _find(self, t):
        for i, ti in enumerate(self.times):
            if abs(ti - t) <= _ATOL:
                return i
        return None

    def get(self, t, default=None):
        i = self._find(t)
        return default if i is None else self.values[i]

    def __getitem__(self, t):
        i = self._find(t)
        if i is None:
            raise KeyError(t)
        return self.values[i]

    def __setitem__(self, t, val):
        i = self._find(t)
        if i is None:
            import bisect
            i = bisect.bisect_left(self.times, t)
            self.times.insert(i, float(t))
            self.values.insert(i, val)
        else:
            self.values[i] = val

    def delete(self, t):
        i = self._find(t)
        if i is not None:
            del self.times[i]
            del self.values[i]
        return self

    def __eq__(self, other):
        if not isinstance(other, TimeSequence) or self.times != other.times or len(self) != len(other):
            return False
        return all(np.array_equal(_arr(a), _arr(b)) for a, b in zip(self.values, other.values))

    __hash__ = None

    def copy(self):
        return TimeSequence(list(self.times), [_copy(v) for v in self.values])

    def map(self, f):
        return TimeSequence(list(self.times), [f(v) for v in self.values])

    def __repr__(self):
        return f"TimeSequence with {len(self)} entries"


def _arr(v):
    return v.values if isinstance(v, LatticeValue) else np.asarray(v)


def _copy(v):
    if isinstance(v, LatticeValue):
        return LatticeValue(v.lattice, np.array(v.values))
    return np.array(v) if isinstance(v, np.ndarray) else v


def _axpby(a, x, b, y):
    if isinstance(x, LatticeValue):
        return LatticeValue(x.lattice, a * x.values + b * y.values)
    return a * np.asarray(x) + b * np.asarray(y)


def differentiate(tseq: TimeSequence) -> TimeSequence:
    """Symmetric-difference derivative at the midpoints (src/timesequence.jl:193-211)."""
    if len(tseq) < 2:
        raise ValueError(f"Cannot differentiate TimeSequence of length {len(tseq)}")
    ts, vs = tseq.times, tseq.values
    out_t, out_v = [], []
    for i in range(1, len(ts)):
        dt = ts[i] - ts[i - 1]
        out_v.append(_axpby(1 / dt, vs[i], -1 / dt, vs[i - 1]))
        out_t.append(ts[i - 1] + dt / 2)
    return TimeSequence(out_t, out_v)


def integrate(tseq: TimeSequence) -> TimeSequence:
    """Cumulative trapezoidal integral, zero at the first time (src/timesequence.jl:252-271)."""
    if len(tseq) < 2:
        raise ValueError(f"Cannot integrate TimeSequence of length {len(tseq)}")
    ts, vs = tseq.times, tseq.values
    acc = _axpby(0.0, vs[0], 0.0, vs[0])
    out = [acc]
    for i in range(1, len(ts)):
        dt = ts[i] - ts[i - 1]
        acc = _axpby(1.0, acc, 1.0, _axpby(dt / 2, vs[i], dt / 2, vs[i - 1]))
        out.append(acc)
    return TimeSequence(list(ts), out)
