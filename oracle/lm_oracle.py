"""CPU oracle for the LatticeModels.jl time-evolution path.

TEST INFRASTRUCTURE ONLY.  This module restates, in numpy/scipy, the semantics of
LatticeModels.jl v1.0.7 for the path

    Evolution(t -> tightbinding_hamiltonian(l; field=...), P_0)  ->  localdensity, DensityCurrents

It is the checker for the GPU library: only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it.  The product path (the ``lmgpu`` package and
``liblmgpu.so``) never calls into it.

Every function cites the reference file:line it restates (paths relative to the
LatticeModels.jl repository root).

Pinning: the reference is Julia and cannot run here, so this oracle is pinned against the
known-answer values held by the reference's own tests and doctests (site order, nnz counts,
the 4x4 spectrum, line-integral identities, flux replication counts, current identities,
evolution against the exact exponent).  See ``tests/test_oracle_golden.py``.
"""
from __future__ import annotations

import bisect
import math
from dataclasses import dataclass, field as dc_field
from typing import List, Optional, Sequence, Tuple

import numpy as np
import scipy.sparse as sp

TWO_PI = 2.0 * math.pi
CURRENTS_EPS = 1e-10  # src/currents.jl:4
FLUX_EPS = 1e-11      # src/zoo/magneticfields.jl:76, :94


# ----------------------------------------------------------------------------------------
# a1: SquareLattice site order            src/lattices/bravais/lattice.jl:101-111, :161-172
#                                         src/lattices/bravais/unitcell.jl:113-132
# ----------------------------------------------------------------------------------------
def _cartesian_indices(depth: int, ndim: int):
    """CartesianIndex(-d,..,-d):CartesianIndex(d,..,d), first index fastest (src/core/utils.jl:24-26)."""
    rng = range(-depth, depth + 1)
    res = []

    def rec(idx, k):  # the last index varies slowest
        if k < 0:
            res.append(tuple(idx))
            return
        for v in rng:
            idx[k] = v
            rec(idx, k - 1)

    rec([0] * ndim, ndim - 1)
    return res


@dataclass
class SquareLattice:
    """SquareLattice(Lx, Ly; boundaries) restated (src/zoo/lattices.jl:131).

    Sites are Bravais pointers (x, y), 1-based, sorted lexicographically
    (src/lattices/bravais/unitcell.jl:126-132); coordinates equal the lattice coordinates
    because the square unit cell is the identity with its basis site at the origin.
    ``periodic``/``twist`` describe ``boundaries=(:axis1 => Θx, :axis2 => Θy)``
    (src/core/boundaries.jl:46-76): a periodic axis has twist 0.
    """
    Lx: int
    Ly: int
    periodic: Tuple[bool, bool] = (False, False)
    twist: Tuple[float, float] = (0.0, 0.0)

    def __post_init__(self):
        if self.Lx < 1 or self.Ly < 1:
            raise ValueError("lattice sizes must be positive")
        # add_bravaispointers! iterates CartesianIndices(reverse(axes)) -> y fastest,
        # then BravaisLattice requires the pointers sorted (x major).
        ptrs = [(x, y) for x in range(1, self.Lx + 1) for y in range(1, self.Ly + 1)]
        ptrs.sort()
        self.pointers = ptrs
        self.coords = np.array(ptrs, dtype=np.float64)
        self.translations = [(self.Lx, 0), (0, self.Ly)]  # default :axisK -> Bravais[L*e_K]

    @property
    def N(self) -> int:
        return len(self.pointers)

    def site_index(self, x: int, y: int) -> Optional[int]:
        """Binary search over the sorted pointers (src/lattices/bravais/lattice.jl:69-74); 1-based."""
        i = bisect.bisect_left(self.pointers, (x, y))
        if i < len(self.pointers) and self.pointers[i] == (x, y):
            return i + 1
        return None

    def has_boundaries(self) -> bool:
        return any(self.periodic)

    def boundaries(self):
        """Active boundaries as (translation, twist) in axis order (src/core/boundaries.jl:138-153)."""
        out = []
        for ax in range(2):
            if self.periodic[ax]:
                out.append((self.translations[ax], float(self.twist[ax])))
        return out

    def resolve_site(self, x: int, y: int):
        """route + findfactor + resolve_site (src/core/boundaries.jl:251-289).

        Returns (index, factor) or None.  ``factor`` is the twist phase of the boundary crossing.
        """
        idx = self.site_index(x, y)
        if idx is not None:
            return idx, 1.0 + 0.0j
        bcs = self.boundaries()
        if not bcs:
            return None
        for tup in _cartesian_indices(1, len(bcs)):  # depth = 1
            nx, ny = x, y
            for (tr, _), n in zip(bcs, tup):
                # nshifts: n > 0 -> site -= tr (n times); n < 0 -> site += tr
                nx -= n * tr[0]
                ny -= n * tr[1]
            idx = self.site_index(nx, ny)
            if idx is not None:
                if all(n == 0 for n in tup):
                    return idx, 1.0 + 0.0j
                theta = sum(th * n for (_, th), n in zip(bcs, tup))
                return idx, complex(math.cos(theta), math.sin(theta)) if theta != 0.0 else 1.0 + 0.0j
        return None


# ----------------------------------------------------------------------------------------
# a2/a3: nearest-neighbour bonds          src/lattices/bravais/nearestneighbor.jl:97-131
#                                         src/core/bonds.jl:415-422
# ----------------------------------------------------------------------------------------
NN_TRANSLATIONS = [(1, 0), (0, 1)]  # detect_nnhops order for the square unit cell


@dataclass
class Bond:
    src: int            # 1-based index of the source site
    dst: int            # 1-based index of the destination site
    r1: Tuple[float, float]   # source coordinates
    r2: Tuple[float, float]   # unwrapped destination coordinates (ResolvedSite.old_site)
    factor: complex     # boundary twist factor of the destination


def nn_bonds(lat: SquareLattice) -> List[Bond]:
    """Bonds of NearestNeighbor(1) in the reference's iteration order.

    BravaisSiteMapping iterates its translations in order (constructoperator.jl:31-38), each
    translation iterates the sites in index order and drops unresolved destinations
    (src/core/bonds.jl:415-422).
    """
    bonds = []
    for (dx, dy) in NN_TRANSLATIONS:
        for i, (x, y) in enumerate(lat.pointers, start=1):
            r = lat.resolve_site(x + dx, y + dy)
            if r is None:
                continue
            j, fac = r
            bonds.append(Bond(i, j, (float(x), float(y)), (float(x + dx), float(y + dy)), fac))
    return bonds


# ----------------------------------------------------------------------------------------
# a4-a6: gauge fields                     src/zoo/magneticfields.jl
# ----------------------------------------------------------------------------------------
@dataclass
class LandauGauge:
    B: float

    def line_integral(self, p1, p2):  # src/zoo/magneticfields.jl:15
        return (p1[0] + p2[0]) * (p2[1] - p1[1]) * self.B / 2

    def vector_potential(self, p):   # :14
        return (0.0, p[0] * self.B)


@dataclass
class SymmetricGauge:
    B: float

    def line_integral(self, p1, p2):  # :31
        return (p1[0] * p2[1] - p2[0] * p1[1]) / 2 * self.B

    def vector_potential(self, p):   # :30
        return (-p[1] * self.B / 2, p[0] * self.B / 2)


@dataclass
class PointFlux:
    flux: float
    point: Tuple[float, float] = (0.0, 0.0)
    gauge: str = "axial"

    def line_integral(self, p1, p2):
        px, py = self.point
        x1, y1 = p1[0] - px, p1[1] - py
        x2, y2 = p2[0] - px, p2[1] - py
        if self.gauge == "axial":  # :72-85
            # norm(p) of a 2-vector: sqrt(x^2 + y^2) with separate products (no hypot scaling)
            n1 = math.sqrt(x1 * x1 + y1 * y1)
            n2 = math.sqrt(x2 * x2 + y2 * y2)
            if n1 < FLUX_EPS or n2 < FLUX_EPS:
                return 0.0 * self.flux
            nnorm = n1 * n2
            det = x1 * y2 - x2 * y1
            cosang = (x1 * x2 + y1 * y2) / nnorm / (1 + 1e-11)
            sgn = (det > 0) - (det < 0)
            angle = math.acos(cosang) * sgn
            return angle * self.flux / TWO_PI
        # singular gauge :89-104
        sg = x2 - x1
        if abs(sg) < FLUX_EPS:
            return 0.0 * self.flux
        if x1 * x2 > 0 or max(x1, x2) == 0:
            return 0.0 * self.flux
        yint = (-y1 * x2 + y2 * x1) / (x1 - x2)
        return 0.0 * self.flux if yint > 0 else self.flux * ((sg > 0) - (sg < 0))

    def vector_potential(self, p):  # :66-70 (axial only)
        x, y = p[0] - 0.0, p[1] - 0.0
        nsq = x * x + y * y
        return (-y / nsq / TWO_PI * self.flux, x / nsq / TWO_PI * self.flux)


@dataclass
class PointFluxes:
    fluxes: List[float]
    points: List[Tuple[float, float]]
    gauge: str = "axial"

    def line_integral(self, p1, p2):  # :183-184 (sum in order)
        s = 0.0
        first = True
        for f, p in zip(self.fluxes, self.points):
            v = PointFlux(f, p, self.gauge).line_integral(p1, p2)
            s = v if first else s + v
            first = False
        return s


@dataclass
class FieldSum:
    fields: Tuple

    def line_integral(self, p1, p2):  # src/operators/magneticfield.jl:104
        s = None
        for f in self.fields:
            v = f.line_integral(p1, p2)
            s = v if s is None else s + v
        return 0.0 if s is None else s


def line_integral_trapezoid(field, p1, p2, n_steps):
    """Midpoint rule over n_steps (src/operators/magneticfield.jl:26-35)."""
    dp = ((p2[0] - p1[0]) / n_steps, (p2[1] - p1[1]) / n_steps)
    p = (p1[0] + 0.5 * dp[0], p1[1] + 0.5 * dp[1])
    acc = 0.0
    for _ in range(n_steps):
        a = field.vector_potential(p)
        acc += dp[0] * a[0] + dp[1] * a[1]
        p = (p[0] + dp[0], p[1] + dp[1])
    return acc


def adapt_field(fld, lat: SquareLattice):
    """PBC adaptation (src/zoo/magneticfields.jl:237-266, src/operators/magneticfield.jl:4).

    PointFlux/PointFluxes on a lattice with boundaries become singular-gauge PointFluxes
    replicated over the 3^d images -sum(n_i * T_i); other fields are unchanged.
    """
    if isinstance(fld, FieldSum):
        return FieldSum(tuple(adapt_field(f, lat) for f in fld.fields))
    if isinstance(fld, PointFlux):
        if not lat.has_boundaries():
            return fld
        fld = PointFluxes([fld.flux], [fld.point], fld.gauge)
    if isinstance(fld, PointFluxes):
        if not lat.has_boundaries():
            return fld
        bcs = lat.boundaries()
        fl, pts = [], []
        for tup in _cartesian_indices(1, len(bcs)):
            rx = -sum(n * tr[0] for (tr, _), n in zip(bcs, tup))
            ry = -sum(n * tr[1] for (tr, _), n in zip(bcs, tup))
            fl.extend(fld.fluxes)
            pts.extend([(p[0] + rx, p[1] + ry) for p in fld.points])
        return PointFluxes(fl, pts, "singular")
    return fld


def periodic_fluxes(lat: SquareLattice, pf: PointFlux) -> PointFluxes:
    """Replicate a point flux over every unit cell (src/zoo/magneticfields.jl:226-235)."""
    lv0 = (round(pf.point[0]), round(pf.point[1]))
    p0 = (pf.point[0] - lv0[0], pf.point[1] - lv0[1])
    pts = sorted({(p0[0] + x, p0[1] + y) for (x, y) in lat.pointers})
    return PointFluxes([pf.flux] * len(pts), pts, pf.gauge)


# ----------------------------------------------------------------------------------------
# a7: tightbinding_hamiltonian            src/operators/constructoperator.jl:4-47, :136-194
#                                         src/operators/builder.jl:116-141, :274-309
# ----------------------------------------------------------------------------------------
def bond_values(lat: SquareLattice, t1: float = 1.0, field=None, bonds=None):
    """Per-bond H[i,j] = t1 * factor * exp(-2 pi i LI(r_i, r_j_unwrapped)) (builder.jl:282-285)."""
    if bonds is None:
        bonds = nn_bonds(lat)
    fld = adapt_field(field, lat) if field is not None else None
    vals = np.empty(len(bonds), dtype=np.complex128)
    for b, bd in enumerate(bonds):
        li = 0.0 if fld is None else fld.line_integral(bd.r1, bd.r2)
        theta = -TWO_PI * li
        ph = complex(math.cos(theta), math.sin(theta))
        vals[b] = t1 * (bd.factor * ph)
    return bonds, vals


def tightbinding_hamiltonian(lat: SquareLattice, t1: float = 1.0, field=None, onsite=None,
                             return_bonds: bool = False):
    """CSC Hamiltonian with the builder's accumulate-and-conjugate semantics.

    Terms are added in argument order: the on-site LatticeValue first (it precedes the
    ``t1 => NearestNeighbor(1)`` pair, constructoperator.jl:190-194), then every bond
    (i -> j): H[i,j] += t1*f, H[j,i] += conj(t1*f) (builder.jl:296-309).  Zero ``t1`` is
    skipped (constructoperator.jl:49-51).
    """
    N = lat.N
    acc = {}
    if onsite is not None:
        V = np.asarray(onsite, dtype=np.float64)
        for i in range(N):
            acc[(i, i)] = acc.get((i, i), 0j) + complex(V[i])
    bonds, vals = bond_values(lat, t1, field)
    if t1 != 0:
        for bd, v in zip(bonds, vals):
            i, j = bd.src - 1, bd.dst - 1
            acc[(i, j)] = acc.get((i, j), 0j) + v
            if i != j:
                acc[(j, i)] = acc.get((j, i), 0j) + v.conjugate()
    rows = np.fromiter((k[0] for k in acc), dtype=np.int64, count=len(acc))
    cols = np.fromiter((k[1] for k in acc), dtype=np.int64, count=len(acc))
    data = np.fromiter(acc.values(), dtype=np.complex128, count=len(acc))
    H = sp.csc_matrix((data, (rows, cols)), shape=(N, N))
    H.sort_indices()
    if return_bonds:
        return H, bonds, vals
    return H


def tightbinding_hamiltonian_fast(lat: SquareLattice, t1=1.0, field=None, onsite=None):
    """Vectorised equivalent of tightbinding_hamiltonian for large lattices (Landau/none only).

    Same values as the scalar restatement: LI = (x1+x2)*(y2-y1)*B/2 per bond; used by the
    tests at GPU scale where the scalar loop is too slow.
    """
    Lx, Ly, N = lat.Lx, lat.Ly, lat.N
    x = np.repeat(np.arange(1, Lx + 1), Ly).astype(np.float64)
    y = np.tile(np.arange(1, Ly + 1), Lx).astype(np.float64)
    idx = np.arange(N, dtype=np.int64)
    srcs, dsts, vals = [], [], []
    for ax, (dx, dy) in enumerate(NN_TRANSLATIONS):
        x2 = x + dx
        y2 = y + dy
        xi = x2.astype(np.int64)
        yi = y2.astype(np.int64)
        L = (Lx, Ly)[ax]
        coord = xi if ax == 0 else yi
        inside = coord <= L
        fac = np.ones(N, dtype=np.complex128)
        if lat.periodic[ax]:
            wrapped = ~inside
            coord_w = np.where(wrapped, coord - L, coord)
            th = lat.twist[ax]
            if th != 0.0:
                fac[wrapped] = complex(math.cos(th), math.sin(th))
            keep = np.ones(N, dtype=bool)
        else:
            coord_w = coord
            keep = inside
        if ax == 0:
            dst = (coord_w - 1) * Ly + (yi - 1)
        else:
            dst = (xi - 1) * Ly + (coord_w - 1)
        if field is None:
            li = np.zeros(N)
        elif isinstance(field, LandauGauge):
            li = (x + x2) * (y2 - y) * field.B / 2
        else:
            raise NotImplementedError("fast path supports LandauGauge only")
        theta = -TWO_PI * li
        ph = np.cos(theta) + 1j * np.sin(theta)
        v = t1 * (fac * ph)
        srcs.append(idx[keep]); dsts.append(dst[keep]); vals.append(v[keep])
    src = np.concatenate(srcs); dst = np.concatenate(dsts); val = np.concatenate(vals)
    rows = np.concatenate([src, dst]); cols = np.concatenate([dst, src])
    data = np.concatenate([val, np.conj(val)])
    if onsite is not None:
        rows = np.concatenate([idx, rows]); cols = np.concatenate([idx, cols])
        data = np.concatenate([np.asarray(onsite, dtype=np.complex128), data])
    H = sp.csc_matrix((data, (rows, cols)), shape=(N, N))  # duplicates summed
    H.sort_indices()
    return H, src + 1, dst + 1, val


# ----------------------------------------------------------------------------------------
# a12: densitymatrix(H; mu) at T = 0      src/spectrum.jl:48-55, :226-232, :253-257, :317-333
# ----------------------------------------------------------------------------------------
def diagonalize(H):
    """Dense Hermitian eigen (LAPACK, as eigen() on a Hermitian matrix), ascending values."""
    Hd = H.toarray() if sp.issparse(H) else np.asarray(H)
    vals, vecs = np.linalg.eigh(Hd)
    order = np.argsort(vals, kind="stable")
    return vals[order], vecs[:, order]


def densfun(T: float, mu: float, statistics: str = "FermiDirac", degenerate_tol: float = 0.0):
    """src/spectrum.jl:230-232: E -> (E - mu == T == 0) ? 1 : 1 / (exp((E - mu)/T) + s) with
    s = Int(statistics): +1 FermiDirac, -1 BoseEinstein.

    degenerate_tol > 0 reads "E == mu" as |E - mu| <= degenerate_tol.  With the exact test (0,
    the reference's rule) a level that is exactly degenerate at mu is split by the eigensolver's
    rounding: each of its computed eigenvalues lands a few ulps above or below mu, and only
    those below are occupied.  The tolerance occupies the whole level."""
    sgn = 1.0 if statistics == "FermiDirac" else -1.0

    def f(E):
        if T == 0 and abs(E - mu) <= degenerate_tol:
            return 1.0
        with np.errstate(over="ignore", divide="ignore"):
            z = (E - mu) / T if T != 0 else (math.inf if E > mu else -math.inf)
        return 1.0 / (math.exp(z) + sgn) if z < 700 else 0.0
    return f


def ddensfun(T: float, mu: float, statistics: str = "FermiDirac"):
    """src/spectrum.jl:233-235: d f / d mu ... as the reference writes it: -e^z / T / (e^z + s)^2."""
    sgn = 1.0 if statistics == "FermiDirac" else -1.0

    def f(E):
        z = (E - mu) / T
        if z > 700:
            return 0.0
        ez = math.exp(z)
        return -ez / T / (ez + sgn) ** 2
    return f


def densitymatrix_dispatch(H, mu=None, T: float = 0.0, N=None, statistics=None, degenerate_tol: float = 0.0):
    """``densitymatrix(ham; kw...)`` of a one-particle system (src/spectrum.jl:226-333):
    * N given: fixn_densitymatrix -- at T = 0 the Fermi sphere (the lowest N states;
      BoseEinstein: N times the ground state), else mu by the reference's Newton iteration on
      the eigenvalues (start 0, step (N_ev - N) / dN_ev, atol sqrt(eps), 1000 iterations);
    * mu or statistics given: ensemble_densitymatrix with densfun(T, mu, statistics);
    * neither: gibbs_densitymatrix -- the ground state at T = 0 (|T| < 1e-10), else
      exp(-E/T)/Z (evaluated here as exp(-(E - E_min)/T)/Z', the same matrix)."""
    vals, vecs = diagonalize(H)
    stat = statistics or "FermiDirac"
    if N is not None:
        if mu is not None:
            raise ValueError("cannot specify both N and mu")
        if abs(T) < 1e-10:
            if stat == "BoseEinstein":
                return np.outer(vecs[:, 0], vecs[:, 0].conj()) * N
            if len(vals) < N:
                raise ValueError(f"cannot build Fermi sphere with {N} particles: only {len(vals)} bands present")
            V = vecs[:, :N]
            return V @ V.conj().T
        newmu = 0.0
        for _ in range(1000):
            f, df = densfun(T, newmu, stat), ddensfun(T, newmu, stat)
            n_ev = sum(f(e) for e in vals)
            dn_ev = sum(df(e) for e in vals)
            dmu = (n_ev - N) / dn_ev
            if abs(dmu) < math.sqrt(np.finfo(float).eps):
                w = np.array([densfun(T, newmu, stat)(e) for e in vals])
                return (vecs * w) @ vecs.conj().T
            newmu += dmu
        raise ValueError("did not converge")
    if mu is not None or statistics is not None:
        f = densfun(T, 0.0 if mu is None else mu, stat, degenerate_tol)
        w = np.array([f(e) for e in vals])
        return (vecs * w) @ vecs.conj().T
    if abs(T) < 1e-10:
        return np.outer(vecs[:, 0], vecs[:, 0].conj())
    w = np.exp(-(vals - vals[0]) / T)
    w /= w.sum()
    return (vecs * w) @ vecs.conj().T


def densitymatrix(H, mu: float = 0.0, T: float = 0.0, degenerate_tol: float = 0.0):
    """projector(densfun(T, mu), eig) = V * (f(E) .* V') (src/spectrum.jl:226-228)."""
    vals, vecs = diagonalize(H)
    f = densfun(T, mu, degenerate_tol=degenerate_tol)
    w = np.array([f(e) for e in vals])
    return (vecs * w) @ vecs.conj().T, vals, vecs


# ----------------------------------------------------------------------------------------
# a9/a10: CachedExp                         src/evolution.jl:62-128
# ----------------------------------------------------------------------------------------
def _nextpow2(x: float) -> float:
    """Julia nextpow(2, x): smallest 2^n >= x with n >= 0."""
    p = 1.0
    while p < x:
        p *= 2.0
    return p


def cachedexp(A, dt: float, threshold: float = 1e-10, nztol: float = 1e-14):
    """myexp!(P, A, -i*dt) restated: scaling + Taylor until max|term| <= threshold/sf."""
    factor = -1j * dt
    A = sp.csc_matrix(A) if sp.issparse(A) else np.asarray(A)
    sparse = sp.issparse(A)
    N = A.shape[0]
    P = sp.identity(N, dtype=np.complex128, format="csc") if sparse else np.eye(N, dtype=np.complex128)
    mat_norm = (abs(A).max() if A.nnz else 0.0) if sparse else np.abs(A).max()
    if mat_norm == 0 or factor == 0:
        return P
    sf = _nextpow2(mat_norm * abs(factor))
    A = A / sf
    delta = 1.0
    term = P.copy()
    n = 1
    while delta > threshold / sf:
        if sparse:
            term = (A @ term) * (factor / n)
            term = term.tocsc()
            term.data[np.abs(term.data) <= nztol] = 0
            term.eliminate_zeros()
            delta = abs(term).max() if term.nnz else 0.0
        else:
            term = (A @ term) * (factor / n)
            delta = np.abs(term).max()
        P = P + term
        n += 1
    for _ in range(int(round(math.log2(sf)))):
        P = P @ P
    return P


def expm_exact(H, dt: float):
    """Dense exp(-i H dt) via the Hermitian eigendecomposition (FP64)."""
    Hd = H.toarray() if sp.issparse(H) else np.asarray(H)
    w, V = np.linalg.eigh(Hd)
    return (V * np.exp(-1j * dt * w)) @ V.conj().T


def expm_multiply(H, dt: float, X):
    """exp(-i H dt) X for sparse H, via scipy (reference-grade FP64 at GPU-test sizes)."""
    from scipy.sparse.linalg import expm_multiply as _em
    return _em((-1j * dt) * sp.csr_matrix(H), X)


# ----------------------------------------------------------------------------------------
# a8: Evolution / EvolutionIterator        src/evolution.jl:183-298
# ----------------------------------------------------------------------------------------
class OracleCachedExpSolver:
    """CachedExp with update_solver!/step! semantics (src/evolution.jl:62-92)."""

    def __init__(self, threshold=1e-10, nztol=1e-14, exact=False):
        self.threshold = threshold
        self.nztol = nztol
        self.exact = exact
        self.mat = None
        self.factor = 0j
        self.U = None

    def update_solver(self, H, dt, force=False):
        factor = -1j * dt
        if not force and self.U is not None and np.isclose(factor, self.factor, rtol=math.sqrt(np.finfo(float).eps), atol=0) \
                and self.mat is not None and (self.mat is H or _sparse_equal(self.mat, H)):
            return
        self.mat = H
        self.U = expm_exact(H, dt) if self.exact else cachedexp(H, dt, self.threshold, self.nztol)
        self.factor = factor

    def step(self, state):
        U = self.U
        if state.ndim == 1:
            return np.asarray(U @ state).ravel()
        c2 = U @ state
        return np.asarray(c2 @ (U.conj().T if not sp.issparse(U) else U.conj().T.toarray()))


def _sparse_equal(A, B):
    if sp.issparse(A) and sp.issparse(B):
        return A.shape == B.shape and (A != B).nnz == 0
    return np.array_equal(np.asarray(A.todense() if sp.issparse(A) else A),
                          np.asarray(B.todense() if sp.issparse(B) else B))


def evolve(h, state0, times, solver):
    """Yields (H_{k-1}, state_k, t_k) exactly like EvolutionIterator (src/evolution.jl:238-275).

    The first moment has dt = times[0] - 0 (zero for a grid starting at 0) and returns the
    initial state with H(0); afterwards H is evaluated at the left end of each interval.
    """
    state = np.array(state0, copy=True)
    t = 0.0
    for i, ti in enumerate(times):
        dt = ti - times[i - 1] if i > 0 else ti - t
        if dt < -1e-15:
            raise ValueError("negative time step")
        H = h(t)
        if abs(dt) >= 1e-15:
            solver.update_solver(H, dt, False)
            state = solver.step(state)
            t += dt
        yield H, state, t


# ----------------------------------------------------------------------------------------
# a13-a15: observables                     src/operators/latticeutils.jl:41-45,
#                                          src/zoo/currents.jl:81-102, src/currents.jl:223-255
# ----------------------------------------------------------------------------------------
def localdensity(state, weights=None):
    """Re P[i,i] for a density matrix, |psi_i|^2 for a ket, sum_m w_m |psi_im|^2 for a block."""
    s = np.asarray(state)
    if s.ndim == 1:
        return np.abs(s) ** 2
    if weights is not None:
        return (np.abs(s) ** 2) @ np.asarray(weights, dtype=np.float64)
    if s.shape[0] == s.shape[1]:
        return np.real(np.diag(s)).copy()
    return (np.abs(s) ** 2).sum(axis=1)


def density_current(H, state, i, j, weights=None, is_density=None):
    """DensityCurrents(H, P)[i,j] = 2 Im(H[i,j] * P[j,i]) with 0-based i, j."""
    hij = H[i, j]
    s = np.asarray(state)
    if s.ndim == 1:
        pji = s[j] * np.conj(s[i])
    elif is_density or (is_density is None and weights is None and s.shape[0] == s.shape[1]):
        pji = s[j, i]
    else:
        w = np.ones(s.shape[1]) if weights is None else np.asarray(weights)
        pji = np.sum(w * s[j, :] * np.conj(s[i, :]))
    return 2.0 * np.imag(hij * pji)


def bond_currents(H, state, bonds_src, bonds_dst, weights=None, is_density=None):
    """Currents on the bond list (1-based src/dst), vectorised; J_b = 2 Im(H[i,j] P[j,i])."""
    H = sp.csr_matrix(H)
    i = np.asarray(bonds_src) - 1
    j = np.asarray(bonds_dst) - 1
    hij = np.asarray(H[i, j]).ravel()
    s = np.asarray(state)
    if s.ndim == 1:
        pji = s[j] * np.conj(s[i])
    elif is_density or (is_density is None and weights is None and s.shape[0] == s.shape[1]):
        pji = s[j, i]
    else:
        w = np.ones(s.shape[1]) if weights is None else np.asarray(weights)
        pji = np.einsum("bm,bm,m->b", s[j, :], np.conj(s[i, :]), w)
    return 2.0 * np.imag(hij * pji)


def currents_matrix(H, state, bonds_src=None, bonds_dst=None, **kw):
    """Currents(dc[, bonds]): antisymmetric sparse matrix, |J| < 1e-10 dropped (src/currents.jl:223-255)."""
    N = H.shape[0]
    if bonds_src is None:
        I, J = np.tril_indices(N, -1)
        vals = np.array([density_current(H, state, a, b, **kw) for a, b in zip(I, J)])
        src, dst = I + 1, J + 1
    else:
        src, dst = np.asarray(bonds_src), np.asarray(bonds_dst)
        vals = bond_currents(H, state, src, dst, **kw)
    keep = np.abs(vals) >= CURRENTS_EPS
    r = np.concatenate([src[keep] - 1, dst[keep] - 1])
    c = np.concatenate([dst[keep] - 1, src[keep] - 1])
    v = np.concatenate([vals[keep], -vals[keep]])
    return sp.csc_matrix((v, (r, c)), shape=(N, N))


# ----------------------------------------------------------------------------------------
# Chebyshev restatement used only to cross-check the library's coefficient logic.
# ----------------------------------------------------------------------------------------
def bessel_j_seq(x: float, kmax: int) -> np.ndarray:
    """J_0..J_kmax(x) via scipy (checker only)."""
    from scipy.special import jv
    return jv(np.arange(kmax + 1), x)


def chebyshev_expv(H, dt, X, emin, emax, K):
    """exp(-i H dt) X with K Chebyshev orders on [emin, emax] (FP64 reference for the library)."""
    a = (emax - emin) / 2
    b = (emax + emin) / 2
    J = bessel_j_seq(a * dt, K)
    Hs = (sp.csr_matrix(H) - b * sp.identity(H.shape[0], format="csr")) / a
    T0 = np.asarray(X, dtype=np.complex128)
    y = J[0] * T0
    if K >= 1:
        T1 = Hs @ T0
        y = y + 2 * (-1j) * J[1] * T1
        for k in range(2, K + 1):
            T2 = 2 * (Hs @ T1) - T0
            y = y + 2 * ((-1j) ** k) * J[k] * T2
            T0, T1 = T1, T2
    return np.exp(-1j * b * dt) * y


# ----------------------------------------------------------------------------------------
# Seeded synthetic inputs (shared by both paths)
# ----------------------------------------------------------------------------------------
def random_kets(N, M, seed, kind="gaussian", dtype=np.complex128):
    """Seeded ket block (N x M, column-major semantics) normalised per column.

    ``gaussian``: complex Gaussian entries; ``phase``: e^{i theta}/sqrt(N).
    Uses numpy PCG64 via default_rng(seed).
    """
    rng = np.random.default_rng(seed)
    if kind == "gaussian":
        X = rng.standard_normal((N, M)) + 1j * rng.standard_normal((N, M))
        X /= np.linalg.norm(X, axis=0, keepdims=True)
    elif kind == "phase":
        th = rng.uniform(0, TWO_PI, size=(N, M))
        X = np.exp(1j * th) / math.sqrt(N)
    else:
        raise ValueError(kind)
    return np.asfortranarray(X.astype(dtype))


def anderson_disorder(N, W, seed):
    """V_i ~ U[-W/2, W/2] (seeded PCG64)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-W / 2, W / 2, size=N)


# ----------------------------------------------------------------------------------------
# Exact gradient of the density loss (checker for the adjoint kernels)
# ----------------------------------------------------------------------------------------
def density_loss_gradient_exact(lat: SquareLattice, psi0, V, B, target, dt, nsteps, spi, point, t1=1.0):
    """L = sum_i (rho_i(T) - target_i)^2 with psi_{n+1} = exp(-i dt H_n) psi_n,
    H_n = tightbinding(V; PointFlux(B[n // spi], point)); exact dL/dV and dL/dB (FP64).

    Uses the Frechet derivative of the matrix exponential (scipy.linalg.expm_frechet):
    dL/dtheta = sum_n Re <lambda_{n+1}, dU_n psi_n>, lambda_N = 4 (rho - target) psi_N,
    lambda_n = U_n^dagger lambda_{n+1}.
    """
    from scipy.linalg import expm_frechet
    N = lat.N
    bonds = nn_bonds(lat)
    unit = PointFlux(1.0, point)
    psis = [np.asarray(psi0, dtype=np.complex128)]
    Hs, Us = [], []
    for n in range(nsteps):
        H = tightbinding_hamiltonian(lat, t1, field=PointFlux(B[n // spi], point), onsite=V).toarray()
        U = expm_exact(H, dt)
        Hs.append(H); Us.append(U)
        psis.append(U @ psis[-1])
    rho = (np.abs(psis[-1]) ** 2).sum(axis=1)
    loss = float(((rho - target) ** 2).sum())
    lam = 4.0 * (rho - target)[:, None] * psis[-1]
    gV = np.zeros(N)
    gB = np.zeros(len(B))
    for n in range(nsteps - 1, -1, -1):
        H = Hs[n]
        A = -1j * dt * H
        # dH/dB on every bond: -2 pi i LI(unit flux) H_ij, Hermitian partner conj
        DB = np.zeros((N, N), dtype=np.complex128)
        for bd in bonds:
            i, j = bd.src - 1, bd.dst - 1
            d = -2j * math.pi * unit.line_integral(bd.r1, bd.r2) * H[i, j] if H[i, j] != 0 else 0.0
            DB[i, j] += d
            DB[j, i] += np.conj(d)
        _, dU = expm_frechet(A, -1j * dt * DB)
        gB[n // spi] += float(np.real(np.sum(np.conj(lam) * (dU @ psis[n]))))
        for i in range(N):
            E = np.zeros((N, N), dtype=np.complex128)
            E[i, i] = -1j * dt
            _, dU = expm_frechet(A, E)
            gV[i] += float(np.real(np.sum(np.conj(lam) * (dU @ psis[n]))))
        lam = Us[n].conj().T @ lam
    return loss, gV, gB


# ------------------------------------------------------------------------------------------
# Density of states (src/greenfunction.jl:306-339) and Chebyshev moments for the KPM checks.
# ------------------------------------------------------------------------------------------
def dos_eigensystem(evals, E, broaden=0.1):
    """dos(eig, E; broaden) = imag(sum(1 ./ (eig.values .- (E + im*broaden)))) / pi
    (src/greenfunction.jl:306), vectorised over E."""
    E = np.atleast_1d(np.asarray(E, dtype=np.float64))
    ev = np.asarray(evals, dtype=np.float64)
    return np.imag((1.0 / (ev[None, :] - (E[:, None] + 1j * broaden))).sum(axis=1)) / np.pi


def ldos_eigensystem(evals, evecs, E, broaden=0.1):
    """Single-particle local density of states at energy E: sum_n |psi_n(i)|^2 Im 1/(E_n - E - i*broaden) / pi,
    the site-resolved form of dos_eigensystem."""
    w = np.imag(1.0 / (np.asarray(evals) - (E + 1j * broaden))) / np.pi
    return (np.abs(evecs) ** 2) @ w


def kpm_moments(H, emin, emax, nmom, vecs=None, per_column=False):
    """mu_n = sum_v <v|T_n(H~)|v>, H~ = (H - b)/a, by the plain three-term recurrence (no
    doubling relations), FP64.  vecs None: the unit vectors (exact trace)."""
    a, b = 0.5 * (emax - emin), 0.5 * (emax + emin)
    Hs = sp.csr_matrix(H, dtype=np.complex128)
    N = Hs.shape[0]
    Ht = (Hs - b * sp.identity(N, format="csr")) / a
    V = np.eye(N, dtype=np.complex128) if vecs is None else np.asarray(vecs, dtype=np.complex128)
    ncols = V.shape[1]
    mu = np.zeros((ncols, nmom))
    T0 = V.copy()
    T1 = Ht @ V
    for n in range(nmom):
        Tn = T0 if n == 0 else T1 if n == 1 else None
        if n >= 2:
            T2 = 2 * (Ht @ T1) - T0
            T0, T1 = T1, T2
            Tn = T1
        mu[:, n] = np.real(np.sum(np.conj(V) * Tn, axis=0))
    return mu if per_column else mu.sum(axis=0)


# ------------------------------------------------------------------------------------------
# Other lattices and internal degrees of freedom, for the general sparse path (lm_ell_*).
# ------------------------------------------------------------------------------------------
HONEYCOMB_T = np.array([[1.0, 0.5], [0.0, math.sqrt(3) / 2]])      # unit vectors (columns)
HONEYCOMB_BASIS = np.array([[0.0, 0.5], [0.0, math.sqrt(3) / 6]])  # basis sites (columns)


def honeycomb_sites(a: int, b: int):
    """HoneycombLattice(a, b) (src/zoo/lattices.jl:145-151): unit cells (j1, j2), 1 <= j1 <= a,
    1 <= j2 <= b, two basis sites each; sites ordered by (j1, j2, basis index) as BravaisPointer
    isless does (src/lattices/bravais/unitcell.jl:126-132).  Returns coordinates (N x 2) and
    the index function."""
    idx = lambda j1, j2, s: ((j1 - 1) * b + (j2 - 1)) * 2 + (s - 1)
    coords = np.zeros((2 * a * b, 2))
    for j1 in range(1, a + 1):
        for j2 in range(1, b + 1):
            for s in (1, 2):
                coords[idx(j1, j2, s)] = HONEYCOMB_BASIS[:, s - 1] + HONEYCOMB_T @ np.array([j1, j2], dtype=float)
    return coords, idx


def _bond_matrix(N, pairs, coords, t1, field, onsite):
    """H[i,j] += t1 e^{-2 pi i LI(r_i -> r_j)}, H[j,i] += its conjugate for every (i, j) in pairs,
    plus the on-site term (src/operators/builder.jl:296-309)."""
    H = sp.lil_matrix((N, N), dtype=np.complex128)
    for i, j in pairs:
        r1 = (float(coords[i][0]), float(coords[i][1]))
        r2 = (float(coords[j][0]), float(coords[j][1]))
        li = 0.0 if field is None else field.line_integral(r1, r2)
        v = t1 * np.exp(-2j * math.pi * li)
        H[i, j] += v
        H[j, i] += np.conj(v)
    if onsite is not None:
        H.setdiag(H.diagonal() + np.asarray(onsite))
    return H.tocsc()


def honeycomb_hamiltonian(a: int, b: int, t1: float = 1.0, B: float = 0.0, onsite=None, field=None):
    """Nearest-neighbour tight-binding on HoneycombLattice(a, b), open boundaries: site A of
    cell (j1, j2) bonds to B of (j1, j2), (j1-1, j2) and (j1, j2-1) (distance 1/sqrt(3)), with
    H[i,j] = t1 e^{-2 pi i LI(r_i -> r_j)} for LandauGauge(B) (or ``field``), LI = (x1+x2)(y2-y1)B/2
    (src/zoo/magneticfields.jl:11-15), H[j,i] its conjugate, and the on-site term."""
    coords, idx = honeycomb_sites(a, b)
    pairs = []
    for j1 in range(1, a + 1):
        for j2 in range(1, b + 1):
            for (k1, k2) in ((j1, j2), (j1 - 1, j2), (j1, j2 - 1)):
                if 1 <= k1 <= a and 1 <= k2 <= b:
                    pairs.append((idx(j1, j2, 1), idx(k1, k2, 2)))
    fld = field if field is not None else (LandauGauge(B) if B else None)
    return _bond_matrix(2 * a * b, pairs, coords, t1, fld, onsite), coords


def honeycomb_hamiltonian_periodic(a: int, b: int, periodic=(True, True), twist=(0.0, 0.0), t1: float = 1.0,
                                   field=None, onsite=None):
    """HoneycombLattice(a, b) with periodic axes (translations a a1, b a2) and twists: the bond
    from A of cell j to B of cell k = j, j - (1,0), j - (0,1) wraps k back into the patch
    (k1 < 1: k1 + a, factor e^{-i Theta_1}; k2 < 1: k2 + b, e^{-i Theta_2}, the phase of a
    boundary crossed backwards), the line integral runs to the unwrapped position of k
    (src/core/boundaries.jl:251-289)."""
    coords, idx = honeycomb_sites(a, b)
    N = 2 * a * b
    H = sp.lil_matrix((N, N), dtype=np.complex128)
    for j1 in range(1, a + 1):
        for j2 in range(1, b + 1):
            i = idx(j1, j2, 1)
            for (k1, k2) in ((j1, j2), (j1 - 1, j2), (j1, j2 - 1)):
                f = 1.0 + 0.0j
                w1, w2 = k1, k2
                if w1 < 1:
                    if not periodic[0]:
                        continue
                    w1 += a
                    f *= complex(math.cos(twist[0]), -math.sin(twist[0]))
                if w2 < 1:
                    if not periodic[1]:
                        continue
                    w2 += b
                    f *= complex(math.cos(twist[1]), -math.sin(twist[1]))
                j = idx(w1, w2, 2)
                r2 = HONEYCOMB_BASIS[:, 1] + HONEYCOMB_T @ np.array([k1, k2], dtype=float)
                li = 0.0 if field is None else field.line_integral((float(coords[i][0]), float(coords[i][1])),
                                                                   (float(r2[0]), float(r2[1])))
                v = t1 * f * np.exp(-2j * math.pi * li)
                H[i, j] += v
                H[j, i] += np.conj(v)
    if onsite is not None:
        H.setdiag(H.diagonal() + np.asarray(onsite))
    return H.tocsc(), coords


KAGOME_BASIS = np.array([[0.0, 0.5, 0.25], [0.0, 0.0, math.sqrt(3) / 4]])


def kagome_hamiltonian(a: int, b: int, t1: float = 1.0, field=None, onsite=None):
    """Nearest-neighbour tight-binding on KagomeLattice(a, b) (src/zoo/lattices.jl:200-211),
    open boundaries: sites A (0,0), B (1/2,0), C (1/4, sqrt(3)/4) per cell, sites ordered by
    (j1, j2, basis); bonds of length 1/2: A-B, A-C, B-C in the cell, B(j) - A(j + (1,0)),
    C(j) - A(j + (0,1)), C(j) - B(j + (-1,1))."""
    idx = lambda j1, j2, s: ((j1 - 1) * b + (j2 - 1)) * 3 + (s - 1)
    coords = np.zeros((3 * a * b, 2))
    for j1 in range(1, a + 1):
        for j2 in range(1, b + 1):
            for s in (1, 2, 3):
                coords[idx(j1, j2, s)] = KAGOME_BASIS[:, s - 1] + HONEYCOMB_T @ np.array([j1, j2], dtype=float)
    pairs = []
    ok = lambda k1, k2: 1 <= k1 <= a and 1 <= k2 <= b
    for j1 in range(1, a + 1):
        for j2 in range(1, b + 1):
            pairs += [(idx(j1, j2, 1), idx(j1, j2, 2)), (idx(j1, j2, 1), idx(j1, j2, 3)), (idx(j1, j2, 2), idx(j1, j2, 3))]
            if ok(j1 + 1, j2):
                pairs.append((idx(j1, j2, 2), idx(j1 + 1, j2, 1)))
            if ok(j1, j2 + 1):
                pairs.append((idx(j1, j2, 3), idx(j1, j2 + 1, 1)))
            if ok(j1 - 1, j2 + 1):
                pairs.append((idx(j1, j2, 3), idx(j1 - 1, j2 + 1, 2)))
    return _bond_matrix(3 * a * b, pairs, coords, t1, field, onsite), coords


def triangular_hamiltonian(a: int, b: int, t1: float = 1.0, field=None, onsite=None):
    """Nearest-neighbour tight-binding on TriangularLattice(a, b) (src/zoo/lattices.jl:136-143),
    open boundaries: site (j1, j2) bonds to (j1+1, j2), (j1, j2+1) and (j1-1, j2+1)."""
    idx = lambda j1, j2: (j1 - 1) * b + (j2 - 1)
    coords = np.zeros((a * b, 2))
    for j1 in range(1, a + 1):
        for j2 in range(1, b + 1):
            coords[idx(j1, j2)] = HONEYCOMB_T @ np.array([j1, j2], dtype=float)
    pairs = []
    for j1 in range(1, a + 1):
        for j2 in range(1, b + 1):
            for (k1, k2) in ((j1 + 1, j2), (j1, j2 + 1), (j1 - 1, j2 + 1)):
                if 1 <= k1 <= a and 1 <= k2 <= b:
                    pairs.append((idx(j1, j2), idx(k1, k2)))
    return _bond_matrix(a * b, pairs, coords, t1, field, onsite), coords


def qwz_hamiltonian(Lx: int, Ly: int, m=1.0, field=None):
    """qwz(l, m; field) (src/zoo/models.jl:129-137) on SquareLattice(Lx, Ly), open boundaries,
    two internal states per site (matrix index 2 (site - 1) + spin).  The builder places each
    term as written (src/operators/builder.jl:134-151, constructoperator.jl:14-19): for the
    bond (i, i + e) of BravaisTranslation(axis) -- the pair (site, destination(site)),
    src/lattices/bravais/bonds.jl:87-98 -- the block H[i, i+e] = M e^{-2 pi i LI(r_i, r_{i+e})}
    with M = [1 -i; -i -1]/2 (x) or [1 -1; 1 -1]/2 (y), and H[i+e, i] its adjoint; the
    on-site block is m_i sigma_z."""
    lat = SquareLattice(Lx, Ly)
    N = Lx * Ly
    mz = np.array([[1, 0], [0, -1]], dtype=np.complex128)
    Mx = np.array([[1, -1j], [-1j, -1]], dtype=np.complex128) / 2
    My = np.array([[1, -1], [1, -1]], dtype=np.complex128) / 2
    mm = np.broadcast_to(np.asarray(m, dtype=float), (N,))
    fld = adapt_field(field, lat) if field is not None else None
    H = sp.lil_matrix((2 * N, 2 * N), dtype=np.complex128)
    site = lambda x, y: (x - 1) * Ly + (y - 1)
    for x in range(1, Lx + 1):
        for y in range(1, Ly + 1):
            s = site(x, y)
            H[2 * s:2 * s + 2, 2 * s:2 * s + 2] = mm[s] * mz
            for (dx, dy, Mb) in ((1, 0, Mx), (0, 1, My)):
                if x + dx <= Lx and y + dy <= Ly:
                    t = site(x + dx, y + dy)
                    li = 0.0 if fld is None else fld.line_integral((x, y), (x + dx, y + dy))
                    blk = Mb * np.exp(-2j * math.pi * li)
                    H[2 * s:2 * s + 2, 2 * t:2 * t + 2] = blk
                    H[2 * t:2 * t + 2, 2 * s:2 * s + 2] = blk.conj().T
    return H.tocsc()


def csc_arrays(H):
    """(colptr, rowval, nzval) of a scipy CSC matrix in the reference's 1-based layout."""
    H = sp.csc_matrix(H)
    H.sort_indices()
    return (H.indptr.astype(np.int64) + 1, H.indices.astype(np.int64) + 1, np.asarray(H.data, dtype=np.complex128))


def csc_currents(H, state, weights=None, is_density=None):
    """2 Im(H[i,j] P[j,i]) for every stored entry (i, j) of H in CSC order (0 on the diagonal)."""
    H = sp.csc_matrix(H)
    H.sort_indices()
    cols = np.repeat(np.arange(H.shape[1]), np.diff(H.indptr))
    rows = H.indices
    s = np.asarray(state)
    if is_density:
        pji = s[cols, rows]
    else:
        w = np.ones(s.shape[1]) if weights is None else np.asarray(weights)
        pji = np.einsum("bm,bm,m->b", s[cols, :], np.conj(s[rows, :]), w)
    J = 2.0 * np.imag(H.data * pji)
    J[rows == cols] = 0.0
    return J


# ----------------------------------------------------------------------------------------
# f3: currents with internal degrees of freedom      src/zoo/currents.jl:24-27, :81-102, :170-184
#                                                     src/currents.jl:104-109, :223-237
# ----------------------------------------------------------------------------------------
def _dense_state(state, weights=None, is_density=None):
    s = np.asarray(state)
    if s.ndim == 1:
        return np.outer(s, np.conj(s))
    if is_density or (is_density is None and weights is None and s.shape[0] == s.shape[1]):
        return s
    w = np.ones(s.shape[1]) if weights is None else np.asarray(weights, dtype=np.float64)
    return (s * w[None, :]) @ np.conj(s).T


def local_operator_current(H, P, ndof, op, i, j):
    """LocalOperatorCurrents(H, P, op)[i, j] with 0-based sites (src/zoo/currents.jl:170-184):
    T = the (i, j) block of H (``_block``, :24-27); sum over alpha, beta of
    2 Im((op T)[alpha, beta] * P[(j, beta), (i, alpha)]).  op = identity is DensityCurrents
    (:92-102)."""
    n = ndof
    T = np.asarray(sp.csr_matrix(H)[i * n:(i + 1) * n, j * n:(j + 1) * n].todense())
    O = np.eye(n) if op is None else np.asarray(op, dtype=np.complex128)
    OT = O @ T
    tot = 0.0
    for a in range(n):
        for b in range(n):
            tot += 2.0 * np.imag(OT[a, b] * P[j * n + b, i * n + a])
    return tot


def site_currents(H, state, ndof, op=None, weights=None, is_density=None):
    """{(i, j): value} for every ordered pair of distinct sites whose H block is nonzero."""
    P = _dense_state(state, weights, is_density)
    A = sp.coo_matrix(H)
    pairs = sorted({(int(r) // ndof, int(c) // ndof) for r, c in zip(A.row, A.col) if r // ndof != c // ndof})
    return {(i, j): local_operator_current(H, P, ndof, op, i, j) for (i, j) in pairs}


def site_currents_matrix(H, state, ndof, op=None, **kw):
    """Currents(curr) (src/currents.jl:223-237): for every site pair i > j the value curr[i, j]
    at [i, j] and its negative at [j, i]; |value| < 1e-10 dropped.  Pairs with a zero block
    carry zero current and are skipped."""
    nsites = H.shape[0] // ndof
    vals = site_currents(H, state, ndof, op, **kw)
    I, J, V = [], [], []
    for (i, j), v in vals.items():
        if i > j and abs(v) >= CURRENTS_EPS:
            I += [i, j]
            J += [j, i]
            V += [v, -v]
    return sp.csc_matrix((V, (I, J)), shape=(nsites, nsites))


def currentsfromto(M, src):
    """currentsfromto(curr, src) (src/currents.jl:104-109) on a materialised matrix: the sum of
    M[src, j] over every other site j (0-based src)."""
    row = np.asarray(sp.csr_matrix(M)[src, :].todense()).ravel()
    return float(row.sum() - row[src])


def entry_op_currents(H, state, ndof, op=None, weights=None, is_density=None):
    """The per-entry split of local_operator_current: for the stored entry
    (r, c) = ((i, k), (j, beta)) of H with i != j, 2 Im(H[r,c] sum_alpha op[alpha,k] P[c, (i, alpha)]),
    in CSC order (0 for entries inside one site block).  Summing the entries of the (i, j)
    block gives local_operator_current(H, P, ndof, op, i, j)."""
    P = _dense_state(state, weights, is_density)
    A = sp.csc_matrix(H)
    A.sort_indices()
    cols = np.repeat(np.arange(A.shape[1]), np.diff(A.indptr))
    rows = A.indices
    O = np.eye(ndof) if op is None else np.asarray(op, dtype=np.complex128)
    si, k = rows // ndof, rows % ndof
    Q = np.zeros(len(rows), dtype=np.complex128)
    for a in range(ndof):
        Q += O[a, k] * P[cols, si * ndof + a]
    J = 2.0 * np.imag(A.data * Q)
    J[si == cols // ndof] = 0.0
    return J
