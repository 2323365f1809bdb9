"""lmgpu -- GB300 backend for the LatticeModels.jl time-evolution path.

Host-side mirror of the reference's API for ``Evolution(t -> h(t), P_0)`` over
``tightbinding_hamiltonian`` with Landau/point-flux fields, read out through ``localdensity``
and ``DensityCurrents``.  All compute runs in liblmgpu.so (hand-written sm_103a CUDA); this
package only holds the host-side bookkeeping and the ctypes bindings.
"""
from ._lib import LMError, load as load_library
from . import adjoint, kpm
from .adjoint import DensityLossAdjoint
from .batch import Batch
from .bravais import BravaisLattice, HoneycombLattice, KagomeLattice, LatticeHamiltonian, TriangularLattice
from .device import Context, default_context
from .evolution import ChebyshevGPU, Evolution, EvolutionIterator, EvolutionSolver, EvolutionTimestamp
from .fields import FieldSum, LandauGauge, NoField, PointFlux, PointFluxes, SymmetricGauge
from .hamiltonian import Hamiltonian, tightbinding_hamiltonian
from .lattice import LatticeValue, SquareLattice, coordvalues
from .observables import Currents, DensityCurrents, SubCurrents, currentsfrom, currentsfromto, localdensity
from .sparse import LocalOperatorCurrents, SiteCurrents, Sites, SparseHamiltonian, entry_currents
from .spectrum import densitymatrix, diagonalize
from .states import DensityMatrix, DeviceState, Ket, KetBlock, Operator
from .timesequence import (ReadoutRing, TimeSequence, differentiate, integrate, moment_currents,
                           moment_density, timesequences)

__all__ = [
    "adjoint", "kpm", "DensityLossAdjoint", "Batch", "LMError", "load_library", "Context", "default_context",
    "ChebyshevGPU", "Evolution", "EvolutionIterator", "EvolutionSolver", "EvolutionTimestamp",
    "FieldSum", "LandauGauge", "NoField", "PointFlux", "PointFluxes", "SymmetricGauge",
    "Hamiltonian", "tightbinding_hamiltonian", "LatticeValue", "SquareLattice", "coordvalues",
    "Currents", "DensityCurrents", "SubCurrents", "currentsfrom", "currentsfromto", "localdensity", "densitymatrix", "diagonalize",
    "DensityMatrix", "DeviceState", "Ket", "KetBlock", "Operator",
    "LocalOperatorCurrents", "SiteCurrents", "Sites", "SparseHamiltonian", "entry_currents", "ReadoutRing", "TimeSequence", "differentiate", "integrate", "moment_currents", "moment_density",
    "timesequences", "BravaisLattice", "HoneycombLattice", "KagomeLattice", "TriangularLattice", "LatticeHamiltonian",
]
