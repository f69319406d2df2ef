"""rimugpu -- GB300 implementation of Rimu.jl's FCIQMC step and matrix-free H*v.

Python mirror of the Rimu.jl API for this path (ProjectorMonteCarloProblem, solve,
StochasticStyle traits, HubbardReal1D / HubbardRealSpace / HubbardMom1D, BoseFS / FermiFS)
over the C ABI of librimu_gpu (include/rimu_gpu.h).  All compute runs in the CUDA library.
"""
from ._lib import RimuError, load as load_library, library_path
from .addresses import BoseFS, CompositeFS, FermiFS, FermiFS2C, near_uniform, near_uniform_onr
from .hamiltonians import (CubicGrid, HardwallBoundaries, HubbardMom1D, HubbardReal1D,
                           HubbardRealSpace, LadderBoundaries, PeriodicBoundaries,
                           continuum_dispersion, hubbard_dispersion)
from .styles import (Exact, IsDeterministic, IsDynamicSemistochastic, IsStochasticInteger,
                     NoCompression, ThresholdCompression, WithReplacement, default_style)
from .dvec import (FirstOrderTransitionOperator, GPUDVec, GPUWorkingMemory, add_, apply_operator,
                   dot_operator, mul, scale_, working_memory)
from .problem import (AllOverlaps, DoubleLogProjected, DoubleLogUpdate,
                      DoubleLogUpdateAfterTargetWalkers, DontUpdate,
                      LogUpdate, LogUpdateAfterTargetWalkers, NoStats, PMCSimulation,
                      ProjectedEnergy, ProjectorMonteCarloProblem, ReportDFAndInfo, init, solve)
from .stats import blocking_analysis, mean_and_se, projected_energy, shift_estimator
from .hv import BasisOperator, eigsolve, hv
from .batch import BatchedReplicas, solve_batched
from .initiators import CoherentInitiator, Initiator, InitiatorRule, NonInitiator, SimpleInitiator
from .rimuio import load_state, save_state

__all__ = [n for n in dir() if not n.startswith("_")]
