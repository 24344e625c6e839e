"""taufactor_gb300: TauFactor's steady-state voxel diffusion solve on one GB300 (sm_103a).

Drop-in for the through-transport solvers of tldr-group/taufactor v1.2.1
(``taufactor/__init__.py:3-11``): ``Solver``, ``PeriodicSolver``, ``AnisotropicSolver``,
``MultiPhaseSolver``, ``PeriodicMultiPhaseSolver``, ``ElectrodeSolver``,
``PeriodicElectrodeSolver``, ``ImpedanceSolver`` and ``PeriodicImpedanceSolver`` with the same
constructor and ``solve()`` surface. The sweeps run as hand-written CUDA kernels of ``lib/libtaufactor_gb300.so`` through
its C ABI (``include/taufactor_gb300.h``). ``read_tiff`` loads the multi-page TIFF volumes the
reference's examples read with ``tifffile.imread`` (README.md:51-55).
"""
from .batch import BatchSolve, MultiDeviceBatchSolve, split_volumes
from .kappa import DeffFunction, KappaSolver, d_eff
from .solvers import (AnisotropicSolver, ElectrodeSolver, MultiPhaseSolver, PeriodicElectrodeSolver,
                      PeriodicMultiPhaseSolver, PeriodicSolver, SORSolver, Solver, ThroughTransportSolver)
from .impedance import ImpedanceSolver, PeriodicImpedanceSolver
from .tiff import read_tiff, write_tiff

__all__ = ["Solver", "PeriodicSolver", "AnisotropicSolver", "MultiPhaseSolver", "PeriodicMultiPhaseSolver",
           "ElectrodeSolver", "PeriodicElectrodeSolver", "ImpedanceSolver", "PeriodicImpedanceSolver",
           "SORSolver", "ThroughTransportSolver", "BatchSolve", "MultiDeviceBatchSolve", "split_volumes", "KappaSolver", "DeffFunction", "d_eff",
           "read_tiff", "write_tiff"]
__version__ = "0.1.0"
