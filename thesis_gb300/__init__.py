"""GB300-native lattice-Boltzmann time-step engine (sm_103a CUDA + C ABI).

Drop-in for the time-step loop of the reference solver ZPaulo/Thesis
(`lbm-solver_final`): same lattice files and Arguments, one fused CUDA kernel
per step.  `thesis_gb300.solver.Solver` wraps the C ABI declared in
include/thesis_lbm.h; `thesis_gb300.lattice` builds lattices.
"""
from . import lattice  # noqa: F401
