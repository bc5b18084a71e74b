"""GB300-native HEOM propagation engine.

A drop-in for libheom's propagation path (heom_hilb / heom_liou / heom_ado
models stepped by rk4 / lsrk4 / rkdp through qme_solver).  The compute path is
hand-written CUDA for sm_103a behind the C ABI of include/heomgb.h; this package
is its Python mirror (ctypes) plus the workload definitions.
"""
from .params import HeomParams
from .heom import (heom, heom_hilb, heom_liou, heom_ado, redfield_hilb, redfield_liou,
                   solver_base, rk4, lsrk4, rkdp, qme_solver, batch_solver,
                   from_params, SOLVERS)
from ._lib import HeomError, load, launch_count, library_path, probe_fma_peaks

__all__ = ["HeomParams", "heom", "heom_hilb", "heom_liou", "heom_ado", "redfield_hilb", "redfield_liou", "solver_base", "rk4", "lsrk4", "rkdp",
           "qme_solver", "batch_solver", "from_params", "SOLVERS", "HeomError", "load", "launch_count", "library_path",
           "probe_fma_peaks"]
