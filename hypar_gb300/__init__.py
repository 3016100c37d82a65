"""hypar_gb300 -- HyPar's explicit WENO5 right-hand side and Runge-Kutta step
on one GB300 GPU, behind HyPar's own function-pointer surface (C ABI in
include/gbhypar.h, implemented by libgbhypar.so in this directory)."""
from .solver import Ensemble, Inputs, Solver, rk_table, run_case  # noqa: F401
from . import cases  # noqa: F401
