"""GB300 transport sweep for SimpleMOC: device storage, hand-written sm_103a
kernels, and a thin C ABI (include/simplemoc_gb300.h)."""
from ._lib import MocError, LIB_PATH
from .problem import (CONFIGS, CONFIG_DEFAULT, CONFIG_SMALL, HostProblem, ProblemSpec,
                      exp_table, generate)
from .solver import Solver

__all__ = ["MocError", "LIB_PATH", "CONFIGS", "CONFIG_DEFAULT", "CONFIG_SMALL", "HostProblem",
           "ProblemSpec", "exp_table", "generate", "Solver"]
