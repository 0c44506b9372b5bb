"""GB300-native electrostatic global placement (a drop-in for Texo's eplace::place).

The engine is the CUDA library built from texo_gb300/csrc behind the C ABI of
include/texo_gp.h; this package is its Python host mirror.
"""
from .abi import TexoGpError, load  # noqa: F401
from .placer import Placer, default_params, place  # noqa: F401
from .problem import Problem, WORKLOADS, density_problem, synthetic  # noqa: F401
