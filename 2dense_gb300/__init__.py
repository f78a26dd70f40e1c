"""GB300-native (sm_103a, FP64) implementation of 2DENSE's right-hand-side evaluation and
TVD-RK3 time advance, behind the C ABI of include/dense2d.h.

The package holds the CUDA sources (``csrc/``), their build recipe (``build.py``), the ctypes
binding of the C ABI (``_abi.py``) and the host-side mirror of the reference's per-stage
interface (``solver.py``). The compute path is the in-tree ``csrc/_build/libdense2d.so``;
importing ``Solver`` without it raises.
"""
from ._abi import (DenseConfig, DenseError, default_config, load_library, array_sizes,  # noqa: F401
                   LIB_PATH)
from .solver import (BatchSolver, Solver, config_default, init_general,  # noqa: F401
                     read_binary, read_par_namelist, setup_config)
