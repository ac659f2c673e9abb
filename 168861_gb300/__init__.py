"""GB300-native solver hot path of Neurite (explicit and implicit cable/HH steppers).

The compute path is libneurite_gb300.so (hand-written CUDA for sm_103a behind the C ABI
of include/neurite_gb300.h); this package is its host-side mirror.  Import it with
importlib.import_module("168861_gb300") (the directory name starts with a digit).
"""
from . import model  # noqa: F401  (tree descriptions in the reference numbering)
from ._lib import LIB_PATH, NeuriteError, load  # noqa: F401
from .solver import (Batch, Derived, ProblemArrays, Recording, Server, SolverEx,  # noqa: F401
                     SolverIm, State, derive, derive_batch, kernel_launches, measurement_point,
                     simulate, step_size)
