"""clode_gb300: a GB300-native engine for large ensembles of ODE/SDE
initial-value problems, a drop-in for clODE's transient, features and
trajectory paths.

* ``clode_gb300.clode_cpp_wrapper`` — the module clODE's Python package
  imports as ``clode.cpp.clode_cpp_wrapper`` (same classes and names).
* ``include/clode_gb300.h`` — the C ABI underneath it.
* ``clode_gb300.surrogate`` — the learned surrogate (tensor-core MLP) and
  surrogate-screened feature maps.
* ``clode_gb300.shard`` — splitting an ensemble over several GPUs.
* ``clode_gb300/rhs/`` — example model sources (clODE's getRHS format).
"""
import os

RHS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rhs")


def rhs_path(name: str) -> str:
    """Path of a bundled model source, e.g. ``rhs_path("lactotroph.cl")``."""
    return os.path.join(RHS_DIR, name)
