"""GB300-native discrete-group Symanzik Metropolis engine.

A drop-in for the hot path of hlammiv/dym_symanzik_action (`dym-mod-metro`):
CUDA kernels for sm_103a behind the C ABI of include/dymgpu.h
(lib/libdymgpu.so), the `dym-mod-metro` executable (bin/), and this Python
host interface.
"""
from ._lib import DymError  # noqa: F401
from .metro import Group, Lattice, Measurement, SweepStats, checkpoint_info, load_group  # noqa: F401

__all__ = ["DymError", "Group", "Lattice", "Measurement", "SweepStats", "checkpoint_info", "load_group"]
