"""dynoplan_gb300 -- the db-A* / iDb-A* node expansion of dynoplan on one
GB300 (sm_103a): C ABI in include/dpg.h, CUDA kernels in csrc/, Python
handle in gpu.py, seeded synthetic workloads in workloads.py.
"""
from . import workloads  # noqa: F401

__all__ = ["workloads"]
