"""GB300-native explicit hex8 / neo-Hookean transient-dynamics engine.

The compute path is libnimble_gb300.so (hand-written sm_103a CUDA behind the
C ABI of include/nimble_gb300.h); `engine.Model` binds it.
"""
from .mesh import BoundaryCondition, Problem, cube_problem, critical_time_step  # noqa: F401
