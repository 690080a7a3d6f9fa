"""GB300-native edge-element assembly and complex sparse solve for MoVFEM_3DMT.

The hot path of the reference (``global_vfem`` + ``zmumps`` + the receiver Z/rho/phi
evaluation) runs as hand-written sm_103a CUDA kernels behind a C-ABI
(``include/movfem_gpu.h``).  ``movfem_gb300.api`` is the host-side mirror of the
reference's call sites; ``movfem_gb300.mesh`` generates synthetic models in the
reference's mesh layout.
"""
from . import mesh  # noqa: F401

__all__ = ["mesh"]
