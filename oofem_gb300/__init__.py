"""GB300-native (sm_103a) structural hot path of OOFEM: element integration,
material updates, deterministic sparse assembly and Jacobi-PCG, behind a C ABI
(include/oofem_gb300.h, liboofem_gb300.so). See native.py for the Python
mirror of the reference interfaces and meshgen.py for the synthetic meshes."""
from . import meshgen  # noqa: F401

__all__ = ["meshgen", "native", "build"]
