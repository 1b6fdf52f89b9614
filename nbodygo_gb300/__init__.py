"""GB300-native compute cycle of the nbodygo N-body simulator.

The product is libnbgpu.so (include/nbgpu.h): hand-written sm_103a kernels for
nbodygo's direct-sum compute cycle behind a C ABI that the reference's Go
runner can call through cgo.  This package builds it in-tree
(nbodygo_gb300.build) and binds it from Python (nbodygo_gb300.api).
"""
from .api import Simulation, NbgError, load_library, probe_peaks  # noqa: F401
