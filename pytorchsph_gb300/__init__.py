"""GB300-native (sm_103a) hot path of wi-re/pytorchSPH: hashed-grid neighbor search and
the deltaSPH / DFSPH SPH kernel summations, behind the reference's own extension and
module interfaces.

* `pytorchsph_gb300.neighborSearch` — drop-in for the reference's `neighborSearch`
  extension module (cppSrc/neighSearch.cpp:413-418).
* `pytorchsph_gb300.search.GridSearch` — native CSR neighbor search with fused density.
* `pytorchsph_gb300.build.build()` — compiles libsph_gb300.so (nvcc, sm_103a).
"""
from . import build  # noqa: F401

__version__ = "0.1.0"
