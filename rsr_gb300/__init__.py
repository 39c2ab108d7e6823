"""GB300 rasteriser: rsr's tile-binning rasteriser hot path as sm_103a CUDA.

The product is the C-ABI library librsrgpu.so (include/rsrgpu.h), built in
tree by rsr_gb300.build.  This package is its host-side mirror of rsr's
rglv::GL / rglv::GPU calling surface (gl.py, gpu.py) plus the seeded scene
generators used by the tests and the benchmark (scenes.py).
"""
from . import abi  # noqa: F401
