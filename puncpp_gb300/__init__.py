"""GB300 particle-in-cell engine for the PUNC++ per-timestep particle path.

The compute path is libpunc_gpu.so (hand-written sm_103a CUDA behind the C
ABI of include/punc_gpu.h); this package holds its Python front end with the
reference's interface names (punc.py), the synthetic mesh generator
(meshgen.py) and the in-tree build step (build_lib.py).
"""
from . import meshgen  # noqa: F401

__all__ = ["meshgen"]
