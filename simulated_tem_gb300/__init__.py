"""GB300 (sm_103a) imaging hot path of simulated_tem's d2bi.

The CUDA kernels and the C ABI live in ``csrc/`` and build into the in-tree
``libstem.so`` (``build.py``); ``imaging`` is the Python face of the
reference's Lib_DynamicalTwoBeamImaging interface, ``synth`` makes the seeded
synthetic cells of the workloads.
"""
from . import _lib, synth  # noqa: F401
from .imaging import Context, DynamicalTwoBeamImaging, d2bi_condition  # noqa: F401
