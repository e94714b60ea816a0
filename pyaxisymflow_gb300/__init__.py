"""GB300-native (sm_103a) drop-in for PyAxisymFlow's per-timestep grid hot path.

Module paths and callables mirror the reference package ``pyaxisymflow``
(``pyaxisymflow_gb300.kernels.brinkmann_penalize.brinkmann_penalize`` ...).
Every kernel takes CUDA ``torch`` tensors of shape (nr, nz), row-major, and
mutates its outputs in place on torch's current stream, like the numpy
originals. The compute runs in the CUDA library declared by
``include/axisym_gb300.h``; there is no CPU path.
"""
__version__ = "0.1.0"
