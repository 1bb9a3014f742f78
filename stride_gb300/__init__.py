"""GB300-native implementation of Stride's iso-acoustic FDTD hot path.

The compute path is libstrideacc.so (hand-written sm_103a CUDA behind a C ABI, declared in
include/strideacc.h); this package holds the host-side mirror of the reference's operator
interface around it.
"""

__version__ = '0.1.0'
