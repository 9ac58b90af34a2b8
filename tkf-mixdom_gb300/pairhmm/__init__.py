"""GB300-native batched 2D pair-HMM forward/backward and E-step.

Host-side mirror of the reference's (evoldoers/tkf-mixdom) 2D pair-HMM
interface, computing through the CUDA library ``libpairhmm.so`` (C ABI in
include/pairhmm.h).
"""
__version__ = '0.1.0'
