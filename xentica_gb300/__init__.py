"""GB300-native engine for Xentica buffered-state cellular automata.

Same public API as the ``xentica`` package (``core``, ``seeds``, ``tools``,
``bridge``, ``utils``); models run on hand-written sm_103a CUDA kernels
reached through the ``libxk`` C-ABI (``include/xk.h``).
"""
__version__ = "0.2.0+gb300"
