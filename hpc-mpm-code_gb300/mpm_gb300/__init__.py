"""GB300-native MPM transfer path (P2G / grid update / G2P / implicit matvec).

The compute lives in libmpm_gb300.so (hand-written CUDA for sm_103a behind the
C ABI declared in include/mpm_gpu.h); this package holds the in-tree build,
the ctypes binding and the synthetic scene generators.
"""
