"""GB300-native Fourier-domain acceleration search.

The compute path is ``libaccelsearch.so`` (CUDA for sm_103a behind a C ABI,
declared in include/accelsearch.h).  Importing this package does not load
it; :func:`gpu_accelsearch_gb300.native.lib` does, and raises if it is
missing.
"""
__all__ = ["native", "search", "synth"]
