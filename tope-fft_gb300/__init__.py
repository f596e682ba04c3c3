"""GB300-native FFT library behind the topeFFT C interface (matze/tope-fft).

The product is libtopefft.so (C host code + CUDA kernels for sm_103a) with
the headers in include/; this package holds its sources (csrc/), its build
script and a ctypes mirror of the C interface (topefft.py).
"""
from .topefft import *  # noqa: F401,F403
from .topefft import lib, load_library, LIB_PATH  # noqa: F401
