"""GB300-native skeleton hot path of the Muesli skeleton library.

The product is libmsl_gb300.so (CUDA kernels for sm_103a behind the C ABI of
include/msl_gb300.h) plus the drop-in C++ front end under include/ of this
package (DA/DM/DC with map/zip/fold/gather/mapStencil). `abi` is the ctypes
binding used by Python callers; `build` compiles the library.
"""
__version__ = "0.1.0"
