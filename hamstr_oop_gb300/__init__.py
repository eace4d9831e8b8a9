"""GB300-native HAMSTR steady ADI iteration (2D Euler, line-implicit).

The compute path lives in ``csrc/`` (CUDA kernels for sm_103a behind a C ABI,
declared in ``include/hamstr_gpu.h``) and the C++ host in ``csrc/host``; this
package holds the Python bindings, the case generator and the build step.
"""
