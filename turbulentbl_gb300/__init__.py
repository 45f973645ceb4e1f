"""GB300-native time-step library for the turbulentBL boundary-layer DNS.

The product is libtblgpu.so (turbulentbl_gb300/csrc, C ABI in include/tbl_gpu.h);
this package holds the host side: mesh and parameter setup, seeded synthetic
inputs, the 3D.tp restart format, and a ctypes driver over the C ABI.
"""
