"""exanbody_gb300: GB300-native (sm_103a) exaNBody particle hot path.

The compute lives in libxnb_gpu.so (C ABI: include/xnb_gpu.h); `xnb` is its
ctypes binding, `workloads` the seeded synthetic systems, `units` the
reference's internal unit constants.
"""
__version__ = "0.1.0"
