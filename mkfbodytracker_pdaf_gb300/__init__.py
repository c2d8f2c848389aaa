"""GB300-native (sm_103a) filtering hot path of the mkfbodytracker_pdaf tracker.

Compute lives in libmkf_gb300.so (hand-written CUDA behind the C ABI in
include/mkf_gb300.h); this package holds its ctypes binding, the host-side
mirror of the reference's filter classes, the OpenCV-YAML model reader and the
seeded synthetic workloads.
"""
__version__ = "0.1.0"
