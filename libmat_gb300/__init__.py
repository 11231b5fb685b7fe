"""GB300-native restricted power diagram (RPD) engine.

Drop-in for libmat's rpd3d path (compute_clipped_voro_diagram_GPU /
ConvexCellHost).  The compute path is librpd_gb300.so: hand-written sm_103a
CUDA kernels behind a C ABI (include/rpd_gb300.h).  This package holds the
Python host bindings (ctypes) and the synthetic workload generators.
"""
