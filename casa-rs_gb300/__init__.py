"""casa-rs_gb300: the GB300 (sm_103a) imaging hot path of casa-imaging.

csrc/        CUDA kernels and the extern "C" boundary (libcasars_cuda.so)
casars_cuda/ Python host mirror of casa-imaging's gridder, imaging and
             deconvolver seams, over ctypes
build.py     in-tree nvcc build of lib/libcasars_cuda.so
"""
