"""GB300-native WCSPH step (DualSPHysics hot path): hand-written sm_103a CUDA
behind a C ABI (include/gbsph.h, libgbsph.so), with a host-side mirror of the
reference's JSphGpuSingle driver and its case / particle-file formats."""
__version__ = "0.1.0"
