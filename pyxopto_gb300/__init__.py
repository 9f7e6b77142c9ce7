"""pyxopto_gb300 - GB300 (sm_103a) Monte Carlo photon-packet transport for
layered (mcml) and voxelized (mcvox) media, a drop-in for PyXOpto's
OpenCL simulators.  The compute runs in libxopto_gb300.so (hand-written CUDA
kernels behind a C ABI, include/xopto_gb300.h)."""
__version__ = '0.1.0'
