"""GB300-native finite-element hot path for OpenCMP: form assembly into CSR and the Krylov solve,
as hand-written sm_103a CUDA behind a C ABI (libopencmp_gpu.so), with OpenCMP's Model/Solver
interface on top. See include/opencmp_gpu.h for the boundary."""

__version__ = '0.1.0'
