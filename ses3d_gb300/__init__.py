"""GB300-native SES3D: the spectral-element velocity-stress time step of SES3D
(spherical section, GLL bases, SLS attenuation, PML, adjoint Frechet kernels)
as sm_103a CUDA kernels behind a C ABI (include/ses3d_gpu.h).

Modules: formats (reference file formats), synth (seeded synthetic workloads),
solver (Simulation: the host interface over libses3d_gpu.so), build (nvcc build).
"""
from . import formats  # noqa: F401

__version__ = "0.1.0"
