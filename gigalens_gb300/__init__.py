"""GB300-native (sm_103a) substrate for the GIGA-Lens forward model + likelihood.

``gigalens_gb300.{profile,model,simulator,inference}`` mirror the reference's
abstract API (``gigalens/{profile,model,simulator,inference}.py``) and
``gigalens_gb300.cuda`` mirrors the ``gigalens.tf`` substrate: the same class
names, constructor arguments and call signatures, backed by hand-written CUDA
kernels in ``libgigalens_cuda.so`` behind a C ABI (``include/gigalens_cuda.h``).
"""
__version__ = "0.1.0"
