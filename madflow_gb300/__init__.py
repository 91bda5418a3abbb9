"""madflow_gb300: GB300-native (sm_103a) leading-order matrix-element integrand
and VEGAS integrator with madflow's interfaces.

The compute runs in hand-written CUDA kernels behind the C ABI of
``include/madflow_gb300.h`` (library built by ``madflow_gb300.build``);
PyTorch only provides device memory and streams.
"""
__version__ = "0.1"

from .config import DTYPE, DTYPECOMPLEX, DTYPEINT, complex_me, float_me, int_me  # noqa: F401
