"""GB300-native ADER-DG element update with SeisSol's kernel interface.

The compute path is libsei_gb300.so (hand-written CUDA for sm_103a behind the C ABI of
include/sei_gb300.h).  This package is a thin ctypes front-end mirroring the reference's
proxy bindings (app/Proxy/Bindings.cpp:14-60) and kernel interface.  There is no CPU
fallback: without the built library every entry point raises.
"""
from .lib import (  # noqa: F401
    tc_gemm_check,
    mlp_gradient,
    fit_attenuation,
    plasticity_nodes,
    plasticity_relax_factor,
    mlp_predict,
    mlp_num_params,
    Context,
    RSParams,
    LSWParams,
    ISRParams,
    TPParams,
    DR_FIELDS,
    SeiError,
    KERNELS,
    load_library,
    derivatives_size,
    nbasis,
    padded_basis,
)
from .proxy import ProxyConfig, ProxyOutput, run_proxy  # noqa: F401

__all__ = ["Context", "SeiError", "KERNELS", "load_library", "ProxyConfig", "ProxyOutput", "run_proxy",
           "derivatives_size", "nbasis", "padded_basis"]
