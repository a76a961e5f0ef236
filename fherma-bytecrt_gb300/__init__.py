"""GB300-native exact negacyclic multiplier: c = a*b mod (X^N+1) mod q.

Drop-in for ByteCRT's plugin path (fherma_init / fherma_run / fherma_free,
native-smoke/fherma.h:46-48).  The compute path is native: sm_103a kernels in
libbytecrt_gb300.so behind the C ABI of include/bytecrt_gb300.h.
"""
from . import inputs  # noqa: F401
from .native import (BcgError, Multiplier, Plan, Batch, Server, lib, header_functions,  # noqa: F401
                     BCG_OK, BCG_ERR_INVALID, BCG_ERR_CUDA, BCG_ERR_NOMEM,
                     BCG_ERR_DEVICE_TIMEOUT, BCG_ERR_BUSY, BCG_ERR_TIMEOUT)
from .plugin import Point, Inputs, Outputs, fherma_init, fherma_run, fherma_free  # noqa: F401
