"""lcpgrid: GB300 (sm_103a) real-space grid path of LCPAODFT.jl.

The compute lives in liblcpgrid.so (CUDA kernels behind the C ABI of
include/lcpgrid.h); this package is the host-side mirror of the reference's
grid-path functions plus the species-data readers and the synthetic workload
builders.  Importing ``lcpgrid`` requires the shared library to be built.
"""
from ._lib import LCPError, exported_symbols  # noqa: F401
from .api import *  # noqa: F401,F403
from .api import __all__ as _api_all
from .pao import PAO, PCC, Read_PAO, Read_VPS_PCC, get_ialpha_index  # noqa: F401

__all__ = list(_api_all) + ["LCPError", "PAO", "PCC", "Read_PAO", "Read_VPS_PCC", "get_ialpha_index"]
