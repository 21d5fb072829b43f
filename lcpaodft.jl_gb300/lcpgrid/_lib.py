"""ctypes binding of liblcpgrid.so (declarations in include/lcpgrid.h).

The library is the product: every compute call of this package goes through
it.  Importing this module raises ImportError when the shared library has not
been built, so no call can silently fall back to a CPU implementation.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# LCPGRID_BOUNDS_CHECK=1 selects the check build (device bounds checks on every
# gathered index, read with lcp_bounds_check_status)
LIB_PATH = os.path.join(_HERE, "liblcpgrid_check.so" if os.environ.get("LCPGRID_BOUNDS_CHECK") == "1"
                        else "liblcpgrid.so")

LCP_OK, LCP_EINVAL, LCP_ENOMEM, LCP_EDEVICE, LCP_ETIMEDOUT, LCP_ENOTSUP, LCP_ESTATE = range(7)
LCP_XC_LDA, LCP_XC_LSDA, LCP_XC_GGA_PBE = range(3)
SPIN = {"off": 0, "on": 1, "nc": 2}
NCHAN = {"off": 1, "on": 2, "nc": 4}
XC = {"LDA": 0, "LSDA": 1, "GGA_PBE": 2}
PREC = {"fp64": 0, "fp32": 1, "bf16x3": 2}

F_FNAN, F_NATN, F_NCN, F_GRIDN_ATOM, F_GRIDLIST, F_CELLLIST = 0, 1, 2, 3, 4, 5
F_PAIR_ATOM, F_PAIR_NATN, F_PAIR_NCN, F_NUMOLG, F_GLIST1, F_GLIST2, F_ATV_IJK = 6, 7, 8, 9, 10, 11, 12


class LCPError(RuntimeError):
    """Raised for a non-OK status; the reference raises ``error(...)`` there."""

    def __init__(self, status, message):
        super().__init__("%s (status %d)" % (message, status))
        self.status = status


class lcp_pao(ctypes.Structure):
    _fields_ = [("max_l", ctypes.c_int32), ("num_basis", ctypes.c_int32 * 4), ("num_mesh", ctypes.c_int32),
                ("rv", ctypes.POINTER(ctypes.c_double)), ("rwf", ctypes.POINTER(ctypes.c_double))]


class lcp_radial(ctypes.Structure):
    _fields_ = [("num_mesh", ctypes.c_int32), ("xv", ctypes.POINTER(ctypes.c_double)),
                ("rv", ctypes.POINTER(ctypes.c_double)), ("yv", ctypes.POINTER(ctypes.c_double))]


class lcp_ucell_info(ctypes.Structure):
    _fields_ = [("cpycell", ctypes.c_int32), ("natom", ctypes.c_int32), ("nloop", ctypes.c_int32),
                ("ncell", ctypes.c_int32), ("ngrid", ctypes.c_int32 * 3), ("max_numorbs", ctypes.c_int32),
                ("total_hsize", ctypes.c_int64), ("sum_gridn", ctypes.c_int64), ("sum_numolg", ctypes.c_int64),
                ("n_unique", ctypes.c_int64), ("gridvol", ctypes.c_double)]


if not os.path.exists(LIB_PATH):
    raise ImportError("liblcpgrid.so is not built (run `python -m lcpgrid.build` in lcpaodft.jl_gb300/): "
                      + LIB_PATH)

lib = ctypes.CDLL(LIB_PATH)

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_dbl = ctypes.c_double
_pd = ctypes.POINTER(ctypes.c_double)
_pi32 = ctypes.POINTER(ctypes.c_int32)
_ppd = ctypes.POINTER(ctypes.POINTER(ctypes.c_double))

_SIGS = {
    "lcp_last_error": ([], ctypes.c_char_p),
    "lcp_version": ([], ctypes.c_char_p),
    "lcp_ucell_create": ([_i32, _pd, _i32, _pi32, _pd, _pd, _pi32, _pd, _pi32, ctypes.POINTER(_vp)], _i32),
    "lcp_ucell_create_device": ([_vp, _i32, _pd, _i32, _pi32, _pd, _pd, _pi32, _pd, _pi32, ctypes.POINTER(_vp)],
                                _i32),
    "lcp_set_adenpcc_grid": ([_vp, _vp, _i32, _pd, _pd, _i32, ctypes.POINTER(lcp_radial),
                              ctypes.POINTER(lcp_radial), _pd, _pd, _ppd], _i32),
    "lcp_ucell_destroy": ([_vp], None),
    "lcp_ucell_get_info": ([_vp, ctypes.POINTER(lcp_ucell_info)], _i32),
    "lcp_ucell_get_int": ([_vp, _i32, _i64, _pi32, _i64], _i32),
    "lcp_ucell_get_atv": ([_vp, _pd], _i32),
    "lcp_ucell_get_bricks": ([_vp, ctypes.POINTER(ctypes.c_int64)], _i32),
    "lcp_calc_ngrid": ([_dbl, _pd, _pi32], _i32),
    "lcp_ctx_create": ([_i32, ctypes.POINTER(_vp)], _i32),
    "lcp_ctx_destroy": ([_vp], None),
    "lcp_ctx_set_stream": ([_vp, _vp], _i32),
    "lcp_ctx_set_precision": ([_vp, _i32], _i32),
    "lcp_ctx_synchronize": ([_vp], _i32),
    "lcp_ctx_launch_count": ([_vp], _i64),
    "lcp_set_orbitals_grid": ([_vp, _vp, _i32, ctypes.POINTER(lcp_pao), _i32, ctypes.POINTER(_vp)], _i32),
    "lcp_orbs_destroy": ([_vp], None),
    "lcp_orbs_download": ([_vp, _vp, _i32, _i32, _pd, _i64], _i32),
    "lcp_set_density_grid": ([_vp, _vp, _vp, _i32, _ppd, _ppd], _i32),
    "lcp_set_density_grid_noalloc": ([_vp, _vp, _vp, _i32, _ppd, _ppd], _i32),
    "lcp_device_alloc_count": ([ctypes.POINTER(_i64)], _i32),
    "lcp_ctx_set_fault_test": ([_vp, ctypes.c_uint32, _i32], _i32),
    "lcp_ctx_set_xc_arithmetic": ([_vp, _i32], _i32),
    "lcp_ctx_set_step_graphs": ([_vp, _i32], _i32),
    "lcp_bounds_check_status": ([_vp, ctypes.POINTER(_i64)], _i32),
    "lcp_orbs_timings": ([_vp, _pd], _i32),
    "lcp_solve_poisson": ([_vp, _pi32, _pd, _i32, _ppd, _pd, _pd], _i32),
    "lcp_solve_poisson_xyz": ([_vp, _pi32, _pd, _pd, _pd], _i32),
    "lcp_set_xc_grid": ([_vp, _i32, _i32, _i64, _pd, _ppd, _ppd], _i32),
    "lcp_diagonalize_nc_density": ([_vp, _i64, _ppd], _i32),
    "lcp_calc_diff_coef": ([_pd, _pd], _i32),
    "lcp_set_xc_grid_gga": ([_vp, _i32, _pi32, _pd, _pd, _ppd, _ppd, _ppd, _ppd], _i32),
    "lcp_calc_exc1_grid": ([_vp, _i32, _i32, _pi32, _pd, _dbl, _pd, _pd, _ppd, _pd], _i32),
    "lcp_set_vpot_grid": ([_vp, _i32, _i64, _pd, _ppd, _pd, _ppd], _i32),
    "lcp_calc_matrix_elements": ([_vp, _vp, _vp, _i32, _ppd, _ppd], _i32),
    "lcp_calc_eh1": ([_vp, _i32, _i64, _dbl, _pd, _ppd, _pd, _pd], _i32),
    "lcp_calc_exc1": ([_vp, _i32, _i32, _i64, _dbl, _pd, _pd, _ppd, _pd], _i32),
    "lcp_job_create": ([_vp, _vp, _vp, _i32, _i32, _pd, _pd, _pd, ctypes.POINTER(_vp)], _i32),
    "lcp_job_destroy": ([_vp], None),
    "lcp_job_set_dm": ([_vp, _vp, _ppd], _i32),
    "lcp_job_step": ([_vp, _vp], _i32),
    "lcp_job_step_timed": ([_vp, _vp, _pd], _i32),
    "lcp_job_energies": ([_vp, _vp, _pd], _i32),
    "lcp_job_energies_async": ([_vp, _vp, _pd], _i32),
    "lcp_job_footprint": ([_vp, ctypes.POINTER(_i64)], _i32),
    "lcp_job_prepare": ([_vp, _vp], _i32),
    "lcp_ctx_check_status": ([_vp], _i32),
    "lcp_server_create": ([_i32, _i32, _i32, _i64, ctypes.POINTER(_vp)], _i32),
    "lcp_server_destroy": ([_vp], None),
    "lcp_server_add": ([_vp, _vp, _i32, _i64, ctypes.POINTER(_i32)], _i32),
    "lcp_server_remove": ([_vp, _i32], _i32),
    "lcp_server_submit": ([_vp, _i32, _ppd, ctypes.c_uint64], _i32),
    "lcp_server_poll": ([_vp, _i32, _i32, ctypes.POINTER(ctypes.c_uint64), _pd, _pd, ctypes.POINTER(_i32)], _i32),
    "lcp_server_stats": ([_vp, ctypes.POINTER(_i64)], _i32),
    "lcp_server_state": ([_vp, _i32, ctypes.POINTER(_i32)], _i32),
    "lcp_server_set_max_batch": ([_vp, _i32], _i32),
    "lcp_server_batch_stats": ([_vp, ctypes.POINTER(_i64)], _i32),
    "lcp_calc_force3": ([_vp, _vp, _vp, _i32, _ppd, _ppd, _pd], _i32),
    "lcp_brick_shape_candidates": ([_vp, _i32, ctypes.POINTER(_i32), _pd, ctypes.POINTER(_i32)], _i32),
    "lcp_orbs_set_brick_shape": ([_vp, _vp, ctypes.POINTER(_i32)], _i32),
    "lcp_orbs_get_brick_shape": ([_vp, _vp, ctypes.POINTER(_i32)], _i32),
    "lcp_orbs_autotune_bricks": ([_vp, _vp, _i32, ctypes.POINTER(_i32), _pd], _i32),
    "lcp_orbs_release_fp64": ([_vp, _vp], _i32),
    "lcp_batch_create": ([_vp, _i32, ctypes.POINTER(_vp), _i64, ctypes.POINTER(_vp)], _i32),
    "lcp_batch_destroy": ([_vp], None),
    "lcp_batch_step": ([_vp, _vp, _i32], _i32),
    "lcp_batch_check_status": ([_vp, _vp], _i32),
    "lcp_batch_step_timed": ([_vp, _vp, _pd], _i32),
    "lcp_batch_energies": ([_vp, _vp, _pd], _i32),
    "lcp_batch_info": ([_vp, ctypes.POINTER(_i64)], _i32),
    "lcp_job_get_density": ([_vp, _vp, _ppd], _i32),
    "lcp_job_get_hks": ([_vp, _vp, _ppd], _i32),
    "lcp_job_get_vpot": ([_vp, _vp, _ppd], _i32),
    "lcp_probe_fp64_tflops": ([_vp, _pd], _i32),
    "lcp_tc_selftest": ([_vp, _i32, _i32, _i32, _i32, _i32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
                        _i32),
    "lcp_xc_selftest": ([_vp, _i32, _i32, _i64, _pd, _pd, _pd, _pd], _i32),
    "lcp_job_tc_kernel_ms": ([_vp, _vp, _pd], _i32),
}

for _name, (_args, _res) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.argtypes = _args
    _f.restype = _res


def exported_symbols():
    """Names of the C-ABI entry points this binding expects."""
    return sorted(_SIGS)


def check(status):
    if status != LCP_OK:
        msg = lib.lcp_last_error()
        raise LCPError(status, msg.decode() if msg else "lcpgrid error")


def dptr(a):
    """double* of a C-contiguous float64 numpy array (or NULL for None)."""
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_pd)


def iptr(a):
    if a.dtype != np.int32 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("expected a C-contiguous int32 array")
    return a.ctypes.data_as(_pi32)


def dptrs(arrays):
    """double* const* over a list of float64 arrays (kept alive by the caller)."""
    arr = (ctypes.POINTER(ctypes.c_double) * len(arrays))()
    for k, a in enumerate(arrays):
        arr[k] = dptr(a)
    return ctypes.cast(arr, _ppd), arr
