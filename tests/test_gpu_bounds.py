"""The check build (liblcpgrid_check.so): every index the pair and
tensor-core kernels gather with is tested on the device, and the first
violation is recorded in a device word instead of being accessed.  Run on the
reference's 3x3x3 Si fixture and the Si2 24^3 cell (FP64 and split-BF16
density and matrix elements), it must record no violation and give the
oracle's results.  It runs in a child process, which loads the check build
(LCPGRID_BOUNDS_CHECK=1)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r"""
import json, sys
import numpy as np
import lcpgrid as L
from lcpgrid import _lib
from helpers import FIX_LAT, FIX_POS, oracle_pao, product_pao, si2_cell
from oracle import lcp_oracle as O
from test_gpu_parity import psd_dm

assert _lib.LIB_PATH.endswith("liblcpgrid_check.so")
ctx = L.Context(0)
out = {}
lat, pos, ng = si2_cell()
for name, (lat_, pos_, ng_) in (("fixture_3x3x3", (FIX_LAT, FIX_POS, (3, 3, 3))), ("si2_24", (lat, pos, ng))):
    u = L.UCell(1, lat_, 2, [1, 1], pos_, [7.0, 7.0], ng_, [0, 0, 0], Total_NumOrbs=[13, 13], ctx=ctx)
    uo = O.UCell(1, lat_, 2, [1, 1], pos_, [7.0, 7.0], ng_, [0, 0, 0], total_numorbs=[13, 13])
    orbs = L.Set_Orbitals_Grid([product_pao()], u)
    oo = O.set_orbitals_grid([oracle_pao()], uo)
    dm = psd_dm(u, 17)
    V = np.random.default_rng(3).normal(size=u.NN)
    rho_ref = O.set_density_grid("off", uo, oo, dm)[0]
    h_ref = O.calc_matrix_elements(uo, oo, [V], 1)[0]
    for prec in ("fp64", "bf16x3"):
        ctx.set_precision(prec)
        rho = [np.zeros(u.NN)]
        L.Set_Density_Grid("off", u, orbs, dm, rho)
        H = [np.zeros(u.Total_Hsize)]
        L.Calc_MatrixElements_dVH_Vxc_off(u, orbs, [V], H)
        w = _lib.ctypes.c_int64()
        _lib.check(_lib.lib.lcp_bounds_check_status(ctx._h, _lib.ctypes.byref(w)))
        out["%s_%s" % (name, prec)] = {
            "word": int(w.value),
            "drho": float(np.max(np.abs(rho[0] - rho_ref)) / max(np.max(np.abs(rho_ref)), 1e-300)),
            "dH": float(np.max(np.abs(H[0] - h_ref)) / max(np.max(np.abs(h_ref)), 1e-300))}
    ctx.set_precision("fp64")
print("RESULT " + json.dumps(out))
"""


def test_check_build_records_no_violation():
    lib = os.path.join(ROOT, "lcpaodft.jl_gb300", "lcpgrid", "liblcpgrid_check.so")
    assert os.path.exists(lib), "build() makes the check build beside the library"
    env = dict(os.environ, LCPGRID_BOUNDS_CHECK="1")
    env["PYTHONPATH"] = os.pathsep.join([ROOT, os.path.join(ROOT, "lcpaodft.jl_gb300"), HERE,
                                         env.get("PYTHONPATH", "")])
    res = subprocess.run([sys.executable, "-c", CHILD], env=env, cwd=ROOT, capture_output=True, text=True,
                         timeout=900)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    line = [x for x in res.stdout.splitlines() if x.startswith("RESULT ")][-1]
    out = json.loads(line[len("RESULT "):])
    assert len(out) == 4
    for key, r in out.items():
        assert r["word"] == 0, (key, r)
        tol = 1e-12 if key.endswith("fp64") else 5e-6
        assert r["drho"] <= tol and r["dH"] <= tol, (key, r)


def test_normal_build_reports_no_checks():
    import lcpgrid as L
    from lcpgrid import _lib
    if _lib.LIB_PATH.endswith("liblcpgrid_check.so"):
        pytest.skip("this process loaded the check build")
    ctx = L.Context(0)
    w = _lib.ctypes.c_int64()
    with pytest.raises(L.LCPError) as e:
        _lib.check(_lib.lib.lcp_bounds_check_status(ctx._h, _lib.ctypes.byref(w)))
    assert e.value.status == _lib.LCP_ENOTSUP
