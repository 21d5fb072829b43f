"""Grid force term (Force3_nospin / _spin / _nc, src/Force.jl:405-566) on the
GPU against the oracle, whose Force3 the finite-difference identity of
test_oracle_force.py pins.  FP64 drop-in: 1e-10 of the largest component."""
import numpy as np
import pytest

import lcpgrid as L
from helpers import oracle_pao, product_pao, si2_cell
from oracle import lcp_oracle as O
from test_gpu_parity import psd_dm

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def ctx():
    return L.Context(0)


def _si2(ctx):
    lat, pos, ng = si2_cell()
    pos = np.asarray(pos) + np.array([[0.0, 0.0, 0.0], [0.11, -0.05, 0.07]])  # off symmetry: forces are not zero
    u = L.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13])
    uo = O.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], total_numorbs=[13, 13])
    return u, uo, [product_pao()], [oracle_pao()]


def _check(F, Fref):
    assert np.max(np.abs(Fref)) > 1e-6
    np.testing.assert_allclose(F, Fref, rtol=0, atol=TOL * np.max(np.abs(Fref)))


@pytest.mark.parametrize("spin", ["off", "on", "nc"])
def test_force3_vs_oracle(ctx, spin):
    u, uo, paos, opaos = _si2(ctx)
    n = {"off": 1, "on": 2, "nc": 4}[spin]
    dm = psd_dm(u, 70 + n, nspin=n)
    rng = np.random.default_rng(80 + n)
    V = [rng.normal(size=u.NN) * 0.3 for _ in range(n)]
    orbs = L.Set_dOrbitals_Grid(paos, u, ctx=ctx)
    oo = O.set_orbitals_grid(opaos, uo)
    do = O.set_dorbitals_grid(opaos, uo)
    if spin == "off":
        F = L.Force3_nospin(paos, orbs, V, dm, u)
        Fref = O.calc_force3("off", uo, oo, do, V, dm)
    elif spin == "on":
        F = L.Force3_spin(paos, orbs, V, dm, u)
        Fref = O.calc_force3("on", uo, oo, do, V, dm)
    else:
        dvh = rng.normal(size=u.NN) * 0.1
        F = L.Force3_nc(paos, orbs, dvh, V, dm, u)
        Fref = O.calc_force3("nc", uo, oo, do, [dvh + V[0], dvh + V[1], V[2], V[3]], dm)
    _check(F, Fref)


def test_force3_mixed_basis_and_internal_tabulation(ctx):
    """18 / 13 / 4-orbital atoms (the 32-orbital kernel); Orbs_Grid without
    gradient tables makes the call tabulate them, as the reference does."""
    from lcpgrid.workloads import synthetic_species
    specs = [synthetic_species(11, max_l=2, num_basis=(2, 2, 2), rc=8.0),
             synthetic_species(12, max_l=2, num_basis=(2, 2, 1), rc=7.0),
             synthetic_species(13, max_l=1, num_basis=(1, 1), rc=6.0)]
    lat = np.diag([11.0, 10.0, 12.0])
    pos = np.array([[1.0, 2.0, 3.0], [5.5, 6.0, 8.5], [8.0, 1.5, 6.0]])
    args = (lat, 3, [1, 2, 3], pos, [8.0, 7.0, 6.0], (33, 30, 36), [0, 0, 0])
    u = L.UCell(1, *args, Total_NumOrbs=[18, 13, 4])
    uo = O.UCell(1, *args, total_numorbs=[18, 13, 4])
    opaos = [O.PAO(p.Spe_MaxL_Basis, p.Spe_Num_Basis, p.Spe_PAO_RV, p.Spe_PAO_RWF) for p in specs]
    dm = psd_dm(u, 91)
    V = [np.random.default_rng(92).normal(size=u.NN)]
    plain = L.Set_Orbitals_Grid(specs, u, ctx=ctx)
    F = L.Force3_nospin(specs, plain, V, dm, u)
    Fref = O.calc_force3("off", uo, O.set_orbitals_grid(opaos, uo), O.set_dorbitals_grid(opaos, uo), V, dm)
    _check(F, Fref)


def test_force3_needs_gradient_tables(ctx):
    from lcpgrid import _lib
    u, uo, paos, _ = _si2(ctx)
    plain = L.Set_Orbitals_Grid(paos, u, ctx=ctx)
    V = [np.zeros(u.NN)]
    dm = psd_dm(u, 3)
    vp, kv = _lib.dptrs(V)
    dp, kd = _lib.dptrs(dm)
    out = np.zeros((2, 3))
    with pytest.raises(L.LCPError):
        _lib.check(_lib.lib.lcp_calc_force3(ctx._h, u._h, plain._h, 0, vp, dp, _lib.dptr(out)))
