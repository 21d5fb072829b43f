"""Grid setup on the device: the sphere and overlap lists of a UCell built on
the GPU against the host build (bit-exact integer lists), and
Set_AdenPCC_Grid on the GPU against the reference's golden vectors
(test/test_Set_AdenPCC_Grid.jl) and the oracle.

Tolerances: lists identical; densities rtol 1.5e-8 against the golden values
(their printed precision) and 1e-13 of the largest value against the oracle
(the same sums in the same order; log/exp differ by an ulp)."""
from types import SimpleNamespace

import numpy as np
import pytest

import lcpgrid as L
from helpers import FE_LAT, FIX_LAT, FIX_POS, aden_tables, golden, si2_cell
from oracle import lcp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return L.Context(0)


def _cells():
    from lcpgrid.workloads import batch_pool, mx2_monolayer, si64_workload
    lat, pos, ng = si2_cell()
    out = [("si2_24", (1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], [13, 13])),
           ("si_fixture_3x3x3", (1, FIX_LAT, 2, [1, 1], FIX_POS, [7.0, 7.0], (3, 3, 3), [0, 0, 0], [13, 13])),
           ("fe_bcc_3x3x3", (2, FE_LAT, 1, [1], [[0, 0, 0]], [6.0], (3, 3, 3), [0, 0, 0], [13]))]
    for name, wl in (("si64_96", si64_workload()), ("mx2", mx2_monolayer())):
        out.append((name, (1, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"],
                           wl["origin"], wl["numorbs"])))
    for k, c in enumerate(batch_pool(4, seed=77, nmax=12, amax_ang=7.0)):
        out.append(("pool%d" % k, (1, c["latvecs"], c["natom"], c["atom2spe"], c["gxyz"], c["cut"], c["ngrid"],
                                   c["origin"], c["numorbs"])))
    return out


CELLS = _cells()


def _same_lists(uh, ud, max_pairs=None):
    for f in ("CpyCell", "Nloop", "ncell", "Total_Hsize", "sum_gridn", "sum_numolg", "n_unique"):
        assert getattr(uh, f) == getattr(ud, f), f
    for f in ("FNAN", "GridN_Atom", "MPI_atom", "MPI_natn", "MPI_ncn", "MPI_NumOLG"):
        np.testing.assert_array_equal(getattr(uh, f), getattr(ud, f), err_msg=f)
    for a, b in zip(uh.GridListAtom, ud.GridListAtom):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(uh.CellListAtom, ud.CellListAtom):
        np.testing.assert_array_equal(a, b)
    pairs = range(uh.Nloop)
    if max_pairs and uh.Nloop > max_pairs:
        pairs = np.random.default_rng(0).choice(uh.Nloop, size=max_pairs, replace=False)
    for p in pairs:
        g1h, g2h = uh.GListTAtoms(int(p))
        g1d, g2d = ud.GListTAtoms(int(p))
        np.testing.assert_array_equal(g1h, g1d)
        np.testing.assert_array_equal(g2h, g2d)


@pytest.mark.parametrize("name,args", CELLS, ids=[c[0] for c in CELLS])
def test_device_ucell_matches_host(ctx, name, args):
    uh = L.UCell(*args[:8], Total_NumOrbs=args[8])
    try:
        ud = L.UCell(*args[:8], Total_NumOrbs=args[8], device=True, ctx=ctx)
    except L.LCPError as e:
        # only cells whose boxes reach beyond the image cells the device
        # build indexes may be refused, and they say so
        assert e.status == L._lib.LCP_ENOTSUP and "CpyCell" in str(e), (name, e)
        assert name in ("si_fixture_3x3x3", "fe_bcc_3x3x3"), name
        return
    _same_lists(uh, ud, max_pairs=400)


def _species(pao_tag, vps_tag, core):
    (pxv, prv, pden), (vxv, vrv, vpcc) = aden_tables(pao_tag, vps_tag, core)
    pao = SimpleNamespace(Spe_PAO_XV=pxv, Spe_PAO_RV=prv, Spe_Atomic_Den=pden)
    pcc = SimpleNamespace(Spe_VPS_XV=vxv, Spe_VPS_RV=vrv, Spe_Atomic_PCC=vpcc)
    return pao, pcc


def test_adenpcc_golden(ctx):
    """The reference's own Set_AdenPCC_Grid test sets, on the GPU."""
    g = golden()["adenpcc"]
    u = L.UCell(1, FIX_LAT, 2, [1, 1], FIX_POS, [7.0, 7.0], (3, 3, 3), [0, 0, 0], Total_NumOrbs=[13, 13])
    for name, vps in (("Set_AdenPCC_Grid Si LDA", "Si_CA19"), ("Set_AdenPCC_Grid Si GGA-PBE", "Si_PBE19")):
        pao, pcc = _species("Si7.0", vps, 4.0)
        a, p, d = L.Set_AdenPCC_Grid("off", [[2., 2.], [2., 2.]], [[0, 0, 0, 0]] * 2, [pao], [pcc], u, ctx=ctx)
        ref = g[name]
        np.testing.assert_allclose(a, ref["ADensity_Grid"], rtol=1.5e-8)
        np.testing.assert_allclose(p, ref["PCCDensity_Grid"], rtol=1.5e-8)
        np.testing.assert_allclose(d[0], ref["Density_Grid"][0], rtol=1.5e-8)
    ufe = L.UCell(2, FE_LAT, 1, [1], [[0, 0, 0]], [6.0], (3, 3, 3), [0, 0, 0], Total_NumOrbs=[13])
    pao, pcc = _species("Fe6.0H", "Fe_PBE19H", 16.0)
    a, p, d = L.Set_AdenPCC_Grid("on", [[8., 6.]], [[0, 0, 0, 0]], [pao], [pcc], ufe, ctx=ctx)
    ref = g["Set_AdenPCC_Grid BCC_Fe GGA-PBE"]
    np.testing.assert_allclose(a, ref["ADensity_Grid"], rtol=1.5e-8)
    np.testing.assert_allclose(p, ref["PCCDensity_Grid"], rtol=1.5e-8)
    for s in range(2):
        np.testing.assert_allclose(d[s], ref["Density_Grid"][s], rtol=1.5e-8)


@pytest.mark.parametrize("spin", ["off", "on", "nc"])
def test_adenpcc_vs_oracle_on_device_ucell(ctx, spin):
    """Device UCell (Si2, 24^3) -> device Set_AdenPCC_Grid, against the oracle."""
    lat, pos, ng = si2_cell()
    u = L.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13], device=True, ctx=ctx)
    uo = O.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], total_numorbs=[13, 13])
    pao, pcc = _species("Si7.0", "Si_PBE19", 4.0)
    pt, vt = aden_tables("Si7.0", "Si_PBE19", 4.0)
    init = [[2.3, 1.7], [1.9, 2.1]]
    angle = [[0.7, 1.1, 0, 0], [2.0, -0.4, 0, 0]]
    a, p, d = L.Set_AdenPCC_Grid(spin, init, angle, [pao], [pcc], u, ctx=ctx)
    ar, pr, dr = O.set_adenpcc_grid(spin, init, angle, [pt], [vt], uo)
    for got, want in [(a, ar), (p, pr)] + list(zip(d, dr)):
        assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))


def test_adenpcc_two_species(ctx):
    """Two species (Si and Fe tables) on one cell, spin "on": each atom reads
    its own species' density and PCC tables."""
    lat, pos, ng = si2_cell()
    u = L.UCell(2, lat, 2, [1, 2], pos, [7.0, 6.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13], device=True, ctx=ctx)
    uo = O.UCell(2, lat, 2, [1, 2], pos, [7.0, 6.0], ng, [0, 0, 0], total_numorbs=[13, 13])
    sp = [_species("Si7.0", "Si_PBE19", 4.0), _species("Fe6.0H", "Fe_PBE19H", 16.0)]
    tabs = [aden_tables("Si7.0", "Si_PBE19", 4.0), aden_tables("Fe6.0H", "Fe_PBE19H", 16.0)]
    init = [[2.2, 1.8], [8.0, 6.0]]
    a, p, d = L.Set_AdenPCC_Grid("on", init, None, [x[0] for x in sp], [x[1] for x in sp], u, ctx=ctx)
    ar, pr, dr = O.set_adenpcc_grid("on", init, [[0, 0, 0, 0]] * 2, [t[0] for t in tabs], [t[1] for t in tabs], uo)
    for got, want in [(a, ar), (p, pr)] + list(zip(d, dr)):
        assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))
