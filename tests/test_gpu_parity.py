"""GPU parity: every step of the grid path through the C ABI against the
oracle and the reference's golden vectors.

Tolerances (FP64 drop-in): orbital tables 1e-13 absolute; density 1e-8
e/bohr^3 (we expect ~1e-15); grid H 1e-7 Ha (expect ~1e-14); Poisson and xc
grids rtol 1.5e-8 against the reference's golden values and 1e-12 against
the oracle; energies 1e-10 Ha."""
import numpy as np
import pytest

import lcpgrid as L
from helpers import FE_LAT, FIX_LAT, FIX_POS, aden_tables, golden, oracle_pao, product_pao, si2_cell
from oracle import lcp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return L.Context(0)


@pytest.fixture(scope="module")
def fix(ctx):
    u = L.UCell(1, FIX_LAT, 2, [1, 1], FIX_POS, [7.0, 7.0], (3, 3, 3), [0, 0, 0], Total_NumOrbs=[13, 13])
    uo = O.UCell(1, FIX_LAT, 2, [1, 1], FIX_POS, [7.0, 7.0], (3, 3, 3), [0, 0, 0], total_numorbs=[13, 13])
    orbs = L.Set_dOrbitals_Grid([product_pao()], u, ctx=ctx)
    return u, uo, orbs


@pytest.fixture(scope="module")
def si2(ctx):
    lat, pos, ng = si2_cell()
    u = L.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13])
    uo = O.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], total_numorbs=[13, 13])
    orbs = L.Set_dOrbitals_Grid([product_pao()], u, ctx=ctx)
    oo = O.set_orbitals_grid([oracle_pao()], uo)
    return u, uo, orbs, oo


def psd_dm(u, seed, nspin=1, trace=8.0):
    rng = np.random.default_rng(seed)
    no = np.asarray(u.Total_NumOrbs)
    off = np.concatenate([[0], np.cumsum(no)])
    out = []
    for _ in range(nspin):
        C = rng.normal(size=(off[-1], 6))
        M = C @ C.T
        M *= trace / np.trace(M)
        dm = np.zeros(u.Total_Hsize)
        for p, (a, b) in enumerate(zip(u.MPI_atom, u.MPI_natn)):
            blk = M[off[a - 1]:off[a], off[b - 1]:off[b]]
            dm[u.block_offset[p]:u.block_offset[p] + blk.size] = blk.reshape(-1)
        out.append(dm)
    return out


def test_orbitals_golden(fix):
    u, uo, orbs = fix
    for key, ref in golden()["orbs_si_3x3x3"].items():
        a, o = (int(x) - 1 for x in key.split("_"))
        np.testing.assert_allclose(orbs.data(a)[o], ref, rtol=1.5e-8, atol=1e-15)


def test_orbitals_and_gradients_vs_oracle(si2):
    u, uo, orbs, oo = si2
    dref = O.set_dorbitals_grid([oracle_pao()], uo)
    for a in range(2):
        np.testing.assert_allclose(orbs.data(a), oo[a], rtol=0, atol=1e-13)
        for k in range(3):
            np.testing.assert_allclose(orbs.data(a, k + 1), dref[k][a], rtol=0, atol=1e-12)


def test_gradient_tables_fixture(fix):
    """The 3x3x3 fixture has a grid point on atom 1 (the 1e-13 shift branch)."""
    u, uo, orbs = fix
    dref = O.set_dorbitals_grid([oracle_pao()], uo)
    for a in range(2):
        for k in range(3):
            np.testing.assert_allclose(orbs.data(a, k + 1), dref[k][a], rtol=0, atol=1e-12)


def test_density_fp64(si2):
    u, uo, orbs, oo = si2
    dm = psd_dm(u, 11)
    rho = [np.zeros(u.NN)]
    L.Set_Density_Grid("off", u, orbs, dm, rho)
    ref = O.set_density_grid("off", uo, oo, dm)[0]
    assert np.max(np.abs(rho[0] - ref)) <= 1e-8
    assert np.max(np.abs(rho[0] - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_density_fixture_golden_geometry(fix):
    u, uo, orbs = fix
    oo = O.set_orbitals_grid([oracle_pao()], uo)
    dm = psd_dm(u, 5)
    rho = [np.zeros(u.NN)]
    L.Set_Density_Grid("off", u, orbs, dm, rho)
    ref = O.set_density_grid("off", uo, oo, dm)[0]
    np.testing.assert_allclose(rho[0], ref, rtol=0, atol=1e-12)


def test_hamiltonian_fp64(si2):
    u, uo, orbs, oo = si2
    rng = np.random.default_rng(4)
    V = rng.normal(size=u.NN)
    H = [np.zeros(u.Total_Hsize)]
    L.Calc_MatrixElements_dVH_Vxc_off(u, orbs, [V], H)
    ref = O.calc_matrix_elements(uo, oo, [V], 1)[0]
    assert np.max(np.abs(H[0] - ref)) <= 1e-7
    assert np.max(np.abs(H[0] - ref)) <= 1e-12


def test_spin_channels_on_and_nc(si2):
    u, uo, orbs, oo = si2
    for spin, n in (("on", 2), ("nc", 4)):
        dm = psd_dm(u, 20 + n, nspin=n)
        rho = [np.zeros(u.NN) for _ in range(n)]
        L.Set_Density_Grid(spin, u, orbs, dm, rho)
        ref = O.set_density_grid(spin, uo, oo, dm)
        for c in range(n):
            np.testing.assert_allclose(rho[c], ref[c], rtol=0, atol=1e-12)
        rng = np.random.default_rng(n)
        V = [rng.normal(size=u.NN) for _ in range(n)]
        H = [np.zeros(u.Total_Hsize) for _ in range(n)]
        getattr(L, "Calc_MatrixElements_dVH_Vxc_" + spin)(u, orbs, V, H)
        ref = O.calc_matrix_elements(uo, oo, V, n)
        for c in range(n):
            np.testing.assert_allclose(H[c], ref[c], rtol=0, atol=1e-12)


def test_poisson_golden_and_oracle(ctx):
    P = golden()["poisson_si_3x3x3"]
    rec = 2 * np.pi * np.linalg.inv(FIX_LAT.T)
    out = np.zeros(27)
    L.Solve_Poisson_xyz((3, 3, 3), rec, np.array(P["density_xyz"]), out, ctx=ctx)
    np.testing.assert_allclose(out, P["dVHart_Grid"], rtol=1.5e-8, atol=1e-15)
    rng = np.random.default_rng(0)
    for ng in ((24, 24, 24), (15, 14, 17), (9, 10, 11)):
        lat = FIX_LAT * 1.3
        rec = 2 * np.pi * np.linalg.inv(lat.T)
        src = rng.normal(size=int(np.prod(ng)))
        out = np.zeros(src.size)
        L.Solve_Poisson_xyz(ng, rec, src, out, ctx=ctx)
        ref = O.solve_poisson_xyz(ng, rec, src)
        np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * np.max(np.abs(ref)))
    # Solve_Poisson! with SpinPol: 2rho - 2rho_a and rho_up + rho_dn - 2rho_a
    ng = (12, 12, 12)
    mix = L.Rhor_Mixing(ng, FIX_LAT, ctx=ctx)  # the solve runs on the mixing object's context
    r = [rng.uniform(size=1728), rng.uniform(size=1728)]
    ad = rng.uniform(size=1728)
    for spin in ("off", "on"):
        out = np.zeros(1728)
        L.Solve_Poisson(spin, mix, r, ad, out)  # the reference's five arguments
        ref = O.solve_poisson_xyz(ng, mix.Recvecs, O.set_density_xyz(spin, ng, r, ad))
        np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * np.max(np.abs(ref)))


def test_xc_golden(ctx, fix):
    u, uo, orbs = fix
    g = golden()
    pt, vt = aden_tables("Si7.0", "Si_CA19", 4.0)
    a, p, d = O.set_adenpcc_grid("off", [[2., 2.], [2., 2.]], [[0, 0, 0, 0]] * 2, [pt], [vt], uo)
    xf = L.XC_Func("LDA", "off", 1, (3, 3, 3), ctx=ctx)
    L.Set_XC_Grid(xf, p, d)  # the reference's three arguments
    np.testing.assert_allclose(xf.Vxc_Grid[0], g["xc_grid"]["XC_PBE Si LDA"][0], rtol=1.5e-8)
    ufe = O.UCell(2, FE_LAT, 1, [1], [[0, 0, 0]], [6.0], (3, 3, 3), [0, 0, 0])
    pt, vt = aden_tables("Fe6.0H", "Fe_CA19H", 16.0)
    a, p, d = O.set_adenpcc_grid("on", [[8., 6.]], [[0, 0, 0, 0]], [pt], [vt], ufe)
    xf = L.XC_Func("LSDA", "on", 2, (3, 3, 3))
    L.Set_XC_Grid(xf, p, d, ctx=ctx)
    for s in range(2):
        np.testing.assert_allclose(xf.Vxc_Grid[s], g["xc_grid"]["XC_PBE BCC_Fe LSDA"][s], rtol=1.5e-8)


def test_xc_vpot_energies_vs_oracle(ctx):
    rng = np.random.default_rng(9)
    nn = 4096
    rho = [rng.uniform(0, 0.3, nn), rng.uniform(0, 0.3, nn)]
    rho[0][:5] = 0.0  # below the 1e-15 cut
    pcc = rng.uniform(0, 0.01, nn)
    ad = rng.uniform(0, 0.2, nn)
    dvh = rng.normal(size=nn)
    vna = rng.normal(size=nn)
    for spin, xc in (("off", "LDA"), ("on", "LSDA")):
        n = 1 if spin == "off" else 2
        xf = L.XC_Func(xc, spin, n, (16, 16, 16))
        L.Set_XC_Grid(xf, pcc, rho, ctx=ctx)
        ref = O.set_xc_grid(xc, spin, pcc, rho)
        for c in range(n):
            np.testing.assert_allclose(xf.Vxc_Grid[c], ref[c], rtol=1e-13, atol=1e-15)
        vp = [np.zeros(nn) for _ in range(n)]
        L.Set_Vpot_Grid(xf, dvh, vp, Vna_Grid=vna, ctx=ctx)
        vref = O.set_vpot_grid(spin, dvh, ref, vna)
        for c in range(n):
            np.testing.assert_allclose(vp[c], vref[c], rtol=1e-13, atol=1e-14)
        eh = L.Calc_EH1(spin, 0.01, ad, rho, dvh, ctx=ctx)
        assert eh == pytest.approx(O.calc_eh1(spin, 0.01, ad, rho, dvh), rel=1e-12)
        ex = L.Calc_EXC1(spin, xc, type("G", (), {"GridVol": 0.01})(), ad, pcc, rho, ctx=ctx)
        exr = O.calc_exc1(spin, xc, 0.01, ad, pcc, rho)
        np.testing.assert_allclose(ex[:n], exr[:n], rtol=1e-12)


def test_nc_xc_rotation(ctx):
    rng = np.random.default_rng(2)
    nn = 512
    rho = [rng.uniform(0, 0.2, nn), rng.uniform(0, 0.2, nn), rng.uniform(0, 3, nn), rng.uniform(-3, 3, nn)]
    pcc = rng.uniform(0, 0.01, nn)
    xf = L.XC_Func("LSDA", "nc", 4, (8, 8, 8))
    L.Set_XC_Grid(xf, pcc, rho, ctx=ctx)
    ref = O.set_xc_grid("LSDA", "nc", pcc, rho)
    for c in range(4):
        np.testing.assert_allclose(xf.Vxc_Grid[c], ref[c], rtol=1e-12, atol=1e-15)


def test_grid_step_job_vs_oracle(ctx, si2):
    """One full FP64 grid step on the Si2 24^3 cell with the reference's own
    atomic and partial-core densities (Set_AdenPCC_Grid) and a V_na field."""
    u, uo, orbs, oo = si2
    pt, vt = aden_tables("Si7.0", "Si_CA19", 4.0)
    ad, pcc, _ = O.set_adenpcc_grid("off", [[2., 2.], [2., 2.]], [[0, 0, 0, 0]] * 2, [pt], [vt], uo)
    vna = np.random.default_rng(8).normal(scale=0.1, size=u.NN)
    dm = psd_dm(u, 31)
    job = L.GridStepJob(u, orbs, "off", "LDA", ad, pcc, vna)
    job.set_dm(dm)
    job.step()
    e = job.energies()
    rho = O.set_density_grid("off", uo, oo, dm)
    dvh = O.solve_poisson("off", uo, rho, ad)
    vxc = O.set_xc_grid("LDA", "off", pcc, rho)
    vp = O.set_vpot_grid("off", dvh, vxc, vna)
    H = O.calc_matrix_elements(uo, oo, vp, 1)
    eh1 = O.calc_eh1("off", uo.GridVol, ad, rho, dvh)
    exc = O.calc_exc1("off", "LDA", uo.GridVol, ad, pcc, rho)
    eg = O.grid_energy("off", uo, dm, H, eh1, exc)
    np.testing.assert_allclose(job.density()[0], rho[0], rtol=0, atol=1e-12)
    np.testing.assert_allclose(job.vpot()[0], vp[0], rtol=0, atol=1e-11)
    np.testing.assert_allclose(job.hks()[0], H[0], rtol=0, atol=1e-11)
    assert e[0] == pytest.approx(eh1, rel=1e-11)
    assert e[1] == pytest.approx(exc[0], rel=1e-11)
    assert e[4] == pytest.approx(eg, abs=1e-9)


def test_fp32_form_error_bounds(ctx, si2):
    u, uo, orbs, oo = si2
    dm = psd_dm(u, 11)
    V = np.random.default_rng(4).normal(size=u.NN)
    ref_rho = O.set_density_grid("off", uo, oo, dm)[0]
    ref_h = O.calc_matrix_elements(uo, oo, [V], 1)[0]
    ctx.set_precision("fp32")
    try:
        rho = [np.zeros(u.NN)]
        L.Set_Density_Grid("off", u, orbs, dm, rho)
        H = [np.zeros(u.Total_Hsize)]
        L.Calc_MatrixElements_dVH_Vxc_off(u, orbs, [V], H)
    finally:
        ctx.set_precision("fp64")
    assert np.max(np.abs(rho[0] - ref_rho)) <= 1e-5 * np.max(np.abs(ref_rho))
    assert np.max(np.abs(H[0] - ref_h)) <= 1e-5 * np.max(np.abs(ref_h))


def test_errors(ctx, fix, si2):
    u, uo, orbs = fix
    u2 = si2[0]
    with pytest.raises(L.LCPError):
        L.Set_Density_Grid("off", u2, orbs, [np.zeros(u2.Total_Hsize)], [np.zeros(u2.NN)])
    with pytest.raises(L.LCPError):
        L.Set_Density_Grid("bad", u, orbs, [np.zeros(u.Total_Hsize)], [np.zeros(u.NN)])
    with pytest.raises(L.LCPError):
        L.XC_Func("LDA", "on", 2, (3, 3, 3))
    with pytest.raises(L.LCPError):
        L.Set_Orbitals_Grid([product_pao("Si7.0", "s1p1")], u, ctx=ctx)  # basis does not match Total_NumOrbs
