"""GPU parity for GGA-PBE (the gradient stencil, the PBE functional, the
divergence term, the energy and the device-resident step) through the C ABI
against the oracle.

Tolerances (FP64): xc grids, gradients and dE/d(grad rho) within 1e-11 of the
grid's largest magnitude, energies rel 1e-11.  The kernels evaluate the same
expressions as the oracle with shared reciprocals, cbrt for the reference's
truncated 1/3 power (a relative change of at most |ln rho| * 3.3e-16) and
log1p for log(1 + f4), so they agree to rounding (~1e-14)."""
import numpy as np
import pytest

import lcpgrid as L
from helpers import FE_LAT, FIX_LAT, aden_tables, golden, oracle_pao, product_pao, si2_cell
from oracle import lcp_oracle as O

pytestmark = pytest.mark.gpu

SKEW = np.array([[4.2, 0.3, 0.1], [0.5, 3.9, -0.2], [0.2, 0.4, 4.4]])
NG = (12, 10, 14)
TOL = 1e-11


@pytest.fixture(scope="module")
def ctx():
    return L.Context(0)


def smooth_fields(ng, nspin, seed):
    rng = np.random.default_rng(seed)
    n1, n2, n3 = ng
    i, j, k = np.meshgrid(np.arange(n1) / n1, np.arange(n2) / n2, np.arange(n3) / n3, indexing="ij")

    def smooth(a0):
        v = a0 * np.ones(ng)
        for _ in range(4):
            q = rng.integers(-2, 3, size=3)
            v = v + rng.uniform(0.05, 0.25) * a0 * np.cos(2 * np.pi * (q[0] * i + q[1] * j + q[2] * k) + rng.uniform(0, 6))
        return v.ravel()

    pcc = smooth(0.01)
    rho = [smooth(0.05), smooth(0.03)][:nspin]
    for r in rho:
        r[:7] = 0.0  # an empty region: the reference's den_min masks
    return pcc, rho


def close(got, want, tol=TOL):
    scale = max(np.max(np.abs(want)), 1e-300)
    assert np.max(np.abs(np.asarray(got) - want)) <= tol * scale, np.max(np.abs(np.asarray(got) - want)) / scale


def test_diff_coef_matches_oracle():
    for lat, ng in ((SKEW, NG), (FIX_LAT, (3, 3, 3)), (FE_LAT, (24, 24, 24))):
        gl = O.glatvecs_of(lat, ng)
        dc = np.array(L.Calc_Diff_Coef(gl))
        close(dc, O.calc_diff_coef(gl), 1e-12)


@pytest.mark.parametrize("spin", ["off", "on", "nc"])
def test_set_xc_grid_gga_vs_oracle(ctx, spin):
    ns = 1 if spin == "off" else 2
    pcc, rho = smooth_fields(NG, ns, seed={"off": 1, "on": 2, "nc": 3}[spin])
    nn = int(np.prod(NG))
    if spin == "nc":
        rng = np.random.default_rng(5)
        rho = rho + [rng.uniform(0, np.pi, nn), rng.uniform(-np.pi, np.pi, nn)]
    gl = O.glatvecs_of(SKEW, NG)
    xf = L.XC_Func("GGA-PBE", spin, {"off": 1, "on": 2, "nc": 4}[spin], NG, gl)
    L.Set_XC_Grid(xf, pcc, rho, ctx=ctx)
    vref, dref, eref = O.set_xc_grid_gga(spin, NG, pcc, rho, O.calc_diff_coef(gl))
    for c in range(len(vref)):
        close(xf.Vxc_Grid[c], vref[c])
    for s in range(ns):
        for a in range(3):
            close(xf.dDensity_Grid[s][a], dref[s][a])
            close(xf.dEXC_dGD[s][a], eref[s][a])
    # the masked points: no gradient, no potential
    assert np.all(xf.Vxc_Grid[0][:7] == 0.0) and np.all(xf.dDensity_Grid[0][0][:7] == 0.0)


@pytest.mark.parametrize("name,lat,spin", [("Set_AdenPCC_Grid Si GGA-PBE", FIX_LAT, "off"),
                                           ("Set_AdenPCC_Grid BCC_Fe GGA-PBE", FE_LAT, "on")])
def test_reference_gga_fixtures(ctx, name, lat, spin):
    """The inputs of the reference's GGA Set_XC_Grid! test sets
    (test/test_Set_XC_Grid.jl:37-76, 110-148): its own Set_AdenPCC_Grid output
    on the 3x3x3 Si and BCC Fe cells."""
    rec = golden()["adenpcc"][name]
    rho = [np.array(r) for r in rec["Density_Grid"]]
    pcc = np.array(rec["PCCDensity_Grid"])
    ng = (3, 3, 3)
    gl = O.glatvecs_of(lat, ng)
    xf = L.XC_Func("GGA-PBE", spin, len(rho), ng, gl)
    L.Set_XC_Grid(xf, pcc, rho, ctx=ctx)
    vref, dref, eref = O.set_xc_grid_gga(spin, ng, pcc, rho, O.calc_diff_coef(gl))
    for c in range(len(vref)):
        close(xf.Vxc_Grid[c], vref[c])
        close(xf.dEXC_dGD[c][0], eref[c][0])


@pytest.mark.parametrize("spin", ["off", "on"])
def test_calc_exc1_gga_vs_oracle(ctx, spin):
    ns = 1 if spin == "off" else 2
    pcc, rho = smooth_fields(NG, ns, seed=7)
    ad = 0.5 * (rho[0] + rho[-1])
    gv = abs(np.linalg.det(SKEW)) / np.prod(NG)
    grid = type("G", (), {"GridVol": gv, "Ngrid": NG, "Latvecs": SKEW})()
    got = L.Calc_EXC1(spin, "GGA_PBE", grid, ad, pcc, rho, ctx=ctx)
    want = O.calc_exc1(spin, "GGA_PBE", gv, ad, pcc, rho, ngrid=NG, latvecs=SKEW)
    np.testing.assert_allclose(got[:ns], want[:ns], rtol=1e-11)


@pytest.fixture(scope="module")
def si2(ctx):
    lat, pos, ng = si2_cell()
    u = L.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13])
    uo = O.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], total_numorbs=[13, 13])
    orbs = L.Set_Orbitals_Grid([product_pao()], u, ctx=ctx)
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
        M *= trace / nspin / np.trace(M)
        dm = np.zeros(u.Total_Hsize)
        for p, (a, b) in enumerate(zip(u.MPI_atom, u.MPI_natn)):
            blk = M[off[a - 1]:off[a], off[b - 1]:off[b]]
            dm[u.block_offset[p]:u.block_offset[p] + blk.size] = blk.reshape(-1)
        out.append(dm)
    return out


@pytest.mark.parametrize("spin", ["off", "on"])
def test_grid_step_job_gga_vs_oracle(ctx, si2, spin):
    """One FP64 device-resident grid step with GGA-PBE on the Si2 cell, with
    the PBE pseudopotential's partial-core density and a V_na field."""
    u, uo, orbs, oo = si2
    ns = 1 if spin == "off" else 2
    pt, vt = aden_tables("Si7.0", "Si_PBE19", 4.0)
    init = [[2., 2.], [2., 2.]] if spin == "off" else [[2.2, 1.8], [2.1, 1.9]]
    ad, pcc, _ = O.set_adenpcc_grid(spin, init, [[0, 0, 0, 0]] * 2, [pt], [vt], uo)
    vna = np.random.default_rng(8).normal(scale=0.1, size=u.NN)
    dm = psd_dm(u, 31 + ns, ns)
    job = L.GridStepJob(u, orbs, spin, "GGA_PBE", ad, pcc, vna)
    job.set_dm(dm)
    job.step()
    e = job.energies()
    rho = O.set_density_grid(spin, uo, oo, dm)
    dvh = O.solve_poisson(spin, uo, rho, ad)
    gl = O.glatvecs_of(uo.Latvecs, uo.Ngrid)
    vxc, _, _ = O.set_xc_grid_gga(spin, uo.Ngrid, pcc, rho, O.calc_diff_coef(gl))
    vp = O.set_vpot_grid(spin, dvh, vxc, vna)
    H = O.calc_matrix_elements(uo, oo, vp, ns)
    eh1 = O.calc_eh1(spin, uo.GridVol, ad, rho, dvh)
    exc = O.calc_exc1(spin, "GGA_PBE", uo.GridVol, ad, pcc, rho, ngrid=uo.Ngrid, latvecs=uo.Latvecs)
    eg = O.grid_energy(spin, uo, dm, H, eh1, exc)
    for s in range(ns):
        close(job.vpot()[s], vp[s])
        close(job.hks()[s], H[s])
    assert e[0] == pytest.approx(eh1, rel=1e-11)
    assert e[1] == pytest.approx(exc[0], rel=1e-11)
    if spin == "on":
        assert e[2] == pytest.approx(exc[1], rel=1e-11)
    assert e[4] == pytest.approx(eg, abs=1e-9)


def test_gga_split_bf16_energy(ctx, si2):
    """The split-BF16 step with GGA-PBE: energy within 1 uHa/atom of FP64."""
    u, uo, orbs, oo = si2
    pt, vt = aden_tables("Si7.0", "Si_PBE19", 4.0)
    ad, pcc, _ = O.set_adenpcc_grid("off", [[2., 2.], [2., 2.]], [[0, 0, 0, 0]] * 2, [pt], [vt], uo)
    dm = psd_dm(u, 17)
    E = {}
    for prec in ("fp64", "bf16x3"):
        ctx.set_precision(prec)
        try:
            job = L.GridStepJob(u, orbs, "off", "GGA_PBE", ad, pcc)
            job.set_dm(dm)
            job.step()
            E[prec] = job.energies()[4]
        finally:
            ctx.set_precision("fp64")
    assert abs(E["bf16x3"] - E["fp64"]) / u.Natom <= 1e-6, E


@pytest.mark.parametrize("spin", ["off", "on", "nc"])
def test_double_float_gga_matches_fp64(spin):
    """The precision forms' GGA-PBE (stencils and functional in double-float,
    FP64 sums; Context.set_xc_arithmetic) against
    the FP64 drop-in on the same inputs: potentials, gradients and
    dE/d(grad rho) within 1e-12 of each grid's largest magnitude (the
    double-float form is built for about 2^-44), the energy terms to 1e-12."""
    ns = 1 if spin == "off" else 2
    pcc, rho = smooth_fields(NG, ns, seed={"off": 11, "on": 12, "nc": 13}[spin])
    nn = int(np.prod(NG))
    if spin == "nc":
        rng = np.random.default_rng(15)
        rho = rho + [rng.uniform(0, np.pi, nn), rng.uniform(-np.pi, np.pi, nn)]
    gl = O.glatvecs_of(SKEW, NG)
    out = {}
    for df in (False, True):
        c = L.Context(0)
        c.set_xc_arithmetic(df)
        xf = L.XC_Func("GGA-PBE", spin, {"off": 1, "on": 2, "nc": 4}[spin], NG, gl)
        L.Set_XC_Grid(xf, pcc, rho, ctx=c)
        ad = np.zeros(nn)  # no atomic term: it nearly cancels the density term here
        gv = abs(np.linalg.det(SKEW)) / np.prod(NG)
        grid = type("G", (), {"GridVol": gv, "Ngrid": NG, "Latvecs": SKEW})()
        e = L.Calc_EXC1("off" if spin == "off" else "on", "GGA_PBE", grid, ad, pcc, rho[:ns], ctx=c)
        out[df] = (xf, e)
    (x64, e64), (xdf, edf) = out[False], out[True]
    for cch in range(len(x64.Vxc_Grid)):
        close(xdf.Vxc_Grid[cch], x64.Vxc_Grid[cch], 1e-12)
    for s in range(ns):
        for a in range(3):
            close(xdf.dDensity_Grid[s][a], x64.dDensity_Grid[s][a], 1e-12)
            close(xdf.dEXC_dGD[s][a], x64.dEXC_dGD[s][a], 1e-12)
    np.testing.assert_allclose(edf[:ns], e64[:ns], rtol=1e-12)
    assert not np.array_equal(xdf.Vxc_Grid[0], x64.Vxc_Grid[0])  # the other arithmetic did run
