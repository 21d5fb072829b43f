"""GPU parity for the non-collinear ("nc") channel set: the Euler-angle
transform diagonalize_nc_density! and the device-resident step on four
channels (density, diagonalization, Poisson, LSDA or GGA-PBE xc rotated into
four potentials, four-channel grid H, energies) against the oracle.

Tolerances (FP64): angles and densities of the transform 1e-13 absolute on
the same inputs (the kernel rounds every operation of xyz_to_spherical as the
reference does; acos/asin differ by at most an ulp or two); in the step,
Nup/Ndown 1e-12 absolute and the magnetization vector within 1e-11 of its
largest magnitude (the FP64 assembly-order difference of the density); potentials and H within 1e-11
of their largest magnitude, energies rel 1e-11."""
import numpy as np
import pytest

import lcpgrid as L
from helpers import aden_tables, oracle_pao, product_pao, si2_cell
from oracle import lcp_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return L.Context(0)


def close(got, want, tol=1e-11):
    scale = max(np.max(np.abs(want)), 1e-300)
    err = np.max(np.abs(np.asarray(got) - want))
    assert err <= tol * scale, err / scale


def test_diagonalize_nc_density_vs_oracle(ctx):
    rng = np.random.default_rng(12)
    n = 20000
    d = [rng.uniform(0, 0.3, n), rng.uniform(0, 0.3, n), rng.normal(0, 0.05, n), rng.normal(0, 0.05, n)]
    d[2][:50] = 0.0
    d[3][:50] = 0.0  # collinear: phi = 0
    d[0][50:60] = d[1][50:60]
    d[2][50:60] = 0.0
    d[3][50:60] = 0.0  # no spin: theta = pi/2, phi = 0
    d[2][60:70] = 1e-9  # nearly collinear: theta near the poles
    d[3][60:70] = 0.0
    d[2][70:80] = -0.02  # x < 0: phi = pi - asin
    ref = O.diagonalize_nc_density(d)
    got = [x.copy() for x in d]
    old = L.use_context(ctx)  # the module's context: the reference's one-argument call
    try:
        L.diagonalize_nc_density(got)
    finally:
        if old is not None:
            L.use_context(old)
    for c in range(4):
        np.testing.assert_allclose(got[c], ref[c], rtol=0, atol=1e-13)
    assert np.all(got[3][:50] == 0.0) and np.all(got[2][50:60] == 0.5 * np.pi)


@pytest.fixture(scope="module")
def si2(ctx):
    lat, pos, ng = si2_cell()
    u = L.UCell(4, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13])
    uo = O.UCell(4, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], total_numorbs=[13, 13])
    orbs = L.Set_Orbitals_Grid([product_pao()], u, ctx=ctx)
    oo = O.set_orbitals_grid([oracle_pao()], uo)
    return u, uo, orbs, oo


def nc_dm(u, seed, trace=8.0):
    """Four flat pair-block channels of a Hermitian 2x2-spinor density
    matrix: Re11, Re22, Re12, Im12 (Im12 antisymmetric in the orbitals)."""
    rng = np.random.default_rng(seed)
    no = np.asarray(u.Total_NumOrbs)
    off = np.concatenate([[0], np.cumsum(no)])
    n = off[-1]
    C = rng.normal(size=(2 * n, 8)) + 1j * rng.normal(size=(2 * n, 8))
    M = C @ C.conj().T
    M *= trace / np.trace(M).real
    mats = [M[:n, :n].real, M[n:, n:].real, M[:n, n:].real, M[:n, n:].imag]
    out = []
    for m in mats:
        dm = np.zeros(u.Total_Hsize)
        for p, (a, b) in enumerate(zip(u.MPI_atom, u.MPI_natn)):
            blk = m[off[a - 1]:off[a], off[b - 1]:off[b]]
            dm[u.block_offset[p]:u.block_offset[p] + blk.size] = blk.reshape(-1)
        out.append(dm)
    return out


def spin_direction(theta, phi):
    return np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)])


@pytest.mark.parametrize("xc", ["LSDA", "GGA_PBE"])
def test_grid_step_job_nc_vs_oracle(ctx, si2, xc):
    u, uo, orbs, oo = si2
    pt, vt = aden_tables("Si7.0", "Si_CA19" if xc == "LSDA" else "Si_PBE19", 4.0)
    ad, pcc, _ = O.set_adenpcc_grid("on", [[2.2, 1.8], [2.1, 1.9]], [[0, 0, 0, 0]] * 2, [pt], [vt], uo)
    vna = np.random.default_rng(3).normal(scale=0.1, size=u.NN)
    dm = nc_dm(u, 77)
    job = L.GridStepJob(u, orbs, "nc", xc, ad, pcc, vna)
    job.set_dm(dm)
    job.step()
    e = job.energies()
    rho4 = O.set_density_grid("nc", uo, oo, dm)
    rho = O.diagonalize_nc_density(rho4)
    dvh = O.solve_poisson("nc", uo, rho, ad)
    if xc == "LSDA":
        vxc = O.set_xc_grid("LSDA", "nc", pcc, rho)
        exc = O.calc_exc1("nc", "LSDA", uo.GridVol, ad, pcc, rho)
    else:
        gl = O.glatvecs_of(uo.Latvecs, uo.Ngrid)
        vxc, _, _ = O.set_xc_grid_gga("nc", uo.Ngrid, pcc, rho, O.calc_diff_coef(gl))
        exc = O.calc_exc1("nc", "GGA_PBE", uo.GridVol, ad, pcc, rho, ngrid=uo.Ngrid, latvecs=uo.Latvecs)
    vp = O.set_vpot_grid("nc", dvh, vxc, vna)
    H = O.calc_matrix_elements(uo, oo, vp, 4)
    eh1 = O.calc_eh1("nc", uo.GridVol, ad, rho, dvh)
    eg = O.grid_energy("nc", uo, dm, H, eh1, exc)
    dens = job.density()
    for c in range(2):
        np.testing.assert_allclose(dens[c], rho[c], rtol=0, atol=1e-12)
    # the angles through the magnetization (Nup - Ndown) * direction: acos/asin
    # amplify the last-bit differences of the assembled densities near
    # theta = 0, pi and phi = +-pi/2, and the direction of a small
    # magnetization is itself ill-conditioned; the magnetization is not
    close((dens[0] - dens[1]) * spin_direction(dens[2], dens[3]),
          (rho[0] - rho[1]) * spin_direction(rho[2], rho[3]), 1e-11)
    for c in range(4):
        close(job.vpot()[c], vp[c])
        close(job.hks()[c], H[c])
    assert e[0] == pytest.approx(eh1, rel=1e-11)
    assert e[1] == pytest.approx(exc[0], rel=1e-11)
    assert e[2] == pytest.approx(exc[1], rel=1e-11)
    assert e[4] == pytest.approx(eg, abs=1e-9)


def test_nc_split_bf16_energy_and_batch_rejects(ctx, si2):
    u, uo, orbs, oo = si2
    dm = nc_dm(u, 5)
    E = {}
    for prec in ("fp64", "bf16x3"):
        ctx.set_precision(prec)
        try:
            job = L.GridStepJob(u, orbs, "nc", "LSDA")
            job.set_dm(dm)
            job.step()
            E[prec] = job.energies()[4]
            if prec == "bf16x3":
                with pytest.raises(L.LCPError):
                    L.Batch([job])
        finally:
            ctx.set_precision("fp64")
    assert abs(E["bf16x3"] - E["fp64"]) / u.Natom <= 1e-6, E
