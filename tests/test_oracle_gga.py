"""GGA-PBE oracle pins (CPU): the pointwise kernel against the reference's
golden vector (test/test_XC_PBE.jl), the 27-point stencil against exact
derivatives of quadratics, and the grid potential against a finite-difference
derivative of the discrete energy it belongs to."""
import numpy as np
import pytest

from helpers import golden
from oracle import lcp_oracle as o

SKEW = np.array([[4.2, 0.3, 0.1], [0.5, 3.9, -0.2], [0.2, 0.4, 4.4]])
NG = (8, 7, 6)


def test_xc_pbe_golden():
    g = golden()["xc_pbe"]
    ed = [np.array([g["ED"][0]]), np.array([g["ED"][1]])]
    gd = [np.array([x]) for x in g["GDENS"]]
    exc, dexdd, decdd, dexdgd, decdgd = o.xc_pbe(ed, gd)
    for name, val in (("Exc", exc), ("DEXDD", dexdd), ("DECDD", decdd), ("DEXDGD", dexdgd), ("DECDGD", decdgd)):
        got = np.array([v[0] for v in val])
        np.testing.assert_allclose(got, g[name], rtol=1e-13, atol=1e-16, err_msg=name)


@pytest.mark.parametrize("lat", [np.eye(3) * 3.0, SKEW, np.array([[5.1, 0, 5.1], [0, 5.1, 5.1], [5.1, 5.1, 0]])])
def test_diff_coef_exact_on_quadratics(lat):
    gl = o.glatvecs_of(lat, (9, 10, 11))
    dc = o.calc_diff_coef(gl)
    rng = np.random.default_rng(3)
    b = rng.normal(size=3)
    C = rng.normal(size=(3, 3))
    f = []
    for i1 in (-1, 0, 1):
        for j1 in (-1, 0, 1):
            for k1 in (-1, 0, 1):
                r = i1 * gl[0] + j1 * gl[1] + k1 * gl[2]
                f.append(0.7 + b @ r + r @ C @ r)
    np.testing.assert_allclose(dc @ np.array(f), b, rtol=0, atol=1e-10)
    # a centred first-derivative stencil is odd under p -> 26 - p
    np.testing.assert_allclose(dc, -dc[:, ::-1], rtol=0, atol=1e-10 * np.abs(dc).max())


def _fields(spinpol, seed=11):
    rng = np.random.default_rng(seed)
    n1, n2, n3 = NG
    i, j, k = np.meshgrid(np.arange(n1) / n1, np.arange(n2) / n2, np.arange(n3) / n3, indexing="ij")

    def smooth(a0):
        v = a0 * np.ones(NG)
        for _ in range(3):
            q = rng.integers(-1, 2, size=3)
            v = v + rng.uniform(0.05, 0.2) * a0 * np.cos(2 * np.pi * (q[0] * i + q[1] * j + q[2] * k) + rng.uniform(0, 6))
        return v.ravel()

    pcc = smooth(0.01)
    if spinpol == "off":
        return pcc, [smooth(0.05)]
    return pcc, [smooth(0.06), smooth(0.035)]


def _energy(spinpol, dc, pcc, dens):
    """Discrete energy whose derivative Set_Vxc_GGA_PBE! evaluates:
    sum_i rho_tot,i * (Fx + Fc)_i with the stencil gradients."""
    dd = o.set_ddensity_grid(spinpol, NG, dens, pcc, dc)
    up = dens[0] + pcc
    dn = up if spinpol == "off" else dens[1] + pcc
    gd = [dd[0][0], dd[0][1], dd[0][2]] + ([dd[0][0], dd[0][1], dd[0][2]] if spinpol == "off" else
                                          [dd[1][0], dd[1][1], dd[1][2]])
    exc = o.xc_pbe((up, dn), gd)[0]
    return float(np.sum((up + dn) * (exc[0] + exc[1])))


@pytest.mark.parametrize("spinpol", ["off", "on"])
def test_vxc_is_energy_derivative(spinpol):
    dc = o.calc_diff_coef(o.glatvecs_of(SKEW, NG))
    pcc, dens = _fields(spinpol)
    vxc, dd, dexc = o.set_xc_grid_gga(spinpol, NG, pcc, dens, dc)
    rng = np.random.default_rng(5)
    nn = int(np.prod(NG))
    for pt in rng.choice(nn, size=6, replace=False):
        for s in range(len(dens)):
            h = 1e-5 * dens[s][pt]
            dp = [d.copy() for d in dens]
            dm = [d.copy() for d in dens]
            dp[s][pt] += h
            dm[s][pt] -= h
            fd = (_energy(spinpol, dc, pcc, dp) - _energy(spinpol, dc, pcc, dm)) / (2 * h)
            # "off": rho feeds both spin channels, so dE/drho = 2 Vxc
            want = (2.0 if spinpol == "off" else 1.0) * vxc[s][pt]
            assert abs(fd - want) <= 1e-7 * max(1.0, abs(want)), (spinpol, pt, s, fd, want)


def test_nc_rotation_and_masks():
    dc = o.calc_diff_coef(o.glatvecs_of(SKEW, NG))
    pcc, dens = _fields("on", seed=4)
    rng = np.random.default_rng(8)
    nn = int(np.prod(NG))
    th, ph = rng.uniform(0, np.pi, nn), rng.uniform(0, 2 * np.pi, nn)
    v_on, _, _ = o.set_xc_grid_gga("on", NG, pcc, dens, dc)
    v_nc, _, _ = o.set_xc_grid_gga("nc", NG, pcc, dens + [th, ph], dc)
    t0, t1 = 0.5 * (v_on[0] + v_on[1]), 0.5 * (v_on[0] - v_on[1])
    np.testing.assert_allclose(v_nc[0], t0 + np.cos(th) * t1, rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(v_nc[1], t0 - np.cos(th) * t1, rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(v_nc[2], -t1 * np.sin(th) * np.cos(ph), rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(v_nc[3], -t1 * np.sin(th) * np.sin(ph), rtol=1e-14, atol=1e-15)
    # an empty region: gradient and potential vanish where the density is at den_min
    d0 = [dens[0].copy(), dens[1].copy()]
    d0[0][:10] = 0.0
    d0[1][:10] = 0.0
    v, dd, dexc = o.set_xc_grid_gga("on", NG, None, d0, dc)
    assert np.all(dd[0][0][:10] == 0) and np.all(dexc[1][2][:10] == 0) and np.all(v[0][:10] == 0)


def test_exc1_gga_matches_energy():
    pcc, dens = _fields("on", seed=2)
    aden = 0.5 * (dens[0] + dens[1])
    gridvol = abs(np.linalg.det(SKEW)) / np.prod(NG)
    exc = o.calc_exc1("on", "GGA_PBE", gridvol, aden, pcc, dens, ngrid=NG, latvecs=SKEW)
    dc = o.calc_diff_coef(o.glatvecs_of(SKEW, NG))
    temp = aden + pcc
    want = (_energy("on", dc, pcc, dens) - 2 * np.sum(temp * o.lda_ca(2 * temp, 0))) * gridvol
    assert abs(exc[0] + exc[1] - want) <= 1e-12 * abs(want)


def test_diagonalize_nc_density_invariants():
    """Nup, Ndown are the eigenvalues of the 2x2 spin density matrix
    [[Re11, Re12 + i Im12], [Re12 - i Im12, Re22]] and the angles give its
    spin direction (2 Re12, -2 Im12, Re11 - Re22) / r."""
    rng = np.random.default_rng(6)
    n = 500
    d = [rng.uniform(0, 0.3, n), rng.uniform(0, 0.3, n), rng.normal(0, 0.05, n), rng.normal(0, 0.05, n)]
    d[2][:5] = 0.0
    d[3][:5] = 0.0  # collinear points: phi = 0
    d[0][5:8] = d[1][5:8]
    d[2][5:8] = 0.0
    d[3][5:8] = 0.0  # no spin at all: r = 0, theta = pi/2, phi = 0
    nu, nd, th, ph = o.diagonalize_nc_density(d)
    np.testing.assert_allclose(nu + nd, d[0] + d[1], rtol=1e-14)
    np.testing.assert_allclose(nu * nd, d[0] * d[1] - d[2] ** 2 - d[3] ** 2, rtol=1e-12, atol=1e-16)
    r = nu - nd
    m = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)])
    np.testing.assert_allclose(m, np.stack([2 * d[2], -2 * d[3], d[0] - d[1]]), atol=1e-14)
    assert np.all(ph[:5] == 0.0) and np.all(th[5:8] == 0.5 * np.pi) and np.all(ph[5:8] == 0.0)


def test_host_diff_coef_matches_oracle():
    """The library's host Calc_Diff_Coef (C++, no GPU) against the oracle's."""
    import lcpgrid as L
    for lat, ng in ((SKEW, NG), (np.array([[5.1, 0, 5.1], [0, 5.1, 5.1], [5.1, 5.1, 0]]), (24, 24, 24)),
                    (np.eye(3) * 7.0, (30, 32, 34))):
        gl = o.glatvecs_of(lat, ng)
        got = np.array(L.Calc_Diff_Coef(gl))
        want = o.calc_diff_coef(gl)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())
    with pytest.raises(L.LCPError):
        L.Calc_Diff_Coef(np.zeros((3, 3)))  # singular fit: every neighbour at the centre
