"""The precision forms' xc functional in double-float against its FP64
evaluation, point by point (src/XC/LDA_CA.jl:4-41, src/XC/LSDA_CA.jl:1-138).

Densities span 1e-14 .. 30 e/bohr^3, both correlation branches (rs < 1 and
rs >= 1), the cutoff at 1e-15, partial core densities, and spin
polarisations up to the clamped |zeta| = 1.  The double-float evaluation must
agree with FP64 to 1e-12 of each value's magnitude (it is built for about
2^-45) and give exactly 0 below the cutoff.  The FP64 path itself is pinned
to the oracle by the parity tests.
"""
import numpy as np
import pytest

import lcpgrid as L
from lcpgrid import _lib

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _eval(ctx, xc, df, up, dn=None, pcc=None):
    out = np.zeros(3 * up.size)
    _lib.check(_lib.lib.lcp_xc_selftest(ctx._h, xc, int(df), up.size, _lib.dptr(up), _lib.dptr(dn), _lib.dptr(pcc),
                                        _lib.dptr(out)))
    return out.reshape(-1, 3)


def _densities(rng, n):
    rho = 10.0 ** rng.uniform(-14, 1.5, n)
    rho[:8] = [0.0, 1e-16, 4e-16, 5.1e-16, 1e-15, 0.24, 0.2387, 0.25]  # cutoff and rs ~ 1 (rho ~ 0.2387)
    return rho


def _compare(a, b):
    scale = np.maximum(np.abs(b), 1e-300)
    rel = np.abs(a - b) / scale
    return float(np.max(rel[np.abs(b) > 0])) if np.any(np.abs(b) > 0) else 0.0


def test_lda_double_float_matches_fp64():
    ctx = L.Context(0)
    rng = np.random.default_rng(5)
    up = _densities(rng, 200_000) * 0.5
    pcc = np.where(rng.uniform(size=up.size) < 0.3, 10.0 ** rng.uniform(-6, 0, up.size), 0.0)
    for p in (None, pcc):
        f64 = _eval(ctx, _lib.LCP_XC_LDA, False, up, pcc=p)
        dfl = _eval(ctx, _lib.LCP_XC_LDA, True, up, pcc=p)
        den = 2 * (up + (p if p is not None else 0.0))
        zero = den <= 1e-15
        assert np.all(dfl[zero, :2] == 0.0) and np.all(f64[zero, :2] == 0.0)
        assert _compare(dfl[:, 0], f64[:, 0]) <= TOL
        assert _compare(dfl[:, 1], f64[:, 1]) <= TOL
        # both branches were exercised
        rs = 0.6203504908994 / np.cbrt(den[~zero])
        assert np.any(rs < 1) and np.any(rs >= 1)


def test_lsda_double_float_matches_fp64():
    ctx = L.Context(0)
    rng = np.random.default_rng(6)
    tot = _densities(rng, 200_000)
    frac = rng.uniform(0, 1, tot.size)
    frac[8:40] = [0.0, 1.0] * 16  # fully polarised
    frac[40:60] = 0.5             # unpolarised
    up, dn = tot * frac, tot * (1 - frac)
    pcc = np.where(rng.uniform(size=up.size) < 0.3, 10.0 ** rng.uniform(-6, 0, up.size), 0.0)
    for p in (None, pcc):
        f64 = _eval(ctx, _lib.LCP_XC_LSDA, False, up, dn, p)
        dfl = _eval(ctx, _lib.LCP_XC_LSDA, True, up, dn, p)
        # FP64's own conditioning near full polarisation: 1 -+ zeta carries
        # an absolute rounding of ~1e-16 there, which the cube roots of the
        # potentials pass on relative to min(1 + zeta, 1 - zeta)
        u = up + (p if p is not None else 0.0)
        d_ = dn + (p if p is not None else 0.0)
        tot_ = np.maximum(u + d_, 1e-300)
        side = np.minimum(2 * u / tot_, 2 * d_ / tot_)
        tol = TOL + 1e-15 / np.maximum(side, 1e-300)
        mag = np.maximum(np.abs(f64).max(axis=1), 1e-300)
        live = (mag > 1e-300) & (side > 0)
        for k in range(3):
            d = np.abs(dfl[:, k] - f64[:, k]) / mag
            assert np.all(d[live] <= tol[live]), (k, float(np.max(d[live] / tol[live])))
        # fully polarised points (a spin exactly empty): zeta = +-1 exactly in both
        full = (mag > 1e-300) & (side == 0)
        assert np.any(full)
        for k in range(3):
            d = np.abs(dfl[full, k] - f64[full, k]) / mag[full]
            assert float(np.max(d)) <= TOL, k


def test_unknown_functional_rejected():
    ctx = L.Context(0)
    x = np.ones(4)
    with pytest.raises(L.LCPError):
        _eval(ctx, _lib.LCP_XC_GGA_PBE, True, x, x)
