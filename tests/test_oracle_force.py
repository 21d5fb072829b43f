"""The oracle's grid force term (Force3, src/Force.jl:405-566, 3344-3394) is
pinned by an exact identity, as no reference test covers it: with V held
fixed, Force3 for atom i is f_s d/dR_i of sum_pairs <D, H^grid>, H^grid
re-tabulated with atom i moved (f_s = 2 for SpinPol "off": Force3_nospin's
factor 4 is f_s times the two orientations of every pair; the term is the
energy's gradient, its sign taken where the forces are assembled)."""
import numpy as np
import pytest

from helpers import oracle_pao, si2_cell
from oracle import lcp_oracle as O


def _psd_dm(u, seed, nspin=1):
    rng = np.random.default_rng(seed)
    no = np.asarray(u.Total_NumOrbs)
    off = np.concatenate([[0], np.cumsum(no)])
    out = []
    for _ in range(nspin):
        C = rng.normal(size=(off[-1], 6))
        M = C @ C.T
        M *= 8.0 / np.trace(M)
        dm = np.zeros(u.Total_Hsize)
        for p, (a, b, _) in enumerate(u.pairs):
            blk = M[off[a - 1]:off[a], off[b - 1]:off[b]]
            dm[u.block_offset[p]:u.block_offset[p] + blk.size] = blk.reshape(-1)
        out.append(dm)
    return out


def _cell(pos):
    lat, _, ng = si2_cell()
    return O.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], total_numorbs=[13, 13])


def _smooth_pao():
    """Synthetic s2p2d1 species whose radial functions and their derivatives
    vanish at the 7-bohr cutoff, so moving an atom changes no value by a jump
    (the tabulated Si7.0 functions end above zero at their last mesh point)."""
    from lcpgrid.workloads import synthetic_species
    p = synthetic_species(5)
    return O.PAO(p.Spe_MaxL_Basis, p.Spe_Num_Basis, p.Spe_PAO_RV, p.Spe_PAO_RWF)


def _energy(pos, dm, V, pao):
    u = _cell(pos)
    orbs = O.set_orbitals_grid([pao], u)
    H = O.calc_matrix_elements(u, orbs, [V], 1)[0]
    return float(np.dot(dm, H))


@pytest.mark.parametrize("atom,axis", [(0, 0), (1, 2)])
def test_force3_matches_finite_difference(atom, axis):
    lat, pos, ng = si2_cell()
    pos = np.asarray(pos, dtype=np.float64) + np.array([[0.0, 0.0, 0.0], [0.13, -0.07, 0.05]])
    u = _cell(pos)
    dm = _psd_dm(u, 11)
    rng = np.random.default_rng(12)
    V = rng.normal(size=u.NN) * 0.2 - 0.5
    pao = _smooth_pao()
    orbs = O.set_orbitals_grid([pao], u)
    dorbs = O.set_dorbitals_grid([pao], u)
    F = O.calc_force3("off", u, orbs, dorbs, [V], dm)
    h = 1e-4
    pp, pm = pos.copy(), pos.copy()
    pp[atom, axis] += h
    pm[atom, axis] -= h
    dE = (_energy(pp, dm[0], V, pao) - _energy(pm, dm[0], V, pao)) / (2 * h)
    assert F[atom, axis] == pytest.approx(2.0 * dE, rel=2e-5, abs=1e-9)


def test_force3_channels():
    """"on" with equal spin channels equals "off" on the half-filled channel
    (2 * (S + S) vs 4 * S); "nc" with zero off-diagonal channels equals "on"."""
    lat, pos, ng = si2_cell()
    u = _cell(pos)
    dm = _psd_dm(u, 21)
    V = np.random.default_rng(22).normal(size=u.NN)
    orbs = O.set_orbitals_grid([oracle_pao()], u)
    dorbs = O.set_dorbitals_grid([oracle_pao()], u)
    f_off = O.calc_force3("off", u, orbs, dorbs, [V], dm)
    f_on = O.calc_force3("on", u, orbs, dorbs, [V, V], [dm[0], dm[0]])
    np.testing.assert_allclose(f_on, f_off, rtol=1e-12, atol=1e-14)
    z = np.zeros(u.Total_Hsize)
    f_nc = O.calc_force3("nc", u, orbs, dorbs, [V, V, V, V], [dm[0], dm[0], z, z])
    np.testing.assert_allclose(f_nc, f_on, rtol=1e-12, atol=1e-14)
