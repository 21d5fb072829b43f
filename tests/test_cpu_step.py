"""The parallel CPU grid step (oracle/cpu_step.py, the timed CPU baseline and
full-size checker) against the serial oracle functions, and its pair split
against the reference's rule (src/UCell.jl:50-132)."""
import numpy as np
import pytest

from helpers import oracle_pao, si2_cell, species_arrays
from oracle import lcp_oracle as O
from oracle.cpu_step import CpuGridStep, split_weighted_contiguous


def test_split_weighted_contiguous_matches_the_rule():
    rng = np.random.default_rng(3)
    for n, parts in ((10, 3), (57, 8), (16, 16), (200, 7)):
        w = rng.uniform(1, 50, n)
        r = split_weighted_contiguous(w, parts)
        assert len(r) == parts and r[0][0] == 0 and r[-1][1] == n
        assert all(a < b for a, b in r) and all(r[k][1] == r[k + 1][0] for k in range(parts - 1))
        cum = np.cumsum(w)
        for k, (a, b) in enumerate(r[:-1]):
            target = cum[-1] * (k + 1) / parts
            # the boundary is the closer of the two cumulative sums around the target
            # (unless a part would be left empty)
            last = b - 1
            if a < last < n - (parts - k - 1) - 1:
                assert abs(cum[last] - target) <= abs(cum[last + 1] - target) + 1e-9
    with pytest.raises(ValueError):
        split_weighted_contiguous([1.0, 2.0], 3)


def _si2_spec(spinpol):
    lat, pos, ng = si2_cell()
    maxl, nb, rv, rwf = species_arrays("Si7.0")
    return {"latvecs": lat, "natom": 2, "atom2spe": [1, 1], "gxyz": pos, "cut": [7.0, 7.0], "ngrid": ng,
            "origin": [0.0, 0.0, 0.0], "numorbs": [13, 13], "paos": [(maxl, nb, rv, rwf)], "spinpol": spinpol,
            "xc": "LDA" if spinpol == "off" else "LSDA"}


@pytest.mark.parametrize("spinpol", ["off", "on"])
def test_parallel_step_matches_serial_oracle(spinpol):
    spec = _si2_spec(spinpol)
    nspin = 1 if spinpol == "off" else 2
    u = O.UCell(nspin, spec["latvecs"], 2, [1, 1], spec["gxyz"], [7.0, 7.0], spec["ngrid"], [0, 0, 0],
                total_numorbs=[13, 13])
    orbs = O.set_orbitals_grid([oracle_pao()], u)
    rng = np.random.default_rng(11)
    dm = []
    for _ in range(nspin):
        C = rng.normal(size=(26, 6))
        M = C @ C.T
        M *= 4.0 / np.trace(M)
        d = np.zeros(u.Total_Hsize)
        for p, (a, b, _) in enumerate(u.pairs):
            d[u.block_offset[p]:u.block_offset[p] + 169] = M[13 * (a - 1):13 * a, 13 * (b - 1):13 * b].reshape(-1)
        dm.append(d)
    rho = O.set_density_grid(spinpol, u, orbs, dm)
    dvh = O.solve_poisson(spinpol, u, rho, np.zeros(u.NN))
    vp = O.set_vpot_grid(spinpol, dvh, O.set_xc_grid(spec["xc"], spinpol, np.zeros(u.NN), rho))
    H = O.calc_matrix_elements(u, orbs, vp, nspin)
    with CpuGridStep(spec, nproc=3) as cs:
        assert cs.nproc == 3 and sum(len(x) for x in cs.loops) == u.Nloop
        cs.set_dm(dm)
        out = cs.step()
        out2 = cs.step()  # a second step on the same ranks gives the same result
    for s in range(nspin):
        np.testing.assert_allclose(out["density"][s], rho[s], rtol=0, atol=1e-13 * np.max(np.abs(rho[s])))
        np.testing.assert_allclose(out["hks"][s], H[s], rtol=0, atol=1e-13 * np.max(np.abs(H[s])))
        np.testing.assert_array_equal(out["hks"][s], out2["hks"][s])
    eh1 = O.calc_eh1(spinpol, u.GridVol, np.zeros(u.NN), rho, dvh)
    exc = O.calc_exc1(spinpol, spec["xc"], u.GridVol, np.zeros(u.NN), np.zeros(u.NN), rho)
    e = O.grid_energy(spinpol, u, dm, H, eh1, exc)
    assert abs(out["energies"][4] - e) <= 1e-11 * abs(e)
    assert set(out["seconds"]) >= {"density", "poisson", "xc_vpot", "hamiltonian", "energies", "step"}
