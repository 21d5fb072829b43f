"""Batched grid step (lcp_batch_*): many cells' device-resident jobs stepped
together -- one tensor-core launch per contraction over every cell's bricks,
batched FFTs per grid shape, tiled grid kernels over all cells, CUDA-graph
replay.  Each cell's results must match its job stepped alone."""
import numpy as np
import pytest

import lcpgrid as L

pytestmark = pytest.mark.gpu


def _cells(ctx, spin="off", n_pool=6, seed=91, xc=None):
    """Small cells of the batching form (1-3 species, cutoffs 6-9 bohr,
    4/9/13/18 orbitals, grids from Calc_Ngrid at 150 Ry) plus two cells that
    share a grid shape (batched FFT plan with two transforms)."""
    from helpers import product_pao, si2_cell
    from lcpgrid.workloads import batch_pool, psd_density_matrices, smooth_vna
    cells = []
    for c in batch_pool(n_pool, seed=seed, nmax=10, amax_ang=7.0):
        u = L.UCell(2 if spin == "on" else 1, c["latvecs"], c["natom"], c["atom2spe"], c["gxyz"], c["cut"],
                    c["ngrid"], c["origin"], Total_NumOrbs=c["numorbs"])
        cells.append((u, L.Set_Orbitals_Grid(c["paos"], u, ctx=ctx)))
    lat, pos, ng = si2_cell()
    for scale in (1.0, 1.01):
        u = L.UCell(2 if spin == "on" else 1, lat, 2, [1, 1], pos * scale, [7.0, 7.0], ng, [0, 0, 0],
                    Total_NumOrbs=[13, 13])
        cells.append((u, L.Set_Orbitals_Grid([product_pao()], u, ctx=ctx)))
    jobs = []
    nspin = 2 if spin == "on" else 1
    for k, (u, orbs) in enumerate(cells):
        vna = smooth_vna(u.Ngrid, u.Latvecs, 300 + k)
        job = L.GridStepJob(u, orbs, spin, xc or ("LDA" if spin == "off" else "LSDA"), None, None, vna)
        dm = psd_density_matrices(u, 400 + k, nspin=nspin, trace=2.0 * u.Natom)
        job.set_dm(dm)
        jobs.append(job)
    return jobs


def _alone(jobs):
    out = []
    for job in jobs:
        job.step()
        out.append((job.energies(), [x.copy() for x in job.density()], [x.copy() for x in job.hks()]))
    return out


def _compare(jobs, ref, exact_density=True):
    for job, (e, rho, hks) in zip(jobs, ref):
        for a, b in zip(job.density(), rho):
            if exact_density:
                np.testing.assert_array_equal(a, b)  # same kernels, same per-cell D scale
        for a, b in zip(job.hks(), hks):
            # V differs from the single-cell step only by the batched FFT's rounding
            np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 * max(1.0, np.abs(b).max()))
        np.testing.assert_allclose(job.energies(), e, rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("spin", ["off", "on"])
def test_batch_matches_alone(spin):
    ctx = L.Context(0, precision="bf16x3")
    jobs = _cells(ctx, spin)
    ref = _alone(jobs)
    b = L.Batch(jobs)
    info = b.info()
    assert info["cells"] == len(jobs) and info["shape_groups"] < len(jobs)
    b.step(graph=False)
    b.check_status()
    _compare(jobs, ref)
    en = b.energies()
    np.testing.assert_array_equal(en, np.array([j.energies() for j in jobs]))
    b.close()


@pytest.mark.parametrize("spin", ["off", "on"])
def test_batch_gga_matches_alone(spin):
    """GGA-PBE cells: the gradient/PBE and divergence passes run tiled over
    every cell of the batch."""
    ctx = L.Context(0, precision="bf16x3")
    jobs = _cells(ctx, spin, n_pool=4, seed=23, xc="GGA_PBE")
    ref = _alone(jobs)
    b = L.Batch(jobs)
    b.step(graph=False)
    b.check_status()
    _compare(jobs, ref)
    b.close()


def test_batch_graph_replay():
    ctx = L.Context(0, precision="bf16x3")
    jobs = _cells(ctx, "off", n_pool=4, seed=17)
    b = L.Batch(jobs)
    b.step(graph=False)
    eager = b.energies().copy()
    h_eager = [j.hks()[0].copy() for j in jobs]
    for _ in range(3):  # the first call runs and captures, the others replay
        b.step(graph=True)
        np.testing.assert_array_equal(b.energies(), eager)
    assert b.info()["graph"] == 1
    for j, h in zip(jobs, h_eager):
        np.testing.assert_array_equal(j.hks()[0], h)
    # a new D reaches the graph through the jobs' device buffers
    from lcpgrid.workloads import psd_density_matrices
    j0 = jobs[0]
    j0.set_dm(psd_density_matrices(j0.ucell, 999, trace=2.0 * j0.ucell.Natom))
    b.step(graph=True)
    e_new = b.energies()
    assert not np.array_equal(e_new[0], eager[0])
    np.testing.assert_array_equal(e_new[1:], eager[1:])
    j0.step()
    np.testing.assert_allclose(j0.energies(), e_new[0], rtol=1e-11, atol=1e-12)
    b.close()


# Split-BF16 quantises every operand to 2^-27 of its scale, so each grid
# energy term carries a relative error of about 1e-8 (up to 7e-8 measured on
# 20 random 2-10 atom cells; eight-bit parts gave up to 1.4e-7 there, and a
# CPU emulation of the rounding alone gives the same).  These synthetic cells
# carry no neutralising atomic density, so their Hartree terms reach tens of
# Ha/atom.
ENERGY_REL_TOL = 2e-7


def test_batch_energy_within_tolerance_of_fp64():
    """Split-BF16 batch vs the FP64 per-cell step: every energy term within
    ENERGY_REL_TOL, and <= 1 uHa/atom on average over the cells."""
    ctx = L.Context(0, precision="bf16x3")
    jobs = _cells(ctx, "off", n_pool=6, seed=23)
    b = L.Batch(jobs)
    b.step(graph=True)
    e_batch = b.energies()
    ctx.set_precision("fp64")
    per_atom = []
    for k, job in enumerate(jobs):
        job.step()
        e64 = job.energies()
        scale = abs(e64[0]) + abs(e64[1]) + abs(e64[2]) + 2 * abs(e64[3])
        for i in range(5):
            assert abs(e_batch[k, i] - e64[i]) <= ENERGY_REL_TOL * scale, (k, i, e_batch[k], e64)
        per_atom.append(abs(e_batch[k, 4] - e64[4]) / job.ucell.Natom)
    assert np.mean(per_atom) <= 1e-6, per_atom
    b.close()


def test_batch_rejects_mixed_and_fp64():
    ctx = L.Context(0, precision="bf16x3")
    jobs = _cells(ctx, "off", n_pool=1, seed=5)
    jobs_on = _cells(ctx, "on", n_pool=1, seed=5)
    with pytest.raises(L.LCPError):
        L.Batch([jobs[0], jobs_on[0]])
    with pytest.raises(L.LCPError):
        L.Batch([jobs[0], jobs[0]])
    ctx.set_precision("fp64")
    with pytest.raises(L.LCPError):
        L.Batch(jobs)


def test_batch_waves_same_bits():
    """A scratch budget that splits the matrix-element pass into waves
    changes no bit of the results."""
    ctx = L.Context(0, precision="bf16x3")
    jobs = _cells(ctx, "off", n_pool=5, seed=29)
    b1 = L.Batch(jobs)
    b1.step(graph=True)
    e1 = b1.energies().copy()
    h1 = [j.hks()[0].copy() for j in jobs]
    b1.close()
    b2 = L.Batch(jobs, scratch_bytes=1)  # every cell a wave of its own
    assert b2.info()["waves"] == len(jobs)
    b2.step(graph=True)
    np.testing.assert_array_equal(b2.energies(), e1)
    for j, h in zip(jobs, h1):
        np.testing.assert_array_equal(j.hks()[0], h)
    b2.close()


def test_batch_isolates_a_bad_cell():
    """A NaN in one cell's D poisons that cell's results only: every other
    cell of the batch keeps the same bits as in a clean batch."""
    from lcpgrid.workloads import psd_density_matrices
    ctx = L.Context(0, precision="bf16x3")
    jobs = _cells(ctx, "off", n_pool=4, seed=41)
    b = L.Batch(jobs)
    b.step(graph=True)
    clean = b.energies().copy()
    bad = 2
    dm = psd_density_matrices(jobs[bad].ucell, 7, trace=2.0 * jobs[bad].ucell.Natom)
    dm[0][5] = np.nan
    jobs[bad].set_dm(dm)
    b.step(graph=True)
    b.check_status()  # a NaN input is not a device error
    got = b.energies()
    assert np.isnan(got[bad]).any()
    others = [k for k in range(len(jobs)) if k != bad]
    np.testing.assert_array_equal(got[others], clean[others])
    b.close()
