"""Tensor-core building blocks: tcgen05 BF16 products with operands in the
K-major and MN-major canonical shared-memory layouts, against the exact
product of the BF16-rounded inputs (FP32 accumulation tolerance)."""
import numpy as np
import pytest

import lcpgrid as L

pytestmark = pytest.mark.gpu


def bf16(x):
    import torch
    return torch.from_numpy(np.asarray(x, dtype=np.float32)).to(torch.bfloat16).to(torch.float64).numpy()


@pytest.fixture(scope="module")
def ctx():
    return L.Context(0)


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("a_mn,b_mn", [(0, 0), (1, 1), (0, 1), (1, 0)])
@pytest.mark.parametrize("n,k", [(16, 16), (64, 32), (256, 64), (48, 48)])
def test_tc_selftest(ctx, a_mn, b_mn, n, k, order):
    rng = np.random.default_rng(n * 100 + k)
    a = rng.normal(size=(128, k)).astype(np.float32)
    b = rng.normal(size=(n, k)).astype(np.float32)
    d = ctx.tc_selftest(a, b, a_mn=bool(a_mn), b_mn=bool(b_mn), order=order)
    ref = bf16(a) @ bf16(b).T
    np.testing.assert_allclose(d, ref, rtol=0, atol=2e-5 * np.sqrt(k) * np.max(np.abs(ref)))


def _si2(ctx):
    from helpers import product_pao, si2_cell
    lat, pos, ng = si2_cell()
    u = L.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13])
    return u, L.Set_Orbitals_Grid([product_pao()], u, ctx=ctx)


def _si64(ctx):
    from lcpgrid.workloads import psd_density_matrices, si64_workload, smooth_vna
    wl = si64_workload()
    u = L.UCell(1, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"], wl["origin"],
                Total_NumOrbs=wl["numorbs"])
    orbs = L.Set_Orbitals_Grid(wl["paos"], u, ctx=ctx)
    dm = psd_density_matrices(u, wl["dm_seed"], trace=wl["trace"])
    vna = smooth_vna(wl["ngrid"], wl["latvecs"], wl["vna_seed"])
    return u, orbs, dm, vna


def _density(ctx, u, orbs, dm, precision, spin="off"):
    n = {"off": 1, "on": 2}[spin]
    rho = [np.zeros(u.NN) for _ in range(n)]
    ctx.set_precision(precision)
    try:
        L.Set_Density_Grid(spin, u, orbs, dm, rho)
    finally:
        ctx.set_precision("fp64")
    return rho


# Split-BF16 bounds.  Every operand is quantised to 2^-27 of its power-of-two
# scale (three BF16 parts of nine bits) and the part products down to
# mid*lo are accumulated exactly (lo*lo, at most 2^-36 of the scales, is not
# formed), so the error is the input quantisation: about 1.5e-7
# of max|rho| / max|H| on these cells, electron count and <D,H> to ~1e-8
# (with eight-bit parts the same cells gave 1e-6 and 4e-8; the bounds below
# are the ones those passed with a 5x margin, tightened by 5x).
RHO_TOL = 1e-6
H_TOL = 1e-6
SUM_TOL = 5e-8


def test_density_bf16x3_si2(ctx):
    """Split-BF16 density (tcgen05) vs the FP64 drop-in on the Si2 24^3 cell."""
    from test_gpu_parity import psd_dm
    u, orbs = _si2(ctx)
    for spin, n in (("off", 1), ("on", 2)):
        dm = psd_dm(u, 77, nspin=n)
        r64 = _density(ctx, u, orbs, dm, "fp64", spin)
        rtc = _density(ctx, u, orbs, dm, "bf16x3", spin)
        for c in range(n):
            scale = np.max(np.abs(r64[c]))
            err = np.max(np.abs(rtc[c] - r64[c]))
            assert err <= RHO_TOL * scale, (err, scale)
            assert abs(rtc[c].sum() - r64[c].sum()) <= SUM_TOL * abs(r64[c].sum())


def test_density_bf16x3_si64(ctx):
    u, orbs, dm, vna = _si64(ctx)
    r64 = _density(ctx, u, orbs, dm, "fp64")[0]
    rtc = _density(ctx, u, orbs, dm, "bf16x3")[0]
    scale = np.max(np.abs(r64))
    err = np.max(np.abs(rtc - r64))
    assert err <= RHO_TOL * scale, (err, scale)
    assert abs(rtc.sum() - r64.sum()) <= SUM_TOL * abs(r64.sum())


def _hks(ctx, u, orbs, vp, precision, spin="off"):
    n = {"off": 1, "on": 2}[spin]
    H = [np.zeros(u.Total_Hsize) for _ in range(n)]
    ctx.set_precision(precision)
    try:
        getattr(L, "Calc_MatrixElements_dVH_Vxc_" + spin)(u, orbs, vp, H)
    finally:
        ctx.set_precision("fp64")
    return H


def test_hamiltonian_bf16x3_si2(ctx):
    u, orbs = _si2(ctx)
    rng = np.random.default_rng(5)
    for spin, n in (("off", 1), ("on", 2)):
        vp = [rng.normal(size=u.NN) for _ in range(n)]
        h64 = _hks(ctx, u, orbs, vp, "fp64", spin)
        htc = _hks(ctx, u, orbs, vp, "bf16x3", spin)
        for c in range(n):
            scale = np.max(np.abs(h64[c]))
            err = np.max(np.abs(htc[c] - h64[c]))
            assert err <= H_TOL * scale, (err, scale)


def test_hamiltonian_bf16x3_si64(ctx):
    u, orbs, dm, vna = _si64(ctx)
    h64 = _hks(ctx, u, orbs, [vna], "fp64")[0]
    htc = _hks(ctx, u, orbs, [vna], "bf16x3")[0]
    scale = np.max(np.abs(h64))
    err = np.max(np.abs(htc - h64))
    e64, etc = float(np.dot(dm[0], h64)), float(np.dot(dm[0], htc))
    assert err <= H_TOL * scale, (err, scale)
    assert abs(etc - e64) <= SUM_TOL * abs(e64), (etc, e64)


@pytest.mark.parametrize("xc", ["LDA", "GGA_PBE"])
def test_job_energy_bf16x3_si64(ctx, xc):
    """Grid energy of one full step (rho, Poisson, xc, H, energies) on the
    64-atom 96^3 cell: split-BF16 contractions vs FP64, <= 1 uHa/atom."""
    u, orbs, dm, vna = _si64(ctx)
    E = {}
    for prec in ("fp64", "bf16x3"):
        ctx.set_precision(prec)
        try:
            job = L.GridStepJob(u, orbs, "off", xc, None, None, vna)
            job.set_dm(dm)
            job.step()
            E[prec] = job.energies()[4]
        finally:
            ctx.set_precision("fp64")
    assert abs(E["bf16x3"] - E["fp64"]) / u.Natom <= 1e-6, E


def test_job_energy_bf16x3_mx2(ctx):
    """The 432-atom MX2 monolayer (216 x 216 x 320 grid, spin-polarised, two
    species of 18 and 13 orbitals): the largest energies per atom of the
    workloads (grid energy ~159 Ha/atom), split-BF16 vs FP64 <= 1 uHa/atom."""
    from lcpgrid.workloads import mx2_monolayer, psd_density_matrices, smooth_vna
    wl = mx2_monolayer()
    u = L.UCell(1, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"], wl["origin"],
                Total_NumOrbs=wl["numorbs"])
    orbs = L.Set_Orbitals_Grid(wl["paos"], u, ctx=ctx)
    dm = psd_density_matrices(u, wl["dm_seed"], nspin=2, trace=wl["trace"])
    vna = smooth_vna(wl["ngrid"], wl["latvecs"], wl["vna_seed"])
    E = {}
    for prec in ("fp64", "bf16x3"):
        ctx.set_precision(prec)
        try:
            job = L.GridStepJob(u, orbs, "on", "LSDA", None, None, vna)
            job.set_dm(dm)
            job.step()
            E[prec] = job.energies()[4]
            del job
        finally:
            ctx.set_precision("fp64")
    assert abs(E["bf16x3"] - E["fp64"]) / u.Natom <= 1e-6, E


def _mixed_cell(ctx, nrep=1, ngrid=(44, 40, 48)):
    """Three species of 18 (s2p2d2: two 16-orbital chunks), 13 and 4 orbitals,
    cutoffs 8 / 7 / 6 bohr, seeded positions in a 11 x 10 x 12 bohr box."""
    from lcpgrid.workloads import synthetic_species
    paos = [synthetic_species(11, max_l=2, num_basis=(2, 2, 2), rc=8.0),
            synthetic_species(12, max_l=2, num_basis=(2, 2, 1), rc=7.0),
            synthetic_species(13, max_l=1, num_basis=(1, 1), rc=6.0)]
    lat = np.diag([11.0, 10.0, 12.0])
    pos = np.array([[1.0, 2.0, 3.0], [5.5, 6.0, 8.5], [8.0, 1.5, 6.0]])
    u = L.UCell(1, lat, 3, [1, 2, 3], pos, [8.0, 7.0, 6.0], ngrid, [0, 0, 0], Total_NumOrbs=[18, 13, 4])
    return u, L.Set_Orbitals_Grid(paos, u, ctx=ctx)


def test_orbital_chunks_density_and_h(ctx):
    """Atoms of more than 16 orbitals enter the tensor-core path as 16-orbital
    chunks: split-BF16 vs FP64 on a mixed 18 / 13 / 4-orbital cell."""
    from test_gpu_parity import psd_dm
    u, orbs = _mixed_cell(ctx)
    for spin, n in (("off", 1), ("on", 2)):
        dm = psd_dm(u, 31, nspin=n)
        r64 = _density(ctx, u, orbs, dm, "fp64", spin)
        rtc = _density(ctx, u, orbs, dm, "bf16x3", spin)
        for c in range(n):
            scale = np.max(np.abs(r64[c]))
            assert np.max(np.abs(rtc[c] - r64[c])) <= RHO_TOL * scale
            assert abs(rtc[c].sum() - r64[c].sum()) <= SUM_TOL * abs(r64[c].sum())
    rng = np.random.default_rng(8)
    vp = [rng.normal(size=u.NN)]
    h64 = _hks(ctx, u, orbs, vp, "fp64")[0]
    htc = _hks(ctx, u, orbs, vp, "bf16x3")[0]
    assert np.max(np.abs(htc - h64)) <= H_TOL * np.max(np.abs(h64))
    dm = psd_dm(u, 32)[0]
    assert abs(np.dot(dm, htc) - np.dot(dm, h64)) <= SUM_TOL * np.sum(np.abs(dm * h64))


def _check_vs_fp64(ctx, u, orbs, seed):
    from test_gpu_parity import psd_dm
    dm = psd_dm(u, seed)
    r64 = _density(ctx, u, orbs, dm, "fp64")[0]
    rtc = _density(ctx, u, orbs, dm, "bf16x3")[0]
    assert np.max(np.abs(rtc - r64)) <= RHO_TOL * np.max(np.abs(r64))
    assert abs(rtc.sum() - r64.sum()) <= SUM_TOL * abs(r64.sum())
    vp = [np.random.default_rng(seed).normal(size=u.NN)]
    h64 = _hks(ctx, u, orbs, vp, "fp64")[0]
    htc = _hks(ctx, u, orbs, vp, "bf16x3")[0]
    assert np.max(np.abs(htc - h64)) <= H_TOL * np.max(np.abs(h64))
    return rtc, htc


@pytest.mark.parametrize("shape", [(4, 4, 8), (8, 4, 4), (5, 6, 4), (3, 7, 5), None])
def test_ragged_bricks(ctx, shape):
    """Brick sides that do not divide Ngrid (45 x 42 x 49): the last brick of
    an axis is ragged, its slots past the grid empty; split-BF16 vs FP64."""
    u, orbs = _mixed_cell(ctx, ngrid=(45, 42, 49))
    ctx.set_precision("bf16x3")
    try:
        orbs.set_brick_shape(shape)
        got = orbs.brick_shape()
    finally:
        ctx.set_precision("fp64")
    if shape is not None:
        assert got == tuple(shape)
    else:
        assert got == u.brick_shape_candidates(1)[0][0]
    _check_vs_fp64(ctx, u, orbs, 61)


def test_autotune_and_release_fp64(ctx):
    """The measured brick-shape autotuner keeps one of the predicted best
    shapes; after the FP64 tables are released the split-BF16 path gives the
    same bits and the FP64 path refuses."""
    from test_gpu_parity import psd_dm
    u, orbs = _mixed_cell(ctx, ngrid=(45, 42, 49))
    cands = [c[0] for c in u.brick_shape_candidates(8)]
    ctx.set_precision("bf16x3")
    try:
        shape, ms = orbs.autotune_bricks(3)
        assert shape in cands[:8] and ms > 0
        assert orbs.brick_shape() == shape
    finally:
        ctx.set_precision("fp64")
    rtc, htc = _check_vs_fp64(ctx, u, orbs, 62)
    ctx.set_precision("bf16x3")
    try:
        orbs.release_fp64()
    finally:
        ctx.set_precision("fp64")
    dm = psd_dm(u, 62)
    np.testing.assert_array_equal(_density(ctx, u, orbs, dm, "bf16x3")[0], rtc)
    with pytest.raises(L.LCPError):
        _density(ctx, u, orbs, dm, "fp64")
    with pytest.raises(L.LCPError):
        orbs.set_brick_shape((4, 4, 8))


def test_bricks_of_many_images(ctx):
    """A dense cell of 18-orbital atoms with 9-bohr cutoffs: bricks touched by
    more than 64 sub-images (the density kernel then reads the brick's pair
    table from global memory instead of its shared-memory copy)."""
    from lcpgrid.workloads import _place, synthetic_species
    pao = synthetic_species(21, max_l=2, num_basis=(2, 2, 2), rc=9.0)
    side = 12.0
    pos = _place(np.random.default_rng(4), 16, side, 3.5)
    u = L.UCell(1, np.eye(3) * side, 16, [1] * 16, pos, [9.0] * 16, (48, 48, 48), [0, 0, 0],
                Total_NumOrbs=[18] * 16)
    assert u.brick_info()["max_images"] > 64
    orbs = L.Set_Orbitals_Grid([pao], u, ctx=ctx)
    _check_vs_fp64(ctx, u, orbs, 63)


def test_tc_kernel_times_and_form():
    """lcp_job_tc_kernel_ms: one split-BF16 step with events around the two
    tensor-core kernels alone; they take part of the step, the step's results
    are those of an ordinary step, and other precisions are refused."""
    from test_gpu_parity import psd_dm
    c = L.Context(0, precision="bf16x3")
    u, orbs = _si2(c)
    job = L.GridStepJob(u, orbs, "off", "LDA")
    job.set_dm(psd_dm(u, 5))
    job.step()
    e_ref, h_ref = job.energies(), job.hks()[0].copy()
    dens_ms, ham_ms = job.tc_kernel_ms()
    assert dens_ms > 0 and ham_ms > 0
    np.testing.assert_array_equal(job.energies(), e_ref)
    np.testing.assert_array_equal(job.hks()[0], h_ref)
    stages = job.step_timed()
    assert dens_ms <= stages[0] * 1.5 and ham_ms <= stages[4] * 1.5
    # the energies queued without waiting are complete after the synchronising H read
    e = np.full(5, np.nan)
    job.step()
    job.energies_async(e)
    job.hks()
    np.testing.assert_array_equal(e, job.energies())
    c.set_precision("fp64")
    with pytest.raises(L.LCPError):
        job.tc_kernel_ms()
