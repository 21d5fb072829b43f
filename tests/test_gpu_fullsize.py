"""The benchmarked workloads against the oracle, at their full sizes.

* 64-atom Si, 96^3 (the precision-form cell): one FP64 grid step of the
  device-resident job (density, Poisson, LDA + V_na, H, energies) against the
  whole step restated on the host cores (oracle/cpu_step.py, every pair of the
  cell).  Then the split-BF16 step against the same oracle step.
* 432-atom MX2 monolayer, 216x216x320, LSDA (the large spin-polarised cell):
  D is zero outside the pairs among a sample of neighbouring atoms (both
  orientations), so the density is exactly the sample's; the oracle computes
  that density, the potential on the full grid, and the H blocks of the
  sampled pairs, which the GPU's FP64 and split-BF16 steps must match.

Tolerances of the drop-in: rho <= 1e-8 e/bohr^3, H <= 1e-7 Ha, total grid energy
<= 1 uHa/atom for FP64.  Split-BF16: rho and H within 1e-6 of their maximum,
energy within 1 uHa/atom (reference: src/Matrix/Set_Density_Grid.jl:60-169,
src/Hamiltonian.jl:235-324).
"""
import os

import numpy as np
import pytest

import lcpgrid as L

pytestmark = pytest.mark.gpu

RHO_ABS = 1e-8     # e/bohr^3, FP64 form
H_ABS = 1e-7       # Ha, FP64 form
E_ATOM = 1e-6      # Ha per atom, both forms
TC_REL = 1e-6      # split-BF16 rho and H, relative to their maximum


def _spec(wl, vna):
    return {"latvecs": wl["latvecs"], "natom": wl["natom"], "atom2spe": wl["atom2spe"], "gxyz": wl["gxyz"],
            "cut": wl["cut"], "ngrid": wl["ngrid"], "origin": wl["origin"], "numorbs": wl["numorbs"],
            "paos": [(p.Spe_MaxL_Basis, p.Spe_Num_Basis, p.Spe_PAO_RV, p.Spe_PAO_RWF) for p in wl["paos"]],
            "spinpol": wl.get("spinpol", "off"), "xc": "LDA" if wl.get("spinpol", "off") == "off" else "LSDA",
            "vna": vna}


def _job_step(ctx, u, orbs, wl, dm, vna, precision):
    spin = wl.get("spinpol", "off")
    job = L.GridStepJob(u, orbs, spin, "LDA" if spin == "off" else "LSDA", None, None, vna)
    job.set_dm(dm)
    ctx.set_precision(precision)
    try:
        job.step()
    finally:
        ctx.set_precision("fp64")
    return job.energies(), job.density(), job.hks()


def _check(name, e, rho, H, ref, natom, pairs_blocks, fp64):
    """Compares a GPU step with the oracle step (H on the listed blocks)."""
    for s in range(len(rho)):
        drho = np.max(np.abs(rho[s] - ref["density"][s]))
        scale_r = np.max(np.abs(ref["density"][s]))
        h, hr = H[s][pairs_blocks], ref["hks"][s][pairs_blocks]
        dh = np.max(np.abs(h - hr))
        scale_h = np.max(np.abs(hr))
        print("%s spin %d: max|drho| %.3e (max rho %.3e), max|dH| %.3e (max H %.3e)"
              % (name, s, drho, scale_r, dh, scale_h))
        if fp64:
            assert drho <= RHO_ABS
            assert dh <= H_ABS
        else:
            assert drho <= TC_REL * scale_r
            assert dh <= TC_REL * scale_h
    de = abs(float(e[4]) - ref["energies"][4]) / natom
    print("%s: |dE_grid| %.3e Ha/atom, E_H1 %.12g vs %.12g" % (name, de, e[0], ref["energies"][0]))
    assert de <= E_ATOM


def test_si64_full_step_vs_oracle():
    """Every pair of the 64-atom cell, FP64 and split-BF16, against the oracle."""
    from lcpgrid.workloads import psd_density_matrices, si64_workload, smooth_vna
    from oracle.cpu_step import CpuGridStep
    wl = si64_workload()
    vna = smooth_vna(wl["ngrid"], wl["latvecs"], wl["vna_seed"])
    ctx = L.Context(0)
    u = L.UCell(1, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"], wl["origin"],
                Total_NumOrbs=wl["numorbs"])
    orbs = L.Set_Orbitals_Grid(wl["paos"], u, ctx=ctx)
    dm = psd_density_matrices(u, wl["dm_seed"], trace=wl["trace"])
    runs = {p: _job_step(ctx, u, orbs, wl, dm, vna, p) for p in ("fp64", "bf16x3")}
    with CpuGridStep(_spec(wl, vna), nproc=min(16, os.cpu_count() or 1)) as cs:
        assert cs.u.Nloop == u.Nloop
        cs.set_dm(dm)
        ref = cs.step()
    allb = np.arange(u.Total_Hsize)
    _check("si64 fp64", *runs["fp64"], ref, wl["natom"], allb, True)
    _check("si64 bf16x3", *runs["bf16x3"], ref, wl["natom"], allb, False)


def test_mx2_lsda_sample_vs_oracle():
    """The 432-atom LSDA cell with D restricted to the pairs among a sample of
    neighbouring atoms (a metal and every atom within 9 bohr of it)."""
    from lcpgrid.workloads import mx2_monolayer, psd_density_matrices, smooth_vna
    from oracle.cpu_step import CpuGridStep
    wl = mx2_monolayer()
    vna = smooth_vna(wl["ngrid"], wl["latvecs"], wl["vna_seed"])
    ctx = L.Context(0)
    u = L.UCell(2, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"], wl["origin"],
                Total_NumOrbs=wl["numorbs"], device=True, ctx=ctx)
    pos = np.asarray(wl["gxyz"])
    lat = np.asarray(wl["latvecs"])
    d = pos - pos[0]
    frac = d @ np.linalg.inv(lat)
    frac[:, :2] -= np.round(frac[:, :2])  # in-plane minimum image
    dist = np.linalg.norm(frac @ lat, axis=1)
    sample = set(np.nonzero(dist <= 9.0)[0].tolist())
    assert 8 <= len(sample) <= 40
    pairs = [p for p in range(u.Nloop) if u.MPI_atom[p] - 1 in sample and u.MPI_natn[p] - 1 in sample]
    dm = psd_density_matrices(u, wl["dm_seed"], nspin=2, trace=wl["trace"])
    keep = np.zeros(u.Total_Hsize, dtype=bool)
    no = np.asarray(wl["numorbs"])
    for p in pairs:
        o = u.block_offset[p]
        keep[o:o + no[u.MPI_atom[p] - 1] * no[u.MPI_natn[p] - 1]] = True
    dm = [np.where(keep, x, 0.0) for x in dm]
    orbs = L.Set_Orbitals_Grid(wl["paos"], u, ctx=ctx)
    runs = {p: _job_step(ctx, u, orbs, wl, dm, vna, p) for p in ("fp64", "bf16x3")}
    del orbs
    with CpuGridStep(_spec(wl, vna), nproc=4, pairs=pairs) as cs:
        cs.set_dm(dm)
        ref = cs.step()
    blocks = np.nonzero(keep)[0]
    _check("mx2 fp64", *runs["fp64"], ref, wl["natom"], blocks, True)
    _check("mx2 bf16x3", *runs["bf16x3"], ref, wl["natom"], blocks, False)
