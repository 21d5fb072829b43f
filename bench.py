#!/usr/bin/env python
"""Benchmark: one SCF grid step of the 64-atom Si precision-form workload.

A step is density assembly from D, FFT Poisson, LDA xc + potential (+ V_na),
grid matrix elements and the FP64 energy terms, on a 96^3 grid with 13
orbitals per atom (see lcpgrid/workloads.py).  Prints one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision bf16x3|fp32|fp64]
    python bench.py --impl reference ...   (the CPU restatement on the host cores)

The headline form is split-BF16 (tensor cores); the FP64 drop-in is timed in
the same run and reported beside it.  --workload si8 runs the 8-atom cell of
the same crystal and grid spacing (48^3), small enough for a profiler capture.

Multi-GPU runs (torchrun) are independent replicas of the same cell: the
path is never sharded, there is no data-path collective.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "lcpaodft.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "ms per SCF grid step & jobs/s (p50/p99) split-BF16 vs FP64, <=1uHa/atom err"
# DRAM bytes per table block of one split-BF16 stage launch (ncu, 8-atom 48^3
# cell: density_tc_kernel 149.7 + 3.3 MB; hamiltonian_tc_kernel 150.1 + 55.9 MB
# and h_reduce_kernel 93.6 + 3.2 MB, over 12076 blocks)
# DRAM bytes (read + write) per table block of a stage's big kernels, from
# one ncu capture of the 64-atom 96^3 cell (96,608 table blocks): the density
# kernel 1,199.0 + 9.4 MB; the H kernel 1,199.9 + 702.5 MB and the
# partial-block reduction 656.1 + 5.0 MB
TRAFFIC_BLOCKS = 96608
TRAFFIC_PER_BLOCK = {"density": (1199.03e6 + 9.38e6) / TRAFFIC_BLOCKS,
                     "hamiltonian": (1199.94e6 + 702.50e6 + 656.07e6 + 5.00e6) / TRAFFIC_BLOCKS}
UNIT = "grid steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16x3", choices=["bf16x3", "fp32", "fp64"])
    ap.add_argument("--workload", default="si64", choices=["si64", "si8", "mx2", "si2"],
                    help="si64: 64-atom Si 96^3 (default); si8: its 8-atom cell at 48^3; mx2: the 432-atom "
                         "LSDA cell; si2: the plain small case (Si2, real Si7.0 tables, 24^3)")
    ap.add_argument("--fp64-steps", type=int, default=5, help="timed steps of the FP64 drop-in form")
    ap.add_argument("--fp32-steps", type=int, default=3,
                    help="timed steps of the FP32 form (CUDA-core FP32 pair contractions), for comparison")
    ap.add_argument("--cpu-steps", type=int, default=2, help="timed full steps of the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--serving", action="store_true", help="run the serving form instead of the step bench")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving section of the step bench line")
    ap.add_argument("--no-force", action="store_true", help="skip the grid force term section of the step bench line")
    ap.add_argument("--no-gga", action="store_true", help="skip the GGA-PBE section of the step bench line")
    ap.add_argument("--no-nc", action="store_true", help="skip the non-collinear section of the step bench line")
    ap.add_argument("--no-si2", action="store_true", help="skip the plain Si2 section of the step bench line")
    ap.add_argument("--xc", default="auto", choices=["auto", "GGA_PBE"],
                    help="xc of the timed step: auto = LDA ('off') / LSDA ('on'), or GGA_PBE")
    ap.add_argument("--serve-structures", type=int, default=24)
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-rates", default="200,500,1000,2000",
                    help="offered Poisson rates of the sweep, jobs/s (comma-separated)")
    ap.add_argument("--serve-max-batch", type=int, default=16, help="requests per batched serving step")
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--serve-saturate", type=int, default=1500, help="requests of the saturated run")
    ap.add_argument("--serve-fp64-requests", type=int, default=60)
    ap.add_argument("--serve-budget-gb", type=float, default=160.0)
    ap.add_argument("--case", choices=["poisson", "tables"],
                    help="one small kernel case for profiler captures: the 96^3 FFT Poisson solve (double-float, "
                         "then FP64), or the 8-atom 48^3 cell's tabulation and split-BF16 table build")
    ap.add_argument("--batching", action="store_true", help="run the batching form instead of the step bench")
    ap.add_argument("--no-batching", action="store_true", help="skip the batching section of the step bench line")
    ap.add_argument("--batch-cells", type=int, default=256)
    ap.add_argument("--batch-seed", type=int, default=4242)
    ap.add_argument("--batch-threads", type=int, default=16, help="host threads building the cells")
    ap.add_argument("--batch-scratch-gb", type=float, default=48.0, help="budget of the partial H blocks")
    ap.add_argument("--batch-autotune", type=int, default=3, help="brick shapes timed per grid shape (0: model)")
    ap.add_argument("--batch-fp64-sample", type=int, default=16, help="cells also stepped in FP64")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers

def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(value, device="cuda"):
    """The largest of the ranks' values (a replica job's time is its slowest
    rank's); the value itself when no process group is up."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world, ms_per_unit):
    """Whole-job units per second of `world` replicas, each taking
    ms_per_unit (the slowest rank's) per unit."""
    return world * 1000.0 / ms_per_unit


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx = float(parts[2])
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def pair_work(ucell):
    """Algorithmic flops of one grid step's pair contractions, counting each
    unordered pair {(i,j,R), (j,i,-R)} once: density (2*NOi*NOj + 2*NOi) and
    H (2*NOi*NOj + NOi) per lens point and spin."""
    import numpy as np
    no = np.asarray(ucell.Total_NumOrbs, dtype=np.float64)
    a = ucell.MPI_atom - 1
    b = ucell.MPI_natn - 1
    olg = ucell.MPI_NumOLG.astype(np.float64)
    # ordered pairs count each unordered pair twice, except self pairs (i,i,0)
    selfp = (a == b) & (ucell.MPI_ncn == 0)
    w = np.where(selfp, 1.0, 0.5)
    dens = float(np.sum(w * olg * (2 * no[a] * no[b] + 2 * no[a])))
    ham = float(np.sum(w * olg * (2 * no[a] * no[b] + no[a])))
    return dens, ham


def force_work(ucell):
    """Algorithmic flops of the grid force term: per ordered pair and lens
    point, D phi_j (2 NO_i NO_j) and the three gradient dot products (6 NO_i)."""
    import numpy as np
    no = np.asarray(ucell.Total_NumOrbs, dtype=np.float64)
    a = ucell.MPI_atom - 1
    b = ucell.MPI_natn - 1
    olg = ucell.MPI_NumOLG.astype(np.float64)
    return float(np.sum(olg * (2 * no[a] * no[b] + 6 * no[a])))


def force3_section(wl, u, dm, vna, reps=5):
    """Force3 (FP64) on the step's cell: gradient tables, then the call as the
    reference makes it (host V and D in, forces out), timed end to end."""
    import numpy as np

    import lcpgrid as L
    ctx = L.Context(0)
    t0 = time.perf_counter()
    orbs = L.Set_dOrbitals_Grid(wl["paos"], u, ctx=ctx)
    ctx.synchronize()
    t_tab = time.perf_counter() - t0
    V = [np.asarray(vna, dtype=np.float64)] * len(dm)
    fn = L.Force3_nospin if len(dm) == 1 else L.Force3_spin
    F = fn(wl["paos"], orbs, V, dm, u)  # warm-up
    t0 = time.perf_counter()
    for _ in range(reps):
        F = fn(wl["paos"], orbs, V, dm, u)
    ms = (time.perf_counter() - t0) / reps * 1e3
    flops = force_work(u) * len(dm)
    fp64 = ctx.probe_fp64_tflops()
    ach = flops / (ms * 1e-3) / 1e12
    try:
        cpu = force3_cpu_baseline(wl, u, len(dm), reps=2)
    except Exception as exc:  # the CPU side must not hide the GPU figures
        cpu = {"value": None, "error": repr(exc)}
    return {"ms_per_call": ms, "calls": reps, "gradient_tabulation_s": t_tab, "cpu_baseline": cpu,
            "max_abs_force": float(np.max(np.abs(F))),
            "roofline": {"bound": "fp64-alu", "achieved": ach, "peak": fp64, "unit": "TFLOP/s", "frac": ach / fp64,
                         "peak_source": "probe: FP64 FMA loop on this GPU",
                         "note": "end to end: includes the host copies of V and D (%.0f MB)"
                                 % (len(dm) * (u.NN + u.Total_Hsize) * 8 / 1e6)}}


def gga_section(wl, u, orbs, dm, vna, steps=10):
    """The same step with GGA-PBE as its xc (the gradient stencil + PBE pass
    and the divergence pass replace the LDA pass), split-BF16 and FP64, and
    the oracle's GGA pass on the same density for the CPU side."""
    import numpy as np
    import torch

    import lcpgrid as L
    from oracle import lcp_oracle as O
    spin = wl.get("spinpol", "off")
    out = {}
    rho = None
    ctx = orbs.ctx
    keep = ctx.precision
    try:
        for prec in ("bf16x3", "fp64"):
            ctx.set_precision(prec)
            job = L.GridStepJob(u, orbs, spin, "GGA_PBE", None, None, vna)
            job.set_dm(dm)
            for _ in range(3):
                job.step()
            st = np.array([job.step_timed() for _ in range(steps if prec == "bf16x3" else 2)])
            med = np.median(st, axis=0)
            # the step as the headline times it (CUDA events on the library's
            # stream; xc beside the Poisson solve); stage_ms come from the
            # sequential timed step
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            nrep = steps if prec == "bf16x3" else 2
            torch.cuda.synchronize()
            ev[0].record()
            for _ in range(nrep):
                job.step()
            ev[1].record()
            torch.cuda.synchronize()
            out[prec] = {"ms_per_step": ev[0].elapsed_time(ev[1]) / nrep, "xc_pass_ms": float(med[2]),
                         "stage_ms": [float(x) for x in med], "stages_sum_ms": float(med.sum()),
                         "E_grid": float(job.energies()[4])}
            if prec == "fp64":
                rho = [x.copy() for x in job.density()]
    finally:
        ctx.set_precision(keep)
    out["err_per_atom_uHa"] = abs(out["bf16x3"]["E_grid"] - out["fp64"]["E_grid"]) / wl["natom"] * 1e6
    out["points_per_s_xc_pass"] = float(u.NN / (out["bf16x3"]["xc_pass_ms"] * 1e-3))
    # the oracle's GGA pass (gradient, PBE, divergence) on one thread, same grid
    gl = O.glatvecs_of(np.asarray(wl["latvecs"], dtype=np.float64), u.Ngrid)
    t0 = time.perf_counter()
    O.set_xc_grid_gga(spin, u.Ngrid, None, rho, O.calc_diff_coef(gl))
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": cpu_s * 1e3, "unit": "ms per GGA xc pass", "cores": 1, "kind": "port",
                           "sample": "the oracle's gradient + PBE + divergence pass on the same %dx%dx%d density"
                                     % tuple(u.Ngrid)}
    out["roofline"] = {"bound": "fp64-alu", "note": "the PBE pass issues FP64 instructions at 85% of the FP64 "
                       "pipe's peak and the divergence pass at 80% (ncu); DRAM traffic is a few bytes per point"}
    return out


def force3_cpu_baseline(wl, ucell_gpu, nspin, reps=2):
    """The oracle's Force3 (per-pair D phi_j and gradient dot products, as
    _Calc_Force3_Blocked_Kernel!) on the pairs among the first 8 atoms, one
    host core, extrapolated to the cell by the force work per pair."""
    import numpy as np
    from oracle import lcp_oracle as O
    W = _inputs()
    psd_density_matrices_oracle, smooth_vna = W.psd_density_matrices_oracle, W.smooth_vna
    sample = [p for p in range(ucell_gpu.Nloop)
              if ucell_gpu.MPI_atom[p] <= SAMPLE_ATOMS and ucell_gpu.MPI_natn[p] <= SAMPLE_ATOMS]
    no = np.asarray(wl["numorbs"], dtype=np.float64)
    a = ucell_gpu.MPI_atom - 1
    b = ucell_gpu.MPI_natn - 1
    wt = ucell_gpu.MPI_NumOLG.astype(np.float64) * (2 * no[a] * no[b] + 6 * no[a])
    w_sample, w_total = float(wt[sample].sum()), float(wt.sum())
    u = O.UCell(1, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"], wl["origin"],
                total_numorbs=wl["numorbs"], pair_subset=sample)
    pao = wl["paos"][0]
    opao = O.PAO(pao.Spe_MaxL_Basis, pao.Spe_Num_Basis, pao.Spe_PAO_RV, pao.Spe_PAO_RWF)
    first = set(range(SAMPLE_ATOMS))
    orbs = O.set_orbitals_grid([opao], u, atoms=first)
    dorbs = O.set_dorbitals_grid([opao], u, atoms=first)
    dm = psd_density_matrices_oracle(u, wl["dm_seed"], trace=wl["trace"])[0]
    vna = smooth_vna(wl["ngrid"], wl["latvecs"], wl["vna_seed"])
    t0 = time.perf_counter()
    for _ in range(reps):
        O.calc_force3("off", u, orbs, dorbs, [vna], [dm])
    t = (time.perf_counter() - t0) / reps
    ms = t * w_total / w_sample * nspin * 1e3
    return {"value": ms, "unit": "ms per Force3 call", "cores": 1, "kind": "port",
            "sample": "numpy oracle Force3 over the %d pairs among atoms 1-%d (%.2f%% of the force work) x %d, "
                      "extrapolated by (2 NO_i NO_j + 6 NO_i) NumOLG" % (len(sample), SAMPLE_ATOMS,
                                                                        100 * w_sample / w_total, reps)}


def nc_section(wl, u, orbs, vna, steps=10):
    """The same cell with the non-collinear channel set: four D/density/V/H
    channels, diagonalize_nc_density!, LSDA rotated into four potentials;
    split-BF16 step time (CUDA events), FP64 step time, energy error."""
    import torch

    import lcpgrid as L
    from lcpgrid.workloads import psd_nc_density_matrices
    dm = psd_nc_density_matrices(u, wl["dm_seed"], trace=wl["trace"])
    out = {}
    ctx = orbs.ctx
    keep = ctx.precision
    try:
        for prec in ("bf16x3", "fp64"):
            ctx.set_precision(prec)
            job = L.GridStepJob(u, orbs, "nc", "LSDA", None, None, vna)
            job.set_dm(dm)
            for _ in range(2 if prec == "fp64" else 3):
                job.step()
            nrep = steps if prec == "bf16x3" else 1
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            torch.cuda.synchronize()
            ev[0].record()
            for _ in range(nrep):
                job.step()
            ev[1].record()
            torch.cuda.synchronize()
            out[prec] = {"ms_per_step": ev[0].elapsed_time(ev[1]) / nrep, "E_grid": float(job.energies()[4])}
    finally:
        ctx.set_precision(keep)
    out["err_per_atom_uHa"] = abs(out["bf16x3"]["E_grid"] - out["fp64"]["E_grid"]) / wl["natom"] * 1e6
    out["note"] = "four channels: one tensor-core density pass and one H pass per channel"
    return out


# ------------------------------------------------------------------ CPU baseline (oracle port)

SAMPLE_ATOMS = 8  # the Force3 CPU sample: pairs among the first conventional cell's 8 atoms


def _inputs():
    """lcpgrid/workloads.py (with pao.py) loaded by path without importing the
    lcpgrid package, whose __init__ loads liblcpgrid.so: the reference arm and
    the CPU baseline build their inputs without the product library."""
    import importlib.util
    import types
    name = "_lcp_inputs"
    if name + ".workloads" in sys.modules:
        return sys.modules[name + ".workloads"]
    pkgdir = os.path.join(PKG, "lcpgrid")
    pkg = types.ModuleType(name)
    pkg.__path__ = [pkgdir]
    sys.modules[name] = pkg
    for mod in ("pao", "workloads"):
        spec = importlib.util.spec_from_file_location(name + "." + mod, os.path.join(pkgdir, mod + ".py"))
        m = importlib.util.module_from_spec(spec)
        sys.modules[spec.name] = m
        spec.loader.exec_module(m)
    return sys.modules[name + ".workloads"]


SPECIES_TABLES = os.path.join(ROOT, "tests", "golden", "species_tables.npz")


def cpu_spec(wl):
    """Host inputs of the CPU grid step (oracle/cpu_step.py) for a workload."""
    import numpy as np
    from oracle import lcp_oracle as O
    W = _inputs()
    spin = wl.get("spinpol", "off")
    spec = {k: wl[k] for k in ("latvecs", "natom", "atom2spe", "gxyz", "cut", "ngrid", "origin", "numorbs")}
    spec["paos"] = [(q.Spe_MaxL_Basis, q.Spe_Num_Basis, q.Spe_PAO_RV, q.Spe_PAO_RWF) for q in wl["paos"]]
    spec["spinpol"] = spin
    spec["xc"] = "LDA" if spin == "off" else "LSDA"
    if "pcc" in wl:  # the plain case: the reference's own atomic and partial-core densities
        u = O.UCell(1, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"],
                    wl["origin"], total_numorbs=wl["numorbs"], pair_subset=[])
        q, c = wl["paos"][0], wl["pcc"]
        ad, pc, _ = O.set_adenpcc_grid("off", wl["init_nspin"], [[0, 0, 0, 0]] * wl["natom"],
                                       [(q.Spe_PAO_XV, q.Spe_PAO_RV, q.Spe_Atomic_Den)],
                                       [(c.Spe_VPS_XV, c.Spe_VPS_RV, c.Spe_Atomic_PCC)], u)
        spec["aden"], spec["pcc"] = ad, pc
    else:
        spec["vna"] = W.smooth_vna(wl["ngrid"], wl["latvecs"], wl["vna_seed"])
    return spec


def cpu_step_run(wl, steps, warmup=1, nproc=None):
    """The reference's grid step restated on the host cores (oracle/cpu_step.py:
    one process per core as one MPI rank each, the reference's pair split,
    per-pair 512-point blocks with single-threaded BLAS, the rank grids summed,
    Poisson, xc and energies on the full grid), timed over `steps` full steps
    after `warmup`.  Returns (result dict, last step's output)."""
    import numpy as np
    from oracle.cpu_step import CpuGridStep
    W = _inputs()
    spec = cpu_spec(wl)
    with CpuGridStep(spec, nproc=nproc) as cs:
        nspin = cs.nspin
        dm = W.psd_density_matrices_oracle(cs.u, wl["dm_seed"], nspin=nspin, trace=wl["trace"])
        cs.set_dm(dm)
        for _ in range(warmup):
            out = cs.step()
        per, stages = [], []
        for _ in range(steps):
            out = cs.step()
            per.append(out["seconds"]["step"])
            stages.append(out["seconds"])
        ms = float(np.mean(per)) * 1e3
        res = {"value": 1000.0 / ms, "unit": UNIT, "cores": cs.nproc, "kind": "port", "ms_per_step": ms,
               "stage_ms": {k: float(np.mean([x[k] for x in stages])) * 1e3
                            for k in ("density", "poisson", "xc_vpot", "hamiltonian", "energies")},
               "setup_s": cs.setup_s, "E_grid": float(out["energies"][4]),
               "sample": "full step, no extrapolation: %s, all %d pairs, %d timed steps after %d warm-up; "
                         "oracle restatement with one process per host core as one MPI rank each, the "
                         "reference's weighted contiguous pair split, 512-point blocks, 1 BLAS thread per "
                         "process; no product library loaded" % (wl["name"], cs.u.Nloop, steps, warmup)}
    return res, out


def cpu_baseline(wl, steps=2):
    """cpu_baseline of the GPU line: the full CPU step on all host cores.
    Spawned processes (this runs after GPU work)."""
    res, _ = cpu_step_run(wl, steps)
    return res


# ------------------------------------------------------------------ GPU arm

def build_workload(ctx, wl):
    import lcpgrid as L
    from lcpgrid.workloads import psd_density_matrices, smooth_vna
    t0 = time.perf_counter()
    nspin = 2 if wl.get("spinpol", "off") == "on" else 1
    u = L.UCell(nspin, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"], wl["origin"],
                Total_NumOrbs=wl["numorbs"])
    t_geom = time.perf_counter() - t0
    t0 = time.perf_counter()
    orbs = L.Set_Orbitals_Grid(wl["paos"], u, ctx=ctx)
    ctx.synchronize()
    t_tab = time.perf_counter() - t0
    dm = psd_density_matrices(u, wl["dm_seed"], nspin=nspin, trace=wl["trace"])
    if "pcc" in wl:  # the plain case: atomic and partial-core densities, no V_na
        ad, pc, _ = L.Set_AdenPCC_Grid("off", wl["init_nspin"], None, wl["paos"], [wl["pcc"]], u, ctx=ctx)
        wl["_aden_pcc"] = (ad, pc)
        vna = None
    else:
        vna = smooth_vna(wl["ngrid"], wl["latvecs"], wl["vna_seed"])
    return u, orbs, dm, vna, t_geom, t_tab


def workload(args):
    import numpy as np
    W = _inputs()
    if args.workload == "si8":
        return W.si64_workload(nrep=1, ngrid=(48, 48, 48))
    if args.workload == "mx2":
        return W.mx2_monolayer()
    if args.workload == "si2":
        return W.si2_workload(np.load(SPECIES_TABLES))
    return W.si64_workload()


def run_ours(args):
    import numpy as np
    import torch

    import lcpgrid as L

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    wl = workload(args)
    ctx = L.Context(local)
    u, orbs, dm, vna, t_geom, t_tab = build_workload(ctx, wl)
    # the same UCell with its sphere and overlap lists built on the GPU
    t_geom_dev = []
    for _ in range(2):
        t0 = time.perf_counter()
        L.UCell(u.Nspin, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"],
                wl["origin"], Total_NumOrbs=wl["numorbs"], device=True, ctx=ctx)
        t_geom_dev.append(time.perf_counter() - t0)
    # a dedicated (non-default) stream: the library launches on it and the
    # CUDA events below are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    # FP64 reference energy of this step (the drop-in), for the error of other forms
    spin = wl.get("spinpol", "off")
    nspin = len(dm)
    xc = args.xc if args.xc != "auto" else ("LDA" if spin == "off" else "LSDA")
    ad, pc = wl.get("_aden_pcc", (None, None))
    job = L.GridStepJob(u, orbs, spin, xc, ad, pc, vna)
    job.set_dm(dm)
    ctx.set_precision("fp64")
    job.step()
    e_fp64 = job.energies()
    h_fp64 = [h.copy() for h in job.hks()]
    rho_fp64 = [r.copy() for r in job.density()]
    fp64_ms = None
    if args.precision != "fp64" and args.fp64_steps > 0:
        fe = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        fe[0].record(stream)
        for _ in range(args.fp64_steps):
            job.step()
        fe[1].record(stream)
        torch.cuda.synchronize()
        fp64_ms = fe[0].elapsed_time(fe[1]) / args.fp64_steps
    # the FP32 form of the same step (density and H in FP32 on the CUDA
    # cores, the rest FP64), the third precision of the comparison
    fp32_form = None
    if args.precision == "bf16x3" and args.fp32_steps > 0:
        ctx.set_precision("fp32")
        job.step()
        e_fp32 = job.energies()
        fe = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        fe[0].record(stream)
        for _ in range(args.fp32_steps):
            job.step()
        fe[1].record(stream)
        torch.cuda.synchronize()
        fp32_form = {"ms_per_step": fe[0].elapsed_time(fe[1]) / args.fp32_steps, "steps": args.fp32_steps,
                     "err_per_atom_uHa": abs(e_fp32[4] - e_fp64[4]) / u.Natom * 1e6,
                     "rel_err": abs(e_fp32[4] - e_fp64[4]) / abs(e_fp64[4])}
    ctx.set_precision(args.precision)

    for _ in range(max(3, args.warmup)):
        job.step()
    torch.cuda.synchronize()
    stages = job.step_timed()

    # timed, device-resident: inputs larger than L2 (phi tables ~1 GB)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    l0 = ctx.launch_count
    ev[0].record(stream)
    for k in range(args.steps):
        job.step()
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    launches = ctx.launch_count - l0
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    per = np.array([ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)])
    total_ms = max_over_ranks(float(ev[0].elapsed_time(ev[-1])))
    e_now = job.energies()
    h_now = job.hks()
    rho_now = job.density()

    # e2e through the public API: pinned host D in, H and energies out, every step
    pin_dm = [torch.empty(u.Total_Hsize, dtype=torch.float64, pin_memory=True) for _ in range(nspin)]
    for c in range(nspin):
        pin_dm[c].numpy()[:] = dm[c]
    pin_h = [torch.empty(u.Total_Hsize, dtype=torch.float64, pin_memory=True) for _ in range(nspin)]
    pin_e = torch.empty(5, dtype=torch.float64, pin_memory=True)
    e2e_n = max(1, args.e2e_steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_n):
        job.set_dm([x.numpy() for x in pin_dm])
        job.step()
        job.energies_async(pin_e.numpy())  # completed by the synchronising H read below
        job.hks(out=[x.numpy() for x in pin_h])
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_n)
    e2e_e = pin_e.numpy().copy()

    # the tensor-core kernels alone (CUDA events around each launch), median of 5 steps
    tc_ms = None
    if args.precision == "bf16x3":
        tc_ms = np.median(np.array([job.tc_kernel_ms() for _ in range(5)]), axis=0)

    dens_flops, ham_flops = pair_work(u)
    dens_flops *= nspin  # the stages cover every spin channel
    ham_flops *= nspin
    peaks, psrc = measured_peaks()
    # dominant kernel: the larger of the two pair contractions
    names = ["density", "poisson", "xc_vpot", "energy_sums", "hamiltonian", "dot_finish"]
    dom = int(np.argmax(stages))
    dom_flops = dens_flops if names[dom] == "density" else ham_flops
    if args.precision == "fp64":
        fp64_peak = ctx.probe_fp64_tflops()
        roof = {"bound": "fp64-alu", "kernel": names[dom], "achieved": dom_flops / (stages[dom] * 1e-3) / 1e12,
                "peak": fp64_peak, "unit": "TFLOP/s", "peak_source": "probe: FP64 FMA loop on this GPU",
                "traffic": None}
    else:
        pk = peaks.get("bf16_tflops_sustained", 1700.0)
        roof = {"bound": "tensor", "kernel": names[dom], "achieved": dom_flops / (stages[dom] * 1e-3) / 1e12,
                "peak": pk, "unit": "TFLOP/s", "peak_source": psrc + " bf16_tflops_sustained", "traffic": None}
        if tc_ms is not None:
            kms = float(tc_ms[0] if names[dom] == "density" else tc_ms[1])
            roof["kernel"] = "density_tc_kernel" if names[dom] == "density" else "hamiltonian_tc_kernel"
            roof["kernel_ms"] = kms
            roof["stage_ms"] = float(stages[dom])
            roof["achieved_stage"] = roof["achieved"]
            roof["achieved"] = dom_flops / (kms * 1e-3) / 1e12
        if args.precision == "bf16x3":
            # DRAM bytes (read + write) per launch of the stage's big kernels,
            # measured with ncu on the 64-atom cell and scaled by table blocks
            # (every brick image is one block)
            per_block = TRAFFIC_PER_BLOCK.get(names[dom])
            nblocks = u.brick_info()["blocks"]
            if per_block is not None:
                roof["traffic"] = per_block * nblocks
                roof["traffic_gbs"] = roof["traffic"] / (stages[dom] * 1e-3) / 1e9
                roof["traffic_frac_hbm"] = roof["traffic_gbs"] / peaks.get("hbm_gbs", 6800.0)
                roof["traffic_note"] = ("ncu DRAM read+write of the stage's kernels per table block (capture "
                                        "of %d blocks), x %d blocks here" % (TRAFFIC_BLOCKS, nblocks))
                roof["note"] = ("FP64-algorithm flops (folded pairs, no padding) over the kernel's launch time "
                                "(achieved_stage: over the stage); split-BF16 forms 8 bf16 products on "
                                "16-orbital blocks, so frac <= ~1/8 before padding")
    roof["frac"] = roof["achieved"] / roof["peak"] if roof["peak"] else None

    # tabulation and Poisson against the HBM roofline (algorithmic bytes:
    # tables written + sphere indices read; FP64 tables read + three BF16
    # parts written; 80 bytes per grid point per solve)
    tab_ms, split_ms = orbs.timings()
    gridn = np.asarray(u.GridN_Atom, dtype=np.float64)
    elems = float(np.sum(gridn * np.asarray(wl["numorbs"], dtype=np.float64)))
    hbm = peaks.get("hbm_gbs", 6800.0)
    tab_bytes = elems * 8 + float(gridn.sum()) * 8
    split_bytes = elems * (8 + 6)
    pois_bytes = 80.0 * u.NN
    gbs = lambda b, ms: b / (ms * 1e-3) / 1e9 if ms else None
    tabulation = {"kernel_ms": tab_ms, "bytes": tab_bytes, "gbs": gbs(tab_bytes, tab_ms),
                  "split_tables_ms": split_ms, "split_bytes": split_bytes, "split_gbs": gbs(split_bytes, split_ms),
                  "peak_gbs": hbm, "peak_source": psrc + " hbm_gbs",
                  "note": "FP64 tables written + sphere indices read (bytes); split-BF16 build: FP64 tables read and "
                          "three BF16 parts written.  The FP64 tabulation is FP64-pipe bound (spline and Y_lm per "
                          "point), not HBM bound"}
    tabulation["frac"] = tabulation["gbs"] / hbm if tabulation["gbs"] else None
    tabulation["split_frac"] = tabulation["split_gbs"] / hbm if tabulation["split_gbs"] else None
    poisson = {"ms": float(stages[1]), "bytes": pois_bytes, "gbs": gbs(pois_bytes, float(stages[1])),
               "peak_gbs": hbm, "transform": "fp64" if args.precision == "fp64" else "double-float (FP32 pipe), FP64 "
               "scaling", "note": "80 bytes per grid point per solve (five passes over the half spectrum, source and "
               "output); the spectrum (%.0f MB) %s" % (u.NN * 8 / 1e6, "stays in L2" if u.NN * 8 < 64e6 else
                                                        "exceeds L2")}
    poisson["frac"] = poisson["gbs"] / hbm if poisson["gbs"] else None

    ms_step = total_ms / args.steps
    line = {
        "metric": METRIC, "value": replica_rate(world, ms_step), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_step,
        "p50_ms": float(np.percentile(per, 50)), "p99_ms": float(np.percentile(per, 99)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp32": "f32", "bf16x3": "bf16x3/f32-acc"}[args.precision],
        "data": "synthetic (seeded: Gaussian radial functions, PSD D, smooth V_na)",
        "config": {"workload": wl["name"], "atoms": wl["natom"], "orbitals_per_atom": sorted(set(wl["numorbs"])),
                   "ngrid": list(wl["ngrid"]), "pairs": int(u.Nloop), "folded_pairs": int(u.n_unique),
                   "lens_points": int(u.sum_numolg), "precision": args.precision, "spinpol": spin,
                   "xc": xc,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2 (phi tables %.0f MB)"
                         % (sum(np.asarray(u.GridN_Atom, float) * np.asarray(wl["numorbs"])) * 8 / 1e6)},
        "stage_ms": dict(zip(names, [float(x) for x in stages])),
        "setup_s": {"ucell_host": t_geom, "ucell_device": min(t_geom_dev), "tabulation": t_tab},
        "roofline": roof,
        "tabulation": tabulation,
        "poisson": poisson,
        "e2e": {"value": replica_rate(world, e2e_s * 1e3), "unit": UNIT, "h2d_bytes_per_step": int(nspin * u.Total_Hsize * 8),
                "d2h_bytes_per_step": int(nspin * u.Total_Hsize * 8 + 40), "ms_per_step": e2e_s * 1e3},
        "energy": {"E_grid": float(e_now[4]), "E_grid_fp64": float(e_fp64[4]),
                   "err_per_atom_uHa": abs(float(e_now[4] - e_fp64[4])) / wl["natom"] * 1e6,
                   "rel_err": abs(float(e_now[4] - e_fp64[4])) / abs(float(e_fp64[4])),
                   "max_abs_dH": float(max(np.max(np.abs(a - b)) for a, b in zip(h_now, h_fp64))),
                   "max_abs_dH_note": "each form with its own V; the H bound of 1e-7 Ha is the FP64 drop-in's, "
                                      "the precision form states its error",
                   "max_abs_drho": float(max(np.max(np.abs(a - b)) for a, b in zip(rho_now, rho_fp64))),
                   "max_abs_rho": float(max(np.max(np.abs(b)) for b in rho_fp64)),
                   "terms": ["E_H1", "E_xc1 up", "E_xc1 down", "sum <D,H>", "E_grid"],
                   "terms_rel_err": [abs(float(a - b)) / max(abs(float(b)), 1e-300) for a, b in zip(e_now, e_fp64)],
                   "terms_this_form": [float(x) for x in e_now], "terms_fp64": [float(x) for x in e_fp64]},
        "fp64_dropin": None if fp64_ms is None else {
            "ms_per_step": fp64_ms, "steps": args.fp64_steps, "speedup_of_this_form": fp64_ms / ms_step},
        "fp32_form": fp32_form,
        "clocks": clk,
        "gpu_launches": int(launches),
        "gpu_launches_note": "kernels of this library per timed region (the FFT Poisson solve is 5 of them per step)",
    }
    plain = args.workload == "si2"
    if rank == 0 and not args.no_force and world == 1 and not plain:
        try:
            line["force3"] = force3_section(wl, u, dm, vna)
        except Exception as exc:  # the force section must not hide the step line
            line["force3"] = {"error": repr(exc)}
    if rank == 0 and not args.no_gga and world == 1 and not plain:
        try:
            line["gga_pbe"] = gga_section(wl, u, orbs, dm, vna)
        except Exception as exc:  # the GGA section must not hide the step line
            line["gga_pbe"] = {"error": repr(exc)}
    if rank == 0 and not args.no_nc and world == 1 and spin == "off" and not plain:
        try:
            line["nc"] = nc_section(wl, u, orbs, vna)
        except Exception as exc:  # the nc section must not hide the step line
            line["nc"] = {"error": repr(exc)}
    if rank == 0 and not args.no_serving and world == 1 and not plain:
        # the serving form on the same GPU: Poisson stream of mixed-size structures
        try:
            line["serving"] = serving(args)
        except Exception as exc:  # the serving run must not hide the step line
            line["serving"] = {"error": repr(exc)}
    if rank == 0 and not args.no_batching and world == 1 and not plain:
        # the batching form on the same GPU: 256 mixed cells in one batched step
        try:
            del job
            torch.cuda.synchronize()
            line["batching"] = batching(args)
        except Exception as exc:  # the batching run must not hide the step line
            line["batching"] = {"error": repr(exc)}
    if rank == 0 and world == 1 and args.workload == "si64" and not args.no_si2:
        try:
            line["plain_si2"] = si2_section(args)
        except Exception as exc:  # the plain case must not hide the step line
            line["plain_si2"] = {"error": repr(exc)}
    if rank == 0 and not args.no_cpu_baseline and args.workload == "mx2":
        line["cpu_baseline"] = {"value": None, "note": "the CPU baseline is timed on the 64-atom cell (the "
                                                       "default workload) and the Si2 cell"}
    elif rank == 0 and not args.no_cpu_baseline:
        try:
            cb, cout = cpu_step_run(wl, args.cpu_steps)
            # the full-size FP64 check: the GPU's FP64 step against the CPU restatement
            cb["vs_gpu_fp64"] = {
                "max_abs_drho": float(max(np.max(np.abs(a - b)) for a, b in zip(rho_fp64, cout["density"]))),
                "max_abs_dH": float(max(np.max(np.abs(a - b)) for a, b in zip(h_fp64, cout["hks"]))),
                "dE_per_atom_uHa": abs(float(e_fp64[4]) - cout["energies"][4]) / wl["natom"] * 1e6}
            line["cpu_baseline"] = cb
        except Exception as exc:  # the baseline must not hide the GPU line
            line["cpu_baseline"] = {"value": None, "error": repr(exc)}
    if rank == 0:
        emit(line)
    if world > 1:
        dist.destroy_process_group()


def si2_section(args, steps=50):
    """The plain small case: the Si2 primitive cell with the real Si7.0-s2p2d1
    tables, LDA with the reference's atomic and partial-core densities, 24^3.
    The whole step on the GPU in FP64 and in split-BF16 (CUDA events on the
    library's stream, device-resident) beside the full CPU step on the host
    cores, with the GPU results against the CPU restatement."""
    import numpy as np
    import torch

    import lcpgrid as L
    wl = workload(argparse.Namespace(workload="si2"))
    ctx = L.Context(0)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    u, orbs, dm, vna, _, _ = build_workload(ctx, wl)
    ad, pc = wl["_aden_pcc"]
    job = L.GridStepJob(u, orbs, "off", "LDA", ad, pc, None)
    job.set_dm(dm)
    out, res = {}, {}
    for prec in ("fp64", "bf16x3"):
        ctx.set_precision(prec)
        for _ in range(5):
            job.step()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        for _ in range(steps):
            job.step()
        ev[1].record(stream)
        torch.cuda.synchronize()
        res[prec] = (job.energies(), job.density()[0].copy(), job.hks()[0].copy())
        out[prec] = {"ms_per_step": ev[0].elapsed_time(ev[1]) / steps}
    cb, cout = cpu_step_run(wl, 3)
    for prec, (e, rho, H) in res.items():
        out[prec].update({"E_grid": float(e[4]),
                          "dE_per_atom_uHa_vs_cpu": abs(float(e[4]) - cout["energies"][4]) / 2 * 1e6,
                          "max_abs_drho_vs_cpu": float(np.max(np.abs(rho - cout["density"][0]))),
                          "max_abs_dH_vs_cpu": float(np.max(np.abs(H - cout["hks"][0])))})
    out["cpu"] = {"ms_per_step": cb["ms_per_step"], "cores": cb["cores"], "E_grid": cb["E_grid"]}
    out["config"] = {"workload": wl["name"], "pairs": int(u.Nloop), "ngrid": list(wl["ngrid"])}
    return out


def emit(line):
    """Prints the JSON line on stdout, with its bulky lists (the brick-shape
    autotune log, the serving pool's per-structure lists) moved to lines on
    stderr, and a compact summary of every form's numbers as the line's last
    key."""
    bat = line.get("batching")
    if isinstance(bat, dict) and "autotune" in bat:
        print(json.dumps({"batching_autotune": bat.pop("autotune")}), file=sys.stderr)
    srv = line.get("serving")
    if isinstance(srv, dict):
        side = {}
        if isinstance(srv.get("pool_step_ms"), dict) and "per_structure" in srv["pool_step_ms"]:
            side["pool_step_ms_per_structure"] = srv["pool_step_ms"].pop("per_structure")
        if isinstance(srv.get("structures"), dict) and "atoms" in srv["structures"]:
            side["structure_atoms"] = srv["structures"].pop("atoms")
        if side:
            print(json.dumps({"serving_lists": side}), file=sys.stderr)
    line["summary"] = summary(line)
    print(json.dumps(line))


def summary(line):
    """The headline numbers of every form, short keys (ms unless named)."""
    def g(d, *keys):
        for k in keys:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return float("%.5g" % d) if isinstance(d, float) else d
    s = {"step": g(line, "ms_per_step"), "e2e": g(line, "e2e", "ms_per_step"),
         "fp64": g(line, "fp64_dropin", "ms_per_step"), "fp32": g(line, "fp32_form", "ms_per_step"),
         "err_uHa_atom": g(line, "energy", "err_per_atom_uHa"), "max_dH": g(line, "energy", "max_abs_dH"),
         "max_drho": g(line, "energy", "max_abs_drho"), "roof_frac": g(line, "roofline", "frac"),
         "roof_traffic_frac_hbm": g(line, "roofline", "traffic_frac_hbm"),
         "tab_ms": g(line, "tabulation", "kernel_ms"), "tab_frac": g(line, "tabulation", "frac"),
         "split_tab_ms": g(line, "tabulation", "split_tables_ms"), "split_tab_frac": g(line, "tabulation", "split_frac"),
         "poisson_ms": g(line, "poisson", "ms"), "poisson_frac": g(line, "poisson", "frac"),
         "cpu_full_step": g(line, "cpu_baseline", "ms_per_step"), "cpu_cores": g(line, "cpu_baseline", "cores"),
         "cpu_vs_gpu_fp64_dE_uHa": g(line, "cpu_baseline", "vs_gpu_fp64", "dE_per_atom_uHa"),
         "cpu_vs_gpu_fp64_drho": g(line, "cpu_baseline", "vs_gpu_fp64", "max_abs_drho"),
         "cpu_vs_gpu_fp64_dH": g(line, "cpu_baseline", "vs_gpu_fp64", "max_abs_dH"),
         "si2_fp64": g(line, "plain_si2", "fp64", "ms_per_step"), "si2_bf16": g(line, "plain_si2", "bf16x3", "ms_per_step"),
         "si2_cpu": g(line, "plain_si2", "cpu", "ms_per_step"),
         "si2_fp64_dE_uHa": g(line, "plain_si2", "fp64", "dE_per_atom_uHa_vs_cpu"),
         "force3": g(line, "force3", "ms_per_call"), "gga": g(line, "gga_pbe", "bf16x3", "ms_per_step"),
         "gga_err_uHa": g(line, "gga_pbe", "err_per_atom_uHa"), "nc": g(line, "nc", "bf16x3", "ms_per_step"),
         "nc_fp64": g(line, "nc", "fp64", "ms_per_step"),
         "batch_ms": g(line, "batching", "ms_per_step"), "batch_cells_s": g(line, "batching", "value"),
         "batch_vs_1by1": g(line, "batching", "batch_speedup_vs_one_by_one"),
         "batch_err_uHa": g(line, "batching", "fp64_per_cell_sample", "max_err_per_atom_uHa")}
    sv = line.get("serving")
    if isinstance(sv, dict):
        s["serve_sat_bf16"] = g(sv, "saturated_bf16x3", "jobs_per_s")
        s["serve_sat_fp64"] = g(sv, "saturated_fp64_dropin", "jobs_per_s")
        s["serve_sat_unbatched"] = g(sv, "saturated_bf16x3_unbatched", "jobs_per_s")
        s["serve_back_to_back"] = g(sv, "pool_step_ms", "jobs_per_s_back_to_back")
        s["serve_vs_fp64"] = g(sv, "jobs_per_s_vs_fp64")
        s["serve_err_uHa"] = g(sv, "max_err_per_atom_uHa")
        s["serve_sweep"] = [[g(r, "offered_rate"), g(r, "jobs_per_s"), g(r, "p50_ms"), g(r, "p99_ms")]
                            for r in sv.get("sweep", [sv.get("stream")]) if isinstance(r, dict)]
    return {k: v for k, v in s.items() if v is not None}


def run_reference(args):
    """The reference arm: the reference's grid step on the host cores (the
    oracle restatement of its MPI-parallel algorithm, oracle/cpu_step.py), on
    this arm's workload, metric and unit; W untimed and K timed full steps.
    Nothing of the product library is loaded.  Under torchrun only rank 0
    runs."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    wl = workload(args)
    t0 = time.perf_counter()
    cb, _ = cpu_step_run(wl, args.steps, warmup=args.warmup)
    wall = time.perf_counter() - t0
    v = cb["value"]
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": cb["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": wl["name"], "atoms": wl["natom"], "ngrid": list(wl["ngrid"]), "precision": "fp64"},
        "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
        "note": "Julia is not available on this machine; the reference's CPU path is timed through its numpy "
                "restatement (oracle/cpu_step.py): every pair of the cell, one process per host core as one MPI "
                "rank each, measured full steps with no extrapolation; liblcpgrid.so is not loaded"}))


# ------------------------------------------------------------------ serving form

def serving(args, wl_pool=None):
    """The serving form: a pool of device-resident structures (2-216 atoms,
    log-uniform), grid-step requests arriving as Poisson streams at each
    offered rate of `--serve-rates` for `--serve-seconds`, served by
    lcp_server in split-BF16 with `--serve-slots` slots, each stepping the
    requests it takes as one batched step (continuous batching, up to
    `--serve-max-batch` requests).  Reports per rate the served jobs/s,
    submission-to-result latency p50/p99 and the mean batch, the saturated
    throughput of the same pool in split-BF16 and in the FP64 drop-in (one
    structure at a time), and the worst total-energy error of a structure vs
    FP64."""
    import numpy as np
    import torch

    import lcpgrid as L
    from lcpgrid.workloads import psd_density_matrices, serving_pool, smooth_vna

    pool = wl_pool or serving_pool(args.serve_structures)
    ctx = L.Context(0)
    jobs, dms, natoms = [], [], []
    t0 = time.perf_counter()
    for w in pool:
        # sphere and overlap lists built on the GPU (the same lists as the host build)
        u = L.UCell(1, w["latvecs"], w["natom"], w["atom2spe"], w["gxyz"], w["cut"], w["ngrid"], w["origin"],
                    Total_NumOrbs=w["numorbs"], device=True, ctx=ctx)
        orbs = L.Set_Orbitals_Grid(w["paos"], u, ctx=ctx)
        vna = smooth_vna(w["ngrid"], w["latvecs"], w["vna_seed"])
        jobs.append(L.GridStepJob(u, orbs, "off", "LDA", None, None, vna))
        dms.append(psd_density_matrices(u, w["dm_seed"], trace=w["trace"]))
        natoms.append(w["natom"])
    t_setup = time.perf_counter() - t0

    # every structure stepped alone (split-BF16, CUDA events): the pool's mean
    # device time per request, i.e. the jobs/s of a GPU that runs one request
    # after another with no host gaps
    tctx = L.Context(0, precision="bf16x3")
    tstream = torch.cuda.Stream()
    tctx.set_stream(tstream.cuda_stream)
    alone_ms = []
    for j, d in zip(jobs, dms):
        j.set_dm(d)
        j.step(tctx)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        ev[0].record(tstream)
        for _ in range(5):
            j.step(tctx)
        ev[1].record(tstream)
        torch.cuda.synchronize()
        alone_ms.append(ev[0].elapsed_time(ev[1]) / 5)
    tctx.close()

    def run_server(precision, nslots, rate, seconds, max_requests, max_batch=None):
        srv_max_batch = (args.serve_max_batch if max_batch is None else max_batch) if precision == "bf16x3" else 1
        srv = L.Server(0, nslots=nslots, precision=precision, budget_bytes=args.serve_budget_gb * 1e9,
                       max_batch=srv_max_batch)
        ids = [srv.add(j) for j in jobs]
        # warm-up: every structure once (split-BF16 tables, FFT plans, workspaces)
        for sid in ids:
            srv.submit(sid, dms[sid], tag=sid)
        got = 0
        energies = {}
        while got < len(ids):
            for tag, e, lat in srv.poll(wait_ms=5000):
                energies[tag] = e
                got += 1
        rng = np.random.default_rng(99)
        if rate > 0:
            gaps = rng.exponential(1.0 / rate, size=max_requests)
            n_req = int(min(max_requests, np.searchsorted(np.cumsum(gaps), seconds)))
        else:
            gaps = np.zeros(max_requests)
            n_req = max_requests
        picks = rng.integers(0, len(ids), size=n_req)
        lat_ms, done = [], 0
        t_start = time.perf_counter()
        t_next = t_start
        for k in range(n_req):
            t_next += gaps[k]
            while True:
                now = time.perf_counter()
                if now >= t_next:
                    break
                for _tag, _e, lat in srv.poll(wait_ms=0):
                    lat_ms.append(lat)
                time.sleep(min(2e-4, t_next - now))
            srv.submit(ids[picks[k]], dms[picks[k]], tag=10_000 + k)
        while len(lat_ms) < n_req:
            for _tag, _e, lat in srv.poll(wait_ms=5000):
                lat_ms.append(lat)
        t_end = time.perf_counter()
        nb, nbr, _, t_asm, t_bat = srv.batch_stats()
        srv.close()
        lat = np.array(lat_ms)
        return {"jobs_per_s": n_req / (t_end - t_start), "requests": n_req,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "offered_rate": rate, "slots": nslots, "precision": precision,
                "batched_steps": nb, "mean_batch": (nbr / nb) if nb else 1.0,
                "batch_assemble_ms": (t_asm / nb) if nb else None, "batch_wall_ms": (t_bat / nb) if nb else None,
                "max_batch": srv_max_batch}, energies

    sweep, e_tc = [], None
    for rate in [float(x) for x in args.serve_rates.split(",") if x]:
        res, e = run_server("bf16x3", args.serve_slots, rate, args.serve_seconds, 100000)
        sweep.append(res)
        e_tc = e_tc or e
    sat_tc, e_sat = run_server("bf16x3", args.serve_slots, 0, 0, args.serve_saturate)
    # the same saturated stream with every request stepping alone (no batching)
    sat_alone, _ = run_server("bf16x3", args.serve_slots, 0, 0, args.serve_saturate, max_batch=1)
    e_tc = e_tc or e_sat
    sat_64, e_64 = run_server("fp64", 1, 0, 0, args.serve_fp64_requests)
    err = max(abs(e_tc[k][4] - e_64[k][4]) / natoms[k] * 1e6 for k in range(len(jobs)))
    return {
        "sweep": sweep, "saturated_bf16x3": sat_tc, "saturated_bf16x3_unbatched": sat_alone,
        "saturated_fp64_dropin": sat_64,
        "jobs_per_s_vs_fp64": sat_tc["jobs_per_s"] / sat_64["jobs_per_s"],
        "max_err_per_atom_uHa": err,
        "pool_step_ms": {"per_structure": alone_ms, "mean": float(np.mean(alone_ms)),
                         "jobs_per_s_back_to_back": 1000.0 / float(np.mean(alone_ms)),
                         "note": "each structure's split-BF16 step alone on the device (CUDA events); requests pick "
                                 "structures uniformly, so 1000 / mean is the jobs/s of back-to-back single steps"},
        "structures": {"count": len(jobs), "atoms": natoms, "setup_s": t_setup,
                       "resident_bytes": int(sum(j.footprint() for j in jobs))},
    }


# ------------------------------------------------------------------ batching form

def batching(args):
    """The batching form: `--batch-cells` independent cells (2-64 atoms, 1-3
    species, cutoffs 6-9 bohr, 4/9/13/18 orbitals, cubic 4-12 A lattices,
    random positions >= 3.5 bohr apart, grids from Calc_Ngrid at 150 Ry)
    stepped together by lcp_batch: one persistent tensor-core launch per
    contraction over the bricks of every cell (the matrix elements in waves
    under `--batch-scratch-gb`), batched FFTs per grid shape, the whole step
    one CUDA graph.  Brick shapes: the measured autotuner on the largest cell
    of each grid shape, applied to the cells of that shape where the model
    ranks it among its best four, else the model's best.  Reported beside it:
    the same batch launched eagerly, the same cells stepped one by one as
    split-BF16 jobs, and the FP64 per-cell path with its energies on a sample
    of cells (the error of the batched energies vs FP64)."""
    import threading
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np
    import torch

    import lcpgrid as L
    from lcpgrid.workloads import batch_pool, psd_density_matrices, smooth_vna

    t_all = time.perf_counter()
    pool = batch_pool(args.batch_cells, seed=args.batch_seed)
    n = len(pool)

    def mk_ucell(w):
        return L.UCell(1, w["latvecs"], w["natom"], w["atom2spe"], w["gxyz"], w["cut"], w["ngrid"], w["origin"],
                       Total_NumOrbs=w["numorbs"])

    t0 = time.perf_counter()
    with ThreadPoolExecutor(args.batch_threads) as ex:
        ucells = list(ex.map(mk_ucell, pool))
    t_geom = time.perf_counter() - t0

    ctx = L.Context(0, precision="bf16x3")
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    classes = {}
    for k, w in enumerate(pool):
        classes.setdefault(tuple(w["ngrid"]), []).append(k)
    sample = set(range(0, n, max(1, n // max(1, args.batch_fp64_sample)))) if args.batch_fp64_sample else set()

    # brick shapes: measured autotune of each grid shape's largest cell
    t0 = time.perf_counter()
    tuned, tuned_orbs, tune_log = {}, {}, []
    if args.batch_autotune > 0:
        for ng, ks in classes.items():
            k = max(ks, key=lambda i: pool[i]["natom"])
            orbs = L.Set_Orbitals_Grid(pool[k]["paos"], ucells[k], ctx=ctx)
            shape, ms = orbs.autotune_bricks(args.batch_autotune)
            tuned[ng] = shape
            tuned_orbs[k] = orbs
            tune_log.append({"ngrid": list(ng), "cell_atoms": pool[k]["natom"], "shape": list(shape),
                             "model_best": list(ucells[k].brick_shape_candidates(1)[0][0]), "ms": ms})
    t_tune = time.perf_counter() - t0

    local = threading.local()
    ctxs, lock = [], threading.Lock()

    def thread_ctx():
        c = getattr(local, "ctx", None)
        if c is None:
            c = local.ctx = L.Context(0, precision="bf16x3")
            with lock:
                ctxs.append(c)
        return c

    def prepare(k):
        w, u = pool[k], ucells[k]
        orbs = tuned_orbs.get(k)
        if orbs is None:
            orbs = L.Set_Orbitals_Grid(w["paos"], u, ctx=thread_ctx())
            shape = tuned.get(tuple(w["ngrid"]))
            if shape is not None and shape in [c[0] for c in u.brick_shape_candidates(4)]:
                orbs.set_brick_shape(shape)
        vna = smooth_vna(w["ngrid"], w["latvecs"], w["vna_seed"])
        job = L.GridStepJob(u, orbs, "off", "LDA", None, None, vna)
        try:
            job.prepare()
        except L.LCPError as exc:
            if exc.status != 5:  # LCP_ENOTSUP: too many atom images per brick for the class's shape
                raise
            orbs.set_brick_shape(None)  # the model's best shape within the limit
            job.prepare()
        if k not in sample:
            orbs.release_fp64()  # the batch needs the split-BF16 tables only
        dm = psd_density_matrices(u, w["dm_seed"], trace=w["trace"])
        job.set_dm(dm)
        return job

    t0 = time.perf_counter()
    with ThreadPoolExecutor(args.batch_threads) as ex:
        jobs = list(ex.map(prepare, range(n)))
    for c in ctxs:
        c.synchronize()
    ctx.synchronize()
    t_prep = time.perf_counter() - t0

    t0 = time.perf_counter()
    b = L.Batch(jobs, scratch_bytes=int(args.batch_scratch_gb * 1e9), ctx=ctx)
    t_batch = time.perf_counter() - t0
    info = b.info()
    torch.cuda.synchronize()
    b.step(graph=True)  # runs eagerly and captures the graph
    torch.cuda.synchronize()
    for _ in range(max(3, args.warmup)):
        b.step(graph=True)
    stages = b.step_timed()
    torch.cuda.synchronize()

    def timed(fn, reps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(reps + 1)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        for r in range(reps):
            fn()
            ev[r + 1].record(stream)
        torch.cuda.synchronize()
        return np.array([ev[r].elapsed_time(ev[r + 1]) for r in range(reps)])

    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    l0 = ctx.launch_count
    g_ms = timed(lambda: b.step(graph=True), args.steps)
    launches = (ctx.launch_count - l0) / args.steps
    clk = clocks.stop()
    e_ms = timed(lambda: b.step(graph=False), max(2, args.steps // 4))
    e_batch = b.energies()
    b.check_status()

    # the same cells stepped one by one (split-BF16 jobs on this context)
    def one_by_one():
        for j in jobs:
            j.step(ctx)
    seq_ms = timed(one_by_one, 2)
    e_seq = np.array([j.energies() for j in jobs])

    # FP64 per-cell path on the sample (these cells kept their FP64 tables)
    fp64 = None
    if sample:
        ctx.set_precision("fp64")
        ks = sorted(sample)
        for k in ks:
            jobs[k].step(ctx)  # warm-up (FFT plans)
        f_ms = timed(lambda: [jobs[k].step(ctx) for k in ks], 1)
        e64 = np.array([jobs[k].energies() for k in ks])
        ctx.set_precision("bf16x3")
        err = np.abs(e_batch[ks, 4] - e64[:, 4]) / np.array([pool[k]["natom"] for k in ks]) * 1e6
        rel = np.abs(e_batch[ks, 4] - e64[:, 4]) / np.abs(e64[:, 4])
        # the batch's per-cell time on the same cells, by their share of the pair work
        fp64 = {"cells": len(ks), "ms_all_sample_cells": float(f_ms[0]),
                "ms_per_cell": float(f_ms[0]) / len(ks),
                "max_err_per_atom_uHa": float(err.max()), "mean_err_per_atom_uHa": float(err.mean()),
                "max_rel_err": float(rel.max())}

    dens = ham = 0.0
    for u in ucells:
        d, h = pair_work(u)
        dens += d
        ham += h
    peaks, psrc = measured_peaks()
    names = ["density", "poisson", "xc_vpot", "energy_sums", "hamiltonian", "dot_finish"]
    dom = int(np.argmax(stages))
    dom_flops = dens if names[dom] == "density" else ham
    pk = peaks.get("bf16_tflops_sustained", 1700.0)
    roof = {"bound": "tensor", "kernel": names[dom] + " (all cells)",
            "achieved": dom_flops / (stages[dom] * 1e-3) / 1e12, "peak": pk, "unit": "TFLOP/s",
            "peak_source": psrc + " bf16_tflops_sustained", "traffic": None,
            "note": "algorithmic flops counted per unordered pair and lens point; eager stage time"}
    roof["frac"] = roof["achieved"] / pk
    ms = float(np.median(g_ms))
    natoms = np.array([w["natom"] for w in pool])
    return {
        "metric": "batching: ms per batched SCF grid step of %d cells & cell steps/s, split-BF16" % n,
        "value": n * 1000.0 / ms, "unit": "cell grid steps/s", "higher_is_better": True, "n_gpus": 1,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "p50_ms": float(np.percentile(g_ms, 50)), "p99_ms": float(np.percentile(g_ms, 99)),
        "dtype": "bf16x3/f32-acc", "scaling": "weak", "vs_baseline": None,
        "data": "synthetic (seeded: random cells, Gaussian radial functions, PSD D, smooth V_na)",
        "config": {"workload": "batch_pool(%d, seed=%d)" % (n, args.batch_seed), "cells": n,
                   "atoms_total": int(natoms.sum()), "atoms_range": [int(natoms.min()), int(natoms.max())],
                   "grid_shapes": len(classes), "grid_points_total": int(sum(np.prod(w["ngrid"]) for w in pool)),
                   "bricks": info["bricks"], "h_waves": info["waves"],
                   "workspace_gb": info["workspace_bytes"] / 1e9, "l2": "inputs larger than L2"},
        "stage_ms": dict(zip(names, [float(x) for x in stages])),
        "eager_ms_per_step": float(np.median(e_ms)),
        "graph_speedup_vs_eager": float(np.median(e_ms)) / ms,
        "one_by_one_ms": float(np.median(seq_ms)),
        "batch_speedup_vs_one_by_one": float(np.median(seq_ms)) / ms,
        "one_by_one_max_abs_dE": float(np.max(np.abs(e_seq - e_batch))),
        "fp64_per_cell_sample": fp64,
        "roofline": roof,
        "autotune": tune_log,
        "setup_s": {"geometry": t_geom, "autotune": t_tune, "tabulate_prepare": t_prep, "batch_create": t_batch,
                    "total": time.perf_counter() - t_all},
        "clocks": clk,
        "gpu_launches": launches,
        "gpu_launches_note": "kernels of this library per batched step (graph nodes; 5 FFT kernels per grid shape)",
    }


def run_case(args):
    """Small cases of single kernels, sized for profiler captures; prints their
    device times (CUDA events on the library's stream)."""
    import numpy as np
    import torch

    import lcpgrid as L
    out = {"case": args.case}
    ctx = L.Context(0, precision="bf16x3")
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    if args.case == "poisson":
        ng = (96, 96, 96)
        lat = np.eye(3) * 20.52
        rec = 2 * np.pi * np.linalg.inv(lat.T)
        src = np.random.default_rng(0).normal(size=int(np.prod(ng)))
        res = np.zeros(src.size)
        for prec in ("bf16x3", "fp64"):
            ctx.set_precision(prec)
            t0 = time.perf_counter()
            L.Solve_Poisson_xyz(ng, rec, src, res, ctx=ctx)  # host in and out, as the reference calls it
            out[prec + "_call_ms"] = (time.perf_counter() - t0) * 1e3
    else:
        wl = _inputs().si64_workload(nrep=1, ngrid=(48, 48, 48))
        u = L.UCell(1, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"], wl["origin"],
                    Total_NumOrbs=wl["numorbs"], ctx=ctx)
        orbs = L.Set_Orbitals_Grid(wl["paos"], u)
        job = L.GridStepJob(u, orbs, "off", "LDA")
        job.prepare()
        out["tabulation_ms"], out["split_tables_ms"] = orbs.timings()
    ctx.synchronize()
    print(json.dumps(out))


def main():
    args = parse()
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.batching:
        print(json.dumps(batching(args)))
    elif args.serving:
        res = serving(args)
        print(json.dumps({"metric": "serving: jobs/s (p50/p99 latency) split-BF16 vs FP64 drop-in, mixed-size stream",
                          "value": res["saturated_bf16x3"]["jobs_per_s"], "unit": "jobs/s", "higher_is_better": True,
                          "n_gpus": 1, "data": "synthetic (seeded random Si-density cells, 2-216 atoms)",
                          "config": {"workload": "serving_pool", "slots": args.serve_slots,
                                     "rates": args.serve_rates, "max_batch": args.serve_max_batch}, **res}))
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
