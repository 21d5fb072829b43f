"""The reference's SCF grid step on the host cores: the timed CPU baseline and
the full-size checker of the GPU step.

TEST AND BENCHMARK INFRASTRUCTURE ONLY.  Only ``tests/`` and the CPU legs of
``bench.py`` use this module.  It loads nothing of the product library: the
geometry, orbitals and every stage come from ``oracle/lcp_oracle.py``.

It restates how LCPAODFT.jl runs one grid step under MPI, with one spawned
process per host core standing in for one MPI rank:

* the pair list is split into contiguous ranges of near-equal work
  NO_atom * NO_jatom * min(GridN_atom, GridN_jatom)
  (``split_system_grid`` / ``_split_weighted_contiguous``, src/UCell.jl:50-132);
* every rank builds the overlap lists of its own pairs
  (``Calc_AtomOverlap_Grid``, src/UCell.jl:425-516) and the orbital tables of
  the atoms they touch (src/Matrix/Set_Orbitals_Grid.jl:26-277);
* density: per pair, 512-point blocks gathered from the two orbital tables,
  a small GEMM with the pair's D block and a dot per point into the atom's
  local sphere array, folded into the rank's grid; the ranks' grids are then
  summed (the Allreduce of src/Matrix/Set_Density_Grid.jl:60-169);
* Poisson (src/Poisson.jl:1-108), xc (src/XC/XC_Func.jl:111-145) and the
  potential (src/Matrix/Set_Vpot_Grid.jl:1-19) on the full grid;
* matrix elements: per pair, the same blocks with V at the atom's points and
  a small GEMM into the pair's H block (src/Hamiltonian.jl:235-324, 384-429);
  the ranks' blocks are disjoint;
* the energy terms E_H1, E_xc1 (src/Energy.jl:655-700) and sum <D, H>.

Each process runs single-threaded BLAS, as the reference pins BLAS to one
thread per rank (src/DFT_Setup.jl:368).  Stage results are exchanged through
file-backed shared maps in a temporary directory.  One difference from the
reference's order of additions: a rank sums the local sphere arrays of
consecutive pairs of the same atom before folding them into its grid (the
reference folds after every pair).  The sums differ in rounding only.
"""
import multiprocessing as mp
import os
import shutil
import tempfile
import time

import numpy as np

from . import lcp_oracle as O

_NSPIN = {"off": 1, "on": 2}


def split_weighted_contiguous(weights, nparts):
    """Contiguous ranges (start, stop) of near-equal summed weight
    (src/UCell.jl:50-72): each boundary is the first cumulative sum reaching
    rank * total / nparts, moved one item back when that lands closer, and
    every part keeps at least one item."""
    w = np.asarray(weights, dtype=np.float64)
    n = w.size
    if n < nparts:
        raise ValueError("number of work items must be at least the number of parts")
    cum = np.cumsum(w)
    total = cum[-1]
    out = []
    first = 0  # 0-based start of the current part
    for rank in range(1, nparts):
        target = total * rank / nparts
        b = int(np.searchsorted(cum, target, side="left"))  # 0-based first index with cum >= target
        last_allowed = n - (nparts - rank) - 1
        b = min(max(b, first), last_allowed)
        if b < last_allowed:
            prev_err = np.inf if b == first else abs(cum[b - 1] - target)
            cur_err = abs(cum[b] - target)
            if prev_err < cur_err:
                b -= 1
            b = max(b, first)
        out.append((first, b + 1))
        first = b + 1
    out.append((first, n))
    return out


def pair_work_weights(ucell):
    """Work weight of each pair (src/UCell.jl:86-99)."""
    no = np.asarray(ucell.Total_NumOrbs, dtype=np.float64)
    gn = np.asarray(ucell.GridN_Atom, dtype=np.float64)
    a = np.asarray(ucell.MPI_atom) - 1
    b = np.asarray(ucell.MPI_natn) - 1
    return np.maximum(no[a] * no[b] * np.minimum(gn[a], gn[b]), 1.0)


def _ucell(spec, pair_subset):
    return O.UCell(_NSPIN[spec["spinpol"]], spec["latvecs"], spec["natom"], spec["atom2spe"], spec["gxyz"],
                   spec["cut"], spec["ngrid"], spec["origin"], total_numorbs=spec["numorbs"],
                   pair_subset=pair_subset)


def _paos(spec):
    return [O.PAO(maxl, nb, rv, rwf) for (maxl, nb, rv, rwf) in spec["paos"]]


def _maps(folder, nproc, nspin, nn, hsize, mode):
    return {
        "dm": np.memmap(os.path.join(folder, "dm"), dtype=np.float64, mode=mode, shape=(nspin, hsize)),
        "rho": np.memmap(os.path.join(folder, "rho"), dtype=np.float64, mode=mode, shape=(nproc, nspin, nn)),
        "vpot": np.memmap(os.path.join(folder, "vpot"), dtype=np.float64, mode=mode, shape=(nspin, nn)),
        "hks": np.memmap(os.path.join(folder, "hks"), dtype=np.float64, mode=mode, shape=(nspin, hsize)),
    }


def _density_part(u, orbs, dm, loops, nspin, out):
    """This rank's share of the density: out[s] (NN) = sum over its pairs."""
    out[:] = 0.0
    cur, local = None, None

    def fold():
        gl = u.GridListAtom[cur]
        for s in range(nspin):
            out[s] += np.bincount(gl, weights=local[:, s], minlength=out.shape[1])

    for loop in loops:
        atom, jatom, _ = u.pairs[loop]
        a, b = atom - 1, jatom - 1
        if a != cur:
            if cur is not None:
                fold()
            cur = a
            local = np.zeros((u.GridN_Atom[a], nspin))
        g1 = u.MPI_GListTAtoms1[loop]
        if g1.size == 0:
            continue
        g2 = u.MPI_GListTAtoms2[loop]
        no0, no1 = int(u.Total_NumOrbs[a]), int(u.Total_NumOrbs[b])
        off = int(u.block_offset[loop])
        # D block [ist, jst]; tables point-major [GridN, NO], the memory order of the
        # reference's column-major Matrix(NO, GridN), so a gather reads whole rows
        Dt = [dm[s][off:off + no0 * no1].reshape(no0, no1) for s in range(nspin)]
        phi_a, phi_b = orbs[a], orbs[b]
        for bs in range(0, g1.size, O.DENSITY_BLOCK):
            i1 = g1[bs:bs + O.DENSITY_BLOCK]
            i2 = g2[bs:bs + O.DENSITY_BLOCK]
            ob1 = phi_a[i1]                                       # [points, NO0]
            ob2 = phi_b[i2]                                       # [points, NO1]
            for s in range(nspin):
                P = ob2 @ Dt[s].T                                 # src/Matrix/Set_Density_Grid.jl:290
                local[i1, s] += np.einsum("po,po->p", ob1, P)     # :293-297 (i1 has no repeats in a pair)
    if cur is not None:
        fold()


def _hamiltonian_part(u, orbs, vpot, loops, nspin, hks):
    """This rank's H blocks (src/Hamiltonian.jl:384-429), scaled by GridVol."""
    for loop in loops:
        atom, jatom, _ = u.pairs[loop]
        a, b = atom - 1, jatom - 1
        no0, no1 = int(u.Total_NumOrbs[a]), int(u.Total_NumOrbs[b])
        off = int(u.block_offset[loop])
        g1 = u.MPI_GListTAtoms1[loop]
        acc = [np.zeros((no1, no0)) for _ in range(nspin)]
        if g1.size:
            g2 = u.MPI_GListTAtoms2[loop]
            gl = u.GridListAtom[a]
            phi_a, phi_b = orbs[a], orbs[b]
            for bs in range(0, g1.size, O.DENSITY_BLOCK):
                i1 = g1[bs:bs + O.DENSITY_BLOCK]
                i2 = g2[bs:bs + O.DENSITY_BLOCK]
                ob1 = phi_a[i1]                                   # [points, NO0]
                ob2 = phi_b[i2]                                   # [points, NO1]
                pts = gl[i1]
                for s in range(nspin):
                    acc[s] += ob2.T @ (ob1 * vpot[s][pts][:, None])  # [jst, ist] (:420)
        for s in range(nspin):
            hks[s][off:off + no0 * no1] = (acc[s] * u.GridVol).T.reshape(-1)


def _worker(rank, nproc, spec, loops, folder, conn):
    """One rank: geometry, its overlap lists and orbital tables, then the
    density and matrix-element passes on command."""
    try:
        nspin = _NSPIN[spec["spinpol"]]
        u = _ucell(spec, loops)
        need = sorted({u.pairs[p][0] - 1 for p in loops} | {u.pairs[p][1] - 1 for p in loops})
        orbs = [None if t is None else np.ascontiguousarray(t.T)
                for t in O.set_orbitals_grid(_paos(spec), u, atoms=set(need))]  # [GridN, NO] per atom
        maps = _maps(folder, nproc, nspin, u.NN, u.Total_Hsize, "r+")
        conn.send(("ready", None))
        while True:
            cmd = conn.recv()
            if cmd == "density":
                t0 = time.perf_counter()
                _density_part(u, orbs, maps["dm"], loops, nspin, maps["rho"][rank])
                conn.send(("done", time.perf_counter() - t0))
            elif cmd == "hamiltonian":
                t0 = time.perf_counter()
                _hamiltonian_part(u, orbs, maps["vpot"], loops, nspin, maps["hks"])
                conn.send(("done", time.perf_counter() - t0))
            else:
                break
    except Exception as exc:  # reported to the parent, which raises
        conn.send(("error", repr(exc)))
    finally:
        conn.close()


class CpuGridStep:
    """The reference's grid step, MPI-style, over ``nproc`` spawned processes.

    ``spec``: a dict of host inputs -- latvecs, natom, atom2spe, gxyz, cut,
    ngrid, origin, numorbs, paos (list of (max_l, num_basis, RV, RWF)),
    spinpol ("off" / "on"), xc ("LDA" / "LSDA"), optional vna, aden, pcc (NN).
    ``pairs``: restrict the work to these 0-based pair indices (the rest of
    D must be zero for the density to be complete; the other H blocks stay 0).
    """

    def __init__(self, spec, nproc=None, pairs=None):
        os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")  # inherited by the spawned ranks
        os.environ.setdefault("OMP_NUM_THREADS", "1")
        self.spec = dict(spec)
        self.spinpol = spec["spinpol"]
        if self.spinpol not in _NSPIN:
            raise ValueError("the CPU step covers SpinPol off and on")
        self.nspin = _NSPIN[self.spinpol]
        t0 = time.perf_counter()
        self.u = _ucell(spec, [])  # geometry and pair list; each rank builds its own overlap lists
        u = self.u
        sel = np.arange(u.Nloop) if pairs is None else np.asarray(sorted(set(pairs)), dtype=np.int64)
        nproc = int(nproc or os.cpu_count() or 1)
        nproc = max(1, min(nproc, sel.size))
        w = pair_work_weights(u)[sel]
        ranges = split_weighted_contiguous(w, nproc)
        self.loops = [sel[a:b].tolist() for a, b in ranges]
        self.nproc = nproc
        nn = u.NN
        self.vna = spec.get("vna")
        self.aden = np.zeros(nn) if spec.get("aden") is None else np.asarray(spec["aden"], dtype=np.float64)
        self.pcc = np.zeros(nn) if spec.get("pcc") is None else np.asarray(spec["pcc"], dtype=np.float64)
        self.folder = tempfile.mkdtemp(prefix="lcp_cpu_step_")
        self.maps = _maps(self.folder, nproc, self.nspin, nn, u.Total_Hsize, "w+")
        ctx = mp.get_context("spawn")
        self.conns, self.procs = [], []
        for r in range(nproc):
            parent, child = ctx.Pipe()
            p = ctx.Process(target=_worker, args=(r, nproc, self.spec, self.loops[r], self.folder, child),
                            daemon=True)
            p.start()
            child.close()
            self.conns.append(parent)
            self.procs.append(p)
        self._gather("ready")
        self.setup_s = time.perf_counter() - t0

    def _gather(self, want):
        out = []
        for c, p in zip(self.conns, self.procs):
            while not c.poll(1.0):  # a rank that died (e.g. at start-up) ends the wait
                if not p.is_alive():
                    self.close()
                    raise RuntimeError("CPU step rank exited (code %s)" % p.exitcode)
            tag, val = c.recv()
            if tag == "error":
                self.close()
                raise RuntimeError("CPU step rank failed: " + val)
            assert tag == want
            out.append(val)
        return out

    def set_dm(self, dm):
        for s in range(self.nspin):
            self.maps["dm"][s] = dm[s]
        self.maps["dm"].flush()

    def step(self):
        """One grid step on the current D: returns a dict of the density (per
        channel), V, H (per channel), the energy terms and stage seconds."""
        u, ns = self.u, self.nspin
        times = {}
        t_all = time.perf_counter()
        t0 = t_all
        for c in self.conns:
            c.send("density")
        self._gather("done")
        rho = [np.array(x) for x in self.maps["rho"].sum(axis=0)]  # the ranks' Allreduce
        times["density"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        dvh = O.solve_poisson(self.spinpol, u, rho, self.aden)
        times["poisson"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        vxc = O.set_xc_grid(self.spec["xc"], self.spinpol, self.pcc, rho)
        vpot = O.set_vpot_grid(self.spinpol, dvh, vxc, self.vna)
        for s in range(ns):
            self.maps["vpot"][s] = vpot[s]
        times["xc_vpot"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        for c in self.conns:
            c.send("hamiltonian")
        self._gather("done")
        hks = [np.array(self.maps["hks"][s]) for s in range(ns)]
        times["hamiltonian"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        dm = [np.array(self.maps["dm"][s]) for s in range(ns)]
        eh1 = O.calc_eh1(self.spinpol, u.GridVol, self.aden, rho, dvh)
        exc = O.calc_exc1(self.spinpol, self.spec["xc"], u.GridVol, self.aden, self.pcc, rho)
        e = O.grid_energy(self.spinpol, u, dm, hks, eh1, exc)
        e_dh = sum(float(np.dot(dm[s], hks[s])) for s in range(ns))
        times["energies"] = time.perf_counter() - t0
        times["step"] = time.perf_counter() - t_all
        return {"density": rho, "vpot": vpot, "hks": hks,
                "energies": [eh1, exc[0], exc[0] if self.spinpol == "off" else exc[1], e_dh, e],
                "seconds": times}

    def close(self):
        for c in getattr(self, "conns", []):
            try:
                c.send("quit")
            except Exception:
                pass
        for p in getattr(self, "procs", []):
            p.join(timeout=10)
            if p.is_alive():
                p.terminate()
        self.conns, self.procs = [], []
        self.maps = {}
        if getattr(self, "folder", None):
            shutil.rmtree(self.folder, ignore_errors=True)
            self.folder = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
