"""Host-side mirror of LCPAODFT.jl's grid-path interface over the C ABI.

Each function keeps the reference's name, argument order and meaning.  The
Julia ``!`` suffix (mutates its last arguments) maps to writing into the numpy
arrays passed in; errors the reference raises with ``error()`` raise
``LCPError``.  All arithmetic runs in liblcpgrid.so on the GPU.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import LCPError, check, dptr, dptrs, iptr, lib

__all__ = ["Context", "UCell", "DeviceOrbitalsGrid", "Rhor_Mixing", "XC_Func", "GridStepJob", "Batch", "Server",
           "Set_Orbitals_Grid", "Set_dOrbitals_Grid", "Set_AdenPCC_Grid", "Set_Density_Grid", "diagonalize_nc_density", "Solve_Poisson", "Solve_Poisson_xyz",
           "Calc_Diff_Coef", "Set_XC_Grid", "Set_Vpot_Grid", "Calc_MatrixElements_dVH_Vxc_off", "Calc_MatrixElements_dVH_Vxc_on",
           "Calc_MatrixElements_dVH_Vxc_nc", "Force3_nospin", "Force3_spin", "Force3_nc", "Calc_EH1", "Calc_EXC1", "Calc_Ngrid", "default_context",
           "use_context"]


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """A device context (CUDA stream, FFT plans, workspaces) on one GPU.

    ``precision`` selects the arithmetic of the pair contractions:
    "fp64" (the drop-in), "fp32" or "bf16x3"."""

    def __init__(self, device=0, precision="fp64"):
        h = ctypes.c_void_p()
        check(lib.lcp_ctx_create(int(device), ctypes.byref(h)))
        self._h = h
        self.device = int(device)
        self.set_precision(precision)

    def set_precision(self, precision):
        check(lib.lcp_ctx_set_precision(self._h, _lib.PREC[precision]))
        self.precision = precision

    def set_stream(self, stream_handle):
        """Run on an external cudaStream_t (an int handle, e.g. torch's
        ``torch.cuda.current_stream().cuda_stream``); None restores the own stream."""
        check(lib.lcp_ctx_set_stream(self._h, ctypes.c_void_p(stream_handle) if stream_handle else None))

    def synchronize(self):
        check(lib.lcp_ctx_synchronize(self._h))

    def probe_fp64_tflops(self):
        """Measured FP64 FMA throughput of the device (TFLOP/s)."""
        out = ctypes.c_double()
        check(lib.lcp_probe_fp64_tflops(self._h, ctypes.byref(out)))
        return out.value

    def tc_selftest(self, a, b, a_mn=False, b_mn=False, order=0):
        """d = bf16(a) @ bf16(b).T on the tensor cores (a: 128 x k, b: n x k)."""
        a = np.ascontiguousarray(a, dtype=np.float32)
        b = np.ascontiguousarray(b, dtype=np.float32)
        d = np.zeros((128, b.shape[0]), dtype=np.float32)
        check(lib.lcp_tc_selftest(self._h, int(a_mn), int(b_mn), int(order), b.shape[0], a.shape[1], a.ctypes.data,
                                  b.ctypes.data, d.ctypes.data))
        return d

    def set_fault_test(self, poll_limit=0, stall=0):
        """Failure-path tests only: poll limit of the split-BF16 density
        kernel's bounded waits (0: default) and its stall switch (1: one
        epilogue warp withholds its stage releases, so the kernel times out
        and unwinds; the call raises LCPError LCP_ETIMEDOUT)."""
        check(lib.lcp_ctx_set_fault_test(self._h, int(poll_limit), int(stall)))

    def set_xc_arithmetic(self, double_float):
        """Arithmetic of this context's drop-in GGA-PBE calls (Set_XC_Grid,
        Calc_EXC1 with an XC_Func "GGA_PBE"): False = FP64 (default), True =
        double-float as the precision forms' grid step."""
        check(lib.lcp_ctx_set_xc_arithmetic(self._h, int(bool(double_float))))

    def set_step_graphs(self, on):
        """Whether GridStepJob.step on this context replays its launches as a
        CUDA graph (True, the default; captured at a job's second step) or
        launches them one by one (False).  Same results either way."""
        check(lib.lcp_ctx_set_step_graphs(self._h, int(bool(on))))

    @property
    def launch_count(self):
        return int(lib.lcp_ctx_launch_count(self._h))

    def close(self):
        if getattr(self, "_h", None):
            lib.lcp_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_DEFAULT = {}


def default_context(device=0):
    """The module's context on `device`: the one installed by use_context, else
    an FP64 context made on first use.  Functions whose reference signature has
    no argument that could carry a context (diagonalize_nc_density, Calc_EH1,
    the inner Solve_Poisson) run on it."""
    if device not in _DEFAULT:
        _DEFAULT[device] = Context(device)
    return _DEFAULT[device]


def use_context(ctx):
    """Installs `ctx` as the module's context on its device; returns the one it
    replaces (or None).  This is the counterpart of the Julia binding's
    module-level context, which lets the reference's call sites stay unchanged."""
    old = _DEFAULT.get(ctx.device)
    _DEFAULT[ctx.device] = ctx
    return old


def _ctx_of(*objs, ctx=None):
    """The context a call runs on: an explicit keyword, else the first object
    that carries one, else the module's default."""
    if ctx is not None:
        return ctx
    for o in objs:
        c = getattr(o, "ctx", None)
        if c is not None:
            return c
    return default_context()


class UCell:
    """``UCell(Nspin, Latvecs, Natom, atom2spe, Gxyz, Atoms_Cut1, Ngrid, Grid_Origin; Total_NumOrbs)``
    (src/UCell.jl:210-294), built by the library: on the host, or with
    ``device=True`` its sphere and overlap lists on the GPU of ``ctx`` (the
    same lists bit for bit; LCPError LCP_ENOTSUP for cells whose atoms' grid
    boxes reach image cells outside -CpyCell..CpyCell-1).

    Lists are exposed with the reference's names: GridN_Atom, GridListAtom,
    CellListAtom (per atom), FNAN, natn, ncn, MPI_atom/MPI_natn/MPI_ncn,
    MPI_NumOLG and MPI_GListTAtoms1/2 (per pair).

    ``ctx`` (keyword) is the context of the device build and of the calls that
    take this UCell (Set_Orbitals_Grid, Set_AdenPCC_Grid); without it they use
    the module's default context."""

    def __init__(self, Nspin, Latvecs, Natom, atom2spe, Gxyz, Atoms_Cut1, Ngrid, Grid_Origin, Total_NumOrbs=None,
                 device=False, ctx=None):
        self.ctx = ctx
        self.Latvecs = _f64(Latvecs).reshape(3, 3)
        self.Natom = int(Natom)
        self.atom2spe = np.ascontiguousarray(atom2spe, dtype=np.int32)
        self.Gxyz = _f64(Gxyz).reshape(self.Natom, 3)
        self.Atoms_Cut1 = _f64(Atoms_Cut1)
        self.Ngrid = tuple(int(x) for x in Ngrid)
        self.Grid_Origin = _f64(Grid_Origin)
        self.Nspin = int(Nspin)
        self.Total_NumOrbs = np.zeros(self.Natom, dtype=np.int32) if Total_NumOrbs is None else \
            np.ascontiguousarray(Total_NumOrbs, dtype=np.int32)
        if self.atom2spe.size != self.Natom or self.Atoms_Cut1.size != self.Natom or self.Total_NumOrbs.size != self.Natom:
            raise LCPError(_lib.LCP_EINVAL, "per-atom arrays must have Natom entries")
        h = ctypes.c_void_p()
        ng = np.array(self.Ngrid, dtype=np.int32)
        args = (self.Nspin, dptr(self.Latvecs), self.Natom, iptr(self.atom2spe), dptr(self.Gxyz),
                dptr(self.Atoms_Cut1), iptr(ng), dptr(self.Grid_Origin), iptr(self.Total_NumOrbs), ctypes.byref(h))
        if device:
            check(lib.lcp_ucell_create_device(_ctx_of(ctx=ctx)._h, *args))
        else:
            check(lib.lcp_ucell_create(*args))
        self._h = h
        info = _lib.lcp_ucell_info()
        check(lib.lcp_ucell_get_info(self._h, ctypes.byref(info)))
        self.CpyCell = info.cpycell
        self.Nloop = info.nloop
        self.ncell = info.ncell
        self.Total_Hsize = int(info.total_hsize)
        self.GridVol = info.gridvol
        self.sum_gridn = int(info.sum_gridn)
        self.sum_numolg = int(info.sum_numolg)
        self.n_unique = int(info.n_unique)
        self.max_numorbs = info.max_numorbs
        self.FNAN = self._ints(_lib.F_FNAN, 0, self.Natom)
        self.GridN_Atom = self._ints(_lib.F_GRIDN_ATOM, 0, self.Natom)
        self.MPI_atom = self._ints(_lib.F_PAIR_ATOM, 0, self.Nloop)
        self.MPI_natn = self._ints(_lib.F_PAIR_NATN, 0, self.Nloop)
        self.MPI_ncn = self._ints(_lib.F_PAIR_NCN, 0, self.Nloop)
        self.MPI_NumOLG = self._ints(_lib.F_NUMOLG, 0, self.Nloop)
        offs = [0]
        for a, b in zip(self.MPI_atom, self.MPI_natn):
            offs.append(offs[-1] + int(self.Total_NumOrbs[a - 1]) * int(self.Total_NumOrbs[b - 1]))
        self.block_offset = np.array(offs[:-1], dtype=np.int64)

    def _ints(self, field, index, count):
        out = np.zeros(int(count), dtype=np.int32)
        check(lib.lcp_ucell_get_int(self._h, field, int(index), iptr(out), int(count)))
        return out

    @property
    def natn(self):
        return [self._ints(_lib.F_NATN, a, self.FNAN[a] + 1) for a in range(self.Natom)]

    @property
    def ncn(self):
        return [self._ints(_lib.F_NCN, a, self.FNAN[a] + 1) for a in range(self.Natom)]

    @property
    def GridListAtom(self):
        return [self._ints(_lib.F_GRIDLIST, a, self.GridN_Atom[a]) for a in range(self.Natom)]

    @property
    def CellListAtom(self):
        return [self._ints(_lib.F_CELLLIST, a, self.GridN_Atom[a]) for a in range(self.Natom)]

    def GListTAtoms(self, pair):
        """(MPI_GListTAtoms1[pair], MPI_GListTAtoms2[pair]), 0-based pair index."""
        n = int(self.MPI_NumOLG[pair])
        return self._ints(_lib.F_GLIST1, pair, n), self._ints(_lib.F_GLIST2, pair, n)

    @property
    def atv(self):
        out = np.zeros((self.ncell, 3))
        check(lib.lcp_ucell_get_atv(self._h, dptr(out)))
        return out

    @property
    def atv_ijk(self):
        return self._ints(_lib.F_ATV_IJK, 0, self.ncell * 3).reshape(self.ncell, 3)

    @property
    def NN(self):
        return int(np.prod(self.Ngrid))

    def brick_shape_candidates(self, max_shapes=8):
        """[(shape, predicted cost)] best first."""
        sh = np.zeros(3 * max_shapes, dtype=np.int32)
        cost = np.zeros(max_shapes)
        n = ctypes.c_int32()
        check(lib.lcp_brick_shape_candidates(self._h, int(max_shapes), iptr(sh), dptr(cost), ctypes.byref(n)))
        return [(tuple(int(x) for x in sh[3 * k:3 * k + 3]), float(cost[k])) for k in range(n.value)]

    def brick_info(self):
        """Grid-brick tiling of the tensor-core path."""
        out = (ctypes.c_int64 * 14)()
        check(lib.lcp_ucell_get_bricks(self._h, out))
        v = list(out)
        return {"bdim": v[0:3], "nbricks_axis": v[3:6], "points": v[6], "bricks": v[7], "blocks": v[8],
                "max_images": v[9], "images": v[10], "paired": v[11], "h_slots": v[12], "sub_pairs": v[13]}

    def Recvecs(self):
        """2*pi*inv(Latvecs') (src/Mixing/DFT_Mixing.jl:91)."""
        return 2 * np.pi * np.linalg.inv(self.Latvecs.T)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib.lcp_ucell_destroy(self._h)
                self._h = None
        except Exception:
            pass


class DeviceOrbitalsGrid:
    """Device-resident orbital tables, the GPU counterpart of
    ``PackedOrbitalsGrid`` (src/Matrix/Set_Orbitals_Grid.jl:1-23).

    ``data(atom)`` copies atom's table to the host as [NumOrbs, GridN], the
    shape of ``PackedOrbitalsGrid.data[atom]``; component 1..3 selects the
    gradient tables when they were tabulated."""

    def __init__(self, ctx, ucell, handle, with_grad):
        self.ctx = ctx
        self.ucell = ucell
        self._h = handle
        self.with_grad = with_grad

    def data(self, atom, component=0):
        a = int(atom)
        n = int(self.ucell.GridN_Atom[a]) * int(self.ucell.Total_NumOrbs[a])
        out = np.zeros(n)
        check(lib.lcp_orbs_download(self.ctx._h, self._h, int(component), a, dptr(out), n))
        return out.reshape(int(self.ucell.GridN_Atom[a]), int(self.ucell.Total_NumOrbs[a])).T.copy()

    def __len__(self):
        return self.ucell.Natom

    def __getitem__(self, atom):
        return self.data(atom)

    def set_brick_shape(self, shape=None):
        """Brick shape of the split-BF16 tables (None: the predicted best)."""
        sh = np.zeros(3, dtype=np.int32) if shape is None else np.asarray(shape, dtype=np.int32)
        check(lib.lcp_orbs_set_brick_shape(self.ctx._h, self._h, iptr(sh)))

    def brick_shape(self):
        sh = np.zeros(3, dtype=np.int32)
        check(lib.lcp_orbs_get_brick_shape(self.ctx._h, self._h, iptr(sh)))
        return tuple(int(x) for x in sh)

    def autotune_bricks(self, ncand=3):
        """Times the split-BF16 passes for the ncand best predicted brick
        shapes and keeps the fastest: (shape, ms per density + H pass)."""
        sh = np.zeros(3, dtype=np.int32)
        ms = ctypes.c_double()
        check(lib.lcp_orbs_autotune_bricks(self.ctx._h, self._h, int(ncand), iptr(sh), ctypes.byref(ms)))
        return tuple(int(x) for x in sh), float(ms.value)

    def timings(self):
        """(tabulation kernel ms, split-BF16 table build ms), device times."""
        out = np.zeros(2)
        check(lib.lcp_orbs_timings(self._h, dptr(out)))
        return float(out[0]), float(out[1])

    def release_fp64(self):
        """Keep only the split-BF16 tables (frees the FP64 tables)."""
        check(lib.lcp_orbs_release_fp64(self.ctx._h, self._h))

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib.lcp_orbs_destroy(self._h)
                self._h = None
        except Exception:
            pass


def _paos_struct(paos):
    arr = (_lib.lcp_pao * len(paos))()
    keep = []
    for k, p in enumerate(paos):
        rv = _f64(p.Spe_PAO_RV)
        rwf = p.packed_rwf()
        keep += [rv, rwf]
        arr[k].max_l = p.Spe_MaxL_Basis
        for l in range(4):
            arr[k].num_basis[l] = p.Spe_Num_Basis[l] if l <= p.Spe_MaxL_Basis else 0
        arr[k].num_mesh = rv.size
        arr[k].rv = dptr(rv)
        arr[k].rwf = dptr(rwf)
    return arr, keep


def _tabulate(pao, ucell, ctx, grad):
    ctx = _ctx_of(ucell, ctx=ctx)
    arr, keep = _paos_struct(list(pao))
    h = ctypes.c_void_p()
    check(lib.lcp_set_orbitals_grid(ctx._h, ucell._h, len(keep) // 2, arr, 1 if grad else 0, ctypes.byref(h)))
    return DeviceOrbitalsGrid(ctx, ucell, h, grad)


def Set_Orbitals_Grid(pao, ucell, *, ctx=None):
    """src/Matrix/Set_Orbitals_Grid.jl:26-42.  Runs on ``ctx`` (keyword), else
    ucell's context, else the module's default."""
    return _tabulate(pao, ucell, ctx, False)


def Set_dOrbitals_Grid(pao, ucell, *, ctx=None):
    """Values and gradient tables (src/Matrix/Set_dOrbitals_Grid.jl:1-20);
    ``.data(atom, k)`` for k = 1, 2, 3 gives d/dx, d/dy, d/dz."""
    return _tabulate(pao, ucell, ctx, True)


def _spin(SpinPol):
    s = SpinPol.lower()
    if s not in _lib.SPIN:
        raise LCPError(_lib.LCP_EINVAL, "please check SpinPol.")
    return s


def Set_Density_Grid(SpinPol, ucell, Orbs_Grid, DM, Density_Grid):
    """``Set_Density_Grid!`` (src/Matrix/Set_Density_Grid.jl:1-9): fills Density_Grid[s]."""
    s = _spin(SpinPol)
    n = _lib.NCHAN[s]
    dm = [_f64(DM[c]) for c in range(n)]
    for c in range(n):
        if Density_Grid[c].dtype != np.float64 or not Density_Grid[c].flags["C_CONTIGUOUS"]:
            raise TypeError("Density_Grid must hold C-contiguous float64 arrays")
        if dm[c].size != ucell.Total_Hsize or Density_Grid[c].size != ucell.NN:
            raise LCPError(_lib.LCP_EINVAL, "DM/Density_Grid sizes do not match the UCell")
    pdm, k1 = dptrs(dm)
    pr, k2 = dptrs([Density_Grid[c] for c in range(n)])
    check(lib.lcp_set_density_grid(Orbs_Grid.ctx._h, ucell._h, Orbs_Grid._h, _lib.SPIN[s], pdm, pr))


def diagonalize_nc_density(Density_Grid, *, ctx=None):
    """``diagonalize_nc_density!`` (src/Matrix/Set_Density_Grid.jl:243-261):
    the four "nc" channels (Re11, Re22, Re12, Im12) become (Nup, Ndown,
    theta, phi) in place.  Runs on the module's default context (or ``ctx``)."""
    ctx = _ctx_of(ctx=ctx)
    for c in range(4):
        if Density_Grid[c].dtype != np.float64 or not Density_Grid[c].flags["C_CONTIGUOUS"]:
            raise TypeError("Density_Grid must hold C-contiguous float64 arrays")
    nn = Density_Grid[0].size
    if any(Density_Grid[c].size != nn for c in range(4)):
        raise LCPError(_lib.LCP_EINVAL, "Density_Grid channels differ in size")
    p, keep = dptrs([Density_Grid[c] for c in range(4)])
    check(lib.lcp_diagonalize_nc_density(ctx._h, nn, p))


def _radial(xv, rv, yv, keep):
    arrs = [_f64(xv), _f64(rv), _f64(yv)]
    if arrs[2].size != arrs[0].size + 4 or arrs[1].size != arrs[0].size:
        raise LCPError(_lib.LCP_EINVAL, "radial table sizes: xv and rv n, values n + 4")
    keep.extend(arrs)
    return _lib.lcp_radial(arrs[0].size, dptr(arrs[0]), dptr(arrs[1]), dptr(arrs[2]))


def Set_AdenPCC_Grid(SpinPol, Init_Atoms_Nspin, Init_Atoms_Angle, pao, pspot, ucell, *, ctx=None):
    """``Set_AdenPCC_Grid(SpinPol, Init_Atoms_Nspin, Init_Atoms_Angle, pao, pspot, ucell)``
    (src/Matrix/Set_AdenPCC_Grid.jl:1-142) on the GPU: returns (ADensity_Grid,
    PCCDensity_Grid, Density_Grid).  ``pao[spe]`` carries Spe_PAO_XV,
    Spe_PAO_RV and Spe_Atomic_Den; ``pspot[spe]`` Spe_VPS_XV, Spe_VPS_RV and
    Spe_Atomic_PCC (``PCC`` objects).  Runs on ucell's context (or ``ctx``)."""
    ctx = _ctx_of(ucell, ctx=ctx)
    s = _spin(SpinPol)
    keep = []
    den = (_lib.lcp_radial * len(pao))(*[_radial(p.Spe_PAO_XV, p.Spe_PAO_RV, p.Spe_Atomic_Den, keep) for p in pao])
    pcc = (_lib.lcp_radial * len(pspot))(*[_radial(p.Spe_VPS_XV, p.Spe_VPS_RV, p.Spe_Atomic_PCC, keep)
                                           for p in pspot])
    nsp = _f64([[float(x[0]), float(x[1])] for x in Init_Atoms_Nspin])
    ang = _f64([[float(x[0]), float(x[1])] for x in Init_Atoms_Angle]) if Init_Atoms_Angle is not None else None
    if nsp.shape != (ucell.Natom, 2) or (ang is not None and ang.shape != (ucell.Natom, 2)):
        raise LCPError(_lib.LCP_EINVAL, "Init_Atoms_Nspin / Init_Atoms_Angle need Natom entries")
    nn = ucell.NN
    ad, pc = np.zeros(nn), np.zeros(nn)
    dens = [np.zeros(nn) for _ in range(_lib.NCHAN[s])]
    pr, k2 = dptrs(dens)
    check(lib.lcp_set_adenpcc_grid(ctx._h, ucell._h, _lib.SPIN[s], dptr(nsp), dptr(ang), len(pao), den, pcc,
                                   dptr(ad), dptr(pc), pr))
    return ad, pc, dens


class Rhor_Mixing:
    """The parts of ``DFT_Mixing`` the Poisson solve reads: Ngrid and Recvecs
    (src/Mixing/DFT_Mixing.jl:47-95), and the device context the solve runs on
    (the module's default when None)."""

    def __init__(self, Ngrid, Latvecs, ctx=None):
        self.ctx = ctx
        self.Ngrid = tuple(int(x) for x in Ngrid)
        self.Latvecs = _f64(Latvecs).reshape(3, 3)
        self.Recvecs = 2 * np.pi * np.linalg.inv(self.Latvecs.T)


def Solve_Poisson(SpinPol, dft_mixing, Density_Grid, ADensity_Grid, dVHart_Grid, *, ctx=None):
    """``Solve_Poisson!`` (src/Poisson.jl:1-7): fills dVHart_Grid.  Runs on
    dft_mixing's context (or ``ctx``)."""
    ctx = _ctx_of(dft_mixing, ctx=ctx)
    s = _spin(SpinPol)
    nr = 1 if s == "off" else 2
    rho = [_f64(Density_Grid[c]) for c in range(nr)]
    pr, keep = dptrs(rho)
    ng = np.array(dft_mixing.Ngrid, dtype=np.int32)
    rv = _f64(dft_mixing.Recvecs)
    ad = None if ADensity_Grid is None else _f64(ADensity_Grid)
    check(lib.lcp_solve_poisson(ctx._h, iptr(ng), dptr(rv), _lib.SPIN[s], pr, dptr(ad), dptr(dVHart_Grid)))


def Solve_Poisson_xyz(Ngrid, Recvecs, Density_xyz, dVHart_Grid, *, ctx=None):
    """Inner ``Solve_Poisson!(Ngrid, Recvecs, Density_xyz, dVHart_Grid)`` for a
    real Density_xyz (src/Poisson.jl:29-108), on the module's default context
    (or ``ctx``)."""
    ctx = _ctx_of(ctx=ctx)
    ng = np.array(Ngrid, dtype=np.int32)
    src = _f64(np.real(np.asarray(Density_xyz)).reshape(-1))
    check(lib.lcp_solve_poisson_xyz(ctx._h, iptr(ng), dptr(_f64(Recvecs)), dptr(src), dptr(dVHart_Grid)))


def _xc_name(xc_type):
    """xc_type spellings accepted by the reference (src/DFT_Setup.jl:436-447)."""
    x = xc_type.strip().upper().replace("-", "_")
    if x in ("GGA", "PBE"):
        x = "GGA_PBE"
    if x not in _lib.XC:
        raise LCPError(_lib.LCP_EINVAL, "please check xc_type name")
    return x


def Calc_Diff_Coef(gLatvecs):
    """``Calc_Diff_Coef(gLatvecs)`` (src/XC/GGA_PBE.jl:1-39): the x, y, z
    weights of the 27-point gradient stencil, as three length-27 arrays."""
    out = np.zeros(81)
    check(lib.lcp_calc_diff_coef(dptr(_f64(gLatvecs).reshape(3, 3)), dptr(out)))
    return [out[0:27].copy(), out[27:54].copy(), out[54:81].copy()]


class XC_Func:
    """``XC_Func(xc_type, SpinPol, Nspin, Ngrid, gLatvecs)``
    (src/XC/XC_Func.jl:47-108).  GGA_PBE needs gLatvecs (rows Latvecs[i] /
    Ngrid[i]) for its Diff_Coef and carries dDensity_Grid and dEXC_dGD.
    ``ctx`` is the device context of Set_XC_Grid / Set_Vpot_Grid on this
    object (the module's default when None)."""

    def __init__(self, xc_type, SpinPol, Nspin, Ngrid, gLatvecs=None, ctx=None):
        self.ctx = ctx
        xc = _xc_name(xc_type)
        sp = SpinPol.lower()
        if sp not in _lib.SPIN:
            raise LCPError(_lib.LCP_EINVAL, "please check SpinPol name")
        if xc == "LDA" and sp != "off" or xc == "LSDA" and sp == "off":
            raise LCPError(_lib.LCP_EINVAL, "please check xc_type and SpinPol")
        self.xc_type = xc
        self.SpinPol = sp
        self.Nspin = int(Nspin)
        self.Ngrid = tuple(int(x) for x in Ngrid)
        nn = int(np.prod(self.Ngrid))
        self.Vxc_Grid = [np.zeros(nn) for _ in range(_lib.NCHAN[sp])]
        if xc == "GGA_PBE":
            if gLatvecs is None:
                raise LCPError(_lib.LCP_EINVAL, "GGA_PBE needs gLatvecs")
            self.Diff_Coef = Calc_Diff_Coef(gLatvecs)
            ns = max(self.Nspin, 1 if sp == "off" else 2)
            self.dDensity_Grid = [[np.zeros(nn) for _ in range(3)] for _ in range(ns)]
            self.dEXC_dGD = [[np.zeros(nn) for _ in range(3)] for _ in range(ns)]


def Set_XC_Grid(xc_func, PCCDensity_Grid, Density_Grid, *, ctx=None):
    """``Set_XC_Grid!`` (src/XC/XC_Func.jl:111-160): fills xc_func.Vxc_Grid
    (and, for GGA_PBE, xc_func.dDensity_Grid and xc_func.dEXC_dGD).  Runs on
    xc_func's context (or ``ctx``)."""
    ctx = _ctx_of(xc_func, ctx=ctx)
    n = _lib.NCHAN[xc_func.SpinPol]
    nn = int(np.prod(xc_func.Ngrid))
    rho = [_f64(Density_Grid[c]) for c in range(n)]
    pr, k1 = dptrs(rho)
    pv, k2 = dptrs(xc_func.Vxc_Grid)
    pcc = None if PCCDensity_Grid is None else _f64(PCCDensity_Grid)
    if xc_func.xc_type == "GGA_PBE":
        ns = 1 if xc_func.SpinPol == "off" else 2
        ng = np.array(xc_func.Ngrid, dtype=np.int32)
        dc = _f64(np.concatenate(xc_func.Diff_Coef))
        pd, k3 = dptrs([xc_func.dDensity_Grid[s][a] for s in range(ns) for a in range(3)])
        pe, k4 = dptrs([xc_func.dEXC_dGD[s][a] for s in range(ns) for a in range(3)])
        check(lib.lcp_set_xc_grid_gga(ctx._h, _lib.SPIN[xc_func.SpinPol], iptr(ng), dptr(dc), dptr(pcc), pr, pv,
                                      pd, pe))
        return
    check(lib.lcp_set_xc_grid(ctx._h, _lib.XC[xc_func.xc_type], _lib.SPIN[xc_func.SpinPol], nn, dptr(pcc), pr, pv))


def Set_Vpot_Grid(xc_func, dVHart_Grid, Vpot_Grid, *, Vna_Grid=None, ctx=None):
    """``Set_Vpot_Grid!`` (src/Matrix/Set_Vpot_Grid.jl:1-19); Vna_Grid
    (keyword), when given, is added to the spin-diagonal channels.  Runs on
    xc_func's context (or ``ctx``)."""
    ctx = _ctx_of(xc_func, ctx=ctx)
    n = _lib.NCHAN[xc_func.SpinPol]
    nn = int(np.prod(xc_func.Ngrid))
    px, k1 = dptrs([_f64(v) for v in xc_func.Vxc_Grid])
    pv, k2 = dptrs([Vpot_Grid[c] for c in range(n)])
    vna = None if Vna_Grid is None else _f64(Vna_Grid)
    check(lib.lcp_set_vpot_grid(ctx._h, _lib.SPIN[xc_func.SpinPol], nn, dptr(_f64(dVHart_Grid)), px, dptr(vna), pv))


def _matrix_elements(spin, ucell, Orbs_Grid, Vpot_Grid, MPI_Hks):
    n = _lib.NCHAN[spin]
    pv, k1 = dptrs([_f64(Vpot_Grid[c]) for c in range(n)])
    for c in range(n):
        if MPI_Hks[c].size != ucell.Total_Hsize:
            raise LCPError(_lib.LCP_EINVAL, "MPI_Hks size does not match Total_Hsize")
    ph, k2 = dptrs([MPI_Hks[c] for c in range(n)])
    check(lib.lcp_calc_matrix_elements(Orbs_Grid.ctx._h, ucell._h, Orbs_Grid._h, _lib.SPIN[spin], pv, ph))


def Calc_MatrixElements_dVH_Vxc_off(ucell, Orbs_Grid, Vpot_Grid, MPI_Hks):
    """src/Hamiltonian.jl:235-277."""
    _matrix_elements("off", ucell, Orbs_Grid, Vpot_Grid, MPI_Hks)


def Calc_MatrixElements_dVH_Vxc_on(ucell, Orbs_Grid, Vpot_Grid, MPI_Hks):
    """src/Hamiltonian.jl:280-324."""
    _matrix_elements("on", ucell, Orbs_Grid, Vpot_Grid, MPI_Hks)


def Calc_MatrixElements_dVH_Vxc_nc(ucell, Orbs_Grid, Vpot_Grid, MPI_Hks):
    """src/Hamiltonian.jl:327-380."""
    _matrix_elements("nc", ucell, Orbs_Grid, Vpot_Grid, MPI_Hks)


def _force3(spin, pao, Orbs_Grid, Vpot, DM, ucell):
    """The reference tabulates the gradient tables inside Force3; here they
    come with Orbs_Grid when it was made by Set_dOrbitals_Grid, else they are
    tabulated (on Orbs_Grid's context) for this call."""
    orbs = Orbs_Grid if getattr(Orbs_Grid, "with_grad", False) else Set_dOrbitals_Grid(pao, ucell, ctx=Orbs_Grid.ctx)
    n = _lib.NCHAN[spin]
    vp, keep_v = dptrs([_f64(Vpot[c]) for c in range(n)])
    dp, keep_d = dptrs([_f64(DM[c]) for c in range(n)])
    out = np.zeros((ucell.Natom, 3))
    check(lib.lcp_calc_force3(orbs.ctx._h, ucell._h, orbs._h, _lib.SPIN[spin], vp, dp, dptr(out)))
    return out


def Force3_nospin(pao, Orbs_Grid, Vpot_Grid, DM, ucell):
    """src/Force.jl:405-446: VpotForce [Natom, 3]; DM as flat pair blocks."""
    return _force3("off", pao, Orbs_Grid, Vpot_Grid, DM, ucell)


def Force3_spin(pao, Orbs_Grid, Vpot_Grid, DM, ucell):
    """src/Force.jl:449-499."""
    return _force3("on", pao, Orbs_Grid, Vpot_Grid, DM, ucell)


def Force3_nc(pao, Orbs_Grid, dVHart_Grid, Vxc_Grid, DM, ucell):
    """src/Force.jl:502-566: Vpot1 = dVHart + Vxc1, Vpot2 = dVHart + Vxc2."""
    dv = _f64(dVHart_Grid)
    V = [dv + _f64(Vxc_Grid[0]), dv + _f64(Vxc_Grid[1]), _f64(Vxc_Grid[2]), _f64(Vxc_Grid[3])]
    return _force3("nc", pao, Orbs_Grid, V, DM, ucell)


def Calc_EH1(SpinPol, GridVol, ADensity_Grid, Density_Grid, dVHart_Grid, *, ctx=None):
    """src/Energy.jl:655-666, on the module's default context (or ``ctx``)."""
    ctx = _ctx_of(ctx=ctx)
    s = _spin(SpinPol)
    nr = 1 if s == "off" else 2
    rho = [_f64(Density_Grid[c]) for c in range(nr)]
    pr, keep = dptrs(rho)
    out = ctypes.c_double()
    ad = None if ADensity_Grid is None else _f64(ADensity_Grid)
    check(lib.lcp_calc_eh1(ctx._h, _lib.SPIN[s], rho[0].size, float(GridVol), dptr(ad), pr, dptr(_f64(dVHart_Grid)),
                           ctypes.byref(out)))
    return out.value


def Calc_EXC1(SpinPol, xc_type, system_grid, ADensity_Grid, PCCDensity_Grid, Density_Grid, *, ctx=None):
    """src/Energy.jl:669-700; ``system_grid`` supplies GridVol, and for
    GGA_PBE also Ngrid and Latvecs (a UCell works).  Runs on system_grid's
    context when it carries one (or ``ctx``), else the module's default."""
    ctx = _ctx_of(system_grid, ctx=ctx)
    s = _spin(SpinPol)
    nr = 1 if s == "off" else 2
    rho = [_f64(Density_Grid[c]) for c in range(nr)]
    pr, keep = dptrs(rho)
    out = np.zeros(2)
    ad = None if ADensity_Grid is None else _f64(ADensity_Grid)
    pcc = None if PCCDensity_Grid is None else _f64(PCCDensity_Grid)
    xc = _xc_name(xc_type)
    if xc == "GGA_PBE":
        ng = np.array(system_grid.Ngrid, dtype=np.int32)
        lat = _f64(system_grid.Latvecs).reshape(3, 3)
        check(lib.lcp_calc_exc1_grid(ctx._h, _lib.XC[xc], _lib.SPIN[s], iptr(ng), dptr(lat),
                                     float(system_grid.GridVol), dptr(ad), dptr(pcc), pr, dptr(out)))
        return out
    check(lib.lcp_calc_exc1(ctx._h, _lib.XC[xc], _lib.SPIN[s], rho[0].size, float(system_grid.GridVol),
                            dptr(ad), dptr(pcc), pr, dptr(out)))
    return out


def Calc_Ngrid(Ecut, Latvecs):
    """src/utils/Calc_Ngrid.jl:1-20."""
    out = np.zeros(3, dtype=np.int32)
    check(lib.lcp_calc_ngrid(float(Ecut), dptr(_f64(Latvecs).reshape(-1)), iptr(out)))
    return tuple(int(x) for x in out)


class GridStepJob:
    """Device-resident SCF grid step: density from D, Poisson, xc, potential
    (+ V_na), grid H and the FP64 energy terms, all on the GPU."""

    def __init__(self, ucell, Orbs_Grid, SpinPol, xc_type, ADensity_Grid=None, PCCDensity_Grid=None, Vna_Grid=None):
        self.ctx = Orbs_Grid.ctx
        self.ucell = ucell
        self.orbs = Orbs_Grid  # the device job reads these tables: keep them alive
        self.SpinPol = _spin(SpinPol)
        self.nspin = _lib.NCHAN[self.SpinPol]
        keep = [None if x is None else _f64(x) for x in (ADensity_Grid, PCCDensity_Grid, Vna_Grid)]
        h = ctypes.c_void_p()
        check(lib.lcp_job_create(self.ctx._h, ucell._h, Orbs_Grid._h, _lib.SPIN[self.SpinPol],
                                 _lib.XC[_xc_name(xc_type)], dptr(keep[0]), dptr(keep[1]), dptr(keep[2]),
                                 ctypes.byref(h)))
        self._h = h

    def set_dm(self, DM):
        p, keep = dptrs([_f64(DM[c]) for c in range(self.nspin)])
        check(lib.lcp_job_set_dm(self.ctx._h, self._h, p))

    def step(self, ctx=None):
        """One step on `ctx` (default: the context of the job's orbitals)."""
        check(lib.lcp_job_step((ctx or self.ctx)._h, self._h))

    def step_timed(self):
        """One step with per-stage CUDA-event times (ms): density, Poisson,
        xc+potential, energy sums, grid H, <D,H> + energy."""
        out = np.zeros(6)
        check(lib.lcp_job_step_timed(self.ctx._h, self._h, dptr(out)))
        return out

    def energies(self):
        """[E_H1, EXC1[1], EXC1[2], sum_s <D_s, H_s>, E_grid]."""
        out = np.zeros(5)
        check(lib.lcp_job_energies(self.ctx._h, self._h, dptr(out)))
        return out

    def energies_async(self, out):
        """Queues the copy of the last step's energies into ``out`` (5
        float64, e.g. pinned) on the context stream without waiting: the next
        call that synchronises (``hks``, ``density``, ``energies``) completes
        it.  ``out`` must stay alive until then."""
        if out.dtype != np.float64 or out.size != 5 or not out.flags["C_CONTIGUOUS"]:
            raise TypeError("out must be 5 contiguous float64")
        check(lib.lcp_job_energies_async(self.ctx._h, self._h, dptr(out)))
        return out

    def tc_kernel_ms(self):
        """One split-BF16 step with CUDA events around its tensor-core kernels
        alone: (density kernel ms, grid-H kernel ms), summed over channels."""
        out = np.zeros(2)
        check(lib.lcp_job_tc_kernel_ms(self.ctx._h, self._h, dptr(out)))
        return float(out[0]), float(out[1])

    def prepare(self):
        """Builds what the context's precision needs of the orbital tables
        (split-BF16 brick tables, FP32 copy) ahead of the first step."""
        check(lib.lcp_job_prepare(self.ctx._h, self._h))

    def footprint(self):
        """Device bytes of the job and its orbital tables."""
        out = ctypes.c_int64()
        check(lib.lcp_job_footprint(self._h, ctypes.byref(out)))
        return int(out.value)

    def _get(self, fn, n, out=None):
        outs = out if out is not None else [np.zeros(n) for _ in range(self.nspin)]
        for o in outs:
            if o.dtype != np.float64 or o.size != n or not o.flags["C_CONTIGUOUS"]:
                raise TypeError("output arrays must be C-contiguous float64 of the grid / H size")
        p, keep = dptrs(outs)
        check(fn(self.ctx._h, self._h, p))
        return outs

    def density(self, out=None):
        return self._get(lib.lcp_job_get_density, self.ucell.NN, out)

    def hks(self, out=None):
        """H of the last step; `out` (one array per spin, e.g. in pinned memory)
        receives it in place."""
        return self._get(lib.lcp_job_get_hks, self.ucell.Total_Hsize, out)

    def vpot(self, out=None):
        return self._get(lib.lcp_job_get_vpot, self.ucell.NN, out)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib.lcp_job_destroy(self._h)
                self._h = None
        except Exception:
            pass


class Batch:
    """Batched grid step over the device-resident jobs of many cells
    (lcp_batch_*): one persistent tensor-core launch per contraction over the
    bricks of every cell, batched FFTs per grid shape, tiled grid kernels over
    all cells, replayed as one CUDA graph.  Results land in the jobs (read
    them with job.energies() / job.hks() / job.density())."""

    GRAPH, EAGER = 0, 1

    def __init__(self, jobs, scratch_bytes=0, ctx=None):
        """scratch_bytes: budget of the partial H blocks (0: none); the cells
        are then stepped in waves of the matrix-element pass.  ctx: the
        split-BF16 context that steps the batch (default: the first job's)."""
        self.jobs = list(jobs)  # the batch reads their buffers: keep them alive
        if not self.jobs:
            raise ValueError("a batch needs at least one job")
        self.ctx = ctx if ctx is not None else self.jobs[0].ctx
        arr = (ctypes.c_void_p * len(self.jobs))(*[j._h.value for j in self.jobs])
        h = ctypes.c_void_p()
        check(lib.lcp_batch_create(self.ctx._h, len(self.jobs), arr, int(scratch_bytes), ctypes.byref(h)))
        self._h = h

    def step(self, graph=True):
        check(lib.lcp_batch_step(self.ctx._h, self._h, self.GRAPH if graph else self.EAGER))

    def step_timed(self):
        """One eager step with per-stage CUDA-event times (ms), as
        GridStepJob.step_timed, for all cells together."""
        out = np.zeros(6)
        check(lib.lcp_batch_step_timed(self.ctx._h, self._h, dptr(out)))
        return out

    def check_status(self):
        check(lib.lcp_batch_check_status(self.ctx._h, self._h))

    def energies(self):
        """[njobs, 5]: each job's energies (as GridStepJob.energies)."""
        out = np.zeros(5 * len(self.jobs))
        check(lib.lcp_batch_energies(self.ctx._h, self._h, dptr(out)))
        return out.reshape(-1, 5)

    def info(self):
        """dict: cells, shape groups, bricks, kernels per step, workspace bytes,
        graph captured, H sub-blocks, waves of the H pass."""
        out = (ctypes.c_int64 * 8)()
        check(lib.lcp_batch_info(self._h, out))
        keys = ("cells", "shape_groups", "bricks", "kernels_per_step", "workspace_bytes", "graph", "h_subblocks",
                "waves")
        return {k: int(v) for k, v in zip(keys, out)}

    def close(self):
        if getattr(self, "_h", None):
            lib.lcp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving engine for SCF grid-step requests on device-resident structures
    (lcp_server_*): `nslots` execution slots at one precision, each stepping
    the pending requests it takes as one batched step (split-BF16: up to
    `max_batch` requests per step, 16 by default; FP64/FP32: one), structures
    admitted by device footprint against `budget_bytes`, with an admission
    queue for those that do not fit yet."""

    ADMITTED, WAITING, ADMITTING = 0, 1, 2

    def __init__(self, device=0, nslots=4, precision="bf16x3", budget_bytes=160e9, max_batch=None):
        h = ctypes.c_void_p()
        check(lib.lcp_server_create(int(device), int(nslots), _lib.PREC[precision], int(budget_bytes),
                                    ctypes.byref(h)))
        self._h = h
        self._jobs = {}
        if max_batch is not None:
            self.set_max_batch(max_batch)

    def set_max_batch(self, n):
        """Requests per batched step (1: every request steps alone)."""
        check(lib.lcp_server_set_max_batch(self._h, int(n)))

    def state(self, sid):
        """Server.ADMITTED, WAITING (admission queue) or ADMITTING."""
        out = ctypes.c_int32()
        check(lib.lcp_server_state(self._h, int(sid), ctypes.byref(out)))
        return out.value

    def batch_stats(self):
        """(batched steps run, requests they carried, structures waiting for
        admission, ms assembling those batches, their wall ms)."""
        out = (ctypes.c_int64 * 5)()
        check(lib.lcp_server_batch_stats(self._h, out))
        return tuple(int(x) for x in out[:3]) + (out[3] / 1000.0, out[4] / 1000.0)

    def add(self, job):
        """Adds a GridStepJob (kept alive by the server object); returns its id.
        It is admitted now when its footprint fits the free budget, else it
        waits in the admission queue (its requests wait with it) until
        removals free the budget.  Raises LCPError (LCP_ENOMEM) only when the
        footprint exceeds the whole budget."""
        i = ctypes.c_int32()
        check(lib.lcp_server_add(self._h, job._h, job.nspin, job.ucell.Total_Hsize, ctypes.byref(i)))
        self._jobs[i.value] = job
        return i.value

    def remove(self, sid):
        check(lib.lcp_server_remove(self._h, int(sid)))
        self._jobs.pop(sid, None)

    def submit(self, sid, DM, tag):
        job = self._jobs[sid]
        p, keep = dptrs([_f64(DM[c]) for c in range(job.nspin)])
        check(lib.lcp_server_submit(self._h, int(sid), p, ctypes.c_uint64(int(tag))))

    def poll(self, max_results=4096, wait_ms=0):
        """Completed requests: list of (tag, energies[5], latency_ms)."""
        tags = (ctypes.c_uint64 * max_results)()
        en = np.zeros(5 * max_results)
        lat = np.zeros(max_results)
        n = ctypes.c_int32()
        check(lib.lcp_server_poll(self._h, int(max_results), int(wait_ms), tags, dptr(en), dptr(lat),
                                  ctypes.byref(n)))
        return [(int(tags[k]), en[5 * k:5 * k + 5].copy(), float(lat[k])) for k in range(n.value)]

    def stats(self):
        """(submitted, completed, resident bytes, budget bytes)."""
        out = (ctypes.c_int64 * 4)()
        check(lib.lcp_server_stats(self._h, out))
        return tuple(int(x) for x in out)

    def close(self):
        if getattr(self, "_h", None):
            lib.lcp_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

