"""CPU oracle: a numpy restatement of LCPAODFT.jl's real-space grid path.

TEST INFRASTRUCTURE ONLY.  This module is the checker the parity tests, the
smoke check and the CPU-baseline leg of ``bench.py`` compare the CUDA path
against.  Nothing in the product library imports or calls it.

Every function states the reference file and lines it follows (paths are
relative to the LCPAODFT.jl project root).  Reference behaviour is kept,
including its quirks, with two deliberate differences that only matter where
the reference itself throws a BoundsError:

* the radial spline index ``m`` is clamped so that ``m-2 >= 1`` and
  ``m+1 <= Nmesh`` (``src/Matrix/Set_Orbitals_Grid.jl:198-221`` and
  ``src/Matrix/Set_dOrbitals_Grid.jl:202-225`` read ``RV[m-2]`` for
  ``RV[1] <= R < RV[2]``);
* nothing else.  The stale-coordinate behaviour of ``Find_CGrids!`` for image
  cells outside ``+-CpyCell`` (``src/utils/Find_CGrid.jl:11-16``) is
  reproduced as written.

Parity is pinned against the reference's own golden vectors
(``tests/golden/golden_vectors.json``, extracted from ``test/*.jl``):
sphere lists and neighbour lists (``test/test_UCell.jl``), orbital values
(``test/test_Set_Orbs_Grid.jl``), the Poisson solve (``test/test_Poisson.jl``),
the xc kernels and grids (``test/test_LDA_CA.jl``, ``test/test_LSDA_CA.jl``,
``test/test_Set_XC_Grid.jl``), the atomic/PCC densities
(``test/test_Set_AdenPCC_Grid.jl``) and grid sizes (``test/test_Calc_Ngrid.jl``).
Density assembly and grid matrix elements have no reference test; they are
pinned by exact identities checked in ``tests/test_oracle.py``.
"""
import math

import numpy as np

PI = math.pi
ANG_TO_BOHR = 1.8897259886  # src/LCPAODFT.jl:18
DENSITY_BLOCK = 512          # src/LCPAODFT.jl:54-55


# --------------------------------------------------------------------------
# lattice helpers


def generation_atv(N, latvecs):
    """Image-cell tables (src/utils/Generation_ATV.jl:51-88).

    Returns ``atv`` [(2N+1)^3, 3] (cell translation vectors, cell 0 first),
    ``atv_ijk`` [(2N+1)^3, 3] and ``ratv`` [(2N+1)]^3 mapping (i+N, j+N, k+N)
    to the cell number.
    """
    n = 2 * N + 1
    atv = np.zeros((n ** 3, 3))
    ijk = np.zeros((n ** 3, 3), dtype=np.int64)
    ratv = np.zeros((n, n, n), dtype=np.int64)
    L = np.asarray(latvecs, dtype=np.float64)
    rn = 1
    for i in range(-N, N + 1):
        for j in range(-N, N + 1):
            for k in range(-N, N + 1):
                if i == 0 and j == 0 and k == 0:
                    ratv[N, N, N] = 0
                    continue
                for c in range(3):
                    atv[rn, c] = i * L[0, c] + j * L[1, c] + k * L[2, c]
                ijk[rn] = (i, j, k)
                ratv[i + N, j + N, k + N] = rn
                rn += 1
    return atv, ijk, ratv


def _estimate_fnan(natom, gxyz, cut, atv):
    """src/UCell.jl:573-608."""
    fnan = np.zeros(natom, dtype=np.int64)
    for a in range(natom):
        for b in range(natom):
            rcut = cut[a] + cut[b]
            d = np.abs(gxyz[a][None, :] - gxyz[b][None, :] - atv)
            ok = (d[:, 0] <= rcut) & (d[:, 1] <= rcut) & (d[:, 2] <= rcut)
            r = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
            ok &= r <= rcut
            if a == b:
                ok[0] = False
            fnan[a] += int(ok.sum())
    return fnan


def trn_system(natom, gxyz, cut, atv):
    """Neighbour lists (src/UCell.jl:612-672): self first, then (jatom, Rn) order."""
    natn, ncn, dis = [], [], []
    for a in range(natom):
        na, nc, ds = [a + 1], [0], [0.0]
        for b in range(natom):
            rcut = cut[a] + cut[b]
            for rn in range(atv.shape[0]):
                if a == b and rn == 0:
                    continue
                dx = abs(gxyz[a][0] - gxyz[b][0] - atv[rn, 0])
                dy = abs(gxyz[a][1] - gxyz[b][1] - atv[rn, 1])
                dz = abs(gxyz[a][2] - gxyz[b][2] - atv[rn, 2])
                if dx <= rcut and dy <= rcut and dz <= rcut:
                    r = math.sqrt(dx * dx + dy * dy + dz * dz)
                    if r <= rcut:
                        na.append(b + 1)
                        nc.append(rn)
                        ds.append(r)
        natn.append(na)
        ncn.append(nc)
        dis.append(ds)
    fnan = np.array([len(x) - 1 for x in natn], dtype=np.int64)
    return fnan, natn, ncn, dis


def get_fnan(latvecs, natom, gxyz, cut):
    """CpyCell search (src/UCell.jl:520-556)."""
    cpy = 0
    tf = 0
    count = 1
    po = 0
    while po == 0 and count < 7:
        cpy += 1
        atv, _, _ = generation_atv(cpy, latvecs)
        tf_prev = tf
        tf = int(_estimate_fnan(natom, gxyz, cut, atv).sum())
        if tf == tf_prev:
            po = 1
        count += 1
    if count == 7 or po == 0:
        raise RuntimeError("please check Get_FNAN")
    atv, _, _ = generation_atv(cpy, latvecs)
    fnan, natn, ncn, dis = trn_system(natom, gxyz, cut, atv)
    return cpy, fnan, natn, ncn, dis


def calc_ngrid(ecut, latvecs):
    """src/utils/Calc_Ngrid.jl:1-76."""
    L = np.asarray(latvecs, dtype=np.float64)
    vol = abs(np.linalg.det(L))
    temp = vol / PI * math.sqrt(ecut)
    ns = [temp / np.linalg.norm(np.cross(L[1], L[2])),
          temp / np.linalg.norm(np.cross(L[2], L[0])),
          temp / np.linalg.norm(np.cross(L[0], L[1]))]
    out = []
    for n in ns:
        lgn = math.log(n)
        best = (1e10, 0, 0, 0, 0)
        l2, l3, l5, l7 = math.log(2), math.log(3), math.log(5), math.log(7)
        for p in range(0, math.ceil(lgn / l2) + 1):
            for q in range(0, math.ceil((lgn - p * l2) / l3) + 1):
                for r in range(0, math.ceil((lgn - p * l2 - q * l3) / l5) + 1):
                    for s in range(0, math.ceil((lgn - p * l2 - q * l3 - r * l5) / l7) + 1):
                        lg = p * l2 + q * l3 + r * l5 + s * l7
                        if abs(lg - lgn) < best[0]:
                            best = (abs(lg - lgn), p, q, r, s)
        _, p, q, r, s = best
        out.append(2 ** p * 3 ** q * 5 ** r * 7 ** s)
    return tuple(out)


# --------------------------------------------------------------------------
# UCell: sphere lists and pair overlaps


def _glatvecs(latvecs, ngrid):
    L = np.asarray(latvecs, dtype=np.float64)
    g = np.empty((3, 3))
    for d in range(3):
        g[d, :] = L[d, :] / ngrid[d]
    return g


def calc_atoms_grid(latvecs, natom, cpy, gxyz, cut, ngrid, origin):
    """Per-atom cutoff-sphere point lists (src/UCell.jl:297-411).

    Returns GridN_Atom, GridListAtom (flat C-order grid index) and CellListAtom
    (image cell number), each list stably sorted by grid index.  The loop order
    (n3 fastest) and the stale ``Cxyz`` of ``Find_CGrids!`` for image cells
    outside ``+-CpyCell`` (src/utils/Find_CGrid.jl:11-27) are kept.
    """
    N1, N2, N3 = (int(x) for x in ngrid)
    L = np.asarray(latvecs, dtype=np.float64)
    atv, _, ratv = generation_atv(cpy, L)
    gL = _glatvecs(L, ngrid)
    grec = 2 * PI * np.linalg.inv(gL.T)
    org = np.asarray(origin, dtype=np.float64)
    kindex = [(1, 2), (2, 0), (0, 1)]
    last_c = np.zeros(3)          # Cxyz persists across points and atoms (:330)
    gn, glist, clist = [], [], []
    for a in range(natom):
        Gx, Gy, Gz = (float(v) for v in gxyz[a])
        rcut = cut[a] + 0.5
        nmin = [0, 0, 0]
        nmax = [0, 0, 0]
        for k in range(3):
            i, j = kindex[k]
            vx = L[i, 1] * L[j, 2] - L[i, 2] * L[j, 1]
            vy = L[i, 2] * L[j, 0] - L[i, 0] * L[j, 2]
            vz = L[i, 0] * L[j, 1] - L[i, 1] * L[j, 0]
            coef = 1.0 / math.sqrt(vx * vx + vy * vy + vz * vz)
            vx, vy, vz = vx * coef, vy * coef, vz * coef
            cx, cy, cz = Gx + rcut * vx - org[0], Gy + rcut * vy - org[1], Gz + rcut * vz - org[2]
            nmax[k] = math.trunc((cx * grec[k, 0] + cy * grec[k, 1] + cz * grec[k, 2]) * 0.5 / PI)
            cx, cy, cz = Gx - rcut * vx - org[0], Gy - rcut * vy - org[1], Gz - rcut * vz - org[2]
            nmin[k] = math.trunc((cx * grec[k, 0] + cy * grec[k, 1] + cz * grec[k, 2]) * 0.5 / PI)
            if nmax[k] < nmin[k]:
                nmin[k], nmax[k] = nmax[k], nmin[k]
        n1, n2, n3 = np.meshgrid(np.arange(nmin[0], nmax[0] + 1), np.arange(nmin[1], nmax[1] + 1),
                                 np.arange(nmin[2], nmax[2] + 1), indexing="ij")
        n1, n2, n3 = n1.ravel(), n2.ravel(), n3.ravel()
        # Find_ln: floor division / modulo (src/utils/Find_CGrid.jl:32-49)
        l1, nn1 = np.floor_divide(n1, N1), np.mod(n1, N1)
        l2, nn2 = np.floor_divide(n2, N2), np.mod(n2, N2)
        l3, nn3 = np.floor_divide(n3, N3), np.mod(n3, N3)
        s1, s2, s3 = l1 + 1, l2 + 1, l3 + 1  # the shifted index the range check uses
        inr = (np.abs(s1) <= cpy) & (np.abs(s2) <= cpy) & (np.abs(s3) <= cpy)
        rn = np.zeros(n1.shape, dtype=np.int64)
        rn[inr] = ratv[cpy + s1[inr] - 1, cpy + s2[inr] - 1, cpy + s3[inr] - 1]
        c = np.empty((n1.size, 3))
        for d in range(3):
            c[:, d] = atv[rn, d] + nn1 * gL[0, d] + nn2 * gL[1, d] + nn3 * gL[2, d] + org[d]
        if not inr.all():
            # stale Cxyz: out-of-range points reuse the last in-range coordinates
            idx = np.where(inr, np.arange(n1.size), -1)
            idx = np.maximum.accumulate(idx)
            prev = np.where(idx[:, None] >= 0, c[np.maximum(idx, 0)], last_c[None, :])
            c = np.where(inr[:, None], c, prev)
        if n1.size:
            last_c = c[-1].copy()
        dx, dy, dz = c[:, 0] - Gx, c[:, 1] - Gy, c[:, 2] - Gz
        R = np.sqrt(dx * dx + dy * dy + dz * dz)
        keep = R <= cut[a]
        N = nn1 * (N2 * N3) + nn2 * N3 + nn3
        gl = N[keep].astype(np.int64)
        cl = rn[keep].astype(np.int64)
        order = np.argsort(gl, kind="stable")
        glist.append(gl[order])
        clist.append(cl[order])
        gn.append(int(keep.sum()))
    return np.array(gn, dtype=np.int64), glist, clist


def calc_atom_overlap_grid_literal(cpy, pairs, gridN, glist, clist, atv_ijk, ratv):
    """Literal restatement of the merge walk (src/UCell.jl:425-516).

    Pure-Python loops: only for small cases.  ``pairs`` is a list of
    (atom, jatom, cell) with 1-based atoms.
    """
    out1, out2 = [], []
    for atom, jatom, cell in pairs:
        a, b = atom - 1, jatom - 1
        l1, l2, l3 = atv_ijk[cell]
        t1, t2 = [], []
        nc = 0
        gi, ci = glist[a], clist[a]
        for nh in range(gridN[b]):
            gnh = int(glist[b][nh])
            grh = int(clist[b][nh])
            ll = atv_ijk[grh]
            lll1, lll2, lll3 = l1 + ll[0], l2 + ll[1], l3 + ll[2]
            if gi[0] <= gnh:
                if gnh == 0:
                    nc = 0
                else:
                    while gnh <= gi[nc] and nc != 0:
                        nc = max(nc - 10, 0)
                if abs(lll1) <= cpy and abs(lll2) <= cpy and abs(lll3) <= cpy:
                    grh1 = ratv[lll1 + cpy, lll2 + cpy, lll3 + cpy]
                    po = 0
                    while po == 0 and nc < gridN[a]:
                        gnc, grc = gi[nc], ci[nc]
                        if gnc == gnh and grc == grh1:
                            t1.append(nc)
                            t2.append(nh)
                            po = 1
                        elif gnh < gnc:
                            po = 1
                        nc += 1
                    nc = max(nc - 1, 0)
        out1.append(np.array(t1, dtype=np.int64))
        out2.append(np.array(t2, dtype=np.int64))
    return out1, out2


def calc_atom_overlap_grid(cpy, pairs, glist, clist, atv_ijk, ratv):
    """Vectorised equivalent of the merge walk (src/UCell.jl:425-516).

    For each pair (atom, jatom, cell R), keeps every point Nh of jatom's list
    whose physical twin (same grid index, image cell = cell(Nh) + R) is in
    atom's list, in Nh order.  ``tests/test_oracle.py`` checks it against
    ``calc_atom_overlap_grid_literal``.
    """
    n = 2 * cpy + 1
    keys_i = {}
    out1, out2 = [], []
    for atom, jatom, cell in pairs:
        a, b = atom - 1, jatom - 1
        if a not in keys_i:
            k = glist[a] * (n ** 3) + clist[a]
            order = np.argsort(k, kind="stable")
            keys_i[a] = (k[order], order)
        ks, order = keys_i[a]
        if ks.size == 0:
            out1.append(np.zeros(0, dtype=np.int64))
            out2.append(np.zeros(0, dtype=np.int64))
            continue
        ll = atv_ijk[clist[b]] + atv_ijk[cell][None, :]
        inr = np.all(np.abs(ll) <= cpy, axis=1)
        grh1 = np.full(ll.shape[0], -1, dtype=np.int64)
        grh1[inr] = ratv[ll[inr, 0] + cpy, ll[inr, 1] + cpy, ll[inr, 2] + cpy]
        kj = glist[b] * (n ** 3) + grh1
        pos = np.minimum(np.searchsorted(ks, kj), ks.size - 1)
        hit = inr & (ks[pos] == kj)
        nh = np.nonzero(hit)[0]
        out1.append(order[pos[nh]].astype(np.int64))
        out2.append(nh.astype(np.int64))
    return out1, out2


class UCell:
    """Grid geometry of one cell, field names as in ``struct UCell``
    (src/UCell.jl:1-46) and built as ``UCell(Nspin, Latvecs, ...)``
    (src/UCell.jl:210-294) with one MPI rank."""

    def __init__(self, nspin, latvecs, natom, atom2spe, gxyz, cut, ngrid, origin,
                 total_numorbs=None, overlap="vectorised", pair_subset=None):
        self.Nspin = nspin
        self.Latvecs = np.asarray(latvecs, dtype=np.float64)
        self.Natom = natom
        self.atom2spe = list(atom2spe)
        self.Gxyz = [np.asarray(g, dtype=np.float64) for g in gxyz]
        self.Atoms_Cut1 = [float(c) for c in cut]
        self.Ngrid = tuple(int(x) for x in ngrid)
        self.Grid_Origin = np.asarray(origin, dtype=np.float64)
        cpy, fnan, natn, ncn, dis = get_fnan(self.Latvecs, natom, self.Gxyz, self.Atoms_Cut1)
        self.CpyCell, self.FNAN, self.natn, self.ncn, self.Dis = cpy, fnan, natn, ncn, dis
        self.atv, self.atv_ijk, self.ratv = generation_atv(cpy, self.Latvecs)
        if total_numorbs is None:
            total_numorbs = [0] * natom
        self.Total_NumOrbs = np.asarray(total_numorbs, dtype=np.int64)
        self.GridVol = abs(np.linalg.det(self.Latvecs)) / float(np.prod(self.Ngrid))
        self.GridN_Atom, self.GridListAtom, self.CellListAtom = calc_atoms_grid(
            self.Latvecs, natom, cpy, self.Gxyz, self.Atoms_Cut1, self.Ngrid, self.Grid_Origin)
        # one rank: the whole flattened pair list (src/UCell.jl:76-132)
        self.pairs = [(a + 1, natn[a][r], ncn[a][r]) for a in range(natom) for r in range(fnan[a] + 1)]
        self.MPI_atom = np.array([p[0] for p in self.pairs], dtype=np.int64)
        self.MPI_natn = np.array([p[1] for p in self.pairs], dtype=np.int64)
        self.MPI_ncn = np.array([p[2] for p in self.pairs], dtype=np.int64)
        self.Nloop = len(self.pairs)
        off = [0]
        for a, b, _ in self.pairs:
            off.append(off[-1] + int(self.Total_NumOrbs[a - 1] * self.Total_NumOrbs[b - 1]))
        self.block_offset = np.array(off[:-1], dtype=np.int64)
        self.Total_Hsize = off[-1]
        # pair_subset: overlap lists of these pair indices only (others empty),
        # for bounded samples of large cells
        sel = list(range(self.Nloop)) if pair_subset is None else sorted(set(pair_subset))
        plist = [self.pairs[p] for p in sel]
        if overlap == "vectorised":
            s1, s2 = calc_atom_overlap_grid(cpy, plist, self.GridListAtom, self.CellListAtom, self.atv_ijk, self.ratv)
        else:
            s1, s2 = calc_atom_overlap_grid_literal(cpy, plist, self.GridN_Atom, self.GridListAtom,
                                                    self.CellListAtom, self.atv_ijk, self.ratv)
        empty = np.zeros(0, dtype=np.int64)
        g1 = [empty] * self.Nloop
        g2 = [empty] * self.Nloop
        for k, p in enumerate(sel):
            g1[p], g2[p] = s1[k], s2[k]
        self.MPI_GListTAtoms1, self.MPI_GListTAtoms2 = g1, g2
        self.MPI_NumOLG = np.array([x.size for x in g1], dtype=np.int64)

    @property
    def NN(self):
        return int(np.prod(self.Ngrid))

    def recvecs(self):
        """2*pi*inv(Latvecs') (src/Mixing/DFT_Mixing.jl:91)."""
        return 2 * PI * np.linalg.inv(self.Latvecs.T)


# --------------------------------------------------------------------------
# PAO data


class PAO:
    """The fields of ``struct PAO`` the grid path reads (src/Atoms/Read_PAO.jl:1-18)."""

    def __init__(self, max_l, num_basis, rv, rwf, xv=None, atomic_den=None, cutoff=None):
        self.Spe_MaxL_Basis = int(max_l)
        self.Spe_Num_Basis = [int(x) for x in num_basis]
        self.Spe_PAO_RV = np.asarray(rv, dtype=np.float64)
        self.Spe_Num_Mesh_PAO = self.Spe_PAO_RV.size
        # rwf[l][p] -> array over the mesh
        self.Spe_PAO_RWF = [[np.asarray(rwf[l][p], dtype=np.float64) for p in range(self.Spe_Num_Basis[l])]
                            for l in range(self.Spe_MaxL_Basis + 1)]
        self.Spe_PAO_XV = None if xv is None else np.asarray(xv, dtype=np.float64)
        self.Spe_Atomic_Den = None if atomic_den is None else np.asarray(atomic_den, dtype=np.float64)
        self.Spe_Atom_Cut1 = cutoff
        self.Spe_Total_NumOrbs = sum(self.Spe_Num_Basis[l] * (2 * l + 1) for l in range(self.Spe_MaxL_Basis + 1))


def get_ialpha_index(orb):
    """Basis string -> (MaxL, Num_Basis) (src/Atoms/Read_PAO.jl:49-76)."""
    if len(orb) % 2 == 1:
        raise ValueError("please check input data")
    maxl = len(orb) // 2 - 1
    letters = "spdf"
    num = []
    for L in range(maxl + 1):
        if L > 3:
            raise ValueError("please check basis")
        pair = orb[2 * L:2 * L + 2]
        if pair[0] != letters[L]:
            raise ValueError("please check basis")
        num.append(int(pair[1:]))
    return maxl, num


def normalize_atomic_den(core_charge, xv, den_raw):
    """Renormalised, edge-extrapolated atomic density (src/Atoms/Read_PAO.jl:290-303).

    Returns the (N+4)-long array laid out as ``Spe_Atomic_Den`` (entry i+1 holds
    mesh point i in 1-based terms)."""
    n = xv.size
    den = np.zeros(n + 4)
    den[1:n + 1] = den_raw
    s = 0.0
    dx = xv[1] - xv[0]
    for i in range(n):
        s += den[i + 1] * math.exp(3 * xv[i])
    s *= 4 * PI * dx
    den[1:n + 1] = den[1:n + 1] * core_charge / s
    den[0] = 2 * den[1] - den[2]
    den[n + 1] = 2 * den[n] - den[n - 1]
    return den


def pcc_array(pcc_raw):
    """``Spe_Atomic_PCC`` layout (src/Atoms/Read_VPS.jl:245-268)."""
    n = pcc_raw.size
    out = np.zeros(n + 4)
    out[1:n + 1] = pcc_raw
    out[0] = 2 * out[1] - out[2]
    out[n + 1] = 2 * out[n] - out[n - 1]
    return out


# --------------------------------------------------------------------------
# angular functions


def xyz_to_spherical(x, y, z):
    """src/utils/xyz_to_spherical.jl:1-31 (vectorised)."""
    x, y, z = np.broadcast_arrays(np.asarray(x, float), np.asarray(y, float), np.asarray(z, float))
    min_r = 1e-14
    dum = x * x + y * y
    r = np.sqrt(dum + z * z)
    r1 = np.sqrt(dum)
    with np.errstate(divide="ignore", invalid="ignore"):
        d1 = np.where(r < np.abs(z), np.sign(z), z / r)
        theta = np.arccos(np.clip(d1, -1.0, 1.0))
        d2 = np.where(r1 < np.abs(y), np.sign(y), y / r1)
        ph = np.where(x >= 0.0, np.arcsin(np.clip(d2, -1, 1)), PI - np.arcsin(np.clip(d2, -1, 1)))
    ph = np.where(min_r <= r1, ph, 0.0)
    theta = np.where(min_r <= r, theta, 0.5 * PI)
    ph = np.where(min_r <= r, ph, 0.0)
    return r, theta, ph


def _trig(theta, ph):
    return np.sin(theta), np.cos(theta), np.sin(ph), np.cos(ph)


# orbital order within l (src/Matrix/Set_Orbitals_Grid.jl:242-268)
M_ORDER = {0: [0], 1: [1, -1, 0], 2: [0, 2, -2, 1, -1], 3: [0, 1, -1, 2, -2, 3, -3]}


def ylm_real(l, m, theta, ph):
    """src/utils/Ylm_real.jl:1-53."""
    siQ, coQ, siP, coP = _trig(theta, ph)
    if l == 0:
        return np.full(np.shape(theta), 0.5 * math.sqrt(1 / PI))
    if l == 1:
        c = math.sqrt(3 / 4 / PI)
        return {-1: c * siQ * siP, 0: c * coQ, 1: c * siQ * coP}[m]
    if l == 2:
        if m == -2:
            return 0.5 * math.sqrt(15 / PI) * siQ * siQ * siP * coP
        if m == -1:
            return 0.5 * math.sqrt(15 / PI) * siQ * coQ * siP
        if m == 0:
            return 0.25 * math.sqrt(5 / PI) * (3 * coQ * coQ - 1)
        if m == 1:
            return 0.5 * math.sqrt(15 / PI) * siQ * coQ * coP
        return 0.25 * math.sqrt(15 / PI) * siQ * siQ * (1 - 2 * siP * siP)
    if l == 3:
        if m == -3:
            return 0.25 * math.sqrt(35 / 2 / PI) * siQ * siQ * siQ * (3 * siP - 4 * siP * siP * siP)
        if m == -2:
            return 0.5 * math.sqrt(105 / PI) * siQ * siQ * coQ * siP * coP
        if m == -1:
            return 0.25 * math.sqrt(21 / 2 / PI) * siQ * (5 * coQ * coQ - 1) * siP
        if m == 0:
            return 0.25 * math.sqrt(7 / PI) * (5 * coQ * coQ * coQ - 3 * coQ)
        if m == 1:
            return 0.25 * math.sqrt(21 / 2 / PI) * siQ * (5 * coQ * coQ - 1) * coP
        if m == 2:
            return 0.25 * math.sqrt(105 / PI) * siQ * siQ * coQ * (coP * coP - siP * siP)
        return 0.25 * math.sqrt(35 / 2 / PI) * siQ * siQ * siQ * (4 * coP * coP * coP - 3 * coP)
    raise ValueError("please check Ylm_real.jl")


def dylm_dtheta(l, m, theta, ph):
    """src/utils/Ylm_real.jl:56-108."""
    siQ, coQ, siP, coP = _trig(theta, ph)
    z = np.zeros(np.shape(theta))
    if l == 0:
        return z
    if l == 1:
        c = math.sqrt(3 / 4 / PI)
        return {-1: c * coQ * siP, 0: -c * siQ, 1: c * coQ * coP}[m]
    if l == 2:
        s = math.sqrt(15 / PI)
        if m == -2:
            return s * siQ * coQ * siP * coP
        if m == -1:
            return 0.5 * s * (1 - 2 * siQ * siQ) * siP
        if m == 0:
            return -1.5 * math.sqrt(5 / PI) * siQ * coQ
        if m == 1:
            return 0.5 * s * (1 - 2 * siQ * siQ) * coP
        return 0.5 * s * siQ * coQ * (1 - 2 * siP * siP)
    if l == 3:
        if m == -3:
            return 0.75 * math.sqrt(35 / 2 / PI) * siQ * siQ * coQ * siP * (3 - 4 * siP * siP)
        if m == -2:
            return 0.5 * math.sqrt(105 / PI) * coP * siP * siQ * (2 * coQ * coQ - siQ * siQ)
        if m == -1:
            return 0.25 * math.sqrt(21 / 2 / PI) * siP * coQ * (15 * coQ * coQ - 11)
        if m == 0:
            return 0.25 * math.sqrt(7 / PI) * siQ * (-15 * coQ * coQ + 3)
        if m == 1:
            return 0.25 * math.sqrt(21 / 2 / PI) * coP * coQ * (15 * coQ * coQ - 11)
        if m == 2:
            return 0.25 * math.sqrt(105 / PI) * (coP * coP - siP * siP) * siQ * (2 * coQ * coQ - siQ * siQ)
        return 0.75 * math.sqrt(35 / 2 / PI) * coP * coQ * siQ * siQ * (-3 + 4 * coP * coP)
    raise ValueError("please check Ylm_real.jl")


def dylm_dphi(l, m, theta, ph):
    """src/utils/Ylm_real.jl:111-162."""
    siQ, coQ, siP, coP = _trig(theta, ph)
    z = np.zeros(np.shape(theta))
    if l == 0:
        return z
    if l == 1:
        c = math.sqrt(3 / 4 / PI)
        return {-1: c * coP, 0: z, 1: -c * siP}[m]
    if l == 2:
        s = math.sqrt(15 / PI)
        if m == -2:
            return 0.5 * s * siQ * (1 - 2 * siP * siP)
        if m == -1:
            return 0.5 * s * coQ * coP
        if m == 0:
            return z
        if m == 1:
            return -0.5 * s * coQ * siP
        return -s * siQ * siP * coP
    if l == 3:
        if m == -3:
            return 0.75 * math.sqrt(35 / 2 / PI) * coP * siQ * siQ * (1 - 4 * siP * siP)
        if m == -2:
            return 0.5 * math.sqrt(105 / PI) * coQ * siQ * (coP * coP - siP * siP)
        if m == -1:
            return 0.25 * math.sqrt(21 / 2 / PI) * coP * (5 * coQ * coQ - 1)
        if m == 0:
            return z
        if m == 1:
            return 0.25 * math.sqrt(21 / 2 / PI) * siP * (-5 * coQ * coQ + 1)
        if m == 2:
            return -math.sqrt(105 / PI) * coP * coQ * siP * siQ
        return 0.75 * math.sqrt(35 / 2 / PI) * siP * siQ * siQ * (1 - 4 * coP * coP)
    raise ValueError("please check Ylm_real.jl")


# --------------------------------------------------------------------------
# radial interpolation


def _spline_setup(rv, R):
    """Binary search + spline geometry (src/Matrix/Set_Orbitals_Grid.jl:187-214).

    Returns 0-based m with RV[m-1] < R <= RV[m], clamped to [2, N-2]."""
    n = rv.size
    m = np.searchsorted(rv, R, side="left")
    m = np.clip(m, 2, n - 2)
    h1 = rv[m - 1] - rv[m - 2]
    h2 = rv[m] - rv[m - 1]
    h3 = rv[m + 1] - rv[m]
    return m, h1, h2, h3


def _hermite(f1, f2, f3, f4, h1, h2, h3, x1, x2):
    y1 = x1 / h2
    y2 = x2 / h2
    y12 = y1 * y1
    y22 = y2 * y2
    dum = h1 + h2
    dum1 = h1 / h2 / dum
    dum2 = h2 / h1 / dum
    dum = h2 + h3
    dum3 = h2 / h3 / dum
    dum4 = h3 / h2 / dum
    dum = f3 - f2
    g1 = dum * dum1 + (f2 - f1) * dum2
    g2 = (f4 - f3) * dum3 + dum * dum4
    A = 3 * f2 + h2 * g1
    B = 2 * f2 + h2 * g1
    C = 3 * f3 - h2 * g2
    D = 2 * f3 - h2 * g2
    E = A + B * y2
    F = C - D * y1
    f = y22 * E + y12 * F
    df = (2 * y2 * E + y22 * B + 2.0 * y1 * F - y12 * D) / h2
    return f, df


def _extrapolation_coeffs(rv, rwf, l):
    """Small-R polynomial (src/Matrix/Set_Orbitals_Grid.jl:124-185)."""
    m = 4  # 1-based m = 5
    rm = rv[m]
    h1 = rv[m - 1] - rv[m - 2]
    h2 = rv[m] - rv[m - 1]
    h3 = rv[m + 1] - rv[m]
    f1, f2, f3, f4 = rwf[m - 2], rwf[m - 1], rwf[m], rwf[m + 1]
    y1 = (rm - rv[m - 1]) / h2
    y2 = (rm - rv[m]) / h2
    y12, y22 = y1 * y1, y2 * y2
    dum = h1 + h2
    dum1 = h1 / h2 / dum
    dum2 = h2 / h1 / dum
    dum = h2 + h3
    dum3 = h2 / h3 / dum
    dum4 = h3 / h2 / dum
    dum = f3 - f2
    g1 = dum * dum1 + (f2 - f1) * dum2
    g2 = (f4 - f3) * dum3 + dum * dum4
    A = 3 * f2 + h2 * g1
    B = 2 * f2 + h2 * g1
    C = 3 * f3 - h2 * g2
    D = 2 * f3 - h2 * g2
    E = A + B * y2
    F = C - D * y1
    f = y22 * E + y12 * F
    df = (2 * y2 / h2) * E + y22 * B / h2 + (2 * y1 / h2) * F - y12 * D / h2
    if l == 0:
        a, b, c = 0.0, 0.5 * df / rm, 0.0
        d = f - b * (rm * rm)
    elif l == 1:
        a = (rm * df - f) / (2 * (rm * rm * rm))
        b = 0.0
        c = df - 3 * a * (rm * rm)
        d = 0.0
    else:
        b = (3 * f - rm * df) / (rm * rm)
        a = (f - b * (rm * rm)) / (rm * rm * rm)
        c = d = 0.0
    return a, b, c, d


def _extrapolation_coeffs_d(rv, rwf, l):
    """Same as above with the derivative expression of
    src/Matrix/Set_dOrbitals_Grid.jl:160-186."""
    m = 4
    rm = rv[m]
    h1 = rv[m - 1] - rv[m - 2]
    h2 = rv[m] - rv[m - 1]
    h3 = rv[m + 1] - rv[m]
    f1, f2, f3, f4 = rwf[m - 2], rwf[m - 1], rwf[m], rwf[m + 1]
    f, df = _hermite(f1, f2, f3, f4, h1, h2, h3, rm - rv[m - 1], rm - rv[m])
    if l == 0:
        a, b, c = 0.0, 0.5 * df / rm, 0.0
        d = f - b * (rm * rm)
    elif l == 1:
        a = (rm * df - f) / (2 * (rm * rm * rm))
        b = 0.0
        c = df - 3 * a * (rm * rm)
        d = 0.0
    else:
        b = (3 * f - rm * df) / (rm * rm)
        a = (f - b * (rm * rm)) / (rm * rm * rm)
        c = d = 0.0
    return a, b, c, d


def _point_geometry(ucell, atom):
    """Atom-relative coordinates of atom's sphere points
    (src/Matrix/Set_Orbitals_Grid.jl:96-110)."""
    N1, N2, N3 = ucell.Ngrid
    gL = _glatvecs(ucell.Latvecs, ucell.Ngrid)
    gnc = ucell.GridListAtom[atom]
    grc = ucell.CellListAtom[atom]
    n1 = gnc // (N2 * N3)
    n2 = (gnc - n1 * N2 * N3) // N3
    n3 = gnc - n1 * N2 * N3 - n2 * N3
    o = ucell.Grid_Origin
    G = ucell.Gxyz[atom]
    out = []
    for d in range(3):
        c = n1 * gL[0, d] + n2 * gL[1, d] + n3 * gL[2, d] + o[d]
        out.append(c + ucell.atv[grc, d] - G[d])
    return out


def set_orbitals_grid(paos, ucell, atoms=None):
    """phi per atom, [NumOrbs, GridN] (src/Matrix/Set_Orbitals_Grid.jl:26-277).
    ``atoms`` restricts the tabulation to those 0-based atoms (others None)."""
    res = []
    for atom in range(ucell.Natom):
        if atoms is not None and atom not in atoms:
            res.append(None)
            continue
        pao = paos[ucell.atom2spe[atom] - 1]
        rv = pao.Spe_PAO_RV
        n = rv.size
        x, y, z = _point_geometry(ucell, atom)
        R, theta, ph = xyz_to_spherical(x, y, z)
        outside = rv[-1] < R
        inner = R < rv[0]
        m, h1, h2, h3 = _spline_setup(rv, R)
        rows = []
        for l in range(pao.Spe_MaxL_Basis + 1):
            for p in range(pao.Spe_Num_Basis[l]):
                w = pao.Spe_PAO_RWF[l][p]
                f1, f2, f3, f4 = w[m - 2], w[m - 1], w[m], w[m + 1]
                f4 = np.where(m == n - 2, f1, f4)  # :226-229
                f, _ = _hermite(f1, f2, f3, f4, h1, h2, h3, R - rv[m - 1], R - rv[m])
                a, b, c, d = _extrapolation_coeffs(rv, w, l)
                fe = a * (R * R * R) + b * (R * R) + c * R + d
                rf = np.where(outside, 0.0, np.where(inner, fe, f))
                for mm in M_ORDER[l]:
                    af = ylm_real(l, mm, theta, ph)
                    rows.append(np.where(outside, 0.0, rf * af))
        res.append(np.array(rows) if rows else np.zeros((0, R.size)))
    return res


def set_dorbitals_grid(paos, ucell, atoms=None):
    """Gradient tables [3][atom] -> [NumOrbs, GridN]
    (src/Matrix/Set_dOrbitals_Grid.jl:23-362).  ``atoms`` restricts the
    tabulation to those 0-based atoms (others None)."""
    rmin = 1.0e-13
    out = [[], [], []]
    for atom in range(ucell.Natom):
        if atoms is not None and atom not in atoms:
            for k in range(3):
                out[k].append(None)
            continue
        pao = paos[ucell.atom2spe[atom] - 1]
        rv = pao.Spe_PAO_RV
        x, y, z = _point_geometry(ucell, atom)
        R, theta, ph = xyz_to_spherical(x, y, z)
        small = R < rmin
        if np.any(small):
            x = np.where(small, x + rmin, x)
            y = np.where(small, y + rmin, y)
            z = np.where(small, z + rmin, z)
            R, theta, ph = xyz_to_spherical(x, y, z)
        outside = rv[-1] < R
        inner = R < rv[0]
        m, h1, h2, h3 = _spline_setup(rv, R)
        siQ, coQ, siP, coP = _trig(theta, ph)
        dRx, dRy, dRz = siQ * coP, siQ * siP, coQ
        big = R > rmin
        with np.errstate(divide="ignore", invalid="ignore"):
            dQx = np.where(big, coQ * coP / R, 0.0)
            dQy = np.where(big, coQ * siP / R, 0.0)
            dQz = np.where(big, -siQ / R, 0.0)
            dPx = np.where(big, -siP / R, 0.0)
            dPy = np.where(big, coP / R, 0.0)
        dPz = 0.0
        rows = [[], [], []]
        for l in range(pao.Spe_MaxL_Basis + 1):
            for p in range(pao.Spe_Num_Basis[l]):
                w = pao.Spe_PAO_RWF[l][p]
                f, df = _hermite(w[m - 2], w[m - 1], w[m], w[m + 1], h1, h2, h3, R - rv[m - 1], R - rv[m])
                a, b, c, d = _extrapolation_coeffs_d(rv, w, l)
                fe = a * (R * R * R) + b * (R * R) + c * R + d
                dfe = 3 * a * (R * R) + 2 * b * R + c
                rf = np.where(outside, 0.0, np.where(inner, fe, f))
                drf = np.where(outside, 0.0, np.where(inner, dfe, df))
                for mm in M_ORDER[l]:
                    af = ylm_real(l, mm, theta, ph)
                    aq = dylm_dtheta(l, mm, theta, ph)
                    ap = dylm_dphi(l, mm, theta, ph)
                    # AF/dAFQ/dAFP are not refreshed for points beyond RV[end]
                    # (po == 1, :255); RF and dRF are zero there, so the products are 0
                    dchidr = drf * af
                    dchidt = rf * aq
                    dchidp = rf * ap
                    gx = -dRx * dchidr - dQx * dchidt - dPx * dchidp
                    gy = -dRy * dchidr - dQy * dchidt - dPy * dchidp
                    gz = -dRz * dchidr - dQz * dchidt - dPz * dchidp
                    rows[0].append(np.where(outside, 0.0, gx))
                    rows[1].append(np.where(outside, 0.0, gy))
                    rows[2].append(np.where(outside, 0.0, gz))
        for k in range(3):
            out[k].append(np.array(rows[k]))
    return out


# --------------------------------------------------------------------------
# density and grid matrix elements


def set_density_grid(spinpol, ucell, orbs, dm):
    """Density on the grid (src/Matrix/Set_Density_Grid.jl:60-304).

    ``dm`` is a list of Nspin flat arrays in the pair-block layout; returns a
    list of Nspin grids of length NN (per-spin density for "off")."""
    nspin = {"off": 1, "on": 2, "nc": 4}[spinpol]
    NN = ucell.NN
    rho = [np.zeros(NN) for _ in range(nspin)]
    for loop, (atom, jatom, _) in enumerate(ucell.pairs):
        a, b = atom - 1, jatom - 1
        no0, no1 = int(ucell.Total_NumOrbs[a]), int(ucell.Total_NumOrbs[b])
        off = int(ucell.block_offset[loop])
        g1 = ucell.MPI_GListTAtoms1[loop]
        g2 = ucell.MPI_GListTAtoms2[loop]
        if g1.size == 0:
            continue
        local = np.zeros((ucell.GridN_Atom[a], nspin))
        for s in range(nspin):
            D = dm[s][off:off + no0 * no1].reshape(no0, no1).T  # [jst, ist]
            for bs in range(0, g1.size, DENSITY_BLOCK):
                i1 = g1[bs:bs + DENSITY_BLOCK]
                i2 = g2[bs:bs + DENSITY_BLOCK]
                P = D.T @ orbs[b][:, i2]                     # :290
                val = np.einsum("op,op->p", orbs[a][:, i1], P)  # :293-297
                np.add.at(local[:, s], i1, val)
        for s in range(nspin):
            np.add.at(rho[s], ucell.GridListAtom[a], local[:, s])
    return rho


def calc_matrix_elements(ucell, orbs, vpot, nchannels):
    """Grid matrix elements, flat pair-block layout, scaled by GridVol
    (src/Hamiltonian.jl:235-429)."""
    H = [np.zeros(ucell.Total_Hsize) for _ in range(nchannels)]
    for loop, (atom, jatom, _) in enumerate(ucell.pairs):
        a, b = atom - 1, jatom - 1
        no0, no1 = int(ucell.Total_NumOrbs[a]), int(ucell.Total_NumOrbs[b])
        off = int(ucell.block_offset[loop])
        g1 = ucell.MPI_GListTAtoms1[loop]
        g2 = ucell.MPI_GListTAtoms2[loop]
        if g1.size == 0:
            continue
        for bs in range(0, g1.size, DENSITY_BLOCK):
            i1 = g1[bs:bs + DENSITY_BLOCK]
            i2 = g2[bs:bs + DENSITY_BLOCK]
            ob1 = orbs[a][:, i1]
            ob2 = orbs[b][:, i2]
            for ch in range(nchannels):
                v = vpot[ch][ucell.GridListAtom[a][i1]]
                W = ob1 * v[None, :]
                prod = ob2 @ W.T                       # [jst, ist] (:420)
                H[ch][off:off + no0 * no1] += prod.T.reshape(-1)  # column-major [jst, ist]
    for ch in range(nchannels):
        H[ch] *= ucell.GridVol
    return H


# --------------------------------------------------------------------------
# Poisson, xc, potentials, energies


def calc_force3(spinpol, ucell, orbs, dorbs, vpot, dm):
    """Grid force term: Force3_nospin / Force3_spin / Force3_nc
    (src/Force.jl:405-566) with _Calc_Force3_Blocked_Kernel!
    (src/Force.jl:3344-3394).  For every ordered pair (atom, jatom, R) of the
    neighbour list, in list order, the sum over the overlap points of
    V(p) * (d phi_atom(p) . D_pair phi_jatom(p)); the channel sums are
    weighted (off: 4; on: 2, 2; nc: 2, 2, 4, -4) and scaled by GridVol.

    ``vpot`` holds the channels' potentials as the reference passes them (off:
    [Vpot]; on: [Vpot_up, Vpot_down]; nc: [dVH + Vxc1, dVH + Vxc2, Vxc3,
    Vxc4]); ``dm`` the flat pair-block density matrices per channel;
    ``dorbs`` the gradient tables of set_dorbitals_grid.  Returns [Natom, 3]."""
    coef = {"off": [4.0], "on": [2.0, 2.0], "nc": [2.0, 2.0, 4.0, -4.0]}[spinpol]
    F = np.zeros((ucell.Natom, 3))
    for loop, (atom, jatom, _) in enumerate(ucell.pairs):
        a, b = atom - 1, jatom - 1
        no0, no1 = int(ucell.Total_NumOrbs[a]), int(ucell.Total_NumOrbs[b])
        off = int(ucell.block_offset[loop])
        g1 = ucell.MPI_GListTAtoms1[loop]
        g2 = ucell.MPI_GListTAtoms2[loop]
        if g1.size == 0:
            continue
        gidx = ucell.GridListAtom[a][g1]
        for c, w in enumerate(coef):
            D = dm[c][off:off + no0 * no1].reshape(no0, no1)   # [ist, jst]
            P = D @ orbs[b][:, g2]                              # :3371-3373
            V = vpot[c][gidx]
            for k in range(3):
                local = np.einsum("op,op->p", dorbs[k][a][:, g1], P)  # :3380-3386
                F[a, k] += w * float(np.sum(V * local)) * ucell.GridVol
    return F


def set_density_xyz(spinpol, ngrid, density, adensity):
    """src/Poisson.jl:10-26."""
    if spinpol == "off":
        d = 2 * density[0] - 2 * adensity
    else:
        d = density[0] + density[1] - 2 * adensity
    return d.reshape(ngrid).astype(np.complex128)


def solve_poisson_xyz(ngrid, recvecs, density_xyz):
    """Inner FFT solve (src/Poisson.jl:29-108): pencil passes k, j, i; 4*pi/G^2;
    G=0 set to zero; inverse passes i, j, k (normalised by 1/N); real part."""
    N1, N2, N3 = ngrid
    a = np.array(density_xyz, dtype=np.complex128).reshape(N1, N2, N3)
    a = np.fft.fft(a, axis=2)
    a = np.fft.fft(a, axis=1)
    a = np.fft.fft(a, axis=0)
    i = np.arange(N1)
    j = np.arange(N2)
    k = np.arange(N3)
    s1 = np.where(i < N1 // 2, i, i - N1)[:, None, None]
    s2 = np.where(j < N2 // 2, j, j - N2)[None, :, None]
    s3 = np.where(k < N3 // 2, k, k - N3)[None, None, :]
    Rv = np.asarray(recvecs, dtype=np.float64)
    Gx = s1 * Rv[0, 0] + s2 * Rv[1, 0] + s3 * Rv[2, 0]
    Gy = s1 * Rv[0, 1] + s2 * Rv[1, 1] + s3 * Rv[2, 1]
    Gz = s1 * Rv[0, 2] + s2 * Rv[1, 2] + s3 * Rv[2, 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        a = 4 * PI * a / (Gx * Gx + Gy * Gy + Gz * Gz)
    a[0, 0, 0] = 0.0
    a = np.fft.ifft(a, axis=0)
    a = np.fft.ifft(a, axis=1)
    a = np.fft.ifft(a, axis=2)
    return np.real(a).reshape(-1).copy()


def solve_poisson(spinpol, ucell, density, adensity):
    """src/Poisson.jl:1-7."""
    return solve_poisson_xyz(ucell.Ngrid, ucell.recvecs(), set_density_xyz(spinpol, ucell.Ngrid, density, adensity))


def lda_ca(den, switch):
    """Ceperley-Alder / Perdew-Zunger LDA (src/XC/LDA_CA.jl:4-41), vectorised."""
    den = np.asarray(den, dtype=np.float64)
    out = np.zeros_like(den)
    ok = den > 1e-15
    d = den[ok]
    coe = 0.6203504908994
    rs = coe * d ** (-1 / 3)
    tmp0 = 0.458165293632163 / rs
    Ex = -tmp0
    dEx = tmp0 / rs
    big = rs >= 1.0
    Ec = np.empty_like(rs)
    dEc = np.empty_like(rs)
    t = np.sqrt(rs[big])
    dum = 1.0 + 1.0529 * t + 0.3334 * rs[big]
    t1 = 0.1423 / dum
    Ec[big] = -t1
    dEc[big] = t1 / dum * (0.52645 / t + 0.3334)
    lr = np.log(rs[~big])
    r = rs[~big]
    Ec[~big] = -0.0480 + 0.0311 * lr + r * (0.0020 * lr - 0.0116)
    dEc[~big] = 0.0311 / r + 0.0020 * lr - 0.0096
    if switch == 0:
        v = Ex + Ec
    elif switch == 1:
        v = Ex + Ec - 1 / 3 * rs * (dEx + dEc)
    elif switch == 2:
        v = 1 / 3 * rs * (dEx + dEc)
    elif switch == 3:
        v = -1 / 3 / coe / coe / coe * rs * rs * rs * rs * (dEx + dEc)
    else:
        raise ValueError("please check switch")
    out[ok] = v
    return out


def lsda_ca(up, down, switch):
    """src/XC/LSDA_CA.jl:1-138, vectorised; returns (first, second)."""
    up = np.asarray(up, dtype=np.float64)
    down = np.asarray(down, dtype=np.float64)
    tden = up + down
    min_den = 1e-15
    o1 = np.zeros_like(tden)
    o2 = np.zeros_like(tden)
    ok = tden > min_den
    u, d, t = up[ok], down[ok], tden[ok]
    zeta = (u - d) / t
    zeta = np.where(zeta > 1.0, 1 - min_den, zeta)
    zeta = np.where(zeta < -1.0, -1 + min_den, zeta)
    coe = 0.6203504908994
    rs = np.where(t < min_den, 62035.04908994, coe * t ** (-1 / 3))
    tmp0 = 0.458165293632163 / rs
    ExP = -tmp0
    dExP = tmp0 / rs
    ExF = 1.25992104989487 * ExP
    dExF = 1.25992104989487 * dExP
    big = rs >= 1.0
    EcP = np.empty_like(rs)
    dEcP = np.empty_like(rs)
    EcF = np.empty_like(rs)
    dEcF = np.empty_like(rs)
    sq = np.sqrt(rs[big])
    r = rs[big]
    dum = 1.0 + 1.0529 * sq + 0.3334 * r
    t1 = 0.1423 / dum
    EcP[big] = -t1
    dEcP[big] = t1 / dum * (0.52645 / sq + 0.3334)
    dum = 1.0 + 1.3981 * sq + 0.2611 * r
    t1 = 0.0843 / dum
    EcF[big] = -t1
    dEcF[big] = t1 / dum * (0.69905 / sq + 0.2611)
    lr = np.log(rs[~big])
    r = rs[~big]
    EcP[~big] = -0.0480 + 0.0311 * lr + r * (0.0020 * lr - 0.0116)
    dEcP[~big] = 0.0311 / r + 0.0020 * lr - 0.0096
    EcF[~big] = -0.0269 + 0.01555 * lr + r * (0.0007 * lr - 0.0048)
    dEcF[~big] = 0.01555 / r + 0.0007 * lr - 0.0041
    if switch == 0:
        z0 = (1 + zeta) ** (4 / 3)
        z1 = (1 - zeta) ** (4 / 3)
        fz = 1.92366105093154 * (z0 + z1 - 2.0)
        exc = ExP + EcP + (ExF + EcF - ExP - EcP) * fz
        a, b = exc, exc
    elif switch in (1, 2):
        z0 = (1 + zeta) ** (1 / 3)
        z1 = (1 - zeta) ** (1 / 3)
        z02 = z0 * z0
        z04 = z02 * z02
        z12 = z1 * z1
        z14 = z12 * z12
        fz = 1.92366105093154 * (z04 + z14 - 2.0)
        dfz = 2.56488140124205 * (z0 - z1)
        tmp0 = ExF + EcF - ExP - EcP
        exc = ExP + EcP + tmp0 * fz
        dexc = dExP + dEcP + (dExF + dEcF - dExP - dEcP) * fz
        if switch == 1:
            vxc = exc - 1 / 3 * rs * dexc
            a = vxc + tmp0 * (1 - zeta) * dfz
            b = vxc + tmp0 * (-1 - zeta) * dfz
        else:
            tmp1 = 1 / 3 * rs * dexc
            tmp2 = tmp0 * dfz
            a = tmp1 - tmp2 * (1 - zeta)
            b = tmp1 - tmp2 * (-1 - zeta)
    else:
        raise ValueError("please check switch")
    o1[ok] = a
    o2[ok] = b
    return o1, o2


def diagonalize_nc_density(density):
    """diagonalize_nc_density! (src/Matrix/Set_Density_Grid.jl:243-261) with
    EulerAngle_Spin (src/utils/EulerAngle_Spin.jl:1-6): (Re11, Re22, Re12,
    Im12) -> (Nup, Ndown, theta, phi), returned as new arrays."""
    re11, re22, re12, im12 = (np.asarray(d, dtype=np.float64) for d in density[:4])
    r, theta, ph = xyz_to_spherical(2 * re12, -2 * im12, re11 - re22)
    return [0.5 * (re11 + re22 + r), 0.5 * (re11 + re22 - r), theta, ph]


def set_xc_grid(xc_type, spinpol, pcc, density):
    """V_xc on the grid (src/XC/XC_Func.jl:111-145)."""
    if xc_type == "LDA":
        return [lda_ca(2 * (density[0] + pcc), 1)]
    u, d = lsda_ca(density[0] + pcc, density[1] + pcc, 1)
    if spinpol == "nc":
        tmp0 = 0.5 * (u + d)
        tmp1 = 0.5 * (u - d)
        th, ph = density[2], density[3]
        return [tmp0 + tmp1 * np.cos(th), tmp0 - tmp1 * np.cos(th),
                tmp1 * np.sin(th) * np.cos(ph), -tmp1 * np.sin(th) * np.sin(ph)]
    return [u, d]


def set_vpot_grid(spinpol, dvhart, vxc, vna=None):
    """src/Matrix/Set_Vpot_Grid.jl:1-19, plus an optional neutral-atom field
    added to the diagonal channels."""
    extra = 0.0 if vna is None else vna
    if spinpol == "off":
        return [dvhart + vxc[0] + extra]
    if spinpol == "on":
        return [dvhart + vxc[0] + extra, dvhart + vxc[1] + extra]
    return [dvhart + vxc[0] + extra, dvhart + vxc[1] + extra, vxc[2].copy(), vxc[3].copy()]


def calc_eh1(spinpol, gridvol, adensity, density, dvhart):
    """src/Energy.jl:655-666."""
    if spinpol == "off":
        e = np.dot(2 * (density[0] - adensity), dvhart)
    else:
        e = np.dot(density[0] + density[1] - 2 * adensity, dvhart)
    return e * gridvol * 0.5


def calc_exc1(spinpol, xc_type, gridvol, adensity, pcc, density, ngrid=None, latvecs=None):
    """src/Energy.jl:669-700 with Calc_Vxc_Grid switch 0 (src/XC/XC_Func.jl:164-189).

    Returns the two-entry EXC vector; for "off" the caller sets EXC[2]=EXC[1]
    (src/Energy.jl:646-648).  GGA_PBE needs the grid (``ngrid``, ``latvecs``)
    for its gradient stencil."""
    if xc_type == "LDA":
        eps = [lda_ca(2 * (density[0] + pcc), 0)]
    elif xc_type == "GGA_PBE":
        dc = calc_diff_coef(glatvecs_of(latvecs, ngrid))
        eps = calc_vxc_grid_gga(spinpol, ngrid, pcc, density, dc)
    else:
        u, d = lsda_ca(density[0] + pcc, density[1] + pcc, 0)
        eps = [u, d]
    spinmax = 1 if spinpol == "off" else 2
    exc = [0.0, 0.0]
    temp = adensity + pcc
    for s in range(spinmax):
        acc = np.sum((density[s] + pcc) * eps[s] - temp * lda_ca(2 * temp, 0))
        exc[s] = acc * gridvol
    return exc


# --------------------------------------------------------------------------
# GGA-PBE: pointwise kernel (src/XC/XC_PBE.jl) and the 27-point gradient
# stencil (src/XC/GGA_PBE.jl), vectorised over grid points.

DEN_MIN = 1.0e-14  # src/LCPAODFT.jl:71 (also the local den_min of src/XC/XC_PBE.jl)


def pw92c(d1, d2):
    """XC_PW92C (src/XC/XC_PBE.jl:1-126): returns (Ec, Vc1, Vc2, d1, d2), the
    densities as the function leaves them (it resets both to den_min/2 where
    their sum is <= den_min)."""
    d1 = np.array(d1, dtype=np.float64, copy=True)
    d2 = np.array(d2, dtype=np.float64, copy=True)
    dtot = d1 + d2
    low = dtot <= DEN_MIN
    d1[low] = 0.5e-14
    d2[low] = 0.5e-14
    dtot = np.where(low, DEN_MIN, dtot)
    rs = np.where(low, 6203.504908994, 0.6203504908994 * dtot ** (-1 / 3))
    tmp0 = 1.0 / dtot
    zeta = tmp0 * (d1 - d2)
    zeta = np.where(zeta > 0.99, 0.99, zeta)
    zeta = np.where(zeta < -1.0, -0.99, zeta)
    drsdd = -(1 / 3) * rs * tmp0
    dzdd1 = tmp0 * (1 - zeta)
    dzdd2 = tmp0 * (-1 - zeta)
    srs = np.sqrt(rs)

    def g(A, a1, b1, b2, b3, b4):
        b = b1 * srs + rs * (b2 + b3 * srs + b4 * rs)
        dbdrs = b1 * 0.5 / srs + b2 + b3 * 1.5 * srs + b4 * 2 * rs
        c = 1 + 1 / (2 * A * b)
        dcdrs = -(c - 1) * dbdrs / b
        dum = np.log(c)
        dum1 = 1 + a1 * rs
        return -2 * A * dum1 * dum, -2 * A * (a1 * dum + dum1 * dcdrs / c)

    G0, dG0 = g(0.0310910, 0.2137000, 7.5957000, 3.5876000, 1.6382000, 0.4929400)
    G1, dG1 = g(0.0155450, 0.2054800, 14.1189000, 6.1977000, 3.3662000, 0.6251700)
    G2, dG2 = g(0.0168870, 0.1112500, 10.3570000, 3.6231000, 0.8802600, 0.4967100)
    c = 1.92366105093154
    fpp0 = 1.70992093416137
    tmp1 = np.cbrt(1 + zeta)
    tmp2 = np.cbrt(1 - zeta)
    f = (tmp1 ** 4 + tmp2 ** 4 - 2) * c
    dfdz = (4 / 3) * (tmp1 - tmp2) * c
    z3 = zeta ** 3
    z4 = z3 * zeta
    Ec = G0 - G2 * f / fpp0 * (1 - z4) + (G1 - G0) * f * z4
    dEcdrs = dG0 - dG2 * f / fpp0 * (1 - z4) + (dG1 - dG0) * f * z4
    dEcdz = -G2 / fpp0 * (dfdz * (1 - z4) - f * 4 * z3) + (G1 - G0) * (dfdz * z4 + f * 4 * z3)
    dum = dEcdrs * drsdd
    Vc1 = Ec + dtot * (dum + dEcdz * dzdd1)
    Vc2 = Ec + dtot * (dum + dEcdz * dzdd2)
    return Ec, Vc1, Vc2, d1, d2


def xc_ex_unpolarised(ds):
    """XC_EX with NSP = 1 (src/XC/XC_PBE.jl:132-184): returns (EX1, VX1)."""
    D = np.maximum(ds, DEN_MIN)
    RS = 0.6203504908994 * D ** (-0.333333333333333)
    VXP = -0.610887057710857 / RS
    return 0.75 * VXP, VXP


def xc_pbe(ed, gdens):
    """XC_PBE! (src/XC/XC_PBE.jl:187-476), vectorised.

    ``ed`` = (rho_up, rho_down) arrays, ``gdens`` = the six gradient arrays
    (d/dx, d/dy, d/dz of up, then of down).  Returns (Exc[2], DEXDD[2],
    DECDD[2], DEXDGD[6], DECDGD[6]) as lists of arrays, in the reference's
    output order."""
    THD = 1 / 3
    beta = 0.06672455060314922
    gamma = (1 - math.log(2)) / (PI * PI)
    kappa = 0.8040
    mu = beta * PI * PI / 3
    GD_min = 1e-14
    d1 = np.maximum(0.5 * DEN_MIN, np.asarray(ed[0], dtype=np.float64))
    d2 = np.maximum(0.5 * DEN_MIN, np.asarray(ed[1], dtype=np.float64))
    dt = d1 + d2
    g = [np.asarray(x, dtype=np.float64) for x in gdens]
    GDT = [g[0] + g[3], g[1] + g[4], g[2] + g[5]]
    GDM = [np.sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]),
           np.sqrt(g[3] * g[3] + g[4] * g[4] + g[5] * g[5])]
    GDMT = np.maximum(GD_min, np.sqrt(GDT[0] * GDT[0] + GDT[1] * GDT[1] + GDT[2] * GDT[2]))

    # local correlation; XC_PW92C writes the densities back (:15-24)
    Ec_unif, Vc1_unif, Vc2_unif, d1, d2 = pw92c(d1, d2)

    # correlation energy (:241-267)
    kF = np.cbrt(3 * PI * PI * dt)
    ks = np.sqrt(4 * kF / PI)
    zeta = (d1 - d2) / dt
    zeta = np.where(zeta > 0.99, 0.99, zeta)
    zeta = np.where(zeta < -1.0, -0.99, zeta)
    phi = 0.5 * ((1 + zeta) ** (2 / 3) + (1 - zeta) ** (2 / 3))
    t = GDMT / (2 * phi * ks * dt)
    f1 = Ec_unif / (gamma * phi ** 3)
    f2 = np.exp(-f1)
    A = beta / gamma / (f2 - 1)
    f3 = t * t + A * t ** 4
    f4 = beta / gamma * f3 / (1 + A * f3)
    H = gamma * phi ** 3 * np.log(1 + f4)
    Fc = Ec_unif + H

    # correlation derivatives (:273-342)
    DKFDD = 1 / 3 * kF / dt
    DKSDD = 0.5 * ks * DKFDD / kF
    DPDZ = 0.5 * 2 / 3 * (1 / np.cbrt(1 + zeta) - 1 / np.cbrt(1 - zeta))
    DFCDD = []
    for Vc_unif, DZDD in ((Vc1_unif, 1 / dt - zeta / dt), (Vc2_unif, -1 / dt - zeta / dt)):
        DECUDD = (Vc_unif - Ec_unif) / dt
        DPDD = DPDZ * DZDD
        DTDD = (-t) * (DPDD / phi + DKSDD / ks + 1 / dt)
        DF1DD = f1 * (DECUDD / Ec_unif - 3 * DPDD / phi)
        DF2DD = -f2 * DF1DD
        DADD = -A * DF2DD / (f2 - 1)
        DF3DD = (2 * t + 4 * A * t ** 3) * DTDD + DADD * t ** 4
        DF4DD = f4 * (DF3DD / f3 - (DADD * f3 + A * DF3DD) / (1 + A * f3))
        DHDD = 3 * H * DPDD / phi + gamma * phi ** 3 * DF4DD / (1 + f4)
        DFCDD.append(Vc_unif + H + dt * DHDD)
    DFCDGD = []
    for x in range(3):
        DTDGD = (t / GDMT) * GDT[x] / GDMT
        DF3DGD = DTDGD * (2.0 * t + 4.0 * A * t * t * t)
        DF4DGD = f4 * DF3DGD * (1.0 / f3 - A / (1.0 + A * f3))
        DHDGD = gamma * phi * phi * phi * DF4DGD / (1.0 + f4)
        DFCDGD.append(dt * DHDGD)

    # exchange, spin by spin (:348-451)
    Fx = np.zeros_like(dt)
    DFXDD = []
    DFXDGD = []
    for ds_, gdm, gs in ((d1, GDM[0], g[0:3]), (d2, GDM[1], g[3:6])):
        DS = np.maximum(DEN_MIN, 2 * ds_)
        GDMS = np.maximum(GD_min, 2 * gdm)
        KFS = np.cbrt(3 * PI * PI * DS)
        s = GDMS / (2 * KFS * DS)
        f1x = 1 + mu * s * s / kappa
        f = 1 + kappa - kappa / f1x
        Ex_unif, Vx1_unif = xc_ex_unpolarised(DS)
        Fx = Fx + DS * Ex_unif * f
        DKFDDx = THD * KFS / DS
        DSDD = s * (-(DKFDDx / KFS) - 1 / DS)
        DF1DD = 2 * (f1x - 1) * DSDD / s
        DFDD = kappa * DF1DD / (f1x * f1x)
        DFXDD.append(Vx1_unif * f + DS * Ex_unif * DFDD)
        for x in range(3):
            GDS = 2 * gs[x]
            DSDGD = (s / GDMS) * GDS / GDMS
            DF1DGD = 2 * mu * s * DSDGD / kappa
            DFDGD = kappa * DF1DGD / (f1x * f1x)
            DFXDGD.append(DS * Ex_unif * DFDGD)
    Fx = 0.5 * Fx / dt
    return [Fx, Fc], DFXDD, DFCDD, DFXDGD, DFCDGD + DFCDGD


def calc_diff_coef(glatvecs):
    """Calc_Diff_Coef (src/XC/GGA_PBE.jl:1-39): the x, y, z first-derivative
    weights of the tri-quadratic fit through the 27 neighbours
    (i1, j1, k1) in -1..1 (k1 fastest), as a (3, 27) array."""
    gL = np.asarray(glatvecs, dtype=np.float64)
    M = np.zeros((27, 27))
    p = 0
    for i1 in (-1, 0, 1):
        for j1 in (-1, 0, 1):
            for k1 in (-1, 0, 1):
                x, y, z = i1 * gL[0] + j1 * gL[1] + k1 * gL[2]
                q = 0
                for i2 in range(3):
                    for j2 in range(3):
                        for k2 in range(3):
                            M[p, q] = x ** i2 * y ** j2 * z ** k2
                            q += 1
                p += 1
    inv = np.linalg.inv(M)
    # rows 10, 4, 2 (1-based) of the inverse: the x, y, z monomial coefficients
    return np.stack([inv[9], inv[3], inv[1]])


def _stencil(ngrid, f, coef):
    """sum_p coef[p] * f[neighbour p] with periodic wrap (transform2primcell,
    src/XC/GGA_PBE.jl:42-50); the neighbour order is i1, j1, k1 in -1..1, k1
    fastest, as in src/XC/GGA_PBE.jl:77-90."""
    a = np.asarray(f, dtype=np.float64).reshape(ngrid)
    out = np.zeros(a.shape)
    p = 0
    for i1 in (-1, 0, 1):
        for j1 in (-1, 0, 1):
            for k1 in (-1, 0, 1):
                out += coef[p] * np.roll(a, shift=(-i1, -j1, -k1), axis=(0, 1, 2))
                p += 1
    return out.ravel()


def _gga_spin_densities(spinpol, density):
    """(ED up, ED down) before the PCC is added and the centre-point test value
    (2 rho for "off", rho_up + rho_down otherwise)."""
    if spinpol == "off":
        r = np.asarray(density[0], dtype=np.float64)
        return r, r, 2 * r
    r0 = np.asarray(density[0], dtype=np.float64)
    r1 = np.asarray(density[1], dtype=np.float64)
    return r0, r1, r0 + r1


def set_ddensity_grid(spinpol, ngrid, density, pcc, diff_coef):
    """Set_dDensity_Grid! (src/XC/GGA_PBE.jl:53-159): per spin, the three
    gradient components of rho_s + pcc, zero where the centre test value is
    <= den_min.  Returns [spin][xyz] arrays (one spin for "off")."""
    r0, r1, test = _gga_spin_densities(spinpol, density)
    pc = np.zeros_like(r0) if pcc is None else np.asarray(pcc, dtype=np.float64)
    on = DEN_MIN < test
    out = []
    for r in ((r0,) if spinpol == "off" else (r0, r1)):
        out.append([np.where(on, _stencil(ngrid, r + pc, diff_coef[a]), 0.0) for a in range(3)])
    return out


def _gga_gdens(spinpol, dden):
    up = dden[0]
    dn = dden[0] if spinpol == "off" else dden[1]
    return [up[0], up[1], up[2], dn[0], dn[1], dn[2]]


def set_xc_grid_gga(spinpol, ngrid, pcc, density, diff_coef):
    """Set_XC_Grid!(xc_func::XC_GGA_PBE, ...) (src/XC/XC_Func.jl:148-160):
    Set_dDensity_Grid! then Set_Vxc_GGA_PBE! (src/XC/GGA_PBE.jl:162-193,
    274-462).  Returns (Vxc_Grid, dDensity_Grid, dEXC_dGD)."""
    r0, r1, test = _gga_spin_densities(spinpol, density)
    pc = np.zeros_like(r0) if pcc is None else np.asarray(pcc, dtype=np.float64)
    dden = set_ddensity_grid(spinpol, ngrid, density, pcc, diff_coef)
    # pointwise pass: 2 ED >= den_min ("off", :301) / ED1 + ED2 > den_min (:393)
    act = test >= DEN_MIN if spinpol == "off" else test > DEN_MIN
    _, dexdd, decdd, dexdgd, decdgd = xc_pbe((r0 + pc, r1 + pc), _gga_gdens(spinpol, dden))
    ns = 1 if spinpol == "off" else 2
    vxc = [np.where(act, dexdd[s] + decdd[s], 0.0) for s in range(ns)]
    dexc = [[np.where(act, dexdgd[3 * s + a] + decdgd[3 * s + a], 0.0) for a in range(3)] for s in range(ns)]
    # divergence pass: centre test value > den_min (:328, :426)
    on = test > DEN_MIN
    for s in range(ns):
        tmp = _stencil(ngrid, dexc[s][0], diff_coef[0])
        tmp = tmp + _stencil(ngrid, dexc[s][1], diff_coef[1])
        tmp = tmp + _stencil(ngrid, dexc[s][2], diff_coef[2])
        vxc[s] = np.where(on, vxc[s] - tmp, vxc[s])
    if spinpol == "nc":
        tmp0 = 0.5 * (vxc[0] + vxc[1])
        tmp1 = 0.5 * (vxc[0] - vxc[1])
        th, ph = np.asarray(density[2]), np.asarray(density[3])
        vxc = [tmp0 + np.cos(th) * tmp1, tmp0 - np.cos(th) * tmp1,
               -tmp1 * np.sin(th) * np.cos(ph), -tmp1 * np.sin(th) * np.sin(ph)]
    return vxc, dden, dexc


def calc_vxc_grid_gga(spinpol, ngrid, pcc, density, diff_coef):
    """_Calc_Vxc_Grid_GGA! (src/XC/XC_Func.jl:193-215 with the five-argument
    _Set_Vxc_GGA_PBE_* of src/XC/GGA_PBE.jl:196-271): the PBE energy per
    particle Exc[1] + Exc[2] where the centre test value is > den_min, else 0;
    the same array for both spins."""
    r0, r1, test = _gga_spin_densities(spinpol, density)
    pc = np.zeros_like(r0) if pcc is None else np.asarray(pcc, dtype=np.float64)
    dden = set_ddensity_grid(spinpol, ngrid, density, pcc, diff_coef)
    exc = xc_pbe((r0 + pc, r1 + pc), _gga_gdens(spinpol, dden))[0]
    e = np.where(test > DEN_MIN, exc[0] + exc[1], 0.0)
    return [e] if spinpol == "off" else [e, e.copy()]


def glatvecs_of(latvecs, ngrid):
    """gtv of Calc_EXC1 (src/Energy.jl:676-679): Latvecs rows / Ngrid."""
    return _glatvecs(latvecs, ngrid)


def grid_energy(spinpol, ucell, dm, H, eh1, exc):
    """Job energy scalar: f_s * sum_s <D_s, H^grid_s> + E_H1 + E_xc1 (the sum over
    all channels, four for "nc"), with f_s = 2
    for "off" (as src/Energy.jl:475-505 doubles the kinetic term) and
    E_xc1 = EXC[1] + EXC[2] with EXC[2] = EXC[1] for "off" (src/Energy.jl:646-648)."""
    fs = 2.0 if spinpol == "off" else 1.0
    nspin = {"off": 1, "on": 2, "nc": 4}[spinpol]
    e_dh = sum(float(np.dot(dm[s], H[s])) for s in range(nspin))
    e_xc = exc[0] + (exc[0] if spinpol == "off" else exc[1])
    return fs * e_dh + eh1 + e_xc


# --------------------------------------------------------------------------
# atomic and partial-core densities (config-1 inputs)


def kumof(n, x, xv, rv, yv):
    """Uniform-x cubic interpolation (src/utils/KumoF.jl:1-60), vectorised.
    ``yv`` uses the (N+4)-long layout of Spe_Atomic_Den / Spe_Atomic_PCC."""
    x = np.asarray(x, dtype=np.float64)
    out = np.empty_like(x)
    low = x < xv[0]
    if np.any(low):
        r = np.exp(x[low])
        m = 5
        rm = rv[m - 1]
        h1 = rv[m - 2] - rv[m - 3]
        h2 = rv[m - 1] - rv[m - 2]
        h3 = rv[m] - rv[m - 1]
        f1, f2, f3, f4 = yv[m - 3], yv[m - 2], yv[m - 1], yv[m]
        g1 = ((f3 - f2) * h1 / h2 + (f2 - f1) * h2 / h1) / (h1 + h2)
        g2 = ((f4 - f3) * h2 / h3 + (f3 - f2) * h3 / h2) / (h2 + h3)
        x1 = rm - rv[m - 2]
        x2 = rm - rv[m - 1]
        y1 = x1 / h2
        y2 = x2 / h2
        y12, y22 = y1 * y1, y2 * y2
        A = 2 * f2 + h2 * g1
        B = 2 * f3 - h2 * g2
        C = 3 * f2 + h2 * g1
        D = 3 * f3 - h2 * g2
        E = C + A * y2
        F = D - B * y1
        f = y22 * E + y12 * F
        df = (2 * y2 / h2) * E + y22 * A / h2 + (2 * y1 / h2) * F - y12 * B / h2
        a = 0.5 * df / rm
        b = f - a * rm * rm
        out[low] = a * r * r + b
    hi = ~low
    if np.any(hi):
        xmin, xmax = xv[0], xv[-1]
        xx = np.minimum(x[hi], xmax)
        xx = np.maximum(xx, xmin)
        tmp = (n - 1) * (xx - xmin) / (xmax - xmin)
        i = np.floor(tmp).astype(np.int64)
        dt = tmp - i
        i = i + 1  # 1-based i; yv[i+1] is 0-based yv[i]
        d0 = yv[i] - yv[i - 1]
        d1 = yv[i + 1] - yv[i]
        d2 = yv[i + 2] - yv[i + 1]
        a = d0 - 2 * d1 + d2
        b = -2 * d0 + 3 * d1 - d2
        c = d0 + d1
        out[hi] = yv[i] + 0.5 * (((a * dt + b) * dt + c) * dt)
    return out


def set_adenpcc_grid(spinpol, init_nspin, init_angle, pao_tables, vps_tables, ucell):
    """src/Matrix/Set_AdenPCC_Grid.jl:1-142.

    ``pao_tables[spe] = (xv, rv, atomic_den)``, ``vps_tables[spe] = (xv, rv, pcc)``
    with the (N+4)-long density layouts."""
    nspin = {"off": 1, "on": 2, "nc": 4}[spinpol]
    NN = ucell.NN
    aden = np.zeros(NN)
    pccd = np.zeros(NN)
    dens = [np.zeros(NN) for _ in range(nspin)]
    for atom in range(ucell.Natom):
        spe = ucell.atom2spe[atom] - 1
        pxv, prv, pden = pao_tables[spe]
        vxv, vrv, vpcc = vps_tables[spe]
        nu, nd = init_nspin[atom]
        nele = nu + nd
        ou = nu / nele if nele > 1e-15 else 0.0
        od = nd / nele if nele > 1e-15 else 0.0
        th, ph = init_angle[atom][0], init_angle[atom][1]
        dx, dy, dz = _point_geometry(ucell, atom)
        with np.errstate(divide="ignore"):
            x = 0.5 * np.log(dx * dx + dy * dy + dz * dz)
        ad = kumof(pxv.size, x, pxv, prv, pden)
        pc = kumof(vxv.size, x, vxv, vrv, vpcc)
        g = ucell.GridListAtom[atom]
        np.add.at(aden, g, 0.5 * ad)
        np.add.at(pccd, g, 0.5 * pc)
        if spinpol == "off":
            np.add.at(dens[0], g, 0.5 * ad)
        elif spinpol == "on":
            np.add.at(dens[0], g, ou * ad)
            np.add.at(dens[1], g, od * ad)
        else:
            mag = (ou - od) * ad
            np.add.at(dens[0], g, ad)
            np.add.at(dens[1], g, mag * math.sin(th) * math.cos(ph))
            np.add.at(dens[2], g, mag * math.sin(th) * math.sin(ph))
            np.add.at(dens[3], g, mag * math.cos(th))
    if spinpol == "nc":
        rho, mx, my, mz = dens
        dens = [0.5 * (rho + mz), 0.5 * (rho - mz), 0.5 * mx, -0.5 * my]
    return aden, pccd, dens
