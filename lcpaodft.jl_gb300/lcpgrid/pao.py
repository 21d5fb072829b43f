"""Species data for the grid path: the fields of ``struct PAO`` it reads
(src/Atoms/Read_PAO.jl:1-18) and the partial-core density of ``struct Pspot``
(src/Atoms/Read_VPS.jl:1-19), read from OpenMX-format ``.pao``/``.vps`` files
or built from tables.  Host-side input handling only."""
import math
import os

import numpy as np

ANG_TO_BOHR = 1.8897259886  # src/LCPAODFT.jl:18


def get_ialpha_index(Spe_orbitals):
    """Basis string such as "s2p2d1" -> (Spe_MaxL_Basis, Spe_Num_Basis)
    (src/Atoms/Read_PAO.jl:49-76)."""
    if len(Spe_orbitals) % 2 == 1:
        raise ValueError("please check input data: %r" % Spe_orbitals)
    maxl = len(Spe_orbitals) // 2 - 1
    if maxl > 3:
        raise ValueError("please check basis")
    num = []
    for L in range(maxl + 1):
        pair = Spe_orbitals[2 * L:2 * L + 2]
        if pair[0] != "spdf"[L]:
            raise ValueError("please check basis: %r" % Spe_orbitals)
        num.append(int(pair[1:]))
    return maxl, num


class PAO:
    """Radial tables of one species.

    ``Spe_PAO_RWF[l][p]`` is the radial function R_lp on the mesh ``Spe_PAO_RV``;
    ``Spe_Atomic_Den`` (optional) uses the reference's (N+4)-long layout."""

    def __init__(self, Spe_MaxL_Basis, Spe_Num_Basis, Spe_PAO_RV, Spe_PAO_RWF, Spe_PAO_XV=None,
                 Spe_Atomic_Den=None, Spe_Atom_Cut1=None, Atom_symbol="", Atom_orbital="", Atom_extra=""):
        self.Atom_symbol = Atom_symbol
        self.Atom_orbital = Atom_orbital
        self.Atom_extra = Atom_extra
        self.Spe_MaxL_Basis = int(Spe_MaxL_Basis)
        self.Spe_Num_Basis = [int(x) for x in Spe_Num_Basis]
        self.Spe_PAO_RV = np.ascontiguousarray(Spe_PAO_RV, dtype=np.float64)
        self.Spe_Num_Mesh_PAO = int(self.Spe_PAO_RV.size)
        self.Spe_PAO_RWF = [[np.ascontiguousarray(Spe_PAO_RWF[l][p], dtype=np.float64)
                             for p in range(self.Spe_Num_Basis[l])] for l in range(self.Spe_MaxL_Basis + 1)]
        self.Spe_PAO_XV = None if Spe_PAO_XV is None else np.asarray(Spe_PAO_XV, dtype=np.float64)
        self.Spe_Atomic_Den = None if Spe_Atomic_Den is None else np.asarray(Spe_Atomic_Den, dtype=np.float64)
        self.Spe_Atom_Cut1 = Spe_Atom_Cut1
        self.Spe_Total_NumOrbs = sum(n * (2 * l + 1) for l, n in enumerate(self.Spe_Num_Basis))
        for l in range(self.Spe_MaxL_Basis + 1):
            for p in range(self.Spe_Num_Basis[l]):
                if self.Spe_PAO_RWF[l][p].size != self.Spe_Num_Mesh_PAO:
                    raise ValueError("radial function (%d,%d) does not match the mesh" % (l, p))

    def packed_rwf(self):
        """RWF flattened in (l, p, mesh) order, the layout of lcp_pao.rwf."""
        rows = [self.Spe_PAO_RWF[l][p] for l in range(self.Spe_MaxL_Basis + 1) for p in range(self.Spe_Num_Basis[l])]
        if not rows:
            return np.zeros(0)
        return np.ascontiguousarray(np.concatenate(rows))


def _read_lines(path):
    with open(path) as f:
        return [ln.strip() for ln in f]


def normalize_atomic_den(core_charge, xv, den_raw):
    """Spe_Atomic_Den renormalised to ``core_charge`` electrons and extended at
    both ends (src/Atoms/Read_PAO.jl:290-303)."""
    n = xv.size
    den = np.zeros(n + 4)
    den[1:n + 1] = den_raw
    s = 0.0
    dx = xv[1] - xv[0]
    for i in range(n):
        s += den[i + 1] * math.exp(3 * xv[i])
    s *= 4 * math.pi * dx
    den[1:n + 1] = den[1:n + 1] * core_charge / s
    den[0] = 2 * den[1] - den[2]
    den[n + 1] = 2 * den[n] - den[n - 1]
    return den


def Read_PAO(Spe_Core_Charge, Atom_symbol, Atom_cutoff, Atom_orb, Atom_extra, data_dir):
    """Read ``<data_dir>/<symbol><cutoff><extra>.pao`` (src/Atoms/Read_PAO.jl:114-331)."""
    name = "%s%s%s.pao" % (Atom_symbol, repr(float(Atom_cutoff)), Atom_extra)
    lines = _read_lines(os.path.join(data_dir, name))
    mesh = cutoff = lmax = mul = None
    for ln in lines:
        parts = ln.split()
        if not parts:
            continue
        if "grid.num.output" in ln:
            mesh = int(parts[1])
        elif "radial.cutoff.pao" in ln:
            cutoff = float(parts[1])
        elif "PAO.Lmax" in ln:
            lmax = int(parts[1])
        elif "PAO.Mul" in ln:
            mul = int(parts[1])
    if mesh is None or cutoff is None or lmax is None or mul is None:
        raise ValueError("please check po")
    if abs(cutoff - Atom_cutoff) > 1e-10:
        raise ValueError("Please check Spe_Atom_Cut1")
    i0 = next(i for i, ln in enumerate(lines) if "<valence.charge.density" in ln)
    block = np.array([[float(x) for x in lines[i0 + 1 + k].split()[:3]] for k in range(mesh)])
    if "valence.charge.density>" not in lines[i0 + 1 + mesh]:
        raise ValueError("please check valence_charge_density")
    xv, rv, den = block[:, 0].copy(), block[:, 1].copy(), block[:, 2].copy()
    maxl, nb = get_ialpha_index(Atom_orb)
    if maxl > lmax or any(n > mul for n in nb):
        raise ValueError("basis %s exceeds the PAO file" % Atom_orb)
    rwf = []
    for L in range(maxl + 1):
        tag = "<pseudo.atomic.orbitals.L=%d" % L
        j0 = next(i for i, ln in enumerate(lines) if tag in ln)
        rows = np.array([[float(x) for x in lines[j0 + 1 + k].split()] for k in range(mesh)])
        rwf.append([rows[:, p + 2].copy() for p in range(nb[L])])
    return PAO(maxl, nb, rv, rwf, Spe_PAO_XV=xv, Spe_Atomic_Den=normalize_atomic_den(Spe_Core_Charge, xv, den),
               Spe_Atom_Cut1=cutoff, Atom_symbol=Atom_symbol, Atom_orbital=Atom_orb, Atom_extra=Atom_extra)


class PCC:
    """The partial-core density of one species (src/Atoms/Read_VPS.jl:245-268)."""

    def __init__(self, xv, rv, pcc_raw):
        self.Spe_VPS_XV = np.asarray(xv, dtype=np.float64)
        self.Spe_VPS_RV = np.asarray(rv, dtype=np.float64)
        n = self.Spe_VPS_XV.size
        self.Spe_Num_Mesh_VPS = n
        a = np.zeros(n + 4)
        a[1:n + 1] = pcc_raw
        a[0] = 2 * a[1] - a[2]
        a[n + 1] = 2 * a[n] - a[n - 1]
        self.Spe_Atomic_PCC = a


def Read_VPS_PCC(Atom_symbol, Atom_extra, xc_type, data_dir):
    """PCC section of ``<symbol>_CA19<extra>.vps`` / ``_PBE19`` (src/Atoms/Read_VPS.jl:51-370)."""
    tag = "CA19" if xc_type in ("LDA", "LSDA") else "PBE19"
    lines = _read_lines(os.path.join(data_dir, "%s_%s%s.vps" % (Atom_symbol, tag, Atom_extra)))
    mesh = None
    for ln in lines:
        if "grid.num.output" in ln:
            mesh = int(ln.split()[1])
    i0 = next(i for i, ln in enumerate(lines) if "<Pseudo.Potentials" in ln)
    pp = np.array([[float(x) for x in lines[i0 + 1 + k].split()[:2]] for k in range(mesh)])
    j0 = next(i for i, ln in enumerate(lines) if "<density.PCC" in ln)
    pcc = np.array([float(lines[j0 + 1 + k].split()[2]) for k in range(mesh)])
    return PCC(pp[:, 0], pp[:, 1], pcc)
