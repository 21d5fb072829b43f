"""Seeded synthetic inputs for the grid-step workloads.

* ``si2_primitive``: the plain small case -- Si diamond primitive cell
  (a = 5.43 A, fcc vectors as examples/Si/Si.jl:5-10), Si7.0-s2p2d1 basis,
  grid from Calc_Ngrid(150 Ry) = 24^3.
* ``si64_supercell``: the precision-form cell -- 64-atom cubic Si
  (2x2x2 conventional cells, a = 10.86 A), 13 orbitals per atom with
  synthetic radial functions (sums of 3 Gaussians, exponents 0.2-3 bohr^-2,
  smooth cutoff at 7 bohr) tabulated on a 1000-point log mesh, grid 96^3,
  PSD density matrix with trace 256, smooth V_na with |G| < 3 bohr^-1 and
  amplitude 0.5 Ha.
* ``batch_pool``: the batching form -- independent cells of 2-64 atoms with
  1-3 species (cutoffs from {6, 7, 8, 9} bohr, 4/9/13/18 orbitals),
  cubic lattice constants of 4-12 A, random positions at least 3.5 bohr
  apart, grids from Calc_Ngrid at 150 Ry (24^3-96^3).
* ``mx2_monolayer``: the large spin-polarised cell -- a 12 x 12 MX2
  monolayer (trigonal prismatic, a = 3.19 A, 20 A of vacuum), 144 metal atoms
  of 18 orbitals (rc 8) and 288 chalcogens of 13 (rc 7), grid 216 x 216 x 320,
  LSDA with two PSD spin density matrices.
* ``serving_pool``: the serving form -- random Si-density cells of 2-216
  atoms (log-uniform) with the 64-atom workload's species.

Everything is generated from a seed with numpy; nothing is read from disk.
"""
import math

import numpy as np

from .pao import ANG_TO_BOHR, PAO

DIAMOND_BASIS = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                          [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])


def synthetic_species(seed, max_l=2, num_basis=(2, 2, 1), rc=7.0, nmesh=1000, r_lo=1e-4, r_hi=None):
    """Radial functions R_lp(r) = sum_k c_k exp(-alpha_k r^2) r^l * (1-(r/rc)^2)^3,
    alpha_k ~ U[0.2, 3], c_k ~ N(0,1), normalised (int R^2 r^2 dr = 1), zero beyond rc,
    tabulated on a log mesh x = log r uniform in [log r_lo, log r_hi]."""
    rng = np.random.default_rng(seed)
    r_hi = r_hi if r_hi is not None else rc + 1.0
    x = np.linspace(math.log(r_lo), math.log(r_hi), nmesh)
    rv = np.exp(x)
    fine = np.linspace(0.0, rc, 20001)
    rwf = []
    for l in range(max_l + 1):
        row = []
        for _ in range(num_basis[l]):
            alpha = rng.uniform(0.2, 3.0, size=3)
            c = rng.normal(size=3)

            def f(r):
                cut = np.where(r < rc, (1 - (r / rc) ** 2) ** 3, 0.0)
                return (c[None, :] * np.exp(-alpha[None, :] * (r[:, None] ** 2))).sum(1) * r ** l * cut

            norm = math.sqrt(np.trapezoid(f(fine) ** 2 * fine ** 2, fine))
            row.append(f(rv) / norm)
        rwf.append(row)
    return PAO(max_l, list(num_basis), rv, rwf, Spe_PAO_XV=x, Spe_Atom_Cut1=rc)


def si2_primitive():
    """Lattice (rows), Cartesian positions (bohr) of the Si2 primitive cell."""
    a = 5.43 * ANG_TO_BOHR
    lat = np.array([[0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]]) * a
    frac = np.array([[0, 0, 0], [0.25, 0.25, 0.25]])
    return lat, frac @ lat


def si2_workload(tables, seed=2024):
    """The plain small case: the Si2 primitive cell with the real Si7.0-s2p2d1
    radial tables and the Si_CA19 partial-core density, read from ``tables``
    (a mapping with the arrays pao_Si7.0_{xv,rv,den,rwf} and
    vps_Si_CA19_{xv,rv,pcc}, e.g. the species-table fixture of the tests),
    LDA, grid Calc_Ngrid(150 Ry) = 24^3, Tr D = 4 per atom.  "pcc" holds the
    PCC table object; the atomic densities come from Set_AdenPCC_Grid with two
    electrons per spin per atom."""
    lat, pos = si2_primitive()
    xv, rv = np.asarray(tables["pao_Si7.0_xv"]), np.asarray(tables["pao_Si7.0_rv"])
    rwf = np.asarray(tables["pao_Si7.0_rwf"])
    from .pao import PCC, get_ialpha_index, normalize_atomic_den
    maxl, nb = get_ialpha_index("s2p2d1")
    pao = PAO(maxl, nb, rv, [[rwf[l, p] for p in range(nb[l])] for l in range(maxl + 1)], Spe_PAO_XV=xv,
              Spe_Atomic_Den=normalize_atomic_den(4.0, xv, np.asarray(tables["pao_Si7.0_den"])),
              Spe_Atom_Cut1=7.0, Atom_symbol="Si")
    pcc = PCC(tables["vps_Si_CA19_xv"], tables["vps_Si_CA19_rv"], tables["vps_Si_CA19_pcc"])
    return {
        "name": "si2_fcc_24x24x24", "latvecs": lat, "gxyz": pos, "natom": 2, "atom2spe": [1, 1],
        "cut": [7.0, 7.0], "ngrid": (24, 24, 24), "origin": [0.0, 0.0, 0.0], "numorbs": [13, 13],
        "paos": [pao], "pcc": pcc, "init_nspin": [[2.0, 2.0], [2.0, 2.0]],
        "vna_seed": seed + 1, "dm_seed": seed + 2, "trace": 8.0,
    }


def si_supercell(nrep=2, a_ang=5.43):
    """Cubic diamond Si supercell of nrep^3 conventional cells (8*nrep^3 atoms)."""
    a = a_ang * ANG_TO_BOHR
    lat = np.eye(3) * a * nrep
    pos = []
    for i in range(nrep):
        for j in range(nrep):
            for k in range(nrep):
                for b in DIAMOND_BASIS:
                    pos.append((np.array([i, j, k]) + b) * a)
    return lat, np.array(pos)


def psd_density_matrices_oracle(ucell, seed, nspin=1, trace=256.0, nocc=None):
    """Same matrices for a UCell whose pair list is ``pairs`` of (atom, jatom, cell)."""
    class _View:
        Total_NumOrbs = ucell.Total_NumOrbs
        Total_Hsize = ucell.Total_Hsize
        MPI_atom = np.array([p[0] for p in ucell.pairs])
        MPI_natn = np.array([p[1] for p in ucell.pairs])
        block_offset = ucell.block_offset
    return psd_density_matrices(_View, seed, nspin, trace, nocc)


def psd_density_matrices(ucell, seed, nspin=1, trace=256.0, nocc=None):
    """Flat pair-block density matrices D(i,j,R) = M[i-block, j-block] of a
    seeded PSD M = C C^T (the Gamma-point Bloch sum), scaled to Tr(M) = trace.

    Blocks follow the reference layout: for pair (atom, jatom), entry
    a*NO(jatom) + b holds D between orbital a of atom and b of jatom."""
    rng = np.random.default_rng(seed)
    no = np.asarray(ucell.Total_NumOrbs, dtype=np.int64)
    off = np.concatenate([[0], np.cumsum(no)])
    norb = int(off[-1])
    nocc = nocc or max(1, norb // 4)
    out = []
    for _ in range(nspin):
        C = rng.normal(size=(norb, nocc))
        M = C @ C.T
        M *= trace / np.trace(M)
        dm = np.zeros(ucell.Total_Hsize)
        for p, (a, b) in enumerate(zip(ucell.MPI_atom, ucell.MPI_natn)):
            i, j = a - 1, b - 1
            blk = M[off[i]:off[i + 1], off[j]:off[j + 1]]
            dm[ucell.block_offset[p]:ucell.block_offset[p] + blk.size] = blk.reshape(-1)
        out.append(dm)
    return out


def psd_nc_density_matrices(ucell, seed, trace=256.0, nocc=None):
    """The four "nc" channels (Re11, Re22, Re12, Im12) of a seeded Hermitian
    positive semi-definite 2x2-spinor density matrix M = C C^H (2 Norb x 2 Norb,
    complex C), scaled to Tr(M) = trace, in the flat pair-block layout."""
    rng = np.random.default_rng(seed)
    no = np.asarray(ucell.Total_NumOrbs, dtype=np.int64)
    off = np.concatenate([[0], np.cumsum(no)])
    norb = int(off[-1])
    nocc = nocc or max(1, norb // 4)
    C = rng.normal(size=(2 * norb, nocc)) + 1j * rng.normal(size=(2 * norb, nocc))
    M = C @ C.conj().T
    M *= trace / np.trace(M).real
    mats = [M[:norb, :norb].real, M[norb:, norb:].real, M[:norb, norb:].real, M[:norb, norb:].imag]
    out = []
    for m in mats:
        dm = np.zeros(ucell.Total_Hsize)
        for p, (a, b) in enumerate(zip(ucell.MPI_atom, ucell.MPI_natn)):
            i, j = a - 1, b - 1
            blk = m[off[i]:off[i + 1], off[j]:off[j + 1]]
            dm[ucell.block_offset[p]:ucell.block_offset[p] + blk.size] = blk.reshape(-1)
        out.append(dm)
    return out


def smooth_vna(ngrid, latvecs, seed, gmax=3.0, amplitude=0.5):
    """Real field from Fourier modes with |G| < gmax, random phases,
    scaled to max |V| = amplitude (Ha), C-order flat."""
    rng = np.random.default_rng(seed)
    N1, N2, N3 = ngrid
    rec = 2 * np.pi * np.linalg.inv(np.asarray(latvecs, float).T)

    def sf(n):
        i = np.arange(n)
        return np.where(i < n // 2, i, i - n)

    s1, s2, s3 = np.meshgrid(sf(N1), sf(N2), sf(N3), indexing="ij")
    G = s1[..., None] * rec[0] + s2[..., None] * rec[1] + s3[..., None] * rec[2]
    mask = np.linalg.norm(G, axis=-1) < gmax
    coef = np.zeros((N1, N2, N3), dtype=np.complex128)
    n = int(mask.sum())
    coef[mask] = rng.normal(size=n) * np.exp(2j * np.pi * rng.uniform(size=n))
    coef[0, 0, 0] = 0.0
    v = np.real(np.fft.ifftn(coef))
    v *= amplitude / np.max(np.abs(v))
    return np.ascontiguousarray(v.reshape(-1))


def si64_workload(seed=1234, ngrid=(96, 96, 96), nrep=2):
    """The 64-atom precision-form workload (nrep = 2; nrep = 1 is its 8-atom
    cell); returns a dict of host inputs.  Tr D = 4 per atom (Si's valence
    electrons): 256 for the 64-atom cell."""
    lat, pos = si_supercell(nrep)
    natom = pos.shape[0]
    pao = synthetic_species(seed)
    return {
        "name": "si%d_cubic_%dx%dx%d" % (natom, *ngrid),
        "latvecs": lat, "gxyz": pos, "natom": natom, "atom2spe": [1] * natom,
        "cut": [7.0] * natom, "ngrid": tuple(ngrid), "origin": [0.0, 0.0, 0.0],
        "numorbs": [pao.Spe_Total_NumOrbs] * natom, "paos": [pao],
        "vna_seed": seed + 1, "dm_seed": seed + 2, "trace": 4.0 * natom,
    }


SI_DENSITY = 64 / (10.86 * ANG_TO_BOHR) ** 3  # atoms per bohr^3 of diamond Si
GRID_SPACING = 10.86 * ANG_TO_BOHR / 96       # bohr, as the 64-atom 96^3 cell (0.2138)


def random_si_cell(natom, seed, min_sep=3.5):
    """Cubic cell at the density of diamond Si with `natom` atoms at seeded
    random positions, pairwise (periodic) distances >= min_sep bohr (sequential
    rejection sampling); grid at the 64-atom cell's spacing, each dimension a
    multiple of 8 (>= 24)."""
    rng = np.random.default_rng(seed)
    side = (natom / SI_DENSITY) ** (1.0 / 3.0)
    lat = np.eye(3) * side
    for _attempt in range(100):
        pos = []
        for _ in range(natom):
            for _try in range(10000):
                x = rng.uniform(0, side, size=3)
                ok = True
                for y in pos:
                    d = x - y
                    d -= side * np.round(d / side)
                    if d @ d < min_sep * min_sep:
                        ok = False
                        break
                if ok:
                    pos.append(x)
                    break
            else:
                break
        if len(pos) == natom:
            break
    else:
        raise RuntimeError("could not place %d atoms" % natom)
    n = max(24, int(math.ceil(side / GRID_SPACING / 8.0)) * 8)
    return lat, np.array(pos), (n, n, n)


def serving_pool(nstruct=24, seed=777, nmin=2, nmax=216):
    """Structures of the serving form: sizes log-uniform in [nmin, nmax] atoms,
    random Si-density cells with the synthetic 13-orbital species of the
    64-atom workload (rc 7), a PSD D (4 electrons per atom) and a smooth V_na."""
    rng = np.random.default_rng(seed)
    pao = synthetic_species(1234)
    out = []
    for k in range(nstruct):
        natom = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        lat, pos, ngrid = random_si_cell(natom, seed + 1 + k)
        out.append({"name": "rand%d_%d" % (natom, k), "latvecs": lat, "gxyz": pos, "natom": natom,
                    "atom2spe": [1] * natom, "cut": [7.0] * natom, "ngrid": ngrid, "origin": [0.0, 0.0, 0.0],
                    "numorbs": [pao.Spe_Total_NumOrbs] * natom, "paos": [pao],
                    "vna_seed": seed + 1000 + k, "dm_seed": seed + 2000 + k, "trace": 2.0 * natom})
    return out


def calc_ngrid(ecut, latvecs):
    """Calc_Ngrid (src/utils/Calc_Ngrid.jl:1-76): per axis the 2^p 3^q 5^r 7^s
    nearest in log to |det L| sqrt(Ecut) / (pi |a_j x a_k|)."""
    L = np.asarray(latvecs, float)
    temp = abs(np.linalg.det(L)) / math.pi * math.sqrt(ecut)
    out = []
    for d in range(3):
        lgn = math.log(temp / np.linalg.norm(np.cross(L[(d + 1) % 3], L[(d + 2) % 3])))
        best, bk = 1e10, 1
        l2, l3, l5, l7 = (math.log(x) for x in (2, 3, 5, 7))
        for p in range(int(math.ceil(lgn / l2)) + 1):
            for q in range(int(math.ceil((lgn - p * l2) / l3)) + 1):
                for r in range(int(math.ceil((lgn - p * l2 - q * l3) / l5)) + 1):
                    for t in range(int(math.ceil((lgn - p * l2 - q * l3 - r * l5) / l7)) + 1):
                        lg = p * l2 + q * l3 + r * l5 + t * l7
                        if abs(lg - lgn) < best:
                            best, bk = abs(lg - lgn), 2 ** p * 3 ** q * 5 ** r * 7 ** t
        out.append(bk)
    return tuple(out)


BATCH_CUTOFFS = (6.0, 7.0, 8.0, 9.0)
BATCH_BASES = {4: (1, 1, 0), 9: (1, 1, 1), 13: (2, 2, 1), 18: (2, 2, 2)}  # orbitals: (s, p, d) radial functions


def _place(rng, natom, side, min_sep, tries=20000):
    pos = []
    for _ in range(natom):
        for _try in range(tries):
            x = rng.uniform(0, side, size=3)
            if all(((x - y) - side * np.round((x - y) / side)) @ ((x - y) - side * np.round((x - y) / side))
                   >= min_sep * min_sep for y in pos):
                pos.append(x)
                break
        else:
            return None
    return np.array(pos)


def batch_pool(ncells=256, seed=4242, nmin=2, nmax=64, min_sep=3.5, ecut=150.0, amax_ang=12.0):
    """Cells of the batching form.  Per cell: natom ~ U{nmin..nmax}, 1-3
    species each with a cutoff from BATCH_CUTOFFS and a basis from
    BATCH_BASES (synthetic radial functions), atoms assigned species
    uniformly; a cubic lattice constant ~ U[a0, amax_ang] A with a0 = max(4 A, the
    side at which the spheres of radius min_sep/2 fill 20% of the cell),
    random positions at least min_sep bohr apart (the box is redrawn larger
    when placement fails); grid Calc_Ngrid(ecut); a PSD D with trace
    2 * natom and a smooth V_na."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(ncells):
        natom = int(rng.integers(nmin, nmax + 1))
        nspe = int(rng.integers(1, 4))
        species = []
        for s_ in range(nspe):
            rc = float(BATCH_CUTOFFS[rng.integers(len(BATCH_CUTOFFS))])
            no = list(BATCH_BASES)[rng.integers(len(BATCH_BASES))]
            nb = BATCH_BASES[no]
            max_l = 2 if nb[2] else 1
            species.append(synthetic_species(int(rng.integers(1 << 30)), max_l=max_l,
                                             num_basis=nb[:max_l + 1], rc=rc))
        a2s = [int(x) + 1 for x in rng.integers(0, nspe, size=natom)]
        a0 = max(4.0 * ANG_TO_BOHR, (natom * (4.0 / 3.0) * math.pi * (min_sep / 2) ** 3 / 0.2) ** (1.0 / 3.0))
        side = rng.uniform(a0, max(a0, amax_ang * ANG_TO_BOHR))
        cell_rng = np.random.default_rng(int(rng.integers(1 << 30)))
        while True:
            pos = _place(cell_rng, natom, side, min_sep)
            if pos is not None:
                break
            side *= 1.05
        lat = np.eye(3) * side
        ngrid = calc_ngrid(ecut, lat)
        out.append({"name": "cell%d_%datoms_%dspe" % (k, natom, nspe), "latvecs": lat, "gxyz": pos,
                    "natom": natom, "atom2spe": a2s, "cut": [species[s - 1].Spe_Atom_Cut1 for s in a2s],
                    "ngrid": ngrid, "origin": [0.0, 0.0, 0.0],
                    "numorbs": [species[s - 1].Spe_Total_NumOrbs for s in a2s], "paos": species,
                    "vna_seed": seed + 1000 + k, "dm_seed": seed + 2000 + k, "trace": 2.0 * natom})
    return out


def mx2_monolayer(seed=555, nrep=12, a_ang=3.19, vacuum_ang=20.0, xx_ang=3.13, ngrid=(216, 216, 320)):
    """The 12 x 12 MX2 monolayer: hexagonal cell a1 = a (1, 0, 0), a2 = a (1/2,
    sqrt(3)/2, 0) repeated nrep x nrep, c = vacuum + the X-X layer thickness;
    metal at in-plane fraction (0, 0) of each primitive cell, chalcogens at
    (1/3, 2/3) at +-xx/2 about the metal plane (trigonal prismatic).  Species:
    metal s2p2d2 (18 orbitals, rc 8), chalcogen s2p2d1 (13 orbitals, rc 7),
    synthetic radial functions.  Two PSD spin density matrices of trace
    3 * natom each (up and down)."""
    a = a_ang * ANG_TO_BOHR
    c = (vacuum_ang + xx_ang) * ANG_TO_BOHR
    a1 = np.array([a, 0.0, 0.0])
    a2 = np.array([a / 2, a * math.sqrt(3) / 2, 0.0])
    lat = np.array([nrep * a1, nrep * a2, [0.0, 0.0, c]])
    z0 = c / 2
    dz = xx_ang * ANG_TO_BOHR / 2
    pos, spe = [], []
    for i in range(nrep):
        for j in range(nrep):
            o = i * a1 + j * a2
            pos.append(o + [0, 0, z0])
            spe.append(1)
            x = o + a1 / 3.0 + 2.0 * a2 / 3.0  # in-plane fraction (1/3, 2/3)
            pos.append(x + [0, 0, z0 + dz])
            spe.append(2)
            pos.append(x + [0, 0, z0 - dz])
            spe.append(2)
    paos = [synthetic_species(seed, max_l=2, num_basis=(2, 2, 2), rc=8.0),
            synthetic_species(seed + 1, max_l=2, num_basis=(2, 2, 1), rc=7.0)]
    natom = len(pos)
    return {
        "name": "mx2_%dx%d_%dx%dx%d" % (nrep, nrep, *ngrid),
        "latvecs": lat, "gxyz": np.array(pos), "natom": natom, "atom2spe": spe,
        "cut": [8.0 if t == 1 else 7.0 for t in spe], "ngrid": tuple(ngrid), "origin": [0.0, 0.0, 0.0],
        "numorbs": [18 if t == 1 else 13 for t in spe], "paos": paos, "spinpol": "on",
        "vna_seed": seed + 2, "dm_seed": seed + 3, "trace": 3.0 * natom,
    }
