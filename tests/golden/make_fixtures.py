"""Generate the golden fixtures used by the parity tests.

This script is run once, in a checkout that has the reference project
(LCPAODFT.jl) available, and its outputs are committed next to it:

* ``golden_vectors.json`` -- the numeric expectations written inline in the
  reference's own unit tests (``test/test_UCell.jl``, ``test_Set_Orbs_Grid.jl``,
  ``test_Poisson.jl``, ``test_LDA_CA.jl``, ``test_LSDA_CA.jl``, ``test_XC_PBE.jl``,
  ``test_Set_XC_Grid.jl``, ``test_Set_AdenPCC_Grid.jl``, ``test_Calc_Ngrid.jl``,
  ``test_Read_PAO.jl``).  The Julia test files are read as text; the array
  literals after ``≈`` / ``==`` are parsed as JSON.  Nothing is executed.
* ``species_tables.npz`` -- the radial tables of the OpenMX-format data files
  the fixtures use (``DFT_DATA19/PAO/Si7.0.pao``, ``Fe6.0H.pao`` and the
  ``Si_CA19``/``Si_PBE19``/``Fe_CA19H``/``Fe_PBE19H`` ``.vps`` files), reduced to
  the arrays the grid path reads: the log mesh (XV, RV), the raw valence
  density, the first three radial multiplicities per L, and the raw PCC density.

Usage::

    python tests/golden/make_fixtures.py REFERENCE_ROOT
    LCP_REFERENCE_ROOT=... python tests/golden/make_fixtures.py

REFERENCE_ROOT is a checkout of LCPAODFT.jl (its test/ and DFT_DATA19/
folders are read as text).  The GPU tests never run this script: they read
only the committed outputs.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
KEEP_MUL = 3  # radial multiplicities kept per L (s2p2d1 / s2p2d2 need 2)


def _arrays_after(line, op):
    """Return the JSON value of the array literal that follows ``op`` in ``line``."""
    idx = line.index(op) + len(op)
    text = line[idx:].strip()
    text = re.sub(r"Int32|Float64", "", text)
    return json.loads(text)


def _test_lines(path):
    with open(path) as f:
        for raw in f:
            line = raw.strip()
            if line.startswith("@test") or line.startswith("Bref"):
                yield line


def parse_ucell(ref):
    out = {}
    for line in _test_lines(os.path.join(ref, "test/test_UCell.jl")):
        m = re.match(r"@test (\S+) (==|≈) (.*)$", line)
        if not m:
            continue
        lhs, op, rhs = m.groups()
        key = lhs.split(".")[-1]
        try:
            out[key] = json.loads(rhs)
        except json.JSONDecodeError:
            pass
    return out


def parse_orbs(ref):
    out = {}
    for line in _test_lines(os.path.join(ref, "test/test_Set_Orbs_Grid.jl")):
        m = re.match(r"@test Orbs_Grid\[(\d+)\]\[(\d+)\] ≈ (.*)$", line)
        if m:
            out["%s_%s" % (m.group(1), m.group(2))] = json.loads(m.group(3))
    return out


def parse_poisson(ref):
    path = os.path.join(ref, "test/test_Poisson.jl")
    with open(path) as f:
        text = f.read()
    inp = json.loads(re.search(r"ADensity_Grid = (\[.*?\])\n", text).group(1))
    outv = json.loads(re.search(r"@test dVHart_Grid ≈ (\[.*?\])\n", text).group(1))
    return {"density_xyz": inp, "dVHart_Grid": outv}


def parse_lda(ref):
    path = os.path.join(ref, "test/test_LDA_CA.jl")
    res = {}
    switch = None
    with open(path) as f:
        for line in f:
            line = line.strip()
            m = re.match(r"@\. B = LDA_CA\(A, (\d)\)", line)
            if m:
                switch = int(m.group(1))
            if line.startswith("Bref"):
                res[str(switch)] = json.loads(line.split("=", 1)[1])
    return {"input": [0.1 * i for i in range(1, 11)], "atol": 1e-15, "switch": res}


def parse_lsda(ref):
    path = os.path.join(ref, "test/test_LSDA_CA.jl")
    res = {}
    switch = None
    with open(path) as f:
        for line in f:
            line = line.strip()
            m = re.match(r"B1\[i\], B2\[i\] = LSDA_CA\(A1\[i\], A2\[i\], (\d)\)", line)
            if m:
                switch = int(m.group(1))
            m = re.match(r"@test (B1|B2) ≈ (.*)$", line)
            if m:
                res.setdefault(str(switch), {})[m.group(1)] = json.loads(m.group(2))
    return {"up": [0.1 * i for i in range(1, 11)],
            "down": [0.1 * i - 0.1 for i in range(1, 11)], "switch": res}


def parse_xc_pbe(ref):
    """Inputs and expected outputs of the pointwise PBE kernel (test/test_XC_PBE.jl)."""
    path = os.path.join(ref, "test/test_XC_PBE.jl")
    res = {}
    with open(path) as f:
        for line in f:
            line = line.strip()
            m = re.match(r"(ED|GDENS) = (\[.*\])$", line)
            if m:
                res[m.group(1)] = json.loads(m.group(2))
            m = re.match(r"@test (Exc|DEXDD|DECDD|DEXDGD|DECDGD) ≈ (.*)$", line)
            if m:
                res[m.group(1)] = json.loads(m.group(2))
    return res


def _testsets(path):
    with open(path) as f:
        text = f.read()
    return re.findall(r'@testset "([^"]+)" begin(.*?)\nend', text, flags=re.S)


def parse_xc_grid(ref):
    out = {}
    for name, body in _testsets(os.path.join(ref, "test/test_Set_XC_Grid.jl")):
        m = re.search(r"@test xc_func\.Vxc_Grid ≈ (.*?)(?:\n|$)", body)
        if m:
            out[name] = json.loads(m.group(1))
    return out


def parse_adenpcc(ref):
    out = {}
    for name, body in _testsets(os.path.join(ref, "test/test_Set_AdenPCC_Grid.jl")):
        rec = {}
        for key in ("ADensity_Grid", "PCCDensity_Grid", "Density_Grid"):
            m = re.search(r"@test %s ≈ (.*?)(?:\n|$)" % key, body)
            if m:
                rec[key] = json.loads(m.group(1))
        out[name] = rec
    return out


def parse_ngrid(ref):
    cases = []
    ang_to_bohr = 1.8897259886  # src/LCPAODFT.jl:18
    for name, body in _testsets(os.path.join(ref, "test/test_Calc_Ngrid.jl")):
        m = re.search(r"(?:Latvecs|Lattice) = \[(.*?)\](\*\"Ang\")?", body, flags=re.S)
        lat = m.group(1)
        rows = [[float(x) for x in r.split()] for r in lat.replace("\n", " ").split(";")]
        if m.group(2):
            rows = [[x * ang_to_bohr for x in r] for r in rows]
        ecut = None
        for line in body.splitlines():
            line = line.strip()
            m = re.match(r"Ecut = ([0-9.]+)", line)
            if m:
                ecut = float(m.group(1))
            m = re.match(r"@test Ngrid == \((\d+),\s*(\d+),\s*(\d+)\)", line)
            if m:
                cases.append({"set": name, "Latvecs": rows, "Ecut": ecut,
                              "Ngrid": [int(m.group(i)) for i in (1, 2, 3)]})
    return cases


def parse_read_pao(ref):
    out = {}
    for name, body in _testsets(os.path.join(ref, "test/test_Read_PAO.jl")):
        rec = {}
        for key in ("Spe_MaxL_Basis", "Spe_Num_Basis", "Spe_Total_NumOrbs",
                    "Spe_Num_Mesh_PAO", "Spe_Atom_Cut1", "Spe_PAO_Lmax", "Spe_PAO_Mul"):
            m = re.search(r"@test pao\.%s == (.*?)(?:\n|$)" % key, body)
            if m:
                rec[key] = json.loads(m.group(1))
        out[name] = rec
    return out


# ---------------------------------------------------------------- data files

def read_pao_file(path):
    """Plain reader of the OpenMX ``.pao`` sections the grid path uses."""
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    scal = {}
    for ln in lines:
        parts = ln.split()
        if not parts:
            continue
        if "grid.num.output" in ln:
            scal["mesh"] = int(parts[1])
        elif "radial.cutoff.pao" in ln:
            scal["cutoff"] = float(parts[1])
        elif "PAO.Lmax" in ln:
            scal["lmax"] = int(parts[1])
        elif "PAO.Mul" in ln:
            scal["mul"] = int(parts[1])
    n = scal["mesh"]
    i0 = next(i for i, ln in enumerate(lines) if "<valence.charge.density" in ln)
    block = np.array([[float(x) for x in lines[i0 + 1 + k].split()[:3]] for k in range(n)])
    rwf = np.zeros((scal["lmax"] + 1, KEEP_MUL, n))
    for L in range(scal["lmax"] + 1):
        tag = "<pseudo.atomic.orbitals.L=%d" % L
        j0 = next(i for i, ln in enumerate(lines) if tag in ln)
        for k in range(n):
            parts = lines[j0 + 1 + k].split()
            for mul in range(min(KEEP_MUL, scal["mul"])):
                rwf[L, mul, k] = float(parts[mul + 2])
    return scal, block[:, 0], block[:, 1], block[:, 2], rwf


def read_vps_file(path):
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    scal = {}
    for ln in lines:
        parts = ln.split()
        if not parts:
            continue
        if "grid.num.output" in ln:
            scal["mesh"] = int(parts[1])
        elif ln.startswith("AtomSpecies"):
            scal["AtomSpecies"] = float(parts[1])
        elif ln.startswith("total.electron"):
            scal["total_electron"] = float(parts[1])
        elif ln.startswith("valence.electron"):
            scal["valence_electron"] = float(parts[1])
        elif "charge.pcc.calc" in ln:
            scal["is_pcc"] = parts[1].lower() == "on"
    n = scal["mesh"]
    i0 = next(i for i, ln in enumerate(lines) if "<Pseudo.Potentials" in ln)
    pp = np.array([[float(x) for x in lines[i0 + 1 + k].split()[:2]] for k in range(n)])
    j0 = next(i for i, ln in enumerate(lines) if "<density.PCC" in ln)
    pcc = np.array([float(lines[j0 + 1 + k].split()[2]) for k in range(n)])
    return scal, pp[:, 0], pp[:, 1], pcc


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LCP_REFERENCE_ROOT")
    if not ref:
        sys.exit("usage: make_fixtures.py REFERENCE_ROOT (or set LCP_REFERENCE_ROOT)")
    gold = {
        "ucell_si_3x3x3": parse_ucell(ref),
        "orbs_si_3x3x3": parse_orbs(ref),
        "poisson_si_3x3x3": parse_poisson(ref),
        "lda_ca": parse_lda(ref),
        "lsda_ca": parse_lsda(ref),
        "xc_pbe": parse_xc_pbe(ref),
        "xc_grid": parse_xc_grid(ref),
        "adenpcc": parse_adenpcc(ref),
        "calc_ngrid": parse_ngrid(ref),
        "read_pao": parse_read_pao(ref),
    }
    with open(os.path.join(HERE, "golden_vectors.json"), "w") as f:
        json.dump(gold, f)

    arrays = {}
    meta = {}
    for tag, fname in (("Si7.0", "PAO/Si7.0.pao"), ("Fe6.0H", "PAO/Fe6.0H.pao")):
        scal, xv, rv, den, rwf = read_pao_file(os.path.join(ref, "DFT_DATA19", fname))
        meta["pao:" + tag] = scal
        arrays["pao_%s_xv" % tag] = xv
        arrays["pao_%s_rv" % tag] = rv
        arrays["pao_%s_den" % tag] = den
        arrays["pao_%s_rwf" % tag] = rwf
    for tag in ("Si_CA19", "Si_PBE19", "Fe_CA19H", "Fe_PBE19H"):
        scal, xv, rv, pcc = read_vps_file(os.path.join(ref, "DFT_DATA19/VPS", tag + ".vps"))
        meta["vps:" + tag] = scal
        arrays["vps_%s_xv" % tag] = xv
        arrays["vps_%s_rv" % tag] = rv
        arrays["vps_%s_pcc" % tag] = pcc
    arrays["meta_json"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "species_tables.npz"), **arrays)
    print("wrote", os.path.join(HERE, "golden_vectors.json"), "and species_tables.npz")


if __name__ == "__main__":
    main()
