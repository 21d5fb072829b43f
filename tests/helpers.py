"""Shared test inputs: the reference's 3x3x3 Si fixture, the Si2 24^3 cell and
species tables from tests/golden/species_tables.npz."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

FIX_LAT = np.array([[5.10, 0.0, 5.10], [0.0, 5.10, 5.10], [5.10, 5.10, 0.0]])
FIX_POS = np.array([[0.0, 0.0, 0.0], [2.55, 2.55, 2.55]])
FE_LAT = np.array([[-2.71176, 2.71176, 2.71176], [2.71176, -2.71176, 2.71176], [2.71176, 2.71176, -2.71176]])

_CACHE = {}


def golden():
    if "g" not in _CACHE:
        with open(os.path.join(GOLDEN, "golden_vectors.json")) as f:
            _CACHE["g"] = json.load(f)
    return _CACHE["g"]


def tables():
    if "t" not in _CACHE:
        _CACHE["t"] = dict(np.load(os.path.join(GOLDEN, "species_tables.npz")))
    return _CACHE["t"]


def species_arrays(tag, basis="s2p2d1"):
    """(max_l, num_basis, rv, rwf[l][p]) of a fixture species."""
    from oracle.lcp_oracle import get_ialpha_index
    t = tables()
    maxl, nb = get_ialpha_index(basis)
    rwf = t["pao_%s_rwf" % tag]
    return maxl, nb, t["pao_%s_rv" % tag], [[rwf[l, p] for p in range(nb[l])] for l in range(maxl + 1)]


def oracle_pao(tag="Si7.0", basis="s2p2d1"):
    from oracle.lcp_oracle import PAO
    maxl, nb, rv, rwf = species_arrays(tag, basis)
    return PAO(maxl, nb, rv, rwf)


def product_pao(tag="Si7.0", basis="s2p2d1"):
    from lcpgrid.pao import PAO
    maxl, nb, rv, rwf = species_arrays(tag, basis)
    return PAO(maxl, nb, rv, rwf)


def aden_tables(pao_tag, vps_tag, core):
    from oracle import lcp_oracle as O
    t = tables()
    xv, rv = t["pao_%s_xv" % pao_tag], t["pao_%s_rv" % pao_tag]
    den = O.normalize_atomic_den(core, xv, t["pao_%s_den" % pao_tag])
    pcc = O.pcc_array(t["vps_%s_pcc" % vps_tag])
    return (xv, rv, den), (t["vps_%s_xv" % vps_tag], t["vps_%s_rv" % vps_tag], pcc)


def si2_cell():
    """Si2 primitive cell at Calc_Ngrid(150) = 24^3 (examples/Si/Si.jl:5-10)."""
    a = 5.43 * 1.8897259886
    lat = np.array([[0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]]) * a
    pos = np.array([[0, 0, 0], [0.25, 0.25, 0.25]]) @ lat
    return lat, pos, (24, 24, 24)
