"""The library's host geometry (UCell construction in C++) against the
reference's golden lists and the oracle -- bit-exact integer lists."""
import numpy as np
import pytest

import lcpgrid as L
from helpers import FE_LAT, FIX_LAT, FIX_POS, golden, si2_cell
from oracle import lcp_oracle as O


def _compare(lat, natom, pos, cut, ng, orbs, origin=(0, 0, 0), nspin=1):
    u = L.UCell(nspin, lat, natom, [1] * natom, pos, cut, ng, list(origin), Total_NumOrbs=orbs)
    uo = O.UCell(nspin, lat, natom, [1] * natom, pos, cut, ng, list(origin), total_numorbs=orbs)
    assert u.CpyCell == uo.CpyCell
    assert list(u.FNAN) == list(uo.FNAN)
    assert [list(x) for x in u.natn] == [list(x) for x in uo.natn]
    assert [list(x) for x in u.ncn] == [list(x) for x in uo.ncn]
    assert list(u.GridN_Atom) == list(uo.GridN_Atom)
    for a in range(natom):
        assert np.array_equal(u.GridListAtom[a], uo.GridListAtom[a])
        assert np.array_equal(u.CellListAtom[a], uo.CellListAtom[a])
    assert list(u.MPI_NumOLG) == list(uo.MPI_NumOLG)
    assert u.Total_Hsize == uo.Total_Hsize
    return u, uo


def test_golden_fixture():
    G = golden()["ucell_si_3x3x3"]
    u = L.UCell(1, FIX_LAT, 2, [1, 1], FIX_POS, [7.0, 7.0], (3, 3, 3), [0, 0, 0], Total_NumOrbs=[13, 13])
    assert u.CpyCell == G["CpyCell"]
    assert u.GridVol == pytest.approx(G["GridVol"], rel=1e-15)
    assert list(u.FNAN) == G["FNAN"]
    assert [list(x) for x in u.natn] == G["natn"]
    assert [list(x) for x in u.ncn] == G["ncn"]
    assert list(u.GridN_Atom) == G["GridN_Atom"]
    assert [list(x) for x in u.GridListAtom] == G["GridListAtom"]
    assert [list(x) for x in u.CellListAtom] == G["CellListAtom"]
    assert np.allclose(u.atv[-1], G["atv[end]"]) and list(u.atv_ijk[-1]) == G["atv_ijk[end]"]


def test_overlap_lists_match_oracle_fixture():
    u, uo = _compare(FIX_LAT, 2, FIX_POS, [7.0, 7.0], (3, 3, 3), [13, 13])
    for p in range(u.Nloop):
        g1, g2 = u.GListTAtoms(p)
        assert np.array_equal(g1, uo.MPI_GListTAtoms1[p])
        assert np.array_equal(g2, uo.MPI_GListTAtoms2[p])


def test_si2_24cubed():
    lat, pos, ng = si2_cell()
    u, uo = _compare(lat, 2, pos, [7.0, 7.0], ng, [13, 13])
    for p in range(0, u.Nloop, 7):
        g1, g2 = u.GListTAtoms(p)
        assert np.array_equal(g1, uo.MPI_GListTAtoms1[p])
        assert np.array_equal(g2, uo.MPI_GListTAtoms2[p])
    # every pair appears with its partner, the folded list keeps one of each
    assert u.n_unique == (u.Nloop + 2) // 2


def test_odd_grid_offcentre_origin_and_mixed_cutoffs():
    lat = np.array([[7.1, 0.3, 0.0], [0.2, 6.3, 0.1], [0.0, 0.4, 8.2]])
    pos = np.array([[0.3, 0.2, 0.1], [3.4, 3.0, 4.1], [5.9, 1.1, 2.2]])
    _compare(lat, 3, pos, [4.0, 5.5, 3.0], (15, 14, 17), [4, 9, 13], origin=(0.11, -0.07, 0.05))


def test_single_atom_bcc():
    _compare(FE_LAT, 1, [[0, 0, 0]], [6.0], (9, 9, 9), [13])


def test_calc_ngrid_golden():
    for c in golden()["calc_ngrid"]:
        assert list(L.Calc_Ngrid(c["Ecut"], c["Latvecs"])) == c["Ngrid"]


def test_invalid_inputs_raise():
    with pytest.raises(L.LCPError):
        L.UCell(1, np.zeros((3, 3)), 1, [1], [[0, 0, 0]], [5.0], (8, 8, 8), [0, 0, 0])
    with pytest.raises(L.LCPError):
        L.UCell(1, FIX_LAT, 1, [1], [[0, 0, 0]], [5.0], (0, 8, 8), [0, 0, 0])
    with pytest.raises(L.LCPError):
        L.UCell(3, FIX_LAT, 1, [1], [[0, 0, 0]], [5.0], (8, 8, 8), [0, 0, 0])
    with pytest.raises(L.LCPError):
        L.Calc_Ngrid(-1.0, FIX_LAT)
