"""The oracle against the reference's golden vectors, and the exact identities
that pin density assembly and grid matrix elements (no reference test covers
those)."""
import numpy as np
import pytest

from helpers import FE_LAT, FIX_LAT, FIX_POS, aden_tables, golden, oracle_pao, si2_cell
from oracle import lcp_oracle as O


@pytest.fixture(scope="module")
def fixture_cell():
    return O.UCell(1, FIX_LAT, 2, [1, 1], FIX_POS, [7.0, 7.0], (3, 3, 3), [0, 0, 0], total_numorbs=[13, 13])


def test_ucell_golden(fixture_cell):
    u, G = fixture_cell, golden()["ucell_si_3x3x3"]
    assert u.CpyCell == G["CpyCell"]
    assert u.GridVol == pytest.approx(G["GridVol"], rel=1e-14)
    assert list(u.FNAN) == G["FNAN"]
    assert [list(x) for x in u.natn] == G["natn"]
    assert [list(x) for x in u.ncn] == G["ncn"]
    assert list(u.GridN_Atom) == G["GridN_Atom"]
    assert [list(map(int, x)) for x in u.GridListAtom] == G["GridListAtom"]
    assert [list(map(int, x)) for x in u.CellListAtom] == G["CellListAtom"]
    assert np.allclose(u.atv[-1], G["atv[end]"]) and list(u.atv_ijk[-1]) == G["atv_ijk[end]"]


def test_overlap_vectorised_equals_literal(fixture_cell):
    u = fixture_cell
    g1, g2 = O.calc_atom_overlap_grid_literal(u.CpyCell, u.pairs, u.GridN_Atom, u.GridListAtom, u.CellListAtom,
                                              u.atv_ijk, u.ratv)
    for p in range(u.Nloop):
        assert np.array_equal(g1[p], u.MPI_GListTAtoms1[p])
        assert np.array_equal(g2[p], u.MPI_GListTAtoms2[p])


def test_orbitals_golden(fixture_cell):
    orbs = O.set_orbitals_grid([oracle_pao()], fixture_cell)
    gv = golden()["orbs_si_3x3x3"]
    for key, ref in gv.items():
        a, o = (int(x) - 1 for x in key.split("_"))
        np.testing.assert_allclose(orbs[a][o], ref, rtol=1.5e-8, atol=1e-15)


def test_poisson_golden():
    P = golden()["poisson_si_3x3x3"]
    rec = 2 * np.pi * np.linalg.inv(FIX_LAT.T)
    v = O.solve_poisson_xyz((3, 3, 3), rec, np.array(P["density_xyz"]))
    np.testing.assert_allclose(v, P["dVHart_Grid"], rtol=1.5e-8, atol=1e-15)


def test_lda_lsda_golden():
    g = golden()
    x = np.array(g["lda_ca"]["input"])
    for s, ref in g["lda_ca"]["switch"].items():
        np.testing.assert_allclose(O.lda_ca(x, int(s)), ref, atol=1e-15, rtol=0)
    up, dn = np.array(g["lsda_ca"]["up"]), np.array(g["lsda_ca"]["down"])
    for s, ref in g["lsda_ca"]["switch"].items():
        a, b = O.lsda_ca(up, dn, int(s))
        np.testing.assert_allclose(a, ref["B1"], rtol=1.5e-8)
        np.testing.assert_allclose(b, ref["B2"], rtol=1.5e-8)


def test_adenpcc_and_xc_golden(fixture_cell):
    g = golden()
    for name, vps in (("Set_AdenPCC_Grid Si LDA", "Si_CA19"), ("Set_AdenPCC_Grid Si GGA-PBE", "Si_PBE19")):
        pt, vt = aden_tables("Si7.0", vps, 4.0)
        a, p, d = O.set_adenpcc_grid("off", [[2., 2.], [2., 2.]], [[0, 0, 0, 0]] * 2, [pt], [vt], fixture_cell)
        ref = g["adenpcc"][name]
        np.testing.assert_allclose(a, ref["ADensity_Grid"], rtol=1.5e-8)
        np.testing.assert_allclose(p, ref["PCCDensity_Grid"], rtol=1.5e-8)
        np.testing.assert_allclose(d[0], ref["Density_Grid"][0], rtol=1.5e-8)
        if vps == "Si_CA19":
            vxc = O.set_xc_grid("LDA", "off", p, d)
            np.testing.assert_allclose(vxc[0], g["xc_grid"]["XC_PBE Si LDA"][0], rtol=1.5e-8)
    ufe = O.UCell(2, FE_LAT, 1, [1], [[0, 0, 0]], [6.0], (3, 3, 3), [0, 0, 0])
    pt, vt = aden_tables("Fe6.0H", "Fe_PBE19H", 16.0)
    a, p, d = O.set_adenpcc_grid("on", [[8., 6.]], [[0, 0, 0, 0]], [pt], [vt], ufe)
    ref = g["adenpcc"]["Set_AdenPCC_Grid BCC_Fe GGA-PBE"]
    np.testing.assert_allclose(a, ref["ADensity_Grid"], rtol=1.5e-8)
    np.testing.assert_allclose(p, ref["PCCDensity_Grid"], rtol=1.5e-8)
    for s in range(2):
        np.testing.assert_allclose(d[s], ref["Density_Grid"][s], rtol=1.5e-8)
    pt, vt = aden_tables("Fe6.0H", "Fe_CA19H", 16.0)
    a, p, d = O.set_adenpcc_grid("on", [[8., 6.]], [[0, 0, 0, 0]], [pt], [vt], ufe)
    vxc = O.set_xc_grid("LSDA", "on", p, d)
    for s in range(2):
        np.testing.assert_allclose(vxc[s], g["xc_grid"]["XC_PBE BCC_Fe LSDA"][s], rtol=1.5e-8)


def test_calc_ngrid_golden():
    for c in golden()["calc_ngrid"]:
        assert list(O.calc_ngrid(c["Ecut"], c["Latvecs"])) == c["Ngrid"]


def _psd_dm(u, seed, trace=8.0):
    rng = np.random.default_rng(seed)
    no = u.Total_NumOrbs
    off = np.concatenate([[0], np.cumsum(no)])
    C = rng.normal(size=(off[-1], 6))
    M = C @ C.T
    M *= trace / np.trace(M)
    dm = np.zeros(u.Total_Hsize)
    for p, (a, b, _) in enumerate(u.pairs):
        blk = M[off[a - 1]:off[a], off[b - 1]:off[b]]
        dm[u.block_offset[p]:u.block_offset[p] + blk.size] = blk.reshape(-1)
    return dm


def test_density_and_h_identities():
    """Exact identities of the restated contractions on the Si2 24^3 cell:
    (i) H with V = 1 is the grid overlap S, (ii) dV*sum(rho*V) = <D, H>,
    (iii) dV*sum(rho) = <D, S> (electron count), (iv) rho >= 0 for a PSD
    Gamma-point D, (v) H(i,j,R) = H(j,i,-R)^T."""
    lat, pos, ng = si2_cell()
    u = O.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], total_numorbs=[13, 13])
    orbs = O.set_orbitals_grid([oracle_pao()], u)
    dm = _psd_dm(u, 7)
    rho = O.set_density_grid("off", u, orbs, [dm])[0]
    rng = np.random.default_rng(3)
    V = rng.normal(size=u.NN)
    H = O.calc_matrix_elements(u, orbs, [V], 1)[0]
    S = O.calc_matrix_elements(u, orbs, [np.ones(u.NN)], 1)[0]
    assert np.dot(rho, V) * u.GridVol == pytest.approx(np.dot(dm, H), rel=1e-11)
    assert np.sum(rho) * u.GridVol == pytest.approx(np.dot(dm, S), rel=1e-11)
    assert rho.min() > -1e-12
    # partner symmetry
    idx = {(a, b, c): p for p, (a, b, c) in enumerate(u.pairs)}
    ijk = u.atv_ijk
    n = 2 * u.CpyCell + 1
    for p, (a, b, c) in enumerate(u.pairs[:40]):
        mc = u.ratv[tuple(-ijk[c] + u.CpyCell)]
        q = idx[(b, a, mc)]
        no = 13
        hp = H[u.block_offset[p]:u.block_offset[p] + no * no].reshape(no, no)
        hq = H[u.block_offset[q]:u.block_offset[q] + no * no].reshape(no, no)
        np.testing.assert_allclose(hp, hq.T, rtol=1e-12, atol=1e-15)
