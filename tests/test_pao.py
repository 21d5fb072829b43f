"""Species data readers: basis strings, the .pao/.vps section parsers (on a
file written from the fixture tables) and the atomic-density normalisation."""
import numpy as np
import pytest

from helpers import golden, tables
from lcpgrid import pao as P
from oracle import lcp_oracle as O


def test_get_ialpha_index():
    assert P.get_ialpha_index("s2p2d1") == (2, [2, 2, 1])
    assert P.get_ialpha_index("s1") == (0, [1])
    assert P.get_ialpha_index("s3p2d2f1") == (3, [3, 2, 2, 1])
    for bad in ("s2p", "s2d1", "s1p1d1f1g1"):
        with pytest.raises(ValueError):
            P.get_ialpha_index(bad)


def _write_pao(path, tag, cutoff):
    t = tables()
    xv, rv, den, rwf = t["pao_%s_xv" % tag], t["pao_%s_rv" % tag], t["pao_%s_den" % tag], t["pao_%s_rwf" % tag]
    n = xv.size
    lines = ["grid.num.output  %d" % n, "radial.cutoff.pao  %s" % cutoff, "PAO.Lmax  %d" % (rwf.shape[0] - 1),
             "PAO.Mul  %d" % rwf.shape[1], "<valence.charge.density"]
    lines += ["%.15f %.15f %.15e" % (xv[i], rv[i], den[i]) for i in range(n)]
    lines.append("valence.charge.density>")
    for L in range(rwf.shape[0]):
        lines.append("<pseudo.atomic.orbitals.L=%d" % L)
        lines += [" ".join(["%.15f" % xv[i], "%.15f" % rv[i]] + ["%.17e" % rwf[L, m, i] for m in range(rwf.shape[1])])
                  for i in range(n)]
        lines.append("pseudo.atomic.orbitals.L=%d>" % L)
    path.write_text("\n".join(lines) + "\n")


def test_read_pao_roundtrip(tmp_path):
    _write_pao(tmp_path / "Si7.0.pao", "Si7.0", 7.0)
    pao = P.Read_PAO(4.0, "Si", 7.0, "s2p2d1", "", str(tmp_path))
    facts = golden()["read_pao"]["Read_PAO Si LDA"]
    assert pao.Spe_MaxL_Basis == facts["Spe_MaxL_Basis"]
    assert pao.Spe_Num_Basis == facts["Spe_Num_Basis"]
    assert pao.Spe_Total_NumOrbs == facts["Spe_Total_NumOrbs"]
    assert pao.Spe_Num_Mesh_PAO == facts["Spe_Num_Mesh_PAO"]
    assert pao.Spe_Atom_Cut1 == facts["Spe_Atom_Cut1"]
    t = tables()
    np.testing.assert_array_equal(pao.Spe_PAO_RV, t["pao_Si7.0_rv"])
    np.testing.assert_array_equal(pao.Spe_PAO_RWF[1][1], t["pao_Si7.0_rwf"][1, 1])
    ref = O.normalize_atomic_den(4.0, t["pao_Si7.0_xv"], t["pao_Si7.0_den"])
    np.testing.assert_allclose(pao.Spe_Atomic_Den, ref, rtol=1e-14)
    with pytest.raises(ValueError):
        P.Read_PAO(4.0, "Si", 7.0, "s4p2d1", "", str(tmp_path))
