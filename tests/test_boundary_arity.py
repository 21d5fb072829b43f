"""Every Python mirror of a reference grid-path function takes exactly the
reference's positional arguments, in the reference's order and under its names.

The reference's call sites (src/KSsolve_SCF.jl:62,144,180,184-185,189,232,252
and the force/energy callers) pass these arguments positionally, so a
drop-in must accept that call unchanged.  Options of this library (the
device context, the synthetic V_na field) are keyword-only; the context
otherwise travels in an argument the reference already passes (ucell,
dft_mixing, xc_func, Orbs_Grid) or is the module's default.
"""
import inspect

import pytest

import lcpgrid as L

# (mirror, reference file:line, positional parameters of the reference method;
# the Julia '!' suffix is dropped from the names)
REFERENCE = [
    ("Set_Orbitals_Grid", "src/Matrix/Set_Orbitals_Grid.jl:26", ["pao", "ucell"]),
    ("Set_dOrbitals_Grid", "src/Matrix/Set_dOrbitals_Grid.jl:1", ["pao", "ucell"]),
    ("Set_Density_Grid", "src/Matrix/Set_Density_Grid.jl:1", ["SpinPol", "ucell", "Orbs_Grid", "DM", "Density_Grid"]),
    ("diagonalize_nc_density", "src/Matrix/Set_Density_Grid.jl:243", ["Density_Grid"]),
    ("Solve_Poisson", "src/Poisson.jl:1", ["SpinPol", "dft_mixing", "Density_Grid", "ADensity_Grid", "dVHart_Grid"]),
    ("Solve_Poisson_xyz", "src/Poisson.jl:29", ["Ngrid", "Recvecs", "Density_xyz", "dVHart_Grid"]),
    ("Set_XC_Grid", "src/XC/XC_Func.jl:111,117,148", ["xc_func", "PCCDensity_Grid", "Density_Grid"]),
    ("Set_Vpot_Grid", "src/Matrix/Set_Vpot_Grid.jl:1", ["xc_func", "dVHart_Grid", "Vpot_Grid"]),
    ("Calc_MatrixElements_dVH_Vxc_off", "src/Hamiltonian.jl:235", ["ucell", "Orbs_Grid", "Vpot_Grid", "MPI_Hks"]),
    ("Calc_MatrixElements_dVH_Vxc_on", "src/Hamiltonian.jl:280", ["ucell", "Orbs_Grid", "Vpot_Grid", "MPI_Hks"]),
    ("Calc_MatrixElements_dVH_Vxc_nc", "src/Hamiltonian.jl:327", ["ucell", "Orbs_Grid", "Vpot_Grid", "MPI_Hks"]),
    ("Calc_EH1", "src/Energy.jl:655", ["SpinPol", "GridVol", "ADensity_Grid", "Density_Grid", "dVHart_Grid"]),
    ("Calc_EXC1", "src/Energy.jl:669",
     ["SpinPol", "xc_type", "system_grid", "ADensity_Grid", "PCCDensity_Grid", "Density_Grid"]),
    ("Set_AdenPCC_Grid", "src/Matrix/Set_AdenPCC_Grid.jl:1",
     ["SpinPol", "Init_Atoms_Nspin", "Init_Atoms_Angle", "pao", "pspot", "ucell"]),
    ("Force3_nospin", "src/Force.jl:407", ["pao", "Orbs_Grid", "Vpot_Grid", "DM", "ucell"]),
    ("Force3_spin", "src/Force.jl:454", ["pao", "Orbs_Grid", "Vpot_Grid", "DM", "ucell"]),
    ("Force3_nc", "src/Force.jl:506", ["pao", "Orbs_Grid", "dVHart_Grid", "Vxc_Grid", "DM", "ucell"]),
    ("Calc_Diff_Coef", "src/XC/GGA_PBE.jl:1", ["gLatvecs"]),
    ("Calc_Ngrid", "src/utils/Calc_Ngrid.jl:1", ["Ecut", "Latvecs"]),
]

# constructors: the reference's positional parameters come first (optional
# extras of this library follow with defaults)
CONSTRUCTORS = [
    ("UCell", "src/UCell.jl:210",
     ["Nspin", "Latvecs", "Natom", "atom2spe", "Gxyz", "Atoms_Cut1", "Ngrid", "Grid_Origin"]),
    ("XC_Func", "src/XC/XC_Func.jl:47", ["xc_type", "SpinPol", "Nspin", "Ngrid", "gLatvecs"]),
]

_POS = (inspect.Parameter.POSITIONAL_ONLY, inspect.Parameter.POSITIONAL_OR_KEYWORD)


@pytest.mark.parametrize("name,where,params", REFERENCE, ids=[r[0] for r in REFERENCE])
def test_mirror_takes_the_reference_arguments(name, where, params):
    sig = inspect.signature(getattr(L, name))
    pos = [p for p in sig.parameters.values() if p.kind in _POS]
    assert [p.name for p in pos] == params, "%s differs from %s" % (name, where)
    # every extra is keyword-only, so the reference's positional call binds as is
    assert all(p.default is inspect.Parameter.empty for p in pos), name
    extras = [p for p in sig.parameters.values() if p.kind not in _POS]
    assert all(p.kind == inspect.Parameter.KEYWORD_ONLY and p.default is not inspect.Parameter.empty
               for p in extras), name
    sig.bind(*params)  # the reference's call form


@pytest.mark.parametrize("name,where,params", CONSTRUCTORS, ids=[c[0] for c in CONSTRUCTORS])
def test_constructor_leads_with_the_reference_arguments(name, where, params):
    sig = inspect.signature(getattr(L, name).__init__)
    names = [p.name for p in sig.parameters.values()][1:]  # without self
    assert names[:len(params)] == params, "%s differs from %s" % (name, where)


def test_context_rides_on_the_passed_objects():
    """The context of a reference-arity call comes from an argument the
    reference passes, else from the module (use_context)."""
    from lcpgrid.api import _ctx_of

    class Holder:
        def __init__(self, ctx):
            self.ctx = ctx

    a, b = object(), object()
    assert _ctx_of(Holder(a)) is a
    assert _ctx_of(Holder(None), Holder(b)) is b
    assert _ctx_of(Holder(a), ctx=b) is b
