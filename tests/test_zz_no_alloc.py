"""The split-BF16 density entry point that allocates no device memory
(lcp_set_density_grid_noalloc), called through the C ABI with device buffers.

It serves callers that cannot call cudaMalloc when they run the density:
hosts whose own pool allocator owns the device memory, and serving loops that
cannot take the device-wide synchronisation of cudaMalloc/cudaFree.  Its
result must match the allocating entry point lcp_set_density_grid at split-
BF16 precision, within the split-BF16 density bound, on consecutive calls
that share its fixed scratch array.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import lcpgrid as L
from lcpgrid import _lib

pytestmark = pytest.mark.gpu

RHO_TOL = 5e-6  # split-BF16 density bound, relative to max |rho| (as the other tensor-core tests)


def _device_ptrs(tensors):
    arr = (ctypes.POINTER(ctypes.c_double) * len(tensors))()
    for k, t in enumerate(tensors):
        arr[k] = ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctypes.c_double))
    return ctypes.cast(arr, _lib._ppd), arr


def _noalloc(ctx, u, orbs, spin, dm_dev, rho_dev):
    pd, k1 = _device_ptrs(dm_dev)
    pr, k2 = _device_ptrs(rho_dev)
    _lib.check(_lib.lib.lcp_set_density_grid_noalloc(ctx._h, u._h, orbs._h, _lib.SPIN[spin], pd, pr))


def _alloc_count():
    n = ctypes.c_int64()
    _lib.check(_lib.lib.lcp_device_alloc_count(ctypes.byref(n)))
    return n.value


def _reference(ctx, u, orbs, spin, dm):
    out = [np.zeros(u.NN) for _ in dm]
    ctx.set_precision("bf16x3")
    try:
        L.Set_Density_Grid(spin, u, orbs, dm, out)
    finally:
        ctx.set_precision("fp64")
    return out


def test_density_noalloc_matches_allocating_entry():
    torch = pytest.importorskip("torch")
    from helpers import product_pao, si2_cell
    from test_gpu_parity import psd_dm
    ctx = L.Context(0)
    lat, pos, ng = si2_cell()
    u = L.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13])
    orbs = L.Set_Orbitals_Grid([product_pao()], u, ctx=ctx)
    from lcpgrid.workloads import psd_nc_density_matrices
    for spin, n in (("off", 1), ("on", 2), ("nc", 4)):
        if spin == "nc":
            dms = [psd_nc_density_matrices(u, seed, trace=4.0) for seed in (101, 202)]
        else:
            dms = [psd_dm(u, seed, nspin=n) for seed in (101, 202)]
        refs = [_reference(ctx, u, orbs, spin, dm) for dm in dms]  # also builds the split-BF16 tables
        outs = []
        for dm in dms:  # two calls in a row on the shared scratch
            dm_dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in dm]
            rho_dev = [torch.full((u.NN,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(n)]
            torch.cuda.synchronize()
            before = _alloc_count()
            _noalloc(ctx, u, orbs, spin, dm_dev, rho_dev)
            assert _alloc_count() == before  # the call made no device allocation of its own
            outs.append([r.cpu().numpy() for r in rho_dev])
        for ref, out in zip(refs, outs):
            for c in range(n):
                scale = np.max(np.abs(ref[c]))
                assert np.all(np.isfinite(out[c]))
                assert np.max(np.abs(out[c] - ref[c])) <= RHO_TOL * scale


def test_density_noalloc_rejections():
    torch = pytest.importorskip("torch")
    from helpers import product_pao, si2_cell
    from lcpgrid.workloads import si_supercell
    ctx = L.Context(0)
    # orbitals whose split-BF16 tables were never built
    lat, pos, ng = si2_cell()
    u = L.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13])
    orbs = L.Set_Orbitals_Grid([product_pao()], u, ctx=ctx)
    dm_dev = [torch.zeros(u.Total_Hsize, dtype=torch.float64, device="cuda")]
    rho_dev = [torch.zeros(u.NN, dtype=torch.float64, device="cuda")]
    with pytest.raises(L.LCPError) as e:
        _noalloc(ctx, u, orbs, "off", dm_dev, rho_dev)
    assert e.value.status == _lib.LCP_ESTATE
    # a cell with more neighbour pairs than the fixed scratch holds (216 Si, coarse grid)
    lat, pos = si_supercell(3)
    nat = pos.shape[0]
    big = L.UCell(1, lat, nat, [1] * nat, pos, [7.0] * nat, (48, 48, 48), [0, 0, 0], Total_NumOrbs=[13] * nat)
    assert big.Nloop > 10921
    borbs = L.Set_Orbitals_Grid([product_pao()], big, ctx=ctx)
    dm_dev = [torch.zeros(big.Total_Hsize, dtype=torch.float64, device="cuda")]
    rho_dev = [torch.zeros(big.NN, dtype=torch.float64, device="cuda")]
    with pytest.raises(L.LCPError) as e:
        _noalloc(ctx, big, borbs, "off", dm_dev, rho_dev)
    assert e.value.status == _lib.LCP_EINVAL
