"""Failure paths of the tensor-core kernels, driven without a GPU fault.

The split-BF16 density kernel is warp-specialised: producers fill a ring of
shared-memory stages, the MMA warp and the epilogue consume and release them,
and every wait on an mbarrier is bounded.  Here one epilogue warp withholds
its stage releases (a signal that nothing else gives) and the poll limit is
short, so the producers' waits run out: the kernel must record LCP_ETIMEDOUT
in the context's error word, stop every role, wait for its copies and MMAs in
flight, free its tensor memory and return.  The call then raises, and the same
context runs the next density and a whole grid step normally, with the same
bits as before the failure.
"""
import time

import numpy as np
import pytest

import lcpgrid as L
from lcpgrid import _lib

pytestmark = pytest.mark.gpu


def test_density_kernel_wait_runs_out_and_unwinds():
    from helpers import product_pao, si2_cell
    from test_gpu_parity import psd_dm
    ctx = L.Context(0, precision="bf16x3")
    lat, pos, ng = si2_cell()
    u = L.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13], ctx=ctx)
    orbs = L.Set_Orbitals_Grid([product_pao()], u)
    assert u.brick_info()["max_images"] > 8  # more K steps than ring stages: the ring must wrap
    dm = psd_dm(u, 5)
    ref = [np.zeros(u.NN)]
    L.Set_Density_Grid("off", u, orbs, dm, ref)

    ctx.set_fault_test(poll_limit=4096, stall=1)
    out = [np.zeros(u.NN)]
    t0 = time.perf_counter()
    with pytest.raises(L.LCPError) as e:
        L.Set_Density_Grid("off", u, orbs, dm, out)
    assert e.value.status == _lib.LCP_ETIMEDOUT
    assert time.perf_counter() - t0 < 10.0  # the short limit, not the default one

    ctx.set_fault_test(0, 0)
    again = [np.zeros(u.NN)]
    L.Set_Density_Grid("off", u, orbs, dm, again)
    np.testing.assert_array_equal(again[0], ref[0])
    job = L.GridStepJob(u, orbs, "off", "LDA")
    job.set_dm(dm)
    job.step()
    assert np.all(np.isfinite(job.energies()))
    with pytest.raises(L.LCPError):
        ctx.set_fault_test(0, 2)  # only the one stall mode exists
