"""lcp_job_step replays its launches as one CUDA graph from a job's second
step on a context.  The replay must give the same bits as the launches issued
one by one, in every precision form and spin setting, count the same kernels,
and be captured again when the device buffers it points into change (here:
another job on the same context growing the shared workspaces, which
reallocates them)."""
import numpy as np
import pytest

import lcpgrid as L

pytestmark = pytest.mark.gpu


def _run(ctx, job, dm, n):
    """n steps with the same D; the H, density and energies of each."""
    out = []
    for _ in range(n):
        job.set_dm(dm)
        l0 = ctx.launch_count
        job.step()
        out.append((job.hks(), job.density(), job.energies(), ctx.launch_count - l0))
    return out


def _same(a, b, exact=True, launches=True):
    """Equal bits; or, for the FP64/FP32 pair kernels (whose blocks add into
    rho and H atomically, in no fixed order), equal to rounding.  And the
    same kernel count, unless one of them is a job's first step (which also
    builds the tables its form needs)."""
    for x, y in zip(a[0] + a[1] + [a[2]], b[0] + b[1] + [b[2]]):
        if exact:
            assert np.array_equal(x, y)
        else:
            np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-14 * np.max(np.abs(y)))
    if launches:
        assert a[3] == b[3]


@pytest.mark.parametrize("precision", ["fp64", "fp32", "bf16x3"])
@pytest.mark.parametrize("spin", ["off", "on"])
def test_graph_replay_same_bits(precision, spin):
    from test_gpu_parity import psd_dm
    from test_gpu_tc import _si2
    ctx = L.Context(0)
    u, orbs = _si2(ctx)
    dm = psd_dm(u, 41, nspin=2 if spin == "on" else 1)
    ctx.set_precision(precision)
    job = L.GridStepJob(u, orbs, spin, "LSDA" if spin == "on" else "LDA")
    exact = precision == "bf16x3"  # the tensor-core form sums in a fixed order
    ctx.set_step_graphs(False)
    first, ref = _run(ctx, job, dm, 2)
    _same(first, ref, exact, launches=False)
    ctx.set_step_graphs(True)
    # direct step (records the signature), capture + launch, then replays
    for r in _run(ctx, job, dm, 4):
        _same(ref, r, exact)


def test_graph_recaptured_after_workspace_growth():
    from test_gpu_parity import psd_dm
    from test_gpu_tc import _mixed_cell, _si2
    ctx = L.Context(0)
    ctx.set_precision("bf16x3")
    u, orbs = _si2(ctx)
    dm = psd_dm(u, 43)
    job = L.GridStepJob(u, orbs, "off", "LDA")
    ref = _run(ctx, job, dm, 3)[2]  # the third step replays the graph
    # a larger cell on the same context: its step grows (reallocates) the
    # context's D-block, partial-block and V-weight workspaces
    u2, orbs2 = _mixed_cell(ctx)
    job2 = L.GridStepJob(u2, orbs2, "off", "LDA")
    _run(ctx, job2, psd_dm(u2, 44), 1)
    for r in _run(ctx, job, dm, 3):  # direct, captured again, replayed
        _same(ref, r)
