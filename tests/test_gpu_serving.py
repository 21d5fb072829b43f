"""Serving engine (lcp_server_*): grid-step requests on several
device-resident structures, batched per slot and concurrent across slots.
Each result must be the same alone and in a mixed, batched stream, and
structures are admitted by device footprint, queued while they do not fit."""
import numpy as np
import pytest

import lcpgrid as L

pytestmark = pytest.mark.gpu


def _structures(ctx):
    """Four small cells of different size and grid: Si2 primitive (24^3), the
    8-atom Si cell (40^3), a 3-species 18/13/4-orbital cell and Si2 again."""
    from helpers import product_pao, si2_cell
    from lcpgrid.workloads import psd_density_matrices, si64_workload, smooth_vna
    from test_gpu_tc import _mixed_cell
    out = []
    lat, pos, ng = si2_cell()
    u = L.UCell(1, lat, 2, [1, 1], pos, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13])
    out.append((u, L.Set_Orbitals_Grid([product_pao()], u, ctx=ctx)))
    wl = si64_workload(nrep=1, ngrid=(40, 40, 40))
    u = L.UCell(1, wl["latvecs"], wl["natom"], wl["atom2spe"], wl["gxyz"], wl["cut"], wl["ngrid"], wl["origin"],
                Total_NumOrbs=wl["numorbs"])
    out.append((u, L.Set_Orbitals_Grid(wl["paos"], u, ctx=ctx)))
    out.append(_mixed_cell(ctx))
    u = L.UCell(1, lat, 2, [1, 1], pos * 1.01, [7.0, 7.0], ng, [0, 0, 0], Total_NumOrbs=[13, 13])
    out.append((u, L.Set_Orbitals_Grid([product_pao()], u, ctx=ctx)))
    jobs = []
    for k, (u, orbs) in enumerate(out):
        vna = smooth_vna(u.Ngrid, u.Latvecs, 40 + k)
        job = L.GridStepJob(u, orbs, "off", "LDA", None, None, vna)
        dm = psd_density_matrices(u, 50 + k, trace=4.0 * u.Natom)
        jobs.append((job, dm))
    return jobs


def test_server_results_alone_and_mixed():
    ctx = L.Context(0)
    jobs = _structures(ctx)
    srv = L.Server(0, nslots=3, precision="bf16x3", budget_bytes=64e9)
    ids = [srv.add(job) for job, _ in jobs]
    alone = {}
    for sid, (job, dm) in zip(ids, jobs):
        srv.submit(sid, dm, tag=sid)
        got = []
        while not got:
            got = srv.poll(wait_ms=2000)
        assert got[0][0] == sid
        alone[sid] = got[0][1]
    # the same requests interleaved and concurrent (several per structure)
    rng = np.random.default_rng(3)
    order = list(rng.permutation(np.repeat(ids, 5)))
    for n, sid in enumerate(order):
        srv.submit(int(sid), jobs[ids.index(sid)][1], tag=1000 + n)
    results = []
    while len(results) < len(order):
        results += srv.poll(wait_ms=2000)
    assert srv.stats()[:2] == (len(ids) + len(order), len(ids) + len(order))
    for tag, e, lat in results:
        sid = int(order[tag - 1000])
        np.testing.assert_allclose(e, alone[sid], rtol=1e-12, atol=0)
        assert lat > 0
    # and the same as the job's own step on its context
    ctx.set_precision("bf16x3")
    try:
        for sid, (job, dm) in zip(ids, jobs):
            job.set_dm(dm)
            job.step()
            np.testing.assert_allclose(job.energies(), alone[sid], rtol=1e-12, atol=0)
    finally:
        ctx.set_precision("fp64")
    srv.close()


def test_server_batches_requests():
    """With one slot and requests already queued, the slot steps them as
    batches of several structures; every result equals the request alone."""
    ctx = L.Context(0)
    jobs = _structures(ctx)
    srv = L.Server(0, nslots=1, precision="bf16x3", budget_bytes=64e9, max_batch=1)
    ids = [srv.add(job) for job, _ in jobs]
    alone = {}
    for sid, (job, dm) in zip(ids, jobs):
        srv.submit(sid, dm, tag=sid)
        got = []
        while not got:
            got = srv.poll(wait_ms=2000)
        alone[sid] = got[0][1]
    assert srv.batch_stats()[0] == 0
    srv.set_max_batch(8)
    order = [int(x) for x in np.repeat(ids, 4)]
    for n, sid in enumerate(order):
        srv.submit(sid, jobs[ids.index(sid)][1], tag=100 + n)
    results = []
    while len(results) < len(order):
        results += srv.poll(wait_ms=2000)
    nb, nreq, nwait, t_asm, t_batch = srv.batch_stats()
    assert nb >= 1 and nreq >= 2 * nb and nwait == 0 and 0 < t_asm <= t_batch
    for tag, e, lat in results:
        np.testing.assert_allclose(e, alone[order[tag - 100]], rtol=1e-12, atol=0)
    srv.close()
    with pytest.raises(L.LCPError) as ex:
        L.Server(0, nslots=1, precision="fp64", budget_bytes=1e9, max_batch=4)
    assert ex.value.status == 5  # LCP_ENOTSUP: batched steps are split-BF16


def test_server_admission_by_footprint():
    ctx = L.Context(0)
    jobs = _structures(ctx)
    # admission measures the footprint with the split-BF16 tables built
    probe = L.Server(0, nslots=1, precision="bf16x3", budget_bytes=1e12)
    for job, _ in jobs[:2]:
        probe.remove(probe.add(job))
    probe.close()
    fp = [job.footprint() for job, _ in jobs]
    assert min(fp) > 0
    with pytest.raises(L.LCPError) as e:  # larger than the whole budget: refused
        L.Server(0, nslots=1, precision="bf16x3", budget_bytes=fp[1] // 2).add(jobs[1][0])
    assert e.value.status == 2  # LCP_ENOMEM
    srv = L.Server(0, nslots=2, precision="bf16x3", budget_bytes=fp[1] + fp[0] // 2)
    a = srv.add(jobs[0][0])
    b = srv.add(jobs[1][0])  # does not fit beside a: queued
    assert srv.state(a) == L.Server.ADMITTED and srv.state(b) == L.Server.WAITING
    assert srv.batch_stats()[2] == 1
    srv.submit(b, jobs[1][1], tag=7)  # waits with its structure
    srv.submit(a, jobs[0][1], tag=6)
    got = []
    while not got:
        got = srv.poll(wait_ms=2000)
    assert [g[0] for g in got] == [6]
    assert srv.poll(wait_ms=300) == []  # b's request cannot run before b is admitted
    srv.remove(a)  # frees the budget: b is admitted and its request runs
    assert srv.state(b) == L.Server.ADMITTED
    got = []
    while not got:
        got = srv.poll(wait_ms=2000)
    assert got[0][0] == 7 and np.isfinite(got[0][1]).all()
    assert srv.stats()[2] == fp[1]
    srv.close()
