"""Serving loop: continuous batching of docking jobs of different sizes.

Each job's result is the same alone and in a mix with other jobs that arrive
while it runs (bit for bit: its draws are its own and every pose is scored
independently); admission respects the HBM budget; latencies are reported."""
import numpy as np
import pytest

import gdock_gb300 as gd
from gdock_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def jobs(k):
    sizes = [(30, 25), (70, 40), (45, 60), (25, 20), (90, 50)]
    out = []
    for i in range(k):
        nr, nl = sizes[i % len(sizes)]
        c = synth.make_complex(nr, nl, 4, seed=500 + i)
        out.append((c.receptor, gd.position_ligand(c.receptor, c.ligand), c.restraint_pairs))
    return out


def ga_cfg():
    return _lib.ga_default_cfg(pop_size=24, max_generations=30, early_stopping=1, convergence_window=4,
                               convergence_threshold=0.005)


def run_alone(ctx, job, seed):
    srv = gd.Server(ctx, max_slots=4, ga=ga_cfg())
    jid = srv.submit(*job, seed=seed)
    while srv.step():
        pass
    srv.step()
    out = srv.result(jid)
    srv.close()
    return out


def test_same_result_alone_and_in_the_mix():
    ctx = gd.Context(0)
    J = jobs(5)
    alone = [run_alone(ctx, J[i], 1000 + i) for i in range(5)]
    srv = gd.Server(ctx, max_slots=3, ga=ga_cfg())
    ids = [srv.submit(*J[0], seed=1000), srv.submit(*J[1], seed=1001)]
    for _ in range(3):
        srv.step()
    ids += [srv.submit(*J[i], seed=1000 + i) for i in (2, 3, 4)]  # arrive while others run
    while srv.step():
        pass
    for i, jid in enumerate(ids):
        res, genes, e, hist = srv.result(jid)
        a_res, a_genes, a_e, a_hist = alone[i]
        assert res.status == _lib.GD_JOB_DONE and a_res.status == _lib.GD_JOB_DONE
        assert res.generations == a_res.generations
        np.testing.assert_array_equal(genes, a_genes)
        assert e.tobytes() == a_e.tobytes()
        np.testing.assert_array_equal(hist, a_hist)
    st = srv.stats()
    assert st.completed == 5 and st.queued == 0 and st.resident == 0
    assert st.latency_p99_s >= st.latency_p50_s > 0
    srv.close()


def test_server_matches_batched_ga_run():
    ctx = gd.Context(0)
    (rec, lig, pairs), = jobs(1)
    cfg = ga_cfg()
    cfg.seed = 77
    cx = gd.Complex(rec, lig, pairs, ctx=ctx)
    ref = gd.run_ga([cx], cfg, gd.GD_PREC_F32, use_graph=False, ctx=ctx, hall_of_fame=True)
    res, genes, e, hist = run_alone(ctx, (rec, lig, pairs), 77)
    assert res.generations == ref.generations[0]
    np.testing.assert_array_equal(genes, ref.genes[0])
    assert e.tobytes() == ref.energies[0].tobytes()
    # the served job's Hall of Fame equals the batched run's
    srv = gd.Server(ctx, max_slots=2, ga=cfg)
    jid = srv.submit(rec, lig, pairs, seed=77)
    while srv.step():
        pass
    h = srv.hall_of_fame(jid)
    assert len(h) > 0 and h.tobytes() == ref.hall_of_fame[0].tobytes()
    srv.close()


def test_admission_by_hbm_budget_tick_by_tick():
    """A budget of one byte holds one resident job at a time (the first job
    is admitted even over it): driven tick by tick, at most one job is ever
    resident, the jobs finish in submission order (first come first served),
    and the device time of the generations is counted."""
    ctx = gd.Context(0)
    J = jobs(4)
    srv = gd.Server(ctx, max_slots=4, hbm_budget=1, ga=ga_cfg())
    ids = [srv.submit(*J[i], seed=7 + i) for i in range(4)]
    done_order, ticks = [], 0
    while True:
        resident = srv.step()
        ticks += 1
        assert resident <= 1, ticks
        assert srv.stats().resident == resident
        for jid in ids:
            if jid not in done_order and srv.result(jid)[0].status == _lib.GD_JOB_DONE:
                done_order.append(jid)
        if len(done_order) == len(ids):
            break
        assert ticks < 4 * 40, "jobs did not finish"
    assert done_order == ids
    st = srv.stats()
    assert st.completed == 4 and st.queued == 0 and st.resident == 0
    assert 0.0 < st.gpu_busy_s <= st.elapsed_s
    for jid in ids:
        res = srv.result(jid)[0]
        assert res.queue_s >= 0 and res.latency_s >= res.queue_s
    srv.close()


def test_background_thread_with_budget():
    ctx = gd.Context(0)
    J = jobs(4)
    srv = gd.Server(ctx, max_slots=4, hbm_budget=1, ga=ga_cfg())
    srv.start()
    ids = [srv.submit(*J[i], seed=7 + i) for i in range(4)]
    for jid in ids:
        assert srv.wait(jid, 300.0) == _lib.GD_JOB_DONE
    st = srv.stats()
    srv.stop()
    assert st.completed == 4 and st.resident == 0
    for jid in ids:
        res = srv.result(jid)[0]
        assert res.queue_s >= 0 and res.latency_s >= res.queue_s
    srv.close()


def test_worker_error_fails_jobs_and_refuses_submissions():
    """A tick that fails (here a bounded wait that runs out, GD_TUNE_FAULT)
    stops the server's thread: resident and queued jobs end FAILED with the
    tick's status, and later submissions are refused with GD_ERR_STATE."""
    ctx = gd.Context(0)
    try:
        J = jobs(2)
        srv = gd.Server(ctx, max_slots=4, ga=ga_cfg())
        ctx.set_tuning(_lib.GD_TUNE_FAULT, 1)
        ids = [srv.submit(*J[0], seed=7), srv.submit(*J[1], seed=8)]
        srv.start()
        for jid in ids:
            assert srv.wait(jid, 60.0) == _lib.GD_JOB_FAILED
        ctx.set_tuning(_lib.GD_TUNE_FAULT, 0)
        for jid in ids:
            res = srv.result(jid)[0]
            assert res.status == _lib.GD_JOB_FAILED and res.error == 4  # GD_ERR_TIMEOUT
        with pytest.raises(gd.GdError) as ei:
            srv.submit(*J[0], seed=9)
        assert ei.value.status == 6  # GD_ERR_STATE
        assert "timed out" in str(ei.value) or "wait" in str(ei.value)
        srv.stop()
        srv.close()
    finally:
        ctx.close()
