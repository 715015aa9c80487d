"""Edge cases of the GA's Hall of Fame and per-generation metrics, the
evaluator and the server's Hall of Fame, against the oracle where it
applies."""
import ctypes as C

import numpy as np
import pytest

import gdock_gb300 as gd
from conftest import make_mol, tatom
from gdock_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def job(nr=30, nl=36, k=4, seed=81):
    c = synth.make_complex(nr, nl, k, seed=seed)
    return c, gd.position_ligand(c.receptor, c.ligand)


def hof_list(recs):
    return [(tuple(r["genes"].tolist()), float(r["fitness"]), int(r["generation"])) for r in recs]


@pytest.mark.parametrize("pop,elitism,cap,top_k", [(2, 0, 1, 1), (2, 2, 3, 50), (8, 1, 1, 8), (40, 5, 2, 100)])
def test_hall_of_fame_small_settings(oracle, pop, elitism, cap, top_k):
    # the smallest population, no elites, a capacity of one entry, top_k
    # larger than the population: the device equals the oracle's HallOfFame
    c, lig = job()
    cfg = _lib.ga_default_cfg(pop_size=pop, elitism=elitism, max_generations=9, seed=12, early_stopping=0,
                              hof_max_size=cap, hof_top_k=top_k)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    res = gd.run_ga([cx], cfg, gd.GD_PREC_F64, use_graph=False, hall_of_fame=True)
    draws = _lib.ga_draw(cfg, cfg.seed, cfg.max_generations)
    hof = oracle.HallOfFame(max_size=cap, top_k=top_k)
    genes, _, _, _ = oracle.run_ga(c.receptor, lig, c.restraint_pairs, cfg, draws, hof=hof)
    np.testing.assert_array_equal(res.genes[0], genes)
    got = hof_list(res.hall_of_fame[0])
    assert [(g, gen) for g, _, gen in got] == [(g, gen) for g, _, gen in hof.entries]
    assert len(got) <= cap


def test_hall_of_fame_off_and_zero_generations():
    c, lig = job()
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    off = _lib.ga_default_cfg(pop_size=16, max_generations=4, seed=3, early_stopping=0, hof_max_size=0)
    res = gd.run_ga([cx], off, gd.GD_PREC_F32, hall_of_fame=True)
    assert len(res.hall_of_fame[0]) == 0
    zero = _lib.ga_default_cfg(pop_size=16, max_generations=0, seed=3, early_stopping=0)
    ev = gd.Evaluator(cx, lig)
    res = gd.run_ga([cx], zero, gd.GD_PREC_F32, hall_of_fame=True, evaluators=[ev])
    assert res.generations[0] == 0 and len(res.hall_of_fame[0]) == 0
    assert res.best_metrics.shape == (1, 0) and res.mean_dockq.shape == (1, 0)


def test_metrics_need_the_jobs_own_complex():
    c, lig = job()
    ctx = gd.Context(0)
    a = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
    b = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
    ev_b = gd.Evaluator(b, lig)
    cfg = _lib.ga_default_cfg(pop_size=16, max_generations=2, seed=3, early_stopping=0)
    with pytest.raises(gd.GdError):
        gd.run_ga([a], cfg, gd.GD_PREC_F32, ctx=ctx, evaluators=[ev_b])
    # the context stays usable
    assert gd.run_ga([a], cfg, gd.GD_PREC_F32, ctx=ctx).generations[0] == 2


def test_evaluator_empty_reference_and_identity(oracle):
    rec = make_mol([tatom(0, 0, 0, resseq=1, chain="A"), tatom(4, 0, 0, resseq=2, chain="A")])
    lig = make_mol([tatom(3, 1, 0, resseq=7, chain="B"), tatom(3, -1, 0, resseq=8, chain="B")])
    cx = gd.Complex(rec, lig, [])
    empty = make_mol([])
    m = gd.Evaluator(cx, empty).eval_metrics(np.zeros((3, 6)))
    # no reference atoms: rmsd, irmsd and fnat are 0 (src/evaluator.rs:92-95,112-115,139-141)
    assert (m["rmsd"] == 0).all() and (m["irmsd"] == 0).all() and (m["fnat"] == 0).all()
    np.testing.assert_allclose(m["dockq"], 1.0 / 3.0 * 2.0)
    # the ligand's own placement as the reference, at the identity pose
    genes = np.zeros((1, 6))
    got = gd.Evaluator(cx, lig).eval_metrics(genes)
    ref = oracle.Evaluator(rec, lig).eval_metrics(lig, genes)
    np.testing.assert_array_equal(np.array([got[k][0] for k in ("rmsd", "irmsd", "fnat", "dockq")]), ref[0])
    assert got["fnat"][0] == 1.0


def test_server_hall_of_fame_capacity_and_state():
    c, lig = job()
    cfg = _lib.ga_default_cfg(pop_size=16, max_generations=6, seed=5, early_stopping=0, hof_max_size=20, hof_top_k=4)
    ctx = gd.Context(0)
    srv = gd.Server(ctx, max_slots=2, ga=cfg)
    jid = srv.submit(c.receptor, lig, c.restraint_pairs, seed=5)
    k = C.c_int32(0)
    # not finished yet: GD_ERR_STATE
    assert ctx.lib.gd_server_hall_of_fame(srv.h, jid, None, 0, C.byref(k)) == _lib.GD_ERR_STATE
    while srv.step():
        pass
    h = srv.hall_of_fame(jid)
    assert len(h) > 1
    # too small a buffer: GD_ERR_CAPACITY with the count
    buf = np.zeros(1, dtype=_lib.HOF_ENTRY_DTYPE)
    st = ctx.lib.gd_server_hall_of_fame(srv.h, jid, buf.ctypes.data, 1, C.byref(k))
    assert st == _lib.GD_ERR_CAPACITY and k.value == len(h)
    srv.close()
