"""Device GA against the oracle's replay of the same draws.

Plain FP64 form: the device population equals the oracle's bit for bit
after every generation (selection only depends on fitness comparisons, and
those agree); energies within 1e-12.  Batched jobs give the same result alone
and in a mix of uneven complexes."""
import numpy as np
import pytest

import gdock_gb300 as gd
from gdock_gb300 import _lib, synth

pytestmark = pytest.mark.gpu
NAMES = ("fitness", "vdw", "elec", "desolv", "air", "restraint_penalty")


def setup_job(nr, nl, k, seed):
    c = synth.make_complex(nr, nl, k, seed=seed)
    return c, gd.position_ligand(c.receptor, c.ligand)


def check_energies(e, ref, tol):
    for k, name in enumerate(NAMES):
        err = np.abs(e[name] - ref[:, k]) / np.maximum(np.abs(ref[:, k]), 1.0)
        assert err.max() <= tol, (name, float(err.max()))


@pytest.mark.parametrize("early", [False, True])
def test_ga_fp64_matches_oracle(oracle, early):
    c, lig = setup_job(30, 36, 4, seed=77)
    cfg = _lib.ga_default_cfg(pop_size=24, max_generations=12 if not early else 40, seed=5,
                              early_stopping=1 if early else 0, convergence_window=3, convergence_threshold=0.01)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    res = gd.run_ga([cx], cfg, gd.GD_PREC_F64, use_graph=False)
    draws = _lib.ga_draw(cfg, cfg.seed, cfg.max_generations)
    genes, e, gens, hist = oracle.run_ga(c.receptor, lig, c.restraint_pairs, cfg, draws)
    assert res.generations[0] == gens
    np.testing.assert_array_equal(res.genes[0], genes)
    check_energies(res.energies[0], e, 1e-12)
    np.testing.assert_allclose(res.history[0][:len(hist)], hist, rtol=1e-12)
    if early:
        assert gens < cfg.max_generations


def test_ga_fp32_graph_runs_and_scores_final_population(oracle):
    c, lig = setup_job(30, 36, 4, seed=78)
    cfg = _lib.ga_default_cfg(pop_size=32, max_generations=8, seed=9, early_stopping=0)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    res = gd.run_ga([cx], cfg, gd.GD_PREC_F32, use_graph=True)
    assert res.generations[0] == 8
    ref = oracle.score_poses(c.receptor, lig, c.restraint_pairs, res.genes[0])
    check_energies(res.energies[0], ref, 1e-5)
    # best-of-generation never gets worse than the elites allow
    h = res.history[0]
    assert np.isfinite(h).all()


def test_batched_jobs_same_alone_and_in_the_mix():
    jobs = [setup_job(25, 20, 3, 101), setup_job(70, 45, 6, 102), setup_job(40, 60, 5, 103)]
    cfg = _lib.ga_default_cfg(pop_size=20, max_generations=6, seed=11, early_stopping=0)
    ctx = gd.Context(0)
    cxs = [gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx) for c, lig in jobs]
    mix = gd.run_ga(cxs, cfg, gd.GD_PREC_F32, use_graph=True, ctx=ctx)
    for j, cx in enumerate(cxs):
        c1 = _lib.ga_default_cfg(pop_size=20, max_generations=6, seed=11 + j, early_stopping=0)
        alone = gd.run_ga([cx], c1, gd.GD_PREC_F32, use_graph=True, ctx=ctx)
        np.testing.assert_array_equal(alone.genes[0], mix.genes[j])
        assert alone.energies[0].tobytes() == mix.energies[j].tobytes()
        np.testing.assert_array_equal(alone.history[0], mix.history[j])


def hof_list(recs):
    return [(tuple(r["genes"].tolist()), float(r["fitness"]), int(r["generation"])) for r in recs]


@pytest.mark.parametrize("early,cap,top_k,pop", [(False, 500, 10, 24), (True, 500, 10, 24), (False, 7, 3, 24),
                                                 (False, 40, 10, 24), (False, 90, 60, 300), (False, 500, 300, 300)])
def test_ga_hall_of_fame_matches_oracle(oracle, early, cap, top_k, pop):
    # plain FP64: the device Hall of Fame equals the oracle's HallOfFame fed
    # with the same populations, entry for entry and in order (small caps
    # exercise the prune, src/commands/run.rs:174-179; populations over 256
    # and top_k over 32 exercise several pre-check rounds per generation)
    c, lig = setup_job(30, 36, 4, seed=79)
    cfg = _lib.ga_default_cfg(pop_size=pop, max_generations=14 if not early else 40, seed=6,
                              early_stopping=1 if early else 0, convergence_window=3, convergence_threshold=0.01,
                              hof_max_size=cap, hof_top_k=top_k)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    res = gd.run_ga([cx], cfg, gd.GD_PREC_F64, use_graph=False, hall_of_fame=True)
    draws = _lib.ga_draw(cfg, cfg.seed, cfg.max_generations)
    hof = oracle.HallOfFame(max_size=cap, top_k=top_k)
    genes, _, gens, _ = oracle.run_ga(c.receptor, lig, c.restraint_pairs, cfg, draws, hof=hof)
    np.testing.assert_array_equal(res.genes[0], genes)
    got = hof_list(res.hall_of_fame[0])
    assert len(got) == len(hof.entries) <= cap
    assert [(g, gen) for g, _, gen in got] == [(g, gen) for g, _, gen in hof.entries]
    np.testing.assert_allclose([x[1] for x in got], [x[1] for x in hof.entries], rtol=1e-12)


def test_ga_hall_of_fame_fp32_graph_invariants(oracle):
    # FP32 graph form, several jobs: every job's entries are pairwise
    # dissimilar, at most hof_max_size, each at most top_k per generation,
    # and the mix equals each job alone
    jobs = [setup_job(25, 20, 3, 111), setup_job(60, 45, 6, 112)]
    ctx = gd.Context(0)
    cxs = [gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx) for c, lig in jobs]
    cfg = _lib.ga_default_cfg(pop_size=32, max_generations=12, seed=21, early_stopping=0, hof_max_size=30,
                              hof_top_k=4)
    mix = gd.run_ga(cxs, cfg, gd.GD_PREC_F32, use_graph=True, ctx=ctx, hall_of_fame=True)
    sim = oracle.HallOfFame().genes_are_similar
    for j, cx in enumerate(cxs):
        h = hof_list(mix.hall_of_fame[j])
        assert 0 < len(h) <= 30
        for a in range(len(h)):
            for b in range(a + 1, len(h)):
                assert not sim(h[a][0], h[b][0])
        per_gen = np.bincount([x[2] for x in h])
        assert per_gen.max() <= 4
        c1 = _lib.ga_default_cfg(pop_size=32, max_generations=12, seed=21 + j, early_stopping=0, hof_max_size=30,
                                 hof_top_k=4)
        alone = gd.run_ga([cx], c1, gd.GD_PREC_F32, use_graph=True, ctx=ctx, hall_of_fame=True)
        assert alone.hall_of_fame[0].tobytes() == mix.hall_of_fame[j].tobytes()


@pytest.mark.parametrize("prec,graph", [(gd.GD_PREC_F64, False), (gd.GD_PREC_F32, True)])
def test_ga_dockq_every_generation(oracle, prec, graph):
    # the metrics of every generation's best pose and the mean DockQ, on the
    # device inside the GA, against the oracle's evaluator run on the same
    # populations (FP64: the populations are the oracle's bit for bit; FP32:
    # the device populations are re-evaluated by the oracle)
    import dataclasses
    c, lig = setup_job(30, 36, 4, seed=80)
    reference = dataclasses.replace(lig, x=lig.x + 1.5)
    cfg = _lib.ga_default_cfg(pop_size=24, max_generations=10, seed=8, early_stopping=0)
    ctx = gd.Context(0)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
    other = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
    ev = gd.Evaluator(cx, reference)
    res = gd.run_ga([cx, other], cfg, prec, use_graph=graph, ctx=ctx, evaluators=[ev, None])
    assert np.isnan(res.mean_dockq[1]).all()  # the job without an evaluator
    oev = oracle.Evaluator(c.receptor, reference)
    assert len(oev.native_contacts) > 0
    if prec == gd.GD_PREC_F64:
        draws = _lib.ga_draw(cfg, cfg.seed, cfg.max_generations)
        out = []
        oracle.run_ga(c.receptor, lig, c.restraint_pairs, cfg, draws, evaluator=oev, metrics_out=out)
        ref_best = np.array([b for b, _ in out])
        ref_mean = np.array([m for _, m in out])
        got = np.stack([res.best_metrics[0][k] for k in ("rmsd", "irmsd", "fnat", "dockq")], axis=1)
        # device frames use CUDA sincos: coordinates agree to a few ulp
        np.testing.assert_allclose(got, ref_best, rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(res.mean_dockq[0], ref_mean, rtol=1e-9)
    else:
        assert np.isfinite(res.mean_dockq[0]).all()
        assert ((res.best_metrics[0]["dockq"] > 0) & (res.best_metrics[0]["dockq"] <= 1)).all()
