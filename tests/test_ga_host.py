"""Host-side GA pieces (no GPU): the seeded draws and the oracle's evolve,
checked against the properties the reference's GA tests assert
(src/population.rs:423-530, src/ga.rs:61-191, src/chromosome.rs:160-250)."""
import math

import numpy as np
import pytest

from gdock_gb300 import _lib


@pytest.fixture(scope="module")
def cfg():
    return _lib.ga_default_cfg(pop_size=20, max_generations=4)


def test_draws_are_deterministic_and_in_range(cfg):
    a = _lib.ga_draw(cfg, 42, 4)
    b = _lib.ga_draw(cfg, 42, 4)
    c = _lib.ga_draw(cfg, 43, 4)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    assert not np.array_equal(a["init"], c["init"])
    init = a["init"]
    assert ((init[:, :3] >= 0) & (init[:, :3] <= 2 * math.pi)).all()  # src/chromosome.rs:28-30
    assert ((init[:, 3:] >= -50) & (init[:, 3:] <= 50)).all()           # :32-34
    assert ((a["tour"] >= 0) & (a["tour"] < 20)).all()
    for g in range(4):
        assert sorted(a["perm"][g].tolist()) == list(range(20))
    assert ((a["cross_u"] >= 0) & (a["cross_u"] < 1)).all()
    trig = a["mut_u"] <= 0.1
    assert (a["mut_z"][~trig] == 0).all() and (a["mut_z"][trig] != 0).all()


def test_evolve_preserves_size_and_elites(oracle, cfg):  # src/population.rs:470-530
    d = _lib.ga_draw(cfg, 42, 1)
    genes = d["init"]
    fit = np.arange(20) * 5.0
    go, fo = oracle.evolve(genes, fit, d, 0)
    assert go.shape == (20, 6)
    for e in range(5):  # the five best individuals survive with their genes
        assert any(np.array_equal(go[i], genes[e]) for i in range(20))
        assert e * 5.0 in fo[:5]


def test_evolve_elites_first_and_sorted_rest(oracle, cfg):
    d = _lib.ga_draw(cfg, 7, 1)
    rng = np.random.default_rng(0)
    fit = rng.normal(size=20)
    go, fo = oracle.evolve(d["init"], fit, d, 0)
    order = np.argsort(fit, kind="stable")[:5]
    np.testing.assert_array_equal(fo[:5], fit[order])
    assert (np.diff(fo[5:]) <= 0).all()  # the rest: descending carried fitness


def test_crossover_complementary_and_bounds(oracle):
    """With no mutation each offspring gene comes from one parent and the
    pair is complementary (src/ga.rs:152-176); with full mutation genes stay
    in bounds (src/chromosome.rs:196-224)."""
    c = _lib.ga_default_cfg(pop_size=2, elitism=0, mutation_rate=0.0)
    d = _lib.ga_draw(c, 42, 1)
    d["tour"][0] = [0, 0, 0, 1, 1, 1]
    d["perm"][0] = [0, 1]
    p = np.array([[1, 2, 3, 4, 5, 6], [7, 8, 9, 10, 11, 12]], float)
    go, fo = oracle.evolve(p, np.array([100.0, 200.0]), d, 0, elitism=0, mutation_rate=0.0)
    kids = sorted(go.tolist())
    for i in range(6):
        assert {kids[0][i], kids[1][i]} == {p[0][i], p[1][i]}
    assert sorted(fo.tolist()) == [100.0, 200.0]  # offspring carry their parents' fitness
    c2 = _lib.ga_default_cfg(pop_size=40, mutation_rate=1.0)
    d2 = _lib.ga_draw(c2, 3, 5)
    genes, fit = d2["init"], np.zeros(40)
    for g in range(5):
        genes, fit = oracle.evolve(genes, fit, d2, g, mutation_rate=1.0)
        assert ((genes[:, :3] >= 0) & (genes[:, :3] <= 2 * math.pi)).all()
        assert ((genes[:, 3:] >= -50) & (genes[:, 3:] <= 50)).all()


def test_ga_close_comparisons_counts(oracle):
    # n = 4, tournament 2: best-of-generation 3 + elitism 3 + tournaments 4 +
    # offspring 3 comparisons; the two equal values and the 1e-12 pair are close
    f = [-10.0, -10.0, -5.0, -5.0 * (1 + 1e-12)]
    tour = [0, 1, 2, 3, 0, 2, 1, 3]
    perm = [0, 1, 2, 3]
    total, ties, close = oracle.ga_close_comparisons(f, tour, perm, tournament=2)
    assert total == 3 + 3 + 4 + 3
    # bookkeeping: (0,1) tie; elitism adjacent: (-10,-10) tie, (-5(1+1e-12), -5) close;
    # tournaments: (0,1) tie, (2,3) close; offspring: winners 0, 3, 0, 1 -> carried
    # -10, -5.000..., -10, -10: two ties
    assert ties == 1 + 1 + 1 + 2 and close == 0 + 1 + 1 + 0
