"""Known-answer tests of the oracle's HallOfFame against the assertions of
gdock's own tests (src/commands/run.rs:915-1033)."""
import math

import pytest


@pytest.fixture
def HoF(oracle):
    return oracle.HallOfFame


def test_new(HoF):  # src/commands/run.rs:915-919
    assert len(HoF().entries) == 0


def test_add_entry(HoF):  # :922-929
    h = HoF()
    assert h.try_add([0.0] * 6, -100.0, 1)
    assert len(h.entries) == 1


def test_rejects_duplicates(HoF):  # :932-941
    h = HoF()
    h.try_add([0.0] * 6, -100.0, 1)
    assert not h.try_add([0.0] * 6, -100.0, 2)
    assert len(h.entries) == 1


def test_accepts_different_genes(HoF):  # :944-956
    h = HoF()
    h.try_add([0.0] * 6, -100.0, 1)
    assert h.try_add([math.pi, math.pi, math.pi, 0.0, 0.0, 0.0], -90.0, 2)
    assert len(h.entries) == 2


def test_accepts_different_translations(HoF):  # :959-971
    h = HoF()
    h.try_add([0.0] * 6, -100.0, 1)
    assert h.try_add([0.0, 0.0, 0.0, 10.0, 10.0, 10.0], -90.0, 2)
    assert len(h.entries) == 2


def test_rejects_similar_genes(HoF):  # :974-986
    h = HoF()
    h.try_add([0.0] * 6, -100.0, 1)
    assert not h.try_add([0.1, 0.1, 0.1, 0.5, 0.5, 0.5], -90.0, 2)
    assert len(h.entries) == 1


def test_prune_keeps_best(HoF):  # :989-1013
    h = HoF(max_size=3)
    for i in range(5):
        h.try_add([float(i), 0.0, 0.0, i * 10.0, 0.0, 0.0], -(100.0 - i * 10.0), i)
    assert len(h.entries) == 3
    f = [e[1] for e in h.entries]
    assert f[0] <= f[1] <= f[2]
    assert f == [-100.0, -90.0, -80.0]


def test_angular_difference(HoF):  # :1016-1033
    assert abs(HoF.angular_difference(0.0, 0.0)) < 0.001
    assert HoF.angular_difference(0.0, 2.0 * math.pi - 0.1) < 0.2
    assert abs(HoF.angular_difference(0.0, math.pi) - math.pi) < 0.001


def test_add_from_population_top_k_and_order(HoF):  # :193-213
    h = HoF(top_k=2)
    genes = [[0.0] * 6, [0.05] * 6, [1.0, 0, 0, 0, 0, 0], [2.0, 0, 0, 0, 0, 0]]
    fitness = [-3.0, -5.0, -1.0, -5.0]  # stable order: 1, 3, 0, 2
    h.add_from_population(genes, fitness, 0)
    assert [e[0][0] for e in h.entries] == [0.05, 2.0]
    h.add_from_population(genes, fitness, 1)  # 1 and 3 now duplicates: 0 is similar to 1, so 2 goes in
    assert [e[0][0] for e in h.entries] == [0.05, 2.0, 1.0]
