"""GPU parity of contacts and FCC clustering: bit-exact against the oracle."""
import numpy as np
import pytest

import gdock_gb300 as gd
from gdock_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    c = synth.make_complex(50, 76, 6, seed=21)
    lig = gd.position_ligand(c.receptor, c.ligand)
    return c, lig


def near_genes(rng, n, spread):
    """Poses around a few seeds so that clusters exist."""
    base = synth.random_genes(rng, 4, max_displacement=12.0)
    g = base[rng.integers(0, 4, n)].copy()
    g[:, :3] = np.mod(g[:, :3] + rng.normal(0, 0.05 * spread, (n, 3)), 2 * np.pi)
    g[:, 3:] += rng.normal(0, 0.5 * spread, (n, 3))
    return g


def test_contacts_bit_exact(oracle, setup):
    c, lig = setup
    genes = near_genes(np.random.default_rng(0), 24, 1.0)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    got = cx.pose_contacts(genes)
    n_nonempty = 0
    for g, keys in zip(genes, got):
        ref = oracle.pose_contacts(c.receptor, lig, g)
        np.testing.assert_array_equal(keys, ref)
        n_nonempty += len(ref) > 0
    assert n_nonempty > 0


def test_cluster_matches_oracle(oracle, setup):
    c, lig = setup
    rng = np.random.default_rng(1)
    genes = near_genes(rng, 60, 1.0)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    sets = [oracle.pose_contacts(c.receptor, lig, g) for g in genes]
    want = oracle.cluster(sets)
    got = cx.cluster(genes)
    assert [(r.center_idx, r.members) for r in got] == want
    assert all(r.size == len(r.members) for r in got)
    got2 = gd.cluster_sets(sets)
    assert [(r.center_idx, r.members) for r in got2] == want
    for ms in (1, 2):
        cfg = gd.ClusteringConfig(min_cluster_size=ms)
        assert [(r.center_idx, r.members) for r in gd.cluster_sets(sets, cfg)] == oracle.cluster(sets, min_size=ms)


def test_cluster_edge_cases(oracle):
    assert gd.cluster_sets([]) == []
    s = [np.array([], np.int64)] * 5
    got = gd.cluster_sets(s, gd.ClusteringConfig(min_cluster_size=1))
    assert [(r.center_idx, r.members) for r in got] == oracle.cluster(s, min_size=1)
    rng = np.random.default_rng(3)
    for trial in range(5):
        n = int(rng.integers(2, 140))
        u = rng.integers(1, 200)
        sets = [np.unique(rng.integers(0, u, int(rng.integers(0, 30))).astype(np.int64)) for _ in range(n)]
        for ms in (1, 4):
            cfg = gd.ClusteringConfig(min_cluster_size=ms)
            got = [(r.center_idx, r.members) for r in gd.cluster_sets(sets, cfg)]
            assert got == oracle.cluster(sets, min_size=ms), trial


def test_cluster_large_dense_groups(oracle):
    """Groups of near-identical contact sets give clusters larger than a row
    of the adjacency bit matrix (the popcount update) next to small ones."""
    rng = np.random.default_rng(11)
    protos = [np.unique(rng.integers(0, 400, 60)) for _ in range(3)]
    sets = []
    for k in range(330):
        base = protos[k % 3] if k < 300 else np.unique(rng.integers(0, 400, int(rng.integers(0, 40))))
        keep = base[rng.random(base.size) > 0.1]
        extra = rng.integers(0, 400, 3)
        sets.append(np.unique(np.concatenate([keep, extra])).astype(np.int64))
    for ms in (1, 4, 50):
        cfg = gd.ClusteringConfig(min_cluster_size=ms)
        got = [(r.center_idx, r.members) for r in gd.cluster_sets(sets, cfg)]
        assert got == oracle.cluster(sets, min_size=ms), ms
    assert max(len(m) for _, m in got) > 330 // 32


def test_multichain_receptor_contacts(oracle):
    """A receptor of two chains: receptor-only inter-chain contacts count in
    every pose's set (src/clustering.rs:82-91)."""
    c = synth.make_complex(40, 30, 3, seed=8)
    rec = c.receptor
    chains = ["A" if i < len(rec) // 2 else "C" for i in range(len(rec))]
    rec = gd.Molecule(**{**rec.__dict__, "chainid": chains})
    lig = gd.position_ligand(rec, c.ligand)
    genes = near_genes(np.random.default_rng(4), 8, 1.0)
    cx = gd.Complex(rec, lig, c.restraint_pairs)
    got = cx.pose_contacts(genes)
    for g, keys in zip(genes, got):
        np.testing.assert_array_equal(keys, oracle.pose_contacts(rec, lig, g))


@pytest.mark.parametrize("mode", [1, 2])
def test_cluster_device_fcc_paths(oracle, setup, mode):
    """Both ways of counting common contacts on the device (GD_TUNE_FCC:
    bitsets, contact postings) give the oracle's clusters, from converged to
    spread-out poses and at extreme cutoffs."""
    from gdock_gb300 import _lib
    c, lig = setup
    ctx = gd.Context(0)
    ctx.set_tuning(_lib.GD_TUNE_FCC, mode)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
    rng = np.random.default_rng(40 + mode)
    for spread in (0.3, 1.0, 6.0):
        genes = near_genes(rng, 80, spread)
        sets = [oracle.pose_contacts(c.receptor, lig, g) for g in genes]
        for ms in (1, 4):
            got = cx.cluster(genes, gd.ClusteringConfig(min_cluster_size=ms))
            assert [(r.center_idx, r.members) for r in got] == oracle.cluster(sets, min_size=ms), (spread, ms)
        for cut, strict in ((0.0, 0.75), (1.0, 1.0), (0.3, 0.5)):
            cfg = gd.ClusteringConfig(fcc_cutoff=cut, strictness=strict, min_cluster_size=1)
            got = cx.cluster(genes, cfg)
            want = oracle.cluster(sets, fcc_cutoff=cut, strictness=strict, min_size=1)
            assert [(r.center_idx, r.members) for r in got] == want, (spread, cut, strict)


@pytest.mark.parametrize("mode", [1, 2])
def test_multichain_cluster_on_device(oracle, mode):
    """Receptor and ligand of two chains each: the device clusters them (the
    contact bitmaps for receptor-ligand pairs, the inter-chain contacts within
    each molecule as a count every pose shares) and gives the oracle's
    clusters of the oracle's contact sets, with both ways of counting common
    contacts (GD_TUNE_FCC)."""
    from gdock_gb300 import _lib
    c = synth.make_complex(40, 30, 3, seed=8)
    rec, lig0 = c.receptor, c.ligand
    rec = gd.Molecule(**{**rec.__dict__, "chainid": ["A" if i < len(rec) // 2 else "C" for i in range(len(rec))]})
    lig0 = gd.Molecule(**{**lig0.__dict__, "chainid": ["B" if i < len(lig0) // 2 else "D" for i in range(len(lig0))]})
    lig = gd.position_ligand(rec, lig0)
    ctx = gd.Context(0)
    try:
        ctx.set_tuning(_lib.GD_TUNE_FCC, mode)
        cx = gd.Complex(rec, lig, c.restraint_pairs, ctx=ctx)
        rng = np.random.default_rng(70 + mode)
        for spread in (0.3, 1.0, 4.0):
            genes = near_genes(rng, 60, spread)
            sets = [oracle.pose_contacts(rec, lig, g) for g in genes]
            for ms in (1, 4):
                got = cx.cluster(genes, gd.ClusteringConfig(min_cluster_size=ms))
                assert ctx.get_tuning(_lib.GD_INFO_LAST_CONTACTS) == 2  # the bitmap kernel ran
                assert ctx.get_tuning(_lib.GD_INFO_LAST_FCC) == mode
                assert [(r.center_idx, r.members) for r in got] == oracle.cluster(sets, min_size=ms), (spread, ms)
        cx.close()
    finally:
        ctx.close()
