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


@pytest.mark.parametrize("mode", [1, 2])
def test_cluster_sets_both_pair_counts(oracle, mode):
    """gd_cluster_sets counts common contacts with bitsets or with postings
    built on the host (GD_TUNE_FCC): the oracle's clusters either way, for
    dense groups, spread-out sets and empty ones."""
    from gdock_gb300 import _lib
    ctx = gd.Context(0)
    try:
        ctx.set_tuning(_lib.GD_TUNE_FCC, mode)
        rng = np.random.default_rng(90 + mode)
        protos = [np.unique(rng.integers(0, 5000, 80)) for _ in range(4)]
        sets = []
        for k in range(260):
            if k % 13 == 0:
                sets.append(np.zeros(0, np.int64))
            elif k < 200:
                base = protos[k % 4]
                sets.append(np.unique(np.concatenate([base[rng.random(base.size) > 0.15],
                                                      rng.integers(0, 5000, 4)])).astype(np.int64))
            else:
                sets.append(np.unique(rng.integers(0, 200000, int(rng.integers(1, 60)))).astype(np.int64))
        for ms in (1, 4):
            got = gd.cluster_sets(sets, gd.ClusteringConfig(min_cluster_size=ms), ctx=ctx)
            assert ctx.get_tuning(_lib.GD_INFO_LAST_FCC) == mode
            assert [(r.center_idx, r.members) for r in got] == oracle.cluster(sets, min_size=ms), ms
        cfg = gd.ClusteringConfig(fcc_cutoff=0.3, strictness=0.5, min_cluster_size=1)
        got = gd.cluster_sets(sets, cfg, ctx=ctx)
        assert [(r.center_idx, r.members) for r in got] == oracle.cluster(sets, fcc_cutoff=0.3, strictness=0.5,
                                                                          min_size=1)
        # over 65,536 keys: the host side runs on several threads
        big = [np.unique(np.concatenate([protos[k % 4][rng.random(protos[k % 4].size) > 0.2],
                                         rng.integers(0, 50000, 8)])).astype(np.int64) for k in range(1100)]
        assert sum(len(b) for b in big) > 65536
        got = gd.cluster_sets(big, gd.ClusteringConfig(min_cluster_size=4), ctx=ctx)
        assert [(r.center_idx, r.members) for r in got] == oracle.cluster(big, min_size=4)
    finally:
        ctx.close()


def test_multichain_pose_contacts_many_poses(oracle):
    """Per-pose contact keys of a two-chain receptor and a two-chain ligand
    over 300 poses (the host builds the keys on several threads from 256
    poses up): each pose's keys are the oracle's."""
    c = synth.make_complex(40, 30, 3, seed=12)
    rec, lig0 = c.receptor, c.ligand
    rec = gd.Molecule(**{**rec.__dict__, "chainid": ["A" if i < len(rec) // 2 else "C" for i in range(len(rec))]})
    lig0 = gd.Molecule(**{**lig0.__dict__, "chainid": ["B" if i < len(lig0) // 2 else "D" for i in range(len(lig0))]})
    lig = gd.position_ligand(rec, lig0)
    genes = near_genes(np.random.default_rng(13), 300, 2.0)
    cx = gd.Complex(rec, lig, c.restraint_pairs)
    got = cx.pose_contacts(genes)
    assert len(got) == 300
    for g, keys in zip(genes, got):
        np.testing.assert_array_equal(keys, oracle.pose_contacts(rec, lig, g))
