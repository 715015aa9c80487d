"""Contacts and FCC clustering at the large-complex size against the oracle,
and the automatic choice between the two device pair counts.

The large-complex workload is a receptor of 2,000 residues (~16,800 atoms)
and a ligand of 500 (~4,200 atoms).  A sample of 192 of its poses (most of
them around four seeds, so that clusters form) has its contacts computed by
the oracle on all host threads; the device's contacts (both contact kernels)
and clusters (both FCC pair counts) must be identical
(src/clustering.rs:62-293).
"""
import numpy as np
import pytest

import gdock_gb300 as gd
from gdock_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def large():
    c = synth.make_complex(2000, 500, 30, seed=5)
    lig = gd.position_ligand(c.receptor, c.ligand)
    rng = np.random.default_rng(77)
    seeds = synth.random_genes(rng, 4, max_displacement=18.0)
    g = seeds[rng.integers(0, 4, 160)].copy()
    g[:, :3] = np.mod(g[:, :3] + rng.normal(0.0, 0.03, (160, 3)), 2 * np.pi)
    g[:, 3:] += rng.normal(0.0, 0.4, (160, 3))
    genes = np.concatenate([g, synth.random_genes(rng, 32, max_displacement=30.0)])
    return c, lig, genes


def test_large_complex_contacts_and_clusters(oracle, large):
    c, lig, genes = large
    sets = oracle.pose_contacts_many(c.receptor, lig, genes)
    assert sum(len(s) > 0 for s in sets) > 150
    ctx = gd.Context(0)
    try:
        cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
        for mode, kernel in ((0, 2), (1, 1)):
            ctx.set_tuning(_lib.GD_TUNE_CONTACTS, mode)
            got = cx.pose_contacts(genes)
            assert ctx.get_tuning(_lib.GD_INFO_LAST_CONTACTS) == kernel
            for i, (a, b) in enumerate(zip(got, sets)):
                np.testing.assert_array_equal(a, b, err_msg=f"pose {i}, contact pass {kernel}")
        for fcc in (1, 2, 0):
            ctx.set_tuning(_lib.GD_TUNE_FCC, fcc)
            for ms in (1, 4):
                want = oracle.cluster(sets, min_size=ms)
                got = cx.cluster(genes, gd.ClusteringConfig(min_cluster_size=ms))
                assert [(r.center_idx, r.members) for r in got] == want, (fcc, ms)
                assert ctx.get_tuning(_lib.GD_INFO_LAST_FCC) == (fcc or 1)  # bitsets at this size
            assert max(len(m) for _, m in want) >= 4
        cx.close()
    finally:
        ctx.close()


def test_automatic_postings_and_budget_fallback():
    """16,384 poses drawn as gdock draws its genes (angles in [0, 2pi),
    displacements in [-50, 50]^3) on the single-complex workload: contacts
    spread over most residue pairs, each pose with few of them, so the
    automatic choice counts common contacts by postings.  With an HBM budget
    that holds the bitsets but not the n x n posting counts, the call falls
    back to the bitsets, succeeds without an error message, and gives the same
    clusters; so does forcing the bitsets."""
    c = synth.make_complex(300, 150, 12, seed=2026)
    lig = gd.position_ligand(c.receptor, c.ligand)
    genes = synth.random_genes(np.random.default_rng(8), 16384, max_displacement=50.0)
    cfg = gd.ClusteringConfig(min_cluster_size=1)
    ctx = gd.Context(0)
    try:
        cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
        auto = [(r.center_idx, r.members) for r in cx.cluster(genes, cfg)]
        assert ctx.get_tuning(_lib.GD_INFO_LAST_FCC) == 2
        ctx.set_tuning(_lib.GD_TUNE_FCC, 1)
        assert [(r.center_idx, r.members) for r in cx.cluster(genes, cfg)] == auto
        assert ctx.get_tuning(_lib.GD_INFO_LAST_FCC) == 1
        resident = ctx.bytes_in_use
        cx.close()
    finally:
        ctx.close()
    # counts: 16,384^2 x 4 B = 1 GiB; bitsets: ~90 MB of compacted words
    # plus a 32 MiB adjacency matrix
    budget = resident + (320 << 20)
    ctx = gd.Context(0, hbm_budget_bytes=budget)
    try:
        cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
        got = [(r.center_idx, r.members) for r in cx.cluster(genes, cfg)]
        assert ctx.get_tuning(_lib.GD_INFO_LAST_FCC) == 1
        assert ctx.lib.gd_last_error(ctx.h).decode() == ""
        assert got == auto
        assert ctx.bytes_in_use <= budget
        cx.close()
    finally:
        ctx.close()
