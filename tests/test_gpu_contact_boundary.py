"""Contact decisions at the 5 A cutoff, decided within a few ulps.

gdock counts a residue contact when any atom pair has ``distance <= 5.0``
(src/clustering.rs:95-104, ``dist <= contact_distance``).  The device makes
that decision on the exact FP64 squared distance against the largest d2 whose
square root is <= 5 (the per-residue lists, k_contacts_rl), or in FP32 with a
guard band whose pairs are re-decided in FP64 (the contact bitmaps,
k_contact_bits).  Here ligand atoms sit at 5 * (1 + k * 2^-52) A from a
receptor atom, k in {-3, -1, 0, 1, 3}, along several directions, each in a
residue of its own, so that every single pair decision shows in the keys.

The ligand is built of mirrored pairs (p, -p) in that order, so its centroid
sums to exactly 0 and the identity pose leaves every coordinate unchanged:
the oracle and the device then see exactly the distances placed here.
"""
import numpy as np
import pytest

import gdock_gb300 as gd
from gdock_gb300 import _lib
from conftest import make_mol, tatom

pytestmark = pytest.mark.gpu

KS = (-3, -1, 0, 1, 3)
DIRS = [(1, 0, 0), (0, 1, 0), (0, 0, 1), (-1, 0, 0), (0.6, 0.8, 0), (0, -0.8, 0.6),
        (1 / 3, 2 / 3, 2 / 3), (2 / 7, -3 / 7, 6 / 7), (-0.48, 0.6, 0.64), (0.1, 0.2, np.sqrt(0.95))]


def boundary_ligand(center=(0.0, 0.0, 0.0)):
    """Ligand atoms at 5(1 + k 2^-52) from `center` (one residue each), each
    followed by its mirror image through the origin (a residue of its own)."""
    pts = []
    for u in DIRS:
        u = np.asarray(u, dtype=np.float64)
        u /= np.linalg.norm(u)
        for k in KS:
            d = 5.0 * (1.0 + k * 2.0 ** -52)
            pts.append(np.asarray(center) + d * u)
    atoms = []
    for i, p in enumerate(pts):
        for s, q in ((1, p), (-1, -p)):
            atoms.append(tatom(*q, "C", name="CB", resseq=len(atoms) + 1, serial=1000 + len(atoms), chain="B"))
    return make_mol(atoms), np.array(pts)


def exact_distances(rec, pts):
    """The reference's distance, sqrt((dx*dx + dy*dy) + dz*dz), per point to
    the receptor's first atom."""
    dx, dy, dz = pts[:, 0] - rec.x[0], pts[:, 1] - rec.y[0], pts[:, 2] - rec.z[0]
    return np.sqrt((dx * dx + dy * dy) + dz * dz)


def check_spread(d):
    """The placed distances straddle the cutoff: some at exactly 5, some a
    few ulps on either side."""
    ulp = np.spacing(5.0)
    assert np.any(d == 5.0)
    assert np.any((d > 5.0) & (d <= 5.0 + 8 * ulp))
    assert np.any((d < 5.0) & (d >= 5.0 - 8 * ulp))


def contacts_all_paths(oracle, rec, lig, genes, paths):
    ctx = gd.Context(0)
    try:
        cx = gd.Complex(rec, lig, [], ctx=ctx)
        want = [oracle.pose_contacts(rec, lig, g) for g in genes]
        for mode, kernel in paths:
            ctx.set_tuning(_lib.GD_TUNE_CONTACTS, mode)
            got = cx.pose_contacts(genes)
            assert ctx.get_tuning(_lib.GD_INFO_LAST_CONTACTS) == kernel, (mode, kernel)
            for a, b in zip(got, want):
                np.testing.assert_array_equal(a, b, err_msg=f"contact pass {kernel}")
        cx.close()
    finally:
        ctx.close()
    return want


def test_single_chain_boundary_pairs_both_kernels(oracle):
    """Single-chain receptor and ligand: the bitmap kernel (FP32 + FP64 guard
    re-decisions) and the list kernel (exact FP64) against the oracle."""
    rec = make_mol([tatom(0.0, 0.0, 0.0, "C", name="CA", resseq=1, serial=1, chain="A")])
    lig, pts = boundary_ligand()
    check_spread(exact_distances(rec, pts))
    genes = np.zeros((3, 6))
    genes[2, 3] = 100.0  # one pose far away: no contact at all
    want = contacts_all_paths(oracle, rec, lig, genes, [(0, 2), (1, 1)])
    n_in = len(want[0])
    # every ligand residue within 5 A of the receptor atom is a contact: the
    # mirrored points are the same distances, so twice the points at <= 5
    d = exact_distances(rec, pts)
    assert n_in == 2 * int(np.sum(d <= 5.0)) and 0 < n_in < 2 * len(pts)
    assert len(want[2]) == 0


def test_multi_chain_receptor_boundary_pairs(oracle):
    """A receptor of two chains takes the per-residue list path (and adds its
    own inter-chain contacts): the same boundary decisions."""
    rec = make_mol([tatom(0.0, 0.0, 0.0, "C", name="CA", resseq=1, serial=1, chain="A"),
                    tatom(0.0, 0.0, 60.0, "C", name="CA", resseq=2, serial=2, chain="C"),
                    tatom(0.0, 0.0, 64.0, "N", name="N", resseq=3, serial=3, chain="A")])
    lig, pts = boundary_ligand()
    check_spread(exact_distances(rec, pts))
    genes = np.zeros((2, 6))
    want = contacts_all_paths(oracle, rec, lig, genes, [(0, 1)])
    assert len(want[0]) > 1  # includes the receptor's own A-C contact at 4 A


def test_boundary_away_from_the_origin(oracle):
    """The same placement around a receptor atom at (31.25, -17.5, 12.0): the
    differences of the coordinates now round, so the distances land on other
    sides of the cutoff; whatever they are, both kernels agree with the
    oracle."""
    c = (31.25, -17.5, 12.0)
    rec = make_mol([tatom(*c, "O", name="O", resseq=7, serial=1, chain="A"),
                    tatom(-30.0, 20.0, -10.0, "C", name="CA", resseq=8, serial=2, chain="A")])
    lig, pts = boundary_ligand(center=c)
    d = exact_distances(rec, pts)
    assert np.all(np.abs(d - 5.0) < 1e-13)
    contacts_all_paths(oracle, rec, lig, np.zeros((1, 6)), [(0, 2), (1, 1)])


@pytest.mark.parametrize("fcc_mode", [1, 2])
def test_cluster_on_boundary_contacts(oracle, fcc_mode):
    """gd_cluster on the boundary geometry and on its variant with a
    two-chain receptor (contact bitmaps both, then both FCC pair counts): the
    oracle's clusters of the oracle's contact sets."""
    rec1 = make_mol([tatom(0.0, 0.0, 0.0, "C", name="CA", resseq=1, serial=1, chain="A")])
    rec2 = make_mol([tatom(0.0, 0.0, 0.0, "C", name="CA", resseq=1, serial=1, chain="A"),
                     tatom(0.0, 0.0, 60.0, "C", name="CA", resseq=2, serial=2, chain="C")])
    lig, _ = boundary_ligand()
    genes = np.zeros((9, 6))
    genes[6:, 3] = (100.0, 200.0, 300.0)  # empty contact sets
    for rec, kernel in ((rec1, 2), (rec2, 2)):
        ctx = gd.Context(0)
        try:
            ctx.set_tuning(_lib.GD_TUNE_FCC, fcc_mode)
            cx = gd.Complex(rec, lig, [], ctx=ctx)
            sets = [oracle.pose_contacts(rec, lig, g) for g in genes]
            for ms in (1, 4):
                got = cx.cluster(genes, gd.ClusteringConfig(min_cluster_size=ms))
                assert ctx.get_tuning(_lib.GD_INFO_LAST_CONTACTS) == kernel
                assert [(r.center_idx, r.members) for r in got] == oracle.cluster(sets, min_size=ms)
            cx.close()
        finally:
            ctx.close()


def test_hydrogens_make_no_contacts(oracle):
    """calculate_contacts skips atoms whose element is H (src/clustering.rs:
    67-70): hydrogens 3 A apart across the chains, or 3 A from a heavy atom,
    make no contact; a heavy pair at 4 A does.  Both contact kernels."""
    rec = make_mol([tatom(0.0, 0.0, 0.0, "C", name="CA", resseq=1, serial=1, chain="A"),
                    tatom(0.0, 0.0, 20.0, "H", name="HA", resseq=2, serial=2, chain="A"),
                    tatom(0.0, 30.0, 0.0, "N", name="N", resseq=3, serial=3, chain="A")])
    lig = make_mol([tatom(0.0, 0.0, 23.0, "H", name="H", resseq=1, serial=11, chain="B"),
                    tatom(4.0, 0.0, 0.0, "C", name="CB", resseq=2, serial=12, chain="B"),
                    tatom(-3.0, 0.0, 0.0, "H", name="HB", resseq=3, serial=13, chain="B"),
                    tatom(0.0, 27.0, 0.0, "H", name="H2", resseq=4, serial=14, chain="B")])
    genes = np.zeros((2, 6))
    genes[1, 3] = 0.5
    want = contacts_all_paths(oracle, rec, lig, genes, [(0, 2), (1, 1)])
    for keys in want:
        assert keys.tolist() == [oracle.contact_key("A", 1, "B", 2)]


def two_chain_ligand(half):
    """Two ligand atoms on chains B and D at (0, 0, +-half): mirrored, so the
    centroid is exactly 0 and the identity pose keeps their distance 2 * half."""
    return make_mol([tatom(0.0, 0.0, half, "C", name="CB", resseq=1, serial=101, chain="B"),
                     tatom(0.0, 0.0, -half, "C", name="CB", resseq=1, serial=102, chain="D")])


def test_cluster_ligand_chains_constant_or_per_pose(oracle):
    """A two-chain ligand's own inter-chain contact is in every pose's set.
    Far from the cutoff (4 A) it is a constant and the device path clusters;
    at exactly 5 A the FP64 rounding of a pose's transform can put it on
    either side, so the per-pose host path decides it (contact lists).  Both
    give the oracle's clusters."""
    rng = np.random.default_rng(5)
    genes = np.zeros((12, 6))
    genes[:, :3] = rng.uniform(0.0, 2 * np.pi, (12, 3))
    genes[1:, 3:] = rng.normal(0.0, 0.4, (11, 3))
    rec = make_mol([tatom(0.0, 0.0, 6.5, "C", name="CA", resseq=1, serial=1, chain="A"),
                    tatom(0.0, 0.0, -6.5, "N", name="N", resseq=2, serial=2, chain="A")])
    for half, kernel in ((2.0, 2), (2.5, 1)):
        lig = two_chain_ligand(half)
        ctx = gd.Context(0)
        try:
            cx = gd.Complex(rec, lig, [], ctx=ctx)
            sets = [oracle.pose_contacts(rec, lig, g) for g in genes]
            got = cx.cluster(genes, gd.ClusteringConfig(min_cluster_size=1))
            assert ctx.get_tuning(_lib.GD_INFO_LAST_CONTACTS) == kernel, half
            assert [(r.center_idx, r.members) for r in got] == oracle.cluster(sets, min_size=1), half
            cx.close()
        finally:
            ctx.close()
