"""Known-answer tests pinning the CPU oracle to the reference's own tests.

Each test restates an assertion of gdock's in-file unit tests (cited by
file:line) against the oracle, so the oracle is checked before it is used as
the checker for the GPU path.
"""
import math

import numpy as np
import pytest

from conftest import make_mol, tatom


def mols(rec_atoms, lig_atoms):
    return make_mol(rec_atoms), make_mol(lig_atoms)


# --- src/fitness.rs tests ------------------------------------------------------

def test_vdw_far_atoms_zero(oracle):  # src/fitness.rs:357-367
    r, l = mols([tatom(0, 0, 0)], [tatom(20, 0, 0)])
    assert oracle.vdw_energy(r, l) == 0.0


def test_vdw_close_atoms_finite(oracle):  # src/fitness.rs:369-379
    r, l = mols([tatom(0, 0, 0)], [tatom(5, 0, 0)])
    assert math.isfinite(oracle.vdw_energy(r, l))
    # with distinct serials the pair is scored (the reference fixture gives
    # both atoms serial 1, which skips the pair)
    r2, l2 = mols([tatom(0, 0, 0, serial=1)], [tatom(5, 0, 0, serial=2)])
    e = oracle.vdw_energy(r2, l2)
    assert math.isfinite(e) and e < 0.0


def test_vdw_equal_serial_skipped(oracle):  # src/fitness.rs:92
    r, l = mols([tatom(0, 0, 0, serial=7)], [tatom(4, 0, 0, serial=7)])
    assert oracle.vdw_energy(r, l) == 0.0


def test_vdw_very_close_capped(oracle):  # src/fitness.rs:381-393
    for s in (1, 2):
        r, l = mols([tatom(0, 0, 0)], [tatom(1, 0, 0, serial=s)])
        e = oracle.vdw_energy(r, l)
        assert math.isfinite(e) and e <= 500.0


def test_vdw_softcore_value(oracle):
    # hand evaluation of src/fitness.rs:57-70 at r = 3, eps = -0.1 both, Rmin/2 = 2
    r, l = mols([tatom(0, 0, 0, serial=1)], [tatom(3, 0, 0, serial=2)])
    eps = math.sqrt(0.01)
    rmin6 = 4.0 ** 6
    ratio = rmin6 / (3.0 ** 6 + 0.5 * rmin6)
    assert oracle.vdw_energy(r, l) == pytest.approx(eps * (ratio * ratio - 2 * ratio), rel=1e-15)


def test_elec_neutral_zero(oracle):  # src/fitness.rs:395-405
    r, l = mols([tatom(0, 0, 0)], [tatom(5, 0, 0)])
    assert oracle.elec_energy(r, l) == 0.0


def test_elec_opposite_negative(oracle):  # src/fitness.rs:407-421
    r, l = mols([tatom(0, 0, 0, charge=1.0)], [tatom(5, 0, 0, charge=-1.0)])
    e = oracle.elec_energy(r, l)
    assert e < 0.0 and math.isfinite(e)
    assert e == 332.0636 * (1.0 * -1.0) / 25.0


def test_elec_same_positive(oracle):  # src/fitness.rs:423-436
    r, l = mols([tatom(0, 0, 0, charge=1.0)], [tatom(5, 0, 0, charge=1.0)])
    assert oracle.elec_energy(r, l) > 0.0


def test_elec_cutoffs(oracle):  # src/fitness.rs:292 (1 < r < 15, open at both ends)
    for d, nz in ((0.5, False), (1.0, False), (1.5, True), (14.9, True), (15.0, False), (16.0, False)):
        r, l = mols([tatom(0, 0, 0, charge=1.0)], [tatom(d, 0, 0, charge=1.0)])
        assert (oracle.elec_energy(r, l) != 0.0) == nz, d


def _ring(element):
    return [tatom(3.0 * math.cos(i), 3.0 * math.sin(i), 0.0, element) for i in range(15)]


def test_desolv_hydrophobic_negative(oracle):  # src/fitness.rs:438-461
    r, l = mols([tatom(0, 0, 0, "C")], _ring("C"))
    assert oracle.desolv_energy(r, l) < 0.0


def test_desolv_hydrophilic_positive(oracle):  # src/fitness.rs:463-486
    r, l = mols([tatom(0, 0, 0, "O")], _ring("C"))
    assert oracle.desolv_energy(r, l) > 0.0


def test_desolv_value(oracle):
    # receptor O buried by 15 C (burial saturates at 1), each ring C buried by 1 O
    r, l = mols([tatom(0, 0, 0, "O")], _ring("C"))
    rec_term = -(-0.160) * 1.0 * 1.7 * 1.7 * 4.0 * math.pi
    lig_term = -(0.012 * 0.1 * 1.7 * 1.7 * 4.0 * math.pi) * 15
    assert oracle.desolv_energy(r, l) == pytest.approx(rec_term + lig_term, rel=1e-14)


def _ca(x, resseq):
    return tatom(x, 0, 0, name="CA", resseq=resseq)


def test_air_satisfied_zero(oracle):  # src/fitness.rs:488-506
    r, l = mols([_ca(0, 1)], [_ca(5, 10)])
    assert oracle.air_energy([(1, 10)], r, l) == 0.0


def test_air_violated_positive(oracle):  # src/fitness.rs:508-526
    r, l = mols([_ca(0, 1)], [_ca(15, 10)])
    e = oracle.air_energy([(1, 10)], r, l)
    assert e > 0.0 and e == 10.0 * 8.0 * 8.0


def test_satisfaction_ratios(oracle):  # src/fitness.rs:528-607
    r, l = mols([_ca(0, 1)], [_ca(5, 10)])
    assert oracle.satisfaction_ratio([(1, 10)], r, l) == 1.0
    r, l = mols([_ca(0, 1)], [_ca(15, 10)])
    assert oracle.satisfaction_ratio([(1, 10)], r, l) == 0.0
    r, l = mols([], [])
    assert oracle.satisfaction_ratio(np.zeros((0, 2)), r, l) == 0.0
    r, l = mols([_ca(0, 1), _ca(0, 2)], [_ca(5, 10), _ca(15, 11)])
    assert oracle.satisfaction_ratio([(1, 10), (2, 11)], r, l) == 0.5


def test_restraint_boundary_seven_satisfied(oracle):  # src/restraints.rs:173-187
    r, l = mols([_ca(0, 1)], [_ca(7.0, 10)])
    assert oracle.satisfaction_ratio([(1, 10)], r, l) == 1.0
    r, l = mols([_ca(0, 1)], [_ca(10.0, 10)])
    assert oracle.satisfaction_ratio([(1, 10)], r, l) == 0.0


def test_restraints_missing_ca_dropped(oracle):  # src/restraints.rs:64-73
    r, l = mols([_ca(0, 1)], [_ca(5, 10)])
    kept = oracle.kept_restraints([(1, 10), (2, 10), (1, 99)], r, l)
    assert kept.tolist() == [[1, 10]]


# --- transform: src/structure.rs, src/chromosome.rs tests ----------------------

def test_rotate_zero_angles_identity(oracle):  # src/structure.rs:433-444
    lig = make_mol([tatom(1, 0, 0)])
    x, y, z = oracle.apply_genes(lig, [0, 0, 0, 0, 0, 0])
    assert abs(x[0] - 1) < 1e-10 and abs(y[0]) < 1e-10 and abs(z[0]) < 1e-10


def test_rotate_preserves_center(oracle):  # src/structure.rs:446-461
    lig = make_mol([tatom(1, 0, 0), tatom(-1, 0, 0)])
    x, y, z = oracle.apply_genes(lig, [0, 0, math.pi / 2, 0, 0, 0])
    assert abs(x.sum() / 2) < 1e-10 and abs(y.sum() / 2) < 1e-10 and abs(z.sum() / 2) < 1e-10


def test_translation_only(oracle):  # src/chromosome.rs:256-279
    lig = make_mol([tatom(0, 0, 0)])
    x, y, z = oracle.apply_genes(lig, [0, 0, 0, 5, 10, 15])
    assert abs(x[0] - 5) < 1e-6 and abs(y[0] - 10) < 1e-6 and abs(z[0] - 15) < 1e-6


def test_rotation_is_rz_ry_rx(oracle):
    """The matrix of src/structure.rs:96-103 is Rz(alpha) Ry(beta) Rx(gamma)."""
    rng = np.random.default_rng(0)
    pts = rng.normal(size=(5, 3))
    pts -= pts.mean(axis=0)
    lig = make_mol([tatom(*p) for p in pts])
    a, b, g = 0.3, 1.1, 2.5
    x, y, z = oracle.apply_genes(lig, [a, b, g, 0, 0, 0])
    c = np.array(lig.center_of_mass())
    Rz = np.array([[math.cos(a), -math.sin(a), 0], [math.sin(a), math.cos(a), 0], [0, 0, 1]])
    Ry = np.array([[math.cos(b), 0, math.sin(b)], [0, 1, 0], [-math.sin(b), 0, math.cos(b)]])
    Rx = np.array([[1, 0, 0], [0, math.cos(g), -math.sin(g)], [0, math.sin(g), math.cos(g)]])
    want = (pts - c) @ (Rz @ Ry @ Rx).T + c
    np.testing.assert_allclose(np.stack([x, y, z], 1), want, atol=1e-12)


# --- src/clustering.rs tests ---------------------------------------------------

K = None


def _k(o, s):
    return [o.contact_key(*t) for t in s]


def test_fcc_identical(oracle):  # src/clustering.rs:308-317
    a = sorted(_k(oracle, [("A", 1, "B", 2), ("A", 3, "B", 4)]))
    f, fv = oracle.pairwise_fcc([a, a])
    assert f[0, 1] == 1.0 and fv[0, 1] == 1.0


def test_fcc_disjoint(oracle):  # src/clustering.rs:319-330
    f, fv = oracle.pairwise_fcc([_k(oracle, [("A", 1, "B", 2)]), _k(oracle, [("A", 5, "B", 6)])])
    assert f[0, 1] == 0.0 and fv[0, 1] == 0.0


def test_fcc_partial(oracle):  # src/clustering.rs:332-345
    a = sorted(_k(oracle, [("A", 1, "B", 2), ("A", 3, "B", 4)]))
    b = sorted(_k(oracle, [("A", 1, "B", 2), ("A", 5, "B", 6)]))
    f, fv = oracle.pairwise_fcc([a, b])
    assert f[0, 1] == 0.5 and fv[0, 1] == 0.5


def test_fcc_empty(oracle):  # src/clustering.rs:347-355
    f, fv = oracle.pairwise_fcc([[], []])
    assert (f == 0).all() and (fv == 0).all()


def test_cluster_empty(oracle):  # src/clustering.rs:357-363
    assert oracle.cluster([]) == []


def test_cluster_greedy_semantics(oracle):
    """Hand-built sets: five near-identical poses, a pair, a singleton and an
    empty set.  Only the group of five reaches the minimum size of 4."""
    base = _k(oracle, [("A", i, "B", i + 1) for i in range(10)])
    sets = [sorted(base) for _ in range(4)] + [sorted(base[:8])]
    sets += [sorted(_k(oracle, [("A", 50, "B", 1), ("A", 51, "B", 2)]))] * 2
    sets += [sorted(_k(oracle, [("A", 80, "B", 9)]))] + [[]]
    cl = oracle.cluster(sets)
    assert cl == [(0, [0, 1, 2, 3, 4])]
    cl2 = oracle.cluster(sets, min_size=1)
    assert [c for c, _ in cl2] == [0, 5, 7, 8]


def test_contacts_real_data(oracle):  # src/clustering.rs:365-392
    from gdock_gb300 import pdb
    import os
    from pathlib import Path
    if not os.environ.get("GDOCK_REF"):
        pytest.skip("GDOCK_REF (a gdock checkout) not set")
    ref = Path(os.environ["GDOCK_REF"]) / "data" / "2oob_A.pdb"
    if not ref.exists():
        pytest.skip(f"no data/2oob_A.pdb under GDOCK_REF={os.environ['GDOCK_REF']}")
    r = pdb.read_pdb(ref)[0]
    l = pdb.read_pdb(ref.with_name("2oob_B.pdb"))[0]
    keys = oracle.contacts(pdb.combine_molecules(r, l))
    assert len(keys) > 0
    for k in keys.tolist():
        assert (k >> 48) & 0xff != (k >> 16) & 0xff
