"""Known-answer tests of the oracle's evaluator (DockQ, L-RMSD, i-RMSD, Fnat)
against the assertions of gdock's own tests in src/evaluator.rs, and of the
host-side Metrics.rank and atom-name packing."""
import math

import numpy as np
import pytest

from conftest import make_mol, tatom
from golden_data import GOLDEN, GoldenMol, load


def ca(x, resseq, chain):  # src/evaluator.rs:238-259 (create_test_atom)
    return tatom(x, 0.0, 0.0, resseq=resseq, chain=chain)


def one_one(oracle):
    rec, ref = make_mol([ca(0.0, 1, "A")]), make_mol([ca(3.0, 10, "B")])
    return oracle.Evaluator(rec, ref), ref


def atoms(oracle, mol):
    return oracle._atoms(mol)


def test_contacts_within_distance(oracle):  # src/evaluator.rs:311-324
    c = oracle._contacts(atoms(oracle, make_mol([ca(0, 1, "A")])), atoms(oracle, make_mol([ca(3, 10, "B")])))
    assert len(c) == 1 and c[0][1] == 1 and c[0][4] == 10


def test_contacts_beyond_distance(oracle):  # src/evaluator.rs:326-337
    c = oracle._contacts(atoms(oracle, make_mol([ca(0, 1, "A")])), atoms(oracle, make_mol([ca(10, 10, "B")])))
    assert c == []


def test_calculate_interface(oracle):  # src/evaluator.rs:339-361
    rec = make_mol([ca(0, 1, "A"), ca(0, 2, "A"), ca(20, 3, "A")])
    ev = oracle.Evaluator(rec, make_mol([ca(3, 10, "B")]))
    assert ev.interface == ({1, 2}, {10})


def test_evaluator_creation(oracle):  # src/evaluator.rs:363-375
    ev, _ = one_one(oracle)
    assert len(ev.interface[0]) == 1 and len(ev.interface[1]) == 1


def test_rmsd_identical(oracle):  # src/evaluator.rs:377-390
    ev, ref = one_one(oracle)
    assert ev.calc_rmsd(atoms(oracle, ref)) == 0.0


def test_rmsd_different(oracle):  # src/evaluator.rs:400-420: sqrt(3), the sum is of distances
    ev, _ = one_one(oracle)
    rmsd = ev.calc_rmsd(atoms(oracle, make_mol([ca(6, 10, "B")])))
    assert abs(rmsd - math.sqrt(3.0)) < 1e-10


def test_fnat_perfect(oracle):  # src/evaluator.rs:422-435
    ev, ref = one_one(oracle)
    assert ev.calc_fnat(atoms(oracle, ref)) == 1.0


def test_fnat_no_contacts(oracle):  # src/evaluator.rs:437-452
    ev, _ = one_one(oracle)
    assert ev.calc_fnat(atoms(oracle, make_mol([ca(20, 10, "B")]))) == 0.0


def test_metrics_complete_and_dockq(oracle):  # src/evaluator.rs:454-490
    ev, ref = one_one(oracle)
    rmsd, irmsd, fnat, dockq = ev.calc_metrics(ref)
    assert (rmsd, irmsd, fnat) == (0.0, 0.0, 1.0)
    assert abs(dockq - 1.0) < 1e-10


def test_fnat_counts_identities(oracle):
    # a docked contact counts when its (chain, residue, name) pair is native,
    # whichever atoms make it (src/evaluator.rs:126-143)
    rec = make_mol([ca(0, 1, "A")])
    ref = make_mol([ca(3, 10, "B"), dict(ca(30, 10, "B"), name="CB")])
    ev = oracle.Evaluator(rec, ref)
    assert ev.native_contacts == [("A", 1, "CA", "B", 10, "CA")]
    # ligand whose CB sits where the native CA was: not native
    lig = make_mol([ca(30, 10, "B"), dict(ca(3, 10, "B"), name="CB")])
    assert ev.calc_fnat(atoms(oracle, lig)) == 0.0


@pytest.mark.parametrize("dockq,rank", [(0.85, "High"), (0.6, "Medium"), (0.3, "Low"), (0.8, "High"),
                                        (0.5, "Medium")])
def test_metrics_rank(dockq, rank):  # src/evaluator.rs:281-309
    import gdock_gb300 as gd
    assert gd.Metrics(1.0, 1.0, 0.5, dockq).rank() == rank


def test_pack_names():
    from gdock_gb300._lib import pack_names
    p = pack_names(["CA", " N  ", "OXT", "HD21"])
    assert p.tolist() == [0x4143, 0x4E, 0x54584F, 0x31324448]
    with pytest.raises(ValueError):
        pack_names(["ABCDE"])


def test_golden_dockq_fixture(oracle):
    # the committed fixture is the oracle's output on gdock's 2oob structures
    d, rec, lig = load("2oob.npz")
    q = np.load(GOLDEN / "2oob_dockq.npz")
    ev = oracle.Evaluator(rec, GoldenMol(q, "ref"))
    assert [len(ev.interface[0]), len(ev.interface[1]), len(ev.native_contacts)] == q["interface_sizes"].tolist()
    got = ev.eval_metrics(lig, q["genes"][::6])
    np.testing.assert_array_equal(got, q["metrics"][::6])
