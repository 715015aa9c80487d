"""DockQ evaluator on the GPU (gd_evaluate_poses) against the oracle's
restatement of src/evaluator.rs: the committed 2oob fixture, the reference's
own single-atom cases, and seeded synthetic molecules with ragged sizes."""
import numpy as np
import pytest

import gdock_gb300 as gd
from conftest import make_mol, tatom
from golden_data import GOLDEN, GoldenMol, load

pytestmark = pytest.mark.gpu
FIELDS = ("rmsd", "irmsd", "fnat", "dockq")
TOL = 1e-12  # rmsd/irmsd: the device sums distances in another order; fnat is exact


def check(got, ref):
    for k, name in enumerate(FIELDS):
        if name == "fnat":
            np.testing.assert_array_equal(got[name], ref[:, k], err_msg=name)
        else:
            err = np.abs(got[name] - ref[:, k]) / np.maximum(np.abs(ref[:, k]), 1e-300)
            assert err.max() <= TOL, (name, float(err.max()))


def test_2oob_fixture():
    d, rec, lig = load("2oob.npz")
    q = np.load(GOLDEN / "2oob_dockq.npz")
    cx = gd.Complex(rec, lig, [])
    ev = gd.Evaluator(cx, GoldenMol(q, "ref"))
    check(ev.eval_metrics(q["genes"]), q["metrics"])
    assert ev.eval_metrics(np.zeros((0, 6))).shape == (0,)


def test_reference_single_atom_cases():
    # src/evaluator.rs:377-490 through the device: the ligand is the moving
    # molecule, posed by its genes
    rec = make_mol([tatom(0, 0, 0, resseq=1, chain="A")])
    ref = make_mol([tatom(3, 0, 0, resseq=10, chain="B")])
    cx = gd.Complex(rec, ref, [])
    ev = gd.Evaluator(cx, ref)
    m = ev.calc_metrics([0, 0, 0, 0, 0, 0])
    assert (m.rmsd, m.irmsd, m.fnat) == (0.0, 0.0, 1.0) and abs(m.dockq - 1.0) < 1e-10
    m = ev.calc_metrics([0, 0, 0, 3, 0, 0])  # 3 A away: sqrt(3)
    assert abs(m.rmsd - np.sqrt(3.0)) < 1e-10 and m.fnat == 0.0
    m = ev.calc_metrics([0, 0, 0, 17, 0, 0])
    assert m.fnat == 0.0


def synth(rng, n, chain, resseq0, centre, spread, names=("N", "CA", "C", "O", "CB", "CG", "OXT")):
    atoms = []
    for i in range(n):
        p = centre + rng.normal(0, spread, 3)
        atoms.append(tatom(*p, resseq=resseq0 + i // 7, chain=chain, name=names[i % len(names)]))
    return make_mol(atoms)


@pytest.mark.parametrize("seed,nr,nl,nref", [(1, 400, 300, 300), (2, 333, 257, 190), (3, 150, 97, 140),
                                             (4, 64, 33, 33)])
def test_synthetic_vs_oracle(oracle, seed, nr, nl, nref):
    # ragged sizes; the reference may have fewer or more atoms than the
    # ligand (zip truncates, the divisor stays the reference's count)
    rng = np.random.default_rng(seed)
    rec = synth(rng, nr, "A", 1, np.zeros(3), 8.0)
    lig = synth(rng, nl, "B", 1, np.array([14.0, 0, 0]), 6.0)
    ref = synth(rng, nref, "B", 1, np.array([13.0, 1.0, 0]), 6.0)
    genes = np.empty((37, 6))
    genes[:, :3] = rng.uniform(0, 2 * np.pi, (37, 3))
    genes[:, 3:] = rng.normal(0, 2.0, (37, 3))
    genes[0] = 0.0
    cx = gd.Complex(rec, lig, [])
    got = gd.Evaluator(cx, ref).eval_metrics(genes)
    check(got, oracle.Evaluator(rec, ref).eval_metrics(lig, genes))


def test_no_interface(oracle):
    rng = np.random.default_rng(9)
    rec = synth(rng, 50, "A", 1, np.zeros(3), 3.0)
    lig = synth(rng, 40, "B", 1, np.array([60.0, 0, 0]), 3.0)
    cx = gd.Complex(rec, lig, [])
    ev = gd.Evaluator(cx, lig)  # reference far from the receptor: no native contacts
    genes = rng.normal(0, 1.0, (5, 6))
    got = ev.eval_metrics(genes)
    check(got, oracle.Evaluator(rec, lig).eval_metrics(lig, genes))
    assert (got["fnat"] == 0).all() and (got["irmsd"] == 0).all()
