"""Generate the golden fixtures of tests/golden from gdock's own test data.

Reads the reference's structures (data/2oob_A.pdb, data/2oob_B.pdb,
data/1h590A_0A.pdb, data/1h590B_0A_poses.pdb, and data/2oob_B_ref.pdb, the
reference ligand of the DockQ evaluator, under the reference checkout),
parses them with gdock_gb300.pdb (gdock's reader and parameter assignment),
and stores the parsed atom arrays together with the CPU oracle's outputs:
energies of seeded poses and of the 100 MODELs of the `score` example,
contacts, clusters and the evaluator's metrics.  The GPU tests compare against these files, so they
need neither the reference checkout nor the oracle at run time.

Usage: python tests/golden/make_golden.py [path/to/gdock]  (default: $GDOCK_REF)
"""
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from gdock_gb300 import pdb  # noqa: E402
import oracle  # noqa: E402

FIELDS = ("serial", "resseq", "x", "y", "z", "epsilon", "rmin2", "charge", "vdw_radius")
# README example restraints of 2oob (receptor resseq : ligand resseq)
RESTRAINTS_2OOB = [(933, 6), (936, 8), (940, 42), (941, 44), (946, 45), (950, 46)]


def pack(prefix, mol, d):
    for f in FIELDS:
        d[f"{prefix}_{f}"] = np.asarray(getattr(mol, f))
    d[f"{prefix}_chain"] = mol.chain_code
    d[f"{prefix}_element"] = mol.element_class
    d[f"{prefix}_is_ca"] = mol.is_ca
    d[f"{prefix}_name"] = np.array(mol.name)
    d[f"{prefix}_resname"] = np.array(mol.resname)


def main(ref: Path):
    data = ref / "data"
    rec = pdb.read_pdb(data / "2oob_A.pdb")[0]
    lig_native = pdb.read_pdb(data / "2oob_B.pdb")[0]
    lig = pdb.position_ligand(rec, lig_native)
    # genes of the crystal placement: no rotation, centroid shift back
    native_shift = np.array(lig_native.center_of_mass()) - np.array(lig.center_of_mass())
    d = {}
    pack("rec", rec, d)
    pack("lig", lig, d)
    d["restraints"] = np.array(RESTRAINTS_2OOB, np.int32)
    rng = np.random.default_rng(2024)
    genes = np.empty((48, 6))
    genes[:16, :3] = rng.uniform(0, 2 * np.pi, (16, 3))      # random poses
    genes[:16, 3:] = rng.uniform(-12, 12, (16, 3))
    genes[16:, :3] = np.mod(rng.normal(0, 0.05, (32, 3)), 2 * np.pi)  # near the crystal placement
    genes[16:, 3:] = native_shift + rng.normal(0, 1.0, (32, 3))
    d["genes"] = genes
    d["energies"] = oracle.score_poses(rec, lig, RESTRAINTS_2OOB, genes)
    sets = [oracle.pose_contacts(rec, lig, g) for g in genes[8:40]]
    d["contact_offsets"] = np.cumsum([0] + [len(s) for s in sets]).astype(np.int64)
    d["contact_keys"] = np.concatenate(sets).astype(np.int64) if sets else np.zeros(0, np.int64)
    cl = oracle.cluster(sets, min_size=1)
    d["cluster_centers"] = np.array([c for c, _ in cl], np.int32)
    d["cluster_members"] = np.concatenate([np.array(m, np.int32) for _, m in cl])
    d["cluster_sizes"] = np.array([len(m) for _, m in cl], np.int32)
    np.savez_compressed(HERE / "2oob.npz", **d)

    # evaluator::Evaluator of the crystal ligand (chain B of data/2oob.pdb)
    ref_lig = pdb.read_pdb(data / "2oob_B_ref.pdb")[0]
    q = {}
    pack("ref", ref_lig, q)
    ev = oracle.Evaluator(rec, ref_lig)
    q["genes"] = genes
    q["metrics"] = ev.eval_metrics(lig, genes)
    q["interface_sizes"] = np.array([len(ev.interface[0]), len(ev.interface[1]), len(ev.native_contacts)], np.int64)
    np.savez_compressed(HERE / "2oob_dockq.npz", **q)

    rec2 = pdb.read_pdb(data / "1h590A_0A.pdb")[0]
    models = pdb.read_pdb(data / "1h590B_0A_poses.pdb")
    e = {}
    pack("rec", rec2, e)
    pack("lig", models[0], e)
    e["models_xyz"] = np.stack([m.xyz() for m in models])
    e["energies"] = oracle.score_models(rec2, models[0], [], e["models_xyz"])
    np.savez_compressed(HERE / "1h590_score.npz", **e)
    print("wrote", HERE / "2oob.npz", HERE / "2oob_dockq.npz", HERE / "1h590_score.npz")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GDOCK_REF")
    if not ref:
        sys.exit("usage: make_golden.py path/to/gdock (or set GDOCK_REF to a gdock checkout)")
    main(Path(ref))
