"""GPU path against the committed golden fixtures (gdock's 2oob and 1h590
test structures, oracle outputs), through the C ABI."""
import numpy as np
import pytest

import gdock_gb300 as gd
from golden_data import cluster_list, contact_sets, load

pytestmark = pytest.mark.gpu
NAMES = ("fitness", "vdw", "elec", "desolv", "air", "restraint_penalty")


def check(e, ref, tol):
    for k, name in enumerate(NAMES):
        if name in ("air", "restraint_penalty"):
            np.testing.assert_array_equal(e[name], ref[:, k], err_msg=name)
        else:
            err = np.abs(e[name] - ref[:, k]) / np.maximum(np.abs(ref[:, k]), 1.0)
            assert err.max() <= tol, (name, float(err.max()))


@pytest.mark.parametrize("prec,tol", [(gd.GD_PREC_F64, 1e-12), (gd.GD_PREC_F32, 1e-5)])
def test_2oob_poses(prec, tol):
    d, rec, lig = load("2oob.npz")
    cx = gd.Complex(rec, lig, d["restraints"].tolist())
    check(cx.score_poses(d["genes"], prec), d["energies"], tol)


def test_2oob_contacts_and_clusters():
    d, rec, lig = load("2oob.npz")
    cx = gd.Complex(rec, lig, d["restraints"].tolist())
    got = cx.pose_contacts(d["genes"][8:40])
    for a, b in zip(got, contact_sets(d)):
        np.testing.assert_array_equal(a, b)
    cl = cx.cluster(d["genes"][8:40], gd.ClusteringConfig(min_cluster_size=1))
    assert [(r.center_idx, r.members) for r in cl] == cluster_list(d)


@pytest.mark.parametrize("prec,tol", [(gd.GD_PREC_F64, 1e-12), (gd.GD_PREC_F32, 1e-5)])
def test_1h590_score_command(prec, tol):
    d, rec, lig = load("1h590_score.npz")
    cx = gd.Complex(rec, lig, [])
    check(cx.score_models(d["models_xyz"], prec), d["energies"], tol)
