"""Parity at the full benchmark sizes, through properties that do not need
the oracle on every pose:

- the single-complex scoring configuration (2,559 x 1,221 atoms, 65,536
  SO(3)-uniform poses): FP32 against the plain FP64 form on a sample of the
  poses, both against the oracle on a few; every pose's FP32 record is the
  same bits when the pose is scored alone, in another order or in a smaller
  batch (batch independence);
- the large complex (16,574 x 4,238 atoms): FP32 and FP64 against the oracle
  on a few poses.
"""
import numpy as np
import pytest

import gdock_gb300 as gd
from gdock_gb300 import position_ligand, synth

pytestmark = pytest.mark.gpu
NAMES = ("fitness", "vdw", "elec", "desolv", "air", "restraint_penalty")


def check(e, ref, tol):
    for k, name in enumerate(NAMES):
        if name in ("air", "restraint_penalty"):
            np.testing.assert_array_equal(e[name], ref[:, k], err_msg=name)
        else:
            err = np.abs(e[name] - ref[:, k]) / np.maximum(np.abs(ref[:, k]), 1.0)
            assert err.max() <= tol, (name, float(err.max()))


def as_array(e):
    return np.stack([e[k] for k in NAMES], axis=1)


@pytest.fixture(scope="module")
def c2():
    c = synth.make_complex(300, 150, 12, seed=2026)
    lig = position_ligand(c.receptor, c.ligand)
    genes = synth.quaternion_genes(np.random.default_rng(2027), 65536, half_box=20.0)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    return c, lig, genes, cx


def test_c2_full_batch_f32_against_f64_and_oracle(oracle, c2):
    c, lig, genes, cx = c2
    e32 = cx.score_poses(genes, gd.GD_PREC_F32)
    sample = np.arange(0, 65536, 256)
    e64 = cx.score_poses(genes[sample], gd.GD_PREC_F64)
    check(e32[sample], as_array(e64), 1e-5)
    few = sample[:4]
    ref = oracle.score_poses(c.receptor, lig, c.restraint_pairs, genes[few])
    check(e64[:4], ref, 1e-12)
    check(e32[few], ref, 1e-5)
    # desolvation decisions are exact: FP32 and FP64 desolvation agree to
    # the rounding of the table sums
    d = np.abs(e32["desolv"][sample] - e64["desolv"]) / np.maximum(np.abs(e64["desolv"]), 1.0)
    assert d.max() <= 1e-12


def test_c2_batch_independence(c2):
    _, _, genes, cx = c2
    full = cx.score_poses(genes, gd.GD_PREC_F32)
    rng = np.random.default_rng(5)
    idx = rng.choice(65536, size=1000, replace=False)
    part = cx.score_poses(genes[idx], gd.GD_PREC_F32)  # another batch, another order
    assert part.tobytes() == full[idx].tobytes()
    for k in idx[:3]:
        alone = cx.score_poses(genes[k:k + 1], gd.GD_PREC_F32)
        assert alone.tobytes() == full[k:k + 1].tobytes()


def test_c5_size_against_oracle(oracle):
    c = synth.make_complex(2000, 500, 30, seed=55)
    lig = position_ligand(c.receptor, c.ligand)
    genes = synth.quaternion_genes(np.random.default_rng(56), 8, half_box=20.0)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    e32 = cx.score_poses(genes, gd.GD_PREC_F32)
    e64 = cx.score_poses(genes, gd.GD_PREC_F64)
    check(e32, as_array(e64), 1e-5)
    ref = oracle.score_poses(c.receptor, lig, c.restraint_pairs, genes[:2])
    check(e64[:2], ref, 1e-12)


def test_receptor_beyond_the_segment_list(oracle):
    """A receptor of 35,946 atoms has 562 segments of 64, more than a chunk's
    culled-segment list holds (512): such chunks take every segment.  FP32
    (both work-item modes, bit-identical) against FP64 and FP64 against the
    oracle, with poses inside, at the surface of and far from the receptor."""
    from gdock_gb300 import _lib
    c = synth.make_complex(4300, 60, 4, seed=9)
    assert len(c.receptor) > 512 * 64
    lig = position_ligand(c.receptor, c.ligand)
    rng = np.random.default_rng(10)
    genes = np.concatenate([synth.quaternion_genes(rng, 8, half_box=20.0),
                            synth.random_genes(rng, 6, max_displacement=50.0)])
    genes[-1, 3:] = (400.0, 0.0, 0.0)  # nothing within reach
    ctx = gd.Context(0)
    try:
        cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
        out = {}
        for mode in (1, 2):
            ctx.set_tuning(_lib.GD_TUNE_SPLIT, mode)
            out[mode] = cx.score_poses(genes, gd.GD_PREC_F32)
        assert out[1].tobytes() == out[2].tobytes()
        e64 = cx.score_poses(genes, gd.GD_PREC_F64)
        check(out[1], as_array(e64), 1e-5)
        ref = oracle.score_poses(c.receptor, lig, c.restraint_pairs, genes[[0, len(genes) - 1]])
        check(e64[[0, len(genes) - 1]], ref, 1e-12)
        assert e64["vdw"][-1] == 0.0 and e64["elec"][-1] == 0.0
        cx.close()
    finally:
        ctx.close()
