"""GPU parity of the scoring path through the C ABI against the CPU oracle.

FP64 (plain) form: every energy component within 1e-12 relative of the
oracle (summation order is the only difference); AIR and the restraint
penalty bit-identical (same restraint order, same arithmetic).
FP32 form: every component within 1e-5 relative, measured against
max(|E_ref|, 1 kcal/mol).
"""
import math

import numpy as np
import pytest

import gdock_gb300 as gd
from gdock_gb300 import synth
from conftest import make_mol, tatom

pytestmark = pytest.mark.gpu

FIELDS = ("vdw", "elec", "desolv", "air", "restraint_penalty", "fitness")
F64_TOL = 1e-12
F32_TOL = 1e-5


def rel_err(got, ref, floor=1.0):
    return np.abs(got - ref) / np.maximum(np.abs(ref), floor)


def check(e, ref, tol, exact_air=True):
    for k, name in enumerate(("fitness", "vdw", "elec", "desolv", "air", "restraint_penalty")):
        r = ref[:, k]
        g = e[name]
        if name in ("air", "restraint_penalty") and exact_air:
            np.testing.assert_array_equal(g, r, err_msg=name)
        else:
            err = rel_err(g, r)
            assert err.max() <= tol, (name, err.max(), int(err.argmax()))


@pytest.fixture(scope="module")
def c1():
    return synth.make_complex(50, 76, 6, seed=11)


def positioned(c):
    return gd.position_ligand(c.receptor, c.ligand)


@pytest.mark.parametrize("prec,tol", [(gd.GD_PREC_F64, F64_TOL), (gd.GD_PREC_F32, F32_TOL)])
def test_c1_random_genes(oracle, c1, prec, tol):
    lig = positioned(c1)
    rng = np.random.default_rng(5)
    genes = synth.random_genes(rng, 48)
    genes[:16, 3:] = rng.uniform(-8, 8, size=(16, 3))  # overlapping poses: many pairs in range
    cx = gd.Complex(c1.receptor, lig, c1.restraint_pairs)
    assert cx.num_restraints == len(oracle.kept_restraints(c1.restraint_pairs, c1.receptor, lig))
    e = cx.score_poses(genes, prec)
    ref = oracle.score_poses(c1.receptor, lig, c1.restraint_pairs, genes)
    check(e, ref, tol)


@pytest.mark.parametrize("nr_res,nl_res", [(3, 2), (33, 35), (40, 70), (150, 140)])
def test_sizes_around_tiles(oracle, nr_res, nl_res):
    """Receptor/ligand sizes around the 256-atom tile and slot boundaries."""
    c = synth.make_complex(nr_res, nl_res, 4, seed=nr_res * 7 + nl_res)
    lig = positioned(c)
    rng = np.random.default_rng(nr_res)
    genes = synth.random_genes(rng, 9, max_displacement=6.0)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    ref = oracle.score_poses(c.receptor, lig, c.restraint_pairs, genes)
    check(cx.score_poses(genes, gd.GD_PREC_F64), ref, F64_TOL)
    check(cx.score_poses(genes, gd.GD_PREC_F32), ref, F32_TOL)


def test_single_pose_and_no_restraints(oracle, c1):
    lig = positioned(c1)
    genes = np.array([[0.1, 0.2, 0.3, 1.0, -1.0, 2.0]])
    cx = gd.Complex(c1.receptor, lig, [])
    assert cx.num_restraints == 0
    e = cx.score_poses(genes)
    ref = oracle.score_poses(c1.receptor, lig, [], genes)
    check(e, ref, F64_TOL)
    assert e["air"][0] == 0.0 and e["restraint_penalty"][0] == 0.0


def test_missing_restraint_pairs_dropped(oracle, c1):
    lig = positioned(c1)
    pairs = list(c1.restraint_pairs) + [(9999, 1), (1, 9999)]
    cx = gd.Complex(c1.receptor, lig, pairs)
    assert cx.num_restraints == len(c1.restraint_pairs)


def test_equal_serials_skip_vdw_pairs(oracle):
    """Receptor and ligand numbered from 1: equal serials drop the vdW pair
    (src/fitness.rs:92)."""
    c = synth.make_complex(30, 25, 3, seed=3, overlap_serials=True)
    lig = positioned(c)
    genes = synth.random_genes(np.random.default_rng(1), 12, max_displacement=5.0)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs)
    ref = oracle.score_poses(c.receptor, lig, c.restraint_pairs, genes)
    check(cx.score_poses(genes, gd.GD_PREC_F64), ref, F64_TOL)
    check(cx.score_poses(genes, gd.GD_PREC_F32), ref, F32_TOL)


def test_models_path_matches_oracle(oracle, c1):
    """score command: explicit model coordinates, no transform."""
    lig = positioned(c1)
    genes = synth.random_genes(np.random.default_rng(2), 5, max_displacement=10.0)
    xyz = np.stack([np.stack(oracle.apply_genes(lig, g), axis=1) for g in genes])
    cx = gd.Complex(c1.receptor, c1.ligand, c1.restraint_pairs)
    ref = oracle.score_models(c1.receptor, c1.ligand, c1.restraint_pairs, xyz)
    check(cx.score_models(xyz, gd.GD_PREC_F64), ref, F64_TOL)
    check(cx.score_models(xyz, gd.GD_PREC_F32), ref, F32_TOL)
    # genes path and models path agree
    cx2 = gd.Complex(c1.receptor, lig, c1.restraint_pairs)
    a = cx2.score_poses(genes)
    ref2 = oracle.score_poses(c1.receptor, lig, c1.restraint_pairs, genes)
    check(a, ref2, F64_TOL)


def test_reference_kats_through_abi(oracle):
    """The reference's fitness unit tests, re-run through the GPU path."""
    r = make_mol([tatom(0, 0, 0, charge=1.0)])
    l = make_mol([tatom(5, 0, 0, charge=-1.0, serial=2)])
    assert gd.elec_energy(r, l) == pytest.approx(332.0636 * -1.0 / 25.0, rel=1e-15)
    l20 = make_mol([tatom(20, 0, 0, serial=2)])
    assert gd.vdw_energy(r, l20) == 0.0
    l1 = make_mol([tatom(1, 0, 0)])  # serial 1 == receptor serial: skipped
    assert gd.vdw_energy(r, l1) == 0.0
    ring = make_mol([tatom(3 * math.cos(i), 3 * math.sin(i), 0, "C", serial=10 + i) for i in range(15)])
    assert gd.desolv_energy(make_mol([tatom(0, 0, 0, "C")]), ring) < 0
    assert gd.desolv_energy(make_mol([tatom(0, 0, 0, "O")]), ring) > 0
    ca_r = make_mol([tatom(0, 0, 0, name="CA", resseq=1)])
    for d, air, sat in ((5.0, 0.0, 1.0), (7.0, 0.0, 1.0), (15.0, 640.0, 0.0)):
        ca_l = make_mol([tatom(d, 0, 0, name="CA", resseq=10, serial=2)])
        assert gd.air_energy([(1, 10)], ca_r, ca_l) == air
        assert gd.satisfaction_ratio([(1, 10)], ca_r, ca_l) == pytest.approx(sat)


def test_cutoff_boundaries_f32_matches_f64(oracle):
    """Ligand atoms placed within a few ulps of every cutoff (1, 8, 12 and
    15 A), each as a model of its own, so that every single pair decision
    shows in the energies: the FP32 form's guard band must reproduce the
    exact FP64 decisions.  Desolvation is a sum of table entries picked by
    exact counts (<= 1e-12); an elec or vdW decision that flipped would add or
    drop a whole pair term (0.8 kcal/mol for elec at 15 A, 3e-4 for vdW at
    12 A), far above the FP32 rounding of one term allowed here."""
    rec = make_mol([tatom(0, 0, 0, "O", charge=0.8, serial=1)])
    lig = make_mol([tatom(0, 0, 0, "N", charge=-0.7, serial=100)])
    pts = []
    for c in (1.0, 8.0, 12.0, 15.0):
        for k in (-3, -1, 0, 1, 3):
            d = c * (1 + k * 2.0 ** -52)
            for u in ((1.0, 2.0, 2.0), (0.0, 0.0, 1.0), (0.6, -0.8, 0.0)):
                pts.append(d * np.asarray(u) / np.linalg.norm(u))
    xyz = np.asarray(pts)[:, None, :]
    cx = gd.Complex(rec, lig, [])
    e64 = cx.score_models(xyz, gd.GD_PREC_F64)
    e32 = cx.score_models(xyz, gd.GD_PREC_F32)
    ref = oracle.score_models(rec, lig, [], xyz)
    check(e64, ref, F64_TOL)
    # the reference's decisions (src/fitness.rs): which models have a term
    for k, name in ((1, "vdw"), (2, "elec"), (3, "desolv")):
        np.testing.assert_array_equal(e32[name] != 0.0, ref[:, k] != 0.0, err_msg=name)
    assert np.any(ref[:, 2] == 0.0) and np.any(ref[:, 2] != 0.0)
    np.testing.assert_array_less(rel_err(e32["desolv"], e64["desolv"], 1e-300), 1e-12 + 1e-300)
    # FP32 rounding of one term: relative for elec; for vdW against a floor of
    # 0.01 kcal/mol (at 1 A its soft-core value is a difference of nearly
    # equal numbers), still 30x below a flipped 12 A term
    for name, floor in (("vdw", 1e-2), ("elec", 1e-300)):
        err = rel_err(e32[name], e64[name], floor)
        assert err.max() <= 1e-5, (name, float(err.max()), int(err.argmax()))


def test_elec_cutoff_band_in_far_rows(oracle):
    """A compact ligand slot about 15 A from a receptor atom (beyond the vdW
    reach, so its row takes the Coulomb-only path) with atoms within a few
    ulps of the 15 A elec cutoff: the FP32 form must match the FP64 one."""
    rec = make_mol([tatom(0, 0, 0, "O", charge=0.8, serial=1)])
    pts = []
    rng = np.random.default_rng(7)
    for k in range(32):
        u = np.array([1.0, 2.0, 2.0]) / 3.0 + rng.normal(0.0, 0.01, 3)
        u /= np.linalg.norm(u)
        d = 15.0 * (1 + (k % 7 - 3) * 2.0 ** -52)
        pts.append(tatom(*(d * u), "N", charge=-0.7, serial=100 + k))
    lig = make_mol(pts)
    cx = gd.Complex(rec, lig, [])
    xyz = lig.xyz()[None]
    e64 = cx.score_models(xyz, gd.GD_PREC_F64)
    e32 = cx.score_models(xyz, gd.GD_PREC_F32)
    ref = oracle.score_models(rec, lig, [], xyz)
    check(e64, ref, F64_TOL)
    assert abs(e32["elec"][0] - e64["elec"][0]) <= 1e-5 * max(1.0, abs(e64["elec"][0]))
    assert e32["vdw"][0] == 0.0 and e64["vdw"][0] == 0.0


def test_receptor_near_shared_counter_limit():
    """A receptor just under the shared-memory burial-counter limit (4,096
    atoms) needs more than 48 KB of dynamic shared memory per CTA: the FP32
    kernel must launch on a fresh context and agree with the FP64 form."""
    c = synth.make_complex(470, 40, 5, seed=3)
    assert 3600 < len(c.receptor) <= 4096
    ctx = gd.Context(0)
    try:
        lig = gd.position_ligand(c.receptor, c.ligand)
        cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
        genes = synth.quaternion_genes(np.random.default_rng(5), 64, half_box=10.0)
        e64 = cx.score_poses(genes, gd.GD_PREC_F64)
        e32 = cx.score_poses(genes, gd.GD_PREC_F32)
        for name in ("vdw", "elec", "desolv", "air"):
            assert np.allclose(e32[name], e64[name], rtol=1e-5, atol=1e-5), name
        cx.close()
    finally:
        ctx.close()


def test_split_items_bit_identical():
    """Poses split into ligand chunks (small launches) give exactly the
    energies of whole-pose work items, for single-chunk and many-chunk
    ligands and for receptors above the shared-counter limit."""
    from gdock_gb300 import _lib
    cases = [synth.make_complex(50, 76, 6, seed=11), synth.make_complex(120, 20, 4, seed=5),
             synth.make_complex(560, 90, 8, seed=9)]
    ctx = gd.Context(0)
    try:
        for c in cases:
            lig = gd.position_ligand(c.receptor, c.ligand)
            cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
            genes = synth.quaternion_genes(np.random.default_rng(3), 40, half_box=8.0)
            out = {}
            for mode in (1, 2):
                ctx.set_tuning(_lib.GD_TUNE_SPLIT, mode)
                out[mode] = cx.score_poses(genes, gd.GD_PREC_F32)
            ctx.set_tuning(_lib.GD_TUNE_SPLIT, 0)
            for name in FIELDS:
                assert np.array_equal(out[1][name], out[2][name]), (len(c.receptor), len(lig), name)
            cx.close()
    finally:
        ctx.close()


def test_bounded_wait_times_out_and_context_recovers(c1):
    """Failure detection without a fault: with GD_TUNE_FAULT one receptor
    stage copy is never issued, the bounded wait on it runs out, the kernel
    drains its other copies and returns, and the call reports GD_ERR_TIMEOUT;
    the same context then scores normally."""
    import time
    from gdock_gb300 import _lib
    ctx = gd.Context(0)
    try:
        cx = gd.Complex(c1.receptor, positioned(c1), c1.restraint_pairs, ctx=ctx)
        genes = synth.quaternion_genes(np.random.default_rng(2), 64, half_box=8.0)
        ref = cx.score_poses(genes, gd.GD_PREC_F32)
        ctx.set_tuning(_lib.GD_TUNE_FAULT, 1)
        t0 = time.time()
        with pytest.raises(gd.GdError) as ei:
            cx.score_poses(genes, gd.GD_PREC_F32)
        ctx.set_tuning(_lib.GD_TUNE_FAULT, 0)
        assert ei.value.status == 4  # GD_ERR_TIMEOUT
        assert time.time() - t0 < 30
        again = cx.score_poses(genes, gd.GD_PREC_F32)
        for name in FIELDS:
            assert np.array_equal(again[name], ref[name]), name
        cx.close()
    finally:
        ctx.close()


def test_autotuner_sets_the_fastest_candidate(c1):
    """gd_autotune_f32 times every candidate on device-resident poses, sets
    the context's knobs to the fastest, and scoring stays within tolerance."""
    import ctypes as C
    import torch
    from gdock_gb300 import _lib
    ctx = gd.Context(0)
    try:
        cx = gd.Complex(c1.receptor, positioned(c1), c1.restraint_pairs, ctx=ctx)
        genes = synth.quaternion_genes(np.random.default_rng(4), 512, half_box=8.0)
        frames = torch.from_numpy(_lib.make_frames(genes)).to("cuda:0")
        out = torch.zeros((len(genes), 6), dtype=torch.float64, device="cuda:0")
        rates = (C.c_double * len(_lib.AUTOTUNE_CANDIDATES))()
        best = C.c_int32(-1)
        ctx.check(ctx.lib.gd_autotune_f32(cx.h, frames.data_ptr(), len(genes), float(np.abs(genes[:, 3:]).max()),
                                          out.data_ptr(), None, rates, C.byref(best)))
        assert 0 <= best.value < len(_lib.AUTOTUNE_CANDIDATES)
        assert all(r > 0 for r in rates) and rates[best.value] == max(rates)
        tune, split = _lib.AUTOTUNE_CANDIDATES[best.value]
        assert ctx.lib.gd_context_get_tuning(ctx.h, _lib.GD_TUNE_F32_SLOTS) == tune
        assert ctx.lib.gd_context_get_tuning(ctx.h, _lib.GD_TUNE_SPLIT) == split
        e32 = cx.score_poses(genes, gd.GD_PREC_F32)
        e64 = cx.score_poses(genes, gd.GD_PREC_F64)
        for name in ("vdw", "elec"):
            assert np.all(rel_err(e32[name], e64[name]) <= F32_TOL), name
        for name in ("desolv", "air"):
            assert np.array_equal(e32[name], e64[name]) or np.all(rel_err(e32[name], e64[name]) <= 1e-12), name
        cx.close()
    finally:
        ctx.close()


@pytest.mark.parametrize("split", [1, 2])
def test_empty_molecules(oracle, split):
    """An empty ligand or receptor scores zero pair terms (and the receptor's
    or ligand's desolvation at zero burial), in both forms and both work-item
    modes, like the oracle."""
    from gdock_gb300 import _lib
    c = synth.make_complex(30, 20, 0, seed=3)
    empty = make_mol([])
    ctx = gd.Context(0)
    try:
        ctx.set_tuning(_lib.GD_TUNE_SPLIT, split)
        genes = synth.quaternion_genes(np.random.default_rng(1), 3, half_box=5.0)
        for rec, lig in ((c.receptor, empty), (empty, c.ligand)):
            cx = gd.Complex(rec, lig, [], ctx=ctx)
            ref = oracle.score_poses(rec, lig, [], genes)
            for prec, tol in ((gd.GD_PREC_F64, F64_TOL), (gd.GD_PREC_F32, F32_TOL)):
                check(cx.score_poses(genes, prec), ref, tol)
            cx.close()
    finally:
        ctx.close()


def test_deterministic(c1):
    lig = positioned(c1)
    genes = synth.random_genes(np.random.default_rng(9), 20)
    cx = gd.Complex(c1.receptor, lig, c1.restraint_pairs)
    for prec in (gd.GD_PREC_F64, gd.GD_PREC_F32):
        a, b = cx.score_poses(genes, prec), cx.score_poses(genes, prec)
        assert a.tobytes() == b.tobytes()


def test_invalid_arguments_rejected(c1):
    from gdock_gb300 import _lib
    cx = gd.Complex(c1.receptor, positioned(c1), c1.restraint_pairs)
    g = np.zeros((1, 6))
    out = np.zeros(1, dtype=_lib.POSE_ENERGY_DTYPE)
    lib = cx.lib
    assert lib.gd_score_poses(cx.h, _lib.ptr(g), 1, 7, _lib.ptr(out)) == _lib.GD_ERR_INVALID_ARG
    assert lib.gd_score_poses(cx.h, None, 1, 0, _lib.ptr(out)) == _lib.GD_ERR_INVALID_ARG
    assert lib.gd_score_poses(cx.h, _lib.ptr(g), -1, 0, _lib.ptr(out)) == _lib.GD_ERR_INVALID_ARG
    assert lib.gd_score_poses(None, _lib.ptr(g), 1, 0, _lib.ptr(out)) == _lib.GD_ERR_INVALID_ARG
    assert b"precision" in lib.gd_last_error(cx.ctx.h) or lib.gd_last_error(cx.ctx.h)
    with pytest.raises(ValueError):
        cx.score_poses(g, 7)
    # nothing was corrupted: a valid call still works
    assert np.isfinite(cx.score_poses(g)["fitness"]).all()


def test_hbm_budget_enforced(c1):
    ctx = gd.Context(0, hbm_budget_bytes=1 << 16)
    with pytest.raises(gd.GdError) as ei:
        gd.Complex(c1.receptor, positioned(c1), c1.restraint_pairs, ctx=ctx)
    assert ei.value.status == 2  # GD_ERR_OOM
    ctx.close()


def test_clamped_lj_variant(oracle):
    """Well depths above 50 kcal/mol make the soft-core LJ reach the
    reference's clamp to [-50, 500] (src/fitness.rs:66-68): the kernels' clamp
    variants, FP64 and FP32 (with segment culling on rigid poses), against the
    oracle; equal serials on top select the variant with both."""
    rng = np.random.default_rng(12)
    for overlap in (False, True):
        rec = make_mol([tatom(*rng.uniform(-6, 6, 3), "C", charge=rng.uniform(-0.5, 0.5), serial=1 + i,
                              epsilon=-120.0 if i % 3 == 0 else -0.1, rmin2=2.2) for i in range(90)])
        lig = make_mol([tatom(*rng.uniform(-4, 4, 3), "N", charge=rng.uniform(-0.5, 0.5),
                              serial=(1 + i) if overlap else 500 + i, epsilon=-80.0 if i % 2 else -0.2, rmin2=1.9)
                        for i in range(70)])
        lig = gd.position_ligand(rec, lig)
        genes = synth.random_genes(rng, 24, max_displacement=6.0)
        cx = gd.Complex(rec, lig, [])
        ref = oracle.score_poses(rec, lig, [], genes)
        check(cx.score_poses(genes, gd.GD_PREC_F64), ref, F64_TOL)
        check(cx.score_poses(genes, gd.GD_PREC_F32), ref, F32_TOL)
        assert np.any(np.abs(ref[:, 1]) > 100.0)  # the clamp is reached


def _first_atoms(mol, n):
    """The molecule's first n atoms (every per-atom field sliced)."""
    import dataclasses
    return dataclasses.replace(mol, **{f.name: getattr(mol, f.name)[:n] for f in dataclasses.fields(mol)})


@pytest.mark.parametrize("nr,nl", [(1, 1), (7, 33), (64, 32), (65, 129), (129, 128), (200, 257), (513, 95)])
def test_exact_atom_counts_around_runs_slots_and_chunks(oracle, nr, nl):
    """Receptors cut at, or one past, the 8-atom runs and 64-atom segments of
    the FP32 kernel, ligands at, or one past, its 32-atom slots and 128-atom
    chunks: FP64 and FP32 (whole poses and split items, bit-identical to each
    other) against the oracle."""
    from gdock_gb300 import _lib
    c = synth.make_complex(80, 40, 0, seed=nr + 3 * nl)
    rec = _first_atoms(c.receptor, nr)
    lig = gd.position_ligand(rec, _first_atoms(c.ligand, nl))
    assert (len(rec), len(lig)) == (nr, nl)
    genes = synth.quaternion_genes(np.random.default_rng(nr * 7 + nl), 24, half_box=6.0)
    ref = oracle.score_poses(rec, lig, [], genes)
    ctx = gd.Context(0)
    try:
        cx = gd.Complex(rec, lig, [], ctx=ctx)
        check(cx.score_poses(genes, gd.GD_PREC_F64), ref, F64_TOL)
        out = {}
        for mode in (1, 2):
            ctx.set_tuning(_lib.GD_TUNE_SPLIT, mode)
            out[mode] = cx.score_poses(genes, gd.GD_PREC_F32)
            check(out[mode], ref, F32_TOL)
        for name in FIELDS:
            assert np.array_equal(out[1][name], out[2][name]), name
        cx.close()
    finally:
        ctx.close()


def test_receptor_parts_do_not_change_the_energies(oracle):
    """Split launches may cut each ligand chunk's receptor into R interleaved
    segment sets (GD_TUNE_RPARTS; automatically for launches with few poses).
    The vdW and Coulomb sums are per-segment fixed-point integers, so R = 1,
    2, 3 and 8, and whole-pose items, give bit-identical energies, all within
    the FP32 tolerance of the oracle."""
    from gdock_gb300 import _lib
    cases = [synth.make_complex(50, 76, 6, seed=11), synth.make_complex(300, 150, 12, seed=2),
             synth.make_complex(12, 40, 2, seed=4)]
    ctx = gd.Context(0)
    try:
        for c in cases:
            lig = gd.position_ligand(c.receptor, c.ligand)
            cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
            genes = synth.quaternion_genes(np.random.default_rng(len(c.receptor)), 30, half_box=10.0)
            ref = oracle.score_poses(c.receptor, lig, c.restraint_pairs, genes)
            ctx.set_tuning(_lib.GD_TUNE_SPLIT, 1)
            whole = cx.score_poses(genes, gd.GD_PREC_F32)
            check(whole, ref, F32_TOL)
            ctx.set_tuning(_lib.GD_TUNE_SPLIT, 2)
            for r in (0, 1, 2, 3, 8):
                ctx.set_tuning(_lib.GD_TUNE_RPARTS, r)
                assert ctx.get_tuning(_lib.GD_TUNE_RPARTS) == r
                got = cx.score_poses(genes, gd.GD_PREC_F32)
                for name in FIELDS:
                    assert np.array_equal(got[name], whole[name]), (len(c.receptor), r, name)
            ctx.set_tuning(_lib.GD_TUNE_RPARTS, 0)
            ctx.set_tuning(_lib.GD_TUNE_SPLIT, 0)
            cx.close()
        with pytest.raises(gd.GdError):
            ctx.set_tuning(_lib.GD_TUNE_RPARTS, 9)
    finally:
        ctx.close()


def test_fp32_sum_range_is_reported(oracle):
    """Charges so large that one segment's FP32 Coulomb partial leaves the
    fixed-point range (2^24 kcal/mol) make the FP32 call fail with a status
    instead of wrapping; the FP64 form still scores them, and the context
    keeps working."""
    rec = make_mol([tatom(0.0, 0.0, 0.0, "C", charge=3000.0, resseq=1, serial=1, chain="A"),
                    tatom(1.5, 0.0, 0.0, "C", charge=3000.0, resseq=2, serial=2, chain="A")])
    lig = make_mol([tatom(0.0, 2.0, 0.0, "C", charge=3000.0, resseq=1, serial=11, chain="B"),
                    tatom(0.0, -2.0, 0.0, "C", charge=-3000.0, resseq=2, serial=12, chain="B")])
    genes = np.zeros((2, 6))
    ctx = gd.Context(0)
    try:
        cx = gd.Complex(rec, lig, [], ctx=ctx)
        with pytest.raises(gd.GdError):
            cx.score_poses(genes, gd.GD_PREC_F32)
        check(cx.score_poses(genes, gd.GD_PREC_F64), oracle.score_poses(rec, lig, [], genes), F64_TOL)
        cx.close()
        c = synth.make_complex(20, 10, 0, seed=3)
        lig2 = gd.position_ligand(c.receptor, c.ligand)
        cx2 = gd.Complex(c.receptor, lig2, [], ctx=ctx)
        g2 = synth.random_genes(np.random.default_rng(2), 4, max_displacement=5.0)
        check(cx2.score_poses(g2, gd.GD_PREC_F32), oracle.score_poses(c.receptor, lig2, [], g2), F32_TOL)
        cx2.close()
    finally:
        ctx.close()
