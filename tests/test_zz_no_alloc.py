"""Scoring without device allocation, through the C ABI.

gd_score_frames_device_noalloc serves hosts that must not allocate GPU memory
while they score (their memory is handed to a pool allocator at start-up, or
their loop cannot take an allocation's latency).  It must give the same
energies as gd_score_frames_device on the same device-resident poses, call
after call, without the library allocating anything.  This file is collected
last so that a failure here leaves every other test already run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative, floor 1 kcal/mol: the FP32 form's tolerance


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    import gdock_gb300 as gd
    from gdock_gb300 import _lib, synth

    c = synth.make_complex(60, 50, 4, seed=31)
    lig = gd.position_ligand(c.receptor, c.ligand)
    n = 300
    genes = synth.random_genes(np.random.default_rng(3), n, max_displacement=10.0)
    max_disp = float(np.abs(genes[:, 3:]).max())
    ctx = gd.Context(0)
    cx = gd.Complex(c.receptor, lig, c.restraint_pairs, ctx=ctx)
    lib = ctx.lib
    stream = torch.cuda.Stream()
    frames = torch.from_numpy(_lib.make_frames(genes)).to("cuda")
    ref = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    ctx.check(lib.gd_score_frames_device(cx.h, frames.data_ptr(), n, gd.GD_PREC_F32, max_disp, ref.data_ptr(),
                                         stream.cuda_stream))
    stream.synchronize()
    ctx.sync()
    want = ref.cpu().numpy()
    in_use = ctx.bytes_in_use
    for call in range(2):
        out = torch.full((n, 6), float("nan"), dtype=torch.float64, device="cuda")
        st = lib.gd_score_frames_device_noalloc(cx.h, frames.data_ptr(), n, max_disp, out.data_ptr(),
                                                stream.cuda_stream)
        assert st == _lib.GD_OK, lib.gd_last_error(ctx.h)
        stream.synchronize()
        ctx.sync()
        got = out.cpu().numpy()
        err = np.abs(got - want) / np.maximum(np.abs(want), 1.0)
        assert np.isfinite(got).all(), call
        assert err.max() <= TOL, (call, float(err.max()))
    assert ctx.bytes_in_use == in_use  # the library allocated nothing


def test_noalloc_rejects_large_receptor():
    pytest.importorskip("torch")
    import gdock_gb300 as gd
    from gdock_gb300 import _lib, synth

    c = synth.make_complex(520, 20, 2, seed=5)  # > 4096 receptor atoms
    assert len(c.receptor) > 4096
    ctx = gd.Context(0)
    cx = gd.Complex(c.receptor, gd.position_ligand(c.receptor, c.ligand), c.restraint_pairs, ctx=ctx)
    st = ctx.lib.gd_score_frames_device_noalloc(cx.h, None, 0, 10.0, None, None)
    assert st == _lib.GD_ERR_INVALID_ARG
    assert b"4096" in ctx.lib.gd_last_error(ctx.h)
