"""The C-ABI library builds, loads without a GPU, and exports every entry
point include/gdock_gb300.h declares."""
import ctypes
import re
from pathlib import Path

from gdock_gb300 import _lib, build

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    hdr = (ROOT / "include" / "gdock_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(gd_[a-z_0-9]+)\s*\(", hdr, re.M)))


def test_header_matches_binding_table():
    assert sorted(_lib.EXPORTS) == declared_symbols()


def test_library_exports_all_symbols():
    lib = ctypes.CDLL(str(build.build()))
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.gd_abi_version() == 1


def test_status_strings():
    lib = _lib.load()
    for s in range(7):
        assert lib.gd_status_string(s)


def test_make_frames_host_side():
    import math
    import numpy as np
    f = _lib.make_frames(np.array([[0.3, 1.1, 2.5, 1.0, -2.0, 3.0]]))[0]
    ca, sa, cb, sb, cg, sg = (math.cos(0.3), math.sin(0.3), math.cos(1.1), math.sin(1.1), math.cos(2.5),
                              math.sin(2.5))
    assert f[:6].tolist() == [ca, sa, cb, sb, cg, sg]
    assert f[6] == -sa * cg + ca * sb * sg and f[9] == -ca * sg + sa * sb * cg
    assert f[10:13].tolist() == [1.0, -2.0, 3.0]


def test_context_without_gpu_fails_loudly():
    import pytest
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(_lib.GdError):
        _lib.Context(0)


def test_debug_library_builds_and_exports_all_symbols():
    # the debug variant: the same sources with the kernels' index checks
    # compiled in (-DGD_DEBUG_CHECKS)
    path = build.build(debug=True)
    assert path.name == "libgdock_gb300_debug.so"
    lib = ctypes.CDLL(str(path))
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.gd_abi_version() == 1
