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


def test_header_is_plain_c_and_links(tmp_path):
    """The header compiles as C99 with warnings as errors, and a C program that
    takes the address of every entry point links against the library (no
    call is made: no GPU is needed).  This is what an FFI binding generator
    or a C host sees."""
    import shutil
    import subprocess
    import pytest
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = build.build()
    names = declared_symbols()
    src = tmp_path / "use_abi.c"
    src.write_text("#include \"gdock_gb300.h\"\n#include <stdio.h>\n"
                   "typedef void (*any_fn)(void);\n"
                   "int main(void) {\n  any_fn p[] = {\n"
                   + "".join(f"    (any_fn)&{n},\n" for n in names)
                   + "  };\n  printf(\"%d %d\\n\", (int)(sizeof(p) / sizeof(p[0])), (int)sizeof(gd_pose_frame));\n"
                   "  return 0;\n}\n")
    exe = tmp_path / "use_abi"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", f"-I{ROOT / 'include'}",
                        str(src), "-o", str(exe), f"-L{lib.parent}", "-lgdock_gb300",
                        f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == [str(len(names)), "128"]


def test_frames_on_the_host_pool():
    """Large batches build their frames on a pool of host threads kept across
    calls: the frames equal the one-pose calls', repeated calls and
    concurrent callers agree, and a process forked after the pool exists
    builds its own (the child has none of the parent's threads) instead of
    waiting on them."""
    import os
    import threading
    import time
    import warnings
    import numpy as np
    from gdock_gb300 import synth
    g = synth.random_genes(np.random.default_rng(1), 20000)
    a = _lib.make_frames(g)
    assert np.array_equal(a[::997], np.stack([_lib.make_frames(g[i:i + 1])[0] for i in range(0, 20000, 997)]))
    for _ in range(3):
        assert np.array_equal(_lib.make_frames(g), a)
    ok = []
    ts = [threading.Thread(target=lambda: ok.append(np.array_equal(_lib.make_frames(g), a))) for _ in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert ok == [True] * 4
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", DeprecationWarning)
        pid = os.fork()
    if pid == 0:
        os._exit(0 if np.array_equal(_lib.make_frames(g), a) else 3)
    t_end = time.time() + 60
    while True:
        done, status = os.waitpid(pid, os.WNOHANG)
        if done:
            break
        if time.time() > t_end:
            os.kill(pid, 9)
            os.waitpid(pid, 0)
            raise AssertionError("the forked child did not finish building frames")
        time.sleep(0.05)
    assert os.WIFEXITED(status) and os.WEXITSTATUS(status) == 0
