"""The GPU tests again through the debug library (kernel index checks
compiled in): every call returns GD_OK and every result still matches, so no
check fired on the workloads the tests cover.  A failed check would make the
call fail with "device index check failed at site N"."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
FILES = ["test_gpu_golden.py", "test_gpu_scoring.py", "test_gpu_ga.py", "test_gpu_cluster.py",
         "test_gpu_evaluator.py", "test_gpu_server.py", "test_gpu_full_size.py",
         "test_gpu_edge_cases.py", "test_gpu_contact_boundary.py", "test_gpu_cluster_large.py"]


def test_gpu_suite_under_debug_library():
    from gdock_gb300 import build
    build.build(debug=True)
    env = dict(os.environ, GD_LIBRARY="debug")
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
           *[str(ROOT / "tests" / f) for f in FILES]]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "passed" in r.stdout
