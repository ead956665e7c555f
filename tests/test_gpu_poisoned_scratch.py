"""The REV arenas are not cleared: the cone kernels write zeros on the part of
every line the gather can read, and a zeroing kernel prepares the adjoint's
gradient arena (line_read_span in ee_kernels.cu).  With EE_DEBUG_POISON=1
the engine fills those arenas with NaN before each chunk, so any sample read
without having been written turns a dose or gradient into NaN.  This runs the
parity, golden, plan and loss tests in a child process with that option."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_parity_with_poisoned_rev_arenas():
    env = dict(os.environ, EE_DEBUG_POISON="1")
    tests = ["tests/test_gpu_parity.py", "tests/test_gpu_golden.py", "tests/test_gpu_plan.py", "tests/test_gpu_loss.py"]
    r = subprocess.run([sys.executable, "-m", "pytest", *tests, "-x", "-q", "-m", "gpu", "-p", "no:cacheprovider",
                        "--basetemp", os.path.join(ROOT, ".pytest_tmp", "poison")],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    print(r.stdout[-3000:])
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
