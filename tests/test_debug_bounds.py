"""The bounds-checked build (-DLTP_DEBUG_BOUNDS): every scatter into a
scratch or table array, and every conflict-word index, is checked against
its capacity; a violation becomes LTP_E_DEVICE_ASSERT from ltp_batch_finish
instead of a fault.  CPU: the variant builds.  GPU: the parity and
order-entry suites pass on it, so no check fires on any of their cases."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_bounds_checked_build_compiles():
    from ltpmg_gb300 import _build

    lib = _build.build(debug_bounds=True)
    assert os.path.exists(lib) and lib.endswith("_debug.so")


@pytest.mark.gpu
def test_parity_suites_on_the_bounds_checked_build():
    from ltpmg_gb300 import _build

    lib = _build.build(debug_bounds=True)
    env = dict(os.environ, LTPMG_LIB=lib)
    # the 8 GiB largest-table case adds nothing here and takes the longest
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-m", "gpu", "-k", "not largest_table",
                        os.path.join(HERE, "test_gpu_parity.py"), os.path.join(HERE, "test_tpcc.py"),
                        os.path.join(HERE, "test_wide.py")],
                       env=env, capture_output=True, text=True, timeout=1200, cwd=os.path.dirname(HERE))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
