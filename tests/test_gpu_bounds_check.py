"""Bounds-checked build (OC_BOUNDS_CHECK) on the parity cases.

The checked library range-checks every index its kernels read from the mesh
tables (cell ids and degrees, DoF offsets, face records, boundary ids,
static-data and face-pass offsets).  On valid meshes it must flag nothing and
give the regular library's results (the checks only read indices; the same
arithmetic is compiled around them); its self-test shows that a failed check
reaches the host as OC_ERR_BOUNDS with the site and the index.  One library is
loaded per process, so the checked one runs in a child process.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checked_results(tmp_path_factory):
    from oceano_gb300.build import build
    build(bounds_check=True)
    out = tmp_path_factory.mktemp("bounds") / "checked.npz"
    env = dict(os.environ, OCEANO_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_cases.py"), str(out)],
                       env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return dict(np.load(out))


def test_checked_build_flags_nothing_and_matches(gpu_lib, checked_results):
    """Every case and precision: no OC_ERR_BOUNDS (the child would have raised),
    and the regular build's u^{n+1}, transport speed and velocity: FP64 form
    within 1e-14 of the scale; mixed form within 1e-7 (the two builds compile the
    same expressions, but the compiler's FP32 contraction and ordering choices
    around the extra checks may differ by a rounding)."""
    from bounds_cases import run_all
    assert int(checked_results["_checked"][0]) == 1
    assert gpu_lib.oc_bounds_checked() == 0
    ref = run_all()
    assert set(ref) <= set(checked_results)
    for k, v in ref.items():
        got = checked_results[k]
        scale = max(np.abs(v).max(), 1e-300)
        tol = 1e-7 if "/mixed/" in k else 1e-14
        assert np.abs(got - v).max() <= tol * scale, (k, np.abs(got - v).max() / scale)


def test_checked_build_reports_a_failed_check(gpu_lib, checked_results):
    """The self-test's out-of-range index (5 in [0, 3)) arrives as OC_ERR_BOUNDS
    with its site and index; the regular build compiles the check away."""
    from oceano_gb300 import _lib
    from bounds_cases import selftest
    assert int(checked_results["_selftest_status"][0]) == _lib.OC_ERR_BOUNDS
    msg = str(checked_results["_selftest_message"])
    assert "self-test" in msg and "index 5" in msg
    st, _ = selftest()
    assert st == _lib.OC_OK
