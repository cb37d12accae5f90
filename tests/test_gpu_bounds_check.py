"""The bounds-check build (-DFB_BOUNDS_CHECK; the stand-in for a memory
sanitizer): the kernels check their shared- and global-memory index ranges
before using them and report an index out of range through the device
status word (FB_ERR_DEVICE).  A fixed set of cases (tests/bounds_cases.py:
2D in both precisions, methods and column kernels, the headline field's
shape, direct sums, 1D, 3D, a batch) must run under it with status 0 and give
bitwise the results of the normal build.  No case feeds bad indices on
purpose: malformed inputs are rejected on the host before any launch."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fast-barnes-py_gb300")


def run_cases(tmp_path, lib, tag):
    env = dict(os.environ)
    if lib:
        env["FASTBARNES_GB300_LIB"] = lib
    else:
        env.pop("FASTBARNES_GB300_LIB", None)
    path = str(tmp_path / f"{tag}.npz")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "bounds_cases.py"), path], env=env,
                       capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, f"{tag} run failed:\n{r.stdout[-3000:]}\n{r.stderr[-3000:]}"
    return np.load(path)


def test_bounds_checked_build_reports_nothing_and_matches(tmp_path):
    r = subprocess.run([sys.executable, os.path.join(PKG, "build.py"), "--bounds-check"], capture_output=True,
                       text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    checked_lib = r.stdout.strip().splitlines()[-1]
    assert checked_lib.endswith("libfastbarnes_gb300_checked.so")
    checked = run_cases(tmp_path, checked_lib, "checked")
    plain = run_cases(tmp_path, None, "plain")
    assert "bounds-check build" in str(checked["version"])
    assert "bounds-check build" not in str(plain["version"])
    names = [k for k in plain.files if k != "version"]
    assert sorted(names) == sorted(k for k in checked.files if k != "version")
    for k in names:
        assert np.array_equal(checked[k], plain[k], equal_nan=True), k
