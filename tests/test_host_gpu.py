"""The C++ drivers (mirrors of src/advection.cpp and src/conv1d.cpp) on the
GPU through the C ABI: the reference's analytic check (mean L1 < 1e-6 after
10 steps, validation_unittests.cpp:34-65) for every strategy name, the
impl_selector error for an unknown name, and conv1d's constant-fill checks."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def apps(bkma):
    from bkma_gb300 import build
    exes = build.build_host_apps()
    return {os.path.basename(e): e for e in exes}


ADV_INI = """[problem]
n0 = 8
n1 = 256
n2 = 4
maxIter = 10
dt = 0.0001
minRealX = 0
maxRealX = 1
minRealVx = 0
maxRealVx = 1
[impl]
kernelImpl = {impl}
[optimization]
gpu = true
"""


@pytest.mark.parametrize("impl,extra", [("AdaptiveWg", []), ("NDRange", []), ("BasicRange", []),
                                        ("Plain", []), ("AdaptiveWg", ["--fp32"]),
                                        ("GB300", ["--fp32"])])
def test_advection_driver(apps, tmp_path, impl, extra):
    ini = tmp_path / "adv.ini"
    ini.write_text(ADV_INI.format(impl=impl))
    r = subprocess.run([apps["advection"], str(ini)] + extra, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    m = re.search(r"Highest L1 error found: (\S+) \(lowest is (\S+)\)", r.stdout)
    assert m, r.stdout
    assert float(m.group(1)) < 1e-6
    assert "PERF_DIAGS:" in r.stdout and "upd_cells_per_sec" in r.stdout


def _l1(apps, tmp_path, impl, extra):
    ini = tmp_path / "adv.ini"
    ini.write_text(ADV_INI.format(impl=impl))
    r = subprocess.run([apps["advection"], str(ini)] + extra, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    return re.search(r"Highest L1 error found: (\S+) \(lowest is (\S+)\)", r.stdout).groups()


@pytest.mark.parametrize("impl,extra", [("AdaptiveWg", ["--fp32"]), ("AdaptiveWg", []),
                                        ("BasicRange", ["--fp32"])])
def test_advection_driver_fused_same_result(apps, tmp_path, impl, extra):
    """--fused K gives the bits of one step per launch in FP32, so the printed
    validation errors are the same. FP64 fused steps run FP64 arithmetic while
    one step per launch runs the FP32-pair kernel (2e-13 max|f| per step
    apart), so the FP64 errors agree to 1e-13; --hi-lo stays within the check."""
    fused = _l1(apps, tmp_path, impl, extra + ["--fused", "4"])
    one = _l1(apps, tmp_path, impl, extra)
    if "--fp32" in extra:
        assert fused == one
    else:
        assert all(abs(float(a) - float(b)) <= 1e-13 for a, b in zip(fused, one)), (fused, one)
    if "--fp32" in extra:
        hi, _ = _l1(apps, tmp_path, impl, extra + ["--fused", "10", "--hi-lo"])
        assert float(hi) < 1e-6


def test_advection_driver_unknown_impl(apps, tmp_path):
    ini = tmp_path / "adv.ini"
    ini.write_text(ADV_INI.format(impl="Hierarchical"))
    r = subprocess.run([apps["advection"], str(ini)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "Hierarchical is not a valid implementation name." in r.stderr


def test_conv1d_driver(apps, tmp_path):
    ini = tmp_path / "conv.ini"
    ini.write_text("[problem]\nlength = 64\nchannel_in = 3\nk = 3\ntotal_batch_size = 64\n"
                   "batch_size_n2 = 4\n")
    r = subprocess.run([apps["conv1d"], str(ini)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "All values data[:,i1,:] are equal." in r.stdout
    m = re.search(r"Normalized Array after: (\S+)", r.stdout)
    assert m and abs(float(m.group(1)) - (1 + 3 * 3 * 1.5 * 7.3)) < 1e-9
