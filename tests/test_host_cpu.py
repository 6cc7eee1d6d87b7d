"""The C++ host's .ini parsing (parallel-advection_gb300/host) against the
reference's own ConfigMap + ADVParams/Conv1dParams parsing, recorded in
tests/golden/params.json: same keys, same defaults, same strtof rounding,
same comment / continuation quirks. Runs without a GPU."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "params.json")))


@pytest.fixture(scope="module")
def params_bin(bkma):
    from bkma_gb300 import build
    exes = build.build_host_apps()
    exe = [e for e in exes if e.endswith("/params")][0]
    return exe


def _parse(exe, kind, path):
    out = subprocess.run([exe, kind, path], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def _compare(got, want):
    for k, v in want.items():
        assert k in got, k
        if isinstance(v, float):
            assert got[k] == v, (k, got[k], v)  # bit-exact (strtof then widen)
        else:
            assert got[k] == v, (k, got[k], v)


@pytest.mark.parametrize("case", sorted(k for k in GOLDEN if k.startswith("ini:")))
def test_ini_cases_match_reference(params_bin, tmp_path, case):
    entry = GOLDEN[case]
    p = tmp_path / "case.ini"
    p.write_text(entry["text"])
    kind = "conv" if case.startswith("ini:conv") else "adv"
    _compare(_parse(params_bin, kind, str(p)), entry["parsed"])


@pytest.mark.parametrize("name,kind", [("advection.ini", "adv"), ("conv1d.ini", "conv")])
def test_reference_ini_files(params_bin, name, kind):
    from oracle import reference_dir
    ref = reference_dir()
    path = os.path.join(ref, "src", name) if ref else ""
    if not os.path.exists(path):
        pytest.skip("reference checkout not available")
    _compare(_parse(params_bin, kind, path), GOLDEN[name])


def test_missing_file(params_bin):
    r = subprocess.run([params_bin, "adv", "/nonexistent.ini"], capture_output=True, text=True)
    assert r.returncode == 1
