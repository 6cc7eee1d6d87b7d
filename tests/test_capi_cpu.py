"""The C-ABI library loads without a GPU, exports every function that
include/bkma_gb300.h declares, and rejects bad descriptors before touching the
device (no compute calls here)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "bkma_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(bkma_[a-z0-9_]+)\s*\(", txt)))


def test_every_declared_symbol_is_exported(bkma):
    lib = bkma.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_python_signatures_cover_header(bkma):
    from bkma_gb300 import _lib
    assert set(_declared()) == set(_lib.SIGNATURES)


def test_abi_version(bkma):
    assert bkma.load().bkma_abi_version() == 1


@pytest.mark.parametrize("name,impl,inplace", [("NDRange", 1, True), ("adaptivewg", 1, True),
                                                ("BasicRange", 1, False), ("plain", 2, True),
                                                ("GB300", 1, True)])
def test_impl_selector(bkma, name, impl, inplace):
    assert bkma.impl_from_name(name) == (impl, inplace)


def test_impl_selector_unknown_name_message(bkma):
    with pytest.raises(bkma.BkmaError) as e:
        bkma.impl_from_name("Hierarchical")
    assert e.value.status == 2
    assert "Hierarchical is not a valid implementation name." in str(e.value)
    assert "Should be: {BasicRange, NDRange, AdaptiveWg}" in str(e.value)


@pytest.mark.parametrize("kw,msg", [
    (dict(n0=0), "positive"),
    (dict(degree=4, weights="lagrange"), "degree"),
    (dict(degree=3), "degree 5 only"),
    (dict(impl="plain", dtype="f32"), "plain form"),
    (dict(i0_offset=9), "i0_offset"),
    (dict(i0_count=9), "i0_count"),
    (dict(maxX=-1.0), "maxX"),
    (dict(n0=2**31), "n0 must be < 2^31"),
    (dict(n0=2**28, n1=2**16, n2=2**8), "2^50"),
    (dict(maxVx=float("inf")), "must be finite"),
    (dict(velocity=[0.1] * 7 + [float("nan")]), "velocity values must be finite"),
])
def test_adv_descriptor_validation(bkma, kw, msg):
    args = dict(n0=8, n1=64, n2=3)
    args.update(kw)
    n0, n1, n2 = args.pop("n0"), args.pop("n1"), args.pop("n2")
    with pytest.raises(bkma.BkmaError) as e:
        bkma.AdvectionPlan(n0, n1, n2, **args)
    assert e.value.status == 1
    assert msg in str(e.value)


@pytest.mark.parametrize("kw,msg", [
    (dict(batch=0), "positive"),
    (dict(ksize=100), "ksize"),
    (dict(semantics="reference", cout=5, dtype="f64"), "channel_out"),
    (dict(semantics="reference", dtype="f32"), "FP64"),
    (dict(cout=3), "cin == cout"),
])
def test_conv_descriptor_validation(bkma, kw, msg):
    args = dict(batch=2, cin=4, cout=4, length=32, ksize=3, dtype="f64")
    args.update(kw)
    with pytest.raises(bkma.BkmaError) as e:
        bkma.Conv1dPlan(args.pop("batch"), args.pop("cin"), args.pop("cout"), args.pop("length"),
                        args.pop("ksize"), **args)
    assert e.value.status == 1
    assert msg in str(e.value)


def test_null_arguments(bkma):
    lib = bkma.load()
    assert lib.bkma_adv_step(None, None, None, 1, None) == 1
    assert lib.bkma_conv_run(None, None, None, None, None, None) == 1
    assert lib.bkma_adv_plan_create(None, None) == 1


def test_long_error_message_is_truncated(bkma):
    """The error text lives in a fixed per-thread buffer: an unknown name of
    5000 characters gives the error status and a message cut to 1023 bytes."""
    with pytest.raises(bkma.BkmaError) as e:
        bkma.impl_from_name("x" * 5000)
    assert e.value.status == 2
    assert len(bkma.load().bkma_last_error()) == 1023


_OOM_CHILD = r"""
import resource, sys
sys.path.insert(0, sys.argv[1])
import bkma_gb300
from bkma_gb300 import _lib
bkma_gb300.load()
vm = [l for l in open("/proc/self/status") if l.startswith("VmSize:")][0].split()[1]
lim = int(vm) * 1024 + (1 << 30)  # 1 GiB above the current address space
resource.setrlimit(resource.RLIMIT_AS, (lim, resource.getrlimit(resource.RLIMIT_AS)[1]))
try:
    bkma_gb300.AdvectionPlan(2**30, 64, 1, dtype="f32")  # 4 GiB of line tables first
except bkma_gb300.BkmaError as e:
    print("STATUS", e.status, str(e))
    sys.exit(0)
print("NO ERROR")
"""


def test_host_allocation_failure_is_a_status(bkma):
    """A plan whose host-side line tables cannot be allocated returns
    BKMA_ERR_HOST through the C ABI (no C++ exception reaches the caller).
    The child process caps its address space, so the allocation fails at once
    and no memory is touched."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-c", _OOM_CHILD, os.path.join(ROOT, "parallel-advection_gb300")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "STATUS 6 BKMA_ERR_HOST: bkma_adv_plan_create: " in r.stdout, r.stdout + r.stderr[-2000:]


def test_tensor_arguments_are_checked_before_any_launch(bkma):
    """The Python mirror refuses what a kernel would read out of bounds:
    host tensors and arrays (the device checks are in the GPU tests). Raw
    integer addresses and None pass through, as through the C ABI."""
    import numpy as np
    import torch
    from bkma_gb300 import _dev
    for bad in (torch.zeros(4), np.zeros(4, dtype=np.float32)):
        with pytest.raises(bkma.BkmaError) as e:
            _dev(bad, "data", "f32", 4)
        assert e.value.status == 1 and "data: not a CUDA tensor" in str(e.value)
    assert _dev(None, "out") is None
    assert _dev(4096, "data", "f32", 1 << 20) == 4096


def test_host_array_checks_need_no_device(bkma):
    """run_host refuses a mistyped or misshapen host array before the C ABI
    is called (an object without a plan handle shows no call is made)."""
    import numpy as np
    plan = bkma.AdvectionPlan.__new__(bkma.AdvectionPlan)
    plan.dtype, plan.lines, plan.n1, plan.n2, plan._h = "f32", 4, 16, 2, None
    for bad in (np.zeros((4, 16, 2)), np.zeros((4, 16, 3), dtype=np.float32),
                np.zeros((4, 2, 16), dtype=np.float32).transpose(0, 2, 1)):
        with pytest.raises(bkma.BkmaError) as e:
            plan.run_host(bad)
        assert e.value.status == 1 and "(4, 16, 2)" in str(e.value)


_C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "bkma_gb300.h"

int main(void) {
    int32_t impl = -1, inplace = -1;
    bkma_adv_plan *plan = NULL;
    bkma_adv_desc d;
    if (bkma_abi_version() != BKMA_ABI_VERSION) return 1;
    if (bkma_impl_from_name("AdaptiveWg", &impl, &inplace) != BKMA_OK) return 2;
    if (impl != BKMA_ADV_STAGED || inplace != 1) return 3;
    if (bkma_impl_from_name("Hierarchical", &impl, &inplace) != BKMA_ERR_UNSUPPORTED) return 4;
    if (strstr(bkma_last_error(), "not a valid implementation name") == NULL) return 5;
    memset(&d, 0, sizeof d);
    d.n0 = 0; /* invalid: refused before any device work */
    if (bkma_adv_plan_create(&d, &plan) != BKMA_ERR_INVALID_ARG || plan != NULL) return 6;
    printf("ok\n");
    return 0;
}
"""


def test_header_is_c_and_links_from_c(bkma, tmp_path):
    """include/bkma_gb300.h compiles as C99 (-Wall -Werror -pedantic) and a C
    program links against the library and calls the entry points that need
    no GPU, with the documented statuses."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from bkma_gb300 import _lib
    libdir = os.path.dirname(_lib.LIB_PATH)
    src = tmp_path / "caller.c"
    src.write_text(_C_CALLER)
    exe = tmp_path / "caller"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-lbkma_gb300", f"-Wl,-rpath,{libdir}"],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
