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
