"""Generate the golden fixtures in tests/golden/ from the reference's OWN code.

Runs only where the reference checkout exists (BKMA_REFERENCE_DIR, or the
directory oracle/build_ref.sh found it in): it builds
oracle/_ref/libbkma_ref.so (the reference's
AdvectionSolver, ConvSolver, ConfigMap/ADVParams/Conv1dParams compiled on the
CPU with oracle/ref_shim) and records what that code outputs. The committed
.npz/.json files are what tests/test_oracle_golden.py checks the oracle
restatement against; nothing at test time needs the reference.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from oracle import AdvParams, Reference, build_ref, reference_dir  # noqa: E402

# INI texts exercising the reference parser: strtof rounding of reals,
# base-0 strtol (hex), ';' inline comments vs '#' kept in values,
# case-insensitive keys, continuation lines, booleans, defaults.
INI_CASES = {
    "adv_plain": """[problem]
n0 = 512
n1 = 1024
n2 = 1
maxIter = 10
dt = 0.001
minRealX = 0
maxRealX = 1
minRealVx = -1
maxRealVx = 1
[impl]
kernelImpl = NDRange
inplace = false
[optimization]
gpu = yes
pref_wg_size = 0x80
""",
    "adv_quirks": """# leading comment
; another
[Problem]
N0 = 96 # hash is not a comment here, strtol stops at the space
n1 = 1000 ; semicolon after whitespace is a comment
n2 = 7
maxIter = 3
dt = 0.1
minRealX = -0.5
maxRealX = 2.5
minRealVx = -3
maxRealVx = 3.3
[impl]
kernelImpl = adaptivewg
inplace = off
[optimization]
gpu = 0
seq_size0 = 2
""",
    "adv_defaults": """[problem]
n1 = 256
""",
    "adv_continuation": """[problem]
n0 = 8
dt = 0.5
  0.25
n2 = abc
""",
    "conv_custom": """[problem]
length = 64
channel_in = 5
channel_out = 9
k = 7
total_batch_size = 4096
batch_size_n2 = 16
[impl]
kernelImpl = AdaptiveWg
inplace = true
""",
}


def main():
    so = build_ref()
    REF_DIR = reference_dir()
    if not so or not REF_DIR:
        raise SystemExit("reference sources not found; cannot regenerate fixtures")
    ref = Reference(so)
    out_json = {}

    # ---- .ini parsing through ConfigMap + ADVParams/Conv1dParams setup
    out_json["advection.ini"] = ref.adv_params_from_ini(os.path.join(REF_DIR, "src/advection.ini"))
    out_json["conv1d.ini"] = ref.conv_params_from_ini(os.path.join(REF_DIR, "src/conv1d.ini"))
    out_json["adv_default_ctor"] = ref.adv_params_default()
    with tempfile.TemporaryDirectory() as td:
        for name, text in INI_CASES.items():
            p = os.path.join(td, name + ".ini")
            with open(p, "w") as f:
                f.write(text)
            if name.startswith("conv"):
                out_json["ini:" + name] = {"text": text, "parsed": ref.conv_params_from_ini(p)}
            else:
                out_json["ini:" + name] = {"text": text, "parsed": ref.adv_params_from_ini(p)}
    with open(os.path.join(HERE, "params.json"), "w") as f:
        json.dump(out_json, f, indent=1, sort_keys=True)

    rng = np.random.default_rng(20240601)
    arrays = {}

    # ---- lag_basis at fixed points
    px = np.concatenate([[2.0, 2.5, 2.999999999999], rng.uniform(2.0, 3.0, 61)])
    arrays["lag_px"] = px
    arrays["lag_coef"] = np.stack([ref.lag_basis(float(x)) for x in px])

    # ---- stencils (departure cell + weights) of AdvectionSolver::operator()
    stencil_cases = [
        # n0, n1, dt, minX, maxX, minVx, maxVx
        (8, 64, 0.001, 0.0, 1.0, -1.0, 1.0),
        (6, 1000, 0.0010000000474974513, 0.0, 1.0, -1.0, 1.0),
        (5, 999, 0.37, -0.5, 2.5, -3.0, 3.3),          # CFL >> 1, wraps
        (4, 128, 0.5, 0.0, 1.0, -4.0, 4.0),             # shift of many periods
        (3, 100, 1e-4, 0.0, 1.0, 0.0, 1.0),             # default-like
    ]
    # Each point's stencil is stored sparse: the nodes with a non-zero weight
    # (sorted, padded with -1) and those weights. Weights can be exactly 0
    # (a foot point on a node), so the tap window is not recovered here; the
    # test rebuilds the same sparse form from the oracle's departure cell.
    st_meta, st_nodes, st_vals = [], [], []
    for ci, (n0, n1, dt, mnx, mxx, mnv, mxv) in enumerate(stencil_cases):
        p = AdvParams(n0=n0, n1=n1, n2=1, dt=dt, minX=mnx, maxX=mxx, minVx=mnv, maxVx=mxv)
        for i0 in range(n0):
            for i1 in range(n1):
                w = ref.adv_stencil(p, i0, i1)
                nz = np.nonzero(w)[0]
                assert len(nz) <= 6
                nodes = np.full(6, -1, dtype=np.int64)
                vals = np.zeros(6)
                nodes[:len(nz)] = nz
                vals[:len(nz)] = w[nz]
                st_meta.append((ci, i0, i1))
                st_nodes.append(nodes)
                st_vals.append(vals)
    arrays["stencil_cases"] = np.array(stencil_cases, dtype=np.float64)
    arrays["stencil_meta"] = np.array(st_meta, dtype=np.int64)
    arrays["stencil_nodes"] = np.array(st_nodes, dtype=np.int64)
    arrays["stencil_vals"] = np.array(st_vals, dtype=np.float64)

    # ---- whole-field advection runs (AdaptiveWg schedule around the solver)
    adv_cases = {
        "small": dict(n0=8, n1=64, n2=3, dt=0.0010000000474974513, minVx=-1.0, maxVx=1.0,
                      steps=[1, 2, 5]),
        "odd": dict(n0=5, n1=999, n2=2, dt=0.37, minX=-0.5, maxX=2.5, minVx=-3.0, maxVx=3.3,
                    steps=[1, 3]),
        "default": dict(n0=16, n1=1024, n2=1, dt=1e-4, minVx=0.0, maxVx=1.0, steps=[10]),
    }
    for name, c in adv_cases.items():
        steps = c.pop("steps")
        p = AdvParams(**c)
        d = p.c  # noqa
        x = np.arange(p.n1) * ((p.maxX - p.minX) / p.n1) + p.minX
        f0 = np.sin(4 * np.pi * x)[None, :, None] + 0.01 * rng.standard_normal((p.n0, p.n1, p.n2))
        f0 = np.ascontiguousarray(f0)
        arrays[f"adv_{name}_params"] = np.array([p.n0, p.n1, p.n2, p.dt, p.minX, p.maxX,
                                                 p.minVx, p.maxVx])
        arrays[f"adv_{name}_init"] = f0
        cur = f0.copy()
        done = 0
        for s in steps:
            ref.adv_step(p, cur, s - done)
            done = s
            arrays[f"adv_{name}_step{s}"] = cur.copy()

    # ---- conv1d through ConvSolver + AdaptiveWg packing
    conv_cases = {
        "rand": dict(n0=3, C=3, L=16, n2=2, K=3),
        "wide": dict(n0=2, C=4, L=40, n2=5, K=7),
    }
    for name, c in conv_cases.items():
        n1 = c["C"] * c["L"]
        data = rng.standard_normal((c["n0"], n1, c["n2"]))
        w = rng.standard_normal((c["K"], c["C"], c["C"]))
        b = rng.standard_normal(c["C"])
        arrays[f"conv_{name}_meta"] = np.array([c["n0"], c["C"], c["L"], c["n2"], c["K"]])
        arrays[f"conv_{name}_in"] = data.copy()
        arrays[f"conv_{name}_w"] = w
        arrays[f"conv_{name}_b"] = b
        ref.conv_step(data, w, b, c["K"], c["C"], c["L"])
        arrays[f"conv_{name}_out"] = data
    # constant fills of fill_buffer_conv1d (src/tools/init.hpp:50-72)
    n0, C, L, n2, K = 2, 3, 32, 2, 3
    data = np.full((n0, C * L, n2), 7.3)
    w = np.full((K, C, C), 1.5)
    b = np.full(C, 1.0)
    ref.conv_step(data, w, b, K, C, L)
    arrays["conv_const_meta"] = np.array([n0, C, L, n2, K])
    arrays["conv_const_out"] = data

    np.savez_compressed(os.path.join(HERE, "reference_vectors.npz"), **arrays)
    total = sum(a.nbytes for a in arrays.values())
    print(f"wrote {len(arrays)} arrays ({total/1e6:.2f} MB raw) and params.json")


if __name__ == "__main__":
    main()
