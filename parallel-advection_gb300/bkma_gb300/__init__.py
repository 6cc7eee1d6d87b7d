"""bkma_gb300: GB300-native BKMA hot paths (semi-Lagrangian advection and
in-place conv1d) behind the C ABI of include/bkma_gb300.h.

Python front-end over libbkma_gb300.so (ctypes). Device buffers are torch
CUDA tensors (torch is the allocator and stream provider only); every
computation runs in the library's CUDA kernels. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import BkmaError, check, load  # noqa: F401

_DT = {"f32": _lib.BKMA_F32, "f64": _lib.BKMA_F64, "bf16": _lib.BKMA_BF16}
_IMPL = {"auto": _lib.BKMA_ADV_AUTO, "staged": _lib.BKMA_ADV_STAGED, "plain": _lib.BKMA_ADV_PLAIN}
_W = {"reference": _lib.BKMA_W_REFERENCE, "lagrange": _lib.BKMA_W_LAGRANGE,
      "table": _lib.BKMA_W_TABLE}


def _dev(t, name: str, dtype: str | None = None, numel: int | None = None) -> int | None:
    """Device address of a tensor argument, after the checks a kernel cannot
    make on a raw pointer: a CUDA tensor on the current device, contiguous, of
    `dtype`, with at least `numel` elements (a host, short or mistyped buffer
    would be read or written out of bounds on the GPU). None stays None; an
    integer is a raw device address the caller vouches for, as through the C
    ABI itself."""
    if t is None or isinstance(t, int):
        return t

    def bad(why):
        return BkmaError(_lib.BKMA_ERR_INVALID_ARG, f"{name}: {why}")
    if not getattr(t, "is_cuda", False):
        raise bad("not a CUDA tensor (the library runs on the GPU only)")
    import torch
    if t.device.index != torch.cuda.current_device():
        raise bad(f"on {t.device}, but the current device is cuda:{torch.cuda.current_device()}")
    if not t.is_contiguous():
        raise bad("not contiguous")
    if dtype is not None and _dtype_name(t) != dtype:
        raise bad(f"dtype {t.dtype}, the plan computes in {dtype}")
    if numel is not None and t.numel() < numel:
        raise bad(f"{t.numel()} elements, {numel} needed")
    return t.data_ptr()


def _stream(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def shard_lines(n0: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous slab of velocity lines for one rank: (i0_offset, i0_count).
    Lines are independent, so shards need no exchange; the first n0 % world
    ranks take one extra line."""
    if world < 1 or not (0 <= rank < world) or n0 < world:
        raise ValueError("need world >= 1, 0 <= rank < world and n0 >= world")
    base, extra = divmod(n0, world)
    offset = rank * base + min(rank, extra)
    return offset, base + (1 if rank < extra else 0)


def fill(data, value: float, stream=None):
    """fill_buffer_conv1d's constant fill of a CUDA tensor (F32/F64/BF16)."""
    check(load().bkma_fill(_dev(data, "data"), data.numel(), _DT[_dtype_name(data)], value,
                           _stream(stream)))
    return data


def conv_check(data, nw: int, stream=None) -> tuple[float, bool]:
    """sum_and_normalize_conv1d + validate_conv1d on a (n0, n1, n2) CUDA
    tensor: (mean of the first nw values per line, all equal per i1)."""
    n0, n1, n2 = data.shape
    mean, equal = C.c_double(), C.c_int32()
    check(load().bkma_conv_check(_dev(data, "data"), _DT[_dtype_name(data)], n0, n1, n2, nw,
                                 C.byref(mean), C.byref(equal), _stream(stream)))
    return mean.value, bool(equal.value)


def impl_from_name(name: str) -> tuple[int, bool]:
    """impl_selector (src/tools/impl_selector.hpp:31-49) over the C ABI."""
    impl, inplace = C.c_int32(), C.c_int32()
    check(load().bkma_impl_from_name(name.encode(), C.byref(impl), C.byref(inplace)))
    return impl.value, bool(inplace.value)


class AdvectionPlan:
    """AdvectionSolver + create_optim_params (src/solvers/AdvectionSolver.hpp,
    src/tools/init.hpp:76-102): per-line FP64 departure and weights, tile
    choice; `step` is bkma_run (src/core/bkma_run.hpp:10-62)."""

    def __init__(self, n0: int, n1: int, n2: int, *, dtype: str = "f32", degree: int = 5,
                 weights: str = "reference", impl: str = "auto", dt: float = 1e-4,
                 minX: float = 0.0, maxX: float = 1.0, minVx: float = 0.0, maxVx: float = 1.0,
                 velocity=None, i0_offset: int = 0, i0_count: int = 0, inplace: bool = True):
        lib = load()
        self.dtype = dtype
        d = _lib.AdvDesc()
        d.n0, d.n1, d.n2 = n0, n1, n2
        d.i0_offset, d.i0_count = i0_offset, i0_count
        d.dtype, d.degree, d.weights = _DT[dtype], degree, _W[weights]
        d.impl, d.inplace = (_IMPL[impl] if isinstance(impl, str) else impl), int(inplace)
        d.dt, d.minX, d.maxX, d.minVx, d.maxVx = dt, minX, maxX, minVx, maxVx
        self._vel = None
        if velocity is not None:
            self._vel = np.ascontiguousarray(velocity, dtype=np.float64)
            d.velocity = self._vel.ctypes.data_as(C.POINTER(C.c_double))
        self.desc = d
        self.n0, self.n1, self.n2 = n0, n1, n2
        self.lines = i0_count or (n0 - i0_offset)
        h = C.c_void_p()
        check(lib.bkma_adv_plan_create(C.byref(d), C.byref(h)))
        self._h = h

    @property
    def shape(self):
        return (self.lines, self.n1, self.n2)

    def info(self) -> dict:
        i = _lib.AdvPlanInfo()
        check(load().bkma_adv_plan_info_get(self._h, C.byref(i)))
        return {n: getattr(i, n) for n, _ in i._fields_}

    def step(self, data, out=None, nsteps: int = 1, stream=None):
        n = self.lines * self.n1 * self.n2
        check(load().bkma_adv_step(self._h, _dev(data, "data", self.dtype, n),
                                   _dev(out, "out", self.dtype, n), nsteps, _stream(stream)))
        return data if out is None else out

    def run_host(self, host: np.ndarray, nsteps: int = 1, stream=None) -> np.ndarray:
        want = np.float32 if self.dtype == "f32" else np.float64
        if not (isinstance(host, np.ndarray) and host.dtype == want and host.flags["C_CONTIGUOUS"]
                and host.shape == self.shape):
            raise BkmaError(_lib.BKMA_ERR_INVALID_ARG,
                            f"host: a C-contiguous {np.dtype(want).name} array of shape "
                            f"{self.shape} is needed")
        check(load().bkma_adv_run_host(self._h, host.ctypes.data, nsteps, _stream(stream)))
        return host

    def _field(self, t, name: str) -> int | None:
        return _dev(t, name, self.dtype, self.lines * self.n1 * self.n2)

    def set_tile(self, W: int, R: int = 1, threads: int = 256, path: int = 0):
        check(load().bkma_adv_plan_set_tile(self._h, W, R, threads, path))
        return self.info()

    def status(self, stream=None):
        """Raise if a bounded device wait timed out since the last query."""
        check(load().bkma_adv_plan_status(self._h, _stream(stream)))

    def set_wait_limit(self, polls: int):
        """Polls of each bounded device wait before it gives up (0: at once)."""
        check(load().bkma_adv_plan_set_wait_limit(self._h, polls))

    def set_fusion(self, steps_per_launch: int):
        """Time steps per kernel launch (shared-memory strips; 1 = off)."""
        check(load().bkma_adv_plan_set_fusion(self._h, steps_per_launch))

    def set_fused_state(self, state: str):
        """On-chip state of fused steps: "f32" (bit-identical to one step
        per launch) or "f32x2" (hi + lo FP32 pair, one FP32 rounding per
        launch)."""
        check(load().bkma_adv_plan_set_fused_state(self._h, {"f32": 0, "f32x2": 1}[state]))

    def autotune(self, field, stream=None):
        check(load().bkma_adv_plan_autotune(self._h, self._field(field, "field"),
                                            _stream(stream)))
        return self.info()

    def fill(self, data, mode: int = 0, amp: float = 0.0, seed: int = 0, stream=None):
        check(load().bkma_adv_fill(self._h, self._field(data, "data"), mode, amp, seed,
                                   _stream(stream)))
        return data

    def error_norms(self, data, ref, stream=None) -> dict:
        out = (C.c_double * 4)()
        dd = _DT[_dtype_name(data)]
        rd = _DT[_dtype_name(ref)]
        n = self.lines * self.n1 * self.n2
        check(load().bkma_adv_error_norms(self._h, _dev(data, "data", None, n), dd,
                                          _dev(ref, "ref", None, n), rd, out,
                                          _stream(stream)))
        maxabs, maxref, se, sr = list(out)
        return {"max_abs": maxabs, "max_ref": maxref,
                "max_rel": maxabs / maxref if maxref else 0.0,
                "l2_rel": (se / sr) ** 0.5 if sr else 0.0}

    def validate(self, data, max_iter: int, stream=None) -> tuple[float, float]:
        hi, lo = C.c_double(), C.c_double()
        check(load().bkma_adv_validate(self._h, self._field(data, "data"), max_iter,
                                       C.byref(hi), C.byref(lo),
                                       _stream(stream)))
        return hi.value, lo.value

    def line_table(self) -> tuple[np.ndarray, np.ndarray]:
        off = np.zeros(self.lines, dtype=np.int32)
        sh = np.zeros(self.lines, dtype=np.float64)
        check(load().bkma_adv_plan_line_table(
            self._h, off.ctypes.data_as(C.POINTER(C.c_int32)),
            sh.ctypes.data_as(C.POINTER(C.c_double))))
        return off, sh

    def set_weights(self, weights, on_device: bool | None = None):
        if isinstance(weights, np.ndarray):
            w = np.ascontiguousarray(weights, dtype=np.float32)
            check(load().bkma_adv_plan_set_weights(self._h, w.ctypes.data, 0))
        else:
            n = self.lines * (self.desc.degree + 1)
            check(load().bkma_adv_plan_set_weights(self._h, _dev(weights, "weights", "f32", n), 1))

    def close(self):
        if getattr(self, "_h", None):
            load().bkma_adv_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AdvectionBatch:
    """Many independent fields advanced by one persistent, graph-captured
    launch per step. `fields`: dicts with keys data (CUDA tensor n0 x n1 x n2),
    degree (3 or 5), weights ("reference" for degree 5, "lagrange"), dt, minX,
    maxX, minVx, maxVx, velocity (optional array of n0)."""

    def __init__(self, fields, dtype: str = "f32"):
        arr = (_lib.AdvField * len(fields))()
        self._keep = []
        self.cells = 0
        for i, f in enumerate(fields):
            t = f["data"]
            n0, n1, n2 = t.shape
            a = arr[i]
            if len(t.shape) != 3:
                raise BkmaError(_lib.BKMA_ERR_INVALID_ARG, f"field {i}: data must be n0 x n1 x n2")
            a.data = _dev(t, f"field {i}", dtype)
            a.n0, a.n1, a.n2 = n0, n1, n2
            a.degree = f.get("degree", 5)
            a.weights = _W[f.get("weights", "reference" if a.degree == 5 else "lagrange")]
            a.dt = f.get("dt", 1e-3)
            a.minX, a.maxX = f.get("minX", 0.0), f.get("maxX", 1.0)
            a.minVx, a.maxVx = f.get("minVx", -1.0), f.get("maxVx", 1.0)
            v = f.get("velocity")
            if v is not None:
                v = np.ascontiguousarray(v, dtype=np.float64)
                self._keep.append(v)
                a.velocity = v.ctypes.data_as(C.POINTER(C.c_double))
            self._keep.append(t)
            self.cells += n0 * n1 * n2
        self.nfields = len(fields)
        h = C.c_void_p()
        check(load().bkma_adv_batch_create(arr, len(fields), _DT[dtype], C.byref(h)))
        self._h = h

    def step(self, nsteps: int = 1, stream=None):
        check(load().bkma_adv_batch_step(self._h, nsteps, _stream(stream)))

    def autotune(self, stream=None):
        check(load().bkma_adv_batch_autotune(self._h, _stream(stream)))
        return self.tiles()

    def launches_per_step(self) -> int:
        """Kernel launches in one step's graph (staged + streamed groups)."""
        cells, launches = C.c_int64(), C.c_int32()
        check(load().bkma_adv_batch_info(self._h, C.byref(cells), C.byref(launches)))
        return launches.value

    def tiles(self) -> dict:
        W = (C.c_int32 * self.nfields)()
        R = (C.c_int32 * self.nfields)()
        nt, th, sm = C.c_int64(), C.c_int32(), C.c_int64()
        check(load().bkma_adv_batch_tiles(self._h, W, R, C.byref(nt), C.byref(th), C.byref(sm)))
        return {"W": list(W), "R": list(R), "tiles": nt.value, "threads": th.value,
                "smem_bytes": sm.value}

    def close(self):
        if getattr(self, "_h", None):
            load().bkma_adv_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LearnedStencil:
    """Learned stencil of 4 or 6 points (bkma_mlp_*): training data, training,
    gradient and inference all run in the library's CUDA kernels."""

    NP = 1252  # parameters of a 4-point model

    def __init__(self, seed: int = 0, npts: int = 4):
        h = C.c_void_p()
        check(load().bkma_mlp_create_stencil(seed, npts, C.byref(h)))
        self._h = h
        k, n = C.c_int32(), C.c_int32()
        check(load().bkma_mlp_info(h, C.byref(k), C.byref(n)))
        self.npts, self.NP = k.value, n.value

    @staticmethod
    def samples(n: int, seed: int, first: int = 0, device=None, n1: int = 1024, npts: int = 4,
                exact: bool = False):
        """Training samples (alpha[n], taps[n][npts], target[n]) of random
        periodic lines sampled on n1 cells; the target is the degree-9
        Lagrange value, or with exact=True the line's own value."""
        import torch
        dev = device or torch.device("cuda", torch.cuda.current_device())
        a = torch.empty(n, dtype=torch.float32, device=dev)
        f = torch.empty(n, npts, dtype=torch.float32, device=dev)
        t = torch.empty(n, dtype=torch.float32, device=dev)
        check(load().bkma_mlp_samples_grid(n, seed, first, n1, npts, int(exact), a.data_ptr(),
                                           f.data_ptr(), t.data_ptr(), _stream(None)))
        return a, f, t

    def params(self) -> np.ndarray:
        p = np.zeros(self.NP, dtype=np.float32)
        check(load().bkma_mlp_params(self._h, p.ctypes.data, 0))
        return p

    def set_params(self, p):
        q = np.ascontiguousarray(p, dtype=np.float32)
        if q.shape != (self.NP,):
            raise BkmaError(_lib.BKMA_ERR_INVALID_ARG, f"params: {self.NP} values needed")
        check(load().bkma_mlp_params(self._h, q.ctypes.data, 1))

    def _samples(self, a, f, t) -> tuple[int, int, int]:
        n = a.numel()
        return (_dev(a, "alpha", "f32"), _dev(f, "taps", "f32", self.npts * n),
                _dev(t, "target", "f32", n))

    def grad(self, a, f, t) -> tuple[float, np.ndarray]:
        g = np.zeros(self.NP, dtype=np.float32)
        loss = C.c_double()
        check(load().bkma_mlp_grad(self._h, *self._samples(a, f, t), a.numel(),
                                   g.ctypes.data, C.byref(loss), _stream(None)))
        return loss.value, g

    def train(self, a, f, t, steps: int, batch: int = 4096, lr: float = 3e-3,
              seed: int = 1) -> float:
        loss = C.c_double()
        check(load().bkma_mlp_train(self._h, *self._samples(a, f, t), a.numel(),
                                    steps, batch, lr, seed, C.byref(loss), _stream(None)))
        return loss.value

    def infer(self, alpha):
        import torch
        out = torch.empty(alpha.numel(), self.npts, dtype=torch.float32, device=alpha.device)
        check(load().bkma_mlp_infer(self._h, _dev(alpha, "alpha", "f32"), alpha.numel(),
                                    out.data_ptr(),
                                    _stream(None)))
        return out

    def plan_for(self, n0: int, n1: int, n2: int, **kw) -> "AdvectionPlan":
        """An FP32 advection plan whose per-line weights come from the network
        (the Lagrange tap layout of degree npts - 1, the plan's own departure
        offsets)."""
        import torch
        plan = AdvectionPlan(n0, n1, n2, dtype="f32", degree=self.npts - 1, weights="table", **kw)
        _, shifts = plan.line_table()
        a = torch.tensor(shifts, dtype=torch.float32, device="cuda")
        w = self.infer(a)
        plan.set_weights(w)
        torch.cuda.synchronize()
        return plan

    def close(self):
        if getattr(self, "_h", None):
            load().bkma_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _dtype_name(t) -> str:
    s = str(t.dtype)
    if "float32" in s:
        return "f32"
    if "float64" in s:
        return "f64"
    if "bfloat16" in s:
        return "bf16"
    raise ValueError(f"unsupported dtype {t.dtype}")


class Conv1dPlan:
    """ConvSolver + bkma_run for conv1d (src/solvers/ConvSolver.hpp,
    src/conv1d.cpp:52-87)."""

    def __init__(self, batch: int, cin: int, cout: int, length: int, ksize: int, *,
                 dtype: str = "bf16", semantics: str = "torch", impl: str = "auto",
                 inplace: bool = True, n2: int = 1):
        d = _lib.ConvDesc()
        d.batch, d.cin, d.cout, d.length, d.ksize, d.n2 = batch, cin, cout, length, ksize, n2
        d.dtype = _DT[dtype]
        d.semantics = {"torch": _lib.BKMA_CONV_TORCH, "reference": _lib.BKMA_CONV_REFERENCE}[semantics]
        d.impl = {"auto": _lib.BKMA_CONV_AUTO, "tensor": _lib.BKMA_CONV_TENSOR,
                  "plain": _lib.BKMA_CONV_PLAIN}[impl]
        d.inplace = int(inplace)
        self.desc = d
        self.dtype, self.semantics = dtype, semantics
        h = C.c_void_p()
        check(load().bkma_conv_plan_create(C.byref(d), C.byref(h)))
        self._h = h

    def scratch_bytes(self) -> int:
        b = C.c_int64()
        check(load().bkma_conv_plan_scratch_bytes(self._h, C.byref(b)))
        return b.value

    def run(self, data, weight, bias=None, out=None, stream=None):
        d = self.desc
        dt = self.dtype
        if self.semantics == "reference":
            n_x = n_out = d.batch * d.cin * d.length * d.n2
        else:
            n_x = d.batch * d.cin * d.length
            n_out = d.batch * d.cout * (d.length - d.ksize + 1)
        check(load().bkma_conv_run(self._h, _dev(data, "data", dt, n_x),
                                   _dev(out, "out", dt, n_out),
                                   _dev(weight, "weight", dt, d.cout * d.cin * d.ksize),
                                   _dev(bias, "bias", dt, d.cout), _stream(stream)))
        return data if out is None else out

    def status(self, stream=None):
        """Raise if a bounded device wait of the tensor kernel timed out."""
        check(load().bkma_conv_plan_status(self._h, _stream(stream)))

    def set_wait_limit(self, polls: int):
        """Polls of each bounded device wait before it gives up (0: at once)."""
        check(load().bkma_conv_plan_set_wait_limit(self._h, polls))

    def close(self):
        if getattr(self, "_h", None):
            load().bkma_conv_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
