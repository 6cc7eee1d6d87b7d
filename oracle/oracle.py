"""ctypes front-end for the CPU oracle (oracle/libbkma_oracle.so) and, when it
has been built in this checkout, for the reference's own solver code
(oracle/_ref/libbkma_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's cpu_baseline / reference arm, always as the checker or the CPU
baseline. The product library never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libbkma_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libbkma_ref.so")

_dp = C.POINTER(C.c_double)


def build(force: bool = False) -> str:
    """Compile the C restatement with make (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < max(
        os.path.getmtime(os.path.join(HERE, f)) for f in ("bkma_oracle.c", "bkma_oracle.h")
    ):
        subprocess.run(["make", "-s", "-C", HERE, "libbkma_oracle.so"], check=True)
    return ORACLE_SO


def reference_dir() -> str | None:
    """The reference checkout's root: BKMA_REFERENCE_DIR when set, else the
    directory build_ref.sh compiled from (recorded in _ref/reference_dir.txt),
    else None (no checkout on this machine)."""
    env = os.environ.get("BKMA_REFERENCE_DIR")
    if env:
        return env if os.path.isdir(env) else None
    rec = os.path.join(HERE, "_ref", "reference_dir.txt")
    if os.path.exists(rec):
        d = open(rec).read().strip()
        return d if os.path.isdir(d) else None
    return None


def build_ref() -> str | None:
    """Compile the reference's solver/config sources (only where they exist)."""
    subprocess.run([os.path.join(HERE, "build_ref.sh")], check=True,
                   stdout=subprocess.DEVNULL)
    return REF_SO if os.path.exists(REF_SO) else None


class _AdvParamsC(C.Structure):
    _fields_ = [("n0", C.c_int64), ("n1", C.c_int64), ("n2", C.c_int64),
                ("dt", C.c_double), ("minX", C.c_double), ("maxX", C.c_double),
                ("minVx", C.c_double), ("maxVx", C.c_double),
                ("width", C.c_double), ("dx", C.c_double), ("dvx", C.c_double),
                ("inv_dx", C.c_double)]


@dataclass
class AdvParams:
    """Mirror of the reference ADVParams physical fields
    (src/config/AdvectionParams.hpp:10-57)."""
    n0: int = 32
    n1: int = 1024
    n2: int = 32
    dt: float = 0.0001
    minX: float = 0.0
    maxX: float = 1.0
    minVx: float = 0.0
    maxVx: float = 1.0
    derived: dict = field(default_factory=dict)

    def c(self, lib) -> _AdvParamsC:
        p = _AdvParamsC(self.n0, self.n1, self.n2, self.dt, self.minX, self.maxX,
                        self.minVx, self.maxVx, 0, 0, 0, 0)
        lib.bko_adv_update_deltas(C.byref(p))
        self.derived = dict(width=p.width, dx=p.dx, dvx=p.dvx, inv_dx=p.inv_dx)
        return p


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


class Oracle:
    def __init__(self, path: str | None = None):
        self.lib = C.CDLL(path or build())
        L = self.lib
        L.bko_adv_update_deltas.argtypes = [C.POINTER(_AdvParamsC)]
        L.bko_coord.restype = C.c_double
        L.bko_coord.argtypes = [C.c_int, C.c_double, C.c_double]
        L.bko_lag_basis_ref5.argtypes = [C.c_double, _dp]
        L.bko_lag_basis_textbook.argtypes = [C.c_int, C.c_double, _dp]
        L.bko_displ_v.restype = C.c_double
        L.bko_displ_v.argtypes = [C.POINTER(_AdvParamsC), C.c_int, C.c_double]
        L.bko_line_velocity.restype = C.c_double
        L.bko_line_velocity.argtypes = [C.POINTER(_AdvParamsC), C.c_int64]
        L.bko_departure.restype = C.c_int
        L.bko_departure.argtypes = [C.POINTER(_AdvParamsC), C.c_int, C.c_double, _dp]
        L.bko_adv_step.argtypes = [C.POINTER(_AdvParamsC), _dp, C.c_int64, C.c_int64,
                                   _dp, C.c_int, C.c_int, C.c_int]
        L.bko_fill_adv.argtypes = [C.POINTER(_AdvParamsC), _dp]
        L.bko_validate_adv.restype = C.c_double
        L.bko_validate_adv.argtypes = [C.POINTER(_AdvParamsC), _dp, C.c_int64]
        L.bko_conv_ref_step.argtypes = [_dp, C.c_int64, C.c_int64, C.c_int64, _dp, _dp,
                                        C.c_int64, C.c_int64, C.c_int64, C.c_int]
        L.bko_conv_torch.argtypes = [_dp, _dp, C.c_int64, C.c_int64, C.c_int64,
                                     C.c_int64, C.c_int64, _dp, _dp, C.c_int]
        L.bko_uniform.restype = C.c_double
        L.bko_uniform.argtypes = [C.c_uint64, C.c_uint64]

    # ---- advection -------------------------------------------------------
    def lag_basis_ref5(self, px: float) -> np.ndarray:
        c = np.zeros(6)
        self.lib.bko_lag_basis_ref5(px, _ptr(c))
        return c

    def lag_basis_textbook(self, npts: int, px: float) -> np.ndarray:
        c = np.zeros(npts)
        self.lib.bko_lag_basis_textbook(npts, px, _ptr(c))
        return c

    def line_velocity(self, p: AdvParams, i0: int) -> float:
        return self.lib.bko_line_velocity(C.byref(p.c(self.lib)), i0)

    def departure(self, p: AdvParams, i1: int, vx: float):
        d = C.c_double(0)
        left = self.lib.bko_departure(C.byref(p.c(self.lib)), i1, vx, C.byref(d))
        return left, d.value

    def adv_step(self, p: AdvParams, data: np.ndarray, nsteps: int = 1, *,
                 i0_offset: int = 0, velocity: np.ndarray | None = None,
                 degree: int = 5, ref_weights: bool = True, nthreads: int = 0):
        """nsteps in-place steps of the FP64 field data[n0_local][n1][n2]."""
        pc = p.c(self.lib)
        assert data.shape[1:] == (p.n1, p.n2)
        vel = None
        if velocity is not None:
            vel = np.ascontiguousarray(velocity, dtype=np.float64)
            assert vel.shape == (data.shape[0],)
        for _ in range(nsteps):
            self.lib.bko_adv_step(C.byref(pc), _ptr(data), data.shape[0], i0_offset,
                                  _ptr(vel) if vel is not None else None, degree,
                                  int(ref_weights), nthreads)
        return data

    def fill_adv(self, p: AdvParams) -> np.ndarray:
        a = np.zeros((p.n0, p.n1, p.n2))
        self.lib.bko_fill_adv(C.byref(p.c(self.lib)), _ptr(a))
        return a

    def validate_adv(self, p: AdvParams, data: np.ndarray, max_iter: int) -> float:
        return self.lib.bko_validate_adv(C.byref(p.c(self.lib)), _ptr(data), max_iter)

    # ---- conv1d ----------------------------------------------------------
    def conv_ref_step(self, data: np.ndarray, weight: np.ndarray, bias: np.ndarray,
                      K: int, cin: int, length: int, nthreads: int = 0):
        n0, n1, n2 = data.shape
        self.lib.bko_conv_ref_step(_ptr(data), n0, n1, n2, _ptr(weight), _ptr(bias),
                                   K, cin, length, nthreads)
        return data

    def conv_torch(self, x: np.ndarray, w: np.ndarray, bias: np.ndarray | None,
                   inplace: bool = False, nthreads: int = 0) -> np.ndarray:
        B, cin, L = x.shape
        cout, cin2, K = w.shape
        assert cin2 == cin
        out = x if inplace else np.zeros((B, cout, L - K + 1))
        self.lib.bko_conv_torch(_ptr(x), _ptr(out), B, cin, cout, L, K, _ptr(w),
                                _ptr(bias) if bias is not None else None, nthreads)
        return out

    def uniform(self, seed: int, idx: int) -> float:
        return self.lib.bko_uniform(seed, idx)


class _RefAdvParamsC(C.Structure):
    _fields_ = [("n0", C.c_int64), ("n1", C.c_int64), ("n2", C.c_int64),
                ("max_iter", C.c_int64), ("dt", C.c_double), ("minX", C.c_double),
                ("maxX", C.c_double), ("minVx", C.c_double), ("maxVx", C.c_double),
                ("width", C.c_double), ("dx", C.c_double), ("dvx", C.c_double),
                ("inv_dx", C.c_double), ("inplace", C.c_int32), ("gpu", C.c_int32),
                ("pref_wg_size", C.c_int64), ("seq_size0", C.c_int64),
                ("seq_size2", C.c_int64), ("kernel_impl", C.c_char * 64)]


class _RefConvParamsC(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("length", "channel_in", "channel_out", "k",
                                         "total_batch_size", "batch_size_n2", "n0",
                                         "n1", "n2", "n_write")] + [
        ("inplace", C.c_int32), ("gpu", C.c_int32), ("pref_wg_size", C.c_int64),
        ("seq_size0", C.c_int64), ("seq_size2", C.c_int64), ("kernel_impl", C.c_char * 64)]


def _struct_dict(s) -> dict:
    out = {}
    for name, _ in s._fields_:
        v = getattr(s, name)
        out[name] = v.decode() if isinstance(v, bytes) else v
    return out


class Reference:
    """The reference's own AdvectionSolver / ConvSolver / ConfigMap, compiled
    on the CPU by oracle/build_ref.sh. Only available where the reference
    checkout exists (fixture generation, pinning tests)."""

    def __init__(self, path: str = REF_SO):
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_adv_params_from_ini.argtypes = [C.c_char_p, C.POINTER(_RefAdvParamsC)]
        L.ref_adv_params_default.argtypes = [C.POINTER(_RefAdvParamsC)]
        L.ref_adv_step.argtypes = [C.POINTER(_RefAdvParamsC), _dp, C.c_int]
        L.ref_adv_stencil.argtypes = [C.POINTER(_RefAdvParamsC), C.c_int64, C.c_int64, _dp]
        L.ref_lag_basis.argtypes = [C.c_double, _dp]
        L.ref_conv_params_from_ini.argtypes = [C.c_char_p, C.POINTER(_RefConvParamsC)]
        L.ref_conv_step.argtypes = [_dp, C.c_int64, C.c_int64, C.c_int64, _dp, _dp,
                                    C.c_int64, C.c_int64, C.c_int64]

    @staticmethod
    def _p(p: AdvParams) -> _RefAdvParamsC:
        s = _RefAdvParamsC()
        s.n0, s.n1, s.n2 = p.n0, p.n1, p.n2
        s.dt, s.minX, s.maxX, s.minVx, s.maxVx = p.dt, p.minX, p.maxX, p.minVx, p.maxVx
        return s

    def adv_params_from_ini(self, path: str) -> dict:
        s = _RefAdvParamsC()
        if self.lib.ref_adv_params_from_ini(path.encode(), C.byref(s)) != 0:
            raise FileNotFoundError(path)
        return _struct_dict(s)

    def adv_params_default(self) -> dict:
        s = _RefAdvParamsC()
        self.lib.ref_adv_params_default(C.byref(s))
        return _struct_dict(s)

    def conv_params_from_ini(self, path: str) -> dict:
        s = _RefConvParamsC()
        if self.lib.ref_conv_params_from_ini(path.encode(), C.byref(s)) != 0:
            raise FileNotFoundError(path)
        return _struct_dict(s)

    def adv_step(self, p: AdvParams, data: np.ndarray, nsteps: int = 1):
        self.lib.ref_adv_step(C.byref(self._p(p)), _ptr(data), nsteps)
        return data

    def adv_stencil(self, p: AdvParams, i0: int, i1: int) -> np.ndarray:
        out = np.zeros(p.n1)
        self.lib.ref_adv_stencil(C.byref(self._p(p)), i0, i1, _ptr(out))
        return out

    def lag_basis(self, px: float) -> np.ndarray:
        c = np.zeros(6)
        self.lib.ref_lag_basis(px, _ptr(c))
        return c

    def conv_step(self, data: np.ndarray, weight: np.ndarray, bias: np.ndarray, K: int,
                  cin: int, length: int):
        n0, n1, n2 = data.shape
        self.lib.ref_conv_step(_ptr(data), n0, n1, n2, _ptr(weight), _ptr(bias), K, cin,
                               length)
        return data
