"""Device-resident level state and Array4 views over torch CUDA tensors.

PyTorch is used only for device memory and streams; every computation is a
call into the C ABI (``hydroexa_gb300.capi``).

Layout in HBM: each field is a plane of ``ny`` rows of ``pitch`` elements, x
fastest (the amrex::Array4 order).  A level's state is three planes (h, hu, hv),
its terrain two (z, Manning n); ``Level.state`` is one (3, ny, pitch) tensor and
``Level.terrain`` one (2, ny, pitch) tensor, so a whole component set is one
allocation and the planes of a component set are ``ny * pitch`` apart.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from . import capi

_REAL = {torch.float64: (ctypes.c_double, capi.Array4F64, capi.LevelF64, "f64"),
         torch.float32: (ctypes.c_float, capi.Array4F32, capi.LevelF32, "f32")}


def _stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t: torch.Tensor, real):
    return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(real))


def array4(t: torch.Tensor, lo=(0, 0)):
    """Array4 view of a contiguous (ncomp, ny, nx) or (ny, nx) tensor whose
    element [c, 0, 0] is cell ``lo``."""
    if t.dim() == 2:
        t = t.unsqueeze(0)
    assert t.is_contiguous(), "array4 needs a contiguous tensor"
    nc, ny, nx = t.shape
    if t.dtype == torch.int8:
        real, A4 = ctypes.c_byte, capi.Array4I8
    else:
        real, A4, _, _ = _REAL[t.dtype]
    a = A4()
    a.p = _ptr(t, real)
    a.jstride = nx
    a.nstride = nx * ny
    a.lo[0], a.lo[1] = int(lo[0]), int(lo[1])
    a.hi[0], a.hi[1] = int(lo[0]) + nx - 1, int(lo[1]) + ny - 1
    a.ncomp = nc
    return a


def box(lo, hi) -> capi.Box:
    b = capi.Box()
    b.lo[0], b.lo[1] = int(lo[0]), int(lo[1])
    b.hi[0], b.hi[1] = int(hi[0]), int(hi[1])
    return b


class DtAccum:
    """Device dt accumulator (min CFL bound, max |vel|) -- compute_dt_Impl's ReduceOps."""

    def __init__(self, device="cuda"):
        n = int(capi.lib().hx_dt_accum_bytes())
        self.buf = torch.zeros(n, dtype=torch.uint8, device=device)

    @property
    def ptr(self):
        return ctypes.c_void_p(self.buf.data_ptr())

    def reset(self, stream=None):
        capi.check(capi.lib().hx_dt_accum_reset(self.ptr, _stream_handle(stream)), "hx_dt_accum_reset")

    def read(self, dtype=torch.float64, stream=None):
        real, _, _, sfx = _REAL[dtype]
        m, v = real(), real()
        capi.check(getattr(capi.lib(), f"hx_dt_accum_read_{sfx}")(self.ptr, ctypes.byref(m), ctypes.byref(v),
                                                                   _stream_handle(stream)), "hx_dt_accum_read")
        return float(m.value), float(v.value)


class Status:
    """Device status word (HX_STATUS_* bits)."""

    def __init__(self, device="cuda"):
        self.buf = torch.zeros(1, dtype=torch.int32, device=device)

    @property
    def ptr(self):
        return ctypes.c_void_p(self.buf.data_ptr())

    def clear(self, stream=None):
        capi.check(capi.lib().hx_status_clear(self.ptr, _stream_handle(stream)), "hx_status_clear")

    def read(self, stream=None) -> int:
        return capi.check(capi.lib().hx_status_read(self.ptr, _stream_handle(stream)), "hx_status_read")


@dataclass
class Geometry:
    """Cell counts, sizes and physical-boundary codes of one level."""
    nx: int
    ny: int
    dx: float
    dy: float
    bc_lo: tuple = (0, 0)
    bc_hi: tuple = (0, 0)


class Level:
    """One single-box level resident in HBM: state (3, ny, pitch), terrain (2, ny, pitch)."""

    def __init__(self, geom: Geometry, state: torch.Tensor, terrain: torch.Tensor):
        assert state.is_cuda and terrain.is_cuda, "level fields must be CUDA tensors"
        assert state.dtype == terrain.dtype and state.dtype in _REAL
        assert state.shape[0] == 3 and terrain.shape[0] == 2
        assert state.is_contiguous() and terrain.is_contiguous()
        self.geom = geom
        self.state = state
        self.terrain = terrain
        self.alt = torch.empty_like(state)
        self.dtype = state.dtype
        self.pitch = state.shape[2]
        self.work = torch.zeros(int(capi.lib().hx_level_run_work_bytes()), dtype=torch.uint8, device=state.device)
        self.status = Status(state.device)
        self.time = torch.zeros(1, dtype=state.dtype, device=state.device)

    @classmethod
    def from_numpy(cls, geom: Geometry, h, hu, hv, z, n, dtype=torch.float64, device="cuda"):
        import numpy as np
        st = torch.from_numpy(np.stack([h, hu, hv]).astype(np.float64 if dtype == torch.float64 else np.float32))
        tr = torch.from_numpy(np.stack([z, n]).astype(np.float64 if dtype == torch.float64 else np.float32))
        return cls(geom, st.to(device).contiguous(), tr.to(device).contiguous())

    def _desc(self, state: torch.Tensor):
        real, _, Lv, _ = _REAL[self.dtype]
        g = self.geom
        d = Lv()
        d.h, d.hu, d.hv = (_ptr(state[k], real) for k in range(3))
        d.z, d.n = _ptr(self.terrain[0], real), _ptr(self.terrain[1], real)
        d.pitch = self.pitch
        d.nx, d.ny = g.nx, g.ny
        d.dx, d.dy = g.dx, g.dy
        d.bc_lo[0], d.bc_lo[1] = g.bc_lo
        d.bc_hi[0], d.bc_hi[1] = g.bc_hi
        return d

    @property
    def sfx(self):
        return _REAL[self.dtype][3]

    def advance(self, method: int, dt: float, out: torch.Tensor | None = None, next_dt: DtAccum | None = None,
                arith: int = capi.HX_ARITH_EXACT, stream=None) -> torch.Tensor:
        """One advance by a host dt, writing ``out`` (default: a new tensor)."""
        out = torch.empty_like(self.state) if out is None else out
        real = _REAL[self.dtype][0]
        d = self._desc(self.state)
        capi.check(getattr(capi.lib(), f"hx_level_advance_{self.sfx}")(
            method, ctypes.byref(d), dt, *(ctypes.c_void_p(out[k].data_ptr()) for k in range(3)),
            next_dt.ptr if next_dt is not None else None, self.status.ptr, arith, _stream_handle(stream)),
            "hx_level_advance")
        del real
        return out

    def advance_epilogue(self, dt: float, out: torch.Tensor | None = None, eta: bool = True, diag: bool = True,
                         next_dt: DtAccum | None = None, arith: int = capi.HX_ARITH_EXACT, stream=None):
        """One hydrostatic advance whose update also writes eta = h + z of the
        new state (DeriveEtaFrom) and its conservation diagnostics (mass,
        x- and y-momentum, kinetic energy, min h; ComputeMassDiagnostics).
        Returns (new state, eta plane or None, 5 diagnostics on the device or None)."""
        out = torch.empty_like(self.state) if out is None else out
        e = torch.empty_like(self.state[0]) if eta else None
        dg = torch.empty(5, dtype=torch.float64, device=self.state.device) if diag else None
        work = getattr(self, "_diag_work", None)  # kept: the kernel may still use it when this returns
        if diag and work is None:
            b = box((0, 0), (self.geom.nx - 1, self.geom.ny - 1))
            work = self._diag_work = torch.empty(int(capi.lib().hx_diagnostics_work_bytes(b)), dtype=torch.uint8,
                                                 device=self.state.device)
        d = self._desc(self.state)
        vp = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
        capi.check(getattr(capi.lib(), f"hx_level_advance_epilogue_{self.sfx}")(
            ctypes.byref(d), dt, *(ctypes.c_void_p(out[k].data_ptr()) for k in range(3)),
            next_dt.ptr if next_dt is not None else None, self.status.ptr, arith, vp(e), vp(dg),
            vp(work) if diag else None,
            _stream_handle(stream)), "hx_level_advance_epilogue")
        return out, e, dg

    def compute_dt(self, stream=None):
        """(min per-cell CFL bound, max |vel|) of the current state, before the CFL factor."""
        acc = getattr(self, "_acc", None)
        if acc is None:
            acc = self._acc = DtAccum(self.state.device)
        acc.reset(stream)
        d = self._desc(self.state)
        capi.check(getattr(capi.lib(), f"hx_level_dt_reduce_{self.sfx}")(ctypes.byref(d), acc.ptr,
                                                                          _stream_handle(stream)), "hx_level_dt_reduce")
        return acc.read(self.dtype, stream)

    def run(self, method: int, nsteps: int, cfl: float, arith: int = capi.HX_ARITH_EXACT, stream=None,
            check_status: bool = True) -> int:
        """nsteps of the single-level time loop; the state ends in ``self.state``.

        Returns the device status bits (read with a stream synchronisation when
        ``check_status``)."""
        self.status.clear(stream)
        d = self._desc(self.state)
        fin = ctypes.c_int(0)
        capi.check(getattr(capi.lib(), f"hx_level_run_{self.sfx}")(
            method, ctypes.byref(d), *(ctypes.c_void_p(self.alt[k].data_ptr()) for k in range(3)), nsteps, cfl,
            ctypes.c_void_p(self.work.data_ptr()), self.status.ptr, ctypes.c_void_p(self.time.data_ptr()), arith,
            ctypes.byref(fin), _stream_handle(stream)), "hx_level_run")
        if fin.value:
            self.state, self.alt = self.alt, self.state
        return self.status.read(stream) if check_status else 0
