"""Inputs-file parameters of the reference solver, same keys and defaults.

Keys and defaults follow include/utils/Params.H:32-111 and the parsing in
src/HydroEXA.cpp:10-81 (plus amr.blocking_factor, src/HydroEXA.cpp:108-109, and
HydroEXA.log_verbosity).  The file format is AMReX ParmParse's
``prefix.key = v1 v2 ...`` with ``#`` comments and quoted strings.
"""
from __future__ import annotations

import shlex
from dataclasses import dataclass, field
from pathlib import Path


@dataclass
class RuntimeParameters:
    etime: float = 0.0
    max_time: float = 1.0
    mass_diag_freq: float = -1.0
    iteration: int = 0
    log_progress_every: int = 10
    wall_elapsed: float = 0.0


@dataclass
class IOParameters:
    io_freq: float = 1.0
    chk_freq: float = -1.0
    plot_freq: float = -1.0
    async_io: bool = False
    chk_type: str = "native"
    plot_file: str = "plt"
    plot_type: str = "native"
    chk_file: str = "chk"
    input_file: str = "input.h5"
    restart_chkfile: str = "restart"


@dataclass
class AMRParameters:
    regrid_int: int = 2
    do_reflux: int = 1
    do_subcycle: int = 1
    terrain_ref_lev: int = 0
    max_amr_level: int = 0
    blocking_factor: int = 8


@dataclass
class BCParams:
    lo_bc: list = field(default_factory=lambda: [0, 0])
    hi_bc: list = field(default_factory=lambda: [0, 0])


@dataclass
class PhysicsParameters:
    cfl: float = 0.5
    model: str = "Roe"
    h_grad_thresh: list = field(default_factory=list)
    umag_grad_thresh: list = field(default_factory=list)
    z_grad_thresh: list = field(default_factory=list)
    bc_params: BCParams = field(default_factory=BCParams)
    log_verbosity: int = 1


@dataclass
class Parameters:
    runtime: RuntimeParameters
    io: IOParameters
    amr: AMRParameters
    physics: PhysicsParameters
    raw: dict


def parse_inputs(text: str) -> dict:
    """ParmParse-style ``key = values`` lines -> {key: [tokens]} (later keys win)."""
    table = {}
    for line in text.splitlines():
        line = line.split("#", 1)[0].strip()
        if not line or "=" not in line:
            continue
        key, val = line.split("=", 1)
        table[key.strip()] = shlex.split(val.strip())
    return table


def _get(table, key, conv, default):
    v = table.get(key)
    if not v:
        return default
    return conv(v[0])


def _bool(s: str) -> bool:
    return s.lower() in ("1", "true", "t", "yes")


def read_parameters(source) -> Parameters:
    """Parse an inputs file (path or text) as HydroEXA::ReadParameters does."""
    p = Path(source) if not isinstance(source, str) or "\n" not in source else None
    text = p.read_text() if p is not None and p.exists() else str(source)
    t = parse_inputs(text)
    io = IOParameters()
    io.chk_freq = _get(t, "io.chk_freq", float, io.chk_freq)
    io.chk_type = _get(t, "io.chk_type", str, io.chk_type)
    io.plot_freq = _get(t, "io.plot_freq", float, io.plot_freq)
    io.async_io = _get(t, "io.async_io", _bool, io.async_io)
    io.input_file = _get(t, "io.input_file", str, io.input_file)
    io.plot_file = _get(t, "io.plot_file", str, io.plot_file)
    io.chk_file = _get(t, "io.chk_file", str, io.chk_file)
    io.restart_chkfile = _get(t, "io.restart", str, io.restart_chkfile)
    amr = AMRParameters()
    amr.regrid_int = _get(t, "amr.regrid_int", int, amr.regrid_int)
    amr.do_reflux = _get(t, "amr.do_reflux", int, amr.do_reflux)
    amr.do_subcycle = _get(t, "amr.do_subcycle", int, amr.do_subcycle)
    amr.terrain_ref_lev = _get(t, "amr.terrain_ref_lev", int, amr.terrain_ref_lev)
    amr.max_amr_level = _get(t, "amr.max_level", int, amr.max_amr_level)
    amr.blocking_factor = _get(t, "amr.blocking_factor", int, amr.blocking_factor)
    if amr.blocking_factor <= 0:
        raise ValueError("amr.blocking_factor must be greater than zero.")
    rt = RuntimeParameters()
    ph = PhysicsParameters()
    ph.model = _get(t, "HydroEXA.model", str, ph.model)
    ph.cfl = _get(t, "HydroEXA.cfl", float, ph.cfl)
    rt.max_time = _get(t, "HydroEXA.max_time", float, rt.max_time)
    rt.mass_diag_freq = _get(t, "HydroEXA.mass_diag_freq", float, rt.mass_diag_freq)
    rt.log_progress_every = _get(t, "HydroEXA.log_progress_every", int, rt.log_progress_every)
    ph.log_verbosity = _get(t, "HydroEXA.log_verbosity", int, ph.log_verbosity)
    for key in ("h_grad_thresh", "umag_grad_thresh", "z_grad_thresh"):
        if t.get("HydroEXA." + key):
            setattr(ph, key, [float(x) for x in t["HydroEXA." + key]])
    for key in ("lo_bc", "hi_bc"):
        vals = t.get("HydroEXA." + key)
        if vals:
            dst = getattr(ph.bc_params, key)
            for i in range(min(2, len(vals))):
                dst[i] = int(vals[i])
    return Parameters(rt, io, amr, ph, t)
