"""The allocation-free time loop, hx_level_run_static_f64.

It exists for callers that cannot allocate device memory of their own: in
HydroEXA the AMReX arena reserves most of the GPU at start-up and serves every
later request, so a library cudaMalloc in the middle of the time loop can fail
or compete with it.  The call keeps its scratch (alternate state planes and
CFL accumulators) in one fixed array inside the library.  This file checks,
through the C ABI, that two calls in a row give exactly what the scratch-taking
hx_level_run_f64 gives on the same inputs, in both arithmetic forms (equality:
the same kernels run), that leftovers of the first call do not leak into the
second, that rows padded past nx keep their padding, and that an oversized
level is refused.  It is named
to run last, and works alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest
import torch

from hydroexa_gb300 import capi, workloads
from hydroexa_gb300.level import Level

pytestmark = pytest.mark.gpu


def _static_run(lev: Level, method: int, nsteps: int, cfl: float, stream, arith=capi.HX_ARITH_EXACT):
    d = lev._desc(lev.state)
    status = torch.zeros(1, dtype=torch.int32, device=lev.state.device)
    t = torch.zeros(1, dtype=torch.float64, device=lev.state.device)
    rc = capi.lib().hx_level_run_static_f64(method, ctypes.byref(d), nsteps, cfl,
                                            ctypes.c_void_p(status.data_ptr()), ctypes.c_void_p(t.data_ptr()),
                                            arith, ctypes.c_void_p(stream.cuda_stream))
    return rc, status, t


def _padded_level(case, pitch, device, fill=12345.0):
    """The case's level stored with rows of ``pitch`` > nx elements, the padding set to ``fill``."""
    ny, nx = case.h.shape
    st = np.full((3, ny, pitch), fill)
    tr = np.full((2, ny, pitch), fill)
    for k, a in enumerate((case.h, case.hu, case.hv)):
        st[k, :, :nx] = a
    tr[0, :, :nx] = case.z
    tr[1, :, :nx] = case.n
    return Level(case.geom, torch.from_numpy(st).to(device), torch.from_numpy(tr).to(device))


@pytest.mark.parametrize("arith", [capi.HX_ARITH_EXACT, capi.HX_ARITH_FAST])
def test_static_run_matches_scratch_run_twice(cuda, hxlib, arith):
    """Both arithmetic forms: the same kernels and the same first CFL reduction
    as hx_level_run_f64, so the results are equal bit for bit in either form
    (the fast form's own tolerance against the oracle does not enter)."""
    stream = torch.cuda.current_stream(cuda)
    calls = [
        (workloads.fractal_dam_break(96, 80, seed=61, amplitude=1.5, nodata_frac=0.15), capi.HX_METHOD_HYDROSTATIC_ROE, 7),
        (workloads.dam_break(64, 48), capi.HX_METHOD_ROE, 10),
    ]
    for case, method, nsteps in calls:
        ref = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, device=cuda)
        assert ref.run(method, nsteps, case.cfl, arith=arith, stream=stream) == 0
        lev = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, device=cuda)
        rc, status, t = _static_run(lev, method, nsteps, case.cfl, stream, arith)
        assert rc == capi.HX_OK, capi.lib().hx_last_error()
        torch.cuda.synchronize(cuda)
        assert int(status.item()) == 0
        assert torch.equal(lev.state, ref.state)
        assert t.item() == ref.time.item()


def test_static_run_keeps_row_padding(cuda, hxlib):
    """A level whose rows are longer than nx (pitch > nx): after an odd number
    of steps the result comes back from the array into the valid cells only,
    the caller's padding keeps its values, and the valid cells equal the
    scratch-taking run's."""
    stream = torch.cuda.current_stream(cuda)
    case = workloads.fractal_dam_break(90, 70, seed=62, amplitude=1.0, nodata_frac=0.1)
    ref = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, device=cuda)
    assert ref.run(capi.HX_METHOD_HYDROSTATIC_ROE, 5, case.cfl, arith=capi.HX_ARITH_EXACT, stream=stream) == 0
    lev = _padded_level(case, 96, cuda)
    rc, status, _ = _static_run(lev, capi.HX_METHOD_HYDROSTATIC_ROE, 5, case.cfl, stream)
    assert rc == capi.HX_OK, capi.lib().hx_last_error()
    torch.cuda.synchronize(cuda)
    assert int(status.item()) == 0
    assert torch.equal(lev.state[:, :, :90], ref.state)
    assert bool((lev.state[:, :, 90:] == 12345.0).all())


def test_static_run_refuses_oversized_level(cuda, hxlib):
    case = workloads.dam_break(1024, 512)
    assert case.cells > capi.HX_STATIC_RUN_MAX_CELLS
    lev = Level.from_numpy(case.geom, case.h, case.hu, case.hv, case.z, case.n, device=cuda)
    before = lev.state.clone()
    rc, _, _ = _static_run(lev, capi.HX_METHOD_HYDROSTATIC_ROE, 3, case.cfl, torch.cuda.current_stream(cuda))
    assert rc == capi.HX_ERR_ARG
    assert b"exceeds the static scratch" in capi.lib().hx_last_error()
    assert torch.equal(lev.state, before)
    assert np.isfinite(before.cpu().numpy()).all()
