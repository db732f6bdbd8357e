"""plume_timestep_noalloc against the time step of plume_step.

The no-allocation entry point serves callers that cannot allocate GPU memory
(their device memory belongs to their own pool, or an allocation would
synchronise the device).  It takes the particle arrays as device pointers
and keeps its scratch in a fixed device array inside the library.  This
test calls it through the C ABI twice in a row on the same device arrays
and compares each result with the dt that plume_step computes for the same
particles (same formula, CFL * min(h / c) over bc_type 100/99): the two must
agree to rounding (relative 1e-15).  It allocates its device arrays with
torch, so it also runs alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_timestep_noalloc_matches_plume_step():
    import torch
    import plume_gpu
    from plume_gpu import Solver, cases

    plume_gpu.build()
    L = plume_gpu.lib()
    case = cases.plume_small(seed=2)
    ps = case.particles
    dev = torch.device("cuda:0")
    h = torch.from_numpy(ps.h.copy()).to(dev)
    c = torch.from_numpy(ps.c.copy()).to(dev)
    bc = torch.from_numpy(ps.bc_type.copy()).to(dev)
    out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    got = []
    for _ in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        rc = L.plume_timestep_noalloc(C.c_void_p(h.data_ptr()), C.c_void_p(c.data_ptr()),
                                      C.c_void_p(bc.data_ptr()), ps.n, case.options.cfl,
                                      C.c_void_p(out.data_ptr()), None)
        assert rc == 0
        torch.cuda.synchronize()
        got.append(float(out.item()))
    s = Solver(case)
    dt_step = s.step()  # first step: no output time within reach, no clipping
    s.close()
    for v in got:
        assert np.isfinite(v) and v > 0
        assert abs(v - dt_step) <= 1e-15 * dt_step, (v, dt_step)


def test_timestep_noalloc_rejects_oversize():
    import plume_gpu
    plume_gpu.build()
    L = plume_gpu.lib()
    big = 1024 * 16384 + 1
    rc = L.plume_timestep_noalloc(C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), big, 0.8,
                                  C.c_void_p(8), None)
    assert rc == 5  # PLUME_E_CAPACITY, checked before any device work
