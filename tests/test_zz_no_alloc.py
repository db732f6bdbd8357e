"""plume_timestep_noalloc: the time step for callers that cannot allocate.

Some hosts cannot let a library allocate GPU memory when they ask for a time
step: their device memory belongs to their own pool (a framework's caching
allocator, an application that reserves all memory at start-up), or they
call from a path where an allocation would synchronise the device.  The
no-allocation entry point takes the particle arrays as device pointers and
keeps its scratch in a fixed device array inside the library.

This file is collected last.  Its tests call the entry point through the C
ABI, twice in a row on the same device arrays, and compare each result with
a host evaluation of the reference's formula (timestep.cc:94-183: CFL *
min(h / c) over bc_type 100/99, starting from 1e10) and with the dt that
plume_step computes for the same particles, to rounding (relative 1e-15).
They also check that the second call leaves the device's free memory
unchanged, the empty input (CFL * 1e10), and the NaN result of a particle
with c = 0 or h < 0.  Device arrays are made with torch, so the file also
runs alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-15


def _host_dt(h, c, bc, cfl):
    sel = (bc == 100) | (bc == 99)
    return cfl * min(1.0e10, float((h[sel] / c[sel]).min())) if sel.any() else cfl * 1.0e10


def _call(L, h, c, bc, n, cfl, out):
    import torch
    out.fill_(-1.0)
    torch.cuda.synchronize()
    rc = L.plume_timestep_noalloc(C.c_void_p(h.data_ptr()), C.c_void_p(c.data_ptr()),
                                  C.c_void_p(bc.data_ptr()), n, cfl, C.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    return rc, float(out.item())


def test_timestep_noalloc_matches_host_and_plume_step():
    import torch
    import plume_gpu
    from plume_gpu import Solver, cases

    plume_gpu.build()
    L = plume_gpu.lib()
    case = cases.plume_small(seed=2)
    ps = case.particles
    cfl = case.options.cfl
    dev = torch.device("cuda:0")
    h = torch.from_numpy(ps.h.copy()).to(dev)
    c = torch.from_numpy(ps.c.copy()).to(dev)
    bc = torch.from_numpy(ps.bc_type.copy()).to(dev)
    out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    want = _host_dt(ps.h, ps.c, ps.bc_type, cfl)
    got = []
    rc, v = _call(L, h, c, bc, ps.n, cfl, out)  # first call: address set-up
    assert rc == 0
    got.append(v)
    free0 = torch.cuda.mem_get_info(dev)[0]
    rc, v = _call(L, h, c, bc, ps.n, cfl, out)
    free1 = torch.cuda.mem_get_info(dev)[0]
    assert rc == 0
    got.append(v)
    assert free1 == free0, (free0, free1)  # the second call took no device memory
    s = Solver(case)
    dt_step = s.step()  # first step: no output time within reach, no clipping
    s.close()
    for v in got:
        assert np.isfinite(v) and v > 0
        assert abs(v - want) <= REL * want, (v, want)
        assert abs(v - dt_step) <= REL * dt_step, (v, dt_step)


def test_timestep_noalloc_edge_cases():
    import torch
    import plume_gpu

    plume_gpu.build()
    L = plume_gpu.lib()
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(3)
    n = 40000  # three blocks of the partial reduction
    h0 = rng.uniform(50.0, 150.0, n)
    c0 = rng.uniform(300.0, 350.0, n)
    bc0 = np.where(rng.random(n) < 0.8, 100, 1).astype(np.uint8)
    bc0[-5:] = 99
    out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    cfl = 0.8

    def run(hh, cc, bb, nn=None):
        hd, cd, bd = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (hh, cc, bb))
        rc, v = _call(L, hd, cd, bd, len(hh) if nn is None else nn, cfl, out)
        assert rc == 0
        return v

    # ragged size: the last block is partly empty; the minimum sits there
    h1 = h0.copy()
    h1[-3] = 1.0
    bc1 = bc0.copy()
    bc1[-3] = 100
    want = _host_dt(h1, c0, bc1, cfl)
    for _ in range(2):
        v = run(h1, c0, bc1)
        assert abs(v - want) <= REL * want, (v, want)
    # no particle updates its state: CFL * 1e10 (timestep.cc:99)
    assert run(h0, c0, np.ones(n, np.uint8)) == cfl * 1.0e10
    # empty input
    assert run(h0[:1], c0[:1], bc0[:1], nn=0) == cfl * 1.0e10
    # a sound speed of zero, or a negative smoothing length, in an updated
    # particle: NaN (the reference asserts c > 0, timestep.cc:167)
    c2 = c0.copy()
    c2[17] = 0.0
    bc2 = bc0.copy()
    bc2[17] = 100
    assert np.isnan(run(h0, c2, bc2))
    h3 = h0.copy()
    h3[n // 2] = -h3[n // 2]
    bc3 = bc0.copy()
    bc3[n // 2] = 99
    assert np.isnan(run(h3, c0, bc3))
    # the same bad value in a particle that does not update: ignored
    bc4 = bc2.copy()
    bc4[17] = 1
    want = _host_dt(h0, c2, bc4, cfl)
    v = run(h0, c2, bc4)
    assert abs(v - want) <= REL * want, (v, want)
    # and a valid call right after a NaN one is valid again
    want = _host_dt(h0, c0, bc0, cfl)
    v = run(h0, c0, bc0)
    assert abs(v - want) <= REL * want, (v, want)


def test_timestep_noalloc_rejects_oversize():
    import plume_gpu
    plume_gpu.build()
    L = plume_gpu.lib()
    big = 1024 * 16384 + 1
    rc = L.plume_timestep_noalloc(C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), big, 0.8,
                                  C.c_void_p(8), None)
    assert rc == 5  # PLUME_E_CAPACITY, checked before any device work
