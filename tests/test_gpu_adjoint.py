"""The hand-written adjoint of the 3D FP64 particle step against finite
differences of full forward runs.

The adjoint differentiates the step with its discrete decisions frozen
(neighbour lists, the particle that sets dt, conversions, deletions); a
finite difference sees them move, plus the jumps of the Gaussian's box
cut-off (|s_k| = 3).  The checks therefore start from a developed state with
h off the lattice spacing (h = 1.3 dx: no lattice offset sits on the
cut-off), use per-component random directions of small size, and require
agreement to 1e-5 (one step) and 1e-3 (windows of several steps), the bar
of the vent-parameter gradient.
"""
import copy
import dataclasses

import numpy as np
import pytest

from plume_gpu import Solver, cases
from plume_gpu.abi import ParticleSet
from plume_gpu.adjoint import FIELDS

pytestmark = pytest.mark.gpu


def _developed(steps, seed=0):
    base = cases.plume_small(seed=seed)
    base.particles.h[:] *= 1.3
    base.step0 = 0
    s = Solver(base)
    s.steps(steps)
    ps = s.download().sorted_by_key()
    t = s.time()
    s.close()
    return dataclasses.replace(base, particles=ps, step0=0), t


def _run(case, t, ps, nsteps, record_every=0):
    s = Solver(dataclasses.replace(case, particles=ps))
    s.set_time(t[0], t[1], t[2], case.options.timeoutput)
    if record_every:
        s.adjoint_record(nsteps, record_every)
    else:
        s.steps(nsteps)
    return s, s.download().sorted_by_key()


OUT = {"x": ["x", "y", "z"], "v": ["vx", "vy", "vz"], "vs": ["vsx", "vsy", "vsz"], "rho": ["rho"],
       "e": ["e"], "h": ["h"]}
DIRS = [("x", 1.0), ("y", 1.0), ("z", 1.0), ("vx", 1.0), ("vz", 1.0), ("vsy", 1.0), ("mass", None),
        ("h", None), ("rho", None), ("e", None), ("p", None), ("c", None)]


def _check(case, t, nsteps, every, rel, tol, min_good):
    rng = np.random.default_rng(3)
    ps0 = case.particles
    s, fin = _run(case, t, ps0.take(np.arange(ps0.n)), nsteps, every)
    W = {f: rng.standard_normal(fin.n) / max(np.abs(getattr(fin, f)).mean(), 1e-12)
         for flds in OUT.values() for f in flds}

    def J(fn):
        assert np.array_equal(fn.key, fin.key)
        return sum(float((W[f] * getattr(fn, f)).sum()) for f in W)

    fb = ParticleSet(fin.n)
    fb.key[:] = fin.key
    for f in W:
        getattr(fb, f)[:] = W[f]
    ib, _ = s.adjoint_backward(fb)
    ib = ib.take(np.argsort(ib.key))
    assert np.array_equal(ib.key, np.sort(ps0.key))
    # the context continues from the window's final state
    np.testing.assert_array_equal(s.download().sorted_by_key().x, fin.x)
    errs = {}
    for f, scale in DIRS:
        mag = scale if scale is not None else np.abs(getattr(ps0, f)).mean()
        u = rng.standard_normal(ps0.n) * rel * mag
        vals = []
        for sgn in (1, -1):
            ps = ps0.take(np.arange(ps0.n))
            getattr(ps, f)[:] = getattr(ps0, f) + sgn * u
            vals.append(J(_run(case, t, ps, nsteps)[1]))
        fd = (vals[0] - vals[1]) / 2
        ad = float((getattr(ib, f) * u).sum())
        errs[f] = abs(fd - ad) / max(abs(fd), abs(ad), 1e-300)
    print({k: "%.1e" % v for k, v in errs.items()})
    good = sum(e <= tol for e in errs.values())
    assert good >= min_good, errs
    assert max(errs.values()) <= 100 * tol, errs
    return errs


def test_adjoint_one_step_matches_finite_differences():
    case, t = _developed(5)
    _check(case, t, nsteps=1, every=1, rel=1e-6, tol=1e-5, min_good=len(DIRS) - 1)


def test_adjoint_window_with_checkpoints_and_adaptive_h():
    # steps 49..52: two checkpoint segments, adaptive h at step 50.  In this
    # near-hydrostatic state the second adaptive iteration gives h ~ 1.5 dx,
    # so its search length 2h puts the cut-off |s| = 3 on the lattice offset
    # 9 dx; directions of 1e-9 keep the finite differences clear of it.
    case, t = _developed(48)
    _check(case, t, nsteps=4, every=2, rel=1e-9, tol=1e-3, min_good=len(DIRS) - 1)


def test_vent_parameter_gradient_matches_finite_differences():
    torch = pytest.importorskip("torch")
    from plume_gpu import adjoint
    case = cases.plume_small(seed=2)
    case.particles.h[:] *= 1.3
    theta = np.array([150.0, 1053.0, 0.95])
    obj = dict(z_ash=40.0, width=20.0, z_target=60.0, r_scale=30.0)
    J, g = adjoint.value_and_grad(theta, case, nsteps=12, every=4, **obj)
    assert np.isfinite(J) and np.all(np.isfinite(g))
    J0 = adjoint.forward_value(theta, case, 12, **obj)
    assert abs(J - J0) <= 1e-9 * abs(J0)
    fd = adjoint.finite_difference(theta, case, 12, rel=1e-4, **obj)
    print("adjoint", g, "central differences", fd)
    np.testing.assert_allclose(g, fd, rtol=1e-3, atol=1e-3 * np.abs(fd).max())
