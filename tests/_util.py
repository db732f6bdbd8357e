"""Shared helpers of the test suite."""
from __future__ import annotations

import os

import numpy as np

from plume_gpu import cases
from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS, ParticleSet

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MASK = np.uint64(0xFFFFFFFFFFFFFFFF)


def mix64(k):
    z = (np.asarray(k, dtype=np.uint64) + np.uint64(0x9E3779B97F4A7C15)) & MASK
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & MASK
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & MASK
    return z ^ (z >> np.uint64(31))


def set_summary(ki, kj):
    """per-i count and xor-hash of the j set, for i in sorted unique order"""
    order = np.lexsort((kj, ki))
    ki, kj = ki[order], kj[order]
    keys, start = np.unique(ki, return_index=True)
    cnt = np.diff(np.append(start, len(ki)))
    with np.errstate(over="ignore"):
        h = np.bitwise_xor.reduceat(mix64(kj), start) if len(ki) else np.zeros(0, np.uint64)
    return keys, cnt, h


def unpack(d, prefix) -> ParticleSet:
    ps = ParticleSet(0)
    ps.key = np.array(d[prefix + "key"], dtype=np.uint64)
    for f in DOUBLE_FIELDS + BYTE_FIELDS:
        setattr(ps, f, np.array(d[prefix + f]))
    return ps


def gsph_case(name):
    """the cases of the GSPH fixtures (tests/golden/make_golden.py)"""
    if name == "gsph_1d_sod":
        c = cases.sod_1d(n_real=200, method=cases.METHOD_GSPH)
    elif name == "gsph_1d_2000_end":
        c = cases.sod_1d(n_real=2000, method=cases.METHOD_GSPH)
    elif name == "gsph_1d_grad":
        c = cases.sod_1d(n_real=200, ghosts=0, eta=2.0, method=cases.METHOD_GSPH)
        c.options.gsph_recon = cases.RECON_EACH
    elif name == "gsph_3d":
        c = cases.plume_3d(half_width=200.0, height=400.0, dx=50.0, vent_radius=50.0,
                           vent_dx=25.0, duct_depth=300.0, seed=5, name="gsph_3d")
        c.options.method = cases.METHOD_GSPH
        c.step0 = 48
    elif name in GSPH_SOLVER_CASES:
        # the other Riemann solvers on the Sod tube and the 3D cube above
        base, solver, wave, method = GSPH_SOLVER_CASES[name]
        c = gsph_case(base)
        c.options.gsph_solver = solver
        c.options.gsph_wave_speed = wave
        c.options.method = method
        c.name = name
    else:
        raise KeyError(name)
    c.options.gsph_gradients = 1
    return c


# fixture name -> (base case, RIEMANN_SOLVER, HLL_WAVE_SPEED_EVA), with the
# reference build that made it (tests/golden/make_golden.py)
GSPH_SOLVER_CASES = {
    "gsph_1d_my2": ("gsph_1d_sod", cases.RIEMANN_HLLC_MY, 2, cases.METHOD_GSPH),
    "gsph_1d_my3": ("gsph_1d_sod", cases.RIEMANN_HLLC_MY, 3, cases.METHOD_GSPH),
    "gsph_1d_vl": ("gsph_1d_sod", cases.RIEMANN_VANLEER, 0, cases.METHOD_GSPH),
    "gsph_3d_my3": ("gsph_3d", cases.RIEMANN_HLLC_MY, 3, cases.METHOD_GSPH),
    "gsph_3d_vl": ("gsph_3d", cases.RIEMANN_VANLEER, 0, cases.METHOD_GSPH),
    # the random choice method (USE_GSPH 2) with the bases' solvers set aside
    "gsph_1d_rcm": ("gsph_1d_sod", cases.RIEMANN_HLLC, 0, cases.METHOD_GSPH_RCM),
    "gsph_3d_rcm": ("gsph_3d", cases.RIEMANN_HLLC, 0, cases.METHOD_GSPH_RCM),
}
# steps the reference completes on each (the next stops on assert(c > 0))
GSPH_SOLVER_STEPS = {"gsph_1d_my2": 1, "gsph_1d_my3": 1, "gsph_1d_vl": 7, "gsph_3d_my3": 1, "gsph_3d_vl": 2,
                     "gsph_1d_rcm": 20, "gsph_3d_rcm": 2}
GSPH_SOLVER_FAILS = {"gsph_1d_my2": True, "gsph_1d_my3": True, "gsph_1d_vl": True, "gsph_3d_my3": True,
                     "gsph_3d_vl": True, "gsph_1d_rcm": False, "gsph_3d_rcm": False}
GSPH_SOLVER_BUILDS = {"gsph_1d_my2": "ref1d_gsph_my2", "gsph_1d_my3": "ref1d_gsph_my3",
                      "gsph_1d_vl": "ref1d_gsph_vl", "gsph_3d_my3": "ref3d_gsph_my3",
                      "gsph_3d_vl": "ref3d_gsph_vl", "gsph_1d_rcm": "ref1d_gsph_rcm",
                      "gsph_3d_rcm": "ref3d_gsph_rcm"}


def adapt_case():
    """the plume of the domain-growth fixture, before cases.adapt_scenario"""
    c = cases.plume_3d(half_width=300.0, height=600.0, dx=50.0, vent_radius=50.0,
                       vent_dx=25.0, duct_depth=300.0, seed=6, name="adapt_3d")
    c.step0 = 48
    return c


def golden_case(name):
    """(case with the fixture's input particles, fixture dict)"""
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    if name.startswith("gsph_"):
        c = gsph_case(name)
    elif name == "sod_1d_200":
        c = cases.sod_1d(n_real=200, kernel=cases.KERNEL_M4)
    elif name == "sod_1d_2000_end":
        c = cases.sod_1d(n_real=2000)
    elif name == "shock_tube_1d":
        c = cases.shock_tube_1d()
    elif name == "plume_3d_small":
        c = cases.plume_3d(half_width=300.0, height=600.0, dx=50.0, vent_radius=50.0,
                           vent_dx=25.0, duct_depth=300.0, seed=3, name="plume_3d_small")
    elif name == "plume_3d_bc":
        c = cases.plume_3d(half_width=300.0, height=600.0, dx=50.0, vent_radius=50.0,
                           vent_dx=25.0, duct_depth=300.0, seed=4, name="plume_3d_bc")
    else:
        raise KeyError(name)
    c.particles = unpack(d, "in_")
    c.step0 = int(d["step0"])
    c.pre_adaptive = bool(int(d["pre_adaptive"]))
    return c, d


def field_errors(a: ParticleSet, b: ParticleSet, fields=DOUBLE_FIELDS):
    """max |a-b| / max|b| per field, after matching by key"""
    a = a.sorted_by_key()
    b = b.sorted_by_key()
    assert a.n == b.n, (a.n, b.n)
    assert np.array_equal(a.key, b.key)
    out = {}
    for f in fields:
        x, y = getattr(a, f), getattr(b, f)
        scale = max(float(np.abs(y).max()) if y.size else 0.0, 1e-300)
        out[f] = float(np.abs(x - y).max() / scale) if y.size else 0.0
    return out


# fields that are positive by construction: their error is bounded per
# particle (the max-normalised bound would let a small value drift)
POSITIVE_FIELDS = ("mass", "h", "rho", "e", "p", "c", "T", "gamma", "cp")


def particle_rel_errors(a: ParticleSet, b: ParticleSet, fields=POSITIVE_FIELDS):
    """max over particles of |a_i - b_i| / |b_i| per field (b_i != 0), after
    matching by key"""
    a = a.sorted_by_key()
    b = b.sorted_by_key()
    assert np.array_equal(a.key, b.key)
    out = {}
    for f in fields:
        x, y = getattr(a, f), getattr(b, f)
        nz = y != 0
        out[f] = float((np.abs(x[nz] - y[nz]) / np.abs(y[nz])).max()) if nz.any() else 0.0
    return out


def inlet_fixture():
    """(case, inlet, fixture) of tests/golden/inlet_3d.npz: the plume of
    cases.duct_scenario with the particles the reference's setup_erupt kept
    and the duct it built (keys after the case's), and the inlet of
    add_new_erupt for that duct (keys after the duct's)"""
    import dataclasses
    d = dict(np.load(os.path.join(GOLDEN, "inlet_3d.npz")))
    c, _, duct = cases.duct_scenario(adapt_case())
    inp = unpack(d, "in_")
    kept = inp.take(np.nonzero(np.isin(inp.key, d["kept_key"]))[0])
    born = unpack(d, "duct_")
    born.key = np.arange(born.n, dtype=np.uint64) + np.uint64(int(inp.key.max()) + 1)
    ps = ParticleSet.concat([kept, born])
    c = dataclasses.replace(c, particles=ps, step0=int(d["step0"]))
    inl = cases.duct_inlet(duct, born, int(born.key.max()) + 1)
    return c, inl, d


def match_by_position(ours: ParticleSet, ref: ParticleSet, tol: float = 1e-6):
    """rows of `ours` in the order of `ref`'s rows, matched by nearest
    position (both sets created with keys of their own)"""
    from scipy.spatial import cKDTree
    assert ours.n == ref.n, (ours.n, ref.n)
    pa = np.stack([ours.x, ours.y, ours.z], axis=1)
    pb = np.stack([ref.x, ref.y, ref.z], axis=1)
    dist, idx = cKDTree(pa).query(pb)
    assert dist.max() <= tol, dist.max()
    assert len(np.unique(idx)) == ref.n
    return ours.take(idx)
