"""Ghost layers after a domain adaptation -- TEST INFRASTRUCTURE.

A numpy restatement of the reference's add_pressure_ghost
(src/plume/add_pressure_ghost.cc:37-316) and add_wall_ghost
(src/plume/add_wall_ghost.cc:44-293), add_air (src/plume/add_air.cc:490-795)
and setup_erupt (src/plume/setup_erupt.cc:44-388) with initial_air
(src/plume/sph_lib.cc:831-866), air_prop_hydro (:543-592) and
Particle::update_second_var (src/datstr/particle.cc:528-604), used by the
tests only, as the checker of the device's plume_add_pressure_ghost and
plume_add_wall_ghost.

For every bucket whose involvement state is NONE, that holds no pressure
ghost and that has a neighbour (of the 26 inside the grid) whose state is
not NONE: the bucket is marked active, and a lattice of spacing dx =
smoothing_length (Nx = round(edge / dx) per axis, points at corner + dx/2 +
i dx) is filled with air particles -- in MIXED buckets on or below the
ground only the points above the ground plane, in OVERGROUND and PRESS_BC
buckets all of them, in UNDERGROUND buckets none.  A new particle is a
pressure ghost (bc 1, phase 1, Y 0, involved 0, at rest) with h =
smoothing_length and the hydrostatic air state of its height: T and p of
the fitted profile, rho = p / (Ra T), e = p / (rho (gamma - 1)), and the
mass of its dx^3 box by the reference's three-point rule in z with the
coefficients as written there (0.1666667, 0.6666666, 0.1666667); then the
mixture EOS sets gamma, p, c, T and cp.

add_wall_ghost: every on-ground MIXED bucket (bottom face below the
ground) that holds particles but no wall ghost gets wall ghosts (bc 2) on
the lattice points below the ground plane, and the bucket below it is made
active and gets its whole lattice; same air state.

Rows come out bucket by bucket in linear bucket order (x fastest), then by
lattice index (i, j, k), k fastest.
"""
from __future__ import annotations

import math

import numpy as np

from .binding import ParticleSet  # noqa: F401  (sets sys.path)
from plume_gpu.abi import (BC_PRESSURE, BC_REAL, BC_WALL, BUCKET_ABSORBING, BUCKET_MIXED, BUCKET_PRESS_BC,
                           BUCKET_UNDERGROUND, Atmosphere, ParticleSet as PS)

OVERGROUND, MIXED, UNDERGROUND, PRESS_BC = 3, 2, 1, 4


def bucket_types(flags, face):
    """the reference bucket type of every bucket from the grid flags (the
    explicit bits when any bucket carries one, else absorbing buckets wholly
    below the ground are UNDERGROUND and the other absorbing ones PRESS_BC)"""
    flags = np.asarray(flags, dtype=np.uint8)
    face = np.asarray(face, dtype=np.int8).reshape(-1, 6)
    explicit = bool(np.any(flags & (BUCKET_UNDERGROUND | BUCKET_PRESS_BC)))
    t = np.full(len(flags), OVERGROUND, dtype=np.int8)
    absorb = (flags & BUCKET_ABSORBING) != 0
    if explicit:
        t[(flags & BUCKET_PRESS_BC) != 0] = PRESS_BC
        t[(flags & BUCKET_UNDERGROUND) != 0] = UNDERGROUND
    else:
        under = absorb & (face[:, 4] == -1) & (face[:, 5] == -1)
        t[absorb & under] = UNDERGROUND
        t[absorb & ~under] = PRESS_BC
    t[(flags & BUCKET_MIXED) != 0] = MIXED
    return t


def _T(a: Atmosphere, h):
    # determine_temperature_hydro, sph_lib.cc:503-515
    if h < 0:
        return a.Ta0
    if h < a.H1:
        return a.Ta0 - a.miu1 * h
    if h < a.H2:
        return a.Ta0 - a.miu1 * a.H1
    return a.Ta0 - a.miu1 * a.H1 + a.miu2 * (h - a.H2)


def _p(a: Atmosphere, h):
    # determine_pressure_hydro, sph_lib.cc:488-500
    if h < 0:
        return a.pa0
    if h < a.H1:
        return a.Ata1 * (a.Ta0 - a.miu1 * h) ** a.Ate1
    if h < a.H2:
        return a.Ata2 * math.exp(a.Atb2 * h)
    return a.AtC3 * (a.Atb3 * h + a.Ata3) ** a.Ate3


def air_state(a: Atmosphere, x, y, z, sml):
    """(rho, e, p, mass) of initial_air for a particle at (x, y, z) with
    smoothing length sml (box of edge sml around it)"""
    T = _T(a, z)
    p = _p(a, z)
    rho = p / (a.Ra * T)
    e = p / (rho * (a.gamma - 1))
    s2 = 0.5 * sml
    lo, hi = z - s2, z + s2
    d1 = _p(a, lo) / (a.Ra * _T(a, lo))
    d2 = _p(a, hi) / (a.Ra * _T(a, hi))
    vol = ((x + s2) - (x - s2)) * ((y + s2) - (y - s2)) * (hi - lo)
    mass = vol * (0.1666667 * d1 + 0.6666666 * rho + 0.1666667 * d2)
    return rho, e, p, mass


def add_pressure_ghost(grid, binv, ps, opt, atm: Atmosphere | None = None):
    """(new particles, buckets that were marked active) for the grid, the
    per-bucket involvement states and the particle table after the
    adaptation; opt gives the smoothing length (sml_phase2) and the EOS
    constants."""
    atm = atm or Atmosphere()
    nb = np.array(grid.nb)
    mind = np.array(grid.mindom, dtype=np.float64)
    d = float(grid.del_)
    flags = np.asarray(grid.flags, dtype=np.uint8)
    face = np.asarray(grid.face_index, dtype=np.int8).reshape(-1, 6)
    typ = bucket_types(flags, face)
    binv = np.asarray(binv, dtype=np.uint8)
    # buckets holding a pressure ghost
    pos = np.stack([ps.x, ps.y, ps.z], axis=1)
    b3 = np.clip(np.floor((pos - mind) / d).astype(np.int64), 0, nb - 1)
    pb = (b3[:, 2] * nb[1] + b3[:, 1]) * nb[0] + b3[:, 0]
    has_pg = np.zeros(len(flags), dtype=bool)
    has_pg[pb[ps.bc_type == BC_PRESSURE]] = True
    dx = float(opt.sml_phase2)
    dx2 = 0.5 * dx
    ground = float(grid.domain_lo[2])
    rows = []
    marked = []
    for b in range(len(flags)):
        if binv[b] != 0 or has_pg[b]:
            continue
        i, j, k = b % nb[0], (b // nb[0]) % nb[1], b // (nb[0] * nb[1])
        hit = False
        for ii in (i - 1, i, i + 1):
            for jj in (j - 1, j, j + 1):
                for kk in (k - 1, k, k + 1):
                    if (ii, jj, kk) == (i, j, k) or not (0 <= ii < nb[0] and 0 <= jj < nb[1] and 0 <= kk < nb[2]):
                        continue
                    if binv[(kk * nb[1] + jj) * nb[0] + ii] != 0:
                        hit = True
        if not hit:
            continue
        marked.append(b)
        if typ[b] == UNDERGROUND:
            continue
        lo = np.array([mind[0] + i * d, mind[1] + j * d, mind[2] + k * d])
        hi = np.array([mind[0] + (i + 1) * d, mind[1] + (j + 1) * d, mind[2] + (k + 1) * d])
        n3 = _lattice(lo, hi, dx)
        onground = typ[b] == MIXED and face[b, 4] == -1
        for qi in range(n3[0]):
            for qj in range(n3[1]):
                for qk in range(n3[2]):
                    c = (lo[0] + dx2 + qi * dx, lo[1] + dx2 + qj * dx, lo[2] + dx2 + qk * dx)
                    if onground and not (c[2] > ground):
                        continue
                    rows.append(c)
    return _air_particles(rows, BC_PRESSURE, dx, opt, atm), np.array(marked, dtype=np.int64)


def _lattice(lo, hi, dx):
    # C round: halves away from zero (the quotients are positive)
    return [int(math.floor((hi[a] - lo[a]) / dx + 0.5)) for a in range(3)]


def add_wall_ghost(grid, ps, opt, atm: Atmosphere | None = None):
    """(new particles, buckets below that were marked active)"""
    atm = atm or Atmosphere()
    nb = np.array(grid.nb)
    mind = np.array(grid.mindom, dtype=np.float64)
    d = float(grid.del_)
    flags = np.asarray(grid.flags, dtype=np.uint8)
    face = np.asarray(grid.face_index, dtype=np.int8).reshape(-1, 6)
    typ = bucket_types(flags, face)
    pos = np.stack([ps.x, ps.y, ps.z], axis=1)
    b3 = np.clip(np.floor((pos - mind) / d).astype(np.int64), 0, nb - 1)
    pb = (b3[:, 2] * nb[1] + b3[:, 1]) * nb[0] + b3[:, 0]
    count = np.bincount(pb, minlength=len(flags))
    has_wg = np.zeros(len(flags), dtype=bool)
    has_wg[pb[ps.bc_type == BC_WALL]] = True
    dx = float(opt.sml_phase2)
    dx2 = 0.5 * dx
    ground = float(grid.domain_lo[2])
    rows, marked = [], []

    def corners(b):
        i, j, k = b % nb[0], (b // nb[0]) % nb[1], b // (nb[0] * nb[1])
        lo = np.array([mind[0] + i * d, mind[1] + j * d, mind[2] + k * d])
        hi = np.array([mind[0] + (i + 1) * d, mind[1] + (j + 1) * d, mind[2] + (k + 1) * d])
        return lo, hi
    for b in range(len(flags)):
        if not (typ[b] == MIXED and face[b, 4] == -1 and count[b] > 0 and not has_wg[b]):
            continue
        lo, hi = corners(b)
        n3 = _lattice(lo, hi, dx)
        for qi in range(n3[0]):
            for qj in range(n3[1]):
                for qk in range(n3[2]):
                    c = (lo[0] + dx2 + qi * dx, lo[1] + dx2 + qj * dx, lo[2] + dx2 + qk * dx)
                    if c[2] < ground:
                        rows.append(c)
        down = b - nb[0] * nb[1]
        marked.append(down)
        lo, hi = corners(down)
        n3 = _lattice(lo, hi, dx)
        for qi in range(n3[0]):
            for qj in range(n3[1]):
                for qk in range(n3[2]):
                    rows.append((lo[0] + dx2 + qi * dx, lo[1] + dx2 + qj * dx, lo[2] + dx2 + qk * dx))
    return _air_particles(rows, BC_WALL, dx, opt, atm), np.array(marked, dtype=np.int64)


def add_air(grid, binv, ps, opt, atm: Atmosphere | None = None):
    """(new particles, buckets marked active): add_air (add_air.cc:490-795)
    fills every empty bucket whose involvement state is not NONE -- MIXED
    buckets on or below the ground above the ground plane only, other MIXED
    and OVERGROUND buckets whole, PRESS_BC and UNDERGROUND buckets not at
    all -- with real air (bc 100, potentially involved)"""
    atm = atm or Atmosphere()
    nb = np.array(grid.nb)
    mind = np.array(grid.mindom, dtype=np.float64)
    d = float(grid.del_)
    flags = np.asarray(grid.flags, dtype=np.uint8)
    face = np.asarray(grid.face_index, dtype=np.int8).reshape(-1, 6)
    typ = bucket_types(flags, face)
    binv = np.asarray(binv, dtype=np.uint8)
    pos = np.stack([ps.x, ps.y, ps.z], axis=1)
    b3 = np.clip(np.floor((pos - mind) / d).astype(np.int64), 0, nb - 1)
    pb = (b3[:, 2] * nb[1] + b3[:, 1]) * nb[0] + b3[:, 0]
    count = np.bincount(pb, minlength=len(flags))
    dx = float(opt.sml_phase2)
    dx2 = 0.5 * dx
    ground = float(grid.domain_lo[2])
    rows, marked = [], []
    for b in range(len(flags)):
        if binv[b] == 0 or count[b] > 0:
            continue
        marked.append(b)
        if typ[b] not in (MIXED, OVERGROUND):
            continue
        i, j, k = b % nb[0], (b // nb[0]) % nb[1], b // (nb[0] * nb[1])
        lo = np.array([mind[0] + i * d, mind[1] + j * d, mind[2] + k * d])
        hi = np.array([mind[0] + (i + 1) * d, mind[1] + (j + 1) * d, mind[2] + (k + 1) * d])
        n3 = _lattice(lo, hi, dx)
        onground = typ[b] == MIXED and face[b, 4] == -1
        for qi in range(n3[0]):
            for qj in range(n3[1]):
                for qk in range(n3[2]):
                    c = (lo[0] + dx2 + qi * dx, lo[1] + dx2 + qj * dx, lo[2] + dx2 + qk * dx)
                    if onground and not (c[2] > ground):
                        continue
                    rows.append(c)
    out = _air_particles(rows, BC_REAL, dx, opt, atm)
    out.involved[:] = 1
    return out, np.array(marked, dtype=np.int64)


def duct_lattice(duct):
    """the points of setup_erupt's vent duct (setup_erupt.cc:104-230), in
    its order: z from the top down, then x from the axis outward (+ side,
    then - side), then y likewise, keeping x^2 + y^2 <= radius^2; positions
    accumulated by repeated steps of sml as there.  Returns (points, mass,
    sml) with mass and sml of Compute_mass (sph_lib.cc:1024-1040)."""
    r = duct["radius"]
    rng = [(-r, r), (-r, r), (duct["z_top"] - duct["depth"], duct["z_top"])]
    dom = [rng[a][1] - rng[a][0] for a in range(3)]
    vol = 1.0
    for a in range(3):
        vol *= dom[a]
    sml = np.cbrt(vol / duct["np"])
    mss = duct["rho"] * vol / duct["np"]
    s2 = 0.5 * sml

    def side(c0, lo, hi):
        out = []
        v = c0 + s2
        while v <= hi:
            out.append(v)
            v += sml
        v = c0 - s2
        while v >= lo:
            out.append(v)
            v -= sml
        return out
    xs = side(duct["x0"], -r, r)
    ys = side(duct["y0"], -r, r)
    pts = []
    z = rng[2][1] - s2
    while z >= rng[2][0]:
        for x in xs:
            for y in ys:
                if x * x + y * y <= r * r:
                    pts.append((x, y, z))
        z -= sml
    return pts, mss, sml


def setup_erupt(ps, duct, opt):
    """(new erupt ghosts, mask of the particles setup_erupt removes): the
    duct of duct_lattice with the state of the erupt-ghost constructor
    (particle.cc:210-316: rho, e, vertical velocity of the profile, Y 1,
    phase 2, the mixture EOS, then p, c and gamma as given), and the
    particles other than erupt ghosts inside the duct removed
    (setup_erupt.cc:296-310)"""
    pts, mss, sml = duct_lattice(duct)
    r = duct["radius"]
    zlo, ztop = duct["z_top"] - duct["depth"], duct["z_top"]
    d2 = ps.x * ps.x + ps.y * ps.y
    gone = (d2 <= r * r) & (ps.z <= ztop) & (ps.z >= zlo) & (ps.bc_type != 0)
    n = len(pts)
    out = PS(n)
    if n:
        xyz = np.array(pts)
        out.x, out.y, out.z = xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy()
    out.mass[:] = mss
    out.h[:] = sml
    out.rho[:] = duct["rho"]
    out.e[:] = duct["e"]
    out.Y[:] = 1.0
    out.phase[:] = 2
    out.bc_type[:] = 0
    for q in range(n):
        dist = out.x[q] * out.x[q] + out.y[q] * out.y[q]
        out.vz[q] = duct["u_avg"] if duct["profile"] == 0 else duct["u_avg"] * 2 * (1 - dist / (r * r))
        # Particle::update_second_var with Y = 1
        ng = opt.ng0 * 1.0
        ns = 1.0 - ng
        na = 1.0 - 1.0
        cvm = ns * opt.cvs + ng * opt.cvg + na * opt.cva
        out.T[q] = duct["e"] / cvm
        out.cp[q] = cvm if opt.lans else 0.0
    out.p[:] = duct["p"]
    out.c[:] = duct["c"]
    out.gamma[:] = duct["gamma"]
    return out, gone


def _air_particles(rows, bc, dx, opt, atm):
    """particles at rest at the given points with the state of initial_air
    and the mixture EOS (Particle::update_second_var with Y = 0)"""
    n = len(rows)
    out = PS(n)
    if n:
        xyz = np.array(rows)
        out.x, out.y, out.z = xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy()
    out.h[:] = dx
    out.phase[:] = 1
    out.bc_type[:] = bc
    for r in range(n):
        rho, e, p, m = air_state(atm, out.x[r], out.y[r], out.z[r], dx)
        out.rho[r], out.e[r], out.mass[r] = rho, e, m
        # Particle::update_second_var with Y = 0 (air): particle.cc:528-604
        cvm, rm = opt.cva, opt.ra
        out.gamma[r] = 1 + rm / cvm
        out.p[r] = rm * rho * e / cvm
        out.c[r] = np.sqrt(out.gamma[r] * out.p[r] / rho)
        out.T[r] = e / cvm
        out.cp[r] = cvm if opt.lans else 0.0
    return out
