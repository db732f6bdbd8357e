"""Workload builders: particles, bucket grid and options of each workload.

The host-side set-up keeps the reference's conventions (its set-up code is
not part of the accelerated path):

* 1D shock tubes follow set_up_shock_tube (src/plume/add_air.cc:37-485):
  creation order (left no-save reals, left ghosts, left reals, right reals,
  right no-save reals, right ghosts), equal mass (EQUAL_PART_MASS) or equal
  spacing, ghost h = 1.1 dx (ADAPTIVE_SML_GHOST 11), initial gamma 1.4 and
  sound speed 340 from the Particle constructor (particle.cc:422-520).
* The 3D plume follows the bucket geometry of the preprocessor
  (src/preproc/preprocess.cc:100-177: bucket edge PARTICLE_DENSITY*h0, domain
  padded by 1.5 buckets, bucket types of determine_bucket_type :404-439), a
  cubic air lattice in the original domain, pressure ghosts (bc 1) on the
  sides and top, wall ghosts (bc 2) under the ground and an eruption duct of
  erupt ghosts (bc 0) under the vent like setup_erupt (setup_erupt.cc:44-387:
  a lattice centred on the vent axis, depth 1.5*8*h0, pressure-balanced
  mixture density rhov = pv0/(Rg*Tv0)/ng0, energy ev0).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .abi import (BC_ERUPT, BC_NOSAVE_REAL, BC_PRESSURE, BC_REAL, BC_WALL,
                  BINV_NONE, BINV_POTENTIAL, BUCKET_PRESS_BC, BUCKET_UNDERGROUND,
                  BUCKET_ABSORBING, BUCKET_MIXED, KERNEL_GAUSS, KERNEL_M4,
                  METHOD_GSPH, METHOD_GSPH_RCM, METHOD_SPH, PREC_FP64, RECON_EACH, RECON_ZEROTH, RIEMANN_HLLC,
                  RIEMANN_HLLC_MY, RIEMANN_VANLEER,
                  Grid, Options, ParticleSet)


@dataclass
class Case:
    name: str
    options: Options
    grid: Grid
    particles: ParticleSet
    pre_adaptive: bool = False   # 1D main calls adaptive_sml once before the loop
    step0: int = 0               # TimeProps::step at the start
    info: dict | None = None


def _f32(v: float) -> float:
    return float(np.float32(v))


# ----------------------------------------------------------------------------
# 1D shock tubes
# ----------------------------------------------------------------------------
def _shock_tube(rho_l, p_l, u_l, rho_r, p_r, u_r, middle, lo, hi, s0, nb, nnsrp_l,
                nnsrp_r, equal_mass):
    """Particle placement of set_up_shock_tube (add_air.cc:37-485).

    When the no-save-real count on the left is 0 the first left ghost sits
    at lo - dx/2 (the reference leaves that start position unset)."""
    dx_l = s0
    dx_r = dx_l * rho_l / rho_r if equal_mass else s0
    smlen = max(dx_r, dx_l)
    dx2_l = 0.5 * dx_l
    gmm, sndspd = 1.4, 340.0
    rows = []  # (x, m, h, rho, u, p, bc, involved)

    def rho_at(x):
        return rho_r if x > middle else rho_l

    def p_at(x):
        return p_r if x > middle else p_l

    def u_at(x):
        return u_r if x > middle else u_l

    x = lo - dx2_l
    for k in range(nnsrp_l):
        x = lo - (dx2_l + k * dx_l)
        d = rho_at(x)
        rows.append((x, d * dx_l, smlen, d, u_l, p_l, BC_NOSAVE_REAL, 0))
    if nnsrp_l == 0:
        x = lo - dx2_l + dx_l
    for k in range(nb):
        x -= dx_l
        d = rho_at(x)
        rows.append((x, d * dx_l, dx_l * 1.1, d, u_l, p_l, BC_ERUPT, 0))
    x = lo + dx2_l
    while x <= middle:
        d = rho_at(x)
        rows.append((x, d * dx_l, smlen, d, u_at(x), p_at(x), BC_REAL, 2))
        x += dx_l
    # right-state particles from one right spacing after the last left one
    # (with rho_l < rho_r the first of them can sit just left of `middle`;
    # it still carries the right state, so every real has the same mass)
    x = x - dx_l + dx_r
    while x <= hi:
        rows.append((x, rho_r * dx_r, smlen, rho_r, u_r, p_r, BC_REAL, 2))
        x += dx_r
    for k in range(nnsrp_r):
        d = rho_at(x)
        rows.append((x, d * dx_r, smlen, d, u_r, p_r, BC_NOSAVE_REAL, 2))
        x += dx_r
    for k in range(nb):
        d = rho_at(x)
        rows.append((x, d * dx_r, dx_r * 1.1, d, u_r, p_r, BC_ERUPT, 2))
        x += dx_r
    n = len(rows)
    ps = ParticleSet(n)
    arr = np.array([r[:6] for r in rows], dtype=np.float64)
    ps.key[:] = np.arange(n, dtype=np.uint64)
    ps.x[:] = arr[:, 0]
    ps.mass[:] = arr[:, 1]
    ps.h[:] = arr[:, 2]
    ps.rho[:] = arr[:, 3]
    ps.vx[:] = arr[:, 4]
    ps.p[:] = arr[:, 5]
    ps.e[:] = ps.p / ((gmm - 1) * ps.rho)
    ps.gamma[:] = gmm
    ps.c[:] = sndspd
    ps.Y[:] = 0.0
    ps.phase[:] = 1
    ps.bc_type[:] = np.array([r[6] for r in rows], dtype=np.uint8)
    ps.involved[:] = np.array([r[7] for r in rows], dtype=np.uint8)
    return ps


def options_1d(kernel=KERNEL_GAUSS, eta=1.0, cfl=0.1, cva=717.0, precision=PREC_FP64,
               max_time=0.2, timeoutput=0.1) -> Options:
    """1D switches of src/plume/options.h:16-410 (method SPH unless set;
    the GSPH switches are the 1D defaults: HLLC, zeroth-order states) and the
    1D constants of parameters.h:1225-1448."""
    return Options(dim=1, precision=precision, kernel=kernel, lans=0, energy_smooth=0,
                   pghost_contrib=2, adaptive_sml=1, sml_interval=1, num_loop=5,
                   thresh=1e-5, c_smooth=2.0, eta_smooth=eta, alpha=1.0, beta=2.0,
                   ata=0.01, cfl=cfl, cutoff2=12.0, list_factor=4.25, g=0.0, ng0=0.05,
                   cvs=1100.0, cvg=1348.0, cva=cva, rg=462.0, ra=287.0, vent_z=0.0,
                   sml_phase2=0.0, max_time=_f32(max_time), timeoutput=_f32(timeoutput),
                   stat_erupt=0.0, end_erupt=7200.0, gsph_solver=RIEMANN_HLLC,
                   gsph_recon=RECON_ZEROTH, gsph_vol=0, gsph_mono=0)


def _grid_1d(ps: ParticleSet, opt: Options, cells_per_h: float = 0.5, travel: float = 0.0) -> Grid:
    """A 1D cell grid over the particle span (tiling of the GPU sweeps only;
    1D neighbour lists are every particle, add_air.cc:470-479), padded by
    `travel` for particles that move out of the initial span."""
    span_lo = float(ps.x.min())
    span_hi = float(ps.x.max())
    hmax = float(ps.h.max())
    pad = 8.0 * max(hmax, (span_hi - span_lo) * 1e-3) + travel
    lo = span_lo - pad
    hi = span_hi + pad
    cell = max(hmax * cells_per_h, (hi - lo) / 2.0e6)
    nb = int(math.ceil((hi - lo) / cell))
    return Grid(mindom=(lo, 0.0, 0.0), del_=cell, nb=(nb, 1, 1), subcells=1,
                domain_lo=(lo, 0.0, 0.0), domain_hi=(hi, 0.0, 0.0))


def sod_1d(n_real: int = 2000, ghosts: int = 10, kernel: int = KERNEL_GAUSS,
           precision: int = PREC_FP64, t_end: float = 0.2,
           states=((1.0, 1.0, 0.0), (0.125, 0.1, 0.0)), eta: float = 1.3,
           method: int = METHOD_SPH) -> Case:
    """The 1D Sod workload: [0,1] split at 0.5, equal-mass particles, ideal
    gas gamma = 1.4 (R = 287, Cv = 717.5), h = eta m/rho (eta 1.3),
    alpha=1, beta=2, CFL 0.3, `ghosts` ghosts per end, run to t = 0.2;
    method SPH (artificial viscosity) or GSPH (HLLC Riemann solver, the
    reference's 1D default).

    The kernel defaults to the reference's Gaussian: with the cubic-spline
    kernel swapped in, the reference's own step (built from its sources)
    drives the wall-adjacent particle to negative internal energy and stops
    on its sound-speed assertion (timestep.cc:167) at step 31, so the
    spline variant is only run for its first steps."""
    (rl, pl, ul), (rr, pr, ur) = states
    # input smoothing length (simulation.data, read with stof) giving n_real
    target = 0.5 / n_real * (1 + rr / rl)
    best = None
    for k in range(-400, 401):
        s0 = _f32(target * (1 + k * 2e-5))
        ps = _shock_tube(rl, pl, ul, rr, pr, ur, 0.5, 0.0, 1.0, s0, ghosts, 0, 0, True)
        nr = int(ps.need_neigh().sum())
        if nr == n_real:
            best = (abs(k), s0, ps)
            if k >= 0:
                break
    if best is None:
        raise ValueError(f"no spacing gives {n_real} particles")
    s0, ps = best[1], best[2]
    opt = options_1d(kernel=kernel, eta=eta, cfl=0.3, cva=717.5, precision=precision,
                     max_time=t_end, timeoutput=t_end / 2)
    opt.capacity = ps.n
    opt.method = method
    return Case("sod_1d", opt, _grid_1d(ps, opt), ps, pre_adaptive=True,
                info={"s0": s0, "n_real": n_real, "ghosts_per_end": ghosts})


def shock_tube_1d(test: int = 1, s0: float = 0.003, kernel: int = KERNEL_GAUSS,
                  precision: int = PREC_FP64) -> Case:
    """The reference's shipped 1D shock-tube deck (SHOCK_TUBE_TESTS 1,
    bin/simulation_1D_shocktube_Sod.data): [-0.4,0.4] split at 0, rho 1/0.25,
    p 1/0.1795, 35 ghosts and 40/20 no-save reals per side, equal spacing,
    Gaussian kernel, eta 1.0, CFL 0.1, t_end 0.17."""
    if test != 1:
        raise ValueError("only SHOCK_TUBE_TESTS 1 is provided")
    s0 = _f32(s0)
    ps = _shock_tube(1.0, 1.0, 0.0, 0.25, 0.1795, 0.0, 0.0, -0.4, 0.4, s0, 35, 40, 20, False)
    opt = options_1d(kernel=kernel, eta=1.0, cfl=0.1, cva=717.0, precision=precision,
                     max_time=0.17, timeoutput=0.1)
    opt.capacity = ps.n
    return Case("shock_tube_1d", opt, _grid_1d(ps, opt), ps, pre_adaptive=True,
                info={"s0": s0})


def riemann_member(rho_l, p_l, u_l, rho_r, p_r, u_r, n_real: int, ghosts: int = 10,
                   kernel: int = KERNEL_GAUSS, precision: int = PREC_FP64,
                   t_end: float = 0.2, name: str = "riemann") -> Case:
    """One 1D Riemann problem on [0,1] split at 0.5 with equal-mass particles
    (about n_real of them, h = 1.3 m/rho), ideal gas gamma = 1.4, alpha=1,
    beta=2, CFL 0.3, `ghosts` ghosts per end, run to t_end: the Sod set-up
    with other states.  The grid is padded for the ghosts' travel
    (|u| t_end)."""
    s0 = _f32(0.5 * (1.0 + rho_r / rho_l) / n_real)
    ps = _shock_tube(rho_l, p_l, u_l, rho_r, p_r, u_r, 0.5, 0.0, 1.0, s0, ghosts, 0, 0, True)
    opt = options_1d(kernel=kernel, eta=1.3, cfl=0.3, cva=717.5, precision=precision,
                     max_time=t_end, timeoutput=t_end / 2)
    opt.max_steps = 1 << 30
    opt.capacity = ps.n
    travel = 1.5 * max(abs(u_l), abs(u_r)) * t_end + 0.05
    return Case(name, opt, _grid_1d(ps, opt, travel=travel), ps, pre_adaptive=True,
                info={"s0": s0, "states": ((rho_l, p_l, u_l), (rho_r, p_r, u_r)),
                      "n_real": int(ps.need_neigh().sum())})


def riemann_ensemble(members: int = 256, seed: int = 1, n_lo: int = 500, n_hi: int = 8000,
                     kernel: int = KERNEL_GAUSS, precision: int = PREC_FP64,
                     t_end: float = 0.2) -> list:
    """The 1D ensemble workload: `members` Riemann problems with real
    particle counts log-uniform in [n_lo, n_hi] and left/right states drawn
    from `seed` (rho in [0.1, 1], p in [0.01, 1], u in [-1, 1] per side)."""
    rng = np.random.default_rng(seed)
    cases = []
    for k in range(members):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        rl, rr = rng.uniform(0.1, 1.0, 2)
        pl, pr = rng.uniform(0.01, 1.0, 2)
        ul, ur = rng.uniform(-1.0, 1.0, 2)
        cases.append(riemann_member(float(rl), float(pl), float(ul), float(rr), float(pr), float(ur),
                                    n, kernel=kernel, precision=precision, t_end=t_end,
                                    name=f"riemann_{k}"))
    return cases


# ----------------------------------------------------------------------------
# 3D plume
# ----------------------------------------------------------------------------
def atmosphere(z, T0=288.0, lapse=6.5e-3, z_trop=11000.0, p0=101325.0, R=287.0,
               g=9.80665):
    """Hydrostatic atmosphere: T = T0 - lapse*z to z_trop, isothermal above."""
    z = np.asarray(z, dtype=np.float64)
    zt = np.minimum(z, z_trop)
    T = T0 - lapse * zt
    p = p0 * (T / T0) ** (g / (R * lapse))
    Tt = T0 - lapse * z_trop
    pt = p0 * (Tt / T0) ** (g / (R * lapse))
    above = z > z_trop
    p = np.where(above, pt * np.exp(-g * (z - z_trop) / (R * Tt)), p)
    T = np.where(above, Tt, T)
    rho = p / (R * T)
    return T, p, rho


def _face(crd, lo, hi):
    # determine_face_index, bucket.cc:459-470
    return -1 if crd < lo else (1 if crd > hi else 0)


def plume_grid(lo, hi, h0, subcells=4) -> Grid:
    """Bucket grid of the preprocessor (preprocess.cc:100-177, :404-464):
    the original domain [lo, hi] padded by EXT_DOM_COF = EXT_DOM_COF_BOT =
    1.5 buckets of edge PARTICLE_DENSITY * h0 = 8 h0; bucket types from the
    face indices (a bucket outside the domain on some axis is UNDERGROUND
    when it lies wholly below the ground, else PRESS_BC -- both absorbing
    here; one straddling the domain's edge is MIXED; and every bucket that
    straddles the ground is MIXED, whatever its other axes say)."""
    del_ = 8.0 * h0                     # PARTICLE_DENSITY * smoothing length
    mind = [lo[a] - 1.5 * del_ for a in range(3)]
    maxd = [hi[a] + 1.5 * del_ for a in range(3)]
    nb = [int(math.ceil((maxd[a] - mind[a]) / del_)) for a in range(3)]
    nbk = nb[0] * nb[1] * nb[2]
    flags = np.zeros(nbk, dtype=np.uint8)
    face = np.zeros(6 * nbk, dtype=np.int8)
    for k in range(nb[2]):
        for j in range(nb[1]):
            for i in range(nb[0]):
                b = (k * nb[1] + j) * nb[0] + i
                c0 = [mind[0] + i * del_, mind[1] + j * del_, mind[2] + k * del_]
                c1 = [mind[0] + (i + 1) * del_, mind[1] + (j + 1) * del_,
                      mind[2] + (k + 1) * del_]
                bt = []
                for a in range(3):
                    bt += [_face(c0[a], lo[a], hi[a]), _face(c1[a], lo[a], hi[a])]
                flag = [abs(bt[2 * a] + bt[2 * a + 1]) for a in range(3)]
                face[6 * b:6 * b + 6] = bt
                if bt[4] == -1 and bt[5] == 0:
                    flags[b] = BUCKET_MIXED              # straddles the ground (:462-463)
                elif 2 in flag:
                    flags[b] = BUCKET_ABSORBING          # underground or pressure bc
                elif 1 in flag:
                    flags[b] = BUCKET_MIXED
    return Grid(mindom=tuple(mind), del_=del_, nb=tuple(nb), subcells=subcells,
                flags=flags, face_index=face, domain_lo=tuple(lo), domain_hi=tuple(hi))


def wall_images(case):
    """The image table of search_bnd_images (bnd_image.cc:35-245) for a flat
    ground at the domain's lower z: a wall ghost whose bucket is MIXED and
    has an on-ground MIXED bucket (bottom face below ground, top face inside,
    bucket.h:524-527) among itself and its 26 neighbours gets the image
    2 intsct - x, intsct = (x, y, z_ground) (bucket.cc:294-360 for flat
    ground).  Returns (ghost keys, (n, 3) image points)."""
    g, ps = case.grid, case.particles
    nb = np.array(g.nb)
    mind = np.array(g.mindom)
    zg = g.domain_lo[2]
    wall = np.nonzero(ps.bc_type == BC_WALL)[0]
    pos = np.stack([ps.x[wall], ps.y[wall], ps.z[wall]], axis=1)
    b3 = np.clip(np.floor((pos - mind) / g.del_).astype(np.int64), 0, nb - 1)
    flags = np.asarray(g.flags)
    face = np.asarray(g.face_index).reshape(-1, 6)
    mixed = (flags & BUCKET_MIXED) != 0
    onground = mixed & (face[:, 4] == -1) & (face[:, 5] == 0)

    def lin(b):
        return (b[:, 2] * nb[1] + b[:, 1]) * nb[0] + b[:, 0]
    sel = mixed[lin(b3)]
    near = np.zeros(len(wall), dtype=bool)
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                q = b3 + np.array([dx, dy, dz])
                ok = np.all((q >= 0) & (q < nb), axis=1)
                qq = np.where(ok[:, None], q, 0)
                near |= ok & onground[lin(qq)]
    sel &= near
    keys = ps.key[wall[sel]]
    img = pos[sel].copy()
    img[:, 2] = 2 * zg - img[:, 2]
    return keys, img


def adapt_scenario(case, clear_beyond=False):
    """A domain-growth set-up on a plume built by plume_3d: explicit bucket
    types (absorbing buckets below the ground UNDERGROUND, the other
    absorbing ones PRESS_BC), involvement NONE where absorbing and POTENTIAL
    elsewhere (dataread.cc:457); then the outermost non-absorbing bucket
    layer on the +x side becomes a NONE layer of pressure ghosts (absorbing,
    its real particles bc 1, as add_pressure_ghost leaves the ring around
    the domain), and the particles of the layer inside it that sit in the
    outer half of their bucket are marked involved (2).  The scan then finds
    involved particles next to the pressure layer, and adapt_domain converts
    that layer.  clear_beyond: the particles of the bucket layer outside it
    are removed, so that add_pressure_ghost refills those buckets after
    the adaptation.  Returns (new case, per-bucket involvement states)."""
    import dataclasses
    g0 = case.grid
    nb = np.array(g0.nb)
    flags = np.array(g0.flags, dtype=np.uint8).copy()
    face = np.asarray(g0.face_index, dtype=np.int8).reshape(-1, 6)
    absorbing = (flags & BUCKET_ABSORBING) != 0
    under = absorbing & (face[:, 4] == -1) & (face[:, 5] == -1)
    flags[under] |= BUCKET_UNDERGROUND
    flags[absorbing & ~under] |= BUCKET_PRESS_BC
    binv = np.where(absorbing, BINV_NONE, BINV_POTENTIAL).astype(np.uint8)
    idx = np.arange(len(flags))
    bx = idx % nb[0]
    # non-absorbing buckets not wholly beyond the domain in +x (the
    # ground-straddling MIXED ring outside the domain is left as it is)
    cand = ~absorbing & (face[:, 0] != 1)
    bx_max = int(bx[cand].max())
    layer = cand & (bx == bx_max)
    inner = cand & (bx == bx_max - 1)
    flags[layer] |= BUCKET_ABSORBING
    binv[layer] = BINV_NONE
    ps = case.particles.copy()
    pos = np.stack([ps.x, ps.y, ps.z], axis=1)
    mind = np.array(g0.mindom)
    b3 = np.clip(np.floor((pos - mind) / g0.del_).astype(np.int64), 0, nb - 1)
    pb = (b3[:, 2] * nb[1] + b3[:, 1]) * nb[0] + b3[:, 0]
    real = (ps.bc_type == BC_REAL) | (ps.bc_type == BC_NOSAVE_REAL)
    ps.bc_type[layer[pb] & real] = BC_PRESSURE
    ps.involved[layer[pb] & real] = 0
    outer_half = (pos[:, 0] - (mind[0] + b3[:, 0] * g0.del_)) > 0.5 * g0.del_
    ps.involved[inner[pb] & real & outer_half] = 2
    if clear_beyond:
        ps = ps.take(np.nonzero(b3[:, 0] != bx_max + 1)[0])
    grid = dataclasses.replace(g0, flags=flags, face_index=np.array(g0.face_index).copy())
    return dataclasses.replace(case, grid=grid, particles=ps, name=case.name + "_adapt"), binv


def wall_scenario(case):
    """A wall-ghost set-up on a plume built by plume_3d: in the on-ground
    MIXED buckets of the column of buckets second from the -x side of the
    original domain, the wall ghosts are removed, and so is every particle
    of the buckets below them, so that add_wall_ghost refills both.
    Returns (new case, per-bucket involvement states: NONE where absorbing,
    POTENTIAL elsewhere)."""
    import dataclasses
    g = case.grid
    nb = np.array(g.nb)
    flags = np.asarray(g.flags, dtype=np.uint8)
    face = np.asarray(g.face_index, dtype=np.int8).reshape(-1, 6)
    idx = np.arange(len(flags))
    bx, by, bz = idx % nb[0], (idx // nb[0]) % nb[1], idx // (nb[0] * nb[1])
    onground = ((flags & BUCKET_MIXED) != 0) & (face[:, 4] == -1)
    col = int(bx[onground & (face[:, 0] == -1) & (face[:, 1] == 0)].min()) + 1
    target = onground & (bx == col)
    below = np.zeros(len(flags), dtype=bool)
    for b in idx[target]:
        if bz[b] > 0:
            below[b - nb[0] * nb[1]] = True
    ps = case.particles
    pos = np.stack([ps.x, ps.y, ps.z], axis=1)
    b3 = np.clip(np.floor((pos - np.array(g.mindom)) / g.del_).astype(np.int64), 0, nb - 1)
    pb = (b3[:, 2] * nb[1] + b3[:, 1]) * nb[0] + b3[:, 0]
    drop = (target[pb] & (ps.bc_type == BC_WALL)) | below[pb]
    ps = ps.take(np.nonzero(~drop)[0])
    binv = np.where((flags & BUCKET_ABSORBING) != 0, BINV_NONE, BINV_POTENTIAL).astype(np.uint8)
    return dataclasses.replace(case, particles=ps, name=case.name + "_walls"), binv


def air_scenario(case):
    """An add_air set-up on a plume built by plume_3d: every particle of a
    block of buckets is removed -- 2 x 2 buckets across, from the ground
    up through three layers, in the +x +y quarter next to the vent axis
    (on-ground MIXED and OVERGROUND buckets) -- so that add_air refills
    them.  Returns (new case, per-bucket involvement states: NONE where
    absorbing, POTENTIAL elsewhere)."""
    import dataclasses
    g = case.grid
    nb = np.array(g.nb)
    flags = np.asarray(g.flags, dtype=np.uint8)
    face = np.asarray(g.face_index, dtype=np.int8).reshape(-1, 6)
    idx = np.arange(len(flags))
    bx, by, bz = idx % nb[0], (idx // nb[0]) % nb[1], idx // (nb[0] * nb[1])
    mind = np.array(g.mindom)
    cx = int(np.floor((0.0 - mind[0]) / g.del_)) + 1
    cy = int(np.floor((0.0 - mind[1]) / g.del_)) + 1
    k0 = int(bz[(face[:, 4] == -1) & (face[:, 5] == 0)].min())
    block = ((bx >= cx) & (bx < cx + 2) & (by >= cy) & (by < cy + 2) & (bz >= k0) & (bz < k0 + 3)
             & ((flags & BUCKET_ABSORBING) == 0))
    ps = case.particles
    pos = np.stack([ps.x, ps.y, ps.z], axis=1)
    b3 = np.clip(np.floor((pos - mind) / g.del_).astype(np.int64), 0, nb - 1)
    pb = (b3[:, 2] * nb[1] + b3[:, 1]) * nb[0] + b3[:, 0]
    ps = ps.take(np.nonzero(~block[pb])[0])
    binv = np.where((flags & BUCKET_ABSORBING) != 0, BINV_NONE, BINV_POTENTIAL).astype(np.uint8)
    return dataclasses.replace(case, particles=ps, name=case.name + "_air"), binv


def duct_scenario(case):
    """A setup_erupt set-up on a plume built by plume_3d: its erupt ghosts
    (the vent duct) removed, so that setup_erupt builds the duct again.
    Returns (new case, per-bucket involvement states: NONE where absorbing,
    POTENTIAL elsewhere) and the duct of the reference's constants
    (parameters.h: radius rv_P 120 m, 1,080 particles, depth
    EXT_DOM_COF * PARTICLE_DENSITY smoothing lengths below the ground,
    parabolic profile of mean speed Vv0_P 75 m/s); the vent state
    (rho, e, p, gamma, c) is left for the caller."""
    import dataclasses
    ps = case.particles
    ps = ps.take(np.nonzero(ps.bc_type != BC_ERUPT)[0])
    flags = np.asarray(case.grid.flags, dtype=np.uint8)
    binv = np.where((flags & BUCKET_ABSORBING) != 0, BINV_NONE, BINV_POTENTIAL).astype(np.uint8)
    duct = dict(x0=0.0, y0=0.0, z_top=float(case.grid.domain_lo[2]), depth=case.options.sml_phase2 * 1.5 * 8,
                radius=120.0, np=1080, profile=1, u_avg=75.0)
    return dataclasses.replace(case, particles=ps, name=case.name + "_duct"), binv, duct


def duct_inlet(duct: dict, born: ParticleSet, key_base: int) -> dict:
    """The inlet of add_new_erupt (setup_erupt.cc:389-673) for a vent duct
    that setup_erupt built (setup_erupt.cc:44-388) from the duct description
    of duct_scenario: the columns of the reference's loops (x from the vent
    axis + sml/2 outward by repeated steps of sml, + side then - side, y the
    same inside each, kept where x^2 + y^2 <= radius^2), each with the
    speed of the velocity profile (profile 1: parabolic_vel, 2 u_avg
    (1 - r^2 / R^2), sph_lib.cc:1223-1227; 0: uniform_vel), the bottom of
    the duct (simprops bot = z_top - depth), and the state of the duct's
    particles (sml_of_phase2, mass_of_phase2, rhov, ev0, pv0, gamma_v,
    sound speed 340, mass fraction 1)."""
    sml = float(born.h[0])
    sml2 = 0.5 * sml
    rv = float(duct["radius"])
    rvsq = rv * rv
    x0, y0 = float(duct["x0"]), float(duct["y0"])

    def speed(rsq):
        if int(duct["profile"]) == 1:
            umax = float(duct["u_avg"]) * 2
            return umax * (1 - (rsq / (rv * rv)))
        return float(duct["u_avg"])

    xy, vel = [], []

    def row(x):
        for sgn in (1, -1):
            y = y0 + sgn * sml2
            while (y <= rv) if sgn > 0 else (y >= -rv):
                rsq = 0.0
                rsq += x * x
                rsq += y * y
                if rsq <= rvsq:
                    xy.append((x, y))
                    vel.append(speed(rsq))
                y = y + sml if sgn > 0 else y - sml

    x = x0 + sml2
    while x <= rv:
        row(x)
        x += sml
    x = x0 - sml2
    while x >= -rv:
        row(x)
        x -= sml
    i0 = 0
    return {"col_xy": np.array(xy, dtype=np.float64), "col_vel": np.array(vel, dtype=np.float64),
            "bot": float(duct["z_top"]) - float(duct["depth"]), "spacing": sml,
            "mass": float(born.mass[i0]), "h": sml, "rho": float(born.rho[i0]), "e": float(born.e[i0]),
            "p": float(born.p[i0]), "gamma": float(born.gamma[i0]), "c": float(born.c[i0]), "Y": 1.0,
            "key_base": int(key_base)}


def inlet(case):
    """The eruption inlet of add_new_erupt (setup_erupt.cc:389-673) for a
    plume built by plume_3d: the duct's particle columns (spacing vent_dx,
    inside the vent radius), bottom = the duct's lowest particle, the vent
    state of the Particle constructor (particle.cc:210-316: p = the vent
    pressure, c = 340 m/s, gamma of the vent mixture) and uniform inflow at
    the vent velocity (ERUPT_VELOCITY_PROF 0).  Keys continue after the
    case's largest key."""
    ps, info, opt = case.particles, case.info, case.options
    vent = (ps.bc_type == BC_ERUPT) & (ps.phase == 2)
    vdx = info["vent_dx"]
    cols = np.unique(np.round(np.stack([ps.x[vent], ps.y[vent]], axis=1) / (0.5 * vdx)).astype(np.int64),
                     axis=0) * (0.5 * vdx)
    v0 = float(ps.vz[vent].max())
    i0 = int(np.nonzero(vent)[0][0])
    return {"col_xy": cols.astype(np.float64), "col_vel": np.full(len(cols), v0),
            "bot": float(ps.z[vent].min()), "spacing": vdx, "mass": float(ps.mass[i0]), "h": vdx,
            "rho": float(ps.rho[i0]), "e": float(ps.e[i0]), "p": info.get("p0", 101325.0),
            "gamma": float(ps.gamma[i0]), "c": 340.0, "Y": 1.0,
            "key_base": int(ps.key.max()) + 1}


def options_3d(precision=PREC_FP64, h0=150.0, cva=711.0) -> Options:
    """3D plume switches (options.h:416-837 with ATMOSPHERE_TYPE 1, USE_GSPH 0)
    and constants (parameters.h:862-1041 with cp = 998, ash 0.95)."""
    return Options(dim=3, precision=precision, kernel=KERNEL_GAUSS, lans=1, energy_smooth=1,
                   pghost_contrib=1, adaptive_sml=1, sml_interval=50, num_loop=2,
                   thresh=1e-5, c_smooth=2.0, eta_smooth=1.5, alpha=0.3, beta=0.6,
                   ata=0.01, cfl=0.8, cutoff2=8.0, list_factor=4.25, g=9.80665,
                   ng0=0.05, cvs=1100.0, cvg=1348.0, cva=cva, rg=462.0, ra=287.0,
                   vent_z=0.0, sml_phase2=h0, max_time=_f32(1.0e5), timeoutput=_f32(1.0e5),
                   stat_erupt=0.0, end_erupt=_f32(72000.0), max_per_bucket=1 << 30)


def _eos(opt: Options, ps: ParticleSet, sel=slice(None)):
    """Particle::update_second_var (particle.cc:528-604), vectorised."""
    Y = ps.Y[sel]
    na = 1 - Y
    ng = opt.ng0 * Y
    ns = Y - ng
    Cvm = ns * opt.cvs + ng * opt.cvg + na * opt.cva
    Rm = ng * opt.rg + na * opt.ra
    Rmg = Rm / (ng + na)
    gam = 1 + Rm / Cvm
    desmg = ps.rho[sel] * (na + ng)
    p = Rmg * desmg * ps.e[sel] / Cvm
    ps.gamma[sel] = gam
    ps.p[sel] = p
    ps.c[sel] = np.sqrt(gam * p / desmg)
    ps.T[sel] = ps.e[sel] / Cvm
    if opt.lans:
        ps.cp[sel] = Cvm


def plume_3d(half_width=1.0e4, height=2.0e4, dx=150.0, vent_radius=100.0,
             vent_velocity=150.0, vent_T=1053.0, ash=0.95, ghost_layers=6,
             vent_dx=None, duct_depth=None, jitter=0.01, seed=0, precision=PREC_FP64,
             T0=288.0, lapse=6.5e-3, p0=101325.0, subcells=4, name="plume_3d") -> Case:
    """The 3D dusty-gas plume workload (20 x 20 x 20 km, 150 m lattice,
    hydrostatic 288 K atmosphere with 6.5 K/km lapse to 11 km, air cp = 998 and
    R = 287, vent of radius 100 m at ground centre injecting at 150 m/s and
    1053 K with ash mass fraction 0.95, outflow ghosts on sides and top,
    +-1% lattice jitter from `seed`), and smaller copies of it for tests."""
    opt = options_3d(precision=precision, h0=dx)
    lo = (-half_width, -half_width, 0.0)
    hi = (half_width, half_width, height)
    grid = plume_grid(lo, hi, dx, subcells=subcells)
    rng = np.random.default_rng(seed)
    g = opt.g
    # lattice centred on the vent axis: x = (i + 1/2) dx
    nxh = int(math.ceil(half_width / dx)) + ghost_layers
    xs = (np.arange(-nxh, nxh) + 0.5) * dx
    nz = int(math.ceil(height / dx)) + ghost_layers
    zs = (np.arange(-ghost_layers, nz) + 0.5) * dx
    X, Yc, Z = np.meshgrid(xs, xs, zs, indexing="ij")
    X = X.ravel(); Yc = Yc.ravel(); Z = Z.ravel()
    inside = (np.abs(X) < half_width) & (np.abs(Yc) < half_width) & (Z > 0) & (Z < height)
    pad = ghost_layers * dx
    near = (np.abs(X) < half_width + pad) & (np.abs(Yc) < half_width + pad) & \
           (Z < height + pad) & (Z > -pad)
    rv = vent_radius
    vdx = vent_dx if vent_dx is not None else min(dx, rv / 2.0)
    duct = duct_depth if duct_depth is not None else 1.5 * 8.0 * dx
    in_duct_col = (X ** 2 + Yc ** 2) <= (rv + 0.5 * dx) ** 2
    press = near & ~inside & (Z > 0)
    wall = near & (Z < 0) & ~(in_duct_col & (Z > -duct))
    parts = []

    def lattice_set(mask, bc, jit):
        n = int(mask.sum())
        ps = ParticleSet(n)
        x, y, z = X[mask].copy(), Yc[mask].copy(), Z[mask].copy()
        if jit:
            x += rng.uniform(-jitter, jitter, n) * dx
            y += rng.uniform(-jitter, jitter, n) * dx
            z += rng.uniform(-jitter, jitter, n) * dx
        ps.x[:], ps.y[:], ps.z[:] = x, y, z
        zz = np.abs(z) if bc == BC_WALL else z
        T, p, rho = atmosphere(zz, T0=T0, lapse=lapse, p0=p0, R=opt.ra, g=g)
        ps.rho[:] = rho
        ps.e[:] = opt.cva * T
        ps.mass[:] = rho * dx ** 3
        ps.h[:] = dx
        ps.Y[:] = 0.0
        ps.phase[:] = 1
        ps.bc_type[:] = bc
        ps.involved[:] = 0
        return ps

    parts.append(lattice_set(inside, BC_REAL, jitter > 0))
    parts.append(lattice_set(press, BC_PRESSURE, jitter > 0))
    parts.append(lattice_set(wall, BC_WALL, jitter > 0))
    # eruption duct (setup_erupt.cc:44-387): lattice of spacing vdx centred on
    # the vent axis, from z = -vdx/2 down to -duct
    nv = int(math.ceil(rv / vdx))
    vx = (np.arange(-nv, nv) + 0.5) * vdx
    vz = -(np.arange(int(duct // vdx)) + 0.5) * vdx
    VX, VY, VZ = np.meshgrid(vx, vx, vz, indexing="ij")
    VX = VX.ravel(); VY = VY.ravel(); VZ = VZ.ravel()
    m = (VX ** 2 + VY ** 2) <= rv * rv
    ne = int(m.sum())
    ev = ParticleSet(ne)
    ev.x[:], ev.y[:], ev.z[:] = VX[m], VY[m], VZ[m]
    ng0 = 1.0 - ash
    Tv = vent_T
    pv = p0
    rhov = pv / (opt.rg * Tv) / ng0          # rhov_P = pv0/(Rg Tv0)/ng0
    ev.rho[:] = rhov
    ev.e[:] = (ng0 * opt.cvg + (1 - ng0) * opt.cvs) * Tv   # ev0_P
    ev.vz[:] = vent_velocity
    ev.mass[:] = rhov * vdx ** 3
    ev.h[:] = vdx
    ev.Y[:] = 1.0
    ev.phase[:] = 2
    ev.bc_type[:] = BC_ERUPT
    ev.involved[:] = 0
    parts.append(ev)
    ps = ParticleSet.concat(parts)
    ps.key[:] = np.arange(ps.n, dtype=np.uint64)
    opt.ng0 = ng0
    _eos(opt, ps)
    opt.capacity = int(ps.n * 1.25) + 1024
    info = {"dx": dx, "vent_dx": vdx, "duct_depth": duct, "n_air": int(inside.sum()),
            "n_vent": ne, "rhov": rhov, "half_width": half_width, "height": height}
    return Case(name, opt, grid, ps, info=info)


def plume_small(seed=0, precision=PREC_FP64, subcells=4) -> Case:
    """A 800 m cube of the 3D plume at 50 m spacing (test size)."""
    return plume_3d(half_width=400.0, height=800.0, dx=50.0, vent_radius=50.0,
                    vent_velocity=150.0, vent_dx=25.0, duct_depth=300.0, seed=seed,
                    precision=precision, subcells=subcells, name="plume_small")


def plume_config2(seed=0, precision=PREC_FP64, subcells=4) -> Case:
    """The full 3D plume workload: 20 x 20 x 20 km at 150 m (134^3 air)."""
    return plume_3d(seed=seed, precision=precision, subcells=subcells, name="plume_3d_config2")


def plume_ensemble(members: int = 64, seed: int = 2, dx: float = 60.0, n_lo: float = 5.0e4,
                   n_hi: float = 4.0e5, precision: int = PREC_FP64, subcells: int = 4,
                   vent_radius: float = 100.0, duct_depth: float | None = None) -> list:
    """The 3D ensemble workload: `members` small copies of the plume at `dx`
    spacing, each a cube whose side gives about N_k air particles, N_k
    log-uniform in [n_lo, n_hi]; vent velocity U[80, 200] m/s, temperature
    U[900, 1200] K and ash mass fraction U[0.9, 0.98] per member, drawn from
    `seed` (the lattice jitter of member k uses seed + 1000 k)."""
    rng = np.random.default_rng(seed)
    cases = []
    for k in range(members):
        n = math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))
        side = dx * n ** (1.0 / 3.0)
        v = float(rng.uniform(80.0, 200.0))
        T = float(rng.uniform(900.0, 1200.0))
        ash = float(rng.uniform(0.9, 0.98))
        c = plume_3d(half_width=0.5 * side, height=side, dx=dx, vent_radius=vent_radius,
                     vent_velocity=v, vent_T=T, ash=ash, duct_depth=duct_depth,
                     seed=seed + 1000 * k, precision=precision, subcells=subcells,
                     name=f"plume_member_{k}")
        c.info.update({"vent_velocity": v, "vent_T": T, "ash": ash})
        cases.append(c)
    return cases
