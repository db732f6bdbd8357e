"""Host-side mirror of the reference's per-step interface over the C ABI.

`Solver` owns one plume_ctx (one CUDA stream on the current device).  Its
methods follow the reference free functions the library replaces
(src/plume/particler.h): `step()` is one pass of the hot loop of
src/plume/main.cc:217-471 (3D) / :676-750 (1D); `adaptive_sml()` is the
pre-loop call of the 1D solver (main.cc:643-649); errors are raised as
`PlumeError` carrying the PLUME_E_* status, where the reference asserts.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .abi import (DOUBLE_FIELDS, STATUS_NAMES, ParticleSet, PlumeGrid, PlumeOptions, PlumeSoA,
                  PlumeStepLog)


def generate_grid(lo, hi, h0: float, subcells: int = 4):
    """the preprocessor's bucket grid for the flat-ground domain [lo, hi]
    and smoothing length h0, computed on the device (plume_grid_generate);
    the same grid as cases.plume_grid, with the explicit UNDERGROUND /
    PRESS_BC bits on the absorbing buckets"""
    from .abi import Grid
    L = _lib.lib()
    lo3 = (C.c_double * 3)(*[float(v) for v in lo])
    hi3 = (C.c_double * 3)(*[float(v) for v in hi])
    g = PlumeGrid()
    n = C.c_size_t()
    rc = L.plume_grid_generate(lo3, hi3, float(h0), int(subcells), C.byref(g), None, None, 0, C.byref(n))
    if rc:
        raise PlumeError(rc, "plume_grid_generate")
    flags = np.zeros(n.value, dtype=np.uint8)
    face = np.zeros(6 * n.value, dtype=np.int8)
    rc = L.plume_grid_generate(lo3, hi3, float(h0), int(subcells), C.byref(g),
                               flags.ctypes.data_as(C.POINTER(C.c_uint8)),
                               face.ctypes.data_as(C.POINTER(C.c_int8)), n.value, C.byref(n))
    if rc:
        raise PlumeError(rc, "plume_grid_generate")
    return Grid(mindom=tuple(g.mindom), del_=g.del_, nb=tuple(g.nb), subcells=g.subcells, flags=flags,
                face_index=face, domain_lo=tuple(g.domain_lo), domain_hi=tuple(g.domain_hi))


class PlumeError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} {detail}".strip())


class Solver:
    def __init__(self, case):
        self.case = case
        self.L = _lib.lib()
        self._opt = case.options.to_c()
        if self._opt.capacity == 0:
            self._opt.capacity = max(case.particles.n, 1)
        self._grid = case.grid.to_c()
        self.ctx = C.c_void_p()
        rc = self.L.plume_create(C.byref(self._opt), C.byref(self._grid), C.byref(self.ctx))
        if rc:
            buf = C.create_string_buffer(512)
            self.L.plume_last_error(None, buf, 512)
            raise PlumeError(rc, "plume_create", buf.value.decode())
        if case.particles.n:
            self.upload(case.particles)
        if case.step0:
            self.set_time(0.0, case.step0, 0, case.options.timeoutput)

    # -- helpers ------------------------------------------------------------
    def _check(self, rc, where):
        if rc:
            buf = C.create_string_buffer(512)
            self.L.plume_last_error(self.ctx, buf, 512)
            raise PlumeError(rc, where, buf.value.decode())

    def close(self):
        if self.ctx:
            self.L.plume_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- particles ----------------------------------------------------------
    def upload(self, ps: ParticleSet):
        s = ps.soa()
        self._check(self.L.plume_upload(self.ctx, C.byref(s), ps.n), "plume_upload")

    def upload_device(self, soa: PlumeSoA, n: int):
        self._check(self.L.plume_upload_device(self.ctx, C.byref(soa), n), "plume_upload_device")

    def append(self, ps: ParticleSet):
        s = ps.soa()
        self._check(self.L.plume_append(self.ctx, C.byref(s), ps.n), "plume_append")

    def set_ghost_state(self, keys, state, Y=None):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        state = np.ascontiguousarray(state, dtype=np.float64)
        yp = None
        if Y is not None:
            Y = np.ascontiguousarray(Y, dtype=np.float64)
            yp = Y.ctypes.data_as(C.POINTER(C.c_double))
        self._check(self.L.plume_set_ghost_state(
            self.ctx, keys.ctypes.data_as(C.POINTER(C.c_uint64)),
            state.ctypes.data_as(C.POINTER(C.c_double)), yp, len(keys)), "plume_set_ghost_state")

    def count(self):
        nt, nr = C.c_size_t(), C.c_size_t()
        self._check(self.L.plume_count(self.ctx, C.byref(nt), C.byref(nr)), "plume_count")
        return nt.value, nr.value

    def download_into(self, ps: ParticleSet) -> int:
        """download into existing arrays (e.g. pinned host buffers); returns
        the particle count"""
        s = ps.soa()
        n = C.c_size_t()
        self._check(self.L.plume_download(self.ctx, C.byref(s), ps.n, C.byref(n)), "plume_download")
        return n.value

    def download(self) -> ParticleSet:
        nt, _ = self.count()
        ps = ParticleSet(nt)
        s = ps.soa()
        n = C.c_size_t()
        self._check(self.L.plume_download(self.ctx, C.byref(s), nt, C.byref(n)), "plume_download")
        if n.value != nt:
            ps = ps.take(np.arange(n.value))
        return ps

    # -- time stepping ------------------------------------------------------
    def adaptive_sml(self):
        self._check(self.L.plume_adapt_sml(self.ctx), "plume_adapt_sml")

    def step(self) -> float:
        dt = C.c_double()
        self._check(self.L.plume_step(self.ctx, C.byref(dt)), "plume_step")
        return dt.value

    def steps(self, n: int, log: bool = False):
        if log:
            arr = (PlumeStepLog * max(n, 1))()
            self._check(self.L.plume_steps(self.ctx, n, arr), "plume_steps")
            return [{"dt": a.dt, "time": a.time, "step": a.step, "n_total": a.n_total,
                     "n_real": a.n_real, "n_lost": a.n_lost} for a in arr[:n]]
        self._check(self.L.plume_steps(self.ctx, n, None), "plume_steps")
        return None

    # -- wall boundary -------------------------------------------------------
    def set_wall_images(self, keys, xyz):
        """image table of the wall boundary (keys of wall ghosts, (n, 3)
        image points); empty arrays clear it"""
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        self._check(self.L.plume_set_wall_images(self.ctx, keys.ctypes.data_as(C.POINTER(C.c_uint64)),
                                                 xyz.ctypes.data_as(C.POINTER(C.c_double)), len(keys)),
                    "plume_set_wall_images")

    def set_inlet(self, inlet: dict | None, reserve_per_step: int = 0):
        """eruption inlet (cases.inlet); None clears it; the reserve defaults
        to 4 particles per column"""
        from .abi import PlumeInlet
        if inlet is None:
            self._check(self.L.plume_set_inlet(self.ctx, None, 0), "plume_set_inlet")
            return
        xy = np.ascontiguousarray(inlet["col_xy"], dtype=np.float64).reshape(-1)
        vel = np.ascontiguousarray(inlet["col_vel"], dtype=np.float64)
        self._inlet_keep = (xy, vel)
        s = PlumeInlet(len(vel), xy.ctypes.data_as(C.POINTER(C.c_double)),
                       vel.ctypes.data_as(C.POINTER(C.c_double)), None, inlet["bot"], inlet["spacing"],
                       inlet["mass"], inlet["h"], inlet["rho"], inlet["e"], inlet["p"], inlet["gamma"],
                       inlet["c"], inlet["Y"], inlet["key_base"])
        res = reserve_per_step or 4 * len(vel)
        self._check(self.L.plume_set_inlet(self.ctx, C.byref(s), res), "plume_set_inlet")

    def apply_bcond(self):
        self._check(self.L.plume_apply_bcond(self.ctx), "plume_apply_bcond")

    # -- domain growth --------------------------------------------------------
    def set_bucket_involvement(self, state):
        """per-bucket involvement states (abi.BINV_*), x fastest"""
        st = np.ascontiguousarray(state, dtype=np.uint8)
        self._check(self.L.plume_set_bucket_involvement(self.ctx, st.ctypes.data_as(C.POINTER(C.c_uint8)),
                                                        len(st)), "plume_set_bucket_involvement")

    def bucket_involvement(self):
        st = np.zeros(self.case.grid.nbuckets, dtype=np.uint8)
        self._check(self.L.plume_get_bucket_involvement(self.ctx, st.ctypes.data_as(C.POINTER(C.c_uint8)),
                                                        len(st)), "plume_get_bucket_involvement")
        return st

    def scan_outside_layer(self) -> int:
        """scan_outside_layer: the count that asks for adapt_domain"""
        a = C.c_int(0)
        self._check(self.L.plume_scan_outside_layer(self.ctx, C.byref(a)), "plume_scan_outside_layer")
        return a.value

    def adapt_domain(self):
        self._check(self.L.plume_adapt_domain(self.ctx), "plume_adapt_domain")

    def add_pressure_ghost(self, key_base: int, atmosphere=None) -> int:
        """the pressure-ghost layers that follow an adaptation
        (add_pressure_ghost), on the device; new keys from key_base; returns
        how many particles were added"""
        from .abi import Atmosphere
        a = (atmosphere or Atmosphere()).to_c()
        n = C.c_size_t()
        self._check(self.L.plume_add_pressure_ghost(self.ctx, C.byref(a), int(key_base), C.byref(n)),
                    "plume_add_pressure_ghost")
        return n.value

    def add_wall_ghost(self, key_base: int, atmosphere=None) -> int:
        """the wall-ghost layers of a grown domain (add_wall_ghost), on the
        device; new keys from key_base; returns how many were added"""
        from .abi import Atmosphere
        a = (atmosphere or Atmosphere()).to_c()
        n = C.c_size_t()
        self._check(self.L.plume_add_wall_ghost(self.ctx, C.byref(a), int(key_base), C.byref(n)),
                    "plume_add_wall_ghost")
        return n.value

    def add_air(self, key_base: int, atmosphere=None) -> int:
        """the air of add_air in the empty buckets, on the device; new keys
        from key_base; returns how many particles were added"""
        from .abi import Atmosphere
        a = (atmosphere or Atmosphere()).to_c()
        n = C.c_size_t()
        self._check(self.L.plume_add_air(self.ctx, C.byref(a), int(key_base), C.byref(n)), "plume_add_air")
        return n.value

    def setup_erupt(self, duct: dict, key_base: int):
        """the initial vent duct of setup_erupt, on the device (duct: the
        PlumeDuct fields); returns (added, removed, mass, spacing)"""
        from .abi import PlumeDuct
        d = PlumeDuct(**{k: duct[k] for k, _ in PlumeDuct._fields_})
        na, nr, m, h = C.c_size_t(), C.c_size_t(), C.c_double(), C.c_double()
        self._check(self.L.plume_setup_erupt(self.ctx, C.byref(d), int(key_base), C.byref(na), C.byref(nr),
                                             C.byref(m), C.byref(h)), "plume_setup_erupt")
        return na.value, nr.value, m.value, h.value

    def search_bnd_images(self) -> int:
        """the wall-image table of search_bnd_images (flat ground), found on
        the device from the current wall ghosts and installed; returns the
        number of images"""
        n = C.c_size_t()
        self._check(self.L.plume_search_bnd_images(self.ctx, C.byref(n)), "plume_search_bnd_images")
        return n.value

    def adapt_step(self, key_base: int, atmosphere=None):
        """the adaptation block of the 3D loop (scan, adapt_domain, both
        ghost layers, the image table when wall images are in use);
        returns (the scan's count, particles added)"""
        from .abi import Atmosphere
        a = (atmosphere or Atmosphere()).to_c()
        ad, n = C.c_int(), C.c_size_t()
        self._check(self.L.plume_adapt_step(self.ctx, C.byref(a), int(key_base), C.byref(ad), C.byref(n)),
                    "plume_adapt_step")
        return ad.value, n.value

    # -- output snapshots -----------------------------------------------------
    def snapshot_begin(self, host: ParticleSet):
        """queue a copy of the current particles into host's arrays (the
        fields write_h5part writes, h5part_writer.cc:41-275) and return;
        stepping may continue while the copy runs.  Arrays in page-locked
        memory (pinned_set) are written by the device directly."""
        s = host.soa()
        self._check(self.L.plume_snapshot_begin(self.ctx, C.byref(s), host.n), "plume_snapshot_begin")
        self._snap = (host, s)

    def snapshot_end(self):
        """wait for the snapshot: (rows, time, step)"""
        n, t, st = C.c_size_t(), C.c_double(), C.c_int()
        self._check(self.L.plume_snapshot_end(self.ctx, C.byref(n), C.byref(t), C.byref(st)),
                    "plume_snapshot_end")
        host, _ = self._snap
        self._snap = None
        return host.take(slice(0, n.value)), t.value, st.value

    # -- GSPH -----------------------------------------------------------------
    def gsph_gradients(self):
        """(keys, (n, (D+2)*D) gradients) of the last GSPH step
        (calc_gradients: d rho, d v_0.., d p; x_k fastest)"""
        n = C.c_size_t(0)
        self._check(self.L.plume_gsph_gradients(self.ctx, None, None, 0, C.byref(n)), "plume_gsph_gradients")
        D = self.case.options.dim
        keys = np.zeros(n.value, dtype=np.uint64)
        grad = np.zeros((n.value, (D + 2) * D))
        self._check(self.L.plume_gsph_gradients(self.ctx, keys.ctypes.data_as(C.POINTER(C.c_uint64)),
                                                grad.ctypes.data_as(C.POINTER(C.c_double)), n.value,
                                                C.byref(n)), "plume_gsph_gradients")
        return keys[:n.value], grad[:n.value]

    # -- adjoint --------------------------------------------------------------
    def adjoint_record(self, nsteps: int, checkpoint_every: int = 25):
        """nsteps steps keeping checkpoints for adjoint_backward"""
        self._adj_n0 = self.count()[0]
        self._check(self.L.plume_adjoint_record(self.ctx, nsteps, checkpoint_every),
                    "plume_adjoint_record")

    def adjoint_backward(self, final_bar: ParticleSet):
        """(adjoint of the window's first state as a ParticleSet with keys,
        adjoint of ng0) from the adjoint of the final state (rows by key)"""
        out = ParticleSet(self._adj_n0)
        s_in, s_out = final_bar.soa(), out.soa()
        n0 = C.c_size_t()
        g = C.c_double()
        self._check(self.L.plume_adjoint_backward(self.ctx, C.byref(s_in), final_bar.n, C.byref(s_out),
                                                  out.n, C.byref(n0), C.byref(g)), "plume_adjoint_backward")
        if n0.value != out.n:
            out = out.take(np.arange(n0.value))
        return out, g.value

    def time(self):
        t, s, o = C.c_double(), C.c_int(), C.c_int()
        self._check(self.L.plume_get_time(self.ctx, C.byref(t), C.byref(s), C.byref(o)),
                    "plume_get_time")
        return t.value, s.value, o.value

    def set_time(self, time: float, step: int, ioutput: int, next_output: float):
        self._check(self.L.plume_set_time(self.ctx, time, step, ioutput, next_output),
                    "plume_set_time")

    def pairs(self, mode: int = 0):
        n = C.c_size_t()
        self._check(self.L.plume_neighbor_pairs(self.ctx, mode, None, None, 0, C.byref(n)),
                    "plume_neighbor_pairs")
        ki = np.zeros(n.value, dtype=np.uint64)
        kj = np.zeros(n.value, dtype=np.uint64)
        self._check(self.L.plume_neighbor_pairs(
            self.ctx, mode, ki.ctypes.data_as(C.POINTER(C.c_uint64)),
            kj.ctypes.data_as(C.POINTER(C.c_uint64)), n.value, C.byref(n)), "plume_neighbor_pairs")
        return ki, kj

    def pairs_of(self, keys, mode: int = 0):
        """pairs() of the need_neigh particles whose keys are in `keys`"""
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        kp = keys.ctypes.data_as(C.POINTER(C.c_uint64))
        n = C.c_size_t()
        self._check(self.L.plume_neighbor_pairs_of(self.ctx, mode, kp, len(keys), None, None, 0, C.byref(n)),
                    "plume_neighbor_pairs_of")
        ki = np.zeros(n.value, dtype=np.uint64)
        kj = np.zeros(n.value, dtype=np.uint64)
        self._check(self.L.plume_neighbor_pairs_of(
            self.ctx, mode, kp, len(keys), ki.ctypes.data_as(C.POINTER(C.c_uint64)),
            kj.ctypes.data_as(C.POINTER(C.c_uint64)), n.value, C.byref(n)), "plume_neighbor_pairs_of")
        return ki, kj

    def phase_times(self):
        ms = (C.c_float * 14)()
        self._check(self.L.plume_phase_times(self.ctx, ms, 14), "plume_phase_times")
        names = ["search", "adaptive", "lists", "momentum", "commit_mom", "density", "commit_dens",
                 "velocity", "position", "dt", "total", "mom_kernel", "inlet", "wall_bc"]
        return dict(zip(names, list(ms)))

    def launches(self) -> int:
        n = C.c_uint64()
        self._check(self.L.plume_launch_count(self.ctx, C.byref(n)), "plume_launch_count")
        return int(n.value)


class Ensemble(Solver):
    """Independent runs (members) stepped together in one context.

    `cases` are per-member `Case`s (options, grid, particles).  Members
    share the options the sweeps read (kernel, switches, viscosity,
    cut-offs); their grids, particles, mixture constants, end times and
    time states are their own.  Particle keys are the members' own keys:
    a downloaded row is identified by (member, key)."""

    def __init__(self, cases):
        self.cases = list(cases)
        self.case = self.cases[0]
        self.L = _lib.lib()
        m = len(self.cases)
        self._opts = (PlumeOptions * m)()
        self._grids = (PlumeGrid * m)()
        for k, c in enumerate(self.cases):
            o = c.options.to_c()
            if o.capacity == 0:
                o.capacity = max(c.particles.n, 1)
            self._opts[k] = o
            self._grids[k] = c.grid.to_c()
        self.nmem = m
        self.ctx = C.c_void_p()
        rc = self.L.plume_batch_create(self._opts, self._grids, m, C.byref(self.ctx))
        if rc:
            buf = C.create_string_buffer(512)
            self.L.plume_last_error(None, buf, 512)
            raise PlumeError(rc, "plume_batch_create", buf.value.decode())
        parts = [c.particles for c in self.cases]
        members = np.concatenate([np.full(p.n, k, dtype=np.uint16) for k, p in enumerate(parts)])
        self.upload_members(ParticleSet.concat(parts), members)

    def upload_members(self, ps: ParticleSet, members):
        members = np.ascontiguousarray(members, dtype=np.uint16)
        s = ps.soa()
        self._check(self.L.plume_batch_upload(self.ctx, C.byref(s),
                                              members.ctypes.data_as(C.POINTER(C.c_uint16)), ps.n),
                    "plume_batch_upload")

    def append_members(self, ps: ParticleSet, members):
        members = np.ascontiguousarray(members, dtype=np.uint16)
        s = ps.soa()
        self._check(self.L.plume_batch_append(self.ctx, C.byref(s),
                                              members.ctypes.data_as(C.POINTER(C.c_uint16)), ps.n),
                    "plume_batch_append")

    def download_members(self):
        """(ParticleSet in device order, member id of every row)"""
        nt, _ = self.count()
        ps = ParticleSet(nt)
        mem = np.zeros(nt, dtype=np.uint16)
        s = ps.soa()
        n = C.c_size_t()
        self._check(self.L.plume_batch_download(self.ctx, C.byref(s),
                                                mem.ctypes.data_as(C.POINTER(C.c_uint16)), nt,
                                                C.byref(n)), "plume_batch_download")
        if n.value != nt:
            ps, mem = ps.take(np.arange(n.value)), mem[:n.value]
        return ps, mem

    def split(self):
        """per-member ParticleSets, rows sorted by key"""
        ps, mem = self.download_members()
        out = []
        for k in range(self.nmem):
            idx = np.nonzero(mem == k)[0]
            sub = ps.take(idx)
            out.append(sub.take(np.argsort(sub.key, kind="stable")))
        return out

    def member_times(self):
        """(time, step, running, status) per member"""
        t = np.zeros(self.nmem)
        st = np.zeros(self.nmem, dtype=np.int32)
        run = np.zeros(self.nmem, dtype=np.int32)
        status = np.zeros(self.nmem, dtype=np.int32)
        self._check(self.L.plume_batch_time(self.ctx, t.ctypes.data_as(C.POINTER(C.c_double)),
                                            st.ctypes.data_as(C.POINTER(C.c_int)),
                                            run.ctypes.data_as(C.POINTER(C.c_int)),
                                            status.ctypes.data_as(C.POINTER(C.c_int))),
                    "plume_batch_time")
        return t, st, run.astype(bool), status

    def run(self, max_steps: int, graph_steps: int = 0) -> int:
        """steps every running member until all reached their end time (or
        max_steps); graph_steps > 0 replays CUDA graphs of that many steps"""
        done = C.c_int()
        self._check(self.L.plume_batch_run(self.ctx, max_steps, graph_steps, C.byref(done)),
                    "plume_batch_run")
        return done.value
