"""ctypes binding of liboracle.so (oracle/sph_oracle.c) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm use it.  Builds the library with `make -C oracle` when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "plume-sph_gb300"))

from plume_gpu.abi import (BYTE_FIELDS, DOUBLE_FIELDS, PlumeGrid, PlumeOptions, PlumeSoA,  # noqa: E402
                           ParticleSet)

_LIB = None


class OracleTime(C.Structure):
    _fields_ = [("time", C.c_double), ("dtime", C.c_double), ("ndtimeoutput", C.c_double),
                ("step", C.c_int), ("ioutput", C.c_int)]


def build():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.oracle_steps.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                   C.POINTER(PlumeSoA), C.POINTER(C.c_size_t),
                                   C.POINTER(OracleTime), C.c_int, C.POINTER(C.c_double), C.c_int]
        L.oracle_adaptive.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                      C.POINTER(PlumeSoA), C.c_size_t, C.c_int]
        L.oracle_pairs.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                   C.POINTER(PlumeSoA), C.c_size_t, C.c_int,
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_size_t,
                                   C.POINTER(C.c_size_t)]
        L.oracle_pairs_of.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                      C.POINTER(PlumeSoA), C.c_size_t, C.c_int,
                                      C.POINTER(C.c_uint64), C.c_size_t,
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_size_t,
                                      C.POINTER(C.c_size_t)]
        L.oracle_sample_step_seconds.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                                 C.POINTER(PlumeSoA), C.c_size_t, C.c_size_t,
                                                 C.c_int]
        L.oracle_sample_step_seconds.restype = C.c_double
        L.oracle_apply_bcond.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                         C.POINTER(PlumeSoA), C.c_size_t, C.POINTER(C.c_uint64),
                                         C.POINTER(C.c_double), C.c_size_t]
        L.oracle_steps_inlet.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                         C.POINTER(PlumeSoA), C.POINTER(C.c_size_t), C.c_size_t,
                                         C.POINTER(OracleTime), C.c_int, C.POINTER(C.c_double), C.c_int,
                                         C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.c_size_t,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.POINTER(C.c_uint64), C.c_size_t, C.POINTER(C.c_double),
                                         C.c_uint64]
        L.oracle_steps_bc.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                      C.POINTER(PlumeSoA), C.POINTER(C.c_size_t),
                                      C.POINTER(OracleTime), C.c_int, C.POINTER(C.c_double), C.c_int,
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.c_size_t]
        L.oracle_steps_grad.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                        C.POINTER(PlumeSoA), C.POINTER(C.c_size_t),
                                        C.POINTER(OracleTime), C.c_int, C.POINTER(C.c_double), C.c_int,
                                        C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_size_t,
                                        C.POINTER(C.c_size_t)]
        L.oracle_scan_outside_layer.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid),
                                                C.POINTER(PlumeSoA), C.c_size_t, C.POINTER(C.c_uint8),
                                                C.POINTER(C.c_int)]
        L.oracle_adapt_domain.argtypes = [C.POINTER(PlumeOptions), C.POINTER(PlumeGrid), C.POINTER(PlumeSoA),
                                          C.c_size_t, C.POINTER(C.c_uint8), C.POINTER(C.c_uint8)]
        _LIB = L
    return _LIB


class OracleRun:
    """Stateful wrapper: particles + time of one oracle run."""

    def __init__(self, case, nthreads: int = 0):
        self.case = case
        self.ps = case.particles.copy()
        self.opt = case.options.to_c()
        self.grid = case.grid.to_c()
        self.t = OracleTime(0.0, 0.0, case.options.timeoutput, case.step0, 0)
        self.nthreads = nthreads

    def adaptive(self):
        s = self.ps.soa()
        rc = lib().oracle_adaptive(C.byref(self.opt), C.byref(self.grid), C.byref(s),
                                   self.ps.n, self.nthreads)
        if rc:
            raise RuntimeError(f"oracle_adaptive failed: {rc}")

    def set_images(self, keys, xyz):
        """wall images (apply_bcond): applied at the end of every step"""
        self.img_key = np.ascontiguousarray(keys, dtype=np.uint64)
        self.img_xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)

    def apply_bcond(self):
        s = self.ps.soa()
        rc = lib().oracle_apply_bcond(C.byref(self.opt), C.byref(self.grid), C.byref(s), self.ps.n,
                                      self.img_key.ctypes.data_as(C.POINTER(C.c_uint64)),
                                      self.img_xyz.ctypes.data_as(C.POINTER(C.c_double)), len(self.img_key))
        if rc:
            raise RuntimeError(f"oracle_apply_bcond failed: {rc}")

    def set_inlet(self, inlet: dict):
        """eruption inlet (plume_gpu.cases.inlet), applied in every step"""
        self.inlet = inlet
        self.inlet_count = np.zeros(len(inlet["col_vel"]), dtype=np.uint64)

    def _steps_inlet(self, nsteps, dts):
        inl = self.inlet
        cap = self.ps.n + nsteps * 8 * len(inl["col_vel"])
        big = ParticleSet(cap)
        for f in ["key"] + list(DOUBLE_FIELDS) + list(BYTE_FIELDS):
            getattr(big, f)[:self.ps.n] = getattr(self.ps, f)
        s = big.soa()
        n = C.c_size_t(self.ps.n)
        keys = getattr(self, "img_key", None)
        ik = keys if keys is not None else np.zeros(0, np.uint64)
        ix = self.img_xyz if keys is not None else np.zeros(0)
        xy = np.ascontiguousarray(inl["col_xy"], dtype=np.float64).reshape(-1)
        vel = np.ascontiguousarray(inl["col_vel"], dtype=np.float64)
        par = np.array([inl[k] for k in ("bot", "spacing", "mass", "h", "rho", "e", "p", "gamma", "c", "Y")],
                       dtype=np.float64)
        D = C.POINTER(C.c_double)
        rc = lib().oracle_steps_inlet(C.byref(self.opt), C.byref(self.grid), C.byref(s), C.byref(n), cap,
                                      C.byref(self.t), nsteps, dts, self.nthreads,
                                      ik.ctypes.data_as(C.POINTER(C.c_uint64)), ix.ctypes.data_as(D), len(ik),
                                      xy.ctypes.data_as(D), vel.ctypes.data_as(D),
                                      self.inlet_count.ctypes.data_as(C.POINTER(C.c_uint64)), len(vel),
                                      par.ctypes.data_as(D), int(inl["key_base"]))
        if rc:
            raise RuntimeError(f"oracle_steps_inlet failed: {rc}")
        self.ps = big.take(np.arange(n.value))
        return np.array(dts[:nsteps])

    def steps(self, nsteps: int):
        s = self.ps.soa()
        n = C.c_size_t(self.ps.n)
        dts = (C.c_double * max(nsteps, 1))()
        if getattr(self, "inlet", None) is not None:
            return self._steps_inlet(nsteps, dts)
        if getattr(self, "img_key", None) is not None:
            rc = lib().oracle_steps_bc(C.byref(self.opt), C.byref(self.grid), C.byref(s), C.byref(n),
                                       C.byref(self.t), nsteps, dts, self.nthreads,
                                       self.img_key.ctypes.data_as(C.POINTER(C.c_uint64)),
                                       self.img_xyz.ctypes.data_as(C.POINTER(C.c_double)),
                                       len(self.img_key))
        else:
            rc = lib().oracle_steps(C.byref(self.opt), C.byref(self.grid), C.byref(s), C.byref(n),
                                    C.byref(self.t), nsteps, dts, self.nthreads)
        if rc:
            raise RuntimeError(f"oracle_steps failed: {rc}")
        if n.value != self.ps.n:
            self.ps = self.ps.take(np.arange(n.value))
        return np.array(dts[:nsteps])

    def steps_grad(self, nsteps: int):
        """steps(), keeping the GSPH gradients of the last step in
        self.grad = (keys, (n, (D+2)*D) array), or None"""
        s = self.ps.soa()
        n = C.c_size_t(self.ps.n)
        dts = (C.c_double * max(nsteps, 1))()
        D = self.case.options.dim
        cap = self.ps.n
        g = np.zeros((cap, (D + 2) * D))
        gk = np.zeros(cap, dtype=np.uint64)
        ng = C.c_size_t(0)
        rc = lib().oracle_steps_grad(C.byref(self.opt), C.byref(self.grid), C.byref(s), C.byref(n),
                                     C.byref(self.t), nsteps, dts, self.nthreads,
                                     g.ctypes.data_as(C.POINTER(C.c_double)),
                                     gk.ctypes.data_as(C.POINTER(C.c_uint64)), cap, C.byref(ng))
        if rc:
            raise RuntimeError(f"oracle_steps_grad failed: {rc}")
        self.grad = (gk[:ng.value], g[:ng.value]) if ng.value else None
        if n.value != self.ps.n:
            self.ps = self.ps.take(np.arange(n.value))
        return np.array(dts[:nsteps])

    def append(self, ps):
        """rows added to the table (particles created outside a step)"""
        out = ParticleSet(self.ps.n + ps.n)
        for f in ["key"] + list(DOUBLE_FIELDS) + list(BYTE_FIELDS):
            getattr(out, f)[:self.ps.n] = getattr(self.ps, f)
            getattr(out, f)[self.ps.n:] = getattr(ps, f)
        self.ps = out

    def scan_outside_layer(self, binv):
        """scan_outside_layer on the current particles; binv (uint8 per
        bucket) is updated in place; returns the count"""
        s = self.ps.soa()
        a = C.c_int(0)
        rc = lib().oracle_scan_outside_layer(C.byref(self.opt), C.byref(self.grid), C.byref(s), self.ps.n,
                                             binv.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(a))
        if rc:
            raise RuntimeError(f"oracle_scan_outside_layer failed: {rc}")
        return a.value

    def adapt_domain(self, binv):
        """adapt_domain; binv and the grid's flags (absorbing bit) updated in place"""
        s = self.ps.soa()
        flags = self.case.grid.flags
        fp = flags.ctypes.data_as(C.POINTER(C.c_uint8)) if flags is not None else None
        rc = lib().oracle_adapt_domain(C.byref(self.opt), C.byref(self.grid), C.byref(s), self.ps.n,
                                       binv.ctypes.data_as(C.POINTER(C.c_uint8)), fp)
        if rc:
            raise RuntimeError(f"oracle_adapt_domain failed: {rc}")

    def pairs(self, mode: int = 0):
        s = self.ps.soa()
        cnt = C.c_size_t(0)
        L = lib()
        rc = L.oracle_pairs(C.byref(self.opt), C.byref(self.grid), C.byref(s), self.ps.n, mode,
                            None, None, 0, C.byref(cnt))
        if rc:
            raise RuntimeError(f"oracle_pairs failed: {rc}")
        ki = np.zeros(cnt.value, dtype=np.uint64)
        kj = np.zeros(cnt.value, dtype=np.uint64)
        rc = L.oracle_pairs(C.byref(self.opt), C.byref(self.grid), C.byref(s), self.ps.n, mode,
                            ki.ctypes.data_as(C.POINTER(C.c_uint64)),
                            kj.ctypes.data_as(C.POINTER(C.c_uint64)), cnt.value, C.byref(cnt))
        if rc:
            raise RuntimeError(f"oracle_pairs failed: {rc}")
        return ki, kj


def _pairs_of(self, keys, mode: int = 0):
    """pairs() of the need_neigh particles whose keys are in `keys`"""
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    kp = keys.ctypes.data_as(C.POINTER(C.c_uint64))
    s = self.ps.soa()
    cnt = C.c_size_t(0)
    L = lib()
    rc = L.oracle_pairs_of(C.byref(self.opt), C.byref(self.grid), C.byref(s), self.ps.n, mode, kp, len(keys),
                           None, None, 0, C.byref(cnt))
    if rc:
        raise RuntimeError(f"oracle_pairs_of failed: {rc}")
    ki = np.zeros(cnt.value, dtype=np.uint64)
    kj = np.zeros(cnt.value, dtype=np.uint64)
    rc = L.oracle_pairs_of(C.byref(self.opt), C.byref(self.grid), C.byref(s), self.ps.n, mode, kp, len(keys),
                           ki.ctypes.data_as(C.POINTER(C.c_uint64)), kj.ctypes.data_as(C.POINTER(C.c_uint64)),
                           cnt.value, C.byref(cnt))
    if rc:
        raise RuntimeError(f"oracle_pairs_of failed: {rc}")
    return ki, kj


OracleRun.pairs_of = _pairs_of


def sample_step_seconds(case, ntarget: int, nthreads: int = 0) -> float:
    ps = case.particles
    s = ps.soa()
    opt = case.options.to_c()
    grid = case.grid.to_c()
    return lib().oracle_sample_step_seconds(C.byref(opt), C.byref(grid), C.byref(s), ps.n,
                                            ntarget, nthreads)
