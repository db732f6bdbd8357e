"""ctypes mirror of include/plume_gpu.h and the particle container.

`ParticleSet` holds particles as numpy structure-of-arrays with the fields of
the reference `Particle` record (src/datstr/particle.h:27-140): key, coords,
velocity (state_vars[1..D]), smoothed velocity (LANS), mass, smoothing
length, density (state_vars[0]), internal energy (state_vars[D+1]),
pressure, mass fraction, gamma, sound speed, temperature, specific heat,
phase, bc_type and the involved flag.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

# ---- status codes (plume_gpu.h) ------------------------------------------
PLUME_OK = 0
PLUME_E_INVALID = 1
PLUME_E_CUDA = 2
PLUME_E_NONFINITE = 3
PLUME_E_NONPOSITIVE = 4
PLUME_E_CAPACITY = 5
PLUME_E_OUTSIDE_GRID = 6
PLUME_E_BUCKET_FULL = 7
PLUME_E_TIMEOUT = 8
PLUME_E_NOT_BUILT = 9
STATUS_NAMES = {
    0: "PLUME_OK", 1: "PLUME_E_INVALID", 2: "PLUME_E_CUDA", 3: "PLUME_E_NONFINITE",
    4: "PLUME_E_NONPOSITIVE", 5: "PLUME_E_CAPACITY", 6: "PLUME_E_OUTSIDE_GRID",
    7: "PLUME_E_BUCKET_FULL", 8: "PLUME_E_TIMEOUT", 9: "PLUME_E_NOT_BUILT",
}

BC_ERUPT, BC_PRESSURE, BC_WALL, BC_NOSAVE_REAL, BC_REAL = 0, 1, 2, 99, 100
BUCKET_ABSORBING, BUCKET_MIXED, BUCKET_INACTIVE = 0x1, 0x2, 0x4
BUCKET_UNDERGROUND, BUCKET_PRESS_BC = 0x8, 0x10
BINV_NONE, BINV_POTENTIAL, BINV_INVOLVED, BINV_BOTH = 0, 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1
KERNEL_GAUSS, KERNEL_M4 = 0, 1
METHOD_SPH, METHOD_GSPH, METHOD_GSPH_RCM = 0, 1, 2
RIEMANN_ROE, RIEMANN_HLLC, RIEMANN_HLLC_MY, RIEMANN_VANLEER = 0, 1, 2, 3
RECON_NONE, RECON_EACH, RECON_PAIRWISE, RECON_ALL, RECON_ZEROTH, RECON_EACH_SHOCK = 0, 1, 2, 3, 4, 10

# field order of the double arrays (also the order of the oracle case files)
DOUBLE_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "vsx", "vsy", "vsz", "mass", "h",
                 "rho", "e", "p", "Y", "gamma", "c", "T", "cp")
BYTE_FIELDS = ("phase", "bc_type", "involved")


class PlumeOptions(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("precision", C.c_int), ("kernel", C.c_int),
        ("lans", C.c_int), ("energy_smooth", C.c_int), ("pghost_contrib", C.c_int),
        ("adaptive_sml", C.c_int), ("sml_interval", C.c_int), ("num_loop", C.c_int),
        ("thresh", C.c_double), ("c_smooth", C.c_double), ("eta_smooth", C.c_double),
        ("alpha", C.c_double), ("beta", C.c_double), ("ata", C.c_double),
        ("cfl", C.c_double), ("cutoff2", C.c_double), ("list_factor", C.c_double),
        ("g", C.c_double),
        ("ng0", C.c_double), ("cvs", C.c_double), ("cvg", C.c_double),
        ("cva", C.c_double), ("rg", C.c_double), ("ra", C.c_double),
        ("vent_z", C.c_double), ("sml_phase2", C.c_double),
        ("max_time", C.c_double), ("timeoutput", C.c_double),
        ("stat_erupt", C.c_double), ("end_erupt", C.c_double),
        ("max_steps", C.c_int), ("max_per_bucket", C.c_int),
        ("capacity", C.c_size_t),
        ("method", C.c_int), ("gsph_solver", C.c_int), ("gsph_recon", C.c_int), ("gsph_vol", C.c_int),
        ("gsph_mono", C.c_int), ("gsph_gradients", C.c_int), ("gsph_wave_speed", C.c_int),
    ]


class PlumeAtmosphere(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("Ta0", "pa0", "Ra", "gamma", "H1", "H2", "H3", "miu1", "miu2",
                                          "Ata1", "Ate1", "Ata2", "Atb2", "Ata3", "Atb3", "AtC3", "Ate3")]


@dataclass
class Atmosphere:
    """The hydrostatic atmosphere of ATMOSPHERE_TYPE 1 (air_prop_hydro,
    sph_lib.cc:488-592): temperature and the fitted pressure profile, with
    the values of the 3D section of parameters.h:902-935."""
    Ta0: float = 265.24
    pa0: float = 0.831e5
    Ra: float = 287.0
    gamma: float = 1.4
    H1: float = 11000.0
    H2: float = 20000.0
    H3: float = 100000.0
    miu1: float = 6.5 / 1000
    miu2: float = 2.0 / 1000
    Ata1: float = 1.561024741e-8
    Ate1: float = 5.258643795
    Ata2: float = 1.321758528e+5
    Atb2: float = -0.16963e-3
    Ata3: float = 4.7248e+03
    Atb3: float = 58.5117
    AtC3: float = 5642.519912
    Ate3: float = -0.1709059897e-1

    def to_c(self) -> PlumeAtmosphere:
        a = PlumeAtmosphere()
        for n, _ in PlumeAtmosphere._fields_:
            setattr(a, n, float(getattr(self, n)))
        return a


class PlumeDuct(C.Structure):
    _fields_ = [("x0", C.c_double), ("y0", C.c_double), ("z_top", C.c_double), ("depth", C.c_double),
                ("radius", C.c_double), ("np", C.c_int), ("profile", C.c_int), ("u_avg", C.c_double),
                ("rho", C.c_double), ("e", C.c_double), ("p", C.c_double), ("gamma", C.c_double),
                ("c", C.c_double)]


class PlumeGrid(C.Structure):
    _fields_ = [
        ("mindom", C.c_double * 3), ("del_", C.c_double), ("nb", C.c_int * 3),
        ("subcells", C.c_int),
        ("flags", C.POINTER(C.c_uint8)), ("face_index", C.POINTER(C.c_int8)),
        ("domain_lo", C.c_double * 3), ("domain_hi", C.c_double * 3),
    ]


_DP = C.POINTER(C.c_double)
_BP = C.POINTER(C.c_uint8)


class PlumeSoA(C.Structure):
    _fields_ = [("key", C.POINTER(C.c_uint64))] + [(f, _DP) for f in DOUBLE_FIELDS] + \
               [(f, _BP) for f in BYTE_FIELDS]


class PlumeInlet(C.Structure):
    _fields_ = [("ncol", C.c_size_t), ("col_xy", C.POINTER(C.c_double)), ("col_vel", C.POINTER(C.c_double)),
                ("col_count", C.POINTER(C.c_ulonglong)), ("bot", C.c_double), ("spacing", C.c_double),
                ("mass", C.c_double), ("h", C.c_double), ("rho", C.c_double), ("e", C.c_double),
                ("p", C.c_double), ("gamma", C.c_double), ("c", C.c_double), ("Y", C.c_double),
                ("key_base", C.c_uint64)]


class PlumeStepLog(C.Structure):
    _fields_ = [("dt", C.c_double), ("time", C.c_double), ("step", C.c_int),
                ("status", C.c_int), ("n_total", C.c_uint64), ("n_real", C.c_uint64),
                ("n_lost", C.c_uint64)]


@dataclass
class Options:
    """Python view of PlumeOptions.  Defaults are the reference's 3D plume
    switches (src/plume/options.h:416-837) and constants
    (src/plume/parameters.h:862-1041)."""
    dim: int = 3
    precision: int = PREC_FP64
    kernel: int = KERNEL_GAUSS
    lans: int = 1
    energy_smooth: int = 1
    pghost_contrib: int = 1
    adaptive_sml: int = 1
    sml_interval: int = 50
    num_loop: int = 2
    thresh: float = 1e-5
    c_smooth: float = 2.0
    eta_smooth: float = 1.5
    alpha: float = 0.3
    beta: float = 0.6
    ata: float = 0.01
    cfl: float = 0.8
    cutoff2: float = 8.0
    list_factor: float = 4.25
    g: float = 9.80665
    ng0: float = 0.05
    cvs: float = 1100.0
    cvg: float = 1348.0
    cva: float = 711.0
    rg: float = 462.0
    ra: float = 287.0
    vent_z: float = 0.0
    sml_phase2: float = 150.0
    max_time: float = 1.0e9
    timeoutput: float = 1.0e9
    stat_erupt: float = 0.0
    end_erupt: float = 1.0e9
    max_steps: int = 1 << 30
    max_per_bucket: int = 1 << 30
    capacity: int = 0
    # GSPH switches: the reference's 3D defaults (options.h:545-593)
    method: int = METHOD_SPH
    gsph_solver: int = RIEMANN_ROE
    gsph_recon: int = RECON_EACH_SHOCK
    gsph_vol: int = 3
    gsph_mono: int = 1
    gsph_gradients: int = 0
    gsph_wave_speed: int = 0

    def to_c(self) -> PlumeOptions:
        o = PlumeOptions()
        for name, _ in PlumeOptions._fields_:
            setattr(o, name, getattr(self, name))
        return o


@dataclass
class Grid:
    """Bucket grid (src/datstr/bucket.h; geometry of preprocess.cc:100-177)."""
    mindom: tuple = (0.0, 0.0, 0.0)
    del_: float = 1.0
    nb: tuple = (1, 1, 1)
    subcells: int = 4
    flags: np.ndarray | None = None        # uint8 per bucket, x fastest
    face_index: np.ndarray | None = None   # int8, 6 per bucket
    domain_lo: tuple = (0.0, 0.0, 0.0)
    domain_hi: tuple = (0.0, 0.0, 0.0)
    _keep: list = field(default_factory=list, repr=False)

    @property
    def nbuckets(self) -> int:
        return int(self.nb[0]) * int(self.nb[1]) * int(self.nb[2])

    def to_c(self) -> PlumeGrid:
        g = PlumeGrid()
        g.mindom = (C.c_double * 3)(*self.mindom)
        g.del_ = self.del_
        g.nb = (C.c_int * 3)(*[int(v) for v in self.nb])
        g.subcells = int(self.subcells)
        self._keep = []
        if self.flags is not None:
            f = np.ascontiguousarray(self.flags, dtype=np.uint8)
            self._keep.append(f)
            g.flags = f.ctypes.data_as(_BP)
        if self.face_index is not None:
            fi = np.ascontiguousarray(self.face_index, dtype=np.int8)
            self._keep.append(fi)
            g.face_index = fi.ctypes.data_as(C.POINTER(C.c_int8))
        g.domain_lo = (C.c_double * 3)(*self.domain_lo)
        g.domain_hi = (C.c_double * 3)(*self.domain_hi)
        return g


class ParticleSet:
    """Particles as numpy structure-of-arrays."""

    def __init__(self, n: int = 0):
        self.key = np.zeros(n, dtype=np.uint64)
        for f in DOUBLE_FIELDS:
            setattr(self, f, np.zeros(n, dtype=np.float64))
        for f in BYTE_FIELDS:
            setattr(self, f, np.zeros(n, dtype=np.uint8))

    @property
    def n(self) -> int:
        return int(self.key.shape[0])

    def copy(self) -> "ParticleSet":
        out = ParticleSet(0)
        out.key = self.key.copy()
        for f in DOUBLE_FIELDS + BYTE_FIELDS:
            setattr(out, f, getattr(self, f).copy())
        return out

    @staticmethod
    def concat(parts) -> "ParticleSet":
        out = ParticleSet(0)
        out.key = np.concatenate([p.key for p in parts])
        for f in DOUBLE_FIELDS + BYTE_FIELDS:
            setattr(out, f, np.concatenate([getattr(p, f) for p in parts]))
        return out

    def take(self, idx) -> "ParticleSet":
        out = ParticleSet(0)
        out.key = self.key[idx]
        for f in DOUBLE_FIELDS + BYTE_FIELDS:
            setattr(out, f, getattr(self, f)[idx])
        return out

    def sorted_by_key(self) -> "ParticleSet":
        return self.take(np.argsort(self.key, kind="stable"))

    def soa(self) -> PlumeSoA:
        """ctypes view (arrays must stay alive while it is used)."""
        s = PlumeSoA()
        for f in DOUBLE_FIELDS + BYTE_FIELDS:
            a = getattr(self, f)
            if not a.flags["C_CONTIGUOUS"]:
                a = np.ascontiguousarray(a)
                setattr(self, f, a)
        s.key = self.key.ctypes.data_as(C.POINTER(C.c_uint64))
        for f in DOUBLE_FIELDS:
            setattr(s, f, getattr(self, f).ctypes.data_as(_DP))
        for f in BYTE_FIELDS:
            setattr(s, f, getattr(self, f).ctypes.data_as(_BP))
        return s

    def need_neigh(self) -> np.ndarray:
        return (self.bc_type == BC_REAL) | (self.bc_type == BC_NOSAVE_REAL)

    def __repr__(self) -> str:
        return f"ParticleSet(n={self.n}, real={int(self.need_neigh().sum())})"
