"""Case / result files of the reference harness oracle/ref/driver.cc --
TEST INFRASTRUCTURE (used by tests/golden/make_golden.py only)."""
from __future__ import annotations

import os
import struct
import subprocess

import numpy as np

from .binding import ParticleSet  # noqa: F401  (sets sys.path)
from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS, ParticleSet as PS

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root() -> str:
    """the reference source tree: $PLUME_REFERENCE, else a directory named
    "reference" beside this checkout"""
    return os.environ.get("PLUME_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                             "reference")


def build_ref(ref_root: str | None = None):
    ref_root = ref_root or reference_root()
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}", "-j8"], check=True)


def write_case(path, case, nsteps, dump_last=False, images=None, binv=None, adapt=False):
    """images: optional (ghost keys, image points (n, 3)) of the wall
    boundary (3D); binv: optional per-bucket involvement states; adapt: 1 runs
    scan_outside_layer / adapt_domain after the steps, 2 also
    add_pressure_ghost (ref3d_adapt)"""
    o, g, ps = case.options, case.grid, case.particles
    with open(path, "wb") as fp:
        fp.write(b"PLSPHIN1")
        fp.write(struct.pack("<6i", o.dim, nsteps, ps.n, int(case.pre_adaptive), int(case.step0),
                             int(dump_last)))
        fp.write(struct.pack("<5d", o.max_time, o.timeoutput, o.stat_erupt, o.end_erupt,
                             o.sml_phase2))
        if o.dim == 3:
            fp.write(struct.pack("<3d", *g.mindom))
            fp.write(struct.pack("<d", g.del_))
            fp.write(struct.pack("<3i", *g.nb))
            fp.write(np.ascontiguousarray(g.flags, dtype=np.uint8).tobytes())
            fp.write(np.ascontiguousarray(g.face_index, dtype=np.int8).tobytes())
            fp.write(struct.pack("<3d", *g.domain_lo))
            fp.write(struct.pack("<3d", *g.domain_hi))
        fp.write(ps.key.astype("<u8").tobytes())
        for f in DOUBLE_FIELDS:
            fp.write(getattr(ps, f).astype("<f8").tobytes())
        for f in BYTE_FIELDS:
            fp.write(getattr(ps, f).astype(np.uint8).tobytes())
        if images is not None or binv is not None:
            keys, xyz = images if images is not None else (np.zeros(0, np.uint64), np.zeros((0, 3)))
            fp.write(struct.pack("<q", len(keys)))
            fp.write(np.ascontiguousarray(keys, dtype="<u8").tobytes())
            fp.write(np.ascontiguousarray(xyz, dtype="<f8").reshape(-1).tobytes())
        if binv is not None:
            fp.write(struct.pack("<q", len(binv)))
            fp.write(np.ascontiguousarray(binv, dtype=np.uint8).tobytes())
            fp.write(struct.pack("<i", int(adapt)))


def read_result(path):
    """Returns (steps, lists): steps = list of dict(dt, time, step, ioutput,
    particles); lists = dict key_i -> np.ndarray of key_j in list order."""
    data = open(path, "rb").read()
    off = 0

    def take(fmt):
        nonlocal off
        v = struct.unpack_from(fmt, data, off)
        off += struct.calcsize(fmt)
        return v

    assert data[:8] == b"PLSPHOU1"
    off = 8
    dim, nsteps = take("<2i")
    steps = []
    for _ in range(nsteps):
        dt, t = take("<2d")
        st, io = take("<2i")
        (n,) = take("<q")
        ps = PS(n)
        ps.key = np.frombuffer(data, "<u8", n, off).copy(); off += 8 * n
        for f in DOUBLE_FIELDS:
            setattr(ps, f, np.frombuffer(data, "<f8", n, off).copy()); off += 8 * n
        for f in BYTE_FIELDS:
            setattr(ps, f, np.frombuffer(data, np.uint8, n, off).copy()); off += n
        steps.append({"dt": dt, "time": t, "step": st, "ioutput": io, "particles": ps})
    (nl,) = take("<q")
    lists = {}
    for _ in range(nl):
        (ki,) = take("<Q")
        (ln,) = take("<q")
        lists[ki] = np.frombuffer(data, "<u8", ln, off).copy(); off += 8 * ln
    if data[off:off + 4] == b"GRAD":
        # GSPH builds: the last step's gradients, (n, (D+2)*D) by key
        off += 4
        (ng,) = take("<q")
        gk = np.frombuffer(data, "<u8", ng, off).copy(); off += 8 * ng
        nq = (dim + 2) * dim
        g = np.frombuffer(data, "<f8", ng * nq, off).copy().reshape(ng, nq); off += 8 * ng * nq
        steps[-1]["grad"] = (gk, g)
    if data[off:off + 4] == b"ADPT":
        # domain growth: the scan's count and the buckets' states after it
        off += 4
        (na,) = take("<i")
        (nbk,) = take("<q")
        st = np.frombuffer(data, np.uint8, nbk, off).copy(); off += nbk
        steps[-1]["adapt"] = (int(na), st)
    if data[off:off + 4] == b"PGHO":
        # the particles the reference created during the run (pressure
        # ghosts of add_pressure_ghost), by key, and bucket activity
        off += 4
        (nn,) = take("<q")
        born = PS(int(nn))
        for f in DOUBLE_FIELDS:
            setattr(born, f, np.frombuffer(data, "<f8", nn, off).copy()); off += 8 * nn
        for f in BYTE_FIELDS:
            setattr(born, f, np.frombuffer(data, np.uint8, nn, off).copy()); off += nn
        nbk = len(steps[-1]["adapt"][1])
        act = np.frombuffer(data, np.uint8, nbk, off).copy(); off += nbk
        steps[-1]["born"] = born
        steps[-1]["active"] = act
    return steps, lists


def run_ref(variant, case, nsteps, workdir, dump_last=False, images=None, binv=None, adapt=False):
    os.makedirs(workdir, exist_ok=True)
    cin = os.path.join(workdir, f"{case.name}.case")
    cout = os.path.join(workdir, f"{case.name}.out")
    write_case(cin, case, nsteps, dump_last, images, binv, adapt)
    exe = os.path.join(HERE, "_ref", variant, "driver")
    subprocess.run([exe, cin, cout], check=True, cwd=workdir)
    return read_result(cout)


# bucket records of oracle/ref/preproc_dump.cc (KEYLENGTH 2, NEIGH_SIZE 27)
_PP_KEYLEN, _PP_NEIGH = 2, 27


def run_preproc(lo, hi, h0, workdir, nproc=1):
    """the reference's preprocessor on the flat-ground domain [lo, hi] with
    smoothing length h0: (htvars, dict of per-bucket arrays over all
    processes' records: key (n, 2), type, proc, index (n, 6), lo (n, 3),
    hi (n, 3), neighs (n, 27, 2), neigh_proc (n, 27))"""
    os.makedirs(workdir, exist_ok=True)
    out = os.path.join(workdir, "funky_dump.bin")
    if os.path.exists(out):
        os.remove(out)
    env = dict(os.environ, ORACLE_DOMAIN=" ".join(repr(float(v)) for v in list(lo) + list(hi)))
    exe = os.path.join(HERE, "_ref", "preproc", "preprocess")
    subprocess.run([exe, str(nproc), repr(float(h0)), "0"], check=True, cwd=workdir, env=env,
                   stdout=subprocess.DEVNULL)
    data = open(out, "rb").read()
    rec = np.dtype([("key", "<u4", _PP_KEYLEN), ("type", "<i4"), ("proc", "<i4"), ("index", "<i4", 6),
                    ("xc", "<f8", 2), ("yc", "<f8", 2), ("zc", "<f8", 2),
                    ("neighs", "<u4", _PP_NEIGH * _PP_KEYLEN), ("neigh_proc", "<i4", _PP_NEIGH)])
    off, parts, ht = 0, [], None
    while off < len(data):
        off += 4  # myid
        ht = np.frombuffer(data, "<f8", 6, off).copy(); off += 48
        (nb,) = np.frombuffer(data, "<i8", 1, off); off += 8
        parts.append(np.frombuffer(data, rec, int(nb), off)); off += int(nb) * rec.itemsize
        (npart,) = np.frombuffer(data, "<i8", 1, off); off += 8 + 4 * int(npart)
    r = np.concatenate(parts)
    return ht, {"key": r["key"].copy(), "type": r["type"].copy(), "proc": r["proc"].copy(),
                "index": r["index"].copy(),
                "lo": np.stack([r["xc"][:, 0], r["yc"][:, 0], r["zc"][:, 0]], axis=1),
                "hi": np.stack([r["xc"][:, 1], r["yc"][:, 1], r["zc"][:, 1]], axis=1),
                "neighs": r["neighs"].reshape(-1, _PP_NEIGH, _PP_KEYLEN).copy(),
                "neigh_proc": r["neigh_proc"].copy()}

