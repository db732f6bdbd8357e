"""Output side of the particle step: host buffers for snapshots and the
reference's text output.

* ``pinned_set(n)``: a ParticleSet whose arrays live in page-locked host
  memory, so that ``Solver.snapshot_begin`` has the device write them
  directly while stepping continues.
* ``real_rows(ps)``: the rows the reference's writers output, the
  non-guest particles with bc_type 100 (h5part_writer.cc:86-88, 470-472;
  a single-GPU table has no guests).
* ``write_csv(path, ps)``: the 1D shock-tube output of write_csv
  (h5part_writer.cc:448-490): the file is opened for appending, a header
  line is written on every call, then one line per real particle of
  ``rho,x,u,e,Y,p,phase,bc_type,guest,involved,h,mass`` with the C++
  stream defaults (six significant digits, the ``%g`` form of printf).
  The guest column is Particle::get_guest, 1 for a particle owned here
  (particle.h:622-626), so 1 on every row of a single-GPU table.
  The header is written as the reference writes it, the last two names
  run together (``smlenpmass``).
"""
from __future__ import annotations

import numpy as np

from .abi import BC_REAL, BYTE_FIELDS, DOUBLE_FIELDS, ParticleSet

CSV_HEADER = "RHO,X,U,E,KS,P,PHASE,BCTP,GUEST_FLAG,INVOLVE_FLAG,smlenpmass\n"


def pinned_set(n: int) -> ParticleSet:
    """ParticleSet of n rows in page-locked host memory (torch's pinned
    allocator; the tensors stay referenced by the set)."""
    import torch
    out = ParticleSet(0)
    keep = []

    def pin(dtype, tdtype):
        t = torch.zeros(n, dtype=tdtype, pin_memory=True)
        keep.append(t)
        return t.numpy().view(dtype)
    out.key = pin(np.uint64, torch.int64)
    for f in DOUBLE_FIELDS:
        setattr(out, f, pin(np.float64, torch.float64))
    for f in BYTE_FIELDS:
        setattr(out, f, pin(np.uint8, torch.uint8))
    out._pinned = keep
    return out


def real_rows(ps: ParticleSet) -> ParticleSet:
    return ps.take(np.nonzero(ps.bc_type == BC_REAL)[0])


def _g(v: float) -> str:
    return "%g" % v


def csv_lines(ps: ParticleSet, order=None) -> list[str]:
    """the lines write_csv appends for ps (header first): its real
    particles, in the row order ``order`` (indices into ps; default:
    ascending x)"""
    idx = np.argsort(ps.x, kind="stable") if order is None else np.asarray(order, dtype=np.int64)
    idx = idx[ps.bc_type[idx] == BC_REAL]
    r = ps
    lines = [CSV_HEADER]
    for i in idx:
        lines.append(",".join((_g(r.rho[i]), _g(r.x[i]), _g(r.vx[i]), _g(r.e[i]), _g(r.Y[i]),
                               _g(r.p[i]), str(int(r.phase[i])), str(int(r.bc_type[i])), "1",
                               str(int(r.involved[i])), _g(r.h[i]), _g(r.mass[i]))) + "\n")
    return lines


def write_csv(path: str, ps: ParticleSet, order=None) -> int:
    """append the shock-tube output of ps to path; returns the rows written"""
    lines = csv_lines(ps, order)
    with open(path, "a") as f:
        f.writelines(lines)
    return len(lines) - 1
