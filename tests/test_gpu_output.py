"""Output snapshots (plume_snapshot_begin / plume_snapshot_end): the copy
queued at step k holds the state of step k, bit for bit, while the run
keeps stepping; the run itself is not perturbed.  The twin is a second
context stepped the same way and read with plume_download."""
import numpy as np
import pytest

from plume_gpu import ParticleSet, PlumeError, Solver, cases
from plume_gpu.abi import BYTE_FIELDS
from plume_gpu.output import csv_lines, pinned_set, real_rows

pytestmark = pytest.mark.gpu

SNAP_DOUBLES = ("x", "y", "z", "vx", "vy", "vz", "mass", "h", "rho", "e", "p", "Y")


def _plume():
    # steps 49..: adaptive_sml at step 50, erupt ghosts turning real,
    # outflow deletions (rows leave the table between snapshots)
    case = cases.plume_3d(half_width=300.0, height=600.0, dx=50.0, vent_radius=50.0,
                          vent_dx=25.0, duct_depth=300.0, seed=5, name="plume_small_b")
    case.step0 = 48
    return case


def _same(a, b, fields=SNAP_DOUBLES + BYTE_FIELDS):
    a, b = a.sorted_by_key(), b.sorted_by_key()
    assert a.n == b.n
    np.testing.assert_array_equal(a.key, b.key)
    for f in fields:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


@pytest.mark.parametrize("pinned", [True, False])
def test_snapshot_while_stepping_equals_twin_download(pinned):
    case = _plume()
    a, b = Solver(case), Solver(case)
    a.steps(3)
    b.steps(3)
    n = a.count()[0]
    host = pinned_set(n + 64) if pinned else ParticleSet(n + 64)
    a.snapshot_begin(host)
    a.steps(2)  # queued behind the staging copy, overlapping the host copy
    snap, t, step = a.snapshot_end()
    tb, sb, _ = b.time()
    assert (t, step) == (tb, sb)
    _same(snap, b.download())
    b.steps(2)
    _same(a.download(), b.download(), fields=tuple(SNAP_DOUBLES) + BYTE_FIELDS)
    # back to back, the second one after more steps
    a.snapshot_begin(host)
    snap2, t2, step2 = a.snapshot_end()
    assert step2 == step + 2
    _same(snap2, b.download())
    assert real_rows(snap2).n == int(np.sum(snap2.bc_type == 100)) > 0


def test_snapshot_errors():
    case = _plume()
    s = Solver(case)
    s.steps(1)
    with pytest.raises(PlumeError):
        s.snapshot_end()  # none in flight
    small = ParticleSet(8)
    with pytest.raises(PlumeError):
        s.snapshot_begin(small)  # capacity
    host = ParticleSet(s.count()[0])
    s.snapshot_begin(host)
    with pytest.raises(PlumeError):
        s.snapshot_begin(host)  # one in flight
    s.snapshot_end()


def test_snapshot_csv_of_sod_tube():
    """1D: a snapshot written as the shock-tube CSV equals the CSV of a
    plain download"""
    case = cases.sod_1d(n_real=200)
    a, b = Solver(case), Solver(case)
    for s in (a, b):
        if case.pre_adaptive:
            s.adaptive_sml()
        s.steps(10)
    host = pinned_set(a.count()[0])
    a.snapshot_begin(host)
    snap, _, _ = a.snapshot_end()
    assert csv_lines(snap) == csv_lines(b.download())


@pytest.mark.parametrize("name", ["plume_20km", "plume_600m", "ragged"])
def test_device_grid_equals_preprocessor(name):
    """plume_grid_generate against the reference preprocessor's buckets
    (tests/golden/grid_3d.npz) and cases.plume_grid"""
    import os
    from plume_gpu import generate_grid
    from plume_gpu.abi import (BUCKET_ABSORBING, BUCKET_MIXED, BUCKET_PRESS_BC,
                               BUCKET_UNDERGROUND)
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "grid_3d.npz"))
    dom = d[f"{name}_domain"]
    g = generate_grid(tuple(dom[:3]), tuple(dom[3:6]), float(dom[6]))
    h = cases.plume_grid(tuple(dom[:3]), tuple(dom[3:6]), float(dom[6]))
    assert (g.mindom, g.del_, g.nb) == (h.mindom, h.del_, h.nb)
    np.testing.assert_array_equal(g.face_index, h.face_index)
    np.testing.assert_array_equal(g.flags & (BUCKET_ABSORBING | BUCKET_MIXED), h.flags)
    ht, typ, lo = d[f"{name}_ht"], d[f"{name}_type"], d[f"{name}_lo"]
    nb = np.array(g.nb)
    np.testing.assert_array_equal(ht[0::2], np.array(g.mindom))
    ijk = np.rint((lo - np.array(g.mindom)) / g.del_).astype(np.int64)
    b = (ijk[:, 2] * nb[1] + ijk[:, 1]) * nb[0] + ijk[:, 0]
    f = g.flags[b]
    np.testing.assert_array_equal(f & BUCKET_UNDERGROUND != 0, typ == 1)
    np.testing.assert_array_equal(f & BUCKET_PRESS_BC != 0, typ == 4)
    np.testing.assert_array_equal(f & BUCKET_MIXED != 0, typ == 2)
    np.testing.assert_array_equal(f == 0, typ == 3)
    np.testing.assert_array_equal(g.face_index.reshape(-1, 6)[b], d[f"{name}_index"])
