"""Domain growth on the GPU (scan_outside_layer, adapt_domain) against the
reference's own functions (tests/golden/adapt_3d.npz) and the oracle."""
import os

import numpy as np
import pytest

from oracle.binding import OracleRun
from plume_gpu import Solver, cases
from plume_gpu.abi import BINV_BOTH, BINV_NONE, BINV_POTENTIAL
from _util import adapt_case, unpack

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "adapt_3d.npz")


def _fixture():
    d = dict(np.load(GOLDEN))
    c, binv = cases.adapt_scenario(adapt_case())
    c.particles = unpack(d, "in_")
    c.grid.flags = np.array(d["flags"], dtype=np.uint8)
    return c, d


def test_domain_growth_matches_reference():
    c, d = _fixture()
    s = Solver(c)
    s.set_bucket_involvement(d["binv_in"])
    s.steps(int(d["nsteps"]))
    a = s.scan_outside_layer()
    assert a == int(d["adapt"])
    st = s.bucket_involvement()
    assert np.count_nonzero(st == BINV_BOTH) == np.count_nonzero(d["binv_out"] == BINV_BOTH)
    s.adapt_domain()
    np.testing.assert_array_equal(s.bucket_involvement(), d["binv_out"])
    g = s.download().sorted_by_key()
    np.testing.assert_array_equal(g.key, d["out_key"])
    np.testing.assert_array_equal(g.bc_type, d["out_bc_type"])
    np.testing.assert_array_equal(g.involved, d["out_involved"])
    np.testing.assert_allclose(g.x, d["out_x"], rtol=0, atol=1e-9)


def test_converted_buckets_stop_absorbing():
    """after adapt_domain a real particle may enter the converted layer:
    two more steps on the device and the oracle lose the same particles"""
    c, d = _fixture()
    s = Solver(c)
    s.set_bucket_involvement(d["binv_in"])
    s.steps(1)
    s.scan_outside_layer()
    s.adapt_domain()
    s.steps(2)
    o = OracleRun(c)
    o.steps(1)
    b = np.array(d["binv_in"], dtype=np.uint8)
    o.scan_outside_layer(b)
    o.adapt_domain(b)
    o.steps(2)
    g, r = s.download().sorted_by_key(), o.ps.sorted_by_key()
    np.testing.assert_array_equal(g.key, r.key)
    np.testing.assert_array_equal(g.bc_type, r.bc_type)
    err = np.abs(g.rho - r.rho).max() / np.abs(r.rho).max()
    assert err <= 1e-10, err


def test_default_involvement_follows_absorbing_flags():
    c, _ = _fixture()
    s = Solver(c)
    st = s.bucket_involvement()
    absorbing = (c.grid.flags & cases.BUCKET_ABSORBING) != 0
    np.testing.assert_array_equal(st, np.where(absorbing, BINV_NONE, BINV_POTENTIAL))


def _pg_fixture():
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "adapt_pg_3d.npz")))
    c, _ = cases.adapt_scenario(adapt_case(), clear_beyond=True)
    c.particles = unpack(d, "in_")
    c.grid.flags = np.array(d["flags"], dtype=np.uint8)
    return c, d


def _by_position(ps):
    return ps.take(np.lexsort((ps.z, ps.y, ps.x)))


def test_pressure_ghosts_after_adaptation_match_reference():
    """one step, scan_outside_layer, adapt_domain and add_pressure_ghost on
    the device: the new particles are the reference's (matched by position;
    positions, bc types and flags exact, the air state within 1e-14 of it:
    CUDA's pow against libm's), their keys the requested range; then two
    steps on the device and the oracle (which appends the same particles)
    agree at the FP64 tolerance"""
    from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS
    c, d = _pg_fixture()
    c.options.capacity = c.particles.n + 40000
    s = Solver(c)
    s.set_bucket_involvement(d["binv_in"])
    s.steps(int(d["nsteps"]))
    assert s.scan_outside_layer() == int(d["adapt"])
    s.adapt_domain()
    n0 = s.count()[0]
    base = 1 << 40
    added = s.add_pressure_ghost(base)
    ref = unpack(d, "born_")
    assert added == ref.n > 1000
    g = s.download()
    new = g.take(np.nonzero(g.key >= base)[0])
    assert new.n == added and g.n == n0 + added
    np.testing.assert_array_equal(np.sort(new.key), base + np.arange(added, dtype=np.uint64))
    a, b = _by_position(new), _by_position(ref)
    for f in ("x", "y", "z", "vx", "vy", "vz", "vsx", "vsy", "vsz", "h", "Y"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    for f in ("mass", "rho", "e", "p", "gamma", "c", "T", "cp"):
        np.testing.assert_allclose(getattr(a, f), getattr(b, f), rtol=1e-14, atol=0, err_msg=f)
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    # the layers in the following steps
    from oracle.ghosts import add_pressure_ghost
    o = OracleRun(c)
    o.steps(1)
    bi = np.array(d["binv_in"], dtype=np.uint8)
    o.scan_outside_layer(bi)
    o.adapt_domain(bi)
    extra, _ = add_pressure_ghost(c.grid, bi, o.ps, c.options)
    # the oracle's rows in the device's key order: by position
    pos = {(x, y, z): k for x, y, z, k in zip(new.x, new.y, new.z, new.key)}
    extra.key = np.array([pos[(x, y, z)] for x, y, z in zip(extra.x, extra.y, extra.z)], dtype=np.uint64)
    o.append(extra)
    s.steps(2)
    o.steps(2)
    gs, os_ = s.download().sorted_by_key(), o.ps.sorted_by_key()
    np.testing.assert_array_equal(gs.key, os_.key)
    np.testing.assert_array_equal(gs.bc_type, os_.bc_type)
    for f in DOUBLE_FIELDS:
        x, y = getattr(gs, f), getattr(os_, f)
        assert np.abs(x - y).max() <= 1e-10 * max(np.abs(y).max(), 1e-300), f


def test_pressure_ghosts_beyond_capacity_are_refused():
    """a table without room for the new layers: PLUME_E_CAPACITY, and the
    context keeps its particles"""
    from plume_gpu import PlumeError
    c, d = _pg_fixture()
    s = Solver(c)
    s.set_bucket_involvement(d["binv_in"])
    s.steps(int(d["nsteps"]))
    s.scan_outside_layer()
    s.adapt_domain()
    n0 = s.count()[0]
    with pytest.raises(PlumeError) as e:
        s.add_pressure_ghost(1 << 40)
    assert e.value.status == 5
    assert s.count()[0] == n0


def test_pressure_ghosts_need_a_3d_single_run():
    from plume_gpu import PlumeError
    case = cases.sod_1d(n_real=200)
    s = Solver(case)
    with pytest.raises(PlumeError):
        s.add_pressure_ghost(1 << 40)


def test_wall_ghosts_match_reference():
    """one step, then add_wall_ghost on the device (cases.wall_scenario):
    the new wall ghosts are the reference's (tests/golden/wall_ghost_3d.npz,
    matched by position; air state within 1e-14); two further steps agree
    with the oracle, which appends the same particles"""
    from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS
    from oracle.ghosts import add_wall_ghost
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "wall_ghost_3d.npz")))
    c, _ = cases.wall_scenario(adapt_case())
    c.particles = unpack(d, "in_")
    c.options.capacity = c.particles.n + 10000
    s = Solver(c)
    s.steps(int(d["nsteps"]))
    base = 1 << 41
    added = s.add_wall_ghost(base)
    ref = unpack(d, "born_")
    assert added == ref.n > 1000
    g = s.download()
    new = g.take(np.nonzero(g.key >= base)[0])
    a, b = _by_position(new), _by_position(ref)
    for f in ("x", "y", "z", "vx", "vy", "vz", "h", "Y"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    for f in ("mass", "rho", "e", "p", "gamma", "c", "T", "cp"):
        np.testing.assert_allclose(getattr(a, f), getattr(b, f), rtol=1e-14, atol=0, err_msg=f)
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    assert s.add_wall_ghost(base + added) == 0  # the buckets hold wall ghosts now
    o = OracleRun(c)
    o.steps(1)
    extra, _ = add_wall_ghost(c.grid, o.ps, c.options)
    pos = {(x, y, z): k for x, y, z, k in zip(new.x, new.y, new.z, new.key)}
    extra.key = np.array([pos[(x, y, z)] for x, y, z in zip(extra.x, extra.y, extra.z)], dtype=np.uint64)
    o.append(extra)
    s.steps(2)
    o.steps(2)
    gs, os_ = s.download().sorted_by_key(), o.ps.sorted_by_key()
    np.testing.assert_array_equal(gs.key, os_.key)
    for f in DOUBLE_FIELDS:
        x, y = getattr(gs, f), getattr(os_, f)
        assert np.abs(x - y).max() <= 1e-10 * max(np.abs(y).max(), 1e-300), f


def test_device_image_search_equals_host_table():
    """plume_search_bnd_images on the wall-boundary plume finds the table of
    cases.wall_images (the fixture's images): same count, and a run with
    either table computes the same bits through apply_bcond and two steps"""
    from _util import golden_case
    from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS
    case, d = golden_case("plume_3d_bc")
    a = Solver(case)
    a.set_wall_images(d["img_key"], d["img_xyz"])
    b = Solver(case)
    assert b.search_bnd_images() == len(d["img_key"]) > 1000
    for s in (a, b):
        s.apply_bcond()
        s.steps(2)
    ga, gb = a.download().sorted_by_key(), b.download().sorted_by_key()
    for f in DOUBLE_FIELDS + BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(ga, f), getattr(gb, f), err_msg=f)


def test_device_image_search_after_wall_ghosts():
    """after add_wall_ghost the device search finds the images of the new
    wall ghosts too: the count of cases.wall_images on the new table"""
    import dataclasses
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "wall_ghost_3d.npz")))
    c, _ = cases.wall_scenario(adapt_case())
    c.particles = unpack(d, "in_")
    c.options.capacity = c.particles.n + 10000
    s = Solver(c)
    s.steps(1)
    before = s.search_bnd_images()
    s.add_wall_ghost(1 << 41)
    after = s.search_bnd_images()
    keys, _ = cases.wall_images(dataclasses.replace(c, particles=s.download()))
    assert after == len(keys) > before


def test_adapt_step_equals_the_calls_in_order():
    """plume_adapt_step on the pressure-ghost set-up with wall images in
    use equals scan, adapt_domain, both ghost layers, the image search and
    apply_bcond called one by one, bit for bit, through two more steps"""
    from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS
    c, d = _pg_fixture()
    c.options.capacity = c.particles.n + 60000
    keys, xyz = cases.wall_images(c)
    runs = []
    for one_call in (True, False):
        s = Solver(c)
        s.set_wall_images(keys, xyz)
        s.set_bucket_involvement(d["binv_in"])
        s.steps(1)
        if one_call:
            adapted, added = s.adapt_step(1 << 40)
        else:
            adapted = s.scan_outside_layer()
            s.adapt_domain()
            added = s.add_pressure_ghost(1 << 40)
            added += s.add_wall_ghost((1 << 40) + added)
            s.search_bnd_images()
            s.apply_bcond()
        assert adapted == int(d["adapt"]) and added >= int(d["born_x"].size)
        s.steps(2)
        runs.append((s, s.download().sorted_by_key()))
    (s, a), (_, b) = runs
    for f in DOUBLE_FIELDS + BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    np.testing.assert_array_equal(a.key, b.key)


def test_add_air_matches_reference():
    """one step, then add_air on the device (cases.air_scenario): the new
    air particles are the reference's (tests/golden/add_air_3d.npz, matched
    by position; air state within 1e-14); a second call adds nothing; two
    further steps agree with the oracle, which appends the same particles"""
    from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS
    from oracle.ghosts import add_air
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "add_air_3d.npz")))
    c, binv = cases.air_scenario(adapt_case())
    c.particles = unpack(d, "in_")
    c.options.capacity = c.particles.n + 10000
    s = Solver(c)
    s.set_bucket_involvement(binv)
    s.steps(int(d["nsteps"]))
    base = 1 << 42
    added = s.add_air(base)
    ref = unpack(d, "born_")
    assert added == ref.n > 1000
    g = s.download()
    new = g.take(np.nonzero(g.key >= base)[0])
    a, b = _by_position(new), _by_position(ref)
    for f in ("x", "y", "z", "vx", "vy", "vz", "h", "Y"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    for f in ("mass", "rho", "e", "p", "gamma", "c", "T", "cp"):
        np.testing.assert_allclose(getattr(a, f), getattr(b, f), rtol=1e-14, atol=0, err_msg=f)
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    assert s.add_air(base + added) == 0
    o = OracleRun(c)
    o.steps(1)
    extra, _ = add_air(c.grid, binv, o.ps, c.options)
    pos = {(x, y, z): k for x, y, z, k in zip(new.x, new.y, new.z, new.key)}
    extra.key = np.array([pos[(x, y, z)] for x, y, z in zip(extra.x, extra.y, extra.z)], dtype=np.uint64)
    o.append(extra)
    s.steps(2)
    o.steps(2)
    gs, os_ = s.download().sorted_by_key(), o.ps.sorted_by_key()
    np.testing.assert_array_equal(gs.key, os_.key)
    np.testing.assert_array_equal(gs.bc_type, os_.bc_type)
    for f in DOUBLE_FIELDS:
        x, y = getattr(gs, f), getattr(os_, f)
        assert np.abs(x - y).max() <= 1e-10 * max(np.abs(y).max(), 1e-300), f


def test_setup_erupt_matches_reference():
    """one step, then setup_erupt on the device (cases.duct_scenario): the
    new erupt ghosts are the reference's (tests/golden/setup_erupt_3d.npz,
    matched by position), the same particles are removed,
    and two further steps agree with the oracle doing the same"""
    from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS
    from oracle.ghosts import setup_erupt
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "setup_erupt_3d.npz")))
    c, binv, duct = cases.duct_scenario(adapt_case())
    c.particles = unpack(d, "in_")
    b = unpack(d, "born_")
    duct.update(rho=float(b.rho[0]), e=float(b.e[0]), p=float(b.p[0]), gamma=float(b.gamma[0]), c=float(b.c[0]))
    c.options.capacity = c.particles.n + 5000
    s = Solver(c)
    s.steps(int(d["nsteps"]))
    base = 1 << 43
    added, removed, mass, sml = s.setup_erupt(duct, base)
    assert added == b.n > 500 and removed > 0
    g = s.download()
    np.testing.assert_array_equal(np.sort(g.key[g.key < base]), d["kept_key"])
    new = g.take(np.nonzero(g.key >= base)[0])
    # the spacing is cbrt(volume / np) of the host's libm: equal to the
    # fixture's (x86) to the last place or one unit off, so positions,
    # which accumulate it, compare to 1e-13
    x, y = _by_position(new), _by_position(b)
    for f in DOUBLE_FIELDS:
        np.testing.assert_allclose(getattr(x, f), getattr(y, f), rtol=1e-13, atol=1e-12, err_msg=f)
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(x, f), getattr(y, f), err_msg=f)
    assert abs(mass / float(b.mass[0]) - 1) < 1e-15 and abs(sml / float(b.h[0]) - 1) < 1e-15
    o = OracleRun(c)
    o.steps(1)
    extra, gone = setup_erupt(o.ps, duct, c.options)
    o.ps = o.ps.take(np.nonzero(~gone)[0])
    pos = {(px, py, pz): k for px, py, pz, k in zip(new.x, new.y, new.z, new.key)}
    extra.key = np.array([pos[(px, py, pz)] for px, py, pz in zip(extra.x, extra.y, extra.z)], dtype=np.uint64)
    o.append(extra)
    s.steps(2)
    o.steps(2)
    gs, os_ = s.download().sorted_by_key(), o.ps.sorted_by_key()
    np.testing.assert_array_equal(gs.key, os_.key)
    for f in DOUBLE_FIELDS:
        u, v = getattr(gs, f), getattr(os_, f)
        assert np.abs(u - v).max() <= 1e-10 * max(np.abs(v).max(), 1e-300), f
