"""The CPU oracle against golden vectors of the reference's own sources.

tests/golden/*.npz were produced by tests/golden/make_golden.py, which runs
the reference solver's hot-path functions (compiled from the Plume-SPH tree
by oracle/Makefile).  1D runs must agree to the last bit; the 3D run agrees
to the last bit on its first step and to rounding afterwards (the
reference re-orders bucket lists when particles move, update_pos.cc:171-463,
which changes the summation order).
"""
import os

import numpy as np
import pytest

from oracle.binding import OracleRun
from plume_gpu import cases
from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS, RIEMANN_ROE
from _util import GOLDEN, field_errors, golden_case, set_summary, unpack


@pytest.mark.parametrize("name", ["sod_1d_200", "shock_tube_1d"])
def test_oracle_1d_bit_exact(name):
    case, d = golden_case(name)
    o = OracleRun(case)
    if case.pre_adaptive:
        o.adaptive()
    dts = o.steps(int(d["nsteps"]))
    np.testing.assert_array_equal(dts, d["dt"])
    assert o.t.step == int(d["step"][-1])
    assert o.t.time == float(d["time"][-1])
    ref = unpack(d, "out_")
    err = field_errors(o.ps, ref)
    assert max(err.values()) == 0.0, err
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(o.ps.sorted_by_key(), f), getattr(ref, f))


def test_oracle_sod_2000_full_run_bit_exact():
    """The 1D Sod workload (2,000 particles, Gaussian kernel) to t = 0.2:
    2,549 steps, final state identical to the reference's."""
    case, d = golden_case("sod_1d_2000_end")
    o = OracleRun(case, nthreads=0)
    o.adaptive()
    o.steps(int(d["nsteps"]))
    assert o.t.step == int(d["step"][-1])
    assert o.t.time == float(d["time"][-1])
    err = field_errors(o.ps, unpack(d, "out_"))
    assert max(err.values()) == 0.0, err


def test_oracle_1d_lists_are_all_particles():
    case, d = golden_case("sod_1d_200")
    o = OracleRun(case)
    ki, kj = o.pairs(mode=0)
    keys, cnt, h = set_summary(ki, kj)
    np.testing.assert_array_equal(keys, d["list_key"])
    np.testing.assert_array_equal(cnt, d["list_count"])
    np.testing.assert_array_equal(h, d["list_hash"])


def test_oracle_3d_plume_steps():
    case, d = golden_case("plume_3d_small")
    o = OracleRun(case)
    dts = o.steps(int(d["nsteps"]))
    np.testing.assert_allclose(dts, d["dt"], rtol=1e-12, atol=0)
    assert o.t.step == int(d["step"][-1])
    ref = unpack(d, "out_")
    err = field_errors(o.ps, ref)
    assert max(err.values()) < 1e-12, err
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(o.ps.sorted_by_key(), f), getattr(ref, f))


def test_oracle_3d_first_step_bit_exact():
    case, d = golden_case("plume_3d_small")
    o = OracleRun(case)
    o.steps(1)
    assert o.t.step == int(d["step"][0])
    np.testing.assert_array_equal(o.t.time, d["time"][0])


def test_oracle_3d_neighbour_sets_match_reference():
    case, d = golden_case("plume_3d_small")
    case.particles = unpack(d, "pre_")
    o = OracleRun(case)
    ki, kj = o.pairs(mode=0)
    keys, cnt, h = set_summary(ki, kj)
    # the reference dumps lists after the step: erupt ghosts that turned real
    # during it hold no list yet, so compare the particles that were
    # need_neigh when the lists were built
    pre = case.particles
    live = np.isin(d["list_key"], pre.key[pre.need_neigh()])
    np.testing.assert_array_equal(keys, d["list_key"][live])
    np.testing.assert_array_equal(cnt, d["list_count"][live])
    np.testing.assert_array_equal(h, d["list_hash"][live])
    # full lists of sampled particles (as sets: the reference re-orders
    # bucket lists when particles move, update_pos.cc:438-445)
    offs = d["sample_offs"]
    for r, k in enumerate(d["sample_key"]):
        if not live[np.searchsorted(d["list_key"], k)]:
            continue
        want = np.sort(d["sample_flat"][offs[r]:offs[r + 1]])
        got = np.sort(kj[ki == k])
        np.testing.assert_array_equal(got, want)


def test_oracle_wall_boundary_matches_reference():
    # apply_bcond of the reference (bcond.cc) before the loop and after each
    # of steps 49..51, flat-ground images
    case, d = golden_case("plume_3d_bc")
    o = OracleRun(case)
    o.set_images(d["img_key"], d["img_xyz"])
    o.apply_bcond()
    dts = o.steps(int(d["nsteps"]))
    np.testing.assert_allclose(dts, d["dt"], rtol=1e-12, atol=0)
    ref = unpack(d, "out_")
    err = field_errors(o.ps, ref)
    assert max(err.values()) < 1e-12, err
    walls = ref.sorted_by_key().bc_type == 2
    moved = ref.sorted_by_key().rho[walls] != case.particles.sorted_by_key().rho[walls]
    assert moved.sum() > 1000  # the boundary did set ghost states


def test_wall_image_table_restates_search_bnd_images():
    case, d = golden_case("plume_3d_bc")
    k, x = cases.wall_images(case)
    np.testing.assert_array_equal(k, d["img_key"])
    np.testing.assert_array_equal(x, d["img_xyz"])
    ps = case.particles
    row = {int(kk): i for i, kk in enumerate(ps.key)}
    g = np.array([[ps.x[row[int(kk)]], ps.y[row[int(kk)]], ps.z[row[int(kk)]]] for kk in k])
    np.testing.assert_array_equal(x[:, :2], g[:, :2])
    np.testing.assert_allclose(x[:, 2], -g[:, 2], rtol=0, atol=0)  # mirrored in z = 0


# ---------------------------------------------------------------- GSPH
def _grad_by_key(keys, grad, want):
    m = {int(k): r for r, k in enumerate(keys)}
    return grad[np.array([m[int(k)] for k in want])]


@pytest.mark.parametrize("name", ["gsph_1d_sod", "gsph_1d_grad"])
def test_oracle_gsph_1d_bit_exact(name):
    """GSPH (HLLC) steps and the last step's calc_gradients, bit for bit:
    zeroth-order states (the 1D default), and linear states (MINI_DERIVATIVE
    _COND 1) on a ghost-free tube that runs the reference's own
    calc_gradients."""
    case, d = golden_case(name)
    o = OracleRun(case)
    o.adaptive()
    dts = o.steps_grad(int(d["nsteps"]))
    np.testing.assert_array_equal(dts, d["dt"])
    err = field_errors(o.ps, unpack(d, "out_"))
    assert max(err.values()) == 0.0, err
    gk, g = o.grad
    np.testing.assert_array_equal(_grad_by_key(gk, g, d["grad_key"]), d["grad"])
    assert np.count_nonzero(np.abs(d["grad"]).sum(axis=1)) > 100


def test_oracle_gsph_differs_from_sph():
    """the method switch reaches the step: GSPH and SPH part after one step"""
    case, _ = golden_case("gsph_1d_sod")
    a = OracleRun(case)
    a.adaptive()
    a.steps(1)
    case.options.method = cases.METHOD_SPH
    b = OracleRun(case)
    b.adaptive()
    b.steps(1)
    assert max(field_errors(a.ps, b.ps, fields=("vx", "e")).values()) > 1e-6


def test_oracle_gsph_3d_matches_reference():
    """3D GSPH with the reference's 3D switches (Roe solver, cubic interface
    position, MINI_DERIVATIVE_COND 10, modified monotonicity, LANS), steps
    49..50: gradients of the last step bit for bit, fields to rounding."""
    case, d = golden_case("gsph_3d")
    assert case.options.gsph_solver == RIEMANN_ROE and case.options.gsph_recon == 10
    o = OracleRun(case)
    dts = o.steps_grad(int(d["nsteps"]))
    np.testing.assert_allclose(dts, d["dt"], rtol=1e-12, atol=0)
    ref = unpack(d, "out_")
    err = field_errors(o.ps, ref)
    assert max(err.values()) < 1e-12, err
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(o.ps.sorted_by_key(), f), getattr(ref, f))
    gk, g = o.grad
    gref = d["grad"]
    gerr = np.abs(_grad_by_key(gk, g, d["grad_key"]) - gref).max(axis=0) / (np.abs(gref).max(axis=0) + 1e-300)
    assert gerr.max() < 1e-12, gerr


# ---------------------------------------------------------------- domain growth
def _adapt_fixture():
    from _util import adapt_case
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "adapt_3d.npz")))
    c, binv = cases.adapt_scenario(adapt_case())
    c.particles = unpack(d, "in_")
    c.grid.flags = np.array(d["flags"], dtype=np.uint8)
    np.testing.assert_array_equal(binv, d["binv_in"])
    return c, d


def test_oracle_domain_growth_matches_reference():
    """one step, then scan_outside_layer and adapt_domain: the scan's count,
    every bucket's involvement state and every particle's bc type and
    involvement identical to the reference's"""
    c, d = _adapt_fixture()
    o = OracleRun(c)
    o.steps(int(d["nsteps"]))
    binv = np.array(d["binv_in"], dtype=np.uint8)
    a = o.scan_outside_layer(binv)
    assert a == int(d["adapt"]) and a > 0
    o.adapt_domain(binv)
    np.testing.assert_array_equal(binv, d["binv_out"])
    ps = o.ps.sorted_by_key()
    np.testing.assert_array_equal(ps.key, d["out_key"])
    np.testing.assert_array_equal(ps.bc_type, d["out_bc_type"])
    np.testing.assert_array_equal(ps.involved, d["out_involved"])
    np.testing.assert_allclose(ps.x, d["out_x"], rtol=0, atol=1e-9)
    assert (d["binv_out"] == 1).sum() > (d["binv_in"] == 1).sum()  # buckets were converted
    # the converted buckets stopped absorbing
    conv = (d["binv_in"] == 0) & (d["binv_out"] == 1)
    assert not np.any(c.grid.flags[conv] & cases.BUCKET_ABSORBING)


def test_oracle_gsph_sod_2000_full_run_bit_exact():
    """The 1D Sod workload (2,000 particles) with GSPH (HLLC) to t = 0.2:
    2,173 steps, final state identical to the reference's GSPH build"""
    case, d = golden_case("gsph_1d_2000_end")
    case.options.gsph_gradients = 0  # zeroth-order states read no gradients
    o = OracleRun(case)
    o.adaptive()
    o.steps(int(d["nsteps"]))
    assert o.t.step == int(d["step"][-1])
    assert o.t.time == float(d["time"][-1])
    err = field_errors(o.ps, unpack(d, "out_"))
    assert max(err.values()) == 0.0, err


def test_csv_writer_matches_reference_write_csv(tmp_path):
    """the 1D text output (plume_gpu.output.write_csv) of the reference's
    final Sod state is byte-for-byte the text the reference's write_csv
    wrote for it (tests/golden/sod_1d_csv.npz); a second call appends a
    second header and the rows again"""
    from plume_gpu.output import CSV_HEADER, write_csv
    d = np.load(os.path.join(GOLDEN, "sod_1d_csv.npz"))
    ps = unpack(d, "out_")  # sorted by key: the reference's row order
    path = tmp_path / "pvplot_out.csv"
    n = write_csv(str(path), ps, order=np.arange(ps.n))
    text = path.read_text()
    assert text == str(d["csv"])
    assert n == int(np.sum(ps.bc_type == 100)) > 0
    write_csv(str(path), ps, order=np.arange(ps.n))
    assert path.read_text() == 2 * str(d["csv"])
    assert text.startswith(CSV_HEADER)


@pytest.mark.parametrize("name", ["plume_20km", "plume_600m", "ragged"])
def test_bucket_grid_matches_reference_preprocessor(name):
    """cases.plume_grid against the buckets of the reference's preprocess.cc
    (tests/golden/grid_3d.npz): hash-table bounds, bucket count and corners,
    bucket_index per face, and bucket types (UNDERGROUND / PRESS_BC are the
    absorbing buckets, MIXED the mixed ones, OVERGROUND neither)"""
    from plume_gpu.abi import BUCKET_ABSORBING, BUCKET_MIXED
    d = np.load(os.path.join(GOLDEN, "grid_3d.npz"))
    dom = d[f"{name}_domain"]
    g = cases.plume_grid(tuple(dom[:3]), tuple(dom[3:6]), float(dom[6]))
    ht, typ, idx, lo = d[f"{name}_ht"], d[f"{name}_type"], d[f"{name}_index"], d[f"{name}_lo"]
    nb = np.array(g.nb)
    assert typ.shape[0] == nb.prod()
    np.testing.assert_array_equal(ht[0::2], np.array(g.mindom))
    np.testing.assert_array_equal(ht[1::2], np.array(g.mindom) + nb * g.del_)
    ijk = np.rint((lo - np.array(g.mindom)) / g.del_).astype(np.int64)
    np.testing.assert_array_equal(lo, np.array(g.mindom) + ijk * g.del_)
    b = (ijk[:, 2] * nb[1] + ijk[:, 1]) * nb[0] + ijk[:, 0]
    assert len(np.unique(b)) == len(b)
    face = np.asarray(g.face_index).reshape(-1, 6)
    np.testing.assert_array_equal(face[b], idx)
    flags = np.asarray(g.flags)[b]
    want = np.select([np.isin(typ, (1, 4)), typ == 2], [BUCKET_ABSORBING, BUCKET_MIXED], 0)
    assert set(np.unique(typ)) <= {1, 2, 3, 4}
    np.testing.assert_array_equal(flags & (BUCKET_ABSORBING | BUCKET_MIXED), want)


def _adapt_pg_fixture():
    from _util import adapt_case
    d = dict(np.load(os.path.join(GOLDEN, "adapt_pg_3d.npz")))
    c, binv = cases.adapt_scenario(adapt_case(), clear_beyond=True)
    c.particles = unpack(d, "in_")
    c.grid.flags = np.array(d["flags"], dtype=np.uint8)
    np.testing.assert_array_equal(binv, d["binv_in"])
    return c, d


def _by_position(ps):
    return ps.take(np.lexsort((ps.z, ps.y, ps.x)))


def test_oracle_pressure_ghosts_after_adaptation_match_reference():
    """one step, scan_outside_layer, adapt_domain, then add_pressure_ghost:
    the oracle's new pressure ghosts (oracle/ghosts.py) are the reference's,
    field for field and bit for bit (matched by position: the reference's
    keys are Hilbert keys of the creation step)"""
    from oracle.ghosts import add_pressure_ghost
    c, d = _adapt_pg_fixture()
    o = OracleRun(c)
    o.steps(int(d["nsteps"]))
    binv = np.array(d["binv_in"], dtype=np.uint8)
    assert o.scan_outside_layer(binv) == int(d["adapt"]) > 0
    o.adapt_domain(binv)
    np.testing.assert_array_equal(binv, d["binv_out"])
    new, marked = add_pressure_ghost(c.grid, binv, o.ps, c.options)
    ref = unpack(d, "born_")
    assert new.n == ref.n > 1000
    a, b = _by_position(new), _by_position(ref)
    for f in DOUBLE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    assert np.all(d["active"] == 1) and len(marked) > 0


def test_oracle_wall_ghosts_match_reference():
    """one step, then add_wall_ghost on cases.wall_scenario: the oracle's
    new wall ghosts (oracle/ghosts.py) are the reference's, bit for bit"""
    from _util import adapt_case
    from oracle.ghosts import add_wall_ghost
    d = dict(np.load(os.path.join(GOLDEN, "wall_ghost_3d.npz")))
    c, binv = cases.wall_scenario(adapt_case())
    c.particles = unpack(d, "in_")
    np.testing.assert_array_equal(binv, d["binv_in"])
    o = OracleRun(c)
    o.steps(int(d["nsteps"]))
    new, marked = add_wall_ghost(c.grid, o.ps, c.options)
    ref = unpack(d, "born_")
    assert new.n == ref.n > 1000 and len(marked) > 0
    a, b = _by_position(new), _by_position(ref)
    for f in DOUBLE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


def test_oracle_add_air_matches_reference():
    """one step, then add_air on cases.air_scenario: the oracle's new air
    particles (oracle/ghosts.py) are the reference's, bit for bit"""
    from _util import adapt_case
    from oracle.ghosts import add_air
    d = dict(np.load(os.path.join(GOLDEN, "add_air_3d.npz")))
    c, binv = cases.air_scenario(adapt_case())
    c.particles = unpack(d, "in_")
    np.testing.assert_array_equal(binv, d["binv_in"])
    o = OracleRun(c)
    o.steps(int(d["nsteps"]))
    new, marked = add_air(c.grid, binv, o.ps, c.options)
    ref = unpack(d, "born_")
    assert new.n == ref.n > 1000 and len(marked) > 0
    a, b = _by_position(new), _by_position(ref)
    for f in DOUBLE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


def _duct_state(d):
    """the vent state the reference's erupt ghosts carry (rhov_P, ev0_P,
    pv0_P, gamma_v_P, sndspd of its build)"""
    b = unpack(d, "born_")
    return dict(rho=float(b.rho[0]), e=float(b.e[0]), p=float(b.p[0]), gamma=float(b.gamma[0]),
                c=float(b.c[0]))


def test_oracle_setup_erupt_matches_reference():
    """one step, then setup_erupt on cases.duct_scenario: the oracle's new
    erupt ghosts (oracle/ghosts.py) are the reference's bit for bit, and it
    removes the same particles"""
    from _util import adapt_case
    from oracle.ghosts import setup_erupt
    d = dict(np.load(os.path.join(GOLDEN, "setup_erupt_3d.npz")))
    c, binv, duct = cases.duct_scenario(adapt_case())
    c.particles = unpack(d, "in_")
    duct.update(_duct_state(d))
    o = OracleRun(c)
    o.steps(int(d["nsteps"]))
    new, gone = setup_erupt(o.ps, duct, c.options)
    ref = unpack(d, "born_")
    assert new.n == ref.n > 500 and gone.sum() > 0
    np.testing.assert_array_equal(np.sort(o.ps.key[~gone]), d["kept_key"])
    a, b = _by_position(new), _by_position(ref)
    for f in DOUBLE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


def test_oracle_inlet_matches_reference_add_new_erupt():
    """The reference's own add_new_erupt (setup_erupt.cc:389-673) against
    the oracle's restatement: the duct that setup_erupt built, then six
    steps with the inlet in each (main.cc:414-421).  Per-step dt and time
    within 1e-12 (later 3D steps sum in the reference's re-ordered bucket
    lists); the case's particles within 1e-10 (max-normalised) and the
    particles the run created (duct and inlet; matched by position, the
    reference keys them by Hilbert keys of the creation step) the same count
    with the same types and fields within 1e-10."""
    from _util import inlet_fixture, match_by_position
    c, inl, d = inlet_fixture()
    o = OracleRun(c)
    o.set_inlet(inl)
    dts = o.steps(int(d["nsteps"]))
    np.testing.assert_allclose(dts, d["dt"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(o.t.time, float(d["time"][-1]), rtol=1e-12, atol=0)
    base = int(inl["key_base"]) - len(unpack(d, "duct_").key)
    case_rows = o.ps.key < np.uint64(base)
    err = field_errors(o.ps.take(np.nonzero(case_rows)[0]), unpack(d, "out_"))
    assert max(err.values()) <= 1e-10, err
    ref = unpack(d, "born_")
    born = match_by_position(o.ps.take(np.nonzero(~case_rows)[0]), ref)
    injected = int((o.ps.key >= np.uint64(inl["key_base"])).sum())
    assert injected == ref.n - unpack(d, "duct_").n > 0
    for f in BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(born, f), getattr(ref, f), err_msg=f)
    for f in DOUBLE_FIELDS:
        x, y = getattr(born, f), getattr(ref, f)
        scale = max(float(np.abs(y).max()), 1e-300)
        assert float(np.abs(x - y).max()) <= 1e-10 * scale, f


def test_duct_inlet_columns_follow_the_reference_loops():
    """cases.duct_inlet: one column per duct lattice column of setup_erupt
    (the same loops), every column inside the vent radius"""
    from _util import inlet_fixture
    c, inl, d = inlet_fixture()
    duct = unpack(d, "duct_")
    cols = {(float(x), float(y)) for x, y in zip(duct.x, duct.y)}
    got = {(float(x), float(y)) for x, y in inl["col_xy"]}
    assert got == cols
    assert np.all((inl["col_xy"] ** 2).sum(1) <= 120.0 ** 2)


def _finite_and_nan_match(a, b, tol, fields=DOUBLE_FIELDS):
    """fields of a against b after matching by key: the same NaN entries, the
    finite ones within tol of max |b|; returns the NaN count of b"""
    a, b = a.sorted_by_key(), b.sorted_by_key()
    assert np.array_equal(a.key, b.key)
    nans = 0
    for f in fields:
        x, y = getattr(a, f), getattr(b, f)
        np.testing.assert_array_equal(np.isnan(x), np.isnan(y), err_msg=f)
        fin = ~np.isnan(y)
        nans += int((~fin).sum())
        if fin.any():
            scale = max(float(np.abs(y[fin]).max()), 1e-300)
            assert float(np.abs(x[fin] - y[fin]).max()) <= tol * scale, f
    return nans


@pytest.mark.parametrize("name", ["gsph_1d_my2", "gsph_1d_my3", "gsph_1d_vl", "gsph_3d_my3", "gsph_3d_vl",
                                  "gsph_1d_rcm", "gsph_3d_rcm"])
def test_oracle_gsph_other_solvers_match_reference(name):
    """HLLC_RP_Solver_my (HLL_WAVE_SPEED_EVA 2, 3) and VanLeer_RP_Solver
    against the reference's own builds over the steps it completes: the
    same dt, the same fields (1D bit for bit, 3D to rounding) and the same
    NaN entries.  The reference's HLLC_RP_Solver_my takes u* = sqrt(2 (E*_l -
    e*_l)), NaN where that is negative, so its first step already leaves
    NaN energies (the next step stops on assert(c > 0)); Van Leer's solver
    leaves NaN positions at the Sod tube's step 8 and the plume's fourth
    step."""
    from _util import GSPH_SOLVER_CASES
    case, d = golden_case(name)
    assert case.options.gsph_solver == GSPH_SOLVER_CASES[name][1]
    o = OracleRun(case)
    if case.pre_adaptive:
        o.adaptive()
    dts = o.steps_grad(int(d["nsteps"]))
    np.testing.assert_allclose(dts, d["dt"], rtol=1e-12, atol=0)
    tol = 0.0 if case.options.dim == 1 else 1e-12
    nans = _finite_and_nan_match(o.ps, unpack(d, "out_"), tol)
    assert (nans > 0) == name.startswith(("gsph_1d_my", "gsph_3d_my"))
    if name == "gsph_1d_vl":
        o.steps(1)  # step 8: the reference's positions turn NaN there
        assert np.isnan(o.ps.x).any()
