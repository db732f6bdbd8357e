"""Ensembles: members stepped together in one context (plume_batch_*).

A member of an ensemble must compute exactly what it computes alone, so the
FP64 and mixed ensembles are compared with single-member runs of the same
members bit for bit (same positions, same cell order inside the member, same
per-member dt), and one FP64 member with the oracle (1e-10, as in the
single-run parity tests).  CUDA-graph replays must give the same bits as
steps issued one by one.  The mixed ensemble's density error against the
FP64 ensemble is reported per member.
"""
import copy
import dataclasses

import numpy as np
import pytest

from oracle.binding import OracleRun
from plume_gpu import PREC_MIXED, Ensemble, PlumeError, Solver, cases
from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS
from _util import field_errors

pytestmark = pytest.mark.gpu

PLUME_E_NONPOSITIVE = 4


def _riemann(n_members, seed=5, n_lo=150, n_hi=600, t_end=0.2, precision=0):
    return cases.riemann_ensemble(n_members, seed=seed, n_lo=n_lo, n_hi=n_hi, t_end=t_end,
                                  precision=precision)


def _solo(case, nsteps):
    s = Solver(case)
    if case.pre_adaptive:
        s.adaptive_sml()
    s.steps(nsteps)
    return s


def _assert_identical(a, b, label):
    a, b = a.sorted_by_key(), b.sorted_by_key()
    assert a.n == b.n, (label, a.n, b.n)
    for f in DOUBLE_FIELDS + BYTE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f"{label}: {f}")


@pytest.mark.parametrize("precision", [0, PREC_MIXED])
def test_1d_ensemble_members_equal_single_runs(precision):
    # some seed-5 members drive a sound speed to <= 0 within 40 steps (member
    # 2 at its 29th step, in the oracle and in the reference's own build,
    # assertion timestep.cc:167): they stop with that status, the others
    # must equal their single runs bit for bit
    cs = _riemann(6, precision=precision)
    ens = Ensemble(cs)
    ens.adaptive_sml()
    ens.steps(40)
    parts = ens.split()
    t, st, run, status = ens.member_times()
    assert status[2] == PLUME_E_NONPOSITIVE and not run[2]
    n_ok = 0
    for k, c in enumerate(cs):
        s = Solver(c)
        s.adaptive_sml()
        try:
            s.steps(40)
        except PlumeError as e:
            assert status[k] == e.status and not run[k], k
            continue
        assert status[k] == 0 and run[k], k
        _assert_identical(parts[k], s.download(), f"member {k}")
        ts, ss, _ = s.time()
        assert t[k] == ts and st[k] == ss
        n_ok += 1
    assert n_ok >= 3


def test_failed_member_stops_where_the_oracle_fails():
    cs = _riemann(6)
    o = OracleRun(cs[2])
    o.adaptive()
    failed_at = None
    for k in range(40):
        try:
            o.steps(1)
        except Exception:
            failed_at = k + 1
            break
    assert failed_at is not None
    ens = Ensemble(cs)
    ens.adaptive_sml()
    ens.steps(40)
    t, st, run, status = ens.member_times()
    # the failing step completes; the member is stopped from the next one
    assert status[2] == PLUME_E_NONPOSITIVE and st[2] == failed_at


def test_1d_ensemble_member_matches_oracle():
    cs = _riemann(3, seed=9)
    ens = Ensemble(cs)
    ens.adaptive_sml()
    ens.steps(20)
    parts = ens.split()
    o = OracleRun(cs[2])
    o.adaptive()
    o.steps(20)
    err = field_errors(parts[2], o.ps)
    assert max(err.values()) <= 1e-10, err


def test_graph_replay_equals_single_steps_and_members_stop_at_their_end():
    # short end times: members end after different step counts
    cs = _riemann(5, seed=3, t_end=0.004)
    for c, te in zip(cs, [0.002, 0.004, 0.003, 0.0025, 0.004]):
        c.options.max_time = float(np.float32(te))
    a = Ensemble(cs)
    a.adaptive_sml()
    na = a.run(100000, graph_steps=16)
    b = Ensemble(cs)
    b.adaptive_sml()
    nb = b.run(100000, graph_steps=0)
    ta, sa, ra, fa = a.member_times()
    tb, sb, rb, fb = b.member_times()
    assert not ra.any() and not rb.any() and not fa.any() and not fb.any()
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(ta, tb)
    assert nb == int(sb.max()) and na >= nb
    pa, pb = a.split(), b.split()
    for k, c in enumerate(cs):
        _assert_identical(pa[k], pb[k], f"member {k} graph vs steps")
        assert ta[k] == c.options.max_time
        # a single run stepped while TimeProps::ifend is false
        solo = Solver(c)
        solo.adaptive_sml()
        while solo.time()[0] < c.options.max_time:
            solo.step()
        _assert_identical(pa[k], solo.download(), f"member {k} vs single run")


@pytest.mark.parametrize("precision", [0, PREC_MIXED])
def test_3d_ensemble_members_equal_single_runs(precision):
    cs = cases.plume_ensemble(3, seed=4, dx=50.0, n_lo=2000, n_hi=6000, duct_depth=300.0,
                              precision=precision)
    for c in cs:
        c.step0 = 49  # the first step runs adaptive_sml (every 50 steps)
    ens = Ensemble(cs)
    ens.set_time(0.0, 49, 0, cs[0].options.timeoutput)
    ens.steps(3)
    parts = ens.split()
    for k, c in enumerate(cs):
        solo = Solver(c)
        solo.steps(3)
        _assert_identical(parts[k], solo.download(), f"3D member {k}")


def _l1(a, b, sel):
    return np.abs(b.rho[sel] - a.rho[sel]).sum() / np.abs(a.rho[sel]).sum()


def test_mixed_one_step_density_error_vs_fp64():
    # the mixed arithmetic itself: one mixed and one FP64 step (adaptive h,
    # momentum, density, position) from the same FP64 state of each member
    errs = []
    for c in _riemann(8, seed=11):
        s = Solver(c)
        s.adaptive_sml()
        try:
            s.steps(20)
        except PlumeError:
            continue
        ps = s.download()
        t, st, io = s.time()
        out = {}
        for prec in (0, PREC_MIXED):
            opt = copy.deepcopy(c.options)
            opt.precision = prec
            s2 = Solver(dataclasses.replace(c, options=opt, particles=ps, step0=0))
            s2.set_time(t, st, io, c.options.timeoutput)
            s2.steps(1)
            out[prec] = s2.download().sorted_by_key()
        r = out[0].need_neigh()
        errs.append(_l1(out[0], out[PREC_MIXED], r))
    print("one-step mixed vs FP64 relative L1 density error per member:",
          ["%.2e" % e for e in errs])
    assert len(errs) >= 4
    assert max(errs) <= 1e-6, errs


def test_mixed_ensemble_density_error_vs_fp64():
    # after 50 steps; the particles next to the tube-end ghosts amplify
    # per-step differences by orders of magnitude on some members, so the
    # error is reported per member with the members' sensitivity to a one-ulp
    # change of the FP64 positions
    n = 8
    f64 = Ensemble(_riemann(n, seed=11))
    mix = Ensemble(_riemann(n, seed=11, precision=PREC_MIXED))
    cs = _riemann(n, seed=11)
    for c in cs:
        c.particles.x[:] = np.nextafter(c.particles.x, np.inf)
    ulp = Ensemble(cs)
    for e in (f64, mix, ulp):
        e.adaptive_sml()
        e.steps(50)
    fa, fb = f64.member_times()[3], mix.member_times()[3]
    np.testing.assert_array_equal(fa, fb)  # the same members fail
    rows = []
    for k, (a, b, u) in enumerate(zip(f64.split(), mix.split(), ulp.split())):
        if fa[k]:
            continue
        r = a.need_neigh()
        rows.append((k, _l1(a, b, r), _l1(a, u, r)))
    print("member, mixed vs FP64 L1 density error, one-ulp FP64 sensitivity (50 steps):",
          ["%d %.2e %.2e" % row for row in rows])
    errs = np.array([row[1] for row in rows])
    assert len(errs) >= n // 2
    assert np.median(errs) <= 1e-3 and errs.max() <= 1e-2, errs
