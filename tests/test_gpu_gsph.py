"""Godunov SPH (USE_GSPH 1) on the GPU against the oracle and the reference's
own GSPH builds (tests/golden/gsph_*.npz).

FP64 runs compare at the FP64 tolerance of the SPH tests (relative error
<= 1e-10 per field: the device sums in cell order, the reference in list
order); the gradients of the last step (calc_gradients) compare at the same
tolerance.  The mixed path (FP32 pair arithmetic, FP32 Riemann problems)
compares with the FP64 GSPH run at the relative L1 density bar of the SPH
mixed path, 1e-4.
"""
import numpy as np
import pytest

from oracle.binding import OracleRun
from plume_gpu import Solver, cases
from plume_gpu.abi import PREC_MIXED
from _util import field_errors, golden_case, unpack

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def _grad_err(keys, grad, ref_keys, ref_grad):
    m = {int(k): r for r, k in enumerate(keys)}
    g = grad[np.array([m[int(k)] for k in ref_keys])]
    scale = np.abs(ref_grad).max(axis=0) + 1e-300
    return float((np.abs(g - ref_grad).max(axis=0) / scale).max())


@pytest.mark.parametrize("name", ["gsph_1d_sod", "gsph_1d_grad", "gsph_3d"])
def test_gsph_fp64_matches_reference(name):
    case, d = golden_case(name)
    s = Solver(case)
    if case.pre_adaptive:
        s.adaptive_sml()
    log = s.steps(int(d["nsteps"]), log=True)
    np.testing.assert_allclose([r["dt"] for r in log], d["dt"], rtol=1e-12, atol=0)
    err = field_errors(s.download(), unpack(d, "out_"))
    assert max(err.values()) <= FP64_TOL, err
    keys, grad = s.gsph_gradients()
    assert _grad_err(keys, grad, d["grad_key"], d["grad"]) <= FP64_TOL


def test_gsph_1d_longer_run_matches_oracle():
    """200 steps of the GSPH Sod tube against the oracle"""
    case, _ = golden_case("gsph_1d_sod")
    s = Solver(case)
    s.adaptive_sml()
    s.steps(200)
    o = OracleRun(case)
    o.adaptive()
    o.steps(200)
    err = field_errors(s.download(), o.ps)
    assert max(err.values()) <= 1e-8, err


def test_gsph_unlimited_reconstruction_fails_like_the_oracle():
    """MINI_DERIVATIVE_COND 0 (linear states, no fallback) drives states
    negative on this plume; both stop with the same status"""
    case, _ = golden_case("gsph_3d")
    case.options.gsph_recon = 0
    s = Solver(case)
    with pytest.raises(RuntimeError) as e:
        s.steps(2)
    assert e.value.status == 6  # PLUME_E_OUTSIDE_GRID
    o = OracleRun(case)
    with pytest.raises(RuntimeError, match="failed: 6"):
        o.steps(2)


@pytest.mark.parametrize("recon", [1, 2, 3, 10])
def test_gsph_reconstructions_match_oracle(recon):
    """every MINI_DERIVATIVE_COND on the 3D fixture's state, the other 3D
    switches as the reference's defaults"""
    case, _ = golden_case("gsph_3d")
    case.options.gsph_recon = recon
    s = Solver(case)
    s.steps(2)
    o = OracleRun(case)
    o.steps(2)
    err = field_errors(s.download(), o.ps)
    assert max(err.values()) <= FP64_TOL, err


def test_gsph_hllc_and_linear_interface_3d():
    case, _ = golden_case("gsph_3d")
    case.options.gsph_solver = cases.RIEMANN_HLLC
    case.options.gsph_vol = 1
    case.options.gsph_mono = 0
    s = Solver(case)
    s.steps(2)
    o = OracleRun(case)
    o.steps(2)
    err = field_errors(s.download(), o.ps)
    assert max(err.values()) <= FP64_TOL, err


@pytest.mark.parametrize("name", ["gsph_1d_sod", "gsph_3d"])
def test_gsph_mixed_density_error(name):
    case, _ = golden_case(name)
    out = {}
    for prec in (0, PREC_MIXED):
        c = case.__class__(**{**case.__dict__, "particles": case.particles.copy()})
        c.options = case.options.__class__(**{**case.options.__dict__, "precision": prec})
        s = Solver(c)
        if c.pre_adaptive:
            s.adaptive_sml()
        s.steps(10 if c.options.dim == 1 else 2)
        out[prec] = s.download().sorted_by_key()
    a, b = out[0], out[PREC_MIXED]
    sel = a.need_neigh()
    err = np.abs(b.rho[sel] - a.rho[sel]).sum() / np.abs(a.rho[sel]).sum()
    assert err <= 1e-4, err
    assert np.abs(b.vx[sel] - a.vx[sel]).sum() / max(np.abs(a.vx[sel]).sum(), 1e-300) <= 1e-3


def test_gsph_gradients_absent_without_request():
    """zeroth-order states and gsph_gradients 0: no gradient pass"""
    case, _ = golden_case("gsph_1d_sod")
    case.options.gsph_gradients = 0
    s = Solver(case)
    s.adaptive_sml()
    s.steps(1)
    with pytest.raises(RuntimeError):
        s.gsph_gradients()
