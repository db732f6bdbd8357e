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
