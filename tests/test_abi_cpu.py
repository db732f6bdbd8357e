"""Host-side checks that need no GPU: the C-ABI library builds and exports
every entry point declared in include/plume_gpu.h, the ctypes structs match
the header's layout, and the input reader and workload builders follow the
reference's conventions."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import plume_gpu
from plume_gpu import abi, cases, inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "plume_gpu.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*\*?\s*(plume_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    plume_gpu.build()
    lib = C.CDLL(plume_gpu._lib.LIBPATH)
    names = header_functions()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.plume_version and C.c_char_p(lib.plume_version.restype and None) is not None


def test_ctypes_struct_layout_matches_header():
    # compile a probe with the header and compare offsets/sizes
    import subprocess
    import tempfile
    probe = r'''
#include <stdio.h>
#include <stddef.h>
#include "plume_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(PlumeOptions), sizeof(PlumeGrid), sizeof(PlumeSoA), sizeof(PlumeStepLog));
  printf("%zu %zu %zu\n", offsetof(PlumeOptions, capacity), offsetof(PlumeGrid, domain_hi), offsetof(PlumeSoA, involved));
  printf("%zu %zu %zu %zu %zu\n", sizeof(PlumeAtmosphere), offsetof(PlumeAtmosphere, Ate3), sizeof(PlumeDuct),
         offsetof(PlumeDuct, u_avg), offsetof(PlumeDuct, c));
  printf("%zu %zu\n", sizeof(PlumeInlet), offsetof(PlumeOptions, gsph_gradients));
  return 0;
}'''
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "p.c")
        open(src, "w").write(probe)
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    sizes = [int(v) for v in out]
    assert sizes[0] == C.sizeof(abi.PlumeOptions)
    assert sizes[1] == C.sizeof(abi.PlumeGrid)
    assert sizes[2] == C.sizeof(abi.PlumeSoA)
    assert sizes[3] == C.sizeof(abi.PlumeStepLog)
    assert sizes[4] == abi.PlumeOptions.capacity.offset
    assert sizes[5] == abi.PlumeGrid.domain_hi.offset
    assert sizes[6] == abi.PlumeSoA.involved.offset
    assert sizes[7] == C.sizeof(abi.PlumeAtmosphere)
    assert sizes[8] == abi.PlumeAtmosphere.Ate3.offset
    assert sizes[9] == C.sizeof(abi.PlumeDuct)
    assert sizes[10] == abi.PlumeDuct.u_avg.offset
    assert sizes[11] == abi.PlumeDuct.c.offset
    assert sizes[12] == C.sizeof(abi.PlumeInlet)
    assert sizes[13] == abi.PlumeOptions.gsph_gradients.offset


def test_read_data_uses_single_precision(tmp_path):
    # the shipped Sod deck of the reference (values after the last ':')
    sim = inputs.SimulationData(max_time=0.17, max_steps=100000000, timeoutput=0.1, stat_erupt=0.0,
                                end_erupt=7200.0, format=1, p_constant=2587463, gamma=1.4,
                                smoothing_length=0.003, idom=(-0.4, 0.4, 0, 0, 0, 0))
    inputs.write_data(str(tmp_path), sim)
    got = inputs.read_data(str(tmp_path))
    assert got.smoothing_length == float(np.float32(0.003))
    assert got.max_time == float(np.float32(0.17))
    assert got.max_steps == 100000000
    assert got.idom[0] == float(np.float32(-0.4))


def test_sod_builder_counts_and_equal_mass():
    c = cases.sod_1d(n_real=2000)
    ps = c.particles
    real = ps.need_neigh()
    assert int(real.sum()) == 2000
    assert int((ps.bc_type == 0).sum()) == 20
    assert np.allclose(ps.mass[real], ps.mass[real][0], rtol=1e-12)
    assert ps.x[real].min() > 0 and ps.x[real].max() < 1
    assert c.options.eta_smooth == 1.3 and c.options.cfl == 0.3
    assert abs(1 + c.options.ra / c.options.cva - 1.4) < 1e-15


def test_plume_builder_geometry():
    c = cases.plume_small()
    g, ps = c.grid, c.particles
    assert g.del_ == 8 * 50.0
    # every particle inside the bucket grid
    for a, f in enumerate("xyz"):
        v = getattr(ps, f)
        assert v.min() >= g.mindom[a] and v.max() < g.mindom[a] + g.nb[a] * g.del_
    # vent particles are pressure balanced with the air at the ground
    vent = ps.bc_type == abi.BC_ERUPT
    air = ps.bc_type == abi.BC_REAL
    assert vent.sum() > 0
    assert np.allclose(ps.p[vent], 101325.0, rtol=1e-9)
    assert np.all(ps.Y[vent] == 1.0) and np.all(ps.Y[air] == 0.0)
    # bucket types: mixed buckets straddle the domain faces
    assert (g.flags & abi.BUCKET_MIXED).any() and (g.flags & abi.BUCKET_ABSORBING).any()


def test_config2_size():
    """the benchmark's workload, pinned: 134^3 air particles of the 20 km
    cube at 150 m, the ghosts and the vent duct, the wall images of its
    ground and the inlet's duct columns"""
    c = cases.plume_config2()
    assert int(c.particles.need_neigh().sum()) == 2388148
    assert c.particles.n == 3091228
    assert len(cases.wall_images(c)[0]) == 85248
    assert len(cases.inlet(c)["col_vel"]) == 12


def test_riemann_ensemble_builder():
    a = cases.riemann_ensemble(256, seed=1)
    b = cases.riemann_ensemble(256, seed=1)
    n = np.array([c.info["n_real"] for c in a])
    assert len(a) == 256 and n.min() >= 480 and n.max() <= 8100
    # log-uniform counts: about half the members below the geometric mean
    assert 0.35 < (n < np.sqrt(500 * 8000)).mean() < 0.65
    for ca, cb in zip(a, b):
        assert ca.info["states"] == cb.info["states"]
        (rl, pl, ul), (rr, pr, ur) = ca.info["states"]
        assert 0.1 <= min(rl, rr) and max(rl, rr) <= 1.0
        assert 0.01 <= min(pl, pr) and max(pl, pr) <= 1.0
        assert -1.0 <= min(ul, ur) and max(ul, ur) <= 1.0
        ps = ca.particles
        r = ps.need_neigh()
        np.testing.assert_allclose(ps.mass[r], ps.mass[r][0], rtol=1e-6)  # equal mass
        # the grid covers the ghosts' travel to t_end
        g = ca.grid
        lo, hi = g.mindom[0], g.mindom[0] + g.nb[0] * g.del_
        reach = max(abs(ul), abs(ur)) * ca.options.max_time
        assert lo < ps.x.min() - reach and hi > ps.x.max() + reach


def test_plume_ensemble_builder():
    cs = cases.plume_ensemble(6, seed=2, dx=60.0, n_lo=2.0e3, n_hi=2.0e4, duct_depth=300.0)
    for c in cs:
        assert 80.0 <= c.info["vent_velocity"] <= 200.0
        assert 900.0 <= c.info["vent_T"] <= 1200.0
        assert 0.9 <= c.info["ash"] <= 0.98
        assert abs(c.options.ng0 - (1.0 - c.info["ash"])) < 1e-12
        assert 1.0e3 <= c.info["n_air"] <= 4.0e4
        assert c.options.capacity >= c.particles.n
    # the shared options are equal across members (the batch create checks it)
    keys = ["dim", "precision", "kernel", "lans", "alpha", "beta", "cutoff2", "list_factor"]
    for k in keys:
        assert len({getattr(c.options, k) for c in cs}) == 1, k


def test_reference_side_bridge_compiles_and_round_trips():
    """plume-sph_gb300/bridge/gpu_bridge.cc, the binding a Plume-SPH build
    adds to src/plume/, compiled against the reference's own headers
    (particle.h, thashtab.h, parameters.h) and linked with the reference's
    particle and hash-table objects and libplume_gpu.so; its self-test packs
    a table, applies a device-like change (reorder, delete, update, create)
    and unpacks it without a GPU"""
    import subprocess
    sys_ref = os.environ.get("PLUME_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
    if not os.path.isdir(os.path.join(sys_ref, "src", "datstr")):
        pytest.skip("the reference tree is not present")
    plume_gpu.build()
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "bridge", f"REF={sys_ref}"],
                   check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "bridge", "gpu_bridge_selftest")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "self-test: ok" in r.stdout
