"""Generate the golden vectors that pin the CPU oracle.

Runs the reference solver's own hot-path sources (compiled by
`make -C oracle ref` from the Plume-SPH tree, driven by oracle/ref/driver.cc)
on three small workloads and stores inputs, per-step dt, the final particle
state and a summary of the reference's neighbour lists:

  sod_1d_200.npz       1D Sod, 200 equal-mass reals, cubic-spline kernel
                       (kernel-swap build), h = 1.3 m/rho, CFL 0.3, 20 steps
  sod_1d_2000_end.npz  the 1D Sod workload: 2,000 equal-mass reals, Gaussian
                       kernel, run to t = 0.2 (final state only), plus the
                       final state of a second reference run whose input
                       differs by one ulp in the x of the wall-adjacent
                       particle (the scheme's own sensitivity floor)
  shock_tube_1d.npz    the reference's shipped 1D deck (Gaussian kernel,
                       SHOCK_TUBE_TESTS 1, h0 = 0.003, 397 particles), 20 steps
  plume_3d_small.npz   3D plume, 600 m cube at 50 m spacing with pressure,
                       wall and erupt ghosts, LANS + energy smoothing, steps
                       49..51 (step 50 runs adaptive_sml)
  plume_3d_bc.npz      the same plume (seed 4) with the wall boundary: the
                       flat-ground image table of cases.wall_images, the
                       reference's apply_bcond before the loop and after each
                       of steps 49..51
  gsph_*.npz           GSPH builds (make_gsph)
  adapt_3d.npz         domain growth: scan_outside_layer + adapt_domain
                       (make_adapt)

Usage (in a container that has the reference tree):
  python tests/golden/make_golden.py [--ref REFERENCE_TREE]
(default: $PLUME_REFERENCE, else a directory named "reference" beside this
checkout)
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "plume-sph_gb300"))
sys.path.insert(0, os.path.dirname(HERE))

from plume_gpu import cases  # noqa: E402
from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS  # noqa: E402
from oracle import refio  # noqa: E402
from _util import adapt_case, gsph_case  # noqa: E402

MASK = np.uint64(0xFFFFFFFFFFFFFFFF)


def mix64(k):
    """splitmix64 finaliser (order-independent list hashing)."""
    z = (np.asarray(k, dtype=np.uint64) + np.uint64(0x9E3779B97F4A7C15)) & MASK
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & MASK
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & MASK
    return z ^ (z >> np.uint64(31))


def list_summary(keys_i, lists_by_i):
    """count and order-independent hash of each particle's neighbour set"""
    cnt = np.zeros(len(keys_i), dtype=np.int64)
    hsh = np.zeros(len(keys_i), dtype=np.uint64)
    for r, k in enumerate(keys_i):
        lj = lists_by_i[int(k)]
        cnt[r] = len(lj)
        with np.errstate(over="ignore"):
            hsh[r] = np.bitwise_xor.reduce(mix64(lj)) if len(lj) else np.uint64(0)
    return cnt, hsh


def pack(prefix, ps):
    out = {f"{prefix}key": ps.key}
    for f in DOUBLE_FIELDS + BYTE_FIELDS:
        out[f"{prefix}{f}"] = getattr(ps, f)
    return out


def make(case, variant, nsteps, path, sample_lists=64, dump_last=False, perturb_key=None, images=None):
    steps, lists = refio.run_ref(variant, case, nsteps, "/tmp/plume_golden", dump_last, images)
    extra = {}
    if perturb_key is not None:
        pc = case.__class__(**{**case.__dict__, "particles": case.particles.copy()})
        k = int(np.nonzero(pc.particles.key == perturb_key)[0][0])
        pc.particles.x[k] = np.nextafter(pc.particles.x[k], np.inf)
        psteps, _ = refio.run_ref(variant, pc, nsteps, "/tmp/plume_golden_p", dump_last)
        extra.update(pack("ulp_", psteps[-1]["particles"].sorted_by_key()))
        extra["ulp_key"] = np.uint64(perturb_key)
        extra["ulp_step"] = psteps[-1]["step"]
    if dump_last:
        nsteps = steps[-1]["step"] - case.step0
    o = case.options
    d = {
        "dim": o.dim, "nsteps": nsteps, "pre_adaptive": int(case.pre_adaptive),
        "step0": case.step0, "dt": np.array([s["dt"] for s in steps]),
        "time": np.array([s["time"] for s in steps]),
        "step": np.array([s["step"] for s in steps]),
    }
    d.update(pack("in_", case.particles))
    d.update(pack("out_", steps[-1]["particles"].sorted_by_key()))
    ki = np.array(sorted(lists.keys()), dtype=np.uint64)
    cnt, hsh = list_summary(ki, lists)
    d.update({"list_key": ki, "list_count": cnt, "list_hash": hsh})
    rng = np.random.default_rng(7)
    pick = rng.choice(len(ki), size=min(sample_lists, len(ki)), replace=False)
    flat, offs = [], [0]
    for r in sorted(pick):
        flat.append(np.asarray(lists[int(ki[r])], dtype=np.uint64))
        offs.append(offs[-1] + len(flat[-1]))
    d.update({"sample_key": ki[sorted(pick)], "sample_offs": np.array(offs, dtype=np.int64),
              "sample_flat": np.concatenate(flat) if flat else np.zeros(0, np.uint64)})
    if o.dim == 3:
        # the lists of the last step were built from the state before it
        d.update(pack("pre_", (steps[-2]["particles"] if len(steps) > 1 else case.particles).sorted_by_key()))
    d.update(extra)
    if images is not None:
        d["img_key"] = np.asarray(images[0], dtype=np.uint64)
        d["img_xyz"] = np.asarray(images[1], dtype=np.float64)
    if "grad" in steps[-1]:
        d["grad_key"], d["grad"] = steps[-1]["grad"]
    np.savez_compressed(path, **d)
    print(f"wrote {path}: {os.path.getsize(path) / 1e6:.2f} MB")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    a = ap.parse_args()
    refio.build_ref(a.ref)
    make(cases.sod_1d(n_real=200, kernel=cases.KERNEL_M4), "ref1d_sod", 20,
         os.path.join(HERE, "sod_1d_200.npz"))
    sod = cases.sod_1d(n_real=2000)
    wall = int(sod.particles.key[sod.particles.need_neigh()][0])  # first real particle
    make(sod, "ref1d_sodg", -1, os.path.join(HERE, "sod_1d_2000_end.npz"),
         sample_lists=4, dump_last=True, perturb_key=wall)
    make(cases.shock_tube_1d(), "ref1d_gauss", 20, os.path.join(HERE, "shock_tube_1d.npz"))
    c = cases.plume_3d(half_width=300.0, height=600.0, dx=50.0, vent_radius=50.0,
                       vent_dx=25.0, duct_depth=300.0, seed=3, name="plume_3d_small")
    c.step0 = 48
    make(c, "ref3d_plume", 3, os.path.join(HERE, "plume_3d_small.npz"))
    make_bc()
    make_gsph()
    make_gsph_end()
    make_adapt()
    make_adapt_pg()
    make_wall_ghost()
    make_air()
    make_duct()
    make_inlet()
    make_csv()
    make_grid()


def make_gsph_end():
    """gsph_1d_2000_end.npz: the 1D Sod workload (2,000 reals) with GSPH
    (HLLC, zeroth-order states) to t = 0.2, final state only, plus the
    reference's one-ulp sensitivity run"""
    sod = cases.sod_1d(n_real=2000, method=cases.METHOD_GSPH)
    wall = int(sod.particles.key[sod.particles.need_neigh()][0])
    make(sod, "ref1d_gsph", -1, os.path.join(HERE, "gsph_1d_2000_end.npz"),
         sample_lists=4, dump_last=True, perturb_key=wall)


def make_gsph():
    """GSPH (USE_GSPH 1) fixtures with the last step's gradients:
      gsph_1d_sod.npz   1D Sod, 200 reals, HLLC, zeroth-order states, 20 steps
      gsph_1d_grad.npz  ghost-free 1D Sod with h = 2 m/rho, linear states
                        (MINI_DERIVATIVE_COND 1), the reference's own
                        calc_gradients, 20 steps
      gsph_3d.npz       a 400 m cube of the 3D plume (seed 5) with the 3D GSPH defaults
                        (Roe, cubic interface, MINI_DERIVATIVE_COND 10,
                        modified monotonicity), steps 49..50"""
    make(gsph_case("gsph_1d_sod"), "ref1d_gsph", 20, os.path.join(HERE, "gsph_1d_sod.npz"))
    make(gsph_case("gsph_1d_grad"), "ref1d_gsph_grad", 20, os.path.join(HERE, "gsph_1d_grad.npz"))
    make(gsph_case("gsph_3d"), "ref3d_gsph", 2, os.path.join(HERE, "gsph_3d.npz"))
    make_gsph_solvers()


def make_gsph_solvers():
    """gsph_1d_my2 / my3 / vl, gsph_3d_my3 / vl: the Sod tube and the 3D cube
    of gsph_1d_sod / gsph_3d with the reference's other Riemann solvers,
    HLLC_RP_Solver_my (HLL_WAVE_SPEED_EVA 2 and 3) and VanLeer_RP_Solver,
    over the steps the reference completes: with HLLC_RP_Solver_my its step
    2 stops on assert(c > 0) (timestep.cc), with Van Leer's solver the Sod
    tube's step 9"""
    from _util import GSPH_SOLVER_BUILDS, GSPH_SOLVER_STEPS
    for name, build in GSPH_SOLVER_BUILDS.items():
        make(gsph_case(name), build, GSPH_SOLVER_STEPS[name], os.path.join(HERE, name + ".npz"))


def make_adapt():
    """adapt_3d.npz: domain growth on the small plume (seed 6): one step
    (step 49), then the reference's scan_outside_layer and adapt_domain on
    the set-up of cases.adapt_scenario; stores the input, the bucket flags
    and involvement states before and after, the scan's count, and the
    particles' key, bc type, involvement and x after adapt_domain."""
    c = adapt_case()
    c, binv = cases.adapt_scenario(c)
    steps, _ = refio.run_ref("ref3d_adapt", c, 1, "/tmp/plume_golden", binv=binv, adapt=True)
    na, st = steps[-1]["adapt"]
    out = steps[-1]["particles"].sorted_by_key()
    d = {"nsteps": 1, "step0": c.step0, "pre_adaptive": 0, "dim": 3,
         "flags": np.asarray(c.grid.flags, dtype=np.uint8), "binv_in": binv, "binv_out": st,
         "adapt": np.int64(na), "out_key": out.key, "out_bc_type": out.bc_type,
         "out_involved": out.involved, "out_x": out.x}
    d.update(pack("in_", c.particles))
    path = os.path.join(HERE, "adapt_3d.npz")
    np.savez_compressed(path, **d)
    print(f"wrote {path}: {os.path.getsize(path) / 1e6:.2f} MB")


def make_adapt_pg():
    """adapt_pg_3d.npz: the domain-growth set-up with the bucket layer
    outside the converted one emptied (cases.adapt_scenario, clear_beyond):
    one step, scan_outside_layer, adapt_domain, then the reference's
    add_pressure_ghost.  Stores the input, flags and involvement states, and
    the particles add_pressure_ghost created (by the reference's key) with
    every bucket's activity after it."""
    c = adapt_case()
    c, binv = cases.adapt_scenario(c, clear_beyond=True)
    steps, _ = refio.run_ref("ref3d_adapt", c, 1, "/tmp/plume_golden", binv=binv, adapt=2)
    na, st = steps[-1]["adapt"]
    d = {"nsteps": 1, "step0": c.step0, "pre_adaptive": 0, "dim": 3,
         "flags": np.asarray(c.grid.flags, dtype=np.uint8), "binv_in": binv, "binv_out": st,
         "adapt": np.int64(na), "active": steps[-1]["active"]}
    d.update(pack("in_", c.particles))
    d.update(pack("born_", steps[-1]["born"]))
    path = os.path.join(HERE, "adapt_pg_3d.npz")
    np.savez_compressed(path, **d)
    print(f"wrote {path}: {os.path.getsize(path) / 1e6:.2f} MB")


def make_wall_ghost():
    """wall_ghost_3d.npz: cases.wall_scenario on the domain-growth plume
    (seed 6): one step, then the reference's add_wall_ghost.  Stores the
    input, flags and involvement states, and the particles add_wall_ghost
    created with every bucket's activity after it."""
    c, binv = cases.wall_scenario(adapt_case())
    steps, _ = refio.run_ref("ref3d_adapt", c, 1, "/tmp/plume_golden", binv=binv, adapt=3)
    d = {"nsteps": 1, "step0": c.step0, "pre_adaptive": 0, "dim": 3,
         "flags": np.asarray(c.grid.flags, dtype=np.uint8), "binv_in": binv,
         "active": steps[-1]["active"]}
    d.update(pack("in_", c.particles))
    d.update(pack("born_", steps[-1]["born"]))
    path = os.path.join(HERE, "wall_ghost_3d.npz")
    np.savez_compressed(path, **d)
    print(f"wrote {path}: {os.path.getsize(path) / 1e6:.2f} MB")


def make_air():
    """add_air_3d.npz: cases.air_scenario on the domain-growth plume (seed
    6): one step, then the reference's add_air.  Stores the input, flags and
    involvement states, and the particles add_air created."""
    c, binv = cases.air_scenario(adapt_case())
    steps, _ = refio.run_ref("ref3d_adapt", c, 1, "/tmp/plume_golden", binv=binv, adapt=4)
    d = {"nsteps": 1, "step0": c.step0, "pre_adaptive": 0, "dim": 3,
         "flags": np.asarray(c.grid.flags, dtype=np.uint8), "binv_in": binv,
         "active": steps[-1]["active"]}
    d.update(pack("in_", c.particles))
    d.update(pack("born_", steps[-1]["born"]))
    path = os.path.join(HERE, "add_air_3d.npz")
    np.savez_compressed(path, **d)
    print(f"wrote {path}: {os.path.getsize(path) / 1e6:.2f} MB")


def make_duct():
    """setup_erupt_3d.npz: cases.duct_scenario on the domain-growth plume
    (seed 6): one step, then the reference's setup_erupt.  Stores the input,
    the particles setup_erupt created, and the keys of the case particles
    left after it."""
    c, binv, _ = cases.duct_scenario(adapt_case())
    steps, _ = refio.run_ref("ref3d_adapt", c, 1, "/tmp/plume_golden", binv=binv, adapt=5)
    d = {"nsteps": 1, "step0": c.step0, "pre_adaptive": 0, "dim": 3, "binv_in": binv,
         "kept_key": np.sort(steps[-1]["particles"].key)}
    d.update(pack("in_", c.particles))
    d.update(pack("born_", steps[-1]["born"]))
    path = os.path.join(HERE, "setup_erupt_3d.npz")
    np.savez_compressed(path, **d)
    print(f"wrote {path}: {os.path.getsize(path) / 1e6:.2f} MB")


INLET_STEPS = 6


def make_inlet():
    """inlet_3d.npz: the reference's own add_new_erupt.  cases.duct_scenario
    on the domain-growth plume (seed 6); the reference's setup_erupt alone
    gives the duct and the case particles it keeps (mode 5, no step); then
    setup_erupt before the loop and INLET_STEPS steps with add_new_erupt in
    each (mode 6).  Stores the input, the duct, the kept keys, the case
    particles after the steps, the step times, and every particle the run
    created (duct and inlet) in its final state."""
    c, binv, duct = cases.duct_scenario(adapt_case())
    s5, _ = refio.run_ref("ref3d_adapt", c, 0, "/tmp/plume_golden", binv=binv, adapt=5)
    s6, _ = refio.run_ref("ref3d_adapt", c, INLET_STEPS, "/tmp/plume_golden", binv=binv, adapt=6)
    d = {"nsteps": INLET_STEPS, "step0": c.step0, "pre_adaptive": 0, "dim": 3, "binv_in": binv,
         "kept_key": np.sort(s5[-1]["particles"].key),
         "dt": np.array([r["dt"] for r in s6[:INLET_STEPS]]),
         "time": np.array([r["time"] for r in s6[:INLET_STEPS]]),
         "duct": np.array([duct[k] for k in ("x0", "y0", "z_top", "depth", "radius", "np", "profile",
                                             "u_avg")], dtype=np.float64)}
    d.update(pack("in_", c.particles))
    d.update(pack("duct_", s5[-1]["born"]))
    d.update(pack("out_", s6[INLET_STEPS - 1]["particles"]))
    d.update(pack("born_", s6[-1]["born"]))
    path = os.path.join(HERE, "inlet_3d.npz")
    np.savez_compressed(path, **d)
    print(f"wrote {path}: {os.path.getsize(path) / 1e6:.2f} MB")


GRID_DOMAINS = (
    # (name, lo, hi, h0, nproc): the 20 km plume domain at 150 m, the 600 m
    # test plume at 50 m, and a ragged domain above 1.5 km (bucket counts
    # rounded up, records split over three processes)
    ("plume_20km", (-1.0e4, -1.0e4, 0.0), (1.0e4, 1.0e4, 2.0e4), 150.0, 1),
    ("plume_600m", (-300.0, -300.0, 0.0), (300.0, 300.0, 600.0), 50.0, 1),
    ("ragged", (-2400.0, -2350.0, 1500.0), (2410.0, 2400.0, 14000.0), 137.3, 3),
)


def make_grid():
    """grid_3d.npz: the reference preprocessor's buckets (type,
    bucket_index, lower corner) and hash-table bounds for GRID_DOMAINS"""
    d = {}
    for name, lo, hi, h0, nproc in GRID_DOMAINS:
        ht, r = refio.run_preproc(lo, hi, h0, "/tmp/plume_golden_grid", nproc)
        d[f"{name}_ht"] = ht
        d[f"{name}_type"] = r["type"].astype(np.int8)
        d[f"{name}_index"] = r["index"].astype(np.int8)
        d[f"{name}_lo"] = r["lo"]
        d[f"{name}_domain"] = np.array(list(lo) + list(hi) + [h0])
    path = os.path.join(HERE, "grid_3d.npz")
    np.savez_compressed(path, **d)
    print(f"wrote {path}: {os.path.getsize(path) / 1e6:.2f} MB")


def make_csv():
    """sod_1d_csv.npz: the 1D Sod tube (200 reals, Gaussian kernel) after 20
    steps and the text the reference's write_csv appends for that state
    (h5part_writer.cc:448-490; rows in key order, see oracle/ref/driver.cc)"""
    case = cases.sod_1d(n_real=200)
    work = "/tmp/plume_golden_csv"
    os.makedirs(work, exist_ok=True)
    out = os.path.join(work, "pvplot_out.csv")
    if os.path.exists(out):
        os.remove(out)
    steps, _ = refio.run_ref("ref1d_csv", case, 20, work, dump_last=True)
    with open(out) as f:
        text = f.read()
    d = {"nsteps": 20, "step0": case.step0, "pre_adaptive": int(case.pre_adaptive), "dim": 1,
         "csv": np.array(text)}
    d.update(pack("out_", steps[-1]["particles"].sorted_by_key()))
    path = os.path.join(HERE, "sod_1d_csv.npz")
    np.savez_compressed(path, **d)
    print(f"wrote {path}: {os.path.getsize(path) / 1e6:.2f} MB")


def make_bc():
    c = cases.plume_3d(half_width=300.0, height=600.0, dx=50.0, vent_radius=50.0,
                       vent_dx=25.0, duct_depth=300.0, seed=4, name="plume_3d_bc")
    c.step0 = 48
    make(c, "ref3d_plume", 3, os.path.join(HERE, "plume_3d_bc.npz"), images=cases.wall_images(c))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--gsph":
        refio.build_ref()
        make_gsph()
    elif len(sys.argv) > 1 and sys.argv[1] == "--adapt":
        refio.build_ref()
        make_adapt()
    elif len(sys.argv) > 1 and sys.argv[1] == "--duct":
        refio.build_ref()
        make_duct()
    elif len(sys.argv) > 1 and sys.argv[1] == "--gsph-solvers":
        refio.build_ref()
        make_gsph_solvers()
    elif len(sys.argv) > 1 and sys.argv[1] == "--inlet":
        refio.build_ref()
        make_inlet()
    elif len(sys.argv) > 1 and sys.argv[1] == "--air":
        refio.build_ref()
        make_air()
    elif len(sys.argv) > 1 and sys.argv[1] == "--wall-ghost":
        refio.build_ref()
        make_wall_ghost()
    elif len(sys.argv) > 1 and sys.argv[1] == "--adapt-pg":
        refio.build_ref()
        make_adapt_pg()
    elif len(sys.argv) > 1 and sys.argv[1] == "--grid":
        refio.build_ref()
        make_grid()
    elif len(sys.argv) > 1 and sys.argv[1] == "--csv":
        refio.build_ref()
        make_csv()
    elif len(sys.argv) > 1 and sys.argv[1] == "--gsph-end":
        refio.build_ref()
        make_gsph_end()
    else:
        main()
