"""Benchmark of the Plume-SPH particle step on GB300.

Workload: the 3D dusty-gas plume (20 x 20 x 20 km, 150 m lattice = 134^3
air particles, hydrostatic 288 K atmosphere, 100 m vent at 150 m/s / 1053 K
with ash mass fraction 0.95, outflow ghosts, +-1% jitter, seed 0), synthetic
inputs built by plume_gpu.cases.plume_config2.  A step is one pass of the
hot loop (dt, neighbour search, adaptive h every 50 steps, momentum/energy,
density, LANS filter, position update).  The metric is particle-steps/s:
need_neigh particles x steps / seconds.

  value     mixed-precision path, particles resident in HBM, CUDA events
            on the library stream over exactly K steps
  e2e       K steps through the C ABI with host buffers: every step
            uploads the particle table from pinned host memory, steps, and
            downloads it (the drop-in use by a host that keeps its own
            particle table); its window is centred on the next adaptive-h
            pass, so it holds passes at the rate of the timed window
  fp64      the FP64 path on the same workload (for the FP64 / mixed ratio)
  roofline  the momentum/energy sweep (dominant kernel)
  cpu_baseline  the CPU oracle (restatement of the reference path) on a
            bounded sample of the same workload, all host threads
  ensembles the batched path (many members per launch, CUDA graphs):
            256 1D Riemann problems (500-8,000 particles each, seed 1) and
            64 small 3D plumes (60 m lattice, 5e4-4e5 air particles each,
            seed 2), mixed and FP64, on a bounded number of steps

Timed window.  Config 2 starts from the lattice with h = dx; the first
adaptive-h pass (step 50, every 50 steps after) raises h to about 1.5 dx,
which more than triples the pairs per particle, and the 2,000-step run
spends 97 % of its steps there.  The run therefore steps untimed to just
before step 100 - K/2 (the plume develops, the inlet injects, h adapts at
step 50), warms up, and times K steps centred on the second adaptive pass:
the window holds every phase of the reference loop (dt, search, wall
boundary, adaptive h, momentum/energy, density, LANS filter, position,
inlet) at the smoothing lengths of the bulk of the run.  With the default
K = 50 (steps 75-124) it holds one adaptive-h pass per 50 steps, the rate of
a real run; a shorter K still holds one pass (a heavier share).

`--impl reference` times the reference's CPU path on the host cores: the
oracle port (OpenMP over all cores) on a bounded sample of the same state,
extrapolated to the whole table.  The reference's own C++ sources are not on
the GPU machine (they build from the reference tree, which only the build
container holds); its single-core speed against the port on the same sample
is measured there and recorded beside the numbers.
Multi-GPU: replicas only (independent copies per rank).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "plume-sph_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s"
WORKLOAD = "plume3d_20km_150m_134cube"

# algorithmic bytes per particle of the momentum/energy sweep kernel:
# i-side and j-side fields read once from HBM (neighbour reuse on chip),
# outputs written once.  Fields read: x,y,z, vx,vy,vz, vsx,vsy,vsz, h, mass,
# rho, p, c, T, cp, e, hlist (18 x 8 B) + xr,yr,zr (3 x 4 B, mixed) + bc,
# bkt (1 + 4 B); written: new v (3 x 8 B) + new e (8 B).
MOM_BYTES_READ = 18 * 8 + 3 * 4 + 1 + 4
MOM_BYTES_WRITE = 4 * 8
# algorithmic FLOPs of one in-support pair of the momentum sweep (3D with
# LANS and heat terms): 80 FLOP + 2 SFU
MOM_FLOP_PER_PAIR = 80
# ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of the
# momentum sweep on the small plume with 4^3 cells per bucket at step 99
# (h ~ 1.5 dx, the regime of the timed window): 397.9 MB + 16.8 MB for
# 778,952 particles, most of it the neighbour lists (8 B per window, read
# once per sweep), which the algorithmic bytes above do not count
MOM_DRAM_BYTES_PER_PARTICLE = 414.7e6 / 778952


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        return dist, dist.get_rank(), ws
    return None, 0, 1


def reduce_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def pinned_particles(ps, extra: int = 0):
    """copy of a ParticleSet whose arrays live in pinned host memory, with
    `extra` more rows of room (the table grows when the inlet injects)"""
    import torch
    from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS, ParticleSet
    out = ParticleSet(0)
    keep = []

    def pin(a):
        t = torch.zeros((a.shape[0] + extra,) + a.shape[1:], dtype=getattr(torch, str(a.dtype))
                        if a.dtype != np.uint64 else torch.int64, pin_memory=True)
        v = t.numpy().view(a.dtype)
        v[:a.shape[0]] = a
        keep.append(t)
        return v
    out.key = pin(ps.key)
    for f in DOUBLE_FIELDS + BYTE_FIELDS:
        setattr(out, f, pin(getattr(ps, f)))
    out._pinned = keep
    return out


SML_INTERVAL = 50


def timed_window(warmup: int, steps: int, interval: int = SML_INTERVAL):
    """(untimed preparation steps, first timed step): K timed steps centred on
    the second adaptive-h pass (step 2 * interval), starting after the first"""
    first = max(interval + 1, 2 * interval - steps // 2)
    return first - warmup - 1, first


def e2e_window(last: int, steps: int, interval: int = SML_INTERVAL) -> int:
    """first step of the e2e leg's window: K steps centred on the next
    adaptive-h pass after the timed window (ending at step `last`), so that
    it holds passes at the timed window's rate"""
    next_pass = (last // interval + 1) * interval
    return max(last + 1, next_pass - steps // 2)


def cpu_state(case):
    """the CPU sample's state: the workload after one adaptive-h pass (the
    smoothing lengths of the bulk of the run), computed by the oracle"""
    import dataclasses
    from oracle.binding import OracleRun
    o = OracleRun(case)
    o.adaptive()
    return dataclasses.replace(case, particles=o.ps)


def density_l1(ref, other, jet_radius=2000.0):
    """relative L1 density error of `other` against `ref` over the
    need_neigh particles present in both (matched by key); also over the
    particles farther than jet_radius from the vent axis (the ambient
    atmosphere, outside the jet)"""
    a, b = ref.sorted_by_key(), other.sorted_by_key()
    common, ia, ib = np.intersect1d(a.key, b.key, return_indices=True)
    real = a.need_neigh()[ia] & b.need_neigh()[ib]
    ra, rb = a.rho[ia][real], b.rho[ib][real]
    far = (a.x[ia][real] ** 2 + a.y[ia][real] ** 2) > jet_radius ** 2
    return {"l1": float(np.abs(rb - ra).sum() / np.abs(ra).sum()),
            "max_rel": float((np.abs(rb - ra) / np.abs(ra)).max()),
            "particles": int(real.sum()),
            "l1_beyond_2km_of_the_vent_axis": float(np.abs(rb - ra)[far].sum() / np.abs(ra)[far].sum())
            if far.any() else None,
            "particles_within_2km": int((~far).sum())}


def cpu_sample(case, budget_s: float = 12.0, nthreads: int = 0):
    """oracle on a bounded sample: the first `ntarget` air particles get the
    full per-step work (list build + sweeps)"""
    from oracle.binding import sample_step_seconds
    nt = 4000
    t = sample_step_seconds(case, nt, nthreads)
    if t <= 0:
        raise RuntimeError("oracle sample failed")
    per = t / nt
    nt2 = int(min(max(budget_s / per, nt), case.particles.need_neigh().sum()))
    t2 = sample_step_seconds(case, nt2, nthreads)
    return nt2, t2


def _member_l1(pa, pb, fa, fb):
    """per-member relative L1 density error of b against a (members that
    stopped on an error in either run are left out)"""
    out = []
    for k, (a, b) in enumerate(zip(pa, pb)):
        if fa[k] or fb[k]:
            continue
        r = a.need_neigh()
        out.append(float(np.abs(b.rho[r] - a.rho[r]).sum() / np.abs(a.rho[r]).sum()))
    return np.array(out)


def ensemble_1d(steps=400, warm=50, graph=50, members=256):
    """The 1D ensemble: `members` Riemann problems stepped together; the mixed
    run replays CUDA graphs of `graph` steps, the FP64 run the same.
    Particle-steps count each member's real particles for the steps it took."""
    from plume_gpu import PREC_FP64, PREC_MIXED, Ensemble, cases
    res, parts = {}, {}
    for prec in (PREC_MIXED, PREC_FP64, "fp64_perturbed"):
        cs = cases.riemann_ensemble(members, seed=1,
                                    precision=PREC_FP64 if prec == "fp64_perturbed" else prec)
        if prec == "fp64_perturbed":
            # FP64 from positions moved by one FP32 rounding (2^-24 relative):
            # the spread an FP32-size change of the state alone produces
            for c in cs:
                c.particles.x[:] = c.particles.x * (1.0 + 2.0 ** -24)
        nreal = np.array([c.info["n_real"] for c in cs], dtype=np.float64)
        e = Ensemble(cs)
        e.adaptive_sml()
        e.run(warm, graph_steps=graph)
        st0 = e.member_times()[1]
        import torch
        torch.cuda.nvtx.range_push(f"riemann1d_{prec}")  # lets a profiler select these launches
        n = e.run(steps, graph_steps=graph)
        torch.cuda.nvtx.range_pop()
        t = e.phase_times()["total"] / 1000.0
        _, st1, run1, status = e.member_times()
        ps = float((nreal * (st1 - st0)).sum())
        res[prec] = {"value": ps / t, "unit": METRIC, "steps": n, "ms_per_step": 1000.0 * t / max(n, 1),
                     "members_running": int(run1.sum()), "members_failed": int((status != 0).sum()),
                     "launches": e.launches()}
        parts[prec] = (e.split(), status != 0)
        e.close()
    err = _member_l1(parts[PREC_FP64][0], parts[PREC_MIXED][0], parts[PREC_FP64][1], parts[PREC_MIXED][1])
    ctl = _member_l1(parts[PREC_FP64][0], parts["fp64_perturbed"][0], parts[PREC_FP64][1],
                     parts["fp64_perturbed"][1])
    return {"workload": f"riemann1d_{members}_members_500_8000", "members": members,
            "particles": int(sum(c.particles.n for c in cases.riemann_ensemble(members, seed=1))),
            "graph_steps": graph, "warmup_steps": warm,
            "mixed": res[PREC_MIXED], "fp64": res[PREC_FP64],
            "mixed_over_fp64": res[PREC_MIXED]["value"] / res[PREC_FP64]["value"],
            "l1_density_vs_fp64": {"after_steps": warm + steps, "members": int(len(err)),
                                   "median": float(np.median(err)) if len(err) else None,
                                   "max": float(err.max()) if len(err) else None,
                                   "frac_le_1e-4": float((err <= 1e-4).mean()) if len(err) else None},
            "l1_density_fp64_fp32_perturbed_vs_fp64": {
                "members": int(len(ctl)), "median": float(np.median(ctl)) if len(ctl) else None,
                "max": float(ctl.max()) if len(ctl) else None,
                "frac_le_1e-4": float((ctl <= 1e-4).mean()) if len(ctl) else None},
            "note": "members stop where the reference asserts (sound speed or density <= 0 next to "
                    "the moving tube-end ghosts); particles next to those ghosts amplify per-step "
                    "differences, so late errors grow on some members (one-step error ~1e-7)"}


def ensemble_3d(steps=10, warm=10, members=64, fp64_steps=2):
    """The 3D ensemble: `members` small plumes (60 m lattice) stepped
    together, mixed with CUDA graphs of `steps` steps; FP64 for a few steps."""
    from plume_gpu import PREC_FP64, PREC_MIXED, Ensemble, cases
    from plume_gpu.autotune import tune_ensemble, with_subcells
    out = {}
    cs = cases.plume_ensemble(members, seed=2, precision=PREC_MIXED)
    t0 = time.perf_counter()
    cs, tuning = tune_ensemble(cs, candidates=(2, 3, 4, 5, 6), classes=3, steps=3)
    tuning["seconds"] = time.perf_counter() - t0
    tiles = [c.grid.subcells for c in cs]
    n_air = int(sum(c.info["n_air"] for c in cs))
    n_all = int(sum(c.particles.n for c in cs))
    e = Ensemble(cs)
    e.run(warm, graph_steps=steps)
    _, nr0 = e.count()
    n = e.run(steps, graph_steps=steps)
    t = e.phase_times()["total"] / 1000.0
    _, nr1 = e.count()
    status = e.member_times()[3]
    out["mixed"] = {"value": 0.5 * (nr0 + nr1) * n / t, "unit": METRIC, "steps": n,
                    "ms_per_step": 1000.0 * t / n, "members_failed": int((status != 0).sum()),
                    "launches": e.launches()}
    e.close()
    del cs
    cs = [with_subcells(c, s) for c, s in
          zip(cases.plume_ensemble(members, seed=2, precision=PREC_FP64), tiles)]
    e = Ensemble(cs)
    e.run(1)
    _, nr0 = e.count()
    n = e.run(fp64_steps)
    t = e.phase_times()["total"] / 1000.0
    _, nr1 = e.count()
    out["fp64"] = {"value": 0.5 * (nr0 + nr1) * n / t, "unit": METRIC, "steps": n,
                   "ms_per_step": 1000.0 * t / n}
    e.close()
    return {"workload": f"plume3d_{members}_members_60m", "members": members, "n_air": n_air,
            "particles": n_all, "graph_steps": steps, "autotune": tuning, **out,
            "mixed_over_fp64": out["mixed"]["value"] / out["fp64"]["value"]}


def adjoint_leg(steps=300, every=25, n_air=2.0e5, fd_rels=(), fd_steps=60, fd_rel=1e-10):
    """Gradient of the plume observable w.r.t. (vent velocity, temperature,
    ash fraction) through the hand-written adjoint on the config-4 geometry
    (60 m lattice) sized for n_air air particles: the time of one FP64
    forward solve, of the recorded forward + backward, their ratio, and
    central differences of full forward runs for each relative step in
    fd_rels.  The forward map is piecewise smooth (erupt-to-real
    conversions, the Gaussian's box cut-off): differences with steps that
    cross its jumps measure the jumps; small steps converge to the adjoint."""
    import torch
    from plume_gpu import adjoint, cases
    dx = 60.0
    side = dx * n_air ** (1.0 / 3.0)
    case = cases.plume_3d(half_width=0.5 * side, height=side, dx=dx, vent_radius=100.0, seed=2,
                          name="plume_adjoint")
    theta = np.array([150.0, 1053.0, 0.95])
    obj = dict(z_ash=3000.0, width=50.0, z_target=1000.0, r_scale=200.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J0 = adjoint.forward_value(theta, case, steps, **obj)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    J, g = adjoint.value_and_grad(theta, case, steps, every, **obj)
    t_grad = time.perf_counter() - t0
    out = {"workload": f"plume3d_60m_{int(case.info['n_air'])}air", "n_particles": int(case.particles.n),
           "steps": steps, "checkpoint_every": every, "objective": obj, "J": J, "J_forward": J0,
           "grad": g.tolist(), "forward_s": t_fwd, "gradient_s": t_grad,
           "gradient_over_forward": t_grad / t_fwd}
    out["fd"] = []
    for rel in fd_rels:
        t0 = time.perf_counter()
        gf = adjoint.finite_difference(theta, case, steps, rel=rel, **obj)
        out["fd"].append({"steps": steps, "rel_step": rel, "grad": gf.tolist(),
                          "rel_err": (np.abs(g - gf) / np.maximum(np.abs(g), 1e-300)).tolist(),
                          "seconds": time.perf_counter() - t0})
    # the same geometry and objective over fd_steps steps: the adjoint
    # gradient against central differences with a relative step small enough
    # to cross none of the forward map's jumps (the Gaussian's box cut-off,
    # erupt-to-real conversions); over much longer windows the map is
    # chaotic and no difference step can confirm the gradient
    if fd_steps:
        t0 = time.perf_counter()
        _, gs = adjoint.value_and_grad(theta, case, fd_steps, every, **obj)
        gf = adjoint.finite_difference(theta, case, fd_steps, rel=fd_rel, **obj)
        out["fd"].append({"steps": fd_steps, "rel_step": fd_rel, "grad_adjoint": gs.tolist(),
                          "grad": gf.tolist(),
                          "rel_err": (np.abs(gs - gf) / np.maximum(np.abs(gs), 1e-300)).tolist(),
                          "seconds": time.perf_counter() - t0})
    return out


def gsph_leg(steps=20):
    """Godunov SPH (USE_GSPH 1): particle-steps/s of the GSPH step on the
    1D Sod tube (2,000 reals, HLLC, zeroth-order states, FP64) and on a
    3D plume (4 km cube at 50 m, the reference's 3D GSPH switches: Roe,
    MINI_DERIVATIVE_COND 10 with calc_gradients every step, cubic interface,
    LANS), FP64 and mixed; device time from the step events."""
    from plume_gpu import Solver, cases
    from plume_gpu.abi import METHOD_GSPH, PREC_FP64, PREC_MIXED
    out = {}

    def timed(case, n, pre=False):
        s = Solver(case)
        if pre:
            s.adaptive_sml()
        s.steps(3)
        _, nr0 = s.count()
        s.steps(n)
        ph = s.phase_times()
        _, nr1 = s.count()
        s.close()
        t = ph["total"] / 1000.0
        return {"value": 0.5 * (nr0 + nr1) * n / t, "unit": METRIC, "ms_per_step": 1000.0 * t / n,
                "momentum_ms": ph["momentum"] / n, "n_real": int(nr1)}

    out["sod1d_2000_fp64"] = timed(cases.sod_1d(n_real=2000, method=METHOD_GSPH), steps, pre=True)
    for prec, tag in ((PREC_FP64, "fp64"), (PREC_MIXED, "mixed")):
        c = small_plume(prec)
        c.options.method = METHOD_GSPH
        out["plume3d_4km_50m_" + tag] = timed(c, max(3, steps // 4))
    return out


def small_plume(prec):
    """the test-size workload of --small (4 km tall plume at 50 m)"""
    from plume_gpu import cases
    return cases.plume_3d(half_width=2000.0, height=4000.0, dx=50.0, vent_radius=50.0,
                          vent_dx=25.0, duct_depth=600.0, seed=0, precision=prec,
                          name="plume_small_bench")


def run_reference(args, dist, rank, ws):
    """--impl reference: the reference CPU path (oracle port) on host cores"""
    if rank != 0:
        return 0
    from plume_gpu import cases
    case = cpu_state(small_plume(0) if args.small else cases.plume_config2(seed=0))
    ncores = os.cpu_count() or 1
    vals = []
    nt = None
    for k in range(args.warmup + args.steps):
        if nt is None:
            nt, t = cpu_sample(case, budget_s=max(2.0, 60.0 / (args.warmup + args.steps)))
        else:
            from oracle.binding import sample_step_seconds
            t = sample_step_seconds(case, nt, 0)
        if k >= args.warmup:
            vals.append(nt / t)
    v = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * case.particles.need_neigh().sum() / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD if not args.small else "plume3d_small",
                                         "n_air": int(case.particles.need_neigh().sum()),
                                         "inputs": "host memory"},
        "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": ncores, "kind": "port",
                         "sample": f"extrapolated: one step's neighbour lists and sweeps for the first "
                                   f"{nt} of {int(case.particles.need_neigh().sum())} air particles "
                                   f"({100.0 * nt / case.particles.need_neigh().sum():.1f} %), per-particle "
                                   f"work for all {case.particles.n}, on the state after one adaptive-h "
                                   f"pass; scaled to the whole table"},
        "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--small", action="store_true", help="test-size workload")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble legs")
    ap.add_argument("--no-tune", action="store_true", help="fixed cell tiles (4^3 per bucket)")
    ap.add_argument("--subcells", type=int, default=0, help="fixed cell tiles (N^3 per bucket), no tuning")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg")
    ap.add_argument("--no-gsph", action="store_true", help="skip the GSPH leg")
    ap.add_argument("--no-wall-bc", action="store_true",
                    help="leave the wall ghosts' states fixed (no apply_bcond in the step)")
    ap.add_argument("--no-inlet", action="store_true",
                    help="no eruption inlet (add_new_erupt) in the step")
    ap.add_argument("--only-riemann1d", action="store_true",
                    help="run only the 1D Riemann ensemble leg (--steps timed steps after --warmup) "
                         "and print its object")
    ap.add_argument("--accuracy-control", action="store_true",
                    help="with --accuracy-steps: also run the FP64 path from positions moved by one FP32 "
                         "rounding and report its density error against FP64")
    ap.add_argument("--accuracy-steps", type=int, default=0,
                    help="also report the mixed path's density error against FP64 after this "
                         "many steps (beyond the timed window's end)")
    ap.add_argument("--adjoint-fd", action="store_true",
                    help="also check the adjoint gradient by central differences, relative "
                         "steps 1e-4 and 1e-10 (12 forward solves)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    dist, rank, ws = dist_init()
    if args.impl == "reference":
        rc = run_reference(args, dist, rank, ws)
        if dist is not None:
            dist.destroy_process_group()
        return rc

    import torch
    import plume_gpu
    from plume_gpu import PREC_FP64, PREC_MIXED, Solver, cases
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    plume_gpu.build()
    if args.only_riemann1d:
        print(json.dumps(ensemble_1d(steps=args.steps, warm=args.warmup)), flush=True)
        return 0

    def make(prec):
        if args.small:
            return small_plume(prec)
        return cases.plume_config2(seed=0, precision=prec)

    case = make(PREC_MIXED)
    tuning = None
    import dataclasses
    from plume_gpu.autotune import tune_subcells, with_subcells
    if args.subcells:
        case = with_subcells(case, args.subcells)
    elif not args.no_tune:
        # tuned at the smoothing lengths of the timed window (after one
        # adaptive-h pass)
        t0 = time.perf_counter()
        best, table = tune_subcells(dataclasses.replace(case, pre_adaptive=True),
                                    candidates=(3, 4, 5, 6), steps=3, warmup=2)
        tuning = {"subcells": best, "ms_per_step": {str(k): round(v, 3) for k, v in table.items()},
                  "state": "after one adaptive-h pass", "seconds": time.perf_counter() - t0}
        case = with_subcells(case, best)
    n_air0 = int(case.particles.need_neigh().sum())
    images = None if args.no_wall_bc else cases.wall_images(case)
    inlet = None if args.no_inlet else cases.inlet(case)
    prep, first = timed_window(args.warmup, args.steps)
    last = first + args.steps - 1
    n_passes = last // SML_INTERVAL - (first - 1) // SML_INTERVAL  # adaptive-h passes in the window

    def solver(c):
        s = Solver(c)
        if images is not None:
            s.set_wall_images(*images)
        if inlet is not None:
            s.set_inlet(inlet)
        return s

    sol = solver(case)
    # untimed: the plume develops, h adapts at step 50; then the warm-up
    sol.steps(prep)
    sol.steps(args.warmup)
    barrier(dist)
    torch.cuda.synchronize()
    _, n_real_before = sol.count()
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed launches
        log = sol.steps(args.steps, log=False)
        torch.cuda.nvtx.range_pop()
        phases = sol.phase_times()
    torch.cuda.synchronize()
    launches = sol.launches()
    _, n_real_after = sol.count()
    t_dev = phases["total"] / 1000.0
    t_max = reduce_max(dist, t_dev)
    # particle-steps: need_neigh particles of each step (count at the start
    # and end of the timed region; the inlet adds < 0.1 %)
    n_real = 0.5 * (n_real_before + n_real_after)
    value = ws * n_real * args.steps / t_max
    ms_per_step = 1000.0 * t_max / args.steps
    step_end = sol.time()[1]
    mixed_end = sol.download() if not args.no_fp64 else None

    # dominant kernel: momentum sweep
    peak_hbm, peak_kind = load_peaks()
    nt, _ = sol.count()
    # the momentum pair-sweep kernel alone (CUDA events around its launch)
    mom_ms = phases["mom_kernel"] / args.steps
    alg_bytes = nt * MOM_BYTES_READ + n_real * MOM_BYTES_WRITE
    achieved_gbs = alg_bytes / (mom_ms / 1000.0) / 1e9
    npairs = None
    try:
        # in-support pairs of the momentum sweep (count only)
        import ctypes as C
        n = C.c_size_t()
        rc = sol.L.plume_neighbor_pairs(sol.ctx, 1, None, None, 0, C.byref(n))
        npairs = int(n.value) if rc == 0 else None
    except Exception:
        npairs = None
    fp32_tflops = (npairs * MOM_FLOP_PER_PAIR / (mom_ms / 1000.0) / 1e12) if npairs else None
    sm_max = 2070.0
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12  # FFMA lanes x 2 FLOP x clock
    # DRAM bytes of one launch: ncu's dram__bytes_read.sum + write.sum per
    # particle on the small plume, scaled by the particles of this workload
    traffic = MOM_DRAM_BYTES_PER_PARTICLE * nt

    # e2e: through the C ABI with pinned host buffers, every step
    # upload -> step -> download
    from plume_gpu.abi import BYTE_FIELDS, DOUBLE_FIELDS
    # the e2e window: K steps centred on the next adaptive-h pass (untimed
    # steps up to it), so that it holds passes at the timed window's rate
    e2e_steps = max(2, args.steps)
    sol.steps(e2e_window(last, e2e_steps) - (last + 1))
    e2e_first = sol.time()[1] + 1
    snap = sol.download()
    grow = 0 if inlet is None else 4 * len(inlet["col_vel"]) * (e2e_steps + 1)
    host = pinned_particles(snap, extra=grow)  # pinned copy of the whole particle table
    n_host = snap.n
    del snap
    bytes_per = 8 + 8 * len(DOUBLE_FIELDS) + len(BYTE_FIELDS)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nrs, h2d, d2h = 0, 0, 0
    for _ in range(e2e_steps):
        view = host.take(slice(0, n_host))
        sol.upload(view)
        h2d += n_host * bytes_per
        sol.steps(1)
        n_host = sol.download_into(host)
        d2h += n_host * bytes_per
        nrs += sol.count()[1]  # particles the step updated (device count)
    torch.cuda.synchronize()
    t_e2e = reduce_max(dist, time.perf_counter() - t0)
    e2e_value = ws * nrs / t_e2e
    h2d //= e2e_steps
    d2h //= e2e_steps
    sol.close()

    # FP64 path on the same workload: the same steps from the same inputs
    # (its last 3 steps timed), and the mixed path's density error against
    # it at the end of the timed window; --accuracy-steps N (> the window's
    # end) adds the error after N steps (a separate mixed run to step N)
    fp64 = None
    accuracy = None
    if not args.no_fp64:
        sub = case.grid.subcells
        s64 = solver(with_subcells(make(PREC_FP64), sub))
        k64 = 3
        s64.steps(step_end - k64)
        _, nr0 = s64.count()
        s64.steps(k64)
        ph64 = s64.phase_times()
        _, nr1 = s64.count()
        t64 = reduce_max(dist, ph64["total"] / 1000.0)
        fp64 = {"value": ws * 0.5 * (nr0 + nr1) * k64 / t64, "unit": METRIC, "steps": k64,
                "timed_steps": [step_end - k64 + 1, step_end],
                "ms_per_step": 1000.0 * t64 / k64,
                "momentum_ms": ph64["momentum"] / k64}
        accuracy = [dict(step=step_end, **density_l1(s64.download(), mixed_end))]
        del mixed_end
        if args.accuracy_steps > step_end:
            s64.steps(args.accuracy_steps - step_end)
            ref = s64.download()
            s64.close()
            sm = solver(case)
            sm.steps(args.accuracy_steps)
            entry = dict(step=args.accuracy_steps, **density_l1(ref, sm.download()))
            sm.close()
            if args.accuracy_control:
                # the FP64 path from positions moved by one FP32 rounding
                # (2^-24 relative): the spread an FP32-size change of the
                # state alone produces over the same steps
                cp = with_subcells(make(PREC_FP64), sub)
                for f in ("x", "y", "z"):
                    setattr(cp.particles, f, getattr(cp.particles, f) * (1.0 + 2.0 ** -24))
                sp = solver(cp)
                sp.steps(args.accuracy_steps)
                entry["fp64_fp32_perturbed_vs_fp64"] = density_l1(ref, sp.download())
                sp.close()
            accuracy.append(entry)
        else:
            s64.close()
    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            ncpu = os.cpu_count() or 1
            cs = cpu_state(make(PREC_FP64))
            ntg, tc = cpu_sample(cs, budget_s=12.0)
            cpu = {"value": ntg / tc, "unit": METRIC, "cores": ncpu, "kind": "port",
                   "sample": f"extrapolated: one step's neighbour lists and sweeps for the first {ntg} of "
                             f"{n_air0} air particles ({100.0 * ntg / n_air0:.1f} %), per-particle work "
                             f"for all, on the state after one adaptive-h pass"}
        except Exception as e:  # the oracle is optional on the box
            cpu = {"value": None, "unit": METRIC, "cores": 0, "kind": "port", "sample": f"failed: {e}"}

    ens = None
    if not args.no_ensemble and not args.small:
        ens = {}
        try:
            ens["riemann1d"] = ensemble_1d()
        except Exception as e:
            ens["riemann1d"] = {"failed": str(e)}
        try:
            ens["plume3d"] = ensemble_3d()
        except Exception as e:
            ens["plume3d"] = {"failed": str(e)}

    adj = None
    if not args.no_adjoint and not args.small:
        try:
            adj = adjoint_leg(fd_rels=(1e-4, 1e-10) if args.adjoint_fd else ())
        except Exception as e:
            adj = {"failed": str(e)}

    gsph = None
    if not args.no_gsph and not args.small:
        try:
            gsph = gsph_leg()
        except Exception as e:
            gsph = {"failed": str(e)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-mixed", "data": "synthetic",
            "config": {"workload": WORKLOAD if not args.small else "plume3d_small",
                       "n_air": n_air0, "n_particles": int(case.particles.n),
                       "precision": "fp32 pair arithmetic, fp64 positions and updates",
                       "parallelism": f"replicas{ws}", "l2": "working set > L2 (state ~0.6 GB)",
                       "subcells": int(case.grid.subcells), "autotune": tuning,
                       "wall_images": 0 if images is None else int(len(images[0])),
                       "inlet_columns": 0 if inlet is None else int(len(inlet["col_vel"])),
                       "timed_steps": [first, last],
                       "window": f"steps {first}-{last} after {prep + args.warmup} untimed steps from the "
                                 f"lattice (h = dx until the adaptive-h pass of step 50); the window "
                                 f"holds {n_passes} adaptive-h pass(es), one per "
                                 f"{args.steps / max(1, n_passes):.0f} steps (a run: one per {SML_INTERVAL})"},
            "gpu_launches": launches,
            "phases_ms_per_step": {k: v / args.steps for k, v in phases.items()},
            "clocks": clk.summary(),
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps,
                    "timed_steps": [e2e_first, e2e_first + e2e_steps - 1]},
            "fp64": fp64,
            "mixed_over_fp64": (value / fp64["value"]) if fp64 else None,
            "l1_density_vs_fp64": accuracy,
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peak_hbm,
                         "unit": "GB/s", "frac": achieved_gbs / peak_hbm, "traffic": traffic,
                         "kernel": "k_sweep3_list<float,WMom>", "peak_kind": peak_kind,
                         "pipe": {"bound": "fp32", "achieved_tflops": fp32_tflops,
                                  "peak_tflops": fp32_peak,
                                  "frac": (fp32_tflops / fp32_peak) if fp32_tflops else None,
                                  "pairs_per_launch": npairs,
                                  "flop_per_pair": MOM_FLOP_PER_PAIR}},
            "cpu_baseline": cpu,
            "ensembles": ens,
            "adjoint": adj,
            "gsph": gsph,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
