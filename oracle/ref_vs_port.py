"""Single-core speed of the reference's own build against the oracle port --
TEST INFRASTRUCTURE (a measurement recipe, not part of the product).

Runs the same 3D plume state through the reference harness
(oracle/_ref/ref3d_plume/driver, the reference's own hot-path sources, built
by `make -C oracle ref`) and through the oracle's C restatement
(liboracle.so), both on one thread, and prints the wall time of each step.
Steps 50 and 51 are timed: step 50 builds the lists at h = dx and runs the
adaptive-h pass, step 51 runs at h ~ 1.5 dx (the smoothing length of most of
a long run).  The ratio at step 51 says how the port's CPU figures translate
to the reference's own code.

  python oracle/ref_vs_port.py [--half-width 3000] [--dx 150]

Needs the reference build (only where the reference tree is present).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for _p in (ROOT, os.path.join(ROOT, "plume-sph_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

from oracle import refio  # noqa: E402
from oracle.binding import OracleRun  # noqa: E402
from plume_gpu import cases  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--half-width", type=float, default=3000.0)
    ap.add_argument("--dx", type=float, default=150.0)
    ap.add_argument("--workdir", default="/tmp/plume_ref_vs_port")
    a = ap.parse_args()
    case = cases.plume_3d(half_width=a.half_width, height=2 * a.half_width, dx=a.dx, seed=0,
                          name="plume_ref_vs_port")
    case.step0 = 49
    nsteps = 2
    n_air = int(case.particles.need_neigh().sum())
    os.makedirs(a.workdir, exist_ok=True)
    cin = os.path.join(a.workdir, "case.bin")
    cout = os.path.join(a.workdir, "out.bin")
    refio.write_case(cin, case, nsteps)
    exe = os.path.join(HERE, "_ref", "ref3d_plume", "driver")
    t0 = time.perf_counter()
    r = subprocess.run([exe, cin, cout], cwd=a.workdir, capture_output=True, text=True,
                       env=dict(os.environ, ORACLE_STEP_TIMES="1"), check=True)
    ref_total = time.perf_counter() - t0
    ref = {int(ln.split()[1]): float(ln.split()[2]) for ln in r.stderr.splitlines()
           if ln.startswith("STEP_SECONDS")}
    o = OracleRun(case, nthreads=1)
    port = {}
    for _ in range(nsteps):
        t0 = time.perf_counter()
        o.steps(1)
        port[int(o.t.step)] = time.perf_counter() - t0
    last = max(ref)
    out = {"workload": f"plume3d_{int(2 * a.half_width)}m_{int(a.dx)}m", "n_air": n_air,
           "n_particles": int(case.particles.n), "threads": 1,
           "reference_step_seconds": ref, "port_step_seconds": port,
           "reference_run_seconds": ref_total,
           "reference_over_port_step51": ref[last] / port[last],
           "reference_particle_steps_per_s_step51": n_air / ref[last],
           "port_particle_steps_per_s_step51": n_air / port[last]}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
