"""Gradients of plume observables through the particle step (torch).

`PlumeSteps` is a torch.autograd.Function over a window of FP64 particle
steps: its forward runs the steps on the GPU (plume_adjoint_record, keeping
checkpoints), its backward is the library's hand-written adjoint
(plume_adjoint_backward: segment recompute from the checkpoints, then the
stage-by-stage reverse of every step).  Inputs are the particle fields of
the window's first state and the EOS constant ng0; outputs are the fields of
the final state.  Around it, plain torch code maps the vent parameters
theta = (vent velocity, vent temperature, ash mass fraction) to the first
state (`vent_initial_state`, the builder's formulas for the eruption duct
and the EOS of every particle) and the final state to an observable
(`plume_objective`), so `J.backward()` gives dJ/dtheta.

Discrete decisions (neighbour lists, the particle that sets dt, erupt-to-real
conversions, deletions) are those of the forward run; `finite_difference`
checks the gradient with central differences of full forward runs.
"""
from __future__ import annotations

import copy
import dataclasses

import numpy as np
import torch

from .abi import BC_ERUPT, ParticleSet
from .solver import Solver

# the fields the adjoint carries, in the library's order
FIELDS = ("x", "y", "z", "vx", "vy", "vz", "vsx", "vsy", "vsz", "mass", "h", "rho", "e", "p", "Y",
          "c", "T", "cp")


def eos_torch(opt, rho, Y, e, ng0):
    """Particle::update_second_var (particle.cc:528-604) in torch, the same
    operation order as the library's EOS; returns (gamma, p, c, T, cp)"""
    na = 1 - Y
    ng = ng0 * Y
    ns = Y - ng
    Cvm = ns * opt.cvs + ng * opt.cvg + na * opt.cva
    Rm = ng * opt.rg + na * opt.ra
    Rmg = Rm / (ng + na)
    gam = 1 + Rm / Cvm
    desmg = rho * (na + ng)
    p = Rmg * desmg * e / Cvm
    c = torch.sqrt(gam * p / desmg)
    T = e / Cvm
    return gam, p, c, T, Cvm


class PlumeSteps(torch.autograd.Function):
    """nsteps FP64 steps of `case` from first-state fields (18 float64
    tensors in FIELDS order, rows in case.particles order) and ng0; returns
    the final fields as an (18, n_final) tensor and the final keys."""

    @staticmethod
    def forward(ctx, ng0, *args):
        fields, (case, nsteps, every) = args[:18], args[18:]
        ps = case.particles.take(np.arange(case.particles.n))
        for f, t in zip(FIELDS, fields):
            getattr(ps, f)[:] = t.detach().cpu().numpy()
        opt = copy.deepcopy(case.options)
        opt.ng0 = float(ng0)
        g, _, _, _, _ = eos_torch(opt, torch.from_numpy(ps.rho), torch.from_numpy(ps.Y),
                                  torch.from_numpy(ps.e), float(ng0))
        ps.gamma[:] = g.numpy()
        sol = Solver(dataclasses.replace(case, options=opt, particles=ps))
        sol.adjoint_record(nsteps, every)
        fin = sol.download()
        ctx.sol = sol
        ctx.n0 = ps.n
        ctx.keys0 = ps.key.copy()
        ctx.device = fields[0].device
        ctx.fin_keys = fin.key.copy()
        out = torch.from_numpy(np.stack([getattr(fin, f) for f in FIELDS])).to(ctx.device)
        keys = torch.from_numpy(fin.key.astype(np.int64)).to(ctx.device)
        ctx.mark_non_differentiable(keys)
        return out, keys

    @staticmethod
    def backward(ctx, gout, gkeys):
        fb = ParticleSet(len(ctx.fin_keys))
        fb.key[:] = ctx.fin_keys
        g = gout.detach().cpu().numpy()
        for k, f in enumerate(FIELDS):
            getattr(fb, f)[:] = g[k]
        ib, ng0b = ctx.sol.adjoint_backward(fb)
        # rows of the first state -> the input order, by key
        order = np.argsort(ctx.keys0, kind="stable")
        pos = order[np.searchsorted(ctx.keys0[order], ib.key)]
        grads = []
        for f in FIELDS:
            a = np.zeros(ctx.n0)
            a[pos] = getattr(ib, f)
            grads.append(torch.from_numpy(a).to(ctx.device))
        ctx.sol.close()
        return (torch.tensor(ng0b, dtype=torch.float64, device=ctx.device), *grads, None, None, None)


def vent_initial_state(theta, case):
    """The first state of `case` as a function of theta = (vent velocity
    m/s, vent temperature K, ash mass fraction): the eruption duct's
    particles get the builder's vent state (vz = V, rho = p0 / (Rg T) / ng0,
    e = (ng0 Cvg + (1 - ng0) Cvs) T, m = rho dx_vent^3, ng0 = 1 - ash) and
    every particle its EOS fields.  Returns (ng0, 18 field tensors)."""
    opt = case.options
    ps = case.particles
    V, Tv, ash = theta[0], theta[1], theta[2]
    ng0 = 1 - ash
    vent = torch.from_numpy((ps.bc_type == BC_ERUPT) & (ps.phase == 2))
    base = {f: torch.from_numpy(getattr(ps, f).copy()) for f in FIELDS}
    vdx = case.info["vent_dx"]
    p0 = case.info.get("p0", 101325.0)
    rhov = p0 / (opt.rg * Tv) / ng0
    ev = (ng0 * opt.cvg + (1 - ng0) * opt.cvs) * Tv
    out = dict(base)
    out["vz"] = torch.where(vent, V * torch.ones_like(base["vz"]), base["vz"])
    out["rho"] = torch.where(vent, rhov * torch.ones_like(base["rho"]), base["rho"])
    out["e"] = torch.where(vent, ev * torch.ones_like(base["e"]), base["e"])
    out["mass"] = torch.where(vent, rhov * vdx ** 3 * torch.ones_like(base["mass"]), base["mass"])
    _, p, c, T, cp = eos_torch(opt, out["rho"], out["Y"], out["e"], ng0)
    out["p"], out["c"], out["T"] = p, c, T
    if opt.lans:
        out["cp"] = cp
    return ng0, [out[f] for f in FIELDS]


def plume_objective(final, z_ash=3000.0, width=50.0, z_target=1000.0, r_scale=200.0):
    """Observable of the final state (18 x n tensor in FIELDS order): the
    ash mass above z_ash, sum m Y sigmoid((z - z_ash) / width), plus
    (z_R - z_target)^2 with z_R the height of the largest horizontal radius
    of the ash, a soft maximum: sum w z / sum w, w = m Y exp(r / r_scale),
    r = sqrt(x^2 + y^2).  Smooth versions of the sharp definitions, so that
    the gradient exists."""
    x, y, z, m, Y = final[0], final[1], final[2], final[9], final[14]
    ash = m * Y
    above = (ash * torch.sigmoid((z - z_ash) / width)).sum()
    r = torch.sqrt(x * x + y * y)
    w = ash * torch.exp((r - r.max().detach()) / r_scale)
    zR = (w * z).sum() / w.sum()
    return above + (zR - z_target) ** 2


def value_and_grad(theta, case, nsteps, every=25, **obj):
    """J(theta) and dJ/dtheta through PlumeSteps"""
    th = torch.as_tensor(theta, dtype=torch.float64).clone().requires_grad_(True)
    ng0, fields = vent_initial_state(th, case)
    final, _ = PlumeSteps.apply(ng0, *fields, case, nsteps, every)
    J = plume_objective(final, **obj)
    J.backward()
    return float(J.detach()), th.grad.numpy().copy()


def forward_value(theta, case, nsteps, **obj):
    """J(theta) from a plain forward run (no adjoint recording)"""
    th = torch.as_tensor(theta, dtype=torch.float64)
    ng0, fields = vent_initial_state(th, case)
    ps = case.particles.take(np.arange(case.particles.n))
    for f, t in zip(FIELDS, fields):
        getattr(ps, f)[:] = t.numpy()
    opt = copy.deepcopy(case.options)
    opt.ng0 = float(ng0)
    g, _, _, _, _ = eos_torch(opt, torch.from_numpy(ps.rho), torch.from_numpy(ps.Y),
                              torch.from_numpy(ps.e), float(ng0))
    ps.gamma[:] = g.numpy()
    sol = Solver(dataclasses.replace(case, options=opt, particles=ps))
    sol.steps(nsteps)
    fin = sol.download()
    sol.close()
    final = torch.from_numpy(np.stack([getattr(fin, f) for f in FIELDS]))
    return float(plume_objective(final, **obj))


def finite_difference(theta, case, nsteps, rel=1e-4, **obj):
    """central differences of forward_value, step rel * |theta_k|"""
    theta = np.asarray(theta, dtype=np.float64)
    g = np.zeros(3)
    for k in range(3):
        d = rel * abs(theta[k])
        tp, tm = theta.copy(), theta.copy()
        tp[k] += d
        tm[k] -= d
        g[k] = (forward_value(tp, case, nsteps, **obj) - forward_value(tm, case, nsteps, **obj)) / (2 * d)
    return g
