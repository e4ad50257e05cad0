"""Fits the parameters of the multigrid V-cycle behind solver="mg" on
systems the plain pipeline itself generates.

A training case is a seeded 1-3 drop pair (synth.random_pair_scenes) solved
with flof.py's parameters (flof.py:913-915) by the multiscale driver: every
pyramid level and multistep contributes its own linear system, assembled
from that pair exactly as the plain solve assembles it.  The objective is
the number of preconditioned CG iterations all solves of all cases need to
reach the stop rule (the reference's, at the requested cgAccuracy), with the
wall time breaking ties.  The parameters are few (two damping factors, the
coarse Laplacian scale, the coarsest-level sweeps), so a coordinate search
over a grid of candidate values, repeated until no move improves the
objective, finds them; each evaluation is a handful of solves on the GPU.
Held-out cases check the fit.
"""
from __future__ import annotations

import time

from . import api, synth

GRID = {
    "omega0": (0.6, 0.7, 0.8, 0.85, 0.9, 0.95, 1.0),
    "omegac": (0.6, 0.7, 0.8, 0.85, 0.9, 0.95, 1.0),
    "lam": (0.35, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0),
    "coarse_sweeps": (8, 16, 24, 32, 48),
}
DEFAULT = {"omega0": 0.95, "omegac": 1.0, "lam": 0.9, "coarse_sweeps": 8}
START = {"omega0": 0.8, "omegac": 0.8, "lam": 0.5, "coarse_sweeps": 24}  # before the fit


def cases(n: int, dims=(32, 32, 32, 32), base_seed: int = 20000, ctx=None):
    """n training pairs (seeds base_seed + k) as device grids."""
    ctx = ctx or api.context()
    out = []
    for k in range(n):
        s0, s1 = synth.random_pair_scenes(base_seed + k)
        g0 = api.Grid4Real(dims=dims, ctx=ctx).from_numpy(synth.flow_input(s0, dims))
        g1 = api.Grid4Real(dims=dims, ctx=ctx).from_numpy(synth.flow_input(s1, dims))
        out.append((g0, g1))
    return out


def evaluate(ctx, data, params: dict, solve_params: dict):
    """(total preconditioned iterations, seconds, plain-finisher solves) of
    the cases' multiscale solves with the V-cycle parameters `params`."""
    ctx.set_mg_params(params["omega0"], params["omegac"], params["lam"], params["coarse_sweeps"])
    f0 = ctx.mg_fallbacks()
    iters = 0
    t = time.perf_counter()
    for g0, g1 in data:
        v = api.Grid4Vec4(dims=g0.dims, ctx=ctx)
        api.opticalFlowMultiscale4d(v, g0, g1, solver="mg", **solve_params)
        iters += sum(s[1] for s in api.last_solve_stats()["solves"])
    ctx.synchronize()
    return iters, time.perf_counter() - t, ctx.mg_fallbacks() - f0


def fit(ctx=None, train: int = 6, dims=(32, 32, 32, 32), cg_accuracy: float = 1e-4,
        start: dict | None = None, max_rounds: int = 3, log=None):
    """Coordinate search from `start` (START when None);
    returns (best parameters, history)."""
    ctx = ctx or api.context()
    sp = dict(wSmooth=0.001, wEnergy=0.0001, cgAccuracy=cg_accuracy, postVelBlur=4, cfl=999,
              multiStep=3, minGridSize=20, doFinalProject=False, resetBndWidth=0.1)
    data = cases(train, dims, ctx=ctx)
    best = dict(start or START)
    hist = []

    def score(p):
        it, sec, fb = evaluate(ctx, data, p, sp)
        hist.append((dict(p), it, sec, fb))
        if log:
            log(f"  {p} -> {it} iterations, {sec * 1e3:.1f} ms, {fb} plain finishes")
        return (it + 1000 * fb, sec)

    cur = score(best)
    for _ in range(max_rounds):
        moved = False
        for key, values in GRID.items():
            for v in values:
                if v == best[key]:
                    continue
                cand = dict(best, **{key: v})
                s = score(cand)
                # fewer iterations, or as many in clearly less time
                if s[0] < cur[0] or (s[0] == cur[0] and s[1] < 0.97 * cur[1]):
                    cur, best, moved = s, cand, True
        if not moved:
            break
    ctx.set_mg_params(best["omega0"], best["omegac"], best["lam"], best["coarse_sweeps"])
    return best, hist
