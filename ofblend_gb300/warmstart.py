"""Training data and training loop of the learned warm start.

A sample is (i0c, i1c, target) on the coarsest grid of the multiscale solve:
the two inputs restricted level by level as opticalFlowMultiscaleTemplate
does (optflow4d.cpp:976-997: interpolGridTempl to half size), and the plain
solver's final deformation restricted the same way and halved per level
(velocities are in cells of each level's grid).  Everything stays on the GPU.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf

import numpy as np

from . import api, synth


def coarsen(grid, res: int, vec: bool):
    """Restrict a cubic 4D grid level by level (half size each) to res^4;
    Vec4 grids are halved in magnitude at every level."""
    g = grid
    while g.dims[0] > res:
        d = tuple(x // 2 for x in g.dims)
        h = (api.Grid4Vec4 if vec else api.Grid4Real)(dims=d, ctx=grid.ctx)
        (api.interpolateGrid4dVec if vec else api.interpolateGrid4d)(h, g)
        if vec:
            h.multConst(0.5)
        g = h
    return g


def _pair_inputs(seed: int, dims):
    s0, s1 = synth.random_pair_scenes(seed)
    return synth.flow_input(s0, dims), synth.flow_input(s1, dims)


def make_samples(n: int, dims=(32, 32, 32, 32), res: int = 16, base_seed: int = 10000,
                 solve_params: dict | None = None, ctx=None, workers: int | None = None):
    """n training samples from seeded 1-3 drop pairs (seeds base_seed + k):
    the plain solver computes each deformation, which is then coarsened.
    The host synthesises the input SDFs of the next pairs on `workers`
    threads while the GPU solves the current one (the library's calls
    release the interpreter lock); the samples are the same as a sequential
    run's.  The synthesis works on 32^3 slices and scales little past two
    threads."""
    ctx = ctx or api.context()
    sp = dict(solve_params or {})
    workers = workers or 2
    ahead = 2 * workers
    out = []
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        pending = collections.deque(ex.submit(_pair_inputs, base_seed + k, dims)
                                    for k in range(min(n, ahead)))
        for k in range(n):
            a0, a1 = pending.popleft().result()
            if k + ahead < n:
                pending.append(ex.submit(_pair_inputs, base_seed + k + ahead, dims))
            g0 = api.Grid4Real(dims=dims, ctx=ctx).from_numpy(a0)
            g1 = api.Grid4Real(dims=dims, ctx=ctx).from_numpy(a1)
            v = api.Grid4Vec4(dims=dims, ctx=ctx)
            api.opticalFlowMultiscale4d(v, g0, g1, **sp)
            out.append((coarsen(g0, res, False), coarsen(g1, res, False), coarsen(v, res, True)))
    return out


def train(model, samples, epochs: int = 10, batch: int = 8, lr: float = 1e-3, seed: int = 0,
          log=None):
    """Adam over shuffled mini-batches; returns the mean loss of each epoch."""
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(len(samples))
        tot, nb = 0.0, 0
        for b0 in range(0, len(order), batch):
            bs = [samples[i] for i in order[b0:b0 + batch]]
            tot += model.train_step(bs, lr)
            nb += 1
        hist.append(tot / max(nb, 1))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.5f}")
    return hist
