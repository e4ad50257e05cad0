"""Seeded synthetic 4D level-set inputs: falling drops over a liquid pool.

The reference builds its inputs with a FLIP liquid simulation
(scenes/dataGen2Drop.py:113-326) that is not part of the hot path; these
analytic stand-ins have the same structure: a 4D (x, y, z, t) grid of signed
distances in cells, negative inside the liquid, x fastest.

All lengths are defined on a 32-cell base domain and scaled to the target
resolution; time runs over the same fraction of the fall for any t extent.

  pool plane:  phi = y - y_pool,          y_pool = 6 + U(-1, 1)
  sphere:      phi = |p - c(t)| - r,      r = U(4, 6)  (or the given range)
  ellipsoid:   phi ~ (|(p - c)/a| - 1) * min(a), semi-axes a_i = U(4, 10)
  fall:        c_y(tau) = 24 - 0.5 * 0.05 * tau^2,  tau = t * 32 / T
  start (x,z): U(8, 24) each

The union is the minimum over components; the result is scaled to cells of
the target grid and clamped to [-4, 4].  Cell centres sit at index + 0.5, the
reference's sampling convention (source/util/vector4d.h:423).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BASE = 32.0
GRAVITY = 0.05
LS_FACTOR = np.float32(-0.1 / 20.0)  # scenes/flof.py:319


@dataclass
class Drop:
    x0: float
    z0: float
    y0: float
    radius: float = 5.0
    axes: tuple | None = None  # semi-axes for an ellipsoid drop


@dataclass
class Scene:
    pool: float
    drops: list = field(default_factory=list)


def make_scene(seed: int, kind: str = "sphere", ndrops: int = 1,
               radius_range=(4.0, 6.0), axes_range=(4.0, 10.0)) -> Scene:
    """Draw one data set's geometry from numpy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    pool = 6.0 + rng.uniform(-1.0, 1.0)
    drops = []
    for _ in range(ndrops):
        if kind == "ellipsoid":
            axes = tuple(float(a) for a in rng.uniform(axes_range[0], axes_range[1], size=3))
            x0 = rng.uniform(8.0, 24.0)
            z0 = rng.uniform(8.0, 24.0)
            drops.append(Drop(x0=float(x0), z0=float(z0), y0=24.0, radius=min(axes), axes=axes))
        else:
            r = rng.uniform(radius_range[0], radius_range[1])
            x0 = rng.uniform(8.0, 24.0)
            z0 = rng.uniform(8.0, 24.0)
            drops.append(Drop(x0=float(x0), z0=float(z0), y0=24.0, radius=float(r)))
    return Scene(pool=float(pool), drops=drops)


def scene_for(data_id: int) -> Scene:
    """Data sets 0 and 1 are sphere drops (seeds 1 and 2); data set 2 is an
    elongated ellipsoid drop (seed 3)."""
    if data_id == 2:
        return make_scene(3, kind="ellipsoid")
    return make_scene(data_id + 1, kind="sphere")


def sdf_slice(scene: Scene, res: tuple, t: int, T: int, clamp: float = 4.0,
              out: np.ndarray | None = None) -> np.ndarray:
    """Signed distance of time step t of T on an (X, Y, Z) grid, returned as
    a float32 (Z, Y, X) array in target-grid cells."""
    X, Y, Z = res
    s = X / BASE
    tau = t * BASE / T
    xs = ((np.arange(X, dtype=np.float64) + 0.5) / s)[None, None, :]
    ys = ((np.arange(Y, dtype=np.float64) + 0.5) / s)[None, :, None]
    zs = ((np.arange(Z, dtype=np.float64) + 0.5) / s)[:, None, None]
    phi = np.broadcast_to(ys - scene.pool, (Z, Y, X)).copy()
    for d in scene.drops:
        cy = d.y0 - 0.5 * GRAVITY * tau * tau
        dx, dy, dz = xs - d.x0, ys - cy, zs - d.z0
        if d.axes is None:
            ph = np.sqrt(dx * dx + dy * dy + dz * dz) - d.radius
        else:
            a, b, c = d.axes
            k0 = np.sqrt((dx / a) ** 2 + (dy / b) ** 2 + (dz / c) ** 2)
            ph = (k0 - 1.0) * min(d.axes)
        np.minimum(phi, ph, out=phi)
    phi *= s
    np.clip(phi, -clamp, clamp, out=phi)
    if out is None:
        return phi.astype(np.float32)
    out[...] = phi
    return out


def sdf4d(scene: Scene, dims: tuple, clamp: float = 4.0) -> np.ndarray:
    """Full 4D SDF of size dims = (X, Y, Z, T) as a float32 (T, Z, Y, X) array."""
    X, Y, Z, T = dims
    out = np.empty((T, Z, Y, X), dtype=np.float32)
    for t in range(T):
        sdf_slice(scene, (X, Y, Z), t, T, clamp, out=out[t])
    return out


def flow_input(scene: Scene, dims: tuple) -> np.ndarray:
    """The solver's input: lsFactor * SDF (scenes/flof.py:319, :520)."""
    return (sdf4d(scene, dims) * LS_FACTOR).astype(np.float32)


def random_pair_scenes(seed: int, ndrops_range=(1, 3), radius_range=(3.0, 8.0)):
    """Two independent multi-drop scenes for batched / training pairs."""
    rng = np.random.default_rng(seed)
    n0 = int(rng.integers(ndrops_range[0], ndrops_range[1] + 1))
    n1 = int(rng.integers(ndrops_range[0], ndrops_range[1] + 1))
    kinds = ["sphere", "ellipsoid"]
    k0 = kinds[int(rng.integers(0, 2))]
    k1 = kinds[int(rng.integers(0, 2))]
    s0 = make_scene(int(rng.integers(1 << 30)), kind=k0, ndrops=n0, radius_range=radius_range,
                    axes_range=radius_range)
    s1 = make_scene(int(rng.integers(1 << 30)), kind=k1, ndrops=n1, radius_range=radius_range,
                    axes_range=radius_range)
    return s0, s1


BATCH_SIZES = (24, 32, 40, 48, 64)
BATCH_T = (16, 32, 48)


def batch_pairs(n: int = 64, base_seed: int = 1000):
    """n deformation pairs of uneven sizes: spatial resolution from
    BATCH_SIZES and t extent from BATCH_T, 1-3 drops of radius U(3, 8) per
    data set; pair k draws from seed base_seed + k.  Returns a list of
    (dims, scene0, scene1) with dims = (S, S, S, T)."""
    out = []
    for k in range(n):
        rng = np.random.default_rng(base_seed + k)
        S = int(BATCH_SIZES[int(rng.integers(0, len(BATCH_SIZES)))])
        T = int(BATCH_T[int(rng.integers(0, len(BATCH_T)))])
        s0, s1 = random_pair_scenes(base_seed + k)
        out.append(((S, S, S, T), s0, s1))
    return out
