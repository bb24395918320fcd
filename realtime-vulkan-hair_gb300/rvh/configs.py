"""Seeded synthetic workloads (all inputs generated here; no external data).

  plain_small   1 head (sphere r=1 at the origin), 1,024 strands x 16 points,
                length 0.5, uniform roots on the upper hemisphere, no grid,
                DFTL damping 0.9, wind 2 sin(0.5 t) x, a sphere r=0.3 orbiting
                at radius 1.2 (omega 0.5 rad/s) at y=0; 120 steps of dt=1/60.
  full_head     100,000 strands x 32 points, Poisson-disk roots, lengths
                U(0.4,0.8), 4 ellipsoids (axes U(0.2,0.5)), 64^3 grid over the
                hair bounds, friction 0.05, repulsion 0.02, wind + gusts (0.5).
  batched       256 heads: strands log-uniform in [512, 65536], points in
                {8,16,24,32}, lengths U(0.2,1.0), grids 32^3..64^3, 0-4 ellipsoids.
  served        1,000 resident characters sized as `batched`.
  adjoint       4,096 strands x 32 points, 60 steps, no grid.
The head sphere is collider 0 in every workload (the reference makes
colliders[0] a sphere, compute.comp:160-169), so hair rests on the head.

`gen` (optional, every builder): where the inputs come from, an object with
generate_head(**desc) and wind_at(desc, step, t) -- rvh.api (the library,
the default) or any other statement of include/rvh_scene.h with the same
results.
"""
import math

import numpy as np

from . import api
from . import types as T

DT = np.float32(1.0 / 60.0)


class AssetSpec:
    def __init__(self, records, rest, params, colliders, n_points, orbit=None, strand_wind=None, wind=None,
                 gen=None):
        self.records = records
        self.rest = rest
        self.params = params
        self.colliders = colliders
        self.n_points = n_points
        self.orbit = orbit            # optional api.Orbit appended as the last collider each frame
        self.strand_wind = strand_wind
        self.wind = wind              # api.WindDesc
        self.gen = api if gen is None else gen

    @property
    def n_strands(self):
        return self.records.shape[0]

    @property
    def n_total_points(self):
        return self.records.shape[0] * self.n_points

    def time(self, step):
        """totalTime of frame `step` (0-based): Scene::UpdateTime adds dt before the dispatch."""
        return float(np.float32((step + 1) * DT))

    def frame(self, step):
        t = self.time(step)
        w = self.gen.wind_at(self.wind, step, t) if self.wind is not None else (0.0, 0.0, 0.0)
        return T.frame(DT, t, w)

    def colliders_at(self, step):
        cols = list(self.colliders)
        if self.orbit is not None:
            cols.append(api.sphere_on_orbit(self.orbit, self.time(step)))
        return cols


def _wind(seed, gust):
    w = T.WindDesc()
    w.amplitude = 2.0
    w.omega = 0.5
    w.dir[:] = (1.0, 0.0, 0.0)
    w.gust_sigma = gust
    w.seed = seed
    return w


def plain_small(n_strands=1024, n_points=16, seed=0):
    rec, rest, p, cols = api.generate_head(seed=seed, n_strands=n_strands, n_points=n_points,
                                           root_sampling=0, sort_roots=1, length_min=0.5, length_max=0.5,
                                           head_collider=1, n_ellipsoids=0, grid_res=0, friction=0.0,
                                           repulsion=0.0, dftl_damping=0.9)
    orbit = api.Orbit()
    orbit.center[:] = (0.0, 0.0, 0.0)
    orbit.orbit_radius = 1.2
    orbit.omega = 0.5
    orbit.phase = 0.0
    orbit.sphere_radius = 0.3
    return AssetSpec(rec, rest, p, cols, n_points, orbit=orbit, wind=_wind(seed, 0.0))


def full_head(n_strands=100000, n_points=32, seed=1, grid_res=64):
    rec, rest, p, cols = api.generate_head(seed=seed, n_strands=n_strands, n_points=n_points,
                                           root_sampling=1, sort_roots=1, length_min=0.4, length_max=0.8,
                                           head_collider=1, n_ellipsoids=4, axis_min=0.2, axis_max=0.5,
                                           grid_res=grid_res, friction=0.05, repulsion=0.02, dftl_damping=0.9)
    return AssetSpec(rec, rest, p, cols, n_points, wind=_wind(seed, 0.5))


def batched_sizes(n_assets=256, seed=2, smin=512, smax=65536):
    """(n_strands, n_points, grid_res, n_ellipsoids) per asset, seeded."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_assets):
        ns = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax)))))
        n = int(rng.choice([8, 16, 24, 32]))
        res = int(rng.integers(32, 65))
        ne = int(rng.integers(0, 5))
        out.append((ns, n, res, ne))
    return out


def batched(n_assets=256, seed=2, scale=1.0, smin=512, smax=65536, gen=None, indices=None):
    """`scale` shrinks every asset's strand count (parity tests use small batches);
    `indices` builds only those assets of the workload, in that order."""
    gen = api if gen is None else gen
    sizes = batched_sizes(n_assets, seed, smin, smax)
    specs = []
    for i in (range(n_assets) if indices is None else indices):
        ns, n, res, ne = sizes[i]
        ns = max(1, int(ns * scale))
        rec, rest, p, cols = gen.generate_head(seed=seed * 100003 + i, n_strands=ns, n_points=n,
                                               root_sampling=0, sort_roots=1, length_min=0.2, length_max=1.0,
                                               head_collider=1, n_ellipsoids=ne, axis_min=0.2, axis_max=0.5,
                                               grid_res=res, friction=0.05, repulsion=0.02, dftl_damping=0.9)
        specs.append(AssetSpec(rec, rest, p, cols, n, wind=_wind(seed * 7919 + i, 0.5), gen=gen))
    return specs


def adjoint_case(n_strands=4096, n_points=32, seed=4, n_ellipsoids=2, max_root_height=0.85):
    """Roots above `max_root_height` (near the crown, where a strand starts
    pointing straight up like an inverted pendulum) are skipped: there the
    loss is so nonlinear that central differences at h = 1e-4 do not converge."""
    rec, rest, p, cols = api.generate_head(seed=seed, n_strands=2 * n_strands, n_points=n_points,
                                           root_sampling=0, sort_roots=1, length_min=0.4, length_max=0.8,
                                           head_collider=1, n_ellipsoids=n_ellipsoids, axis_min=0.2,
                                           axis_max=0.5, grid_res=0, friction=0.0, repulsion=0.0,
                                           dftl_damping=0.9)
    keep = np.nonzero(rec[:, 0, 1] < max_root_height)[0][:n_strands]
    rec, rest = np.ascontiguousarray(rec[keep]), np.ascontiguousarray(rest[keep])
    n_strands = rec.shape[0]
    rng = np.random.default_rng(seed)
    tips = rec[:, n_points - 1, :3].astype(np.float64)
    targets = tips + rng.normal(0.0, 0.05, size=tips.shape)
    wind = rng.normal(0.0, 0.5, size=(n_strands, 3)).astype(np.float32)
    v0 = rng.normal(0.0, 0.1, size=(n_strands, n_points, 3)).astype(np.float32)
    v0[:, 0, :] = 0.0
    rec[:, n_points:2 * n_points, :3] = v0
    spec = AssetSpec(rec, rest, p, cols, n_points, strand_wind=wind, wind=_wind(seed, 0.0))
    return spec, targets
