"""Synthetic scenes of the benchmark workloads (seeded, deterministic).

The reference measures no public dataset; these procedural scenes stand in
for its Configs/ scenes at the sizes the workloads name.  Seeds are
0x5EED0000 + workload index.  Each builder returns a Workload with the
scene, the light and camera views, the light-map parameters and the
visibility parameters.

  hard_pcf_1024     ground quad 20 x 20 at y = 0 + UV sphere 64 x 32 (r 1,
                    centre (0, 1.2, 0)); spot light at (4, 8, 4) aimed at the
                    origin, 60 deg; 1024^2 FP32 map with constant bias 1e-3;
                    camera 1024 x 768; 3 x 3 PCF.
  pcss_1080p        ground + 64 icospheres (subdivision 3, 1,280 triangles
                    each: 81,922 triangles); centres U([-8,8] x [0.2,3] x
                    [-8,8]), radii U[0.2, 1]; square area light of side 0.5
                    at (0, 12, 0) aimed down (90 deg frustum so the whole
                    ground is inside the map); 2048^2 map with the
                    reference's polygon offset (4, 20); camera 1920 x 1080;
                    PCSS with 16 Poisson blocker taps and 32 filter taps.
  batched_720p      256 scenes (seed base + 2): ground + an icosphere field
                    whose triangle count is log-uniform in [1k, 500k]; 1-8
                    spot lights (60 deg) at uniform points of the upper
                    hemisphere of radius 10 (elevation >= 15 deg) aimed at
                    the origin, each with a map side drawn from {512, 1024,
                    2048, 4096}; camera 1280 x 720 on a circle of radius 15,
                    height 8; 5 x 5 PCF, polygon offset (4, 20).
  pcss_1080p_batch  16 pcss_1080p frames of different seeded sphere fields
                    (seed base + 1 + 16 k), same light, camera and PCSS:
                    the frames the batched and surrogate paths are measured
                    on against the plain single-frame pass.
  heavy_2160p       1024 x 1024 UV-grid sphere (r 2) displaced by Perlin
                    noise of amplitude 0.3 + ground; 8 spot lights, 4096^2
                    maps, camera 3840 x 2160.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _capi as api
from .shadow import MapParams, Scene, ShadowParams, ViewSpec

SEED_BASE = 0x5EED0000


@dataclass
class Workload:
    name: str
    scene: Scene
    light: ViewSpec
    camera: ViewSpec
    map_params: MapParams
    params: ShadowParams
    lights: list | None = None  # extra light eyes for multi-light workloads


def hard_pcf_1024(width: int = 1024, height: int = 768, map_size: int = 1024) -> Workload:
    s = Scene()
    s.ground(10.0, 0.0)
    s.uv_sphere(64, 32, 1.0, (0.0, 1.2, 0.0))
    light = ViewSpec(eye=(4.0, 8.0, 4.0), at=(0.0, 0.0, 0.0), width=map_size, height=map_size, fovy_deg=60.0)
    camera = ViewSpec(eye=(0.0, 6.0, -9.0), at=(0.0, 0.6, 0.0), width=width, height=height)
    mp = MapParams(map_size, map_size, bias_mode=api.GI_BIAS_CONSTANT, constant_bias=1e-3)
    p = ShadowParams.defaults(api.GI_TECH_PCF)
    p.kernel_order = 3
    return Workload("hard_pcf_1024", s, light, camera, mp, p)


def pcss_1080p(width: int = 1920, height: int = 1080, map_size: int = 2048, spheres: int = 64,
               technique: int = api.GI_TECH_PCSS_POISSON) -> Workload:
    s = Scene()
    s.ground(10.0, 0.0)
    s.icosphere_field(spheres, 3, (-8.0, 0.2, -8.0), (8.0, 3.0, 8.0), 0.2, 1.0, SEED_BASE + 1)
    light = ViewSpec(eye=(0.0, 12.0, 0.0), at=(0.0, 0.0, 0.0), width=map_size, height=map_size, fovy_deg=90.0)
    camera = ViewSpec(eye=(0.0, 14.0, -20.0), at=(0.0, 0.0, 0.0), width=width, height=height)
    mp = MapParams(map_size, map_size, bias_mode=api.GI_BIAS_POLYGON_OFFSET, offset_factor=4.0,
                   offset_units=20.0)
    p = ShadowParams.defaults(technique)
    p.light_radius = 0.25  # square light of side 0.5
    # With near 1 / far 1000 every blocker depth of this scene is about 0.9,
    # below the reference's 0.99 cut-off, so PCSS would return 1 everywhere;
    # the cut-off is disabled for this workload.
    p.pcss_min_blocker_depth = 0.0
    return Workload("pcss_1080p", s, light, camera, mp, p)


def heavy_2160p(width: int = 3840, height: int = 2160, map_size: int = 4096, grid: int = 1024,
                lights: int = 8, technique: int = api.GI_TECH_PCSS_POISSON) -> Workload:
    s = Scene()
    s.ground(10.0, 0.0)
    s.displaced_sphere(grid, grid, 2.0, 0.3, (0.0, 2.6, 0.0), SEED_BASE + 4)
    eyes = []
    for k in range(lights):
        a = 2.0 * math.pi * k / lights
        eyes.append((10.0 * math.cos(a) * 0.7, 10.0 * 0.7, 10.0 * math.sin(a) * 0.7))
    light = ViewSpec(eye=eyes[0], at=(0.0, 0.0, 0.0), width=map_size, height=map_size, fovy_deg=90.0)
    camera = ViewSpec(eye=(0.0, 9.0, -14.0), at=(0.0, 1.5, 0.0), width=width, height=height)
    mp = MapParams(map_size, map_size, bias_mode=api.GI_BIAS_POLYGON_OFFSET, offset_factor=4.0,
                   offset_units=20.0)
    p = ShadowParams.defaults(technique)
    p.light_radius = 0.25
    p.pcss_min_blocker_depth = 0.0
    return Workload("heavy_2160p", s, light, camera, mp, p, lights=eyes)


@dataclass
class BatchFrame:
    scene: Scene
    camera: ViewSpec
    lights: list = field(default_factory=list)
    maps: list = field(default_factory=list)
    params: ShadowParams | None = None
    triangles: int = 0


def batched_720p(scenes: int = 256, width: int = 1280, height: int = 720, tri_min: int = 1000,
                 tri_max: int = 500_000, map_sides=(512, 1024, 2048, 4096), max_lights: int = 8,
                 seed: int = SEED_BASE + 2) -> list[BatchFrame]:
    """The batched workload: `scenes` seeded scenes of varied size and light count."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(scenes):
        target = math.exp(rng.uniform(math.log(tri_min), math.log(tri_max)))
        level = int(min(6, max(0, round(math.log(target / (20 * 24), 4)))))
        count = max(1, int(round(target / (20 * 4 ** level))))
        s = Scene()
        s.ground(10.0, 0.0)
        s.icosphere_field(count, level, (-6.0, 0.2, -6.0), (6.0, 2.5, 6.0), 0.2, 0.8, seed * 1000 + k)
        az = rng.uniform(0.0, 2.0 * math.pi)
        camera = ViewSpec(eye=(15.0 * math.cos(az), 8.0, 15.0 * math.sin(az)), at=(0.0, 0.5, 0.0),
                          width=width, height=height, up=(0.0, 1.0, 0.0))
        lights, maps = [], []
        for _ in range(int(rng.integers(1, max_lights + 1))):
            phi = rng.uniform(0.0, 2.0 * math.pi)
            # uniform over the area of the hemisphere cap above 15 deg elevation
            cos_p = rng.uniform(math.sin(math.radians(15.0)), 1.0)
            y = 10.0 * cos_p
            r = 10.0 * math.sqrt(1.0 - cos_p * cos_p)
            side = int(rng.choice(map_sides))
            lights.append(ViewSpec(eye=(r * math.cos(phi), y, r * math.sin(phi)), at=(0.0, 0.0, 0.0),
                                   width=side, height=side, fovy_deg=60.0, up=(0.0, 1.0, 0.0)))
            maps.append(MapParams(side, side, bias_mode=api.GI_BIAS_POLYGON_OFFSET, offset_factor=4.0,
                                  offset_units=20.0))
        p = ShadowParams.defaults(api.GI_TECH_PCF)
        p.kernel_order = 5
        out.append(BatchFrame(s, camera, lights, maps, p, int(s.info().num_triangles)))
    return out


def pcss_1080p_batch(frames: int = 16, width: int = 1920, height: int = 1080, map_size: int = 2048,
                     spheres: int = 64) -> list[BatchFrame]:
    """pcss_1080p frames of `frames` different seeded sphere fields (one light each)."""
    out = []
    for k in range(frames):
        w = pcss_1080p(width, height, map_size, spheres)
        if k:
            s = Scene()
            s.ground(10.0, 0.0)
            s.icosphere_field(spheres, 3, (-8.0, 0.2, -8.0), (8.0, 3.0, 8.0), 0.2, 1.0, SEED_BASE + 1 + 16 * k)
            w.scene.close()
            w.scene = s
        out.append(BatchFrame(w.scene, w.camera, [w.light], [w.map_params], w.params,
                              int(w.scene.info().num_triangles)))
    return out
