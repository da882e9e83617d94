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
  heavy_2160p       1024 x 1024 UV-grid sphere (r 2) displaced by Perlin
                    noise of amplitude 0.3 + ground; 8 spot lights, 4096^2
                    maps, camera 3840 x 2160.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

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
    mp = MapParams(map_size, map_size, bias_mode=api.GI_BIAS_POLYGON_OFFSET)
    p = ShadowParams.defaults(technique)
    p.light_radius = 0.25
    p.pcss_min_blocker_depth = 0.0
    return Workload("heavy_2160p", s, light, camera, mp, p, lights=eyes)
