"""GB300-native shadow-visibility engine (sm_103a CUDA behind a C ABI).

Covers the shadow-visibility path of MarcioCerqueira/GlobalIllumination:
light-view depth maps, the G-buffer, per-pixel visibility (hard test, PCF,
PCSS, RBSM family) and shadow-volume stencil counts.  See shadow.py for the
technique interface and include/gi_shadow.h for the C ABI.
"""
from . import _capi
from ._capi import GIError
from .shadow import (Batch, Context, debug_fail_allocation, area_light_adaptive, area_light_samples, area_light_visibility, edt_inputs, edt_mean_filter, edt_soft_shadows,
                     pba_chain_rows, pba_voronoi, phong_shade, Frame, FrameBuffers, MapParams, Scene, ShadowParams, TECHNIQUES, ViewSpec,
                     allocate_frame, compute_hard_shadows, compute_visibility, frame_setup, hierarchical_shadow_map, light_map_minmax,
                     poisson_table, render_frame, render_frame_passes, render_gbuffer, render_shadow_map,
                     render_soft_shadows, shadow_volume_counts, shadow_volume_counts_silhouette, shadow_volume_geometry, soft_moment_map)

__all__ = [
    "Batch", "Context", "Frame", "debug_fail_allocation", "area_light_adaptive", "area_light_samples", "area_light_visibility", "edt_inputs", "edt_mean_filter", "edt_soft_shadows", "pba_chain_rows", "pba_voronoi", "phong_shade", "FrameBuffers", "GIError", "MapParams", "Scene", "ShadowParams", "TECHNIQUES",
    "ViewSpec", "allocate_frame", "compute_hard_shadows", "compute_visibility", "frame_setup",
    "poisson_table", "render_frame", "render_frame_passes", "render_gbuffer", "render_shadow_map", "render_soft_shadows",
    "shadow_volume_counts", "shadow_volume_counts_silhouette", "shadow_volume_geometry", "soft_moment_map", "hierarchical_shadow_map", "light_map_minmax", "_capi",
]
