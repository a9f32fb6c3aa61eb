"""voidray_gb300 — GB300 (sm_103a) wavefront path-tracing backend for voidray.

The compute path is the native library ``_lib/libvoidray_gb300.so`` (C ABI in
``include/voidray_gpu.h``); this package mirrors voidray_renderer's scene,
camera, material and settings API on top of it.
"""
from ._native import EXPORTED, VR_MISS, VoidrayError, lib
from .renderer import Checkpoint, Renderer, RenderAction, RendererStats
from .scene import (AnalyticSurface, ImageTexture, SampleType, Camera, ColorManagementSettings, CpuRenderTarget, Environment, Environments, Estimator, Material,
                    Materials, Mesh, MicrofacetBSDF, RenderMode, RenderSettings, Scene, SceneAcceleration, Settings,
                    Surfaces, Tonemap, LegacyTonemap, Vertex, degrees_to_radians, hex_color, iterative_render, render_device,
                    tonemap, tonemap_legacy)

__all__ = [
    "EXPORTED", "VR_MISS", "VoidrayError", "lib", "AnalyticSurface", "ImageTexture", "SampleType", "Camera", "ColorManagementSettings", "CpuRenderTarget",
    "Environment", "Environments", "Estimator", "Material", "Materials", "Mesh", "MicrofacetBSDF", "RenderMode",
    "RenderSettings", "Scene", "SceneAcceleration", "Settings", "Surfaces", "Tonemap", "Vertex",
    "degrees_to_radians", "hex_color", "iterative_render", "render_device", "tonemap", "Renderer", "RenderAction",
    "RendererStats", "Checkpoint", "LegacyTonemap", "tonemap_legacy",
]
