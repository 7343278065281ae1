"""rayna_gb300 — GB300 (sm_103a) path-tracing library with rayna_engine's API.

The per-sample path-tracing hot path of rayna_engine (camera rays, BVH
traversal, sphere / triangle / SDF / medium intersection, material scatter,
radiance accumulation) runs as hand-written CUDA behind the C ABI of
include/rayna_gpu.h. This package is the host-side mirror of the reference's
scene, camera, options and Renderer types over that ABI.
"""
from .scene import (  # noqa: F401
    Angle, AxisBoxMesh, BvhMesh, Camera, CylinderMesh, DielectricMaterial, InfinitePlaneMesh, IsotropicMaterial,
    LambertianMaterial, ObjectTransform, ParallelogramMesh, Planar,
    LightMaterial, MetalMaterial, NoSkybox, ObjectList, RaymarchedIsosurfaceMesh, RenderMode, RenderOpts,
    Scene, SdfMandelbulb, SdfSphere, SdfTorus, SimpleObject, SimpleSkybox, SolidTexture, SphereMesh,
    StandardScene, Transform3, Triangle, UnsupportedVariant, VolumetricObject, WhiteSkybox, flatten,
    ColourSource, DynamicTexture, HdrImageSkybox, Image, ImageTexture, LocalNoiseTexture, Perlin, ScalePoint,
    UvCheckerTexture, UvNoiseTexture, WorldCheckerTexture, WorldNoiseTexture,
)
from .renderer import Render, Renderer, RenderStats  # noqa: F401
from ._abi import RaynaError, load_library  # noqa: F401
