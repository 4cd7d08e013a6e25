"""caustic: GB300 (sm_103a) drop-in for the caustic-tracer CPU path tracer.

Mirrors the reference's module surface (src/tracer/index.ts:5-20): scene
model, Rng, packScene, camera, renderImage/accumulatePass and the ray
queries, with the hot path in libcaustic_gb300.so (CUDA). Names follow the
reference in snake_case.
"""
from .camera import CameraFrame, camera_at, camera_frame, camera_position, generate_ray
from .pack import PackedScene, pack_scene
from .rng import Rng, pcg_hash, seed_for
from .scene import (CameraSettings, CheckerTexture, Dielectric, Emissive, Lambertian, Mesh, Metal, Quad,
                    Scene, SceneObject, SkyGradient, SkyNone, Sphere, Triangle, material_emission,
                    primitive_count, quad_triangles, triangle_area, triangle_normal)
from .scenes import (CORNELL_BOX, batch_scene, batch_workload, caustic_scene, cornell_box, cornell_unit_box,
                     furnace_scene, random_test_scene, soup_rays, triangle_soup)
from .batch import BatchRenderer, Job
from .tonemap import decode_ppm, encode_ppm, ppm_device, tonemap_buffer, tonemap_device
from .tracer import (DEFAULT_TRACE_OPTIONS, T_MIN, DeviceScene, Hits, PickResult, RenderOptions, TraceOptions,
                     accumulate_pass, intersect_closest, make_rays, occluded, pick, pick_many, render_image,
                     set_traversal)
from .serve import RenderServer, Request
from ._native import CausticError, NativeLibraryError
