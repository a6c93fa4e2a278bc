"""PathTracer render-pass interface of the reference, on top of libxr.

Mirrors src/pathTracer.h:12-57 / src/pathTracer.cpp:35-201 for headless use:
PostTracerInit(scenes) uploads a scene and builds its BVH (LoadCurrentScene +
CreateAccelerationStructures), DrawFrame() advances the frame counter modulo
10000 (pathTracer.cpp:135) and renders, GetUniformBufferObject() builds the UBO
with the previous frame's matrices (pathTracer.cpp:169-201).  The camera is
scripted (position/yaw/pitch) instead of the interactive fly camera.
"""
from __future__ import annotations

from dataclasses import dataclass, field

from . import _lib as L
from .api import Renderer, Scene, camera_ubo, params_default, params_reference


@dataclass
class UserSettings:
    """src/Editor/UserSettings.h:5-30 (fields the ReSTIR GI mode reads) + the reuse knobs."""
    scene_index: int = 0
    enable_sky_lighting: bool = False
    enable_reuse: bool = True
    number_of_bounces: int = 4
    fov: float = 45.0
    compat_reference: bool = False
    temporal_on: bool = True
    spatial_on: bool = True
    m_cap_temporal: int = 20
    m_cap_spatial: int = 120
    n_neighbours: int = 5
    radius_px: float = 30.0
    visibility: bool = True
    seed: int = 1


@dataclass
class PathTracer:
    settings: UserSettings
    width: int
    height: int
    device: int = 0
    scenes: list = field(default_factory=list)

    def __post_init__(self):
        self.renderer = Renderer(self.width, self.height, self.device)
        self.current_frame_total = 0
        self.camera = L.XrCamera()
        self._prev_ubo = None
        self._apply_settings()

    def _apply_settings(self) -> None:
        s = self.settings
        if s.compat_reference:
            p = params_reference(self.width, self.height)
        else:
            p = params_default(self.width, self.height, temporal_on=int(s.temporal_on), spatial_on=int(s.spatial_on),
                               m_cap_temporal=s.m_cap_temporal, m_cap_spatial=s.m_cap_spatial,
                               n_neighbours=s.n_neighbours, radius_px=s.radius_px, visibility=int(s.visibility),
                               seed=s.seed)
        self.renderer.set_params(p)

    # pathTracer.cpp:35-41
    def PostTracerInit(self, scene_list: list[Scene]) -> None:
        self.scenes = list(scene_list)
        self.LoadCurrentScene(self.settings.scene_index)

    # pathTracer.cpp:162-167 + ApplicationRT.cpp:55-66
    def LoadCurrentScene(self, index: int) -> None:
        sc = self.scenes[index]
        self.renderer.upload_scene(sc)
        self.renderer.build_bvh()
        self.camera = L.XrCamera.from_buffer_copy(sc.camera)
        self.camera.fov_deg = self.settings.fov
        self._prev_ubo = None

    # pathTracer.cpp:169-201
    def GetUniformBufferObject(self) -> L.XrUniformBufferObject:
        u = camera_ubo(self.camera, self.width, self.height, self._prev_ubo, self.current_frame_total,
                       self.settings.number_of_bounces, self.settings.enable_sky_lighting, self.settings.enable_reuse)
        self._prev_ubo = u
        return u

    # pathTracer.cpp:57-81 (frame counter) + ApplicationReSTIRGI::Render
    def DrawFrame(self) -> None:
        self.current_frame_total = (self.current_frame_total + 1) % 10000
        self.Render(self.GetUniformBufferObject())

    def Render(self, ubo: L.XrUniformBufferObject) -> None:
        self.renderer.render(ubo)

    def close(self) -> None:
        self.renderer.close()
