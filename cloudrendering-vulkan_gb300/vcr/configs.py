"""The five scene configurations the project is measured on, as vcr structs.

Cloud: seeded Perlin fBm (lacunarity 2, gain 0.5, base frequency 4 over the
longest axis) times an ellipsoidal falloff, clamped to [0, 1]; voxel size
1 / longest axis so the cloud spans one unit along it (x, y centred, z from
0, as SetCloudProperties lays it out, main.cpp:145-163).  sigma_t =
density_scaling * density (base_scaling 1).

Light: a sun at 30 deg elevation to the -x side (light travels +x and down,
as the reference default (1,-1,0) does); irradiance 1; constant sky 0.1.
Camera: pinhole at (0, 0, -0.4) looking +z at the cloud, vertical FOV 90 deg.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

from . import _abi
from . import cloud_from_grid, camera_look, fbm_desc, grid_desc, params_set_phase_g

SUN_ELEVATION_DEG = 30.0
SUN_AZIMUTH_DEG = 180.0  # toward the sun: -x (side lighting, like the reference default (1,-1,0))


def sun_travel_dir(elev_deg: float = SUN_ELEVATION_DEG, az_deg: float = SUN_AZIMUTH_DEG):
    """Unit direction the sunlight travels (from the sun into the scene)."""
    e, a = math.radians(elev_deg), math.radians(az_deg)
    to_sun = (math.cos(e) * math.cos(a), math.sin(e), math.cos(e) * math.sin(a))
    return tuple(-c for c in to_sun)


@dataclass
class Scene:
    name: str
    size: tuple
    octaves: int
    density_scaling: float
    width: int
    height: int
    passes: int
    spp: int = 1
    max_events: int = 64
    albedo: float = 0.99
    g: float = 0.857
    precision: int = _abi.PREC_FP32
    seed: int = 1
    extra: dict = field(default_factory=dict)

    def digest(self) -> str:
        """The first 16 hex digits of the SHA-256 of the scene's fields as
        canonical JSON: the same configuration hashes the same in every
        output that names it (pure Python; loads no library)."""
        import hashlib
        import json
        from dataclasses import asdict
        blob = json.dumps(asdict(self), sort_keys=True, separators=(",", ":"))
        return hashlib.sha256(blob.encode()).hexdigest()[:16]

    def grid_desc(self):
        n = max(self.size)
        return grid_desc(self.size, (1.0 / n,) * 3)

    def fbm(self):
        return fbm_desc(seed=self.seed, octaves=self.octaves)

    def cloud(self):
        c = cloud_from_grid(self.grid_desc(), 1.0, self.density_scaling)
        return c

    @staticmethod
    def camera_pose():
        """(position, forward, vertical FOV in degrees, near plane)."""
        return (0.0, 0.0, -0.4), (0.0, 0.0, 1.0), 90.0, 0.1

    def camera(self, width=None, height=None):
        pos, fwd, fov, near = self.camera_pose()
        return camera_look(pos, fwd, fov, near, width or self.width, height or self.height)

    def params(self, tracker=_abi.TRACKER_DDA):
        p = self.params_fields(tracker)
        params_set_phase_g(p, self.g)
        return p

    def params_fields(self, tracker=_abi.TRACKER_DDA):
        """The parameter struct without the phase function (set by
        params_set_phase_g): plain field values, no library call."""
        p = _abi.Params()
        p.max_events = self.max_events
        p.light_intensity = 1.0
        p.albedo = self.albedo
        sd = sun_travel_dir()
        for i in range(3):
            p.sun_dir[i] = sd[i]
            p.sky[i] = 0.1
        p.sky_mode = _abi.SKY_CONSTANT
        p.rng_mode = _abi.RNG_PCG
        p.nee_mode = _abi.NEE_RATIO
        p.tracker = tracker
        p.nrc_events = 0
        return p


C1_PT = Scene("C1-pt-128^3-512x512", (128, 128, 128), 6, 8.0, 512, 512, 256)
C2_PPM = Scene("C2-ppm-256^3-960x540", (256, 256, 256), 6, 16.0, 960, 540, 64,
               extra=dict(photons=1 << 20, r0=0.01, alpha=0.7))
C3_PPB = Scene("C3-ppb-256^3-1280x720", (256, 256, 256), 6, 16.0, 1280, 720, 32, extra=dict(beams=262144))
C4_BATCH = Scene("C4-batched-512^3-fp16", (512, 512, 512), 6, 16.0, 1024, 1024, 1, spp=4,
                 precision=_abi.PREC_FP16, extra=dict(views=64, suns=8))
C5_NRC = Scene("C5-nrc-1024x512x1024-fp16-1920x1080", (1024, 512, 1024), 8, 32.0, 1920, 1080, 1,
               precision=_abi.PREC_FP16, extra=dict(train_samples=65536, nrc_events=2))

ALL = [C1_PT, C2_PPM, C3_PPB, C4_BATCH, C5_NRC]

C4_ELEVATIONS = tuple(5.0 + 75.0 * i / 7.0 for i in range(8))  # 5 .. 80 deg


def c4_views(count=64, seed=1, fov_y_deg=60.0):
    """The batched configuration's views: square frames with sides drawn
    uniformly from [256, 1024] (numpy generator seeded `seed`); cameras on a
    ring around the cloud centre (0, 0, 0.5) at radius 1.4, 0.25 above its
    plane, looking at the centre; view v uses sun elevation index v mod 8
    (C4_ELEVATIONS) at the default azimuth.  Returns (camera, w, h, sun)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    sides = rng.integers(256, 1025, size=count)
    centre = np.array([0.0, 0.0, 0.5])
    out = []
    for v in range(count):
        a = 2.0 * math.pi * v / count
        pos = centre + np.array([1.4 * math.sin(a), 0.25, -1.4 * math.cos(a)])
        fwd = centre - pos
        fwd = fwd / np.linalg.norm(fwd)
        s = int(sides[v])
        cam = camera_look(tuple(pos), tuple(fwd), fov_y_deg, 0.1, s, s)
        out.append((cam, s, s, sun_travel_dir(C4_ELEVATIONS[v % 8])))
    return out


def setup_context(ctx, scene: Scene, tracker=_abi.TRACKER_DDA, precision=None, width=None, height=None):
    """Generate the scene's grid on the device and bind cloud, camera, params, frame."""
    ctx.grid_generate(scene.grid_desc(), scene.fbm(), scene.precision if precision is None else precision)
    ctx.set_cloud(scene.cloud())
    ctx.set_camera(scene.camera(width, height))
    ctx.set_params(scene.params(tracker))
    ctx.set_frame(width or scene.width, height or scene.height)
