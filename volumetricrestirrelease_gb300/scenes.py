"""Synthetic scenes for the workloads of this path.

The reference renders GVDB (.vbx) clouds that are not available here; these procedural scenes
stand in for them with the shapes, sizes and value ranges of the benchmark configurations:

  small  : 128^3 dense fBm (4 octaves, seed 1, lacunarity 2, gain 0.5) x smooth sphere mask
           r = 0.45 in the unit box, sigma_t 20/unit, albedo 0.9, g = 0; one point light
           (intensity 50) at (2,2,2) + constant white environment 0.2; camera (0,0,-2.5),
           45 deg FOV, 256x256; max path length 2, 8 candidates, temporal + 3 spatial
           neighbours (radius 10), static camera.
  full   : 512^3 sparse fBm (6 octaves) thresholded at 0.35 and remapped to [0,1] in 8^3
           bricks, 4-level conservative pyramid; sigma_t 40, albedo 0.95, g = 0.6; 16 point
           lights on a sphere of radius 3 (intensity 10) + procedural 512x256 sky; 1920x1080;
           max path length 3, 32 candidates, temporal + 3 spatial neighbours; the camera
           orbits 0.5 deg per frame.
  small_fp16 : `small` with FP16 bricks.
  batch  : 32 independent instances: resolutions drawn from {256^2, 512^2, 960x540, 1280x720,
           1920x1080}, sparse fBm grids of 128^3..512^3 (seeded per instance), 8 of them fire
           plumes (temperature 500..3000 K, blackbody emission, density falling off with
           height); max path length 3, 16..32 candidates, temporal + spatial, FP16 bricks and
           the learned target (2^15 training samples per instance and frame, 2^20 per batch).
  fire   : 128^3 fire plume (fBm turbulence, density falling off with height) with a
           temperature grid of 500..3000 K emitting blackbody radiance; sigma_t 30, albedo 0.6;
           one point light + dim sky; max path length 3, 16 candidates, temporal + spatial.
"""
import math
from dataclasses import dataclass, field

import numpy as np

from . import capi


@dataclass
class SceneDesc:
    name: str
    width: int
    height: int
    volume: capi.ProceduralDesc
    medium: capi.Medium
    lights: list
    env_rgb: np.ndarray            # (H, W, 3) float32 lat-long
    env_scale: tuple = (1.0, 1.0, 1.0)
    options: dict = field(default_factory=dict)
    camera_radius: float = 2.5
    camera_height: float = 0.0
    orbit_deg_per_frame: float = 0.0
    fov_deg: float = 45.0
    frames: int = 16
    fire: tuple = None             # (t_min, t_max, le_scale, cutoff, scale) for emissive plumes
    orbit_start_deg: float = 0.0
    anim_frames: int = 0           # animated volume: number of frames in the cycle
    anim_shift: tuple = None       # world displacement of the volume per animation frame

    def camera(self, frame=0):
        ang = math.radians(self.orbit_start_deg + self.orbit_deg_per_frame * frame)
        pos = (-self.camera_radius * math.sin(ang), self.camera_height, -self.camera_radius * math.cos(ang))
        c = capi.Camera()
        c.pos[:] = [float(np.float32(v)) for v in pos]
        c.target[:] = [0.0, 0.0, 0.0]
        c.up[:] = [0.0, 1.0, 0.0]
        c.fov_y = float(np.float32(math.radians(self.fov_deg)))
        c.near_z = 0.01
        c.far_z = 1000.0
        return c


def _procedural(kind, res, octaves, seed, threshold, world_min, voxel_size, fp16=False, num_mips=4,
                base_frequency=4.0, mask_radius=0.45):
    d = capi.ProceduralDesc()
    d.kind = kind
    d.res = res
    d.num_mips = num_mips
    d.octaves = octaves
    d.seed = seed
    d.lacunarity = 2.0
    d.gain = 0.5
    d.base_frequency = base_frequency
    d.mask_radius = mask_radius
    d.threshold = threshold
    d.world_min[:] = list(world_min)
    d.voxel_size = voxel_size
    d.fp16 = 1 if fp16 else 0
    return d


def _medium(sigma_t, albedo, g):
    m = capi.Medium()
    ss = np.float32(sigma_t * albedo)
    sa = np.float32(sigma_t) - ss
    m.sigma_s[:] = [float(ss)] * 3
    m.sigma_a[:] = [float(sa)] * 3
    m.g = g
    m.density_scale = 1.0
    return m


def constant_env(value, w=8, h=4):
    return np.full((h, w, 3), value, dtype=np.float32)


def sky_env(w=512, h=256):
    """Procedural sky in lat-long layout (v = 0 at +y): zenith-to-horizon gradient, a dim
    ground and a soft sun lobe."""
    v = (np.arange(h, dtype=np.float64) + 0.5) / h
    u = (np.arange(w, dtype=np.float64) + 0.5) / w
    uu, vv = np.meshgrid(u, v)
    theta = vv * math.pi                       # 0 at +y
    phi = (uu - 0.5) * 2.0 * math.pi
    d = np.stack([np.sin(theta) * np.sin(phi), np.cos(theta), -np.sin(theta) * np.cos(phi)], -1)
    up = np.clip(d[..., 1], 0.0, 1.0)
    zen = np.array([0.25, 0.45, 0.95])
    hor = np.array([0.85, 0.9, 1.0])
    sky = hor + (zen - hor) * up[..., None] ** 0.6
    ground = np.array([0.25, 0.22, 0.2]) * np.ones_like(sky)
    col = np.where((d[..., 1] >= 0)[..., None], sky, ground)
    sun = np.array([0.3, 0.8, 0.5])
    sun /= np.linalg.norm(sun)
    lobe = np.clip(d @ sun, 0.0, 1.0) ** 256
    col = col + lobe[..., None] * np.array([40.0, 36.0, 30.0])
    return col.astype(np.float32)


def sphere_lights(n, radius, intensity):
    lights = []
    ga = math.pi * (3.0 - math.sqrt(5.0))
    for i in range(n):
        y = 1.0 - 2.0 * (i + 0.5) / n
        r = math.sqrt(max(0.0, 1.0 - y * y))
        t = ga * i
        l = capi.PointLight()
        l.pos[:] = [radius * r * math.cos(t), radius * y, radius * r * math.sin(t)]
        l.intensity[:] = [intensity] * 3
        lights.append(l)
    return lights


def small(width=256, height=256, fp16=False):
    light = capi.PointLight()
    light.pos[:] = [2.0, 2.0, 2.0]
    light.intensity[:] = [50.0, 50.0, 50.0]
    return SceneDesc(
        name="small_fp16" if fp16 else "small", width=width, height=height,
        volume=_procedural(0, 128, 4, 1, 0.0, (-0.5, -0.5, -0.5), 1.0 / 128.0, fp16=fp16),
        medium=_medium(20.0, 0.9, 0.0), lights=[light], env_rgb=constant_env(0.2),
        options=dict(mMaxBounces=2, mInitialM=8, mEnableTemporalReuse=1, mEnableSpatialReuse=1, mSpatialSampleCount=4,
                     mSampleRadius=10.0, mUseAnalyticLights=1, mUseEnvironmentLights=1),
        camera_radius=2.5, frames=16)


def full(width=1920, height=1080, fp16=False):
    return SceneDesc(
        name="full_fp16" if fp16 else "full", width=width, height=height,
        volume=_procedural(1, 512, 6, 7, 0.35, (-1.0, -1.0, -1.0), 2.0 / 512.0, fp16=fp16, base_frequency=3.0),
        medium=_medium(40.0, 0.95, 0.6), lights=sphere_lights(16, 3.0, 10.0), env_rgb=sky_env(),
        options=dict(mMaxBounces=3, mInitialM=32, mEnableTemporalReuse=1, mEnableSpatialReuse=1, mSpatialSampleCount=4,
                     mSampleRadius=10.0, mUseAnalyticLights=1, mUseEnvironmentLights=1),
        camera_radius=2.4, camera_height=0.3, orbit_deg_per_frame=0.5, frames=64)


def fire(width=256, height=256, fp16=False, res=128, seed=11):
    light = capi.PointLight()
    light.pos[:] = [2.0, 3.0, -2.0]
    light.intensity[:] = [40.0, 40.0, 40.0]
    vol = _procedural(2, res, 5, seed, 0.0, (-0.5, -0.5, -0.5), 1.0 / res, fp16=fp16, num_mips=3, base_frequency=5.0)
    return SceneDesc(
        name="fire_fp16" if fp16 else "fire", width=width, height=height, volume=vol,
        medium=_medium(30.0, 0.6, 0.2), lights=[light], env_rgb=constant_env(0.05),
        options=dict(mMaxBounces=3, mInitialM=16, mEnableTemporalReuse=1, mEnableSpatialReuse=1, mSpatialSampleCount=4,
                     mSampleRadius=10.0, mUseAnalyticLights=1, mUseEnvironmentLights=1),
        camera_radius=2.2, frames=16, fire=(500.0, 3000.0, 100.0, 0.0, 1.0))


BATCH_RESOLUTIONS = ((256, 256), (512, 512), (960, 540), (1280, 720), (1920, 1080))
BATCH_GRIDS = (128, 192, 256, 320, 384, 448, 512)


def batch(n=32, fires=8, seed=2024, learned=True, fp16=True, scale=1.0):
    """The batched workload: a list of SceneDesc, fire plumes first.  `scale` shrinks the
    resolutions (for tests)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = BATCH_RESOLUTIONS[int(rng.integers(len(BATCH_RESOLUTIONS)))]
        w, h = max(8, int(w * scale)), max(8, int(h * scale))
        M = int(rng.integers(16, 33))
        ang = float(rng.uniform(0.0, 360.0))
        if i < fires:
            res = int(rng.choice((128, 192, 256)))
            sc = fire(width=w, height=h, fp16=fp16, res=res, seed=1000 + i)
        else:
            res = int(rng.choice(BATCH_GRIDS))
            sc = full(width=w, height=h, fp16=fp16)
            sc.volume = _procedural(1, res, 6, 100 + i, float(rng.uniform(0.3, 0.4)), (-1.0, -1.0, -1.0), 2.0 / res,
                                    fp16=fp16, num_mips=4 if res % 64 == 0 else 3, base_frequency=float(rng.uniform(2.5, 3.5)))
        sc.name = f"batch{i}"
        sc.options = dict(sc.options, mMaxBounces=3, mInitialM=M, mEnableTemporalReuse=1, mEnableSpatialReuse=1)
        if learned:
            sc.options.update(mUseLearnedPHat=1, mLearnedTrainSamples=32768, mLearnedBatch=16384)
        sc.orbit_deg_per_frame = 0.5
        sc.orbit_start_deg = ang
        out.append(sc)
    return out


def animated(width=128, height=96, frames=4, fp16=False, fire=False, shift_voxels=(1.5, 0.0, 0.75), res=64):
    """A drifting cloud (or fire plume): the same procedural volume displaced by a fixed world
    offset per animation frame, with a velocity grid equal to that offset.  Use make_animation."""
    voxel = 1.0 / res
    light = capi.PointLight()
    light.pos[:] = [2.0, 2.0, 2.0]
    light.intensity[:] = [50.0, 50.0, 50.0]
    shift = tuple(v * voxel for v in shift_voxels)
    fire_params = (500.0, 3000.0, 0.02, 0.0, 1.0) if fire else None
    return SceneDesc(
        name="animated_fire" if fire else "animated", width=width, height=height,
        volume=_procedural(0, res, 3, 5, 0.0, (-0.5, -0.5, -0.5), voxel, fp16=fp16, num_mips=3),
        medium=_medium(20.0, 0.9, 0.2), lights=[light], env_rgb=constant_env(0.2),
        options=dict(mMaxBounces=2, mInitialM=6, mEnableTemporalReuse=1, mEnableSpatialReuse=1, mSpatialSampleCount=4,
                     mSampleRadius=8.0, mUseAnalyticLights=1, mUseEnvironmentLights=1),
        camera_radius=2.0, frames=2 * frames + 1, fire=fire_params, anim_frames=frames, anim_shift=shift)


def make_animation(sc, lib=None):
    """(frames, temperatures or None, velocity components) for an animated SceneDesc: frame i is
    the scene's volume with its world_min moved by i * anim_shift; velocity is anim_shift everywhere
    in the frame's box."""
    import ctypes as C
    from .restir import Volume
    lib = lib or capi.load()
    frames, temps, vels = [], [], []
    d = sc.volume
    for i in range(sc.anim_frames):
        di = capi.ProceduralDesc()
        C.pointer(di)[0] = d
        for k in range(3):
            di.world_min[k] = d.world_min[k] + i * sc.anim_shift[k]
        if sc.fire:
            dv, tv = Volume.fire(di, sc.fire[0], sc.fire[1], lib=lib)
            frames.append(dv)
            temps.append(tv)
        else:
            frames.append(Volume.procedural(di, lib=lib))
        for k in range(3):
            g = np.full((d.res, d.res, d.res), sc.anim_shift[k], np.float32)
            vels.append(Volume.signed(g, tuple(di.world_min), d.voxel_size, lib=lib))
    return frames, (temps if sc.fire else None), vels


def make_volumes(sc, lib=None):
    """(density volume, temperature volume or None) of a scene."""
    from .restir import Volume
    if sc.fire:
        return Volume.fire(sc.volume, sc.fire[0], sc.fire[1], lib=lib)
    return Volume.procedural(sc.volume, lib=lib), None


CONFIGS = {"small": small, "full": full, "small_fp16": lambda **k: small(fp16=True, **k), "fire": fire, "batch": batch}
