"""Host-side mirror of the reference render pass interface.

`VolumetricReSTIR` keeps the names and behaviour of the reference's pass
(Source/RenderPasses/VolumetricReSTIR/VolumetricReSTIR.h:36-315):

  * construction from a parameter dictionary (VolumetricReSTIR::create, .cpp:61-70); unknown
    keys produce a warning, as serializePass does (.h:305-311);
  * `mParams` / `setParams` with the VolumetricReSTIRParams field names; any change resets the
    temporal history like mOptionsChanged (.cpp:349-359);
  * `setScene` binds the volume, medium, lights and environment (.cpp:1218-1256);
  * `execute` renders one frame into a device RGBA32F buffer (`accumulated_color`).

All rendering goes through libvrestir.so (CUDA); PyTorch only provides device buffers and the
current stream.
"""
import ctypes as C
import warnings

import numpy as np

from . import capi


class Volume:
    """Host-side sparse brick grid with its mip pyramids (owned by the library)."""

    def __init__(self, handle, lib):
        self._h = handle
        self._lib = lib

    @classmethod
    def procedural(cls, desc, lib=None):
        lib = lib or capi.load()
        h = C.c_void_p()
        r = lib.vr_volume_create_procedural(C.byref(desc), C.byref(h))
        if r != capi.VR_OK:
            raise ValueError(f"vr_volume_create_procedural failed ({r})")
        return cls(h, lib)

    @classmethod
    def fire(cls, desc, t_min, t_max, lib=None):
        """Fire plume: (density volume, temperature volume)."""
        lib = lib or capi.load()
        hd, ht = C.c_void_p(), C.c_void_p()
        r = lib.vr_volume_create_fire(C.byref(desc), t_min, t_max, C.byref(hd), C.byref(ht))
        if r != capi.VR_OK:
            raise ValueError(f"vr_volume_create_fire failed ({r})")
        return cls(hd, lib), cls(ht, lib)

    @classmethod
    def load_vbx(cls, path, num_mips=4, fp16=False, signed=False, lib=None):
        """A GVDB .vbx file (grid 0); signed: a velocity component (mip 0 only)."""
        lib = lib or capi.load()
        h = C.c_void_p()
        flags = (1 if fp16 else 0) | (2 if signed else 0)
        r = lib.vr_volume_load_vbx(str(path).encode(), num_mips, flags, C.byref(h))
        if r != capi.VR_OK:
            raise ValueError(f"vr_volume_load_vbx failed ({r}): {lib.vr_volume_vbx_error().decode()}")
        return cls(h, lib)

    def save_vbx(self, path):
        r = self._lib.vr_volume_save_vbx(self._h, str(path).encode())
        if r != capi.VR_OK:
            raise ValueError(f"vr_volume_save_vbx failed ({r}): {self._lib.vr_volume_vbx_error().decode()}")

    @classmethod
    def signed(cls, values, world_min, voxel_size, fp16=False, lib=None):
        """Signed scalar grid, mip 0 only (a velocity component)."""
        lib = lib or capi.load()
        d = np.ascontiguousarray(values, dtype=np.float32)
        assert d.ndim == 3 and d.shape[0] == d.shape[1] == d.shape[2]
        wm = (C.c_float * 3)(*world_min)
        h = C.c_void_p()
        r = lib.vr_volume_create_dense_signed(d.ctypes.data_as(C.POINTER(C.c_float)), d.shape[0], wm, voxel_size,
                                              1 if fp16 else 0, C.byref(h))
        if r != capi.VR_OK:
            raise ValueError(f"vr_volume_create_dense_signed failed ({r})")
        return cls(h, lib)

    @classmethod
    def dense(cls, density, world_min, voxel_size, num_mips=4, fp16=False, lib=None):
        lib = lib or capi.load()
        d = np.ascontiguousarray(density, dtype=np.float32)
        assert d.ndim == 3 and d.shape[0] == d.shape[1] == d.shape[2]
        wm = (C.c_float * 3)(*world_min)
        h = C.c_void_p()
        r = lib.vr_volume_create_dense(d.ctypes.data_as(C.POINTER(C.c_float)), d.shape[0], num_mips, wm,
                                       voxel_size, 1 if fp16 else 0, C.byref(h))
        if r != capi.VR_OK:
            raise ValueError(f"vr_volume_create_dense failed ({r})")
        return cls(h, lib)

    def compress_bc4(self):
        """Re-encode the coarse normal mips and every conservative mip as BC4 blocks (the
        reference's default texture form); normal mip 0 keeps its storage.  Returns self."""
        r = self._lib.vr_volume_compress_bc4(self._h)
        if r != capi.VR_OK:
            raise ValueError(f"vr_volume_compress_bc4 failed ({r})")
        return self

    def info(self):
        i = capi.VolumeInfo()
        self._lib.vr_volume_get_info(self._h, C.byref(i))
        return i

    def slot(self, s):
        v = capi.GridView()
        self._lib.vr_volume_get_slot(self._h, s, C.byref(v))
        return v

    def views(self):
        arr = (capi.GridView * capi.VR_NUM_SLOTS)()
        for s in range(capi.VR_NUM_SLOTS):
            self._lib.vr_volume_get_slot(self._h, s, C.byref(arr[s]))
        return arr

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.vr_volume_destroy(self._h)
            self._h = None


def blackbody_lut(lib=None):
    """The library's blackbody table: (128, 3) linear sRGB for 50 K .. 6400 K."""
    lib = lib or capi.load()
    out = np.zeros(384, np.float32)
    lib.vr_blackbody_lut(out.ctypes.data_as(C.POINTER(C.c_float)))
    return out.reshape(128, 3)


def env_struct(rgb, scale=(1.0, 1.0, 1.0), rotation=None):
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    e = capi.EnvMap()
    e.rgb = rgb.ctypes.data_as(C.POINTER(C.c_float))
    e.height, e.width = rgb.shape[0], rgb.shape[1]
    e.scale[:] = list(scale)
    e.rotation[:] = list(rotation) if rotation is not None else [1, 0, 0, 0, 1, 0, 0, 0, 1]
    return e, rgb


def load_gvdb_volume(vbx, num_mips=1, fp16=False, lib=None):
    """The file layout Scene::addGVDBVolume reads (Scene.cpp:2769-2816): with num_mips > 1, `vbx`
    is a folder <dir>/<name> holding <name>_mip0.vbx (this loader rebuilds the finer mips and the
    conservative <name>_mip<k>c.vbx from mip 0); with num_mips == 1 it is the file itself.
    <name>_temperature.vbx and <name>_velocity_{x,y,z}.vbx in the folder are picked up when
    present.  Returns (density, temperature or None, [vx, vy, vz] or None)."""
    import os
    vbx = str(vbx)
    name = os.path.basename(vbx.rstrip("/\\"))
    density_file = os.path.join(vbx, f"{name}_mip0.vbx") if num_mips > 1 else vbx
    density = Volume.load_vbx(density_file, num_mips=num_mips, fp16=fp16, lib=lib)
    folder = vbx if num_mips > 1 else os.path.dirname(vbx)
    base = name if num_mips > 1 else os.path.splitext(name)[0]
    tf = os.path.join(folder, f"{base}_temperature.vbx")
    temperature = Volume.load_vbx(tf, num_mips=1, fp16=fp16, lib=lib) if os.path.exists(tf) else None
    vfs = [os.path.join(folder, f"{base}_velocity_{a}.vbx") for a in "xyz"]
    velocity = [Volume.load_vbx(f, signed=True, lib=lib) for f in vfs] if all(os.path.exists(f) for f in vfs) else None
    return density, temperature, velocity


class VolumetricReSTIR:
    """The per-frame Volumetric ReSTIR loop on one GB300."""

    def __init__(self, width, height, params=None, lib=None):
        self._lib = lib or capi.load()
        self._opts = capi.default_options(self._lib)
        if params:
            self._apply(params)
        err = C.c_int32()
        self._h = self._lib.vr_create(C.byref(self._opts), width, height, C.byref(err))
        if not self._h:
            raise RuntimeError(f"vr_create failed ({err.value})")
        self.width, self.height = width, height
        self._keep = []

    # ---- options (VolumetricReSTIRParams) ----
    def _apply(self, params):
        names = {k for k, _ in capi.Options._fields_}
        for k, v in params.items():
            if k not in names:
                warnings.warn(f"Unknown field '{k}' in a VolumetricReSTIR dictionary")
                continue
            setattr(self._opts, k, v)

    @property
    def mParams(self):
        return self._opts.as_dict()

    def setParams(self, **params):
        self._apply(params)
        self._check(self._lib.vr_set_options(self._h, C.byref(self._opts)))

    # ---- scene ----
    def setScene(self, volume, medium, lights=(), env_rgb=None, env_scale=(1.0, 1.0, 1.0)):
        self._volume = volume
        self._check(self._lib.vr_set_volume(self._h, volume._h, C.byref(medium)))
        arr = (capi.PointLight * max(1, len(lights)))(*lights) if lights else None
        env = None
        if env_rgb is not None:
            env, keep = env_struct(env_rgb, env_scale)
            self._keep = [keep]
        self._check(self._lib.vr_set_lights(self._h, arr, len(lights), C.byref(env) if env is not None else None))

    # ---- frames ----
    def setEmission(self, temperature, le_scale, cutoff=0.0, scale=1.0, lut=None):
        """Volume emission from a temperature volume (None switches it off)."""
        self._temperature = temperature
        lp = None
        if lut is not None:
            self._lut = np.ascontiguousarray(lut, np.float32).reshape(384)
            lp = self._lut.ctypes.data_as(C.POINTER(C.c_float))
        self._check(self._lib.vr_set_emission(self._h, temperature._h if temperature is not None else None, le_scale, cutoff,
                                              scale, lp))

    def set_animation(self, frames, temperature=None, velocity=None, velocity_scale=1.0):
        """Animated volume sequence (Scene::addGVDBVolumeSequence): frames are Volumes with the
        bound volume's res, box and mips; temperature one Volume (or None) per frame; velocity
        three component Volumes per frame (x, y, z; world units per frame).  Each execute()
        advances one frame, cyclically.  An empty list returns to the static volume."""
        n = len(frames)
        self._anim_keep = list(frames) + [t for t in (temperature or []) if t is not None] + list(velocity or [])
        fa = (C.c_void_p * max(1, n))(*[f._h for f in frames])
        ta = va = None
        if temperature is not None:
            if len(temperature) != n:
                raise ValueError("one temperature entry per frame")
            ta = (C.c_void_p * n)(*[t._h if t is not None else None for t in temperature])
        if velocity is not None:
            if len(velocity) != 3 * n:
                raise ValueError("three velocity components per frame")
            va = (C.c_void_p * (3 * n))(*[v._h for v in velocity])
        self._check(self._lib.vr_set_animation(self._h, fa, n, ta, va, velocity_scale))

    def animation_frame(self):
        return int(self._lib.vr_animation_frame(self._h))

    def execute(self, camera, out_ptr, mvec_ptr=None, stream=0):
        """Renders one frame into device memory (width*height float4)."""
        self._check(self._lib.vr_render_frame(self._h, C.byref(camera), C.c_void_p(out_ptr),
                                              C.c_void_p(mvec_ptr) if mvec_ptr else None, C.c_void_p(stream)))

    def set_frame_hook(self, fn):
        """Post-process hook run after every frame (the slot of the reference graph's
        OptixDenoiser): fn(rgba_ptr, mvec_ptr_or_0, width, height, stream) enqueues its work on
        the frame's stream and may rewrite the image in place.  None removes it."""
        if fn is None:
            self._hook = None
            self._check(self._lib.vr_set_frame_hook(self._h, None, None))
            return

        def call(user, rgba, mvec, w, h, stream):
            fn(rgba or 0, mvec or 0, w, h, stream or 0)
        self._hook = capi.FRAME_HOOK(call)            # kept alive with the context
        self._check(self._lib.vr_set_frame_hook(self._h, C.cast(self._hook, C.c_void_p), None))

    def execute_host(self, camera, stream=0):
        out = np.empty((self.height, self.width, 4), np.float32)
        self._check(self._lib.vr_render_frame_host(self._h, C.byref(camera), out.ctypes.data_as(C.POINTER(C.c_float)),
                                                   C.c_void_p(stream)))
        return out

    def render_reference(self, camera, accum_ptr, first_frame, num_frames, stream=0):
        self._check(self._lib.vr_render_reference(self._h, C.byref(camera), first_frame, num_frames,
                                                  C.c_void_p(accum_ptr), C.c_void_p(stream)))

    # ---- state ----
    def export_reservoirs(self, which=0):
        n = self.width * self.height
        rb = self._lib.vr_reservoir_bytes(self._h)
        buf = np.zeros(n * rb, np.uint8)
        self._check(self._lib.vr_export_reservoirs(self._h, which, buf.ctypes.data_as(C.c_void_p), buf.nbytes))
        return buf

    def export_extra(self, which=0):
        n = self.width * self.height * max(self._opts.mMaxBounces - 1, 0) * 3
        out = np.zeros(max(n, 1), np.float32)
        self._check(self._lib.vr_export_extra_bounces(self._h, which, out.ctypes.data_as(C.POINTER(C.c_float)), out.nbytes))
        return out[:n]

    def export_features(self):
        out = np.zeros(self.width * self.height * 2, np.int32)
        self._check(self._lib.vr_export_features(self._h, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def export_state(self):
        n = self._lib.vr_state_bytes(self._h)
        buf = np.zeros(n, np.uint8)
        self._check(self._lib.vr_export_state(self._h, buf.ctypes.data_as(C.c_void_p), buf.nbytes))
        return buf

    def import_state(self, buf):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        self._check(self._lib.vr_import_state(self._h, buf.ctypes.data_as(C.c_void_p), buf.nbytes))

    @property
    def frame_count(self):
        return self._lib.vr_frame_count(self._h)

    def last_timings(self):
        ms = (C.c_float * 16)()
        n = C.c_int32()
        self._lib.vr_last_timings(self._h, ms, 16, C.byref(n))
        return list(ms[: n.value])

    def kernel_time_totals(self, reset=True):
        ms = (C.c_float * 8)()
        n = C.c_int32()
        self._check(self._lib.vr_kernel_time_totals(self._h, ms, 8, C.byref(n), 1 if reset else 0))
        return list(ms[:6]), n.value

    def last_launch_count(self):
        return self._lib.vr_last_launch_count(self._h)

    # ---- learned target (transmittance network) ----
    def net_params(self):
        out = np.zeros(capi.NET_PARAMS, np.float32)
        self._check(self._lib.vr_net_get_params(self._h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def set_net_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == capi.NET_PARAMS
        self._check(self._lib.vr_net_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def net_infer(self, queries_ptr, n, out_ptr, stream=0):
        self._check(self._lib.vr_net_infer(self._h, C.c_void_p(queries_ptr), n, C.c_void_p(out_ptr), C.c_void_p(stream)))

    def net_gradients(self, samples_ptr, n):
        g = np.zeros(capi.NET_PARAMS, np.float32)
        loss = C.c_float()
        self._check(self._lib.vr_net_gradients(self._h, C.c_void_p(samples_ptr), n, g.ctypes.data_as(C.POINTER(C.c_float)),
                                               C.byref(loss)))
        return loss.value, g

    def net_train_step(self, samples_ptr, n):
        loss = C.c_float()
        self._check(self._lib.vr_net_train_step(self._h, C.c_void_p(samples_ptr), n, C.byref(loss)))
        return loss.value

    def net_box(self):
        out = np.zeros(6, np.float32)
        cnt = C.c_int64()
        self._check(self._lib.vr_export_learned(self._h, 4, out.ctypes.data_as(C.c_void_p), out.nbytes, C.byref(cnt)))
        return out[:3].copy(), out[3:].copy()

    def export_learned(self, which):
        """0: T per vertex slot, 1: query list (n, 8), 2: training samples (n, 8), 3: step losses."""
        cnt = C.c_int64()
        self._check(self._lib.vr_export_learned(self._h, which, None, 0, C.byref(cnt)))
        n = cnt.value * (8 if which in (1, 2) else 1)
        out = np.zeros(max(n, 1), np.float32)
        self._check(self._lib.vr_export_learned(self._h, which, out.ctypes.data_as(C.c_void_p), out.nbytes, C.byref(cnt)))
        out = out[:n]
        return out.reshape(-1, 8) if which in (1, 2) else out

    def _check(self, r):
        if r != capi.VR_OK:
            msg = self._lib.vr_last_error(self._h).decode() if getattr(self, "_h", None) else ""
            raise RuntimeError(f"libvrestir error {r}: {msg}")

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.vr_destroy(self._h)
            self._h = None


class Batch:
    """Many VolumetricReSTIR instances rendered by persistent batched launches (and a CUDA graph)."""

    def __init__(self, renderers, graph=True):
        self._r = list(renderers)
        self._lib = self._r[0]._lib
        arr = (C.c_void_p * len(self._r))(*[r._h for r in self._r])
        h = C.c_void_p()
        rc = self._lib.vr_batch_create(arr, len(self._r), C.byref(h))
        if rc != capi.VR_OK:
            raise RuntimeError(f"vr_batch_create failed ({rc})")
        self._h = h
        self._lib.vr_batch_set_graph(self._h, 1 if graph else 0)

    def _args(self, cams, out_ptrs):
        ca = (capi.Camera * len(cams))(*cams)
        oa = (C.c_void_p * len(out_ptrs))(*out_ptrs)
        return ca, oa

    def render(self, cams, out_ptrs, stream=0):
        ca, oa = self._args(cams, out_ptrs)
        self._check(self._lib.vr_batch_render(self._h, ca, oa, C.c_void_p(stream)))

    def autotune(self, cams, out_ptrs, stream=0, max_trials=0):
        ca, oa = self._args(cams, out_ptrs)
        ms = (C.c_float * 16)()
        self._check(self._lib.vr_batch_autotune(self._h, ca, oa, C.c_void_p(stream), ms, max_trials))
        return list(ms[: (max_trials or 9)]), self.launch_shape()

    def set_launch_shape(self, tile_w, blocks_per_sm):
        self._check(self._lib.vr_batch_set_launch_shape(self._h, tile_w, blocks_per_sm))

    def launch_shape(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        self._lib.vr_batch_get_launch_shape(self._h, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def last_launch_count(self):
        return self._lib.vr_batch_last_launch_count(self._h)

    def set_graph(self, on):
        self._lib.vr_batch_set_graph(self._h, 1 if on else 0)

    def _check(self, r):
        if r != capi.VR_OK:
            raise RuntimeError(f"libvrestir batch error {r}: {self._lib.vr_batch_last_error(self._h).decode()}")

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.vr_batch_destroy(self._h)
            self._h = None


class Accumulator:
    """Running per-pixel sums of RGBA32F frames (AccumulatePass, Accumulate.cs.slang:55-125):
    precision 0 = double, 1 = single, 2 = compensated single."""

    def __init__(self, width, height, precision=0, lib=None):
        self._lib = lib or capi.load()
        h = C.c_void_p()
        rc = self._lib.vr_accumulator_create(width, height, precision, C.byref(h))
        if rc != capi.VR_OK:
            raise RuntimeError(f"vr_accumulator_create failed ({rc})")
        self._h = h

    def add(self, frame_ptr, mean_out_ptr=None, stream=0):
        """Adds one device frame; writes the running mean to mean_out_ptr (device RGBA32F) if given."""
        rc = self._lib.vr_accumulate(self._h, C.c_void_p(frame_ptr), C.c_void_p(mean_out_ptr) if mean_out_ptr else None,
                                     C.c_void_p(stream))
        if rc != capi.VR_OK:
            raise RuntimeError(f"vr_accumulate failed ({rc})")

    def reset(self):
        self._lib.vr_accumulator_reset(self._h)

    @property
    def count(self):
        return self._lib.vr_accumulator_count(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.vr_accumulator_destroy(self._h)
            self._h = None


RESERVOIR_DTYPE_36 = np.dtype([("runningSum", "<f4"), ("M", "<f4"), ("depth", "<f4"), ("p_y", "<f4"),
                               ("lightUV", "<f4", 2), ("lightID", "<i4"), ("sampledPixel", "<i4"),
                               ("extraBounceStartId", "<i4")])
RESERVOIR_DTYPE_40 = np.dtype([("runningSum", "<f4"), ("M", "<f4"), ("depth", "<f4"), ("p_y", "<f4"),
                               ("lightUV", "<f4", 2), ("lightID", "<i4"), ("sampledPixel", "<i4"),
                               ("extraBounceStartId", "<i4"), ("p_partial", "<f4")])
RESERVOIR_DTYPE_32 = np.dtype([("runningSum", "<f4"), ("M", "<f4"), ("depth", "<f4"), ("p_y", "<f4"),
                               ("lightUV", "<f4", 2), ("lightID", "<i4"), ("sampledPixel", "<i4")])


def as_reservoirs(buf, max_bounces, vertex_reuse=False):
    if max_bounces > 1 and vertex_reuse:
        return np.frombuffer(buf.tobytes(), RESERVOIR_DTYPE_40)
    return np.frombuffer(buf.tobytes(), RESERVOIR_DTYPE_36 if max_bounces > 1 else RESERVOIR_DTYPE_32)
