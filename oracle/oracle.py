"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, and only
as the checker; the product path never calls it.
"""
import ctypes as C
import pathlib

import numpy as np

from . import build as _build

HERE = pathlib.Path(__file__).resolve().parent


def _load():
    lib = C.CDLL(str(_build.build()))
    P = C.c_void_p
    sig = {
        "vro_create": (P, [P, C.c_int, C.c_int]),
        "vro_destroy": (None, [P]),
        "vro_bc4_decode_block": (None, [C.c_uint64, P]),
        "vro_set_threads": (None, [P, C.c_int]),
        "vro_set_options": (None, [P, P]),
        "vro_set_volume": (C.c_int, [P, P, C.c_int, P, C.c_float, C.c_float, C.c_int]),
        "vro_set_lights": (C.c_int, [P, P, C.c_int, P]),
        "vro_render_frame": (C.c_int, [P, P, P, P]),
        "vro_frame_count": (C.c_int, [P]),
        "vro_voxel_reads": (None, [P]),
        "vro_export_reservoirs": (C.c_int, [P, C.c_int, P]),
        "vro_export_extra": (C.c_int, [P, C.c_int, P]),
        "vro_export_features": (C.c_int, [P, P]),
        "vro_env_importance": (C.c_int, [P, C.c_int, P]),
        "vro_render_reference": (C.c_int, [P, P, C.c_int, C.c_int, P]),
        "vro_transmittance": (C.c_float, [P, P, P, C.c_float, C.c_int, C.c_int, C.c_int, C.c_float, C.c_uint32]),
        "vro_sample_distance": (None, [P, P, P, C.c_int, C.c_int, C.c_uint32, P]),
        "vro_density_world": (C.c_float, [P, P, C.c_int]),
        "vro_math": (C.c_int, [C.c_int, P, P, P, C.c_int]),
        "vro_rng": (None, [P, C.c_int, C.c_int, P]),
        "vro_xoshiro": (None, [P, C.c_int, P]),
        "vro_splitmix": (None, [C.c_uint64, C.c_int, P]),
        "vro_set_net": (None, [P, P, P, P]),
        "vro_set_emission": (None, [P, P, P, C.c_float, C.c_float, C.c_float]),
        "vro_set_animation": (None, [P, P, C.c_int, P, P, C.c_float, P, C.c_float, C.c_float, C.c_float]),
        "vro_set_lp_T": (None, [P, P, C.c_int64]),
        "vro_export_lp": (C.c_int64, [P, C.c_int, P, C.c_int64]),
        "vro_net_forward": (None, [P, P, P, C.c_float, P, C.c_int, P]),
        "vro_net_gradients": (None, [P, P, P, P, C.c_int, C.c_int, C.c_float, P, P]),
        "vro_volume_procedural": (P, [P]),
        "vro_volume_info": (C.c_int, [P, P]),
        "vro_volume_slot": (C.c_int, [P, C.c_int, P]),
        "vro_volume_destroy": (None, [P]),
    }
    for k, (r, a) in sig.items():
        f = getattr(lib, k)
        f.restype = r
        f.argtypes = a
    return lib


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = _load()
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleVolume:
    """A procedural input grid built by the oracle's library (no GPU library involved), with the
    views()/info()/slot() interface of restir.Volume that Oracle.set_volume reads."""

    def __init__(self, desc):
        self.L = lib()
        self._h = self.L.vro_volume_procedural(C.byref(desc))
        if not self._h:
            raise ValueError("vro_volume_procedural failed")

    def info(self):
        from volumetricrestirrelease_gb300 import capi
        i = capi.VolumeInfo()
        self.L.vro_volume_info(self._h, C.byref(i))
        return i

    def slot(self, s):
        from volumetricrestirrelease_gb300 import capi
        v = capi.GridView()
        self.L.vro_volume_slot(self._h, s, C.byref(v))
        return v

    def views(self):
        from volumetricrestirrelease_gb300 import capi
        arr = (capi.GridView * capi.VR_NUM_SLOTS)()
        for s in range(capi.VR_NUM_SLOTS):
            self.L.vro_volume_slot(self._h, s, C.byref(arr[s]))
        return arr

    def __del__(self):
        if getattr(self, "_h", None):
            self.L.vro_volume_destroy(self._h)
            self._h = None


class Oracle:
    """CPU restatement of the pass, driven through the same data as the GPU library."""

    def __init__(self, width, height, options, threads=0):
        self.L = lib()
        self.width, self.height = width, height
        self._opts = options
        self._h = self.L.vro_create(C.byref(options), width, height)
        if threads:
            self.L.vro_set_threads(self._h, threads)
        self.max_bounces = options.mMaxBounces

    def set_options(self, options):
        self._opts = options
        self.max_bounces = options.mMaxBounces
        self.L.vro_set_options(self._h, C.byref(options))

    def set_volume(self, volume, medium):
        views = volume.views()
        info = volume.info()
        self._volume = volume
        self.L.vro_set_volume(self._h, C.cast(views, C.c_void_p), 16, C.byref(medium), info.voxel_size,
                              info.supervoxel_diag, info.num_mips)

    def set_lights(self, lights, env_rgb=None, env_scale=(1.0, 1.0, 1.0)):
        from volumetricrestirrelease_gb300 import capi
        from volumetricrestirrelease_gb300.restir import env_struct
        arr = (capi.PointLight * max(1, len(lights)))(*lights) if lights else None
        env = None
        if env_rgb is not None:
            env, self._env_keep = env_struct(env_rgb, env_scale)
        self.L.vro_set_lights(self._h, C.cast(arr, C.c_void_p) if arr else None, len(lights),
                              C.byref(env) if env is not None else None)

    def render_frame(self, camera, mvec=False):
        out = np.zeros((self.height, self.width, 4), np.float32)
        mv = np.zeros((self.height, self.width, 2), np.float32) if mvec else None
        r = self.L.vro_render_frame(self._h, C.byref(camera), _ptr(out), _ptr(mv) if mv is not None else None)
        if r != 0:
            raise RuntimeError(f"oracle frame status {r}")
        return (out, mv) if mvec else out

    def render_reference(self, camera, first_frame, num_frames, accum=None):
        if accum is None:
            accum = np.zeros((self.height, self.width, 3), np.float64)
        r = self.L.vro_render_reference(self._h, C.byref(camera), first_frame, num_frames, _ptr(accum))
        if r != 0:
            raise RuntimeError(f"oracle reference status {r}")
        return accum

    def set_animation(self, frames, temperature=None, velocity=None, velocity_scale=1.0):
        """Mirror of VolumetricReSTIR.set_animation: frames (density volumes), temperature (one
        per frame, entries may be None) and velocity (3 component volumes per frame)."""
        from volumetricrestirrelease_gb300 import capi
        from volumetricrestirrelease_gb300.restir import blackbody_lut
        n = len(frames)
        self._anim_keep = list(frames) + list(temperature or []) + list(velocity or [])
        views = (capi.GridView * max(1, 16 * n))()
        for i, f in enumerate(frames):
            fv = f.views()
            for k in range(16):
                views[16 * i + k] = fv[k]
        tv = vv = None
        if temperature is not None:
            tv = (capi.GridView * n)()
            for i, t in enumerate(temperature):
                if t is not None:
                    tv[i] = t.slot(0)
        if velocity is not None:
            vv = (capi.GridView * (3 * n))()
            for i, v in enumerate(velocity):
                vv[i] = v.slot(0)
        # the parameters of the last set_emission, else Scene::addGVDBVolume's defaults
        le, cut, sc, lut = getattr(self, "_emis_params", (0.005, 1.0, 100.0, None))
        self._anim_lut = np.ascontiguousarray(blackbody_lut() if lut is None else lut, np.float32).reshape(384)
        self._anim_arrays = (views, tv, vv)
        self.L.vro_set_animation(self._h, C.cast(views, C.c_void_p), n, C.cast(tv, C.c_void_p) if tv is not None else None,
                                 C.cast(vv, C.c_void_p) if vv is not None else None, velocity_scale, _ptr(self._anim_lut),
                                 le, cut, sc)

    def set_emission(self, temperature, le_scale, cutoff=0.0, scale=1.0, lut=None):
        from volumetricrestirrelease_gb300.restir import blackbody_lut
        if temperature is None:
            self.L.vro_set_emission(self._h, None, None, 0.0, 0.0, 1.0)
            return
        self._emis_params = (le_scale, cutoff, scale, lut)
        self._tview = temperature.slot(0)
        self._tvol = temperature
        self._lut = np.ascontiguousarray(blackbody_lut() if lut is None else lut, np.float32).reshape(384)
        self.L.vro_set_emission(self._h, C.byref(self._tview), _ptr(self._lut), le_scale, cutoff, scale)

    # ---- learned target ----
    def set_net(self, params, box):
        """params: VR_NET_PARAMS float32; box: (bmin[3], binv[3])."""
        self._net = np.ascontiguousarray(params, np.float32)
        self._box = [np.ascontiguousarray(b, np.float32) for b in box]
        self.L.vro_set_net(self._h, _ptr(self._net), _ptr(self._box[0]), _ptr(self._box[1]))

    def set_lp_T(self, T=None):
        """Per-slot transmittance to use instead of the CPU network (None: use the network)."""
        if T is None:
            self.L.vro_set_lp_T(self._h, None, 0)
        else:
            self._T = np.ascontiguousarray(T, np.float32)
            self.L.vro_set_lp_T(self._h, _ptr(self._T), self._T.size)

    def export_lp(self, which):
        n = self.L.vro_export_lp(self._h, which, None, 0)
        out = np.zeros(n, np.float32)
        self.L.vro_export_lp(self._h, which, _ptr(out), n)
        return out.reshape(-1, 8) if which in (0, 2) else out

    def export_reservoirs(self, which=0):
        from volumetricrestirrelease_gb300.restir import RESERVOIR_DTYPE_40
        out = np.zeros(self.width * self.height, RESERVOIR_DTYPE_40)
        self.L.vro_export_reservoirs(self._h, which, _ptr(out))
        return out

    def export_extra(self, which=0):
        n = self.width * self.height * max(self.max_bounces - 1, 1) * 3
        out = np.zeros(n, np.float32)
        self.L.vro_export_extra(self._h, which, _ptr(out))
        return out[: self.width * self.height * max(self.max_bounces - 1, 0) * 3]

    def export_features(self):
        out = np.zeros(self.width * self.height * 2, np.int32)
        self.L.vro_export_features(self._h, _ptr(out))
        return out

    def env_importance(self, mip):
        d = 512 >> mip
        out = np.zeros(d * d, np.float32)
        self.L.vro_env_importance(self._h, mip, _ptr(out))
        return out

    @property
    def frame_count(self):
        return self.L.vro_frame_count(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            self.L.vro_destroy(self._h)
            self._h = None


# VolumetricReSTIRParams defaults (VolumetricReSTIR.h:130-207) and the learned target's, so that
# CPU-only runs fill a vr_options without the GPU library (a test checks them against
# vr_options_default)
OPTION_DEFAULTS = dict(
    mMaxBounces=1, mEnableTemporalReuse=1, mEnableSpatialReuse=1, mUseReference=0, mUseEnvironmentLights=1,
    mUseAnalyticLights=0, mBaselineSamplePerPixel=1, mVisualizeTotalTransmittance=0, mInitialBaseMipLevel=1,
    mInitialM=4, mInitialLightSamples=1, mInitialLightingMipLevel=2, mInitialVisibilityUseLinearSampler=0,
    mInitialLightingUseLinearSampler=1, mInitialLightingTrackingMethod=2, mInitialVisibilityTStepScale=1.0,
    mInitialLightingTStepScale=2.0, mInitialUseRussianRoulette=1, mInitialUseCoarserGridForIndirectBounce=1,
    mTemporalReuseMThreshold=4.0, mTemporalReprojectionMode=0, mTemporalMISMethod=1, mTemporalReprojectionMipLevel=1,
    mSpatialReuseRounds=1, mSpatialVisibilityMipLevel=1, mSpatialLightingMipLevel=1, mSpatialVisibilityUseLinearSampler=1,
    mSpatialLightingUseLinearSampler=1, mSpatialVisibilityTStepScale=1.0, mSpatialLightingTStepScale=1.0,
    mSpatialVisibilityTrackingMethod=2, mSpatialLightingTrackingMethod=2, mRandomSamplerType=1, mSampleRadius=10.0,
    mSpatialSampleCount=4, mSpatialMISMethod=1, mFinalLightSamples=1, mFinalVisibilitySamples=1,
    mFinalVisibilityTrackingMethod=1, mFinalLightTrackingMethod=1, mFinalTStepScale=0.2, mUseLearnedPHat=0,
    mLearnedTrainSamples=1 << 20, mLearnedBatch=16384, mLearnedLearningRate=1e-3, mLearnedTFloor=0.02, mLearnedSeed=1,
    mLearnedTargetMethod=2, mLearnedLoss=0, mUsePrevVolumeForReproj=1, mVertexReuse=0, mVertexReuseStartBounce=1)


def default_options(**overrides):
    from volumetricrestirrelease_gb300 import capi
    o = capi.Options()
    for k, v in {**OPTION_DEFAULTS, **overrides}.items():
        setattr(o, k, v)
    return o


NET_PARAMS = 16705


def _splitmix64(state):
    state = (state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return state, z ^ (z >> 31)


def net_init(seed):
    """The learned target's initial weights for a seed: He-uniform hidden matrices from a
    SplitMix64 stream, small output weights (T starts near 1), zero biases, layer 0's four pad
    columns zero."""
    w = np.zeros(NET_PARAMS, np.float32)
    st = (0x6C7E3A91D2B54F08 ^ (seed << 17)) & 0xFFFFFFFFFFFFFFFF

    def uni():
        nonlocal st
        st, z = _splitmix64(st)
        return np.float32(np.float32((z >> 40) * (1.0 / 16777216.0)) * np.float32(2.0) - np.float32(1.0))
    for l in range(4):
        bound = np.float32(np.sqrt(np.float32(6.0) / np.float32(60 if l == 0 else 64)))
        base = l * (4096 + 64)
        for r in range(64):
            for k in range(64):
                u = uni()
                w[base + r * 64 + k] = 0.0 if (l == 0 and k >= 60) else u * bound
    ob = np.float32(np.float32(0.1) * np.sqrt(np.float32(6.0) / np.float32(64)))
    for k in range(64):
        w[4 * (4096 + 64) + k] = uni() * ob
    return w


class CpuTrainer:
    """Adam on the transmittance network with the oracle's gradient (BF16 operands, FP32 sums),
    the batch split over host threads (each chunk's mean gradient, averaged in chunk order)."""

    def __init__(self, params, box, lr=1e-3, threads=0, loss_log=0, floor=0.02):
        import os
        self.w = np.ascontiguousarray(params, np.float32).copy()
        self.m = np.zeros_like(self.w)
        self.v = np.zeros_like(self.w)
        self.t = 0
        self.lr = lr
        self.box = [np.ascontiguousarray(b, np.float32) for b in box]
        self.threads = threads or os.cpu_count() or 1
        self.loss_log, self.floor = loss_log, floor

    def step(self, samples):
        import concurrent.futures as cf
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 8)
        parts = np.array_split(np.arange(len(s)), self.threads)
        parts = [p for p in parts if len(p)]
        L = lib()
        grads = [np.zeros(NET_PARAMS, np.float32) for _ in parts]
        losses = [np.zeros(1, np.float32) for _ in parts]
        chunks = [np.ascontiguousarray(s[p[0]:p[-1] + 1]) for p in parts]

        def run(i):
            L.vro_net_gradients(_ptr(self.w), _ptr(self.box[0]), _ptr(self.box[1]), _ptr(chunks[i]), len(chunks[i]),
                                int(self.loss_log), float(self.floor), _ptr(grads[i]), _ptr(losses[i]))
        with cf.ThreadPoolExecutor(len(parts)) as ex:
            list(ex.map(run, range(len(parts))))
        g = np.zeros(NET_PARAMS, np.float64)
        for gi, p in zip(grads, parts):
            g += gi.astype(np.float64) * (len(p) / len(s))
        g = g.astype(np.float32)
        self.t += 1
        self.m = np.float32(0.9) * self.m + np.float32(0.1) * g
        self.v = np.float32(0.999) * self.v + np.float32(0.001) * g * g
        c1 = np.float32(1.0 - 0.9 ** self.t)
        c2 = np.float32(1.0 - 0.999 ** self.t)
        self.w = (self.w - np.float32(self.lr) * (self.m / c1) / (np.sqrt(self.v / c2) + np.float32(1e-8))).astype(np.float32)
        return float(sum(float(l[0]) * len(p) for l, p in zip(losses, parts)) / len(s))


def voxel_reads():
    """Voxel reads per pass since the last call: features, initial, temporal, spatial, final,
    reference, (unused), and the learned-target select share (p_hat of the winner)."""
    out = np.zeros(8, np.uint64)
    lib().vro_voxel_reads(_ptr(out))
    return out


def math_op(op, a, b=None):
    a = np.ascontiguousarray(a, np.float32)
    out = np.zeros_like(a)
    bb = np.ascontiguousarray(b, np.float32) if b is not None else None
    lib().vro_math(op, _ptr(a), _ptr(bb) if bb is not None else None, _ptr(out), a.size)
    return out


def rng(cases, draws):
    cases = np.ascontiguousarray(cases, np.uint32)
    out = np.zeros((len(cases), draws), np.float32)
    lib().vro_rng(_ptr(cases), len(cases), draws, _ptr(out))
    return out


def net_forward(params, box, floor, queries):
    """CPU network: T for (n, 8) query records (index-order FP32 accumulation)."""
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 8)
    P = np.ascontiguousarray(params, np.float32)
    b0, b1 = [np.ascontiguousarray(b, np.float32) for b in box]
    out = np.zeros(len(q), np.float32)
    lib().vro_net_forward(_ptr(P), _ptr(b0), _ptr(b1), float(floor), _ptr(q), len(q), _ptr(out))
    return out


def net_gradients(params, box, samples, loss_log=0, floor=0.02):
    """Loss and gradient of the training step with the training kernel's numerics."""
    s = np.ascontiguousarray(samples, np.float32).reshape(-1, 8)
    P = np.ascontiguousarray(params, np.float32)
    b0, b1 = [np.ascontiguousarray(b, np.float32) for b in box]
    g = np.zeros(len(P), np.float32)
    loss = np.zeros(1, np.float32)
    lib().vro_net_gradients(_ptr(P), _ptr(b0), _ptr(b1), _ptr(s), len(s), int(loss_log), float(floor), _ptr(g), _ptr(loss))
    return float(loss[0]), g
