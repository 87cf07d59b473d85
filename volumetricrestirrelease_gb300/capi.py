"""ctypes binding of the C ABI declared in include/vrestir.h (libvrestir.so).

The library is the in-tree build of the CUDA kernels (volumetricrestirrelease_gb300/_lib/).
Loading fails loudly if it is missing: there is no CPU fallback for the frame loop.
"""
import ctypes as C
import os
import pathlib

PKG = pathlib.Path(__file__).resolve().parent
DEFAULT_LIB = PKG / "_lib" / "libvrestir.so"

VR_OK, VR_ERR_INVALID_ARG, VR_ERR_OOM, VR_ERR_CUDA, VR_ERR_LOOP_LIMIT, VR_ERR_UNSUPPORTED, VR_ERR_STATE = range(7)
VR_MIS_NONE, VR_MIS_TALBOT = 0, 1
VR_SAMPLER_HAMMERSLEY, VR_SAMPLER_R2 = 0, 1
(VR_TRACK_RATIO, VR_TRACK_ANALYTIC, VR_TRACK_RAY_MARCHING, VR_TRACK_RESIDUAL_RATIO,
 VR_TRACK_ANALOG_RESIDUAL_RATIO) = range(5)
VR_REPROJ_LINEAR, VR_REPROJ_NONE, VR_REPROJ_NO_BACKGROUND = range(3)
VR_NUM_MAX_MIPS = 8
VR_NUM_SLOTS = 16

_i32, _u32, _f32 = C.c_int32, C.c_uint32, C.c_float


class Options(C.Structure):
    """vr_options: the option surface of VolumetricReSTIRParams (VolumetricReSTIR.h:130-207)."""
    _fields_ = [
        ("mMaxBounces", _i32), ("mEnableTemporalReuse", _i32), ("mEnableSpatialReuse", _i32),
        ("mUseReference", _i32), ("mUseEnvironmentLights", _i32), ("mUseAnalyticLights", _i32),
        ("mBaselineSamplePerPixel", _i32), ("mVisualizeTotalTransmittance", _i32),
        ("mInitialBaseMipLevel", _i32), ("mInitialM", _i32), ("mInitialLightSamples", _i32),
        ("mInitialLightingMipLevel", _i32), ("mInitialVisibilityUseLinearSampler", _i32),
        ("mInitialLightingUseLinearSampler", _i32), ("mInitialLightingTrackingMethod", _u32),
        ("mInitialVisibilityTStepScale", _f32), ("mInitialLightingTStepScale", _f32),
        ("mInitialUseRussianRoulette", _i32), ("mInitialUseCoarserGridForIndirectBounce", _i32),
        ("mTemporalReuseMThreshold", _f32), ("mTemporalReprojectionMode", _u32), ("mTemporalMISMethod", _u32),
        ("mTemporalReprojectionMipLevel", _i32), ("mSpatialReuseRounds", _i32), ("mSpatialVisibilityMipLevel", _i32),
        ("mSpatialLightingMipLevel", _i32), ("mSpatialVisibilityUseLinearSampler", _i32),
        ("mSpatialLightingUseLinearSampler", _i32), ("mSpatialVisibilityTStepScale", _f32),
        ("mSpatialLightingTStepScale", _f32), ("mSpatialVisibilityTrackingMethod", _u32),
        ("mSpatialLightingTrackingMethod", _u32), ("mRandomSamplerType", _u32), ("mSampleRadius", _f32),
        ("mSpatialSampleCount", _i32), ("mSpatialMISMethod", _u32), ("mFinalLightSamples", _i32),
        ("mFinalVisibilitySamples", _i32), ("mFinalVisibilityTrackingMethod", _u32),
        ("mFinalLightTrackingMethod", _u32), ("mFinalTStepScale", _f32),
        ("mUseLearnedPHat", _i32), ("mLearnedTrainSamples", _i32), ("mLearnedBatch", _i32),
        ("mLearnedLearningRate", _f32), ("mLearnedTFloor", _f32), ("mLearnedSeed", _u32),
        ("mLearnedTargetMethod", _u32), ("mLearnedLoss", _i32), ("mUsePrevVolumeForReproj", _i32),
        ("mVertexReuse", _i32), ("mVertexReuseStartBounce", _i32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Medium(C.Structure):
    _fields_ = [("sigma_a", _f32 * 3), ("sigma_s", _f32 * 3), ("g", _f32), ("density_scale", _f32)]


class ProceduralDesc(C.Structure):
    _fields_ = [("kind", _i32), ("res", _i32), ("num_mips", _i32), ("octaves", _i32), ("seed", _u32),
                ("lacunarity", _f32), ("gain", _f32), ("base_frequency", _f32), ("mask_radius", _f32),
                ("threshold", _f32), ("world_min", _f32 * 3), ("voxel_size", _f32), ("fp16", _i32)]


class GridView(C.Structure):
    _fields_ = [("valid", _i32), ("res", _i32 * 3), ("bmin", _f32 * 3), ("bmax", _f32 * 3),
                ("world_to_index", _f32 * 16), ("max_value", _f32), ("num_l1", _i32), ("num_bricks", _i32),
                ("root_child", C.POINTER(_i32)), ("l1_vmin", C.POINTER(_i32)), ("l1_child", C.POINTER(_i32)),
                ("brick_vmin", C.POINTER(_i32)), ("brick_bounds", C.POINTER(_f32)),
                ("brick_f32", C.POINTER(_f32)), ("brick_f16", C.POINTER(C.c_uint16)),
                ("brick_bc4", C.POINTER(C.c_uint64)), ("bc4_scale", _f32)]


class VolumeInfo(C.Structure):
    _fields_ = [("num_mips", _i32), ("res", _i32), ("voxel_size", _f32), ("supervoxel_diag", _f32),
                ("num_bricks", _i32 * VR_NUM_SLOTS), ("device_bytes", C.c_int64), ("fp16", _i32), ("world_min", _f32 * 3),
                ("bc4", _i32)]


# void (*)(void* user, float* rgba, float* mvec, int32_t width, int32_t height, void* stream)
FRAME_HOOK = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_void_p, _i32, _i32, C.c_void_p)


class PointLight(C.Structure):
    _fields_ = [("pos", _f32 * 3), ("intensity", _f32 * 3)]


class EnvMap(C.Structure):
    _fields_ = [("rgb", C.POINTER(_f32)), ("width", _i32), ("height", _i32), ("scale", _f32 * 3),
                ("rotation", _f32 * 9)]


class Camera(C.Structure):
    _fields_ = [("pos", _f32 * 3), ("target", _f32 * 3), ("up", _f32 * 3), ("fov_y", _f32),
                ("near_z", _f32), ("far_z", _f32)]


class ReservoirAoS(C.Structure):
    _fields_ = [("runningSum", _f32), ("M", _f32), ("depth", _f32), ("p_y", _f32), ("lightUV", _f32 * 2),
                ("lightID", _i32), ("sampledPixel", _i32), ("extraBounceStartId", _i32), ("p_partial", _f32)]


# exported entry points and their signatures (include/vrestir.h)
_P = C.c_void_p
SIGNATURES = {
    "vr_options_default": (None, [C.POINTER(Options)]),
    "vr_volume_create_procedural": (_i32, [C.POINTER(ProceduralDesc), C.POINTER(_P)]),
    "vr_volume_create_fire": (_i32, [C.POINTER(ProceduralDesc), _f32, _f32, C.POINTER(_P), C.POINTER(_P)]),
    "vr_blackbody_lut": (None, [C.POINTER(_f32)]),
    "vr_set_emission": (_i32, [_P, _P, _f32, _f32, _f32, C.POINTER(_f32)]),
    "vr_volume_create_dense": (_i32, [C.POINTER(_f32), _i32, _i32, C.POINTER(_f32), _f32, _i32, C.POINTER(_P)]),
    "vr_volume_destroy": (None, [_P]),
    "vr_volume_compress_bc4": (_i32, [_P]),
    "vr_set_frame_hook": (_i32, [_P, _P, _P]),
    "vr_volume_get_info": (_i32, [_P, C.POINTER(VolumeInfo)]),
    "vr_volume_get_slot": (_i32, [_P, _i32, C.POINTER(GridView)]),
    "vr_create": (_P, [C.POINTER(Options), _i32, _i32, C.POINTER(_i32)]),
    "vr_destroy": (None, [_P]),
    "vr_last_error": (C.c_char_p, [_P]),
    "vr_set_options": (_i32, [_P, C.POINTER(Options)]),
    "vr_get_options": (_i32, [_P, C.POINTER(Options)]),
    "vr_resize": (_i32, [_P, _i32, _i32]),
    "vr_set_volume": (_i32, [_P, _P, C.POINTER(Medium)]),
    "vr_set_lights": (_i32, [_P, C.POINTER(PointLight), _i32, C.POINTER(EnvMap)]),
    "vr_render_frame": (_i32, [_P, C.POINTER(Camera), _P, _P, _P]),
    "vr_render_frame_host": (_i32, [_P, C.POINTER(Camera), C.POINTER(_f32), _P]),
    "vr_render_reference": (_i32, [_P, C.POINTER(Camera), _i32, _i32, _P, _P]),
    "vr_render_frame_noalloc": (_i32, [_P, C.POINTER(Camera), _i32, _P, _P]),
    "vr_reservoir_bytes": (_i32, [_P]),
    "vr_export_reservoirs": (_i32, [_P, _i32, _P, C.c_size_t]),
    "vr_export_extra_bounces": (_i32, [_P, _i32, C.POINTER(_f32), C.c_size_t]),
    "vr_export_features": (_i32, [_P, _P, C.c_size_t]),
    "vr_state_bytes": (C.c_int64, [_P]),
    "vr_export_state": (_i32, [_P, _P, C.c_size_t]),
    "vr_import_state": (_i32, [_P, _P, C.c_size_t]),
    "vr_frame_count": (_i32, [_P]),
    "vr_last_timings": (_i32, [_P, C.POINTER(_f32), _i32, C.POINTER(_i32)]),
    "vr_last_launch_count": (_i32, [_P]),
    "vr_kernel_time_totals": (_i32, [_P, C.POINTER(_f32), _i32, C.POINTER(_i32), _i32]),
    "vr_last_transfer_bytes": (_i32, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "vr_selftest_math": (_i32, [_i32, C.POINTER(_f32), C.POINTER(_f32), C.POINTER(_f32), _i32]),
    "vr_selftest_rng": (_i32, [C.POINTER(_u32), _i32, _i32, C.POINTER(_f32)]),
    "vr_selftest_umma": (_i32, [C.POINTER(C.c_uint16), C.POINTER(C.c_uint16), C.POINTER(_f32), _i32]),
    "vr_set_block_size": (_i32, [_P, _i32]),
    "vr_set_animation": (_i32, [_P, C.POINTER(_P), _i32, C.POINTER(_P), C.POINTER(_P), _f32]),
    "vr_render_frame_host_async": (_i32, [_P, C.POINTER(Camera), C.POINTER(_f32), _P]),
    "vr_host_frames_wait": (_i32, [_P]),
    "vr_debug_fail_allocation": (None, [_i32]),
    "vr_volume_create_dense_signed": (_i32, [_P, _i32, C.POINTER(_f32), _f32, _i32, C.POINTER(_P)]),
    "vr_volume_load_vbx": (_i32, [C.c_char_p, _i32, _i32, C.POINTER(_P)]),
    "vr_volume_save_vbx": (_i32, [_P, C.c_char_p]),
    "vr_volume_vbx_error": (C.c_char_p, []),
    "vr_accumulator_create": (_i32, [_i32, _i32, _i32, C.POINTER(_P)]),
    "vr_accumulator_destroy": (None, [_P]),
    "vr_accumulator_reset": (None, [_P]),
    "vr_accumulator_count": (C.c_int64, [_P]),
    "vr_accumulate": (_i32, [_P, _P, _P, _P]),
    "vr_error_measure": (_i32, [_P, _P, _P, _i32, _i32, _i32, _f32, C.POINTER(C.c_double), _P, _P]),
    "vr_animation_frame": (_i32, [_P]),
    "vr_batch_create": (_i32, [C.POINTER(_P), _i32, C.POINTER(_P)]),
    "vr_batch_destroy": (None, [_P]),
    "vr_batch_last_error": (C.c_char_p, [_P]),
    "vr_batch_render": (_i32, [_P, C.POINTER(Camera), C.POINTER(_P), _P]),
    "vr_batch_set_graph": (_i32, [_P, _i32]),
    "vr_batch_set_launch_shape": (_i32, [_P, _i32, _i32]),
    "vr_batch_get_launch_shape": (_i32, [_P, C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_i32)]),
    "vr_batch_autotune": (_i32, [_P, C.POINTER(Camera), C.POINTER(_P), _P, C.POINTER(_f32), _i32]),
    "vr_batch_last_launch_count": (_i32, [_P]),
    "vr_net_get_params": (_i32, [_P, C.POINTER(_f32)]),
    "vr_net_set_params": (_i32, [_P, C.POINTER(_f32)]),
    "vr_net_infer": (_i32, [_P, _P, _i32, _P, _P]),
    "vr_net_gradients": (_i32, [_P, _P, _i32, C.POINTER(_f32), C.POINTER(_f32)]),
    "vr_net_train_step": (_i32, [_P, _P, _i32, C.POINTER(_f32)]),
    "vr_export_learned": (_i32, [_P, _i32, _P, C.c_size_t, C.POINTER(C.c_int64)]),
}

NET_PARAMS = 16705

_LIB = None


def load(path=None):
    """Loads libvrestir.so (default: the in-tree build) and sets all signatures."""
    global _LIB
    if path is None and _LIB is not None:
        return _LIB
    p = pathlib.Path(path or os.environ.get("VRESTIR_LIB", DEFAULT_LIB))
    if not p.exists():
        raise RuntimeError(f"libvrestir.so not built ({p}); run __graft_entry__.build() -- there is no CPU fallback")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def default_options(lib=None):
    o = Options()
    (lib or load()).vr_options_default(C.byref(o))
    return o
