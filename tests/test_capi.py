"""The C-ABI library loads and exports every entry point include/vrestir.h declares; host-side
option handling (no GPU calls)."""
import ctypes as C
import pathlib
import re

from volumetricrestirrelease_gb300 import capi

HEADER = pathlib.Path(__file__).resolve().parents[1] / "include" / "vrestir.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vr_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "vr_render_frame" in syms and "vr_create" in syms and len(syms) >= 25


def test_library_exports_every_declared_symbol(vlib):
    missing = [s for s in declared_symbols() if not hasattr(vlib, s)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_header():
    assert set(declared_symbols()) <= set(capi.SIGNATURES), set(declared_symbols()) - set(capi.SIGNATURES)


def test_default_options_match_reference(vlib):
    # VolumetricReSTIR.h:130-207 defaults
    o = capi.default_options(vlib)
    assert o.mMaxBounces == 1 and o.mEnableTemporalReuse == 1 and o.mEnableSpatialReuse == 1
    assert o.mInitialM == 4 and o.mInitialBaseMipLevel == 1 and o.mInitialLightingMipLevel == 2
    assert o.mInitialVisibilityUseLinearSampler == 0 and o.mInitialLightingUseLinearSampler == 1
    assert o.mInitialLightingTrackingMethod == capi.VR_TRACK_RAY_MARCHING
    assert abs(o.mInitialLightingTStepScale - 2.0) < 1e-7 and o.mTemporalReuseMThreshold == 4.0
    assert o.mSpatialSampleCount == 4 and o.mSampleRadius == 10.0 and o.mRandomSamplerType == capi.VR_SAMPLER_R2
    assert o.mFinalVisibilityTrackingMethod == capi.VR_TRACK_ANALYTIC and abs(o.mFinalTStepScale - 0.2) < 1e-7
    assert o.mUseEnvironmentLights == 1 and o.mUseAnalyticLights == 0 and o.mSpatialMISMethod == capi.VR_MIS_TALBOT


def test_struct_sizes_match_header():
    assert C.sizeof(capi.ReservoirAoS) == 40
    assert C.sizeof(capi.PointLight) == 24
    assert C.sizeof(capi.Camera) == 48


def test_volume_arguments_rejected(vlib):
    from volumetricrestirrelease_gb300 import scenes
    d = scenes.small().volume
    d.res = 100                       # not a multiple of 8 * 2^(mips-1)
    h = C.c_void_p()
    assert vlib.vr_volume_create_procedural(C.byref(d), C.byref(h)) == capi.VR_ERR_INVALID_ARG
    d = scenes.small().volume
    d.num_mips = 9
    assert vlib.vr_volume_create_procedural(C.byref(d), C.byref(h)) == capi.VR_ERR_INVALID_ARG
    assert vlib.vr_volume_create_procedural(None, C.byref(h)) == capi.VR_ERR_INVALID_ARG
