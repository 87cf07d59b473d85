// vr_oracle.cpp -- CPU restatement of the VolumetricReSTIR per-frame loop.
//
// TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU path is checked against and the
// timed CPU baseline of bench.py; nothing in the product library links or calls it.
//
// It transcribes, function by function and in the same operation order, the reference's
// shader logic (paths relative to the reference repository; RP = Source/RenderPasses/
// VolumetricReSTIR, FS = Source/Falcor):
//   RP/TraceRays.cs.slang, RP/ComputeInitialSample.slang, RP/TemporalReuse.cs.slang,
//   RP/SpatialReuse.cs.slang, RP/CopyReservoirs.cs.slang, RP/FinalShading.cs.slang,
//   RP/GenerateFeatures.cs.slang, RP/Reservoir.slang, RP/ReSTIRHelper.slang,
//   RP/VolumeUtils.slang, RP/VolumeTrackingAdapterGVDB.slang, RP/VolumeBase.slang,
//   RP/VolumePathTracingFunctions.slang, FS/Scene/GVDB/{gvdb,gvdbNodes,gvdbDda}.slang,
//   FS/Scene/Camera/Camera.slang, FS/Experimental/Scene/Lights/{EnvMap,EnvMapSampler,
//   EnvMapSamplerSetup.cs,LightHelpers}.slang, FS/Utils/Math/MathHelpers.slang,
//   FS/Utils/Helpers.slang, and the pass driver RP/VolumetricReSTIR.cpp:303-906.
// Surface scenes, vertex reuse, mesh lights and animated volumes are outside the path.
//
// Parity: the reference itself cannot run here (D3D12 + Slang only), so this restatement
// is pinned only through the RNG known-answer vectors of the reference's own generator
// sources and through analytic known answers; see tests/.  Texture hardware filtering
// and BC4 atlas compression are replaced by software trilinear on FP32/FP16 bricks.
// Elementary functions come from the project's deterministic math header (vr_math.h).
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <thread>
#include <vector>

#include "../include/vrestir.h"
#include "../volumetricrestirrelease_gb300/csrc/vr_math.h"

using namespace vr;

namespace oracle {

static const float kRayTMax = FLT_MAX;                  // VolumeBase.slang:11
static const int kSelfEmissionLightID = -3;             // HostDeviceSharedConstants.slang:19
static const int kNumMaxMips = 8;
static const float kM_PI = 3.14159265358979323846f;
static const float kM_2PI = 6.28318530717958647693f;
static const float kM_PI_4 = 0.785398163397448309616f;
static const float kM_1_PI = 0.318309886183790671538f;
static const float kM_1_2PI = 0.159154943091895335769f;
static const float kM_1_4PI = 0.079577471545947667884f;
static const int kMaxBrickSteps = 128;                  // VolumeTrackingAdapterGVDB.slang:4
static const int kMaxDeltaIters = 1 << 20;              // bound on delta-tracking loops

// ---------------------------------------------------------------------------------------
// Reservoir (HostDeviceSharedDefinitions.h:16-45, Reservoir.slang)
// ---------------------------------------------------------------------------------------
struct Reservoir {
    float runningSum, M, depth, p_y;
    float lightUV[2];
    int lightID, sampledPixel, extraBounceStartId;
    float p_partial;            // vertex reuse: the suffix's share of p_hat (HostDeviceSharedDefinitions.h:29-31)
};
static Reservoir createNewReservoir() {                 // Reservoir.slang:19-23
    Reservoir r;
    r.runningSum = 0.f; r.M = 0.f; r.depth = FLT_MAX; r.p_y = 0.f;
    r.lightUV[0] = 0.f; r.lightUV[1] = 0.f; r.lightID = 0; r.sampledPixel = 0;
    r.extraBounceStartId = 0;
    r.p_partial = 0.f;
    return r;
}
static void copySample(const Reservoir& from, Reservoir& to) {
    to.depth = from.depth; to.p_y = from.p_y;
    to.lightUV[0] = from.lightUV[0]; to.lightUV[1] = from.lightUV[1];
    to.lightID = from.lightID; to.extraBounceStartId = from.extraBounceStartId;
    to.sampledPixel = from.sampledPixel;
    to.p_partial = from.p_partial;          // Reservoir.slang:46-48, 76-78 (vertex reuse)
}
// Reservoir.slang:26-57
static bool simpleResampleStep(const Reservoir& reservoir, Reservoir& state, Rng& sg) {
    float sampleWeight = reservoir.runningSum;
    state.M += reservoir.M;
    if (sampleWeight <= 0.0f) return false;
    state.runningSum += sampleWeight;
    bool selectSample = next1D(sg) * state.runningSum < sampleWeight;
    if (selectSample) copySample(reservoir, state);
    return selectSample;
}
// simpleResampleStep with its uniform drawn beforehand (the learned-target pass)
static bool simpleResampleStepU(const Reservoir& reservoir, Reservoir& state, float u) {
    float w = reservoir.runningSum;
    state.M += reservoir.M;
    if (w <= 0.0f) return false;
    state.runningSum += w;
    bool sel = u * state.runningSum < w;
    if (sel) copySample(reservoir, state);
    return sel;
}
// Reservoir.slang:59-87
static bool simpleResampleStepWithMaxM(const Reservoir& reservoir, float MThreshold, Reservoir& state, Rng& sg) {
    float correctedM = fmin_(MThreshold, reservoir.M);
    float sampleWeight = correctedM == 0.0f ? 0.0f : correctedM / reservoir.M * reservoir.runningSum;
    state.M += correctedM;
    if (sampleWeight <= 0.0f) return false;
    state.runningSum += sampleWeight;
    bool selectSample = next1D(sg) * state.runningSum < sampleWeight;
    if (selectSample) copySample(reservoir, state);
    return selectSample;
}

struct Features { int noReflectiveSurface; float transmittance; };   // HostDeviceSharedDefinitions.h:66-70

// ---------------------------------------------------------------------------------------
// codecs (ReSTIRHelper.slang:10-89)
// ---------------------------------------------------------------------------------------
static f3 decodeEmissivePosition(int lightID, const float lightUV[2]) {
    return mk3(lightUV[0], lightUV[1], asfloat(lightID));
}
static void encodeEmissivePosition(f3 pos, int& lightID, float lightUV[2]) {
    lightID = asint(pos.z); lightUV[0] = pos.x; lightUV[1] = pos.y;
}
struct f4 { float x, y, z, w; };
static f4 decodeWiDist(f3 input, bool reuseAsVertex = false) {     // ReSTIRHelper.slang:21-39
    if (reuseAsVertex) {
        if (input.x == kRayTMax) return f4{0.f, 0.f, 0.f, kRayTMax};
        return f4{input.x, input.y, input.z, -1.f};
    }
    f3 wi;
    wi.x = input.x; wi.y = input.y;
    wi.z = sqrt_(1.0f - (input.x * input.x + input.y * input.y));
    if (isnan_(wi.z)) wi.z = 0.f;
    if (input.z < 0) { wi.z = -wi.z; input.z = -input.z; }
    return f4{wi.x, wi.y, wi.z, input.z};
}
static f3 encodeWiDist(f3 dir, float dist) {
    f3 wi = mk3(dir.x, dir.y, dist);
    if (dir.z < 0) wi.z = -wi.z;
    return wi;
}
static int decodeMaxIndirectBounces(int storage, int maxBounces) {
    return maxBounces == 1 ? 0 : (storage >> 20);
}
static int encodeMaxIndirectBounces(int storage, int bounce) { return (bounce << 20) | (storage & 0xFFFFF); }
static int decodePathTag(int storage) { return (storage >> 16) & 0xF; }
static int encodePathTag(int storage, int tag) { return (tag << 16) | (storage & (int)0xFFF0FFFF); }

// ---------------------------------------------------------------------------------------
// scene data
// ---------------------------------------------------------------------------------------
struct Ray { f3 origin, dir; float tMin, tMax; f3 at(float t) const { return origin + dir * t; } };

struct Slot {
    bool valid = false;
    int res[3] = {0, 0, 0};
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
    float M[16];
    float maxValue = 0.f;
    std::vector<int32_t> root, l1vmin, l1child, bvmin;
    std::vector<float> bounds, data;      // data: 1000 per brick, decoded to float
};

struct EnvMap {
    std::vector<float> rgb;  // width*height*3
    int w = 0, h = 0;
    f3 scale;
    float rot[9];            // local->world (row-vector)
    float inv[9];            // world->local
    // importance map: 512x512 with full mip chain (EnvMapSampler.cpp:83-100)
    int impDim = 512, baseMip = 9;
    std::vector<std::vector<float>> imp;   // imp[m] is (512>>m)^2
};

struct CamFrame {
    f3 posW, U, V, W;
    float view[16], proj[16];   // column-major as glm
};

struct MediumI {
    float sigma_t;
    f3 sigma_s, sigma_a;
    float g;
    float dscale;
    float tStep;           // world voxel size at mip 0
    float superDiag;
    int numMips;
};

struct Emission {             // VolumeDesc.hasEmission, LeScale, temperatureCutOff/Scale + the LUT
    bool has = false;
    Slot slot;                 // temperature grid, mip 0
    bool lastHas = false;      // VolumeDesc.lastFrameHasEmission
    Slot prevSlot;             // the previous animation frame's temperature grid
    float leScale = 0.f, cutoff = 0.f, scale = 1.f;
    float lut[128][3];
};

// slots [kPrevSlotOffset, kPrevSlotOffset + VR_NUM_SLOTS): the previous animation frame's mips
// (the role of kPrevFrameDensityGridOffset, HostDeviceSharedConstants.slang:27)
constexpr int kPrevSlotOffset = VR_NUM_SLOTS;

struct Scene {
    Slot slots[2 * VR_NUM_SLOTS];
    MediumI med;
    // VolumeDesc.hasAnimation / usePrevGridForReproj / hasVelocity / velocityScale
    bool hasAnimation = false, usePrevGrid = true, hasVelocity = false;
    float velocityScale = 1.f;
    Slot vel[3];               // velocity components, world units per frame
    std::vector<vr_point_light> lights;
    EnvMap env;
    bool hasEnv = false;
    Emission emis;
};

// ---------------------------------------------------------------------------------------
// matrices: mul(float4(v), M) with M stored row-major, row-vector convention
// ---------------------------------------------------------------------------------------
static f3 mulPoint(f3 p, const float* M, float* wOut = nullptr) {
    float o[4];
    for (int j = 0; j < 4; ++j) o[j] = p.x * M[0 * 4 + j] + p.y * M[1 * 4 + j] + p.z * M[2 * 4 + j] + 1.0f * M[3 * 4 + j];
    if (wOut) *wOut = o[3];
    return mk3(o[0] / o[3], o[1] / o[3], o[2] / o[3]);
}
static f3 mulVec(f3 d, const float* M) {
    float o[3];
    for (int j = 0; j < 3; ++j) o[j] = d.x * M[0 * 4 + j] + d.y * M[1 * 4 + j] + d.z * M[2 * 4 + j] + 0.0f * M[3 * 4 + j];
    return mk3(o[0], o[1], o[2]);
}
static f3 mul33(f3 d, const float* R) {
    return mk3(d.x * R[0] + d.y * R[3] + d.z * R[6], d.x * R[1] + d.y * R[4] + d.z * R[7],
               d.x * R[2] + d.y * R[5] + d.z * R[8]);
}

// ---------------------------------------------------------------------------------------
// GVDB lookups (gvdb.slang, gvdbNodes.slang, VolumeBase.slang) on the restated brick grid
// ---------------------------------------------------------------------------------------
static const int kLevDim[3] = {3, 4, 5};
static const int kLevRes[3] = {8, 16, 32};
static const float kLevVdel[3] = {1.f, 8.f, 128.f};

static Ray WorldToMedium(const Scene& sc, const Ray& r, int mip) {          // VolumeBase.slang:97-103
    Ray o;
    o.origin = mulPoint(r.origin, sc.slots[mip].M);
    o.dir = mulVec(r.dir, sc.slots[mip].M);
    o.tMin = r.tMin; o.tMax = r.tMax;
    return o;
}
static f3 WorldToMediumP(const Scene& sc, f3 p, int mip) { return mulPoint(p, sc.slots[mip].M); }

// getChild (gvdbNodes.slang:114-120); lev 2 = root, lev 1 = level-1 node.  Flat indices
// outside the stored lists read as empty.
static int getChild(const Slot& s, int nodeId, int clev, int b) {
    if (clev == 2) {
        if (b < 0 || b >= 32768) return -1;
        return s.root[b];
    }
    if (b < 0 || b >= 4096) return -1;
    return s.l1child[(size_t)nodeId * 4096 + b];
}
static f3 nodeVmin(const Slot& s, int lev, int id) {
    if (lev == 2) return mk3(0.f);
    if (lev == 1) return mk3((float)s.l1vmin[id * 4], (float)s.l1vmin[id * 4 + 1], (float)s.l1vmin[id * 4 + 2]);
    return mk3((float)s.bvmin[id * 4], (float)s.bvmin[id * 4 + 1], (float)s.bvmin[id * 4 + 2]);
}

// instrumentation: voxel reads per pass (algorithmic brick bytes for the roofline)
// voxel reads per pass (instrumentation for the roofline's algorithmic bytes); a pass may
// attribute part of its reads to another counter through tl_voxSplit
static thread_local uint64_t tl_voxReads = 0;
static thread_local uint64_t tl_voxSplit = 0;
static std::atomic<uint64_t> g_voxReads[8];
static float voxel(const Slot& s, int brick, int x, int y, int z) {     // local coords in [-1, 8]
    ++tl_voxReads;
    x = std::min(std::max(x, -1), 8); y = std::min(std::max(y, -1), 8); z = std::min(std::max(z, -1), 8);
    return s.data[(size_t)brick * 1000 + ((z + 1) * 10 + (y + 1)) * 10 + (x + 1)];
}
static float lerp_(float a, float b, float t) { return a + (b - a) * t; }
// software trilinear filter at brick-local position p (voxel centres at integer + 0.5)
static float trilinear(const Slot& s, int brick, f3 p) {
    float qx = p.x - 0.5f, qy = p.y - 0.5f, qz = p.z - 0.5f;
    float fx0 = floor_(qx), fy0 = floor_(qy), fz0 = floor_(qz);
    int ix = f2i(fx0), iy = f2i(fy0), iz = f2i(fz0);
    float fx = qx - fx0, fy = qy - fy0, fz = qz - fz0;
    float c000 = voxel(s, brick, ix, iy, iz), c100 = voxel(s, brick, ix + 1, iy, iz);
    float c010 = voxel(s, brick, ix, iy + 1, iz), c110 = voxel(s, brick, ix + 1, iy + 1, iz);
    float c001 = voxel(s, brick, ix, iy, iz + 1), c101 = voxel(s, brick, ix + 1, iy, iz + 1);
    float c011 = voxel(s, brick, ix, iy + 1, iz + 1), c111 = voxel(s, brick, ix + 1, iy + 1, iz + 1);
    float x00 = lerp_(c000, c100, fx), x10 = lerp_(c010, c110, fx);
    float x01 = lerp_(c001, c101, fx), x11 = lerp_(c011, c111, fx);
    float y0 = lerp_(x00, x10, fy), y1 = lerp_(x01, x11, fy);
    return lerp_(y0, y1, fz);
}
static float pointSample(const Slot& s, int brick, f3 p) {
    return voxel(s, brick, f2i(floor_(p.x)), f2i(floor_(p.y)), f2i(floor_(p.z)));
}
// DensityInAtlas (VolumeBase.slang:255-263): the atlas coordinate is the brick-local one
static float DensityInAtlas(const Scene& sc, int mip, int brick, f3 pLocal, bool linear) {
    const Slot& s = sc.slots[mip];
    float v = linear ? trilinear(s, brick, pLocal) : pointSample(s, brick, pLocal);
    return v * 1.0f * sc.med.dscale;
}
// FetchEightVoxelsInAtlas (VolumeBase.slang:245-253) at integer cell p
static void FetchEight(const Scene& sc, int mip, int brick, const int p[3], float v[8]) {
    const Slot& s = sc.slots[mip];
    for (int i = 0; i < 8; ++i)
        v[i] = voxel(s, brick, p[0] + (i % 2), p[1] + (i % 4) / 2, p[2] + i / 4) * 1.0f * sc.med.dscale;
}
// getNodeUnrolledThreeLevel (gvdbNodes.slang:175-223)
static int findBrick(const Slot& s, f3 pos, f3& vmin) {
    f3 v = mk3(0.f);
    if (pos.x < v.x || pos.y < v.y || pos.z < v.z || pos.x >= v.x + 4096.f || pos.y >= v.y + 4096.f || pos.z >= v.z + 4096.f) return -1;
    int px = f2i(pos.x - v.x) / 128, py = f2i(pos.y - v.y) / 128, pz = f2i(pos.z - v.z) / 128;
    int b = (((pz << 5) + py) << 5) + px;
    int l1 = getChild(s, 0, 2, b);
    if (l1 < 0) return -1;
    v = nodeVmin(s, 1, l1);
    if (pos.x < v.x || pos.y < v.y || pos.z < v.z || pos.x >= v.x + 128.f || pos.y >= v.y + 128.f || pos.z >= v.z + 128.f) return -1;
    px = f2i(pos.x - v.x) / 8; py = f2i(pos.y - v.y) / 8; pz = f2i(pos.z - v.z) / 8;
    b = (((pz << 4) + py) << 4) + px;
    int br = getChild(s, l1, 1, b);
    if (br < 0) return -1;
    vmin = nodeVmin(s, 0, br);
    return br;
}
// Density (VolumeBase.slang:234-238) + getValueAtPoint (gvdb.slang:6-27)
static float Density(const Scene& sc, f3 p, int mip) {
    const Slot& s = sc.slots[mip];
    if (p.x < s.bmin[0] || p.y < s.bmin[1] || p.z < s.bmin[2] || p.x >= s.bmax[0] || p.y >= s.bmax[1] || p.z >= s.bmax[2]) return 0.f;
    f3 vmin;
    int br = findBrick(s, p, vmin);
    if (br < 0) return 0.f;
    return trilinear(s, br, p - vmin) * sc.med.dscale;
}
static float DensityWorldSpace(const Scene& sc, f3 p, int mip) { return Density(sc, WorldToMediumP(sc, p, mip), mip); }

// TemperatureWorldSpace / ConvertTempToColor / EmissionWorldSpace (VolumeBase.slang:196-232);
// the LUT's hardware linear filter restated in software: texel centres at (i + 0.5) / 128,
// clamped addressing
static float TemperatureWorldSpace(const Scene& sc, f3 pw, bool isLastFrame = false) {
    const Slot& s = isLastFrame ? sc.emis.prevSlot : sc.emis.slot;
    f3 p = mulPoint(pw, s.M);
    if (p.x < s.bmin[0] || p.y < s.bmin[1] || p.z < s.bmin[2] || p.x >= s.bmax[0] || p.y >= s.bmax[1] || p.z >= s.bmax[2]) return 0.f;
    f3 vmin;
    int br = findBrick(s, p, vmin);
    if (br < 0) return 0.f;
    return trilinear(s, br, p - vmin);
}
static f3 ConvertTempToColor(const Scene& sc, float temp) {
    temp = fmin_(6400.f, (temp - sc.emis.cutoff) * sc.emis.scale);
    const float q = (temp - 25.f) / 6400.f;
    const float x = q * 128.f - 0.5f;
    const float fl = floor_(x);
    const float f = x - fl;
    int i0 = f2i(fl), i1 = i0 + 1;
    i0 = std::min(127, std::max(0, i0));
    i1 = std::min(127, std::max(0, i1));
    const f3 a = mk3(sc.emis.lut[i0][0], sc.emis.lut[i0][1], sc.emis.lut[i0][2]);
    const f3 b = mk3(sc.emis.lut[i1][0], sc.emis.lut[i1][1], sc.emis.lut[i1][2]);
    return sc.emis.leScale * (a + (b - a) * f);
}
static f3 EmissionWorldSpace(const Scene& sc, f3 pw, bool isLastFrame = false) {
    if (isLastFrame ? !sc.emis.lastHas : !sc.emis.has) return mk3(0.f);
    return ConvertTempToColor(sc, TemperatureWorldSpace(sc, pw, isLastFrame));
}
// VelocityWorld (VolumeBase.slang:182-194): trilinear velocity at mip 0 of each component grid,
// zero outside them (NaN coordinates included)
static f3 VelocityWorld(const Scene& sc, f3 pw) {
    float v[3];
    for (int k = 0; k < 3; ++k) {
        const Slot& s = sc.vel[k];
        const f3 p = mulPoint(pw, s.M);
        v[k] = 0.f;
        if (!(p.x >= s.bmin[0] && p.y >= s.bmin[1] && p.z >= s.bmin[2] && p.x < s.bmax[0] && p.y < s.bmax[1] && p.z < s.bmax[2])) continue;
        f3 vmin;
        const int br = findBrick(s, p, vmin);
        if (br >= 0) v[k] = trilinear(s, br, p - vmin);
    }
    return mk3(v[0], v[1], v[2]);
}

// Bounds3f::IntersectP + IntersectVolumeBound (VolumeBase.slang:131-172)
static bool IntersectVolumeBound(const Scene& sc, const Ray& ray, float& tMin, float& tMax, int mip, bool vertexCenter) {
    const Slot& s = sc.slots[mip];
    float pMin[3] = {s.bmin[0], s.bmin[1], s.bmin[2]}, pMax[3] = {s.bmax[0], s.bmax[1], s.bmax[2]};
    if (vertexCenter) for (int i = 0; i < 3; ++i) { pMin[i] -= 0.5f; pMax[i] -= 0.5f; }
    float o[3] = {ray.origin.x, ray.origin.y, ray.origin.z}, d[3] = {ray.dir.x, ray.dir.y, ray.dir.z};
    float t0 = 0, t1 = ray.tMax;
    for (int i = 0; i < 3; ++i) {
        float invRayDir = 1 / d[i];
        float tNear = (pMin[i] - o[i]) * invRayDir;
        float tFar = (pMax[i] - o[i]) * invRayDir;
        if (tNear > tFar) { float tmp = tNear; tNear = tFar; tFar = tmp; }
        t0 = tNear > t0 ? tNear : t0;
        t1 = tFar < t1 ? tFar : t1;
        if (t0 > t1) return false;
    }
    tMin = t0; tMax = t1;
    return true;
}

// ---------------------------------------------------------------------------------------
// HDDA (gvdbDda.slang:86-157)
// ---------------------------------------------------------------------------------------
struct HDDA {
    f3 pos, dir; int pStep[3];
    f3 tDel, t, tSide; int p[3]; int mask[3];
    void SetFromRay(f3 sp, f3 sd, f3 st) {
        pos = sp; dir = sd;
        pStep[0] = dir.x >= 0 ? 1 : -1; pStep[1] = dir.y >= 0 ? 1 : -1; pStep[2] = dir.z >= 0 ? 1 : -1;
        t = st;
    }
    void Prepare(f3 vmin, float vdel) {
        tDel = mk3(fabs_(vdel / dir.x), fabs_(vdel / dir.y), fabs_(vdel / dir.z));
        f3 pFlt = (pos + dir * t.x - vmin) / mk3(vdel);
        f3 fl = mk3(floor_(pFlt.x), floor_(pFlt.y), floor_(pFlt.z));
        tSide = ((fl - pFlt + mk3(0.5f)) * mk3((float)pStep[0], (float)pStep[1], (float)pStep[2]) + mk3(0.5f)) * tDel + mk3(t.x);
        p[0] = f2i(fl.x); p[1] = f2i(fl.y); p[2] = f2i(fl.z);
    }
    void PrepareLeaf(f3 vmin) {
        tDel = mk3(fabs_(1.0f / dir.x), fabs_(1.0f / dir.y), fabs_(1.0f / dir.z));
        f3 pFlt = pos + dir * t.x - vmin;
        f3 fl = mk3(floor_(pFlt.x), floor_(pFlt.y), floor_(pFlt.z));
        tSide = ((fl - pFlt + mk3(0.5f)) * mk3((float)pStep[0], (float)pStep[1], (float)pStep[2]) + mk3(0.5f)) * tDel + mk3(t.x);
        p[0] = f2i(fl.x); p[1] = f2i(fl.y); p[2] = f2i(fl.z);
    }
    // Next (gvdbDda.slang:140-149).  Deviation: when the three side distances are equal (the ray
    // passes through a cell corner) the reference sets no mask, so Step does not move: the node
    // walk then creeps on by epsilon and re-enters the brick, and the voxel walk inside a brick
    // repeats a zero-length step until its step limit, dropping the rest of that brick.  Here
    // the z axis steps, as it does for the tie z == y < x.  Without NaN side distances (a zero
    // direction component gives an infinite one), z is the reference's choice exactly when
    // neither x nor y is, apart from that tie.
    void Next() {
        mask[0] = (tSide.x < tSide.y) & (tSide.x <= tSide.z);
        mask[1] = (tSide.y < tSide.z) & (tSide.y <= tSide.x);
        mask[2] = !(mask[0] | mask[1]);       // (z < x) & (z <= y) in the reference, or the tie
        t.y = mask[0] ? tSide.x : (mask[1] ? tSide.y : tSide.z);
    }
    // Step (gvdbDda.slang:151-156) advances the masked axes by tDel.  The reference writes
    // tSide += float3(mask) * tDel, whose unmasked terms are 0 * inf = NaN for a zero
    // direction component under IEEE arithmetic and stall the walk; the select form below is
    // the intended semantics (and what a non-IEEE-strict shader compiler produces).
    void Step() {
        t.x = t.y;
        tSide = mk3(mask[0] ? tSide.x + tDel.x : tSide.x, mask[1] ? tSide.y + tDel.y : tSide.y, mask[2] ? tSide.z + tDel.z : tSide.z);
        p[0] += mask[0] * pStep[0]; p[1] += mask[1] * pStep[1]; p[2] += mask[2] * pStep[2];
    }
};
static bool inLeaf(const int p[3]) { return p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] < 8 && p[1] < 8 && p[2] < 8; }
static bool inLeafF(f3 p) { return p.x >= 0 && p.y >= 0 && p.z >= 0 && p.x < 8 && p.y < 8 && p.z < 8; }

// VolumeTrackingGVDB (VolumeUtils.slang:171-282)
template <class Adapter>
static void VolumeTrackingGVDB(const Scene& sc, const Ray& rWorld, int mipLevel, Rng& sg, Adapter& adapter, bool vertexCenter) {
    int nodeid[3];
    float tMax[3];
    const float epsilon = 0.01f;
    const Slot& s = sc.slots[mipLevel];
    int lev = 2, topLev = 2;
    nodeid[lev] = 0;
    Ray ray = WorldToMedium(sc, rWorld, mipLevel);
    if (vertexCenter) ray.origin = ray.origin - mk3(0.5f);
    float tNear, tFar;
    if (!IntersectVolumeBound(sc, ray, tNear, tFar, mipLevel, vertexCenter)) { adapter.ExecuteEndStep(); return; }
    adapter.SetRayInfo(tNear, tFar, ray);
    adapter.ExecuteStartStep();
    f3 tStart = mk3(tNear, tFar, 0);
    f3 vmin = nodeVmin(s, lev, nodeid[lev]);
    int node = nodeid[lev];
    tStart.x += epsilon;
    tMax[lev] = tStart.y;
    int iter = 0;
    HDDA dda;
    dda.SetFromRay(ray.origin, ray.dir, tStart);
    dda.Prepare(vmin, kLevVdel[lev]);
    if (vertexCenter) {
        int it2 = 0;
        while (it2++ < 3 && (dda.p[0] < 0 || dda.p[1] < 0 || dda.p[2] < 0 || dda.p[0] > kLevRes[lev] || dda.p[1] > kLevRes[lev] || dda.p[2] > kLevRes[lev])) {
            dda.Next(); dda.Step(); dda.t.x += epsilon;
        }
    }
    float t = tNear;
    for (; iter < 4096 && lev > 0 && lev <= topLev &&
           (dda.p[0] >= 0 && dda.p[1] >= 0 && dda.p[2] >= 0 && dda.p[0] <= kLevRes[lev] && dda.p[1] <= kLevRes[lev] && dda.p[2] <= kLevRes[lev]);
         iter++) {
        dda.Next();
        int b = (((dda.p[2] << kLevDim[lev]) + dda.p[1]) << kLevDim[lev]) + dda.p[0];
        int child = getChild(s, node, lev, b);
        if (child >= 0) {
            if (lev == 1) {
                nodeid[0] = child;
                t = dda.t.x - epsilon;
                // Deviation from VolumeUtils.slang:240-249: stop when the next occupied brick
                // starts beyond tFar.  The reference enters it with t > tFar, and the analytic
                // and residual-ratio adapters then integrate over a negative interval
                // (t_dist = tFar - t < 0), returning transmittances far above 1 (up to e^60
                // observed: fireflies of 1e26 in the final shading).
                if (t >= tFar) break;
                f3 vmin_leaf = nodeVmin(s, 0, child);
                float bnd[4];
                for (int k = 0; k < 4; ++k) bnd[k] = s.bounds[(size_t)child * 4 + k] * sc.med.dscale;
                bool shouldExit = adapter.ExecuteMainStep(dda, vmin_leaf, child, bnd, mipLevel, t, sg);
                if (shouldExit) return;
                dda.Step();
                dda.t.x += epsilon;
            } else {
                lev--;
                nodeid[lev] = child;
                node = child;
                vmin = nodeVmin(s, lev, child);
                tMax[lev] = dda.t.y;
                dda.Prepare(vmin, kLevVdel[lev]);
            }
        } else {
            dda.Step();
            dda.t.x += epsilon;
        }
        while (lev <= topLev && dda.t.x > tMax[lev]) {
            lev++;
            if (lev <= topLev) {
                node = nodeid[lev];
                vmin = nodeVmin(s, lev, node);
                dda.Prepare(vmin, kLevVdel[lev]);
            }
        }
    }
    adapter.ExecuteEndStep();
}

// ---------------------------------------------------------------------------------------
// adapters (VolumeTrackingAdapterGVDB.slang)
// ---------------------------------------------------------------------------------------
// trilinear optical-depth polynomial coefficients (VolumeTrackingAdapterGVDB.slang:59-99)
static void trilinearCoeffs(const float v[8], f3 d, f3 p0, float& c3, float& c2, float& c1, float& c0) {
    float v_000 = v[0], v_100 = v[1], v_010 = v[2], v_110 = v[3];
    float v_001 = v[4], v_101 = v[5], v_011 = v[6], v_111 = v[7];
    float mxyz = v_111 - v_011 - v_101 - v_110 + v_100 + v_010 + v_001 - v_000;
    float mxy = v_000 - v_100 - v_010 + v_110;
    float mxz = v_000 - v_100 - v_001 + v_101;
    float myz = v_000 - v_010 - v_001 + v_011;
    float mx = v_100 - v_000;
    float my = v_010 - v_000;
    float mz = v_001 - v_000;
    c3 = mxyz * d.x * d.y * d.z;
    c2 = (p0.z * d.x * d.y + p0.y * d.x * d.z + p0.x * d.y * d.z) * mxyz + mxy * d.x * d.y + mxz * d.x * d.z + myz * d.y * d.z;
    c1 = (p0.y * p0.z * d.x + p0.x * p0.z * d.y + p0.x * p0.y * d.z) * mxyz +
         mx * d.x + my * d.y + mz * d.z + (p0.y * d.x + p0.x * d.y) * mxy + (p0.z * d.x + p0.x * d.z) * mxz + (p0.z * d.y + p0.y * d.z) * myz;
    c0 = p0.x * p0.y * p0.z * mxyz + p0.x * p0.y * mxy + p0.x * p0.z * mxz + p0.y * p0.z * myz + p0.x * mx + p0.y * my + p0.z * mz + v_000;
}
static void fetchSigma(const Scene& sc, int mip, int brick, const int p[3], float v[8]) {
    FetchEight(sc, mip, brick, p, v);
    for (int i = 0; i < 8; ++i) v[i] *= sc.med.sigma_t;
}
static f3 leafP0(const HDDA& d, f3 vmin_leaf) {
    return d.pos + d.t.x * d.dir - (mk3((float)d.p[0], (float)d.p[1], (float)d.p[2]) + vmin_leaf);
}
static f3 cellCenter(const int p[3]) { return mk3((float)p[0] + 0.5f, (float)p[1] + 0.5f, (float)p[2] + 0.5f); }

struct MediumTrAnalyticAdapter {                    // :20-136
    const Scene& sc; float Tr = 0.f; bool useLinearSampler; float tNear, tFar; Ray ray;
    MediumTrAnalyticAdapter(const Scene& s, bool lin) : sc(s), useLinearSampler(lin) {}
    void SetRayInfo(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    void ExecuteStartStep() {}
    bool ExecuteMainStep(const HDDA& dda, f3 vmin_leaf, int brick, const float*, int mip, float& t, Rng&) {
        HDDA dl = dda;
        dl.PrepareLeaf(vmin_leaf);
        for (int iter = 0; iter < kMaxBrickSteps && inLeaf(dl.p); iter++) {
            dl.Next();
            float maxDeltaT = dl.t.y - t;
            if (useLinearSampler) {
                float v[8]; fetchSigma(sc, mip, brick, dl.p, v);
                float c3, c2, c1, c0;
                trilinearCoeffs(v, ray.dir, leafP0(dl, vmin_leaf), c3, c2, c1, c0);
                float t_dist = fmin_(tFar - t, maxDeltaT);
                float t2 = t_dist * t_dist, t3 = t2 * t_dist, t4 = t2 * t2;
                Tr += -(c3 * t4 / 4 + c2 * t3 / 3 + c1 * t2 / 2 + c0 * t_dist);
            } else {
                float density = DensityInAtlas(sc, mip, brick, cellCenter(dl.p), false);
                float sigma_t = density * sc.med.sigma_t;
                Tr += -fmin_(tFar - t, maxDeltaT) * sigma_t;
            }
            if (t + maxDeltaT >= tFar) { Tr = exp_(Tr); return true; }
            t += maxDeltaT;
            dl.Step();
        }
        return false;
    }
    void ExecuteEndStep() { Tr = exp_(Tr); }
};

struct MediumTrRayMarchingAdapter {                 // :139-208
    const Scene& sc; float Tr = 0.f; bool useLinearSampler; float tNear, tFar; Ray ray; float tStep; bool hasInitialized = false;
    MediumTrRayMarchingAdapter(const Scene& s, bool lin, float ts) : sc(s), useLinearSampler(lin), tStep(ts) {}
    void SetRayInfo(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    void ExecuteStartStep() { hasInitialized = true; }
    bool ExecuteMainStep(const HDDA& dda, f3 vmin_leaf, int brick, const float*, int mip, float& t, Rng&) {
        t = tNear + (floor_((t - tNear) / tStep) + 0.5f) * tStep;
        if (t < dda.t.x) t += tStep;
        float tStepMultipler = 1.f;
        f3 wp = ray.origin + t * ray.dir;
        f3 p = wp - vmin_leaf;
        const f3 wpt = tStepMultipler * tStep * ray.dir;
        for (int iter = 0; iter < kMaxBrickSteps && inLeafF(p); iter++) {
            if (t >= tFar) { Tr = exp_(Tr); return true; }
            float density = DensityInAtlas(sc, mip, brick, p, useLinearSampler);
            float sigma_t = density * sc.med.sigma_t;
            Tr += -sigma_t * (iter == 0 ? 1.f : tStepMultipler) * tStep;
            p = p + wpt;
            t += tStepMultipler * tStep;
        }
        return false;
    }
    void ExecuteEndStep() { if (hasInitialized) Tr = exp_(Tr); else Tr = 1.f; }
};

struct SampleMediumAnalyticAdapter {                // :211-436
    const Scene& sc;
    float hitDistances[4], outTr[4], pdf[4];
    int numSamples; float opticalThickness = 0.f; float tNear, tFar; Ray ray; bool hasInitialized = false; bool useLinearSampler = false;
    explicit SampleMediumAnalyticAdapter(const Scene& s) : sc(s) {}
    void ExecuteStartStep() { for (int i = 0; i < numSamples; i++) hitDistances[i] = -1; hasInitialized = true; }
    void SetRayInfo(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    static float opticalThick(float t, float c3, float c2, float c1, float c0) {
        float t2 = t * t, t3 = t2 * t, t4 = t2 * t2;
        return c3 * t4 / 4 + c2 * t3 / 3 + c1 * t2 / 2 + c0 * t;
    }
    static float sigmaT(float t, float c3, float c2, float c1, float c0) {
        float t2 = t * t, t3 = t2 * t;
        return c3 * t3 + c2 * t2 + c1 * t + c0;
    }
    bool ExecuteMainStep(const HDDA& dda, f3 vmin_leaf, int brick, const float*, int mip, float& t, Rng& sg) {
        HDDA dl = dda;
        dl.PrepareLeaf(vmin_leaf);
        for (int iter = 0; iter < kMaxBrickSteps && inLeaf(dl.p); iter++) {
            dl.Next();
            float maxDeltaT = fmin_(tFar - t, dl.t.y - t);
            float currentTMax = fmin_(tFar, dl.t.y);
            int finishedCount = 0;
            float deltaThickness = 0.f;
            if (useLinearSampler) {
                float v[8]; fetchSigma(sc, mip, brick, dl.p, v);
                float c3, c2, c1, c0;
                trilinearCoeffs(v, ray.dir, leafP0(dl, vmin_leaf), c3, c2, c1, c0);
                deltaThickness = opticalThick(maxDeltaT, c3, c2, c1, c0);
                for (int sid = 0; sid < numSamples; sid++) {
                    if (hitDistances[sid] == -1) {
                        if (opticalThickness + deltaThickness >= outTr[sid]) {
                            float tau_target = outTr[sid] - opticalThickness;
                            float t_low = 0, t_high = maxDeltaT, tau_low = 0, tau_high = deltaThickness, t_sol = 0;
                            int it = 0;
                            while (it++ < 32 && t_high - t_low > maxDeltaT * 0.001f) {
                                t_sol = t_low + (t_high - t_low) * (tau_target - tau_low) / (tau_high - tau_low);
                                float tau = opticalThick(t_sol, c3, c2, c1, c0);
                                if (tau < tau_target) { t_low = t_sol; tau_low = tau; }
                                else { t_high = t_sol; tau_high = tau; }
                            }
                            hitDistances[sid] = t + t_sol;
                            outTr[sid] = exp_(-outTr[sid]);
                            pdf[sid] = sigmaT(t_sol, c3, c2, c1, c0) * outTr[sid];
                            finishedCount++;
                        }
                    } else finishedCount++;
                }
            } else {
                float density = DensityInAtlas(sc, mip, brick, cellCenter(dl.p), false);
                float sigma_t = density * sc.med.sigma_t;
                for (int sid = 0; sid < numSamples; sid++) {
                    if (hitDistances[sid] == -1) {
                        float dT = -log_(1 - next1D(sg)) / sigma_t;
                        float curT = t + dT;
                        if (isnan_(curT) || isinf_(curT)) curT = kRayTMax;
                        if (curT < currentTMax) {
                            hitDistances[sid] = curT;
                            outTr[sid] = exp_(-(dT * sigma_t + opticalThickness));
                            pdf[sid] = sigma_t * outTr[sid];
                            finishedCount++;
                        }
                    } else finishedCount++;
                }
                deltaThickness = maxDeltaT * sigma_t;
            }
            if (finishedCount == numSamples) return true;
            t = currentTMax;
            opticalThickness += deltaThickness;
            if (t >= tFar) { ExecuteEndStep(); return true; }
            dl.Step();
        }
        return false;
    }
    void ExecuteEndStep() {
        if (hasInitialized) {
            for (int i = 0; i < numSamples; i++)
                if (hitDistances[i] == -1) { hitDistances[i] = kRayTMax; outTr[i] = exp_(-opticalThickness); pdf[i] = outTr[i]; }
        } else {
            for (int i = 0; i < numSamples; i++) { hitDistances[i] = kRayTMax; outTr[i] = 1.f; pdf[i] = 1.f; }
        }
    }
};

struct SampleVolumeCellByDensityAdapter {           // :439-515
    const Scene& sc; int densityBound = 0; float selX = -1, selY = -1; float tNear, tFar; Ray ray; float runningSum = 0.f; float Tr = 0.f;
    explicit SampleVolumeCellByDensityAdapter(const Scene& s) : sc(s) {}
    void ExecuteStartStep() { selX = -1; selY = -1; }
    void SetRayInfo(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    bool ExecuteMainStep(const HDDA& dda, f3 vmin_leaf, int brick, const float*, int mip, float& t, Rng& sg) {
        HDDA dl = dda;
        dl.PrepareLeaf(vmin_leaf);
        for (int iter = 0; iter < kMaxBrickSteps && inLeaf(dl.p); iter++) {
            float density = DensityInAtlas(sc, mip, brick, cellCenter(dl.p), false);
            dl.Next();
            float maxDeltaT = dl.t.y - t;
            float sigma_t = density * sc.med.sigma_t;
            float weight = exp_(Tr) * sigma_t;
            runningSum += weight;
            if (runningSum > 0.f && next1D(sg) < weight / runningSum) {
                densityBound = f2i(density);
                selX = t; selY = fmin_(tFar, t + maxDeltaT);
            }
            Tr += -maxDeltaT * sigma_t;
            if (t + maxDeltaT >= tFar) return true;
            t += maxDeltaT;
            dl.Step();
        }
        return false;
    }
    void ExecuteEndStep() {}
};

struct FeatureRayMarchingAdapter {                  // :518-602
    const Scene& sc; float accuTransmittance = 1.f; float tNear, tFar; Ray ray; float Tr = 0.f; bool useLinearSampler; float tStep;
    bool earlyTerminate = false, hasInitialized = false;
    FeatureRayMarchingAdapter(const Scene& s, bool lin, float ts) : sc(s), useLinearSampler(lin), tStep(ts) {}
    void ExecuteStartStep() { hasInitialized = true; }
    void SetRayInfo(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    bool ExecuteMainStep(const HDDA& dda, f3 vmin_leaf, int brick, const float*, int mip, float& t, Rng&) {
        t = tNear + (floor_((t - tNear) / tStep) + 0.5f) * tStep;
        if (t < dda.t.x) t += tStep;
        f3 wp = ray.origin + t * ray.dir;
        f3 p = wp - vmin_leaf;
        const f3 wpt = tStep * ray.dir;
        for (int iter = 0; iter < kMaxBrickSteps && inLeafF(p); iter++) {
            float curTransmittance = exp_(Tr);
            if (curTransmittance < 0.01f) { earlyTerminate = true; ExecuteEndStep(); return true; }
            float density = DensityInAtlas(sc, mip, brick, p, useLinearSampler);
            float sigma_t = density * sc.med.sigma_t;
            float negOpticalLength = -sigma_t * tStep;
            Tr += negOpticalLength;
            p = p + wpt;
            t += tStep;
        }
        return false;
    }
    void ExecuteEndStep() { if (hasInitialized) accuTransmittance = exp_(Tr); }
};

struct MediumInteraction {                          // VolumeBase.slang:66-94
    f3 p, wo; float g; bool isValid;
};
static float PhaseHG(float cosTheta, float g) {
    float denom = 1 + g * g + 2 * g * cosTheta;
    const float Inv4Pi = 0.07957747154594766788444188168626f;
    return Inv4Pi * (1 - g * g) / (denom * sqrt_(denom));
}
static float phaseFunction(const MediumInteraction& mi, f3 wo, f3 wi) { return PhaseHG(dot(wo, wi), mi.g); }
static void CoordinateSystem(f3 v1, f3& v2, f3& v3) {
    if (fabs_(v1.x) > fabs_(v1.y)) v2 = mk3(-v1.z, 0, v1.x) / sqrt_(v1.x * v1.x + v1.z * v1.z);
    else v2 = mk3(0, v1.z, -v1.y) / sqrt_(v1.y * v1.y + v1.z * v1.z);
    v3 = cross(v1, v2);
}
static float Sample_p(const MediumInteraction& mi, f3 wo, f3& wi, float u0, float u1) {
    float g = mi.g, cosTheta;
    if (fabs_(g) < 1e-3f) cosTheta = 1 - 2 * u0;
    else {
        float sqrTerm = (1 - g * g) / (1 + g - 2 * g * u0);
        cosTheta = -(1 + g * g - sqrTerm * sqrTerm) / (2 * g);
    }
    float sinTheta = sqrt_(fmax_(0, 1 - cosTheta * cosTheta));
    float phi = 2 * kM_PI * u1;
    f3 v1, v2;
    CoordinateSystem(wo, v1, v2);
    wi = sinTheta * cos_(phi) * v1 + sinTheta * sin_(phi) * v2 + cosTheta * wo;
    return PhaseHG(cosTheta, g);
}

struct DecompositionTrackingAdapter {               // :606-707
    const Scene& sc; float tNear, tFar; Ray ray; Ray rWorld; MediumInteraction mi; bool loopLimit = false;
    explicit DecompositionTrackingAdapter(const Scene& s) : sc(s) {}
    void ExecuteStartStep() {}
    void SetRayInfo(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    void setMi(float t) { mi.p = rWorld.at(t); mi.wo = -rWorld.dir; mi.g = sc.med.g; mi.isValid = true; }
    bool ExecuteMainStep(const HDDA& dda, f3 vmin_leaf, int brick, const float* bnd, int mip, float& t, Rng& sg) {
        float minDensity = bnd[0], maxDensity = bnd[1];
        float currentTMax = fmin_(tFar, dda.t.y);
        float t_control;
        if (minDensity == 0.f) t_control = kRayTMax;
        else t_control = t - log_(1 - next1D(sg)) / (minDensity * sc.med.sigma_t);
        float invMaxDensity = 1.f / (maxDensity - minDensity);
        if (maxDensity - minDensity > 0.f) {
            int guard = 0;
            while (true) {
                if (++guard > kMaxDeltaIters) { loopLimit = true; break; }
                t -= log_(1 - next1D(sg)) * invMaxDensity / sc.med.sigma_t;
                if (t >= t_control || t >= currentTMax) break;
                f3 wp = ray.origin + t * ray.dir;
                f3 p = wp - vmin_leaf;
                float density = DensityInAtlas(sc, mip, brick, p, true);
                if ((density - minDensity) * invMaxDensity > next1D(sg)) { setMi(t); return true; }
            }
            t = fmin_(t_control, t);
            if (t < currentTMax) { setMi(t); return true; }
            t = currentTMax;
            if (t >= tFar) { ExecuteEndStep(); return true; }
        } else {
            if (t_control < currentTMax) { setMi(t_control); return true; }
            else { t = currentTMax; return false; }
        }
        return false;
    }
    void ExecuteEndStep() { mi.isValid = false; }
};

struct ResidualRatioTrackingAdapter {               // :710-794
    const Scene& sc; float tNear, tFar; Ray ray; float Tr = 1.f; bool useAnalogResidual, useGlobalMajorant; bool loopLimit = false;
    ResidualRatioTrackingAdapter(const Scene& s, bool analog, bool global) : sc(s), useAnalogResidual(analog || global), useGlobalMajorant(global) {}
    void ExecuteStartStep() { if (useGlobalMajorant) useAnalogResidual = true; }
    void SetRayInfo(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    bool ExecuteMainStep(const HDDA& dda, f3 vmin_leaf, int brick, const float* bnd, int mip, float& t, Rng& sg) {
        const float st = sc.med.sigma_t;
        float mu_min = useGlobalMajorant ? 0.f : bnd[0] * st;
        float mu_max = useGlobalMajorant ? sc.slots[mip].maxValue * sc.med.dscale * st : bnd[1] * st;
        float mu_avg = bnd[2] * st;
        float maxDeltaT = fmin_(tFar - t, dda.t.y - t);
        float currentTMax = fmin_(tFar, dda.t.y);
        float mu_r_temp = mu_max - mu_min;
        float D = sc.med.superDiag;
        float gamma = 2;
        float mu_c = (mu_r_temp == 0.f || useAnalogResidual) ? mu_min
                   : fmin_(mu_avg, fmax_(mu_min, mu_min + mu_r_temp * (pow_(gamma, 1.f / (D * mu_r_temp)) - 1)));
        float mu_r = fmax_(mu_c - mu_min, mu_max - mu_c);
        float inv_mu_r = 1.f / mu_r;
        float T_c = exp_(-mu_c * fmin_(tFar - t, maxDeltaT));
        float T_r = 1;
        if (mu_r > 0.f) {
            int guard = 0;
            while (true) {
                if (++guard > kMaxDeltaIters) { loopLimit = true; break; }
                t -= log_(1 - next1D(sg)) * inv_mu_r;
                if (t >= currentTMax) break;
                f3 wp = ray.origin + t * ray.dir;
                f3 p = wp - vmin_leaf;
                float density = DensityInAtlas(sc, mip, brick, p, true);
                float mu = density * st;
                T_r *= 1 - (mu - mu_c) * inv_mu_r;
            }
        }
        Tr *= T_c * T_r;
        t = currentTMax;
        if (t >= tFar) return true;
        return false;
    }
    void ExecuteEndStep() {}
};

// ---------------------------------------------------------------------------------------
// generic tracking entry points (VolumeUtils.slang:284-362, 573-582)
// ---------------------------------------------------------------------------------------
static float MediumTrAnalyticGeneric(const Scene& sc, const Ray& r, int mip, Rng& sg, bool lin) {
    MediumTrAnalyticAdapter a(sc, lin);
    VolumeTrackingGVDB(sc, r, mip, sg, a, lin);
    return a.Tr;
}
static void SampleMediumAnalyticGeneric(const Scene& sc, const Ray& r, Rng& sg, bool lin, float hit[4], int mip, float pdf[4], float tr[4], int n) {
    SampleMediumAnalyticAdapter a(sc);
    a.numSamples = n;
    a.useLinearSampler = lin;
    if (lin) for (int i = 0; i < n; i++) a.outTr[i] = -log_(1 - next1D(sg));
    VolumeTrackingGVDB(sc, r, mip, sg, a, lin);
    for (int i = 0; i < 4; ++i) { hit[i] = a.hitDistances[i]; tr[i] = a.outTr[i]; pdf[i] = a.pdf[i]; }
}
static void SampleMediumSuperVoxelGeneric(const Scene& sc, const Ray& r, Rng& sg, MediumInteraction& mi, int mip, bool& loopLimit) {
    DecompositionTrackingAdapter a(sc);
    a.rWorld = r;
    a.mi = mi;
    VolumeTrackingGVDB(sc, r, mip, sg, a, false);
    mi = a.mi;
    loopLimit |= a.loopLimit;
}
static float MediumTrResidualRatioTrackingGeneric(const Scene& sc, const Ray& r, int mip, Rng& sg, bool analog, bool global) {
    ResidualRatioTrackingAdapter a(sc, analog, global);
    VolumeTrackingGVDB(sc, r, mip, sg, a, false);
    return a.Tr;
}
static float MediumTrRayMarchingGeneric(const Scene& sc, const Ray& r, int mip, bool lin, float tStepScale, Rng& sg) {
    int eff = mip >= kPrevSlotOffset ? mip - kPrevSlotOffset : mip;
    eff = eff >= kNumMaxMips ? eff - kNumMaxMips : eff;
    MediumTrRayMarchingAdapter a(sc, lin, sc.med.tStep * tStepScale * (float)(eff + 1));
    VolumeTrackingGVDB(sc, r, mip, sg, a, false);
    return a.Tr;
}
static float ReservoirFeatureRayMarching(const Scene& sc, const Ray& r, Rng& sg, int mip, bool lin, float tStepScale) {
    FeatureRayMarchingAdapter a(sc, lin, sc.med.tStep * tStepScale);
    VolumeTrackingGVDB(sc, r, mip, sg, a, false);
    return a.accuTransmittance;
}
// computeVisibility (VolumeUtils.slang:535-551)
static float computeVisibility(const Scene& sc, const Ray& ray, Rng& sg, int samples, int mip, bool lin, uint32_t method, float tStepScale) {
    float visibility = 0;
    for (int i = 0; i < samples; i++) {
        if (method == VR_TRACK_RATIO || method == VR_TRACK_RESIDUAL_RATIO || method == VR_TRACK_ANALOG_RESIDUAL_RATIO)
            visibility += MediumTrResidualRatioTrackingGeneric(sc, ray, mip, sg, method == VR_TRACK_ANALOG_RESIDUAL_RATIO, method == VR_TRACK_RATIO);
        else if (method == VR_TRACK_RAY_MARCHING)
            visibility += MediumTrRayMarchingGeneric(sc, ray, mip, lin, tStepScale, sg);
        else if (method == VR_TRACK_ANALYTIC)
            visibility += MediumTrAnalyticGeneric(sc, ray, mip, sg, lin);
    }
    visibility /= samples;
    return visibility;
}
static float RejectionSampleRandomPointByDensity(const Scene& sc, const Ray& r, Rng& sg, int mip) {
    SampleVolumeCellByDensityAdapter a(sc);
    VolumeTrackingGVDB(sc, r, mip, sg, a, false);
    if (a.selX == -1) return kRayTMax;
    float sampledDepth = a.selX + (a.selY - a.selX) * next1D(sg);
    (void)next1D(sg);     // sampledY = sampleNext1D(sg) * densityBound (unused)
    return sampledDepth;
}

// ---------------------------------------------------------------------------------------
// environment map + importance sampling (EnvMap.slang, EnvMapSampler.slang, MathHelpers.slang)
// ---------------------------------------------------------------------------------------
static float signf_(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
static void world_to_latlong_map(f3 dir, float& u, float& v) {
    f3 p = normalize(dir);
    u = atan2_(p.x, -p.z) * kM_1_2PI + 0.5f;
    v = acos_(p.y) * kM_1_PI;
}
static f3 oct_to_ndir_equal_area_unorm(float px, float py) {
    px = px * 2.f - 1.f; py = py * 2.f - 1.f;
    float d = 1.f - (fabs_(px) + fabs_(py));
    float r = 1.f - fabs_(d);
    float phi = (r > 0.f) ? ((fabs_(py) - fabs_(px)) / r + 1.f) * kM_PI_4 : 0.f;
    float f = r * sqrt_(2.f - r * r);
    float x = f * signf_(px) * cos_(phi);
    float y = f * signf_(py) * sin_(phi);
    float z = signf_(d) * (1.f - r * r);
    return mk3(x, y, z);
}
// bilinear lookup, wrap in u, clamp in v (EnvMap.cpp:107-110 sampler)
static f3 envTex(const EnvMap& e, float u, float v) {
    float x = u * (float)e.w - 0.5f, y = v * (float)e.h - 0.5f;
    float fx0 = floor_(x), fy0 = floor_(y);
    float fx = x - fx0, fy = y - fy0;
    int ix = f2i(fx0), iy = f2i(fy0);
    auto wrap = [&](int i) { int m = i % e.w; return m < 0 ? m + e.w : m; };
    auto clampy = [&](int j) { return j < 0 ? 0 : (j >= e.h ? e.h - 1 : j); };
    int x0 = wrap(ix), x1 = wrap(ix + 1), y0 = clampy(iy), y1 = clampy(iy + 1);
    float c[3];
    for (int k = 0; k < 3; ++k) {
        float a = e.rgb[((size_t)y0 * e.w + x0) * 3 + k], b = e.rgb[((size_t)y0 * e.w + x1) * 3 + k];
        float cc = e.rgb[((size_t)y1 * e.w + x0) * 3 + k], d = e.rgb[((size_t)y1 * e.w + x1) * 3 + k];
        float top = lerp_(a, b, fx), bot = lerp_(cc, d, fx);
        c[k] = lerp_(top, bot, fy);
    }
    return mk3(c[0], c[1], c[2]);
}
static f3 envToLocal(const EnvMap& e, f3 d) { return mul33(d, e.inv); }
static f3 envToWorld(const EnvMap& e, f3 d) { return mul33(d, e.rot); }
static f3 envEval(const Scene& sc, f3 dir) {
    if (!sc.hasEnv) return mk3(0.f);
    float u, v;
    world_to_latlong_map(envToLocal(sc.env, dir), u, v);
    return sc.env.scale * envTex(sc.env, u, v);
}
// EnvMapSamplerSetup.cs.slang:46-72 and generateMips (2x2 box)
static void buildImportanceMap(EnvMap& e) {
    const int dim = e.impDim, spp = 64, sx = 8, sy = 8;
    e.imp.assign(e.baseMip + 1, std::vector<float>());
    e.imp[0].assign((size_t)dim * dim, 0.f);
    const float invSamples = 1.f / (float)(sx * sy);
    const float dimS = (float)(dim * sx);
    (void)spp;
    for (int py = 0; py < dim; ++py)
        for (int px = 0; px < dim; ++px) {
            float L = 0.f;
            for (int y = 0; y < sy; ++y)
                for (int x = 0; x < sx; ++x) {
                    float ppx = ((float)(px * sx + x) + 0.5f) / dimS;
                    float ppy = ((float)(py * sy + y) + 0.5f) / dimS;
                    f3 dir = oct_to_ndir_equal_area_unorm(ppx, ppy);
                    float u, v;
                    world_to_latlong_map(dir, u, v);
                    L += luminance(envTex(e, u, v));
                }
            e.imp[0][(size_t)py * dim + px] = L * invSamples;
        }
    for (int m = 1; m <= e.baseMip; ++m) {
        int d = dim >> m, ds = dim >> (m - 1);
        e.imp[m].assign((size_t)d * d, 0.f);
        for (int y = 0; y < d; ++y)
            for (int x = 0; x < d; ++x) {
                const std::vector<float>& s = e.imp[m - 1];
                float a = s[(size_t)(2 * y) * ds + 2 * x], b = s[(size_t)(2 * y) * ds + 2 * x + 1];
                float c = s[(size_t)(2 * y + 1) * ds + 2 * x], dd = s[(size_t)(2 * y + 1) * ds + 2 * x + 1];
                e.imp[m][(size_t)y * d + x] = (((a + b) + c) + dd) * 0.25f;
            }
    }
}
struct EnvSample { f3 dir; float pdf; f3 Le; };
static void envSample(const Scene& sc, float r0, float r1, EnvSample& res) {     // EnvMapSampler.slang:94-166
    const EnvMap& e = sc.env;
    float px = r0, py = r1;
    unsigned posx = 0, posy = 0;
    for (int mip = e.baseMip - 1; mip >= 0; mip--) {
        posx *= 2; posy *= 2;
        int d = e.impDim >> mip;
        const std::vector<float>& m = e.imp[mip];
        float w[4];
        w[0] = m[(size_t)posy * d + posx];
        w[1] = m[(size_t)posy * d + posx + 1];
        w[2] = m[(size_t)(posy + 1) * d + posx];
        w[3] = m[(size_t)(posy + 1) * d + posx + 1];
        float q[2] = {w[0] + w[2], w[1] + w[3]};
        unsigned offx, offy;
        float dd = q[0] / (q[0] + q[1]);
        if (px < dd) { offx = 0; px = px / dd; }
        else { offx = 1; px = (px - dd) / (1.f - dd); }
        float ee = w[offx] / q[offx];
        if (py < ee) { offy = 0; py = py / ee; }
        else { offy = 1; py = (py - ee) / (1.f - ee); }
        posx += offx; posy += offy;
    }
    float inv = 1.f / (float)e.impDim;
    float uvx = ((float)posx + px) * inv, uvy = ((float)posy + py) * inv;
    f3 dir = oct_to_ndir_equal_area_unorm(uvx, uvy);
    float avg_w = e.imp[e.baseMip][0];
    float pdf = e.imp[0][(size_t)posy * e.impDim + posx] / avg_w;
    res.dir = envToWorld(e, dir);
    res.pdf = pdf * kM_1_4PI;
    res.Le = envEval(sc, res.dir);
}
static void encodeLightUV(const Scene& sc, f3 dir, int& lightID, float uv[2]) {
    dir = envToLocal(sc.env, dir);
    lightID = dir.z < 0 ? -2 : -1;
    uv[0] = dir.x; uv[1] = dir.y;
}
static f3 decodeLightUV(const Scene& sc, const float uv[2], int lightID) {
    f3 dir = mk3(uv[0], uv[1], 0);
    dir.z = sqrt_(1 - uv[0] * uv[0] - uv[1] * uv[1]);
    if (isnan_(dir.z)) dir.z = 0.f;
    if (lightID == -2) dir.z = -dir.z;
    return envToWorld(sc.env, dir);
}

// ---------------------------------------------------------------------------------------
// lights (VolumeUtils.slang:12-149, LightHelpers.slang:223-242)
// ---------------------------------------------------------------------------------------
struct SceneLightSample { f3 dir; float distance; f3 Li; float pdf, pdfArea; f3 rayDir; float rayDistance; };
static void samplePointLight(f3 shadingPosW, const vr_point_light& L, f3& dir, float& dist, f3& Li, float& pdf) {
    f3 pos = mk3(L.pos[0], L.pos[1], L.pos[2]);
    f3 toLight = pos - shadingPosW;
    float distSqr = fmax_(dot(toLight, toLight), 1e-9f);
    dist = sqrt_(distSqr);
    dir = toLight / dist;
    Li = mk3(L.intensity[0], L.intensity[1], L.intensity[2]) / distSqr;
    pdf = 0.f;
}
static bool sampleSceneLights(const Scene& sc, f3 rayOrigin, bool useEnv, bool useAnalytic, Rng& sg, SceneLightSample& ls, int& outLightIndex, float outLightUV[2]) {
    if (!useEnv && !useAnalytic) return false;
    float p[3] = {useEnv ? 1.f : 0.f, useAnalytic ? 1.f : 0.f, 0.f};
    float sum = p[0] + p[1] + p[2];
    if (sum == 0.f) return false;
    float invSum = 1.f / sum;
    p[0] *= invSum; p[1] *= invSum; p[2] *= invSum;
    float u = next1D(sg);
    if (useEnv) {
        if (u < p[0]) {
            float selectionPdf = p[0];
            EnvSample s;
            float r0 = next1D(sg), r1 = next1D(sg);
            envSample(sc, r0, r1, s);
            float pdf = selectionPdf * s.pdf;
            ls.rayDir = ls.dir = s.dir;
            ls.rayDistance = ls.distance = kRayTMax;
            ls.pdf = pdf; ls.pdfArea = pdf;
            ls.Li = pdf > 0.f ? s.Le / pdf : mk3(0.f);
            outLightIndex = -1;
            encodeLightUV(sc, ls.rayDir, outLightIndex, outLightUV);
            return !(isnan_(ls.rayDir.x) || isnan_(ls.rayDir.y) || isnan_(ls.rayDir.z));
        }
        u -= p[0];
    }
    if (useAnalytic) {
        if (u < p[1]) {
            u /= p[1];
            uint32_t lightCount = (uint32_t)sc.lights.size();
            uint32_t lightIndex = std::min(f2u32(u * (float)lightCount), lightCount - 1);
            float selectionPdf = p[1] / (float)lightCount;
            f3 dir, Li; float dist, lpdf;
            samplePointLight(rayOrigin, sc.lights[lightIndex], dir, dist, Li, lpdf);
            outLightIndex = (int)lightIndex;
            ls.rayDir = ls.dir = dir;
            ls.rayDistance = ls.distance = dist;
            if (lpdf == 0) lpdf = 1.f;
            ls.pdf = selectionPdf * lpdf;
            ls.pdfArea = ls.pdf;
            ls.Li = Li / ls.pdf;
            outLightUV[0] = 0; outLightUV[1] = 0;
            return true;
        }
        u -= p[1];
    }
    return false;
}

// ---------------------------------------------------------------------------------------
// options per pass (VolumetricReSTIR.cpp:455-496)
// ---------------------------------------------------------------------------------------
struct SamplingOptions {
    uint32_t visibilityTrackingMethod, lightingTrackingMethod;
    int lightSamples, lightingMipLevel, visibilitySamples, visibilityMipLevel;
    bool visibilityUseLinearSampler, lightingUseLinearSampler;
    float visibilityTStepScale, lightingTStepScale;
    bool useEnvironmentLights, useAnalyticLights;
    int vertexReuseStartBounce = -1;        // vertex reuse (VERTEX_REUSE): first reconnection bounce; -1 off
};

struct Ctx {             // per-call constants
    const Scene* sc;
    const vr_options* o;
    int W, H;
    int maxBounces;
    SamplingOptions initial, spatial, fin;
    bool noReuse;
    bool loopLimit = false;
};

// SampleDirectLighting (VolumeUtils.slang:485-521)
static f3 SampleDirectLighting(const Ctx& c, Rng& sg, float& pdf, const MediumInteraction& mi, const SamplingOptions& o, bool enableShadow,
                               int& outLightIndex, float outLightUV[2], float& outVisibility) {
    pdf = 0.f;
    f3 Ld = mk3(0.f);
    SceneLightSample ls;
    bool valid = sampleSceneLights(*c.sc, mi.p, o.useEnvironmentLights, o.useAnalyticLights, sg, ls, outLightIndex, outLightUV);
    pdf = valid ? ls.pdfArea : 0.f;
    if (!valid) { pdf = 0.f; return mk3(0.f); }
    ls.pdf = 1.f;
    Ray shadowRay{mi.p, ls.rayDir, 0, ls.rayDistance};
    if (enableShadow) {
        float visibility = computeVisibility(*c.sc, shadowRay, sg, o.lightSamples, o.lightingMipLevel, o.lightingUseLinearSampler, o.lightingTrackingMethod, o.lightingTStepScale);
        outVisibility = visibility;
        ls.Li = ls.Li * visibility;
    }
    float p = phaseFunction(mi, mi.wo, ls.dir);
    Ld = Ld + p * ls.Li / ls.pdf;
    return Ld;
}

// ---------------------------------------------------------------------------------------
// ComputeInitialSample (ComputeInitialSample.slang:4-395), volume-only
// ---------------------------------------------------------------------------------------
static Reservoir ComputeInitialSample(Ctx& c, Ray primaryRay, float preHit, float prePdf, float preTr, Rng& sg, f3 extra[3]) {
    const Scene& sc = *c.sc;
    const SamplingOptions& options = c.initial;
    const int maxBounces = c.maxBounces;
    const bool noReuse = c.noReuse;
    float pathPdf = 1.f, pathPHat = 1.f;
    Ray ray = primaryRay;
    Reservoir combined = createNewReservoir();
    Reservoir out = createNewReservoir();
    float primaryScatterDepth = 0;
    const f3 sigma_s = sc.med.sigma_s, sigma_a = sc.med.sigma_a;
    const float sigma_t = sc.med.sigma_t;
    for (int bounce = 0; bounce < maxBounces; bounce++) {
        out = createNewReservoir();
        out.M = 1;
        float curHitDist, pdfDist = 0, Tr;
        MediumInteraction mi;
        if (bounce >= 1 || noReuse) {
            if (noReuse) {
                mi.isValid = false;
                SampleMediumSuperVoxelGeneric(sc, ray, sg, mi, 0, c.loopLimit);
                pdfDist = 1.f; Tr = 1.f;
                curHitDist = mi.isValid ? length(mi.p - ray.origin) : kRayTMax;
            } else {
                int curMip = options.visibilityMipLevel;
                if (c.o->mInitialUseCoarserGridForIndirectBounce)
                    curMip = std::min((options.visibilityMipLevel >= kNumMaxMips ? kNumMaxMips : 0) + sc.med.numMips - 1, curMip + 1);
                float hd[4], pd[4], trs[4];
                SampleMediumAnalyticGeneric(sc, ray, sg, options.visibilityUseLinearSampler, hd, curMip, pd, trs, 1);
                curHitDist = hd[0]; pdfDist = pd[0]; Tr = trs[0];
                mi.p = ray.at(curHitDist); mi.wo = -ray.dir; mi.g = sc.med.g; mi.isValid = curHitDist != kRayTMax;
            }
        } else {
            curHitDist = preHit; pdfDist = prePdf; Tr = preTr;
            mi.p = ray.at(curHitDist); mi.wo = -ray.dir; mi.g = sc.med.g; mi.isValid = curHitDist != kRayTMax;
        }
        pathPdf *= pdfDist;
        const int vrs = options.vertexReuseStartBounce;
        // ComputeInitialSample.slang:88-94: the reconnection vertex in area measure
        if (vrs >= 0 && bounce == vrs && curHitDist != kRayTMax) {
            pathPdf /= curHitDist * curHitDist;
            pathPHat /= curHitDist * curHitDist;
        }
        bool hitEmpty = false;
        float actualVolumeDensity = 0.f;
        if (bounce == 0) {
            if (maxBounces > 1) out.sampledPixel = encodeMaxIndirectBounces(out.sampledPixel, 0);
            out.depth = mi.isValid ? curHitDist : kRayTMax;
            primaryScatterDepth = out.depth;
            out.p_y = pathPdf;
        } else {
            out.depth = primaryScatterDepth;
            if (maxBounces > 1) {
                out.sampledPixel = encodeMaxIndirectBounces(out.sampledPixel, bounce);
                // ComputeInitialSample.slang:114-127: from the reuse bounce on, vertex positions
                if (vrs >= 0 && bounce >= vrs) extra[bounce - 1] = !mi.isValid ? mk3(kRayTMax) : mi.p;
                else extra[bounce - 1] = encodeWiDist(ray.dir, !mi.isValid ? kRayTMax : curHitDist);
            }
            out.p_y = pathPdf;
        }
        if (mi.isValid) actualVolumeDensity = noReuse ? 1.f : DensityWorldSpace(sc, mi.p, 0);
        if ((!mi.isValid && bounce > 0) || (mi.isValid && actualVolumeDensity == 0)) {
            out.p_y = 0.f; out.runningSum = 0.f; hitEmpty = true;
        }
        float pdfDir = 1.f;
        if (!hitEmpty) {
            if (mi.isValid) {
                f3 albedo = sigma_s / sigma_t;
                out.lightID = -1; out.lightUV[0] = 0; out.lightUV[1] = 0;
                float outLightPdf = 0.f, outVisibility = 1.f;
                f3 Ld = mk3(0.f), Le = mk3(0.f);
                if (sc.emis.has && actualVolumeDensity > 0.f) Le = EmissionWorldSpace(sc, mi.p);
                f3 one_minus_albedo = mk3(1.f) - albedo;
                bool shouldComputeLightVisibility = options.lightSamples == 0 ? false : true;
                Ld = SampleDirectLighting(c, sg, outLightPdf, mi, options, shouldComputeLightVisibility, out.lightID, out.lightUV, outVisibility);
                f3 wo = -ray.dir, wi = mk3(0.f);
                if (maxBounces > 1) {
                    float u0 = next1D(sg), u1 = next1D(sg);
                    pdfDir = Sample_p(mi, wo, wi, u0, u1);
                }
                float p_src = out.p_y;
                {
                    float emissionRatio = luminance(one_minus_albedo * Le) / (luminance(one_minus_albedo * Le) + luminance(albedo * Ld));
                    if (isnan_(emissionRatio)) emissionRatio = 0.f;
                    if (next1D(sg) < emissionRatio) { p_src *= emissionRatio; out.lightID = kSelfEmissionLightID; }
                    else p_src *= outLightPdf * (1 - emissionRatio);
                }
                out.runningSum = p_src == 0.f ? 0.f : 1.f;
                out.p_y = p_src;
                {
                    float p_y;
                    pathPHat *= Tr;
                    pathPHat *= actualVolumeDensity;
                    if (out.lightID == kSelfEmissionLightID) p_y = pathPHat * luminance(sigma_a * Le);
                    else p_y = pathPHat * luminance(sigma_s * Ld * outLightPdf);
                    pathPHat *= luminance(sigma_s) * pdfDir;
                    if (noReuse) { p_y /= sigma_t; pathPHat /= sigma_t; }
                    if (out.runningSum > 0.f) {
                        out.runningSum = out.p_y == 0.f ? 0.f : p_y / out.p_y;
                        if (out.lightID == kSelfEmissionLightID && bounce > 0) {
                            if (vrs < 0 || bounce < vrs) {          // ComputeInitialSample.slang:322-330
                                encodeEmissivePosition(mi.p, out.lightID, out.lightUV);
                                p_y /= (curHitDist * curHitDist);
                            }
                            out.sampledPixel = encodePathTag(out.sampledPixel, 1);
                        }
                        out.p_y = p_y;
                    }
                }
                pathPdf *= pdfDir;
                if (maxBounces > 1) {
                    if (bounce < maxBounces - 1) {
                        ray = Ray{mi.p, wi, 0, kRayTMax};
                        if (c.o->mInitialUseRussianRoulette && bounce >= 2) {
                            if (next1D(sg) < albedo.x) pathPdf *= albedo.x;
                            else { hitEmpty = true; combined.M++; }
                        }
                    }
                }
            } else {
                f3 Le = envEval(sc, ray.dir);
                pathPHat *= Tr;
                float p_y = pathPHat * luminance(Le);
                out.runningSum = out.p_y == 0.f ? 0.f : p_y / out.p_y;
                out.p_y = p_y;
                hitEmpty = true;
            }
        }
        if (maxBounces > 1) simpleResampleStep(out, combined, sg);
        if (hitEmpty) break;
    }
    if (maxBounces > 1) { combined.M = 1; return combined; }
    return out;
}

// ---------------------------------------------------------------------------------------
// Learned target (no counterpart in the reference): the product's definition restated.
// A transmittance MLP T(x, w) replaces the marched light visibility of the initial RIS target.
// Network: 5 query scalars (x normalised to the volume box, theta/pi, phi/2pi + 1/2), each
// encoded as sin/cos of 2^k pi s (k < 6, higher bands by the double-angle recurrences) -> 60
// features + 4 zero pads; 4 hidden ReLU layers of 64; T = clamp(exp(o), floor, 1).  Weights
// and activations are rounded to BF16, products accumulated in FP32 in index order.
// ---------------------------------------------------------------------------------------
namespace lpo {
const int kIn = 60, kInPad = 64, kHid = 64, kLayers = 4, kLayerStride = 64 * 64 + 64;
const int kOutW = kLayers * kLayerStride, kOutB = kOutW + 64, kParams = kOutB + 1;

static uint16_t toBf(float f) {
    uint32_t u = f2u(f);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    return (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
}
static float fromBf(uint16_t b) { return u2f((uint32_t)b << 16); }
static float rb(float f) { return fromBf(toBf(f)); }

static void features(const float x[3], const float w[3], const float bmin[3], const float binv[3], float f[kInPad]) {
    float s[5];
    for (int i = 0; i < 3; ++i) s[i] = (x[i] - bmin[i]) * binv[i];
    float wy = w[1] > 1.f ? 1.f : (w[1] < -1.f ? -1.f : w[1]);
    s[3] = acos_(wy) * kM_1_PI;
    s[4] = atan2_(w[2], w[0]) * kM_1_2PI + 0.5f;
    for (int i = 0; i < 5; ++i) {
        float a = s[i] * kM_PI;
        float sn = sin_(a), cs = cos_(a);
        for (int k = 0; k < 6; ++k) {
            f[12 * i + 2 * k] = sn;
            f[12 * i + 2 * k + 1] = cs;
            float s2 = 2.f * sn * cs, c2 = cs * cs - sn * sn;
            sn = s2; cs = c2;
        }
    }
    for (int k = kIn; k < kInPad; ++k) f[k] = 0.f;
}

// The weight matrices rounded to BF16 once, stored input-major ([layer][k][n], then the 64
// output weights), so that a layer's 64 outputs accumulate side by side; each output is still
// summed over k in index order, so the values are those of the row-by-row form.
static void roundedWeights(const float* P, std::vector<float>& wt) {
    wt.assign((size_t)kLayers * 4096 + 64, 0.f);
    for (int l = 0; l < kLayers; ++l)
        for (int n = 0; n < kHid; ++n)
            for (int k = 0; k < kInPad; ++k) wt[(size_t)l * 4096 + (size_t)k * 64 + n] = rb(P[l * kLayerStride + n * 64 + k]);
    for (int k = 0; k < kHid; ++k) wt[(size_t)kLayers * 4096 + k] = rb(P[kOutW + k]);
}

// forward pass keeping the BF16 activations of every layer (act[0] = encoded input); wt from
// roundedWeights(P)
static float forwardR(const float* P, const float* wt, const float x[3], const float w[3], const float bmin[3], const float binv[3],
                      float act[5][64]) {
    float f[kInPad];
    features(x, w, bmin, binv, f);
    for (int k = 0; k < kInPad; ++k) act[0][k] = rb(f[k]);
    for (int l = 0; l < kLayers; ++l) {
        const float* Wl = wt + (size_t)l * 4096;
        float acc[kHid];
        for (int n = 0; n < kHid; ++n) acc[n] = 0.f;
        for (int k = 0; k < kInPad; ++k) {
            const float a = act[l][k];
            for (int n = 0; n < kHid; ++n) acc[n] += Wl[k * 64 + n] * a;
        }
        for (int n = 0; n < kHid; ++n) {
            float z = acc[n] + P[l * kLayerStride + 4096 + n];
            act[l + 1][n] = rb(z > 0.f ? z : 0.f);
        }
    }
    float o = 0.f;
    for (int k = 0; k < kHid; ++k) o += act[4][k] * wt[(size_t)kLayers * 4096 + k];
    return o + P[kOutB];
}
static float forward(const float* P, const float x[3], const float w[3], const float bmin[3], const float binv[3], float act[5][64]) {
    std::vector<float> wt;
    roundedWeights(P, wt);
    return forwardR(P, wt.data(), x, w, bmin, binv, act);
}
static float predict(float o, float floor_) {
    float t = exp_(o);
    t = t < floor_ ? floor_ : t;
    return t > 1.f ? 1.f : t;
}

// gradient of mean((exp(o) - target)^2) with the training kernel's numerics: BF16 weights,
// activations and dZ, FP32 sums (per chunk of 128 samples in sample order, then chunk sums in
// chunk order; the tensor core's own order inside the products differs)
static void gradients(const float* P, const float* samples, int n, const float bmin[3], const float binv[3], int lossLog, float floor_,
                      float* grad, float* loss) {
    const float invB = 1.f / (float)n;
    std::vector<float> wt, Pr(kParams);
    roundedWeights(P, wt);
    for (int i = 0; i < kParams; ++i) Pr[i] = rb(P[i]);      // only the weight entries are read rounded
    std::vector<float> tot(kParams, 0.f), part(kParams);
    float lossTot = 0.f;
    std::vector<float> act((size_t)128 * 5 * 64), g(128), lv(128), dzs((size_t)128 * 64), dhs((size_t)128 * 64);
    for (int c0 = 0; c0 < n; c0 += 128) {
        std::fill(part.begin(), part.end(), 0.f);
        for (int t = 0; t < 128; ++t) {
            const int si = c0 + t;
            float (*a)[64] = reinterpret_cast<float (*)[64]>(&act[(size_t)t * 320]);
            g[t] = 0.f; lv[t] = 0.f;
            bool valid = si < n;
            float x[3] = {0, 0, 0}, w[3] = {0, 0, 0};
            if (valid) {
                const float* q = samples + (size_t)si * 8;
                x[0] = q[0]; x[1] = q[1]; x[2] = q[2]; w[0] = q[3]; w[1] = q[4]; w[2] = q[5];
                valid = q[6] >= 0.f;
            }
            float o;
            if (si < n) o = forwardR(P, wt.data(), x, w, bmin, binv, a);
            else {
                for (int k = 0; k < 64; ++k) a[0][k] = 0.f;
                for (int l = 0; l < kLayers; ++l)
                    for (int m = 0; m < kHid; ++m) {
                        float acc = 0.f;
                        for (int k = 0; k < kInPad; ++k) acc += Pr[l * kLayerStride + m * 64 + k] * a[l][k];
                        float z = acc + P[l * kLayerStride + 4096 + m];
                        a[l + 1][m] = rb(z > 0.f ? z : 0.f);
                    }
                o = 0.f;
                for (int k = 0; k < kHid; ++k) o += a[4][k] * Pr[kOutW + k];
                o += P[kOutB];
            }
            (void)o;
            if (valid) {
                const float y = samples[(size_t)si * 8 + 7];
                if (lossLog) {
                    float d = o - log_(fmax_(y, floor_));
                    g[t] = 2.f * d * invB;
                    lv[t] = d * d * invB;
                } else {
                    float p = exp_(o);
                    float d = p - y;
                    g[t] = 2.f * d * p * invB;
                    lv[t] = d * d * invB;
                }
            }
            for (int k = 0; k < kHid; ++k) dhs[(size_t)t * 64 + k] = g[t] * Pr[kOutW + k];
        }
        for (int k = 0; k < kHid; ++k) {
            float acc = 0.f;
            for (int t = 0; t < 128; ++t) acc += g[t] * act[(size_t)t * 320 + 4 * 64 + k];
            part[kOutW + k] = acc;
        }
        {
            float acc = 0.f, ls = 0.f;
            for (int t = 0; t < 128; ++t) { acc += g[t]; ls += lv[t]; }
            part[kOutB] = acc;
            lossTot += ls;
        }
        for (int l = kLayers - 1; l >= 0; --l) {
            const float* W = Pr.data() + l * kLayerStride;
            for (int t = 0; t < 128; ++t) {
                float* dz = &dzs[(size_t)t * 64];
                float* dh = &dhs[(size_t)t * 64];
                // dZ enters both products of the layer rounded to BF16 (tensor-core operands)
                for (int m = 0; m < kHid; ++m) dz[m] = rb(act[(size_t)t * 320 + (l + 1) * 64 + m] > 0.f ? dh[m] : 0.f);
                if (l > 0)
                    for (int k = 0; k < kHid; ++k) {
                        float acc = 0.f;
                        for (int m = 0; m < kHid; ++m) acc += W[m * 64 + k] * dz[m];
                        dh[k] = acc;
                    }
            }
            for (int m = 0; m < kHid; ++m) {
                float accb = 0.f;
                float acc[64];
                for (int k = 0; k < 64; ++k) acc[k] = 0.f;
                for (int t = 0; t < 128; ++t) {
                    float d = dzs[(size_t)t * 64 + m];
                    accb += d;
                    for (int k = 0; k < 64; ++k) acc[k] += d * act[(size_t)t * 320 + l * 64 + k];
                }
                for (int k = 0; k < 64; ++k) part[l * kLayerStride + m * 64 + k] = acc[k];
                part[l * kLayerStride + 4096 + m] = accb;
            }
        }
        for (int i = 0; i < kParams; ++i) tot[i] += part[i];
    }
    for (int i = 0; i < kParams; ++i) grad[i] = tot[i];
    *loss = lossTot;
}
}  // namespace lpo

// vertex record of the split initial pass (see ComputeInitialSampleLP)
struct LpVertex { float a, b, uv0, uv1; int lightID, sampledPixel, flags; float u; };
const int kLpValid = 1, kLpNeedsT = 2;

// ComputeInitialSample with the shadow ray of the next-event estimate deferred to the network
// and every resampling uniform drawn up front (the random stream does not depend on T).  The
// primary distance sample comes from the pixel's stream (the rounds of TraceRays, all drawn
// before any vertex); every vertex, and the candidate's resampling uniform right after the first
// vertex (ucOut), draws from the candidate's own stream, seeded by (pixel, frame, candidate), so
// that candidates and their indirect vertices can be generated as work apart from the others.
static float ComputeInitialSampleLP(Ctx& c, Ray ray, float preHit, float prePdf, float preTr, LpVertex* rec, f3* extra,
                                    float* queries /* [maxBounces][8] */, int px, int py, int frame, int cid, float* ucOut) {
    const Scene& sc = *c.sc;
    const SamplingOptions& options = c.initial;
    const int maxBounces = c.maxBounces;
    float pathPdf = 1.f, pathPHat = 1.f;
    float primaryScatterDepth = 0;
    const f3 sigma_s = sc.med.sigma_s, sigma_a = sc.med.sigma_a;
    const float sigma_t = sc.med.sigma_t;
    int bounce = 0;
    Rng sg = rng_create((uint32_t)px, (uint32_t)py, 0x40000000u | (((uint32_t)frame * 4096u + (uint32_t)cid) & 0x3FFFFFFFu));
    for (; bounce < maxBounces; bounce++) {
        Reservoir out = createNewReservoir();
        out.M = 1;
        float curHitDist, pdfDist = 0, Tr;
        MediumInteraction mi;
        if (bounce >= 1) {
            int curMip = options.visibilityMipLevel;
            if (c.o->mInitialUseCoarserGridForIndirectBounce)
                curMip = std::min((options.visibilityMipLevel >= kNumMaxMips ? kNumMaxMips : 0) + sc.med.numMips - 1, curMip + 1);
            float hd[4], pd[4], trs[4];
            SampleMediumAnalyticGeneric(sc, ray, sg, options.visibilityUseLinearSampler, hd, curMip, pd, trs, 1);
            curHitDist = hd[0]; pdfDist = pd[0]; Tr = trs[0];
        } else {
            curHitDist = preHit; pdfDist = prePdf; Tr = preTr;
        }
        mi.p = ray.at(curHitDist); mi.wo = -ray.dir; mi.g = sc.med.g; mi.isValid = curHitDist != kRayTMax;
        pathPdf *= pdfDist;
        bool hitEmpty = false;
        float actualVolumeDensity = 0.f;
        if (bounce == 0) {
            if (maxBounces > 1) out.sampledPixel = encodeMaxIndirectBounces(out.sampledPixel, 0);
            out.depth = mi.isValid ? curHitDist : kRayTMax;
            primaryScatterDepth = out.depth;
        } else if (maxBounces > 1) {
            out.sampledPixel = encodeMaxIndirectBounces(out.sampledPixel, bounce);
            extra[bounce - 1] = encodeWiDist(ray.dir, !mi.isValid ? kRayTMax : curHitDist);
        }
        out.p_y = pathPdf;
        if (mi.isValid) actualVolumeDensity = DensityWorldSpace(sc, mi.p, 0);
        if ((!mi.isValid && bounce > 0) || (mi.isValid && actualVolumeDensity == 0)) {
            out.p_y = 0.f; out.runningSum = 0.f; hitEmpty = true;
        }
        int flags = kLpValid;
        float pdfDir = 1.f;
        queries[bounce * 8 + 6] = -1.f;
        if (!hitEmpty) {
            if (mi.isValid) {
                f3 albedo = sigma_s / sigma_t;
                out.lightID = -1; out.lightUV[0] = 0; out.lightUV[1] = 0;
                float outLightPdf = 0.f;
                f3 Ld = mk3(0.f), Le = mk3(0.f);
                if (sc.emis.has && actualVolumeDensity > 0.f) Le = EmissionWorldSpace(sc, mi.p);
                f3 one_minus_albedo = mk3(1.f) - albedo;
                SceneLightSample ls;
                bool lv = sampleSceneLights(sc, mi.p, options.useEnvironmentLights, options.useAnalyticLights, sg, ls, out.lightID, out.lightUV);
                if (lv) {
                    outLightPdf = ls.pdfArea;
                    float p = phaseFunction(mi, mi.wo, ls.dir);
                    Ld = mk3(0.f) + p * ls.Li / 1.f;
                }
                f3 wo = -ray.dir, wi = mk3(0.f);
                if (maxBounces > 1) {
                    float u0 = next1D(sg), u1 = next1D(sg);
                    pdfDir = Sample_p(mi, wo, wi, u0, u1);
                }
                float p_src = out.p_y;
                {
                    float emissionRatio = luminance(one_minus_albedo * Le) / (luminance(one_minus_albedo * Le) + luminance(albedo * Ld));
                    if (isnan_(emissionRatio)) emissionRatio = 0.f;
                    if (next1D(sg) < emissionRatio) { p_src *= emissionRatio; out.lightID = kSelfEmissionLightID; }
                    else p_src *= outLightPdf * (1 - emissionRatio);
                }
                out.runningSum = p_src == 0.f ? 0.f : 1.f;
                out.p_y = p_src;
                {
                    float p_y;
                    pathPHat *= Tr;
                    pathPHat *= actualVolumeDensity;
                    const bool emis = out.lightID == kSelfEmissionLightID;
                    if (emis) p_y = pathPHat * luminance(sigma_a * Le);
                    else p_y = pathPHat * luminance(sigma_s * Ld * outLightPdf);
                    pathPHat *= luminance(sigma_s) * pdfDir;
                    if (out.runningSum > 0.f) {
                        if (!emis && lv && options.lightSamples != 0 && p_y != 0.f) {
                            flags |= kLpNeedsT;
                            out.runningSum = out.p_y;
                            out.p_y = p_y;
                            float* q = queries + bounce * 8;
                            q[0] = mi.p.x; q[1] = mi.p.y; q[2] = mi.p.z; q[3] = ls.rayDir.x; q[4] = ls.rayDir.y; q[5] = ls.rayDir.z;
                            q[6] = ls.rayDistance; q[7] = 0.f;
                        } else {
                            out.runningSum = out.p_y == 0.f ? 0.f : p_y / out.p_y;
                            if (emis && bounce > 0) {
                                encodeEmissivePosition(mi.p, out.lightID, out.lightUV);
                                p_y /= (curHitDist * curHitDist);
                                out.sampledPixel = encodePathTag(out.sampledPixel, 1);
                            }
                            out.p_y = p_y;
                        }
                    }
                }
                pathPdf *= pdfDir;
                if (maxBounces > 1 && bounce < maxBounces - 1) {
                    ray = Ray{mi.p, wi, 0, kRayTMax};
                    if (c.o->mInitialUseRussianRoulette && bounce >= 2) {
                        if (next1D(sg) < albedo.x) pathPdf *= albedo.x;
                        else hitEmpty = true;
                    }
                }
            } else {
                f3 Le = envEval(sc, ray.dir);
                pathPHat *= Tr;
                float p_y = pathPHat * luminance(Le);
                out.runningSum = out.p_y == 0.f ? 0.f : p_y / out.p_y;
                out.p_y = p_y;
                hitEmpty = true;
            }
        }
        const float ub = maxBounces > 1 ? next1D(sg) : 0.f;
        rec[bounce] = LpVertex{out.runningSum, out.p_y, out.lightUV[0], out.lightUV[1], out.lightID, out.sampledPixel, flags, ub};
        if (bounce == 0) *ucOut = next1D(sg);        // the candidate's resampling uniform
        if (hitEmpty) { bounce++; break; }
    }
    for (int b = bounce; b < maxBounces; ++b) { rec[b].flags = 0; queries[b * 8 + 6] = -1.f; }
    return primaryScatterDepth;
}

// ---------------------------------------------------------------------------------------
// evaluate_F_ family (ReSTIRHelper.slang:91-496)
// ---------------------------------------------------------------------------------------
struct ExtraProvider {        // StructuredBuffer/Array data providers (ArrayDataProvider.slang)
    const f3* data;
    f3 get(int i) const { return data[i]; }
};

// precomputedVisibility / lightVisibilityReuse: vertex reuse (ReSTIRHelper.slang:443-496) takes the
// light transmittance from the reservoir's p_partial, or hands the marched one back for it
static f3 evaluate_L_in_volume(const Ctx& c, const MediumInteraction& mi, int lightID, const float lightUV[2], Rng& sg, const SamplingOptions& options, bool cullNonOpaque,
                               int densityGridOffset, float* precomputedVisibility = nullptr, bool lightVisibilityReuse = false) {
    const Scene& sc = *c.sc;
    Ray shadowRay;
    f3 Ld = mk3(0.f);
    if (lightID < 0) {
        f3 wiWorld = decodeLightUV(sc, lightUV, lightID);
        shadowRay = Ray{mi.p, wiWorld, 0, kRayTMax};
        Ld = envEval(sc, wiWorld) * phaseFunction(mi, mi.wo, wiWorld);
    } else if (lightID < (int)sc.lights.size()) {
        f3 dir, Li; float dist, pdf;
        samplePointLight(mi.p, sc.lights[lightID], dir, dist, Li, pdf);
        shadowRay = Ray{mi.p, dir, 0, dist};
        Ld = Li * phaseFunction(mi, mi.wo, dir);
    } else {
        return mk3(0.f);      // mesh lights are outside this path
    }
    float Tr;
    if (lightVisibilityReuse) Tr = *precomputedVisibility;
    else {
        Tr = computeVisibility(sc, shadowRay, sg, options.lightSamples, cullNonOpaque ? options.lightingMipLevel + densityGridOffset : 0,
                               options.lightingUseLinearSampler, options.lightingTrackingMethod, options.lightingTStepScale);
        if (precomputedVisibility) *precomputedVisibility = Tr;
    }
    return Tr * Ld;
}

// spatialReuse and pPartialOut: vertex reuse (ReSTIRHelper.slang:91-420; the reservoir is REUSETYPE
// inout there): spatial reuse takes the suffix's share of p_hat from tap.p_partial; other calls
// write the share they evaluate to *pPartialOut (when given)
static f3 evaluate_F_(const Ctx& c, Reservoir tap, const ExtraProvider& extra, Ray ray, Rng& sg, const SamplingOptions& options,
                      bool noReuse, bool isFinalShading, bool isLastFrame = false, bool spatialReuse = false, float* pPartialOut = nullptr) {
    const int vrs = options.vertexReuseStartBounce;
    const bool vr = vrs >= 0;
    f3 P_prefix = mk3(1.f);
    const Scene& sc = *c.sc;
    const bool useLastFrameGrid = sc.usePrevGrid && isLastFrame && sc.hasAnimation;
    const int mipLevelOffset = useLastFrameGrid ? kPrevSlotOffset : 0;
    bool isBackgroundSample = tap.depth == kRayTMax;
    ray.tMax = tap.depth;
    f3 F = mk3(1.f);
    int maxIndirectBounces = decodeMaxIndirectBounces(tap.sampledPixel, c.maxBounces);
    bool isSelfEmission = c.maxBounces > 1 ? (maxIndirectBounces == 0 && tap.lightID == kSelfEmissionLightID)
                                           : (tap.lightID == kSelfEmissionLightID);
    float visibility = 1.f;
    f3 p_World = ray.at(ray.tMax);
    MediumInteraction mi{ray.at(ray.tMax), -ray.dir, sc.med.g, true};
    {
        f3 sigma_s = mk3(1.f);
        float density = (isBackgroundSample || noReuse) ? 1.f : DensityWorldSpace(sc, p_World, mipLevelOffset);
        if (density == 0.f) return mk3(0.f);
        if (!noReuse)
            visibility = computeVisibility(sc, ray, sg, options.visibilitySamples, options.visibilityMipLevel + mipLevelOffset,
                                           options.visibilityUseLinearSampler, options.visibilityTrackingMethod, options.visibilityTStepScale);
        sigma_s = isBackgroundSample ? mk3(1.f) : (isSelfEmission ? sc.med.sigma_a : sc.med.sigma_s);
        if (noReuse && !isBackgroundSample) sigma_s = sigma_s / sc.med.sigma_t;
        F = F * (visibility * density * sigma_s);
    }
    int bounceId = 0;
    if (any_gt0(F)) {
        if (isBackgroundSample) {
            F = F * envEval(sc, ray.dir);
        } else if (isSelfEmission) {
            F = F * EmissionWorldSpace(*c.sc, p_World, useLastFrameGrid);
        } else {
            bool isScatterSelfEmission = false;
            Ray scatterRay{};
            if (c.maxBounces > 1 && maxIndirectBounces > 0) {
                isScatterSelfEmission = decodePathTag(tap.sampledPixel) == 1;
                int numIndirectBounces = maxIndirectBounces;
                for (; bounceId < numIndirectBounces; bounceId++) {
                    bool isCurrentVertexEmissive = isScatterSelfEmission && bounceId == numIndirectBounces - 1;
                    f4 wiDist = decodeWiDist(extra.get(tap.extraBounceStartId + bounceId), vr && bounceId + 1 >= vrs);
                    if (isCurrentVertexEmissive && (!vr || bounceId + 1 < vrs)) {
                        f3 pe = decodeEmissivePosition(tap.lightID, tap.lightUV);
                        wiDist.x = pe.x; wiDist.y = pe.y; wiDist.z = pe.z; wiDist.w = -1.f;
                    }
                    if (wiDist.w == kRayTMax) return mk3(0.f);
                    float dist = 1.f;
                    if (wiDist.w == -1.f) {
                        f3 disp = mk3(wiDist.x, wiDist.y, wiDist.z) - p_World;
                        dist = length(disp);
                        f3 dir = normalize(disp);
                        scatterRay = Ray{p_World, dir, 0.f, dist};
                    } else {
                        scatterRay = Ray{p_World, mk3(wiDist.x, wiDist.y, wiDist.z), 0.f, wiDist.w};
                    }
                    f3 bsdf = mk3(phaseFunction(mi, mi.wo, scatterRay.dir));
                    F = F * bsdf;
                    if (all_eq0(F)) return mk3(0.f);
                    if (vr && bounceId == vrs) {                 // ReSTIRHelper.slang:289-295
                        if (spatialReuse) return F * tap.p_partial;
                        P_prefix = F;
                    }
                    if (wiDist.w == -1.f) p_World = mk3(wiDist.x, wiDist.y, wiDist.z);
                    else p_World = scatterRay.at(scatterRay.tMax);
                    f3 sig; float scatterDensity;
                    if (!noReuse) {
                        sig = isCurrentVertexEmissive ? sc.med.sigma_a : sc.med.sigma_s;
                        scatterDensity = fmax_(0, DensityWorldSpace(sc, p_World, mipLevelOffset));
                    } else {
                        sig = isCurrentVertexEmissive ? sc.med.sigma_a / sc.med.sigma_t : sc.med.sigma_s / sc.med.sigma_t;
                        scatterDensity = 1.f;
                    }
                    F = F * (scatterDensity * sig);
                    if (vr ? (bounceId + 1 == vrs || (isCurrentVertexEmissive && bounceId + 1 < vrs)) : isCurrentVertexEmissive)
                        F = F * (1.f / (dist * dist));
                    if (all_eq0(F)) return mk3(0.f);
                    float scatterVisibility = 1.f;
                    if (!noReuse)
                        scatterVisibility = computeVisibility(sc, scatterRay, sg, options.visibilitySamples, options.visibilityMipLevel + mipLevelOffset,
                                                              options.visibilityUseLinearSampler, options.visibilityTrackingMethod, options.visibilityTStepScale);
                    F = F * scatterVisibility;
                    mi.wo = -scatterRay.dir;
                    mi.p = p_World;
                    if (all_eq0(F)) return mk3(0.f);
                }
                if (isScatterSelfEmission) F = F * EmissionWorldSpace(*c.sc, p_World, useLastFrameGrid);
                else mi = MediumInteraction{scatterRay.at(scatterRay.tMax), -scatterRay.dir, sc.med.g, true};
            }
            if (!isScatterSelfEmission && any_gt0(F)) {
                const bool lightVisibilityReuse = vr && bounceId == vrs && spatialReuse;
                float precomputedVisibility = tap.p_partial;
                F = F * evaluate_L_in_volume(c, mi, tap.lightID, tap.lightUV, sg, options, !isFinalShading, mipLevelOffset, &precomputedVisibility,
                                             lightVisibilityReuse);
                if (vr && bounceId == vrs && !spatialReuse && pPartialOut) *pPartialOut = precomputedVisibility;
            }
        }
    }
    // ReSTIRHelper.slang:415-419: the suffix's share of p_hat
    if (vr && bounceId > vrs && !spatialReuse && pPartialOut) *pPartialOut = luminance(F / P_prefix);
    return F;
}
static float evaluate_P_hat(const Ctx& c, const Ray& ray, Rng& sg, const ExtraProvider& extra, const SamplingOptions& o, const Reservoir& tap,
                            bool isLastFrame = false, bool spatialReuse = false, float* pPartialOut = nullptr) {
    f3 F = evaluate_F_(c, tap, extra, ray, sg, o, false, false, isLastFrame, spatialReuse, pPartialOut);
    return luminance(F);
}
// resampleNeighbor (spatialReuse false: the tap's p_partial is re-evaluated, the reservoir being
// REUSETYPE inout) and resampleNeighborSpatialReuse (spatialReuse true), ReSTIRHelper.slang:567-600
static void resampleNeighbor(const Ctx& c, Reservoir& tap, const Ray& ray, Rng& sg, const ExtraProvider& extra, const SamplingOptions& o,
                             bool spatialReuse = false) {
    if (tap.runningSum == 0.f) return;
    float p_y_hat = evaluate_P_hat(c, ray, sg, extra, o, tap, false, spatialReuse, spatialReuse ? nullptr : &tap.p_partial);
    float weight = p_y_hat / tap.p_y;
    if (isinf_(weight) || isnan_(weight)) weight = 0.f;
    tap.runningSum *= weight;
    tap.p_y = p_y_hat;
}

// ---------------------------------------------------------------------------------------
// camera (Camera.slang, Camera.cpp:183-189) and reprojection matrices (glm conventions)
// ---------------------------------------------------------------------------------------
static CamFrame makeCamera(const vr_camera& cam, int W, int H) {
    CamFrame f;
    f3 pos = mk3(cam.pos[0], cam.pos[1], cam.pos[2]);
    f3 tgt = mk3(cam.target[0], cam.target[1], cam.target[2]);
    f3 up = mk3(cam.up[0], cam.up[1], cam.up[2]);
    float aspect = (float)W / (float)H;
    float focal = 1.f;
    f.posW = pos;
    f.W = normalize(tgt - pos) * focal;
    f.U = normalize(cross(f.W, up));
    f.V = normalize(cross(f.U, f.W));
    float th = tan_(cam.fov_y * 0.5f);
    float ulen = focal * th * aspect, vlen = focal * th;
    f.U = f.U * ulen;
    f.V = f.V * vlen;
    // view = lookAt(pos, target, up), right-handed, column-major m[col*4+row]
    f3 fw = normalize(tgt - pos);
    f3 s = normalize(cross(fw, up));
    f3 u = cross(s, fw);
    float* v = f.view;
    for (int i = 0; i < 16; ++i) v[i] = 0.f;
    v[0] = s.x; v[4] = s.y; v[8] = s.z;
    v[1] = u.x; v[5] = u.y; v[9] = u.z;
    v[2] = -fw.x; v[6] = -fw.y; v[10] = -fw.z;
    v[12] = -dot(s, pos); v[13] = -dot(u, pos); v[14] = dot(fw, pos); v[15] = 1.f;
    // projection = perspective(fovY, aspect, near, far), depth range [0, 1]
    float* p = f.proj;
    for (int i = 0; i < 16; ++i) p[i] = 0.f;
    p[0] = 1.f / (aspect * th);
    p[5] = 1.f / th;
    p[10] = cam.far_z / (cam.near_z - cam.far_z);
    p[11] = -1.f;
    p[14] = -(cam.far_z * cam.near_z) / (cam.far_z - cam.near_z);
    return f;
}
static f3 rayDirPinhole(const CamFrame& f, int px, int py, int W, int H) {      // Camera.slang:172-181
    float sx = ((float)px + 0.5f) / (float)W, sy = ((float)py + 0.5f) / (float)H;
    float ndcx = 2.f * sx + -1.f, ndcy = -2.f * sy + 1.f;
    return ndcx * f.U + ndcy * f.V + f.W;
}
// glm matrix (column-major) times column vector
static void mulMat4(const float* m, const float in[4], float out[4]) {
    for (int r = 0; r < 4; ++r) out[r] = in[0] * m[0 * 4 + r] + in[1] * m[1 * 4 + r] + in[2] * m[2 * 4 + r] + in[3] * m[3 * 4 + r];
}

// ---------------------------------------------------------------------------------------
// the pass
// ---------------------------------------------------------------------------------------
struct Oracle {
    vr_options opts;
    int W = 0, H = 0;
    Scene sc;
    bool hasVolume = false;
    int frameCount = 0;
    bool optionsChanged = true;
    int temporalSampleAccumulated = 0;
    CamFrame prev{};
    int numThreads = 0;
    bool loopLimit = false;
    // buffers (VolumetricReSTIR.cpp:419-450)
    std::vector<Reservoir> perPixel[2], temporal;
    std::vector<f3> extraPP[2], extraTemporal;
    std::vector<Features> features, temporalFeatures;
    std::vector<float> color;          // perPixelColor[0] (reference mode), rgba
    int lastMaxBounces = 0;

    // animated volume (Scene::addGVDBVolumeSequence / Scene::update): every frame's grids, the
    // current one advanced before each rendered frame
    struct AnimFrame {
        Slot slots[VR_NUM_SLOTS];
        Slot temp, vel[3];
        bool hasTemp = false;
    };
    std::vector<AnimFrame> anim;
    Slot staticSlots[VR_NUM_SLOTS];
    int animId = -1;
    bool animTemp = false, animVel = false;
    float animVelScale = 1.f;
    void animAdvance() {
        if (anim.empty()) return;
        const int n = (int)anim.size();
        animId = (animId + 1) % n;
        const int cur = animId, prv = (cur + n - 1) % n;
        for (int k = 0; k < VR_NUM_SLOTS; ++k) { sc.slots[k] = anim[cur].slots[k]; sc.slots[kPrevSlotOffset + k] = anim[prv].slots[k]; }
        sc.hasAnimation = true;
        if (animTemp) {
            sc.emis.slot = anim[cur].temp; sc.emis.prevSlot = anim[prv].temp;
            sc.emis.has = anim[cur].hasTemp; sc.emis.lastHas = anim[prv].hasTemp;
        }
        if (animVel) {
            for (int k = 0; k < 3; ++k) sc.vel[k] = anim[cur].vel[k];
            sc.hasVelocity = true;
            sc.velocityScale = animVelScale;
        }
    }

    // learned target: network parameters and box, optional externally supplied T per vertex
    // slot, and the frame's per-slot queries and training samples (exports for the tests)
    std::vector<float> lpParams;
    float lpBmin[3] = {0, 0, 0}, lpBinv[3] = {1, 1, 1};
    std::vector<float> lpTIn;
    std::vector<float> lpQueries, lpTrain, lpTUsed;
    std::atomic<int64_t> lpVertices{0};     // vertex records written by the last learned-target frame

    int curPass = 0;     // 0 features, 1 initial, 2 temporal, 3 spatial, 4 final, 5 reference
    template <class F>
    void forRows(F f) {
        int nt = numThreads > 0 ? numThreads : (int)std::thread::hardware_concurrency();
        const int pass = curPass;
        auto row = [&](int y) {
            tl_voxReads = 0;
            tl_voxSplit = 0;
            f(y);
            g_voxReads[pass] += tl_voxReads - tl_voxSplit;
            g_voxReads[7] += tl_voxSplit;
        };
        if (nt <= 1) { for (int y = 0; y < H; ++y) row(y); return; }
        std::atomic<int> next(0);
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t)
            th.emplace_back([&]() { for (int y; (y = next.fetch_add(1)) < H;) row(y); });
        for (auto& t : th) t.join();
    }

    void alloc() {
        size_t n = (size_t)W * H;
        int mb = opts.mMaxBounces;
        for (int i = 0; i < 2; ++i) {
            perPixel[i].assign(n, Reservoir{});
            memset(perPixel[i].data(), 0, n * sizeof(Reservoir));
            extraPP[i].assign(n * (size_t)std::max(mb - 1, 1), mk3(0.f));
        }
        temporal.assign(n, Reservoir{});
        memset(temporal.data(), 0, n * sizeof(Reservoir));
        extraTemporal.assign(n * (size_t)std::max(mb - 1, 1), mk3(0.f));
        features.assign(n, Features{0, 0.f});
        temporalFeatures.assign(n, Features{0, 0.f});
        color.assign(n * 4, 0.f);
        lastMaxBounces = mb;
    }

    void makeOptions(Ctx& c) {
        const vr_options& o = opts;
        c.o = &opts;
        c.sc = &sc;
        c.W = W; c.H = H;
        c.maxBounces = o.mMaxBounces;
        c.noReuse = !o.mEnableSpatialReuse && !o.mEnableTemporalReuse;
        c.initial = SamplingOptions{VR_TRACK_ANALYTIC, o.mInitialLightingTrackingMethod, o.mInitialLightSamples, o.mInitialLightingMipLevel, 1,
                                    o.mInitialVisibilityUseLinearSampler ? o.mInitialBaseMipLevel : o.mInitialBaseMipLevel + kNumMaxMips,
                                    o.mInitialVisibilityUseLinearSampler != 0, o.mInitialLightingUseLinearSampler != 0,
                                    o.mInitialVisibilityTStepScale, o.mInitialLightingTStepScale,
                                    o.mUseEnvironmentLights != 0, o.mUseAnalyticLights != 0};
        c.spatial = SamplingOptions{o.mSpatialVisibilityTrackingMethod, o.mSpatialLightingTrackingMethod, 1, o.mSpatialLightingMipLevel, 1,
                                    o.mSpatialVisibilityMipLevel, o.mSpatialVisibilityUseLinearSampler != 0, o.mSpatialLightingUseLinearSampler != 0,
                                    o.mSpatialVisibilityTStepScale, o.mSpatialLightingTStepScale,
                                    o.mUseEnvironmentLights != 0, o.mUseAnalyticLights != 0};
        bool flA = o.mFinalLightTrackingMethod == VR_TRACK_ANALYTIC || o.mFinalLightTrackingMethod == VR_TRACK_RAY_MARCHING;
        bool fvA = o.mFinalVisibilityTrackingMethod == VR_TRACK_ANALYTIC || o.mFinalVisibilityTrackingMethod == VR_TRACK_RAY_MARCHING;
        c.fin = SamplingOptions{o.mFinalVisibilityTrackingMethod, o.mFinalLightTrackingMethod, flA ? 1 : o.mFinalLightSamples, 0,
                                fvA ? 1 : o.mFinalVisibilitySamples, 0, true, true, o.mFinalTStepScale, o.mFinalTStepScale,
                                o.mUseEnvironmentLights != 0, o.mUseAnalyticLights != 0};
        // VolumetricReSTIR.cpp:118-121, 376-386: the VERTEX_REUSE define, for paths with indirect vertices
        const int vrs = (o.mVertexReuse && o.mMaxBounces > 1) ? o.mVertexReuseStartBounce : -1;
        c.initial.vertexReuseStartBounce = vrs;
        c.spatial.vertexReuseStartBounce = vrs;
        c.fin.vertexReuseStartBounce = vrs;
    }

    // GenerateFeatures.cs.slang:57-101
    void passFeatures(Ctx& c, const CamFrame& cam) {
        forRows([&](int y) {
            for (int x = 0; x < W; ++x) {
                Rng sg{};   // unused by the feature adapter
                Ray ray{cam.posW, normalize(rayDirPinhole(cam, x, y, W, H)), 0, kRayTMax};
                float tr = ReservoirFeatureRayMarching(sc, ray, sg, 0, true, c.initial.visibilityTStepScale);
                features[(size_t)y * W + x] = Features{1, tr};
            }
        });
    }

    // TraceRays.cs.slang:64-200 (ReSTIR branch)
    void passTraceRays(Ctx& c, const CamFrame& cam, int numTotalRounds) {
        const int mb = c.maxBounces, mbe = std::max(mb - 1, 1);
        std::atomic<bool> ll(false);
        forRows([&](int y) {
            Ctx cl = c;
            for (int x = 0; x < W; ++x) {
                Rng sg = rng_create((uint32_t)x, (uint32_t)y, (uint32_t)(numTotalRounds * frameCount));
                int reservoirId = y * W + x;
                Ray ray{cam.posW, normalize(rayDirPinhole(cam, x, y, W, H)), 0.f, kRayTMax};
                f3 finalExtra[3] = {mk3(0.f), mk3(0.f), mk3(0.f)};
                Reservoir fin = createNewReservoir();
                int M = opts.mInitialM;
                int rounds = (M + 3) / 4;
                for (int roundId = 0; roundId < rounds; roundId++) {
                    float hd[4] = {0, 0, 0, 0}, pd[4] = {0, 0, 0, 0}, trs[4] = {0, 0, 0, 0};
                    int roundSamples = roundId == rounds - 1 ? (M - 4 * (rounds - 1)) : 4;
                    if (!c.noReuse)
                        SampleMediumAnalyticGeneric(sc, ray, sg, c.initial.visibilityUseLinearSampler, hd, c.initial.visibilityMipLevel, pd, trs, roundSamples);
                    for (int sid = 0; sid < roundSamples; sid++) {
                        f3 ex[3] = {mk3(0.f), mk3(0.f), mk3(0.f)};
                        Reservoir outR = ComputeInitialSample(cl, ray, hd[sid], pd[sid], trs[sid], sg, ex);
                        bool sel = simpleResampleStep(outR, fin, sg);
                        if (sel && mb > 1) {
                            int mib = decodeMaxIndirectBounces(fin.sampledPixel, mb);
                            for (int b = 0; b < mib; b++) finalExtra[b] = ex[b];
                        }
                    }
                }
                ExtraProvider prov{finalExtra};
                float p_hat = evaluate_P_hat(cl, ray, sg, prov, c.spatial, fin, false, false, &fin.p_partial);
                if (fin.runningSum > 0.f) {
                    fin.runningSum *= fin.p_y == 0.f ? 0.f : p_hat / fin.p_y;
                    fin.p_y = p_hat;
                }
                fin.extraBounceStartId = mb > 1 ? reservoirId * (mb - 1) : 0;
                perPixel[0][reservoirId] = fin;
                if (mb > 1) {
                    int mib = decodeMaxIndirectBounces(fin.sampledPixel, mb);
                    for (int b = 0; b < mib; b++) extraPP[0][(size_t)fin.extraBounceStartId + b] = finalExtra[b];
                }
                (void)mbe;
            }
            if (cl.loopLimit) ll = true;
        });
        if (ll) loopLimit = true;
    }

    // The initial pass with the learned target: candidates recorded with deferred shadow rays,
    // T per query slot from lpTIn (when supplied) or the CPU network, then resampling of the
    // records and the rest of TraceRays
    void passTraceRaysLP(Ctx& c, const CamFrame& cam, int numTotalRounds) {
        const int mb = c.maxBounces, M = opts.mInitialM;
        const size_t N = (size_t)W * H;
        lpQueries.assign((size_t)M * mb * N * 8, 0.f);
        lpTUsed.assign((size_t)M * mb * N, 0.f);
        const bool haveT = lpTIn.size() == (size_t)M * mb * N;
        std::vector<float> lpWt;
        if (!haveT) lpo::roundedWeights(lpParams.data(), lpWt);
        std::atomic<bool> ll(false);
        lpVertices = 0;
        forRows([&](int y) {
            Ctx cl = c;
            std::vector<LpVertex> rec((size_t)M * mb);
            std::vector<f3> ex((size_t)M * std::max(mb - 1, 1));
            std::vector<float> crec((size_t)M * 2), q((size_t)mb * 8), dist((size_t)M * 3);
            for (int x = 0; x < W; ++x) {
                Rng sg = rng_create((uint32_t)x, (uint32_t)y, (uint32_t)(numTotalRounds * frameCount));
                const size_t pid = (size_t)y * W + x;
                Ray ray{cam.posW, normalize(rayDirPinhole(cam, x, y, W, H)), 0.f, kRayTMax};
                // the rounds of primary distance samples from the pixel's stream, then each
                // candidate's vertices from its own stream
                int rounds = (M + 3) / 4;
                for (int roundId = 0, cid = 0; roundId < rounds; roundId++) {
                    float hd[4] = {0, 0, 0, 0}, pd[4] = {0, 0, 0, 0}, trs[4] = {0, 0, 0, 0};
                    int rs = roundId == rounds - 1 ? (M - 4 * (rounds - 1)) : 4;
                    SampleMediumAnalyticGeneric(sc, ray, sg, c.initial.visibilityUseLinearSampler, hd, c.initial.visibilityMipLevel, pd, trs, rs);
                    for (int sid = 0; sid < rs; sid++, cid++) { dist[cid * 3] = hd[sid]; dist[cid * 3 + 1] = pd[sid]; dist[cid * 3 + 2] = trs[sid]; }
                }
                {
                    for (int cid = 0; cid < M; ++cid) {
                        float uc = 0.f;
                        float depth = ComputeInitialSampleLP(cl, ray, dist[cid * 3], dist[cid * 3 + 1], dist[cid * 3 + 2], &rec[(size_t)cid * mb],
                                                             &ex[(size_t)cid * std::max(mb - 1, 1)], q.data(), x, y, frameCount, cid, &uc);
                        crec[cid * 2] = depth;
                        crec[cid * 2 + 1] = uc;
                        int nv = 0;
                        for (int b = 0; b < mb; ++b) nv += (rec[(size_t)cid * mb + b].flags & kLpValid) ? 1 : 0;
                        lpVertices += nv;
                        for (int b = 0; b < mb; ++b) {
                            const size_t slot = (size_t)(cid * mb + b) * N + pid;
                            if (rec[(size_t)cid * mb + b].flags & kLpNeedsT) {
                                memcpy(&lpQueries[slot * 8], &q[b * 8], 8 * sizeof(float));
                                float t;
                                if (haveT) t = lpTIn[slot];
                                else {
                                    float act[5][64];
                                    float o = lpo::forwardR(lpParams.data(), lpWt.data(), &q[b * 8], &q[b * 8 + 3], lpBmin, lpBinv, act);
                                    t = lpo::predict(o, opts.mLearnedTFloor);
                                }
                                lpTUsed[slot] = t;
                            } else {
                                lpQueries[slot * 8 + 6] = -1.f;
                            }
                        }
                    }
                }
                // select
                f3 finalExtra[3] = {mk3(0.f), mk3(0.f), mk3(0.f)};
                Reservoir fin = createNewReservoir();
                for (int ci = 0; ci < M; ++ci) {
                    Reservoir comb = createNewReservoir();
                    for (int b = 0; b < mb; ++b) {
                        const LpVertex& v = rec[(size_t)ci * mb + b];
                        if (!(v.flags & kLpValid)) break;
                        Reservoir out = createNewReservoir();
                        out.M = 1; out.depth = crec[ci * 2];
                        out.runningSum = v.a; out.p_y = v.b; out.lightUV[0] = v.uv0; out.lightUV[1] = v.uv1;
                        out.lightID = v.lightID; out.sampledPixel = v.sampledPixel;
                        if (v.flags & kLpNeedsT) {
                            float p_y = v.b * lpTUsed[(size_t)(ci * mb + b) * N + pid];
                            out.runningSum = v.a == 0.f ? 0.f : p_y / v.a;
                            out.p_y = p_y;
                        }
                        if (mb > 1) simpleResampleStepU(out, comb, v.u);
                        else comb = out;
                    }
                    if (mb > 1) comb.M = 1;
                    bool sel = simpleResampleStepU(comb, fin, crec[ci * 2 + 1]);
                    if (sel && mb > 1) {
                        int mib = decodeMaxIndirectBounces(fin.sampledPixel, mb);
                        for (int b = 0; b < mib; b++) finalExtra[b] = ex[(size_t)ci * (mb - 1) + b];
                    }
                }
                ExtraProvider prov{finalExtra};
                const uint64_t r0 = tl_voxReads;
                float p_hat = evaluate_P_hat(cl, ray, sg, prov, c.spatial, fin);
                tl_voxSplit += tl_voxReads - r0;      // the select kernel's share
                if (fin.runningSum > 0.f) {
                    fin.runningSum *= fin.p_y == 0.f ? 0.f : p_hat / fin.p_y;
                    fin.p_y = p_hat;
                }
                fin.extraBounceStartId = mb > 1 ? (int)pid * (mb - 1) : 0;
                perPixel[0][pid] = fin;
                if (mb > 1) {
                    int mib = decodeMaxIndirectBounces(fin.sampledPixel, mb);
                    for (int b = 0; b < mib; b++) extraPP[0][(size_t)fin.extraBounceStartId + b] = finalExtra[b];
                }
            }
            if (cl.loopLimit) ll = true;
        });
        if (ll) loopLimit = true;
    }

    // training samples of the network, drawn from this frame's queries: a pixel and a starting
    // slot from the sample's own stream, the first slot of the pixel (cyclically) that holds a
    // query (up to 4 pixels tried), and a full-resolution transmittance estimate of its shadow
    // ray as the target
    void passTrainGenLP(Ctx& c) {
        const int S = opts.mLearnedTrainSamples;
        const int numSlots = opts.mInitialM * c.maxBounces;
        const int N = W * H;
        lpTrain.assign((size_t)std::max(S, 0) * 8, 0.f);
        const uint32_t seed = 0x80000000u | ((opts.mLearnedSeed * 0x9E3779B9u + (uint32_t)frameCount) & 0x7FFFFFFFu);
        const int rows = (S + 255) / 256;
        std::atomic<int> next(0);
        std::atomic<bool> ll(false);
        int nt = numThreads > 0 ? numThreads : (int)std::thread::hardware_concurrency();
        auto work = [&]() {
            Ctx cl = c;
            for (int r; (r = next.fetch_add(1)) < rows;) {
                for (int i = r * 256; i < std::min(S, r * 256 + 256); ++i) {
                    Rng sg = rng_create((uint32_t)i & 0x3FFFu, (uint32_t)i >> 14, seed);
                    long slot = -1;
                    for (int att = 0; att < 4 && slot < 0; ++att) {
                        const int pid = std::min(N - 1, (int)(next1D(sg) * (float)N));
                        const int j0 = std::min(numSlots - 1, (int)(next1D(sg) * (float)numSlots));
                        for (int k = 0; k < numSlots; ++k) {
                            int j = j0 + k;
                            if (j >= numSlots) j -= numSlots;
                            const long s = (long)j * N + pid;
                            if (lpQueries[(size_t)s * 8 + 6] >= 0.f) { slot = s; break; }
                        }
                    }
                    float* o = &lpTrain[(size_t)i * 8];
                    if (slot >= 0) {
                        const float* q = &lpQueries[(size_t)slot * 8];
                        Ray sr{mk3(q[0], q[1], q[2]), mk3(q[3], q[4], q[5]), 0, q[6]};
                        float t = computeVisibility(sc, sr, sg, 1, 0, true, opts.mLearnedTargetMethod, 1.f);
                        for (int k = 0; k < 7; ++k) o[k] = q[k];
                        o[7] = t;
                    } else {
                        o[6] = -1.f;
                    }
                }
            }
            if (cl.loopLimit) ll = true;
        };
        if (nt <= 1) work();
        else {
            std::vector<std::thread> th;
            for (int t = 0; t < nt; ++t) th.emplace_back(work);
            for (auto& t : th) t.join();
        }
        if (ll) loopLimit = true;
    }

    // TraceRays.cs.slang:85-103 (reference branch) + IntegrateByVolumePathTracing
    f3 integratePT(Ctx& c, Ray ray, Rng& sg) {
        const Scene& s = sc;
        int maxBounces = c.maxBounces;
        const bool useNEE = true;
        const int lightSamples = std::max(1, c.initial.lightSamples);
        MediumInteraction mi;
        f3 beta = mk3(1.f), L = mk3(0.f);
        if (!useNEE) maxBounces += 1;
        for (int bounce = 0; bounce < maxBounces; bounce++) {
            mi.isValid = false;
            SampleMediumSuperVoxelGeneric(s, ray, sg, mi, 0, c.loopLimit);
            if (mi.isValid) {
                f3 albedo = s.med.sigma_s / s.med.sigma_t;
                f3 one_minus_albedo = mk3(1.f) - albedo;
                { f3 Le = EmissionWorldSpace(s, mi.p); L = L + Le * one_minus_albedo * beta; }
                beta = beta * albedo;
                if (useNEE) {
                    // directLighting (VolumeUtils.slang:453-483)
                    f3 Ld = mk3(0.f);
                    for (int ls_i = 0; ls_i < lightSamples; ls_i++) {
                        SceneLightSample ls; int idx; float uv[2];
                        bool valid = sampleSceneLights(s, mi.p, c.initial.useEnvironmentLights, c.initial.useAnalyticLights, sg, ls, idx, uv);
                        if (!valid) continue;
                        ls.pdf = 1.f;
                        Ray shadowRay{mi.p, ls.rayDir, 0, ls.rayDistance};
                        float visibility = computeVisibility(s, shadowRay, sg, 1, 0, true, VR_TRACK_RESIDUAL_RATIO, 1.f);
                        ls.Li = ls.Li * visibility;
                        float p = phaseFunction(mi, mi.wo, ls.dir);
                        Ld = Ld + p * ls.Li / ls.pdf;
                    }
                    Ld = Ld / (float)lightSamples;
                    L = L + beta * Ld;
                }
                f3 wo = -ray.dir, wi = mk3(0.f);
                if (maxBounces > 1) { float u0 = next1D(sg), u1 = next1D(sg); Sample_p(mi, wo, wi, u0, u1); }
                if (bounce < maxBounces - 1) {
                    ray = Ray{mi.p, wi, 0, kRayTMax};
                    if (c.o->mInitialUseRussianRoulette && bounce >= 2) {
                        if (next1D(sg) < albedo.x) beta = beta / albedo.x;
                        else bounce = maxBounces;
                    }
                }
            } else {
                f3 Le = envEval(s, ray.dir);
                if (!useNEE || bounce == 0) L = L + beta * Le;
                bounce = maxBounces;
            }
        }
        return L;
    }

    // TemporalReuse.cs.slang:80-377
    void passTemporal(Ctx& c, const CamFrame& cam, int numTotalRounds, bool isFirstFrame, float* mvec) {
        if (isFirstFrame) return;
        const int mb = c.maxBounces;
        const uint32_t N = (uint32_t)(W * H);
        forRows([&](int py) {
            Ctx cl = c;
            for (int px = 0; px < W; ++px) {
                Rng sg = rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(numTotalRounds * frameCount + 1));
                int selectedId = -1;
                int pixelId = py * W + px;
                int numUsed = 1;
                Reservoir taps[2];
                taps[0] = perPixel[0][pixelId];
                taps[1] = createNewReservoir();
                Ray ray{cam.posW, normalize(rayDirPinhole(cam, px, py, W, H)), 0, kRayTMax};
                Reservoir output = opts.mTemporalMISMethod == VR_MIS_TALBOT ? createNewReservoir() : taps[0];
                int centerStart = taps[0].extraBounceStartId;
                float temporalOriginalDepth = 0.f;
                int reprojX = 0, reprojY = 0;
                Features cf = features[pixelId];
                bool isBackgroundReservoir = cf.transmittance == 1.f && cf.noReflectiveSurface;
                bool useFallback = true;
                bool earlyOut = false;
                if (opts.mTemporalReprojectionMode != VR_REPROJ_NONE) {
                    float reprojDepth = taps[0].depth;
                    if (reprojDepth == kRayTMax && opts.mTemporalReprojectionMode != VR_REPROJ_NO_BACKGROUND && !isBackgroundReservoir)
                        reprojDepth = RejectionSampleRandomPointByDensity(sc, ray, sg, kNumMaxMips + opts.mTemporalReprojectionMipLevel);
                    f3 p = ray.origin + ray.dir * reprojDepth;
                    // find last frame world position if having velocity grid (TemporalReuse.cs.slang:161-166);
                    // a background point keeps its own pixel below and needs none
                    if (sc.hasVelocity && sc.hasAnimation && reprojDepth != kRayTMax) {
                        f3 v = VelocityWorld(sc, p) * sc.velocityScale;
                        p = p - v;
                    }
                    float in4[4] = {p.x, p.y, p.z, 1.f}, vp[4], cp[4];
                    mulMat4(prev.view, in4, vp);
                    mulMat4(prev.proj, vp, cp);
                    float sx = cp[0] / cp[3], sy = cp[1] / cp[3];
                    int sxi, syi;
                    if (reprojDepth == kRayTMax) { sx = (float)px + 0.5f; sy = (float)py + 0.5f; sxi = px; syi = py; }
                    else {
                        sx = 0.5f * sx + 0.5f; sy = -0.5f * sy + 0.5f;
                        sx *= (float)W; sy *= (float)H;
                        sxi = f2i(sx); syi = f2i(sy);
                    }
                    {
                        uint32_t id = (uint32_t)syi * (uint32_t)W + (uint32_t)sxi;
                        Features tf = id < N ? temporalFeatures[id] : Features{0, 0.f};
                        bool isTapBackground = tf.transmittance == 1.f && tf.noReflectiveSurface;
                        if (isBackgroundReservoir && !isTapBackground) {
                            if (mvec) { mvec[pixelId * 2] = (float)(reprojX - px) / (float)W; mvec[pixelId * 2 + 1] = (float)(reprojY - py) / (float)H; }
                            earlyOut = true;
                        }
                    }
                    if (!earlyOut) {
                        sxi = f2i(sx); syi = f2i(sy);
                        reprojX = sxi; reprojY = syi;
                        if (sxi >= 0 && sxi < W && syi >= 0 && syi < H) {
                            numUsed++;
                            taps[1] = temporal[(size_t)syi * W + sxi];
                        }
                        if (numUsed > 1) useFallback = false;
                    }
                }
                if (earlyOut) continue;
                if (useFallback) { numUsed++; reprojX = px; reprojY = py; taps[1] = temporal[pixelId]; }
                if (mvec) { mvec[pixelId * 2] = (float)(reprojX - px) / (float)W; mvec[pixelId * 2 + 1] = (float)(reprojY - py) / (float)H; }
                float curM = taps[0].M;
                float MaxPrevM = opts.mTemporalReuseMThreshold * curM;
                if (numUsed == 2) {
                    temporalOriginalDepth = taps[1].depth;
                    if (taps[1].depth != kRayTMax) {
                        f3 dir = normalize(rayDirPinhole(prev, reprojX, reprojY, W, H));
                        f3 worldPos = prev.posW + taps[1].depth * dir;
                        taps[1].depth = length(worldPos - ray.origin);
                    }
                }
                float centerPrevFrameDepth = taps[0].depth;
                if (centerPrevFrameDepth != kRayTMax) {
                    f3 worldPos = ray.at(centerPrevFrameDepth);
                    centerPrevFrameDepth = length(worldPos - prev.posW);
                }
                bool hasSelection = output.runningSum > 0.f;
                bool talbot = opts.mTemporalMISMethod == VR_MIS_TALBOT;
                int start = talbot ? 0 : 1;
                if (start == 1) selectedId = 0;
                ExtraProvider curProv{extraPP[0].data()}, tempProv{extraTemporal.data()};
                for (int i = start; i < numUsed; i++) {
                    float talbotMISWeight = 1.f;
                    float neighbor_py = 0.f;
                    if (taps[i].p_y > 0.f) {
                        neighbor_py = taps[i].p_y;
                        if (isnan_(taps[i].runningSum) || isinf_(taps[i].runningSum)) taps[i].runningSum = 0.f;
                        if (i > 0) resampleNeighbor(cl, taps[i], ray, sg, tempProv, cl.spatial);
                    } else { taps[i].p_y = 0.f; taps[i].runningSum = 0.f; }
                    if (talbot && taps[i].runningSum > 0.f) {
                        float p_sum = 0, p_qi = 0, k = 0;
                        for (int j = 0; j < numUsed; j++) {
                            float correctedM = fmin_(MaxPrevM, taps[j].M);
                            k += correctedM;
                            if (j == 0) { p_qi = taps[i].p_y; p_sum += taps[i].p_y * correctedM; }
                            else if (i == j) { p_qi = neighbor_py; p_sum += neighbor_py * correctedM; }
                            else {
                                // j > 0 here: previous-frame camera ray through the reprojected pixel
                                Ray nr{prev.posW, normalize(rayDirPinhole(prev, reprojX, reprojY, W, H)), 0,
                                       i == 0 ? centerPrevFrameDepth : temporalOriginalDepth};
                                float backupDepth = taps[i].depth;
                                taps[i].depth = nr.tMax;
                                float p_y = evaluate_P_hat(cl, nr, sg, i == 0 ? curProv : tempProv, cl.spatial, taps[i], true);
                                taps[i].depth = backupDepth;
                                if (isinf_(p_y) || isnan_(p_y)) p_y = 0.f;
                                p_sum += p_y * correctedM;
                            }
                        }
                        if (p_sum > 0) talbotMISWeight = p_qi * k / p_sum;
                    }
                    taps[i].runningSum *= talbotMISWeight;
                    bool sel = simpleResampleStepWithMaxM(taps[i], MaxPrevM, output, sg);
                    hasSelection |= sel;
                    if (sel) selectedId = i;
                }
                if (mb > 1) {
                    if (hasSelection && selectedId > 0) {
                        int mib = decodeMaxIndirectBounces(output.sampledPixel, mb);
                        for (int b = 0; b < mib; b++) extraPP[0][(size_t)centerStart + b] = extraTemporal[(size_t)output.extraBounceStartId + b];
                    }
                    output.extraBounceStartId = centerStart;
                }
                perPixel[0][pixelId] = output;
            }
        });
    }

    // SpatialReuse.cs.slang:64-81 (offsets are the same for every pixel of a round)
    static void neighborOffsets(const vr_options& o, int r2TimeSeed, int offs[][2]) {
        for (int sid = 0; sid < o.mSpatialSampleCount; ++sid) {
            float ux, uy;
            if (o.mRandomSamplerType == VR_SAMPLER_HAMMERSLEY) {
                ux = (float)sid / (float)o.mSpatialSampleCount;
                uint32_t i = (uint32_t)sid;
                i = (i & 0x55555555u) << 1 | (i & 0xAAAAAAAAu) >> 1;
                i = (i & 0x33333333u) << 2 | (i & 0xCCCCCCCCu) >> 2;
                i = (i & 0x0F0F0F0Fu) << 4 | (i & 0xF0F0F0F0u) >> 4;
                i = (i & 0x00FF00FFu) << 8 | (i & 0xFF00FF00u) >> 8;
                i = (i << 16) | (i >> 16);
                uy = (float)i * 2.3283064365386963e-10f;
            } else {
                double multiplier = (double)(r2TimeSeed * o.mSpatialSampleCount + sid);
                if (sid == 0) { ux = 0; uy = 0; }
                else {
                    double a = 0.754877669 * multiplier, b = 0.569840296 * multiplier;
                    ux = (float)(a - std::floor(a)); uy = (float)(b - std::floor(b));
                }
            }
            float r = sqrt_(ux), phi = kM_2PI * uy;
            float dx = r * cos_(phi), dy = r * sin_(phi);
            offs[sid][0] = f2i(o.mSampleRadius * dx);
            offs[sid][1] = f2i(o.mSampleRadius * dy);
        }
    }

    void passSpatial(Ctx& c, const CamFrame& cam, int roundId, int roundOffset, int in, int out) {
        const int mb = c.maxBounces;
        int numRounds = opts.mSpatialReuseRounds + roundOffset + 1;
        int rid = roundId + roundOffset;
        int r2TimeSeed = ((opts.mSpatialReuseRounds + 1) * frameCount + roundId) % 16;
        int offs[64][2];
        neighborOffsets(opts, r2TimeSeed, offs);
        const int K = opts.mSpatialSampleCount;
        bool talbot = opts.mSpatialMISMethod == VR_MIS_TALBOT;
        forRows([&](int py) {
            Ctx cl = c;
            for (int px = 0; px < W; ++px) {
                Rng sg = rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(numRounds * frameCount + rid));
                const int pixelId = py * W + px;
                Reservoir output = perPixel[in][pixelId];
                int centerStart = output.extraBounceStartId;
                Ray ray{cam.posW, normalize(rayDirPinhole(cam, px, py, W, H)), 0, kRayTMax};
                if (talbot) output = createNewReservoir();
                bool hasSelection = output.runningSum > 0.f;
                bool selfBg = features[pixelId].transmittance == 1.f;
                ExtraProvider prov{extraPP[in].data()};
                if (selfBg) {
                    perPixel[out][pixelId] = talbot ? perPixel[in][pixelId] : output;
                    if (mb > 1) {
                        int mib = decodeMaxIndirectBounces(output.sampledPixel, mb);
                        for (int b = 0; b < mib; b++) extraPP[out][(size_t)output.extraBounceStartId + b] = extraPP[in][(size_t)output.extraBounceStartId + b];
                    }
                    continue;
                }
                for (int sid = talbot ? 0 : 1; sid < K; sid++) {
                    int tx = px + offs[sid][0], ty = py + offs[sid][1];
                    if (!(tx >= 0 && tx < W && ty >= 0 && ty < H)) continue;
                    Reservoir tap = perPixel[in][(size_t)ty * W + tx];
                    float MISWeight = 1.f;
                    if (sid > 0) resampleNeighbor(cl, tap, ray, sg, prov, cl.spatial, true);
                    if (talbot && tap.runningSum > 0.f) {
                        float p_sum = 0, p_qi = 0, k = 0;
                        for (int j = 0; j < K; j++) {
                            int tx2 = px + offs[j][0], ty2 = py + offs[j][1];
                            if (!(tx2 >= 0 && tx2 < W && ty2 >= 0 && ty2 < H)) continue;
                            const Reservoir& tap2 = perPixel[in][(size_t)ty2 * W + tx2];
                            k += tap2.M;
                            if (j == 0) { p_qi = tap.p_y; p_sum += tap.p_y * tap2.M; }
                            else if (sid == j) { p_qi = tap2.p_y; p_sum += tap2.p_y * tap2.M; }
                            else {
                                Ray nr{ray.origin, normalize(rayDirPinhole(cam, tx2, ty2, W, H)), 0, tap.depth};
                                float p_y = evaluate_P_hat(cl, nr, sg, prov, cl.spatial, tap, false, true);
                                if (isinf_(p_y) || isnan_(p_y)) p_y = 0.f;
                                p_sum += p_y * tap2.M;
                            }
                        }
                        if (p_sum > 0) MISWeight = p_qi * k / p_sum;
                    }
                    tap.runningSum *= MISWeight;
                    if (simpleResampleStep(tap, output, sg)) hasSelection = true;
                }
                if (mb > 1) {
                    if (hasSelection) {
                        int mib = decodeMaxIndirectBounces(output.sampledPixel, mb);
                        for (int b = 0; b < mib; b++) extraPP[out][(size_t)centerStart + b] = extraPP[in][(size_t)output.extraBounceStartId + b];
                    }
                    output.extraBounceStartId = centerStart;
                }
                perPixel[out][pixelId] = output;
            }
        });
    }

    // CopyReservoirs.cs.slang:84-94
    void passCopy(int cur) {
        const int mb = opts.mMaxBounces;
        for (size_t i = 0; i < (size_t)W * H; ++i) {
            const Reservoir& r = perPixel[cur][i];
            temporal[i] = r;
            if (mb > 1) {
                int mib = decodeMaxIndirectBounces(r.sampledPixel, mb);
                for (int b = 0; b < mib; b++) extraTemporal[(size_t)r.extraBounceStartId + b] = extraPP[cur][(size_t)r.extraBounceStartId + b];
            }
        }
    }

    // FinalShading.cs.slang:71-143
    void passFinal(Ctx& c, const CamFrame& cam, int numTotalRounds, int cur, float* outRGBA) {
        forRows([&](int py) {
            Ctx cl = c;
            for (int px = 0; px < W; ++px) {
                int pixelId = py * W + px;
                f3 outputColor = mk3(0.f);
                Rng sg = rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(numTotalRounds * frameCount + numTotalRounds - 1));
                if (opts.mUseReference) {
                    outputColor = mk3(color[(size_t)pixelId * 4], color[(size_t)pixelId * 4 + 1], color[(size_t)pixelId * 4 + 2]);
                } else if (opts.mVisualizeTotalTransmittance) {
                    outputColor = mk3(pow_(features[pixelId].transmittance, 2.2f));
                } else {
                    const Reservoir& r = perPixel[cur][pixelId];
                    if (r.runningSum > 0.f) {
                        Ray ray{cam.posW, normalize(rayDirPinhole(cam, px, py, W, H)), 0, r.depth};
                        ExtraProvider prov{extraPP[cur].data()};
                        f3 col = evaluate_F_(cl, r, prov, ray, sg, cl.fin, cl.noReuse, true);
                        float Wt = r.p_y == 0.0f ? 1.f : r.runningSum / (r.p_y * r.M);
                        col = col * Wt;
                        outputColor = outputColor + col;
                    }
                }
                float cc[4] = {outputColor.x, outputColor.y, outputColor.z, 1.f};
                bool bad = false;
                for (int k = 0; k < 4; ++k) bad |= isnan_(cc[k]) || isinf_(cc[k]);
                for (int k = 0; k < 4; ++k) outRGBA[(size_t)pixelId * 4 + k] = bad ? 0.f : cc[k];
            }
        });
    }

    // VolumetricReSTIR::execute (VolumetricReSTIR.cpp:303-906)
    void renderFrame(const vr_camera& camIn, float* outRGBA, float* mvec) {
        if (optionsChanged) { frameCount = 0; temporalSampleAccumulated = 0; optionsChanged = false; }
        sc.usePrevGrid = opts.mUsePrevVolumeForReproj != 0;
        if (perPixel[0].size() != (size_t)W * H || lastMaxBounces != opts.mMaxBounces) alloc();
        Ctx c; makeOptions(c);
        CamFrame cam = makeCamera(camIn, W, H);
        int numTotalRounds = (opts.mEnableSpatialReuse ? opts.mSpatialReuseRounds : 0) + opts.mEnableTemporalReuse + 1 + 1;
        curPass = 0;
        if (!opts.mUseReference) passFeatures(c, cam);
        curPass = opts.mUseReference ? 5 : 1;
        if (opts.mUseReference) {
            forRows([&](int y) {
                Ctx cl = c;
                for (int x = 0; x < W; ++x) {
                    Rng sg = rng_create((uint32_t)x, (uint32_t)y, (uint32_t)(numTotalRounds * frameCount));
                    Ray ray{cam.posW, normalize(rayDirPinhole(cam, x, y, W, H)), 0.f, kRayTMax};
                    f3 avg = mk3(0.f);
                    for (int r = 0; r < opts.mBaselineSamplePerPixel; ++r) avg = avg + integratePT(cl, ray, sg);
                    avg = avg / (float)opts.mBaselineSamplePerPixel;
                    size_t i = (size_t)y * W + x;
                    color[i * 4] = avg.x; color[i * 4 + 1] = avg.y; color[i * 4 + 2] = avg.z; color[i * 4 + 3] = 1.f;
                }
                if (cl.loopLimit) loopLimit = true;
            });
        } else if (opts.mUseLearnedPHat && (opts.mEnableTemporalReuse || opts.mEnableSpatialReuse)) {
            passTraceRaysLP(c, cam, numTotalRounds);
            if (opts.mLearnedTrainSamples > 0) passTrainGenLP(c);
        } else {
            passTraceRays(c, cam, numTotalRounds);
        }
        int totalRoundId = 0;
        if (!opts.mUseReference && opts.mEnableTemporalReuse) {
            curPass = 2;
            passTemporal(c, cam, numTotalRounds, temporalSampleAccumulated == 0, mvec);
            if (!opts.mEnableSpatialReuse) {
                temporal = perPixel[totalRoundId];
                if (opts.mMaxBounces > 1) extraTemporal = extraPP[totalRoundId];
            }
            temporalFeatures = features;
        }
        if (!opts.mUseReference && opts.mEnableSpatialReuse) {
            curPass = 3;
            for (int r = 0; r < opts.mSpatialReuseRounds; ++r) {
                passSpatial(c, cam, r, opts.mEnableTemporalReuse + 1, totalRoundId % 2, (totalRoundId + 1) % 2);
                totalRoundId++;
            }
        }
        if (!opts.mUseReference && opts.mEnableTemporalReuse) passCopy(totalRoundId % 2);
        curPass = 4;
        passFinal(c, cam, numTotalRounds, totalRoundId % 2, outRGBA);
        finalBuffer = totalRoundId % 2;
        temporalSampleAccumulated = 1;
        prev = cam;
        frameCount++;
    }
    int finalBuffer = 0;
};

}  // namespace oracle

// ---------------------------------------------------------------------------------------
// C API (test infrastructure)
// ---------------------------------------------------------------------------------------
using oracle::Oracle;

extern "C" {

void* vro_create(const vr_options* o, int W, int H) {
    Oracle* p = new Oracle();
    p->opts = *o; p->W = W; p->H = H;
    return p;
}
void vro_destroy(void* h) { delete (Oracle*)h; }
void vro_set_threads(void* h, int n) { ((Oracle*)h)->numThreads = n; }
void vro_set_options(void* h, const vr_options* o) {
    Oracle* p = (Oracle*)h;
    p->opts = *o;
    p->optionsChanged = true;
}

// BC4 unorm block (the block layout of BCHelper.h:9-69, the format the reference's textures
// use for the coarse and conservative mips, Scene.cpp:3161-3181): red_0 in bits 0-7, red_1 in
// bits 8-15, texel t's 3-bit index at bit 16 + 3 t.  red_0 > red_1: entries red_0, red_1 and
// (7 - k) red_0 + k red_1 over 7 for k = 1..6; otherwise red_0, red_1, (5 - k) red_0 + k red_1
// over 5 for k = 1..4, then 0 and 1.  Each entry is its integer numerator (over 255 * 7 or
// 255 * 5) times that denominator's reciprocal rounded to float.
static float bc4_entry(uint32_t r0, uint32_t r1, uint32_t idx) {
    const float inv8 = 1.0f / 1785.0f, inv6 = 1.0f / 1275.0f;
    if (r0 > r1) {
        uint32_t k = idx == 0 ? 0u : (idx == 1 ? 7u : idx - 1u);
        return (float)((7u - k) * r0 + k * r1) * inv8;
    }
    if (idx == 6) return 0.0f;
    if (idx == 7) return (float)1275u * inv6;
    uint32_t k = idx == 0 ? 0u : (idx == 1 ? 5u : idx - 1u);
    return (float)((5u - k) * r0 + k * r1) * inv6;
}
static float bc4_texel_value(uint64_t blk, int t) {
    return bc4_entry((uint32_t)(blk & 255u), (uint32_t)((blk >> 8) & 255u), (uint32_t)((blk >> (16 + 3 * t)) & 7u));
}

// the 16 texel values of one BC4 block (format check against hand-computed palettes)
void vro_bc4_decode_block(uint64_t block, float out[16]) {
    for (int t = 0; t < 16; ++t) out[t] = bc4_texel_value(block, t);
}

static void load_slot(const vr_grid_view& v, oracle::Slot& d) {
    {
        d.valid = true;
        for (int i = 0; i < 3; ++i) { d.res[i] = v.res[i]; d.bmin[i] = v.bmin[i]; d.bmax[i] = v.bmax[i]; }
        memcpy(d.M, v.world_to_index, sizeof(d.M));
        d.maxValue = v.max_value;
        d.root.assign(v.root_child, v.root_child + 32768);
        d.l1vmin.assign(v.l1_vmin, v.l1_vmin + (size_t)v.num_l1 * 4);
        d.l1child.assign(v.l1_child, v.l1_child + (size_t)v.num_l1 * 4096);
        d.bvmin.assign(v.brick_vmin, v.brick_vmin + (size_t)v.num_bricks * 4);
        d.bounds.assign(v.brick_bounds, v.brick_bounds + (size_t)v.num_bricks * 4);
        d.data.resize((size_t)v.num_bricks * 1000);
        for (size_t i = 0; i < d.data.size(); ++i) {
            if (v.brick_bc4) {
                // brick b, apron voxel (x, y, z): block z * 9 + (y / 4) * 3 + x / 4 of the
                // brick's 90, texel (y % 4) * 4 + x % 4
                const size_t b = i / 1000;
                const int r = (int)(i % 1000), x = r % 10, y = (r / 10) % 10, z = r / 100;
                const uint64_t blk = v.brick_bc4[b * 90 + (size_t)(z * 9 + (y / 4) * 3 + x / 4)];
                d.data[i] = bc4_texel_value(blk, (y % 4) * 4 + x % 4) * v.bc4_scale;
            } else if (v.brick_f32) d.data[i] = v.brick_f32[i];
            else {
                uint16_t hh = v.brick_f16[i];
                uint32_t sign = ((uint32_t)hh & 0x8000u) << 16, e = (hh >> 10) & 0x1fu, mm = hh & 0x3ffu;
                float f;
                if (e == 0) { f = (float)mm * 5.9604644775390625e-08f; if (sign) f = -f; }
                else if (e == 31) f = u2f(sign | 0x7f800000u | (mm << 13));
                else f = u2f(sign | ((e + 112) << 23) | (mm << 13));
                d.data[i] = f;
            }
        }
    }
}

int vro_set_volume(void* h, const vr_grid_view* views, int numViews, const vr_medium* m, float voxelSize, float superDiag, int numMips) {
    Oracle* p = (Oracle*)h;
    oracle::Scene& sc = p->sc;
    for (int s = 0; s < VR_NUM_SLOTS; ++s) sc.slots[s] = oracle::Slot();
    for (int s = 0; s < numViews && s < VR_NUM_SLOTS; ++s)
        if (views[s].valid) load_slot(views[s], sc.slots[s]);
    for (int s = 0; s < VR_NUM_SLOTS; ++s) p->staticSlots[s] = sc.slots[s];
    p->anim.clear();
    p->animId = -1;
    sc.hasAnimation = false;
    sc.hasVelocity = false;
    sc.med.sigma_s = mk3(m->sigma_s[0], m->sigma_s[1], m->sigma_s[2]);
    sc.med.sigma_a = mk3(m->sigma_a[0], m->sigma_a[1], m->sigma_a[2]);
    sc.med.sigma_t = m->sigma_s[0] + m->sigma_a[0];
    sc.med.g = m->g;
    sc.med.dscale = m->density_scale;
    sc.med.tStep = voxelSize;
    sc.med.superDiag = superDiag;
    sc.med.numMips = numMips;
    p->optionsChanged = true;
    return 0;
}

int vro_set_lights(void* h, const vr_point_light* lights, int n, const vr_env_map* env) {
    Oracle* p = (Oracle*)h;
    p->sc.lights.assign(lights, lights + n);
    p->sc.hasEnv = env != nullptr;
    if (env) {
        oracle::EnvMap& e = p->sc.env;
        e.w = env->width; e.h = env->height;
        e.rgb.assign(env->rgb, env->rgb + (size_t)e.w * e.h * 3);
        e.scale = mk3(env->scale[0], env->scale[1], env->scale[2]);
        memcpy(e.rot, env->rotation, sizeof(e.rot));
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) e.inv[i * 3 + j] = env->rotation[j * 3 + i];   // rotation: inverse = transpose
        oracle::buildImportanceMap(e);
    }
    p->optionsChanged = true;
    return 0;
}

int vro_render_frame(void* h, const vr_camera* cam, float* out_rgba, float* mvec) {
    Oracle* p = (Oracle*)h;
    p->loopLimit = false;
    p->animAdvance();
    p->renderFrame(*cam, out_rgba, mvec);
    return p->loopLimit ? VR_ERR_LOOP_LIMIT : VR_OK;
}

int vro_frame_count(void* h) { return ((Oracle*)h)->frameCount; }
// voxel reads per pass since the last call (0 features, 1 initial, 2 temporal, 3 spatial, 4 final, 5 reference)
void vro_voxel_reads(uint64_t out[8]) { for (int i = 0; i < 8; ++i) out[i] = oracle::g_voxReads[i].exchange(0); }

// which: 0 = final reservoirs of the last frame, 1 = temporal history, 2 = perPixel[0], 3 = perPixel[1]
int vro_export_reservoirs(void* h, int which, vr_reservoir_aos* out) {
    Oracle* p = (Oracle*)h;
    const std::vector<oracle::Reservoir>* src;
    if (which == 0) src = &p->perPixel[p->finalBuffer];
    else if (which == 1) src = &p->temporal;
    else src = &p->perPixel[which - 2];
    for (size_t i = 0; i < src->size(); ++i) {
        const oracle::Reservoir& r = (*src)[i];
        vr_reservoir_aos& o = out[i];
        o.runningSum = r.runningSum; o.M = r.M; o.depth = r.depth; o.p_y = r.p_y;
        o.lightUV[0] = r.lightUV[0]; o.lightUV[1] = r.lightUV[1];
        o.lightID = r.lightID; o.sampledPixel = r.sampledPixel; o.extraBounceStartId = r.extraBounceStartId;
        o.p_partial = r.p_partial;
    }
    return 0;
}
int vro_export_extra(void* h, int which, float* out) {
    Oracle* p = (Oracle*)h;
    const std::vector<f3>* src = which == 0 ? &p->extraPP[p->finalBuffer] : (which == 1 ? &p->extraTemporal : &p->extraPP[which - 2]);
    for (size_t i = 0; i < src->size(); ++i) { out[i * 3] = (*src)[i].x; out[i * 3 + 1] = (*src)[i].y; out[i * 3 + 2] = (*src)[i].z; }
    return 0;
}
int vro_export_features(void* h, int32_t* out) {
    Oracle* p = (Oracle*)h;
    for (size_t i = 0; i < p->features.size(); ++i) { out[i * 2] = p->features[i].noReflectiveSurface; memcpy(&out[i * 2 + 1], &p->features[i].transmittance, 4); }
    return 0;
}
// importance map level m of the environment sampler (for cross-checks)
int vro_env_importance(void* h, int mip, float* out) {
    Oracle* p = (Oracle*)h;
    if (mip < 0 || mip >= (int)p->sc.env.imp.size()) return 1;
    memcpy(out, p->sc.env.imp[mip].data(), p->sc.env.imp[mip].size() * 4);
    return 0;
}

// FP64 reference accumulation: adds num_frames frames of the path tracer into accum (W*H*3)
int vro_render_reference(void* h, const vr_camera* cam, int firstFrame, int numFrames, double* accum) {
    Oracle* p = (Oracle*)h;
    oracle::Ctx c; p->makeOptions(c);
    oracle::CamFrame cf = oracle::makeCamera(*cam, p->W, p->H);
    int numTotalRounds = (p->opts.mEnableSpatialReuse ? p->opts.mSpatialReuseRounds : 0) + p->opts.mEnableTemporalReuse + 1 + 1;
    std::atomic<bool> ll(false);
    p->forRows([&](int y) {
        oracle::Ctx cl = c;
        for (int x = 0; x < p->W; ++x) {
            for (int f = firstFrame; f < firstFrame + numFrames; ++f) {
                Rng sg = rng_create((uint32_t)x, (uint32_t)y, (uint32_t)(numTotalRounds * f));
                oracle::Ray ray{cf.posW, normalize(oracle::rayDirPinhole(cf, x, y, p->W, p->H)), 0.f, oracle::kRayTMax};
                f3 avg = mk3(0.f);
                for (int r = 0; r < p->opts.mBaselineSamplePerPixel; ++r) avg = avg + p->integratePT(cl, ray, sg);
                avg = avg / (float)p->opts.mBaselineSamplePerPixel;
                size_t i = (size_t)y * p->W + x;
                accum[i * 3] += (double)avg.x; accum[i * 3 + 1] += (double)avg.y; accum[i * 3 + 2] += (double)avg.z;
            }
        }
        if (cl.loopLimit) ll = true;
    });
    return ll ? VR_ERR_LOOP_LIMIT : VR_OK;
}

// ---- single-ray probes for analytic known answers ----
// transmittance of a world-space segment with a given tracking method (computeVisibility)
float vro_transmittance(void* h, const float o[3], const float d[3], float tmax, int mip, int linear, int method, float tStepScale, uint32_t seed) {
    Oracle* p = (Oracle*)h;
    Rng sg = rng_create(seed, 0, 0);
    oracle::Ray r{mk3(o[0], o[1], o[2]), mk3(d[0], d[1], d[2]), 0, tmax};
    return oracle::computeVisibility(p->sc, r, sg, 1, mip, linear != 0, (uint32_t)method, tStepScale);
}
// distance sampling along a ray (SampleMediumAnalyticGeneric with one sample)
void vro_sample_distance(void* h, const float o[3], const float d[3], int mip, int linear, uint32_t seed, float out[3]) {
    Oracle* p = (Oracle*)h;
    Rng sg = rng_create(seed, 1, 0);
    oracle::Ray r{mk3(o[0], o[1], o[2]), mk3(d[0], d[1], d[2]), 0, oracle::kRayTMax};
    float hd[4], pd[4], tr[4];
    oracle::SampleMediumAnalyticGeneric(p->sc, r, sg, linear != 0, hd, mip, pd, tr, 1);
    out[0] = hd[0]; out[1] = pd[0]; out[2] = tr[0];
}
float vro_density_world(void* h, const float pw[3], int mip) {
    Oracle* p = (Oracle*)h;
    return oracle::DensityWorldSpace(p->sc, mk3(pw[0], pw[1], pw[2]), mip);
}

// ---- elementary functions and RNG (for tests) ----
int vro_math(int op, const float* a, const float* b, float* out, int n) {
    for (int i = 0; i < n; ++i) {
        float x = a[i], y = b ? b[i] : 0.f, r = 0.f;
        switch (op) {
            case 0: r = exp_(x); break;
            case 1: r = log_(x); break;
            case 2: r = sin_(x); break;
            case 3: r = cos_(x); break;
            case 4: r = atan2_(x, y); break;
            case 5: r = acos_(x); break;
            case 6: r = pow_(x, y); break;
            case 7: r = sqrt_(x); break;
            default: return 1;
        }
        out[i] = r;
    }
    return 0;
}
void vro_rng(const uint32_t* cases, int n, int draws, float* out) {
    for (int c = 0; c < n; ++c) {
        Rng r = rng_create(cases[c * 3], cases[c * 3 + 1], cases[c * 3 + 2]);
        for (int j = 0; j < draws; ++j) out[c * draws + j] = next1D(r);
    }
}
void vro_xoshiro(const uint32_t seed[4], int draws, uint32_t* out) {
    Rng r; for (int k = 0; k < 4; ++k) r.s[k] = seed[k];
    for (int j = 0; j < draws; ++j) out[j] = xoshiro_next(r);
}
void vro_splitmix(uint64_t seed, int draws, uint64_t* out) {
    uint64_t st = seed;
    for (int j = 0; j < draws; ++j) out[j] = splitmix64_next(st);
}

// volume emission: temperature view (mip 0), 128 RGB table, LeScale, cutoff, scale; view NULL = off
void vro_set_emission(void* h, const vr_grid_view* tview, const float* lut, float leScale, float cutoff, float scale) {
    Oracle* p = (Oracle*)h;
    oracle::Emission& e = p->sc.emis;
    e = oracle::Emission();
    p->optionsChanged = true;
    if (!tview || !tview->valid) return;
    load_slot(*tview, e.slot);
    memcpy(e.lut, lut, sizeof(e.lut));
    e.leScale = leScale; e.cutoff = cutoff; e.scale = scale;
    e.has = true;
    e.prevSlot = e.slot;          // a static grid is its own previous frame
    e.lastHas = true;
}

// views: n * VR_NUM_SLOTS density slots; tviews: n temperature grids (valid = 0: no emission in
// that frame) or NULL; vviews: 3n velocity components or NULL; the emission parameters apply to
// the frames' temperature grids.  n = 0 returns to the static volume.
void vro_set_animation(void* h, const vr_grid_view* views, int n, const vr_grid_view* tviews, const vr_grid_view* vviews, float vscale,
                       const float* lut, float leScale, float cutoff, float scale) {
    Oracle* p = (Oracle*)h;
    oracle::Scene& sc = p->sc;
    p->optionsChanged = true;
    p->anim.clear();
    p->animId = -1;
    for (int k = 0; k < VR_NUM_SLOTS; ++k) { sc.slots[k] = p->staticSlots[k]; sc.slots[oracle::kPrevSlotOffset + k] = oracle::Slot(); }
    sc.hasAnimation = false;
    sc.hasVelocity = false;
    for (int k = 0; k < 3; ++k) sc.vel[k] = oracle::Slot();
    if (sc.emis.has) sc.emis.prevSlot = sc.emis.slot;
    sc.emis.lastHas = sc.emis.has;
    p->animTemp = tviews != nullptr;
    p->animVel = vviews != nullptr;
    p->animVelScale = vscale;
    if (n <= 0) { p->animTemp = p->animVel = false; return; }
    p->anim.resize(n);
    for (int i = 0; i < n; ++i) {
        Oracle::AnimFrame& f = p->anim[i];
        for (int k = 0; k < VR_NUM_SLOTS; ++k)
            if (views[(size_t)i * VR_NUM_SLOTS + k].valid) load_slot(views[(size_t)i * VR_NUM_SLOTS + k], f.slots[k]);
        if (tviews && tviews[i].valid) { load_slot(tviews[i], f.temp); f.hasTemp = true; }
        if (vviews)
            for (int k = 0; k < 3; ++k) load_slot(vviews[3 * i + k], f.vel[k]);
    }
    if (tviews) {
        memcpy(sc.emis.lut, lut, sizeof(sc.emis.lut));
        sc.emis.leScale = leScale; sc.emis.cutoff = cutoff; sc.emis.scale = scale;
    }
}

// learned target (test infrastructure)
void vro_set_net(void* h, const float* params, const float bmin[3], const float binv[3]) {
    Oracle* p = (Oracle*)h;
    p->lpParams.assign(params, params + oracle::lpo::kParams);
    for (int i = 0; i < 3; ++i) { p->lpBmin[i] = bmin[i]; p->lpBinv[i] = binv[i]; }
}
void vro_set_lp_T(void* h, const float* T, int64_t n) {
    Oracle* p = (Oracle*)h;
    if (!T || n <= 0) p->lpTIn.clear();
    else p->lpTIn.assign(T, T + n);
}
// which 0: per-slot queries (8 floats, tmax = -1 where none), 1: T used per slot, 2: training samples,
// 3: vertex records written by the last frame (one value)
int64_t vro_export_lp(void* h, int which, float* out, int64_t cap) {
    Oracle* p = (Oracle*)h;
    if (which == 3) {
        if (out && cap >= 1) out[0] = (float)p->lpVertices.load();
        return 1;
    }
    const std::vector<float>& v = which == 0 ? p->lpQueries : which == 1 ? p->lpTUsed : p->lpTrain;
    if (out && cap >= (int64_t)v.size()) memcpy(out, v.data(), v.size() * sizeof(float));
    return (int64_t)v.size();
}
void vro_net_forward(const float* params, const float bmin[3], const float binv[3], float floor_, const float* q, int n, float* out) {
    std::vector<float> wt;
    oracle::lpo::roundedWeights(params, wt);
    for (int i = 0; i < n; ++i) {
        float act[5][64];
        float o = oracle::lpo::forwardR(params, wt.data(), q + (size_t)i * 8, q + (size_t)i * 8 + 3, bmin, binv, act);
        out[i] = oracle::lpo::predict(o, floor_);
    }
}
void vro_net_gradients(const float* params, const float bmin[3], const float binv[3], const float* samples, int n, int lossLog, float floor_,
                       float* grads, float* loss) {
    oracle::lpo::gradients(params, samples, n, bmin, binv, lossLog, floor_, grads, loss);
}

// debugging aid: F of one reservoir (with its suffix records) at pixel (px, py), final options
int vro_eval_F(void* h, const vr_camera* camIn, const vr_reservoir_aos* ra, const float* extra, int px, int py, int frameCount, float out[3]) {
    Oracle* p = (Oracle*)h;
    oracle::Ctx c;
    p->makeOptions(c);
    oracle::CamFrame cam = oracle::makeCamera(*camIn, p->W, p->H);
    const int numTotalRounds = (p->opts.mEnableSpatialReuse ? p->opts.mSpatialReuseRounds : 0) + p->opts.mEnableTemporalReuse + 1 + 1;
    Rng sg = rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(numTotalRounds * frameCount + numTotalRounds - 1));
    oracle::Reservoir r;
    r.runningSum = ra->runningSum; r.M = ra->M; r.depth = ra->depth; r.p_y = ra->p_y;
    r.lightUV[0] = ra->lightUV[0]; r.lightUV[1] = ra->lightUV[1]; r.lightID = ra->lightID; r.sampledPixel = ra->sampledPixel;
    r.extraBounceStartId = 0;
    std::vector<f3> ex(4);
    for (int b = 0; b < 3; ++b) ex[b] = mk3(extra[3 * b], extra[3 * b + 1], extra[3 * b + 2]);
    oracle::ExtraProvider prov{ex.data()};
    oracle::Ray ray{cam.posW, normalize(oracle::rayDirPinhole(cam, px, py, p->W, p->H)), 0, r.depth};
    f3 col = oracle::evaluate_F_(c, r, prov, ray, sg, c.fin, c.noReuse, true);
    out[0] = col.x; out[1] = col.y; out[2] = col.z;
    return 0;
}

}  // extern "C"
