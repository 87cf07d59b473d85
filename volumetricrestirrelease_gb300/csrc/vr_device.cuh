// vr_device.cuh -- device-side volume tracking, lighting and reservoir logic for sm_103a.
//
// One thread owns one pixel and its RNG stream for the whole pass, so every pixel consumes
// random numbers in exactly the order the reference shaders do
// (Source/RenderPasses/VolumetricReSTIR/*.slang).  The scene lives in constant memory; the
// sparse brick grid, reservoirs and the environment's importance map live in HBM and are read
// through the read-only data path (__ldg).  Arithmetic is written in the same operation order
// as the CPU oracle and compiled with -fmad=false so both round identically.
#pragma once

#if defined(__CUDACC__)
#include <cuda_fp16.h>
#endif
#include <stdint.h>

#include "vr_math.h"
#include "vr_bc4.h"
#include "../../include/vrestir.h"

namespace vrd {

using vr::f3;
using vr::mk3;

constexpr float kRayTMax = 3.402823466e+38f;
constexpr int kSelfEmissionLightID = -3;
constexpr int kNumMaxMips = 8;
constexpr float kM_PI = 3.14159265358979323846f;
constexpr float kM_2PI = 6.28318530717958647693f;
constexpr float kM_PI_4 = 0.785398163397448309616f;
constexpr float kM_1_PI = 0.318309886183790671538f;
constexpr float kM_1_2PI = 0.159154943091895335769f;
constexpr float kM_1_4PI = 0.079577471545947667884f;
constexpr int kMaxBrickSteps = 128;
constexpr int kMaxDeltaIters = 1 << 20;
constexpr int kMaxLights = 64;

// status bits reported to the host
constexpr int kStatusLoopLimit = 1;

// ---------------------------------------------------------------------------------------
// device scene (constant memory)
// ---------------------------------------------------------------------------------------
struct DevSlot {
    int valid;
    int res;
    float bmaxf;                 // res as float (bmin = 0)
    float maxValue;
    float M[16];                 // world -> index, row-vector convention
    const int* root;             // 32768
    const int4* l1vmin;
    const int* l1child;          // 4096 per node
    const int4* bvmin;
    const float4* bounds;
    const float* f32;            // 1000 per brick
    const __half* f16;
    const uint2* bc4;            // 90 BC4 blocks per brick (vr_bc4.h), density = decoded * bc4Scale
    float bc4Scale;
};

// slots [0, VR_NUM_SLOTS): the current frame's mips (normal, then conservative); with an
// animated volume, [kPrevSlotOffset, kPrevSlotOffset + VR_NUM_SLOTS) hold the previous animation
// frame's (the reference's kPrevFrameDensityGridOffset, HostDeviceSharedConstants.slang:27)
constexpr int kPrevSlotOffset = VR_NUM_SLOTS;

struct DevScene {
    DevSlot slots[2 * VR_NUM_SLOTS];
    float sigma_t;
    f3 sigma_s, sigma_a;
    float g;
    float dscale;
    float tStep;
    float superDiag;
    int numMips;
    int numLights;
    float lightPos[kMaxLights][3];
    float lightI[kMaxLights][3];
    int hasEnv;
    const float* envRGB;         // w*h*3
    int envW, envH;
    f3 envScale;
    float envRot[9], envInv[9];
    const float* imp;            // importance pyramid, mip m at impOff[m]
    int impOff[12];
    int impDim, impBaseMip;
    int* status;                 // device status word (kStatus* bits)
    // volume emission (VolumeBase.slang:196-232): temperature grid (mip 0), blackbody table
    int hasEmission;
    DevSlot tslot;
    float leScale, tCutoff, tScale;
    float blackbody[128][3];     // radiance of 50 K .. 6400 K in steps of 50 K (texel centres)
    // animated volumes (VolumeDesc.hasAnimation, usePrevGridForReproj, lastFrameHasEmission,
    // hasVelocity, velocityScale; SceneTypes.slang:101-109)
    int hasAnimation, usePrevGrid, lastHasEmission, hasVelocity;
    float velocityScale;
    DevSlot ptslot;              // the previous animation frame's temperature grid
    DevSlot vslot[3];            // velocity components (world units per frame), mip 0
};

struct SamplingOptions {         // HostDeviceSharedDefinitions.h:96-141
    uint32_t visibilityTrackingMethod, lightingTrackingMethod;
    int lightSamples, lightingMipLevel, visibilitySamples, visibilityMipLevel;
    int visibilityUseLinearSampler, lightingUseLinearSampler;
    float visibilityTStepScale, lightingTStepScale;
    int useEnvironmentLights, useAnalyticLights;
    int vertexReuseStartBounce;  // vertex reuse (VERTEX_REUSE): the first reconnection bounce; -1 off
};

struct FrameParams {
    int W, H, N;
    int maxBounces;
    int frameCount;
    int numTotalRounds;
    int noReuse;
    int initialM;
    int baselineSpp;
    int useRR, useCoarser;
    int temporalEnabled, isFirstFrame, reprojMode, temporalTalbot, reprojMip;
    float temporalMThreshold;
    int spatialTalbot, spatialK, spatialRounds;
    int visualizeTr;
    SamplingOptions initial, spatial, fin;
    f3 camPos, camU, camV, camW;
    f3 prevPos, prevU, prevV, prevW;
    float prevView[16], prevProj[16];
};

// SoA reservoir buffer: a = (runningSum, M, depth, p_y), b = (lightUV.x, lightUV.y, lightID,
// sampledPixel) as raw bits; extra-bounce records are float4 planes indexed b*N + pixel.
struct ResBuf {
    float4* a;
    int4* b;
    float4* extra;
    float* pp;             // p_partial per pixel under vertex reuse, else nullptr
};

// Each translation unit that includes this header has its own copy of the scene constants
// (internal linkage); the host uploads the same DevScene to every copy.  The batched kernels
// (many scenes in one launch) keep the scene of the tile being processed in shared memory
// instead: each block loads it from the instance's DevScene in global memory.
#if defined(VR_BATCHED) && defined(VR_HOST_EMULATION)
static thread_local DevScene c_scene;
#elif defined(VR_BATCHED)
static __shared__ DevScene c_scene;
#else
static __constant__ DevScene c_scene;
#endif

// ---------------------------------------------------------------------------------------
// reservoir (Reservoir.slang); extraBounceStartId is carried as the owning pixel
// ---------------------------------------------------------------------------------------
struct Reservoir {
    float runningSum, M, depth, p_y;
    float uv0, uv1;
    int lightID, sampledPixel;
    int startPixel;              // extraBounceStartId / (maxBounces - 1)
    float pp;                    // p_partial (vertex reuse): the suffix's share of p_hat
};
__device__ __forceinline__ Reservoir newReservoir() {
    Reservoir r;
    r.runningSum = 0.f; r.M = 0.f; r.depth = kRayTMax; r.p_y = 0.f;
    r.uv0 = 0.f; r.uv1 = 0.f; r.lightID = 0; r.sampledPixel = 0; r.startPixel = 0; r.pp = 0.f;
    return r;
}
__device__ __forceinline__ Reservoir loadRes(const ResBuf& buf, int i) {
    float4 a = __ldg(&buf.a[i]);
    int4 b = __ldg(&buf.b[i]);
    Reservoir r;
    r.runningSum = a.x; r.M = a.y; r.depth = a.z; r.p_y = a.w;
    r.uv0 = __int_as_float(b.x); r.uv1 = __int_as_float(b.y); r.lightID = b.z; r.sampledPixel = b.w;
    r.startPixel = i;
    r.pp = buf.pp ? __ldg(&buf.pp[i]) : 0.f;
    return r;
}
// coherent load (buffer written earlier in the same kernel)
__device__ __forceinline__ Reservoir loadResRW(const ResBuf& buf, int i) {
    float4 a = buf.a[i];
    int4 b = buf.b[i];
    Reservoir r;
    r.runningSum = a.x; r.M = a.y; r.depth = a.z; r.p_y = a.w;
    r.uv0 = __int_as_float(b.x); r.uv1 = __int_as_float(b.y); r.lightID = b.z; r.sampledPixel = b.w;
    r.startPixel = i;
    r.pp = buf.pp ? buf.pp[i] : 0.f;
    return r;
}
__device__ __forceinline__ void storeRes(const ResBuf& buf, int i, const Reservoir& r) {
    buf.a[i] = make_float4(r.runningSum, r.M, r.depth, r.p_y);
    buf.b[i] = make_int4(__float_as_int(r.uv0), __float_as_int(r.uv1), r.lightID, r.sampledPixel);
    if (buf.pp) buf.pp[i] = r.pp;
}
__device__ __forceinline__ void copySample(const Reservoir& f, Reservoir& t) {
    t.depth = f.depth; t.p_y = f.p_y; t.uv0 = f.uv0; t.uv1 = f.uv1;
    t.lightID = f.lightID; t.startPixel = f.startPixel; t.sampledPixel = f.sampledPixel;
    t.pp = f.pp;                 // Reservoir.slang:46-48, 76-78
}
__device__ __forceinline__ bool resampleStep(const Reservoir& r, Reservoir& s, vr::Rng& sg) {
    float w = r.runningSum;
    s.M += r.M;
    if (w <= 0.0f) return false;
    s.runningSum += w;
    bool sel = vr::next1D(sg) * s.runningSum < w;
    if (sel) copySample(r, s);
    return sel;
}
__device__ __forceinline__ bool resampleStepMaxM(const Reservoir& r, float MThr, Reservoir& s, vr::Rng& sg) {
    float cm = vr::fmin_(MThr, r.M);
    float w = cm == 0.0f ? 0.0f : cm / r.M * r.runningSum;
    s.M += cm;
    if (w <= 0.0f) return false;
    s.runningSum += w;
    bool sel = vr::next1D(sg) * s.runningSum < w;
    if (sel) copySample(r, s);
    return sel;
}
// the stored count never exceeds mb - 1; the clamp only keeps extra-bounce indexing in bounds
__device__ __forceinline__ int decodeBounces(int sp, int mb) { return mb == 1 ? 0 : min(sp >> 20, mb - 1); }
__device__ __forceinline__ int encodeBounces(int sp, int b) { return (b << 20) | (sp & 0xFFFFF); }
__device__ __forceinline__ int decodeTag(int sp) { return (sp >> 16) & 0xF; }
__device__ __forceinline__ int encodeTag(int sp, int tag) { return (tag << 16) | (sp & (int)0xFFF0FFFF); }

// ---------------------------------------------------------------------------------------
// grid access
// ---------------------------------------------------------------------------------------
struct Ray { f3 o, d; float tMin, tMax; };
__device__ __forceinline__ f3 at(const Ray& r, float t) { return r.o + r.d * t; }

__device__ __forceinline__ f3 mulPoint(f3 p, const float* M) {
    float o[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) o[j] = p.x * M[j] + p.y * M[4 + j] + p.z * M[8 + j] + 1.0f * M[12 + j];
    return mk3(o[0] / o[3], o[1] / o[3], o[2] / o[3]);
}
__device__ __forceinline__ f3 mulVec(f3 d, const float* M) {
    float o[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) o[j] = d.x * M[j] + d.y * M[4 + j] + d.z * M[8 + j] + 0.0f * M[12 + j];
    return mk3(o[0], o[1], o[2]);
}
__device__ __forceinline__ f3 mul33(f3 d, const float* R) {
    return mk3(d.x * R[0] + d.y * R[3] + d.z * R[6], d.x * R[1] + d.y * R[4] + d.z * R[7], d.x * R[2] + d.y * R[5] + d.z * R[8]);
}

__device__ __forceinline__ int getChild(const DevSlot& s, int node, int clev, int b) {
    if (clev == 2) return (b >= 0 && b < 32768) ? __ldg(&s.root[b]) : -1;
    return (b >= 0 && b < 4096) ? __ldg(&s.l1child[(size_t)node * 4096 + b]) : -1;
}
__device__ __forceinline__ f3 nodeVmin(const DevSlot& s, int lev, int id) {
    if (lev == 2) return mk3(0.f);
    int4 v = lev == 1 ? __ldg(&s.l1vmin[id]) : __ldg(&s.bvmin[id]);
    return mk3((float)v.x, (float)v.y, (float)v.z);
}
// one voxel of a BC4 brick, apron coordinates in [0, 10)^3
__device__ __forceinline__ float bc4Voxel(const DevSlot& s, int brick, int x, int y, int z) {
    const uint2 b = __ldg(&s.bc4[(size_t)brick * vr::kBc4BlocksPerBrick + vr::bc4_block(x, y, z)]);
    return vr::bc4_decode2(b.x, b.y, vr::bc4_texel(x, y)) * s.bc4Scale;
}
__device__ __forceinline__ float voxel(const DevSlot& s, int brick, int x, int y, int z) {
    x = min(max(x, -1), 8); y = min(max(y, -1), 8); z = min(max(z, -1), 8);
    if (s.bc4) return bc4Voxel(s, brick, x + 1, y + 1, z + 1);
    size_t o = (size_t)brick * 1000 + ((z + 1) * 10 + (y + 1)) * 10 + (x + 1);
    if (s.f32) return __ldg(&s.f32[o]);
    return __half2float(__ldg(&s.f16[o]));
}
__device__ __forceinline__ float lerp_(float a, float b, float t) { return a + (b - a) * t; }
__device__ __forceinline__ float trilinear(const DevSlot& s, int brick, f3 p) {
    float qx = p.x - 0.5f, qy = p.y - 0.5f, qz = p.z - 0.5f;
    float fx0 = vr::floor_(qx), fy0 = vr::floor_(qy), fz0 = vr::floor_(qz);
    int ix = vr::f2i(fx0), iy = vr::f2i(fy0), iz = vr::f2i(fz0);
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
// Unclamped accessors for positions the caller's loop guard keeps inside the brick
// (p in [0, 8]^3 for trilinear, cell in [0, 7]^3 for point and 8-corner fetches): one base
// offset and seven constant displacements into the 10^3 brick.
__device__ __forceinline__ void cornerValues(const DevSlot& s, size_t base, float c[8]) {
    if (s.f32) {
        const float* d = s.f32 + base;
        c[0] = __ldg(d); c[1] = __ldg(d + 1); c[2] = __ldg(d + 10); c[3] = __ldg(d + 11);
        c[4] = __ldg(d + 100); c[5] = __ldg(d + 101); c[6] = __ldg(d + 110); c[7] = __ldg(d + 111);
    } else {
        const __half* d = s.f16 + base;
        c[0] = __half2float(__ldg(d)); c[1] = __half2float(__ldg(d + 1));
        c[2] = __half2float(__ldg(d + 10)); c[3] = __half2float(__ldg(d + 11));
        c[4] = __half2float(__ldg(d + 100)); c[5] = __half2float(__ldg(d + 101));
        c[6] = __half2float(__ldg(d + 110)); c[7] = __half2float(__ldg(d + 111));
    }
}
// the eight corners from apron corner (x, y, z) in [0, 9)^3, in cornerValues' order
__device__ __forceinline__ void cornerValuesAt(const DevSlot& s, int brick, int x, int y, int z, float c[8]) {
    if (s.bc4) {
        // the four corners of a z-slice share one block unless x or y is the last texel of its
        // block: one load per slice, the others only where a corner crosses into the next block
        const uint2* blk = s.bc4 + (size_t)brick * vr::kBc4BlocksPerBrick;
        const bool cx = (x & 3) == 3, cy = (y & 3) == 3;
#pragma unroll
        for (int dz = 0; dz < 2; ++dz) {
            const int zz = z + dz;
            const uint2 b00 = __ldg(&blk[vr::bc4_block(x, y, zz)]);
            const uint2 b10 = cx ? __ldg(&blk[vr::bc4_block(x + 1, y, zz)]) : b00;
            const uint2 b01 = cy ? __ldg(&blk[vr::bc4_block(x, y + 1, zz)]) : b00;
            const uint2 b11 = (cx || cy) ? __ldg(&blk[vr::bc4_block(x + 1, y + 1, zz)]) : b00;
            c[4 * dz + 0] = vr::bc4_decode2(b00.x, b00.y, vr::bc4_texel(x, y)) * s.bc4Scale;
            c[4 * dz + 1] = vr::bc4_decode2(b10.x, b10.y, vr::bc4_texel(x + 1, y)) * s.bc4Scale;
            c[4 * dz + 2] = vr::bc4_decode2(b01.x, b01.y, vr::bc4_texel(x, y + 1)) * s.bc4Scale;
            c[4 * dz + 3] = vr::bc4_decode2(b11.x, b11.y, vr::bc4_texel(x + 1, y + 1)) * s.bc4Scale;
        }
        return;
    }
    cornerValues(s, (size_t)brick * 1000 + (size_t)((z * 10 + y) * 10 + x), c);
}
__device__ __forceinline__ float trilinearIn(const DevSlot& s, int brick, f3 p) {
    float qx = p.x - 0.5f, qy = p.y - 0.5f, qz = p.z - 0.5f;
    float fx0 = vr::floor_(qx), fy0 = vr::floor_(qy), fz0 = vr::floor_(qz);
    int ix = (int)fx0, iy = (int)fy0, iz = (int)fz0;
    float fx = qx - fx0, fy = qy - fy0, fz = qz - fz0;
    float c[8];
    cornerValuesAt(s, brick, ix + 1, iy + 1, iz + 1, c);
    float x00 = lerp_(c[0], c[1], fx), x10 = lerp_(c[2], c[3], fx);
    float x01 = lerp_(c[4], c[5], fx), x11 = lerp_(c[6], c[7], fx);
    float y0 = lerp_(x00, x10, fy), y1 = lerp_(x01, x11, fy);
    return lerp_(y0, y1, fz);
}
__device__ __forceinline__ float voxelIn(const DevSlot& s, int brick, int x, int y, int z) {
    if (s.bc4) return bc4Voxel(s, brick, x + 1, y + 1, z + 1);
    size_t o = (size_t)brick * 1000 + (size_t)(((z + 1) * 10 + (y + 1)) * 10 + (x + 1));
    return s.f32 ? __ldg(&s.f32[o]) : __half2float(__ldg(&s.f16[o]));
}
// density at a brick-local position inside the brick (loop-guarded callers)
__device__ __forceinline__ float densityLocal(int mip, int brick, f3 p, bool linear) {
    const DevSlot& s = c_scene.slots[mip];
    float v = linear ? trilinearIn(s, brick, p) : voxelIn(s, brick, (int)vr::floor_(p.x), (int)vr::floor_(p.y), (int)vr::floor_(p.z));
    return v * 1.0f * c_scene.dscale;
}
// density at a position that may sit a rounding error outside the brick (delta and ratio
// tracking sample free-flight positions): clamped indices
__device__ __forceinline__ float densityLocalClamped(int mip, int brick, f3 p) {
    return trilinear(c_scene.slots[mip], brick, p) * 1.0f * c_scene.dscale;
}
__device__ __forceinline__ float densityCell(int mip, int brick, const int p[3]) {
    return voxelIn(c_scene.slots[mip], brick, p[0], p[1], p[2]) * 1.0f * c_scene.dscale;
}
__device__ __forceinline__ void fetchEightSigma(int mip, int brick, const int p[3], float v[8]) {
    const DevSlot& s = c_scene.slots[mip];
    cornerValuesAt(s, brick, p[0] + 1, p[1] + 1, p[2] + 1, v);
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = v[i] * 1.0f * c_scene.dscale * c_scene.sigma_t;
}
__device__ inline int findBrick(const DevSlot& s, f3 pos, f3& vmin) {
    if (pos.x < 0.f || pos.y < 0.f || pos.z < 0.f || pos.x >= 4096.f || pos.y >= 4096.f || pos.z >= 4096.f) return -1;
    int px = vr::f2i(pos.x) / 128, py = vr::f2i(pos.y) / 128, pz = vr::f2i(pos.z) / 128;
    int l1 = getChild(s, 0, 2, (((pz << 5) + py) << 5) + px);
    if (l1 < 0) return -1;
    f3 v = nodeVmin(s, 1, l1);
    if (pos.x < v.x || pos.y < v.y || pos.z < v.z || pos.x >= v.x + 128.f || pos.y >= v.y + 128.f || pos.z >= v.z + 128.f) return -1;
    px = vr::f2i(pos.x - v.x) / 8; py = vr::f2i(pos.y - v.y) / 8; pz = vr::f2i(pos.z - v.z) / 8;
    int br = getChild(s, l1, 1, (((pz << 4) + py) << 4) + px);
    if (br < 0) return -1;
    vmin = nodeVmin(s, 0, br);
    return br;
}
static __device__ __forceinline__ float densityWorld(f3 pw, int mip) {
    const DevSlot& s = c_scene.slots[mip];
    f3 p = mulPoint(pw, s.M);
    if (p.x < 0.f || p.y < 0.f || p.z < 0.f || p.x >= s.bmaxf || p.y >= s.bmaxf || p.z >= s.bmaxf) return 0.f;
    f3 vmin;
    int br = findBrick(s, p, vmin);
    if (br < 0) return 0.f;
    return trilinearIn(s, br, p - vmin) * c_scene.dscale;
}

// Temperature / ConvertTempToColor / EmissionWorldSpace (VolumeBase.slang:196-232): trilinear
// temperature at mip 0, mapped to a blackbody colour through the 128-texel table with linear
// filtering between texel centres and clamped addressing
static __device__ __noinline__ float temperatureWorld(f3 pw, bool last) {
    const DevSlot& s = last ? c_scene.ptslot : c_scene.tslot;
    f3 p = mulPoint(pw, s.M);
    if (p.x < 0.f || p.y < 0.f || p.z < 0.f || p.x >= s.bmaxf || p.y >= s.bmaxf || p.z >= s.bmaxf) return 0.f;
    f3 vmin;
    int br = findBrick(s, p, vmin);
    if (br < 0) return 0.f;
    return trilinearIn(s, br, p - vmin);
}
__device__ inline f3 tempToColor(float temp) {
    temp = vr::fmin_(6400.f, (temp - c_scene.tCutoff) * c_scene.tScale);
    const float q = (temp - 25.f) / 6400.f;
    const float x = q * 128.f - 0.5f;
    const float fl = vr::floor_(x);
    const float f = x - fl;
    int i0 = vr::f2i(fl), i1 = i0 + 1;
    i0 = i0 < 0 ? 0 : (i0 > 127 ? 127 : i0);
    i1 = i1 < 0 ? 0 : (i1 > 127 ? 127 : i1);
    const f3 a = mk3(c_scene.blackbody[i0][0], c_scene.blackbody[i0][1], c_scene.blackbody[i0][2]);
    const f3 b = mk3(c_scene.blackbody[i1][0], c_scene.blackbody[i1][1], c_scene.blackbody[i1][2]);
    return c_scene.leScale * (a + (b - a) * f);
}
static __device__ __noinline__ f3 emissionWorld(f3 pw, bool last = false) {
    if (last ? !c_scene.lastHasEmission : !c_scene.hasEmission) return mk3(0.f);
    return tempToColor(temperatureWorld(pw, last));
}
// VelocityWorld (VolumeBase.slang:182-194): the trilinear velocity at mip 0, zero outside the
// grids (the points given may be far outside: the comparisons also reject NaN)
static __device__ __noinline__ f3 velocityWorld(f3 pw) {
    float v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const DevSlot& s = c_scene.vslot[k];
        const f3 p = mulPoint(pw, s.M);
        v[k] = 0.f;
        if (!(p.x >= 0.f && p.y >= 0.f && p.z >= 0.f && p.x < s.bmaxf && p.y < s.bmaxf && p.z < s.bmaxf)) continue;
        f3 vmin;
        const int br = findBrick(s, p, vmin);
        if (br >= 0) v[k] = trilinearIn(s, br, p - vmin);
    }
    return mk3(v[0], v[1], v[2]);
}

// ---------------------------------------------------------------------------------------
// hierarchical DDA (gvdbDda.slang:86-157)
// ---------------------------------------------------------------------------------------
struct HDDA {
    f3 pos, dir; int ps[3];
    f3 tDel, t, tSide; int p[3]; int mask[3];
    __device__ __forceinline__ void setFromRay(f3 sp, f3 sd, f3 st) {
        pos = sp; dir = sd;
        ps[0] = dir.x >= 0 ? 1 : -1; ps[1] = dir.y >= 0 ? 1 : -1; ps[2] = dir.z >= 0 ? 1 : -1;
        t = st;
    }
    __device__ __forceinline__ void finishPrepare(f3 pFlt) {
        f3 fl = mk3(vr::floor_(pFlt.x), vr::floor_(pFlt.y), vr::floor_(pFlt.z));
        tSide = ((fl - pFlt + mk3(0.5f)) * mk3((float)ps[0], (float)ps[1], (float)ps[2]) + mk3(0.5f)) * tDel + mk3(t.x);
        p[0] = vr::f2i(fl.x); p[1] = vr::f2i(fl.y); p[2] = vr::f2i(fl.z);
    }
    __device__ __forceinline__ void prepare(f3 vmin, float vdel) {
        tDel = mk3(vr::fabs_(vdel / dir.x), vr::fabs_(vdel / dir.y), vr::fabs_(vdel / dir.z));
        finishPrepare((pos + dir * t.x - vmin) / mk3(vdel));
    }
    __device__ __forceinline__ void prepareLeaf(f3 vmin) {
        tDel = mk3(vr::fabs_(1.0f / dir.x), vr::fabs_(1.0f / dir.y), vr::fabs_(1.0f / dir.z));
        finishPrepare(pos + dir * t.x - vmin);
    }
    // a three-way tie (the ray through a cell corner) steps the z axis; the reference sets no
    // mask there and stalls the walk (see the oracle's HDDA::Next)
    __device__ __forceinline__ void next() {
        mask[0] = (tSide.x < tSide.y) & (tSide.x <= tSide.z);
        mask[1] = (tSide.y < tSide.z) & (tSide.y <= tSide.x);
        mask[2] = !(mask[0] | mask[1]);       // (z < x) & (z <= y), or the three-way tie
        t.y = mask[0] ? tSide.x : (mask[1] ? tSide.y : tSide.z);
    }
    // advances only the masked axes (a zero direction component has tDel = inf)
    __device__ __forceinline__ void step() {
        t.x = t.y;
        tSide = mk3(mask[0] ? tSide.x + tDel.x : tSide.x, mask[1] ? tSide.y + tDel.y : tSide.y, mask[2] ? tSide.z + tDel.z : tSide.z);
        p[0] += mask[0] * ps[0]; p[1] += mask[1] * ps[1]; p[2] += mask[2] * ps[2];
    }
};
__device__ __forceinline__ bool inLeaf(const int p[3]) { return p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] < 8 && p[1] < 8 && p[2] < 8; }
__device__ __forceinline__ bool inLeafF(f3 p) { return p.x >= 0 && p.y >= 0 && p.z >= 0 && p.x < 8 && p.y < 8 && p.z < 8; }

__device__ __forceinline__ bool intersectBound(const Ray& ray, float& tMin, float& tMax, int mip, bool vc) {
    const DevSlot& s = c_scene.slots[mip];
    float lo = vc ? -0.5f : 0.f, hi = vc ? s.bmaxf - 0.5f : s.bmaxf;
    float o[3] = {ray.o.x, ray.o.y, ray.o.z}, d[3] = {ray.d.x, ray.d.y, ray.d.z};
    float t0 = 0, t1 = ray.tMax;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float inv = 1 / d[i];
        float tn = (lo - o[i]) * inv, tf = (hi - o[i]) * inv;
        if (tn > tf) { float tmp = tn; tn = tf; tf = tmp; }
        t0 = tn > t0 ? tn : t0;
        t1 = tf < t1 ? tf : t1;
        if (t0 > t1) return false;
    }
    tMin = t0; tMax = t1;
    return true;
}

// VolumeTrackingGVDB (VolumeUtils.slang:171-282): walks root -> level-1 -> brick, handing
// each non-empty brick to the adapter.
template <class A>
static __device__ __noinline__ void trackVolume(const Ray& rWorld, int mip, vr::Rng& sg, A& ad, bool vc) {
    const DevSlot& s = c_scene.slots[mip];
    const float eps = 0.01f;
    const int kDim[3] = {3, 4, 5}, kRes[3] = {8, 16, 32};
    const float kVdel[3] = {1.f, 8.f, 128.f};
    int nodeid[3];
    float tMax[3];
    int lev = 2;
    nodeid[2] = 0;
    Ray ray;
    ray.o = mulPoint(rWorld.o, s.M);
    ray.d = mulVec(rWorld.d, s.M);
    ray.tMin = rWorld.tMin; ray.tMax = rWorld.tMax;
    if (vc) ray.o = ray.o - mk3(0.5f);
    float tNear, tFar;
    if (!intersectBound(ray, tNear, tFar, mip, vc)) { ad.end(); return; }
    ad.setRay(tNear, tFar, ray);
    ad.start();
    f3 tStart = mk3(tNear, tFar, 0);
    f3 vmin = mk3(0.f);
    int node = 0;
    tStart.x += eps;
    tMax[2] = tStart.y;
    HDDA dda;
    dda.setFromRay(ray.o, ray.d, tStart);
    dda.prepare(vmin, kVdel[2]);
    if (vc) {
        int it2 = 0;
        while (it2++ < 3 && (dda.p[0] < 0 || dda.p[1] < 0 || dda.p[2] < 0 || dda.p[0] > 32 || dda.p[1] > 32 || dda.p[2] > 32)) {
            dda.next(); dda.step(); dda.t.x += eps;
        }
    }
    float t = tNear;
    for (int iter = 0; iter < 4096 && lev > 0 && lev <= 2 &&
                       (dda.p[0] >= 0 && dda.p[1] >= 0 && dda.p[2] >= 0 && dda.p[0] <= kRes[lev] && dda.p[1] <= kRes[lev] && dda.p[2] <= kRes[lev]);
         iter++) {
        dda.next();
        int b = (((dda.p[2] << kDim[lev]) + dda.p[1]) << kDim[lev]) + dda.p[0];
        int child = getChild(s, node, lev, b);
        if (child >= 0) {
            if (lev == 1) {
                nodeid[0] = child;
                t = dda.t.x - eps;
                // the next occupied brick starts beyond the ray's end: nothing left to track
                // (entering it would integrate over a negative interval, see the oracle's
                // VolumeTrackingGVDB)
                if (t >= tFar) break;
                f3 vmin_leaf = nodeVmin(s, 0, child);
                float4 bb = __ldg(&s.bounds[child]);
                float bnd[3] = {bb.x * c_scene.dscale, bb.y * c_scene.dscale, bb.z * c_scene.dscale};
                if (ad.mainStep(dda, vmin_leaf, child, bnd, mip, t, sg)) return;
                dda.step();
                dda.t.x += eps;
            } else {
                lev--;
                nodeid[lev] = child;
                node = child;
                vmin = nodeVmin(s, lev, child);
                tMax[lev] = dda.t.y;
                dda.prepare(vmin, kVdel[lev]);
            }
        } else {
            dda.step();
            dda.t.x += eps;
        }
        while (lev <= 2 && dda.t.x > tMax[lev]) {
            lev++;
            if (lev <= 2) {
                node = nodeid[lev];
                vmin = nodeVmin(s, lev, node);
                dda.prepare(vmin, kVdel[lev]);
            }
        }
    }
    ad.end();
}

// ---------------------------------------------------------------------------------------
// adapters (VolumeTrackingAdapterGVDB.slang)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void trilinearCoeffs(const float v[8], f3 d, f3 p0, float& c3, float& c2, float& c1, float& c0) {
    float v_000 = v[0], v_100 = v[1], v_010 = v[2], v_110 = v[3];
    float v_001 = v[4], v_101 = v[5], v_011 = v[6], v_111 = v[7];
    float mxyz = v_111 - v_011 - v_101 - v_110 + v_100 + v_010 + v_001 - v_000;
    float mxy = v_000 - v_100 - v_010 + v_110;
    float mxz = v_000 - v_100 - v_001 + v_101;
    float myz = v_000 - v_010 - v_001 + v_011;
    float mx = v_100 - v_000, my = v_010 - v_000, mz = v_001 - v_000;
    c3 = mxyz * d.x * d.y * d.z;
    c2 = (p0.z * d.x * d.y + p0.y * d.x * d.z + p0.x * d.y * d.z) * mxyz + mxy * d.x * d.y + mxz * d.x * d.z + myz * d.y * d.z;
    c1 = (p0.y * p0.z * d.x + p0.x * p0.z * d.y + p0.x * p0.y * d.z) * mxyz +
         mx * d.x + my * d.y + mz * d.z + (p0.y * d.x + p0.x * d.y) * mxy + (p0.z * d.x + p0.x * d.z) * mxz + (p0.z * d.y + p0.y * d.z) * myz;
    c0 = p0.x * p0.y * p0.z * mxyz + p0.x * p0.y * mxy + p0.x * p0.z * mxz + p0.y * p0.z * myz + p0.x * mx + p0.y * my + p0.z * mz + v_000;
}
__device__ __forceinline__ f3 leafP0(const HDDA& d, f3 vmin_leaf) {
    return d.pos + d.t.x * d.dir - (mk3((float)d.p[0], (float)d.p[1], (float)d.p[2]) + vmin_leaf);
}

struct TrAnalytic {
    float Tr = 0.f; bool lin; float tNear, tFar; Ray ray;
    __device__ void setRay(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    __device__ void start() {}
    __device__ bool mainStep(const HDDA& dda, f3 vl, int brick, const float*, int mip, float& t, vr::Rng&) {
        HDDA dl = dda;
        dl.prepareLeaf(vl);
        for (int iter = 0; iter < kMaxBrickSteps && inLeaf(dl.p); iter++) {
            dl.next();
            float maxDeltaT = dl.t.y - t;
            if (lin) {
                float v[8]; fetchEightSigma(mip, brick, dl.p, v);
                float c3, c2, c1, c0;
                trilinearCoeffs(v, ray.d, leafP0(dl, vl), c3, c2, c1, c0);
                float td = vr::fmin_(tFar - t, maxDeltaT);
                float t2 = td * td, t3 = t2 * td, t4 = t2 * t2;
                Tr += -(c3 * t4 / 4 + c2 * t3 / 3 + c1 * t2 / 2 + c0 * td);
            } else {
                float sigma_t = densityCell(mip, brick, dl.p) * c_scene.sigma_t;
                Tr += -vr::fmin_(tFar - t, maxDeltaT) * sigma_t;
            }
            if (t + maxDeltaT >= tFar) { Tr = vr::exp_(Tr); return true; }
            t += maxDeltaT;
            dl.step();
        }
        return false;
    }
    __device__ void end() { Tr = vr::exp_(Tr); }
};

struct TrRayMarch {
    float Tr = 0.f; bool lin; float tNear, tFar; Ray ray; float tStep; bool init = false;
    __device__ void setRay(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    __device__ void start() { init = true; }
    __device__ bool mainStep(const HDDA& dda, f3 vl, int brick, const float*, int mip, float& t, vr::Rng&) {
        t = tNear + (vr::floor_((t - tNear) / tStep) + 0.5f) * tStep;
        if (t < dda.t.x) t += tStep;
        const float mult = 1.f;
        f3 wp = ray.o + t * ray.d;
        f3 p = wp - vl;
        const f3 wpt = mult * tStep * ray.d;
        // Two samples per trip: the second sample's position and the exit tests are computed
        // exactly as the next iteration would, so both loads are in flight together while the
        // optical depth is still summed sample by sample.
        int iter = 0;
        while (iter < kMaxBrickSteps && inLeafF(p)) {
            if (t >= tFar) { Tr = vr::exp_(Tr); return true; }
            const f3 p1 = p + wpt;
            const float t1 = t + mult * tStep;
            const bool second = iter + 1 < kMaxBrickSteps && inLeafF(p1) && !(t1 >= tFar);
            float d0 = densityLocal(mip, brick, p, lin);
            float d1 = second ? densityLocal(mip, brick, p1, lin) : 0.f;
            float sigma_t = d0 * c_scene.sigma_t;
            Tr += -sigma_t * (iter == 0 ? 1.f : mult) * tStep;
            p = p1;
            t = t1;
            iter++;
            if (!second) continue;
            sigma_t = d1 * c_scene.sigma_t;
            Tr += -sigma_t * mult * tStep;
            p = p + wpt;
            t += mult * tStep;
            iter++;
        }
        return false;
    }
    __device__ void end() { if (init) Tr = vr::exp_(Tr); else Tr = 1.f; }
};

struct SampleDist {
    float hit[4], tr[4], pdf[4];
    int n; float thick = 0.f; float tNear, tFar; Ray ray; bool init = false; bool lin = false;
    __device__ void setRay(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    __device__ void start() { for (int i = 0; i < n; i++) hit[i] = -1; init = true; }
    __device__ static float thickAt(float t, float c3, float c2, float c1, float c0) {
        float t2 = t * t, t3 = t2 * t, t4 = t2 * t2;
        return c3 * t4 / 4 + c2 * t3 / 3 + c1 * t2 / 2 + c0 * t;
    }
    __device__ static float sigmaAt(float t, float c3, float c2, float c1, float c0) {
        float t2 = t * t, t3 = t2 * t;
        return c3 * t3 + c2 * t2 + c1 * t + c0;
    }
    __device__ bool mainStep(const HDDA& dda, f3 vl, int brick, const float*, int mip, float& t, vr::Rng& sg) {
        HDDA dl = dda;
        dl.prepareLeaf(vl);
        for (int iter = 0; iter < kMaxBrickSteps && inLeaf(dl.p); iter++) {
            dl.next();
            float maxDeltaT = vr::fmin_(tFar - t, dl.t.y - t);
            float curTMax = vr::fmin_(tFar, dl.t.y);
            int finished = 0;
            float dThick = 0.f;
            if (lin) {
                float v[8]; fetchEightSigma(mip, brick, dl.p, v);
                float c3, c2, c1, c0;
                trilinearCoeffs(v, ray.d, leafP0(dl, vl), c3, c2, c1, c0);
                dThick = thickAt(maxDeltaT, c3, c2, c1, c0);
                for (int k = 0; k < n; k++) {
                    if (hit[k] == -1) {
                        if (thick + dThick >= tr[k]) {
                            float target = tr[k] - thick;
                            float tl = 0, th = maxDeltaT, taul = 0, tauh = dThick, ts = 0;
                            int it = 0;
                            while (it++ < 32 && th - tl > maxDeltaT * 0.001f) {
                                ts = tl + (th - tl) * (target - taul) / (tauh - taul);
                                float tau = thickAt(ts, c3, c2, c1, c0);
                                if (tau < target) { tl = ts; taul = tau; } else { th = ts; tauh = tau; }
                            }
                            hit[k] = t + ts;
                            tr[k] = vr::exp_(-tr[k]);
                            pdf[k] = sigmaAt(ts, c3, c2, c1, c0) * tr[k];
                            finished++;
                        }
                    } else finished++;
                }
            } else {
                float sigma_t = densityCell(mip, brick, dl.p) * c_scene.sigma_t;
                for (int k = 0; k < n; k++) {
                    if (hit[k] == -1) {
                        float dT = -vr::log_(1 - vr::next1D(sg)) / sigma_t;
                        float curT = t + dT;
                        if (vr::isnan_(curT) || vr::isinf_(curT)) curT = kRayTMax;
                        if (curT < curTMax) {
                            hit[k] = curT;
                            tr[k] = vr::exp_(-(dT * sigma_t + thick));
                            pdf[k] = sigma_t * tr[k];
                            finished++;
                        }
                    } else finished++;
                }
                dThick = maxDeltaT * sigma_t;
            }
            if (finished == n) return true;
            t = curTMax;
            thick += dThick;
            if (t >= tFar) { end(); return true; }
            dl.step();
        }
        return false;
    }
    __device__ void end() {
        if (init) {
            for (int k = 0; k < n; k++)
                if (hit[k] == -1) { hit[k] = kRayTMax; tr[k] = vr::exp_(-thick); pdf[k] = tr[k]; }
        } else {
            for (int k = 0; k < n; k++) { hit[k] = kRayTMax; tr[k] = 1.f; pdf[k] = 1.f; }
        }
    }
};

struct CellByDensity {
    float selX = -1, selY = -1; float tNear, tFar; Ray ray; float runningSum = 0.f; float Tr = 0.f;
    __device__ void setRay(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    __device__ void start() { selX = -1; selY = -1; }
    __device__ bool mainStep(const HDDA& dda, f3 vl, int brick, const float*, int mip, float& t, vr::Rng& sg) {
        HDDA dl = dda;
        dl.prepareLeaf(vl);
        for (int iter = 0; iter < kMaxBrickSteps && inLeaf(dl.p); iter++) {
            float density = densityCell(mip, brick, dl.p);
            dl.next();
            float maxDeltaT = dl.t.y - t;
            float sigma_t = density * c_scene.sigma_t;
            float weight = vr::exp_(Tr) * sigma_t;
            runningSum += weight;
            if (runningSum > 0.f && vr::next1D(sg) < weight / runningSum) { selX = t; selY = vr::fmin_(tFar, t + maxDeltaT); }
            Tr += -maxDeltaT * sigma_t;
            if (t + maxDeltaT >= tFar) return true;
            t += maxDeltaT;
            dl.step();
        }
        return false;
    }
    __device__ void end() {}
};

// The largest float x with vr::exp_(x) < 0.01f (bits 0xc0935d8f): exp_ is non-decreasing, so
// "exp_(Tr) < 0.01f", the early exit of the feature march, is "Tr <= kFeatureCutoff", without an
// exponential per step (tests/test_feature_cutoff.py checks the equivalence over every float of
// [-5.3, -4.4] and on samples of the rest).
constexpr float kFeatureCutoff = -4.60517073f;
struct FeatureMarch {
    float accu = 1.f; float tNear, tFar; Ray ray; float Tr = 0.f; bool lin; float tStep; bool init = false;
    __device__ void setRay(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    __device__ void start() { init = true; }
    __device__ bool mainStep(const HDDA& dda, f3 vl, int brick, const float*, int mip, float& t, vr::Rng&) {
        t = tNear + (vr::floor_((t - tNear) / tStep) + 0.5f) * tStep;
        if (t < dda.t.x) t += tStep;
        f3 wp = ray.o + t * ray.d;
        f3 p = wp - vl;
        const f3 wpt = tStep * ray.d;
        // two samples per trip, as in TrRayMarch: the second sample's density is loaded with the
        // first (a read inside the brick, used only if the march gets there), and the steps are
        // taken one by one with the early exit tested before each, as in the one-sample loop
        int iter = 0;
        while (iter < kMaxBrickSteps && inLeafF(p)) {
            const f3 p1 = p + wpt;
            const bool second = iter + 1 < kMaxBrickSteps && inLeafF(p1);
            const float d0 = densityLocal(mip, brick, p, lin);
            const float d1 = second ? densityLocal(mip, brick, p1, lin) : 0.f;
            if (Tr <= kFeatureCutoff) { end(); return true; }
            float sigma_t = d0 * c_scene.sigma_t;
            Tr += -sigma_t * tStep;
            p = p1;
            t += tStep;
            iter++;
            if (!second) continue;
            if (Tr <= kFeatureCutoff) { end(); return true; }
            sigma_t = d1 * c_scene.sigma_t;
            Tr += -sigma_t * tStep;
            p = p + wpt;
            t += tStep;
            iter++;
        }
        return false;
    }
    __device__ void end() { if (init) accu = vr::exp_(Tr); }
};

struct MediumInteraction { f3 p, wo; float g; bool valid; };

struct DeltaTrack {
    float tNear, tFar; Ray ray; Ray rWorld; MediumInteraction mi;
    __device__ void setRay(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    __device__ void start() {}
    __device__ void setMi(float t) { mi.p = at(rWorld, t); mi.wo = -rWorld.d; mi.g = c_scene.g; mi.valid = true; }
    __device__ bool mainStep(const HDDA& dda, f3 vl, int brick, const float* bnd, int mip, float& t, vr::Rng& sg) {
        float minD = bnd[0], maxD = bnd[1];
        float curTMax = vr::fmin_(tFar, dda.t.y);
        float tc;
        if (minD == 0.f) tc = kRayTMax;
        else tc = t - vr::log_(1 - vr::next1D(sg)) / (minD * c_scene.sigma_t);
        float invMax = 1.f / (maxD - minD);
        if (maxD - minD > 0.f) {
            int guard = 0;
            while (true) {
                if (++guard > kMaxDeltaIters) { atomicOr(c_scene.status, kStatusLoopLimit); break; }
                t -= vr::log_(1 - vr::next1D(sg)) * invMax / c_scene.sigma_t;
                if (t >= tc || t >= curTMax) break;
                f3 p = (ray.o + t * ray.d) - vl;
                float density = densityLocalClamped(mip, brick, p);
                if ((density - minD) * invMax > vr::next1D(sg)) { setMi(t); return true; }
            }
            t = vr::fmin_(tc, t);
            if (t < curTMax) { setMi(t); return true; }
            t = curTMax;
            if (t >= tFar) { end(); return true; }
        } else {
            if (tc < curTMax) { setMi(tc); return true; }
            t = curTMax;
            return false;
        }
        return false;
    }
    __device__ void end() { mi.valid = false; }
};

struct ResidualRatio {
    float tNear, tFar; Ray ray; float Tr = 1.f; bool analog, global;
    __device__ void setRay(float a, float b, const Ray& r) { tNear = a; tFar = b; ray = r; }
    __device__ void start() { if (global) analog = true; }
    __device__ bool mainStep(const HDDA& dda, f3 vl, int brick, const float* bnd, int mip, float& t, vr::Rng& sg) {
        const float st = c_scene.sigma_t;
        float mu_min = global ? 0.f : bnd[0] * st;
        float mu_max = global ? c_scene.slots[mip].maxValue * c_scene.dscale * st : bnd[1] * st;
        float mu_avg = bnd[2] * st;
        float maxDeltaT = vr::fmin_(tFar - t, dda.t.y - t);
        float curTMax = vr::fmin_(tFar, dda.t.y);
        float mrt = mu_max - mu_min;
        float D = c_scene.superDiag;
        float gamma = 2;
        float mu_c = (mrt == 0.f || analog) ? mu_min : vr::fmin_(mu_avg, vr::fmax_(mu_min, mu_min + mrt * (vr::pow_(gamma, 1.f / (D * mrt)) - 1)));
        float mu_r = vr::fmax_(mu_c - mu_min, mu_max - mu_c);
        float inv = 1.f / mu_r;
        float T_c = vr::exp_(-mu_c * vr::fmin_(tFar - t, maxDeltaT));
        float T_r = 1;
        if (mu_r > 0.f) {
            int guard = 0;
            while (true) {
                if (++guard > kMaxDeltaIters) { atomicOr(c_scene.status, kStatusLoopLimit); break; }
                t -= vr::log_(1 - vr::next1D(sg)) * inv;
                if (t >= curTMax) break;
                f3 p = (ray.o + t * ray.d) - vl;
                float mu = densityLocalClamped(mip, brick, p) * st;
                T_r *= 1 - (mu - mu_c) * inv;
            }
        }
        Tr *= T_c * T_r;
        t = curTMax;
        return t >= tFar;
    }
    __device__ void end() {}
};

// ---------------------------------------------------------------------------------------
// tracking entry points (VolumeUtils.slang:284-362, 535-582)
// ---------------------------------------------------------------------------------------
__device__ inline float trAnalytic(const Ray& r, int mip, vr::Rng& sg, bool lin) {
    TrAnalytic a; a.lin = lin;
    trackVolume(r, mip, sg, a, lin);
    return a.Tr;
}
__device__ inline float trRayMarch(const Ray& r, int mip, bool lin, float tss, vr::Rng& sg) {
    int eff = mip >= kPrevSlotOffset ? mip - kPrevSlotOffset : mip;
    eff = eff >= kNumMaxMips ? eff - kNumMaxMips : eff;
    TrRayMarch a; a.lin = lin; a.tStep = c_scene.tStep * tss * (float)(eff + 1);
    trackVolume(r, mip, sg, a, false);
    return a.Tr;
}
// ---------------------------------------------------------------------------------------
// Resumable ray-marched transmittance: the walk of trackVolume + TrRayMarch (cell-centred) as
// explicit state advanced one tree node or one trip of the march (up to two samples) per call,
// for kernels in which a lane whose march ends takes new work while the rest of its warp goes
// on marching.  Performs the operations of trRayMarch in the same order.
// ---------------------------------------------------------------------------------------
struct MarchWalk {
    HDDA dda;
    f3 p, wpt, vmin;
    float tNear, tFar, t, Tr, tStep;
    float tMax1, tMax2;
    int lev, node, nid1, brick, oiter, iter;
    bool inBrick, lin;
};
__device__ __forceinline__ void marchAscend(const DevSlot& s, MarchWalk& w) {
    const float kVdel[3] = {1.f, 8.f, 128.f};
    while (w.lev <= 2 && w.dda.t.x > (w.lev == 1 ? w.tMax1 : w.tMax2)) {
        w.lev++;
        if (w.lev <= 2) {
            w.node = w.lev == 1 ? w.nid1 : 0;
            w.vmin = nodeVmin(s, w.lev, w.node);
            w.dda.prepare(w.vmin, kVdel[w.lev]);
        }
    }
}
// set-up of a march along rWorld in slot `mip` (the tStep of trRayMarch); false when it ended
// there (w.Tr = 1: the ray misses the volume)
__device__ __forceinline__ bool marchStart(const DevSlot& s, int mip, const Ray& rWorld, float tStep, bool lin, MarchWalk& w) {
    Ray ray;
    ray.o = mulPoint(rWorld.o, s.M);
    ray.d = mulVec(rWorld.d, s.M);
    ray.tMin = rWorld.tMin; ray.tMax = rWorld.tMax;
    w.Tr = 0.f;
    w.tStep = tStep;
    w.lin = lin;
    float tNear, tFar;
    if (!intersectBound(ray, tNear, tFar, mip, false)) { w.Tr = 1.f; return false; }
    w.tNear = tNear;
    w.tFar = tFar;
    f3 tStart = mk3(tNear, tFar, 0);
    w.vmin = mk3(0.f);
    w.node = 0;
    tStart.x += 0.01f;
    w.tMax2 = tStart.y;
    w.dda.setFromRay(ray.o, ray.d, tStart);
    w.dda.prepare(w.vmin, 128.f);
    w.t = tNear;
    w.lev = 2;
    w.oiter = 0;
    w.inBrick = false;
    return true;
}
// one step; true when the march has ended (w.Tr holds the transmittance)
__device__ __forceinline__ bool marchStep(const DevSlot& s, int mip, MarchWalk& w) {
    const float eps = 0.01f;
    if (w.inBrick) {
        // one trip of TrRayMarch::mainStep's loop
        if (!(w.iter < kMaxBrickSteps && inLeafF(w.p))) {
            w.inBrick = false;
            w.dda.step();
            w.dda.t.x += eps;
            marchAscend(s, w);
            w.oiter++;
            return false;
        }
        if (w.t >= w.tFar) { w.Tr = vr::exp_(w.Tr); return true; }
        const float mult = 1.f;
        const f3 p1 = w.p + w.wpt;
        const float t1 = w.t + mult * w.tStep;
        const bool second = w.iter + 1 < kMaxBrickSteps && inLeafF(p1) && !(t1 >= w.tFar);
        const float d0 = densityLocal(mip, w.brick, w.p, w.lin);
        const float d1 = second ? densityLocal(mip, w.brick, p1, w.lin) : 0.f;
        float sigma_t = d0 * c_scene.sigma_t;
        w.Tr += -sigma_t * (w.iter == 0 ? 1.f : mult) * w.tStep;
        w.p = p1;
        w.t = t1;
        w.iter++;
        if (!second) return false;
        sigma_t = d1 * c_scene.sigma_t;
        w.Tr += -sigma_t * mult * w.tStep;
        w.p = w.p + w.wpt;
        w.t += mult * w.tStep;
        w.iter++;
        return false;
    }
    const int kDim[3] = {3, 4, 5}, kRes[3] = {8, 16, 32};
    const float kVdel[3] = {1.f, 8.f, 128.f};
    const int* q = w.dda.p;
    if (!(w.oiter < 4096 && w.lev > 0 && w.lev <= 2 && q[0] >= 0 && q[1] >= 0 && q[2] >= 0 && q[0] <= kRes[w.lev] && q[1] <= kRes[w.lev] &&
          q[2] <= kRes[w.lev])) {
        w.Tr = vr::exp_(w.Tr);
        return true;
    }
    w.dda.next();
    const int b = (((w.dda.p[2] << kDim[w.lev]) + w.dda.p[1]) << kDim[w.lev]) + w.dda.p[0];
    const int child = getChild(s, w.node, w.lev, b);
    if (child >= 0) {
        if (w.lev == 1) {
            w.t = w.dda.t.x - eps;
            if (w.t >= w.tFar) { w.Tr = vr::exp_(w.Tr); return true; }
            const f3 vl = nodeVmin(s, 0, child);
            // TrRayMarch::mainStep's entry: the first sample point of the brick
            w.t = w.tNear + (vr::floor_((w.t - w.tNear) / w.tStep) + 0.5f) * w.tStep;
            if (w.t < w.dda.t.x) w.t += w.tStep;
            const f3 wp = w.dda.pos + w.t * w.dda.dir;
            w.p = wp - vl;
            w.wpt = 1.f * w.tStep * w.dda.dir;
            w.iter = 0;
            w.brick = child;
            w.inBrick = true;
            return false;
        }
        w.lev--;
        w.nid1 = child;
        w.node = child;
        w.vmin = nodeVmin(s, w.lev, child);
        w.tMax1 = w.dda.t.y;
        w.dda.prepare(w.vmin, kVdel[w.lev]);
    } else {
        w.dda.step();
        w.dda.t.x += eps;
    }
    marchAscend(s, w);
    w.oiter++;
    return false;
}

__device__ inline float trResidual(const Ray& r, int mip, vr::Rng& sg, bool analog, bool global) {
    ResidualRatio a; a.analog = analog || global; a.global = global;
    trackVolume(r, mip, sg, a, false);
    return a.Tr;
}
static __device__ __forceinline__ float computeVisibility(const Ray& ray, vr::Rng& sg, int samples, int mip, bool lin, uint32_t method, float tss) {
    float vis = 0;
    for (int i = 0; i < samples; i++) {
        if (method == VR_TRACK_RATIO || method == VR_TRACK_RESIDUAL_RATIO || method == VR_TRACK_ANALOG_RESIDUAL_RATIO)
            vis += trResidual(ray, mip, sg, method == VR_TRACK_ANALOG_RESIDUAL_RATIO, method == VR_TRACK_RATIO);
        else if (method == VR_TRACK_RAY_MARCHING)
            vis += trRayMarch(ray, mip, lin, tss, sg);
        else if (method == VR_TRACK_ANALYTIC)
            vis += trAnalytic(ray, mip, sg, lin);
    }
    vis /= samples;
    return vis;
}
// The learned form's generate and bounce kernels track with their own adapter type, so that
// they call their own instance of the (noinline) traversal rather than the one the other
// kernels of the unit share: measured 3 ms faster per 1080p learned frame (136.9-137.2 ->
// 133.7-133.8 ms), with bit-identical images.
struct SampleDistLp : SampleDist {};
template <class SD = SampleDist>
__device__ inline void sampleDistances(const Ray& r, vr::Rng& sg, bool lin, int mip, int n, float hit[4], float pdf[4], float tr[4]) {
    SD a; a.n = n; a.lin = lin;
    if (lin) for (int i = 0; i < n; i++) a.tr[i] = -vr::log_(1 - vr::next1D(sg));
    trackVolume(r, mip, sg, a, lin);
    for (int i = 0; i < 4; ++i) { hit[i] = a.hit[i]; pdf[i] = a.pdf[i]; tr[i] = a.tr[i]; }
}
__device__ inline void deltaTrack(const Ray& r, vr::Rng& sg, MediumInteraction& mi, int mip) {
    DeltaTrack a; a.rWorld = r; a.mi = mi;
    trackVolume(r, mip, sg, a, false);
    mi = a.mi;
}
__device__ inline float rejectionSampleByDensity(const Ray& r, vr::Rng& sg, int mip) {
    CellByDensity a;
    trackVolume(r, mip, sg, a, false);
    if (a.selX == -1) return kRayTMax;
    float d = a.selX + (a.selY - a.selX) * vr::next1D(sg);
    (void)vr::next1D(sg);
    return d;
}
__device__ inline float featureTransmittance(const Ray& r, float tss) {
    FeatureMarch a; a.lin = true; a.tStep = c_scene.tStep * tss;
    vr::Rng sg;
    trackVolume(r, 0, sg, a, false);
    return a.accu;
}

// ---------------------------------------------------------------------------------------
// phase function (VolumeBase.slang:55-93)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ float phaseHG(float cosT, float g) {
    float denom = 1 + g * g + 2 * g * cosT;
    const float Inv4Pi = 0.07957747154594766788444188168626f;
    return Inv4Pi * (1 - g * g) / (denom * vr::sqrt_(denom));
}
__device__ __forceinline__ float phaseF(const MediumInteraction& mi, f3 wo, f3 wi) { return phaseHG(vr::dot(wo, wi), mi.g); }
__device__ inline float samplePhase(const MediumInteraction& mi, f3 wo, f3& wi, float u0, float u1) {
    float g = mi.g, cosT;
    if (vr::fabs_(g) < 1e-3f) cosT = 1 - 2 * u0;
    else {
        float sq = (1 - g * g) / (1 + g - 2 * g * u0);
        cosT = -(1 + g * g - sq * sq) / (2 * g);
    }
    float sinT = vr::sqrt_(vr::fmax_(0, 1 - cosT * cosT));
    float phi = 2 * kM_PI * u1;
    f3 v1 = wo, v2;
    if (vr::fabs_(v1.x) > vr::fabs_(v1.y)) v2 = mk3(-v1.z, 0, v1.x) / vr::sqrt_(v1.x * v1.x + v1.z * v1.z);
    else v2 = mk3(0, v1.z, -v1.y) / vr::sqrt_(v1.y * v1.y + v1.z * v1.z);
    f3 v3 = vr::cross(v1, v2);
    wi = sinT * vr::cos_(phi) * v2 + sinT * vr::sin_(phi) * v3 + cosT * wo;
    return phaseHG(cosT, g);
}

// ---------------------------------------------------------------------------------------
// environment (EnvMap.slang:45-50, EnvMapSampler.slang:55-166, MathHelpers.slang:92-219)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ float signf_(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
__device__ inline f3 octToDir(float px, float py) {
    px = px * 2.f - 1.f; py = py * 2.f - 1.f;
    float d = 1.f - (vr::fabs_(px) + vr::fabs_(py));
    float r = 1.f - vr::fabs_(d);
    float phi = (r > 0.f) ? ((vr::fabs_(py) - vr::fabs_(px)) / r + 1.f) * kM_PI_4 : 0.f;
    float f = r * vr::sqrt_(2.f - r * r);
    return mk3(f * signf_(px) * vr::cos_(phi), f * signf_(py) * vr::sin_(phi), signf_(d) * (1.f - r * r));
}
static __device__ __noinline__ f3 envEval(f3 dir) {
    if (!c_scene.hasEnv) return mk3(0.f);
    f3 p = vr::normalize(mul33(dir, c_scene.envInv));
    float u = vr::atan2_(p.x, -p.z) * kM_1_2PI + 0.5f;
    float v = vr::acos_(p.y) * kM_1_PI;
    const int W = c_scene.envW, H = c_scene.envH;
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float fx0 = vr::floor_(x), fy0 = vr::floor_(y);
    float fx = x - fx0, fy = y - fy0;
    int ix = vr::f2i(fx0), iy = vr::f2i(fy0);
    int x0 = ix % W; if (x0 < 0) x0 += W;
    int x1 = (ix + 1) % W; if (x1 < 0) x1 += W;
    int y0 = iy < 0 ? 0 : (iy >= H ? H - 1 : iy);
    int y1 = iy + 1 < 0 ? 0 : (iy + 1 >= H ? H - 1 : iy + 1);
    const float* T = c_scene.envRGB;
    float c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float a = __ldg(&T[((size_t)y0 * W + x0) * 3 + k]), b = __ldg(&T[((size_t)y0 * W + x1) * 3 + k]);
        float cc = __ldg(&T[((size_t)y1 * W + x0) * 3 + k]), d = __ldg(&T[((size_t)y1 * W + x1) * 3 + k]);
        c[k] = lerp_(lerp_(a, b, fx), lerp_(cc, d, fx), fy);
    }
    return c_scene.envScale * mk3(c[0], c[1], c[2]);
}
static __device__ __noinline__ void envSample(float px, float py, f3& dirOut, float& pdfOut, f3& LeOut) {
    unsigned posx = 0, posy = 0;
    for (int mip = c_scene.impBaseMip - 1; mip >= 0; mip--) {
        posx *= 2; posy *= 2;
        int d = c_scene.impDim >> mip;
        const float* m = c_scene.imp + c_scene.impOff[mip];
        float w0 = __ldg(&m[(size_t)posy * d + posx]), w1 = __ldg(&m[(size_t)posy * d + posx + 1]);
        float w2 = __ldg(&m[(size_t)(posy + 1) * d + posx]), w3 = __ldg(&m[(size_t)(posy + 1) * d + posx + 1]);
        float q0 = w0 + w2, q1 = w1 + w3;
        unsigned offx, offy;
        float dd = q0 / (q0 + q1);
        if (px < dd) { offx = 0; px = px / dd; } else { offx = 1; px = (px - dd) / (1.f - dd); }
        float ee = offx ? w1 / q1 : w0 / q0;
        if (py < ee) { offy = 0; py = py / ee; } else { offy = 1; py = (py - ee) / (1.f - ee); }
        posx += offx; posy += offy;
    }
    float inv = 1.f / (float)c_scene.impDim;
    f3 dir = octToDir(((float)posx + px) * inv, ((float)posy + py) * inv);
    float avg_w = __ldg(&c_scene.imp[c_scene.impOff[c_scene.impBaseMip]]);
    float pdf = __ldg(&c_scene.imp[(size_t)posy * c_scene.impDim + posx]) / avg_w;
    dirOut = mul33(dir, c_scene.envRot);
    pdfOut = pdf * kM_1_4PI;
    LeOut = envEval(dirOut);
}
__device__ __forceinline__ f3 decodeLightUV(float u0, float u1, int lightID) {
    f3 d = mk3(u0, u1, 0);
    d.z = vr::sqrt_(1 - u0 * u0 - u1 * u1);
    if (vr::isnan_(d.z)) d.z = 0.f;
    if (lightID == -2) d.z = -d.z;
    return mul33(d, c_scene.envRot);
}

// ---------------------------------------------------------------------------------------
// lights (VolumeUtils.slang:12-149, 485-521; LightHelpers.slang:223-242)
// ---------------------------------------------------------------------------------------
struct LightSample { f3 dir; float distance; f3 Li; float pdf, pdfArea; };
__device__ __forceinline__ void pointLight(f3 x, int i, f3& dir, float& dist, f3& Li) {
    f3 toL = mk3(c_scene.lightPos[i][0], c_scene.lightPos[i][1], c_scene.lightPos[i][2]) - x;
    float d2 = vr::fmax_(vr::dot(toL, toL), 1e-9f);
    dist = vr::sqrt_(d2);
    dir = toL / dist;
    Li = mk3(c_scene.lightI[i][0], c_scene.lightI[i][1], c_scene.lightI[i][2]) / d2;
}
__device__ inline bool sampleLights(f3 x, bool useEnv, bool useAn, vr::Rng& sg, LightSample& ls, int& lid, float& uv0, float& uv1) {
    if (!useEnv && !useAn) return false;
    float p0 = useEnv ? 1.f : 0.f, p1 = useAn ? 1.f : 0.f, p2 = 0.f;
    float sum = p0 + p1 + p2;
    if (sum == 0.f) return false;
    float invSum = 1.f / sum;
    p0 *= invSum; p1 *= invSum;
    float u = vr::next1D(sg);
    if (useEnv) {
        if (u < p0) {
            float sel = p0;
            float r0 = vr::next1D(sg), r1 = vr::next1D(sg);
            f3 d, Le; float epdf;
            envSample(r0, r1, d, epdf, Le);
            float pdf = sel * epdf;
            ls.dir = d; ls.distance = kRayTMax; ls.pdf = pdf; ls.pdfArea = pdf;
            ls.Li = pdf > 0.f ? Le / pdf : mk3(0.f);
            f3 loc = mul33(d, c_scene.envInv);
            lid = loc.z < 0 ? -2 : -1;
            uv0 = loc.x; uv1 = loc.y;
            return !(vr::isnan_(d.x) || vr::isnan_(d.y) || vr::isnan_(d.z));
        }
        u -= p0;
    }
    if (useAn) {
        if (u < p1) {
            u /= p1;
            uint32_t n = (uint32_t)c_scene.numLights;
            uint32_t li = min(vr::f2u32(u * (float)n), n - 1);
            float sel = p1 / (float)n;
            f3 d, Li; float dist;
            pointLight(x, (int)li, d, dist, Li);
            lid = (int)li;
            ls.dir = d; ls.distance = dist;
            ls.pdf = sel * 1.f; ls.pdfArea = ls.pdf;
            ls.Li = Li / ls.pdf;
            uv0 = 0; uv1 = 0;
            return true;
        }
    }
    return false;
}
__device__ inline f3 sampleDirectLighting(vr::Rng& sg, float& pdf, const MediumInteraction& mi, const SamplingOptions& o, bool shadow,
                                          int& lid, float& uv0, float& uv1) {
    LightSample ls;
    bool valid = sampleLights(mi.p, o.useEnvironmentLights != 0, o.useAnalyticLights != 0, sg, ls, lid, uv0, uv1);
    if (!valid) { pdf = 0.f; return mk3(0.f); }
    pdf = ls.pdfArea;
    ls.pdf = 1.f;
    if (shadow) {
        Ray sr{mi.p, ls.dir, 0, ls.distance};
        float vis = computeVisibility(sr, sg, o.lightSamples, o.lightingMipLevel, o.lightingUseLinearSampler != 0, o.lightingTrackingMethod, o.lightingTStepScale);
        ls.Li = ls.Li * vis;
    }
    float p = phaseF(mi, mi.wo, ls.dir);
    return mk3(0.f) + p * ls.Li / ls.pdf;
}

// ---------------------------------------------------------------------------------------
// path contribution re-evaluation (ReSTIRHelper.slang:91-496)
// ---------------------------------------------------------------------------------------
// Where evaluateF takes its transmittances from: DirectVis estimates them in place; the split
// spatial round records the segments first and replays the marched values (k_spatial_split).
struct DirectVis {
    __device__ __forceinline__ float operator()(const Ray& r, vr::Rng& sg, int samples, int mip, bool lin, uint32_t method, float tss) {
        return computeVisibility(r, sg, samples, mip, lin, method, tss);
    }
};
// pre / reuse: vertex reuse takes the light transmittance from the reservoir's p_partial, or hands
// the estimated one back for it (ReSTIRHelper.slang:443-496)
template <class V>
__device__ inline f3 evalLightInVolume(const MediumInteraction& mi, int lid, float uv0, float uv1, vr::Rng& sg, const SamplingOptions& o, bool cull,
                                       int off, V& vis, float* pre = nullptr, bool reuse = false) {
    Ray sr;
    f3 Ld;
    if (lid < 0) {
        f3 wi = decodeLightUV(uv0, uv1, lid);
        sr = Ray{mi.p, wi, 0, kRayTMax};
        Ld = envEval(wi) * phaseF(mi, mi.wo, wi);
    } else if (lid < c_scene.numLights) {
        f3 d, Li; float dist;
        pointLight(mi.p, lid, d, dist, Li);
        sr = Ray{mi.p, d, 0, dist};
        Ld = Li * phaseF(mi, mi.wo, d);
    } else {
        return mk3(0.f);
    }
    float Tr;
    if (reuse) Tr = *pre;
    else {
        Tr = vis(sr, sg, o.lightSamples, cull ? o.lightingMipLevel + off : 0, o.lightingUseLinearSampler != 0, o.lightingTrackingMethod, o.lightingTStepScale);
        if (pre) *pre = Tr;
    }
    return Tr * Ld;
}

// extra: the extra-bounce plane base, indexed extra[b * N + tap.startPixel]; lastFrame: the
// sample as of the previous frame (the temporal tap's MIS weight), on the previous animation
// frame's grids when the volume is animated and usePrevGrid is set
// spatialReuse / ppOut: vertex reuse (the reservoir is REUSETYPE inout in ReSTIRHelper.slang:91-420):
// spatial reuse takes the suffix's share of p_hat from tap.pp; other calls write the share they
// evaluate to *ppOut (when given)
template <class V>
static __device__ __noinline__ f3 evaluateFV(const Reservoir& tap, const float4* extra, int N, Ray ray, vr::Rng& sg, const SamplingOptions& o,
                                             int maxBounces, bool noReuse, bool isFinal, bool lastFrame, V& vis, bool spatialReuse = false,
                                             float* ppOut = nullptr) {
    const int vrs = o.vertexReuseStartBounce;
    const bool vreuse = vrs >= 0;
    f3 P_prefix = mk3(1.f);
    int bounceId = 0;
    const bool useLast = lastFrame && c_scene.usePrevGrid && c_scene.hasAnimation;
    const int off = useLast ? kPrevSlotOffset : 0;
    bool isBg = tap.depth == kRayTMax;
    ray.tMax = tap.depth;
    f3 F = mk3(1.f);
    int mib = decodeBounces(tap.sampledPixel, maxBounces);
    bool isSelfEmission = maxBounces > 1 ? (mib == 0 && tap.lightID == kSelfEmissionLightID) : (tap.lightID == kSelfEmissionLightID);
    float visibility = 1.f;
    f3 pW = at(ray, ray.tMax);
    MediumInteraction mi{at(ray, ray.tMax), -ray.d, c_scene.g, true};
    {
        float density = (isBg || noReuse) ? 1.f : densityWorld(pW, off);
        if (density == 0.f) return mk3(0.f);
        if (!noReuse)
            visibility = vis(ray, sg, o.visibilitySamples, o.visibilityMipLevel + off, o.visibilityUseLinearSampler != 0, o.visibilityTrackingMethod, o.visibilityTStepScale);
        f3 sig = isBg ? mk3(1.f) : (isSelfEmission ? c_scene.sigma_a : c_scene.sigma_s);
        if (noReuse && !isBg) sig = sig / c_scene.sigma_t;
        F = F * (visibility * density * sig);
    }
    if (vr::any_gt0(F)) {
        if (isBg) {
            F = F * envEval(ray.d);
        } else if (isSelfEmission) {
            F = F * emissionWorld(pW, useLast);
        } else {
            bool scatterEm = false;
            Ray sr{};
            if (maxBounces > 1 && mib > 0) {
                scatterEm = decodeTag(tap.sampledPixel) == 1;
                for (; bounceId < mib; bounceId++) {
                    const int b = bounceId;
                    bool curEm = scatterEm && b == mib - 1;
                    float4 e = extra[(size_t)b * N + tap.startPixel];
                    float wx, wy, wzz, ww;
                    if (vreuse && b + 1 >= vrs) {
                        // decodeWiDist (ReSTIRHelper.slang:21-39), vertex form (vertex reuse)
                        if (e.x == kRayTMax) { wx = 0.f; wy = 0.f; wzz = 0.f; ww = kRayTMax; }
                        else { wx = e.x; wy = e.y; wzz = e.z; ww = -1.f; }
                    } else {
                        // decodeWiDist, direction form
                        f3 wi = mk3(e.x, e.y, vr::sqrt_(1.0f - (e.x * e.x + e.y * e.y)));
                        if (vr::isnan_(wi.z)) wi.z = 0.f;
                        float wz = e.z;
                        if (wz < 0) { wi.z = -wi.z; wz = -wz; }
                        wx = wi.x; wy = wi.y; wzz = wi.z; ww = wz;
                    }
                    if (curEm && (!vreuse || b + 1 < vrs)) { wx = tap.uv0; wy = tap.uv1; wzz = __int_as_float(tap.lightID); ww = -1.f; }
                    if (ww == kRayTMax) return mk3(0.f);
                    float dist = 1.f;
                    if (ww == -1.f) {
                        f3 disp = mk3(wx, wy, wzz) - pW;
                        dist = vr::length(disp);
                        sr = Ray{pW, vr::normalize(disp), 0.f, dist};
                    } else {
                        sr = Ray{pW, mk3(wx, wy, wzz), 0.f, ww};
                    }
                    F = F * mk3(phaseF(mi, mi.wo, sr.d));
                    if (vr::all_eq0(F)) return mk3(0.f);
                    if (vreuse && b == vrs) {                // ReSTIRHelper.slang:289-295
                        if (spatialReuse) return F * tap.pp;
                        P_prefix = F;
                    }
                    pW = ww == -1.f ? mk3(wx, wy, wzz) : at(sr, sr.tMax);
                    f3 sig; float sd;
                    if (!noReuse) {
                        sig = curEm ? c_scene.sigma_a : c_scene.sigma_s;
                        sd = vr::fmax_(0, densityWorld(pW, off));
                    } else {
                        sig = curEm ? c_scene.sigma_a / c_scene.sigma_t : c_scene.sigma_s / c_scene.sigma_t;
                        sd = 1.f;
                    }
                    F = F * (sd * sig);
                    if (vreuse ? (b + 1 == vrs || (curEm && b + 1 < vrs)) : curEm) F = F * (1.f / (dist * dist));
                    if (vr::all_eq0(F)) return mk3(0.f);
                    float sv = 1.f;
                    if (!noReuse)
                        sv = vis(sr, sg, o.visibilitySamples, o.visibilityMipLevel + off, o.visibilityUseLinearSampler != 0, o.visibilityTrackingMethod, o.visibilityTStepScale);
                    F = F * sv;
                    mi.wo = -sr.d;
                    mi.p = pW;
                    if (vr::all_eq0(F)) return mk3(0.f);
                }
                if (scatterEm) F = F * emissionWorld(pW, useLast);
                else mi = MediumInteraction{at(sr, sr.tMax), -sr.d, c_scene.g, true};
            }
            if (!scatterEm && vr::any_gt0(F)) {
                const bool reuse = vreuse && bounceId == vrs && spatialReuse;
                float pre = tap.pp;
                F = F * evalLightInVolume(mi, tap.lightID, tap.uv0, tap.uv1, sg, o, !isFinal, off, vis, &pre, reuse);
                if (vreuse && bounceId == vrs && !spatialReuse && ppOut) *ppOut = pre;
            }
        }
    }
    // ReSTIRHelper.slang:415-419: the suffix's share of p_hat
    if (vreuse && bounceId > vrs && !spatialReuse && ppOut)
        *ppOut = vr::luminance(mk3(F.x / P_prefix.x, F.y / P_prefix.y, F.z / P_prefix.z));
    return F;
}
__device__ __forceinline__ f3 evaluateF(const Reservoir& tap, const float4* extra, int N, const Ray& ray, vr::Rng& sg, const SamplingOptions& o,
                                        int maxBounces, bool noReuse, bool isFinal, bool lastFrame = false) {
    DirectVis v;
    return evaluateFV<DirectVis>(tap, extra, N, ray, sg, o, maxBounces, noReuse, isFinal, lastFrame, v);
}
// spatialReuse / ppOut as in evaluateFV (vertex reuse)
__device__ __forceinline__ float evalPHat(const Reservoir& tap, const float4* extra, int N, const Ray& ray, vr::Rng& sg, const SamplingOptions& o, int mb,
                                         bool lastFrame = false, bool spatialReuse = false, float* ppOut = nullptr) {
    DirectVis v;
    return vr::luminance(evaluateFV<DirectVis>(tap, extra, N, ray, sg, o, mb, false, false, lastFrame, v, spatialReuse, ppOut));
}
// resampleNeighbor (the tap's p_partial re-evaluated: REUSETYPE inout) and, with spatialReuse,
// resampleNeighborSpatialReuse (ReSTIRHelper.slang:567-600)
__device__ __forceinline__ void resampleNeighbor(Reservoir& tap, const Ray& ray, vr::Rng& sg, const float4* extra, int N, const SamplingOptions& o, int mb,
                                                 bool spatialReuse = false) {
    if (tap.runningSum == 0.f) return;
    float ph = evalPHat(tap, extra, N, ray, sg, o, mb, false, spatialReuse, spatialReuse ? nullptr : &tap.pp);
    float w = ph / tap.p_y;
    if (vr::isinf_(w) || vr::isnan_(w)) w = 0.f;
    tap.runningSum *= w;
    tap.p_y = ph;
}

__device__ __forceinline__ f3 pinholeDir(f3 U, f3 V, f3 W, int px, int py, int Wd, int Ht) {
    float sx = ((float)px + 0.5f) / (float)Wd, sy = ((float)py + 0.5f) / (float)Ht;
    float nx = 2.f * sx + -1.f, ny = -2.f * sy + 1.f;
    return nx * U + ny * V + W;
}

}  // namespace vrd
