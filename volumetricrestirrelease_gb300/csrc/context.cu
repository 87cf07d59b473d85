// context.cu -- host side of libvrestir: the C ABI, the per-frame orchestration
// (VolumetricReSTIR::execute, VolumetricReSTIR.cpp:303-906) and the kernel instantiations.
//
// The context owns every device buffer: the sparse brick grid of each mip slot, the
// environment map with its importance pyramid, and the SoA reservoir buffers (current,
// spatial ping-pong, temporal history), the extra-bounce planes and the feature buffers.
// All work of a call goes on the caller's stream; nothing synchronises except the
// *_host variants, the exports and the status query.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/vrestir.h"
#include "lp_net.h"
// NVTX ranges around the passes of a frame (header-only NVTX 3: no cost unless a profiler attaches)
#if !defined(VR_HOST_EMULATION)
#include <nvtx3/nvToolsExt.h>
#define VR_RANGE(name) nvtxRangePushA(name)
#define VR_RANGE_END() nvtxRangePop()
#else
#define VR_RANGE(name) ((void)0)
#define VR_RANGE_END() ((void)0)
#endif
#include "vr_kernels.cuh"
#include "vr_lp.h"
#include "vr_volume.h"

// per-path-length kernel objects (frame_kernels.cu compiled with VR_MB = 1..4)
namespace vrk {
#define VR_DECL(MB)                                                                                           \
    cudaError_t upload_scene_##MB(const vrd::DevScene&, cudaStream_t);                                         \
    void launch_initial_##MB(const vrd::FrameParams&, const vrd::FrameBuffers&, dim3, dim3, cudaStream_t);     \
    void launch_spatial_##MB(const vrd::FrameParams&, const vrd::FrameBuffers&, const vrd::SpatialParams&, dim3, dim3, const vrd::SpatialSplit*, int, \
                             cudaStream_t);                                                                     \
    void launch_final_##MB(const vrd::FrameParams&, const vrd::FrameBuffers&, int, dim3, dim3, cudaStream_t);  \
    void launch_reference_##MB(const vrd::FrameParams&, int, int, double*, dim3, dim3, cudaStream_t);        \
    void launch_lp_generate_##MB(const vrd::FrameParams&, const vrd::FrameBuffers&, const vrd::LpBuffers&, dim3, dim3, cudaStream_t); \
    void launch_lp_select_##MB(const vrd::FrameParams&, const vrd::FrameBuffers&, const vrd::LpBuffers&, dim3, dim3, cudaStream_t); \
    void launch_lp_train_gen_##MB(const vrd::FrameParams&, const vrd::LpBuffers&, uint32_t, cudaStream_t);          \
    void launch_lp_bounce_##MB(const vrd::FrameParams&, const vrd::LpBuffers&, int, int, int, cudaStream_t);      \
    void launch_lp_sort_##MB(const vrd::LpBuffers&, int, int, cudaStream_t);
VR_DECL(1) VR_DECL(2) VR_DECL(3) VR_DECL(4)
#undef VR_DECL
// the network kernels (lp.cu)
cudaError_t net_setup();
void launch_net_infer(const vrd::NetView&, const float4*, int, const int*, float*, const int*, int*, int, cudaStream_t);
void launch_net_train(const vrd::NetView&, const float4*, int, float*, float*, int*, cudaStream_t);
void launch_net_reduce_adam(const float*, int, const float*, float*, float*, float*, float*, float*, uint16_t*, float*, float, float, float,
                            const float*, int, cudaStream_t);
void launch_net_pack(const float*, uint16_t*, float*, cudaStream_t);
}

using vr::f3;
using vr::mk3;

namespace {

// ---------------------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------------------
struct CamFrame {
    f3 pos, U, V, W;
    float view[16], proj[16];
};

// Camera.cpp:183-189 (pinhole frame, focal distance 1) and the glm lookAt / perspective
// matrices the temporal pass reprojects with (depth range [0, 1]).
CamFrame camera_frame(const vr_camera& c, int W, int H) {
    CamFrame f;
    f3 pos = mk3(c.pos[0], c.pos[1], c.pos[2]);
    f3 tgt = mk3(c.target[0], c.target[1], c.target[2]);
    f3 up = mk3(c.up[0], c.up[1], c.up[2]);
    float aspect = (float)W / (float)H;
    float th = vr::tan_(c.fov_y * 0.5f);
    f.pos = pos;
    f.W = vr::normalize(tgt - pos) * 1.f;
    f.U = vr::normalize(vr::cross(f.W, up));
    f.V = vr::normalize(vr::cross(f.U, f.W));
    f.U = f.U * (1.f * th * aspect);
    f.V = f.V * (1.f * th);
    f3 fw = vr::normalize(tgt - pos);
    f3 s = vr::normalize(vr::cross(fw, up));
    f3 u = vr::cross(s, fw);
    float* v = f.view;
    for (int i = 0; i < 16; ++i) v[i] = 0.f;
    v[0] = s.x; v[4] = s.y; v[8] = s.z;
    v[1] = u.x; v[5] = u.y; v[9] = u.z;
    v[2] = -fw.x; v[6] = -fw.y; v[10] = -fw.z;
    v[12] = -vr::dot(s, pos); v[13] = -vr::dot(u, pos); v[14] = vr::dot(fw, pos); v[15] = 1.f;
    float* p = f.proj;
    for (int i = 0; i < 16; ++i) p[i] = 0.f;
    p[0] = 1.f / (aspect * th);
    p[5] = 1.f / th;
    p[10] = c.far_z / (c.near_z - c.far_z);
    p[11] = -1.f;
    p[14] = -(c.far_z * c.near_z) / (c.far_z - c.near_z);
    return f;
}

// SpatialReuse.cs.slang:64-81: the neighbour offsets of a round are the same for every pixel
void neighbor_offsets(const vr_options& o, int r2TimeSeed, int offs[][2]) {
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
        } else if (sid == 0) {
            ux = 0.f; uy = 0.f;
        } else {
            double m = (double)(r2TimeSeed * o.mSpatialSampleCount + sid);
            double a = 0.754877669 * m, b = 0.569840296 * m;
            ux = (float)(a - std::floor(a));
            uy = (float)(b - std::floor(b));
        }
        float r = vr::sqrt_(ux), phi = vrd::kM_2PI * uy;
        offs[sid][0] = vr::f2i(o.mSampleRadius * (r * vr::cos_(phi)));
        offs[sid][1] = vr::f2i(o.mSampleRadius * (r * vr::sin_(phi)));
    }
}

// lat-long env lookup, octahedral map and importance pyramid (EnvMapSamplerSetup.cs.slang)
struct HostEnv {
    std::vector<float> rgb;
    int w = 0, h = 0;
    std::vector<float> imp;    // concatenated mips
    int off[12] = {};
};
float host_lerp(float a, float b, float t) { return a + (b - a) * t; }
float signf_h(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
void env_tex(const HostEnv& e, float u, float v, float c[3]) {
    float x = u * (float)e.w - 0.5f, y = v * (float)e.h - 0.5f;
    float fx0 = vr::floor_(x), fy0 = vr::floor_(y);
    float fx = x - fx0, fy = y - fy0;
    int ix = vr::f2i(fx0), iy = vr::f2i(fy0);
    int x0 = ix % e.w; if (x0 < 0) x0 += e.w;
    int x1 = (ix + 1) % e.w; if (x1 < 0) x1 += e.w;
    int y0 = iy < 0 ? 0 : (iy >= e.h ? e.h - 1 : iy);
    int y1 = iy + 1 < 0 ? 0 : (iy + 1 >= e.h ? e.h - 1 : iy + 1);
    for (int k = 0; k < 3; ++k) {
        float a = e.rgb[((size_t)y0 * e.w + x0) * 3 + k], b = e.rgb[((size_t)y0 * e.w + x1) * 3 + k];
        float cc = e.rgb[((size_t)y1 * e.w + x0) * 3 + k], d = e.rgb[((size_t)y1 * e.w + x1) * 3 + k];
        c[k] = host_lerp(host_lerp(a, b, fx), host_lerp(cc, d, fx), fy);
    }
}
void build_importance(HostEnv& e) {
    const int dim = 512, sx = 8, sy = 8, base = 9;
    size_t total = 0;
    for (int m = 0; m <= base; ++m) { e.off[m] = (int)total; total += (size_t)(dim >> m) * (dim >> m); }
    e.imp.assign(total, 0.f);
    const float invSamples = 1.f / (float)(sx * sy);
    const float dimS = (float)(dim * sx);
    int nt = std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&]() {
            for (int py; (py = next.fetch_add(1)) < dim;)
                for (int px = 0; px < dim; ++px) {
                    float L = 0.f;
                    for (int y = 0; y < sy; ++y)
                        for (int x = 0; x < sx; ++x) {
                            float ppx = ((float)(px * sx + x) + 0.5f) / dimS, ppy = ((float)(py * sy + y) + 0.5f) / dimS;
                            // oct_to_ndir_equal_area_unorm (MathHelpers.slang:200-219)
                            float qx = ppx * 2.f - 1.f, qy = ppy * 2.f - 1.f;
                            float d = 1.f - (vr::fabs_(qx) + vr::fabs_(qy));
                            float r = 1.f - vr::fabs_(d);
                            float phi = (r > 0.f) ? ((vr::fabs_(qy) - vr::fabs_(qx)) / r + 1.f) * vrd::kM_PI_4 : 0.f;
                            float f = r * vr::sqrt_(2.f - r * r);
                            f3 dir = mk3(f * signf_h(qx) * vr::cos_(phi), f * signf_h(qy) * vr::sin_(phi), signf_h(d) * (1.f - r * r));
                            // world_to_latlong_map (MathHelpers.slang:92-99)
                            f3 pn = vr::normalize(dir);
                            float u = vr::atan2_(pn.x, -pn.z) * vrd::kM_1_2PI + 0.5f;
                            float v = vr::acos_(pn.y) * vrd::kM_1_PI;
                            float c[3];
                            env_tex(e, u, v, c);
                            L += vr::luminance(mk3(c[0], c[1], c[2]));
                        }
                    e.imp[(size_t)py * dim + px] = L * invSamples;
                }
        });
    for (auto& t : th) t.join();
    for (int m = 1; m <= base; ++m) {
        int d = dim >> m, ds = dim >> (m - 1);
        const float* s = &e.imp[e.off[m - 1]];
        float* o = &e.imp[e.off[m]];
        for (int y = 0; y < d; ++y)
            for (int x = 0; x < d; ++x) {
                float a = s[(size_t)(2 * y) * ds + 2 * x], b = s[(size_t)(2 * y) * ds + 2 * x + 1];
                float c = s[(size_t)(2 * y + 1) * ds + 2 * x], dd = s[(size_t)(2 * y + 1) * ds + 2 * x + 1];
                o[(size_t)y * d + x] = (((a + b) + c) + dd) * 0.25f;
            }
    }
}

}  // namespace

// Every device allocation of the library's contexts goes through dev_malloc, so that host-side
// fault injection (vr_debug_fail_allocation) can make the n-th one fail as an out-of-memory would.
static std::atomic<int64_t> g_failAlloc{-1};
template <class T>
static cudaError_t dev_malloc(T** p, size_t bytes) {
    if (g_failAlloc.load() >= 0 && g_failAlloc.fetch_sub(1) == 0) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc((void**)p, bytes);
}

namespace {

template <class T>
T* dalloc(size_t n) {
    T* p = nullptr;
    if (n == 0) n = 1;
    if (dev_malloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
    return p;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------------------
struct vr_context {
    vr_options opts;
    int W = 0, H = 0;
    std::string err;
    // scene
    vrd::DevScene scene{};
    std::vector<void*> sceneAllocs;
    bool hasVolume = false;
    int numMips = 0;
    int staticRes = 0;
    std::vector<void*> envAllocs;
    std::vector<void*> emisAllocs;
    HostEnv env;
    // emission parameters of the last vr_set_emission (the reference's defaults until then)
    bool emisParamsSet = false;
    // animated volume: every frame's grids resident, bound cyclically frame by frame
    struct AnimFrame {
        vrd::DevSlot slots[VR_NUM_SLOTS];
        vrd::DevSlot temp, vel[3];
        bool hasTemp = false;
    };
    std::vector<AnimFrame> anim;
    std::vector<void*> animAllocs;
    vrd::DevSlot staticSlots[VR_NUM_SLOTS]{};   // the volume of vr_set_volume
    int animId = -1;
    bool animTemp = false, animVel = false;
    float animVelScale = 1.f;
    // buffers
    vrd::ResBuf res[3]{};      // 0 = perPixel[0], 1 = perPixel[1], 2 = temporal history
    float* feat[2] = {nullptr, nullptr};
    int featCurIdx = 0;
    float* color = nullptr;
    int allocMB = 0, allocW = 0, allocH = 0;
    // frame state
    int frameCount = 0;
    bool optionsChanged = true;
    int temporalSampleAccumulated = 0;
    CamFrame prev{};
    int finalBuf = 0;
    // instrumentation: per-frame event triples (frame start, after k_initial, after the last
    // kernel), summed only when the caller asks, so timing never synchronises a frame
    cudaEvent_t ev[10] = {};
    int nev = 0;
    std::vector<std::vector<cudaEvent_t>> pendingEv;
    std::vector<cudaEvent_t> freeEv;
    double totalMs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int totalFrames = 0;
    int launches = 0;
    int64_t h2d = 0, d2h = 0;
    int* status = nullptr;    // device status word
    int blockThreads = 128;   // pixel kernels: blocks of 8 x (blockThreads / 8) pixels
    vr_frame_hook hook = nullptr;   // post-process hook (vr_set_frame_hook)
    void* hookUser = nullptr;
    // the network trains on a side stream (non-blocking, so it also overlaps work on the legacy
    // default stream), forked after select and joined at the end of the frame
    cudaStream_t side = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    // pipelined host output: two device staging images, their copies on a copy stream
    float* hostStage[2] = {nullptr, nullptr};
    cudaStream_t copyStream = nullptr;
    cudaEvent_t copyDone[2] = {nullptr, nullptr}, rendered[2] = {nullptr, nullptr};
    bool copyPending[2] = {false, false};
    int hostIdx = 0;
    size_t hostStageBytes = 0;
    // learned target: network (FP32 master weights, Adam moments, BF16 copy) and the buffers
    // of the split initial pass
    float *netW = nullptr, *netM = nullptr, *netV = nullptr, *netG = nullptr, *netBias = nullptr;
    uint16_t* netWbf = nullptr;
    float *netPart = nullptr, *netLossPart = nullptr, *netScalar = nullptr;
    int netPartRows = 0;
    bool netReady = false;
    int64_t adamStep = 0;
    float netBmin[3] = {0, 0, 0}, netBinv[3] = {1, 1, 1};
    int numSMs = 0;
    vrd::LpBuffers lp{};
    vrd::SpatialSplit split{};           // buffers of the split spatial round (allocated when used)
    float* ppPlane[3] = {nullptr, nullptr, nullptr};   // p_partial of res[0..2], bound under vertex reuse
    size_t splitSlots = 0;
    size_t lpSlots = 0;            // allocated vertex slots (M * MB * N)
    int lpM = 0, lpMB = 0;
    float* stepLoss = nullptr;     // loss of each Adam step of the last frame
    int stepLossCap = 0, lastSteps = 0;
    bool lpFrameDone = false;
};

static void free_buffers(vr_context* c) {
    for (int i = 0; i < 3; ++i) {
        cudaFree(c->res[i].a); cudaFree(c->res[i].b); cudaFree(c->res[i].extra);
        c->res[i] = vrd::ResBuf{};
    }
    cudaFree(c->feat[0]); cudaFree(c->feat[1]); cudaFree(c->color);
    c->feat[0] = c->feat[1] = nullptr; c->color = nullptr;
    for (int i = 0; i < 3; ++i) { cudaFree(c->ppPlane[i]); c->ppPlane[i] = nullptr; }
    c->allocMB = 0;
}

static int alloc_buffers(vr_context* c) {
    const int mb = c->opts.mMaxBounces;
    if (c->allocMB == mb && c->allocW == c->W && c->allocH == c->H) return VR_OK;
    free_buffers(c);
    size_t N = (size_t)c->W * c->H;
    size_t ne = N * (size_t)std::max(mb - 1, 1);
    for (int i = 0; i < 3; ++i) {
        c->res[i].a = dalloc<float4>(N);
        c->res[i].b = dalloc<int4>(N);
        c->res[i].extra = dalloc<float4>(ne);
        if (!c->res[i].a || !c->res[i].b || !c->res[i].extra) { c->err = "out of device memory (reservoirs)"; return VR_ERR_OOM; }
        cudaMemset(c->res[i].a, 0, N * sizeof(float4));
        cudaMemset(c->res[i].b, 0, N * sizeof(int4));
        cudaMemset(c->res[i].extra, 0, ne * sizeof(float4));
    }
    for (int i = 0; i < 2; ++i) {
        c->feat[i] = dalloc<float>(N);
        if (!c->feat[i]) { c->err = "out of device memory (features)"; return VR_ERR_OOM; }
        cudaMemset(c->feat[i], 0, N * sizeof(float));
    }
    c->color = dalloc<float>(N * 4);
    if (!c->color) { c->err = "out of device memory (colour)"; return VR_ERR_OOM; }
    cudaMemset(c->color, 0, N * 4 * sizeof(float));
    for (int i = 0; i < 3; ++i) {
        c->ppPlane[i] = dalloc<float>(N);
        if (!c->ppPlane[i]) { c->err = "out of device memory (p_partial)"; return VR_ERR_OOM; }
        cudaMemset(c->ppPlane[i], 0, N * sizeof(float));
    }
    c->allocMB = mb; c->allocW = c->W; c->allocH = c->H;
    return VR_OK;
}

// ---- the split spatial round: recorded segments, their transmittances, the p-hat table ----
static void free_split(vr_context* c) {
    cudaFree(c->split.seg); cudaFree(c->split.tr); cudaFree(c->split.list); cudaFree(c->split.counts); cudaFree(c->split.E);
    c->split = vrd::SpatialSplit{};
    c->splitSlots = 0;
}
// the spatial options take the split round (vrd::spatialSplitEligible, from the options)
static bool split_needed(const vr_context* c) {
    const vr_options& o = c->opts;
    return o.mEnableSpatialReuse && !o.mUseReference && !(o.mVertexReuse && o.mMaxBounces > 1) && o.mSpatialSampleCount <= vrd::kSplitK &&
           o.mSpatialVisibilityTrackingMethod == VR_TRACK_RAY_MARCHING && o.mSpatialLightingTrackingMethod == VR_TRACK_RAY_MARCHING;
}
static int split_alloc(vr_context* c) {
    const size_t N = (size_t)c->W * c->H;
    const size_t slots = N * (size_t)(vrd::kSplitK * vrd::kSplitK) * (size_t)(c->opts.mMaxBounces + 1);
    if (c->split.seg && c->splitSlots == slots) return VR_OK;
    free_split(c);
    if (slots > (size_t)INT32_MAX) { c->err = "image too large for the split spatial round"; return VR_ERR_INVALID_ARG; }
    c->split.seg = dalloc<float4>(2 * slots);
    c->split.tr = dalloc<float>(slots);
    c->split.list = dalloc<uint2>(slots);
    c->split.counts = dalloc<int>(2);
    c->split.E = dalloc<float>(N * vrd::kSplitK * vrd::kSplitK);
    if (!c->split.seg || !c->split.tr || !c->split.list || !c->split.counts || !c->split.E) {
        free_split(c);
        c->err = "out of device memory (split spatial round)";
        return VR_ERR_OOM;
    }
    c->split.capacity = (int)slots;
    c->splitSlots = slots;
    return VR_OK;
}

// ---- learned target: network state and the buffers of the split initial pass ----
static void free_lp(vr_context* c) {
    cudaFree(c->lp.vrecA); cudaFree(c->lp.vrecB); cudaFree(c->lp.crec); cudaFree(c->lp.dist); cudaFree(c->lp.ex); cudaFree(c->lp.T);
    cudaFree(c->lp.query); cudaFree(c->lp.qlist); cudaFree(c->lp.qcount); cudaFree(c->lp.rng); cudaFree(c->lp.train);
    cudaFree(c->lp.paths[0]); cudaFree(c->lp.paths[1]); cudaFree(c->lp.pcount); cudaFree(c->lp.psort); cudaFree(c->lp.hist);
    c->lp = vrd::LpBuffers{};
    c->lpSlots = 0; c->lpM = 0; c->lpMB = 0;
}
static void free_net(vr_context* c) {
    float* fs[] = {c->netW, c->netM, c->netV, c->netG, c->netBias, c->netPart, c->netLossPart, c->netScalar, c->stepLoss};
    for (float* f : fs) cudaFree(f);
    cudaFree(c->netWbf);
    c->netW = c->netM = c->netV = c->netG = c->netBias = c->netPart = c->netLossPart = c->netScalar = c->stepLoss = nullptr;
    c->netWbf = nullptr;
    c->netPartRows = 0; c->stepLossCap = 0; c->netReady = false;
}

// He-uniform hidden weights from a SplitMix64 stream, small output weights (T starts near 1),
// zero biases; layer 0's four pad columns stay zero
static void net_init_params(uint32_t seed, std::vector<float>& w) {
    w.assign(lpn::kParams, 0.f);
    uint64_t st = 0x6C7E3A91D2B54F08ull ^ ((uint64_t)seed << 17);
    auto uni = [&]() { return (float)((vr::splitmix64_next(st) >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f; };
    for (int l = 0; l < lpn::kLayers; ++l) {
        const int fanIn = l == 0 ? lpn::kIn : lpn::kHid;
        const float bound = std::sqrt(6.f / (float)fanIn);
        for (int r = 0; r < lpn::kHid; ++r)
            for (int k = 0; k < lpn::kInPad; ++k) {
                float u = uni();
                w[lpn::w_off(l) + r * lpn::kInPad + k] = (l == 0 && k >= lpn::kIn) ? 0.f : u * bound;
            }
    }
    const float ob = 0.1f * std::sqrt(6.f / (float)lpn::kHid);
    for (int k = 0; k < lpn::kHid; ++k) w[lpn::kOutW + k] = uni() * ob;
}

static int net_alloc(vr_context* c, int partRows) {
    if (!c->netW) {
        c->netW = dalloc<float>(lpn::kParamsPad); c->netM = dalloc<float>(lpn::kParamsPad); c->netV = dalloc<float>(lpn::kParamsPad);
        c->netG = dalloc<float>(lpn::kParamsPad); c->netBias = dalloc<float>(320); c->netWbf = dalloc<uint16_t>(5 * 4096);
        c->netScalar = dalloc<float>(4);
        if (!c->netW || !c->netM || !c->netV || !c->netG || !c->netBias || !c->netWbf || !c->netScalar) {
            cudaFree(c->netW); cudaFree(c->netM); cudaFree(c->netV); cudaFree(c->netG); cudaFree(c->netBias); cudaFree(c->netWbf);
            cudaFree(c->netScalar);
            c->netW = c->netM = c->netV = c->netG = c->netBias = c->netScalar = nullptr;
            c->netWbf = nullptr;
            c->err = "out of device memory (network)"; return VR_ERR_OOM;
        }
        if (vrk::net_setup() != cudaSuccess) { c->err = "network kernel setup failed"; return VR_ERR_CUDA; }
        cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, 0);
        if (c->numSMs <= 0) c->numSMs = 1;
    }
    if (partRows > c->netPartRows) {
        cudaFree(c->netPart); cudaFree(c->netLossPart);
        c->netPart = dalloc<float>((size_t)partRows * lpn::kParamsPad);
        c->netLossPart = dalloc<float>(partRows);
        if (!c->netPart || !c->netLossPart) {
            cudaFree(c->netPart); cudaFree(c->netLossPart);
            c->netPart = c->netLossPart = nullptr;
            c->netPartRows = 0; c->err = "out of device memory (network gradients)"; return VR_ERR_OOM;
        }
        c->netPartRows = partRows;
    }
    return VR_OK;
}

static int net_upload(vr_context* c, const float* host) {
    cudaMemcpy(c->netW, host, lpn::kParams * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(c->netM, 0, lpn::kParamsPad * sizeof(float));
    cudaMemset(c->netV, 0, lpn::kParamsPad * sizeof(float));
    vrk::launch_net_pack(c->netW, c->netWbf, c->netBias, 0);
    if (cudaDeviceSynchronize() != cudaSuccess) { c->err = "network upload failed"; return VR_ERR_CUDA; }
    c->adamStep = 0;
    c->netReady = true;
    return VR_OK;
}

static int net_ensure(vr_context* c, int partRows) {
    int r = net_alloc(c, std::max(partRows, 1));
    if (r) return r;
    if (!c->netReady) {
        std::vector<float> w;
        net_init_params(c->opts.mLearnedSeed, w);
        return net_upload(c, w.data());
    }
    return VR_OK;
}

static vrd::NetView net_view(const vr_context* c) {
    vrd::NetView v;
    v.wbf = c->netWbf; v.bias = c->netBias;
    for (int i = 0; i < 3; ++i) { v.bmin[i] = c->netBmin[i]; v.binv[i] = c->netBinv[i]; }
    v.floor_ = c->opts.mLearnedTFloor;
    v.lossLog = c->opts.mLearnedLoss;
    return v;
}

// vertex reuse in effect: the option, and paths with indirect vertices
static bool vertex_reuse(const vr_context* c) { return c->opts.mVertexReuse && c->opts.mMaxBounces > 1; }

static bool lp_active(const vr_context* c) {
    const vr_options& o = c->opts;
    return o.mUseLearnedPHat && !o.mUseReference && (o.mEnableTemporalReuse || o.mEnableSpatialReuse);
}

static int lp_alloc(vr_context* c) {
    const vr_options& o = c->opts;
    const size_t N = (size_t)c->W * c->H;
    const int M = o.mInitialM, MB = o.mMaxBounces;
    const size_t slots = (size_t)M * MB * N;
    if (slots >= (size_t)INT32_MAX) { c->err = "mInitialM * mMaxBounces * pixels must stay below 2^31 with the learned target"; return VR_ERR_INVALID_ARG; }
    const int S = std::max(0, o.mLearnedTrainSamples);
    int r = net_ensure(c, (std::min(std::max(o.mLearnedBatch, 1), std::max(S, 1)) + 127) / 128);
    if (r) return r;
    if (c->lpSlots != slots || c->lpM != M || c->lpMB != MB || c->lp.trainCount != S) {
        free_lp(c);
        c->lp.vrecA = dalloc<float4>(slots);
        c->lp.vrecB = dalloc<int4>(slots);
        c->lp.crec = dalloc<float2>((size_t)M * N);
        c->lp.dist = dalloc<float4>((size_t)M * N);
        c->lp.ex = dalloc<float4>((size_t)M * std::max(MB - 1, 1) * N);
        c->lp.T = dalloc<float>(slots);
        c->lp.query = dalloc<float4>(2 * slots);
        c->lp.qlist = dalloc<int>(slots);
        c->lp.qcount = dalloc<int>(1);
        c->lp.rng = dalloc<uint4>(N);
        c->lp.train = dalloc<float4>(2 * (size_t)std::max(S, 1));
        // the queue of bounce b is paths[b & 1]: bounce 1 (every path length above 1) in paths[1],
        // bounce 2 in paths[0], bounce 3 in paths[1] again
        const size_t paths = MB > 1 ? (size_t)M * N : 1;
        c->lp.paths[1] = dalloc<float4>(MB > 1 ? 4 * paths : 4);
        c->lp.paths[0] = dalloc<float4>(MB > 2 ? 4 * paths : 4);
        c->lp.psort = dalloc<float4>(4 * paths);
        c->lp.hist = dalloc<int>(2 * vrd::kPathKeys);
        c->lp.pcount = dalloc<int>(16);         // queue lengths [0, MB], walk cursors from 8 on
        if (!c->lp.vrecA || !c->lp.vrecB || !c->lp.crec || !c->lp.dist || !c->lp.ex || !c->lp.T || !c->lp.query || !c->lp.qlist || !c->lp.qcount || !c->lp.rng || !c->lp.train ||
            !c->lp.paths[0] || !c->lp.paths[1] || !c->lp.pcount || !c->lp.psort || !c->lp.hist) {
            free_lp(c);
            c->err = "out of device memory (learned-target buffers)";
            return VR_ERR_OOM;
        }
        cudaMemset(c->lp.T, 0, slots * sizeof(float));
        cudaMemset(c->lp.qcount, 0, sizeof(int));
        cudaMemset(c->lp.pcount, 0, 16 * sizeof(int));
        c->lp.wcursor = c->lp.pcount + 8;
        c->lp.qcapacity = (int)slots;
        c->lp.pcapacity = (int)paths;
        c->lp.numSlots = M * MB;
        c->lp.trainCount = S;
        c->lpSlots = slots; c->lpM = M; c->lpMB = MB;
    }
    const int steps = S > 0 ? std::max(1, S / std::max(1, std::min(o.mLearnedBatch, S))) : 0;
    if (steps > c->stepLossCap) {
        cudaFree(c->stepLoss);
        c->stepLoss = dalloc<float>(steps);
        if (!c->stepLoss) { c->stepLossCap = 0; c->err = "out of device memory (loss log)"; return VR_ERR_OOM; }
        c->stepLossCap = steps;
    }
    return VR_OK;
}

static bool options_valid(const vr_options* o, std::string& why) {
    if (o->mMaxBounces < 1 || o->mMaxBounces > VR_MAX_BOUNCES) { why = "mMaxBounces must be in [1, 4]"; return false; }
    if (o->mInitialM < 1 || o->mInitialM > 4096) { why = "mInitialM must be in [1, 4096]"; return false; }
    if (o->mSpatialSampleCount < 1 || o->mSpatialSampleCount > 32) { why = "mSpatialSampleCount must be in [1, 32]"; return false; }
    if (o->mSpatialReuseRounds < 1 || o->mSpatialReuseRounds > 16) { why = "mSpatialReuseRounds must be in [1, 16]"; return false; }
    if (o->mBaselineSamplePerPixel < 1) { why = "mBaselineSamplePerPixel must be >= 1"; return false; }
    if (o->mInitialBaseMipLevel < 0 || o->mInitialBaseMipLevel >= VR_NUM_MAX_MIPS) { why = "mInitialBaseMipLevel out of range"; return false; }
    if (o->mInitialLightingMipLevel < 0 || o->mInitialLightingMipLevel >= VR_NUM_SLOTS) { why = "mInitialLightingMipLevel out of range"; return false; }
    if (o->mSpatialVisibilityMipLevel < 0 || o->mSpatialVisibilityMipLevel >= VR_NUM_SLOTS) { why = "mSpatialVisibilityMipLevel out of range"; return false; }
    if (o->mSpatialLightingMipLevel < 0 || o->mSpatialLightingMipLevel >= VR_NUM_SLOTS) { why = "mSpatialLightingMipLevel out of range"; return false; }
    if (o->mTemporalReprojectionMipLevel < 0 || o->mTemporalReprojectionMipLevel >= VR_NUM_MAX_MIPS) { why = "mTemporalReprojectionMipLevel out of range"; return false; }
    uint32_t methods[] = {o->mInitialLightingTrackingMethod, o->mSpatialVisibilityTrackingMethod, o->mSpatialLightingTrackingMethod,
                          o->mFinalVisibilityTrackingMethod, o->mFinalLightTrackingMethod};
    for (uint32_t m : methods) if (m > VR_TRACK_ANALOG_RESIDUAL_RATIO) { why = "unknown tracking method"; return false; }
    if (o->mTemporalReprojectionMode > VR_REPROJ_NO_BACKGROUND) { why = "unknown reprojection mode"; return false; }
    if (o->mUsePrevVolumeForReproj != 0 && o->mUsePrevVolumeForReproj != 1) { why = "mUsePrevVolumeForReproj must be 0 or 1"; return false; }
    if (o->mVertexReuse != 0 && o->mVertexReuse != 1) { why = "mVertexReuse must be 0 or 1"; return false; }
    if (o->mVertexReuseStartBounce < 1 || o->mVertexReuseStartBounce > 64) { why = "mVertexReuseStartBounce must be in [1, 64]"; return false; }
    if (o->mVertexReuse && o->mUseLearnedPHat) { why = "mVertexReuse is not available with mUseLearnedPHat"; return false; }
    if (o->mUseLearnedPHat) {
        if (!o->mEnableTemporalReuse && !o->mEnableSpatialReuse) { why = "mUseLearnedPHat needs temporal or spatial reuse"; return false; }
        if (o->mLearnedTrainSamples < 0 || o->mLearnedTrainSamples > (1 << 26)) { why = "mLearnedTrainSamples must be in [0, 2^26]"; return false; }
        if (o->mLearnedBatch < 1 || o->mLearnedBatch > (1 << 20)) { why = "mLearnedBatch must be in [1, 2^20]"; return false; }
        if (!(o->mLearnedLearningRate >= 0.f) || !(o->mLearnedLearningRate < 1.f)) { why = "mLearnedLearningRate must be in [0, 1)"; return false; }
        if (!(o->mLearnedTFloor > 0.f) || !(o->mLearnedTFloor <= 1.f)) { why = "mLearnedTFloor must be in (0, 1]"; return false; }
        if (o->mLearnedTargetMethod > VR_TRACK_ANALOG_RESIDUAL_RATIO) { why = "unknown mLearnedTargetMethod"; return false; }
        if (o->mLearnedLoss < 0 || o->mLearnedLoss > 1) { why = "mLearnedLoss must be 0 or 1"; return false; }
    }
    return true;
}

// every mip slot the options can reach must exist in the bound volume
static bool slots_present(const vr_context* c, std::string& why) {
    const vr_options& o = c->opts;
    auto need = [&](int slot) {
        if (slot < 0 || slot >= VR_NUM_SLOTS || !c->scene.slots[slot].valid) {
            why = "options need mip slot " + std::to_string(slot) + " which the volume does not have";
            return false;
        }
        return true;
    };
    int base = o.mInitialVisibilityUseLinearSampler ? o.mInitialBaseMipLevel : o.mInitialBaseMipLevel + VR_NUM_MAX_MIPS;
    if (!need(base) || !need(o.mInitialLightingMipLevel) || !need(o.mSpatialVisibilityMipLevel) || !need(o.mSpatialLightingMipLevel) ||
        !need(0) || !need(VR_NUM_MAX_MIPS + o.mTemporalReprojectionMipLevel))
        return false;
    if (o.mInitialUseCoarserGridForIndirectBounce && o.mMaxBounces > 1) {
        int cm = std::min((base >= VR_NUM_MAX_MIPS ? VR_NUM_MAX_MIPS : 0) + c->numMips - 1, base + 1);
        if (!need(cm)) return false;
    }
    return true;
}

template <int MB>
static void launch_frame_kernels(vr_context* c, const vrd::FrameParams& P, vrd::FrameBuffers& B, cudaStream_t st);
#if !defined(VR_HOST_EMULATION)
// gathers the records of a slot list (query export)
__global__ void k_gather_queries(const float4* __restrict__ q, const int* __restrict__ slots, int n, float4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t s = (size_t)slots[i];
    out[2 * (size_t)i] = q[2 * s];
    out[2 * (size_t)i + 1] = q[2 * s + 1];
}
#endif
static void lp_train_steps(vr_context* c, const float4* samples, int S, cudaStream_t st, const float* ccTable = nullptr);
static cudaEvent_t take_event(vr_context* c) {
    cudaEvent_t e;
    if (!c->freeEv.empty()) { e = c->freeEv.back(); c->freeEv.pop_back(); }
    else cudaEventCreate(&e);
    return e;
}

extern "C" {

void vr_options_default(vr_options* o) {
    memset(o, 0, sizeof(*o));
    o->mMaxBounces = 1;
    o->mEnableTemporalReuse = 1;
    o->mEnableSpatialReuse = 1;
    o->mUseReference = 0;
    o->mUseEnvironmentLights = 1;
    o->mUseAnalyticLights = 0;
    o->mBaselineSamplePerPixel = 1;
    o->mVisualizeTotalTransmittance = 0;
    o->mInitialBaseMipLevel = 1;
    o->mInitialM = 4;
    o->mInitialLightSamples = 1;
    o->mInitialLightingMipLevel = 2;
    o->mInitialVisibilityUseLinearSampler = 0;
    o->mInitialLightingUseLinearSampler = 1;
    o->mInitialLightingTrackingMethod = VR_TRACK_RAY_MARCHING;
    o->mInitialVisibilityTStepScale = 1.f;
    o->mInitialLightingTStepScale = 2.f;
    o->mInitialUseRussianRoulette = 1;
    o->mInitialUseCoarserGridForIndirectBounce = 1;
    o->mTemporalReuseMThreshold = 4.f;
    o->mTemporalReprojectionMode = VR_REPROJ_LINEAR;
    o->mTemporalMISMethod = VR_MIS_TALBOT;
    o->mTemporalReprojectionMipLevel = 1;
    o->mSpatialReuseRounds = 1;
    o->mSpatialVisibilityMipLevel = 1;
    o->mSpatialLightingMipLevel = 1;
    o->mSpatialVisibilityUseLinearSampler = 1;
    o->mSpatialLightingUseLinearSampler = 1;
    o->mSpatialVisibilityTStepScale = 1.f;
    o->mSpatialLightingTStepScale = 1.f;
    o->mSpatialVisibilityTrackingMethod = VR_TRACK_RAY_MARCHING;
    o->mSpatialLightingTrackingMethod = VR_TRACK_RAY_MARCHING;
    o->mRandomSamplerType = VR_SAMPLER_R2;
    o->mSampleRadius = 10.f;
    o->mSpatialSampleCount = 4;
    o->mSpatialMISMethod = VR_MIS_TALBOT;
    o->mFinalLightSamples = 1;
    o->mFinalVisibilitySamples = 1;
    o->mFinalVisibilityTrackingMethod = VR_TRACK_ANALYTIC;
    o->mFinalLightTrackingMethod = VR_TRACK_ANALYTIC;
    o->mFinalTStepScale = 0.2f;
    o->mUseLearnedPHat = 0;
    o->mLearnedTrainSamples = 1 << 20;
    o->mLearnedBatch = 16384;
    o->mLearnedLearningRate = 1e-3f;
    o->mLearnedTFloor = 0.02f;
    o->mLearnedSeed = 1;
    o->mLearnedTargetMethod = VR_TRACK_RAY_MARCHING;
    o->mLearnedLoss = 0;
    o->mUsePrevVolumeForReproj = 1;
    o->mVertexReuse = 0;
    o->mVertexReuseStartBounce = 1;
}

// ---- volumes ----
int vr_volume_create_procedural(const vr_procedural_desc* d, vr_volume** out) {
    if (!d || !out) return VR_ERR_INVALID_ARG;
    if (d->res <= 0 || d->res > 4096 || d->num_mips < 1 || d->num_mips > VR_NUM_MAX_MIPS || d->octaves < 1 || d->octaves > 16) return VR_ERR_INVALID_ARG;
    if (d->res % (8 << (d->num_mips - 1)) != 0) return VR_ERR_INVALID_ARG;
    if (!(d->voxel_size > 0.f)) return VR_ERR_INVALID_ARG;
    try {
        std::vector<float> g = vr::procedural_density(*d);
        vr_volume* v = new vr_volume();
        if (vr::build_volume(g, d->res, d->num_mips, d->world_min, d->voxel_size, d->fp16 != 0, v->v) != 0) { delete v; return VR_ERR_INVALID_ARG; }
        *out = v;
        return VR_OK;
    } catch (...) {
        return VR_ERR_OOM;
    }
}
int vr_volume_create_dense(const float* density, int32_t res, int32_t num_mips, const float world_min[3], float voxel_size, int32_t fp16, vr_volume** out) {
    if (!density || !out || !world_min) return VR_ERR_INVALID_ARG;
    if (res <= 0 || res > 4096 || num_mips < 1 || num_mips > VR_NUM_MAX_MIPS || res % (8 << (num_mips - 1)) != 0 || !(voxel_size > 0.f)) return VR_ERR_INVALID_ARG;
    try {
        std::vector<float> g(density, density + (size_t)res * res * res);
        for (float& x : g) if (!(x >= 0.f) || vr::isinf_(x)) return VR_ERR_INVALID_ARG;
        vr_volume* v = new vr_volume();
        if (vr::build_volume(g, res, num_mips, world_min, voxel_size, fp16 != 0, v->v) != 0) { delete v; return VR_ERR_INVALID_ARG; }
        *out = v;
        return VR_OK;
    } catch (...) {
        return VR_ERR_OOM;
    }
}
int vr_volume_create_dense_signed(const float* values, int32_t res, const float world_min[3], float voxel_size, int32_t fp16, vr_volume** out) {
    if (!values || !out || !world_min) return VR_ERR_INVALID_ARG;
    if (res <= 0 || res > 4096 || res % 8 != 0 || !(voxel_size > 0.f)) return VR_ERR_INVALID_ARG;
    try {
        std::vector<float> g(values, values + (size_t)res * res * res);
        for (float& x : g) if (!(x == x) || vr::isinf_(x)) return VR_ERR_INVALID_ARG;
        vr_volume* v = new vr_volume();
        if (vr::build_signed_grid(g, res, world_min, voxel_size, fp16 != 0, v->v) != 0) { delete v; return VR_ERR_INVALID_ARG; }
        *out = v;
        return VR_OK;
    } catch (...) {
        return VR_ERR_OOM;
    }
}
static thread_local std::string g_vbxErr;
int vr_volume_load_vbx(const char* path, int32_t num_mips, int32_t flags, vr_volume** out) {
    g_vbxErr.clear();
    if (!path || !out || num_mips < 1 || num_mips > VR_NUM_MAX_MIPS || (flags & ~(VR_VBX_FP16 | VR_VBX_SIGNED))) { g_vbxErr = "invalid argument"; return VR_ERR_INVALID_ARG; }
    try {
        FILE* fp = fopen(path, "rb");
        if (!fp) { g_vbxErr = std::string("cannot open ") + path; return VR_ERR_INVALID_ARG; }
        std::vector<unsigned char> file;
        unsigned char buf[1 << 16];
        size_t k;
        while ((k = fread(buf, 1, sizeof(buf), fp)) > 0) file.insert(file.end(), buf, buf + k);
        fclose(fp);
        vr_volume* v = new vr_volume();
        if (vr::read_vbx(file, (flags & VR_VBX_SIGNED) ? 1 : num_mips, (flags & VR_VBX_FP16) != 0, (flags & VR_VBX_SIGNED) != 0, v->v, g_vbxErr) != 0) {
            delete v;
            return VR_ERR_INVALID_ARG;
        }
        *out = v;
        return VR_OK;
    } catch (...) {
        g_vbxErr = "out of host memory";
        return VR_ERR_OOM;
    }
}
int vr_volume_save_vbx(const vr_volume* v, const char* path) {
    g_vbxErr.clear();
    if (!v || !path) { g_vbxErr = "invalid argument"; return VR_ERR_INVALID_ARG; }
    try {
        std::vector<unsigned char> file;
        if (vr::write_vbx(v->v, file, g_vbxErr) != 0) return VR_ERR_INVALID_ARG;
        FILE* fp = fopen(path, "wb");
        if (!fp) { g_vbxErr = std::string("cannot create ") + path; return VR_ERR_INVALID_ARG; }
        const bool ok = fwrite(file.data(), 1, file.size(), fp) == file.size();
        fclose(fp);
        if (!ok) { g_vbxErr = "write failed"; return VR_ERR_INVALID_ARG; }
        return VR_OK;
    } catch (...) {
        g_vbxErr = "out of host memory";
        return VR_ERR_OOM;
    }
}
const char* vr_volume_vbx_error(void) { return g_vbxErr.c_str(); }
void vr_volume_destroy(vr_volume* v) { delete v; }
int vr_volume_compress_bc4(vr_volume* v) {
    if (!v) return VR_ERR_INVALID_ARG;
    for (int m = 0; m < v->v.num_mips && m < VR_NUM_MAX_MIPS; ++m) {
        if (m > 0) vr::compress_slot_bc4(v->v.slots[m], false);
        vr::compress_slot_bc4(v->v.slots[VR_NUM_MAX_MIPS + m], true);
    }
    v->v.bc4 = 1;
    return VR_OK;
}
int vr_volume_get_info(const vr_volume* v, vr_volume_info* info) {
    if (!v || !info) return VR_ERR_INVALID_ARG;
    memset(info, 0, sizeof(*info));
    info->num_mips = v->v.num_mips;
    info->res = v->v.res;
    info->voxel_size = v->v.voxel_size;
    info->supervoxel_diag = v->v.supervoxel_diag;
    info->fp16 = v->v.fp16;
    info->bc4 = v->v.bc4;
    for (int i = 0; i < 3; ++i) info->world_min[i] = v->v.world_min[i];
    int64_t bytes = 0;
    for (int s = 0; s < VR_NUM_SLOTS; ++s) {
        const vr::GridSlot& g = v->v.slots[s];
        info->num_bricks[s] = g.num_bricks;
        if (!g.valid) continue;
        bytes += (int64_t)g.root_child.size() * 4 + (int64_t)g.l1_vmin.size() * 4 + (int64_t)g.l1_child.size() * 4 +
                 (int64_t)g.brick_vmin.size() * 4 + (int64_t)g.brick_bounds.size() * 4 + (int64_t)g.brick_f32.size() * 4 +
                 (int64_t)g.brick_f16.size() * 2 + (int64_t)g.brick_bc4.size() * 8;
    }
    info->device_bytes = bytes;
    return VR_OK;
}
int vr_volume_get_slot(const vr_volume* v, int32_t slot, vr_grid_view* view) {
    if (!v || !view || slot < 0 || slot >= VR_NUM_SLOTS) return VR_ERR_INVALID_ARG;
    vr::slot_view(v->v.slots[slot], view);
    return VR_OK;
}

// ---- context ----
vr_context* vr_create(const vr_options* opts, int32_t width, int32_t height, int32_t* err) {
    vr_options d;
    if (!opts) { vr_options_default(&d); opts = &d; }
    std::string why;
    if (width <= 0 || height <= 0 || width > 16384 || height > 16384 || !options_valid(opts, why)) {
        if (err) *err = VR_ERR_INVALID_ARG;
        return nullptr;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { if (err) *err = VR_ERR_CUDA; return nullptr; }
    vr_context* c = new vr_context();
    c->opts = *opts;
    c->W = width; c->H = height;
    // persistent grids (walks, marches, network kernels) are sized by the SM count
    cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, dev);
    if (c->numSMs <= 0) c->numSMs = 1;
    for (auto& e : c->ev) cudaEventCreate(&e);
    if (dev_malloc(&c->status, sizeof(int)) != cudaSuccess) { delete c; if (err) *err = VR_ERR_OOM; return nullptr; }
    cudaMemset(c->status, 0, sizeof(int));
    c->scene.status = c->status;
    if (err) *err = VR_OK;
    return c;
}

void vr_destroy(vr_context* c) {
    if (!c) return;
    free_buffers(c);
    free_lp(c);
    free_split(c);
    free_net(c);
    for (void* p : c->sceneAllocs) cudaFree(p);
    for (void* p : c->envAllocs) cudaFree(p);
    for (void* p : c->emisAllocs) cudaFree(p);
    for (void* p : c->animAllocs) cudaFree(p);
    for (auto& e : c->ev) if (e) cudaEventDestroy(e);
    for (auto& v : c->pendingEv) for (auto e : v) cudaEventDestroy(e);
    for (auto e : c->freeEv) cudaEventDestroy(e);
    cudaFree(c->status);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->evFork) cudaEventDestroy(c->evFork);
    if (c->evJoin) cudaEventDestroy(c->evJoin);
    for (int i = 0; i < 2; ++i) {
        if (c->copyDone[i]) { cudaEventSynchronize(c->copyDone[i]); cudaEventDestroy(c->copyDone[i]); }
        if (c->rendered[i]) cudaEventDestroy(c->rendered[i]);
        cudaFree(c->hostStage[i]);
    }
    if (c->copyStream) cudaStreamDestroy(c->copyStream);
    delete c;
}

const char* vr_last_error(const vr_context* c) { return c ? c->err.c_str() : "null context"; }

int vr_set_options(vr_context* c, const vr_options* o) {
    if (!c || !o) return VR_ERR_INVALID_ARG;
    std::string why;
    if (!options_valid(o, why)) { c->err = why; return VR_ERR_INVALID_ARG; }
    c->opts = *o;
    c->optionsChanged = true;
    return VR_OK;
}
int vr_get_options(const vr_context* c, vr_options* o) {
    if (!c || !o) return VR_ERR_INVALID_ARG;
    *o = c->opts;
    return VR_OK;
}
int vr_resize(vr_context* c, int32_t w, int32_t h) {
    if (!c || w <= 0 || h <= 0 || w > 16384 || h > 16384) return VR_ERR_INVALID_ARG;
    c->W = w; c->H = h;
    c->optionsChanged = true;
    return VR_OK;
}

// ---- scene binding ----
int vr_volume_create_fire(const vr_procedural_desc* d, float t_min, float t_max, vr_volume** density, vr_volume** temperature) {
    if (!d || !density || !temperature) return VR_ERR_INVALID_ARG;
    if (d->res <= 0 || d->res > 4096 || d->num_mips < 1 || d->num_mips > VR_NUM_MAX_MIPS || d->octaves < 1 || d->octaves > 16) return VR_ERR_INVALID_ARG;
    if (d->res % (8 << (d->num_mips - 1)) != 0 || !(d->voxel_size > 0.f) || !(t_min >= 0.f) || !(t_max >= t_min)) return VR_ERR_INVALID_ARG;
    try {
        std::vector<float> g, t;
        vr::procedural_fire(*d, t_min, t_max, g, t);
        vr_volume* v = new vr_volume();
        vr_volume* w = new vr_volume();
        if (vr::build_volume(g, d->res, d->num_mips, d->world_min, d->voxel_size, d->fp16 != 0, v->v) != 0 ||
            vr::build_volume(t, d->res, 1, d->world_min, d->voxel_size, d->fp16 != 0, w->v) != 0) {
            delete v; delete w;
            return VR_ERR_INVALID_ARG;
        }
        *density = v;
        *temperature = w;
        return VR_OK;
    } catch (...) {
        return VR_ERR_OOM;
    }
}

void vr_blackbody_lut(float rgb[384]) {
    if (rgb) vr::blackbody_lut(rgb);
}

int vr_set_emission(vr_context* c, const vr_volume* temp, float le_scale, float cutoff, float scale, const float* lut) {
    if (!c) return VR_ERR_INVALID_ARG;
    for (void* p : c->emisAllocs) cudaFree(p);
    c->emisAllocs.clear();
    memset(&c->scene.tslot, 0, sizeof(c->scene.tslot));
    memset(&c->scene.ptslot, 0, sizeof(c->scene.ptslot));
    c->scene.hasEmission = 0;
    c->scene.lastHasEmission = 0;
    c->optionsChanged = true;
    if (!temp) return VR_OK;
    if (!(le_scale >= 0.f) || vr::isinf_(le_scale) || !(scale == scale) || !(cutoff == cutoff)) { c->err = "invalid emission parameters"; return VR_ERR_INVALID_ARG; }
    const vr::GridSlot& g = temp->v.slots[0];
    if (!g.valid) { c->err = "temperature volume has no mip 0"; return VR_ERR_INVALID_ARG; }
    auto up = [&](const void* src, size_t bytes) -> void* {
        void* p = nullptr;
        if (dev_malloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        c->emisAllocs.push_back(p);
        if (bytes) cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
        return p;
    };
    vrd::DevSlot& d = c->scene.tslot;
    c->emisParamsSet = true;
    d.valid = 1;
    d.res = g.res;
    d.bmaxf = (float)g.res;
    d.maxValue = g.max_value;
    memcpy(d.M, g.world_to_index, sizeof(d.M));
    d.root = (const int*)up(g.root_child.data(), g.root_child.size() * 4);
    d.l1vmin = (const int4*)up(g.l1_vmin.data(), g.l1_vmin.size() * 4);
    d.l1child = (const int*)up(g.l1_child.data(), g.l1_child.size() * 4);
    d.bvmin = (const int4*)up(g.brick_vmin.data(), g.brick_vmin.size() * 4);
    d.bounds = (const float4*)up(g.brick_bounds.data(), g.brick_bounds.size() * 4);
    if (!g.brick_f32.empty()) d.f32 = (const float*)up(g.brick_f32.data(), g.brick_f32.size() * 4);
    else if (!g.brick_f16.empty() || g.brick_bc4.empty()) d.f16 = (const __half*)up(g.brick_f16.data(), g.brick_f16.size() * 2);
    else { d.bc4 = (const uint2*)up(g.brick_bc4.data(), g.brick_bc4.size() * 8); d.bc4Scale = g.bc4_scale; }
    if (!d.root || !d.l1vmin || !d.l1child || !d.bvmin || !d.bounds || (!d.f32 && !d.f16 && !d.bc4)) {
        for (void* q : c->emisAllocs) cudaFree(q);
        c->emisAllocs.clear();
        memset(&c->scene.tslot, 0, sizeof(c->scene.tslot));
        c->err = "out of device memory (temperature)"; return VR_ERR_OOM;
    }
    float tab[384];
    if (lut) memcpy(tab, lut, sizeof(tab));
    else vr::blackbody_lut(tab);
    memcpy(c->scene.blackbody, tab, sizeof(tab));
    c->scene.leScale = le_scale;
    c->scene.tCutoff = cutoff;
    c->scene.tScale = scale;
    c->scene.hasEmission = 1;
    c->scene.ptslot = c->scene.tslot;          // a static grid is its own previous frame
    c->scene.lastHasEmission = 1;
    return VR_OK;
}

static void anim_clear(vr_context* c);

int vr_set_volume(vr_context* c, const vr_volume* vol, const vr_medium* m) {
    if (!c || !vol || !m) return VR_ERR_INVALID_ARG;
    anim_clear(c);
    if (!(m->sigma_s[0] + m->sigma_a[0] > 0.f)) { c->err = "sigma_t must be positive"; return VR_ERR_INVALID_ARG; }
    if (m->sigma_s[0] + m->sigma_a[0] != m->sigma_s[1] + m->sigma_a[1] || m->sigma_s[1] + m->sigma_a[1] != m->sigma_s[2] + m->sigma_a[2]) {
        c->err = "sigma_t must be grey (sigma_s + sigma_a equal on all channels)"; return VR_ERR_INVALID_ARG;
    }
    for (void* p : c->sceneAllocs) cudaFree(p);
    c->sceneAllocs.clear();
    const vr::Volume& v = vol->v;
    for (int s = 0; s < VR_NUM_SLOTS; ++s) {
        vrd::DevSlot& d = c->scene.slots[s];
        memset(&d, 0, sizeof(d));
        const vr::GridSlot& g = v.slots[s];
        if (!g.valid) continue;
        auto up = [&](const void* src, size_t bytes) -> void* {
            void* p = nullptr;
            if (dev_malloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
            c->sceneAllocs.push_back(p);
            if (bytes) cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
            return p;
        };
        d.valid = 1;
        d.res = g.res;
        d.bmaxf = (float)g.res;
        d.maxValue = g.max_value;
        memcpy(d.M, g.world_to_index, sizeof(d.M));
        d.root = (const int*)up(g.root_child.data(), g.root_child.size() * 4);
        d.l1vmin = (const int4*)up(g.l1_vmin.data(), g.l1_vmin.size() * 4);
        d.l1child = (const int*)up(g.l1_child.data(), g.l1_child.size() * 4);
        d.bvmin = (const int4*)up(g.brick_vmin.data(), g.brick_vmin.size() * 4);
        d.bounds = (const float4*)up(g.brick_bounds.data(), g.brick_bounds.size() * 4);
        if (!g.brick_f32.empty()) d.f32 = (const float*)up(g.brick_f32.data(), g.brick_f32.size() * 4);
        else if (!g.brick_f16.empty() || g.brick_bc4.empty()) d.f16 = (const __half*)up(g.brick_f16.data(), g.brick_f16.size() * 2);
        else { d.bc4 = (const uint2*)up(g.brick_bc4.data(), g.brick_bc4.size() * 8); d.bc4Scale = g.bc4_scale; }
        if (!d.root || !d.l1vmin || !d.l1child || !d.bvmin || !d.bounds || (!d.f32 && !d.f16 && !d.bc4)) {
            for (void* q : c->sceneAllocs) cudaFree(q);
            c->sceneAllocs.clear();
            memset(c->scene.slots, 0, sizeof(vrd::DevSlot) * VR_NUM_SLOTS);
            c->hasVolume = false;
            c->err = "out of device memory (volume)"; return VR_ERR_OOM;
        }
    }
    c->scene.sigma_s = mk3(m->sigma_s[0], m->sigma_s[1], m->sigma_s[2]);
    c->scene.sigma_a = mk3(m->sigma_a[0], m->sigma_a[1], m->sigma_a[2]);
    c->scene.sigma_t = m->sigma_s[0] + m->sigma_a[0];
    c->scene.g = m->g;
    c->scene.dscale = m->density_scale;
    c->scene.tStep = v.voxel_size;
    c->scene.superDiag = v.supervoxel_diag;
    c->scene.numMips = v.num_mips;
    c->numMips = v.num_mips;
    c->staticRes = v.res;
    for (int i = 0; i < 3; ++i) {
        c->netBmin[i] = v.world_min[i];
        c->netBinv[i] = 1.f / ((float)v.res * v.voxel_size);
    }
    memcpy(c->staticSlots, c->scene.slots, sizeof(c->staticSlots));
    c->hasVolume = true;
    c->optionsChanged = true;
    return VR_OK;
}

// ---- animated volumes ----
static bool upload_grid(const vr::GridSlot& g, vrd::DevSlot& d, std::vector<void*>& allocs) {
    memset(&d, 0, sizeof(d));
    if (!g.valid) return true;
    auto up = [&](const void* src, size_t bytes) -> void* {
        void* p = nullptr;
        if (dev_malloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        allocs.push_back(p);
        if (bytes) cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
        return p;
    };
    d.valid = 1;
    d.res = g.res;
    d.bmaxf = (float)g.res;
    d.maxValue = g.max_value;
    memcpy(d.M, g.world_to_index, sizeof(d.M));
    d.root = (const int*)up(g.root_child.data(), g.root_child.size() * 4);
    d.l1vmin = (const int4*)up(g.l1_vmin.data(), g.l1_vmin.size() * 4);
    d.l1child = (const int*)up(g.l1_child.data(), g.l1_child.size() * 4);
    d.bvmin = (const int4*)up(g.brick_vmin.data(), g.brick_vmin.size() * 4);
    d.bounds = (const float4*)up(g.brick_bounds.data(), g.brick_bounds.size() * 4);
    if (!g.brick_f32.empty()) d.f32 = (const float*)up(g.brick_f32.data(), g.brick_f32.size() * 4);
    else if (!g.brick_f16.empty() || g.brick_bc4.empty()) d.f16 = (const __half*)up(g.brick_f16.data(), g.brick_f16.size() * 2);
    else { d.bc4 = (const uint2*)up(g.brick_bc4.data(), g.brick_bc4.size() * 8); d.bc4Scale = g.bc4_scale; }
    return d.root && d.l1vmin && d.l1child && d.bvmin && d.bounds && (d.f32 || d.f16 || d.bc4);
}

static void anim_clear(vr_context* c) {
    if (c->anim.empty()) return;
    cudaDeviceSynchronize();                 // frames in flight may still read the grids
    for (void* p : c->animAllocs) cudaFree(p);
    c->animAllocs.clear();
    c->anim.clear();
    c->animId = -1;
    c->animTemp = c->animVel = false;
    memcpy(c->scene.slots, c->staticSlots, sizeof(c->staticSlots));
    memset(c->scene.slots + vrd::kPrevSlotOffset, 0, sizeof(vrd::DevSlot) * VR_NUM_SLOTS);
    memset(c->scene.vslot, 0, sizeof(c->scene.vslot));
    c->scene.hasAnimation = 0;
    c->scene.hasVelocity = 0;
    if (c->scene.hasEmission) c->scene.ptslot = c->scene.tslot;
    c->scene.lastHasEmission = c->scene.hasEmission;
}

// Scene::update (Scene.cpp:825-860): the next animation frame becomes current, the one before
// it supplies the previous-frame grids
static void anim_advance(vr_context* c) {
    if (c->anim.empty()) return;
    const int n = (int)c->anim.size();
    c->animId = (c->animId + 1) % n;
    const int cur = c->animId, prv = (cur + n - 1) % n;
    memcpy(c->scene.slots, c->anim[cur].slots, sizeof(c->anim[cur].slots));
    memcpy(c->scene.slots + vrd::kPrevSlotOffset, c->anim[prv].slots, sizeof(c->anim[prv].slots));
    c->scene.hasAnimation = 1;
    if (c->animTemp) {
        c->scene.tslot = c->anim[cur].temp;
        c->scene.ptslot = c->anim[prv].temp;
        c->scene.hasEmission = c->anim[cur].hasTemp;
        c->scene.lastHasEmission = c->anim[prv].hasTemp;
    }
    if (c->animVel) {
        memcpy(c->scene.vslot, c->anim[cur].vel, sizeof(c->scene.vslot));
        c->scene.hasVelocity = 1;
        c->scene.velocityScale = c->animVelScale;
    }
}

// frames share the grid layout and voxel size (the tracking step and the brick structure);
// each keeps its own world placement (its slots' world -> index transforms)
static bool same_layout(const vr::Volume& a, const vr::Volume& b) {
    return a.res == b.res && a.num_mips == b.num_mips && a.voxel_size == b.voxel_size;
}

int vr_set_animation(vr_context* c, const vr_volume* const* frames, int32_t n, const vr_volume* const* temperature,
                     const vr_volume* const* velocity, float velocity_scale) {
    if (!c || n < 0 || (n > 0 && !frames)) return VR_ERR_INVALID_ARG;
    if (!c->hasVolume) { c->err = "no volume bound (vr_set_volume)"; return VR_ERR_STATE; }
    anim_clear(c);
    c->optionsChanged = true;
    if (n == 0) return VR_OK;
    if (!(velocity_scale == velocity_scale) || vr::isinf_(velocity_scale)) { c->err = "invalid velocity scale"; return VR_ERR_INVALID_ARG; }
    const vr::Volume* base = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!frames[i]) { c->err = "null animation frame"; return VR_ERR_INVALID_ARG; }
        if (!base) base = &frames[i]->v;
        if (!same_layout(*base, frames[i]->v) || base->res != c->staticRes || base->num_mips != c->numMips ||
            base->voxel_size != c->scene.tStep) {
            c->err = "animation frames need the res, mip count and voxel size of the bound volume"; return VR_ERR_INVALID_ARG;
        }
        if (temperature && temperature[i] && !temperature[i]->v.slots[0].valid) { c->err = "temperature grid has no mip 0"; return VR_ERR_INVALID_ARG; }
        if (velocity)
            for (int k = 0; k < 3; ++k)
                if (!velocity[3 * i + k] || !velocity[3 * i + k]->v.slots[0].valid) { c->err = "velocity needs 3 grids per frame, each with mip 0"; return VR_ERR_INVALID_ARG; }
    }
    c->anim.resize(n);
    bool ok = true;
    for (int i = 0; i < n && ok; ++i) {
        vr_context::AnimFrame& f = c->anim[i];
        for (int sl = 0; sl < VR_NUM_SLOTS && ok; ++sl) ok = upload_grid(frames[i]->v.slots[sl], f.slots[sl], c->animAllocs);
        if (ok && temperature && temperature[i]) { ok = upload_grid(temperature[i]->v.slots[0], f.temp, c->animAllocs); f.hasTemp = true; }
        if (velocity)
            for (int k = 0; k < 3 && ok; ++k) ok = upload_grid(velocity[3 * i + k]->v.slots[0], f.vel[k], c->animAllocs);
    }
    if (!ok) {
        for (void* p : c->animAllocs) cudaFree(p);
        c->animAllocs.clear();
        c->anim.clear();
        c->err = "out of device memory (animation)";
        return VR_ERR_OOM;
    }
    c->animTemp = temperature != nullptr;
    c->animVel = velocity != nullptr;
    c->animVelScale = velocity_scale;
    if (c->animTemp && !c->emisParamsSet) {
        // Scene::addGVDBVolume defaults (Scene.h:481): LeScale 0.005, cutoff 1, scale 100
        c->scene.leScale = 0.005f;
        c->scene.tCutoff = 1.f;
        c->scene.tScale = 100.f;
        float tab[384];
        vr::blackbody_lut(tab);
        memcpy(c->scene.blackbody, tab, sizeof(tab));
    }
    c->animId = -1;
    return VR_OK;
}

int32_t vr_animation_frame(const vr_context* c) { return c ? c->animId : -1; }

void vr_debug_fail_allocation(int32_t n) { g_failAlloc.store(n < 0 ? -1 : (int64_t)n); }

int vr_set_lights(vr_context* c, const vr_point_light* lights, int32_t n, const vr_env_map* env) {
    if (!c || n < 0 || n > vrd::kMaxLights || (n > 0 && !lights)) { if (c) c->err = "at most 64 point lights"; return VR_ERR_INVALID_ARG; }
    c->scene.numLights = n;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) { c->scene.lightPos[i][k] = lights[i].pos[k]; c->scene.lightI[i][k] = lights[i].intensity[k]; }
    for (void* p : c->envAllocs) cudaFree(p);
    c->envAllocs.clear();
    c->scene.hasEnv = 0;
    c->scene.envRGB = nullptr;
    c->scene.imp = nullptr;
    if (env) {
        if (!env->rgb || env->width <= 0 || env->height <= 0) { c->err = "invalid environment map"; return VR_ERR_INVALID_ARG; }
        HostEnv& e = c->env;
        e.w = env->width; e.h = env->height;
        e.rgb.assign(env->rgb, env->rgb + (size_t)e.w * e.h * 3);
        build_importance(e);
        float *drgb = nullptr, *dimp = nullptr;
        if (dev_malloc(&drgb, e.rgb.size() * 4) != cudaSuccess || dev_malloc(&dimp, e.imp.size() * 4) != cudaSuccess) {
            cudaFree(drgb); cudaFree(dimp);
            c->optionsChanged = true;
            c->err = "out of device memory (env)"; return VR_ERR_OOM;
        }
        c->envAllocs.push_back(drgb); c->envAllocs.push_back(dimp);
        cudaMemcpy(drgb, e.rgb.data(), e.rgb.size() * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dimp, e.imp.data(), e.imp.size() * 4, cudaMemcpyHostToDevice);
        c->scene.envRGB = drgb;
        c->scene.envW = e.w; c->scene.envH = e.h;
        c->scene.envScale = mk3(env->scale[0], env->scale[1], env->scale[2]);
        memcpy(c->scene.envRot, env->rotation, sizeof(c->scene.envRot));
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) c->scene.envInv[i * 3 + j] = env->rotation[j * 3 + i];
        c->scene.imp = dimp;
        memcpy(c->scene.impOff, e.off, sizeof(e.off));
        c->scene.impDim = 512;
        c->scene.impBaseMip = 9;
        c->scene.hasEnv = 1;
    }
    c->optionsChanged = true;
    return VR_OK;
}

static void fill_sampling(vrd::SamplingOptions& s, uint32_t vm, uint32_t lm, int ls, int lmip, int vs, int vmip, int vlin, int llin,
                          float vts, float lts, const vr_options& o) {
    s.visibilityTrackingMethod = vm; s.lightingTrackingMethod = lm;
    s.lightSamples = ls; s.lightingMipLevel = lmip; s.visibilitySamples = vs; s.visibilityMipLevel = vmip;
    s.visibilityUseLinearSampler = vlin; s.lightingUseLinearSampler = llin;
    s.visibilityTStepScale = vts; s.lightingTStepScale = lts;
    s.useEnvironmentLights = o.mUseEnvironmentLights; s.useAnalyticLights = o.mUseAnalyticLights;
    // the VERTEX_REUSE define applies to paths with indirect vertices (VolumetricReSTIR.cpp:376-386)
    s.vertexReuseStartBounce = (o.mVertexReuse && o.mMaxBounces > 1) ? o.mVertexReuseStartBounce : -1;
}

static vrd::FrameParams frame_params(vr_context* c, const CamFrame& cam, int numTotalRounds) {
    const vr_options& o = c->opts;
    vrd::FrameParams P;
    memset(&P, 0, sizeof(P));
    P.W = c->W; P.H = c->H; P.N = c->W * c->H;
    P.maxBounces = o.mMaxBounces;
    P.frameCount = c->frameCount;
    P.numTotalRounds = numTotalRounds;
    P.noReuse = !o.mEnableSpatialReuse && !o.mEnableTemporalReuse;
    P.initialM = o.mInitialM;
    P.baselineSpp = o.mBaselineSamplePerPixel;
    P.useRR = o.mInitialUseRussianRoulette;
    P.useCoarser = o.mInitialUseCoarserGridForIndirectBounce;
    P.temporalEnabled = o.mEnableTemporalReuse && !o.mUseReference;
    P.isFirstFrame = c->temporalSampleAccumulated == 0;
    P.reprojMode = (int)o.mTemporalReprojectionMode;
    P.temporalTalbot = o.mTemporalMISMethod == VR_MIS_TALBOT;
    P.reprojMip = o.mTemporalReprojectionMipLevel;
    P.temporalMThreshold = o.mTemporalReuseMThreshold;
    P.spatialTalbot = o.mSpatialMISMethod == VR_MIS_TALBOT;
    P.spatialK = o.mSpatialSampleCount;
    P.spatialRounds = o.mSpatialReuseRounds;
    P.visualizeTr = o.mVisualizeTotalTransmittance;
    fill_sampling(P.initial, VR_TRACK_ANALYTIC, o.mInitialLightingTrackingMethod, o.mInitialLightSamples, o.mInitialLightingMipLevel, 1,
                  o.mInitialVisibilityUseLinearSampler ? o.mInitialBaseMipLevel : o.mInitialBaseMipLevel + VR_NUM_MAX_MIPS,
                  o.mInitialVisibilityUseLinearSampler != 0, o.mInitialLightingUseLinearSampler != 0, o.mInitialVisibilityTStepScale,
                  o.mInitialLightingTStepScale, o);
    fill_sampling(P.spatial, o.mSpatialVisibilityTrackingMethod, o.mSpatialLightingTrackingMethod, 1, o.mSpatialLightingMipLevel, 1,
                  o.mSpatialVisibilityMipLevel, o.mSpatialVisibilityUseLinearSampler != 0, o.mSpatialLightingUseLinearSampler != 0,
                  o.mSpatialVisibilityTStepScale, o.mSpatialLightingTStepScale, o);
    bool flA = o.mFinalLightTrackingMethod == VR_TRACK_ANALYTIC || o.mFinalLightTrackingMethod == VR_TRACK_RAY_MARCHING;
    bool fvA = o.mFinalVisibilityTrackingMethod == VR_TRACK_ANALYTIC || o.mFinalVisibilityTrackingMethod == VR_TRACK_RAY_MARCHING;
    fill_sampling(P.fin, o.mFinalVisibilityTrackingMethod, o.mFinalLightTrackingMethod, flA ? 1 : o.mFinalLightSamples, 0,
                  fvA ? 1 : o.mFinalVisibilitySamples, 0, 1, 1, o.mFinalTStepScale, o.mFinalTStepScale, o);
    P.camPos = cam.pos; P.camU = cam.U; P.camV = cam.V; P.camW = cam.W;
    P.prevPos = c->prev.pos; P.prevU = c->prev.U; P.prevV = c->prev.V; P.prevW = c->prev.W;
    memcpy(P.prevView, c->prev.view, sizeof(P.prevView));
    memcpy(P.prevProj, c->prev.proj, sizeof(P.prevProj));
    return P;
}

static int check_cuda(vr_context* c, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { c->err = std::string(what) + ": " + cudaGetErrorString(e); return VR_ERR_CUDA; }
    return VR_OK;
}

static int prepare_frame(vr_context* c, const vr_camera* cam) {
    if (!cam) return VR_ERR_INVALID_ARG;
    if (!c->hasVolume) { c->err = "no volume bound (vr_set_volume)"; return VR_ERR_STATE; }
    std::string why;
    if (!slots_present(c, why)) { c->err = why; return VR_ERR_INVALID_ARG; }
    if (c->opts.mUseAnalyticLights && c->scene.numLights == 0) { c->err = "mUseAnalyticLights needs at least one point light"; return VR_ERR_INVALID_ARG; }
    if (c->opts.mUseEnvironmentLights && !c->scene.hasEnv) { c->err = "mUseEnvironmentLights needs an environment map"; return VR_ERR_INVALID_ARG; }
    int r = alloc_buffers(c);
    if (r) return r;
    if (lp_active(c) && (r = lp_alloc(c))) return r;
    if (split_needed(c) && (r = split_alloc(c))) return r;
    if (c->optionsChanged) { c->frameCount = 0; c->temporalSampleAccumulated = 0; c->optionsChanged = false; }
    return VR_OK;
}

static int upload_scene(vr_context* c, cudaStream_t st) {
    cudaError_t e;
    switch (c->opts.mMaxBounces) {
        case 1: e = vrk::upload_scene_1(c->scene, st); break;
        case 2: e = vrk::upload_scene_2(c->scene, st); break;
        case 3: e = vrk::upload_scene_3(c->scene, st); break;
        default: e = vrk::upload_scene_4(c->scene, st); break;
    }
    if (e != cudaSuccess) { c->err = std::string("scene upload: ") + cudaGetErrorString(e); return VR_ERR_CUDA; }
    return VR_OK;
}

int vr_render_frame(vr_context* c, const vr_camera* cam, float* out_rgba, float* out_mvec, void* stream) {
    if (!c || !out_rgba) return VR_ERR_INVALID_ARG;
    int r = prepare_frame(c, cam);
    if (r) return r;
    anim_advance(c);
    c->scene.usePrevGrid = c->opts.mUsePrevVolumeForReproj != 0;
    cudaStream_t st = (cudaStream_t)stream;
    if ((r = upload_scene(c, st))) return r;
    const vr_options& o = c->opts;
    CamFrame cf = camera_frame(*cam, c->W, c->H);
    int numTotalRounds = (o.mEnableSpatialReuse ? o.mSpatialReuseRounds : 0) + o.mEnableTemporalReuse + 1 + 1;
    vrd::FrameParams P = frame_params(c, cf, numTotalRounds);
    vrd::FrameBuffers B;
    memset(&B, 0, sizeof(B));
    B.cur = c->res[0];
    B.sp[0] = c->res[0];
    B.sp[1] = c->res[1];
    B.hist = c->res[2];
    if (vertex_reuse(c)) {
        B.cur.pp = B.sp[0].pp = c->ppPlane[0];
        B.sp[1].pp = c->ppPlane[1];
        B.hist.pp = c->ppPlane[2];
    }
    B.featCur = c->feat[c->featCurIdx];
    B.featPrev = c->feat[c->featCurIdx ^ 1];
    B.color = o.mUseReference ? c->color : nullptr;
    B.out = (float4*)out_rgba;
    B.mvec = (float2*)out_mvec;
    c->nev = 0;
    c->launches = 0;
    c->d2h = 0;
    switch (o.mMaxBounces) {
        case 1: launch_frame_kernels<1>(c, P, B, st); break;
        case 2: launch_frame_kernels<2>(c, P, B, st); break;
        case 3: launch_frame_kernels<3>(c, P, B, st); break;
        default: launch_frame_kernels<4>(c, P, B, st); break;
    }
    if ((r = check_cuda(c, "frame kernels"))) return r;
    c->h2d = (int64_t)sizeof(vrd::DevScene) + (int64_t)c->launches * (int64_t)(sizeof(vrd::FrameParams) + sizeof(vrd::FrameBuffers)) +
             (o.mEnableSpatialReuse && !o.mUseReference ? (int64_t)o.mSpatialReuseRounds * (int64_t)sizeof(vrd::SpatialParams) : 0);
    if (!o.mUseReference && o.mEnableTemporalReuse) c->featCurIdx ^= 1;
    c->temporalSampleAccumulated = 1;
    c->prev = cf;
    c->frameCount++;
    if (c->hook) {
        c->hook(c->hookUser, out_rgba, out_mvec, c->W, c->H, stream);
        if ((r = check_cuda(c, "frame hook"))) return r;
    }
    return VR_OK;
}

int vr_set_frame_hook(vr_context* c, vr_frame_hook fn, void* user) {
    if (!c) return VR_ERR_INVALID_ARG;
    c->hook = fn;
    c->hookUser = fn ? user : nullptr;
    return VR_OK;
}

static int read_status(vr_context* c) {
    int status = 0;
    cudaMemcpy(&status, c->status, 4, cudaMemcpyDeviceToHost);
    if (status) {
        int zero = 0;
        cudaMemcpy(c->status, &zero, 4, cudaMemcpyHostToDevice);
        c->err = "a bounded device loop hit its iteration limit";
        return VR_ERR_LOOP_LIMIT;
    }
    return VR_OK;
}

int vr_render_frame_host_async(vr_context* c, const vr_camera* cam, float* out_rgba_host, void* stream) {
    if (!c || !out_rgba_host) return VR_ERR_INVALID_ARG;
    const size_t bytes = (size_t)c->W * c->H * 16;
    if (!c->copyStream) {
        if (cudaStreamCreateWithFlags(&c->copyStream, cudaStreamNonBlocking) != cudaSuccess) return check_cuda(c, "copy stream");
        for (int i = 0; i < 2; ++i) {
            cudaEventCreateWithFlags(&c->copyDone[i], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&c->rendered[i], cudaEventDisableTiming);
        }
    }
    const int i = c->hostIdx;
    if (c->copyPending[i]) {                       // the copy issued two calls ago
        if (cudaEventSynchronize(c->copyDone[i]) != cudaSuccess) return check_cuda(c, "host copy");
        c->copyPending[i] = false;
    }
    if (!c->hostStage[i] || c->hostStageBytes != bytes) {
        for (int k = 0; k < 2; ++k) {
            if (c->copyPending[k]) { cudaEventSynchronize(c->copyDone[k]); c->copyPending[k] = false; }
            cudaFree(c->hostStage[k]);
            c->hostStage[k] = nullptr;
        }
        for (int k = 0; k < 2; ++k)
            if (dev_malloc(&c->hostStage[k], bytes) != cudaSuccess) { c->err = "out of device memory (output)"; return VR_ERR_OOM; }
        c->hostStageBytes = bytes;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int r = vr_render_frame(c, cam, c->hostStage[i], nullptr, stream);
    if (r) return r;
    cudaEventRecord(c->rendered[i], st);
    cudaStreamWaitEvent(c->copyStream, c->rendered[i], 0);
    cudaMemcpyAsync(out_rgba_host, c->hostStage[i], bytes, cudaMemcpyDeviceToHost, c->copyStream);
    cudaEventRecord(c->copyDone[i], c->copyStream);
    c->copyPending[i] = true;
    c->d2h = (int64_t)bytes;
    c->hostIdx ^= 1;
    return check_cuda(c, "host copy");
}

int vr_host_frames_wait(vr_context* c) {
    if (!c) return VR_ERR_INVALID_ARG;
    for (int i = 0; i < 2; ++i)
        if (c->copyPending[i]) {
            if (cudaEventSynchronize(c->copyDone[i]) != cudaSuccess) return check_cuda(c, "host copy");
            c->copyPending[i] = false;
        }
    return read_status(c);
}

int vr_render_frame_host(vr_context* c, const vr_camera* cam, float* out_rgba_host, void* stream) {
    if (!c || !out_rgba_host) return VR_ERR_INVALID_ARG;
    size_t bytes = (size_t)c->W * c->H * 16;
    float* d = nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    static thread_local std::vector<std::pair<size_t, float*>> scratch;
    for (auto& s : scratch) if (s.first == bytes) d = s.second;
    if (!d) {
        if (dev_malloc(&d, bytes) != cudaSuccess) { c->err = "out of device memory (output)"; return VR_ERR_OOM; }
        scratch.push_back({bytes, d});
    }
    int r = vr_render_frame(c, cam, d, nullptr, stream);
    if (r) return r;
    cudaMemcpyAsync(out_rgba_host, d, bytes, cudaMemcpyDeviceToHost, st);
    c->d2h = (int64_t)bytes;
    if (cudaStreamSynchronize(st) != cudaSuccess) return check_cuda(c, "frame");
    int status = 0;
    cudaMemcpy(&status, c->status, 4, cudaMemcpyDeviceToHost);
    if (status) {
        int zero = 0;
        cudaMemcpy(c->status, &zero, 4, cudaMemcpyHostToDevice);
        c->err = "a bounded device loop hit its iteration limit";
        return VR_ERR_LOOP_LIMIT;
    }
    return VR_OK;
}

int vr_render_reference(vr_context* c, const vr_camera* cam, int32_t first_frame, int32_t num_frames, double* accum, void* stream) {
    if (!c || !accum || num_frames < 0) return VR_ERR_INVALID_ARG;
    int r = prepare_frame(c, cam);
    if (r) return r;
    cudaStream_t st = (cudaStream_t)stream;
    if ((r = upload_scene(c, st))) return r;
    const vr_options& o = c->opts;
    CamFrame cf = camera_frame(*cam, c->W, c->H);
    int numTotalRounds = (o.mEnableSpatialReuse ? o.mSpatialReuseRounds : 0) + o.mEnableTemporalReuse + 1 + 1;
    vrd::FrameParams P = frame_params(c, cf, numTotalRounds);
    dim3 grid((c->W + 7) / 8, (c->H + 15) / 16), block(128);
    // chunks of frames keep each launch short
    for (int f = 0; f < num_frames; f += 16) {
        int cnt = std::min(16, num_frames - f);
        switch (o.mMaxBounces) {
            case 1: vrk::launch_reference_1(P, first_frame + f, cnt, accum, grid, block, st); break;
            case 2: vrk::launch_reference_2(P, first_frame + f, cnt, accum, grid, block, st); break;
            case 3: vrk::launch_reference_3(P, first_frame + f, cnt, accum, grid, block, st); break;
            default: vrk::launch_reference_4(P, first_frame + f, cnt, accum, grid, block, st); break;
        }
    }
    return check_cuda(c, "reference");
}

// ---- exports ----
int32_t vr_reservoir_bytes(const vr_context* c) { return c ? (c->opts.mMaxBounces > 1 ? (vertex_reuse(c) ? 40 : 36) : 32) : 0; }

int vr_export_reservoirs(vr_context* c, int32_t which, void* host, size_t bytes) {
    if (!c || !host || which < 0 || which > 3) return VR_ERR_INVALID_ARG;
    size_t N = (size_t)c->W * c->H;
    int rb = vr_reservoir_bytes(c);
    if (bytes < N * rb) return VR_ERR_INVALID_ARG;
    if (!c->res[0].a) { c->err = "no frame rendered yet"; return VR_ERR_STATE; }
    int idx = which == 0 ? c->finalBuf : (which == 1 ? 2 : which - 2);
    std::vector<float4> a(N);
    std::vector<int4> b(N);
    cudaDeviceSynchronize();
    cudaMemcpy(a.data(), c->res[idx].a, N * 16, cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), c->res[idx].b, N * 16, cudaMemcpyDeviceToHost);
    std::vector<float> pp;
    if (vertex_reuse(c)) {
        pp.resize(N);
        cudaMemcpy(pp.data(), c->ppPlane[idx], N * 4, cudaMemcpyDeviceToHost);
    }
    int mb = c->opts.mMaxBounces;
    char* o = (char*)host;
    for (size_t i = 0; i < N; ++i) {
        vr_reservoir_aos r;
        r.runningSum = a[i].x; r.M = a[i].y; r.depth = a[i].z; r.p_y = a[i].w;
        memcpy(&r.lightUV[0], &b[i].x, 4); memcpy(&r.lightUV[1], &b[i].y, 4);
        r.lightID = b[i].z; r.sampledPixel = b[i].w;
        r.extraBounceStartId = (int32_t)(i * (size_t)(mb - 1));
        r.p_partial = pp.empty() ? 0.f : pp[i];
        memcpy(o + i * rb, &r, rb);
    }
    return check_cuda(c, "export");
}

int vr_export_extra_bounces(vr_context* c, int32_t which, float* host, size_t bytes) {
    if (!c || !host || which < 0 || which > 3) return VR_ERR_INVALID_ARG;
    size_t N = (size_t)c->W * c->H;
    int mb = c->opts.mMaxBounces;
    size_t ne = N * (size_t)std::max(mb - 1, 0);
    if (bytes < ne * 12) return VR_ERR_INVALID_ARG;
    if (ne == 0) return VR_OK;
    int idx = which == 0 ? c->finalBuf : (which == 1 ? 2 : which - 2);
    std::vector<float4> e(ne);
    cudaDeviceSynchronize();
    cudaMemcpy(e.data(), c->res[idx].extra, ne * 16, cudaMemcpyDeviceToHost);
    // device planes are b*N + pixel; the reference layout is pixel*(mb-1) + b
    for (size_t p = 0; p < N; ++p)
        for (int b = 0; b < mb - 1; ++b) {
            const float4& v = e[(size_t)b * N + p];
            float* d = host + (p * (mb - 1) + b) * 3;
            d[0] = v.x; d[1] = v.y; d[2] = v.z;
        }
    return check_cuda(c, "export extra");
}

int vr_export_features(vr_context* c, void* host, size_t bytes) {
    if (!c || !host) return VR_ERR_INVALID_ARG;
    size_t N = (size_t)c->W * c->H;
    if (bytes < N * 8) return VR_ERR_INVALID_ARG;
    if (!c->feat[0]) return VR_ERR_STATE;
    std::vector<float> f(N);
    cudaDeviceSynchronize();
    // the features of the last frame: the buffer before the end-of-frame swap
    bool swapped = !c->opts.mUseReference && c->opts.mEnableTemporalReuse;
    int idx = swapped ? (c->featCurIdx ^ 1) : c->featCurIdx;
    cudaMemcpy(f.data(), c->feat[idx], N * 4, cudaMemcpyDeviceToHost);
    int32_t* o = (int32_t*)host;
    for (size_t i = 0; i < N; ++i) { o[i * 2] = 1; memcpy(&o[i * 2 + 1], &f[i], 4); }
    return check_cuda(c, "export features");
}

int32_t vr_frame_count(const vr_context* c) { return c ? c->frameCount : -1; }

int vr_last_timings(const vr_context* c, float* ms, int32_t max_entries, int32_t* n) {
    if (!c || !ms || !n) return VR_ERR_INVALID_ARG;
    int k = 0;
    for (int i = 0; i + 1 < c->nev && k < max_entries; ++i) {
        cudaEventSynchronize(c->ev[i + 1]);
        float t = 0.f;
        cudaEventElapsedTime(&t, c->ev[i], c->ev[i + 1]);
        ms[k++] = t;
    }
    *n = k;
    return VR_OK;
}
int32_t vr_last_launch_count(const vr_context* c) { return c ? c->launches : 0; }

// frame events, plain: start, after the initial stage, after the spatial/final stage, end;
// learned target: start, after generate, after infer, after select, after the spatial/final
// stage, then the start and end of the training on the side stream.  Totals: 0 initial stage,
// 1 spatial/final stage, 2 training, 3 generate, 4 infer, 5 select
static void drain_events(vr_context* c) {
    for (auto& v : c->pendingEv) {
        for (cudaEvent_t e : v) cudaEventSynchronize(e);
        static const int plain[3][3] = {{0, 1, 0}, {1, 2, 1}, {2, 3, 2}};
        static const int learned[6][3] = {{0, 3, 0}, {3, 4, 1}, {5, 6, 2}, {0, 1, 3}, {1, 2, 4}, {2, 3, 5}};
        const int (*map)[3] = v.size() == 7 ? learned : plain;
        const int nm = v.size() == 7 ? 6 : (v.size() == 4 ? 3 : 0);
        for (int i = 0; i < nm; ++i) {
            float t = 0.f;
            cudaEventElapsedTime(&t, v[map[i][0]], v[map[i][1]]);
            c->totalMs[map[i][2]] += t;
        }
        c->totalFrames++;
        for (auto e : v) c->freeEv.push_back(e);
    }
    c->pendingEv.clear();
}
int vr_kernel_time_totals(vr_context* c, float* ms, int32_t max_entries, int32_t* frames, int32_t reset) {
    if (!c || !ms || !frames) return VR_ERR_INVALID_ARG;
    drain_events(c);
    for (int i = 0; i < max_entries && i < 8; ++i) ms[i] = (float)c->totalMs[i];
    *frames = c->totalFrames;
    if (reset) { for (double& t : c->totalMs) t = 0; c->totalFrames = 0; }
    return VR_OK;
}
// ---- learned target: network ----
int vr_net_get_params(vr_context* c, float* host) {
    if (!c || !host) return VR_ERR_INVALID_ARG;
    int r = net_ensure(c, 1);
    if (r) return r;
    if (cudaMemcpy(host, c->netW, lpn::kParams * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return check_cuda(c, "network export");
    return VR_OK;
}
int vr_net_set_params(vr_context* c, const float* host) {
    if (!c || !host) return VR_ERR_INVALID_ARG;
    for (int i = 0; i < lpn::kParams; ++i)
        if (!(host[i] == host[i]) || vr::isinf_(host[i])) { c->err = "network parameters must be finite"; return VR_ERR_INVALID_ARG; }
    int r = net_alloc(c, 1);
    if (r) return r;
    return net_upload(c, host);
}
int vr_net_infer(vr_context* c, const float* q, int32_t n, float* out, void* stream) {
    if (!c || n < 0 || (n > 0 && (!q || !out))) return VR_ERR_INVALID_ARG;
    int r = net_ensure(c, 1);
    if (r) return r;
    if (n == 0) return VR_OK;
    vrk::launch_net_infer(net_view(c), (const float4*)q, n, nullptr, out, nullptr, c->status, c->numSMs, (cudaStream_t)stream);
    return check_cuda(c, "network inference");
}
static int net_grad_common(vr_context* c, const float* samples, int32_t n, float* loss, bool update, float* grads) {
    if (!c || !samples || n <= 0 || n > (1 << 22)) return VR_ERR_INVALID_ARG;
    int r = net_ensure(c, (n + 127) / 128);
    if (r) return r;
    if (update) {
        lp_train_steps(c, (const float4*)samples, n, 0);
        c->launches -= 2;
    } else {
        vrk::launch_net_train(net_view(c), (const float4*)samples, n, c->netPart, c->netLossPart, c->status, 0);
        vrk::launch_net_reduce_adam(c->netPart, (n + 127) / 128, c->netLossPart, c->netW, c->netM, c->netV, c->netG, c->netScalar, c->netWbf,
                                    c->netBias, 0.f, 1.f, 1.f, nullptr, 0, 0);
    }
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) return check_cuda(c, "network training");
    if (loss) cudaMemcpy(loss, update ? c->stepLoss : c->netScalar, sizeof(float), cudaMemcpyDeviceToHost);
    if (grads) cudaMemcpy(grads, c->netG, lpn::kParams * sizeof(float), cudaMemcpyDeviceToHost);
    return check_cuda(c, "network training");
}
int vr_net_gradients(vr_context* c, const float* samples, int32_t n, float* grads, float* loss) {
    if (!grads) return VR_ERR_INVALID_ARG;
    return net_grad_common(c, samples, n, loss, false, grads);
}
int vr_net_train_step(vr_context* c, const float* samples, int32_t n, float* loss) {
    if (c && c->opts.mLearnedBatch < n) { c->err = "n exceeds mLearnedBatch"; return VR_ERR_INVALID_ARG; }
    if (c && c->stepLossCap < 1) {
        int r = net_alloc(c, (n + 127) / 128);
        if (r) return r;
        c->stepLoss = dalloc<float>(1);
        if (!c->stepLoss) return VR_ERR_OOM;
        c->stepLossCap = 1;
    }
    return net_grad_common(c, samples, n, loss, true, nullptr);
}
int vr_export_learned(vr_context* c, int32_t which, void* host, size_t bytes, int64_t* count) {
    if (!c || !count) return VR_ERR_INVALID_ARG;
    if (which == 4) {
        *count = 6;
        if (!host || bytes < 24) return VR_ERR_INVALID_ARG;
        float* f = (float*)host;
        for (int i = 0; i < 3; ++i) { f[i] = c->netBmin[i]; f[3 + i] = c->netBinv[i]; }
        return VR_OK;
    }
    if (!c->lpFrameDone) { c->err = "no learned-target frame rendered yet"; return VR_ERR_STATE; }
    if (cudaDeviceSynchronize() != cudaSuccess) return check_cuda(c, "export");
    const void* src = nullptr;
    size_t need = 0;
    if (which == 0) { *count = (int64_t)c->lpSlots; src = c->lp.T; need = c->lpSlots * sizeof(float); }
    else if (which == 1) {
        int qc = 0;
        cudaMemcpy(&qc, c->lp.qcount, sizeof(int), cudaMemcpyDeviceToHost);
        *count = std::min(qc, c->lp.qcapacity);
        need = (size_t)*count * 32;
        if (!host) return VR_OK;
        if (bytes < need) { c->err = "export buffer too small"; return VR_ERR_INVALID_ARG; }
        if (!*count) return VR_OK;
        float4* tmp = dalloc<float4>(2 * (size_t)*count);
        if (!tmp) { c->err = "out of device memory (export)"; return VR_ERR_OOM; }
#if !defined(VR_HOST_EMULATION)
        k_gather_queries<<<(int)((*count + 255) / 256), 256>>>(c->lp.query, c->lp.qlist, (int)*count, tmp);
#else
        for (int64_t k = 0; k < *count; ++k) { tmp[2 * k] = c->lp.query[2 * (size_t)c->lp.qlist[k]]; tmp[2 * k + 1] = c->lp.query[2 * (size_t)c->lp.qlist[k] + 1]; }
#endif
        cudaMemcpy(host, tmp, need, cudaMemcpyDeviceToHost);
        cudaFree(tmp);
        return check_cuda(c, "export");
    } else if (which == 2) { *count = c->lp.trainCount; src = c->lp.train; need = (size_t)c->lp.trainCount * 32; }
    else if (which == 3) { *count = c->lastSteps; src = c->stepLoss; need = (size_t)c->lastSteps * sizeof(float); }
    else return VR_ERR_INVALID_ARG;
    if (!host) return VR_OK;
    if (bytes < need) { c->err = "export buffer too small"; return VR_ERR_INVALID_ARG; }
    if (need && cudaMemcpy(host, src, need, cudaMemcpyDeviceToHost) != cudaSuccess) return check_cuda(c, "export");
    return VR_OK;
}

int vr_last_transfer_bytes(const vr_context* c, int64_t* h2d, int64_t* d2h) {
    if (!c || !h2d || !d2h) return VR_ERR_INVALID_ARG;
    *h2d = c->h2d;
    *d2h = c->d2h;
    return VR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// frame launch sequence (VolumetricReSTIR.cpp:499-762)
// ---------------------------------------------------------------------------------------
template <int MB>
static void launch_initial(const vrd::FrameParams& P, const vrd::FrameBuffers& B, dim3 g, dim3 b, cudaStream_t st) {
    if (MB == 1) vrk::launch_initial_1(P, B, g, b, st);
    else if (MB == 2) vrk::launch_initial_2(P, B, g, b, st);
    else if (MB == 3) vrk::launch_initial_3(P, B, g, b, st);
    else vrk::launch_initial_4(P, B, g, b, st);
}
template <int MB>
static void launch_spatial(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::SpatialParams& S, dim3 g, dim3 b,
                           const vrd::SpatialSplit* SS, int persistent, cudaStream_t st) {
    if (MB == 1) vrk::launch_spatial_1(P, B, S, g, b, SS, persistent, st);
    else if (MB == 2) vrk::launch_spatial_2(P, B, S, g, b, SS, persistent, st);
    else if (MB == 3) vrk::launch_spatial_3(P, B, S, g, b, SS, persistent, st);
    else vrk::launch_spatial_4(P, B, S, g, b, SS, persistent, st);
}
template <int MB>
static void launch_final(const vrd::FrameParams& P, const vrd::FrameBuffers& B, int wh, dim3 g, dim3 b, cudaStream_t st) {
    if (MB == 1) vrk::launch_final_1(P, B, wh, g, b, st);
    else if (MB == 2) vrk::launch_final_2(P, B, wh, g, b, st);
    else if (MB == 3) vrk::launch_final_3(P, B, wh, g, b, st);
    else vrk::launch_final_4(P, B, wh, g, b, st);
}

template <int MB>
static void launch_lp_bounce(const vrd::FrameParams& P, const vrd::LpBuffers& L, int bounce, int grid, cudaStream_t st) {
    // sort the queue by coherence key, then the bounce pass over the sorted copy
    if (MB == 1) { vrk::launch_lp_sort_1(L, bounce, grid, st); vrk::launch_lp_bounce_1(P, L, bounce, grid, 1, st); }
    else if (MB == 2) { vrk::launch_lp_sort_2(L, bounce, grid, st); vrk::launch_lp_bounce_2(P, L, bounce, grid, 1, st); }
    else if (MB == 3) { vrk::launch_lp_sort_3(L, bounce, grid, st); vrk::launch_lp_bounce_3(P, L, bounce, grid, 1, st); }
    else { vrk::launch_lp_sort_4(L, bounce, grid, st); vrk::launch_lp_bounce_4(P, L, bounce, grid, 1, st); }
}
template <int MB>
static void launch_lp_generate(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::LpBuffers& L, dim3 g, dim3 b, cudaStream_t st) {
    if (MB == 1) vrk::launch_lp_generate_1(P, B, L, g, b, st);
    else if (MB == 2) vrk::launch_lp_generate_2(P, B, L, g, b, st);
    else if (MB == 3) vrk::launch_lp_generate_3(P, B, L, g, b, st);
    else vrk::launch_lp_generate_4(P, B, L, g, b, st);
}
template <int MB>
static void launch_lp_select(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::LpBuffers& L, dim3 g, dim3 b, cudaStream_t st) {
    if (MB == 1) vrk::launch_lp_select_1(P, B, L, g, b, st);
    else if (MB == 2) vrk::launch_lp_select_2(P, B, L, g, b, st);
    else if (MB == 3) vrk::launch_lp_select_3(P, B, L, g, b, st);
    else vrk::launch_lp_select_4(P, B, L, g, b, st);
}
template <int MB>
static void launch_lp_train_gen(const vrd::FrameParams& P, const vrd::LpBuffers& L, uint32_t seed, cudaStream_t st) {
    if (MB == 1) vrk::launch_lp_train_gen_1(P, L, seed, st);
    else if (MB == 2) vrk::launch_lp_train_gen_2(P, L, seed, st);
    else if (MB == 3) vrk::launch_lp_train_gen_3(P, L, seed, st);
    else vrk::launch_lp_train_gen_4(P, L, seed, st);
}

// seed of the training-sample streams of a frame
static uint32_t lp_train_seed(uint32_t learnedSeed, int frameCount) { return 0x80000000u | ((learnedSeed * 0x9E3779B9u + (uint32_t)frameCount) & 0x7FFFFFFFu); }

// one Adam step per batch over the frame's fresh training samples
// ccTable (device, optional): the bias corrections of each step, [steps][2], instead of
// arguments computed here (graph replay)
static void lp_train_steps(vr_context* c, const float4* samples, int S, cudaStream_t st, const float* ccTable) {
    const vr_options& o = c->opts;
    const int Bt = std::max(1, std::min(o.mLearnedBatch, S));
    const int steps = std::max(1, S / Bt);
    const vrd::NetView nv = net_view(c);
    for (int k = 0; k < steps; ++k) {
        vrk::launch_net_train(nv, samples + 2 * (size_t)k * Bt, Bt, c->netPart, c->netLossPart, c->status, st);
        c->adamStep++;
        const float c1 = (float)(1.0 - std::pow(0.9, (double)c->adamStep));
        const float c2 = (float)(1.0 - std::pow(0.999, (double)c->adamStep));
        vrk::launch_net_reduce_adam(c->netPart, (Bt + 127) / 128, c->netLossPart, c->netW, c->netM, c->netV, c->netG, c->stepLoss + k,
                                    c->netWbf, c->netBias, o.mLearnedLearningRate, c1, c2, ccTable ? ccTable + 2 * k : nullptr, 1, st);
        c->launches += 2;
    }
    c->lastSteps = steps;
}

template <int MB>
static void launch_frame_kernels(vr_context* c, const vrd::FrameParams& P, vrd::FrameBuffers& B, cudaStream_t st) {
    const vr_options& o = c->opts;
    const int rows = c->blockThreads / 8;
    dim3 grid((c->W + 7) / 8, (c->H + rows - 1) / rows), block(c->blockThreads);
    std::vector<cudaEvent_t> frameEv;
    auto mark = [&]() {
        if (c->nev < 10) cudaEventRecord(c->ev[c->nev++], st);
        cudaEvent_t e;
        if (!c->freeEv.empty()) { e = c->freeEv.back(); c->freeEv.pop_back(); }
        else cudaEventCreate(&e);
        cudaEventRecord(e, st);
        frameEv.push_back(e);
    };
    auto rec = [&]() {
        cudaEvent_t e;
        if (!c->freeEv.empty()) { e = c->freeEv.back(); c->freeEv.pop_back(); }
        else cudaEventCreate(&e);
        cudaEventRecord(e, st);
        frameEv.push_back(e);
    };
    cudaEvent_t trainEv[2] = {nullptr, nullptr};
    mark();
    const bool lpOn = lp_active(c);
    if (lpOn) {
        cudaMemsetAsync(c->lp.qcount, 0, sizeof(int), st);
        cudaMemsetAsync(c->lp.pcount, 0, 16 * sizeof(int), st);
        for (int k = 0; k < 3; ++k) { c->lp.kmin[k] = c->netBmin[k]; c->lp.kinv[k] = c->netBinv[k]; }
        VR_RANGE("vr.generate");
        launch_lp_generate<MB>(P, B, c->lp, grid, block, st);
        for (int b = 1; b < MB; ++b) launch_lp_bounce<MB>(P, c->lp, b, c->numSMs * VR_KINIT_MIN_BLOCKS, st);
        c->launches += (P.initial.visibilityUseLinearSampler ? 4 : 5) * (MB - 1);
        VR_RANGE_END();
        rec();
        VR_RANGE("vr.infer");
        vrk::launch_net_infer(net_view(c), c->lp.query, c->lp.qcapacity, c->lp.qcount, c->lp.T, c->lp.qlist, c->status, c->numSMs, st);
        VR_RANGE_END();
        rec();
        VR_RANGE("vr.select");
        launch_lp_select<MB>(P, B, c->lp, grid, block, st);
        VR_RANGE_END();
        c->launches += 3;
        c->lpFrameDone = true;
        // online training of the network on this frame's own queries (used from the next frame
        // on), on the side stream, concurrent with the spatial pass
        if (o.mLearnedTrainSamples > 0) {
            if (!c->side) {
                cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
                cudaEventCreateWithFlags(&c->evFork, cudaEventDisableTiming);
                cudaEventCreateWithFlags(&c->evJoin, cudaEventDisableTiming);
            }
            cudaEventRecord(c->evFork, st);
            cudaStreamWaitEvent(c->side, c->evFork, 0);
            trainEv[0] = take_event(c);
            cudaEventRecord(trainEv[0], c->side);
            c->lp.targetMethod = o.mLearnedTargetMethod;
            launch_lp_train_gen<MB>(P, c->lp, lp_train_seed(o.mLearnedSeed, c->frameCount), c->side);
            c->launches++;
            VR_RANGE("vr.train");
            lp_train_steps(c, c->lp.train, o.mLearnedTrainSamples, c->side);
            VR_RANGE_END();
            trainEv[1] = take_event(c);
            cudaEventRecord(trainEv[1], c->side);
            cudaEventRecord(c->evJoin, c->side);
        } else {
            c->lastSteps = 0;
        }
    } else {
        VR_RANGE("vr.initial");
        launch_initial<MB>(P, B, grid, block, st);
        VR_RANGE_END();
        c->launches++;
    }
    mark();
    int totalRoundId = 0;
    bool temporal = !o.mUseReference && o.mEnableTemporalReuse;
    bool spatial = !o.mUseReference && o.mEnableSpatialReuse;
    size_t N = (size_t)c->W * c->H;
    if (temporal && !spatial) {
        // copyResource(temporal <- perPixel[0]) (VolumetricReSTIR.cpp:632-637)
        cudaMemcpyAsync(c->res[2].a, c->res[0].a, N * 16, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(c->res[2].b, c->res[0].b, N * 16, cudaMemcpyDeviceToDevice, st);
        if (o.mMaxBounces > 1)
            cudaMemcpyAsync(c->res[2].extra, c->res[0].extra, N * (size_t)(o.mMaxBounces - 1) * 16, cudaMemcpyDeviceToDevice, st);
    }
    if (spatial) {
        for (int r = 0; r < o.mSpatialReuseRounds; ++r) {
            vrd::SpatialParams S;
            memset(&S, 0, sizeof(S));
            S.in = totalRoundId % 2;
            S.out = (totalRoundId + 1) % 2;
            int roundOffset = o.mEnableTemporalReuse + 1;
            S.roundId = r;
            S.numRounds = o.mSpatialReuseRounds + roundOffset + 1;
            S.rid = r + roundOffset;
            S.last = r == o.mSpatialReuseRounds - 1;
            S.writeHistory = temporal;
            int r2 = ((o.mSpatialReuseRounds + 1) * c->frameCount + r) % 16;
            neighbor_offsets(o, r2, S.offs);
            VR_RANGE("vr.spatial");
            launch_spatial<MB>(P, B, S, grid, block, c->split.seg ? &c->split : nullptr, c->numSMs * VR_KINIT_MIN_BLOCKS, st);
            if (c->split.seg && vrd::spatialSplitEligible(P)) c->launches += 4;
            VR_RANGE_END();
            c->launches++;
            totalRoundId++;
            if (S.last) mark();
        }
    } else {
        VR_RANGE("vr.final");
        launch_final<MB>(P, B, 0, grid, block, st);
        VR_RANGE_END();
        c->launches++;
        mark();
    }
    c->finalBuf = totalRoundId % 2;
    if (lpOn) {
        if (trainEv[0]) {
            cudaStreamWaitEvent(st, c->evJoin, 0);      // the next frame infers with the new weights
            frameEv.push_back(trainEv[0]);
            frameEv.push_back(trainEv[1]);
        } else {
            rec();
            rec();
        }
    } else {
        rec();
    }
    c->pendingEv.push_back(frameEv);
    if (c->pendingEv.size() > 512) drain_events(c);
}

// ---------------------------------------------------------------------------------------
// self tests
// ---------------------------------------------------------------------------------------
#if !defined(VR_HOST_EMULATION)
__global__ void k_selftest_math(int op, const float* a, const float* b, float* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = a[i], y = b ? b[i] : 0.f, r = 0.f;
    switch (op) {
        case 0: r = vr::exp_(x); break;
        case 1: r = vr::log_(x); break;
        case 2: r = vr::sin_(x); break;
        case 3: r = vr::cos_(x); break;
        case 4: r = vr::atan2_(x, y); break;
        case 5: r = vr::acos_(x); break;
        case 6: r = vr::pow_(x, y); break;
        default: r = vr::sqrt_(x); break;
    }
    out[i] = r;
}
__global__ void k_selftest_rng(const uint32_t* cases, int n, int draws, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vr::Rng r = vr::rng_create(cases[i * 3], cases[i * 3 + 1], cases[i * 3 + 2]);
    for (int j = 0; j < draws; ++j) out[(size_t)i * draws + j] = vr::next1D(r);
}

extern "C" int vr_selftest_math(int32_t op, const float* a, const float* b, float* out, int32_t n) {
    if (!a || !out || n <= 0 || op < 0 || op > 7) return VR_ERR_INVALID_ARG;
    float *da, *db = nullptr, *dout;
    if (dev_malloc(&da, n * 4) != cudaSuccess) return VR_ERR_CUDA;
    dev_malloc(&dout, n * 4);
    cudaMemcpy(da, a, n * 4, cudaMemcpyHostToDevice);
    if (b) { dev_malloc(&db, n * 4); cudaMemcpy(db, b, n * 4, cudaMemcpyHostToDevice); }
    k_selftest_math<<<(n + 255) / 256, 256>>>(op, da, db, dout, n);
    cudaMemcpy(out, dout, n * 4, cudaMemcpyDeviceToHost);
    cudaFree(da); cudaFree(db); cudaFree(dout);
    return cudaGetLastError() == cudaSuccess ? VR_OK : VR_ERR_CUDA;
}
extern "C" int vr_selftest_rng(const uint32_t* cases, int32_t n, int32_t draws, float* out) {
    if (!cases || !out || n <= 0 || draws <= 0) return VR_ERR_INVALID_ARG;
    uint32_t* dc; float* dout;
    if (dev_malloc(&dc, (size_t)n * 12) != cudaSuccess) return VR_ERR_CUDA;
    dev_malloc(&dout, (size_t)n * draws * 4);
    cudaMemcpy(dc, cases, (size_t)n * 12, cudaMemcpyHostToDevice);
    k_selftest_rng<<<(n + 127) / 128, 128>>>(dc, n, draws, dout);
    cudaMemcpy(out, dout, (size_t)n * draws * 4, cudaMemcpyDeviceToHost);
    cudaFree(dc); cudaFree(dout);
    return cudaGetLastError() == cudaSuccess ? VR_OK : VR_ERR_CUDA;
}
#endif  // !VR_HOST_EMULATION

// ---------------------------------------------------------------------------------------
// checkpoint / resume of the history (all device buffers + frame counter + previous camera)
// ---------------------------------------------------------------------------------------
namespace {
struct StateHeader {
    uint32_t magic, version;
    int32_t W, H, maxBounces, frameCount, temporalSampleAccumulated, featCurIdx, finalBuf, optionsChanged;
    CamFrame prev;
};
constexpr uint32_t kStateMagic = 0x56525354u;   // "VRST"
}
extern "C" int64_t vr_state_bytes(const vr_context* c) {
    if (!c) return 0;
    int64_t N = (int64_t)c->W * c->H;
    int64_t ne = N * std::max(c->opts.mMaxBounces - 1, 1);
    return (int64_t)sizeof(StateHeader) + 3 * (N * 32 + ne * 16) + 2 * N * 4 + N * 16 + (vertex_reuse(c) ? 3 * N * 4 : 0);
}
extern "C" int vr_export_state(vr_context* c, void* host, size_t bytes) {
    if (!c || !host || (int64_t)bytes < vr_state_bytes(c)) return VR_ERR_INVALID_ARG;
    int r = alloc_buffers(c);
    if (r) return r;
    size_t N = (size_t)c->W * c->H, ne = N * (size_t)std::max(c->opts.mMaxBounces - 1, 1);
    StateHeader h{kStateMagic, 1, c->W, c->H, c->opts.mMaxBounces, c->frameCount, c->temporalSampleAccumulated,
                  c->featCurIdx, c->finalBuf, c->optionsChanged ? 1 : 0, c->prev};
    char* p = (char*)host;
    memcpy(p, &h, sizeof(h)); p += sizeof(h);
    cudaDeviceSynchronize();
    for (int i = 0; i < 3; ++i) {
        cudaMemcpy(p, c->res[i].a, N * 16, cudaMemcpyDeviceToHost); p += N * 16;
        cudaMemcpy(p, c->res[i].b, N * 16, cudaMemcpyDeviceToHost); p += N * 16;
        cudaMemcpy(p, c->res[i].extra, ne * 16, cudaMemcpyDeviceToHost); p += ne * 16;
    }
    for (int i = 0; i < 2; ++i) { cudaMemcpy(p, c->feat[i], N * 4, cudaMemcpyDeviceToHost); p += N * 4; }
    cudaMemcpy(p, c->color, N * 16, cudaMemcpyDeviceToHost); p += N * 16;
    if (vertex_reuse(c))
        for (int i = 0; i < 3; ++i) { cudaMemcpy(p, c->ppPlane[i], N * 4, cudaMemcpyDeviceToHost); p += N * 4; }
    return check_cuda(c, "export state");
}
extern "C" int vr_import_state(vr_context* c, const void* host, size_t bytes) {
    if (!c || !host || (int64_t)bytes < (int64_t)sizeof(StateHeader)) return VR_ERR_INVALID_ARG;
    StateHeader h;
    memcpy(&h, host, sizeof(h));
    if (h.magic != kStateMagic || h.version != 1 || h.W != c->W || h.H != c->H || h.maxBounces != c->opts.mMaxBounces) {
        c->err = "state blob does not match this context (size or max path length)";
        return VR_ERR_INVALID_ARG;
    }
    if ((int64_t)bytes < vr_state_bytes(c)) return VR_ERR_INVALID_ARG;
    int r = alloc_buffers(c);
    if (r) return r;
    size_t N = (size_t)c->W * c->H, ne = N * (size_t)std::max(c->opts.mMaxBounces - 1, 1);
    const char* p = (const char*)host + sizeof(h);
    for (int i = 0; i < 3; ++i) {
        cudaMemcpy(c->res[i].a, p, N * 16, cudaMemcpyHostToDevice); p += N * 16;
        cudaMemcpy(c->res[i].b, p, N * 16, cudaMemcpyHostToDevice); p += N * 16;
        cudaMemcpy(c->res[i].extra, p, ne * 16, cudaMemcpyHostToDevice); p += ne * 16;
    }
    for (int i = 0; i < 2; ++i) { cudaMemcpy(c->feat[i], p, N * 4, cudaMemcpyHostToDevice); p += N * 4; }
    cudaMemcpy(c->color, p, N * 16, cudaMemcpyHostToDevice); p += N * 16;
    if (vertex_reuse(c))
        for (int i = 0; i < 3; ++i) { cudaMemcpy(c->ppPlane[i], p, N * 4, cudaMemcpyHostToDevice); p += N * 4; }
    c->frameCount = h.frameCount;
    c->temporalSampleAccumulated = h.temporalSampleAccumulated;
    c->featCurIdx = h.featCurIdx;
    c->finalBuf = h.finalBuf;
    c->optionsChanged = h.optionsChanged != 0;
    c->prev = h.prev;
    return check_cuda(c, "import state");
}

// ---------------------------------------------------------------------------------------
// support for the allocation-free frame entry point (noalloc.cu): validation and launch
// parameters from a context, without touching its buffers, counters or history
// ---------------------------------------------------------------------------------------
#include "vr_noalloc.h"
namespace vrk {
int noalloc_prepare(vr_context* c, const vr_camera* cam, int32_t frame_index, NoAllocFrame* f) {
    if (!cam || !f) { c->err = "null camera or frame"; return VR_ERR_INVALID_ARG; }
    if (!c->hasVolume) { c->err = "no volume bound (vr_set_volume)"; return VR_ERR_STATE; }
    const vr_options& o = c->opts;
    if (o.mEnableTemporalReuse || o.mUseReference) {
        c->err = "vr_render_frame_noalloc renders frames without history: disable mEnableTemporalReuse and mUseReference";
        return VR_ERR_INVALID_ARG;
    }
    if (o.mMaxBounces > kNoAllocMaxBounces) { c->err = "vr_render_frame_noalloc supports mMaxBounces <= 2"; return VR_ERR_INVALID_ARG; }
    if (vertex_reuse(c)) { c->err = "vr_render_frame_noalloc does not keep p_partial: disable mVertexReuse"; return VR_ERR_INVALID_ARG; }
    if (lp_active(c)) {
        // the learned target needs its vertex records, queries and network buffers, which this
        // entry point has no room for: refuse rather than render the plain form silently
        c->err = "vr_render_frame_noalloc renders the plain target only: disable mUseLearnedPHat";
        return VR_ERR_INVALID_ARG;
    }
    if ((int64_t)c->W * c->H > kNoAllocMaxPixels) {
        c->err = "vr_render_frame_noalloc supports at most 65536 pixels (e.g. 256x256); its scratch is a fixed static buffer";
        return VR_ERR_INVALID_ARG;
    }
    if (frame_index < 0) { c->err = "frame_index must be >= 0"; return VR_ERR_INVALID_ARG; }
    if (!c->anim.empty()) { c->err = "vr_render_frame_noalloc does not play animated volumes"; return VR_ERR_INVALID_ARG; }
    std::string why;
    if (!slots_present(c, why)) { c->err = why; return VR_ERR_INVALID_ARG; }
    if (o.mUseAnalyticLights && c->scene.numLights == 0) { c->err = "mUseAnalyticLights needs at least one point light"; return VR_ERR_INVALID_ARG; }
    if (o.mUseEnvironmentLights && !c->scene.hasEnv) { c->err = "mUseEnvironmentLights needs an environment map"; return VR_ERR_INVALID_ARG; }
    CamFrame cf = camera_frame(*cam, c->W, c->H);
    int numTotalRounds = (o.mEnableSpatialReuse ? o.mSpatialReuseRounds : 0) + 0 + 1 + 1;
    f->P = frame_params(c, cf, numTotalRounds);
    f->P.frameCount = frame_index;
    f->P.isFirstFrame = 1;
    f->P.temporalEnabled = 0;
    f->scene = &c->scene;
    f->W = c->W; f->H = c->H;
    f->maxBounces = o.mMaxBounces;
    f->spatial = o.mEnableSpatialReuse;
    f->rounds = o.mEnableSpatialReuse ? o.mSpatialReuseRounds : 0;
    for (int r = 0; r < f->rounds; ++r) {
        vrd::SpatialParams& S = f->S[r];
        memset(&S, 0, sizeof(S));
        S.in = r % 2;
        S.out = (r + 1) % 2;
        S.roundId = r;
        S.numRounds = o.mSpatialReuseRounds + 1 + 1;
        S.rid = r + 1;
        S.last = r == o.mSpatialReuseRounds - 1;
        S.writeHistory = 0;
        neighbor_offsets(o, ((o.mSpatialReuseRounds + 1) * frame_index + r) % 16, S.offs);
    }
    return VR_OK;
}
void noalloc_error(vr_context* c, const char* msg) { c->err = msg; }
}  // namespace vrk

// ---------------------------------------------------------------------------------------
// batches: many contexts rendered together by the persistent batched kernels (batch.cu), with
// the launch sequence captured once into a CUDA graph and an autotuned launch shape
// ---------------------------------------------------------------------------------------
#include "vr_batch.h"

namespace vrk {
#define VR_BDECL(MB)                                                                      \
    void launch_batch_pass_##MB(const vrd::BatchLaunch&, int, int, int, cudaStream_t);  \
    void launch_batch_train_gen_##MB(const vrd::BatchLaunch&, int, cudaStream_t);        \
    void launch_batch_lp_bounce_##MB(const vrd::BatchLaunch&, int, int, int, cudaStream_t); \
    void launch_batch_split_march_##MB(const vrd::BatchLaunch&, int, cudaStream_t);      \
    void launch_batch_split_reset_##MB(const vrd::BatchLaunch&, cudaStream_t);          \
    void launch_batch_walk_all_##MB(const vrd::BatchLaunch&, int, int, cudaStream_t);     \
    void launch_batch_vertex0_##MB(const vrd::BatchLaunch&, int, cudaStream_t);
VR_BDECL(1) VR_BDECL(2) VR_BDECL(3) VR_BDECL(4)
#undef VR_BDECL
}  // namespace vrk

struct vr_batch {
    std::vector<vr_context*> ctx;
    int MB = 0, temporal = 0, spatial = 0, rounds = 0;
    int tileW = 8, tileH = 16, blocksPerSM = 5, numSMs = 1;
    // device copy of the per-frame data (instances, scenes, Adam bias corrections) and its
    // pinned staging buffer: one host-to-device copy per frame
    unsigned char* dData = nullptr;
    unsigned char* hStage = nullptr;
    size_t dataBytes = 0;
    cudaEvent_t frameDone = nullptr;
    bool pendingFrame = false;
    // the graph is captured on and launched into a stream of its own, ordered after and before
    // the caller's stream by events (the legacy default stream cannot be captured)
    cudaStream_t gstream = nullptr;
    cudaEvent_t evIn = nullptr, evOut = nullptr;
    // the training steps run on a stream of their own, forked after the select pass and joined
    // at the end of the frame, concurrent with the spatial passes
    cudaStream_t tstream = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    // graph
    bool useGraph = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<int64_t> sig;
    int launches = 0, trainLaunches = 0;
    std::string err;
    // per-frame host state
    std::vector<CamFrame> cfs;
    std::vector<int> steps;
    std::vector<size_t> ccOff;
};

static void batch_drop_graph(vr_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->sig.clear();
}

template <int MB>
static void batch_pass(const vr_batch* b, const vrd::BatchLaunch& BL, int pass, cudaStream_t st) {
    const int nsm = std::max(1, b->numSMs), bps = std::max(1, b->blocksPerSM);
    if (MB == 1) vrk::launch_batch_pass_1(BL, pass, nsm, bps, st);
    else if (MB == 2) vrk::launch_batch_pass_2(BL, pass, nsm, bps, st);
    else if (MB == 3) vrk::launch_batch_pass_3(BL, pass, nsm, bps, st);
    else vrk::launch_batch_pass_4(BL, pass, nsm, bps, st);
}
template <int MB>
static void batch_lp_bounce(const vrd::BatchLaunch& BL, int inst, int bounce, int grid, cudaStream_t st) {
    if (MB == 1) vrk::launch_batch_lp_bounce_1(BL, inst, bounce, grid, st);
    else if (MB == 2) vrk::launch_batch_lp_bounce_2(BL, inst, bounce, grid, st);
    else if (MB == 3) vrk::launch_batch_lp_bounce_3(BL, inst, bounce, grid, st);
    else vrk::launch_batch_lp_bounce_4(BL, inst, bounce, grid, st);
}
template <int MB>
static void batch_split_march(const vrd::BatchLaunch& BL, int grid, cudaStream_t st) {
    if (MB == 1) vrk::launch_batch_split_march_1(BL, grid, st);
    else if (MB == 2) vrk::launch_batch_split_march_2(BL, grid, st);
    else if (MB == 3) vrk::launch_batch_split_march_3(BL, grid, st);
    else vrk::launch_batch_split_march_4(BL, grid, st);
}
template <int MB>
static void batch_walk_all(const vrd::BatchLaunch& BL, int bounce, int grid, cudaStream_t st) {
    if (MB == 1) vrk::launch_batch_walk_all_1(BL, bounce, grid, st);
    else if (MB == 2) vrk::launch_batch_walk_all_2(BL, bounce, grid, st);
    else if (MB == 3) vrk::launch_batch_walk_all_3(BL, bounce, grid, st);
    else vrk::launch_batch_walk_all_4(BL, bounce, grid, st);
}
template <int MB>
static void batch_vertex0(const vrd::BatchLaunch& BL, int grid, cudaStream_t st) {
    if (MB == 1) vrk::launch_batch_vertex0_1(BL, grid, st);
    else if (MB == 2) vrk::launch_batch_vertex0_2(BL, grid, st);
    else if (MB == 3) vrk::launch_batch_vertex0_3(BL, grid, st);
    else vrk::launch_batch_vertex0_4(BL, grid, st);
}
template <int MB>
static void batch_split_reset(const vrd::BatchLaunch& BL, cudaStream_t st) {
    if (MB == 1) vrk::launch_batch_split_reset_1(BL, st);
    else if (MB == 2) vrk::launch_batch_split_reset_2(BL, st);
    else if (MB == 3) vrk::launch_batch_split_reset_3(BL, st);
    else vrk::launch_batch_split_reset_4(BL, st);
}
template <int MB>
static void batch_train_gen(const vrd::BatchLaunch& BL, int grid, cudaStream_t st) {
    if (MB == 1) vrk::launch_batch_train_gen_1(BL, grid, st);
    else if (MB == 2) vrk::launch_batch_train_gen_2(BL, grid, st);
    else if (MB == 3) vrk::launch_batch_train_gen_3(BL, grid, st);
    else vrk::launch_batch_train_gen_4(BL, grid, st);
}

// host side of a batch frame: prepares every context, fills the staging buffer and returns the
// launch descriptor and the signature of the launch sequence (what a captured graph depends on)
static int batch_prepare(vr_batch* b, const vr_camera* cams, float* const* outs, vrd::BatchLaunch& BL, std::vector<int64_t>& sig) {
    const int n = (int)b->ctx.size();
    if (b->pendingFrame) { cudaEventSynchronize(b->frameDone); b->pendingFrame = false; }
    for (int i = 0; i < n; ++i) {
        vr_context* c = b->ctx[i];
        if (!outs[i]) { b->err = "null output buffer"; return VR_ERR_INVALID_ARG; }
        int r = prepare_frame(c, &cams[i]);
        if (r) { b->err = "instance " + std::to_string(i) + ": " + c->err; return r; }
        if (c->opts.mMaxBounces != b->MB || c->opts.mEnableTemporalReuse != b->temporal || c->opts.mEnableSpatialReuse != b->spatial ||
            (b->spatial && c->opts.mSpatialReuseRounds != b->rounds) || c->opts.mUseReference) {
            b->err = "instance " + std::to_string(i) + ": options no longer match the batch";
            return VR_ERR_STATE;
        }
    }
    // staging layout: instances, scenes, Adam tables
    b->steps.assign(n, 0);
    b->ccOff.assign(n, 0);
    size_t ccFloats = 0;
    for (int i = 0; i < n; ++i) {
        vr_context* c = b->ctx[i];
        if (lp_active(c) && c->opts.mLearnedTrainSamples > 0) {
            const int S = c->opts.mLearnedTrainSamples;
            b->steps[i] = std::max(1, S / std::max(1, std::min(c->opts.mLearnedBatch, S)));
            b->ccOff[i] = ccFloats;
            ccFloats += 2 * (size_t)b->steps[i];
        }
    }
    const size_t instBytes = sizeof(vrd::BatchInstance) * n, sceneBytes = sizeof(vrd::DevScene) * n;
    const size_t need = instBytes + sceneBytes + ccFloats * sizeof(float);
    if (need > b->dataBytes) {
        batch_drop_graph(b);
        cudaFree(b->dData);
        cudaFreeHost(b->hStage);
        b->dData = nullptr; b->hStage = nullptr; b->dataBytes = 0;
        if (dev_malloc(&b->dData, need) != cudaSuccess || cudaMallocHost(&b->hStage, need) != cudaSuccess) {
            b->err = "out of memory (batch descriptors)";
            return VR_ERR_OOM;
        }
        b->dataBytes = need;
    }
    vrd::BatchInstance* hInst = (vrd::BatchInstance*)b->hStage;
    vrd::DevScene* hScene = (vrd::DevScene*)(b->hStage + instBytes);
    float* hCC = (float*)(b->hStage + instBytes + sceneBytes);
    const vrd::DevScene* dScene = (const vrd::DevScene*)(b->dData + instBytes);
    b->cfs.resize(n);
    int tiles = 0, chunks = 0, cchunks = 0;
    sig.clear();
    sig.push_back(n); sig.push_back(b->tileW); sig.push_back(b->blocksPerSM); sig.push_back((int64_t)(size_t)b->dData);
    for (int i = 0; i < n; ++i) {
        vr_context* c = b->ctx[i];
        const vr_options& o = c->opts;
        vrd::BatchInstance& I = hInst[i];
        memset(&I, 0, sizeof(I));
        const CamFrame cf = camera_frame(cams[i], c->W, c->H);
        b->cfs[i] = cf;
        const int numTotalRounds = (o.mEnableSpatialReuse ? o.mSpatialReuseRounds : 0) + o.mEnableTemporalReuse + 1 + 1;
        I.P = frame_params(c, cf, numTotalRounds);
        I.B.cur = c->res[0]; I.B.sp[0] = c->res[0]; I.B.sp[1] = c->res[1]; I.B.hist = c->res[2];
        I.B.featCur = c->feat[c->featCurIdx];
        I.B.featPrev = c->feat[c->featCurIdx ^ 1];
        I.B.color = nullptr;
        I.B.out = (float4*)outs[i];
        I.B.mvec = nullptr;
        I.learned = lp_active(c) ? 1 : 0;
        I.walk = I.learned && !o.mInitialVisibilityUseLinearSampler ? 1 : 0;
        if (I.learned) {
            c->lp.targetMethod = o.mLearnedTargetMethod;
            I.L = c->lp;
            I.trainSeed = lp_train_seed(o.mLearnedSeed, c->frameCount);
        }
        I.spatialRounds = o.mEnableSpatialReuse ? o.mSpatialReuseRounds : 0;
        // the split rounds where the single-instance frame takes them (the same result)
        I.split = I.spatialRounds > 0 && c->split.seg && vrd::spatialSplitEligible(I.P) ? 1 : 0;
        if (I.split) I.SS = c->split;
        int totalRoundId = 0;
        for (int r = 0; r < I.spatialRounds; ++r) {
            vrd::SpatialParams& S = I.S[r];
            S.in = totalRoundId % 2;
            S.out = (totalRoundId + 1) % 2;
            const int roundOffset = o.mEnableTemporalReuse + 1;
            S.roundId = r;
            S.numRounds = o.mSpatialReuseRounds + roundOffset + 1;
            S.rid = r + roundOffset;
            S.last = r == o.mSpatialReuseRounds - 1;
            S.writeHistory = o.mEnableTemporalReuse;
            neighbor_offsets(o, ((o.mSpatialReuseRounds + 1) * c->frameCount + r) % 16, S.offs);
            totalRoundId++;
        }
        I.scene = dScene + i;
        hScene[i] = c->scene;
        I.tilesX = (c->W + b->tileW - 1) / b->tileW;
        I.tileStart = tiles;
        tiles += I.tilesX * ((c->H + b->tileH - 1) / b->tileH);
        I.trainChunkStart = chunks;
        if (I.learned && o.mLearnedTrainSamples > 0) chunks += (o.mLearnedTrainSamples + 127) / 128;
        I.candChunkStart = cchunks;
        if (I.learned) cchunks += (int)(((int64_t)o.mInitialM * c->W * c->H + 127) / 128);
        for (int k = 0; k < b->steps[i]; ++k) {
            const double t = (double)(c->adamStep + k + 1);
            hCC[b->ccOff[i] + 2 * k] = (float)(1.0 - std::pow(0.9, t));
            hCC[b->ccOff[i] + 2 * k + 1] = (float)(1.0 - std::pow(0.999, t));
        }
        const int64_t s[] = {c->W, c->H, o.mInitialM, I.learned, I.walk, I.spatialRounds, I.split, o.mLearnedTrainSamples, o.mLearnedBatch, b->steps[i],
                             (int64_t)(size_t)c->res[0].a, (int64_t)(size_t)c->lp.vrecA, (int64_t)(size_t)c->lp.train,
                             (int64_t)(size_t)c->netW, (int64_t)(size_t)c->netPart};
        sig.insert(sig.end(), s, s + sizeof(s) / sizeof(s[0]));
    }
    BL.inst = (const vrd::BatchInstance*)b->dData;
    BL.numInst = n;
    BL.totalTiles = tiles;
    BL.tileW = b->tileW;
    BL.tileH = b->tileH;
    BL.round = 0;
    BL.trainChunks = chunks;
    BL.candChunks = cchunks;
    return VR_OK;
}

template <int MB>
static void batch_launch(vr_batch* b, vrd::BatchLaunch BL, cudaStream_t st) {
    const int n = (int)b->ctx.size();
    const size_t instBytes = sizeof(vrd::BatchInstance) * n, sceneBytes = sizeof(vrd::DevScene) * n;
    cudaMemcpyAsync(b->dData, b->hStage, b->dataBytes, cudaMemcpyHostToDevice, st);
    const float* dCC = (const float*)(b->dData + instBytes + sceneBytes);
    const int grid = std::max(1, b->numSMs * b->blocksPerSM);
    bool anyPlain = false, anyLearned = false, anyTrain = false, anySplit = false, anyUnsplit = false;
    const vrd::BatchInstance* hInst = (const vrd::BatchInstance*)b->hStage;
    for (int i = 0; i < n; ++i) {
        vr_context* c = b->ctx[i];
        if (lp_active(c)) { anyLearned = true; anyTrain |= c->opts.mLearnedTrainSamples > 0; }
        else anyPlain = true;
        if (hInst[i].spatialRounds > 0) (hInst[i].split ? anySplit : anyUnsplit) = true;
    }
    int launches = 0;
    if (anyPlain) { batch_pass<MB>(b, BL, 0, st); launches++; }
    if (anyLearned) {
        for (vr_context* c : b->ctx)
            if (lp_active(c)) {
                cudaMemsetAsync(c->lp.qcount, 0, sizeof(int), st);
                cudaMemsetAsync(c->lp.pcount, 0, 16 * sizeof(int), st);
            }
        batch_pass<MB>(b, BL, 1, st);
        batch_vertex0<MB>(BL, grid, st);
        launches += 2;
        // the bounce passes: one launch each for the walks and the vertices of every walking
        // instance, one per instance and bounce for the others (linear sampler)
        bool anyWalk = false;
        for (int i = 0; i < n; ++i) anyWalk |= hInst[i].walk != 0;
        for (int bn = 1; bn < MB; ++bn) {
            if (anyWalk) { batch_walk_all<MB>(BL, bn, grid, st); launches += 2; }
            for (int i = 0; i < n; ++i)
                if (hInst[i].learned && !hInst[i].walk) { batch_lp_bounce<MB>(BL, i, bn, grid, st); launches++; }
        }
        for (vr_context* c : b->ctx)
            if (lp_active(c)) {
                vrk::launch_net_infer(net_view(c), c->lp.query, c->lp.qcapacity, c->lp.qcount, c->lp.T, c->lp.qlist, c->status, c->numSMs, st);
                launches++;
            }
        batch_pass<MB>(b, BL, 2, st);
        launches++;
        // online training of every learned instance on this frame's queries (used from the next
        // frame on): training samples, then each instance's steps, on the training stream
        if (anyTrain) {
            cudaEventRecord(b->evFork, st);
            cudaStreamWaitEvent(b->tstream, b->evFork, 0);
            batch_train_gen<MB>(BL, grid, b->tstream);
            b->trainLaunches = 1;
            for (int i = 0; i < n; ++i) {
                vr_context* c = b->ctx[i];
                if (!lp_active(c) || c->opts.mLearnedTrainSamples <= 0) continue;
                const int64_t step0 = c->adamStep;
                lp_train_steps(c, c->lp.train, c->opts.mLearnedTrainSamples, b->tstream, dCC + b->ccOff[i]);
                c->adamStep = step0;         // advanced once per frame in batch_finish (graph replays too)
                b->trainLaunches += 2 * b->steps[i];
            }
            cudaEventRecord(b->evJoin, b->tstream);
        }
    }
    if (b->temporal && !b->spatial) {
        for (vr_context* c : b->ctx) {
            const size_t N = (size_t)c->W * c->H;
            cudaMemcpyAsync(c->res[2].a, c->res[0].a, N * 16, cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(c->res[2].b, c->res[0].b, N * 16, cudaMemcpyDeviceToDevice, st);
            if (MB > 1) cudaMemcpyAsync(c->res[2].extra, c->res[0].extra, N * (size_t)(MB - 1) * 16, cudaMemcpyDeviceToDevice, st);
        }
    }
    if (b->spatial) {
        for (int r = 0; r < b->rounds; ++r) {
            BL.round = r;
            if (anySplit) {
                batch_split_reset<MB>(BL, st);
                batch_pass<MB>(b, BL, 5, st);
                batch_split_march<MB>(BL, grid, st);
                batch_split_reset<MB>(BL, st);
                batch_pass<MB>(b, BL, 6, st);
                batch_split_march<MB>(BL, grid, st);
                batch_pass<MB>(b, BL, 7, st);
                launches += 7;
            }
            if (anyUnsplit) {
                batch_pass<MB>(b, BL, 3, st);
                launches++;
            }
        }
    } else {
        batch_pass<MB>(b, BL, 4, st);
        launches++;
    }
    if (anyTrain) {
        cudaStreamWaitEvent(st, b->evJoin, 0);
        launches += b->trainLaunches;
    }
    b->launches = launches;
}

static void batch_finish(vr_batch* b, cudaStream_t st) {
    for (size_t i = 0; i < b->ctx.size(); ++i) {
        vr_context* c = b->ctx[i];
        const vr_options& o = c->opts;
        if (o.mEnableTemporalReuse) c->featCurIdx ^= 1;
        c->temporalSampleAccumulated = 1;
        c->prev = b->cfs[i];
        c->frameCount++;
        c->finalBuf = (o.mEnableSpatialReuse ? o.mSpatialReuseRounds : 0) % 2;
        c->launches = 0;
        if (lp_active(c)) {
            c->lpFrameDone = true;
            c->adamStep += b->steps[i];
            c->lastSteps = b->steps[i];
        }
    }
    cudaEventRecord(b->frameDone, st);
    b->pendingFrame = true;
}

static int batch_frame(vr_batch* b, const vr_camera* cams, float* const* outs, cudaStream_t st) {
    vrd::BatchLaunch BL;
    std::vector<int64_t> sig;
    int r = batch_prepare(b, cams, outs, BL, sig);
    if (r) return r;
    auto launch = [&]() {
        switch (b->MB) {
            case 1: batch_launch<1>(b, BL, st); break;
            case 2: batch_launch<2>(b, BL, st); break;
            case 3: batch_launch<3>(b, BL, st); break;
            default: batch_launch<4>(b, BL, st); break;
        }
    };
    if (!b->useGraph) {
        launch();
    } else {
        const cudaStream_t user = st;
        cudaEventRecord(b->evIn, user);
        cudaStreamWaitEvent(b->gstream, b->evIn, 0);
        st = b->gstream;
        if (!b->exec || sig != b->sig) {
            batch_drop_graph(b);
            if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { b->err = "stream capture failed"; return VR_ERR_CUDA; }
            launch();
            if (cudaStreamEndCapture(st, &b->graph) != cudaSuccess || !b->graph) { b->err = "stream capture failed"; batch_drop_graph(b); return VR_ERR_CUDA; }
            if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) { b->err = "graph instantiation failed"; batch_drop_graph(b); return VR_ERR_CUDA; }
            b->sig = sig;
        }
        if (cudaGraphLaunch(b->exec, st) != cudaSuccess) { b->err = "graph launch failed"; return VR_ERR_CUDA; }
        cudaEventRecord(b->evOut, st);
        cudaStreamWaitEvent(user, b->evOut, 0);
        st = user;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { b->err = std::string("batch frame: ") + cudaGetErrorString(e); return VR_ERR_CUDA; }
    batch_finish(b, st);
    return VR_OK;
}

extern "C" {

int vr_set_block_size(vr_context* c, int32_t threads) {
    if (!c || (threads != 32 && threads != 64 && threads != 128)) return VR_ERR_INVALID_ARG;
    c->blockThreads = threads;
    return VR_OK;
}

int vr_batch_create(vr_context* const* ctxs, int32_t n, vr_batch** out) {
    if (!ctxs || !out || n < 1 || n > 1024) return VR_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) if (!ctxs[i] || !ctxs[i]->anim.empty()) return VR_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) if (vertex_reuse(ctxs[i])) return VR_ERR_UNSUPPORTED;    // batches keep no p_partial
    const vr_options& o0 = ctxs[0]->opts;
    if (o0.mUseReference) return VR_ERR_INVALID_ARG;
    for (int i = 1; i < n; ++i) {
        const vr_options& o = ctxs[i]->opts;
        if (o.mMaxBounces != o0.mMaxBounces || o.mEnableTemporalReuse != o0.mEnableTemporalReuse || o.mEnableSpatialReuse != o0.mEnableSpatialReuse ||
            (o0.mEnableSpatialReuse && o.mSpatialReuseRounds != o0.mSpatialReuseRounds) || o.mUseReference)
            return VR_ERR_INVALID_ARG;
    }
    vr_batch* b = new vr_batch();
    b->ctx.assign(ctxs, ctxs + n);
    b->MB = o0.mMaxBounces;
    b->temporal = o0.mEnableTemporalReuse;
    b->spatial = o0.mEnableSpatialReuse;
    b->rounds = o0.mEnableSpatialReuse ? o0.mSpatialReuseRounds : 0;
    cudaDeviceGetAttribute(&b->numSMs, cudaDevAttrMultiProcessorCount, 0);
    if (b->numSMs <= 0) b->numSMs = 1;
    cudaEventCreateWithFlags(&b->frameDone, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&b->evIn, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&b->evOut, cudaEventDisableTiming);
    cudaStreamCreateWithFlags(&b->gstream, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&b->tstream, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&b->evFork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&b->evJoin, cudaEventDisableTiming);
    *out = b;
    return VR_OK;
}

void vr_batch_destroy(vr_batch* b) {
    if (!b) return;
    if (b->pendingFrame) cudaEventSynchronize(b->frameDone);
    batch_drop_graph(b);
    cudaFree(b->dData);
    cudaFreeHost(b->hStage);
    if (b->frameDone) cudaEventDestroy(b->frameDone);
    if (b->evIn) cudaEventDestroy(b->evIn);
    if (b->evOut) cudaEventDestroy(b->evOut);
    if (b->gstream) cudaStreamDestroy(b->gstream);
    if (b->evFork) cudaEventDestroy(b->evFork);
    if (b->evJoin) cudaEventDestroy(b->evJoin);
    if (b->tstream) cudaStreamDestroy(b->tstream);
    delete b;
}

const char* vr_batch_last_error(const vr_batch* b) { return b ? b->err.c_str() : "null batch"; }

int vr_batch_set_graph(vr_batch* b, int32_t enable) {
    if (!b) return VR_ERR_INVALID_ARG;
    b->useGraph = enable != 0;
    if (!b->useGraph) batch_drop_graph(b);
    return VR_OK;
}

int vr_batch_set_launch_shape(vr_batch* b, int32_t tile_w, int32_t blocks_per_sm) {
    if (!b || (tile_w != 4 && tile_w != 8 && tile_w != 16 && tile_w != 32) || blocks_per_sm < 1 || blocks_per_sm > 32) return VR_ERR_INVALID_ARG;
    b->tileW = tile_w;
    b->tileH = 128 / tile_w;
    b->blocksPerSM = blocks_per_sm;
    return VR_OK;
}

int vr_batch_get_launch_shape(const vr_batch* b, int32_t* tile_w, int32_t* tile_h, int32_t* blocks_per_sm) {
    if (!b || !tile_w || !tile_h || !blocks_per_sm) return VR_ERR_INVALID_ARG;
    *tile_w = b->tileW; *tile_h = b->tileH; *blocks_per_sm = b->blocksPerSM;
    return VR_OK;
}

int vr_batch_render(vr_batch* b, const vr_camera* cams, float* const* outs, void* stream) {
    if (!b || !cams || !outs) return VR_ERR_INVALID_ARG;
    return batch_frame(b, cams, outs, (cudaStream_t)stream);
}

int32_t vr_batch_last_launch_count(const vr_batch* b) { return b ? b->launches : 0; }

int vr_batch_autotune(vr_batch* b, const vr_camera* cams, float* const* outs, void* stream, float* trial_ms, int32_t max_trials) {
    if (!b || !cams || !outs) return VR_ERR_INVALID_ARG;
    // tile widths x blocks per SM (capped per pass at the blocks it is compiled to keep resident)
    static const int shapes[][2] = {{8, 5}, {16, 5}, {32, 5}, {8, 4}, {16, 4}, {32, 4}, {8, 3}, {16, 3}, {32, 3}};
    const int nShapes = (int)(sizeof(shapes) / sizeof(shapes[0]));
    cudaStream_t st = (cudaStream_t)stream;
    const bool graph = b->useGraph;
    b->useGraph = false;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bestK = 0, r = VR_OK;
    for (int k = 0; k < nShapes && (max_trials <= 0 || k < max_trials); ++k) {
        b->tileW = shapes[k][0]; b->tileH = 128 / shapes[k][0]; b->blocksPerSM = shapes[k][1];
        cudaEventRecord(e0, st);
        if ((r = batch_frame(b, cams, outs, st))) break;
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (trial_ms) trial_ms[k] = ms;
        if (ms < best) { best = ms; bestK = k; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->tileW = shapes[bestK][0]; b->tileH = 128 / shapes[bestK][0]; b->blocksPerSM = shapes[bestK][1];
    b->useGraph = graph;
    batch_drop_graph(b);
    return r;
}

}  // extern "C"
