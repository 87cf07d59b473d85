// vr_lp_kernels.cuh -- the initial pass with the learned target, split into generate and select
// around the batched network evaluation, and the generation of the network's training samples.
//
// generate follows ComputeInitialSample (ComputeInitialSample.slang:4-395) and TraceRays
// (TraceRays.cs.slang:104-198) step for step with two changes: the next-event estimate does not
// march its shadow ray (SampleDirectLighting's visibility, VolumeUtils.slang:485-521), and every
// resampling uniform is drawn at generation time whether or not the weight is positive, so the
// random stream is independent of the predicted transmittance.
#pragma once

#include "vr_kernels.cuh"
#include "vr_lp.h"

namespace vrd {

__device__ __forceinline__ bool resampleStepU(const Reservoir& r, Reservoir& s, float u) {
    float w = r.runningSum;
    s.M += r.M;
    if (w <= 0.0f) return false;
    s.runningSum += w;
    bool sel = u * s.runningSum < w;
    if (sel) copySample(r, s);
    return sel;
}

// stores the query of a slot and appends the slot to the compacted list; the threads that reach
// this point together share one atomic
__device__ __forceinline__ void lpAppendQuery(const LpBuffers& L, f3 x, f3 w, float tmax, int slot) {
    L.query[2 * (size_t)slot] = make_float4(x.x, x.y, x.z, w.x);
    L.query[2 * (size_t)slot + 1] = make_float4(w.y, w.z, tmax, __int_as_float(slot));
    const unsigned m = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    const int rank = __popc(m & ((1u << lane) - 1u));
    int base = 0;
    if (lane == leader) base = atomicAdd(L.qcount, __popc(m));
    base = __shfl_sync(m, base, leader);
    const int idx = base + rank;
    if (idx < L.qcapacity) {
        L.qlist[idx] = slot;
    } else if (c_scene.status) {
        atomicOr(c_scene.status, 2);
    }
}

// state of one candidate path between its vertices
struct LpPath {
    Ray ray;
    float pathPdf, pathPHat, primaryDepth;
    int bounce;
};

// random stream of candidate c's indirect vertices (bounces >= 1); the pixel's own stream covers
// the primary distance samples, the first vertex of every candidate and the candidate uniforms
__device__ __forceinline__ vr::Rng lpCandidateStream(int px, int py, int frameCount, int c) {
    return vr::rng_create((uint32_t)px, (uint32_t)py, 0x40000000u | (((uint32_t)frameCount * 4096u + (uint32_t)c) & 0x3FFFFFFFu));
}

// a continuing path in the queue of its next bounce: (o, pathPdf), (d, pathPHat), (pixel,
// candidate, -, -), the candidate stream
__device__ __forceinline__ void lpEnqueue(const LpBuffers& L, int level, const LpPath& cs, int pid, int c, const vr::Rng& g) {
    const unsigned m = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    const int rank = __popc(m & ((1u << lane) - 1u));
    int base = 0;
    if (lane == leader) base = atomicAdd(&L.pcount[level], __popc(m));
    base = __shfl_sync(m, base, leader);
    const size_t i = (size_t)(base + rank);
    if (i >= (size_t)L.pcapacity) {                 // cannot happen: a candidate enters each queue once
        if (c_scene.status) atomicOr(c_scene.status, 2);
        return;
    }
    float4* q = L.paths[level & 1] + 4 * i;
    q[0] = make_float4(cs.ray.o.x, cs.ray.o.y, cs.ray.o.z, cs.pathPdf);
    q[1] = make_float4(cs.ray.d.x, cs.ray.d.y, cs.ray.d.z, cs.pathPHat);
    q[2] = make_float4(__int_as_float(pid), __int_as_float(c), 0.f, 0.f);
    q[3] = make_float4(__uint_as_float(g.s[0]), __uint_as_float(g.s[1]), __uint_as_float(g.s[2]), __uint_as_float(g.s[3]));
}


// one vertex (bounce cs.bounce) of candidate c: writes its record and returns true when the
// path continues, i.e. when the next vertex needs a distance sample along cs.ray
template <int MB>
__device__ __forceinline__ bool lpVertex(const FrameParams& P, LpPath& cs, float hitD, float pdfDist, float Tr, vr::Rng& sg,
                                         const LpBuffers& L, int c, int pid) {
    const SamplingOptions& o = P.initial;
    const int N = P.N;
    const f3 sigma_s = c_scene.sigma_s, sigma_a = c_scene.sigma_a;
    const float sigma_t = c_scene.sigma_t;
    const int bounce = cs.bounce;
    const Ray ray = cs.ray;
    Reservoir out = newReservoir();
    out.M = 1;
    MediumInteraction mi;
    mi.p = at(ray, hitD); mi.wo = -ray.d; mi.g = c_scene.g; mi.valid = hitD != kRayTMax;
    cs.pathPdf *= pdfDist;
    bool hitEmpty = false;
    float density = 0.f;
    if (bounce == 0) {
        if (MB > 1) out.sampledPixel = encodeBounces(out.sampledPixel, 0);
        out.depth = mi.valid ? hitD : kRayTMax;
        cs.primaryDepth = out.depth;
    } else {
        if (MB > 1) {
            out.sampledPixel = encodeBounces(out.sampledPixel, bounce);
            f3 w = mk3(ray.d.x, ray.d.y, !mi.valid ? kRayTMax : hitD);
            if (ray.d.z < 0) w.z = -w.z;
            L.ex[(size_t)(c * (MB - 1) + bounce - 1) * N + pid] = make_float4(w.x, w.y, w.z, 0.f);
        }
    }
    out.p_y = cs.pathPdf;
    if (mi.valid) density = densityWorld(mi.p, 0);
    if ((!mi.valid && bounce > 0) || (mi.valid && density == 0)) {
        out.p_y = 0.f; out.runningSum = 0.f; hitEmpty = true;
    }
    int flags = kLpValid;
    float pdfDir = 1.f;
    if (!hitEmpty) {
        if (mi.valid) {
            f3 albedo = sigma_s / sigma_t;
            out.lightID = -1; out.uv0 = 0; out.uv1 = 0;
            float lightPdf = 0.f;
            const bool emitting = c_scene.hasEmission && density > 0.f;
            f3 Le = mk3(0.f);
            if (emitting) Le = emissionWorld(mi.p);
            f3 oma = mk3(1.f) - albedo;
            LightSample ls;
            const bool lv = sampleLights(mi.p, o.useEnvironmentLights != 0, o.useAnalyticLights != 0, sg, ls, out.lightID, out.uv0, out.uv1);
            f3 Ld = mk3(0.f);
            if (lv) {
                lightPdf = ls.pdfArea;
                float ph = phaseF(mi, mi.wo, ls.dir);
                Ld = mk3(0.f) + ph * ls.Li / 1.f;
            }
            f3 wo = -ray.d, wi = mk3(0.f);
            if (MB > 1) {
                float u0 = vr::next1D(sg), u1 = vr::next1D(sg);
                pdfDir = samplePhase(mi, wo, wi, u0, u1);
            }
            float p_src = out.p_y;
            {
                float er = 0.f;      // 0 without emission (see initialSample)
                if (emitting) {
                    er = vr::luminance(oma * Le) / (vr::luminance(oma * Le) + vr::luminance(albedo * Ld));
                    if (vr::isnan_(er)) er = 0.f;
                }
                if (vr::next1D(sg) < er) { p_src *= er; out.lightID = kSelfEmissionLightID; }
                else p_src *= lightPdf * (1 - er);
            }
            out.runningSum = p_src == 0.f ? 0.f : 1.f;
            out.p_y = p_src;
            {
                float p_y;
                cs.pathPHat *= Tr;
                cs.pathPHat *= density;
                const bool emis = out.lightID == kSelfEmissionLightID;
                if (emis) p_y = cs.pathPHat * vr::luminance(sigma_a * Le);
                else p_y = cs.pathPHat * vr::luminance(sigma_s * Ld * lightPdf);
                cs.pathPHat *= vr::luminance(sigma_s) * pdfDir;
                if (out.runningSum > 0.f) {
                    if (!emis && lv && o.lightSamples != 0 && p_y != 0.f) {
                        // runningSum keeps p_src and p_y the unoccluded target until T is known
                        flags |= kLpNeedsT;
                        out.runningSum = out.p_y;
                        out.p_y = p_y;
                        lpAppendQuery(L, mi.p, ls.dir, ls.distance, (c * MB + bounce) * N + pid);
                    } else {
                        out.runningSum = out.p_y == 0.f ? 0.f : p_y / out.p_y;
                        if (emis && bounce > 0) {
                            out.lightID = vr::asint(mi.p.z); out.uv0 = mi.p.x; out.uv1 = mi.p.y;
                            p_y /= (hitD * hitD);
                            out.sampledPixel = encodeTag(out.sampledPixel, 1);
                        }
                        out.p_y = p_y;
                    }
                }
            }
            cs.pathPdf *= pdfDir;
            if (MB > 1) {
                if (bounce < MB - 1) {
                    cs.ray = Ray{mi.p, wi, 0, kRayTMax};
                    if (P.useRR && bounce >= 2) {
                        if (vr::next1D(sg) < albedo.x) cs.pathPdf *= albedo.x;
                        else hitEmpty = true;
                    }
                }
            }
        } else {
            f3 Le = envEval(ray.d);
            cs.pathPHat *= Tr;
            float p_y = cs.pathPHat * vr::luminance(Le);
            out.runningSum = out.p_y == 0.f ? 0.f : p_y / out.p_y;
            out.p_y = p_y;
            hitEmpty = true;
        }
    }
    const float ub = MB > 1 ? vr::next1D(sg) : 0.f;
    const size_t slot = (size_t)(c * MB + bounce) * N + pid;
    L.vrecA[slot] = make_float4(out.runningSum, out.p_y, out.uv0, out.uv1);
    L.vrecB[slot] = make_int4(out.lightID, out.sampledPixel, flags, __float_as_int(ub));
    // the record after the last vertex of a path that ended early is marked invalid
    if (hitEmpty) {
        if (bounce + 1 < MB) L.vrecB[(size_t)(c * MB + bounce + 1) * N + pid].z = 0;
        return false;
    }
    cs.bounce = bounce + 1;
    return cs.bounce < MB;
}

// the first vertex of candidate c of a pixel from the primary distance sample in L.dist: drawn
// from the candidate's own stream (the vertex, then the candidate's resampling uniform); a path
// that goes on is queued for the bounce passes with that stream
template <int MB>
__device__ __forceinline__ void lpVertex0(const FrameParams& P, const LpBuffers& L, int c, int px, int py) {
    const int N = P.N;
    const int pid = py * P.W + px;
    const float4 d = L.dist[(size_t)c * N + pid];
    LpPath cs;
    cs.ray = Ray{P.camPos, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, P.W, P.H)), 0.f, kRayTMax};
    cs.pathPdf = 1.f; cs.pathPHat = 1.f; cs.primaryDepth = 0.f; cs.bounce = 0;
    vr::Rng g = lpCandidateStream(px, py, P.frameCount, c);
    const bool more = lpVertex<MB>(P, cs, d.x, d.y, d.z, g, L, c, pid);
    const float uc = vr::next1D(g);
    L.crec[(size_t)c * N + pid] = make_float2(cs.primaryDepth, uc);
    if (more) lpEnqueue(L, 1, cs, pid, c, g);
}

// generate, in the order of the learned target: GenerateFeatures, then per pixel the rounds of
// TraceRays (up to 4 primary distance samples in one traversal) from the pixel's stream, whose
// samples go to L.dist (the pixel's stream is then left to the select pass); then, in a launch of
// its own with one thread per candidate, the first vertex of every candidate from the candidate's
// own stream (lpVertex0).  Measured on one GB300 at 1080p, 36 candidates: the generate stage 72.7 ms with
// rounds and vertices alternating per candidate, 63.5 ms with every round first in one kernel,
// 55.8 ms with the vertices in their own launch (74 registers, a flat grid of M x N threads).
template <int MB>
__device__ __forceinline__ void lpRoundsPixel(const FrameParams& P, const FrameBuffers& B, const LpBuffers& L, int px, int py) {
    const int W = P.W, N = P.N;
    const int pid = py * W + px;
    const f3 dir = vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, W, P.H));
    const Ray ray{P.camPos, dir, 0.f, kRayTMax};
    B.featCur[pid] = featureTransmittance(ray, P.initial.visibilityTStepScale);
    vr::Rng sg = vr::rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(P.numTotalRounds * P.frameCount));
    const int M = P.initialM;
    const int rounds = (M + 3) / 4;
    int c = 0;
    for (int rd = 0; rd < rounds; rd++) {
        float hd[4] = {0, 0, 0, 0}, pd[4] = {0, 0, 0, 0}, trs[4] = {0, 0, 0, 0};
        int rs = rd == rounds - 1 ? (M - 4 * (rounds - 1)) : 4;
        sampleDistances<SampleDistLp>(ray, sg, P.initial.visibilityUseLinearSampler != 0, P.initial.visibilityMipLevel, rs, hd, pd, trs);
        for (int s = 0; s < rs; s++, c++) L.dist[(size_t)c * N + pid] = make_float4(hd[s], pd[s], trs[s], 0.f);
    }
    L.rng[pid] = make_uint4(sg.s[0], sg.s[1], sg.s[2], sg.s[3]);
}

// one indirect vertex (bounce b >= 1) of a queued path (entry i of `src`): its distance sample,
// then the vertex; a path that goes on is queued for bounce b + 1
template <int MB>
__device__ __forceinline__ void lpBouncePath(const FrameParams& P, const LpBuffers& L, int b, const float4* src, size_t i) {
    const float4* q = src + 4 * i;
    const float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
    LpPath cs;
    cs.ray = Ray{mk3(q0.x, q0.y, q0.z), mk3(q1.x, q1.y, q1.z), 0.f, kRayTMax};
    cs.pathPdf = q0.w; cs.pathPHat = q1.w; cs.primaryDepth = 0.f; cs.bounce = b;
    const int pid = __float_as_int(q2.x), c = __float_as_int(q2.y);
    vr::Rng g;
    g.s[0] = __float_as_uint(q3.x); g.s[1] = __float_as_uint(q3.y); g.s[2] = __float_as_uint(q3.z); g.s[3] = __float_as_uint(q3.w);
    const SamplingOptions& o = P.initial;
    int curMip = o.visibilityMipLevel;
    if (P.useCoarser) curMip = min((o.visibilityMipLevel >= kNumMaxMips ? kNumMaxMips : 0) + c_scene.numMips - 1, curMip + 1);
    float hd[4], pd[4], trs[4];
    sampleDistances<SampleDistLp>(cs.ray, g, o.visibilityUseLinearSampler != 0, curMip, 1, hd, pd, trs);
    if (lpVertex<MB>(P, cs, hd[0], pd[0], trs[0], g, L, c, pid)) lpEnqueue(L, b + 1, cs, pid, c, g);
}

// the bounce pass b: a persistent grid over the queue of bounce b (or its sorted copy), whose
// length the previous pass left on the device
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) k_lp_bounce(const __grid_constant__ FrameParams P, const __grid_constant__ LpBuffers L,
                                                                        int b, int sorted) {
    const int n = min(L.pcount[b], L.pcapacity);
    const float4* src = sorted ? L.psort : L.paths[b & 1];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)n; i += (size_t)gridDim.x * blockDim.x)
        lpBouncePath<MB>(P, L, b, src, i);
}

// ---------------------------------------------------------------------------------------
// The bounce pass in two kernels: k_lp_walk samples the distance of every queued path, and
// k_lp_vertex then builds the vertices.  k_lp_walk keeps the walk of trackVolume + SampleDist
// (one sample, point-sampled) as explicit per-lane state and advances it one step per loop
// trip, a step being one node of the tree or one voxel of a brick; a lane whose walk ends
// stores its result and takes the next path of the queue (warp-aggregated counter) while the
// other lanes of its warp go on walking, so the lanes of a warp stay on live walks instead of
// waiting for the longest walk of the warp.  Every walk performs the operations of
// trackVolume(..., SampleDist) in the same order, so results are bit-identical.  The result
// goes back into the queue entry: pathPdf * pdf, pathPHat * Tr (the first operations of
// lpVertex on either value), the hit distance and the random state after the walk.
// ---------------------------------------------------------------------------------------
struct LpWalk {
    HDDA dda, dl;               // node-level walk, brick-level walk (dl = dda prepared for the leaf)
    float tFar, t, thick;
    float tMax1, tMax2;         // exits of the level-1 and root nodes
    f3 vmin;                    // origin of the current node
    int lev, node, nid1, brick; // level, current node, level-1 node, brick being walked
    int oiter, biter;           // trip counters of trackVolume's node loop and the brick loop
    float hit, tr, pdf;
    vr::Rng g;
    size_t entry;
    bool inBrick;
};

// trackVolume's climb to the first node whose exit lies beyond the walk
__device__ __forceinline__ void lpWalkAscend(const DevSlot& s, LpWalk& w) {
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
// SampleDist::end
__device__ __forceinline__ void lpWalkEnd(LpWalk& w, bool init) {
    if (init) {
        if (w.hit == -1) { w.hit = kRayTMax; w.tr = vr::exp_(-w.thick); w.pdf = w.tr; }
    } else {
        w.hit = kRayTMax; w.tr = 1.f; w.pdf = 1.f;
    }
}
// trackVolume's set-up; false when the walk ended there (the ray misses the volume)
__device__ __forceinline__ bool lpWalkStart(const DevSlot& s, int mip, const Ray& rWorld, LpWalk& w) {
    Ray ray;
    ray.o = mulPoint(rWorld.o, s.M);
    ray.d = mulVec(rWorld.d, s.M);
    ray.tMin = rWorld.tMin; ray.tMax = rWorld.tMax;
    float tNear, tFar;
    w.thick = 0.f;
    if (!intersectBound(ray, tNear, tFar, mip, false)) { lpWalkEnd(w, false); return false; }
    w.tFar = tFar;
    w.hit = -1;
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
// one step of the walk; true when it has ended (hit, tr and pdf hold the sample)
__device__ __forceinline__ bool lpWalkStep(const DevSlot& s, int mip, LpWalk& w) {
    const float eps = 0.01f;
    if (w.inBrick) {
        // one trip of SampleDist::mainStep's voxel loop (one sample, point-sampled)
        if (!(w.biter < kMaxBrickSteps && inLeaf(w.dl.p))) {
            w.inBrick = false;               // mainStep returned false: the node loop goes on
            w.dda.step();
            w.dda.t.x += eps;
            lpWalkAscend(s, w);
            w.oiter++;
            return false;
        }
        w.dl.next();
        const float maxDeltaT = vr::fmin_(w.tFar - w.t, w.dl.t.y - w.t);
        const float curTMax = vr::fmin_(w.tFar, w.dl.t.y);
        const float sigma_t = densityCell(mip, w.brick, w.dl.p) * c_scene.sigma_t;
        const float dT = -vr::log_(1 - vr::next1D(w.g)) / sigma_t;
        float curT = w.t + dT;
        if (vr::isnan_(curT) || vr::isinf_(curT)) curT = kRayTMax;
        if (curT < curTMax) {
            w.hit = curT;
            w.tr = vr::exp_(-(dT * sigma_t + w.thick));
            w.pdf = sigma_t * w.tr;
            return true;
        }
        const float dThick = maxDeltaT * sigma_t;
        w.t = curTMax;
        w.thick += dThick;
        if (w.t >= w.tFar) { lpWalkEnd(w, true); return true; }
        w.dl.step();
        w.biter++;
        return false;
    }
    // one trip of trackVolume's node loop
    const int kDim[3] = {3, 4, 5}, kRes[3] = {8, 16, 32};
    const float kVdel[3] = {1.f, 8.f, 128.f};
    const int* p = w.dda.p;
    if (!(w.oiter < 4096 && w.lev > 0 && w.lev <= 2 && p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] <= kRes[w.lev] && p[1] <= kRes[w.lev] &&
          p[2] <= kRes[w.lev])) {
        lpWalkEnd(w, true);
        return true;
    }
    w.dda.next();
    const int b = (((w.dda.p[2] << kDim[w.lev]) + w.dda.p[1]) << kDim[w.lev]) + w.dda.p[0];
    const int child = getChild(s, w.node, w.lev, b);
    if (child >= 0) {
        if (w.lev == 1) {
            w.t = w.dda.t.x - eps;
            if (w.t >= w.tFar) { lpWalkEnd(w, true); return true; }
            const f3 vl = nodeVmin(s, 0, child);
            w.brick = child;
            w.dl = w.dda;
            w.dl.prepareLeaf(vl);
            w.biter = 0;
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
    lpWalkAscend(s, w);
    w.oiter++;
    return false;
}

// the distance samples of the queue of bounce b held in `queue` (a frame's sorted copy, or a
// batched instance's queue itself), written back into its entries
template <int MB>
__device__ __forceinline__ void lpWalkPass(const FrameParams& P, const LpBuffers& L, int b, float4* queue) {
    const int n = min(L.pcount[b], L.pcapacity);
    const SamplingOptions& o = P.initial;
    int mip = o.visibilityMipLevel;
    if (P.useCoarser) mip = min((o.visibilityMipLevel >= kNumMaxMips ? kNumMaxMips : 0) + c_scene.numMips - 1, mip + 1);
    const DevSlot& s = c_scene.slots[mip];
    const int lane = threadIdx.x & 31;
    int* cursor = L.wcursor + b;
    LpWalk w;
    bool live = false, exhausted = false;
    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, !live && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(cursor, __popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!live && !exhausted) {
                const int idx = base + __popc(need & ((1u << lane) - 1u));
                if (idx >= n) exhausted = true;
                else {
                    w.entry = (size_t)idx;
                    const float4* q = queue + 4 * w.entry;
                    const float4 q0 = q[0], q1 = q[1], q3 = q[3];
                    w.g.s[0] = __float_as_uint(q3.x); w.g.s[1] = __float_as_uint(q3.y);
                    w.g.s[2] = __float_as_uint(q3.z); w.g.s[3] = __float_as_uint(q3.w);
                    const Ray r{mk3(q0.x, q0.y, q0.z), mk3(q1.x, q1.y, q1.z), 0.f, kRayTMax};
                    live = true;
                    if (!lpWalkStart(s, mip, r, w)) live = false, exhausted = false;
                    if (!live) {
                        float4* qw = queue + 4 * w.entry;
                        qw[0].w *= w.pdf; qw[1].w *= w.tr; qw[2].z = w.hit;
                        qw[3] = make_float4(__uint_as_float(w.g.s[0]), __uint_as_float(w.g.s[1]), __uint_as_float(w.g.s[2]), __uint_as_float(w.g.s[3]));
                    }
                }
            }
        }
        if (__ballot_sync(0xffffffffu, live) == 0) {
            if (__ballot_sync(0xffffffffu, !exhausted) == 0) break;
            continue;
        }
        if (live && lpWalkStep(s, mip, w)) {
            float4* qw = queue + 4 * w.entry;
            qw[0].w *= w.pdf; qw[1].w *= w.tr; qw[2].z = w.hit;
            qw[3] = make_float4(__uint_as_float(w.g.s[0]), __uint_as_float(w.g.s[1]), __uint_as_float(w.g.s[2]), __uint_as_float(w.g.s[3]));
            live = false;
        }
    }
}

template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) k_lp_walk(const __grid_constant__ FrameParams P, const __grid_constant__ LpBuffers L, int b) {
    lpWalkPass<MB>(P, L, b, L.psort);
}

// the vertices of the queue of bounce b from the distances the walks left in its entries
template <int MB>
__device__ __forceinline__ void lpVertexPass(const FrameParams& P, const LpBuffers& L, int b, const float4* queue) {
    const int n = min(L.pcount[b], L.pcapacity);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)n; i += (size_t)gridDim.x * blockDim.x) {
        const float4* q = queue + 4 * i;
        const float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
        LpPath cs;
        cs.ray = Ray{mk3(q0.x, q0.y, q0.z), mk3(q1.x, q1.y, q1.z), 0.f, kRayTMax};
        cs.pathPdf = q0.w; cs.pathPHat = q1.w; cs.primaryDepth = 0.f; cs.bounce = b;
        const int pid = __float_as_int(q2.x), c = __float_as_int(q2.y);
        vr::Rng g;
        g.s[0] = __float_as_uint(q3.x); g.s[1] = __float_as_uint(q3.y); g.s[2] = __float_as_uint(q3.z); g.s[3] = __float_as_uint(q3.w);
        // pdf and Tr are already in pathPdf and pathPHat: x * 1 = x
        if (lpVertex<MB>(P, cs, q2.z, 1.f, 1.f, g, L, c, pid)) lpEnqueue(L, b + 1, cs, pid, c, g);
    }
}
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) k_lp_vertex(const __grid_constant__ FrameParams P, const __grid_constant__ LpBuffers L, int b) {
    lpVertexPass<MB>(P, L, b, L.psort);
}

// Counting sort of a queue by coherence key before its bounce pass: the octant of the direction
// and the 8^3 cell of the volume box holding the origin, so that a warp takes paths that cross
// the same region in the same direction.  The order of a queue changes no result (every path
// writes its own slots), only the divergence of the traversals in a warp.
__device__ __forceinline__ int lpPathKey(const LpBuffers& L, float4 q0, float4 q1) {
    int cell[3];
    const float o[3] = {q0.x, q0.y, q0.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float u = (o[k] - L.kmin[k]) * L.kinv[k] * 8.f;
        cell[k] = u >= 0.f ? (u < 8.f ? (int)u : 7) : 0;       // NaN lands in cell 0
    }
    const int oct = (q1.x < 0.f ? 1 : 0) | (q1.y < 0.f ? 2 : 0) | (q1.z < 0.f ? 4 : 0);
    return (oct << 9) | (cell[2] << 6) | (cell[1] << 3) | cell[0];
}
static __global__ void __launch_bounds__(256) k_path_hist(const __grid_constant__ LpBuffers L, int b) {
    __shared__ int h[kPathKeys];
    for (int i = threadIdx.x; i < kPathKeys; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const int n = min(L.pcount[b], L.pcapacity);
    const float4* q = L.paths[b & 1];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)n; i += (size_t)gridDim.x * blockDim.x)
        atomicAdd(&h[lpPathKey(L, q[4 * i], q[4 * i + 1])], 1);
    __syncthreads();
    for (int i = threadIdx.x; i < kPathKeys; i += blockDim.x)
        if (h[i]) atomicAdd(&L.hist[i], h[i]);
}
// exclusive prefix sums of the key counts into the scatter cursors: one block of 1024 threads,
// 4 keys each
static __global__ void __launch_bounds__(1024) k_path_scan(const __grid_constant__ LpBuffers L) {
    __shared__ int s[1024];
    const int t = threadIdx.x;
    int v[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) { v[k] = L.hist[4 * t + k]; sum += v[k]; }
    s[t] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int add = t >= off ? s[t - off] : 0;
        __syncthreads();
        s[t] += add;
        __syncthreads();
    }
    int base = s[t] - sum;
#pragma unroll
    for (int k = 0; k < 4; ++k) { L.hist[kPathKeys + 4 * t + k] = base; base += v[k]; }
}
static __global__ void __launch_bounds__(256) k_path_scatter(const __grid_constant__ LpBuffers L, int b) {
    const int n = min(L.pcount[b], L.pcapacity);
    const float4* q = L.paths[b & 1];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)n; i += (size_t)gridDim.x * blockDim.x) {
        const float4 a = q[4 * i], c = q[4 * i + 1], d = q[4 * i + 2], e = q[4 * i + 3];
        // one cursor update per key and warp: the lanes holding the same key take consecutive
        // places after the lowest of them reserved them all
        const int key = lpPathKey(L, a, c);
        const unsigned peers = __match_any_sync(__activemask(), key);
        const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&L.hist[kPathKeys + key], __popc(peers));
        const int pos = __shfl_sync(peers, base, leader) + __popc(peers & ((1u << lane) - 1u));
        if (pos < 0 || pos >= n) continue;                    // cannot happen: the cursors cover [0, n)
        float4* o = L.psort + 4 * (size_t)pos;
        o[0] = a; o[1] = c; o[2] = d; o[3] = e;
    }
}
// generate in two launches: the per-pixel part (features and the rounds of primary distance
// samples), then one thread per candidate for the first vertices (candidate c of pixel pid is
// thread c * N + pid: the lanes of a warp take one candidate of neighbouring pixels)
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) k_lp_rounds(const __grid_constant__ FrameParams P, const __grid_constant__ FrameBuffers B, const __grid_constant__ LpBuffers L) {
    const int px = blockIdx.x * 8 + (threadIdx.x & 7);
    const int py = blockIdx.y * (blockDim.x >> 3) + (threadIdx.x >> 3);
    if (px >= P.W || py >= P.H) return;
    lpRoundsPixel<MB>(P, B, L, px, py);
}
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) k_lp_vertex0(const __grid_constant__ FrameParams P, const __grid_constant__ LpBuffers L) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)P.initialM * (size_t)P.N) return;
    const int c = (int)(i / (size_t)P.N), pid = (int)(i - (size_t)c * (size_t)P.N);
    lpVertex0<MB>(P, L, c, pid % P.W, pid / P.W);
}

// select: resample the recorded candidates with the predicted transmittance, then finish
// TraceRays (p_hat of the winner) and run TemporalReuse as k_initial does.
// lpSelectChoose: the candidates of a pixel resampled with the predicted transmittances (the
// recorded vertices replayed with p-hat = unoccluded p-hat x T); the winner's suffix goes to
// B.cur.extra
template <int MB>
__device__ __forceinline__ Reservoir lpSelectChoose(const FrameParams& P, const FrameBuffers& B, const LpBuffers& L, int pid) {
    const int N = P.N;
    Reservoir fin = newReservoir();
    int cSel = -1;
    // a candidate's records are loaded before they are replayed, so that their loads are in
    // flight together: every vertex record's flags (fetched while the previous candidate is
    // replayed), then the record and T of each vertex up to the first invalid one (the slots
    // after it are never used)
    float2 crNext = L.crec[pid];
    int4 rbNext[MB];
#pragma unroll
    for (int b = 0; b < MB; b++) rbNext[b] = L.vrecB[(size_t)b * N + pid];
    for (int c = 0; c < P.initialM; c++) {
        const float2 cr = crNext;
        int4 rb[MB];
#pragma unroll
        for (int b = 0; b < MB; b++) rb[b] = rbNext[b];
        if (c + 1 < P.initialM) {
            crNext = L.crec[(size_t)(c + 1) * N + pid];
#pragma unroll
            for (int b = 0; b < MB; b++) rbNext[b] = L.vrecB[(size_t)((c + 1) * MB + b) * N + pid];
        }
        float4 ra[MB];
        float tv[MB];
        bool alive = true;
#pragma unroll
        for (int b = 0; b < MB; b++) {
            const size_t slot = (size_t)(c * MB + b) * N + pid;
            alive = alive && (rb[b].z & kLpValid);
            ra[b] = alive ? L.vrecA[slot] : make_float4(0.f, 0.f, 0.f, 0.f);
            tv[b] = alive && (rb[b].z & kLpNeedsT) ? L.T[slot] : 1.f;
        }
        Reservoir comb = newReservoir();
#pragma unroll
        for (int b = 0; b < MB; b++) {
            if (!(rb[b].z & kLpValid)) break;
            Reservoir out = newReservoir();
            out.M = 1; out.depth = cr.x;
            out.runningSum = ra[b].x; out.p_y = ra[b].y; out.uv0 = ra[b].z; out.uv1 = ra[b].w;
            out.lightID = rb[b].x; out.sampledPixel = rb[b].y;
            if (rb[b].z & kLpNeedsT) {
                float p_y = ra[b].y * tv[b];
                out.runningSum = ra[b].x == 0.f ? 0.f : p_y / ra[b].x;
                out.p_y = p_y;
            }
            if (MB > 1) resampleStepU(out, comb, __int_as_float(rb[b].w));
            else comb = out;
        }
        if (MB > 1) comb.M = 1;
        if (resampleStepU(comb, fin, cr.y)) cSel = c;
    }
    // the winner's suffix (its candidate's records are not written again in the frame)
    if (MB > 1 && cSel >= 0) {
        const int mib0 = decodeBounces(fin.sampledPixel, MB);
        for (int b = 0; b < mib0; b++) {
            const float4 e = L.ex[(size_t)(cSel * (MB - 1) + b) * N + pid];
            B.cur.extra[(size_t)b * N + pid] = make_float4(e.x, e.y, e.z, 0.f);
        }
    }
    fin.startPixel = pid;
    return fin;
}
// TraceRays' p-hat of the winner (the marched target) in place of the predicted one
__device__ __forceinline__ void lpSelectTarget(Reservoir& fin, float ph) {
    if (fin.runningSum > 0.f) {
        fin.runningSum *= fin.p_y == 0.f ? 0.f : ph / fin.p_y;
        fin.p_y = ph;
    }
}
__device__ __forceinline__ vr::Rng lpPixelStream(const LpBuffers& L, int pid) {
    vr::Rng sg;
    const uint4 s = L.rng[pid];
    sg.s[0] = s.x; sg.s[1] = s.y; sg.s[2] = s.z; sg.s[3] = s.w;
    return sg;
}

template <int MB>
__device__ __forceinline__ void lpSelectPixel(const FrameParams& P, const FrameBuffers& B, const LpBuffers& L, int px, int py) {
    const int pid = py * P.W + px;
    const Ray ray{P.camPos, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, P.W, P.H)), 0.f, kRayTMax};
    vr::Rng sg = lpPixelStream(L, pid);
    Reservoir fin = lpSelectChoose<MB>(P, B, L, pid);
    lpSelectTarget(fin, evalPHat(fin, B.cur.extra, P.N, ray, sg, P.spatial, MB));
    storeRes(B.cur, pid, fin);
    if (P.temporalEnabled && !P.isFirstFrame) temporalReuse<MB>(P, B, px, py, ray);
}

// 4 blocks per SM (128 registers): the spills of the temporal evaluations drop from 188 to 88
// bytes; measured 14.2 -> 13.7 ms per 1080p frame (3 blocks: 14.95 ms)
template <int MB>
__global__ void __launch_bounds__(128, 4) k_lp_select(const __grid_constant__ FrameParams P, const __grid_constant__ FrameBuffers B, const __grid_constant__ LpBuffers L) {
    const int px = blockIdx.x * 8 + (threadIdx.x & 7);
    const int py = blockIdx.y * (blockDim.x >> 3) + (threadIdx.x >> 3);
    if (px >= P.W || py >= P.H) return;
    lpSelectPixel<MB>(P, B, L, px, py);
}

// training samples of the network, drawn from the queries the frame's candidates made: sample i
// picks a pixel and a starting slot from its own stream and takes the first slot of that pixel
// (cyclically from the start) that holds a query, with up to 4 pixels tried; the target is a full-resolution (mip 0,
// trilinear) estimate of the transmittance of the query's shadow ray, by ray marching (default) or
// by (residual) ratio tracking.  A sample that found no query is invalid (tmax = -1).
template <int MB>
__device__ __forceinline__ void lpTrainSample(const FrameParams& P, const LpBuffers& L, uint32_t seed, int i) {
    const int N = P.N, S = L.numSlots;
    vr::Rng sg = vr::rng_create((uint32_t)i & 0x3FFFu, (uint32_t)i >> 14, seed);
    int slot = -1;
    for (int att = 0; att < 4 && slot < 0; ++att) {
        const int pid = min(N - 1, (int)(vr::next1D(sg) * (float)N));
        const int j0 = min(S - 1, (int)(vr::next1D(sg) * (float)S));
        for (int k = 0; k < S; ++k) {
            int j = j0 + k;
            if (j >= S) j -= S;
            if (reinterpret_cast<const int*>(L.vrecB + (size_t)j * N + pid)[2] & kLpNeedsT) { slot = j * N + pid; break; }
        }
    }
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = make_float4(0.f, 0.f, -1.f, 0.f);
    if (slot >= 0) {
        a = L.query[2 * (size_t)slot];
        const float4 q1 = L.query[2 * (size_t)slot + 1];
        Ray sr{mk3(a.x, a.y, a.z), mk3(a.w, q1.x, q1.y), 0, q1.z};
        const float t = computeVisibility(sr, sg, 1, 0, true, L.targetMethod, 1.f);
        b = make_float4(q1.x, q1.y, q1.z, t);
    }
    L.train[2 * (size_t)i] = a;
    L.train[2 * (size_t)i + 1] = b;
}
template <int MB>
__global__ void __launch_bounds__(128) k_lp_train_gen(const __grid_constant__ FrameParams P, const __grid_constant__ LpBuffers L, uint32_t seed) {
    const int i = blockIdx.x * 128 + threadIdx.x;
    if (i >= L.trainCount) return;
    lpTrainSample<MB>(P, L, seed, i);
}


}  // namespace vrd
