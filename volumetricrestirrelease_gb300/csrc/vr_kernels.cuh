// vr_kernels.cuh -- the frame-loop kernels, templated on the maximum path length.
//
// Pass fusion (the reference dispatches six compute passes per frame,
// VolumetricReSTIR.cpp:499-762):
//   k_initial : GenerateFeatures + TraceRays + TemporalReuse for one pixel per thread.  The
//               temporal pass reads only this pixel's new reservoir and previous-frame
//               buffers, so it runs in the same thread right after the initial candidates.
//   k_spatial : one SpatialReuse round; the last round also writes the temporal history
//               (CopyReservoirs) and shades the pixel (FinalShading), both of which read only
//               this pixel's final reservoir.
//   k_final   : FinalShading alone, for configurations without spatial reuse.
//   k_reference: the volume path tracer of the reference mode, accumulated in FP64.
// Each thread keeps its own RNG stream seeded exactly as the pass it restates.
#pragma once

#include "vr_device.cuh"

namespace vrd {

struct FrameBuffers {
    ResBuf cur;            // perPixel[0]: initial + temporal output
    ResBuf sp[2];          // spatial ping-pong (sp[0] aliases cur)
    ResBuf hist;           // temporal history
    float* featCur;        // transmittance feature of this frame
    const float* featPrev; // previous frame's features
    float* color;          // reference-mode colour (rgba)
    float4* out;           // output frame
    float2* mvec;          // optional motion vectors
};

// ---------------------------------------------------------------------------------------
// ComputeInitialSample (ComputeInitialSample.slang:4-395), volume-only
// ---------------------------------------------------------------------------------------
template <int MB>
static __device__ __noinline__ Reservoir initialSample(const FrameParams& P, Ray ray, float preHit, float prePdf, float preTr, vr::Rng& sg, f3 ex[4]) {
    const SamplingOptions& o = P.initial;
    float pathPdf = 1.f, pathPHat = 1.f;
    Reservoir combined = newReservoir();
    Reservoir out = newReservoir();
    float primaryDepth = 0;
    const f3 sigma_s = c_scene.sigma_s, sigma_a = c_scene.sigma_a;
    const float sigma_t = c_scene.sigma_t;
    for (int bounce = 0; bounce < MB; bounce++) {
        out = newReservoir();
        out.M = 1;
        float hitD, pdfDist = 0, Tr;
        MediumInteraction mi;
        if (bounce >= 1 || P.noReuse) {
            if (P.noReuse) {
                mi.valid = false;
                deltaTrack(ray, sg, mi, 0);
                pdfDist = 1.f; Tr = 1.f;
                hitD = mi.valid ? vr::length(mi.p - ray.o) : kRayTMax;
            } else {
                int curMip = o.visibilityMipLevel;
                if (P.useCoarser) curMip = min((o.visibilityMipLevel >= kNumMaxMips ? kNumMaxMips : 0) + c_scene.numMips - 1, curMip + 1);
                float hd[4], pd[4], trs[4];
                sampleDistances(ray, sg, o.visibilityUseLinearSampler != 0, curMip, 1, hd, pd, trs);
                hitD = hd[0]; pdfDist = pd[0]; Tr = trs[0];
                mi.p = at(ray, hitD); mi.wo = -ray.d; mi.g = c_scene.g; mi.valid = hitD != kRayTMax;
            }
        } else {
            hitD = preHit; pdfDist = prePdf; Tr = preTr;
            mi.p = at(ray, hitD); mi.wo = -ray.d; mi.g = c_scene.g; mi.valid = hitD != kRayTMax;
        }
        pathPdf *= pdfDist;
        const int vrs = o.vertexReuseStartBounce;
        // ComputeInitialSample.slang:88-94: the reconnection vertex in area measure (vertex reuse)
        if (vrs >= 0 && bounce == vrs && hitD != kRayTMax) {
            pathPdf /= hitD * hitD;
            pathPHat /= hitD * hitD;
        }
        bool hitEmpty = false;
        float density = 0.f;
        if (bounce == 0) {
            if (MB > 1) out.sampledPixel = encodeBounces(out.sampledPixel, 0);
            out.depth = mi.valid ? hitD : kRayTMax;
            primaryDepth = out.depth;
            out.p_y = pathPdf;
        } else {
            out.depth = primaryDepth;
            if (MB > 1) {
                out.sampledPixel = encodeBounces(out.sampledPixel, bounce);
                if (vrs >= 0 && bounce >= vrs) {
                    // vertex reuse: from the reuse bounce on, the vertex position (ComputeInitialSample.slang:114-127)
                    ex[bounce - 1] = !mi.valid ? mk3(kRayTMax) : mi.p;
                } else {
                    // encodeWiDist (ReSTIRHelper.slang:41-51)
                    f3 w = mk3(ray.d.x, ray.d.y, !mi.valid ? kRayTMax : hitD);
                    if (ray.d.z < 0) w.z = -w.z;
                    ex[bounce - 1] = w;
                }
            }
            out.p_y = pathPdf;
        }
        if (mi.valid) density = P.noReuse ? 1.f : densityWorld(mi.p, 0);
        if ((!mi.valid && bounce > 0) || (mi.valid && density == 0)) {
            out.p_y = 0.f; out.runningSum = 0.f; hitEmpty = true;
        }
        float pdfDir = 1.f;
        if (!hitEmpty) {
            if (mi.valid) {
                f3 albedo = sigma_s / sigma_t;
                out.lightID = -1; out.uv0 = 0; out.uv1 = 0;
                float lightPdf = 0.f;
                // Le and the emission ratio only where the medium emits: without emission the
                // ratio luminance(0) / (0 + luminance(albedo * Ld)) is 0 or NaN -> 0, i.e. 0
                const bool emitting = c_scene.hasEmission && density > 0.f;
                f3 Le = mk3(0.f);
                if (emitting) Le = emissionWorld(mi.p);
                f3 oma = mk3(1.f) - albedo;
                f3 Ld = sampleDirectLighting(sg, lightPdf, mi, o, o.lightSamples != 0, out.lightID, out.uv0, out.uv1);
                f3 wo = -ray.d, wi = mk3(0.f);
                if (MB > 1) {
                    float u0 = vr::next1D(sg), u1 = vr::next1D(sg);
                    pdfDir = samplePhase(mi, wo, wi, u0, u1);
                }
                float p_src = out.p_y;
                {
                    float er = 0.f;
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
                    pathPHat *= Tr;
                    pathPHat *= density;
                    if (out.lightID == kSelfEmissionLightID) p_y = pathPHat * vr::luminance(sigma_a * Le);
                    else p_y = pathPHat * vr::luminance(sigma_s * Ld * lightPdf);
                    pathPHat *= vr::luminance(sigma_s) * pdfDir;
                    if (P.noReuse) { p_y /= sigma_t; pathPHat /= sigma_t; }
                    if (out.runningSum > 0.f) {
                        out.runningSum = out.p_y == 0.f ? 0.f : p_y / out.p_y;
                        if (out.lightID == kSelfEmissionLightID && bounce > 0) {
                            if (vrs < 0 || bounce < vrs) {       // ComputeInitialSample.slang:322-330
                                out.lightID = vr::asint(mi.p.z); out.uv0 = mi.p.x; out.uv1 = mi.p.y;
                                p_y /= (hitD * hitD);
                            }
                            out.sampledPixel = encodeTag(out.sampledPixel, 1);
                        }
                        out.p_y = p_y;
                    }
                }
                pathPdf *= pdfDir;
                if (MB > 1) {
                    if (bounce < MB - 1) {
                        ray = Ray{mi.p, wi, 0, kRayTMax};
                        if (P.useRR && bounce >= 2) {
                            if (vr::next1D(sg) < albedo.x) pathPdf *= albedo.x;
                            else { hitEmpty = true; combined.M++; }
                        }
                    }
                }
            } else {
                f3 Le = envEval(ray.d);
                pathPHat *= Tr;
                float p_y = pathPHat * vr::luminance(Le);
                out.runningSum = out.p_y == 0.f ? 0.f : p_y / out.p_y;
                out.p_y = p_y;
                hitEmpty = true;
            }
        }
        if (MB > 1) resampleStep(out, combined, sg);
        if (hitEmpty) break;
    }
    if (MB > 1) { combined.M = 1; return combined; }
    return out;
}

// ---------------------------------------------------------------------------------------
// volume path tracer (VolumePathTracingFunctions.slang:3-131) with NEE through residual
// ratio tracking (directLighting, VolumeUtils.slang:453-483)
// ---------------------------------------------------------------------------------------
template <int MB>
static __device__ __noinline__ f3 integratePT(const FrameParams& P, Ray ray, vr::Rng& sg) {
    const int maxBounces = MB;
    const int lightSamples = max(1, P.initial.lightSamples);
    MediumInteraction mi;
    f3 beta = mk3(1.f), L = mk3(0.f);
    for (int bounce = 0; bounce < maxBounces; bounce++) {
        mi.valid = false;
        deltaTrack(ray, sg, mi, 0);
        if (mi.valid) {
            f3 albedo = c_scene.sigma_s / c_scene.sigma_t;
            f3 oma = mk3(1.f) - albedo;
            { f3 Le = emissionWorld(mi.p); L = L + Le * oma * beta; }
            beta = beta * albedo;
            f3 Ld = mk3(0.f);
            for (int s = 0; s < lightSamples; s++) {
                LightSample ls; int idx; float u0, u1;
                bool valid = sampleLights(mi.p, P.initial.useEnvironmentLights != 0, P.initial.useAnalyticLights != 0, sg, ls, idx, u0, u1);
                if (!valid) continue;
                ls.pdf = 1.f;
                Ray sr{mi.p, ls.dir, 0, ls.distance};
                float vis = computeVisibility(sr, sg, 1, 0, true, VR_TRACK_RESIDUAL_RATIO, 1.f);
                ls.Li = ls.Li * vis;
                float p = phaseF(mi, mi.wo, ls.dir);
                Ld = Ld + p * ls.Li / ls.pdf;
            }
            Ld = Ld / (float)lightSamples;
            L = L + beta * Ld;
            f3 wo = -ray.d, wi = mk3(0.f);
            if (maxBounces > 1) { float u0 = vr::next1D(sg), u1 = vr::next1D(sg); samplePhase(mi, wo, wi, u0, u1); }
            if (bounce < maxBounces - 1) {
                ray = Ray{mi.p, wi, 0, kRayTMax};
                if (P.useRR && bounce >= 2) {
                    if (vr::next1D(sg) < albedo.x) beta = beta / albedo.x;
                    else bounce = maxBounces;
                }
            }
        } else {
            f3 Le = envEval(ray.d);
            if (bounce == 0) L = L + beta * Le;
            bounce = maxBounces;
        }
    }
    return L;
}

__device__ __forceinline__ void mulMat4(const float* m, const float in[4], float out[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r) out[r] = in[0] * m[r] + in[1] * m[4 + r] + in[2] * m[8 + r] + in[3] * m[12 + r];
}

// ---------------------------------------------------------------------------------------
// TemporalReuse (TemporalReuse.cs.slang:80-377) for one pixel; taps[0] is in `cur`
// ---------------------------------------------------------------------------------------
template <int MB>
static __device__ __noinline__ void temporalReuse(const FrameParams& P, const FrameBuffers& B, int px, int py, const Ray& ray) {
    const int W = P.W, H = P.H, N = P.N;
    const int pixelId = py * W + px;
    vr::Rng sg = vr::rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(P.numTotalRounds * P.frameCount + 1));
    int selectedId = -1;
    int numUsed = 1;
    Reservoir taps[2];
    taps[0] = loadResRW(B.cur, pixelId);
    taps[1] = newReservoir();
    Reservoir output = P.temporalTalbot ? newReservoir() : taps[0];
    const int centerStart = pixelId;
    float tOrigDepth = 0.f;
    int rx = 0, ry = 0;
    const bool isBgRes = B.featCur[pixelId] == 1.f;
    bool useFallback = true;
    if (P.reprojMode != VR_REPROJ_NONE) {
        float rd = taps[0].depth;
        if (rd == kRayTMax && P.reprojMode != VR_REPROJ_NO_BACKGROUND && !isBgRes)
            rd = rejectionSampleByDensity(ray, sg, kNumMaxMips + P.reprojMip);
        f3 p = ray.o + ray.d * rd;
        // the point's position in the previous frame, from the velocity grid (a background point
        // keeps its pixel below, so it needs none)
        if (c_scene.hasVelocity && c_scene.hasAnimation && rd != kRayTMax) {
            const f3 v = velocityWorld(p) * c_scene.velocityScale;
            p = p - v;
        }
        float in4[4] = {p.x, p.y, p.z, 1.f}, vp[4], cp[4];
        mulMat4(P.prevView, in4, vp);
        mulMat4(P.prevProj, vp, cp);
        float sx = cp[0] / cp[3], sy = cp[1] / cp[3];
        int sxi, syi;
        if (rd == kRayTMax) { sx = (float)px + 0.5f; sy = (float)py + 0.5f; sxi = px; syi = py; }
        else {
            sx = 0.5f * sx + 0.5f; sy = -0.5f * sy + 0.5f;
            sx *= (float)W; sy *= (float)H;
            sxi = vr::f2i(sx); syi = vr::f2i(sy);
        }
        {
            uint32_t id = (uint32_t)syi * (uint32_t)W + (uint32_t)sxi;
            float tfT = id < (uint32_t)N ? __ldg(&B.featPrev[id]) : 0.f;
            bool tapBg = tfT == 1.f && id < (uint32_t)N;
            if (isBgRes && !tapBg) {
                if (B.mvec) B.mvec[pixelId] = make_float2((float)(rx - px) / (float)W, (float)(ry - py) / (float)H);
                return;
            }
        }
        sxi = vr::f2i(sx); syi = vr::f2i(sy);
        rx = sxi; ry = syi;
        if (sxi >= 0 && sxi < W && syi >= 0 && syi < H) {
            numUsed++;
            taps[1] = loadRes(B.hist, syi * W + sxi);
        }
        if (numUsed > 1) useFallback = false;
    }
    if (useFallback) { numUsed++; rx = px; ry = py; taps[1] = loadRes(B.hist, pixelId); }
    if (B.mvec) B.mvec[pixelId] = make_float2((float)(rx - px) / (float)W, (float)(ry - py) / (float)H);
    const float MaxPrevM = P.temporalMThreshold * taps[0].M;
    if (numUsed == 2) {
        tOrigDepth = taps[1].depth;
        if (taps[1].depth != kRayTMax) {
            f3 dir = vr::normalize(pinholeDir(P.prevU, P.prevV, P.prevW, rx, ry, W, H));
            f3 wp = P.prevPos + taps[1].depth * dir;
            taps[1].depth = vr::length(wp - ray.o);
        }
    }
    float cPrevDepth = taps[0].depth;
    if (cPrevDepth != kRayTMax) cPrevDepth = vr::length(at(ray, cPrevDepth) - P.prevPos);
    bool hasSel = output.runningSum > 0.f;
    int start = P.temporalTalbot ? 0 : 1;
    if (start == 1) selectedId = 0;
    for (int i = start; i < numUsed; i++) {
        float mis = 1.f;
        float nPy = 0.f;
        if (taps[i].p_y > 0.f) {
            nPy = taps[i].p_y;
            if (vr::isnan_(taps[i].runningSum) || vr::isinf_(taps[i].runningSum)) taps[i].runningSum = 0.f;
            if (i > 0) resampleNeighbor(taps[i], ray, sg, B.hist.extra, N, P.spatial, MB);
        } else { taps[i].p_y = 0.f; taps[i].runningSum = 0.f; }
        if (P.temporalTalbot && taps[i].runningSum > 0.f) {
            float p_sum = 0, p_qi = 0, k = 0;
            for (int j = 0; j < numUsed; j++) {
                float cm = vr::fmin_(MaxPrevM, taps[j].M);
                k += cm;
                if (j == 0) { p_qi = taps[i].p_y; p_sum += taps[i].p_y * cm; }
                else if (i == j) { p_qi = nPy; p_sum += nPy * cm; }
                else {
                    Ray nr{P.prevPos, vr::normalize(pinholeDir(P.prevU, P.prevV, P.prevW, rx, ry, W, H)), 0, i == 0 ? cPrevDepth : tOrigDepth};
                    Reservoir tt = taps[i];
                    tt.depth = nr.tMax;
                    float p_y = evalPHat(tt, i == 0 ? B.cur.extra : B.hist.extra, N, nr, sg, P.spatial, MB, true);
                    if (vr::isinf_(p_y) || vr::isnan_(p_y)) p_y = 0.f;
                    p_sum += p_y * cm;
                }
            }
            if (p_sum > 0) mis = p_qi * k / p_sum;
        }
        taps[i].runningSum *= mis;
        bool sel = resampleStepMaxM(taps[i], MaxPrevM, output, sg);
        hasSel |= sel;
        if (sel) selectedId = i;
    }
    if (MB > 1) {
        if (hasSel && selectedId > 0) {
            int mib = decodeBounces(output.sampledPixel, MB);
            for (int b = 0; b < mib; b++) B.cur.extra[(size_t)b * N + centerStart] = __ldg(&B.hist.extra[(size_t)b * N + output.startPixel]);
        }
        output.startPixel = centerStart;
    }
    storeRes(B.cur, pixelId, output);
}

// ---------------------------------------------------------------------------------------
// k_initial: GenerateFeatures + TraceRays (+ TemporalReuse)
// ---------------------------------------------------------------------------------------
// Register budget: 5 blocks of 128 threads per SM (<= 102 registers per thread).  Measured on
// the full workload against 1, 4 and 6 blocks; the extra residency outweighs the added spills.
#ifndef VR_KINIT_MIN_BLOCKS
#define VR_KINIT_MIN_BLOCKS 5
#endif
#ifndef VR_KSPAT_MIN_BLOCKS
#define VR_KSPAT_MIN_BLOCKS 5
#endif
template <int MB>
__device__ __forceinline__ void initialPixel(const FrameParams& P, const FrameBuffers& B, int px, int py) {
    const int W = P.W, H = P.H, N = P.N;
    const int pid = py * W + px;
    const f3 dir = vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, W, H));
    const Ray ray{P.camPos, dir, 0.f, kRayTMax};
    const bool reference = B.color != nullptr;
    if (!reference) {
        // GenerateFeatures.cs.slang:57-101 (ray-marched transmittance at mip 0, trilinear)
        B.featCur[pid] = featureTransmittance(ray, P.initial.visibilityTStepScale);
    }
    vr::Rng sg = vr::rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(P.numTotalRounds * P.frameCount));
    if (reference) {
        f3 avg = mk3(0.f);
        for (int r = 0; r < P.baselineSpp; ++r) avg = avg + integratePT<MB>(P, ray, sg);
        avg = avg / (float)P.baselineSpp;
        reinterpret_cast<float4*>(B.color)[pid] = make_float4(avg.x, avg.y, avg.z, 1.f);
        return;
    }
    // TraceRays.cs.slang:104-198
    f3 finalEx[4] = {mk3(0.f), mk3(0.f), mk3(0.f), mk3(0.f)};
    Reservoir fin = newReservoir();
    const int M = P.initialM;
    const int rounds = (M + 3) / 4;
    for (int rd = 0; rd < rounds; rd++) {
        float hd[4] = {0, 0, 0, 0}, pd[4] = {0, 0, 0, 0}, trs[4] = {0, 0, 0, 0};
        int rs = rd == rounds - 1 ? (M - 4 * (rounds - 1)) : 4;
        if (!P.noReuse) sampleDistances(ray, sg, P.initial.visibilityUseLinearSampler != 0, P.initial.visibilityMipLevel, rs, hd, pd, trs);
        for (int s = 0; s < rs; s++) {
            f3 ex[4];
            Reservoir o = initialSample<MB>(P, ray, hd[s], pd[s], trs[s], sg, ex);
            bool sel = resampleStep(o, fin, sg);
            if (sel && MB > 1) {
                int mib = decodeBounces(fin.sampledPixel, MB);
                for (int b = 0; b < mib; b++) finalEx[b] = ex[b];
            }
        }
    }
    // the selected suffix goes to this pixel's extra-bounce slots, which the p-hat
    // evaluation below and the later passes read
    const int mib0 = decodeBounces(fin.sampledPixel, MB);
    for (int b = 0; b < mib0; b++) B.cur.extra[(size_t)b * N + pid] = make_float4(finalEx[b].x, finalEx[b].y, finalEx[b].z, 0.f);
    fin.startPixel = pid;
    // TraceRays.cs.slang:176-177 (the reservoir is REUSETYPE inout: vertex reuse updates p_partial)
    float ph = evalPHat(fin, B.cur.extra, N, ray, sg, P.spatial, MB, false, false, &fin.pp);
    if (fin.runningSum > 0.f) {
        fin.runningSum *= fin.p_y == 0.f ? 0.f : ph / fin.p_y;
        fin.p_y = ph;
    }
    storeRes(B.cur, pid, fin);
    if (P.temporalEnabled && !P.isFirstFrame) temporalReuse<MB>(P, B, px, py, ray);
}
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) k_initial(const __grid_constant__ FrameParams P, const __grid_constant__ FrameBuffers B) {
    const int px = blockIdx.x * 8 + (threadIdx.x & 7);
    const int py = blockIdx.y * (blockDim.x >> 3) + (threadIdx.x >> 3);
    if (px >= P.W || py >= P.H) return;
    initialPixel<MB>(P, B, px, py);
}

// ---------------------------------------------------------------------------------------
// FinalShading (FinalShading.cs.slang:71-143) for one pixel
// ---------------------------------------------------------------------------------------
template <int MB>
static __device__ __noinline__ void finalShade(const FrameParams& P, const FrameBuffers& B, const ResBuf& fb, const Reservoir& r, int px, int py) {
    const int pid = py * P.W + px;
    f3 col = mk3(0.f);
    vr::Rng sg = vr::rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(P.numTotalRounds * P.frameCount + P.numTotalRounds - 1));
    if (B.color) {
        float4 c = reinterpret_cast<const float4*>(B.color)[pid];
        col = mk3(c.x, c.y, c.z);
    } else if (P.visualizeTr) {
        col = mk3(vr::pow_(B.featCur[pid], 2.2f));
    } else if (r.runningSum > 0.f) {
        Ray ray{P.camPos, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, P.W, P.H)), 0, r.depth};
        f3 c = evaluateF(r, fb.extra, P.N, ray, sg, P.fin, MB, P.noReuse != 0, true);
        float Wt = r.p_y == 0.0f ? 1.f : r.runningSum / (r.p_y * r.M);
        c = c * Wt;
        col = col + c;
    }
    float cc[4] = {col.x, col.y, col.z, 1.f};
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) bad |= vr::isnan_(cc[k]) || vr::isinf_(cc[k]);
    B.out[pid] = bad ? make_float4(0.f, 0.f, 0.f, 0.f) : make_float4(cc[0], cc[1], cc[2], cc[3]);
}

// CopyReservoirs (CopyReservoirs.cs.slang:84-94) for one pixel
template <int MB>
__device__ __forceinline__ void writeHistory(const FrameBuffers& B, const ResBuf& fb, const Reservoir& r, int pid, int N) {
    storeRes(B.hist, pid, r);
    if (MB > 1) {
        int mib = decodeBounces(r.sampledPixel, MB);
        for (int b = 0; b < mib; b++) B.hist.extra[(size_t)b * N + pid] = fb.extra[(size_t)b * N + pid];
    }
}

// ---------------------------------------------------------------------------------------
// k_spatial: one SpatialReuse round (SpatialReuse.cs.slang:94-264); the last round also
// writes the temporal history and shades the pixel
// ---------------------------------------------------------------------------------------
struct SpatialParams {
    int in, out;
    int roundId;
    int numRounds, rid;            // RNG seed: numRounds * frame + rid
    int last;
    int writeHistory;
    int offs[32][2];
};

template <int MB>
__device__ __forceinline__ void spatialPixel(const FrameParams& P, const FrameBuffers& B, const SpatialParams& S, int px, int py) {
    const int W = P.W, H = P.H, N = P.N;
    const int pid = py * W + px;
    const ResBuf& in = B.sp[S.in];
    const ResBuf& outb = B.sp[S.out];
    vr::Rng sg = vr::rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(S.numRounds * P.frameCount + S.rid));
    Reservoir output = loadRes(in, pid);
    const int centerStart = pid;
    const Ray ray{P.camPos, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, W, H)), 0, kRayTMax};
    if (P.spatialTalbot) output = newReservoir();
    bool hasSel = output.runningSum > 0.f;
    Reservoir result;
    if (__ldg(&B.featCur[pid]) == 1.f) {
        result = P.spatialTalbot ? loadRes(in, pid) : output;
        storeRes(outb, pid, result);
        if (MB > 1) {
            int mib = decodeBounces(output.sampledPixel, MB);
            for (int b = 0; b < mib; b++) outb.extra[(size_t)b * N + output.startPixel] = __ldg(&in.extra[(size_t)b * N + output.startPixel]);
        }
        result.startPixel = pid;
    } else {
        const int K = P.spatialK;
        for (int s = P.spatialTalbot ? 0 : 1; s < K; s++) {
            int tx = px + S.offs[s][0], ty = py + S.offs[s][1];
            if (!(tx >= 0 && tx < W && ty >= 0 && ty < H)) continue;
            Reservoir tap = loadRes(in, ty * W + tx);
            float mis = 1.f;
            if (s > 0) resampleNeighbor(tap, ray, sg, in.extra, N, P.spatial, MB, true);     // resampleNeighborSpatialReuse
            if (P.spatialTalbot && tap.runningSum > 0.f) {
                float p_sum = 0, p_qi = 0, k = 0;
                for (int j = 0; j < K; j++) {
                    int tx2 = px + S.offs[j][0], ty2 = py + S.offs[j][1];
                    if (!(tx2 >= 0 && tx2 < W && ty2 >= 0 && ty2 < H)) continue;
                    float4 a2 = __ldg(&in.a[ty2 * W + tx2]);
                    float M2 = a2.y;
                    k += M2;
                    if (j == 0) { p_qi = tap.p_y; p_sum += tap.p_y * M2; }
                    else if (s == j) { p_qi = a2.w; p_sum += a2.w * M2; }
                    else {
                        Ray nr{ray.o, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, tx2, ty2, W, H)), 0, tap.depth};
                        float p_y = evalPHat(tap, in.extra, N, nr, sg, P.spatial, MB, false, true);    // evaluatePHatReadOnly(..., true)
                        if (vr::isinf_(p_y) || vr::isnan_(p_y)) p_y = 0.f;
                        p_sum += p_y * M2;
                    }
                }
                if (p_sum > 0) mis = p_qi * k / p_sum;
            }
            tap.runningSum *= mis;
            if (resampleStep(tap, output, sg)) hasSel = true;
        }
        if (MB > 1) {
            if (hasSel) {
                int mib = decodeBounces(output.sampledPixel, MB);
                for (int b = 0; b < mib; b++) outb.extra[(size_t)b * N + centerStart] = __ldg(&in.extra[(size_t)b * N + output.startPixel]);
            }
            output.startPixel = centerStart;
        }
        storeRes(outb, pid, output);
        result = output;
    }
    if (S.last) {
        if (S.writeHistory) writeHistory<MB>(B, outb, result, pid, N);
        finalShade<MB>(P, B, outb, result, px, py);
    }
}
template <int MB>
__global__ void __launch_bounds__(128, VR_KSPAT_MIN_BLOCKS) k_spatial(const __grid_constant__ FrameParams P, const __grid_constant__ FrameBuffers B, const __grid_constant__ SpatialParams S) {
    const int px = blockIdx.x * 8 + (threadIdx.x & 7);
    const int py = blockIdx.y * (blockDim.x >> 3) + (threadIdx.x >> 3);
    if (px >= P.W || py >= P.H) return;
    spatialPixel<MB>(P, B, S, px, py);
}

// ---------------------------------------------------------------------------------------
// The SpatialReuse round with its marches split out (the default spatial options: ray-marched
// visibility and light transmittance, one sample each, at most kSplitK taps).
//
// Per pixel the round re-evaluates p-hat up to K^2 - K times, and each evaluation marches the
// camera segment, every suffix segment and the light segment; per thread, the lanes of a warp
// wait for the longest march of every evaluation.  Here the evaluations run twice through
// evaluateFV: first recording the segments they would march (RecordVis, which answers 1 and
// lists the segment), then, after k_split_march has marched every listed segment as resumable
// walks (a lane whose march ends takes the next segment), replaying the marched values
// (ReplayVis).  Transmittance only scales F, so a recording walks the same branches as the
// replay or further, never fewer; the replay consumes a prefix of the recorded segments in the
// same order and evaluates exactly what evaluateF does.  Three per-pixel kernels:
//   k_split_a : records E(s, 0) (each neighbour tap at this pixel's ray, resampleNeighbor)
//               and, for Talbot MIS, E(0, j) (the centre's reservoir at every tap's ray);
//   k_split_b : replays them into E, and records E(s, j) for the taps with weight left;
//   k_split_c : the round itself (SpatialReuse.cs.slang:94-264), E(s, j) replayed in place,
//               then the history copy and the final shading of the last round.
// ---------------------------------------------------------------------------------------
constexpr int kSplitK = 4;
struct SpatialSplit {
    float4* seg;        // [slots][2]: (origin, tMax), (direction, march step) of each recorded segment
    float* tr;          // [slots]: its marched transmittance
    uint2* list;        // recorded segments: (slot, mip | linear << 8)
    int* counts;        // [0] entries in list, [1] next entry of the marches
    float* E;           // [N][kSplitK * kSplitK]: p-hat of tap s at pixel j's ray
    int capacity;       // entries of list
};
__device__ __forceinline__ size_t splitSlot(int pid, int s, int j, int MB) {
    return ((size_t)pid * (kSplitK * kSplitK) + (size_t)(s * kSplitK + j)) * (size_t)(MB + 1);
}
struct RecordVis {
    const SpatialSplit* S;
    size_t base;
    int k;
    __device__ float operator()(const Ray& r, vr::Rng&, int, int mip, bool lin, uint32_t, float tss) {
        const size_t slot = base + (size_t)(k++);
        // the march step of trRayMarch
        int eff = mip >= kPrevSlotOffset ? mip - kPrevSlotOffset : mip;
        eff = eff >= kNumMaxMips ? eff - kNumMaxMips : eff;
        const float tStep = c_scene.tStep * tss * (float)(eff + 1);
        S->seg[2 * slot] = make_float4(r.o.x, r.o.y, r.o.z, r.tMax);
        S->seg[2 * slot + 1] = make_float4(r.d.x, r.d.y, r.d.z, tStep);
        const unsigned m = __activemask();
        const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
        int b = 0;
        if (lane == leader) b = atomicAdd(S->counts, __popc(m));
        b = __shfl_sync(m, b, leader) + __popc(m & ((1u << lane) - 1u));
        if (b < S->capacity) S->list[b] = make_uint2((uint32_t)slot, (uint32_t)mip | (lin ? 256u : 0u));
        else if (c_scene.status) atomicOr(c_scene.status, 2);
        return 1.f;
    }
};
struct ReplayVis {
    const float* tr;
    size_t base;
    int k;
    // computeVisibility's average over its samples, with the marched values
    __device__ float operator()(const Ray&, vr::Rng&, int samples, int, bool, uint32_t, float) {
        float vis = 0;
        for (int i = 0; i < samples; i++) vis += tr[base + (size_t)k];
        k++;
        vis /= samples;
        return vis;
    }
};
__host__ __device__ inline bool spatialSplitEligible(const FrameParams& P) {
    return P.spatial.vertexReuseStartBounce < 0 && P.spatialK <= kSplitK && P.spatial.visibilityTrackingMethod == VR_TRACK_RAY_MARCHING &&
           P.spatial.lightingTrackingMethod == VR_TRACK_RAY_MARCHING && P.spatial.visibilitySamples == 1 && P.spatial.lightSamples == 1;
}

__device__ __forceinline__ bool splitPixel(const FrameParams& P, int& px, int& py) {
    px = blockIdx.x * 8 + (threadIdx.x & 7);
    py = blockIdx.y * (blockDim.x >> 3) + (threadIdx.x >> 3);
    return px < P.W && py < P.H;
}

template <int MB>
__device__ __forceinline__ void splitAPixel(const FrameParams& P, const FrameBuffers& B, const SpatialParams& S, const SpatialSplit& SS, int px, int py) {
    const int W = P.W, H = P.H, N = P.N, K = P.spatialK;
    const int pid = py * W + px;
    if (__ldg(&B.featCur[pid]) == 1.f) return;
    const ResBuf& in = B.sp[S.in];
    const Ray ray{P.camPos, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, W, H)), 0, kRayTMax};
    vr::Rng unused;
    for (int s = P.spatialTalbot ? 0 : 1; s < K; s++) {
        const int tx = px + S.offs[s][0], ty = py + S.offs[s][1];
        if (!(tx >= 0 && tx < W && ty >= 0 && ty < H)) continue;
        const Reservoir tap = loadRes(in, ty * W + tx);
        if (s > 0 && tap.runningSum != 0.f) {
            RecordVis v{&SS, splitSlot(pid, s, 0, MB), 0};
            evaluateFV(tap, in.extra, N, ray, unused, P.spatial, MB, false, false, false, v);
        }
        if (s == 0 && P.spatialTalbot && tap.runningSum > 0.f) {
            for (int j = 1; j < K; j++) {
                const int tx2 = px + S.offs[j][0], ty2 = py + S.offs[j][1];
                if (!(tx2 >= 0 && tx2 < W && ty2 >= 0 && ty2 < H)) continue;
                const Ray nr{ray.o, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, tx2, ty2, W, H)), 0, tap.depth};
                RecordVis v{&SS, splitSlot(pid, 0, j, MB), 0};
                evaluateFV(tap, in.extra, N, nr, unused, P.spatial, MB, false, false, false, v);
            }
        }
    }
}

template <int MB>
__device__ __forceinline__ void splitBPixel(const FrameParams& P, const FrameBuffers& B, const SpatialParams& S, const SpatialSplit& SS, int px, int py) {
    const int W = P.W, H = P.H, N = P.N, K = P.spatialK;
    const int pid = py * W + px;
    if (__ldg(&B.featCur[pid]) == 1.f) return;
    const ResBuf& in = B.sp[S.in];
    const Ray ray{P.camPos, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, W, H)), 0, kRayTMax};
    vr::Rng unused;
    for (int s = P.spatialTalbot ? 0 : 1; s < K; s++) {
        const int tx = px + S.offs[s][0], ty = py + S.offs[s][1];
        if (!(tx >= 0 && tx < W && ty >= 0 && ty < H)) continue;
        const Reservoir tap = loadRes(in, ty * W + tx);
        float rs = tap.runningSum;
        if (s > 0 && tap.runningSum != 0.f) {
            ReplayVis v{SS.tr, splitSlot(pid, s, 0, MB), 0};
            const float ph = vr::luminance(evaluateFV(tap, in.extra, N, ray, unused, P.spatial, MB, false, false, false, v));
            SS.E[(size_t)pid * (kSplitK * kSplitK) + s * kSplitK] = ph;
            float w = ph / tap.p_y;
            if (vr::isinf_(w) || vr::isnan_(w)) w = 0.f;
            rs = tap.runningSum * w;
        }
        if (!P.spatialTalbot || !(rs > 0.f)) continue;
        for (int j = 1; j < K; j++) {
            if (j == s) continue;
            const int tx2 = px + S.offs[j][0], ty2 = py + S.offs[j][1];
            if (!(tx2 >= 0 && tx2 < W && ty2 >= 0 && ty2 < H)) continue;
            const Ray nr{ray.o, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, tx2, ty2, W, H)), 0, tap.depth};
            if (s == 0) {
                ReplayVis v{SS.tr, splitSlot(pid, 0, j, MB), 0};
                SS.E[(size_t)pid * (kSplitK * kSplitK) + j] =
                    vr::luminance(evaluateFV(tap, in.extra, N, nr, unused, P.spatial, MB, false, false, false, v));
            } else {
                RecordVis v{&SS, splitSlot(pid, s, j, MB), 0};
                evaluateFV(tap, in.extra, N, nr, unused, P.spatial, MB, false, false, false, v);
            }
        }
    }
}

// the recorded segments of one list, marched as resumable walks by the warps of the grid: a lane
// whose march ends takes the next listed segment; returns when the list is used up
__device__ __forceinline__ void splitMarchList(const SpatialSplit& SS) {
    const int n = min(SS.counts[0], SS.capacity);
    const int lane = threadIdx.x & 31;
    MarchWalk w;
    uint32_t slot = 0;
    int mip = 0;
    bool live = false, exhausted = false;
    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, !live && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(SS.counts + 1, __popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!live && !exhausted) {
                const int idx = base + __popc(need & ((1u << lane) - 1u));
                if (idx >= n) exhausted = true;
                else {
                    const uint2 e = SS.list[idx];
                    slot = e.x;
                    mip = (int)(e.y & 255u);
                    const float4 a = SS.seg[2 * (size_t)slot], d = SS.seg[2 * (size_t)slot + 1];
                    const Ray r{mk3(a.x, a.y, a.z), mk3(d.x, d.y, d.z), 0.f, a.w};
                    live = marchStart(c_scene.slots[mip], mip, r, d.w, (e.y & 256u) != 0, w);
                    if (!live) SS.tr[slot] = w.Tr;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, live) == 0) {
            if (__ballot_sync(0xffffffffu, !exhausted) == 0) break;
            continue;
        }
        if (live && marchStep(c_scene.slots[mip], mip, w)) {
            SS.tr[slot] = w.Tr;
            live = false;
        }
    }
}

template <int MB>
__device__ __forceinline__ void splitCPixel(const FrameParams& P, const FrameBuffers& B, const SpatialParams& S, const SpatialSplit& SS, int px, int py) {
    const int W = P.W, H = P.H, N = P.N;
    const int pid = py * W + px;
    const ResBuf& in = B.sp[S.in];
    const ResBuf& outb = B.sp[S.out];
    const float* E = SS.E + (size_t)pid * (kSplitK * kSplitK);
    vr::Rng sg = vr::rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(S.numRounds * P.frameCount + S.rid));
    Reservoir output = loadRes(in, pid);
    const int centerStart = pid;
    const Ray ray{P.camPos, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, W, H)), 0, kRayTMax};
    if (P.spatialTalbot) output = newReservoir();
    bool hasSel = output.runningSum > 0.f;
    Reservoir result;
    if (__ldg(&B.featCur[pid]) == 1.f) {
        result = P.spatialTalbot ? loadRes(in, pid) : output;
        storeRes(outb, pid, result);
        if (MB > 1) {
            int mib = decodeBounces(output.sampledPixel, MB);
            for (int b = 0; b < mib; b++) outb.extra[(size_t)b * N + output.startPixel] = __ldg(&in.extra[(size_t)b * N + output.startPixel]);
        }
        result.startPixel = pid;
    } else {
        const int K = P.spatialK;
        vr::Rng unused;
        for (int s = P.spatialTalbot ? 0 : 1; s < K; s++) {
            int tx = px + S.offs[s][0], ty = py + S.offs[s][1];
            if (!(tx >= 0 && tx < W && ty >= 0 && ty < H)) continue;
            Reservoir tap = loadRes(in, ty * W + tx);
            float mis = 1.f;
            if (s > 0 && tap.runningSum != 0.f) {          // resampleNeighbor, p-hat from k_split_b
                const float ph = E[s * kSplitK];
                float w = ph / tap.p_y;
                if (vr::isinf_(w) || vr::isnan_(w)) w = 0.f;
                tap.runningSum *= w;
                tap.p_y = ph;
            }
            if (P.spatialTalbot && tap.runningSum > 0.f) {
                float p_sum = 0, p_qi = 0, k = 0;
                for (int j = 0; j < K; j++) {
                    int tx2 = px + S.offs[j][0], ty2 = py + S.offs[j][1];
                    if (!(tx2 >= 0 && tx2 < W && ty2 >= 0 && ty2 < H)) continue;
                    float4 a2 = __ldg(&in.a[ty2 * W + tx2]);
                    float M2 = a2.y;
                    k += M2;
                    if (j == 0) { p_qi = tap.p_y; p_sum += tap.p_y * M2; }
                    else if (s == j) { p_qi = a2.w; p_sum += a2.w * M2; }
                    else {
                        float p_y;
                        if (s == 0) p_y = E[j];
                        else {
                            Ray nr{ray.o, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, tx2, ty2, W, H)), 0, tap.depth};
                            ReplayVis v{SS.tr, splitSlot(pid, s, j, MB), 0};
                            p_y = vr::luminance(evaluateFV(tap, in.extra, N, nr, unused, P.spatial, MB, false, false, false, v));
                        }
                        if (vr::isinf_(p_y) || vr::isnan_(p_y)) p_y = 0.f;
                        p_sum += p_y * M2;
                    }
                }
                if (p_sum > 0) mis = p_qi * k / p_sum;
            }
            tap.runningSum *= mis;
            if (resampleStep(tap, output, sg)) hasSel = true;
        }
        if (MB > 1) {
            if (hasSel) {
                int mib = decodeBounces(output.sampledPixel, MB);
                for (int b = 0; b < mib; b++) outb.extra[(size_t)b * N + centerStart] = __ldg(&in.extra[(size_t)b * N + output.startPixel]);
            }
            output.startPixel = centerStart;
        }
        storeRes(outb, pid, output);
        result = output;
    }
    if (S.last) {
        if (S.writeHistory) writeHistory<MB>(B, outb, result, pid, N);
        finalShade<MB>(P, B, outb, result, px, py);
    }
}

#ifndef VR_BATCHED
template <int MB>
__global__ void __launch_bounds__(128, VR_KSPAT_MIN_BLOCKS) k_split_a(const __grid_constant__ FrameParams P, const __grid_constant__ FrameBuffers B,
                                                                      const __grid_constant__ SpatialParams S, const __grid_constant__ SpatialSplit SS) {
    int px, py;
    if (splitPixel(P, px, py)) splitAPixel<MB>(P, B, S, SS, px, py);
}
template <int MB>
__global__ void __launch_bounds__(128, VR_KSPAT_MIN_BLOCKS) k_split_b(const __grid_constant__ FrameParams P, const __grid_constant__ FrameBuffers B,
                                                                      const __grid_constant__ SpatialParams S, const __grid_constant__ SpatialSplit SS) {
    int px, py;
    if (splitPixel(P, px, py)) splitBPixel<MB>(P, B, S, SS, px, py);
}
static __global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) k_split_march(const __grid_constant__ SpatialSplit SS) {
    splitMarchList(SS);
}
template <int MB>
__global__ void __launch_bounds__(128, VR_KSPAT_MIN_BLOCKS) k_split_c(const __grid_constant__ FrameParams P, const __grid_constant__ FrameBuffers B,
                                                                      const __grid_constant__ SpatialParams S, const __grid_constant__ SpatialSplit SS) {
    int px, py;
    if (splitPixel(P, px, py)) splitCPixel<MB>(P, B, S, SS, px, py);
}
#endif

// k_final: FinalShading without spatial reuse (optionally after the history copy)
template <int MB>
__device__ __forceinline__ void finalPixel(const FrameParams& P, const FrameBuffers& B, int writeHist, int px, int py) {
    const int pid = py * P.W + px;
    Reservoir r = loadRes(B.cur, pid);
    if (writeHist) writeHistory<MB>(B, B.cur, r, pid, P.N);
    finalShade<MB>(P, B, B.cur, r, px, py);
}
template <int MB>
__global__ void __launch_bounds__(128) k_final(const __grid_constant__ FrameParams P, const __grid_constant__ FrameBuffers B, int writeHist) {
    const int px = blockIdx.x * 8 + (threadIdx.x & 7);
    const int py = blockIdx.y * (blockDim.x >> 3) + (threadIdx.x >> 3);
    if (px >= P.W || py >= P.H) return;
    finalPixel<MB>(P, B, writeHist, px, py);
}

// k_reference: FP64 accumulation of the path tracer over frames [first, first + count)
template <int MB>
__global__ void __launch_bounds__(128) k_reference(const FrameParams P, int first, int count, double* accum) {
    const int px = blockIdx.x * 8 + (threadIdx.x & 7);
    const int py = blockIdx.y * (blockDim.x >> 3) + (threadIdx.x >> 3);
    if (px >= P.W || py >= P.H) return;
    const int pid = py * P.W + px;
    const Ray ray{P.camPos, vr::normalize(pinholeDir(P.camU, P.camV, P.camW, px, py, P.W, P.H)), 0.f, kRayTMax};
    // running FP64 sums, added frame by frame (AccumulatePass accumulateDouble)
    double s0 = accum[(size_t)pid * 3 + 0], s1 = accum[(size_t)pid * 3 + 1], s2 = accum[(size_t)pid * 3 + 2];
    for (int f = first; f < first + count; ++f) {
        vr::Rng sg = vr::rng_create((uint32_t)px, (uint32_t)py, (uint32_t)(P.numTotalRounds * f));
        f3 avg = mk3(0.f);
        for (int r = 0; r < P.baselineSpp; ++r) avg = avg + integratePT<MB>(P, ray, sg);
        avg = avg / (float)P.baselineSpp;
        s0 += (double)avg.x; s1 += (double)avg.y; s2 += (double)avg.z;
    }
    accum[(size_t)pid * 3 + 0] = s0;
    accum[(size_t)pid * 3 + 1] = s1;
    accum[(size_t)pid * 3 + 2] = s2;
}

}  // namespace vrd
