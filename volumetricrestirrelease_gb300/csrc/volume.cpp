// volume.cpp -- host-side construction of the sparse 8^3-brick grid with its normal and
// conservative mip pyramids (the setup that Scene::addGVDBVolume performs in the reference,
// Source/Falcor/Scene/Scene.cpp:2754-3279, on grids produced by the GVDB converter,
// gvdb-voxel-src/source/gvdb_library/src/gvdb_volume_gvdb.cpp:2700-2862).
//
// Layout (one "slot" per mip; slots 0-7 normal mips, 8-15 conservative mips, as the
// reference's gvdb parameter block, HostDeviceSharedConstants.slang:21-27):
//   level 2 (root, origin 0): dense 32^3 child list, each child covering 128^3 voxels
//   level 1 nodes: vmin + dense 16^3 child list, each child an 8^3 brick
//   level 0 bricks: vmin + density bounds (min, max, avg) + 10^3 voxels (apron of 1)
// This keeps the three-level hierarchy the reference's HDDA walks (gvdbNodes.slang:175-223:
// 4096 -> 128 -> 8 voxels) so that traversal order and RNG consumption are the same, while
// storing each brick with its apron contiguously so a trilinear lookup never leaves it.
#include "vr_volume.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "vr_math.h"
#include "vr_bc4.h"

namespace vr {

// ---------------------------------------------------------------------------------------
// parallel helper
// ---------------------------------------------------------------------------------------
template <class F>
static void parallel_for(int n, F f) {
    int nt = (int)std::thread::hardware_concurrency();
    if (nt <= 0) nt = 4;
    nt = std::min(nt, 64);
    if (n < 2 * nt) { for (int i = 0; i < n; ++i) f(i); return; }
    std::atomic<int> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&]() { for (int i; (i = next.fetch_add(1)) < n;) f(i); });
    for (auto& t : th) t.join();
}

// ---------------------------------------------------------------------------------------
// half precision (round to nearest even), written for this project
// ---------------------------------------------------------------------------------------
uint16_t float_to_half(float f) {
    uint32_t x = f2u(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);          // overflow -> inf
    if (ax < 0x38800000u) {                                            // half denormal / zero
        if (ax < 0x33000000u) return (uint16_t)sign;
        uint32_t m = (ax & 0x007fffffu) | 0x00800000u;
        int shift = 126 - (int)(ax >> 23);                             // 14..24
        uint32_t q = m >> shift;                                       // units of 2^-24
        uint32_t rem = m & ((1u << shift) - 1u);
        uint32_t halfway = 1u << (shift - 1);
        if (rem > halfway || (rem == halfway && (q & 1u))) q += 1;
        return (uint16_t)(sign | q);
    }
    uint32_t e = (ax >> 23) - 112;                                     // rebias 127 -> 15
    uint32_t m = ax & 0x007fffffu;
    uint32_t q = (e << 10) | (m >> 13);
    uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) q += 1;
    return (uint16_t)(sign | q);
}

float half_to_float(uint16_t h) {
    uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu;
    uint32_t m = h & 0x3ffu;
    if (e == 0) {
        if (m == 0) return u2f(sign);
        float v = (float)m * 5.9604644775390625e-08f;                  // m * 2^-24, exact
        return sign ? -v : v;
    }
    if (e == 31) return u2f(sign | 0x7f800000u | (m << 13));
    return u2f(sign | ((e + 112) << 23) | (m << 13));
}

// ---------------------------------------------------------------------------------------
// seeded improved Perlin noise (Perlin 2002) and fBm
// ---------------------------------------------------------------------------------------
struct Perlin {
    int perm[512];
    explicit Perlin(uint32_t seed) {
        int p[256];
        for (int i = 0; i < 256; ++i) p[i] = i;
        uint64_t st = 0x5EEDull ^ ((uint64_t)seed << 17) ^ seed;
        for (int i = 255; i > 0; --i) {                 // Fisher-Yates with SplitMix64
            uint64_t r = splitmix64_next(st);
            int j = (int)(r % (uint64_t)(i + 1));
            std::swap(p[i], p[j]);
        }
        for (int i = 0; i < 512; ++i) perm[i] = p[i & 255];
    }
    static float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
    static float lerp(float a, float b, float t) { return a + t * (b - a); }
    static float grad(int h, float x, float y, float z) {
        h &= 15;
        float u = h < 8 ? x : y;
        float v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
        return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
    }
    float noise(float x, float y, float z) const {
        float fx = floor_(x), fy = floor_(y), fz = floor_(z);
        int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
        x -= fx; y -= fy; z -= fz;
        float u = fade(x), v = fade(y), w = fade(z);
        int A = perm[X] + Y, AA = perm[A] + Z, AB = perm[A + 1] + Z;
        int B = perm[X + 1] + Y, BA = perm[B] + Z, BB = perm[B + 1] + Z;
        return lerp(lerp(lerp(grad(perm[AA], x, y, z), grad(perm[BA], x - 1, y, z), u),
                         lerp(grad(perm[AB], x, y - 1, z), grad(perm[BB], x - 1, y - 1, z), u), v),
                    lerp(lerp(grad(perm[AA + 1], x, y, z - 1), grad(perm[BA + 1], x - 1, y, z - 1), u),
                         lerp(grad(perm[AB + 1], x, y - 1, z - 1), grad(perm[BB + 1], x - 1, y - 1, z - 1), u), v),
                    w);
    }
    float fbm(float x, float y, float z, int octaves, float lac, float gain) const {
        float sum = 0.0f, amp = 1.0f, norm = 0.0f;
        for (int o = 0; o < octaves; ++o) {
            sum = sum + amp * noise(x, y, z);
            norm = norm + amp;
            x = x * lac; y = y * lac; z = z * lac;
            amp = amp * gain;
        }
        return sum / norm;
    }
};

static float clamp01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }

std::vector<float> procedural_density(const vr_procedural_desc& d) {
    const int R = d.res;
    std::vector<float> g((size_t)R * R * R, 0.0f);
    Perlin pn(d.seed);
    const float inv = 1.0f / (float)R;
    parallel_for(R, [&](int z) {
        for (int y = 0; y < R; ++y)
            for (int x = 0; x < R; ++x) {
                // voxel centre in the unit cube
                float ux = ((float)x + 0.5f) * inv, uy = ((float)y + 0.5f) * inv, uz = ((float)z + 0.5f) * inv;
                float n = pn.fbm(ux * d.base_frequency + 0.37f, uy * d.base_frequency + 1.91f,
                                 uz * d.base_frequency + 4.13f, d.octaves, d.lacunarity, d.gain);
                float dx = ux - 0.5f, dy = uy - 0.5f, dz = uz - 0.5f;
                float r = sqrt_(dx * dx + dy * dy + dz * dz);
                float v;
                if (d.kind == 0) {
                    // fBm remapped to [0,1] times a smooth sphere mask of radius mask_radius
                    float t = clamp01((d.mask_radius - r) / 0.08f);
                    float mask = t * t * (3.0f - 2.0f * t);
                    v = clamp01(n * 1.25f + 0.5f) * mask;
                } else {
                    // fBm rescaled by 2.6 so it spans about [-1, 1], thresholded and remapped to
                    // [0,1], confined to the inscribed ball (threshold 0.35 occupies ~15% of bricks)
                    float t = clamp01((0.5f - r) / 0.1f);
                    float mask = t * t * (3.0f - 2.0f * t);
                    float sgl = n * 2.6f;
                    v = clamp01((sgl - d.threshold) / (1.0f - d.threshold)) * mask;
                }
                g[((size_t)z * R + y) * R + x] = v;
            }
    });
    return g;
}

// Fire plume: a vertical column whose radius grows with height, fBm turbulence, density
// falling off with height; the temperature follows the same turbulence, hottest at the base,
// in [t_min, t_max] inside the plume and 0 outside.
void procedural_fire(const vr_procedural_desc& d, float t_min, float t_max, std::vector<float>& density, std::vector<float>& temperature) {
    const int R = d.res;
    density.assign((size_t)R * R * R, 0.0f);
    temperature.assign((size_t)R * R * R, 0.0f);
    Perlin pn(d.seed);
    const float inv = 1.0f / (float)R;
    parallel_for(R, [&](int z) {
        for (int y = 0; y < R; ++y)
            for (int x = 0; x < R; ++x) {
                float ux = ((float)x + 0.5f) * inv, uy = ((float)y + 0.5f) * inv, uz = ((float)z + 0.5f) * inv;
                float n = pn.fbm(ux * d.base_frequency + 0.37f, uy * d.base_frequency * 0.7f + 1.91f,
                                 uz * d.base_frequency + 4.13f, d.octaves, d.lacunarity, d.gain);
                float dx = ux - 0.5f, dz = uz - 0.5f;
                float dist = sqrt_(dx * dx + dz * dz);
                float rad = 0.08f + 0.25f * uy + 0.05f * n;
                float t = clamp01((rad - dist) / 0.06f) * clamp01((0.92f - uy) / 0.08f) * clamp01((uy - 0.02f) / 0.03f);
                float env = t * t * (3.0f - 2.0f * t);
                if (env <= 0.f) continue;
                size_t i = ((size_t)z * R + y) * R + x;
                density[i] = clamp01(0.6f + 0.8f * n) * env * exp_(-2.5f * uy);
                temperature[i] = t_min + (t_max - t_min) * clamp01(0.75f + 0.9f * n) * clamp01(1.05f - 0.8f * uy);
            }
    });
}

// ---------------------------------------------------------------------------------------
// mip pyramids (gvdb_volume_gvdb.cpp:2702-2862)
// ---------------------------------------------------------------------------------------
// 2x box downsample for even dimensions: res += wi*wj*wk*density with all weights 0.5, the
// (x, y, z) loop order of the converter; kept only where positive.
static std::vector<float> downsample(const std::vector<float>& src, int R) {
    int H = R / 2;
    std::vector<float> dst((size_t)H * H * H, 0.0f);
    parallel_for(H, [&](int k) {
        for (int j = 0; j < H; ++j)
            for (int i = 0; i < H; ++i) {
                float res = 0.0f;
                for (int ii = 0; ii < 2; ++ii)
                    for (int jj = 0; jj < 2; ++jj)
                        for (int kk = 0; kk < 2; ++kk) {
                            float dv = src[((size_t)(2 * k + kk) * R + (2 * j + jj)) * R + (2 * i + ii)];
                            res += 0.5f * 0.5f * 0.5f * dv;
                        }
                dst[((size_t)k * H + j) * H + i] = res > 0.0f ? res : 0.0f;
            }
    });
    return dst;
}

// Conservative mip 0: an empty voxel takes the sum of the positive values of its 27
// neighbours divided by 27 (gvdb_volume_gvdb.cpp:2753-2800).
static std::vector<float> conservative0(const std::vector<float>& src, int R) {
    std::vector<float> dst(src);
    parallel_for(R, [&](int k) {
        for (int j = 0; j < R; ++j)
            for (int i = 0; i < R; ++i) {
                if (src[((size_t)k * R + j) * R + i] != 0.0f) continue;
                float avg = 0.0f;
                for (int ii = -1; ii <= 1; ++ii)
                    for (int jj = -1; jj <= 1; ++jj)
                        for (int kk = -1; kk <= 1; ++kk) {
                            int x = i + ii, y = j + jj, z = k + kk;
                            if (x < 0 || y < 0 || z < 0 || x >= R || y >= R || z >= R) continue;
                            float tap = src[((size_t)z * R + y) * R + x];
                            avg += tap > 0.0f ? tap : 0.0f;
                        }
                avg /= 27.0f;
                if (avg > 0.0f) dst[((size_t)k * R + j) * R + i] = avg;
            }
    });
    return dst;
}

// ---------------------------------------------------------------------------------------
// brick grid for one slot
// ---------------------------------------------------------------------------------------
// signedValues: any nonzero voxel makes its brick active and values are stored as given
// (velocity components); otherwise only positive voxels count (densities, temperatures)
static void build_slot(GridSlot& s, const std::vector<float>& g, int R, const float wmin[3],
                       float vsize, bool fp16, bool signedValues = false) {
    s.valid = 1;
    s.res = R;
    const int NB = R / 8;                    // bricks per axis
    const int NL = (R + 127) / 128;          // level-1 nodes per axis
    // max value of the slot's grid (mGridValMax)
    float maxv = 0.0f;
    for (float v : g) maxv = std::max(maxv, v);
    s.max_value = maxv;
    // which bricks are active (any voxel > 0)
    std::vector<int32_t> brickId((size_t)NB * NB * NB, -1);
    std::vector<uint8_t> active((size_t)NB * NB * NB, 0);
    parallel_for(NB, [&](int bz) {
        for (int by = 0; by < NB; ++by)
            for (int bx = 0; bx < NB; ++bx) {
                bool any = false;
                for (int z = 0; z < 8 && !any; ++z)
                    for (int y = 0; y < 8 && !any; ++y)
                        for (int x = 0; x < 8; ++x)
                            if (signedValues ? g[((size_t)(bz * 8 + z) * R + (by * 8 + y)) * R + (bx * 8 + x)] != 0.0f
                                             : g[((size_t)(bz * 8 + z) * R + (by * 8 + y)) * R + (bx * 8 + x)] > 0.0f) { any = true; break; }
                active[((size_t)bz * NB + by) * NB + bx] = any ? 1 : 0;
            }
    });
    // level-1 nodes and brick ids in (l1 node, z, y, x) order
    s.root_child.assign(32 * 32 * 32, -1);
    s.l1_vmin.clear(); s.l1_child.clear(); s.brick_vmin.clear();
    int nb = 0;
    for (int lz = 0; lz < NL; ++lz)
        for (int ly = 0; ly < NL; ++ly)
            for (int lx = 0; lx < NL; ++lx) {
                bool any = false;
                for (int bz = lz * 16; bz < std::min(NB, lz * 16 + 16) && !any; ++bz)
                    for (int by = ly * 16; by < std::min(NB, ly * 16 + 16) && !any; ++by)
                        for (int bx = lx * 16; bx < std::min(NB, lx * 16 + 16); ++bx)
                            if (active[((size_t)bz * NB + by) * NB + bx]) { any = true; break; }
                if (!any) continue;
                int l1 = (int)(s.l1_vmin.size() / 4);
                s.root_child[(lz * 32 + ly) * 32 + lx] = l1;
                s.l1_vmin.insert(s.l1_vmin.end(), {lx * 128, ly * 128, lz * 128, 0});
                size_t base = s.l1_child.size();
                s.l1_child.resize(base + 4096, -1);
                for (int cz = 0; cz < 16; ++cz)
                    for (int cy = 0; cy < 16; ++cy)
                        for (int cx = 0; cx < 16; ++cx) {
                            int bx = lx * 16 + cx, by = ly * 16 + cy, bz = lz * 16 + cz;
                            if (bx >= NB || by >= NB || bz >= NB) continue;
                            if (!active[((size_t)bz * NB + by) * NB + bx]) continue;
                            s.l1_child[base + (cz * 16 + cy) * 16 + cx] = nb;
                            brickId[((size_t)bz * NB + by) * NB + bx] = nb;
                            s.brick_vmin.insert(s.brick_vmin.end(), {bx * 8, by * 8, bz * 8, 0});
                            ++nb;
                        }
            }
    s.num_l1 = (int)(s.l1_vmin.size() / 4);
    s.num_bricks = nb;
    s.brick_bounds.assign((size_t)nb * 4, 0.0f);
    if (fp16) { s.brick_f16.assign((size_t)nb * 1000, 0); s.brick_f32.clear(); }
    else { s.brick_f32.assign((size_t)nb * 1000, 0.0f); s.brick_f16.clear(); }
    auto at = [&](int x, int y, int z) -> float {
        if (x < 0 || y < 0 || z < 0 || x >= R || y >= R || z >= R) return 0.0f;
        return g[((size_t)z * R + y) * R + x];
    };
    parallel_for(nb, [&](int b) {
        int vx = s.brick_vmin[b * 4 + 0], vy = s.brick_vmin[b * 4 + 1], vz = s.brick_vmin[b * 4 + 2];
        // density bounds over the 10^3 neighbourhood, sum / 512 (Scene.cpp:2983-3012)
        float sum = 0.0f, mn = FLT_MAX, mx = 0.0f;
        for (int i = -1; i <= 8; ++i)
            for (int j = -1; j <= 8; ++j)
                for (int k = -1; k <= 8; ++k) {
                    float dv = at(vx + i, vy + j, vz + k);
                    mn = std::min(mn, dv);
                    mx = std::max(mx, dv);
                    sum += dv;
                }
        s.brick_bounds[b * 4 + 0] = mn;
        s.brick_bounds[b * 4 + 1] = mx;
        s.brick_bounds[b * 4 + 2] = sum / 512.0f;
        s.brick_bounds[b * 4 + 3] = 0.0f;
        // voxels with apron; values tiny relative to the maximum are stored as 0
        // (Scene.cpp:3117-3119)
        for (int z = 0; z < 10; ++z)
            for (int y = 0; y < 10; ++y)
                for (int x = 0; x < 10; ++x) {
                    float v = at(vx + x - 1, vy + y - 1, vz + z - 1);
                    if (!signedValues && maxv > 0.0f && (double)(v / maxv) < 1e-9) v = 0.0f;
                    size_t o = (size_t)b * 1000 + (z * 10 + y) * 10 + x;
                    if (fp16) s.brick_f16[o] = float_to_half(v);
                    else s.brick_f32[o] = v;
                }
    });
    // world -> index transform of this mip (row-vector convention)
    float vs = vsize;
    for (int k = 0; k < 16; ++k) s.world_to_index[k] = 0.0f;
    float inv = 1.0f / vs;
    s.world_to_index[0] = inv; s.world_to_index[5] = inv; s.world_to_index[10] = inv;
    s.world_to_index[12] = -wmin[0] * inv;
    s.world_to_index[13] = -wmin[1] * inv;
    s.world_to_index[14] = -wmin[2] * inv;
    s.world_to_index[15] = 1.0f;
}

int build_signed_grid(const std::vector<float>& dense, int R, const float wmin[3], float vsize, bool fp16, Volume& vol) {
    if (R <= 0 || R % 8 != 0 || R > 4096) return 1;
    vol.res = R;
    vol.num_mips = 1;
    vol.voxel_size = vsize;
    vol.fp16 = fp16 ? 1 : 0;
    for (int i = 0; i < 3; ++i) vol.world_min[i] = wmin[i];
    vol.supervoxel_diag = 8.0f * sqrt_(vsize * vsize + vsize * vsize + vsize * vsize);
    for (auto& s : vol.slots) s = GridSlot();
    build_slot(vol.slots[0], dense, R, wmin, vsize, fp16, true);
    return 0;
}

int build_volume(const std::vector<float>& dense, int R, int numMips, const float wmin[3],
                 float vsize, bool fp16, Volume& vol) {
    if (R <= 0 || numMips < 1 || numMips > 8) return 1;
    if (R % (8 << (numMips - 1)) != 0) return 1;
    if (R > 4096) return 1;
    vol.res = R;
    vol.num_mips = numMips;
    vol.voxel_size = vsize;
    vol.fp16 = fp16 ? 1 : 0;
    for (int i = 0; i < 3; ++i) vol.world_min[i] = wmin[i];
    // superVoxelWorldSpaceDiagonalLength = 8 * sqrt(|row0|^2 + |row1|^2 + |row2|^2) of the
    // index->model transform of mip 0 (Scene.cpp:3076-3080)
    vol.supervoxel_diag = 8.0f * sqrt_(vsize * vsize + vsize * vsize + vsize * vsize);
    for (auto& s : vol.slots) s = GridSlot();
    std::vector<float> normal = dense, cons;
    int r = R;
    float vs = vsize;
    for (int m = 0; m < numMips; ++m) {
        if (m == 0) cons = conservative0(normal, r);
        else {
            normal = downsample(normal, r * 2);
            cons = downsample(cons, r * 2);
        }
        build_slot(vol.slots[m], normal, r, wmin, vs, fp16);
        build_slot(vol.slots[8 + m], cons, r, wmin, vs, fp16);
        r /= 2;
        vs = vs * 2.0f;
    }
    return 0;
}

// ---------------------------------------------------------------------------------------
// BC4 brick form (Scene.cpp:3161-3181, ATLAS_COMPRESSION 2).  The encoder is this project's
// own: endpoints from the block's extremes (floor of the minimum, ceiling of the maximum, in
// 1/255 steps), the six-value palette when the block holds an exact 0 or 1 (so those stay
// exact, as the reference's encoder arranges) or when the extremes round to one code, the
// eight-value palette otherwise; each texel takes the nearest palette entry.  For the
// conservative grids a nonzero texel never takes a zero entry (the reference's
// FindClosestUNORMConservative keeps nonzero texels nonzero, BCHelper.cpp:229-299), so distance
// sampling on them still reaches every occupied voxel.  Padding texels (x or y of 10, 11) take
// index 0 and do not take part in the endpoints.
// ---------------------------------------------------------------------------------------
float bc4_decode(uint64_t block, int texel) { return bc4_decode2((uint32_t)block, (uint32_t)(block >> 32), texel); }

static uint64_t bc4_encode_block(const float u[16], const bool used[16], bool conservative) {
    bool any = false, has0 = false, has1 = false, anyIn = false;
    float lo = 1.0f, hi = 0.0f, loIn = 1.0f, hiIn = 0.0f;
    for (int t = 0; t < 16; ++t) {
        if (!used[t]) continue;
        const float v = u[t];
        any = true;
        has0 |= v == 0.0f;
        has1 |= v == 1.0f;
        lo = std::min(lo, v);
        hi = std::max(hi, v);
        if (v > 0.0f && v < 1.0f) { anyIn = true; loIn = std::min(loIn, v); hiIn = std::max(hiIn, v); }
    }
    auto code_lo = [](float v) { return (uint32_t)std::min(255.0f, std::floor(255.0f * v)); };
    auto code_hi = [](float v) { return (uint32_t)std::min(255.0f, std::ceil(255.0f * v)); };
    uint32_t r0 = 0, r1 = 0;
    if (!any) {
        r0 = r1 = 0;
    } else if (has0 || has1) {
        r0 = anyIn ? code_lo(loIn) : 0u;                 // r0 <= r1: six-value palette with 0 and 1
        r1 = anyIn ? code_hi(hiIn) : 0u;
    } else {
        const uint32_t a = code_lo(lo), b = code_hi(hi);
        if (b > a) { r0 = b; r1 = a; }                   // eight-value palette
        else { r0 = r1 = a; }
    }
    uint64_t w = (uint64_t)r0 | ((uint64_t)r1 << 8);
    float pal[8];
    for (uint32_t i = 0; i < 8; ++i) pal[i] = bc4_palette(r0, r1, i);
    for (int t = 0; t < 16; ++t) {
        uint32_t best = 0;
        if (used[t]) {
            float bestD = FLT_MAX;
            for (uint32_t i = 0; i < 8; ++i) {
                if (conservative && u[t] > 0.0f && pal[i] == 0.0f) continue;
                const float d = std::fabs(pal[i] - u[t]);
                if (d < bestD) { bestD = d; best = i; }
            }
        }
        w |= (uint64_t)best << (16 + 3 * t);
    }
    return w;
}

void compress_slot_bc4(GridSlot& s, bool conservative) {
    if (!s.valid || !s.brick_bc4.empty()) return;
    const int nb = s.num_bricks;
    auto src = [&](size_t o) { return s.brick_f32.empty() ? half_to_float(s.brick_f16[o]) : s.brick_f32[o]; };
    float scale = 0.0f;
    for (size_t o = 0; o < (size_t)nb * 1000; ++o) scale = std::max(scale, src(o));
    s.bc4_scale = scale;
    s.brick_bc4.assign((size_t)nb * kBc4BlocksPerBrick, 0);
    parallel_for(nb, [&](int b) {
        const size_t base = (size_t)b * 1000;
        for (int z = 0; z < 10; ++z)
            for (int by = 0; by < 3; ++by)
                for (int bx = 0; bx < 3; ++bx) {
                    float u[16];
                    bool used[16];
                    for (int t = 0; t < 16; ++t) {
                        const int x = bx * 4 + (t & 3), y = by * 4 + (t >> 2);
                        used[t] = x < 10 && y < 10;
                        const float v = used[t] ? src(base + (size_t)(z * 10 + y) * 10 + x) : 0.0f;
                        u[t] = scale > 0.0f ? std::min(1.0f, std::max(0.0f, v / scale)) : 0.0f;
                    }
                    s.brick_bc4[(size_t)b * kBc4BlocksPerBrick + bc4_block(bx * 4, by * 4, z)] = bc4_encode_block(u, used, conservative);
                }
        // bounds of the decoded values over the same 10^3 box as build_slot, sum / 512
        float mn = FLT_MAX, mx = 0.0f, sum = 0.0f;
        for (int z = 0; z < 10; ++z)
            for (int y = 0; y < 10; ++y)
                for (int x = 0; x < 10; ++x) {
                    const float v = bc4_decode(s.brick_bc4[(size_t)b * kBc4BlocksPerBrick + bc4_block(x, y, z)], bc4_texel(x, y)) * scale;
                    mn = std::min(mn, v);
                    mx = std::max(mx, v);
                    sum += v;
                }
        s.brick_bounds[(size_t)b * 4 + 0] = mn;
        s.brick_bounds[(size_t)b * 4 + 1] = mx;
        s.brick_bounds[(size_t)b * 4 + 2] = sum / 512.0f;
    });
    s.brick_f32.clear(); s.brick_f32.shrink_to_fit();
    s.brick_f16.clear(); s.brick_f16.shrink_to_fit();
}

void slot_view(const GridSlot& s, vr_grid_view* v) {
    memset(v, 0, sizeof(*v));
    v->valid = s.valid;
    if (!s.valid) return;
    for (int i = 0; i < 3; ++i) { v->res[i] = s.res; v->bmin[i] = 0.0f; v->bmax[i] = (float)s.res; }
    memcpy(v->world_to_index, s.world_to_index, sizeof(v->world_to_index));
    v->max_value = s.max_value;
    v->num_l1 = s.num_l1;
    v->num_bricks = s.num_bricks;
    v->root_child = s.root_child.data();
    v->l1_vmin = s.l1_vmin.data();
    v->l1_child = s.l1_child.data();
    v->brick_vmin = s.brick_vmin.data();
    v->brick_bounds = s.brick_bounds.data();
    v->brick_f32 = s.brick_f32.empty() ? nullptr : s.brick_f32.data();
    v->brick_f16 = s.brick_f16.empty() ? nullptr : s.brick_f16.data();
    v->brick_bc4 = s.brick_bc4.empty() ? nullptr : s.brick_bc4.data();
    v->bc4_scale = s.bc4_scale;
}

// ---------------------------------------------------------------------------------------
// blackbody colour table for volume emission: Planck's law B(lambda, T) integrated over
// 360..830 nm (1 nm steps) against the CIE 1931 colour-matching functions in the multi-lobe
// Gaussian fit of Wyman, Sloan and Shirley ("Simple Analytic Approximations to the CIE XYZ
// Color Matching Functions", JCGT 2013), then XYZ -> linear sRGB (D65) and normalised to unit
// luminance at the last entry.  Entry i is T = 50 + 50 i kelvin (the texel centres of a
// 128-texel table over [25, 6425) K).
// ---------------------------------------------------------------------------------------
static double lobe(double l, double mu, double s1, double s2) {
    const double t = (l - mu) / (l < mu ? s1 : s2);
    return std::exp(-0.5 * t * t);
}
void blackbody_lut(float rgb[384]) {
    const double h = 6.62607015e-34, c = 2.99792458e8, kB = 1.380649e-23;
    double X[128], Y[128], Z[128];
    for (int i = 0; i < 128; ++i) {
        const double T = 50.0 + 50.0 * i;
        double x = 0, y = 0, z = 0;
        for (int nm = 360; nm <= 830; ++nm) {
            const double l = nm * 1e-9;
            const double B = 2.0 * h * c * c / (l * l * l * l * l) / std::expm1(h * c / (l * kB * T));
            const double xb = 1.056 * lobe(nm, 599.8, 37.9, 31.0) + 0.362 * lobe(nm, 442.0, 16.0, 26.7) - 0.065 * lobe(nm, 501.1, 20.4, 26.2);
            const double yb = 0.821 * lobe(nm, 568.8, 46.9, 40.5) + 0.286 * lobe(nm, 530.9, 16.3, 31.1);
            const double zb = 1.217 * lobe(nm, 437.0, 11.8, 36.0) + 0.681 * lobe(nm, 459.0, 26.0, 13.8);
            x += B * xb; y += B * yb; z += B * zb;
        }
        X[i] = x; Y[i] = y; Z[i] = z;
    }
    const double norm = 1.0 / Y[127];
    for (int i = 0; i < 128; ++i) {
        const double x = X[i] * norm, y = Y[i] * norm, z = Z[i] * norm;
        const double r = 3.2406 * x - 1.5372 * y - 0.4986 * z;
        const double g = -0.9689 * x + 1.8758 * y + 0.0415 * z;
        const double b = 0.0557 * x - 0.2040 * y + 1.0570 * z;
        rgb[3 * i + 0] = (float)std::max(r, 0.0);
        rgb[3 * i + 1] = (float)std::max(g, 0.0);
        rgb[3 * i + 2] = (float)std::max(b, 0.0);
    }
}

}  // namespace vr
