// vr_bc4.h -- the BC4 (unsigned) block form of brick storage, shared by the kernels and the
// host library.
//
// The reference stores its coarse density mips and its conservative mips as BC4 textures
// (Scene.cpp:3161-3181 with ATLAS_COMPRESSION 2; the block layout of BCHelper.h:9-69) and lets
// the texture unit decode them.  Here a brick's 10^3 voxels (8^3 and an apron of one) are ten
// z-slices of 10 x 10 texels, each cut into 3 x 3 blocks of 4 x 4 texels (the last row and
// column of blocks half padding): 90 blocks, 720 bytes per brick against 2000 (FP16) or 4000
// (FP32).
//
// A block is one little-endian 64-bit word: bits 0-7 red_0, bits 8-15 red_1, then a 3-bit
// palette index per texel (texel t = 4 y + x at bits 16 + 3 t).  red_0 > red_1 selects the
// eight-value palette (red_0, red_1 and six interpolants), otherwise the six-value one (red_0,
// red_1, four interpolants, 0 and 1).  The decoded unorm value is the integer numerator of the
// palette entry over 255 * 7 (or 255 * 5) times that denominator's reciprocal rounded to float,
// so that every decoder of this project gives the same bits; the density is that value times
// the slot's scale.
#pragma once

#include <stdint.h>

#include "vr_math.h"

namespace vr {

constexpr int kBc4BlocksPerBrick = 90;
constexpr float kBc4Inv8 = 1.0f / 1785.0f;     // 1 / (255 * 7)
constexpr float kBc4Inv6 = 1.0f / 1275.0f;     // 1 / (255 * 5)

// block of apron coordinates (x, y, z) in [0, 10)^3 within its brick, and texel in the block
VR_HD int bc4_block(int x, int y, int z) { return z * 9 + (y >> 2) * 3 + (x >> 2); }
VR_HD int bc4_texel(int x, int y) { return ((y & 3) << 2) | (x & 3); }

// palette entry idx of a block with endpoints r0, r1: numerator w0 r0 + w1 r1 (+ 1275 for the
// six-value palette's entry 7), the weights read from nibble tables (entry idx at bits 4 idx),
// so that the decode has no branches
VR_HD float bc4_palette(uint32_t r0, uint32_t r1, uint32_t idx) {
    const bool eight = r0 > r1;
    const uint32_t t0 = eight ? 0x12345607u : 0x00123405u;    // w0: 7 0 6 5 4 3 2 1 / 5 0 4 3 2 1 0 0
    const uint32_t t1 = eight ? 0x65432170u : 0x00432150u;    // w1: 0 7 1 2 3 4 5 6 / 0 5 1 2 3 4 0 0
    const uint32_t w0 = (t0 >> (4u * idx)) & 15u, w1 = (t1 >> (4u * idx)) & 15u;
    const uint32_t num = w0 * r0 + w1 * r1 + ((!eight && idx == 7u) ? 1275u : 0u);
    return (float)num * (eight ? kBc4Inv8 : kBc4Inv6);
}

// the two 32-bit halves of a block (lo = bits 0-31)
VR_HD float bc4_decode2(uint32_t lo, uint32_t hi, int texel) {
    const uint64_t w = ((uint64_t)hi << 32) | lo;
    const uint32_t idx = (uint32_t)(w >> (16 + 3 * texel)) & 7u;
    return bc4_palette(lo & 255u, (lo >> 8) & 255u, idx);
}

}  // namespace vr
