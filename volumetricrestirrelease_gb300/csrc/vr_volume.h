// vr_volume.h -- host-side sparse brick grid (internal to libvrestir).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/vrestir.h"

namespace vr {

struct GridSlot {
    int valid = 0;
    int res = 0;
    float max_value = 0.0f;
    float world_to_index[16] = {};
    int num_l1 = 0, num_bricks = 0;
    std::vector<int32_t> root_child;   // 32^3
    std::vector<int32_t> l1_vmin;      // 4 per level-1 node
    std::vector<int32_t> l1_child;     // 4096 per level-1 node
    std::vector<int32_t> brick_vmin;   // 4 per brick
    std::vector<float> brick_bounds;   // 4 per brick
    std::vector<float> brick_f32;      // 1000 per brick
    std::vector<uint16_t> brick_f16;   // 1000 per brick
    std::vector<uint64_t> brick_bc4;   // 90 BC4 blocks per brick (10 z-slices x 3 x 3 blocks of 4x4)
    float bc4_scale = 0.0f;            // decoded unorm value x bc4_scale = density
};

struct Volume {
    int res = 0, num_mips = 0, fp16 = 0, bc4 = 0;
    float voxel_size = 0.0f, supervoxel_diag = 0.0f;
    float world_min[3] = {0, 0, 0};
    GridSlot slots[VR_NUM_SLOTS];
};

uint16_t float_to_half(float f);
float half_to_float(uint16_t h);
std::vector<float> procedural_density(const vr_procedural_desc& d);
// mip 0 only, values kept with their sign (bricks where any voxel is nonzero): velocity grids
int build_signed_grid(const std::vector<float>& dense, int R, const float wmin[3], float vsize, bool fp16, Volume& vol);
int build_volume(const std::vector<float>& dense, int R, int numMips, const float wmin[3],
                 float vsize, bool fp16, Volume& vol);
void slot_view(const GridSlot& s, vr_grid_view* v);
// BC4 form: the slot's bricks re-encoded as BC4 blocks, bounds recomputed from the decoded values
void compress_slot_bc4(GridSlot& s, bool conservative);
float bc4_decode(uint64_t block, int texel);
// GVDB .vbx files (vbx.cpp)
int read_vbx(const std::vector<unsigned char>& file, int numMips, bool fp16, bool signedValues, Volume& vol, std::string& err);
int write_vbx(const Volume& vol, std::vector<unsigned char>& out, std::string& err);
void blackbody_lut(float rgb[384]);
void procedural_fire(const vr_procedural_desc& d, float t_min, float t_max, std::vector<float>& density, std::vector<float>& temperature);

}  // namespace vr

struct vr_volume {
    vr::Volume v;
};
