// vro_volume.cpp -- input volumes for the oracle without the GPU library (test infrastructure).
//
// The CPU baseline and the reference arm of the benchmark build their procedural input grid
// here, so that they run with the oracle's own library only.  The grid builder itself
// (procedural fBm, the normal and conservative mip pyramids, the 8^3 bricks with their apron,
// the brick bounds) is the same source file the GPU library compiles, built into this library
// a second time: both sides must render the same input, and the builder's rules are checked on
// their own against a numpy restatement by the volume tests.
#include "../volumetricrestirrelease_gb300/csrc/vr_volume.h"

#include <new>

extern "C" {

void* vro_volume_procedural(const vr_procedural_desc* d) {
    if (!d || d->res <= 0 || d->res > 4096 || d->num_mips < 1 || d->num_mips > VR_NUM_MAX_MIPS) return nullptr;
    if (d->res % (8 << (d->num_mips - 1)) != 0 || !(d->voxel_size > 0.f)) return nullptr;
    try {
        std::vector<float> g = vr::procedural_density(*d);
        vr_volume* v = new vr_volume();
        if (vr::build_volume(g, d->res, d->num_mips, d->world_min, d->voxel_size, d->fp16 != 0, v->v) != 0) {
            delete v;
            return nullptr;
        }
        return v;
    } catch (...) {
        return nullptr;
    }
}

int vro_volume_info(const void* h, vr_volume_info* info) {
    if (!h || !info) return VR_ERR_INVALID_ARG;
    const vr::Volume& v = ((const vr_volume*)h)->v;
    *info = vr_volume_info();
    info->num_mips = v.num_mips;
    info->res = v.res;
    info->voxel_size = v.voxel_size;
    info->supervoxel_diag = v.supervoxel_diag;
    info->fp16 = v.fp16;
    info->bc4 = v.bc4;
    for (int i = 0; i < 3; ++i) info->world_min[i] = v.world_min[i];
    for (int s = 0; s < VR_NUM_SLOTS; ++s) info->num_bricks[s] = v.slots[s].num_bricks;
    return VR_OK;
}

int vro_volume_slot(const void* h, int slot, vr_grid_view* view) {
    if (!h || !view || slot < 0 || slot >= VR_NUM_SLOTS) return VR_ERR_INVALID_ARG;
    vr::slot_view(((const vr_volume*)h)->v.slots[slot], view);
    return VR_OK;
}

void vro_volume_destroy(void* h) { delete (vr_volume*)h; }

}  // extern "C"
