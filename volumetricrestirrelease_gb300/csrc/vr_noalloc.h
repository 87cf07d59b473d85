// vr_noalloc.h -- internal interface between context.cu and noalloc.cu (the allocation-free
// frame entry point).
#pragma once
#include "../../include/vrestir.h"
#include "vr_kernels.cuh"

namespace vrk {
constexpr int64_t kNoAllocMaxPixels = 65536;   // e.g. 256 x 256
constexpr int kNoAllocMaxBounces = 2;

struct NoAllocFrame {
    vrd::FrameParams P;
    const vrd::DevScene* scene;
    int W, H, maxBounces, spatial, rounds;
    vrd::SpatialParams S[16];
};
// Checks the context's options and size against the static scratch and fills the launch
// parameters of one history-free frame; allocates nothing and changes no context state.
int noalloc_prepare(vr_context* c, const vr_camera* cam, int32_t frame_index, NoAllocFrame* f);
void noalloc_error(vr_context* c, const char* msg);
}  // namespace vrk
