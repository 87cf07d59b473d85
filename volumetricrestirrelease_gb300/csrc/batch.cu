// batch.cu -- persistent batched frame kernels: one launch per pass renders the pixels of many
// independent instances (own volume, view, resolution, options and buffers).  Compiled once per
// maximum path length with VR_BATCHED, so the scene constants live in shared memory: each block
// walks a strided slice of one list of pixel tiles over all instances and, whenever its tile
// belongs to another instance, loads that instance's scene, frame parameters and buffer views
// into shared memory.  The per-pixel work is the same code as the single-instance kernels, so
// every pixel is bit-identical to rendering its instance alone; only the grid and the tile
// shape (chosen by the autotuner) differ.
#include <cuda_runtime.h>

#include "vr_batch_kernels.cuh"

#ifndef VR_MB
#error "VR_MB must be defined (1..4)"
#endif
#define VR_CAT2(a, b) a##b
#define VR_CAT(a, b) VR_CAT2(a, b)
namespace vrk {

// pass: 0 initial, 1 generate, 2 select, 3 spatial, 4 final
void VR_CAT(launch_batch_pass_, VR_MB)(const vrd::BatchLaunch& BL, int pass, int grid, cudaStream_t st) {
    switch (pass) {
        case 0: vrd::kb_pixels<VR_MB, vrd::kPassInitial><<<grid, 128, 0, st>>>(BL); break;
        case 1: vrd::kb_pixels<VR_MB, vrd::kPassGenerate><<<grid, 128, 0, st>>>(BL); break;
        case 2: vrd::kb_pixels<VR_MB, vrd::kPassSelect><<<grid, 128, 0, st>>>(BL); break;
        case 3: vrd::kb_pixels<VR_MB, vrd::kPassSpatial><<<grid, 128, 0, st>>>(BL); break;
        default: vrd::kb_pixels<VR_MB, vrd::kPassFinal><<<grid, 128, 0, st>>>(BL); break;
    }
}
// walk: point-sampled distances (the instance's initial visibility sampler), as resumable walks
void VR_CAT(launch_batch_lp_bounce_, VR_MB)(const vrd::BatchLaunch& BL, int inst, int b, int grid, int walk, cudaStream_t st) {
    if (walk) {
        vrd::kb_lp_walk<VR_MB><<<grid, 128, 0, st>>>(BL, inst, b);
        vrd::kb_lp_vertex<VR_MB><<<grid, 128, 0, st>>>(BL, inst, b);
    } else {
        vrd::kb_lp_bounce<VR_MB><<<grid, 128, 0, st>>>(BL, inst, b);
    }
}
void VR_CAT(launch_batch_train_gen_, VR_MB)(const vrd::BatchLaunch& BL, int grid, cudaStream_t st) {
    vrd::kb_train_gen<VR_MB><<<grid, 128, 0, st>>>(BL);
}

}  // namespace vrk
