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

// pass: 0 initial, 1 generate (features and rounds; kb_vertex0 builds the first vertices), 2 select, 3 spatial, 4 final, 5-7 the split spatial round's
// record, replay-and-record and round kernels
// grid: the SMs x the blocks per SM asked for, at most the blocks the pass is compiled to keep resident
void VR_CAT(launch_batch_pass_, VR_MB)(const vrd::BatchLaunch& BL, int pass, int numSMs, int blocksPerSM, cudaStream_t st) {
    const int grid = numSMs * (blocksPerSM < vrd::batchPassBlocks(pass) ? blocksPerSM : vrd::batchPassBlocks(pass));
    switch (pass) {
        case 0: vrd::kb_pixels<VR_MB, vrd::kPassInitial><<<grid, 128, 0, st>>>(BL); break;
        case 1: vrd::kb_pixels<VR_MB, vrd::kPassGenerate><<<grid, 128, 0, st>>>(BL); break;
        case 2: vrd::kb_pixels<VR_MB, vrd::kPassSelect><<<grid, 128, 0, st>>>(BL); break;
        case 3: vrd::kb_pixels<VR_MB, vrd::kPassSpatial><<<grid, 128, 0, st>>>(BL); break;
        case 5: vrd::kb_pixels<VR_MB, vrd::kPassSplitA><<<grid, 128, 0, st>>>(BL); break;
        case 6: vrd::kb_pixels<VR_MB, vrd::kPassSplitB><<<grid, 128, 0, st>>>(BL); break;
        case 7: vrd::kb_pixels<VR_MB, vrd::kPassSplitC><<<grid, 128, 0, st>>>(BL); break;
        default: vrd::kb_pixels<VR_MB, vrd::kPassFinal><<<grid, 128, 0, st>>>(BL); break;
    }
}
// the marches recorded by the split spatial round BL.round of every instance (their list
// counters were cleared before the recording pass)
void VR_CAT(launch_batch_split_march_, VR_MB)(const vrd::BatchLaunch& BL, int grid, cudaStream_t st) {
    vrd::kb_split_march<<<grid, 128, 0, st>>>(BL);
}
void VR_CAT(launch_batch_split_reset_, VR_MB)(const vrd::BatchLaunch& BL, cudaStream_t st) {
    vrd::kb_split_reset<<<(BL.numInst + 127) / 128, 128, 0, st>>>(BL);
}
// the bounce pass b of learned instance `inst` in one pass (linear sampler)
void VR_CAT(launch_batch_lp_bounce_, VR_MB)(const vrd::BatchLaunch& BL, int inst, int b, int grid, cudaStream_t st) {
    vrd::kb_lp_bounce<VR_MB><<<grid, 128, 0, st>>>(BL, inst, b);
}
// the bounce pass b of every walking instance: the walks, then the vertices
void VR_CAT(launch_batch_walk_all_, VR_MB)(const vrd::BatchLaunch& BL, int b, int grid, cudaStream_t st) {
    vrd::kb_lp_walk_all<VR_MB><<<grid, 128, 0, st>>>(BL, b);
    vrd::kb_lp_vertex_all<VR_MB><<<grid, 128, 0, st>>>(BL, b);
}
void VR_CAT(launch_batch_vertex0_, VR_MB)(const vrd::BatchLaunch& BL, int grid, cudaStream_t st) {
    vrd::kb_vertex0<VR_MB><<<grid, 128, 0, st>>>(BL);
}
void VR_CAT(launch_batch_train_gen_, VR_MB)(const vrd::BatchLaunch& BL, int grid, cudaStream_t st) {
    vrd::kb_train_gen<VR_MB><<<grid, 128, 0, st>>>(BL);
}

}  // namespace vrk
