// frame_kernels.cu -- instantiates the frame-loop kernels for one maximum path length.
// Compiled once per VR_MB in {1, 2, 3, 4} so the four variants build in parallel; each
// object has its own copy of the scene constants, uploaded by upload_scene_<MB>.
#include <cuda_runtime.h>

#include "vr_kernels.cuh"
#include "vr_lp_kernels.cuh"

#ifndef VR_MB
#error "VR_MB must be defined (1..4)"
#endif
#define VR_CAT2(a, b) a##b
#define VR_CAT(a, b) VR_CAT2(a, b)

namespace vrk {

cudaError_t VR_CAT(upload_scene_, VR_MB)(const vrd::DevScene& s, cudaStream_t st) {
    return cudaMemcpyToSymbolAsync(vrd::c_scene, &s, sizeof(vrd::DevScene), 0, cudaMemcpyHostToDevice, st);
}
void VR_CAT(launch_initial_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_initial<VR_MB><<<g, b, 0, st>>>(P, B);
}
void VR_CAT(launch_spatial_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::SpatialParams& S, dim3 g, dim3 b,
                                    const vrd::SpatialSplit* SS, int persistent, cudaStream_t st) {
    // the round with its marches split out when its options allow (the same result); else
    // the per-thread round
    if (SS && vrd::spatialSplitEligible(P)) {
        cudaMemsetAsync(SS->counts, 0, 2 * sizeof(int), st);
        vrd::k_split_a<VR_MB><<<g, b, 0, st>>>(P, B, S, *SS);
        vrd::k_split_march<<<persistent, 128, 0, st>>>(*SS);
        cudaMemsetAsync(SS->counts, 0, 2 * sizeof(int), st);
        vrd::k_split_b<VR_MB><<<g, b, 0, st>>>(P, B, S, *SS);
        vrd::k_split_march<<<persistent, 128, 0, st>>>(*SS);
        vrd::k_split_c<VR_MB><<<g, b, 0, st>>>(P, B, S, *SS);
    } else {
        vrd::k_spatial<VR_MB><<<g, b, 0, st>>>(P, B, S);
    }
}
void VR_CAT(launch_final_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, int writeHist, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_final<VR_MB><<<g, b, 0, st>>>(P, B, writeHist);
}
void VR_CAT(launch_reference_, VR_MB)(const vrd::FrameParams& P, int first, int count, double* accum, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_reference<VR_MB><<<g, b, 0, st>>>(P, first, count, accum);
}

void VR_CAT(launch_lp_generate_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::LpBuffers& L, dim3 g, dim3 b,
                                        cudaStream_t st) {
    vrd::k_lp_rounds<VR_MB><<<g, b, 0, st>>>(P, B, L);
    const size_t n = (size_t)P.initialM * (size_t)P.N;
    vrd::k_lp_vertex0<VR_MB><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(P, L);
}
void VR_CAT(launch_lp_select_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::LpBuffers& L, dim3 g, dim3 b,
                                      cudaStream_t st) {
    vrd::k_lp_select<VR_MB><<<g, b, 0, st>>>(P, B, L);
}
void VR_CAT(launch_lp_bounce_, VR_MB)(const vrd::FrameParams& P, const vrd::LpBuffers& L, int b, int grid, int sorted, cudaStream_t st) {
    // point-sampled distances of a sorted queue: the resumable walks, then the vertices
    if (sorted && !P.initial.visibilityUseLinearSampler) {
        vrd::k_lp_walk<VR_MB><<<grid, 128, 0, st>>>(P, L, b);
        vrd::k_lp_vertex<VR_MB><<<grid, 128, 0, st>>>(P, L, b);
    } else {
        vrd::k_lp_bounce<VR_MB><<<grid, 128, 0, st>>>(P, L, b, sorted);
    }
}
// counting sort of the queue of bounce b into L.psort
void VR_CAT(launch_lp_sort_, VR_MB)(const vrd::LpBuffers& L, int b, int grid, cudaStream_t st) {
    cudaMemsetAsync(L.hist, 0, vrd::kPathKeys * sizeof(int), st);
    vrd::k_path_hist<<<grid, 256, 0, st>>>(L, b);
    vrd::k_path_scan<<<1, 1024, 0, st>>>(L);
    vrd::k_path_scatter<<<grid, 256, 0, st>>>(L, b);
}
void VR_CAT(launch_lp_train_gen_, VR_MB)(const vrd::FrameParams& P, const vrd::LpBuffers& L, uint32_t seed, cudaStream_t st) {
    vrd::k_lp_train_gen<VR_MB><<<(L.trainCount + 127) / 128, 128, 0, st>>>(P, L, seed);
}

}  // namespace vrk
