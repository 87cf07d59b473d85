// frame_kernels.cu -- instantiates the frame-loop kernels for one maximum path length.
// Compiled once per VR_MB in {1, 2, 3, 4} so the four variants build in parallel; each
// object has its own copy of the scene constants, uploaded by upload_scene_<MB>.
//
// With VR_LOW_OCC = n it instead builds the per-pixel kernels of the initial and spatial passes
// (plain and learned) at a budget of n blocks per SM, for frames too small to fill the GPU at
// full occupancy (the *_lo_<MB> entry points).  Each budget sits in its own object, so the
// register classes of the shared device functions in either object are the same as when it is
// built alone.
#include <cuda_runtime.h>

#include "vr_kernels.cuh"
#include "vr_lp_kernels.cuh"

#ifndef VR_MB
#error "VR_MB must be defined (1..4)"
#endif
#define VR_CAT2(a, b) a##b
#define VR_CAT(a, b) VR_CAT2(a, b)

#ifdef VR_LOW_OCC
namespace vrk {

#define VR_LO(name) VR_CAT(VR_CAT(name, lo_), VR_MB)
cudaError_t VR_LO(upload_scene_)(const vrd::DevScene& s, cudaStream_t st) {
    return cudaMemcpyToSymbolAsync(vrd::c_scene, &s, sizeof(vrd::DevScene), 0, cudaMemcpyHostToDevice, st);
}
void VR_LO(launch_initial_)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_initial<VR_MB, VR_LOW_OCC><<<g, b, 0, st>>>(P, B);
}
void VR_LO(launch_spatial_)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::SpatialParams& S, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_spatial<VR_MB, VR_LOW_OCC><<<g, b, 0, st>>>(P, B, S);
}
void VR_LO(launch_lp_generate_)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::LpBuffers& L, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_lp_generate<VR_MB, VR_LOW_OCC><<<g, b, 0, st>>>(P, B, L);
}
void VR_LO(launch_lp_select_)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::LpBuffers& L, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_lp_select<VR_MB, VR_LOW_OCC><<<g, b, 0, st>>>(P, B, L);
}
#undef VR_LO

}  // namespace vrk
#else
namespace vrk {

cudaError_t VR_CAT(upload_scene_, VR_MB)(const vrd::DevScene& s, cudaStream_t st) {
    return cudaMemcpyToSymbolAsync(vrd::c_scene, &s, sizeof(vrd::DevScene), 0, cudaMemcpyHostToDevice, st);
}
void VR_CAT(launch_initial_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_initial<VR_MB><<<g, b, 0, st>>>(P, B);
}
void VR_CAT(launch_spatial_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::SpatialParams& S, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_spatial<VR_MB><<<g, b, 0, st>>>(P, B, S);
}
void VR_CAT(launch_final_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, int writeHist, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_final<VR_MB><<<g, b, 0, st>>>(P, B, writeHist);
}
void VR_CAT(launch_reference_, VR_MB)(const vrd::FrameParams& P, int first, int count, double* accum, dim3 g, dim3 b, cudaStream_t st) {
    vrd::k_reference<VR_MB><<<g, b, 0, st>>>(P, first, count, accum);
}

void VR_CAT(launch_lp_generate_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::LpBuffers& L, dim3 g, dim3 b,
                                        cudaStream_t st) {
    vrd::k_lp_generate<VR_MB><<<g, b, 0, st>>>(P, B, L);
}
void VR_CAT(launch_lp_select_, VR_MB)(const vrd::FrameParams& P, const vrd::FrameBuffers& B, const vrd::LpBuffers& L, dim3 g, dim3 b,
                                      cudaStream_t st) {
    vrd::k_lp_select<VR_MB><<<g, b, 0, st>>>(P, B, L);
}
void VR_CAT(launch_lp_train_gen_, VR_MB)(const vrd::FrameParams& P, const vrd::LpBuffers& L, uint32_t seed, cudaStream_t st) {
    vrd::k_lp_train_gen<VR_MB><<<(L.trainCount + 127) / 128, 128, 0, st>>>(P, L, seed);
}

}  // namespace vrk
#endif
