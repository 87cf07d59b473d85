// noalloc.cu -- vr_render_frame_noalloc: one frame without temporal history whose per-pixel
// intermediates (features, reservoirs, path suffixes, the spatial ping-pong buffer) live in a
// fixed static device array instead of buffers the library allocates.
//
// Who needs it: callers that must not allocate GPU memory at render time -- hosts that hand
// out a fixed memory budget up front and forbid later allocations (an engine or plugin host
// that owns the device heap), and real-time loops where a cudaMalloc, which can synchronise
// the whole device, would stall a frame.  The scene (volume, lights) must already be bound to
// the context, which is done once at set-up.
//
// Limits and behaviour:
//   * at most 65536 pixels (for example 256 x 256) and max path length 2; temporal reuse,
//     the reference mode and the learned target must be off (there is no history to keep
//     between calls and no room for the learned target's records);
//   * the scratch array is about 6.3 MiB and every GPU that loads the library holds it until
//     the process exits;
//   * every call on a device shares the one array and it keeps the last call's contents, so
//     each call clears the part it reads before writing; calls whose work overlaps on the GPU
//     (two streams, two host threads) race on it and must be serialised by the caller; they
//     also share this file's copy of the scene constants, which each call rewrites;
//   * the first call on each device looks up the array's device address (cudaGetSymbolAddress,
//     with that device current); make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "vr_noalloc.h"

namespace {

// scratch layout for N = 65536 pixels: two reservoir buffers (a, b, one suffix plane each) and
// the feature buffer, each region 256-byte aligned
constexpr size_t kN = (size_t)vrk::kNoAllocMaxPixels;
constexpr size_t kRegion = kN * 16;                 // float4 / int4 per pixel
constexpr size_t kScratchBytes = 6 * kRegion + kN * 4;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_setup_mutex;

// Device address of the scratch array for the current device; looked up once per device.
cudaError_t scratch_for_current_device(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

template <int MB>
void launch(const vrk::NoAllocFrame& f, const vrd::FrameBuffers& B, cudaStream_t st) {
    dim3 grid((f.W + 7) / 8, (f.H + 15) / 16), block(128);
    vrd::k_initial<MB><<<grid, block, 0, st>>>(f.P, B);
    if (f.spatial) {
        for (int r = 0; r < f.rounds; ++r) vrd::k_spatial<MB><<<grid, block, 0, st>>>(f.P, B, f.S[r]);
    } else {
        vrd::k_final<MB><<<grid, block, 0, st>>>(f.P, B, 0);
    }
}

}  // namespace

extern "C" int vr_render_frame_noalloc(vr_context* ctx, const vr_camera* cam, int32_t frame_index,
                                       float* out_rgba_device, void* stream) {
    if (!ctx || !out_rgba_device) return VR_ERR_INVALID_ARG;
    vrk::NoAllocFrame f;
    int r = vrk::noalloc_prepare(ctx, cam, frame_index, &f);
    if (r != VR_OK) return r;
    void* base = nullptr;
    cudaError_t e = scratch_for_current_device(&base);
    if (e != cudaSuccess) {
        vrk::noalloc_error(ctx, "vr_render_frame_noalloc: cannot get the scratch address on this device");
        return VR_ERR_CUDA;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const size_t N = (size_t)f.W * f.H;
    unsigned char* s = (unsigned char*)base;
    vrd::FrameBuffers B;
    memset(&B, 0, sizeof(B));
    B.cur.a = (float4*)(s + 0 * kRegion);
    B.cur.b = (int4*)(s + 1 * kRegion);
    B.cur.extra = (float4*)(s + 2 * kRegion);
    B.sp[0] = B.cur;
    B.sp[1].a = (float4*)(s + 3 * kRegion);
    B.sp[1].b = (int4*)(s + 4 * kRegion);
    B.sp[1].extra = (float4*)(s + 5 * kRegion);
    B.hist = B.cur;                       // no history: never read or written (temporal off)
    B.featCur = (float*)(s + 6 * kRegion);
    B.featPrev = B.featCur;
    B.color = nullptr;
    B.out = (float4*)out_rgba_device;
    B.mvec = nullptr;
    // the array keeps the previous call's data: clear what this frame may read before writing
    // (the spatial buffer's suffix plane is read for pixels that keep their own reservoir)
    e = cudaMemsetAsync(B.sp[1].extra, 0, N * 16, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.cur.extra, 0, N * 16, st);
    if (e != cudaSuccess) { vrk::noalloc_error(ctx, "vr_render_frame_noalloc: clearing the scratch array failed"); return VR_ERR_CUDA; }
    e = cudaMemcpyToSymbolAsync(vrd::c_scene, f.scene, sizeof(vrd::DevScene), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { vrk::noalloc_error(ctx, "vr_render_frame_noalloc: scene upload failed"); return VR_ERR_CUDA; }
    if (f.maxBounces == 1) launch<1>(f, B, st);
    else launch<2>(f, B, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) { vrk::noalloc_error(ctx, cudaGetErrorString(e)); return VR_ERR_CUDA; }
    return VR_OK;
}
