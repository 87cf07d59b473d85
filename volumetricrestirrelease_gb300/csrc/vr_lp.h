// vr_lp.h -- device-side views of the learned target function (the transmittance network) and
// of the buffers of the split initial pass that uses it.
//
// With the learned target the initial pass runs in three steps so that the network is
// evaluated on the tensor cores in batches:
//   generate : every candidate path is sampled as in the plain pass, except that the light
//              visibility of each next-event estimate is not marched; the vertex's reservoir
//              fields, its resampling uniform and (where the target needs it) a transmittance
//              query (x, w, tmax, slot) are written out.  The first vertices come from one
//              per-pixel kernel, the indirect vertices from one pass per bounce over a queue of
//              the paths that go on (each candidate's indirect vertices use its own stream);
//   infer    : the network predicts T for the compacted list of query slots;
//   select   : the recorded candidates are resampled with p_hat = p_hat_unoccluded * T, then the
//              pass continues as the plain one (p_hat of the winner, temporal reuse).
// The random stream of a pixel does not depend on T: the resampling uniforms are drawn at
// generation time for every vertex and every candidate.
#pragma once

#include <stdint.h>

namespace vrd {

// coherence keys of the path-queue sort: ray octant x 8^3 origin cell
constexpr int kPathKeys = 4096;

struct NetView {
    const uint16_t* wbf;   // BF16 weights: 4 hidden matrices [64 out][64 in] then the 64 output weights
    const float* bias;     // FP32 biases: 4 x 64 hidden, then the output bias
    float bmin[3], binv[3];
    float floor_;          // lower clamp of the predicted transmittance
    int lossLog;           // training loss: 0 squared error of T, 1 squared error of log T
};

// vertex record flags
constexpr int kLpValid = 1;      // the vertex was processed (the plain pass resamples it)
constexpr int kLpNeedsT = 2;     // p_y = y * T and runningSum = p_y / x (x = p_src, y = unoccluded p_hat)
constexpr int kLpRRShift = 8;    // Russian-roulette terminations added to the candidate's M

struct LpBuffers {
    float4* vrecA;     // [M * MB][N]: runningSum (or p_src), p_y (or unoccluded p_hat), uv0, uv1
    int4* vrecB;       // [M * MB][N]: lightID, sampledPixel, flags, resampling uniform (bits)
    float2* crec;      // [M][N]: depth, candidate resampling uniform
    float4* dist;      // [M][N]: the candidate's primary distance sample: hit distance, pdf, Tr
    float4* ex;        // [M * (MB - 1)][N]: encoded direction / distance of each indirect vertex
    float* T;          // [M * MB][N]: predicted transmittance of the vertices with kLpNeedsT
    float4* query;     // [M * MB][N][2]: the query of each slot with kLpNeedsT: (x, y, z, wx), (wy, wz, tmax, slot bits)
    int* qlist;        // compacted list of the slots that hold a query (in arbitrary order)
    int* qcount;
    int qcapacity;
    uint4* rng;        // [N]: the pixel's random state after generation
    float4* paths[2];  // queues of continuing candidate paths, 4 float4 each (the bounce b queue is paths[b & 1])
    int* pcount;       // [MB]: queue lengths by bounce
    int* wcursor;      // [MB]: next entry of each queue for the resumable walks (k_lp_walk)
    int pcapacity;     // entries of each queue (M * N)
    float4* psort;     // a queue sorted by coherence key before its bounce pass (single-context frames)
    int* hist;         // [2][kPathKeys]: key counts, then scatter cursors
    float kmin[3], kinv[3];   // the volume's world box: key cell = floor(8 * (x - kmin) * kinv)
    float4* train;     // [S][2]: (x, y, z, wx), (wy, wz, tmax or -1 when invalid, target)
    int trainCount;
    int numSlots;      // M * MB
    uint32_t targetMethod;   // transmittance estimator of the training targets (mip 0, trilinear)
};

}  // namespace vrd
