// lp_net.h -- the learned target function's network: parameter layout, input encoding and
// numerics, shared by the CUDA kernels (lp.cu) and the CPU check (oracle).
//
// The network predicts the transmittance T(x, w) from a point x of the medium along direction
// w out of the volume (the visibility factor of the next-event estimate in the initial RIS
// target).  Input: x normalised to the volume box and w as (theta/pi, phi/2pi + 1/2), each of
// the 5 scalars encoded as sin/cos of 2^k pi s for k = 0..5 -> 60 features (padded to 64).
// Four hidden layers of 64 (ReLU) and a scalar output o = log T; the prediction is
// clamp(exp(o), floor, 1), the floor keeping the RIS target positive wherever the integrand
// can be.  Weights are stored in BF16 (FP32 master copy for Adam); activations enter each
// layer rounded to BF16 and every product is accumulated in FP32.
#pragma once

#include <stdint.h>

#include "vr_math.h"

namespace lpn {

constexpr int kIn = 60;          // encoded features
constexpr int kInPad = 64;       // padded input width
constexpr int kHid = 64;
constexpr int kLayers = 4;       // hidden layers
constexpr int kBands = 6;
constexpr int kLayerStride = kHid * kInPad + kHid;      // W (64x64) + b (64)
constexpr int kOutW = kLayers * kLayerStride;           // 64 output weights
constexpr int kOutB = kOutW + kHid;                     // output bias
constexpr int kParams = kOutB + 1;                      // 16705
constexpr int kParamsPad = 16708;

VR_HD int w_off(int l) { return l * kLayerStride; }
VR_HD int b_off(int l) { return l * kLayerStride + kHid * kInPad; }

// round-to-nearest-even float -> bf16 bits, and back (written for this project)
VR_HD uint16_t f2bf(float f) {
    uint32_t u = vr::f2u(f);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);   // NaN stays NaN
    uint32_t r = u + 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(r >> 16);
}
VR_HD float bf2f(uint16_t b) { return vr::u2f((uint32_t)b << 16); }
VR_HD float round_bf(float f) { return bf2f(f2bf(f)); }

// 5 normalised scalars of a query (x, w) over the box [bmin, bmin + bsize)
VR_HD void query_scalars(const float x[3], const float w[3], const float bmin[3], const float binv[3], float s[5]) {
    s[0] = (x[0] - bmin[0]) * binv[0];
    s[1] = (x[1] - bmin[1]) * binv[1];
    s[2] = (x[2] - bmin[2]) * binv[2];
    float wy = w[1] > 1.f ? 1.f : (w[1] < -1.f ? -1.f : w[1]);
    s[3] = vr::acos_(wy) * 0.318309886183790671538f;
    s[4] = vr::atan2_(w[2], w[0]) * 0.159154943091895335769f + 0.5f;
}

// 64 features: for scalar i, [sin(2^k pi s), cos(2^k pi s)] for k = 0..5 at 12 i + 2 k; the
// higher bands come from the double-angle recurrences of band 0, then the 4 pad features are 0
VR_HD void encode(const float s[5], float f[kInPad]) {
    for (int i = 0; i < 5; ++i) {
        float a = s[i] * 3.14159265358979323846f;
        float sn = vr::sin_(a), cs = vr::cos_(a);
        for (int k = 0; k < kBands; ++k) {
            f[12 * i + 2 * k] = sn;
            f[12 * i + 2 * k + 1] = cs;
            float s2 = 2.f * sn * cs;
            float c2 = cs * cs - sn * sn;
            sn = s2;
            cs = c2;
        }
    }
    for (int k = kIn; k < kInPad; ++k) f[k] = 0.f;
}

VR_HD float predict_from_logit(float o, float floor_) {
    float t = vr::exp_(o);
    t = t < floor_ ? floor_ : t;
    return t > 1.f ? 1.f : t;
}

}  // namespace lpn
