// vr_math.h -- deterministic arithmetic shared by the CUDA kernels and the CPU oracle.
//
// Bit-exact reservoir selection between the GPU and the CPU transcription needs every
// float operation to round identically on both sides.  Basic operations (+ - * /, sqrt,
// floor, fabs, fmin, fmax) are IEEE-754 exact on both when FMA contraction is disabled
// (nvcc -fmad=false, g++ -ffp-contract=off).  Library transcendental functions are not:
// the GPU's and glibc's expf/logf/sinf... differ in the last bits.  This header therefore
// defines its own elementary functions from textbook methods, using only exact operations:
//
//   * exp  : Cody & Waite argument reduction x = k ln2 + r (ln2 split in a 16-bit head and
//            a tail, so k*head is exact), polynomial for e^r on |r| <= ln2/2, scaling by 2^k
//            through the exponent field.
//   * log  : x = m 2^e with m in [sqrt(1/2), sqrt(2)), s = (m-1)/(m+1),
//            log m = 2 atanh(s) = 2 s (1 + a1 s^2 + ...), plus e ln2 (split).
//   * sin/cos : Cody & Waite reduction by pi/2 (three-part split), polynomials on |r|<=pi/4.
//   * atan : reduction atan(x) = pi/2 - atan(1/x) for |x|>1 and the tan(pi/6) shift
//            atan(x) = pi/6 + atan((sqrt3 x - 1)/(sqrt3 + x)) for x > tan(pi/12).
//   * atan2, acos, pow, tan are composed from the above.
//
// The polynomial coefficients were fitted for this project by weighted least squares on
// Chebyshev nodes in float64 (script: fit_math_coeffs.py beside this file) and rounded
// to float32.  Measured accuracy is a few ulp (tests/test_math.py); what matters for
// parity is that the CPU and the GPU evaluate exactly the same operation sequence.
//
// The RNG restates Falcor's UniformSampleGenerator (SplitMix64 seeding of xoshiro128**):
//   Source/Falcor/Utils/Sampling/UniformSampleGenerator.slang:49-68,
//   Source/Falcor/Utils/Sampling/Pseudorandom/Xoshiro.slang:52-66,
//   Source/Falcor/Utils/Sampling/Pseudorandom/SplitMix64.slang:54-60,
//   Source/Falcor/Utils/Math/BitTricks.slang:45-58 (interleave_32bit),
//   Source/Falcor/Utils/Sampling/SampleGenerator.slang:58-64 (sampleNext1D).
#pragma once

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define VR_HD __host__ __device__ __forceinline__
#else
#define VR_HD inline
#endif

namespace vr {

// ---------------------------------------------------------------------------------------
// bit casts and classification
// ---------------------------------------------------------------------------------------
VR_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
VR_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f; memcpy(&f, &u, 4); return f;
#endif
}
VR_HD int32_t asint(float f) { return (int32_t)f2u(f); }
VR_HD float asfloat(int32_t i) { return u2f((uint32_t)i); }
VR_HD bool isnan_(float x) { return (f2u(x) & 0x7fffffffu) > 0x7f800000u; }
VR_HD bool isinf_(float x) { return (f2u(x) & 0x7fffffffu) == 0x7f800000u; }

// float -> int conversions with one definition on every platform (NaN -> 0, saturating);
// plain C casts of NaN or out-of-range values differ between x86, Arm and the GPU.
VR_HD int32_t f2i(float x) {
    if (isnan_(x)) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int32_t)x;
}
VR_HD uint32_t f2u32(float x) {
    if (isnan_(x) || x <= 0.0f) return 0u;
    if (x >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)x;
}

constexpr float kFltMax = 3.402823466e+38f;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInf = __builtin_huge_valf();

// min/max with one definition everywhere: a NaN operand yields the other operand, and for
// equal operands (including +0/-0) the second one is returned.  Library fminf/fmaxf leave
// the sign of a zero result unspecified, which differs between x86, Arm and the GPU.
VR_HD float fmin_(float a, float b) { if (isnan_(a)) return b; if (isnan_(b)) return a; return a < b ? a : b; }
VR_HD float fmax_(float a, float b) { if (isnan_(a)) return b; if (isnan_(b)) return a; return a > b ? a : b; }
// floor/fabs/sqrt are exact IEEE operations on both sides.
VR_HD float floor_(float a) { return floorf(a); }
VR_HD float fabs_(float a) { return fabsf(a); }
VR_HD float sqrt_(float a) { return sqrtf(a); }

// ---------------------------------------------------------------------------------------
// exp
// ---------------------------------------------------------------------------------------
VR_HD float ldexp_k(float p, int k) {
    // p * 2^k for p in [0.5, 2), k in [-152, 128]; two-step scaling keeps denormals exact.
    if (k > 127) { p = p * 2.0f; k -= 1; }
    if (k < -126) {
        p = p * u2f((uint32_t)(k + 64 + 127) << 23);
        return p * u2f((uint32_t)(-64 + 127) << 23);
    }
    return p * u2f((uint32_t)(k + 127) << 23);
}

VR_HD float exp_(float x) {
    if (isnan_(x)) return x;
    if (x > 88.72283935546875f) return kInf;
    if (x < -103.97283935546875f) return 0.0f;
    const float kLog2e = 1.44269502162933349609f;
    const float kLn2Hi = 0.693145751953125f;          // 16 significant bits
    const float kLn2Lo = 1.428606765330187e-06f;      // ln2 - kLn2Hi
    float kf = floor_(x * kLog2e + 0.5f);
    float r = (x - kf * kLn2Hi) - kf * kLn2Lo;
    float p = 0.00019826495554298162f;
    p = p * r + 0.0013946021208539605f;
    p = p * r + 0.00833342969417572f;
    p = p * r + 0.041666269302368164f;
    p = p * r + 0.1666666567325592f;
    p = p * r + 0.5f;
    p = p * r;
    p = p * r + r;
    p = p + 1.0f;
    return ldexp_k(p, (int)kf);
}

// ---------------------------------------------------------------------------------------
// log
// ---------------------------------------------------------------------------------------
VR_HD float log_(float x) {
    uint32_t u = f2u(x);
    if (isnan_(x)) return x;
    if ((u & 0x7fffffffu) == 0) return -kInf;
    if (u & 0x80000000u) return u2f(0x7fc00000u);
    if (u == 0x7f800000u) return kInf;
    int e = 0;
    if (u < 0x00800000u) {           // denormal: scale by 2^23
        x = x * 8388608.0f;
        u = f2u(x);
        e = -23;
    }
    e += (int)(u >> 23) - 127;
    float m = u2f((u & 0x007fffffu) | 0x3f800000u);   // [1, 2)
    if (m > 1.41421353816986083984f) { m = m * 0.5f; e += 1; }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float q = 0.11792702227830887f;
    q = q * z + 0.14268554747104645f;
    q = q * z + 0.20000170171260834f;
    q = q * z + 0.3333333134651184f;
    q = q * z;
    float lm = (s + s) + (s + s) * q;
    const float kLn2Hi = 0.693145751953125f;
    const float kLn2Lo = 1.428606765330187e-06f;
    float ef = (float)e;
    return ef * kLn2Hi + (lm + ef * kLn2Lo);
}

// ---------------------------------------------------------------------------------------
// sin / cos
// ---------------------------------------------------------------------------------------
VR_HD float sin_poly(float r) {
    float z = r * r;
    float p = 2.725753574850387e-06f;
    p = p * z + -0.00019840168533846736f;
    p = p * z + 0.008333331905305386f;
    p = p * z + -0.1666666716337204f;
    return r + (r * z) * p;
}
VR_HD float cos_poly(float r) {
    float z = r * r;
    float p = -1.6319434337219718e-07f;
    p = p * z + 2.4682052753632888e-05f;
    p = p * z + -0.0013888522516936064f;
    p = p * z + 0.0416666641831398f;
    return (1.0f - 0.5f * z) + (z * z) * p;
}
// Reduces x to r in [-pi/4, pi/4] with quadrant q.  Accurate for |x| < ~1e5.
VR_HD float reduce_pio2(float x, int& q) {
    const float k2OverPi = 0.636619746685028076171875f;
    const float kP1 = 1.5703125f;
    const float kP2 = 0.0004837512969970703f;
    const float kP3 = 7.549790126404332e-08f;
    float kf = floor_(x * k2OverPi + 0.5f);
    float r = ((x - kf * kP1) - kf * kP2) - kf * kP3;
    q = ((int)kf) & 3;
    return r;
}
VR_HD float sin_(float x) {
    if (isnan_(x) || isinf_(x)) return u2f(0x7fc00000u);
    int q; float r = reduce_pio2(x, q);
    switch (q) {
        case 0: return sin_poly(r);
        case 1: return cos_poly(r);
        case 2: return -sin_poly(r);
        default: return -cos_poly(r);
    }
}
VR_HD float cos_(float x) {
    if (isnan_(x) || isinf_(x)) return u2f(0x7fc00000u);
    int q; float r = reduce_pio2(x, q);
    switch (q) {
        case 0: return cos_poly(r);
        case 1: return -sin_poly(r);
        case 2: return -cos_poly(r);
        default: return sin_poly(r);
    }
}
VR_HD float tan_(float x) { return sin_(x) / cos_(x); }

// ---------------------------------------------------------------------------------------
// atan / atan2 / acos / pow
// ---------------------------------------------------------------------------------------
VR_HD float atan_poly(float x) {   // x in [0, tan(pi/12)]
    float z = x * x;
    float p = -0.07840076088905334f;
    p = p * z + 0.11035103350877762f;
    p = p * z + -0.14283795654773712f;
    p = p * z + 0.1999998241662979f;
    p = p * z + -0.3333333432674408f;
    return x + (x * z) * p;
}
VR_HD float atan_pos(float x) {    // x >= 0, finite or +inf
    const float kPio2 = 1.57079637050628662109f;
    const float kPio6 = 0.52359879016876220703f;
    const float kTanPi12 = 0.26794919371604919434f;
    const float kSqrt3 = 1.73205077648162841797f;
    bool inv = false;
    if (x > 1.0f) { x = 1.0f / x; inv = true; }
    float r;
    if (x > kTanPi12) {
        float t = (x * kSqrt3 - 1.0f) / (kSqrt3 + x);
        r = kPio6 + atan_poly(t < 0.0f ? -t : t) * (t < 0.0f ? -1.0f : 1.0f);
    } else {
        r = atan_poly(x);
    }
    return inv ? kPio2 - r : r;
}
VR_HD float atan_(float x) {
    if (isnan_(x)) return x;
    return x < 0.0f ? -atan_pos(-x) : atan_pos(x);
}
VR_HD float atan2_(float y, float x) {
    const float kPi_ = 3.14159274101257324219f;
    const float kPio2 = 1.57079637050628662109f;
    if (isnan_(x) || isnan_(y)) return u2f(0x7fc00000u);
    bool ny = (f2u(y) & 0x80000000u) != 0;
    float ay = fabs_(y), ax = fabs_(x);
    float r;
    if (ax == 0.0f && ay == 0.0f) {
        r = (f2u(x) & 0x80000000u) ? kPi_ : 0.0f;
    } else if (isinf_(ax) && isinf_(ay)) {
        r = (f2u(x) & 0x80000000u) ? 2.35619449615478515625f : 0.78539818525314331055f;
    } else if (ax == 0.0f || isinf_(ay)) {
        r = kPio2;
    } else if (isinf_(ax)) {
        r = (f2u(x) & 0x80000000u) ? kPi_ : 0.0f;
    } else {
        // first-octant style: atan(ay/ax) with the quotient kept <= 1
        float a;
        if (ay <= ax) a = atan_pos(ay / ax);
        else a = kPio2 - atan_pos(ax / ay);
        r = (f2u(x) & 0x80000000u) ? kPi_ - a : a;
    }
    return ny ? -r : r;
}
VR_HD float acos_(float x) {
    if (isnan_(x) || x > 1.0f || x < -1.0f) return u2f(0x7fc00000u);
    float s = sqrt_((1.0f - x) * (1.0f + x));
    return atan2_(s, x);
}
VR_HD float pow_(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (x == 1.0f) return 1.0f;
    if (x == 0.0f) return y > 0.0f ? 0.0f : kInf;
    if (x < 0.0f) return u2f(0x7fc00000u);
    return exp_(y * log_(x));
}

// ---------------------------------------------------------------------------------------
// small vector type (own type: CUDA's float3 is avoided on purpose)
// ---------------------------------------------------------------------------------------
struct f3 { float x, y, z; };
VR_HD f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
VR_HD f3 mk3(float a) { return mk3(a, a, a); }
VR_HD f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
VR_HD f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
VR_HD f3 operator-(f3 a) { return mk3(-a.x, -a.y, -a.z); }
VR_HD f3 operator*(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
VR_HD f3 operator/(f3 a, f3 b) { return mk3(a.x / b.x, a.y / b.y, a.z / b.z); }
VR_HD f3 operator*(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
VR_HD f3 operator*(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
VR_HD f3 operator/(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
VR_HD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
VR_HD float length(f3 a) { return sqrt_(dot(a, a)); }
VR_HD f3 normalize(f3 a) { float l = length(a); return a / l; }
VR_HD f3 cross(f3 a, f3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
VR_HD bool any_gt0(f3 a) { return a.x > 0.0f || a.y > 0.0f || a.z > 0.0f; }
VR_HD bool all_eq0(f3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
// Rec.709 luminance, Source/Falcor/Utils/Color/ColorHelpers.slang:39-42
VR_HD float luminance(f3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }

// ---------------------------------------------------------------------------------------
// RNG: SplitMix64-seeded xoshiro128**
// ---------------------------------------------------------------------------------------
VR_HD uint32_t interleave_32bit(uint32_t vx, uint32_t vy) {
    uint32_t x = vx & 0x0000ffffu, y = vy & 0x0000ffffu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    y = (y | (y << 8)) & 0x00FF00FFu;
    y = (y | (y << 4)) & 0x0F0F0F0Fu;
    y = (y | (y << 2)) & 0x33333333u;
    y = (y | (y << 1)) & 0x55555555u;
    return x | (y << 1);
}

VR_HD uint64_t splitmix64_next(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

VR_HD uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

struct Rng {
    uint32_t s[4];
};

VR_HD uint32_t xoshiro_next(Rng& r) {
    const uint32_t result = rotl32(r.s[0] * 5u, 7) * 9u;
    const uint32_t t = r.s[1] << 9;
    r.s[2] ^= r.s[0];
    r.s[3] ^= r.s[1];
    r.s[1] ^= r.s[2];
    r.s[0] ^= r.s[3];
    r.s[2] ^= t;
    r.s[3] = rotl32(r.s[3], 11);
    return result;
}

VR_HD Rng rng_create(uint32_t px, uint32_t py, uint32_t sampleNumber) {
    uint64_t st = ((uint64_t)sampleNumber << 32) | (uint64_t)interleave_32bit(px, py);
    uint64_t s0 = splitmix64_next(st);
    uint64_t s1 = splitmix64_next(st);
    Rng r;
    r.s[0] = (uint32_t)s0; r.s[1] = (uint32_t)(s0 >> 32);
    r.s[2] = (uint32_t)s1; r.s[3] = (uint32_t)(s1 >> 32);
    return r;
}

VR_HD float next1D(Rng& r) {
    uint32_t bits = xoshiro_next(r);
    return (float)(bits >> 8) * 5.9604644775390625e-08f;   // 2^-24
}

}  // namespace vr
