// rng_golden.cpp -- emits known-answer vectors for the per-pixel RNG from the reference's
// own public-domain generator sources, compiled in place (never copied):
//   Source/Externals/xoshiro/xoshiro128starstar.c, Source/Externals/xoshiro/splitmix64.c
// The seeding follows the reference's GPU unit test
//   Source/Tools/FalcorTest/Tests/Sampling/PseudorandomTests.cpp:57-66, 94-119, 124-149
// (default-constructed std::mt19937, 128 bits of seed per xoshiro instance, 64 bits per
// SplitMix64 instance), and the composition used by the pass's sample generator
//   Source/Falcor/Utils/Sampling/UniformSampleGenerator.slang:49-68 (SplitMix64 seeded with
//   (sampleNumber << 32) | Morton(pixel), two outputs -> xoshiro128** state), and
//   Source/Falcor/Utils/Sampling/SampleGenerator.slang:58-64 (u = (bits >> 8) * 2^-24).
// Test infrastructure only: the output is a JSON fixture under tests/golden/.
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

namespace ref_xoshiro {
#include "xoshiro/xoshiro128starstar.c"
}
namespace ref_splitmix {
#include "xoshiro/splitmix64.c"
}

// Morton interleave written bit by bit (independent of the masked form in the pass).
static uint32_t morton_bitwise(uint32_t x, uint32_t y) {
    uint32_t r = 0;
    for (int b = 0; b < 16; ++b) {
        r |= ((x >> b) & 1u) << (2 * b);
        r |= ((y >> b) & 1u) << (2 * b + 1);
    }
    return r;
}

int main() {
    const int kInstances = 32, kDims = 64;
    std::printf("{\n");
    {
        std::mt19937 mt;
        std::vector<uint32_t> seed(kInstances * 4);
        for (auto& s : seed) s = mt();
        std::printf("\"xoshiro_seed\": [");
        for (size_t i = 0; i < seed.size(); ++i) std::printf("%s%u", i ? "," : "", seed[i]);
        std::printf("],\n\"xoshiro_out\": [");
        for (int i = 0; i < kInstances; ++i) {
            for (int k = 0; k < 4; ++k) ref_xoshiro::s[k] = seed[i * 4 + k];
            for (int j = 0; j < kDims; ++j)
                std::printf("%s%u", (i || j) ? "," : "", ref_xoshiro::next());
        }
        std::printf("],\n");
    }
    {
        std::mt19937 mt;
        std::vector<uint32_t> seed(kInstances * 2);
        for (auto& s : seed) s = mt();
        std::printf("\"splitmix_seed\": [");
        for (size_t i = 0; i < seed.size(); ++i) std::printf("%s%u", i ? "," : "", seed[i]);
        std::printf("],\n\"splitmix_out\": [");
        for (int i = 0; i < kInstances; ++i) {
            ref_splitmix::x = ((uint64_t)seed[i * 2 + 1] << 32) | (uint64_t)seed[i * 2 + 0];
            for (int j = 0; j < kDims; ++j)
                std::printf("%s\"%llu\"", (i || j) ? "," : "", (unsigned long long)ref_splitmix::next());
        }
        std::printf("],\n");
    }
    {
        // pixel sample generator: (px, py, sampleNumber) -> first 16 sampleNext1D bit patterns
        const uint32_t cases[][3] = {
            {0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {255, 255, 0}, {17, 93, 4}, {17, 93, 5}, {17, 93, 6},
            {17, 93, 7}, {1919, 1079, 255}, {1023, 511, 65535}, {640, 360, 4 * 63 + 2}, {3, 7, 123456}};
        const int n = sizeof(cases) / sizeof(cases[0]);
        std::printf("\"pixel_cases\": [");
        for (int c = 0; c < n; ++c)
            std::printf("%s[%u,%u,%u]", c ? "," : "", cases[c][0], cases[c][1], cases[c][2]);
        std::printf("],\n\"pixel_u24\": [");
        for (int c = 0; c < n; ++c) {
            ref_splitmix::x = ((uint64_t)cases[c][2] << 32) | morton_bitwise(cases[c][0], cases[c][1]);
            uint64_t s0 = ref_splitmix::next(), s1 = ref_splitmix::next();
            ref_xoshiro::s[0] = (uint32_t)s0; ref_xoshiro::s[1] = (uint32_t)(s0 >> 32);
            ref_xoshiro::s[2] = (uint32_t)s1; ref_xoshiro::s[3] = (uint32_t)(s1 >> 32);
            for (int j = 0; j < 16; ++j)
                std::printf("%s%u", (c || j) ? "," : "", ref_xoshiro::next() >> 8);
        }
        std::printf("]\n}\n");
    }
    return 0;
}
