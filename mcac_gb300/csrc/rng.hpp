// The C library's rand() stream as a value type usable on host and device.
//
// The reference draws every random number with rand() / RAND_MAX
// (src/tools/tools.cpp:53-57). glibc's rand() is its TYPE_3 additive
// lagged-Fibonacci generator: r[0] = seed (1 when seed is 0), r[i] =
// 16807 * r[i-1] mod (2^31 - 1) for i = 1..30 (Schrage's method, signed
// arithmetic), r[31..33] = r[0..2], then r[i] = r[i-3] + r[i-31] mod 2^32;
// outputs are r[i] >> 1 for i >= 344 (the first 310 values after the seed
// block are discarded). This is the published description of the algorithm
// (e.g. P. Selinger, "The GLIBC pseudo-random number generator"). Each box of
// a batched run owns one stream, seeded like the reference box would be.
#pragma once
#include <stdint.h>

#include "common.hpp"

namespace mcacg {

struct RandStream {
    uint32_t r[34];  // the last 34 values, circular
    int pos;         // index of the next value to produce (mod 34)

    MCACG_HD void seed(uint32_t s) {
        int64_t word = s == 0 ? 1 : int64_t(s);
        uint32_t init[34];
        init[0] = uint32_t(word);
        for (int i = 1; i < 31; ++i) {
            int64_t hi = word / 127773;
            int64_t lo = word % 127773;
            word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            init[i] = uint32_t(word);
        }
        for (int i = 31; i < 34; ++i) init[i] = init[i - 31];
        for (int i = 0; i < 34; ++i) r[i] = init[i];
        pos = 34 % 34;
        // values 34..343 are generated and dropped
        for (int i = 34; i < 344; ++i) step();
    }
    MCACG_HD uint32_t step() {
        // r[i] = r[i-3] + r[i-31] with i = pos (mod 34)
        int i3 = pos - 3;
        if (i3 < 0) i3 += 34;
        int i31 = pos - 31;
        if (i31 < 0) i31 += 34;
        uint32_t v = r[i3] + r[i31];
        r[pos] = v;
        pos = pos + 1 == 34 ? 0 : pos + 1;
        return v;
    }
    // rand(): 31-bit value
    MCACG_HD int next_int() { return int(step() >> 1); }
    // the reference's random(): rand() / RAND_MAX as a double
    MCACG_HD double uniform() {
        double v = next_int();
        return v / 2147483647.0;
    }
    // The device loop's draws: the same rand() values scaled by a product
    // (last bit aside) or drawn in FP32. Its pick and directions follow the
    // reference statistically, and FP64 instructions are scarce on the GPU.
    MCACG_HD double uniform_mul() { return double(next_int()) * (1.0 / 2147483647.0); }
    MCACG_HD float uniform_f() { return float(next_int()) * (1.0f / 2147483647.0f); }
};

}  // namespace mcacg
