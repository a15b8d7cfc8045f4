// glibc-exact x^3, x^4 and x^0.25 for the REFERENCE precision mode.
//
// The reference evaluates pow(T, 4.0f) and pow(T, 3.0f) with the host libm's
// powf (3905/Thermal/NominalPole/main.cpp:1523-1538), and the instantaneous
// equilibrium temperature as pow(x, 0.25f) (main.cpp:1455, 1606).  glibc's powf is not
// correctly rounded: over the floats in [0.5, 5000] about 0.07 % of the
// results differ by one unit in the last place from the correctly rounded
// power.  The device evaluates x^e with a double-float product (exact IEEE
// operations, see emu_pow4/emu_pow3) from 2^-4 up and with one double
// product rounded to float below 2^-4, where the double-float product
// underflows, and then consults an exception table of every positive float
// x below 2^12 (subnormals included) for which this process's powf(x, e)
// differs.  The low end matters: with TI = 0 the night side of a facet
// without neighbours in view falls to 0 K and facets seeing it to tiny
// temperatures (about 0.02 % of the low-range powers differ).
// The table is built here by calling powf itself on every float of that
// range (multi-threaded), so it reproduces whatever libm the host links; no
// libm code or constant is restated.
//
// x^0.25 (e = -4) is evaluated on the device as (float)sqrt(sqrt((double)x))
// (two correctly rounded square roots); about 0.06 % of glibc's powf(x, 0.25f)
// results differ from it.  Its table covers every positive float below 2^44
// (temperatures up to 2048 K), and is only built when a REFERENCE solve needs
// it.  Each table takes one powf call per float of its range, about 2 s on
// 8 host threads.
//
// Build with -ffp-contract=off: the emulation must round each operation.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "atpm_internal.h"

namespace atpm {

// double-float evaluation shared bit-for-bit with the device code
// (atpm_thermal.cu: dev_pow4 / dev_pow3)
float emu_pow4(float x) {
    if (x < 0.0625f) {  // below 2^-4 the double-float product underflows
        const double d = (double)x, d2 = d * d;
        return (float)(d2 * d2);
    }
    float h = x * x;
    float l = std::fma(x, x, -h);        // x^2 = h + l exactly
    float p = h * h;
    float e = std::fma(h, h, -p);        // h^2 = p + e exactly
    float c = std::fma(2.0f * h, l, e);  // 2hl + e (l^2 below the result's ulp)
    return p + c;
}

float emu_pow3(float x) {
    if (x < 0.0625f) {
        const double d = (double)x;
        return (float)((d * d) * d);
    }
    float h = x * x;
    float l = std::fma(x, x, -h);
    float p = h * x;
    float e = std::fma(h, x, -p);        // h x = p + e exactly
    float c = std::fma(l, x, e);
    return p + c;
}

float emu_qroot(float x) { return (float)std::sqrt(std::sqrt((double)x)); }

static inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

static inline uint32_t slot_of(uint32_t key, uint32_t log2slots) {
    return (key * 2654435761u) >> (32 - log2slots);
}

int build_pow_table(int e, HostPowTab* out, char* err, size_t errlen) {
    const bool q = (e == -4);
    // from the smallest subnormal (bits 1); zero needs no entry (0^e = 0)
    const float hi = q ? std::ldexp(1.0f, 44) : 4096.0f;
    const uint32_t lo_bits = 1u, hi_bits = fbits(hi);
    const float ef = q ? 0.25f : (float)e;
    unsigned nth = std::thread::hardware_concurrency();
    if (nth == 0) nth = 4;
    if (nth > 64) nth = 64;
    std::vector<std::vector<uint2>> found(nth);
    std::vector<std::thread> th;
    const uint32_t span = hi_bits - lo_bits;
    for (unsigned t = 0; t < nth; ++t) {
        th.emplace_back([&, t]() {
            uint32_t a = lo_bits + (uint32_t)((uint64_t)span * t / nth);
            uint32_t b = lo_bits + (uint32_t)((uint64_t)span * (t + 1) / nth);
            for (uint32_t u = a; u < b; ++u) {
                float x = bitsf(u);
                volatile float xv = x;
                float ref = std::pow((float)xv, ef);  // libm powf, as the reference
                float dev = q ? emu_qroot(x) : (e == 4) ? emu_pow4(x) : emu_pow3(x);
                if (fbits(ref) != fbits(dev)) found[t].push_back(make_uint2(u, fbits(ref)));
            }
        });
    }
    for (auto& x : th) x.join();
    size_t n = 0;
    for (auto& v : found) n += v.size();
    uint32_t log2slots = 10;
    while ((1ull << log2slots) < 4 * n + 1024) ++log2slots;
    std::vector<uint2> slots((size_t)1 << log2slots, make_uint2(0xFFFFFFFFu, 0u));
    const uint32_t mask = (1u << log2slots) - 1;
    for (auto& v : found)
        for (const uint2& kv : v) {
            uint32_t h = slot_of(kv.x, log2slots);
            while (slots[h].x != 0xFFFFFFFFu) h = (h + 1) & mask;
            slots[h] = kv;
        }
    uint2* d = nullptr;
    cudaError_t ce = cudaMalloc(&d, slots.size() * sizeof(uint2));
    if (ce != cudaSuccess) {
        std::snprintf(err, errlen, "cudaMalloc(pow table): %s", cudaGetErrorString(ce));
        return 1;
    }
    ce = cudaMemcpy(d, slots.data(), slots.size() * sizeof(uint2), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
        cudaFree(d);
        std::snprintf(err, errlen, "cudaMemcpy(pow table): %s", cudaGetErrorString(ce));
        return 1;
    }
    out->slots_dev = d;
    out->log2slots = log2slots;
    out->lo_bits = lo_bits;
    out->hi_bits = hi_bits;
    out->exceptions = (int64_t)n;
    return 0;
}

}  // namespace atpm
