// Host-side tables for the GB300 path: everything the kernels read that the reference computes
// on the CPU once (polyphase weights, cluster orderings, 565 midpoints, single-colour tables,
// gamma exponent tables, 8-bit transform tables). Compiled with -ffp-contract=off so every
// value is produced with the reference's own float/double steps.
#include "ntg_host_tables.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace ntg {

static inline int ex5(int v) { return (v << 3) | (v >> 2); }
static inline int ex6(int v) { return (v << 2) | (v >> 4); }

void build_device_tables(HostTables &t) {
    std::memset(&t, 0, sizeof(t));
    // Cluster orderings (src/nvtt/icbc.h:1906-1975): the orderings new at point count t are the
    // cumulative triples a <= b <= c == t, in (a, b) order.
    int n4 = 0, n3 = 0;
    for (int c = 1; c <= 16; c++) {
        for (int a = 0; a <= c; a++)
            for (int b = a; b <= c; b++) t.four[n4++] = (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)c << 16);
        t.four_total[c - 1] = n4;
        for (int a = 0; a <= c; a++) t.three[n3++] = (uint32_t)a | ((uint32_t)c << 8);
        t.three_total[c - 1] = n3;
    }
    // 565 rounding midpoints (src/nvtt/icbc.h:1516-1525): mean of adjacent expanded values / 255,
    // as six-decimal literals, FLT_MAX last.
    char buf[64];
    for (int i = 0; i < 31; i++) {
        std::snprintf(buf, sizeof buf, "%.6f", (ex5(i) + ex5(i + 1)) / 510.0);
        t.mid5[i] = std::strtof(buf, nullptr);
    }
    t.mid5[31] = 3.402823466e+38F;
    for (int i = 0; i < 63; i++) {
        std::snprintf(buf, sizeof buf, "%.6f", (ex6(i) + ex6(i + 1)) / 510.0);
        t.mid6[i] = std::strtof(buf, nullptr);
    }
    t.mid6[63] = 3.402823466e+38F;
    // icbc single-colour tables, D3D10 decoder: worse of the AMD and NVIDIA interpolation errors
    // (src/nvtt/icbc.h:3166-3262).
    for (int i = 0; i < 256; i++) {
        int best = 256 * 100;
        for (int mn = 0; mn < 32; mn++)
            for (int mx = 0; mx < 32; mx++) {
                int lo = ex5(mn), hi = ex5(mx);
                int amd = std::abs(((43 * hi + 21 * lo + 32) >> 6) - i);
                int nv = std::abs(((2 * mx + mn) * 22) / 8 - i);
                int err = amd > nv ? amd : nv;
                if (err < best) { best = err; t.icbc_match5[i][0] = (uint8_t)mx; t.icbc_match5[i][1] = (uint8_t)mn; }
            }
        best = 256 * 100;
        for (int mn = 0; mn < 64; mn++)
            for (int mx = 0; mx < 64; mx++) {
                int lo = ex6(mn), hi = ex6(mx);
                int amd = std::abs(((43 * hi + 21 * lo + 32) >> 6) - i);
                int nv = std::abs((256 * lo + (hi - lo) / 4 + 128 + (hi - lo) * 80) / 256 - i);
                int err = amd > nv ? amd : nv;
                if (err < best) { best = err; t.icbc_match6[i][0] = (uint8_t)mx; t.icbc_match6[i][1] = (uint8_t)mn; }
            }
    }
    // OMatch5 / OMatch6 and OMatchAlpha5 / OMatchAlpha6 (src/nvtt/SingleColorLookup.cpp:32-89):
    // the one-third point, or the midpoint for the three-colour tables
    for (int pass = 0; pass < 4; pass++) {
        const int size = (pass & 1) == 0 ? 32 : 64;
        const bool mid = pass >= 2;
        uint8_t(*tab)[2] = pass == 0 ? t.opt_match5 : pass == 1 ? t.opt_match6 : pass == 2 ? t.opt_alpha5 : t.opt_alpha6;
        for (int i = 0; i < 256; i++) {
            int best = 256 * 100;
            for (int mn = 0; mn < size; mn++)
                for (int mx = 0; mx < size; mx++) {
                    int lo = (pass & 1) == 0 ? ex5(mn) : ex6(mn), hi = (pass & 1) == 0 ? ex5(mx) : ex6(mx);
                    int err = (mid ? std::abs((hi + lo) / 2 - i) : std::abs((hi * 2 + lo) / 3 - i)) * 100 +
                              std::abs(mx - mn) * 3;
                    if (err < best) { tab[i][0] = (uint8_t)mx; tab[i][1] = (uint8_t)mn; best = err; }
                }
        }
    }
    // Gamma exponent tables (src/nvmath/Gamma.cpp:34-297)
    for (int k = 0; k < 512; k++) {
        float a = 0.0f, b = 0.0f;
        if (k == 255) { a = INFINITY; b = INFINITY; }
        else if (k >= 1 && k <= 254) {
            a = (float)std::pow(2.0, (k - 127) * (5.0 / 11.0));
            b = (float)std::pow(2.0, (k - 127) * (11.0 / 5.0));
        }
        t.pow_5_11[k] = a;
        t.pow_11_5[k] = b;
    }
}

// ---- colour transforms (host scalar forms) ----

static float host_powf_11_5(float x, const HostTables &t) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    uint32_t mu = (u & 0x7FFFFFu) | (127u << 23);
    float m;
    std::memcpy(&m, &mu, 4);
    float pm = (((-0.00916587552f * m + 0.119315466f) * m + 1.01847068f) * m - 0.158338739f) * m + 0.0297184721f;
    return t.pow_11_5[u >> 23] * pm;
}

static float host_powf_5_11(float x, const HostTables &t) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    uint32_t mu = (u & 0x7FFFFFu) | (127u << 23);
    float m;
    std::memcpy(&m, &mu, 4);
    float pm = (((-0.0110083047f * m + 0.0905038750f) * m - 0.324697506f) * m + 0.876040946f) * m + 0.369160989f;
    return t.pow_5_11[u >> 23] * pm;
}

// toSrgb / fromSrgb (src/nvtt/Surface.cpp:1512-1519, 1562-1568)
float host_to_srgb(float f) {
    if (std::isnan(f)) f = 0.0f;
    else if (f <= 0.0f) f = 0.0f;
    else if (f <= 0.0031308f) f = 12.92f * f;
    else if (f <= 1.0f) f = (powf(f, 0.41666f) * 1.055f) - 0.055f;
    else f = 1.0f;
    return f;
}

float host_from_srgb(float f) {
    if (f < 0.0f) f = 0.0f;
    else if (f < 0.04045f) f = f / 12.92f;
    else if (f <= 1.0f) f = powf((f + 0.055f) / 1.055f, 2.4f);
    else f = 1.0f;
    return f;
}

static bool nv_equal(float a, float b) {
    float m = 1.0f;
    if (m < std::fabs(a)) m = std::fabs(a);
    if (m < std::fabs(b)) m = std::fabs(b);
    return std::fabs(a - b) <= 0.0001f * m;
}

float host_xform_in(float v, int xform, float gamma, const HostTables &t) {
    if (xform == 2) return host_from_srgb(v);
    if (xform == 1 && !nv_equal(gamma, 1.0f)) {
        if (gamma == 2.2f) return host_powf_11_5(v, t);
        return powf(v > 0.0f ? v : 0.0f, gamma);
    }
    return v;
}

float host_xform_out(float v, int xform, float gamma, const HostTables &t) {
    if (xform == 2) return host_to_srgb(v);
    if (xform == 1 && !nv_equal(gamma, 1.0f)) {
        if (gamma == 2.2f) return host_powf_5_11(v, t);
        return powf(v > 0.0f ? v : 0.0f, 1.0f / gamma);
    }
    return v;
}

static inline uint8_t quant_u8(float x) {
    float c = x;
    if (!(0.0f < c)) c = 0.0f;  // nv::max(x, 0) keeps 0 for NaN
    if (!(c < 1.0f)) c = 1.0f;
    return (uint8_t)(255 * c);
}

void build_input_lut(int xform, float gamma, const HostTables &t, float lut[256]) {
    for (int v = 0; v < 256; v++) lut[v] = host_xform_in((float)v / 255.0f, xform, gamma, t);
}

void build_composed_lut(int in_xform, int out_xform, float gamma, const HostTables &t, float lut[256]) {
    for (int v = 0; v < 256; v++) lut[v] = host_xform_out(host_xform_in((float)v / 255.0f, in_xform, gamma, t), out_xform, gamma, t);
}

void build_composed_lut8(int in_xform, int out_xform, float gamma, const HostTables &t, uint8_t lut8[512]) {
    float f[256];
    build_composed_lut(in_xform, out_xform, gamma, t, f);
    for (int v = 0; v < 256; v++) lut8[v] = quant_u8(f[v]);
    for (int v = 0; v < 256; v++) lut8[256 + v] = quant_u8((float)v / 255.0f);
}

// Smallest float reaching each 8-bit code of uint8(255 * clamp(toSrgb(x), 0, 1)), by bisection over
// the bit patterns of [0, 2] (non-negative floats order like their bit patterns). Code 255 is only
// reached above 1: toSrgb(1) rounds to just below 1.
void build_srgb_steps(float steps[256]) {
    auto q = [](uint32_t bits) {
        float x;
        std::memcpy(&x, &bits, 4);
        return (int)quant_u8(host_to_srgb(x));
    };
    uint32_t two;
    const float f2 = 2.0f;
    std::memcpy(&two, &f2, 4);
    steps[0] = 0.0f;
    for (int k = 1; k < 256; k++) {
        uint32_t lo = 0, hi = two;  // q(lo) < k <= q(hi)
        while (hi - lo > 1) {
            uint32_t mid = lo + (hi - lo) / 2;
            if (q(mid) >= k) hi = mid; else lo = mid;
        }
        std::memcpy(&steps[k], &hi, 4);
    }
}

// Bucket table of the device's sRGB quantiser: over [2^-14, 2), bucket b covers the floats whose
// bits >> 15 equal (bits of 2^-14 >> 15) + b; buckets[b] = steps at or below its smallest float.
// Returns false unless every bucket holds at most one step beyond that and the first step lies
// above 2^-14, the two facts the device's single correcting comparison relies on.
bool build_srgb_buckets(const float steps[256], uint8_t buckets[kSrgbBuckets]) {
    uint32_t first;
    std::memcpy(&first, &steps[1], 4);
    const uint32_t lo_bits = 113u << 23;  // 2^-14
    if (first <= lo_bits) return false;
    int k = 0;  // steps (1..255) at or below the current bound
    for (int b = 0; b < kSrgbBuckets; b++) {
        const uint32_t lo = lo_bits + ((uint32_t)b << 15), hi = lo + (1u << 15) - 1;
        auto bits = [&](int i) { uint32_t u; std::memcpy(&u, &steps[i], 4); return u; };
        while (k < 255 && bits(k + 1) <= lo) k++;
        buckets[b] = (uint8_t)k;
        int inside = 0;
        for (int i = k + 1; i < 256 && bits(i) <= hi; i++) inside++;
        if (inside > 1) return false;
    }
    return true;
}

// ---- polyphase kernels (src/nvimage/Filter.cpp) ----

static const float kPi = (float)3.1415926535897932384626433833;

static float sincf_ref(float x) {  // src/nvimage/Filter.cpp:47-56
    if (std::fabs(x) < 0.0001f) return 1.0f + x * x * (-1.0f / 6.0f + x * x * 1.0f / 120.0f);
    return sinf(x) / x;
}

static float bessel0_ref(float x) {  // src/nvimage/Filter.cpp:60-79
    const float eps = 1e-6f;
    float xh = 0.5f * x, sum = 1.0f, pw = 1.0f, ds = 1.0f;
    int k = 0;
    while (ds > sum * eps) {
        ++k;
        pw = pw * (xh / k);
        ds = pw * pw;
        sum = sum + ds;
    }
    return sum;
}

float filter_evaluate(int filter, float width, float p0, float p1, float x) {
    if (filter == 0) return std::fabs(x) <= width ? 1.0f : 0.0f;         // BoxFilter
    if (filter == 1) { x = std::fabs(x); return x < width ? width - x : 0.0f; }  // TriangleFilter
    const float sinc_value = sincf_ref(kPi * x * p1);                     // KaiserFilter
    const float t = x / width;
    if ((1 - t * t) >= 0) return sinc_value * bessel0_ref(p0 * sqrtf(1 - t * t)) / bessel0_ref(p0);
    return 0;
}

static float sample_box(int filter, float width, float p0, float p1, float x, float scale, int samples) {
    double sum = 0;
    const float isamples = 1.0f / (float)samples;
    for (int s = 0; s < samples; s++) {
        const float p = (x + ((float)s + 0.5f) * isamples) * scale;
        sum += filter_evaluate(filter, width, p0, p1, p);
    }
    return (float)(sum * isamples);
}

int polyphase_window(float width, int src_len, int dst_len) {
    const float scale = (float)dst_len / (float)src_len;
    const float iscale = 1.0f / scale;
    return (int)ceilf(width * iscale * 2) + 1;
}

// PolyphaseKernel (src/nvimage/Filter.cpp:520-566) plus the window offsets applyKernelX/Y use
// (src/nvimage/FloatImage.cpp:1124-1131).
int build_polyphase(int filter, float width, float p0, float p1, int src_len, int dst_len, float *weights, int *lefts) {
    float scale = (float)dst_len / (float)src_len;
    const float iscale = 1.0f / scale;
    int samples = 32;
    if (scale > 1) { samples = 1; scale = 1; }
    const float kw = width * iscale;
    const int ws = (int)ceilf(kw * 2) + 1;
    for (int i = 0; i < dst_len; i++) {
        const float center = (0.5f + (float)(unsigned)i) * iscale;
        const int left = (int)floorf(center - kw);
        lefts[i] = left;
        float total = 0.0f;
        for (int j = 0; j < ws; j++) {
            const float s = sample_box(filter, width, p0, p1, (float)(left + j) - center, scale, samples);
            weights[(size_t)i * ws + j] = s;
            total += s;
        }
        for (int j = 0; j < ws; j++) weights[(size_t)i * ws + j] /= total;
    }
    return ws;
}

}  // namespace ntg
