// Host-computed tables shared with the kernels (see ntg_host_tables.cpp).
#pragma once

#include <cstddef>
#include <cstdint>

namespace ntg {

// Uploaded verbatim to __constant__ memory on each device.
struct HostTables {
    uint32_t four[968];            // icbc 4-cluster orderings, bytes (a, b, c) = cumulative cluster ends
    uint32_t three[152];           // icbc 3-cluster orderings, bytes (a, b)
    int four_total[16];            // orderings available for 1..16 points
    int three_total[16];
    float mid5[32];                // 565 rounding midpoints
    float mid6[64];
    uint8_t icbc_match5[256][2];   // icbc single-colour tables (D3D10 decoder)
    uint8_t icbc_match6[256][2];
    uint8_t opt_match5[256][2];    // OptimalCompress single-colour tables
    uint8_t opt_match6[256][2];
    uint8_t opt_alpha5[256][2];    // the three-colour (midpoint) variants, for BC1a
    uint8_t opt_alpha6[256][2];
    float pow_5_11[512];           // exponent tables of the gamma-2.2 helpers
    float pow_11_5[512];
};

void build_device_tables(HostTables &t);

// Colour transforms, 0 none / 1 power-law gamma / 2 sRGB.
float host_to_srgb(float f);
float host_from_srgb(float f);
// Float bit patterns of the sRGB curves' power segments: toSrgb's covers the floats above 0.0031308f
// up to 1.0f, toLinearFromSrgb's 0.04045f up to 1.0f (the domains of the device correction tables).
constexpr uint32_t kToSrgbLo = 0x3B4D2E1Du;    // first float above 0.0031308f
constexpr uint32_t kFromSrgbLo = 0x3D25AEE6u;  // 0.04045f
constexpr uint32_t kSrgbHi = 0x3F800000u;      // 1.0f
constexpr uint32_t kToSrgbCount = kSrgbHi - kToSrgbLo + 1, kFromSrgbCount = kSrgbHi - kFromSrgbLo + 1;
float host_xform_in(float v, int xform, float gamma, const HostTables &t);
float host_xform_out(float v, int xform, float gamma, const HostTables &t);
void build_input_lut(int xform, float gamma, const HostTables &t, float lut[256]);
void build_composed_lut(int in_xform, int out_xform, float gamma, const HostTables &t, float lut[256]);
void build_composed_lut8(int in_xform, int out_xform, float gamma, const HostTables &t, uint8_t lut8[512]);
void build_srgb_steps(float steps[256]);
constexpr int kSrgbBuckets = 15 * 256;  // the device quantiser's buckets over [2^-14, 2)
bool build_srgb_buckets(const float steps[256], uint8_t buckets[kSrgbBuckets]);

// Polyphase filtering: 0 box, 1 triangle, 2 kaiser (params: alpha, stretch).
float filter_evaluate(int filter, float width, float p0, float p1, float x);
int polyphase_window(float width, int src_len, int dst_len);
int build_polyphase(int filter, float width, float p0, float p1, int src_len, int dst_len, float *weights, int *lefts);

}  // namespace ntg
