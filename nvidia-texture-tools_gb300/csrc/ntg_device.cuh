// Device-side building blocks shared by the sm_103a kernels.
//
// Every kernel translation unit is compiled with --fmad=false: each product and each sum is
// rounded on its own, as in the reference's scalar CPU code, which is what makes the encoders
// bit-exact. Division and square root use the IEEE-rounded forms (no fast-math).
#pragma once

#include <cstdint>
#include <cfloat>
#include <cuda_runtime.h>

#include "ntg_host_tables.h"

namespace ntg {

// Min/max in the two comparison forms the reference uses; they differ on NaN.
//   ic_*: icbc::max/min and nv::max/min   (src/nvtt/icbc.h:180-190, src/nvcore/Utils.h:159-187)
//   sq_*: std::max/std::min as squish calls them (src/nvtt/squish/maths.h)
__device__ __forceinline__ float ic_max(float a, float b) { return (b < a) ? a : b; }
__device__ __forceinline__ float ic_min(float a, float b) { return (a < b) ? a : b; }
__device__ __forceinline__ float ic_clamp(float x, float a, float b) { return ic_min(ic_max(x, a), b); }
__device__ __forceinline__ float ic_sat(float x) { return ic_clamp(x, 0.0f, 1.0f); }
__device__ __forceinline__ float sq_max(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float sq_min(float a, float b) { return (b < a) ? b : a; }
// Clamp to [0, 1] ahead of a grid snap (k * x + 0.5 truncated or floored). Both reference forms,
// ic_sat(x) and sq_min(1, sq_max(0, x)), turn a NaN into 0 as fmaxf does, and agree with
// fminf(fmaxf(x, 0), 1) everywhere else except in the sign of a zero result, which the snap
// loses (k * -0 + 0.5 = 0.5). Only valid where the clamped value feeds such a snap.
__device__ __forceinline__ float snap_clamp(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
// snap_clamp(x * y) as one instruction: the product rounded to nearest, then clamped to [0, 1] by
// the multiply's saturation, which also turns a NaN into +0 (PTX mul.sat).
__device__ __forceinline__ float mul_sat(float x, float y) {
    float r;
    asm("mul.rn.sat.f32 %0, %1, %2;" : "=f"(r) : "f"(x), "f"(y));
    return r;
}

struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 sat3(f3 a) { return f3{ic_sat(a.x), ic_sat(a.y), ic_sat(a.z)}; }

__device__ __forceinline__ int ex5(int v) { return (v << 3) | (v >> 2); }
__device__ __forceinline__ int ex6(int v) { return (v << 2) | (v >> 4); }

// Tables built on the host (ntg_host_tables.cpp) and uploaded once per device: cluster orderings,
// 565 midpoints, single-colour tables, gamma exponent tables.
// Each translation unit holds its own copy (no relocatable device code) and exports an uploader.
using DeviceTables = HostTables;
static __constant__ DeviceTables c_tab;
#define NTG_DEFINE_TABLE_UPLOAD(fn) \
    int fn(const HostTables &t) { return cudaMemcpyToSymbol(c_tab, &t, sizeof(t)) == cudaSuccess ? 0 : 3; }

__device__ __forceinline__ void put_u16(uint8_t *p, unsigned v) { p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); }

// D3D10 BC1 palette (src/nvtt/icbc.h:2558-2585; src/nvimage/BlockDXT.cpp:43-99).
struct Pal8 { int r[4], g[4], b[4]; };
__device__ __forceinline__ void palette_d3d10(unsigned c0, unsigned c1, Pal8 &p) {
    p.r[0] = ex5((c0 >> 11) & 31); p.g[0] = ex6((c0 >> 5) & 63); p.b[0] = ex5(c0 & 31);
    p.r[1] = ex5((c1 >> 11) & 31); p.g[1] = ex6((c1 >> 5) & 63); p.b[1] = ex5(c1 & 31);
    if (c0 > c1) {
        p.r[2] = (2 * p.r[0] + p.r[1]) / 3; p.g[2] = (2 * p.g[0] + p.g[1]) / 3; p.b[2] = (2 * p.b[0] + p.b[1]) / 3;
        p.r[3] = (2 * p.r[1] + p.r[0]) / 3; p.g[3] = (2 * p.g[1] + p.g[0]) / 3; p.b[3] = (2 * p.b[1] + p.b[0]) / 3;
    } else {
        p.r[2] = (p.r[0] + p.r[1]) / 2; p.g[2] = (p.g[0] + p.g[1]) / 2; p.b[2] = (p.b[0] + p.b[1]) / 2;
        p.r[3] = 0; p.g[3] = 0; p.b[3] = 0;
    }
}

// AlphaBlockDXT5::evaluatePalette, D3D10 (src/nvimage/BlockDXT.cpp:336-378).
__device__ __forceinline__ void alpha_palette(int a0, int a1, int pal[8]) {
    pal[0] = a0; pal[1] = a1;
    if (a0 > a1) {
#pragma unroll
        for (int k = 1; k <= 6; k++) pal[k + 1] = ((7 - k) * a0 + k * a1) / 7;
    } else {
#pragma unroll
        for (int k = 1; k <= 4; k++) pal[k + 1] = ((5 - k) * a0 + k * a1) / 5;
        pal[6] = 0; pal[7] = 255;
    }
}

// _powf_11_5 / _powf_5_11 of src/nvmath/Gamma.cpp:311-357 (exponent table times a quartic).
__device__ __forceinline__ float powf_11_5(float x) {
    uint32_t u = __float_as_uint(x);
    float m = __uint_as_float((u & 0x7FFFFFu) | (127u << 23));
    float pm = (((-0.00916587552f * m + 0.119315466f) * m + 1.01847068f) * m - 0.158338739f) * m + 0.0297184721f;
    return c_tab.pow_11_5[u >> 23] * pm;
}
__device__ __forceinline__ float powf_5_11(float x) {
    uint32_t u = __float_as_uint(x);
    float m = __uint_as_float((u & 0x7FFFFFu) | (127u << 23));
    float pm = (((-0.0110083047f * m + 0.0905038750f) * m - 0.324697506f) * m + 0.876040946f) * m + 0.369160989f;
    return c_tab.pow_5_11[u >> 23] * pm;
}

// The sRGB curves (toSrgb / toLinearFromSrgb, src/nvtt/Surface.cpp:1512-1519, 1562-1568). Their power
// segments call powf, and the device's powf and the host libm's (which the reference uses) differ in
// the last place for ~6% of the floats there. Every float of the two segments' domains is therefore
// given a correction: the host evaluates the segment with its libm, a kernel evaluates the same
// expression below and stores the difference of the two results' bit patterns (within -8..7 on
// every input: 4 bits; the build checks it) in a table per device. The corrected device results
// equal the host's bit for bit, over the whole domain.
// (The domains' bounds kToSrgbLo, kFromSrgbLo, kSrgbHi are in ntg_host_tables.h.)
__device__ __forceinline__ float srgb_pow_segment(float f) { return (powf(f, 0.41666f) * 1.055f) - 0.055f; }
__device__ __forceinline__ float linear_pow_segment(float f) { return powf((f + 0.055f) / 1.055f, 2.4f); }

// y corrected by entry i of a 4-bit table (two entries per byte, low nibble first, two's complement).
__device__ __forceinline__ float srgb_fixed(const uint8_t *fix, uint32_t i, float y) {
    const int b = __ldg(fix + (i >> 1));
    const int d = (i & 1) ? (b >> 4) : (b & 15);
    return __uint_as_float(__float_as_uint(y) + (d >= 8 ? d - 16 : d));
}
__device__ __forceinline__ float to_srgb_exact(float f, const uint8_t *fix) {
    if (isnan(f)) return 0.0f;
    if (f <= 0.0f) return 0.0f;
    if (f <= 0.0031308f) return 12.92f * f;
    if (f <= 1.0f) return srgb_fixed(fix, __float_as_uint(f) - kToSrgbLo, srgb_pow_segment(f));
    return 1.0f;
}
__device__ __forceinline__ float from_srgb_exact(float f, const uint8_t *fix) {
    if (f < 0.0f) return 0.0f;
    if (f < 0.04045f) return f / 12.92f;
    if (f <= 1.0f) return srgb_fixed(fix, __float_as_uint(f) - kFromSrgbLo, linear_pow_segment(f));
    return 1.0f;
}

// Packed FP32 pairs: two floats in one 64-bit register (the first in the low half) added by one
// instruction (add.rn.f32x2, sm_100 and later), which rounds each half exactly as the scalar
// add.rn.f32 does. The products that feed it stay scalar multiplies: a packed multiply whose result
// feeds a packed add is contracted into a packed fused multiply-add after PTX (one rounding instead
// of two, measured on sm_103a), which would change the sums, while a scalar multiply feeding a packed
// add is not. So a tap sum += k * v over four channels is 4 multiplies and 2 packed adds, bit for bit
// the 8 scalar instructions' result.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ void f2_unpack(f32x2 p, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(p));
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// A packed multiply, for products that feed no addition or subtraction (only multiplies, floors,
// comparisons): there is nothing for it to be contracted with.
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// An f3 as a packed (x, y) pair and a scalar z. Sums and differences run x and y in one instruction;
// so do products that feed no sum (p3_mul); products that feed a sum are scalar multiplies, packed
// afterwards (p3 of an f3 product). Each component is rounded exactly as the f3 operations round it.
struct P3 { f32x2 xy; float z; };
__device__ __forceinline__ P3 p3(f3 v) { return P3{f2_pack(v.x, v.y), v.z}; }
__device__ __forceinline__ f3 u3(P3 p) {
    float x, y;
    f2_unpack(p.xy, x, y);
    return f3{x, y, p.z};
}
__device__ __forceinline__ P3 p3_add(P3 a, P3 b) { return P3{f2_add(a.xy, b.xy), a.z + b.z}; }
__device__ __forceinline__ P3 p3_sub(P3 a, P3 b) { return P3{f2_sub(a.xy, b.xy), a.z - b.z}; }
__device__ __forceinline__ P3 p3_mul(P3 a, P3 b) { return P3{f2_mul(a.xy, b.xy), a.z * b.z}; }

// A float4 as two pairs (x, y) and (z, w), and back: the same 16 bytes.
struct F4x2 { f32x2 xy, zw; };
__device__ __forceinline__ float4 f4_of(const F4x2 &p) {
    const ulonglong2 u = make_ulonglong2(p.xy, p.zw);
    return *reinterpret_cast<const float4 *>(&u);
}
// sum += k * v on all four channels.
__device__ __forceinline__ void tap2(F4x2 &sum, float k, const float4 &v) {
    sum.xy = f2_add(sum.xy, f2_pack(k * v.x, k * v.y));
    sum.zw = f2_add(sum.zw, f2_pack(k * v.z, k * v.w));
}

// ColorBlock::init(float) quantiser (src/nvimage/ColorBlock.cpp:103-106).
__device__ __forceinline__ uint32_t quant_u8(float x) { return (uint32_t)(uint8_t)(255 * ic_clamp(x, 0.0f, 1.0f)); }

}  // namespace ntg
