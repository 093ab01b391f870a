// BC3, BC5, BC1a and BC4 encoders for sm_103a.
//
// BC3 = CompressorDXT5::compressBlock (src/nvtt/CompressorDX9.cpp:145-176):
//   alpha : QuickCompress::compressDXT5A (Normal/Production) or OptimalCompress::compressDXT5A
//           (Highest); colour: OptimalCompress::compressDXT1 for single-colour blocks, otherwise
//           squish's WeightedClusterFit::Compress4 over all 969 cluster splits (scalar build).
//   Fastest uses FastCompressorDXT5 = QuickCompress::compressDXT1 + compressDXT5A.
// BC5 = FastCompressorBC5 / ProductionCompressorBC5 (src/nvtt/CompressorDX10.cpp:51-85): the
//   red and green channels as two interpolated-alpha blocks.
//
// One thread encodes one block. The 16 texels stay in registers; the principal-axis sort is a
// fully unrolled stable insertion network, and the weighted points it produces are staged in
// shared memory as [element][thread] because the cluster-split loops index them by running
// counts. Blocks with 16 distinct colours (the common case) all run the same 969-split schedule,
// so those warps do not diverge in the search. Built with --fmad=false.
#include "ntg.h"
#include "ntg_device.cuh"
#include "ntg_internal.h"

namespace ntg {

struct AlphaBlk { int a0, a1; uint64_t idx; };  // idx: 16 x 3-bit, texel i at bits 3i

__device__ __forceinline__ void pack_alpha(const AlphaBlk &b, uint8_t *dst) {
    uint64_t u = (uint64_t)(b.a0 & 255) | ((uint64_t)(b.a1 & 255) << 8) | (b.idx << 16);
    *reinterpret_cast<uint2 *>(dst) = make_uint2((uint32_t)u, (uint32_t)(u >> 32));
}

// computeAlphaIndices of QuickCompress (src/nvtt/QuickCompressDXT.cpp:505-536)
__device__ __forceinline__ unsigned quick_alpha_indices(const int a[16], AlphaBlk &b) {
    int pal[8];
    alpha_palette(b.a0, b.a1, pal);
    unsigned total = 0;
    uint64_t idx = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        unsigned besterr = 256 * 256;
        int best = 8;
#pragma unroll
        for (int p = 0; p < 8; p++) {
            int d = pal[p] - a[i];
            unsigned e = (unsigned)(d * d);
            if (e < besterr) { besterr = e; best = p; }
        }
        total += besterr;
        idx |= (uint64_t)best << (3 * i);
    }
    b.idx = idx;
    return total;
}

// optimizeAlpha8 (src/nvtt/QuickCompressDXT.cpp:538-592)
__device__ __forceinline__ void quick_alpha_refit(const int a[16], AlphaBlk &b) {
    float a2 = 0, b2 = 0, ab = 0, ax = 0, bx = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        unsigned k = (unsigned)(b.idx >> (3 * i)) & 7;
        float alpha = k < 2 ? 1.0f - k : (8.0f - k) / 7.0f;
        float beta = 1 - alpha;
        a2 += alpha * alpha; b2 += beta * beta; ab += alpha * beta;
        ax += alpha * a[i]; bx += beta * a[i];
    }
    const float f = 1.0f / (a2 * b2 - ab * ab);
    float fa = (ax * b2 - bx * ab) * f;
    float fb = (bx * a2 - ax * ab) * f;
    unsigned v0 = (unsigned)ic_min(ic_max(fa, 0.0f), 255.0f);
    unsigned v1 = (unsigned)ic_min(ic_max(fb, 0.0f), 255.0f);
    if (v0 < v1) {
        unsigned t = v0; v0 = v1; v1 = t;
        uint64_t n = 0;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            unsigned k = (unsigned)(b.idx >> (3 * i)) & 7;
            n |= (uint64_t)(k < 2 ? 1 - k : 9 - k) << (3 * i);
        }
        b.idx = n;
    } else if (v0 == v1) {
        b.idx = 0;
    }
    b.a0 = (int)v0; b.a1 = (int)v1;
}

// QuickCompress::compressDXT5A (src/nvtt/QuickCompressDXT.cpp:779-821); its sameIndices()
// compares the endpoint bytes only, kept as is.
__device__ AlphaBlk dxt5a_quick(const int a[16]) {
    int hi = 0, lo = 255;
#pragma unroll
    for (int i = 0; i < 16; i++) { hi = max(hi, a[i]); lo = min(lo, a[i]); }
    AlphaBlk b;
    b.a0 = (uint8_t)(hi - (hi - lo) / 34);
    b.a1 = (uint8_t)(lo + (hi - lo) / 34);
    unsigned best = quick_alpha_indices(a, b);
    AlphaBlk bestb = b;
    for (int it = 0; it < 8; it++) {
        quick_alpha_refit(a, b);
        unsigned e = quick_alpha_indices(a, b);
        if (e >= best) break;
        if (b.a0 == bestb.a0 && b.a1 == bestb.a1) { bestb = b; break; }
        best = e;
        bestb = b;
    }
    return bestb;
}

// computeAlphaError (src/nvtt/OptimalCompressDXT.cpp:189-217), unit weights, early out.
__device__ __forceinline__ float opt_alpha_error(const int a[16], int a0, int a1, float bound) {
    int pal[8];
    alpha_palette(a0, a1, pal);
    float total = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        int md = 0x7fffffff;
#pragma unroll
        for (int p = 0; p < 8; p++) { int d = a[i] - pal[p]; d = d * d; md = d < md ? d : md; }
        total += md * 1.0f;
        if (total > bound) return total;
    }
    return total;
}

// OptimalCompress::compressDXT5A (src/nvtt/OptimalCompressDXT.cpp:512-607), starting from a zeroed
// destination block (the reference starts from whatever the destination held).
__device__ AlphaBlk dxt5a_optimal(const int a[16]) {
    int mina = 255, maxa = 0, mina01 = 255, maxa01 = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        int v = a[i];
        mina = min(mina, v); maxa = max(maxa, v);
        if (v != 0 && v != 255) { mina01 = min(mina01, v); maxa01 = max(maxa01, v); }
    }
    AlphaBlk b;
    if (maxa - mina < 8) { b.a0 = maxa; b.a1 = mina; }
    else if (maxa01 - mina01 < 6) { b.a0 = mina01; b.a1 = maxa01; }
    else {
        float besterr = opt_alpha_error(a, 0, 0, FLT_MAX);
        int ba0 = maxa, ba1 = mina;
        int lo = mina <= 8 ? 0 : mina - 8, hi = maxa >= 255 - 8 ? 255 : maxa + 8;
        for (int a0 = lo + 9; a0 < hi; a0++)
            for (int a1 = lo; a1 < a0 - 8; a1++) {
                float e = opt_alpha_error(a, a0, a1, besterr);
                if (e < besterr) { besterr = e; ba0 = a0; ba1 = a1; }
            }
        lo = mina01 <= 6 ? 0 : mina01 - 6;
        hi = maxa01 >= 255 - 6 ? 255 : maxa01 + 6;
        for (int a0 = lo + 9; a0 < hi; a0++)
            for (int a1 = lo; a1 < a0 - 8; a1++) {
                float e = opt_alpha_error(a, a1, a0, besterr);
                if (e < besterr) { besterr = e; ba0 = a1; ba1 = a0; }
            }
        b.a0 = ba0; b.a1 = ba1;
    }
    int pal[8];
    alpha_palette(b.a0, b.a1, pal);
    uint64_t idx = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        int md = 0x7fffffff, bi = 8;
#pragma unroll
        for (int p = 0; p < 8; p++) { int d = a[i] - pal[p]; d = d * d; if (d < md) { md = d; bi = p; } }
        idx |= (uint64_t)bi << (3 * i);
    }
    b.idx = idx;
    return b;
}

// OptimalCompress::compressDXT1(Color32) (src/nvtt/OptimalCompressDXT.cpp:254-269)
__device__ __forceinline__ uint2 dxt1_single_color(int r, int g, int b) {
    unsigned c0 = ((unsigned)c_tab.opt_match5[r][0] << 11) | ((unsigned)c_tab.opt_match6[g][0] << 5) | c_tab.opt_match5[b][0];
    unsigned c1 = ((unsigned)c_tab.opt_match5[r][1] << 11) | ((unsigned)c_tab.opt_match6[g][1] << 5) | c_tab.opt_match5[b][1];
    uint32_t idx = 0xaaaaaaaau;
    if (c0 < c1) { unsigned t = c0; c0 = c1; c1 = t; idx ^= 0x55555555u; }
    return make_uint2(c0 | (c1 << 16), idx);
}

__device__ __forceinline__ int float_to_int(float a, int limit) {
    int i = (int)(a + 0.5f);
    return i < 0 ? 0 : (i > limit ? limit : i);
}

// squish WeightedClusterFit, scalar build: ColourSet with the header's default
// createMinimalSet = true (src/nvtt/squish/colourset.h:40, colourset.cpp:44-90), SetColourSet
// (src/nvtt/squish/weightedclusterfit.cpp:39-105), ComputeWeightedCovariance /
// ComputePrincipleComponent (src/nvtt/squish/maths.cpp:32-135), Compress4 / Compress3
// (src/nvtt/squish/weightedclusterfit.cpp:476-589, 372-470), WriteColourBlock4 / 3
// (src/nvtt/squish/colourblock.cpp:108-139, 75-106).
//
// The minimal set is kept in texel slots instead of being compacted: a slot is live when its
// texel is the first with that RGB, and its weight collects the weights of the later duplicates
// in texel order. Live slots in slot order are exactly the reference's points in order, so the
// sums run in the same order; dead slots sort last behind +inf keys. Everything stays in
// registers with static indices; `wp` is this thread's [17][thread] float4 staging for the
// split loops, which index points by running counts. In DXT1 mode (BC1a) a texel with alpha 0
// is never live and never matched, and takes index 3 at the end.

// v = n * f, Min(one, Max(zero, v)), then Floor(grid * v + half) * gridrcp
// (src/nvtt/squish/weightedclusterfit.cpp:513-519) per channel, grid (31, 63, 31); the product and
// the clamp are one saturating multiply, which gives the same snapped value as squish's Max/Min
// for every input.
__device__ __forceinline__ f3 snap565(f3 n, float f) {
    const float x = mul_sat(n.x, f), y = mul_sat(n.y, f), z = mul_sat(n.z, f);
    return mk3(floorf(31.0f * x + 0.5f) * (1.0f / 31.0f), floorf(63.0f * y + 0.5f) * (1.0f / 63.0f),
               floorf(31.0f * z + 0.5f) * (1.0f / 31.0f));
}

// The colour set of a block, sorted along its principal axis and staged in `wp`.
struct SquishSet {
    int count;
    uint32_t transparent;  // bit i: texel i has alpha 0 (DXT1 mode only)
    uint64_t first;        // 4 bits per texel: slot of its point
    uint64_t order;        // 4 bits per sorted position: slot
    f3 xsum;
    float wsum;
    f3 axis;               // the principal axis the points are sorted along (arbitrary sign)
    f3 xxsum;              // sum of weight x colour^2 per channel over the points (the error's constant)
};

// The minimal colour set in texel slots (colours, summed weights, live slots, transparent texels,
// each texel's slot) and its principal axis (ComputeWeightedCovariance, ComputePrincipleComponent).
template <bool DXT1>
__device__ __forceinline__ f3 squish_points(const uint32_t px[16], bool weight_by_alpha, f3 metric, float X[16], float Y[16],
                                            float Z[16], float W[16], uint32_t &live_out, uint32_t &transp_out,
                                            uint64_t &first_out) {
    uint32_t live = 0;  // bit i: slot i holds a point
    uint32_t transp = 0;
    uint64_t first = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        X[i] = (float)((px[i] >> 16) & 255) / 255.0f;
        Y[i] = (float)((px[i] >> 8) & 255) / 255.0f;
        Z[i] = (float)(px[i] & 255) / 255.0f;
        W[i] = weight_by_alpha ? (float)((px[i] >> 24) + 1) / 256.0f : 1.0f;
        if (DXT1 && (px[i] >> 24) == 0) transp |= 1u << i;
    }
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const bool skip = DXT1 && ((transp >> i) & 1u);
        bool found = skip;
        int slot = i;
#pragma unroll
        for (int j = 0; j < i; j++) {
            const bool m = !found && !(DXT1 && ((transp >> j) & 1u)) && ((px[i] & 0xFFFFFF) == (px[j] & 0xFFFFFF));
            if (m) { W[j] += W[i]; slot = j; }
            found = found || m;
        }
        if (!found) live |= 1u << i;
        first |= (uint64_t)slot << (4 * i);
    }
    float total = 0.0f;
    f3 cen = mk3(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 16; i++)
        if (live & (1u << i)) { total += W[i]; cen = cen + mk3(X[i], Y[i], Z[i]) * W[i]; }
    cen = cen * (1.0f / total);
    float m0 = 0, m1 = 0, m2 = 0, m3 = 0, m4 = 0, m5 = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        if (!(live & (1u << i))) continue;
        f3 a = (mk3(X[i], Y[i], Z[i]) - cen) * metric;
        f3 b = a * W[i];
        m0 += a.x * b.x; m1 += a.x * b.y; m2 += a.x * b.z;
        m3 += a.y * b.y; m4 += a.y * b.z; m5 += a.z * b.z;
    }
    f3 r0 = mk3(m0, m1, m2), r1 = mk3(m1, m3, m4), r2 = mk3(m2, m4, m5);
    float l0 = dot(r0, r0), l1 = dot(r1, r1), l2 = dot(r2, r2);
    f3 v = (l0 > l1 && l0 > l2) ? r0 : (l1 > l2 ? r1 : r2);
#pragma unroll
    for (int it = 0; it < 8; it++) {
        float x = v.x * m0 + v.y * m1 + v.z * m2;
        float y = v.x * m1 + v.y * m3 + v.z * m4;
        float z = v.x * m2 + v.y * m4 + v.z * m5;
        float norm = sq_max(sq_max(x, y), z);
        float iv = 1.0f / norm;
        if (norm == 0.0f) { v = mk3(0, 0, 0); break; }
        v = mk3(x * iv, y * iv, z * iv);
    }
    live_out = live;
    transp_out = transp;
    first_out = first;
    return v;
}

template <bool DXT1, typename Arr>
__device__ __forceinline__ void squish_prepare(const uint32_t px[16], bool weight_by_alpha, f3 metric, Arr wp,
                                               SquishSet &S) {
    float X[16], Y[16], Z[16], W[16];
    uint32_t live, transp;
    uint64_t first;
    const f3 v = squish_points<DXT1>(px, weight_by_alpha, metric, X, Y, Z, W, live, transp, first);
    const int count = __popc(live);
    // stable insertion sort along the axis; slot numbers carried in a packed 64-bit word
    float dps[16];
    uint64_t order = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        dps[i] = (live & (1u << i)) ? dot(mk3(X[i], Y[i], Z[i]), v) : __int_as_float(0x7f800000);
        order |= (uint64_t)i << (4 * i);
    }
#pragma unroll
    for (int i = 1; i < 16; i++) {
        bool moving = true;
#pragma unroll
        for (int j = i; j > 0; --j) {
            moving = moving && (dps[j] < dps[j - 1]);
            if (moving) {
                float t;
                t = dps[j]; dps[j] = dps[j - 1]; dps[j - 1] = t;
                t = X[j]; X[j] = X[j - 1]; X[j - 1] = t;
                t = Y[j]; Y[j] = Y[j - 1]; Y[j - 1] = t;
                t = Z[j]; Z[j] = Z[j - 1]; Z[j - 1] = t;
                t = W[j]; W[j] = W[j - 1]; W[j - 1] = t;
                uint64_t a = (order >> (4 * j)) & 15, b = (order >> (4 * (j - 1))) & 15;
                order &= ~((uint64_t)0xFF << (4 * (j - 1)));
                order |= (a << (4 * (j - 1))) | (b << (4 * j));
            }
        }
    }
    f3 xsum = mk3(0, 0, 0), xxsum = mk3(0, 0, 0);
    float wsum = 0.0f;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        f3 p = mk3(X[i], Y[i], Z[i]) * W[i];
        wp[i] = make_float4(p.x, p.y, p.z, W[i]);
        if (i < count) { xsum = xsum + p; wsum += W[i]; xxsum = xxsum + p * mk3(X[i], Y[i], Z[i]); }
    }
    wp[16] = make_float4(0, 0, 0, 0);
    S.count = count;
    S.transparent = transp;
    S.first = first;
    S.order = order;
    S.xsum = xsum;
    S.wsum = wsum;
    S.axis = v;
    S.xxsum = xxsum;
}

// Compress4's split search: the first strict minimum, as best error and split key
// c0 << 10 | c1 << 5 | c2 (the endpoints of the winner are recomputed afterwards with the same
// sequence of operations).
template <bool UNIT_METRIC, typename Arr>
__device__ __forceinline__ float squish_search4(const SquishSet &S, f3 msq, Arr wp, int &best) {
    const int count = S.count;
    const f3 xsum = S.xsum;
    const float wsum = S.wsum;
    float besterr = FLT_MAX;
    best = 0;
    f3 x0 = mk3(0, 0, 0);
    float w0 = 0.0f;
    for (int c0 = 0; c0 <= count; c0++) {
        f3 x1 = mk3(0, 0, 0);
        float w1 = 0.0f;
        const float t01 = w0;  // loop invariants of the inner loops, same operands and order
        for (int c1 = 0; c1 <= count - c0; c1++) {
            f3 x2 = mk3(0, 0, 0);
            float w2 = 0.0f;
            const float wr = wsum - w0 - w1;
            const float a2p = t01 + w1 * (4.0f / 9.0f);
            const float w1n = w1 * (1.0f / 9.0f);
            const f3 axp = x0 + (x1 * (2.0f / 3.0f));
            int key = (c0 << 10) | (c1 << 5);
            for (int c2 = 0; c2 <= count - c0 - c1; c2++) {
                const float w3 = wr - w2;
                const float a2 = a2p + w2 * (1.0f / 9.0f);
                const float b2s = w3 + w2 * (4.0f / 9.0f) + w1n;
                const float ab = (w1 + w2) * (2.0f / 9.0f);
                const float f = 1.0f / (a2 * b2s - ab * ab);
                const f3 ax = axp + (x2 * (1.0f / 3.0f));
                const f3 bx = xsum - ax;
                const f3 a = snap565((ax * b2s) - (bx * ab), f);
                const f3 b = snap565((bx * a2) - (ax * ab), f);
                const f3 t = (((a * b) * ab) - (a * ax)) - (b * bx);
                const f3 e1 = (((a * a) * a2) + ((b * b) * b2s)) + (t * 2.0f);
                // x * 1.0f is x exactly: the default unit metric drops the three multiplies
                const float err = UNIT_METRIC ? (e1.x + e1.y) + e1.z : dot(e1, msq);
                if (err < besterr) { besterr = err; best = key; }
                key++;
                const float4 q = wp[c0 + c1 + c2];
                x2 = x2 + mk3(q.x, q.y, q.z);
                w2 += q.w;
            }
            const float4 q = wp[c0 + c1];
            x1 = x1 + mk3(q.x, q.y, q.z);
            w1 += q.w;
        }
        const float4 q = wp[c0];
        x0 = x0 + mk3(q.x, q.y, q.z);
        w0 += q.w;
    }
    return besterr;
}

// Compress3's split search (two clusters ends, key c0 << 5 | c1).
template <bool UNIT_METRIC, typename Arr>
__device__ __forceinline__ float squish_search3(const SquishSet &S, f3 msq, Arr wp, int &best) {
    const int count = S.count;
    float besterr = FLT_MAX;
    best = 0;
    f3 x0 = mk3(0, 0, 0);
    float w0 = 0.0f;
    for (int c0 = 0; c0 <= count; c0++) {
        f3 x1 = mk3(0, 0, 0);
        float w1 = 0.0f;
        int key = c0 << 5;
        for (int c1 = 0; c1 <= count - c0; c1++) {
            const float w2 = S.wsum - w0 - w1;
            const float a2 = w0 + w1 * 0.25f;
            const float b2s = w2 + w1 * 0.25f;
            const float ab = w1 * 0.25f;
            const float f = 1.0f / (a2 * b2s - ab * ab);
            const f3 ax = x0 + x1 * 0.5f;
            const f3 bx = S.xsum - ax;
            const f3 a = snap565((ax * b2s) - (bx * ab), f);
            const f3 b = snap565((bx * a2) - (ax * ab), f);
            const f3 t = (((a * b) * ab) - (a * ax)) - (b * bx);
            const f3 e1 = (((a * a) * a2) + ((b * b) * b2s)) + (t * 2.0f);
            const float err = UNIT_METRIC ? (e1.x + e1.y) + e1.z : dot(e1, msq);
            if (err < besterr) { besterr = err; best = key; }
            key++;
            const float4 q = wp[c0 + c1];
            x1 = x1 + mk3(q.x, q.y, q.z);
            w1 += q.w;
        }
        const float4 q = wp[c0];
        x0 = x0 + mk3(q.x, q.y, q.z);
        w0 += q.w;
    }
    return besterr;
}

// The running sums of a winning split (cluster sizes b0, b1, b2), accumulated as the search did.
template <typename Arr>
__device__ __forceinline__ void split_sums(Arr wp, int b0, int b1, int b2, f3 &x0, f3 &x1, f3 &x2, float &w0, float &w1,
                                           float &w2) {
    x0 = mk3(0, 0, 0); x1 = mk3(0, 0, 0); x2 = mk3(0, 0, 0);
    w0 = 0.0f; w1 = 0.0f; w2 = 0.0f;
    for (int i = 0; i < b0; i++) { const float4 q = wp[i]; x0 = x0 + mk3(q.x, q.y, q.z); w0 += q.w; }
    for (int i = b0; i < b0 + b1; i++) { const float4 q = wp[i]; x1 = x1 + mk3(q.x, q.y, q.z); w1 += q.w; }
    for (int i = b0 + b1; i < b0 + b1 + b2; i++) { const float4 q = wp[i]; x2 = x2 + mk3(q.x, q.y, q.z); w2 += q.w; }
}

// Sorted-position clusters -> slot indices -> texel indices (ColourSet::RemapIndices,
// src/nvtt/squish/colourset.cpp:141-151; transparent texels take 3). Four-colour clusters are
// 0, 2, 3, 1 in order; three-colour ones 0, 2, 1.
template <bool THREE>
__device__ __forceinline__ uint32_t texel_indices(const SquishSet &S, int b0, int b1, int b2) {
    uint32_t slot_idx = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const uint32_t c = i < b0 ? 0u : (i < b0 + b1 ? 2u : ((!THREE && i < b0 + b1 + b2) ? 3u : 1u));
        if (i < S.count) slot_idx |= c << (2 * (int)((S.order >> (4 * i)) & 15));
    }
    uint32_t idx = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const uint32_t v = ((S.transparent >> i) & 1u) ? 3u : ((slot_idx >> (2 * (int)((S.first >> (4 * i)) & 15))) & 3u);
        idx |= v << (2 * i);
    }
    return idx;
}

__device__ __forceinline__ int squish_565(f3 c) {
    return (float_to_int(31.0f * c.x, 31) << 11) | (float_to_int(63.0f * c.y, 63) << 5) | float_to_int(31.0f * c.z, 31);
}

// WriteColourBlock4 of the split with key `best` (cluster sizes b0 << 10 | b1 << 5 | b2).
template <typename Arr>
__device__ __forceinline__ uint2 squish_finish4(const SquishSet &S, Arr wp, int best) {
    const int b0 = best >> 10, b1 = (best >> 5) & 31, b2 = best & 31;
    f3 x0, x1, x2;
    float w0, w1, w2;
    split_sums(wp, b0, b1, b2, x0, x1, x2, w0, w1, w2);
    const float w3 = S.wsum - w0 - w1 - w2;
    const float a2 = w0 + w1 * (4.0f / 9.0f) + w2 * (1.0f / 9.0f);
    const float b2s = w3 + w2 * (4.0f / 9.0f) + w1 * (1.0f / 9.0f);
    const float ab = (w1 + w2) * (2.0f / 9.0f);
    const float f = 1.0f / (a2 * b2s - ab * ab);
    const f3 ax = (x0 + (x1 * (2.0f / 3.0f))) + (x2 * (1.0f / 3.0f));
    const f3 bx = S.xsum - ax;
    const f3 bs = snap565((ax * b2s) - (bx * ab), f);
    const f3 be = snap565((bx * a2) - (ax * ab), f);
    uint32_t idx = texel_indices<false>(S, b0, b1, b2);
    int ea = squish_565(bs), eb = squish_565(be);
    if (ea < eb) { int t = ea; ea = eb; eb = t; idx ^= 0x55555555u; }
    else if (ea == eb) idx = 0;
    return make_uint2((uint32_t)ea | ((uint32_t)eb << 16), idx);
}

template <bool UNIT_METRIC, typename Arr>
__device__ __forceinline__ uint2 squish_block4(const SquishSet &S, f3 msq, Arr wp, float &err) {
    int best;
    err = squish_search4<UNIT_METRIC>(S, msq, wp, best);
    if (!(err < FLT_MAX)) return make_uint2(0, 0);
    return squish_finish4(S, wp, best);
}

template <bool UNIT_METRIC, typename Arr>
__device__ __forceinline__ uint2 squish_block3(const SquishSet &S, f3 msq, Arr wp, float &err) {
    int best;
    err = squish_search3<UNIT_METRIC>(S, msq, wp, best);
    if (!(err < FLT_MAX)) return make_uint2(0, 0);
    const int b0 = best >> 5, b1 = best & 31;
    f3 x0, x1, x2;
    float w0, w1, w2;
    split_sums(wp, b0, b1, 0, x0, x1, x2, w0, w1, w2);
    const float w2r = S.wsum - w0 - w1;
    const float a2 = w0 + w1 * 0.25f;
    const float b2s = w2r + w1 * 0.25f;
    const float ab = w1 * 0.25f;
    const float f = 1.0f / (a2 * b2s - ab * ab);
    const f3 ax = x0 + x1 * 0.5f;
    const f3 bx = S.xsum - ax;
    const f3 bs = snap565((ax * b2s) - (bx * ab), f);
    const f3 be = snap565((bx * a2) - (ax * ab), f);
    uint32_t idx = texel_indices<true>(S, b0, b1, 0);
    int ea = squish_565(bs), eb = squish_565(be);
    // WriteColourBlock3: endpoints ascending; swapping exchanges indices 0 and 1
    if (ea > eb) { int t = ea; ea = eb; eb = t; idx ^= (~idx >> 1) & 0x55555555u; }
    return make_uint2((uint32_t)ea | ((uint32_t)eb << 16), idx);
}

// BC3 colour: Compress4 over the full colour set.
template <bool UNIT_METRIC, typename Arr>
__device__ uint2 squish_compress4(const uint32_t px[16], bool weight_by_alpha, f3 metric, Arr wp) {
    SquishSet S;
    squish_prepare<false>(px, weight_by_alpha, metric, wp, S);
    float err;
    return squish_block4<UNIT_METRIC>(S, metric * metric, wp, err);
}

// BC1a colour (ColourFit::Compress with kDxt1, src/nvtt/squish/colourfit.cpp:39-55): Compress3,
// then Compress4 unless a texel is transparent; a later mode replaces the block only with a
// strictly smaller error.
template <bool UNIT_METRIC, typename Arr>
__device__ uint2 squish_compress_dxt1(const uint32_t px[16], bool weight_by_alpha, f3 metric, Arr wp) {
    SquishSet S;
    squish_prepare<true>(px, weight_by_alpha, metric, wp, S);
    const f3 msq = metric * metric;
    float e3, e4;
    uint2 out = squish_block3<UNIT_METRIC>(S, msq, wp, e3);
    if (!(e3 < FLT_MAX)) e3 = FLT_MAX;
    if (S.transparent == 0) {
        const uint2 four = squish_block4<UNIT_METRIC>(S, msq, wp, e4);
        if (e4 < e3) out = four;
    }
    return out;
}

// OptimalCompress::compressDXT1a(Color32, alphaMask) (src/nvtt/OptimalCompressDXT.cpp:271-292).
__device__ __forceinline__ uint2 dxt1a_single_color(int r, int g, int b, uint32_t alpha_mask) {
    if (alpha_mask == 0) return dxt1_single_color(r, g, b);
    unsigned c0 = ((unsigned)c_tab.opt_alpha5[r][0] << 11) | ((unsigned)c_tab.opt_alpha6[g][0] << 5) | c_tab.opt_alpha5[b][0];
    unsigned c1 = ((unsigned)c_tab.opt_alpha5[r][1] << 11) | ((unsigned)c_tab.opt_alpha6[g][1] << 5) | c_tab.opt_alpha5[b][1];
    if (c0 > c1) { unsigned t = c0; c0 = c1; c1 = t; }
    return make_uint2(c0 | (c1 << 16), 0xaaaaaaaau | alpha_mask);
}

// QuickCompress::compressDXT1 (src/nvtt/QuickCompressDXT.cpp:653-713) with roundAndExpand
// (:122-149), computeIndices4 (:195-227) and optimizeEndPoints4 (:406-452).
__device__ __forceinline__ unsigned quick_round_expand(f3 &v) {
    unsigned r = (unsigned)floorf(ic_clamp(v.x * (31.0f / 255.0f), 0.0f, 31.0f));
    unsigned g = (unsigned)floorf(ic_clamp(v.y * (63.0f / 255.0f), 0.0f, 63.0f));
    unsigned b = (unsigned)floorf(ic_clamp(v.z * (31.0f / 255.0f), 0.0f, 31.0f));
    if (fabsf(v.x - (float)ex5(r + 1)) < fabsf(v.x - (float)ex5(r))) r = min(r + 1, 31u);
    if (fabsf(v.y - (float)ex6(g + 1)) < fabsf(v.y - (float)ex6(g))) g = min(g + 1, 63u);
    if (fabsf(v.z - (float)ex5(b + 1)) < fabsf(v.z - (float)ex5(b))) b = min(b + 1, 31u);
    unsigned w = (r << 11) | (g << 5) | b;
    v = mk3((float)ex5(r), (float)ex6(g), (float)ex5(b));
    return w;
}

__device__ __forceinline__ uint32_t quick_indices4(const f3 blk[16], f3 mx, f3 mn) {
    const float s1 = 1.0f - 1.0f / 3.0f, s2 = 1.0f - 2.0f / 3.0f;
    f3 p2 = mk3(mx.x * s1 + (1.0f / 3.0f) * mn.x, mx.y * s1 + (1.0f / 3.0f) * mn.y, mx.z * s1 + (1.0f / 3.0f) * mn.z);
    f3 p3 = mk3(mx.x * s2 + (2.0f / 3.0f) * mn.x, mx.y * s2 + (2.0f / 3.0f) * mn.y, mx.z * s2 + (2.0f / 3.0f) * mn.z);
    uint32_t idx = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        f3 t;
        t = mx - blk[i]; float d0 = dot(t, t);
        t = mn - blk[i]; float d1 = dot(t, t);
        t = p2 - blk[i]; float d2 = dot(t, t);
        t = p3 - blk[i]; float d3 = dot(t, t);
        unsigned q0 = d0 > d3, q1 = d1 > d2, q2 = d0 > d2, q3 = d1 > d3, q4 = d2 > d3;
        unsigned x0 = q1 & q2, x1 = q0 & q3, x2 = q0 & q4;
        idx |= (x2 | ((x0 | x1) << 1)) << (2 * i);
    }
    return idx;
}

__device__ uint2 quick_dxt1(const uint32_t px[16]) {
    f3 blk[16];
#pragma unroll
    for (int i = 0; i < 16; i++) blk[i] = mk3((float)((px[i] >> 16) & 255), (float)((px[i] >> 8) & 255), (float)(px[i] & 255));
    f3 mx = mk3(0, 0, 0), mn = mk3(255, 255, 255);
#pragma unroll
    for (int i = 0; i < 16; i++) {
        mx = mk3(ic_max(mx.x, blk[i].x), ic_max(mx.y, blk[i].y), ic_max(mx.z, blk[i].z));
        mn = mk3(ic_min(mn.x, blk[i].x), ic_min(mn.y, blk[i].y), ic_min(mn.z, blk[i].z));
    }
    f3 center = (mx + mn) * 0.5f;
    float cx = 0.0f, cy = 0.0f;
#pragma unroll
    for (int i = 0; i < 16; i++) { f3 t = blk[i] - center; cx += t.x * t.z; cy += t.y * t.z; }
    float x0 = mx.x, y0 = mx.y, x1 = mn.x, y1 = mn.y;
    if (cx < 0) { float t = x0; x0 = x1; x1 = t; }
    if (cy < 0) { float t = y0; y0 = y1; y1 = t; }
    mx = mk3(x0, y0, mx.z); mn = mk3(x1, y1, mn.z);
    f3 d = mx - mn;
    const float bias = (8.0f / 255.0f) / 16.0f;
    f3 inset = mk3(d.x / 16.0f - bias, d.y / 16.0f - bias, d.z / 16.0f - bias);
    f3 t = mx - inset;
    mx = mk3(ic_clamp(t.x, 0.0f, 255.0f), ic_clamp(t.y, 0.0f, 255.0f), ic_clamp(t.z, 0.0f, 255.0f));
    t = mn + inset;
    mn = mk3(ic_clamp(t.x, 0.0f, 255.0f), ic_clamp(t.y, 0.0f, 255.0f), ic_clamp(t.z, 0.0f, 255.0f));
    unsigned c0 = quick_round_expand(mx), c1 = quick_round_expand(mn);
    if (c0 < c1) { f3 tv = mx; mx = mn; mn = tv; unsigned tc = c0; c0 = c1; c1 = tc; }
    uint32_t idx = quick_indices4(blk, mx, mn);
    float a2 = 0, b2 = 0, ab = 0;
    f3 ax = mk3(0, 0, 0), bx = mk3(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 16; i++) {
        unsigned bits = idx >> (2 * i);
        float beta = (float)(bits & 1);
        if (bits & 2) beta = (1 + beta) / 3.0f;
        float alpha = 1.0f - beta;
        a2 += alpha * alpha; b2 += beta * beta; ab += alpha * beta;
        ax = ax + blk[i] * alpha; bx = bx + blk[i] * beta;
    }
    float den = a2 * b2 - ab * ab;
    if (!(fabsf(den - 0.0f) <= 0.0001f * ic_max(ic_max(1.0f, fabsf(den)), 0.0f))) {
        float f = 1.0f / den;
        f3 a = ((ax * b2) - (bx * ab)) * f;
        f3 b = ((bx * a2) - (ax * ab)) * f;
        a = mk3(ic_clamp(a.x, 0.0f, 255.0f), ic_clamp(a.y, 0.0f, 255.0f), ic_clamp(a.z, 0.0f, 255.0f));
        b = mk3(ic_clamp(b.x, 0.0f, 255.0f), ic_clamp(b.y, 0.0f, 255.0f), ic_clamp(b.z, 0.0f, 255.0f));
        unsigned e0 = quick_round_expand(a), e1 = quick_round_expand(b);
        if (e0 < e1) { f3 tv = a; a = b; b = tv; unsigned tc = e0; e0 = e1; e1 = tc; }
        c0 = e0; c1 = e1;
        idx = quick_indices4(blk, a, b);
    }
    return make_uint2(c0 | (c1 << 16), idx);
}

__device__ __forceinline__ int find_job(const EncJob *jobs, int njobs, long long blk) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_block <= blk) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Loads a block's 16 texels as BGRA words (b | g << 8 | r << 16 | a << 24), with ColorBlock's
// edge repetition (src/nvimage/ColorBlock.cpp:57-110):
//  - from BGRA8 words, optionally remapped through 8-bit tables (the composed transform +
//    quantiser of an 8-bit source level), or
//  - from a planar FP32 level with ColorBlock::init(float)'s clamp-and-truncate.
__device__ __forceinline__ void load_block(const EncJob &J, int x, int y, uint32_t px[16]) {
    const unsigned bw = min(J.w - x, 4), bh = min(J.h - y, 4);
    const size_t n = (size_t)J.w * J.h;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const unsigned yy = (unsigned)i % bh;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const unsigned xx = (unsigned)e % bw;
            const size_t idx = (size_t)(y + yy) * J.w + x + xx;
            uint32_t p;
            if (J.bgra) {
                p = J.bgra[idx];
                if (J.lut8)
                    p = (uint32_t)J.lut8[p & 255] | ((uint32_t)J.lut8[(p >> 8) & 255] << 8) |
                        ((uint32_t)J.lut8[(p >> 16) & 255] << 16) | ((uint32_t)J.lut8[256 + (p >> 24)] << 24);
            } else {
                p = quant_u8(J.rgba[idx + 2 * n]) | (quant_u8(J.rgba[idx + n]) << 8) | (quant_u8(J.rgba[idx]) << 16) |
                    (quant_u8(J.rgba[idx + 3 * n]) << 24);
            }
            px[4 * i + e] = p;
        }
    }
}

// Resident CTAs of 128 threads per SM the register allocation is sized for: 5 (96 registers, 252 B
// of spill stores) measured 2.6% faster than 4 (127 registers) and 1.9% faster than 6 on C1.
#ifndef NTG_BC3_MIN_CTAS
#define NTG_BC3_MIN_CTAS 5
#endif

template <int QUALITY>
__global__ void __launch_bounds__(128, NTG_BC3_MIN_CTAS) k_bc3(const EncJob *__restrict__ jobs, int njobs, long long nblocks,
                                                              const long long *__restrict__ list,
                                                              const unsigned long long *__restrict__ count) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x, t = threadIdx.x;
    long long gblk = (long long)blockIdx.x * T + t;
    if (gblk >= nblocks) return;
    if (list) {  // a subset of the jobs' blocks (the learned path's fallbacks), *count long
        if ((unsigned long long)gblk >= *count) return;
        gblk = list[gblk];
    }
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    uint32_t px[16];
    load_block(J, 4 * (blk % J.bw), 4 * (blk / J.bw), px);
    int al[16];
#pragma unroll
    for (int i = 0; i < 16; i++) al[i] = (int)(px[i] >> 24);
    AlphaBlk ab = QUALITY == 3 ? dxt5a_optimal(al) : dxt5a_quick(al);
    uint8_t *dst = J.out + 16 * (size_t)blk;
    pack_alpha(ab, dst);
    bool single = true;
#pragma unroll
    for (int i = 1; i < 16; i++) single = single && ((px[i] & 0xFFFFFF) == (px[0] & 0xFFFFFF));
    uint2 col;
    if (single) col = dxt1_single_color((px[0] >> 16) & 255, (px[0] >> 8) & 255, px[0] & 255);
    else if (QUALITY == 0) col = quick_dxt1(px);
    else {
        struct { float4 *b; int s; __device__ float4 &operator[](int k) const { return b[k * s]; } } wp{smem + t, T};
        const f3 metric = mk3(J.cw[0], J.cw[1], J.cw[2]);
        if (metric.x == 1.0f && metric.y == 1.0f && metric.z == 1.0f)
            col = squish_compress4<true>(px, J.alpha_mode == 1, metric, wp);
        else
            col = squish_compress4<false>(px, J.alpha_mode == 1, metric, wp);
    }
    *reinterpret_cast<uint2 *>(dst + 8) = col;
}

template <int QUALITY>
__global__ void __launch_bounds__(128) k_bc5(const EncJob *__restrict__ jobs, int njobs, long long nblocks) {
    const long long gblk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gblk >= nblocks) return;
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    uint32_t px[16];
    load_block(J, 4 * (blk % J.bw), 4 * (blk / J.bw), px);
    int ch[16];
    uint8_t *dst = J.out + 16 * (size_t)blk;
#pragma unroll
    for (int i = 0; i < 16; i++) ch[i] = (int)((px[i] >> 16) & 255);
    pack_alpha(QUALITY >= 2 ? dxt5a_optimal(ch) : dxt5a_quick(ch), dst);
#pragma unroll
    for (int i = 0; i < 16; i++) ch[i] = (int)((px[i] >> 8) & 255);
    pack_alpha(QUALITY >= 2 ? dxt5a_optimal(ch) : dxt5a_quick(ch), dst + 8);
}

// BC1a = CompressorDXT1a::compressBlock (src/nvtt/CompressorDX9.cpp:83-111), Normal quality and
// above: single RGB colour -> OptimalCompress::compressDXT1a with the mask of zero-alpha texels,
// otherwise the squish fit in DXT1 mode.
__global__ void __launch_bounds__(128, NTG_BC3_MIN_CTAS) k_bc1a(const EncJob *__restrict__ jobs, int njobs,
                                                               long long nblocks) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x, t = threadIdx.x;
    const long long gblk = (long long)blockIdx.x * T + t;
    if (gblk >= nblocks) return;
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    uint32_t px[16];
    load_block(J, 4 * (blk % J.bw), 4 * (blk / J.bw), px);
    uint32_t mask = 0;
    bool single = true;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        if ((px[i] >> 24) == 0) mask |= 3u << (2 * i);
        single = single && ((px[i] & 0xFFFFFF) == (px[0] & 0xFFFFFF));
    }
    uint2 col;
    if (single) col = dxt1a_single_color((px[0] >> 16) & 255, (px[0] >> 8) & 255, px[0] & 255, mask);
    else {
        struct { float4 *b; int s; __device__ float4 &operator[](int k) const { return b[k * s]; } } wp{smem + t, T};
        const f3 metric = mk3(J.cw[0], J.cw[1], J.cw[2]);
        if (metric.x == 1.0f && metric.y == 1.0f && metric.z == 1.0f)
            col = squish_compress_dxt1<true>(px, J.alpha_mode == 1, metric, wp);
        else
            col = squish_compress_dxt1<false>(px, J.alpha_mode == 1, metric, wp);
    }
    *reinterpret_cast<uint2 *>(J.out + 8 * (size_t)blk) = col;
}

// BC4 = FastCompressorBC4 / ProductionCompressorBC4 (src/nvtt/CompressorDX10.cpp:40-72): the red
// channel (AlphaBlock4x4::init(src, 0)) as an interpolated-alpha block.
template <int QUALITY>
__global__ void __launch_bounds__(128) k_bc4(const EncJob *__restrict__ jobs, int njobs, long long nblocks) {
    const long long gblk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gblk >= nblocks) return;
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    uint32_t px[16];
    load_block(J, 4 * (blk % J.bw), 4 * (blk / J.bw), px);
    int ch[16];
#pragma unroll
    for (int i = 0; i < 16; i++) ch[i] = (int)((px[i] >> 16) & 255);
    pack_alpha(QUALITY >= 2 ? dxt5a_optimal(ch) : dxt5a_quick(ch), J.out + 8 * (size_t)blk);
}

// ---------------------------------------------------------------------------------------------
// Learned endpoint proposal for the BC3 colour block (no counterpart in the reference). The network
// (the same MLP as BC1's, trained on BC3 blocks) reads the block's 16 texels as the encoder sees them
// (after ColorBlock's quantiser, RGB / 255) in order of their projection on the squish principal axis
// oriented towards brighter colours (stable), each pulled towards the block's weighted mean colour in
// proportion to its fit weight (mu + w (c - mu), w = (alpha + 1) / 256 under transparency), and
// proposes Compress4's winning split as three cumulative weight fractions of the sorted colour set in
// that orientation, and the fit's error. The pruned search evaluates only the splits whose three
// cumulative ends lie within `radius` of the proposal's, with the full search's arithmetic and in its
// order, so a block whose best split is in that window gets exactly the full fit's colour block. A
// block whose pruned error exceeds (1 + margin) x the network's estimate of the full fit's error is
// listed for the full k_bc3. Errors are in 8-bit units: SSE8 = 255^2 x (the search's error + the
// constant it leaves out), V the block's weighted colour variance in the same units; the network's
// error output is log((SSE8 + 1) / (V + 1)).

struct Bc3Frame {
    bool reversed;  // the squish axis points towards darker colours
    float var;      // V
};

__device__ __forceinline__ f3 texel_rgb(uint32_t p) {
    return mk3((float)((p >> 16) & 255) / 255.0f, (float)((p >> 8) & 255) / 255.0f, (float)(p & 255) / 255.0f);
}
__device__ __forceinline__ float texel_weight(uint32_t p, bool weight_by_alpha) {
    return weight_by_alpha ? (float)((p >> 24) + 1) / 256.0f : 1.0f;
}

// The block's frame for its axis `v` (squish's), and, when `row` is given, the network's input row.
// The texels are read again from the packed words at each use, so that only their sort keys are live.
__device__ __forceinline__ Bc3Frame bc3_inputs(const uint32_t px[16], bool weight_by_alpha, f3 metric, f3 v, float *row) {
    Bc3Frame fr;
    fr.reversed = (v.x + v.y + v.z) < 0.0f;
    float ws = 0.0f;
    f3 mu = mk3(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const float w = texel_weight(px[i], weight_by_alpha);
        ws += w;
        mu = mu + texel_rgb(px[i]) * w;
    }
    mu = mu * (1.0f / ws);
    float var = 0.0f;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const f3 d = ((texel_rgb(px[i]) - mu) * metric) * 255.0f;
        var += texel_weight(px[i], weight_by_alpha) * dot(d, d);
    }
    fr.var = var;
    if (row) {
        float key[16];
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const float p = dot(texel_rgb(px[i]), v);
            key[i] = fr.reversed ? -p : p;
        }
#pragma unroll
        for (int i = 0; i < 16; i++) {
            int rank = 0;
#pragma unroll
            for (int j = 0; j < 16; j++) rank += (key[j] < key[i]) | ((key[j] == key[i]) & (j < i));
            const f3 c = mu + (texel_rgb(px[i]) - mu) * texel_weight(px[i], weight_by_alpha);
            row[3 * rank] = c.x; row[3 * rank + 1] = c.y; row[3 * rank + 2] = c.z;
        }
    }
    return fr;
}

// Compress4's splits whose cumulative ends lie in [lo_k, hi_k] (e1 <= e2 <= e3 <= count), in the full
// search's order, with its running sums: every sum is accumulated point by point from its cluster's
// first point as squish_search4's loops accumulate it (the partial sums before a window's start are
// built the same way), and each split's error uses the loops' operations in their order, so every
// evaluated split's error equals the full search's bit for bit. Returns the best error (first strict
// minimum) and its key in `best` (-1 when none compares below FLT_MAX); `evaluated` counts the splits.
template <bool UNIT_METRIC, typename Arr>
__device__ __forceinline__ float squish_window4(const SquishSet &S, f3 msq, Arr wp, int lo1, int hi1, int lo2, int hi2,
                                               int lo3, int hi3, int &best, int &evaluated) {
    const int n = S.count;
    float besterr = FLT_MAX;
    best = -1;
    f3 x0 = mk3(0, 0, 0);
    float w0 = 0.0f;
    for (int i = 0; i < lo1; i++) { const float4 q = wp[i]; x0 = x0 + mk3(q.x, q.y, q.z); w0 += q.w; }
    for (int e1 = lo1; e1 <= hi1; e1++) {
        const int a2lo = max(e1, lo2);
        f3 x1 = mk3(0, 0, 0);
        float w1 = 0.0f;
        for (int i = e1; i < a2lo; i++) { const float4 q = wp[i]; x1 = x1 + mk3(q.x, q.y, q.z); w1 += q.w; }
        for (int e2 = a2lo; e2 <= hi2; e2++) {
            const float wr = S.wsum - w0 - w1;
            const float a2p = w0 + w1 * (4.0f / 9.0f);
            const float w1n = w1 * (1.0f / 9.0f);
            const f3 axp = x0 + (x1 * (2.0f / 3.0f));
            const int a3lo = max(e2, lo3);
            f3 x2 = mk3(0, 0, 0);
            float w2 = 0.0f;
            for (int i = e2; i < a3lo; i++) { const float4 q = wp[i]; x2 = x2 + mk3(q.x, q.y, q.z); w2 += q.w; }
            for (int e3 = a3lo; e3 <= hi3; e3++) {
                const float w3 = wr - w2;
                const float a2 = a2p + w2 * (1.0f / 9.0f);
                const float b2s = w3 + w2 * (4.0f / 9.0f) + w1n;
                const float ab = (w1 + w2) * (2.0f / 9.0f);
                const float f = 1.0f / (a2 * b2s - ab * ab);
                const f3 ax = axp + (x2 * (1.0f / 3.0f));
                const f3 bx = S.xsum - ax;
                const f3 a = snap565((ax * b2s) - (bx * ab), f);
                const f3 b = snap565((bx * a2) - (ax * ab), f);
                const f3 t = (((a * b) * ab) - (a * ax)) - (b * bx);
                const f3 e = (((a * a) * a2) + ((b * b) * b2s)) + (t * 2.0f);
                const float err = UNIT_METRIC ? (e.x + e.y) + e.z : dot(e, msq);
                evaluated++;
                if (err < besterr) { besterr = err; best = (e1 << 10) | ((e2 - e1) << 5) | (e3 - e2); }
                if (e3 < n) { const float4 q = wp[e3]; x2 = x2 + mk3(q.x, q.y, q.z); w2 += q.w; }
            }
            if (e2 < n) { const float4 q = wp[e2]; x1 = x1 + mk3(q.x, q.y, q.z); w1 += q.w; }
        }
        if (e1 < n) { const float4 q = wp[e1]; x0 = x0 + mk3(q.x, q.y, q.z); w0 += q.w; }
    }
    return besterr;
}

// Cumulative end of a weight fraction over the sorted points: the number of leading points whose
// cumulative weight is within it.
template <typename Arr>
__device__ __forceinline__ int frac_count(const SquishSet &S, Arr wp, float frac) {
    const float lim = frac * S.wsum * (1.0f + 1e-5f) + 1e-7f;
    float cum = 0.0f;
    int e = 0;
    for (int i = 0; i < S.count; i++) {
        cum += wp[i].w;
        if (cum <= lim) e = i + 1;
    }
    return e;
}

// The search error of the block's best split in 8-bit units.
__device__ __forceinline__ float squish_sse8(const SquishSet &S, f3 msq, float err) {
    return (err + dot(S.xxsum, msq)) * 65025.0f;
}

// The network's inputs for every block: x [nblocks x 48], staged per warp and written coalesced.
constexpr int BC3_FEAT_STRIDE = 49;

__global__ void __launch_bounds__(64, 8) k_bc3_features(const EncJob *__restrict__ jobs, int njobs, long long nblocks,
                                                        float *__restrict__ x) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31;
    const long long gblk = (long long)blockIdx.x * T + t;
    float *stage = reinterpret_cast<float *>(smem) + (t >> 5) * 32 * BC3_FEAT_STRIDE;
    if (gblk < nblocks) {
        const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
        const int blk = (int)(gblk - J.first_block);
        uint32_t px[16];
        load_block(J, 4 * (blk % J.bw), 4 * (blk / J.bw), px);
        const f3 metric = mk3(J.cw[0], J.cw[1], J.cw[2]);
        float X[16], Y[16], Z[16], W[16];  // only the axis is needed here: the points are not sorted
        uint32_t live, transp;
        uint64_t first;
        const f3 v = squish_points<false>(px, J.alpha_mode == 1, metric, X, Y, Z, W, live, transp, first);
        bc3_inputs(px, J.alpha_mode == 1, metric, v, stage + lane * BC3_FEAT_STRIDE);
    }
    __syncwarp();
    const long long base = (long long)blockIdx.x * T + (t & ~31);
    const int rows = (int)min(32LL, nblocks - base);
    for (int q = lane; q < rows * 48; q += 32) x[base * 48 + q] = stage[(q / 48) * BC3_FEAT_STRIDE + q % 48];
}

// Training targets from the full fit: tg [nblocks x 8] = the winning split's three cumulative weight
// fractions (in the inputs' orientation), 1/3 and 2/3 (the network's three-cluster outputs, unused
// for BC3), log((SSE8 + 1) / (V + 1)), 0, 0. Single-colour blocks (no search) get 0, 0, 0.
__global__ void __launch_bounds__(128) k_bc3_targets(const EncJob *__restrict__ jobs, int njobs, long long nblocks,
                                                     float *__restrict__ tg) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x, t = threadIdx.x;
    const long long gblk = (long long)blockIdx.x * T + t;
    if (gblk >= nblocks) return;
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    uint32_t px[16];
    load_block(J, 4 * (blk % J.bw), 4 * (blk / J.bw), px);
    float *o = tg + gblk * 8;
    o[3] = 1.0f / 3.0f; o[4] = 2.0f / 3.0f; o[6] = 0.0f; o[7] = 0.0f;
    bool single = true;
#pragma unroll
    for (int i = 1; i < 16; i++) single = single && ((px[i] & 0xFFFFFF) == (px[0] & 0xFFFFFF));
    struct { float4 *b; int s; __device__ float4 &operator[](int k) const { return b[k * s]; } } wp{smem + t, T};
    const f3 metric = mk3(J.cw[0], J.cw[1], J.cw[2]);
    SquishSet S;
    squish_prepare<false>(px, J.alpha_mode == 1, metric, wp, S);
    const Bc3Frame fr = bc3_inputs(px, J.alpha_mode == 1, metric, S.axis, nullptr);
    if (single) {
        o[0] = o[1] = o[2] = 0.0f;
        o[5] = logf(1.0f / (fr.var + 1.0f));
        return;
    }
    int best;
    const f3 msq = metric * metric;
    const float err = squish_search4<false>(S, msq, wp, best);
    const int e1 = best >> 10, e2 = e1 + ((best >> 5) & 31), e3 = e2 + (best & 31);
    float c1 = 0.0f, c2 = 0.0f, c3 = 0.0f, cum = 0.0f;
    for (int i = 0; i < S.count; i++) {
        cum += wp[i].w;
        if (i + 1 == e1) c1 = cum;
        if (i + 1 == e2) c2 = cum;
        if (i + 1 == e3) c3 = cum;
    }
    float f1 = c1 / S.wsum, f2 = c2 / S.wsum, f3v = c3 / S.wsum;
    if (fr.reversed) { const float a = f1; f1 = 1.0f - f3v; f2 = 1.0f - f2; f3v = 1.0f - a; }
    o[0] = f1; o[1] = f2; o[2] = f3v;
    const float sse = err < FLT_MAX ? squish_sse8(S, msq, err) : fr.var;
    o[5] = logf((fmaxf(sse, 0.0f) + 1.0f) / (fr.var + 1.0f));
}

// Learned BC3 Normal encode: alpha as k_bc3<1> (QuickCompress DXT5A), colour from the pruned split
// search around the network's proposal y [nblocks x 16]; a listed block is rewritten whole by the
// full k_bc3. radius: the window half-width in each cumulative end. stats[0] += blocks kept here,
// stats[1] = list length, stats[2] += splits evaluated.
template <bool UNIT_METRIC>
__global__ void __launch_bounds__(128, NTG_BC3_MIN_CTAS) k_bc3_learned(const EncJob *__restrict__ jobs, int njobs,
                                                                      long long nblocks, const float *__restrict__ y,
                                                                      int radius, float margin, long long *__restrict__ list,
                                                                      unsigned long long *__restrict__ stats) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x, t = threadIdx.x;
    const long long gblk = (long long)blockIdx.x * T + t;
    if (gblk >= nblocks) return;
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    uint32_t px[16];
    load_block(J, 4 * (blk % J.bw), 4 * (blk / J.bw), px);
    uint8_t *dst = J.out + 16 * (size_t)blk;
    {   // alpha first, so that the texels are dead during the search
        int al[16];
#pragma unroll
        for (int i = 0; i < 16; i++) al[i] = (int)(px[i] >> 24);
        pack_alpha(dxt5a_quick(al), dst);
    }
    bool single = true;
#pragma unroll
    for (int i = 1; i < 16; i++) single = single && ((px[i] & 0xFFFFFF) == (px[0] & 0xFFFFFF));
    bool take = false;
    int evaluated = 0;
    uint2 col = make_uint2(0, 0);
    if (single) {
        col = dxt1_single_color((px[0] >> 16) & 255, (px[0] >> 8) & 255, px[0] & 255);
    } else {
        struct { float4 *b; int s; __device__ float4 &operator[](int k) const { return b[k * s]; } } wp{smem + t, T};
        const f3 metric = mk3(J.cw[0], J.cw[1], J.cw[2]);
        const f3 msq = metric * metric;
        SquishSet S;
        squish_prepare<false>(px, J.alpha_mode == 1, metric, wp, S);
        const Bc3Frame fr = bc3_inputs(px, J.alpha_mode == 1, metric, S.axis, nullptr);
        const float *yp = y + gblk * 16;
        const float pred = (fr.var + 1.0f) * expf(yp[5]) - 1.0f;
        float q1 = yp[0], q2 = yp[1], q3 = yp[2];
        if (fr.reversed) { const float a = q1; q1 = 1.0f - q3; q2 = 1.0f - q2; q3 = 1.0f - a; }
        const int n = S.count;
        const int p1 = frac_count(S, wp, q1), p2 = max(p1, frac_count(S, wp, q2)), p3 = max(p2, frac_count(S, wp, q3));
        int bkey;
        const float best = squish_window4<UNIT_METRIC>(S, msq, wp, max(0, p1 - radius), min(n, p1 + radius),
                                                       max(0, p2 - radius), min(n, p2 + radius), max(0, p3 - radius),
                                                       min(n, p3 + radius), bkey, evaluated);
        take = bkey < 0 || !(squish_sse8(S, msq, best) <= (1.0f + margin) * pred);  // NaN estimates fall back too
        if (!take) col = squish_finish4(S, wp, bkey);
    }
    if (!take) *reinterpret_cast<uint2 *>(dst + 8) = col;
    // the list and the statistics, warp-aggregated
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync(active, take);
    const int lane = threadIdx.x & 31, leader = __ffs(active) - 1;
    unsigned long long kept = take ? 0 : 1, ev = (unsigned long long)evaluated;
    for (int off = 16; off > 0; off >>= 1) {
        kept += __shfl_down_sync(active, kept, off);
        ev += __shfl_down_sync(active, ev, off);
    }
    unsigned long long base = 0;
    if (lane == leader) {
        if (mask) base = atomicAdd(&stats[1], (unsigned long long)__popc(mask));
        atomicAdd(&stats[0], kept);
        atomicAdd(&stats[2], ev);
    }
    base = __shfl_sync(active, base, leader);
    if (take) list[base + __popc(mask & ((1u << lane) - 1))] = gblk;
}

int launch_bc3_features(const EncJob *d_jobs, int njobs, long long nblocks, float *x, cudaStream_t stream) {
    if (nblocks == 0) return 0;
    const int T = 64;
    const size_t sm = 2 * 32 * BC3_FEAT_STRIDE * sizeof(float);
    k_bc3_features<<<(unsigned)((nblocks + T - 1) / T), T, sm, stream>>>(d_jobs, njobs, nblocks, x);
    return launch_status();
}

int launch_bc3_targets(const EncJob *d_jobs, int njobs, long long nblocks, float *tg, cudaStream_t stream) {
    if (nblocks == 0) return 0;
    const int T = 128;
    k_bc3_targets<<<(unsigned)((nblocks + T - 1) / T), T, (size_t)T * 17 * sizeof(float4), stream>>>(d_jobs, njobs, nblocks,
                                                                                                      tg);
    return launch_status();
}

int launch_bc3_learned(const EncJob *d_jobs, int njobs, long long nblocks, const float *y, int radius, float margin,
                       bool unit_metric, long long *list, unsigned long long *stats, cudaStream_t stream) {
    if (nblocks == 0) return 0;
    const int T = 128;
    const size_t sm = (size_t)T * 17 * sizeof(float4);
    const unsigned grid = (unsigned)((nblocks + T - 1) / T);
    if (unit_metric) k_bc3_learned<true><<<grid, T, sm, stream>>>(d_jobs, njobs, nblocks, y, radius, margin, list, stats);
    else k_bc3_learned<false><<<grid, T, sm, stream>>>(d_jobs, njobs, nblocks, y, radius, margin, list, stats);
    return launch_status();
}

// The full BC3 Normal fit over the first *d_count entries of `list` (at most max_count).
int launch_bc3_list(const EncJob *d_jobs, int njobs, const long long *list, const unsigned long long *d_count,
                    long long max_count, cudaStream_t stream) {
    if (max_count == 0) return 0;
    const int T = 128;
    const size_t sm = (size_t)T * 17 * sizeof(float4);
    k_bc3<1><<<(unsigned)((max_count + T - 1) / T), T, sm, stream>>>(d_jobs, njobs, max_count, list, d_count);
    return launch_status();
}

int launch_bc3(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t stream) {
    if (nblocks == 0) return 0;
    const int T = threads == 32 || threads == 64 ? threads : 128;  // blocks per CTA
    const size_t sm = (size_t)T * 17 * sizeof(float4);
    const unsigned grid = (unsigned)((nblocks + T - 1) / T);
    switch (quality) {
        case 0: k_bc3<0><<<grid, T, sm, stream>>>(d_jobs, njobs, nblocks, nullptr, nullptr); break;
        case 3: k_bc3<3><<<grid, T, sm, stream>>>(d_jobs, njobs, nblocks, nullptr, nullptr); break;
        default: k_bc3<1><<<grid, T, sm, stream>>>(d_jobs, njobs, nblocks, nullptr, nullptr); break;
    }
    return launch_status();
}

int launch_bc5(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t stream) {
    if (nblocks == 0) return 0;
    const int T = threads == 32 || threads == 64 ? threads : 128;  // blocks per CTA
    const unsigned grid = (unsigned)((nblocks + T - 1) / T);
    if (quality >= 2) k_bc5<2><<<grid, T, 0, stream>>>(d_jobs, njobs, nblocks);
    else k_bc5<1><<<grid, T, 0, stream>>>(d_jobs, njobs, nblocks);
    return launch_status();
}

int launch_bc1a(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t stream) {
    if (nblocks == 0) return 0;
    if (quality == 0) return NTG_ERROR_UNSUPPORTED_FEATURE;  // see ntg_encode's check
    const int T = threads == 32 || threads == 64 ? threads : 128;  // blocks per CTA
    const size_t sm = (size_t)T * 17 * sizeof(float4);
    k_bc1a<<<(unsigned)((nblocks + T - 1) / T), T, sm, stream>>>(d_jobs, njobs, nblocks);
    return launch_status();
}

int launch_bc4(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t stream) {
    if (nblocks == 0) return 0;
    const int T = threads == 32 || threads == 64 ? threads : 128;  // blocks per CTA
    const unsigned grid = (unsigned)((nblocks + T - 1) / T);
    if (quality >= 2) k_bc4<2><<<grid, T, 0, stream>>>(d_jobs, njobs, nblocks);
    else k_bc4<1><<<grid, T, 0, stream>>>(d_jobs, njobs, nblocks);
    return launch_status();
}

NTG_DEFINE_TABLE_UPLOAD(upload_tables_bc3)

}  // namespace ntg
