// BC1 encoder for sm_103a: the icbc 1.05 fits NVTT's CompressorDXT1 uses
// (src/nvtt/BlockCompressor.cpp:211-222 -> icbc::compress_dxt1, src/nvtt/icbc.h:3485-3559):
//   Quality_Fastest    -> icbc Level1: box fit + least squares
//   Quality_Normal     -> icbc Level8: 4- and 3-colour cluster fit over all orderings
//   Quality_Production -> icbc Level9: Level8 + endpoint refinement
// One thread encodes one 4x4 block. The block's texels, its reduced colour set and its summed-area
// table live in shared memory laid out [element][thread], so the data-dependent element indices of
// the cluster-fit search never conflict on banks. The ordering index of the search loop is the
// same in every thread of a warp, so ordering records are read as constant-cache broadcasts.
// Built with --fmad=false: results are bit-identical to the reference's scalar build.
#include "ntg.h"
#include "ntg_device.cuh"
#include "ntg_internal.h"

namespace ntg {

template <typename T>
struct Lane {  // one thread's view of a [k][thread] shared-memory array
    T *base;
    int stride;
    __device__ __forceinline__ T &operator[](int k) const { return base[k * stride]; }
};

// One thread's 16 weights packed in four float4 slots of a [slot][thread] array (k -> slot k / 4,
// component k % 4), so that every slot holds this thread's data only.
struct LaneW {
    float *base;  // component 0 of this thread's first slot
    int stride;   // floats between consecutive slots of one thread
    __device__ __forceinline__ float &operator[](int k) const { return base[(k >> 2) * stride + (k & 3)]; }
};

// One thread's 16 weights derived from its gathered texels when they are read: saturate(alpha)
// under AlphaMode_Transparency, else 1, and 0 for the texels outside the image (bit k of `valid`
// clear). It needs no storage of its own, and reads right while the slots hold the gathered texels:
// reduce_colors reads slot k's weight before it writes there, and the output stage gathers again.
struct AlphaW {
    const float4 *base;  // this thread's first slot
    int stride;          // float4 between consecutive slots of one thread
    bool transparency;
    uint32_t valid;
    __device__ __forceinline__ float operator[](int k) const {
        return ((valid >> k) & 1u) ? (transparency ? ic_clamp(base[k * stride].w, 0.0f, 1.0f) : 1.0f) : 0.0f;
    }
};

// The device's toSrgb correction table (set once per device when a context is created).
static __device__ const uint8_t *g_to_srgb_fix;

int set_srgb_fix_bc1(const uint8_t *to_srgb) {
    return cudaMemcpyToSymbol(g_to_srgb_fix, &to_srgb, sizeof to_srgb) == cudaSuccess ? 0 : launch_status();
}

// toSrgb (src/nvtt/Surface.cpp:1512-1519), bit-identical to the host libm's
__device__ __forceinline__ float to_srgb(float f) { return to_srgb_exact(f, g_to_srgb_fix); }

__device__ __forceinline__ unsigned to565(f3 v) {
    // vector3_to_color16 (src/nvtt/icbc.h:1580-1595)
    unsigned r = (unsigned)ic_clamp(v.x * 31.0f, 0.0f, 31.0f);
    unsigned g = (unsigned)ic_clamp(v.y * 63.0f, 0.0f, 63.0f);
    unsigned b = (unsigned)ic_clamp(v.z * 31.0f, 0.0f, 31.0f);
    r += (v.x > c_tab.mid5[r]);
    g += (v.y > c_tab.mid6[g]);
    b += (v.z > c_tab.mid5[b]);
    return (r << 11) | (g << 5) | b;
}

__device__ __forceinline__ float round5(float x) { return (float)(int)(x * 31.0f + 0.5f) * (1.0f / 31.0f); }
__device__ __forceinline__ float round6(float x) { return (float)(int)(x * 63.0f + 0.5f) * (1.0f / 63.0f); }
// vround_ept(n * f) (src/nvtt/icbc.h:1572-1578): saturate, then the 5:6:5 grid; the product and the
// clamp are one saturating multiply, equal to saturate(n * f) for every input as far as the snap sees.
__device__ __forceinline__ f3 round_ept(f3 n, float f) {
    return mk3(round5(mul_sat(n.x, f)), round6(mul_sat(n.y, f)), round5(mul_sat(n.z, f)));
}
__device__ __forceinline__ bool is_black(f3 c) { return c.x < 1.0f / 8 && c.y < 1.0f / 8 && c.z < 1.0f / 8; }
__device__ __forceinline__ f3 xyz(float4 v) { return mk3(v.x, v.y, v.z); }

struct Pal3 { f3 p[4]; };
__device__ __forceinline__ void palette_f(unsigned c0, unsigned c1, Pal3 &pf) {
    Pal8 p;
    palette_d3d10(c0, c1, p);
#pragma unroll
    for (int i = 0; i < 4; i++) pf.p[i] = mk3(p.r[i] / 255.0f, p.g[i] / 255.0f, p.b[i] / 255.0f);
}

// compute_indices4 (src/nvtt/icbc.h:2803-2835)
__device__ uint32_t indices4(const Lane<float4> &in, f3 cw, const Pal3 &pal) {
    f3 p0 = pal.p[0] * cw, p1 = pal.p[1] * cw, p2 = pal.p[2] * cw, p3 = pal.p[3] * cw;
    uint32_t idx = 0;
#pragma unroll 4
    for (int i = 0; i < 16; i++) {
        f3 c = xyz(in[i]) * cw;
        f3 t;
        t = c - p0; float d0 = dot(t, t);
        t = c - p1; float d1 = dot(t, t);
        t = c - p2; float d2 = dot(t, t);
        t = c - p3; float d3 = dot(t, t);
        unsigned hi = ((d1 > d2) & (d0 > d2)) | ((d0 > d3) & (d1 > d3));
        unsigned lo = (d0 > d3) & (d2 > d3);
        idx |= ((hi << 1) | lo) << (2 * i);
    }
    return idx;
}

// compute_indices3 (src/nvtt/icbc.h:2837-2882)
__device__ uint32_t indices3(const Lane<float4> &in, f3 cw, bool allow_black, const Pal3 &pal) {
    f3 p0 = pal.p[0] * cw, p1 = pal.p[1] * cw, p2 = pal.p[2] * cw;
    uint32_t idx = 0;
#pragma unroll 4
    for (int i = 0; i < 16; i++) {
        f3 c = xyz(in[i]) * cw;
        f3 t;
        unsigned hi, lo;
        if (allow_black) {
            t = p0 - c; float d0 = dot(t, t);
            t = p1 - c; float d1 = dot(t, t);
            t = p2 - c; float d2 = dot(t, t);
            float d3 = dot(c, c);
            unsigned i1 = d1 < d2, i2 = (d2 <= d0) & (d2 <= d1), i3 = (d3 <= d0) & (d3 <= d1) & (d3 <= d2);
            hi = i2 | i3; lo = i1 | i3;
        } else {
            t = c - p0; float d0 = dot(t, t);
            t = c - p1; float d1 = dot(t, t);
            t = c - p2; float d2 = dot(t, t);
            hi = (d2 <= d0) & (d2 <= d1); lo = d1 < d2;
        }
        idx |= ((hi << 1) | lo) << (2 * i);
    }
    return idx;
}

// compute_indices, live branch (src/nvtt/icbc.h:2885-2941)
__device__ uint32_t indices_any(const Lane<float4> &in, f3 cw, const Pal3 &pal) {
    f3 p0 = pal.p[0] * cw, p1 = pal.p[1] * cw, p2 = pal.p[2] * cw, p3 = pal.p[3] * cw;
    uint32_t idx = 0;
#pragma unroll 4
    for (int i = 0; i < 16; i++) {
        f3 c = xyz(in[i]) * cw;
        f3 t;
        t = c - p0; float d0 = dot(t, t);
        t = c - p1; float d1 = dot(t, t);
        t = c - p2; float d2 = dot(t, t);
        t = c - p3; float d3 = dot(t, t);
        unsigned i1 = (d1 <= d0) & (d1 < d2) & (d1 < d3);
        unsigned i2 = (d2 <= d0) & (d2 <= d1) & (d2 < d3);
        unsigned i3 = (d3 <= d0) & (d3 <= d1) & (d3 <= d2);
        idx |= (((i2 | i3) << 1) | (i1 | i3)) << (2 * i);
    }
    return idx;
}

// evaluate_mse over the input texels (src/nvtt/icbc.h:2733-2756)
template <typename W>
__device__ float block_mse(const Lane<float4> &in, const W &wi, f3 cw, const Pal3 &pal, uint32_t idx) {
    float err = 0.0f;
#pragma unroll 4
    for (int i = 0; i < 16; i++) {
        int k = (idx >> (2 * i)) & 3;
        f3 p = k == 0 ? pal.p[0] : (k == 1 ? pal.p[1] : (k == 2 ? pal.p[2] : pal.p[3]));
        f3 d = ((p - xyz(in[i])) * cw) * 255.0f;
        err += wi[i] * dot(d, d);
    }
    return err;
}

struct Block1 { unsigned c0, c1; uint32_t idx; };

template <typename W>
__device__ float output_block4(const Lane<float4> &in, const W &wi, f3 cw, f3 v0, f3 v1, Block1 &o) {
    unsigned c0 = to565(v0), c1 = to565(v1);
    if (c0 < c1) { unsigned t = c0; c0 = c1; c1 = t; }
    Pal3 pal;
    palette_f(c0, c1, pal);
    o.c0 = c0; o.c1 = c1;
    o.idx = indices4(in, cw, pal);
    return block_mse(in, wi, cw, pal, o.idx);
}

template <typename W>
__device__ float output_block3(const Lane<float4> &in, const W &wi, f3 cw, bool allow_black, f3 v0, f3 v1, Block1 &o) {
    unsigned c0 = to565(v0), c1 = to565(v1);
    if (c0 > c1) { unsigned t = c0; c0 = c1; c1 = t; }
    Pal3 pal;
    palette_f(c0, c1, pal);
    o.c0 = c0; o.c1 = c1;
    o.idx = indices3(in, cw, allow_black, pal);
    return block_mse(in, wi, cw, pal, o.idx);
}

template <typename W>
__device__ __forceinline__ float mse_of(const Lane<float4> &in, const W &wi, f3 cw, const Block1 &o) {
    Pal3 pal;
    palette_f(o.c0, o.c1, pal);
    return block_mse(in, wi, cw, pal, o.idx);
}

// compute_sat (src/nvtt/icbc.h:1812-1882) from n colours (xyz) and weights (w) in `col`.
// Writes the prefix sums in principal-axis order to `sat` (and, when asked, the order itself as
// 4-bit indices into `col`). Returns n.
__device__ int compute_sat(const Lane<float4> &col, int n, const Lane<float4> &sat, uint64_t *order_out = nullptr) {
    // computeCentroid / computeCovariance (src/nvtt/icbc.h:1700-1741)
    f3 c = mk3(0, 0, 0);
    float total = 0.0f;
    for (int i = 0; i < n; i++) { float4 p = col[i]; total += p.w; c = c + xyz(p) * p.w; }
    c = c * (1.0f / total);
    float m0 = 0, m1 = 0, m2 = 0, m3 = 0, m4 = 0, m5 = 0;
    for (int i = 0; i < n; i++) {
        float4 p = col[i];
        f3 a = xyz(p) - c;
        f3 b = a * p.w;
        m0 += a.x * b.x; m1 += a.x * b.y; m2 += a.x * b.z;
        m3 += a.y * b.y; m4 += a.y * b.z; m5 += a.z * b.z;
    }
    // firstEigenVector_PowerMethod (src/nvtt/icbc.h:1760-1790)
    f3 v;
    if (m0 == 0 && m3 == 0 && m5 == 0) {
        v = mk3(0, 0, 0);
    } else {
        f3 r0 = mk3(m0, m1, m2), r1 = mk3(m1, m3, m4), r2 = mk3(m2, m4, m5);
        float l0 = dot(r0, r0), l1 = dot(r1, r1), l2 = dot(r2, r2);
        v = (l0 > l1 && l0 > l2) ? r0 : (l1 > l2 ? r1 : r2);
#pragma unroll
        for (int it = 0; it < 8; it++) {
            float x = v.x * m0 + v.y * m1 + v.z * m2;
            float y = v.x * m1 + v.y * m3 + v.z * m4;
            float z = v.x * m2 + v.y * m4 + v.z * m5;
            float norm = ic_max(ic_max(x, y), z);
            v = mk3(x, y, z) * (1.0f / norm);
        }
    }
    // project and stable insertion sort of (dps, order), packed order in a 64-bit word
    float dps[16];
    uint64_t order = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        dps[i] = i < n ? dot(xyz(col[i]), v) : 0.0f;
        order |= (uint64_t)i << (4 * i);
    }
#pragma unroll
    for (int i = 1; i < 16; i++) {
        bool moving = i < n;
#pragma unroll
        for (int j = i; j > 0; --j) {
            moving = moving && (dps[j] < dps[j - 1]);
            if (moving) {
                float t = dps[j]; dps[j] = dps[j - 1]; dps[j - 1] = t;
                uint64_t a = (order >> (4 * j)) & 15, b = (order >> (4 * (j - 1))) & 15;
                order &= ~((uint64_t)0xFF << (4 * (j - 1)));
                order |= (a << (4 * (j - 1))) | (b << (4 * j));
            }
        }
    }
    if (order_out) *order_out = order;
    float4 acc = col[(int)(order & 15)];
    acc = make_float4(acc.x * acc.w, acc.y * acc.w, acc.z * acc.w, acc.w);
    sat[0] = acc;
    for (int i = 1; i < n; i++) {
        float4 p = col[(int)((order >> (4 * i)) & 15)];
        acc = make_float4(acc.x + p.x * p.w, acc.y + p.y * p.w, acc.z + p.z * p.w, acc.w + p.w);
        sat[i] = acc;
    }
    return n;
}

// compute_sat over `col` in place: the same axis, order and prefix sums, with the colours first
// moved into axis order (each cycle of the permutation followed once) and then summed where they
// lie, so the table needs no storage of its own. Returns n. With `frame_v`, *reversed tells
// whether the first colour in axis order projects above the last on frame_v (axis_reversed).
// The table is a ZERO one: entry k holds the sum of the first k colours (entry 0 zero, n + 1
// entries), so that a cumulative cluster end indexes it directly.
__device__ int compute_sat_inplace(const Lane<float4> &col, int n, const f3 *frame_v = nullptr, bool *reversed = nullptr) {
    // computeCentroid / computeCovariance / firstEigenVector_PowerMethod as in compute_sat
    f3 c = mk3(0, 0, 0);
    float total = 0.0f;
    for (int i = 0; i < n; i++) { float4 p = col[i]; total += p.w; c = c + xyz(p) * p.w; }
    c = c * (1.0f / total);
    float m0 = 0, m1 = 0, m2 = 0, m3 = 0, m4 = 0, m5 = 0;
    for (int i = 0; i < n; i++) {
        float4 p = col[i];
        f3 a = xyz(p) - c;
        f3 b = a * p.w;
        m0 += a.x * b.x; m1 += a.x * b.y; m2 += a.x * b.z;
        m3 += a.y * b.y; m4 += a.y * b.z; m5 += a.z * b.z;
    }
    f3 v;
    if (m0 == 0 && m3 == 0 && m5 == 0) {
        v = mk3(0, 0, 0);
    } else {
        f3 r0 = mk3(m0, m1, m2), r1 = mk3(m1, m3, m4), r2 = mk3(m2, m4, m5);
        float l0 = dot(r0, r0), l1 = dot(r1, r1), l2 = dot(r2, r2);
        v = (l0 > l1 && l0 > l2) ? r0 : (l1 > l2 ? r1 : r2);
#pragma unroll
        for (int it = 0; it < 8; it++) {
            float x = v.x * m0 + v.y * m1 + v.z * m2;
            float y = v.x * m1 + v.y * m3 + v.z * m4;
            float z = v.x * m2 + v.y * m4 + v.z * m5;
            float norm = ic_max(ic_max(x, y), z);
            v = mk3(x, y, z) * (1.0f / norm);
        }
    }
    float dps[16];
    uint64_t order = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        dps[i] = i < n ? dot(xyz(col[i]), v) : 0.0f;
        order |= (uint64_t)i << (4 * i);
    }
#pragma unroll
    for (int i = 1; i < 16; i++) {
        bool moving = i < n;
#pragma unroll
        for (int j = i; j > 0; --j) {
            moving = moving && (dps[j] < dps[j - 1]);
            if (moving) {
                float t = dps[j]; dps[j] = dps[j - 1]; dps[j - 1] = t;
                uint64_t a = (order >> (4 * j)) & 15, b = (order >> (4 * (j - 1))) & 15;
                order &= ~((uint64_t)0xFF << (4 * (j - 1)));
                order |= (a << (4 * (j - 1))) | (b << (4 * j));
            }
        }
    }
    // col[i] <- col[order_i] for i < n (the order is a permutation of [0, n))
    uint32_t done = 0;
    for (int s = 0; s < n; s++) {
        if (done & (1u << s)) continue;
        const float4 first = col[s];
        int i = s;
        for (int step = 0; step < 16; step++) {
            done |= 1u << i;
            const int p = (int)((order >> (4 * i)) & 15);
            if (p == s) break;
            col[i] = col[p];
            i = p;
        }
        col[i] = first;
    }
    if (frame_v) *reversed = dot(xyz(col[0]), *frame_v) > dot(xyz(col[n - 1]), *frame_v);
    float4 acc = col[0];
    acc = make_float4(acc.x * acc.w, acc.y * acc.w, acc.z * acc.w, acc.w);
    col[0] = make_float4(0, 0, 0, 0);
    for (int i = 1; i < n; i++) {
        float4 p = col[i];  // read colour i before its slot takes the sum of the first i
        col[i] = acc;
        acc = make_float4(acc.x + p.x * p.w, acc.y + p.y * p.w, acc.z + p.z * p.w, acc.w + p.w);
    }
    col[n] = acc;
    return n;
}

// round_ept on a packed endpoint: the same operations per channel (saturating scale, k x + 0.5,
// truncation, 1 / k), the additions and the final scale packed for x and y.
__device__ __forceinline__ P3 round_eptp(P3 n, float f) {
    float nx, ny;
    f2_unpack(n.xy, nx, ny);
    const float x = mul_sat(nx, f), y = mul_sat(ny, f), z = mul_sat(n.z, f);
    float gx, gy;
    f2_unpack(f2_add(f2_pack(x * 31.0f, y * 63.0f), f2_pack(0.5f, 0.5f)), gx, gy);
    return P3{f2_mul(f2_pack((float)(int)gx, (float)(int)gy), f2_pack(1.0f / 31.0f, 1.0f / 63.0f)), round5(z)};
}

// Shared solve / snap / residual of cluster_fit_three and cluster_fit_four
// (src/nvtt/icbc.h:2200-2240, 2501-2540): bx = sum - ax, a = snap((ax b2 - bx ab) factor),
// b = snap((bx a2 - ax ab) factor), e2 = 2 (a (b ab - ax) - b bx), e1 = (a a) a2 + ((b b) b2 + e2),
// with x and y packed where that is exact (sums, differences, products that feed no sum).
__device__ __forceinline__ float cf_eval(P3 axq, P3 sum, float a2, float b2, float ab, f3 metric, f3 &pa, f3 &pb) {
    float factor = 1.0f / (a2 * b2 - ab * ab);
    const P3 bxq = p3_sub(sum, axq);
    const f3 ax = u3(axq), bx = u3(bxq);
    const P3 aq = round_eptp(p3_sub(p3(ax * b2), p3(bx * ab)), factor);
    const P3 bq = round_eptp(p3_sub(p3(bx * a2), p3(ax * ab)), factor);
    const f3 a = u3(aq), b = u3(bq);
    const f3 e2 = u3(p3_sub(p3(a * u3(p3_sub(p3(b * ab), axq))), p3(b * bx))) * 2.0f;
    const f3 e1 = u3(p3_add(p3(u3(p3_mul(aq, aq)) * a2), p3_add(p3(u3(p3_mul(bq, bq)) * b2), p3(e2))));
    pa = a; pb = b;
    return dot(e1, metric);
}

// One ordering of cluster_fit_four (src/nvtt/icbc.h:2250-2549): cumulative cluster ends from the
// SAT, solve, snap, residual. The last end is never 0 (the ordering tables leave out the empty
// split, src/nvtt/icbc.h:1913-1914), so its SAT entry needs no check; with a ZERO table (entry 0
// zero) no end does.
// The ordering from the SAT entries of its three cumulative ends.
__device__ __forceinline__ float four_eval_v(float4 v0, float4 v1, float4 v2, f3 sum, float wsum, f3 metric, f3 &a,
                                             f3 &b) {
    float w0 = v0.w, w1 = v1.w, w2 = v2.w;
    const float w3 = wsum - w2;
    const P3 x0 = p3(xyz(v0)), x1 = p3_sub(p3(xyz(v1)), x0), x2 = p3_sub(p3(xyz(v2)), p3(xyz(v1)));
    w2 = w2 - w1;
    w1 = w1 - w0;
    const float a2 = w2 * (1.0f / 9.0f) + (w1 * (4.0f / 9.0f) + w0);
    const float b2 = w1 * (1.0f / 9.0f) + (w2 * (4.0f / 9.0f) + w3);
    const float ab = (w1 + w2) * (2.0f / 9.0f);
    // ax = x2 / 3 + (2 x1 / 3 + x0)
    const P3 ax = p3_add(p3(u3(x2) * (1.0f / 3.0f)), p3_add(p3(u3(x1) * (2.0f / 3.0f)), x0));
    return cf_eval(ax, p3(sum), a2, b2, ab, metric, a, b);
}

template <bool ZERO = false>
__device__ __forceinline__ float four_eval(const Lane<float4> &sat, uint32_t o, f3 sum, float wsum, f3 metric, f3 &a,
                                           f3 &b) {
    const int d = ZERO ? 0 : 1;
    const int c0 = (int)(o & 255) - d, c1 = (int)((o >> 8) & 255) - d, c2 = (int)((o >> 16) & 255) - d;
    const float4 v0 = (ZERO || c0 >= 0) ? sat[c0] : make_float4(0, 0, 0, 0);
    const float4 v1 = (ZERO || c1 >= 0) ? sat[c1] : make_float4(0, 0, 0, 0);
    return four_eval_v(v0, v1, sat[c2], sum, wsum, metric, a, b);
}

// The first strict minimum over all orderings wins, as in the scalar build. The search keeps the
// index of the best ordering; its endpoints are recomputed once at the end. Over a ZERO table the
// orderings are walked as the nest the table lists them in (last end t = 1..n, first end 0..t,
// second end first..t: build_device_tables), so that the last and first ends' entries stay loaded.
template <bool ZERO = false>
__device__ void cluster_fit_four(const Lane<float4> &sat, int n, f3 metric, f3 &start, f3 &end) {
    const float4 s = sat[ZERO ? n : n - 1];
    const f3 sum = xyz(s);
    const float wsum = s.w;
    float best = FLT_MAX;
    int bi = -1;
    if (ZERO) {
        int i = 0;
        for (int t = 1; t <= n; t++) {
            const float4 v2 = sat[t];
            for (int c0 = 0; c0 <= t; c0++) {
                const float4 v0 = sat[c0];
                for (int c1 = c0; c1 <= t; c1++, i++) {
                    f3 a, b;
                    const float e = four_eval_v(v0, sat[c1], v2, sum, wsum, metric, a, b);
                    if (e < best) { best = e; bi = i; }
                }
            }
        }
    } else {
        const int total = c_tab.four_total[n - 1];
        for (int i = 0; i < total; i++) {
            f3 a, b;
            const float e = four_eval<ZERO>(sat, c_tab.four[i], sum, wsum, metric, a, b);
            if (e < best) { best = e; bi = i; }
        }
    }
    start = mk3(0, 0, 0);
    end = mk3(0, 0, 0);
    if (bi >= 0) four_eval<ZERO>(sat, c_tab.four[bi], sum, wsum, metric, start, end);
}

// The full search's best ordering code (0 when none), for training targets.
__device__ uint32_t best_order_four(const Lane<float4> &sat, int n, f3 metric) {
    const float4 s = sat[n - 1];
    const f3 sum = xyz(s);
    float best = FLT_MAX;
    uint32_t bo = 0;
    const int total = c_tab.four_total[n - 1];
    for (int i = 0; i < total; i++) {
        f3 a, b;
        const float e = four_eval(sat, c_tab.four[i], sum, s.w, metric, a, b);
        if (e < best) { best = e; bo = c_tab.four[i]; }
    }
    return bo;
}

// One ordering of cluster_fit_three (src/nvtt/icbc.h:2016-2247); its last end is never 0 either
// (src/nvtt/icbc.h:1948-1949).
__device__ __forceinline__ float three_eval_v(float4 v0, float4 v1, f3 sum, float wsum, f3 metric, f3 &a, f3 &b) {
    float w0 = v0.w, w1 = v1.w;
    const float w2 = wsum - w1;
    const P3 x0 = p3(xyz(v0)), x1 = p3_sub(p3(xyz(v1)), x0);
    w1 = w1 - w0;
    const float ab = w1 * 0.25f;
    const float a2 = w0 + ab;
    const float b2 = w2 + ab;
    const P3 ax = p3_add(x0, p3(u3(x1) * 0.5f));
    return cf_eval(ax, p3(sum), a2, b2, ab, metric, a, b);
}

template <bool ZERO = false>
__device__ __forceinline__ float three_eval(const Lane<float4> &sat, uint32_t o, f3 sum, float wsum, f3 metric, f3 &a,
                                            f3 &b) {
    const int d = ZERO ? 0 : 1;
    const int c0 = (int)(o & 255) - d, c1 = (int)((o >> 8) & 255) - d;
    const float4 v0 = (ZERO || c0 >= 0) ? sat[c0] : make_float4(0, 0, 0, 0);
    return three_eval_v(v0, sat[c1], sum, wsum, metric, a, b);
}

__device__ uint32_t best_order_three(const Lane<float4> &sat, int n, f3 metric) {
    const float4 s = sat[n - 1];
    const f3 sum = xyz(s);
    float best = FLT_MAX;
    uint32_t bo = 0;
    const int total = c_tab.three_total[n - 1];
    for (int i = 0; i < total; i++) {
        f3 a, b;
        const float e = three_eval(sat, c_tab.three[i], sum, s.w, metric, a, b);
        if (e < best) { best = e; bo = c_tab.three[i]; }
    }
    return bo;
}

template <bool ZERO = false>
__device__ void cluster_fit_three(const Lane<float4> &sat, int n, f3 metric, f3 &start, f3 &end) {
    const float4 s = sat[ZERO ? n : n - 1];
    const f3 sum = xyz(s);
    const float wsum = s.w;
    float best = FLT_MAX;
    int bi = -1;
    if (ZERO) {  // the table's nest: last end t = 1..n, first end 0..t
        int i = 0;
        for (int t = 1; t <= n; t++) {
            const float4 v1 = sat[t];
            for (int c0 = 0; c0 <= t; c0++, i++) {
                f3 a, b;
                const float e = three_eval_v(sat[c0], v1, sum, wsum, metric, a, b);
                if (e < best) { best = e; bi = i; }
            }
        }
    } else {
        const int total = c_tab.three_total[n - 1];
        for (int i = 0; i < total; i++) {
            f3 a, b;
            const float e = three_eval<ZERO>(sat, c_tab.three[i], sum, wsum, metric, a, b);
            if (e < best) { best = e; bi = i; }
        }
    }
    start = mk3(0, 0, 0);
    end = mk3(0, 0, 0);
    if (bi >= 0) three_eval<ZERO>(sat, c_tab.three[bi], sum, wsum, metric, start, end);
}

// refine_endpoints (src/nvtt/icbc.h:3329-3406), including the reference's use of the current
// output's palette (not the candidate's) for index selection.
template <typename W>
__device__ float refine_endpoints(const Lane<float4> &in, const W &wi, f3 cw, float err, Block1 &o) {
    const int8_t deltas[16][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1},
                                  {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {-1, -1, 0}, {-1, 0, -1}, {0, -1, -1},
                                  {-1, 1, 0}, {1, -1, 0}, {0, -1, 1}, {0, 1, -1}};
    float best = err;
    int last = 0;
    for (int i = 0; i < 256; i++) {
        Block1 r = o;
        const int8_t *d = deltas[i % 16];
        unsigned c = ((i / 16) & 1) ? r.c0 : r.c1;
        unsigned cr = ((c >> 11) + d[0]) & 31, cg = (((c >> 5) & 63) + d[1]) & 63, cb = ((c & 31) + d[2]) & 31;
        c = (cr << 11) | (cg << 5) | cb;
        if ((i / 16) & 1) r.c0 = c; else r.c1 = c;
        Pal3 pal;
        palette_f(o.c0, o.c1, pal);
        r.idx = indices_any(in, cw, pal);
        float e = mse_of(in, wi, cw, r);
        if (e < best) { best = e; o = r; last = i; }
        if (i - last > 32) break;
    }
    return best;
}

__device__ __forceinline__ void store_block(uint8_t *dst, const Block1 &o) {
    uint2 v;
    v.x = (o.c0 & 0xFFFF) | (o.c1 << 16);
    v.y = o.idx;
    *reinterpret_cast<uint2 *>(dst) = v;
}

// compress_dxt1 with NVTT's arguments: three-colour mode and transparent black enabled
// (src/nvtt/icbc.h:3485-3559, src/nvtt/BlockCompressor.cpp:219-222).
__device__ __forceinline__ int find_job(const EncJob *jobs, int njobs, long long blk) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_block <= blk) lo = mid; else hi = mid - 1;
    }
    return lo;
}


__device__ __forceinline__ void put_weight(const LaneW &w, int k, float v) { w[k] = v; }
__device__ __forceinline__ void put_weight(const Lane<float> &w, int k, float v) { w[k] = v; }
__device__ __forceinline__ void put_weight(const AlphaW &, int, float) {}  // derived when read

// Bit 4y + x set for the texels (x, y) of block `blk` that lie inside the image.
__device__ __forceinline__ uint32_t valid_texels(const EncJob &J, int blk) {
    const int bx = blk % J.bw, by = blk / J.bw;
    const int vw = min(J.w - bx * 4, 4), vh = min(J.h - by * 4, 4);
    const uint32_t row = (1u << vw) - 1u;
    uint32_t m = 0;
    for (int y = 0; y < vh; y++) m |= row << (4 * y);
    return m;
}

// FloatColorCompressorTask gather (src/nvtt/BlockCompressor.cpp:116-166): the block's 16 texels
// after the output transform, weight saturate(alpha) under AlphaMode_Transparency, texels outside
// the image at weight 0.
template <typename W>
__device__ __forceinline__ void gather_block(const EncJob &J, int blk, const Lane<float4> &in, const W &wi) {
    const int bx = blk % J.bw, by = blk / J.bw;
    const size_t n = (size_t)J.w * J.h;
    const int vw = min(J.w - bx * 4, 4), vh = min(J.h - by * 4, 4);
#pragma unroll
    for (int y = 0; y < 4; y++)
#pragma unroll
        for (int x = 0; x < 4; x++) {
            const int k = 4 * y + x;
            if (x < vw && y < vh) {
                const size_t s = (size_t)(by * 4 + y) * J.w + (bx * 4 + x);
                float r, g, b, al;
                if (J.bgra) {
                    // 8-bit source through the composed input/output transform table
                    const uint32_t p = J.bgra[s];
                    r = J.lut_f[(p >> 16) & 255]; g = J.lut_f[(p >> 8) & 255]; b = J.lut_f[p & 255];
                    al = (float)(p >> 24) / 255.0f;
                } else {
                    r = J.rgba[s]; g = J.rgba[n + s]; b = J.rgba[2 * n + s]; al = J.rgba[3 * n + s];
                    if (J.out_xform == 1) { r = powf_5_11(r); g = powf_5_11(g); b = powf_5_11(b); }
                    else if (J.out_xform == 2) { r = to_srgb(r); g = to_srgb(g); b = to_srgb(b); }
                }
                in[k] = make_float4(r, g, b, al);
                put_weight(wi, k, J.alpha_mode == 1 ? ic_clamp(al, 0.0f, 1.0f) : 1.0f);
            } else {
                in[k] = make_float4(0, 0, 0, 0);
                put_weight(wi, k, 0.0f);
            }
        }
}

// reduce_colors (src/nvtt/icbc.h:1638-1683), threshold 1/256: merges near-equal colours of
// positive weight into `col` (weighted mean, summed weight). Returns the colour count.
template <typename W>
__device__ __forceinline__ int reduce_colors(const Lane<float4> &in, const W &wi, const Lane<float4> &col,
                                             bool &any_black) {
    const float thr = 1.0f / 256;
    int cnt = 0;
    any_black = false;
    for (int i = 0; i < 16; i++) {
        float wt = wi[i];
        if (wt > 0) {
            f3 c = xyz(in[i]);
            int j;
            for (j = 0; j < cnt; j++) {
                float4 q = col[j];
                if (fabsf(q.x - c.x) < thr && fabsf(q.y - c.y) < thr && fabsf(q.z - c.z) < thr) {
                    float den = q.w + wt;
                    f3 s = (xyz(q) * q.w) + (c * wt);
                    col[j] = make_float4(s.x / den, s.y / den, s.z / den, q.w + wt);
                    break;
                }
            }
            if (j == cnt) { col[cnt] = make_float4(c.x, c.y, c.z, wt); cnt++; }
            if (is_black(c)) any_black = true;
        }
    }
    return cnt;
}

// compress_dxt1_single_color_optimal (src/nvtt/icbc.h:3274-3289)
__device__ __forceinline__ Block1 single_colour(float4 c) {
    Block1 o;
    int r = (int)(uint8_t)(ic_sat(c.x) * 255 + 0.5f);
    int g = (int)(uint8_t)(ic_sat(c.y) * 255 + 0.5f);
    int b = (int)(uint8_t)(ic_sat(c.z) * 255 + 0.5f);
    o.c0 = ((unsigned)c_tab.icbc_match5[r][0] << 11) | ((unsigned)c_tab.icbc_match6[g][0] << 5) | c_tab.icbc_match5[b][0];
    o.c1 = ((unsigned)c_tab.icbc_match5[r][1] << 11) | ((unsigned)c_tab.icbc_match6[g][1] << 5) | c_tab.icbc_match5[b][1];
    o.idx = 0xaaaaaaaau;
    if (o.c0 < o.c1) { unsigned tt = o.c0; o.c0 = o.c1; o.c1 = tt; o.idx ^= 0x55555555u; }
    return o;
}

template <int LEVEL>  // 0: icbc Level1, 7: Level8, 8: Level9
__global__ void __launch_bounds__(64) k_bc1(const EncJob *__restrict__ jobs, int njobs, long long nblocks,
                                            const long long *__restrict__ list, const unsigned long long *__restrict__ count) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x;
    const int t = threadIdx.x;
    long long gblk = (long long)blockIdx.x * T + t;
    if (gblk >= nblocks) return;
    if (list) {  // a subset of the jobs' blocks (the learned path's fallbacks), *count long
        if ((unsigned long long)gblk >= *count) return;
        gblk = list[gblk];
    }
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    // 17 float4 slots per thread: the texels (16) and one more. The weights are derived from the
    // texels when read (AlphaW). The reduced colours overwrite the texels in place (reduce_colors
    // only writes slots it has already read), the summed-area table overwrites the colours in place
    // with a zero entry first (17 entries), and the texels are gathered again for the output stage
    // once the cluster fits are done.
    Lane<float4> in{smem + t, T};
    Lane<float4> col = in;
    Lane<float4> sat = in;
    const AlphaW wi{smem + t, T, J.alpha_mode == 1, valid_texels(J, blk)};
    const f3 cw = mk3(J.cw[0], J.cw[1], J.cw[2]);
    uint8_t *const out = J.out + 8 * (size_t)blk;

    gather_block(J, blk, in, wi);

    Block1 o{0, 0, 0};
    float err = FLT_MAX;

    if (LEVEL == 0) {
        // Level1: box fit of all 16 texels, inset, diagonal, then least squares
        // (src/nvtt/icbc.h:3096-3151, 2984-3016)
        f3 c0 = mk3(0, 0, 0), c1 = mk3(1, 1, 1);
        for (int i = 0; i < 16; i++) {
            f3 p = xyz(in[i]);
            c0 = mk3(ic_max(c0.x, p.x), ic_max(c0.y, p.y), ic_max(c0.z, p.z));
            c1 = mk3(ic_min(c1.x, p.x), ic_min(c1.y, p.y), ic_min(c1.z, p.z));
        }
        const float bias = (8.0f / 255.0f) / 16.0f;
        f3 d = c0 - c1;
        f3 inset = mk3(d.x / 16.0f, d.y / 16.0f, d.z / 16.0f) - mk3(bias, bias, bias);
        c0 = sat3(c0 - inset);
        c1 = sat3(c1 + inset);
        f3 center = (c0 + c1) * 0.5f;
        float cxz = 0.0f, cyz = 0.0f;
        for (int i = 0; i < 16; i++) { f3 tt = xyz(in[i]) - center; cxz += tt.x * tt.z; cyz += tt.y * tt.z; }
        float x0 = c0.x, y0 = c0.y, x1 = c1.x, y1 = c1.y;
        if (cxz < 0) { float tt = x0; x0 = x1; x1 = tt; }
        if (cyz < 0) { float tt = y0; y0 = y1; y1 = tt; }
        c0 = mk3(x0, y0, c0.z); c1 = mk3(x1, y1, c1.z);
        err = output_block4(in, wi, cw, c0, c1, o);
        // optimize_end_points4 on the 16 input texels
        float a2 = 0, b2 = 0, ab = 0;
        f3 ax = mk3(0, 0, 0), bxs = mk3(0, 0, 0);
        for (int i = 0; i < 16; i++) {
            unsigned bits = o.idx >> (2 * i);
            float beta = (float)(bits & 1);
            if (bits & 2) beta = (1 + beta) / 3.0f;
            float alpha = 1.0f - beta;
            f3 p = xyz(in[i]);
            a2 += alpha * alpha; b2 += beta * beta; ab += alpha * beta;
            ax = ax + p * alpha; bxs = bxs + p * beta;
        }
        float den = a2 * b2 - ab * ab;
        if (!(fabsf(den - 0.0f) < 0.0001f)) {
            float f = 1.0f / den;
            f3 na = sat3(((ax * b2) - (bxs * ab)) * f);
            f3 nb = sat3(((bxs * a2) - (ax * ab)) * f);
            Block1 t2;
            float e2 = output_block4(in, wi, cw, na, nb, t2);
            if (e2 < err) { err = e2; o = t2; }
        }
        store_block(out, o);
        return;
    }

    bool any_black = false;
    const int cnt = reduce_colors(in, wi, col, any_black);

    if (cnt == 0) {
        store_block(out, Block1{0, 0, 0});
        return;
    }
    if (cnt == 1) {
        store_block(out, single_colour(col[0]));
        return;
    }

    // compress_dxt1_cluster_fit (src/nvtt/icbc.h:3292-3325); both fits first, then the output stage
    // (pure functions of the texels and the endpoints, so their order does not matter)
    const f3 metric = cw * cw;
    int sn = compute_sat_inplace(col, cnt);
    f3 s0, s1, t0, t1;
    cluster_fit_four<true>(sat, sn, metric, s0, s1);
    bool run3 = true;
    if (any_black) {
        // the table has replaced the colours: reduce them again (the same colours), then
        // skip_blacks in place, compacting the non-black ones to the front of `col`
        gather_block(J, blk, in, wi);
        bool again = false;
        reduce_colors(in, wi, col, again);
        int m = 0;
        for (int i = 0; i < cnt; i++) {
            float4 q = col[i];
            if (is_black(xyz(q))) continue;
            col[m++] = q;
        }
        if (m == 0) run3 = false;
        else sn = compute_sat_inplace(col, m);
    }
    if (run3) cluster_fit_three<true>(sat, sn, metric, t0, t1);
    gather_block(J, blk, in, wi);
    Block1 cf;
    float cerr = output_block4(in, wi, cw, s0, s1, cf);
    if (run3) {
        Block1 c3;
        float e3 = output_block3(in, wi, cw, true, t0, t1, c3);
        if (e3 < cerr) { cerr = e3; cf = c3; }
    }
    // taken only when its error compares below FLT_MAX: a NaN error leaves the block as the
    // reference leaves it unwritten (this build writes zeros there)
    if (cerr < err) { o = cf; err = cerr; }
    if (LEVEL == 8) err = refine_endpoints(in, wi, cw, err, o);
    store_block(out, o);
}

// The first strict minimum of a search split over the K lanes of a group, lane j having taken the
// orderings i = j (mod K) with its own first strict minimum (e, i) (FLT_MAX, -1 when none): the
// smallest error, and among equal errors the smallest ordering - the ordering the sequential search
// keeps. Every lane of the group returns it.
template <int K>
__device__ __forceinline__ int group_first_min(unsigned gmask, float e, int i) {
#pragma unroll
    for (int off = K / 2; off > 0; off >>= 1) {
        const float eo = __shfl_xor_sync(gmask, e, off, K);
        const int io = __shfl_xor_sync(gmask, i, off, K);
        if (eo < e || (eo == e && io < i)) { e = eo; i = io; }
    }
    return i;
}

// cluster_fit_four / cluster_fit_three over a ZERO table, lane j of K evaluating the orderings
// j, j + K, ... of the icbc tables (listed in the sequential search's order); returns the group's best
// ordering (-1 when none).
template <int K>
__device__ int split_fit_four(unsigned gmask, const Lane<float4> &sat, int n, f3 metric, int j) {
    const float4 s = sat[n];
    const f3 sum = xyz(s);
    float best = FLT_MAX;
    int bi = -1;
    const int total = c_tab.four_total[n - 1];
    for (int i = j; i < total; i += K) {
        f3 a, b;
        const float e = four_eval<true>(sat, c_tab.four[i], sum, s.w, metric, a, b);
        if (e < best) { best = e; bi = i; }
    }
    return group_first_min<K>(gmask, best, bi);
}
template <int K>
__device__ int split_fit_three(unsigned gmask, const Lane<float4> &sat, int n, f3 metric, int j) {
    const float4 s = sat[n];
    const f3 sum = xyz(s);
    float best = FLT_MAX;
    int bi = -1;
    const int total = c_tab.three_total[n - 1];
    for (int i = j; i < total; i += K) {
        f3 a, b;
        const float e = three_eval<true>(sat, c_tab.three[i], sum, s.w, metric, a, b);
        if (e < best) { best = e; bi = i; }
    }
    return group_first_min<K>(gmask, best, bi);
}

// k_bc1 for launches too small to fill the GPU with one thread per block: a group of K lanes of one
// warp encodes each block (64 / K blocks per 64-thread CTA). The group's first lane gathers, reduces
// and builds the summed-area table, in 17 float4 slots of shared memory per block; the K lanes split
// the orderings of each cluster fit; the first lane recomputes the winners' endpoints and runs the
// output stage. The same operations on the same values as k_bc1, so the same blocks.
template <int LEVEL, int K>
__global__ void __launch_bounds__(64) k_bc1_split(const EncJob *__restrict__ jobs, int njobs, long long nblocks) {
    extern __shared__ float4 smem[];
    constexpr int G = 64 / K;  // blocks per CTA
    const int t = threadIdx.x, g = t / K, j = t % K;
    const long long gblk = (long long)blockIdx.x * G + g;
    if (gblk >= nblocks) return;  // the whole group leaves together
    const unsigned gmask = ((1u << K) - 1u) << ((t & 31) & ~(K - 1));
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    Lane<float4> in{smem + 17 * g, 1};  // one block's slots, consecutive: the lanes read different ones
    Lane<float4> col = in;
    Lane<float4> sat = in;
    const AlphaW wi{smem + 17 * g, 1, J.alpha_mode == 1, valid_texels(J, blk)};
    const f3 cw = mk3(J.cw[0], J.cw[1], J.cw[2]);
    const f3 metric = cw * cw;
    uint8_t *const out = J.out + 8 * (size_t)blk;

    int cnt = 0, sn = 0, black = 0;
    if (j == 0) {
        gather_block(J, blk, in, wi);
        bool any_black = false;
        cnt = reduce_colors(in, wi, col, any_black);
        black = any_black;
        if (cnt == 0) store_block(out, Block1{0, 0, 0});
        else if (cnt == 1) store_block(out, single_colour(col[0]));
        else sn = compute_sat_inplace(col, cnt);
    }
    cnt = __shfl_sync(gmask, cnt, 0, K);
    if (cnt <= 1) return;
    sn = __shfl_sync(gmask, sn, 0, K);
    black = __shfl_sync(gmask, black, 0, K);
    __syncwarp(gmask);  // the table is written

    f3 s0 = mk3(0, 0, 0), s1 = mk3(0, 0, 0), t0 = mk3(0, 0, 0), t1 = mk3(0, 0, 0);
    const int b4 = split_fit_four<K>(gmask, sat, sn, metric, j);
    int run3 = 1;
    if (j == 0) {
        if (b4 >= 0) four_eval<true>(sat, c_tab.four[b4], xyz(sat[sn]), sat[sn].w, metric, s0, s1);
    }
    __syncwarp(gmask);  // every lane is done with the table
    if (black) {
        if (j == 0) {
            // the table has replaced the colours: reduce them again, then keep the non-black ones
            gather_block(J, blk, in, wi);
            bool again = false;
            reduce_colors(in, wi, col, again);
            int m = 0;
            for (int i = 0; i < cnt; i++) {
                float4 q = col[i];
                if (is_black(xyz(q))) continue;
                col[m++] = q;
            }
            if (m == 0) run3 = 0;
            else sn = compute_sat_inplace(col, m);
        }
        run3 = __shfl_sync(gmask, run3, 0, K);
        sn = __shfl_sync(gmask, sn, 0, K);
        __syncwarp(gmask);
    }
    if (run3) {
        const int b3 = split_fit_three<K>(gmask, sat, sn, metric, j);
        if (j == 0 && b3 >= 0) three_eval<true>(sat, c_tab.three[b3], xyz(sat[sn]), sat[sn].w, metric, t0, t1);
        __syncwarp(gmask);
    }
    if (j != 0) return;
    gather_block(J, blk, in, wi);
    Block1 o{0, 0, 0};
    float err = FLT_MAX;
    Block1 cf;
    float cerr = output_block4(in, wi, cw, s0, s1, cf);
    if (run3) {
        Block1 c3;
        const float e3 = output_block3(in, wi, cw, true, t0, t1, c3);
        if (e3 < cerr) { cerr = e3; cf = c3; }
    }
    if (cerr < err) { o = cf; err = cerr; }
    if (LEVEL == 8) err = refine_endpoints(in, wi, cw, err, o);
    store_block(out, o);
}

// ---------------------------------------------------------------------------------------------
// Learned endpoint proposal (no counterpart in the reference). The network reads a block's texels
// and proposes its two endpoints and the error of the full cluster fit. The proposal's palette
// assigns each of the block's reduced colours, in the cluster fit's principal-axis order, to a
// cluster; the cumulative cluster ends give an ordering of cluster_fit_four (and of
// cluster_fit_three), and only the orderings within `radius` of it in every cluster end are
// evaluated - with the same arithmetic and in the same order as the full search, so a block whose
// best ordering lies in that neighbourhood gets exactly the full fit's result. A block whose
// pruned result's error exceeds (1 + margin) x the network's estimate of the full fit's error is
// listed for the full fit.

// The network works in each block's principal frame: texels centred on the block's weighted mean,
// divided by its RMS deviation (plus 1/255), rotated onto the principal axis v of their weighted
// covariance (power iteration as in the cluster fit; v points towards brighter colours) and two
// axes orthogonal to it, and sorted along v (stable; texels of weight 0 sit at the mean). The
// endpoints are expressed in the same frame, and the fit's error as a log ratio to the block's
// total weighted variance V (evaluate_mse's units): err_estimate = (V + 1) exp(y6) - 1.
struct Frame {
    f3 mu, v, u1, u2;
    float sigma, var;
    __device__ f3 to(f3 c) const {
        const f3 d = (c - mu) * (1.0f / sigma);
        return mk3(dot(d, v), dot(d, u1), dot(d, u2));
    }
    __device__ f3 from(f3 q) const { return mu + ((v * q.x) + ((u1 * q.y) + (u2 * q.z))) * sigma; }
};

template <typename W>
__device__ __forceinline__ Frame block_frame(const Lane<float4> &in, const W &wi, f3 cw) {
    Frame f;
    float ws = 0.0f;
    f3 m = mk3(0, 0, 0);
    for (int i = 0; i < 16; i++) { const float w = wi[i]; ws += w; m = m + xyz(in[i]) * w; }
    f.mu = ws > 0 ? m * (1.0f / ws) : mk3(0, 0, 0);
    float ss = 0.0f, var = 0.0f, m0 = 0, m1 = 0, m2 = 0, m3 = 0, m4 = 0, m5 = 0;
    for (int i = 0; i < 16; i++) {
        const float w = wi[i];
        const f3 d = xyz(in[i]) - f.mu;
        const f3 dw = (d * cw) * 255.0f;
        ss += w * dot(d, d);
        var += w * dot(dw, dw);
        m0 += w * d.x * d.x; m1 += w * d.x * d.y; m2 += w * d.x * d.z;
        m3 += w * d.y * d.y; m4 += w * d.y * d.z; m5 += w * d.z * d.z;
    }
    f.sigma = (ws > 0 ? sqrtf(ss / (3.0f * ws)) : 0.0f) + 1.0f / 255.0f;
    f.var = var;
    f3 v = mk3(1, 1, 1);
    if (!(m0 == 0 && m3 == 0 && m5 == 0)) {
        const f3 r0 = mk3(m0, m1, m2), r1 = mk3(m1, m3, m4), r2 = mk3(m2, m4, m5);
        const float l0 = dot(r0, r0), l1 = dot(r1, r1), l2 = dot(r2, r2);
        v = (l0 > l1 && l0 > l2) ? r0 : (l1 > l2 ? r1 : r2);
        for (int it = 0; it < 8; it++) {
            const f3 q = mk3(v.x * m0 + v.y * m1 + v.z * m2, v.x * m1 + v.y * m3 + v.z * m4, v.x * m2 + v.y * m4 + v.z * m5);
            const float nrm = sqrtf(dot(q, q));
            if (!(nrm > 0)) break;
            v = q * (1.0f / nrm);
        }
    }
    float vn = sqrtf(dot(v, v));
    v = vn > 0 ? v * (1.0f / vn) : mk3(0.57735027f, 0.57735027f, 0.57735027f);
    if (v.x + v.y + v.z < 0) v = v * -1.0f;
    // the coordinate axis least aligned with v, made orthogonal to it; then their cross product
    const float ax = fabsf(v.x), ay = fabsf(v.y), az = fabsf(v.z);
    f3 e = ax <= ay && ax <= az ? mk3(1, 0, 0) : (ay <= az ? mk3(0, 1, 0) : mk3(0, 0, 1));
    f3 u1 = e - v * dot(e, v);
    u1 = u1 * (1.0f / sqrtf(dot(u1, u1)));
    f.v = v;
    f.u1 = u1;
    f.u2 = mk3(v.y * u1.z - v.z * u1.y, v.z * u1.x - v.x * u1.z, v.x * u1.y - v.y * u1.x);
    return f;
}

// The network's input: the block's 16 texels as RGB in [0, 1] (as the encoder sees them), in
// order of their projection on the block's principal axis v (stable), each pulled towards the block's
// weighted mean colour in proportion to its fit weight, mu + w (c - mu) (w = 1 for opaque texels,
// saturate(alpha) under transparency: a texel of weight 0 sits at the mean), so that the network sees
// how much each texel counts. Each warp stages its 32 rows in shared memory and writes them out as
// one contiguous, coalesced run.
constexpr int FEAT_STRIDE = 49;  // floats per staged row (odd: conflict-free)

__global__ void __launch_bounds__(64) k_bc1_features(const EncJob *__restrict__ jobs, int njobs, long long nblocks,
                                                     float *__restrict__ x) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31;
    const long long gblk = (long long)blockIdx.x * T + t;
    float *stage = reinterpret_cast<float *>(smem + 16 * T) + 16 * T + (t >> 5) * 32 * FEAT_STRIDE;
    if (gblk < nblocks) {
        const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
        Lane<float4> in{smem + t, T};
        Lane<float> wi{reinterpret_cast<float *>(smem + 16 * T) + t, T};
        gather_block(J, (int)(gblk - J.first_block), in, wi);
        const Frame f = block_frame(in, wi, mk3(J.cw[0], J.cw[1], J.cw[2]));
        float key[16];
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const float wk = wi[k];
            const f3 c = wk > 0 ? f.mu + (xyz(in[k]) - f.mu) * fminf(wk, 1.0f) : f.mu;
            in[k] = make_float4(c.x, c.y, c.z, 0.0f);
            const float p = dot(c - f.mu, f.v);
            key[k] = p == p ? p : 0.0f;  // NaN texels rank as the mean, so the ranks stay a permutation
        }
        // stable ranks along the axis (ties keep the texel order), then each texel to its rank
        float *row = stage + lane * FEAT_STRIDE;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            int rank = 0;
#pragma unroll
            for (int j = 0; j < 16; j++) rank += (key[j] < key[i]) | ((key[j] == key[i]) & (j < i));
            const float4 v = in[i];
            row[3 * rank] = v.x; row[3 * rank + 1] = v.y; row[3 * rank + 2] = v.z;
        }
    }
    __syncwarp();
    const long long base = (long long)blockIdx.x * T + (t & ~31);
    const int rows = (int)min(32LL, nblocks - base);
    for (int q = lane; q < rows * 48; q += 32) x[base * 48 + q] = stage[(q / 48) * FEAT_STRIDE + q % 48];
}

// True when the cluster fit's axis order (ascending projection on its own, arbitrarily signed
// principal vector) runs from brighter to darker along the block frame's axis v: the orderings are
// then expressed mirrored, so that the network always sees them darker-first, like its inputs.
__device__ __forceinline__ bool axis_reversed(const Lane<float4> &col, int n, uint64_t order, f3 v) {
    const float first = dot(xyz(col[(int)(order & 15)]), v);
    const float last = dot(xyz(col[(int)((order >> (4 * (n - 1))) & 15)]), v);
    return first > last;
}

// Cumulative weight fraction of the sorted colours up to ordering end e (-1: none).
__device__ __forceinline__ float cum_frac(const Lane<float4> &sat, int e, float wsum) {
    return e < 0 ? 0.0f : sat[e].w / wsum;
}

// Training targets: the orderings the full searches choose for the block, as cumulative weight
// fractions of its colours in principal-axis order - three ends of the four-cluster fit, two of
// the three-cluster fit (over the non-black colours when the block has black ones; 0, 1 when it
// has none to fit) - then log((SSE + 1) / (V + 1)) of the encoded block `J.out` against its
// texels, and 0 twice.
__global__ void __launch_bounds__(64) k_bc1_targets(const EncJob *__restrict__ jobs, int njobs, long long nblocks,
                                                    float *__restrict__ tg) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x, t = threadIdx.x;
    const long long gblk = (long long)blockIdx.x * T + t;
    if (gblk >= nblocks) return;
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    Lane<float4> in{smem + t, T};
    Lane<float4> col{smem + 16 * T + t, T};
    Lane<float4> sat{smem + 32 * T + t, T};
    Lane<float> wi{reinterpret_cast<float *>(smem + 48 * T) + t, T};
    const f3 cw = mk3(J.cw[0], J.cw[1], J.cw[2]);
    gather_block(J, blk, in, wi);
    const uint2 b = *reinterpret_cast<const uint2 *>(J.out + 8 * (size_t)blk);
    Pal3 pal;
    palette_f(b.x & 0xFFFF, b.x >> 16, pal);
    const float sse = block_mse(in, wi, cw, pal, b.y);
    const Frame f = block_frame(in, wi, cw);
    float *o = tg + gblk * 8;
    float w4[3] = {0, 0, 0}, w3[2] = {0, 1};
    bool any_black = false;
    const int cnt = reduce_colors(in, wi, col, any_black);
    if (cnt >= 2) {
        const f3 metric = cw * cw;
        uint64_t order;
        int sn = compute_sat(col, cnt, sat, &order);
        float wsum = sat[sn - 1].w;
        uint32_t bo = best_order_four(sat, sn, metric);
        w4[0] = cum_frac(sat, (int)(bo & 255) - 1, wsum);
        w4[1] = cum_frac(sat, (int)((bo >> 8) & 255) - 1, wsum);
        w4[2] = cum_frac(sat, (int)((bo >> 16) & 255) - 1, wsum);
        if (axis_reversed(col, sn, order, f.v)) { const float a = w4[0]; w4[0] = 1 - w4[2]; w4[1] = 1 - w4[1]; w4[2] = 1 - a; }
        bool run3 = true;
        if (any_black) {
            int m = 0;
            for (int i = 0; i < cnt; i++) {
                float4 q = col[i];
                if (is_black(xyz(q))) continue;
                col[m++] = q;
            }
            if (m == 0) run3 = false;
            else sn = compute_sat(col, m, sat, &order);
        }
        if (run3) {
            wsum = sat[sn - 1].w;
            bo = best_order_three(sat, sn, metric);
            w3[0] = cum_frac(sat, (int)(bo & 255) - 1, wsum);
            w3[1] = cum_frac(sat, (int)((bo >> 8) & 255) - 1, wsum);
            if (axis_reversed(col, sn, order, f.v)) { const float a = w3[0]; w3[0] = 1 - w3[1]; w3[1] = 1 - a; }
        }
    }
    o[0] = w4[0]; o[1] = w4[1]; o[2] = w4[2]; o[3] = w3[0]; o[4] = w3[1];
    o[5] = logf((sse + 1.0f) / (f.var + 1.0f));
    o[6] = 0.0f;
    o[7] = 0.0f;
}

// Ordering end of a cumulative weight fraction: the last sorted colour whose cumulative weight is
// within the fraction (-1 when none is). `sat` is a ZERO table (entry k: the first k colours).
__device__ __forceinline__ int frac_end(const Lane<float4> &sat, int n, float frac) {
    const float lim = frac * sat[n].w * (1.0f + 1e-5f) + 1e-7f;
    int e = -1;
    for (int k = 0; k < n; k++)
        if (sat[k + 1].w <= lim) e = k;
    return e;
}

__device__ __forceinline__ uint32_t pack_order(int e0, int e1, int e2) {
    return (uint32_t)(e0 + 1) | ((uint32_t)(e1 + 1) << 8) | ((uint32_t)(e2 + 1) << 16);
}

// cluster_fit_four over the orderings whose cluster ends lie within r of (e0, e1, e2), in the full
// search's order (last end, then first, then second); returns the number evaluated.
__device__ int pruned_four(const Lane<float4> &sat, int n, f3 metric, int e0, int e1, int e2, int r, f3 &start, f3 &end) {
    const float4 s = sat[n];  // a ZERO table
    const f3 sum = xyz(s);
    const float wsum = s.w;
    float best = FLT_MAX;
    uint32_t bo = 0;
    bool found = false;
    int evaluated = 0;
    for (int c = max(0, e2 - r); c <= min(n - 1, e2 + r); c++)
        for (int a = max(-1, e0 - r); a <= min(c, e0 + r); a++)
            for (int b = max(a, e1 - r); b <= min(c, e1 + r); b++) {
                f3 pa, pb;
                const uint32_t o = pack_order(a, b, c);
                const float e = four_eval<true>(sat, o, sum, wsum, metric, pa, pb);
                evaluated++;
                if (e < best) { best = e; bo = o; found = true; }
            }
    start = mk3(0, 0, 0);
    end = mk3(0, 0, 0);
    if (found) four_eval<true>(sat, bo, sum, wsum, metric, start, end);
    return evaluated;
}

__device__ int pruned_three(const Lane<float4> &sat, int n, f3 metric, int e0, int e1, int r, f3 &start, f3 &end) {
    const float4 s = sat[n];  // a ZERO table
    const f3 sum = xyz(s);
    const float wsum = s.w;
    float best = FLT_MAX;
    uint32_t bo = 0;
    bool found = false;
    int evaluated = 0;
    for (int c = max(0, e1 - r); c <= min(n - 1, e1 + r); c++)
        for (int a = max(-1, e0 - r); a <= min(c, e0 + r); a++) {
            f3 pa, pb;
            const uint32_t o = (uint32_t)(a + 1) | ((uint32_t)(c + 1) << 8);
            const float e = three_eval<true>(sat, o, sum, wsum, metric, pa, pb);
            evaluated++;
            if (e < best) { best = e; bo = o; found = true; }
        }
    start = mk3(0, 0, 0);
    end = mk3(0, 0, 0);
    if (found) three_eval<true>(sat, bo, sum, wsum, metric, start, end);
    return evaluated;
}

// Steepest descent over cluster_fit_four's orderings from (e0, e1, e2): each move evaluates the
// orderings one step away in any of the three ends (up to 26) and goes to the lowest error if it is
// strictly below the current one; at most `moves` moves. Returns the number evaluated.
__device__ int descend_four(const Lane<float4> &sat, int n, f3 metric, int e0, int e1, int e2, int moves, f3 &start,
                            f3 &end) {
    const float4 s = sat[n];  // a ZERO table
    const f3 sum = xyz(s);
    const float wsum = s.w;
    int c = min(max(e2, 0), n - 1), a = min(max(e0, -1), c), b = min(max(e1, a), c);
    f3 pa, pb;
    float best = four_eval<true>(sat, pack_order(a, b, c), sum, wsum, metric, pa, pb);
    int evaluated = 1;
    for (int m = 0; m < moves; m++) {
        float mbest = best;
        int na = a, nb = b, nc = c;
        for (int dc = -1; dc <= 1; dc++)
            for (int da = -1; da <= 1; da++)
                for (int db = -1; db <= 1; db++) {
                    const int cc = c + dc, aa = a + da, bb = b + db;
                    if ((dc | da | db) == 0 || cc < 0 || cc > n - 1 || aa < -1 || aa > bb || bb > cc) continue;
                    const float e = four_eval<true>(sat, pack_order(aa, bb, cc), sum, wsum, metric, pa, pb);
                    evaluated++;
                    if (e < mbest) { mbest = e; na = aa; nb = bb; nc = cc; }
                }
        if (!(mbest < best)) break;
        best = mbest; a = na; b = nb; c = nc;
    }
    start = mk3(0, 0, 0);
    end = mk3(0, 0, 0);
    if (best < FLT_MAX) four_eval<true>(sat, pack_order(a, b, c), sum, wsum, metric, start, end);
    return evaluated;
}

__device__ int descend_three(const Lane<float4> &sat, int n, f3 metric, int e0, int e1, int moves, f3 &start, f3 &end) {
    const float4 s = sat[n];  // a ZERO table
    const f3 sum = xyz(s);
    const float wsum = s.w;
    int c = min(max(e1, 0), n - 1), a = min(max(e0, -1), c);
    f3 pa, pb;
    float best = three_eval<true>(sat, (uint32_t)(a + 1) | ((uint32_t)(c + 1) << 8), sum, wsum, metric, pa, pb);
    int evaluated = 1;
    for (int m = 0; m < moves; m++) {
        float mbest = best;
        int na = a, nc = c;
        for (int dc = -1; dc <= 1; dc++)
            for (int da = -1; da <= 1; da++) {
                const int cc = c + dc, aa = a + da;
                if ((dc | da) == 0 || cc < 0 || cc > n - 1 || aa < -1 || aa > cc) continue;
                const float e = three_eval<true>(sat, (uint32_t)(aa + 1) | ((uint32_t)(cc + 1) << 8), sum, wsum, metric,
                                                 pa, pb);
                evaluated++;
                if (e < mbest) { mbest = e; na = aa; nc = cc; }
            }
        if (!(mbest < best)) break;
        best = mbest; a = na; c = nc;
    }
    start = mk3(0, 0, 0);
    end = mk3(0, 0, 0);
    if (best < FLT_MAX) three_eval<true>(sat, (uint32_t)(a + 1) | ((uint32_t)(c + 1) << 8), sum, wsum, metric, start, end);
    return evaluated;
}

// Least-squares refit of a four-colour block's endpoints (an addition of the learned path; the plain
// Level8 fit has none): the weighted least-squares endpoints of the block's texels for its current
// indices (index 0 -> first endpoint, 1 -> second, 2 -> 2/3 first + 1/3 second, 3 -> 1/3 + 2/3), snapped
// to 5:6:5 and re-indexed by the output stage; kept when the block's error drops, twice at most.
// Returns the block's error. Three-colour blocks are left as they are.
template <typename W>
__device__ float ls_refit(const Lane<float4> &in, const W &wi, f3 cw, float err, Block1 &o) {
    for (int it = 0; it < 2 && o.c0 > o.c1; it++) {
        float a2 = 0, b2 = 0, ab = 0;
        f3 ax = mk3(0, 0, 0), bx = mk3(0, 0, 0);
        for (int i = 0; i < 16; i++) {
            const unsigned bits = (o.idx >> (2 * i)) & 3;
            const float beta = bits == 0 ? 0.0f : (bits == 1 ? 1.0f : (bits == 2 ? 1.0f / 3.0f : 2.0f / 3.0f));
            const float alpha = 1.0f - beta, w = wi[i];
            const f3 p = xyz(in[i]);
            a2 += w * alpha * alpha; b2 += w * beta * beta; ab += w * alpha * beta;
            ax = ax + p * (w * alpha); bx = bx + p * (w * beta);
        }
        const float den = a2 * b2 - ab * ab;
        if (!(fabsf(den) > 1e-6f)) break;
        const float f = 1.0f / den;
        const f3 na = sat3(((ax * b2) - (bx * ab)) * f), nb = sat3(((bx * a2) - (ax * ab)) * f);
        Block1 t;
        const float e = output_block4(in, wi, cw, na, nb, t);
        if (!(e < err)) break;
        err = e;
        o = t;
    }
    return err;
}

// Warp-aggregated append of this thread's block to `list` (count in *n) when `take`.
__device__ __forceinline__ void append_block(bool take, long long gblk, long long *list, unsigned long long *n) {
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync(active, take);
    if (!mask) return;
    const int lane = threadIdx.x & 31, leader = __ffs(active) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(n, (unsigned long long)__popc(mask));
    base = __shfl_sync(active, base, leader);
    if (take) list[base + __popc(mask & ((1u << lane) - 1))] = gblk;
}

// stats[0] += blocks written here, stats[1] = fallback count (list length), stats[2] += orderings evaluated
__global__ void __launch_bounds__(64) k_bc1_learned(const EncJob *__restrict__ jobs, int njobs, long long nblocks,
                                                    const float *__restrict__ y, int radius, float margin,
                                                    long long *__restrict__ fallback, unsigned long long *__restrict__ stats) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x, t = threadIdx.x;
    const long long gblk = (long long)blockIdx.x * T + t;
    if (gblk >= nblocks) return;
    const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
    const int blk = (int)(gblk - J.first_block);
    // the layout of k_bc1: colours reduced over the texels in place, the ZERO SAT built over the
    // colours in place, texels gathered again for the output stage, weights derived from the texels
    Lane<float4> in{smem + t, T};
    Lane<float4> col = in;
    Lane<float4> sat = in;
    const AlphaW wi{smem + t, T, J.alpha_mode == 1, valid_texels(J, blk)};
    const f3 cw = mk3(J.cw[0], J.cw[1], J.cw[2]);
    uint8_t *const out = J.out + 8 * (size_t)blk;
    gather_block(J, blk, in, wi);
    const Frame f = block_frame(in, wi, cw);
    bool any_black = false;
    const int cnt = reduce_colors(in, wi, col, any_black);
    bool take = false;
    int evaluated = 0;
    if (cnt <= 1) {
        store_block(out, cnt == 0 ? Block1{0, 0, 0} : single_colour(col[0]));
    } else {
        const float *yp = y + gblk * 16;
        const float full_pred = (f.var + 1.0f) * expf(yp[5]) - 1.0f;
        const f3 metric = cw * cw;
        bool rev = false;
        int sn = compute_sat_inplace(col, cnt, &f.v, &rev);
        float q0 = yp[0], q1 = yp[1], q2 = yp[2];
        if (rev) { const float a = q0; q0 = 1 - q2; q1 = 1 - q1; q2 = 1 - a; }
        const int e0 = frac_end(sat, sn, q0), e1 = max(e0, frac_end(sat, sn, q1));
        const int e2 = max(max(e1, 0), frac_end(sat, sn, q2));
        f3 s0, s1, t0, t1;
        const bool descent = (radius & NTG_PROPOSAL_DESCENT) != 0;
        const int reach = radius & (NTG_PROPOSAL_DESCENT - 1);  // the flags are above the reach's bits
        evaluated += descent ? descend_four(sat, sn, metric, e0, e1, e2, reach, s0, s1)
                             : pruned_four(sat, sn, metric, e0, e1, e2, reach, s0, s1);
        Block1 o{0, 0, 0}, cf;
        float err = FLT_MAX;
        bool run3 = true;
        if (any_black) {
            // the table has replaced the colours: reduce them again, then skip the black ones
            gather_block(J, blk, in, wi);
            bool again = false;
            reduce_colors(in, wi, col, again);
            int m = 0;
            for (int i = 0; i < cnt; i++) {
                float4 q = col[i];
                if (is_black(xyz(q))) continue;
                col[m++] = q;
            }
            if (m == 0) run3 = false;
            else sn = compute_sat_inplace(col, m, &f.v, &rev);
        }
        if (run3) {
            float r0 = yp[3], r1 = yp[4];
            if (rev) { const float a = r0; r0 = 1 - r1; r1 = 1 - a; }
            const int f0 = frac_end(sat, sn, r0), f1 = max(max(f0, 0), frac_end(sat, sn, r1));
            evaluated += descent ? descend_three(sat, sn, metric, f0, f1, reach, t0, t1)
                                 : pruned_three(sat, sn, metric, f0, f1, reach, t0, t1);
        }
        gather_block(J, blk, in, wi);
        float cerr = output_block4(in, wi, cw, s0, s1, cf);
        if (run3) {
            Block1 b3;
            float e3 = output_block3(in, wi, cw, true, t0, t1, b3);
            if (e3 < cerr) { cerr = e3; cf = b3; }
        }
        if (cerr < err) { o = cf; err = cerr; }
        if (radius & NTG_PROPOSAL_REFIT) err = ls_refit(in, wi, cw, err, o);
        take = !(err <= (1.0f + margin) * full_pred);  // NaN estimates fall back too
        if (!take) store_block(out, o);
    }
    append_block(take, gblk, fallback, &stats[1]);
    // warp-aggregated statistics
    const unsigned active = __activemask();
    unsigned long long written = take ? 0 : 1, ev = (unsigned long long)evaluated;
    for (int off = 16; off > 0; off >>= 1) {
        written += __shfl_down_sync(active, written, off);
        ev += __shfl_down_sync(active, ev, off);
    }
    if ((threadIdx.x & 31) == __ffs(active) - 1) {
        atomicAdd(&stats[0], written);
        atomicAdd(&stats[2], ev);
    }
}

// Work of the Level8 fit (measurement only, outside the encoder): per block the orderings that
// cluster_fit_four and cluster_fit_three evaluate (over the non-black colours when the block has
// black ones), from the same gather and reduce_colors as k_bc1; summed into work[0] and work[1].
__global__ void __launch_bounds__(64) k_bc1_work(const EncJob *__restrict__ jobs, int njobs, long long nblocks,
                                                 unsigned long long *__restrict__ work) {
    extern __shared__ float4 smem[];
    const int T = blockDim.x, t = threadIdx.x;
    const long long gblk = (long long)blockIdx.x * T + t;
    unsigned long long n4 = 0, n3 = 0;
    if (gblk < nblocks) {
        const EncJob &J = jobs[find_job(jobs, njobs, gblk)];
        Lane<float4> in{smem + t, T};
        Lane<float> wi{reinterpret_cast<float *>(smem + 16 * T) + t, T};
        gather_block(J, (int)(gblk - J.first_block), in, wi);
        bool any_black = false;
        const int cnt = reduce_colors(in, wi, in, any_black);
        if (cnt >= 2) {
            n4 = c_tab.four_total[cnt - 1];
            int m = cnt;
            if (any_black) {
                m = 0;
                for (int i = 0; i < cnt; i++) m += !is_black(xyz(in[i]));
            }
            if (m > 0) n3 = c_tab.three_total[m - 1];
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        n4 += __shfl_down_sync(0xffffffffu, n4, off);
        n3 += __shfl_down_sync(0xffffffffu, n3, off);
    }
    if ((t & 31) == 0 && (n4 | n3)) {
        atomicAdd(&work[0], n4);
        atomicAdd(&work[1], n3);
    }
}

// Shared memory of k_bc1 and k_bc1_learned: per thread 17 float4 slots, the texels, then the
// reduced colours, then the SAT (its weights are derived from the texels).
static size_t bc1_fit_smem(int T) { return (size_t)T * 17 * sizeof(float4); }
// k_bc1_work: per thread the texels and 16 stored weights.
static size_t bc1_work_smem(int T) { return (size_t)T * (16 * sizeof(float4) + 16 * sizeof(float)); }

// Blocks the one-thread-per-block fit keeps in flight on a full GB300 (152 SMs x 12 CTAs of 64).
constexpr long long kBc1InFlight = 152LL * 12 * 64;

template <int LEVEL, int K>
static void launch_bc1_split(const EncJob *d_jobs, int njobs, long long nblocks, cudaStream_t stream) {
    constexpr int G = 64 / K;
    k_bc1_split<LEVEL, K><<<(unsigned)((nblocks + G - 1) / G), 64, (size_t)G * 17 * sizeof(float4), stream>>>(
        d_jobs, njobs, nblocks);
}

int launch_bc1(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t stream) {
    if (nblocks == 0) return 0;
    if (quality != 0 && nblocks * 4 <= 2 * kBc1InFlight) {
        // too few blocks to keep the SMs busy one thread each (a single 512x512 chain has 21,847):
        // 8 or 4 lanes per block, for up to two waves of threads
        const bool eight = nblocks * 8 <= 2 * kBc1InFlight;
        if (quality == 2) eight ? launch_bc1_split<8, 8>(d_jobs, njobs, nblocks, stream)
                                : launch_bc1_split<8, 4>(d_jobs, njobs, nblocks, stream);
        else eight ? launch_bc1_split<7, 8>(d_jobs, njobs, nblocks, stream)
                   : launch_bc1_split<7, 4>(d_jobs, njobs, nblocks, stream);
        return launch_status();
    }
    const int T = threads == 32 ? 32 : 64;  // blocks per CTA (one thread per 4x4 block)
    const size_t sm = bc1_fit_smem(T);
    const unsigned grid = (unsigned)((nblocks + T - 1) / T);
    static std::atomic<unsigned long long> configured{0};
    if (first_use_on_device(configured)) {  // the per-thread arrays exceed the 48 KB default
        cudaFuncSetAttribute(k_bc1<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        cudaFuncSetAttribute(k_bc1<7>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        cudaFuncSetAttribute(k_bc1<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    }
    if (quality == 0) k_bc1<0><<<grid, T, sm, stream>>>(d_jobs, njobs, nblocks, nullptr, nullptr);
    else if (quality == 2) k_bc1<8><<<grid, T, sm, stream>>>(d_jobs, njobs, nblocks, nullptr, nullptr);
    else k_bc1<7><<<grid, T, sm, stream>>>(d_jobs, njobs, nblocks, nullptr, nullptr);
    return launch_status();
}

static size_t bc1_smem(int T) { return (size_t)T * (48 * sizeof(float4) + 16 * sizeof(float)); }

template <typename K>
static void allow_smem(K kernel, size_t bytes, std::atomic<unsigned long long> &configured) {
    if (first_use_on_device(configured)) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int launch_bc1_features(const EncJob *d_jobs, int njobs, long long nblocks, float *x, cudaStream_t s) {
    if (nblocks == 0) return 0;
    const int T = 64;
    k_bc1_features<<<(unsigned)((nblocks + T - 1) / T), T,
                     (size_t)T * (16 * sizeof(float4) + 16 * sizeof(float) + FEAT_STRIDE * sizeof(float)), s>>>(
        d_jobs, njobs, nblocks, x);
    return launch_status();
}

int launch_bc1_targets(const EncJob *d_jobs, int njobs, long long nblocks, float *tg, cudaStream_t s) {
    if (nblocks == 0) return 0;
    const int T = 64;  // texels, colours, summed-area table and weights per thread, as k_bc1
    static std::atomic<unsigned long long> configured{0};
    allow_smem(k_bc1_targets, bc1_smem(T), configured);
    k_bc1_targets<<<(unsigned)((nblocks + T - 1) / T), T, bc1_smem(T), s>>>(d_jobs, njobs, nblocks, tg);
    return launch_status();
}

int launch_bc1_learned(const EncJob *d_jobs, int njobs, long long nblocks, const float *y, int radius, float margin,
                       long long *fallback, unsigned long long *stats, cudaStream_t s) {
    if (nblocks == 0) return 0;
    const int T = 64;
    static std::atomic<unsigned long long> configured{0};
    allow_smem(k_bc1_learned, bc1_fit_smem(T), configured);
    k_bc1_learned<<<(unsigned)((nblocks + T - 1) / T), T, bc1_fit_smem(T), s>>>(d_jobs, njobs, nblocks, y, radius, margin,
                                                                            fallback, stats);
    return launch_status();
}

int launch_bc1_work(const EncJob *d_jobs, int njobs, long long nblocks, unsigned long long *work, cudaStream_t s) {
    if (nblocks == 0) return 0;
    const int T = 64;
    k_bc1_work<<<(unsigned)((nblocks + T - 1) / T), T, bc1_work_smem(T), s>>>(d_jobs, njobs, nblocks, work);
    return launch_status();
}

// The full Level8 fit over a list of blocks of the jobs (the learned path's fallbacks); the list's
// length stays on the device, so the sequence needs no host round trip.
int launch_bc1_list(const EncJob *d_jobs, int njobs, const long long *list, const unsigned long long *d_count,
                    long long max_count, cudaStream_t s) {
    if (max_count == 0) return 0;
    const int T = 64;
    static std::atomic<unsigned long long> configured{0};
    allow_smem(k_bc1<7>, bc1_fit_smem(T), configured);
    k_bc1<7><<<(unsigned)((max_count + T - 1) / T), T, bc1_fit_smem(T), s>>>(d_jobs, njobs, max_count, list, d_count);
    return launch_status();
}

NTG_DEFINE_TABLE_UPLOAD(upload_tables_bc1)

}  // namespace ntg
