/* CPU restatement of the NVTT 2.1.2 texture hot path (mip filtering, BC1/BC3/BC5 encoding).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA kernels are checked against and the timed CPU
 * baseline ("port") of the benchmark. The product never calls it.
 *
 * Each function names the reference file:line it follows (paths inside the reference project).
 * Arithmetic follows the reference's scalar paths operation by operation; compile with
 * -ffp-contract=off so that no product and sum fuse. Min/max helpers keep the reference's own
 * comparison forms because they treat NaN differently:
 *   ic_max/ic_min  : icbc::max/min and nv::max/min   (b < a ? a : b) / (a < b ? a : b)
 *   sq_max/sq_min  : std::max/std::min as squish uses them (a < b ? b : a) / (b < a ? b : a)
 */
#include "ntg_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int ora_version(void) { return 20102; }

/* ------------------------------------------------------------------------------------------ */
/* small helpers                                                                                */

typedef struct { float x, y, z; } v3;

static inline float ic_max(float a, float b) { return (b < a) ? a : b; }
static inline float ic_min(float a, float b) { return (a < b) ? a : b; }
static inline float ic_clamp(float x, float a, float b) { return ic_min(ic_max(x, a), b); }
static inline float ic_sat(float x) { return ic_clamp(x, 0.0f, 1.0f); }
static inline float sq_max(float a, float b) { return (a < b) ? b : a; }
static inline float sq_min(float a, float b) { return (b < a) ? b : a; }

static inline v3 mk3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(v3 a, v3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 scl3(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 sat3(v3 a) { return mk3(ic_sat(a.x), ic_sat(a.y), ic_sat(a.z)); }

/* Expand 5/6-bit endpoint channels to 8 bits (BlockDXT1::evaluatePalette,
 * src/nvimage/BlockDXT.cpp:46-57). */
static inline int ex5(int v) { return (v << 3) | (v >> 2); }
static inline int ex6(int v) { return (v << 2) | (v >> 4); }

static void put16(uint8_t *p, unsigned v) { p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); }
static void put32(uint8_t *p, uint32_t v) { put16(p, v & 0xFFFF); put16(p + 2, v >> 16); }
static unsigned get16(const uint8_t *p) { return (unsigned)p[0] | ((unsigned)p[1] << 8); }
static uint32_t get32(const uint8_t *p) { return get16(p) | ((uint32_t)get16(p + 2) << 16); }

/* ------------------------------------------------------------------------------------------ */
/* one-time tables                                                                              */

typedef struct { uint8_t a, b, c, pad; } order4_t; /* cumulative cluster ends */
typedef struct { uint8_t a, b, pad0, pad1; } order3_t;

static order4_t g_four[968];
static int g_four_total[16];
static order3_t g_three[152];
static int g_three_total[16];
static float g_mid5[32], g_mid6[64];
static uint8_t g_icbc_match5[256][2], g_icbc_match6[256][2];
static uint8_t g_opt_match5[256][2], g_opt_match6[256][2];
static uint8_t g_opt_alpha5[256][2], g_opt_alpha6[256][2];
static pthread_once_t g_once = PTHREAD_ONCE_INIT;

/* Cluster orderings of icbc init_cluster_tables (src/nvtt/icbc.h:1906-1975). For every point
 * count t, the orderings new at t are exactly the cumulative triples (A <= B <= C == t), taken in
 * the order A then B ascending -- the order in which the reference's dedup loop first meets them. */
static void init_orderings(void) {
    int n4 = 0, n3 = 0;
    for (int t = 1; t <= 16; t++) {
        for (int a = 0; a <= t; a++)
            for (int b = a; b <= t; b++) {
                g_four[n4].a = (uint8_t)a; g_four[n4].b = (uint8_t)b; g_four[n4].c = (uint8_t)t; n4++;
            }
        g_four_total[t - 1] = n4;
        for (int a = 0; a <= t; a++) { g_three[n3].a = (uint8_t)a; g_three[n3].b = (uint8_t)t; n3++; }
        g_three_total[t - 1] = n3;
    }
}

/* 565 rounding midpoints (src/nvtt/icbc.h:1516-1525): the mean of two adjacent expanded values
 * over 255, as six-decimal literals; the last entry is FLT_MAX. */
static void init_midpoints(void) {
    char buf[64];
    for (int i = 0; i < 31; i++) {
        snprintf(buf, sizeof buf, "%.6f", (ex5(i) + ex5(i + 1)) / 510.0);
        g_mid5[i] = strtof(buf, NULL);
    }
    g_mid5[31] = FLT_MAX;
    for (int i = 0; i < 63; i++) {
        snprintf(buf, sizeof buf, "%.6f", (ex6(i) + ex6(i + 1)) / 510.0);
        g_mid6[i] = strtof(buf, NULL);
    }
    g_mid6[63] = FLT_MAX;
}

/* icbc single-colour tables for the D3D10 decoder: the worse of the AMD and NVIDIA
 * interpolation errors (src/nvtt/icbc.h:3166-3262). */
static void init_icbc_single(void) {
    for (int i = 0; i < 256; i++) {
        int best = 256 * 100;
        for (int mn = 0; mn < 32; mn++)
            for (int mx = 0; mx < 32; mx++) {
                int lo = ex5(mn), hi = ex5(mx);
                int amd = abs(((43 * hi + 21 * lo + 32) >> 6) - i);
                int nv = abs(((2 * mx + mn) * 22) / 8 - i);
                int err = amd > nv ? amd : nv;
                if (err < best) { best = err; g_icbc_match5[i][0] = (uint8_t)mx; g_icbc_match5[i][1] = (uint8_t)mn; }
            }
        best = 256 * 100;
        for (int mn = 0; mn < 64; mn++)
            for (int mx = 0; mx < 64; mx++) {
                int lo = ex6(mn), hi = ex6(mx);
                int amd = abs(((43 * hi + 21 * lo + 32) >> 6) - i);
                int nv = abs((256 * lo + (hi - lo) / 4 + 128 + (hi - lo) * 80) / 256 - i);
                int err = amd > nv ? amd : nv;
                if (err < best) { best = err; g_icbc_match6[i][0] = (uint8_t)mx; g_icbc_match6[i][1] = (uint8_t)mn; }
            }
    }
}

/* OMatch5/OMatch6 and OMatchAlpha5/OMatchAlpha6 of OptimalCompress
 * (src/nvtt/SingleColorLookup.cpp:32-89): interpolation error x100 (the one-third point, or the
 * midpoint for the three-colour tables) plus 3 x endpoint distance. */
static void init_opt_single(void) {
    for (int pass = 0; pass < 4; pass++) {
        const int size = (pass & 1) == 0 ? 32 : 64;
        const int alpha = pass >= 2;
        uint8_t (*tab)[2] = pass == 0 ? g_opt_match5 : pass == 1 ? g_opt_match6 : pass == 2 ? g_opt_alpha5 : g_opt_alpha6;
        for (int i = 0; i < 256; i++) {
            int best = 256 * 100;
            for (int mn = 0; mn < size; mn++)
                for (int mx = 0; mx < size; mx++) {
                    int lo = (pass & 1) == 0 ? ex5(mn) : ex6(mn);
                    int hi = (pass & 1) == 0 ? ex5(mx) : ex6(mx);
                    int err = (alpha ? abs((hi + lo) / 2 - i) : abs((hi * 2 + lo) / 3 - i)) * 100 + abs(mx - mn) * 3;
                    if (err < best) { tab[i][0] = (uint8_t)mx; tab[i][1] = (uint8_t)mn; best = err; }
                }
        }
    }
}

static float g_pow_5_11[512], g_pow_11_5[512];

/* Exponent tables of the gamma-2.2 helpers (src/nvmath/Gamma.cpp:34-297): 2^((k-127)*p) for the
 * biased exponents of positive normal numbers, 0 for zero/subnormal and every negative input,
 * +inf for inf/NaN. */
static void init_gamma_tables(void) {
    for (int k = 0; k < 512; k++) {
        float a = 0.0f, b = 0.0f;
        if (k == 255) { a = INFINITY; b = INFINITY; }
        else if (k >= 1 && k <= 254) {
            a = (float)pow(2.0, (k - 127) * (5.0 / 11.0));
            b = (float)pow(2.0, (k - 127) * (11.0 / 5.0));
        }
        g_pow_5_11[k] = a;
        g_pow_11_5[k] = b;
    }
}

static void init_all(void) {
    init_orderings();
    init_midpoints();
    init_icbc_single();
    init_opt_single();
    init_gamma_tables();
}
static void ensure_init(void) { pthread_once(&g_once, init_all); }

/* ------------------------------------------------------------------------------------------ */
/* BC1 palettes and block layout                                                                */

typedef struct { int r, g, b; } rgb8;

/* D3D10 palette of a BC1 block (icbc evaluate_palette_d3d10, src/nvtt/icbc.h:2558-2585). */
static void palette_d3d10(unsigned c0, unsigned c1, rgb8 pal[4]) {
    pal[0].r = ex5((c0 >> 11) & 31); pal[0].g = ex6((c0 >> 5) & 63); pal[0].b = ex5(c0 & 31);
    pal[1].r = ex5((c1 >> 11) & 31); pal[1].g = ex6((c1 >> 5) & 63); pal[1].b = ex5(c1 & 31);
    if (c0 > c1) {
        pal[2].r = (2 * pal[0].r + pal[1].r) / 3; pal[2].g = (2 * pal[0].g + pal[1].g) / 3; pal[2].b = (2 * pal[0].b + pal[1].b) / 3;
        pal[3].r = (2 * pal[1].r + pal[0].r) / 3; pal[3].g = (2 * pal[1].g + pal[0].g) / 3; pal[3].b = (2 * pal[1].b + pal[0].b) / 3;
    } else {
        pal[2].r = (pal[0].r + pal[1].r) / 2; pal[2].g = (pal[0].g + pal[1].g) / 2; pal[2].b = (pal[0].b + pal[1].b) / 2;
        pal[3].r = 0; pal[3].g = 0; pal[3].b = 0;
    }
}

static void palette_f(unsigned c0, unsigned c1, v3 pf[4]) {
    rgb8 p[4];
    palette_d3d10(c0, c1, p);
    for (int i = 0; i < 4; i++) pf[i] = mk3(p[i].r / 255.0f, p[i].g / 255.0f, p[i].b / 255.0f);
}

/* ------------------------------------------------------------------------------------------ */
/* icbc BC1 encoder (src/nvtt/icbc.h, scalar build)                                             */

typedef struct { float r[16], g[16], b[16], w[16]; } sat_t;

/* vector3_to_color16 (src/nvtt/icbc.h:1580-1595). */
static unsigned to565(v3 v) {
    unsigned r = (unsigned)ic_clamp(v.x * 31.0f, 0.0f, 31.0f);
    unsigned g = (unsigned)ic_clamp(v.y * 63.0f, 0.0f, 63.0f);
    unsigned b = (unsigned)ic_clamp(v.z * 31.0f, 0.0f, 31.0f);
    r += (v.x > g_mid5[r]);
    g += (v.y > g_mid6[g]);
    b += (v.z > g_mid5[b]);
    return (r << 11) | (g << 5) | b;
}

/* vround5/vround6 of the scalar path (src/nvtt/icbc.h:1544-1578). */
static inline float round5(float x) { return (float)(int)(x * 31.0f + 0.5f) * (1.0f / 31.0f); }
static inline float round6(float x) { return (float)(int)(x * 63.0f + 0.5f) * (1.0f / 63.0f); }
static inline v3 round_ept(v3 v) { return mk3(round5(ic_sat(v.x)), round6(ic_sat(v.y)), round5(ic_sat(v.z))); }

static inline int is_black(v3 c) { return c.x < 1.0f / 8 && c.y < 1.0f / 8 && c.z < 1.0f / 8; }

/* reduce_colors (src/nvtt/icbc.h:1638-1683). */
static int reduce_colors(const float *in, const float *wi, float thr, v3 *col, float *w, int *any_black) {
    int n = 0;
    *any_black = 0;
    for (int i = 0; i < 16; i++) {
        v3 c = mk3(in[4 * i], in[4 * i + 1], in[4 * i + 2]);
        float wt = wi[i];
        if (wt > 0) {
            int j;
            for (j = 0; j < n; j++) {
                if (fabsf(col[j].x - c.x) < thr && fabsf(col[j].y - c.y) < thr && fabsf(col[j].z - c.z) < thr) {
                    float den = w[j] + wt;
                    v3 s = add3(scl3(col[j], w[j]), scl3(c, wt));
                    col[j] = mk3(s.x / den, s.y / den, s.z / den);
                    w[j] += wt;
                    break;
                }
            }
            if (j == n) { col[n] = c; w[n] = wt; n++; }
            if (is_black(c)) *any_black = 1;
        }
    }
    return n;
}

static int skip_blacks(const v3 *col, const float *w, int n, v3 *oc, float *ow) {
    int m = 0;
    for (int i = 0; i < n; i++) {
        if (is_black(col[i])) continue;
        oc[m] = col[i]; ow[m] = w[i]; m++;
    }
    return m;
}

/* computeCovariance + firstEigenVector_PowerMethod (src/nvtt/icbc.h:1700-1799). */
static v3 icbc_principal(int n, const v3 *p, const float *w) {
    v3 c = mk3(0, 0, 0);
    float total = 0.0f;
    for (int i = 0; i < n; i++) { total += w[i]; c = add3(c, scl3(p[i], w[i])); }
    c = scl3(c, 1.0f / total);
    float m[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; i++) {
        v3 a = sub3(p[i], c);
        v3 b = scl3(a, w[i]);
        m[0] += a.x * b.x; m[1] += a.x * b.y; m[2] += a.x * b.z;
        m[3] += a.y * b.y; m[4] += a.y * b.z; m[5] += a.z * b.z;
    }
    if (m[0] == 0 && m[3] == 0 && m[5] == 0) return mk3(0, 0, 0);
    v3 r0 = mk3(m[0], m[1], m[2]), r1 = mk3(m[1], m[3], m[4]), r2 = mk3(m[2], m[4], m[5]);
    float l0 = dot3(r0, r0), l1 = dot3(r1, r1), l2 = dot3(r2, r2);
    v3 v = (l0 > l1 && l0 > l2) ? r0 : (l1 > l2 ? r1 : r2);
    for (int it = 0; it < 8; it++) {
        float x = v.x * m[0] + v.y * m[1] + v.z * m[2];
        float y = v.x * m[1] + v.y * m[3] + v.z * m[4];
        float z = v.x * m[2] + v.y * m[4] + v.z * m[5];
        float norm = ic_max(ic_max(x, y), z);
        v = scl3(mk3(x, y, z), 1.0f / norm);
    }
    return v;
}

/* compute_sat (src/nvtt/icbc.h:1812-1882): project, stable insertion sort, prefix sums. */
static int compute_sat(const v3 *col, const float *w, int n, sat_t *s) {
    v3 axis = icbc_principal(n, col, w);
    int order[16];
    float dps[16];
    for (int i = 0; i < n; i++) { order[i] = i; dps[i] = dot3(col[i], axis); }
    for (int i = 0; i < n; i++)
        for (int j = i; j > 0 && dps[j] < dps[j - 1]; --j) {
            float t = dps[j]; dps[j] = dps[j - 1]; dps[j - 1] = t;
            int o = order[j]; order[j] = order[j - 1]; order[j - 1] = o;
        }
    float wt = w[order[0]];
    s->r[0] = col[order[0]].x * wt; s->g[0] = col[order[0]].y * wt; s->b[0] = col[order[0]].z * wt; s->w[0] = wt;
    for (int i = 1; i < n; i++) {
        wt = w[order[i]];
        s->r[i] = s->r[i - 1] + col[order[i]].x * wt;
        s->g[i] = s->g[i - 1] + col[order[i]].y * wt;
        s->b[i] = s->b[i - 1] + col[order[i]].z * wt;
        s->w[i] = s->w[i - 1] + wt;
    }
    for (int i = n; i < 16; i++) s->r[i] = s->g[i] = s->b[i] = s->w[i] = FLT_MAX;
    return n;
}

static inline v3 sat_at(const sat_t *s, int k) { return mk3(s->r[k], s->g[k], s->b[k]); }

/* Shared tail of cluster_fit_three/four (src/nvtt/icbc.h:2200-2240, 2501-2540): solve, snap to
 * the 565 grid, weighted residual. */
static inline float cf_eval(v3 ax, v3 sum, float a2, float b2, float ab, v3 metric, v3 *pa, v3 *pb) {
    float factor = 1.0f / (a2 * b2 - ab * ab);
    v3 bx = sub3(sum, ax);
    v3 a = scl3(sub3(scl3(ax, b2), scl3(bx, ab)), factor);
    v3 b = scl3(sub3(scl3(bx, a2), scl3(ax, ab)), factor);
    a = round_ept(a);
    b = round_ept(b);
    v3 e2 = scl3(sub3(mul3(a, sub3(scl3(b, ab), ax)), mul3(b, bx)), 2.0f);
    v3 e1 = add3(scl3(mul3(a, a), a2), add3(scl3(mul3(b, b), b2), e2));
    *pa = a; *pb = b;
    return dot3(e1, metric);
}

/* cluster_fit_four (src/nvtt/icbc.h:2250-2549), scalar order: first strict minimum wins. */
static void cluster_fit_four(const sat_t *s, int n, v3 metric, v3 *start, v3 *end) {
    v3 sum = sat_at(s, n - 1);
    float wsum = s->w[n - 1];
    float best = FLT_MAX;
    v3 bs = mk3(0, 0, 0), be = mk3(0, 0, 0);
    for (int i = 0; i < g_four_total[n - 1]; i++) {
        int c0 = g_four[i].a - 1, c1 = g_four[i].b - 1, c2 = g_four[i].c - 1;
        v3 x0 = mk3(0, 0, 0), x1 = mk3(0, 0, 0), x2 = mk3(0, 0, 0);
        float w0 = 0, w1 = 0, w2 = 0;
        if (c0 >= 0) { x0 = sat_at(s, c0); w0 = s->w[c0]; }
        if (c1 >= 0) { x1 = sat_at(s, c1); w1 = s->w[c1]; }
        if (c2 >= 0) { x2 = sat_at(s, c2); w2 = s->w[c2]; }
        float w3 = wsum - w2;
        x2 = sub3(x2, x1); x1 = sub3(x1, x0);
        w2 = w2 - w1; w1 = w1 - w0;
        float a2 = w2 * (1.0f / 9.0f) + (w1 * (4.0f / 9.0f) + w0);
        float b2 = w1 * (1.0f / 9.0f) + (w2 * (4.0f / 9.0f) + w3);
        float ab = (w1 + w2) * (2.0f / 9.0f);
        v3 ax = add3(scl3(x2, 1.0f / 3.0f), add3(scl3(x1, 2.0f / 3.0f), x0));
        v3 a, b;
        float e = cf_eval(ax, sum, a2, b2, ab, metric, &a, &b);
        if (e < best) { best = e; bs = a; be = b; }
    }
    *start = bs; *end = be;
}

/* cluster_fit_three (src/nvtt/icbc.h:2016-2247). */
static void cluster_fit_three(const sat_t *s, int n, v3 metric, v3 *start, v3 *end) {
    v3 sum = sat_at(s, n - 1);
    float wsum = s->w[n - 1];
    float best = FLT_MAX;
    v3 bs = mk3(0, 0, 0), be = mk3(0, 0, 0);
    for (int i = 0; i < g_three_total[n - 1]; i++) {
        int c0 = g_three[i].a - 1, c1 = g_three[i].b - 1;
        v3 x0 = mk3(0, 0, 0), x1 = mk3(0, 0, 0);
        float w0 = 0, w1 = 0;
        if (c0 >= 0) { x0 = sat_at(s, c0); w0 = s->w[c0]; }
        if (c1 >= 0) { x1 = sat_at(s, c1); w1 = s->w[c1]; }
        float w2 = wsum - w1;
        x1 = sub3(x1, x0);
        w1 = w1 - w0;
        float ab = w1 * 0.25f;
        float a2 = w0 + ab;
        float b2 = w2 + ab;
        v3 ax = add3(x0, scl3(x1, 0.5f));
        v3 a, b;
        float e = cf_eval(ax, sum, a2, b2, ab, metric, &a, &b);
        if (e < best) { best = e; bs = a; be = b; }
    }
    *start = bs; *end = be;
}

/* compute_indices4 (src/nvtt/icbc.h:2803-2835). */
static uint32_t indices4(const float *in, v3 cw, const v3 pal[4]) {
    v3 p0 = mul3(pal[0], cw), p1 = mul3(pal[1], cw), p2 = mul3(pal[2], cw), p3 = mul3(pal[3], cw);
    uint32_t idx = 0;
    for (int i = 0; i < 16; i++) {
        v3 c = mul3(mk3(in[4 * i], in[4 * i + 1], in[4 * i + 2]), cw);
        v3 t;
        t = sub3(c, p0); float d0 = dot3(t, t);
        t = sub3(c, p1); float d1 = dot3(t, t);
        t = sub3(c, p2); float d2 = dot3(t, t);
        t = sub3(c, p3); float d3 = dot3(t, t);
        unsigned hi = ((d1 > d2) & (d0 > d2)) | ((d0 > d3) & (d1 > d3));
        unsigned lo = (d0 > d3) & (d2 > d3);
        idx |= (uint32_t)((hi << 1) | lo) << (2 * i);
    }
    return idx;
}

/* compute_indices3 (src/nvtt/icbc.h:2837-2882). */
static uint32_t indices3(const float *in, v3 cw, int allow_black, const v3 pal[4]) {
    v3 p0 = mul3(pal[0], cw), p1 = mul3(pal[1], cw), p2 = mul3(pal[2], cw);
    uint32_t idx = 0;
    for (int i = 0; i < 16; i++) {
        v3 c = mul3(mk3(in[4 * i], in[4 * i + 1], in[4 * i + 2]), cw);
        v3 t;
        unsigned hi, lo;
        if (allow_black) {
            t = sub3(p0, c); float d0 = dot3(t, t);
            t = sub3(p1, c); float d1 = dot3(t, t);
            t = sub3(p2, c); float d2 = dot3(t, t);
            float d3 = dot3(c, c);
            unsigned i1 = d1 < d2, i2 = (d2 <= d0) & (d2 <= d1), i3 = (d3 <= d0) & (d3 <= d1) & (d3 <= d2);
            hi = i2 | i3; lo = i1 | i3;
        } else {
            t = sub3(c, p0); float d0 = dot3(t, t);
            t = sub3(c, p1); float d1 = dot3(t, t);
            t = sub3(c, p2); float d2 = dot3(t, t);
            unsigned i1 = d1 < d2, i2 = (d2 <= d0) & (d2 <= d1);
            hi = i2; lo = i1;
        }
        idx |= (uint32_t)((hi << 1) | lo) << (2 * i);
    }
    return idx;
}

/* compute_indices, the live branch (src/nvtt/icbc.h:2885-2941). */
static uint32_t indices_any(const float *in, v3 cw, const v3 pal[4]) {
    v3 p0 = mul3(pal[0], cw), p1 = mul3(pal[1], cw), p2 = mul3(pal[2], cw), p3 = mul3(pal[3], cw);
    uint32_t idx = 0;
    for (int i = 0; i < 16; i++) {
        v3 c = mul3(mk3(in[4 * i], in[4 * i + 1], in[4 * i + 2]), cw);
        v3 t;
        t = sub3(c, p0); float d0 = dot3(t, t);
        t = sub3(c, p1); float d1 = dot3(t, t);
        t = sub3(c, p2); float d2 = dot3(t, t);
        t = sub3(c, p3); float d3 = dot3(t, t);
        unsigned i1 = (d1 <= d0) & (d1 < d2) & (d1 < d3);
        unsigned i2 = (d2 <= d0) & (d2 <= d1) & (d2 < d3);
        unsigned i3 = (d3 <= d0) & (d3 <= d1) & (d3 <= d2);
        idx |= (uint32_t)(((i2 | i3) << 1) | (i1 | i3)) << (2 * i);
    }
    return idx;
}

/* evaluate_mse over the 16 input texels (src/nvtt/icbc.h:2733-2756). */
static float block_mse(const float *in, const float *wi, v3 cw, const v3 pal[4], uint32_t idx) {
    float err = 0.0f;
    for (int i = 0; i < 16; i++) {
        int k = (idx >> (2 * i)) & 3;
        v3 d = scl3(mul3(sub3(pal[k], mk3(in[4 * i], in[4 * i + 1], in[4 * i + 2])), cw), 255.0f);
        err += wi[i] * dot3(d, d);
    }
    return err;
}

typedef struct { unsigned c0, c1; uint32_t idx; } bc1_t;

static float output_block4(const float *in, const float *wi, v3 cw, v3 v0, v3 v1, bc1_t *o) {
    unsigned c0 = to565(v0), c1 = to565(v1);
    if (c0 < c1) { unsigned t = c0; c0 = c1; c1 = t; }
    v3 pal[4];
    palette_f(c0, c1, pal);
    o->c0 = c0; o->c1 = c1;
    o->idx = indices4(in, cw, pal);
    return block_mse(in, wi, cw, pal, o->idx);
}

static float output_block3(const float *in, const float *wi, v3 cw, int allow_black, v3 v0, v3 v1, bc1_t *o) {
    unsigned c0 = to565(v0), c1 = to565(v1);
    if (c0 > c1) { unsigned t = c0; c0 = c1; c1 = t; }
    v3 pal[4];
    palette_f(c0, c1, pal);
    o->c0 = c0; o->c1 = c1;
    o->idx = indices3(in, cw, allow_black, pal);
    return block_mse(in, wi, cw, pal, o->idx);
}

/* optimize_end_points4 on the 16 input texels (src/nvtt/icbc.h:2984-3016). */
static int lsq_endpoints4(uint32_t idx, const float *in, v3 *a, v3 *b) {
    float a2 = 0, b2 = 0, ab = 0;
    v3 ax = mk3(0, 0, 0), bx = mk3(0, 0, 0);
    for (int i = 0; i < 16; i++) {
        unsigned bits = idx >> (2 * i);
        float beta = (float)(bits & 1);
        if (bits & 2) beta = (1 + beta) / 3.0f;
        float alpha = 1.0f - beta;
        v3 c = mk3(in[4 * i], in[4 * i + 1], in[4 * i + 2]);
        a2 += alpha * alpha; b2 += beta * beta; ab += alpha * beta;
        ax = add3(ax, scl3(c, alpha)); bx = add3(bx, scl3(c, beta));
    }
    float den = a2 * b2 - ab * ab;
    if (fabsf(den - 0.0f) < 0.0001f) return 0;
    float f = 1.0f / den;
    *a = sat3(scl3(sub3(scl3(ax, b2), scl3(bx, ab)), f));
    *b = sat3(scl3(sub3(scl3(bx, a2), scl3(ax, ab)), f));
    return 1;
}

static float mse_of(const float *in, const float *wi, v3 cw, const bc1_t *o) {
    v3 pal[4];
    palette_f(o->c0, o->c1, pal);
    return block_mse(in, wi, cw, pal, o->idx);
}

/* refine_endpoints (src/nvtt/icbc.h:3329-3406), including its use of the current output's
 * palette for index selection. */
static float refine_endpoints(const float *in, const float *wi, v3 cw, int three_color_mode, float err, bc1_t *o) {
    static const int8_t deltas[16][3] = {
        {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1},
        {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {-1, -1, 0}, {-1, 0, -1}, {0, -1, -1},
        {-1, 1, 0}, {1, -1, 0}, {0, -1, 1}, {0, 1, -1}};
    float best = err;
    int last = 0;
    for (int i = 0; i < 256; i++) {
        bc1_t r = *o;
        const int8_t *d = deltas[i % 16];
        unsigned *c = ((i / 16) & 1) ? &r.c0 : &r.c1;
        unsigned cr = ((*c >> 11) + d[0]) & 31, cg = (((*c >> 5) & 63) + d[1]) & 63, cb = ((*c & 31) + d[2]) & 31;
        *c = (cr << 11) | (cg << 5) | cb;
        if (!three_color_mode) {
            if (r.c0 == r.c1) r.c1 = (r.c1 & ~(63u << 5)) | ((((r.c1 >> 5) & 63) + 1) & 63) << 5;
            if (r.c0 < r.c1) { unsigned t = r.c0; r.c0 = r.c1; r.c1 = t; }
        }
        v3 pal[4];
        palette_f(o->c0, o->c1, pal);
        r.idx = indices_any(in, cw, pal);
        float e = mse_of(in, wi, cw, &r);
        if (e < best) { best = e; *o = r; last = i; }
        if (i - last > 32) break;
    }
    return best;
}

static void single_color_icbc(v3 c, bc1_t *o) {
    int r = (int)(uint8_t)(ic_sat(c.x) * 255 + 0.5f);
    int g = (int)(uint8_t)(ic_sat(c.y) * 255 + 0.5f);
    int b = (int)(uint8_t)(ic_sat(c.z) * 255 + 0.5f);
    o->c0 = ((unsigned)g_icbc_match5[r][0] << 11) | ((unsigned)g_icbc_match6[g][0] << 5) | g_icbc_match5[b][0];
    o->c1 = ((unsigned)g_icbc_match5[r][1] << 11) | ((unsigned)g_icbc_match6[g][1] << 5) | g_icbc_match5[b][1];
    o->idx = 0xaaaaaaaau;
    if (o->c0 < o->c1) { unsigned t = o->c0; o->c0 = o->c1; o->c1 = t; o->idx ^= 0x55555555u; }
}

/* compress_dxt1 (src/nvtt/icbc.h:3485-3559) with setup_options (:3418-3482). icbc_level is the
 * icbc::Quality value: 0 = Level1 (box + least squares), 7 = Level8, 8 = Level9. */
float ora_bc1_block(int level, const float *in, const float *wi, const float *cw3, int three_color_mode,
                    int three_color_black, uint8_t *out8) {
    ensure_init();
    v3 cw = mk3(cw3[0], cw3[1], cw3[2]);
    int box_fit = 0, lsq = 0, cfit = 0, cfit3 = 0, cfit3_black_only = 0, refine = 0;
    float thr = 0.0f;
    switch (level) {
        case 0: box_fit = 1; lsq = 1; thr = 1.0f / 256; break;
        case 1: box_fit = 1; lsq = 1; cfit = 1; cfit3_black_only = three_color_mode && three_color_black; thr = 1.0f / 24; break;
        case 2: box_fit = 1; cfit = 1; cfit3_black_only = three_color_mode && three_color_black; thr = 1.0f / 32; break;
        case 3: cfit = 1; cfit3_black_only = three_color_mode && three_color_black; thr = 1.0f / 48; break;
        case 4: cfit = 1; cfit3_black_only = three_color_mode && three_color_black; thr = 1.0f / 64; break;
        case 5: cfit = 1; cfit3_black_only = three_color_mode && three_color_black; thr = 1.0f / 96; break;
        case 6: cfit = 1; cfit3_black_only = three_color_mode && three_color_black; thr = 1.0f / 128; break;
        case 7: cfit = 1; cfit3 = three_color_mode; thr = 1.0f / 256; break;
        default: cfit = 1; cfit3 = three_color_mode; thr = 1.0f / 256; refine = 1; break;
    }
    v3 col[16];
    float w[16];
    int any_black = 0, count;
    if (cfit) count = reduce_colors(in, wi, thr, col, w, &any_black);
    else { for (int i = 0; i < 16; i++) col[i] = mk3(in[4 * i], in[4 * i + 1], in[4 * i + 2]); count = 16; }

    bc1_t o = {0, 0, 0};
    float err;
    if (count == 0) {
        put16(out8, 0); put16(out8 + 2, 0); put32(out8 + 4, 0);
        return 0.0f;
    }
    if (count == 1) {
        single_color_icbc(col[0], &o);
        err = mse_of(in, wi, cw, &o);
        put16(out8, o.c0); put16(out8 + 2, o.c1); put32(out8 + 4, o.idx);
        return err;
    }
    err = FLT_MAX;
    if (box_fit) {
        v3 c0 = mk3(0, 0, 0), c1 = mk3(1, 1, 1);
        for (int i = 0; i < count; i++) {
            c0 = mk3(ic_max(c0.x, col[i].x), ic_max(c0.y, col[i].y), ic_max(c0.z, col[i].z));
            c1 = mk3(ic_min(c1.x, col[i].x), ic_min(c1.y, col[i].y), ic_min(c1.z, col[i].z));
        }
        /* inset_bbox (src/nvtt/icbc.h:3143-3149) */
        float bias = (8.0f / 255.0f) / 16.0f;
        v3 d = sub3(c0, c1);
        v3 inset = sub3(mk3(d.x / 16.0f, d.y / 16.0f, d.z / 16.0f), mk3(bias, bias, bias));
        c0 = sat3(sub3(c0, inset));
        c1 = sat3(add3(c1, inset));
        /* select_diagonal (src/nvtt/icbc.h:3107-3141) */
        v3 center = scl3(add3(c0, c1), 0.5f);
        float cxz = 0.0f, cyz = 0.0f;
        for (int i = 0; i < count; i++) {
            v3 t = sub3(col[i], center);
            cxz += t.x * t.z; cyz += t.y * t.z;
        }
        float x0 = c0.x, y0 = c0.y, x1 = c1.x, y1 = c1.y;
        if (cxz < 0) { float t = x0; x0 = x1; x1 = t; }
        if (cyz < 0) { float t = y0; y0 = y1; y1 = t; }
        c0 = mk3(x0, y0, c0.z); c1 = mk3(x1, y1, c1.z);
        err = output_block4(in, wi, cw, c0, c1, &o);
        if (lsq && lsq_endpoints4(o.idx, in, &c0, &c1)) {
            bc1_t t;
            float e = output_block4(in, wi, cw, c0, c1, &t);
            if (e < err) { err = e; o = t; }
        }
    }
    if (cfit) {
        int use_black = any_black && three_color_black;
        int use_three = cfit3 || (use_black && cfit3_black_only);
        v3 metric = mul3(cw, cw);
        sat_t s;
        int sn = compute_sat(col, w, count, &s);
        v3 a, b;
        cluster_fit_four(&s, sn, metric, &a, &b);
        bc1_t cf;
        float cerr = output_block4(in, wi, cw, a, b, &cf);
        int done = 0;
        if (use_three) {
            if (use_black) {
                v3 tc[16];
                float tw[16];
                int tn = skip_blacks(col, w, count, tc, tw);
                if (!tn) done = 1;
                else sn = compute_sat(tc, tw, tn, &s);
            }
            if (!done) {
                cluster_fit_three(&s, sn, metric, &a, &b);
                bc1_t c3;
                float e3 = output_block3(in, wi, cw, three_color_black, a, b, &c3);
                if (e3 < cerr) { cerr = e3; cf = c3; }
            }
        }
        if (cerr < err) { o = cf; err = cerr; }
    }
    if (refine) err = refine_endpoints(in, wi, cw, three_color_mode, err, &o);
    put16(out8, o.c0); put16(out8 + 2, o.c1); put32(out8 + 4, o.idx);
    return err;
}

/* ------------------------------------------------------------------------------------------ */
/* Block gathers                                                                                */

/* FloatColorCompressorTask gather (src/nvtt/BlockCompressor.cpp:116-166): texels outside the
 * image are zero with zero weight; weights are saturate(alpha) under Transparency. */
static void gather_float(const float *rgba, int w, int h, int alpha_mode, int bx, int by, float *col, float *wt) {
    const size_t n = (size_t)w * h;
    int bw = w - bx * 4; if (bw > 4) bw = 4;
    int bh = h - by * 4; if (bh > 4) bh = 4;
    for (int y = 0; y < 4; y++)
        for (int x = 0; x < 4; x++) {
            int k = 4 * y + x;
            if (x < bw && y < bh) {
                size_t s = (size_t)(by * 4 + y) * w + (bx * 4 + x);
                float a = rgba[3 * n + s];
                col[4 * k] = rgba[s]; col[4 * k + 1] = rgba[n + s]; col[4 * k + 2] = rgba[2 * n + s]; col[4 * k + 3] = a;
                wt[k] = alpha_mode == ORA_ALPHA_TRANSPARENCY ? ic_clamp(a, 0.0f, 1.0f) : 1.0f;
            } else {
                col[4 * k] = col[4 * k + 1] = col[4 * k + 2] = col[4 * k + 3] = 0.0f;
                wt[k] = 0.0f;
            }
        }
}

/* ColorBlock::init(float) (src/nvimage/ColorBlock.cpp:80-110): clamp, scale by 255 and
 * truncate; blocks past the edge repeat pixels with i % size. Output is BGRA bytes. */
void ora_colorblock_gather(const float *rgba, int w, int h, int x, int y, uint8_t *bgra) {
    const size_t n = (size_t)w * h;
    unsigned bw = (unsigned)(w - x) < 4u ? (unsigned)(w - x) : 4u;
    unsigned bh = (unsigned)(h - y) < 4u ? (unsigned)(h - y) : 4u;
    for (unsigned i = 0; i < 4; i++) {
        unsigned yy = i % bh;
        for (unsigned e = 0; e < 4; e++) {
            unsigned xx = e % bw;
            size_t idx = (size_t)(y + yy) * w + x + xx;
            uint8_t *c = bgra + 4 * (i * 4 + e);
            c[2] = (uint8_t)(255 * ic_clamp(rgba[idx], 0.0f, 1.0f));
            c[1] = (uint8_t)(255 * ic_clamp(rgba[idx + n], 0.0f, 1.0f));
            c[0] = (uint8_t)(255 * ic_clamp(rgba[idx + 2 * n], 0.0f, 1.0f));
            c[3] = (uint8_t)(255 * ic_clamp(rgba[idx + 3 * n], 0.0f, 1.0f));
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Interpolated alpha / channel blocks                                                          */

/* AlphaBlockDXT5::evaluatePalette, D3D10 (src/nvimage/BlockDXT.cpp:336-378). */
static void alpha_palette(int a0, int a1, int pal[8]) {
    pal[0] = a0; pal[1] = a1;
    if (a0 > a1) {
        for (int k = 1; k <= 6; k++) pal[k + 1] = ((7 - k) * a0 + k * a1) / 7;
    } else {
        for (int k = 1; k <= 4; k++) pal[k + 1] = ((5 - k) * a0 + k * a1) / 5;
        pal[6] = 0; pal[7] = 255;
    }
}

typedef struct { int a0, a1; int idx[16]; } ablk_t;

static void pack_alpha(const ablk_t *b, uint8_t *out8) {
    uint64_t u = (uint64_t)(b->a0 & 255) | ((uint64_t)(b->a1 & 255) << 8);
    for (int i = 0; i < 16; i++) u |= (uint64_t)(b->idx[i] & 7) << (16 + 3 * i);
    for (int i = 0; i < 8; i++) out8[i] = (uint8_t)(u >> (8 * i));
}

/* computeAlphaIndices of QuickCompress (src/nvtt/QuickCompressDXT.cpp:505-536). */
static unsigned quick_alpha_indices(const uint8_t *a, ablk_t *b) {
    int pal[8];
    alpha_palette(b->a0, b->a1, pal);
    unsigned total = 0;
    for (int i = 0; i < 16; i++) {
        unsigned besterr = 256 * 256;
        int best = 8;
        for (int p = 0; p < 8; p++) {
            int d = pal[p] - a[i];
            unsigned e = (unsigned)(d * d);
            if (e < besterr) { besterr = e; best = p; }
        }
        total += besterr;
        b->idx[i] = best;
    }
    return total;
}

/* optimizeAlpha8 (src/nvtt/QuickCompressDXT.cpp:538-592). */
static void quick_alpha_refit(const uint8_t *a, ablk_t *b) {
    float a2 = 0, b2 = 0, ab = 0, ax = 0, bx = 0;
    for (int i = 0; i < 16; i++) {
        unsigned k = (unsigned)b->idx[i];
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
        for (int i = 0; i < 16; i++) b->idx[i] = b->idx[i] < 2 ? 1 - b->idx[i] : 9 - b->idx[i];
    } else if (v0 == v1) {
        for (int i = 0; i < 16; i++) b->idx[i] = 0;
    }
    b->a0 = (int)v0; b->a1 = (int)v1;
}

/* QuickCompress::compressDXT5A (src/nvtt/QuickCompressDXT.cpp:779-821). The reference's
 * sameIndices() compares the two endpoint bytes (its mask keeps only the low 16 bits), and this
 * restatement keeps that. */
void ora_dxt5a_quick(const uint8_t *a, uint8_t *out8) {
    int hi = 0, lo = 255;
    for (int i = 0; i < 16; i++) { if (a[i] > hi) hi = a[i]; if (a[i] < lo) lo = a[i]; }
    ablk_t b;
    b.a0 = (uint8_t)(hi - (hi - lo) / 34);
    b.a1 = (uint8_t)(lo + (hi - lo) / 34);
    unsigned best = quick_alpha_indices(a, &b);
    ablk_t bestb = b;
    for (int it = 0; it < 8; it++) {
        quick_alpha_refit(a, &b);
        unsigned e = quick_alpha_indices(a, &b);
        if (e >= best) break;
        if (b.a0 == bestb.a0 && b.a1 == bestb.a1) { bestb = b; break; }
        best = e;
        bestb = b;
    }
    pack_alpha(&bestb, out8);
}

/* computeAlphaError of OptimalCompress (src/nvtt/OptimalCompressDXT.cpp:189-217), unit weights. */
static float opt_alpha_error(const uint8_t *a, int a0, int a1, float bound) {
    int pal[8];
    alpha_palette(a0, a1, pal);
    float total = 0;
    for (int i = 0; i < 16; i++) {
        int md = 0x7fffffff;
        for (int p = 0; p < 8; p++) { int d = a[i] - pal[p]; d = d * d; if (d < md) md = d; }
        total += md * 1.0f;
        if (total > bound) return total;
    }
    return total;
}

/* OptimalCompress::compressDXT5A (src/nvtt/OptimalCompressDXT.cpp:512-607). The reference starts
 * the search from the error of whatever endpoints the destination block already holds; this
 * restatement (and the GPU kernel) start from a zeroed destination block. */
void ora_dxt5a_optimal(const uint8_t *a, uint8_t *out8) {
    int mina = 255, maxa = 0, mina01 = 255, maxa01 = 0;
    for (int i = 0; i < 16; i++) {
        int v = a[i];
        if (v < mina) mina = v;
        if (v > maxa) maxa = v;
        if (v != 0 && v != 255) { if (v < mina01) mina01 = v; if (v > maxa01) maxa01 = v; }
    }
    ablk_t b;
    if (maxa - mina < 8) { b.a0 = maxa; b.a1 = mina; }
    else if (maxa01 - mina01 < 6) { b.a0 = mina01; b.a1 = maxa01; }
    else {
        float besterr = opt_alpha_error(a, 0, 0, FLT_MAX);
        int ba0 = maxa, ba1 = mina;
        int lo = mina <= 8 ? 0 : mina - 8;
        int hi = maxa >= 255 - 8 ? 255 : maxa + 8;
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
    /* computeAlphaIndices (src/nvtt/OptimalCompressDXT.cpp:219-244) */
    int pal[8];
    alpha_palette(b.a0, b.a1, pal);
    for (int i = 0; i < 16; i++) {
        int md = 0x7fffffff, bi = 8;
        for (int p = 0; p < 8; p++) { int d = a[i] - pal[p]; d = d * d; if (d < md) { md = d; bi = p; } }
        b.idx[i] = bi;
    }
    pack_alpha(&b, out8);
}

/* OptimalCompress::compressDXT1(Color32) (src/nvtt/OptimalCompressDXT.cpp:254-269). */
void ora_dxt1_single_color(int r, int g, int b, uint8_t *out8) {
    ensure_init();
    unsigned c0 = ((unsigned)g_opt_match5[r][0] << 11) | ((unsigned)g_opt_match6[g][0] << 5) | g_opt_match5[b][0];
    unsigned c1 = ((unsigned)g_opt_match5[r][1] << 11) | ((unsigned)g_opt_match6[g][1] << 5) | g_opt_match5[b][1];
    uint32_t idx = 0xaaaaaaaau;
    if (c0 < c1) { unsigned t = c0; c0 = c1; c1 = t; idx ^= 0x55555555u; }
    put16(out8, c0); put16(out8 + 2, c1); put32(out8 + 4, idx);
}

/* OptimalCompress::compressDXT1a(Color32, alphaMask) (src/nvtt/OptimalCompressDXT.cpp:271-292):
 * without transparent texels the four-colour block above; otherwise the three-colour midpoint
 * tables, endpoints ordered col0 <= col1, index 2 everywhere and 3 on the transparent texels. */
void ora_dxt1a_single_color(int r, int g, int b, uint32_t alpha_mask, uint8_t *out8) {
    ensure_init();
    if (alpha_mask == 0) { ora_dxt1_single_color(r, g, b, out8); return; }
    unsigned c0 = ((unsigned)g_opt_alpha5[r][0] << 11) | ((unsigned)g_opt_alpha6[g][0] << 5) | g_opt_alpha5[b][0];
    unsigned c1 = ((unsigned)g_opt_alpha5[r][1] << 11) | ((unsigned)g_opt_alpha6[g][1] << 5) | g_opt_alpha5[b][1];
    if (c0 > c1) { unsigned t = c0; c0 = c1; c1 = t; }
    put16(out8, c0); put16(out8 + 2, c1); put32(out8 + 4, 0xaaaaaaaau | alpha_mask);
}

/* ------------------------------------------------------------------------------------------ */
/* squish weighted cluster fit (BC3 colour, BC1a), scalar build                                 */

/* ColourSet (src/nvtt/squish/colourset.cpp:35-139, no minimal set), WeightedClusterFit::
 * SetColourSet (src/nvtt/squish/weightedclusterfit.cpp:39-105), ComputeWeightedCovariance /
 * ComputePrincipleComponent (src/nvtt/squish/maths.cpp:32-135), Compress4 (scalar,
 * src/nvtt/squish/weightedclusterfit.cpp:476-589), WriteColourBlock4
 * (src/nvtt/squish/colourblock.cpp:108-139). */
static int float_to_int(float a, int limit) {
    int i = (int)(a + 0.5f);
    if (i < 0) i = 0; else if (i > limit) i = limit;
    return i;
}
static int float_to_565(v3 c) {
    return (float_to_int(31.0f * c.x, 31) << 11) | (float_to_int(63.0f * c.y, 63) << 5) | float_to_int(31.0f * c.z, 31);
}

/* The colour set and the sorted, weighted points of one block. */
typedef struct {
    int count, transparent;
    int remap[16];          /* point of each texel; -1 = transparent (DXT1 mode) */
    int order[16];          /* point of each sorted position */
    v3 wp[17];              /* weighted points in axis order (the tail entries are read, never used) */
    float ww[17];
    v3 xsum, msq;
    float wsum;
} squish_set;

static void squish_prepare(const uint8_t *bgra, int weight_by_alpha, int dxt1, v3 metric, squish_set *S) {
    /* ColourSet with the header's default createMinimalSet = true
     * (src/nvtt/squish/colourset.h:40, src/nvtt/squish/colourset.cpp:44-90): texels with equal RGB
     * bytes share one point whose weight is the sum of theirs, points in first-occurrence order.
     * In DXT1 mode a texel with alpha 0 is left out (remap -1) and never matched. */
    v3 pts[16];
    float wts[16];
    int count = 0;
    S->transparent = 0;
    for (int i = 0; i < 16; i++) {
        if (dxt1 && bgra[4 * i + 3] == 0) { S->remap[i] = -1; S->transparent = 1; continue; }
        const float wi = weight_by_alpha ? (float)(bgra[4 * i + 3] + 1) / 256.0f : 1.0f;
        for (int j = 0;; ++j) {
            if (j == i) {
                pts[count] = mk3((float)bgra[4 * i + 2] / 255.0f, (float)bgra[4 * i + 1] / 255.0f, (float)bgra[4 * i + 0] / 255.0f);
                wts[count] = wi;
                S->remap[i] = count;
                ++count;
                break;
            }
            if (bgra[4 * i] == bgra[4 * j] && bgra[4 * i + 1] == bgra[4 * j + 1] && bgra[4 * i + 2] == bgra[4 * j + 2] &&
                (bgra[4 * j + 3] != 0 || !dxt1)) {
                const int index = S->remap[j];
                wts[index] += wi;
                S->remap[i] = index;
                break;
            }
        }
    }
    S->count = count;
    /* weighted covariance */
    float total = 0.0f;
    v3 cen = mk3(0, 0, 0);
    for (int i = 0; i < count; i++) { total += wts[i]; cen = add3(cen, scl3(pts[i], wts[i])); }
    cen = scl3(cen, 1.0f / total);
    float m[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < count; i++) {
        v3 a = mul3(sub3(pts[i], cen), metric);
        v3 b = scl3(a, wts[i]);
        m[0] += a.x * b.x; m[1] += a.x * b.y; m[2] += a.x * b.z;
        m[3] += a.y * b.y; m[4] += a.y * b.z; m[5] += a.z * b.z;
    }
    /* principal component, power iteration */
    v3 r0 = mk3(m[0], m[1], m[2]), r1 = mk3(m[1], m[3], m[4]), r2 = mk3(m[2], m[4], m[5]);
    float l0 = dot3(r0, r0), l1 = dot3(r1, r1), l2 = dot3(r2, r2);
    v3 v = (l0 > l1 && l0 > l2) ? r0 : (l1 > l2 ? r1 : r2);
    for (int it = 0; it < 8; it++) {
        float x = v.x * m[0] + v.y * m[1] + v.z * m[2];
        float y = v.x * m[1] + v.y * m[3] + v.z * m[4];
        float z = v.x * m[2] + v.y * m[4] + v.z * m[5];
        float norm = sq_max(sq_max(x, y), z);
        float iv = 1.0f / norm;
        if (norm == 0.0f) { v = mk3(0, 0, 0); break; }
        v = mk3(x * iv, y * iv, z * iv);
    }
    /* order along the axis (stable) */
    float dps[16];
    for (int i = 0; i < count; i++) { dps[i] = dot3(pts[i], v); S->order[i] = i; }
    for (int i = 0; i < count; i++)
        for (int j = i; j > 0 && dps[j] < dps[j - 1]; --j) {
            float t = dps[j]; dps[j] = dps[j - 1]; dps[j - 1] = t;
            int o = S->order[j]; S->order[j] = S->order[j - 1]; S->order[j - 1] = o;
        }
    S->xsum = mk3(0, 0, 0);
    S->wsum = 0.0f;
    for (int i = 0; i < count; i++) {
        int p = S->order[i];
        S->wp[i] = scl3(pts[p], wts[p]);
        S->xsum = add3(S->xsum, S->wp[i]);
        S->ww[i] = wts[p];
        S->wsum += S->ww[i];
    }
    for (int i = count; i < 17; i++) { S->wp[i] = mk3(0, 0, 0); S->ww[i] = 0.0f; }
    S->msq = mul3(metric, metric);
}

/* Min(one, Max(zero, v)) then Floor(grid * v + half) * gridrcp, grid (31, 63, 31)
 * (src/nvtt/squish/weightedclusterfit.cpp:516-519). */
static v3 squish_snap(v3 a) {
    a = mk3(sq_min(1.0f, sq_max(0.0f, a.x)), sq_min(1.0f, sq_max(0.0f, a.y)), sq_min(1.0f, sq_max(0.0f, a.z)));
    return mk3(floorf(31.0f * a.x + 0.5f) * (1.0f / 31.0f), floorf(63.0f * a.y + 0.5f) * (1.0f / 63.0f),
               floorf(31.0f * a.z + 0.5f) * (1.0f / 31.0f));
}

/* Compress4's split search (scalar, src/nvtt/squish/weightedclusterfit.cpp:476-545): the first
 * strict minimum; the winner's endpoints and cluster sizes. */
static float squish_search4(const squish_set *S, v3 *bs, v3 *be, int *b0, int *b1, int *b2) {
    const int count = S->count;
    float besterr = FLT_MAX;
    *bs = mk3(0, 0, 0); *be = mk3(0, 0, 0);
    *b0 = *b1 = *b2 = 0;
    v3 x0 = mk3(0, 0, 0);
    float w0 = 0.0f;
    for (int c0 = 0; c0 <= count; c0++) {
        v3 x1 = mk3(0, 0, 0);
        float w1 = 0.0f;
        for (int c1 = 0; c1 <= count - c0; c1++) {
            v3 x2 = mk3(0, 0, 0);
            float w2 = 0.0f;
            for (int c2 = 0; c2 <= count - c0 - c1; c2++) {
                float w3 = S->wsum - w0 - w1 - w2;
                float a2 = w0 + w1 * (4.0f / 9.0f) + w2 * (1.0f / 9.0f);
                float b2s = w3 + w2 * (4.0f / 9.0f) + w1 * (1.0f / 9.0f);
                float ab = (w1 + w2) * (2.0f / 9.0f);
                float f = 1.0f / (a2 * b2s - ab * ab);
                v3 ax = add3(add3(x0, scl3(x1, 2.0f / 3.0f)), scl3(x2, 1.0f / 3.0f));
                v3 bx = sub3(S->xsum, ax);
                v3 a = squish_snap(scl3(sub3(scl3(ax, b2s), scl3(bx, ab)), f));
                v3 b = squish_snap(scl3(sub3(scl3(bx, a2), scl3(ax, ab)), f));
                v3 t = sub3(sub3(scl3(mul3(a, b), ab), mul3(a, ax)), mul3(b, bx));
                v3 e1 = add3(add3(scl3(mul3(a, a), a2), scl3(mul3(b, b), b2s)), scl3(t, 2.0f));
                float err = dot3(e1, S->msq);
                if (err < besterr) { besterr = err; *bs = a; *be = b; *b0 = c0; *b1 = c1; *b2 = c2; }
                x2 = add3(x2, S->wp[c0 + c1 + c2]);
                w2 += S->ww[c0 + c1 + c2];
            }
            x1 = add3(x1, S->wp[c0 + c1]);
            w1 += S->ww[c0 + c1];
        }
        x0 = add3(x0, S->wp[c0]);
        w0 += S->ww[c0];
    }
    return besterr;
}

/* Compress3's split search (scalar, src/nvtt/squish/weightedclusterfit.cpp:372-431). */
static float squish_search3(const squish_set *S, v3 *bs, v3 *be, int *b0, int *b1) {
    const int count = S->count;
    float besterr = FLT_MAX;
    *bs = mk3(0, 0, 0); *be = mk3(0, 0, 0);
    *b0 = *b1 = 0;
    v3 x0 = mk3(0, 0, 0);
    float w0 = 0.0f;
    for (int c0 = 0; c0 <= count; c0++) {
        v3 x1 = mk3(0, 0, 0);
        float w1 = 0.0f;
        for (int c1 = 0; c1 <= count - c0; c1++) {
            float w2 = S->wsum - w0 - w1;
            float a2 = w0 + w1 * 0.25f;
            float b2s = w2 + w1 * 0.25f;
            float ab = w1 * 0.25f;
            float f = 1.0f / (a2 * b2s - ab * ab);
            v3 ax = add3(x0, scl3(x1, 0.5f));
            v3 bx = sub3(S->xsum, ax);
            v3 a = squish_snap(scl3(sub3(scl3(ax, b2s), scl3(bx, ab)), f));
            v3 b = squish_snap(scl3(sub3(scl3(bx, a2), scl3(ax, ab)), f));
            v3 t = sub3(sub3(scl3(mul3(a, b), ab), mul3(a, ax)), mul3(b, bx));
            v3 e1 = add3(add3(scl3(mul3(a, a), a2), scl3(mul3(b, b), b2s)), scl3(t, 2.0f));
            float err = dot3(e1, S->msq);
            if (err < besterr) { besterr = err; *bs = a; *be = b; *b0 = c0; *b1 = c1; }
            x1 = add3(x1, S->wp[c0 + c1]);
            w1 += S->ww[c0 + c1];
        }
        x0 = add3(x0, S->wp[c0]);
        w0 += S->ww[c0];
    }
    return besterr;
}

/* Cluster of each sorted position -> point indices -> texel indices (ColourSet::RemapIndices,
 * src/nvtt/squish/colourset.cpp:141-151: transparent texels take index 3). */
static void squish_texel_indices(const squish_set *S, int b0, int b1, int b2, int three, uint8_t idx[16]) {
    uint8_t point_idx[16];
    for (int i = 0; i < S->count; i++)
        point_idx[S->order[i]] = three ? (i < b0 ? 0 : (i < b0 + b1 ? 2 : 1))
                                       : (i < b0 ? 0 : (i < b0 + b1 ? 2 : (i < b0 + b1 + b2 ? 3 : 1)));
    for (int i = 0; i < 16; i++) idx[i] = S->remap[i] < 0 ? 3 : point_idx[S->remap[i]];
}

static void write_colour_block(int a, int b, const uint8_t rem[16], uint8_t *out8) {
    out8[0] = (uint8_t)(a & 0xff); out8[1] = (uint8_t)(a >> 8);
    out8[2] = (uint8_t)(b & 0xff); out8[3] = (uint8_t)(b >> 8);
    for (int i = 0; i < 4; i++)
        out8[4 + i] = (uint8_t)(rem[4 * i] | (rem[4 * i + 1] << 2) | (rem[4 * i + 2] << 4) | (rem[4 * i + 3] << 6));
}

/* WriteColourBlock4 (src/nvtt/squish/colourblock.cpp:108-139). */
static void write_colour_block4(v3 s, v3 e, const uint8_t idx[16], uint8_t *out8) {
    int a = float_to_565(s), b = float_to_565(e);
    uint8_t rem[16];
    if (a < b) { int t = a; a = b; b = t; for (int i = 0; i < 16; i++) rem[i] = (idx[i] ^ 1) & 3; }
    else if (a == b) { memset(rem, 0, 16); }
    else memcpy(rem, idx, 16);
    write_colour_block(a, b, rem, out8);
}

/* WriteColourBlock3 (src/nvtt/squish/colourblock.cpp:75-106). */
static void write_colour_block3(v3 s, v3 e, const uint8_t idx[16], uint8_t *out8) {
    int a = float_to_565(s), b = float_to_565(e);
    uint8_t rem[16];
    if (a <= b) memcpy(rem, idx, 16);
    else {
        int t = a; a = b; b = t;
        for (int i = 0; i < 16; i++) rem[i] = idx[i] == 0 ? 1 : (idx[i] == 1 ? 0 : idx[i]);
    }
    write_colour_block(a, b, rem, out8);
}

static void squish_compress4(const uint8_t *bgra, int weight_by_alpha, v3 metric, uint8_t *out8) {
    squish_set S;
    squish_prepare(bgra, weight_by_alpha, 0, metric, &S);
    v3 bs, be;
    int b0, b1, b2;
    const float besterr = squish_search4(&S, &bs, &be, &b0, &b1, &b2);
    if (!(besterr < FLT_MAX)) { memset(out8, 0, 8); return; }
    uint8_t idx[16];
    squish_texel_indices(&S, b0, b1, b2, 0, idx);
    write_colour_block4(bs, be, idx, out8);
}

/* WeightedClusterFit with kDxt1 (ColourFit::Compress, src/nvtt/squish/colourfit.cpp:39-55):
 * Compress3, then Compress4 unless a texel is transparent; a mode replaces the block only with a
 * strictly smaller error. */
static void squish_compress_dxt1(const uint8_t *bgra, int weight_by_alpha, v3 metric, uint8_t *out8) {
    squish_set S;
    squish_prepare(bgra, weight_by_alpha, 1, metric, &S);
    float best = FLT_MAX;
    v3 bs, be;
    int b0, b1, b2;
    uint8_t idx[16];
    memset(out8, 0, 8);
    const float e3 = squish_search3(&S, &bs, &be, &b0, &b1);
    if (e3 < best) {
        squish_texel_indices(&S, b0, b1, 0, 1, idx);
        write_colour_block3(bs, be, idx, out8);
        best = e3;
    }
    if (!S.transparent) {
        const float e4 = squish_search4(&S, &bs, &be, &b0, &b1, &b2);
        if (e4 < best) {
            squish_texel_indices(&S, b0, b1, b2, 0, idx);
            write_colour_block4(bs, be, idx, out8);
        }
    }
}

/* CompressorDXT1a::compressBlock (src/nvtt/CompressorDX9.cpp:83-111) for Normal quality and
 * above: the single-colour test looks at RGB only (ColorBlock::isSingleColor,
 * src/nvimage/ColorBlock.cpp:136-149). */
void ora_bc1a_block(const uint8_t *bgra, int alpha_mode, const float *cw3, uint8_t *out8) {
    ensure_init();
    uint32_t mask = 0;
    for (int i = 0; i < 16; i++)
        if (bgra[4 * i + 3] == 0) mask |= 3u << (2 * i);
    int single = 1;
    for (int i = 1; i < 16; i++)
        if (bgra[4 * i] != bgra[0] || bgra[4 * i + 1] != bgra[1] || bgra[4 * i + 2] != bgra[2]) single = 0;
    if (single) ora_dxt1a_single_color(bgra[2], bgra[1], bgra[0], mask, out8);
    else squish_compress_dxt1(bgra, alpha_mode == ORA_ALPHA_TRANSPARENCY, mk3(cw3[0], cw3[1], cw3[2]), out8);
}

/* FastCompressorBC4 / ProductionCompressorBC4 (src/nvtt/CompressorDX10.cpp:40-72): the red
 * channel as an interpolated-alpha block; Fastest and Normal use the quick fit. */
void ora_bc4_block(const uint8_t *bgra, int quality, uint8_t *out8) {
    uint8_t r[16];
    for (int i = 0; i < 16; i++) r[i] = bgra[4 * i + 2];
    if (quality == ORA_Q_FASTEST || quality == ORA_Q_NORMAL) ora_dxt5a_quick(r, out8);
    else ora_dxt5a_optimal(r, out8);
}

/* ------------------------------------------------------------------------------------------ */
/* QuickCompress::compressDXT1 (BC3 colour at Fastest)                                        */

/* roundAndExpand (src/nvtt/QuickCompressDXT.cpp:122-149); floor of a value in [0, 31]. */
static unsigned quick_round_expand(v3 *v) {
    unsigned r = (unsigned)floorf(ic_clamp(v->x * (31.0f / 255.0f), 0.0f, 31.0f));
    unsigned g = (unsigned)floorf(ic_clamp(v->y * (63.0f / 255.0f), 0.0f, 63.0f));
    unsigned b = (unsigned)floorf(ic_clamp(v->z * (31.0f / 255.0f), 0.0f, 31.0f));
    if (fabsf(v->x - (float)ex5(r + 1)) < fabsf(v->x - (float)ex5(r))) r = r + 1 < 31u ? r + 1 : 31u;
    if (fabsf(v->y - (float)ex6(g + 1)) < fabsf(v->y - (float)ex6(g))) g = g + 1 < 63u ? g + 1 : 63u;
    if (fabsf(v->z - (float)ex5(b + 1)) < fabsf(v->z - (float)ex5(b))) b = b + 1 < 31u ? b + 1 : 31u;
    unsigned w = (r << 11) | (g << 5) | b;
    *v = mk3((float)ex5(r), (float)ex6(g), (float)ex5(b));
    return w;
}

/* computeIndices4 (src/nvtt/QuickCompressDXT.cpp:195-227). */
static uint32_t quick_indices4(const v3 *blk, v3 maxc, v3 minc) {
    v3 pal[4];
    pal[0] = maxc; pal[1] = minc;
    float s1 = 1.0f - 1.0f / 3.0f, s2 = 1.0f - 2.0f / 3.0f;
    pal[2] = mk3(maxc.x * s1 + (1.0f / 3.0f) * minc.x, maxc.y * s1 + (1.0f / 3.0f) * minc.y, maxc.z * s1 + (1.0f / 3.0f) * minc.z);
    pal[3] = mk3(maxc.x * s2 + (2.0f / 3.0f) * minc.x, maxc.y * s2 + (2.0f / 3.0f) * minc.y, maxc.z * s2 + (2.0f / 3.0f) * minc.z);
    uint32_t idx = 0;
    for (int i = 0; i < 16; i++) {
        v3 t;
        t = sub3(pal[0], blk[i]); float d0 = dot3(t, t);
        t = sub3(pal[1], blk[i]); float d1 = dot3(t, t);
        t = sub3(pal[2], blk[i]); float d2 = dot3(t, t);
        t = sub3(pal[3], blk[i]); float d3 = dot3(t, t);
        unsigned b0 = d0 > d3, b1 = d1 > d2, b2 = d0 > d2, b3 = d1 > d3, b4 = d2 > d3;
        unsigned x0 = b1 & b2, x1 = b0 & b3, x2 = b0 & b4;
        idx |= (x2 | ((x0 | x1) << 1)) << (2 * i);
    }
    return idx;
}

void ora_quick_dxt1(const uint8_t *bgra, uint8_t *out8) {
    ensure_init();
    int single = 1;
    for (int i = 1; i < 16; i++)
        if (bgra[4 * i] != bgra[0] || bgra[4 * i + 1] != bgra[1] || bgra[4 * i + 2] != bgra[2]) single = 0;
    if (single) { ora_dxt1_single_color(bgra[2], bgra[1], bgra[0], out8); return; }
    v3 blk[16];
    for (int i = 0; i < 16; i++) blk[i] = mk3(bgra[4 * i + 2], bgra[4 * i + 1], bgra[4 * i + 0]);
    v3 mx = mk3(0, 0, 0), mn = mk3(255, 255, 255);
    for (int i = 0; i < 16; i++) {
        mx = mk3(ic_max(mx.x, blk[i].x), ic_max(mx.y, blk[i].y), ic_max(mx.z, blk[i].z));
        mn = mk3(ic_min(mn.x, blk[i].x), ic_min(mn.y, blk[i].y), ic_min(mn.z, blk[i].z));
    }
    /* selectDiagonal (:85-106) */
    v3 center = scl3(add3(mx, mn), 0.5f);
    float cx = 0.0f, cy = 0.0f;
    for (int i = 0; i < 16; i++) { v3 t = sub3(blk[i], center); cx += t.x * t.z; cy += t.y * t.z; }
    float x0 = mx.x, y0 = mx.y, x1 = mn.x, y1 = mn.y;
    if (cx < 0) { float t = x0; x0 = x1; x1 = t; }
    if (cy < 0) { float t = y0; y0 = y1; y1 = t; }
    mx = mk3(x0, y0, mx.z); mn = mk3(x1, y1, mn.z);
    /* insetBBox (:108-113) */
    v3 d = sub3(mx, mn);
    float bias = (8.0f / 255.0f) / 16.0f;
    v3 inset = mk3(d.x / 16.0f - bias, d.y / 16.0f - bias, d.z / 16.0f - bias);
    v3 t = sub3(mx, inset);
    mx = mk3(ic_clamp(t.x, 0.0f, 255.0f), ic_clamp(t.y, 0.0f, 255.0f), ic_clamp(t.z, 0.0f, 255.0f));
    t = add3(mn, inset);
    mn = mk3(ic_clamp(t.x, 0.0f, 255.0f), ic_clamp(t.y, 0.0f, 255.0f), ic_clamp(t.z, 0.0f, 255.0f));
    unsigned c0 = quick_round_expand(&mx), c1 = quick_round_expand(&mn);
    if (c0 < c1) { v3 tv = mx; mx = mn; mn = tv; unsigned tc = c0; c0 = c1; c1 = tc; }
    uint32_t idx = quick_indices4(blk, mx, mn);
    /* optimizeEndPoints4 (:406-452) */
    float a2 = 0, b2 = 0, ab = 0;
    v3 ax = mk3(0, 0, 0), bx = mk3(0, 0, 0);
    for (int i = 0; i < 16; i++) {
        unsigned bits = idx >> (2 * i);
        float beta = (float)(bits & 1);
        if (bits & 2) beta = (1 + beta) / 3.0f;
        float alpha = 1.0f - beta;
        a2 += alpha * alpha; b2 += beta * beta; ab += alpha * beta;
        ax = add3(ax, scl3(blk[i], alpha)); bx = add3(bx, scl3(blk[i], beta));
    }
    float den = a2 * b2 - ab * ab;
    if (!(fabsf(den - 0.0f) <= 0.0001f * ic_max(ic_max(1.0f, fabsf(den)), fabsf(0.0f)))) {
        float f = 1.0f / den;
        v3 a = scl3(sub3(scl3(ax, b2), scl3(bx, ab)), f);
        v3 b = scl3(sub3(scl3(bx, a2), scl3(ax, ab)), f);
        a = mk3(ic_clamp(a.x, 0.0f, 255.0f), ic_clamp(a.y, 0.0f, 255.0f), ic_clamp(a.z, 0.0f, 255.0f));
        b = mk3(ic_clamp(b.x, 0.0f, 255.0f), ic_clamp(b.y, 0.0f, 255.0f), ic_clamp(b.z, 0.0f, 255.0f));
        unsigned e0 = quick_round_expand(&a), e1 = quick_round_expand(&b);
        if (e0 < e1) { v3 tv = a; a = b; b = tv; unsigned tc = e0; e0 = e1; e1 = tc; }
        c0 = e0; c1 = e1;
        idx = quick_indices4(blk, a, b);
    }
    put16(out8, c0); put16(out8 + 2, c1); put32(out8 + 4, idx);
}

/* ------------------------------------------------------------------------------------------ */
/* BC3 / BC5 blocks and images                                                                  */

/* CompressorDXT5::compressBlock (src/nvtt/CompressorDX9.cpp:145-176) and FastCompressorDXT5
 * (src/nvtt/CompressorDX9.cpp:47-51). */
void ora_bc3_block(const uint8_t *bgra, int alpha_mode, int quality, const float *cw3, uint8_t *out16) {
    ensure_init();
    uint8_t a[16];
    for (int i = 0; i < 16; i++) a[i] = bgra[4 * i + 3];
    if (quality == ORA_Q_FASTEST) {
        ora_dxt5a_quick(a, out16);
        ora_quick_dxt1(bgra, out16 + 8);
        return;
    }
    if (quality == ORA_Q_HIGHEST) ora_dxt5a_optimal(a, out16);
    else ora_dxt5a_quick(a, out16);
    int single = 1;
    for (int i = 1; i < 16; i++)
        if (bgra[4 * i] != bgra[0] || bgra[4 * i + 1] != bgra[1] || bgra[4 * i + 2] != bgra[2]) single = 0;
    if (single) ora_dxt1_single_color(bgra[2], bgra[1], bgra[0], out16 + 8);
    else squish_compress4(bgra, alpha_mode == ORA_ALPHA_TRANSPARENCY, mk3(cw3[0], cw3[1], cw3[2]), out16 + 8);
}

/* FastCompressorBC5 / ProductionCompressorBC5 (src/nvtt/CompressorDX10.cpp:51-85). */
void ora_bc5_block(const uint8_t *bgra, int quality, uint8_t *out16) {
    uint8_t r[16], g[16];
    for (int i = 0; i < 16; i++) { r[i] = bgra[4 * i + 2]; g[i] = bgra[4 * i + 1]; }
    if (quality == ORA_Q_FASTEST || quality == ORA_Q_NORMAL) { ora_dxt5a_quick(r, out16); ora_dxt5a_quick(g, out16 + 8); }
    else { ora_dxt5a_optimal(r, out16); ora_dxt5a_optimal(g, out16 + 8); }
}

/* A small fork/join pool over block indices (the reference dispatches the same per-block task
 * through its thread pool, src/nvtt/BlockCompressor.cpp:169-205). */
typedef struct {
    void (*fn)(void *, int);
    void *ctx;
    int count;
    atomic_int next;
} job_t;

static void *job_worker(void *p) {
    job_t *j = (job_t *)p;
    for (;;) {
        int i = atomic_fetch_add(&j->next, 64);
        if (i >= j->count) break;
        int e = i + 64 < j->count ? i + 64 : j->count;
        for (; i < e; i++) j->fn(j->ctx, i);
    }
    return NULL;
}

static void run_jobs(void (*fn)(void *, int), void *ctx, int count, int threads) {
    job_t j;
    j.fn = fn; j.ctx = ctx; j.count = count;
    atomic_init(&j.next, 0);
    if (threads <= 1) { job_worker(&j); return; }
    if (threads > 256) threads = 256;
    pthread_t th[256];
    for (int t = 1; t < threads; t++) pthread_create(&th[t], NULL, job_worker, &j);
    job_worker(&j);
    for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
}

typedef struct {
    const float *rgba;
    const uint8_t *bgra;
    int w, h, bw, alpha_mode, quality, level;
    float cw[3];
    uint8_t *out;
} img_ctx;

static void bc1_task(void *p, int i) {
    img_ctx *c = (img_ctx *)p;
    float col[64], wt[16];
    gather_float(c->rgba, c->w, c->h, c->alpha_mode, i % c->bw, i / c->bw, col, wt);
    ora_bc1_block(c->level, col, wt, c->cw, 1, 1, c->out + 8 * (size_t)i);
}

void ora_bc1_image(const float *rgba, int w, int h, int alpha_mode, int quality, const float *cw3, uint8_t *out, int threads) {
    ensure_init();
    img_ctx c = {rgba, NULL, w, h, (w + 3) / 4, alpha_mode, quality, 7, {cw3[0], cw3[1], cw3[2]}, out};
    c.level = quality == ORA_Q_FASTEST ? 0 : (quality == ORA_Q_PRODUCTION ? 8 : 7);
    run_jobs(bc1_task, &c, c.bw * ((h + 3) / 4), threads);
}

static void bc3_task(void *p, int i) {
    img_ctx *c = (img_ctx *)p;
    uint8_t blk[64];
    ora_colorblock_gather(c->rgba, c->w, c->h, 4 * (i % c->bw), 4 * (i / c->bw), blk);
    ora_bc3_block(blk, c->alpha_mode, c->quality, c->cw, c->out + 16 * (size_t)i);
}

void ora_bc3_image(const float *rgba, int w, int h, int alpha_mode, int quality, const float *cw3, uint8_t *out, int threads) {
    ensure_init();
    img_ctx c = {rgba, NULL, w, h, (w + 3) / 4, alpha_mode, quality, 0, {cw3[0], cw3[1], cw3[2]}, out};
    run_jobs(bc3_task, &c, c.bw * ((h + 3) / 4), threads);
}

static void bc3u8_task(void *p, int i) {
    img_ctx *c = (img_ctx *)p;
    uint8_t blk[64];
    int x = 4 * (i % c->bw), y = 4 * (i / c->bw);
    unsigned bw = (unsigned)(c->w - x) < 4u ? (unsigned)(c->w - x) : 4u;
    unsigned bh = (unsigned)(c->h - y) < 4u ? (unsigned)(c->h - y) : 4u;
    for (unsigned r = 0; r < 4; r++)
        for (unsigned e = 0; e < 4; e++)
            memcpy(blk + 4 * (r * 4 + e), c->bgra + 4 * ((size_t)(y + r % bh) * c->w + x + e % bw), 4);
    ora_bc3_block(blk, c->alpha_mode, c->quality, c->cw, c->out + 16 * (size_t)i);
}

void ora_bc3_image_u8(const uint8_t *bgra, int w, int h, int alpha_mode, int quality, const float *cw3, uint8_t *out, int threads) {
    ensure_init();
    img_ctx c = {NULL, bgra, w, h, (w + 3) / 4, alpha_mode, quality, 0, {cw3[0], cw3[1], cw3[2]}, out};
    run_jobs(bc3u8_task, &c, c.bw * ((h + 3) / 4), threads);
}

static void bc5_task(void *p, int i) {
    img_ctx *c = (img_ctx *)p;
    uint8_t blk[64];
    ora_colorblock_gather(c->rgba, c->w, c->h, 4 * (i % c->bw), 4 * (i / c->bw), blk);
    ora_bc5_block(blk, c->quality, c->out + 16 * (size_t)i);
}

void ora_bc5_image(const float *rgba, int w, int h, int quality, uint8_t *out, int threads) {
    ensure_init();
    img_ctx c = {rgba, NULL, w, h, (w + 3) / 4, 0, quality, 0, {1, 1, 1}, out};
    run_jobs(bc5_task, &c, c.bw * ((h + 3) / 4), threads);
}

static void bc1a_task(void *p, int i) {
    img_ctx *c = (img_ctx *)p;
    uint8_t blk[64];
    ora_colorblock_gather(c->rgba, c->w, c->h, 4 * (i % c->bw), 4 * (i / c->bw), blk);
    ora_bc1a_block(blk, c->alpha_mode, c->cw, c->out + 8 * (size_t)i);
}

void ora_bc1a_image(const float *rgba, int w, int h, int alpha_mode, const float *cw3, uint8_t *out, int threads) {
    ensure_init();
    img_ctx c = {rgba, NULL, w, h, (w + 3) / 4, alpha_mode, 1, 0, {cw3[0], cw3[1], cw3[2]}, out};
    run_jobs(bc1a_task, &c, c.bw * ((h + 3) / 4), threads);
}

static void bc4_task(void *p, int i) {
    img_ctx *c = (img_ctx *)p;
    uint8_t blk[64];
    ora_colorblock_gather(c->rgba, c->w, c->h, 4 * (i % c->bw), 4 * (i / c->bw), blk);
    ora_bc4_block(blk, c->quality, c->out + 8 * (size_t)i);
}

void ora_bc4_image(const float *rgba, int w, int h, int quality, uint8_t *out, int threads) {
    ensure_init();
    img_ctx c = {rgba, NULL, w, h, (w + 3) / 4, 0, quality, 0, {1, 1, 1}, out};
    run_jobs(bc4_task, &c, c.bw * ((h + 3) / 4), threads);
}

/* ------------------------------------------------------------------------------------------ */
/* Filters (src/nvimage/Filter.cpp)                                                             */

static const float ORA_PI = (float)3.1415926535897932384626433833;

/* sincf (src/nvimage/Filter.cpp:47-56) */
static float ora_sincf(float x) {
    if (fabsf(x) < 0.0001f) return 1.0f + x * x * (-1.0f / 6.0f + x * x * 1.0f / 120.0f);
    return sinf(x) / x;
}

/* bessel0 (src/nvimage/Filter.cpp:60-79) */
static float ora_bessel0(float x) {
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

/* Box/Triangle/Kaiser evaluate (src/nvimage/Filter.cpp:133-148, 258-265). */
float ora_filter_evaluate(int filter, float width, float p0, float p1, float x) {
    if (filter == ORA_FILTER_BOX) return fabsf(x) <= width ? 1.0f : 0.0f;
    if (filter == ORA_FILTER_TRIANGLE) { x = fabsf(x); return x < width ? width - x : 0.0f; }
    float sinc_value = ora_sincf(ORA_PI * x * p1);
    float t = x / width;
    if ((1 - t * t) >= 0) return sinc_value * ora_bessel0(p0 * sqrtf(1 - t * t)) / ora_bessel0(p0);
    return 0;
}

/* Filter::sampleBox (src/nvimage/Filter.cpp:88-103). */
static float sample_box(int filter, float width, float p0, float p1, float x, float scale, int samples) {
    double sum = 0;
    float isamples = 1.0f / (float)samples;
    for (int s = 0; s < samples; s++) {
        float p = (x + ((float)s + 0.5f) * isamples) * scale;
        sum += ora_filter_evaluate(filter, width, p0, p1, p);
    }
    return (float)(sum * isamples);
}

/* PolyphaseKernel (src/nvimage/Filter.cpp:520-566). */
int ora_polyphase(int filter, float width, float p0, float p1, int src_len, int dst_len, float *weights, int cap) {
    float scale = (float)dst_len / (float)src_len;
    const float iscale = 1.0f / scale;
    int samples = 32;
    if (scale > 1) { samples = 1; scale = 1; }
    const float kw = width * iscale;
    const int ws = (int)ceilf(kw * 2) + 1;
    if ((long long)ws * dst_len > cap) return ws;
    for (int i = 0; i < dst_len; i++) {
        const float center = (0.5f + (float)(unsigned)i) * iscale;
        const int left = (int)floorf(center - kw);
        float total = 0.0f;
        for (int j = 0; j < ws; j++) {
            float s = sample_box(filter, width, p0, p1, (float)(left + j) - center, scale, samples);
            weights[i * ws + j] = s;
            total += s;
        }
        for (int j = 0; j < ws; j++) weights[i * ws + j] /= total;
    }
    return ws;
}

/* Leftmost source index of output i, as applyKernelX/Y recompute it
 * (src/nvimage/FloatImage.cpp:1124-1131). */
int ora_polyphase_left(float width, int src_len, int dst_len, int i) {
    const float scale = (float)dst_len / (float)src_len;
    const float iscale = 1.0f / scale;
    const float kw = width * iscale;
    const float center = (0.5f + (float)(unsigned)i) * iscale;
    return (int)floorf(center - kw);
}

/* wrapClamp/wrapRepeat/wrapMirror (src/nvimage/FloatImage.h:298-317). */
static int wrap_index(int x, int w, int wm) {
    if (wm == ORA_WRAP_CLAMP) return x < 0 ? 0 : (x > w - 1 ? w - 1 : x);
    if (wm == ORA_WRAP_REPEAT) return x >= 0 ? x % w : (x + 1) % w + w - 1;
    if (w == 1) x = 0;
    x = abs(x);
    while (x >= w) x = abs(w + w - x - 2);
    return x;
}

/* FloatImage::fastDownSample (src/nvimage/FloatImage.cpp:559-737). */
void ora_fast_downsample(const float *src0, int W, int H, int channels, float *dst0) {
    const unsigned w = W / 2 > 1 ? (unsigned)W / 2 : 1, h = H / 2 > 1 ? (unsigned)H / 2 : 1;
    const size_t sn = (size_t)W * H, dn = (size_t)w * h;
    for (int c = 0; c < channels; c++) {
        const float *src = src0 + c * sn;
        float *dst = dst0 + c * dn;
        if (W == 1 || H == 1) {
            const unsigned n = w * h;
            if (((unsigned)W * (unsigned)H) & 1) {
                const float scale = 1.0f / (2 * n + 1);
                for (unsigned x = 0; x < n; x++) {
                    const float w0 = (float)(n - x), w1 = (float)(n - 0), w2 = (float)(1 + x);
                    *dst++ = scale * (w0 * src[0] + w1 * src[1] + w2 * src[2]);
                    src += 2;
                }
            } else {
                for (unsigned x = 0; x < n; x++) { *dst++ = 0.5f * (src[0] + src[1]); src += 2; }
            }
        } else if ((W & 1) == 0 && (H & 1) == 0) {
            for (unsigned y = 0; y < h; y++) {
                for (unsigned x = 0; x < w; x++) { *dst++ = 0.25f * (src[0] + src[1] + src[W] + src[W + 1]); src += 2; }
                src += W;
            }
        } else if ((W & 1) && (H & 1)) {
            const float scale = 1.0f / (float)((unsigned)W * (unsigned)H);
            for (unsigned y = 0; y < h; y++) {
                const float v0 = (float)(h - y), v1 = (float)(h - 0), v2 = (float)(1 + y);
                for (unsigned x = 0; x < w; x++) {
                    const float w0 = (float)(w - x), w1 = (float)(w - 0), w2 = (float)(1 + x);
                    float f = 0.0f;
                    f += v0 * (w0 * src[2 * x] + w1 * src[2 * x + 1] + w2 * src[2 * x + 2]);
                    f += v1 * (w0 * src[W + 2 * x] + w1 * src[W + 2 * x + 1] + w2 * src[W + 2 * x + 2]);
                    f += v2 * (w0 * src[2 * W + 2 * x] + w1 * src[2 * W + 2 * x + 1] + w2 * src[2 * W + 2 * x + 2]);
                    *dst++ = f * scale;
                }
                src += 2 * W;
            }
        } else if (W & 1) {
            const float scale = 1.0f / (float)(2 * (unsigned)W);
            for (unsigned y = 0; y < h; y++) {
                for (unsigned x = 0; x < w; x++) {
                    const float w0 = (float)(w - x), w1 = (float)(w - 0), w2 = (float)(1 + x);
                    float f = 0.0f;
                    f += w0 * (src[2 * x + 0] + src[W + 2 * x + 0]);
                    f += w1 * (src[2 * x + 1] + src[W + 2 * x + 1]);
                    f += w2 * (src[2 * x + 2] + src[W + 2 * x + 2]);
                    *dst++ = f * scale;
                }
                src += 2 * W;
            }
        } else {
            const float scale = 1.0f / (float)(2 * (unsigned)H);
            for (unsigned y = 0; y < h; y++) {
                const float v0 = (float)(h - y), v1 = (float)(h - 0), v2 = (float)(1 + y);
                for (unsigned x = 0; x < w; x++) {
                    float f = 0.0f;
                    f += v0 * (src[2 * x] + src[2 * x + 1]);
                    f += v1 * (src[W + 2 * x] + src[W + 2 * x + 1]);
                    f += v2 * (src[2 * W + 2 * x] + src[2 * W + 2 * x + 1]);
                    *dst++ = f * scale;
                }
                src += 2 * W;
            }
        }
    }
}

/* FloatImage::resize 2D (src/nvimage/FloatImage.cpp:761-808) with applyKernelX/Y
 * (:1115-1176): X pass into a w' x H plane, then Y pass, sums in tap order. */
void ora_resize(const float *src, int W, int H, int channels, int w, int h, int filter, float width, float p0, float p1, int wrap, float *dst) {
    int wsx = ora_polyphase(filter, width, p0, p1, W, w, NULL, 0);
    int wsy = ora_polyphase(filter, width, p0, p1, H, h, NULL, 0);
    float *kx = (float *)malloc(sizeof(float) * wsx * w), *ky = (float *)malloc(sizeof(float) * wsy * h);
    ora_polyphase(filter, width, p0, p1, W, w, kx, wsx * w);
    ora_polyphase(filter, width, p0, p1, H, h, ky, wsy * h);
    float *tmp = (float *)malloc(sizeof(float) * (size_t)w * H);
    for (int c = 0; c < channels; c++) {
        const float *sp = src + (size_t)c * W * H;
        for (int y = 0; y < H; y++)
            for (int i = 0; i < w; i++) {
                int left = ora_polyphase_left(width, W, w, i);
                float sum = 0;
                for (int j = 0; j < wsx; j++) sum += kx[i * wsx + j] * sp[(size_t)y * W + wrap_index(left + j, W, wrap)];
                tmp[(size_t)y * w + i] = sum;
            }
        float *dp = dst + (size_t)c * w * h;
        for (int x = 0; x < w; x++)
            for (int i = 0; i < h; i++) {
                int left = ora_polyphase_left(width, H, h, i);
                float sum = 0;
                for (int j = 0; j < wsy; j++) sum += ky[i * wsy + j] * tmp[(size_t)wrap_index(left + j, H, wrap) * w + x];
                dp[(size_t)i * w + x] = sum;
            }
    }
    free(tmp); free(kx); free(ky);
}

/* Alpha-weighted separable resize from the reference's weighted kernels
 * (src/nvimage/FloatImage.cpp:1212-1281): alpha plane with the plain kernels, colour planes
 * weighted by (alpha + 1/256) and renormalised per output texel. */
void ora_resize_weighted(const float *src, int W, int H, int w, int h, int filter, float width, float p0, float p1, int wrap, float *dst) {
    int wsx = ora_polyphase(filter, width, p0, p1, W, w, NULL, 0);
    int wsy = ora_polyphase(filter, width, p0, p1, H, h, NULL, 0);
    float *kx = (float *)malloc(sizeof(float) * wsx * w), *ky = (float *)malloc(sizeof(float) * wsy * h);
    ora_polyphase(filter, width, p0, p1, W, w, kx, wsx * w);
    ora_polyphase(filter, width, p0, p1, H, h, ky, wsy * h);
    const size_t sn = (size_t)W * H, tn = (size_t)w * H, dn = (size_t)w * h;
    float *tmp = (float *)malloc(sizeof(float) * 4 * tn);
    const float *sa = src + 3 * sn;
    for (int c = 0; c < 4; c++) {
        const float *sp = src + c * sn;
        for (int y = 0; y < H; y++)
            for (int i = 0; i < w; i++) {
                int left = ora_polyphase_left(width, W, w, i);
                float sum = 0, norm = 0;
                for (int j = 0; j < wsx; j++) {
                    size_t s = (size_t)y * W + wrap_index(left + j, W, wrap);
                    if (c == 3) sum += kx[i * wsx + j] * sp[s];
                    else { float wt = kx[i * wsx + j] * (sa[s] + (1.0f / 256.0f)); norm += wt; sum += wt * sp[s]; }
                }
                tmp[c * tn + (size_t)y * w + i] = c == 3 ? sum : sum / norm;
            }
    }
    const float *ta = tmp + 3 * tn;
    for (int c = 0; c < 4; c++) {
        const float *tp = tmp + c * tn;
        for (int x = 0; x < w; x++)
            for (int i = 0; i < h; i++) {
                int left = ora_polyphase_left(width, H, h, i);
                float sum = 0, norm = 0;
                for (int j = 0; j < wsy; j++) {
                    size_t s = (size_t)wrap_index(left + j, H, wrap) * w + x;
                    if (c == 3) sum += ky[i * wsy + j] * tp[s];
                    else { float wt = ky[i * wsy + j] * (ta[s] + (1.0f / 256.0f)); norm += wt; sum += wt * tp[s]; }
                }
                dst[c * dn + (size_t)i * w + x] = c == 3 ? sum : sum / norm;
            }
    }
    free(tmp); free(kx); free(ky);
}

/* ------------------------------------------------------------------------------------------ */
/* Colour transforms                                                                            */

/* Surface::setImage(InputFormat_BGRA_8UB) (src/nvtt/Surface.cpp:728-760). */
void ora_set_image_bgra8(const uint8_t *bgra, int n, float *rgba) {
    for (int i = 0; i < n; i++) {
        rgba[i] = (float)bgra[4 * i + 2] / 255.0f;
        rgba[n + i] = (float)bgra[4 * i + 1] / 255.0f;
        rgba[2 * n + i] = (float)bgra[4 * i + 0] / 255.0f;
        rgba[3 * n + i] = (float)bgra[4 * i + 3] / 255.0f;
    }
}

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* _powf_11_5 / _powf_5_11 (src/nvmath/Gamma.cpp:311-357). */
void ora_powf_11_5(const float *src, float *dst, int n) {
    ensure_init();
    for (int i = 0; i < n; i++) {
        uint32_t u = f2u(src[i]);
        int k = (int)(u >> 23);
        float m = u2f((u & ((1u << 23) - 1)) | (127u << 23));
        float pm = (((-0.00916587552f * m + 0.119315466f) * m + 1.01847068f) * m - 0.158338739f) * m + 0.0297184721f;
        dst[i] = g_pow_11_5[k] * pm;
    }
}
void ora_powf_5_11(const float *src, float *dst, int n) {
    ensure_init();
    for (int i = 0; i < n; i++) {
        uint32_t u = f2u(src[i]);
        int k = (int)(u >> 23);
        float m = u2f((u & ((1u << 23) - 1)) | (127u << 23));
        float pm = (((-0.0110083047f * m + 0.0905038750f) * m - 0.324697506f) * m + 0.876040946f) * m + 0.369160989f;
        dst[i] = g_pow_5_11[k] * pm;
    }
}

/* toSrgb / fromSrgb (src/nvtt/Surface.cpp:1512-1519, 1562-1568). */
void ora_to_srgb(const float *src, float *dst, int n) {
    for (int i = 0; i < n; i++) {
        float f = src[i];
        if (isnan(f)) f = 0.0f;
        else if (f <= 0.0f) f = 0.0f;
        else if (f <= 0.0031308f) f = 12.92f * f;
        else if (f <= 1.0f) f = (powf(f, 0.41666f) * 1.055f) - 0.055f;
        else f = 1.0f;
        dst[i] = f;
    }
}
void ora_from_srgb(const float *src, float *dst, int n) {
    for (int i = 0; i < n; i++) {
        float f = src[i];
        if (f < 0.0f) f = 0.0f;
        else if (f < 0.04045f) f = f / 12.92f;
        else if (f <= 1.0f) f = powf((f + 0.055f) / 1.055f, 2.4f);
        else f = 1.0f;
        dst[i] = f;
    }
}

/* nv::equal with the default relative epsilon (src/nvmath/nvmath.h:139-143). */
static int nv_equal(float a, float b) {
    return fabsf(a - b) <= 0.0001f * ic_max(ic_max(1.0f, fabsf(a)), fabsf(b));
}

static void xform_in(float *img, int n, int x, float gamma) {
    if (x == ORA_XFORM_SRGB) ora_from_srgb(img, img, 3 * n);
    else if (x == ORA_XFORM_GAMMA && !nv_equal(gamma, 1.0f)) {
        if (gamma == 2.2f) ora_powf_11_5(img, img, 3 * n);
        else for (int i = 0; i < 3 * n; i++) img[i] = powf(ic_max(0.0f, img[i]), gamma);
    }
}
static void xform_out(float *img, int n, int x, float gamma) {
    if (x == ORA_XFORM_SRGB) ora_to_srgb(img, img, 3 * n);
    else if (x == ORA_XFORM_GAMMA && !nv_equal(gamma, 1.0f)) {
        if (gamma == 2.2f) ora_powf_5_11(img, img, 3 * n);
        else for (int i = 0; i < 3 * n; i++) img[i] = powf(ic_max(0.0f, img[i]), 1.0f / gamma);
    }
}

/* Surface flow of the reference's Surface API (src/nvtt/tests/imperativeapi.cpp:32-86 shape):
 * setImage -> input transform -> per level { emit linear; copy -> output transform; emit } ->
 * buildNextMipmap (src/nvtt/Surface.cpp:1344-1406). Returns the number of levels. */
int ora_mip_chain(const uint8_t *bgra, int w, int h, int filter, float width, float p0, float p1, int wrap,
                  int alpha_mode, int in_xform, int out_xform, float gamma, int max_levels, float *linear, float *encoded) {
    float *img = (float *)malloc(sizeof(float) * 4 * (size_t)w * h);
    ora_set_image_bgra8(bgra, w * h, img);
    xform_in(img, w * h, in_xform, gamma);
    size_t off = 0;
    int levels = 0;
    for (;;) {
        const size_t n = (size_t)w * h;
        if (linear) memcpy(linear + off, img, sizeof(float) * 4 * n);
        if (encoded) {
            memcpy(encoded + off, img, sizeof(float) * 4 * n);
            xform_out(encoded + off, (int)n, out_xform, gamma);
        }
        off += 4 * n;
        levels++;
        if (levels >= max_levels || (w == 1 && h == 1)) break;
        int nw = w / 2 > 1 ? w / 2 : 1, nh = h / 2 > 1 ? h / 2 : 1;
        float *next = (float *)malloc(sizeof(float) * 4 * (size_t)nw * nh);
        if (alpha_mode != ORA_ALPHA_TRANSPARENCY && filter == ORA_FILTER_BOX && width == 0.5f)
            ora_fast_downsample(img, w, h, 4, next);
        else
            ora_resize(img, w, h, 4, nw, nh, filter, width, p0, p1, wrap, next);
        free(img);
        img = next; w = nw; h = nh;
    }
    free(img);
    return levels;
}

/* ------------------------------------------------------------------------------------------ */
/* Target extent of the InputOptions resize step (nv::getTargetExtent, src/nvtt/Surface.cpp:220-326,
 * 2D textures, no shape restriction) with the rounding helpers of src/nvtt/Surface.cpp:60-105 and
 * nextPowerOfTwo (src/nvcore/Utils.h:205-229). The reference tests RoundMode_ToNextMultipleOfFour
 * twice in its else-if chain, so RoundMode_ToNearestMultipleOfFour leaves the extents as they are. */
static unsigned next_pow2(unsigned x) {
    x--;
    x |= x >> 1; x |= x >> 2; x |= x >> 4; x |= x >> 8; x |= x >> 16;
    return x + 1;
}
static unsigned prev_pow2(unsigned v) { return next_pow2(v + 1) / 2; }
static unsigned nearest_pow2(unsigned v) {
    const unsigned np2 = next_pow2(v), pp2 = prev_pow2(v);
    return np2 - v <= v - pp2 ? np2 : pp2;
}

void ora_target_extent(int w, int h, int max_extent, int round_mode, int *out_w, int *out_h) {
    if (round_mode != 0 && max_extent > 0) max_extent = (int)prev_pow2((unsigned)max_extent);
    const int m = w > h ? w : h;
    if (max_extent > 0 && m > max_extent) {
        w = (w * max_extent) / m; if (w < 1) w = 1;
        h = (h * max_extent) / m; if (h < 1) h = 1;
    }
    switch (round_mode) {
        case 1: w = (int)next_pow2((unsigned)w); h = (int)next_pow2((unsigned)h); break;
        case 2: w = (int)nearest_pow2((unsigned)w); h = (int)nearest_pow2((unsigned)h); break;
        case 3: w = (int)prev_pow2((unsigned)w); h = (int)prev_pow2((unsigned)h); break;
        case 4: w = (int)(((unsigned)w + 3) & ~3u); h = (int)(((unsigned)h + 3) & ~3u); break;
        case 6: w = (int)((unsigned)w & ~3u); h = (int)((unsigned)h & ~3u); break;
        default: break;
    }
    *out_w = w;
    *out_h = h;
}

/* ------------------------------------------------------------------------------------------ */
/* Decode (Surface::setImage2D, D3D10) and RMSE                                                 */

static void decode_bc1(const uint8_t *b, uint8_t rgba[16][4]) {
    rgb8 pal[4];
    unsigned c0 = get16(b), c1 = get16(b + 2);
    palette_d3d10(c0, c1, pal);
    uint32_t idx = get32(b + 4);
    for (int i = 0; i < 16; i++) {
        int k = (idx >> (2 * i)) & 3;
        rgba[i][0] = (uint8_t)pal[k].r; rgba[i][1] = (uint8_t)pal[k].g; rgba[i][2] = (uint8_t)pal[k].b;
        rgba[i][3] = (c0 <= c1 && k == 3) ? 0 : 255;
    }
}

static void decode_alpha(const uint8_t *b, uint8_t out[16]) {
    int pal[8];
    alpha_palette(b[0], b[1], pal);
    uint64_t u = 0;
    for (int i = 0; i < 8; i++) u |= (uint64_t)b[i] << (8 * i);
    for (int i = 0; i < 16; i++) out[i] = (uint8_t)pal[(u >> (16 + 3 * i)) & 7];
}

/* Block decode into a planar FP32 image, 1/255 scale (src/nvtt/Surface.cpp:908-1116). BC5
 * decodes to (x, y, 0, 1) as the reference does for ATI2. */
int ora_decode(int format, const uint8_t *blocks, int w, int h, float *rgba) {
    const int bw = (w + 3) / 4, bh = (h + 3) / 4;
    const size_t n = (size_t)w * h;
    const int bs = format == ORA_FMT_BC1 || format == ORA_FMT_BC1A || format == ORA_FMT_BC4 ? 8 : 16;
    for (int by = 0; by < bh; by++)
        for (int bx = 0; bx < bw; bx++) {
            const uint8_t *b = blocks + (size_t)(by * bw + bx) * bs;
            uint8_t px[16][4];
            if (format == ORA_FMT_BC1 || format == ORA_FMT_BC1A) decode_bc1(b, px);
            else if (format == ORA_FMT_BC4) {  /* BlockATI1::decodeBlock (src/nvimage/BlockDXT.cpp:513-526) */
                uint8_t x[16];
                decode_alpha(b, x);
                for (int i = 0; i < 16; i++) { px[i][0] = px[i][1] = px[i][2] = x[i]; px[i][3] = 255; }
            }
            else if (format == ORA_FMT_BC3) {
                uint8_t a[16];
                decode_bc1(b + 8, px);
                decode_alpha(b, a);
                for (int i = 0; i < 16; i++) px[i][3] = a[i];
            } else if (format == ORA_FMT_BC5) {
                uint8_t x[16], y[16];
                decode_alpha(b, x);
                decode_alpha(b + 8, y);
                for (int i = 0; i < 16; i++) { px[i][0] = x[i]; px[i][1] = y[i]; px[i][2] = 0; px[i][3] = 255; }
            } else return -1;
            for (int yy = 0; yy < 4; yy++)
                for (int xx = 0; xx < 4; xx++) {
                    int X = bx * 4 + xx, Y = by * 4 + yy;
                    if (X >= w || Y >= h) continue;
                    size_t s = (size_t)Y * w + X;
                    for (int c = 0; c < 4; c++) rgba[c * n + s] = px[yy * 4 + xx][c] / 255.0f;
                }
        }
    return 0;
}

/* nv::rmsColorError / rmsAlphaError (src/nvimage/ErrorMetric.cpp:13-71). */
int ora_rms(int format, const float *ref, const uint8_t *blocks, int w, int h, int alpha_mode, float *rms_color, float *rms_alpha) {
    const size_t n = (size_t)w * h;
    float *dec = (float *)malloc(sizeof(float) * 4 * n);
    if (ora_decode(format, blocks, w, h, dec)) { free(dec); return -1; }
    double mse = 0, msa = 0;
    for (size_t i = 0; i < n; i++) {
        float r = ref[i] - dec[i], g = ref[n + i] - dec[n + i], b = ref[2 * n + i] - dec[2 * n + i];
        float a = 1;
        if (alpha_mode == ORA_ALPHA_TRANSPARENCY) a = ref[3 * n + i] * ref[3 * n + i];
        mse += (r * r) * a;
        mse += (g * g) * a;
        mse += (b * b) * a;
        float da = dec[3 * n + i] - ref[3 * n + i];
        msa += da * da;
    }
    *rms_color = (float)sqrt(mse / n);
    *rms_alpha = (float)sqrt(msa / n);
    free(dec);
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Check of a toSrgb quantiser step table: counts the floats in [0, 2] whose 8-bit code by
 * counting steps differs from uint8(255 * clamp(toSrgb(x), 0, 1)) computed directly. */
typedef struct { const float *steps; uint32_t lo, hi; long long bad; } srgb_scan_t;

static int srgb_code(float x) {
    float s;
    ora_to_srgb(&x, &s, 1);
    return (int)(uint8_t)(255 * ic_clamp(s, 0.0f, 1.0f));
}

static void *srgb_scan(void *p) {
    srgb_scan_t *t = (srgb_scan_t *)p;
    for (uint32_t b = t->lo; b < t->hi; b++) {
        const float x = u2f(b);
        int k = 0;
        while (k < 255 && t->steps[k + 1] <= x) k++;
        if (k != srgb_code(x)) t->bad++;
    }
    return NULL;
}

long long ora_count_srgb_step_mismatches(const float *steps, int threads) {
    const uint32_t hi = f2u(2.0f) + 1;
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    pthread_t th[64];
    srgb_scan_t jobs[64];
    for (int i = 0; i < threads; i++) {
        jobs[i].steps = steps;
        jobs[i].lo = (uint32_t)((uint64_t)hi * i / threads);
        jobs[i].hi = (uint32_t)((uint64_t)hi * (i + 1) / threads);
        jobs[i].bad = 0;
        pthread_create(&th[i], NULL, srgb_scan, &jobs[i]);
    }
    long long bad = 0;
    for (int i = 0; i < threads; i++) { pthread_join(th[i], NULL); bad += jobs[i].bad; }
    return bad;
}
