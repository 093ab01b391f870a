// Mip-chain kernels for sm_103a: Surface::setImage + colour transforms, FloatImage::fastDownSample
// and the separable polyphase resize (Box / Triangle / Kaiser) of Surface::buildNextMipmap.
//
// Data layout in HBM: each level is planar FP32 (plane c at c * w * h), as FloatImage stores it.
// A level can also be emitted as interleaved BGRA8 words already passed through the output
// transform and ColorBlock's truncating quantiser: that is what the BC3/BC5 encoders read.
//
// Exactness: kernels are built with --fmad=false; polyphase weights and window offsets come from
// the host (computed with the reference's own float/double steps), and every output is the
// sequential tap-order sum the reference computes, so levels are bit-identical to the CPU path.
#include <algorithm>

#include "ntg_async.cuh"
#include "ntg_device.cuh"
#include "ntg_internal.h"

namespace ntg {

// Polls of each mbarrier wait of the TMA-staged tile kernels before it gives up, and the word such a
// wait sets (1) before its kernel drains its copy in flight and returns.
constexpr int kMipWaitPolls = 1 << 22;
__device__ int g_mip_wait_polls = kMipWaitPolls;
__device__ unsigned int g_mip_status = 0;


// ---------------------------------------------------------------------------------------------
// Surface::setImage(InputFormat_BGRA_8UB) (src/nvtt/Surface.cpp:728-760) fused with the input
// transform. The input is 8-bit, so toLinear / toLinearFromSrgb of RGB collapse into a 256-entry
// table built on the host; alpha is v / 255.

__global__ void k_set_image(const uint32_t *__restrict__ bgra, size_t n, const float *__restrict__ lut,
                            float *__restrict__ out) {
    __shared__ float s_lut[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_lut[i] = lut[i];
    __syncthreads();
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t p = bgra[i];
        out[i] = s_lut[(p >> 16) & 255];
        out[n + i] = s_lut[(p >> 8) & 255];
        out[2 * n + i] = s_lut[p & 255];
        out[3 * n + i] = (float)(p >> 24) / 255.0f;
    }
}

// ---------------------------------------------------------------------------------------------
// Output transform + quantiser for the BC3/BC5 path: x -> uint8(255 * clamp(xform(x), 0, 1))
// (ColorBlock::init(float), src/nvimage/ColorBlock.cpp:103-106).
//   xform 0: identity; 1: toGamma(2.2) = powf_5_11, evaluated exactly on the device;
//   2: toSrgb, whose 8-bit result is a monotone step function of x: the host tabulates its 255
//      steps (the smallest float reaching each code) with the same libm the reference uses, and
//      the device counts the steps at or below x.
struct Quant {
    int xform;
    const float *steps;  // 256 entries, steps[0] unused, for xform 2
};

__device__ __forceinline__ uint32_t quantize(float x, int xform, const float *s_steps) {
    if (xform == 0) return quant_u8(x);
    if (xform == 1) return quant_u8(powf_5_11(x));
    // branch-free search over the sorted step table; NaN compares false everywhere -> 0
    int lo = 0;
#pragma unroll
    for (int b = 128; b >= 1; b >>= 1)
        if (lo + b <= 255 && s_steps[lo + b] <= x) lo += b;
    return (uint32_t)lo;
}

__device__ __forceinline__ uint32_t quantize_bgra(float r, float g, float b, float a, int xform, const float *s_steps) {
    return quantize(b, xform, s_steps) | (quantize(g, xform, s_steps) << 8) | (quantize(r, xform, s_steps) << 16) |
           (quant_u8(a) << 24);
}

// The sRGB quantiser with a bucket table over [2^-14, 2): buckets[b] (b = float bits >> 15, from the
// bucket of 2^-14) counts the steps at or below the smallest float of bucket b. The host checks,
// when it builds the table, that no bucket holds more than one step and that the first step lies
// above 2^-14; one comparison then finishes the count. Same code as quantize() for every float:
// below 2^-14 (negatives and NaN included) nothing is passed, from 2 on everything is.
constexpr int QB_LO = 113 << 8;   // (bits of 2^-14) >> 15; kSrgbBuckets buckets reach 2.0
__device__ __forceinline__ uint32_t quantize_srgb(float x, const float *s_steps, const uint8_t *s_buckets) {
    if (!(x >= 6.103515625e-05f)) return 0;
    if (x >= 2.0f) return 255;
    int c = s_buckets[(int)(__float_as_uint(x) >> 15) - QB_LO];
    if (c < 255 && s_steps[c + 1] <= x) c++;
    return (uint32_t)c;
}

__device__ __forceinline__ uint32_t quantize_srgb_bgra(float4 v, const float *s_steps, const uint8_t *s_buckets) {
    return quantize_srgb(v.z, s_steps, s_buckets) | (quantize_srgb(v.y, s_steps, s_buckets) << 8) |
           (quantize_srgb(v.x, s_steps, s_buckets) << 16) | (quant_u8(v.w) << 24);
}

// Self-check of quantize_srgb against the step search over every float bit pattern below 2^31
// (all non-negative floats, infinities and NaNs included): counts the disagreements.
__global__ void k_check_srgb(const float *__restrict__ steps, unsigned long long *__restrict__ bad) {
    __shared__ float s_steps[256];
    __shared__ uint8_t s_buckets[kSrgbBuckets];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_steps[i] = steps[i];
    const uint8_t *b = reinterpret_cast<const uint8_t *>(steps + 256);
    for (int i = threadIdx.x; i < kSrgbBuckets; i += blockDim.x) s_buckets[i] = b[i];
    __syncthreads();
    unsigned long long n = 0;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < 0x80000000u; u += gridDim.x * blockDim.x) {
        const float x = __uint_as_float(u);
        n += quantize(x, 2, s_steps) != quantize_srgb(x, s_steps, s_buckets);
        n += quantize(-x, 2, s_steps) != quantize_srgb(-x, s_steps, s_buckets);
    }
    if (n) atomicAdd(bad, n);
}

int launch_check_srgb(const float *steps, unsigned long long *bad, cudaStream_t s) {
    if (cudaMemsetAsync(bad, 0, sizeof *bad, s) != cudaSuccess) return launch_status();
    k_check_srgb<<<152 * 8, 256, 0, s>>>(steps, bad);
    return launch_status();
}

// Emits the quantised BGRA8 words of a planar FP32 level (used for level 0 of a chain).
__global__ void k_quantize_level(const float *__restrict__ rgba, size_t n, Quant q, uint32_t *__restrict__ out) {
    __shared__ float s_steps[256];
    if (q.xform == 2)
        for (int i = threadIdx.x; i < 256; i += blockDim.x) s_steps[i] = q.steps[i];
    __syncthreads();
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = quantize_bgra(rgba[i], rgba[n + i], rgba[2 * n + i], rgba[3 * n + i], q.xform, s_steps);
}

// ---------------------------------------------------------------------------------------------
// Job lists. Every mip kernel takes an array of MipJob (one level step of one texture) and a
// running unit count per job, so one launch covers a level of any number of textures; a unit is a
// destination texel (box), a PTW x PTH tile (general polyphase), a 32-column x `strip`-row tile
// (2:1 polyphase from FP32) or a 64 x 16 tile (2:1 polyphase from BGRA8). A unit finds its job by
// binary search over `first_unit`.
__device__ __forceinline__ int find_mip_job(const MipJob *__restrict__ jobs, int njobs, long long u) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_unit <= u) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The sRGB quantiser steps are one table for every job (they depend on no option); a CTA copies
// it into shared memory once, so the 8-step search of each quantised channel stays on chip.
__device__ __forceinline__ void load_steps(const MipJob *__restrict__ jobs, float *s_steps) {
    const float *steps = jobs[0].steps;
    if (steps)
        for (int i = threadIdx.x; i < 256; i += blockDim.x) s_steps[i] = __ldg(steps + i);
}

// ---------------------------------------------------------------------------------------------
// FloatImage::fastDownSample (src/nvimage/FloatImage.cpp:559-737): 2x2 box for even sizes,
// pair average for 1-D images and the three-tap polyphase box for odd sizes. One thread per
// destination texel, all four channels.
__global__ void k_fast_down(const MipJob *__restrict__ jobs, int njobs, long long units) {
    __shared__ float s_steps[256];
    load_steps(jobs, s_steps);
    __syncthreads();
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < units;
         u += (long long)gridDim.x * blockDim.x) {
        const MipJob &L = jobs[find_mip_job(jobs, njobs, u)];
        const int W = L.W, H = L.H;
        const float *src0 = L.src;
        const unsigned w = W / 2 > 1 ? (unsigned)W / 2 : 1u, h = H / 2 > 1 ? (unsigned)H / 2 : 1u;
        const size_t sn = (size_t)W * H, dn = (size_t)w * h;
        const unsigned t = (unsigned)(u - L.first_unit);  // levels hold < 2^32 texels: 32-bit division
        const unsigned x = t % w, y = t / w;
        float v[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const float *src = src0 + c * sn;
            float f;
            if (W == 1 || H == 1) {
                const unsigned n = w * h, i = (unsigned)t;
                const float *s = src + 2 * (size_t)i;
                if (((unsigned)W * (unsigned)H) & 1) {
                    const float scale = 1.0f / (2 * n + 1);
                    const float w0 = (float)(n - i), w1 = (float)(n - 0), w2 = (float)(1 + i);
                    f = scale * (w0 * s[0] + w1 * s[1] + w2 * s[2]);
                } else {
                    f = 0.5f * (s[0] + s[1]);
                }
            } else if ((W & 1) == 0 && (H & 1) == 0) {
                const float *s = src + (size_t)(2 * y) * W + 2 * x;
                f = 0.25f * (s[0] + s[1] + s[W] + s[W + 1]);
            } else if ((W & 1) && (H & 1)) {
                const float scale = 1.0f / (float)((unsigned)W * (unsigned)H);
                const float v0 = (float)(h - y), v1 = (float)(h - 0), v2 = (float)(1 + y);
                const float w0 = (float)(w - x), w1 = (float)(w - 0), w2 = (float)(1 + x);
                const float *s = src + (size_t)(2 * y) * W + 2 * x;
                float acc = 0.0f;
                acc += v0 * (w0 * s[0] + w1 * s[1] + w2 * s[2]);
                acc += v1 * (w0 * s[W] + w1 * s[W + 1] + w2 * s[W + 2]);
                acc += v2 * (w0 * s[2 * W] + w1 * s[2 * W + 1] + w2 * s[2 * W + 2]);
                f = acc * scale;
            } else if (W & 1) {
                const float scale = 1.0f / (float)(2 * (unsigned)W);
                const float w0 = (float)(w - x), w1 = (float)(w - 0), w2 = (float)(1 + x);
                const float *s = src + (size_t)(2 * y) * W + 2 * x;
                float acc = 0.0f;
                acc += w0 * (s[0] + s[W]);
                acc += w1 * (s[1] + s[W + 1]);
                acc += w2 * (s[2] + s[W + 2]);
                f = acc * scale;
            } else {
                const float scale = 1.0f / (float)(2 * (unsigned)H);
                const float v0 = (float)(h - y), v1 = (float)(h - 0), v2 = (float)(1 + y);
                const float *s = src + (size_t)(2 * y) * W + 2 * x;
                float acc = 0.0f;
                acc += v0 * (s[0] + s[1]);
                acc += v1 * (s[W] + s[W + 1]);
                acc += v2 * (s[2 * W] + s[2 * W + 1]);
                f = acc * scale;
            }
            v[c] = f;
            L.dst[c * dn + t] = f;
        }
        if (L.q_out) L.q_out[t] = quantize_bgra(v[0], v[1], v[2], v[3], L.xform, s_steps);
    }
}

// ---------------------------------------------------------------------------------------------
// Separable polyphase resize: FloatImage::resize 2D (src/nvimage/FloatImage.cpp:761-808) =
// applyKernelX over every source row into a (w' x H) plane, then applyKernelY (:1115-1176). Wrap
// modes follow FloatImage::index (src/nvimage/FloatImage.h:298-317). The weighted variants apply the
// alpha-weighted kernels (:1212-1281) to RGB. Channel arithmetic is the reference's, lane by lane:
// each sum starts at 0 and adds k * v in tap order, so levels are bit-identical.
__device__ __forceinline__ int wrap_index(int x, int w, int wm) {
    if (wm == 0) return x < 0 ? 0 : (x > w - 1 ? w - 1 : x);
    if (wm == 1) return x >= 0 ? x % w : (x + 1) % w + w - 1;
    if (w == 1) return 0;
    x = abs(x);
    while (x >= w) x = abs(w + w - x - 2);
    return x;
}

// Windows at the level's edges. A TMA box reads 0 where it reaches past the level; with the clamp
// and mirror wraps the texel that belongs there (the wrapped position) usually lies inside the same
// box, so the threads that read such a position read the wrapped one instead (a column or row index
// remap inside shared memory: no extra copy from global memory, no extra barrier). box_remap(x) is
// that index for position x of a box starting at b0; in_box checks, per tile, that the needed
// positions lo..hi (of a level of n) map into the box [b0, b0 + bn) with at most one reflection.
// Tiles where they do not (the repeat wrap, levels narrower than a window) are copied by the
// threads with the wrap applied.
__device__ __forceinline__ bool in_box(int lo, int hi, int b0, int bn, int n, int wrap) {
    if (lo >= 0 && hi < n) return true;
    if (wrap == 1) return false;
    if (wrap == 0) return true;  // clamp: 0 and n - 1 lie in the box whenever lo < 0 or hi >= n
    if (lo < 0 && (-lo >= n || -lo >= b0 + bn)) return false;
    if (hi >= n && (hi >= 2 * n - 1 || 2 * n - 2 - hi < b0)) return false;
    return true;
}
__device__ __forceinline__ int box_remap(int x, int b0, int n, int wrap) { return wrap_index(b0 + x, n, wrap) - b0; }

template <bool SRC_U8>
__device__ __forceinline__ float4 load_texel(const MipJob &L, size_t s, size_t sn) {
    if (SRC_U8) {
        const uint32_t p = __ldg(L.bgra8 + s);
        return make_float4(__ldg(L.lut + ((p >> 16) & 255)), __ldg(L.lut + ((p >> 8) & 255)), __ldg(L.lut + (p & 255)),
                           (float)(p >> 24) / 255.0f);
    }
    return make_float4(__ldg(L.src + s), __ldg(L.src + sn + s), __ldg(L.src + 2 * sn + s), __ldg(L.src + 3 * sn + s));
}

// One tap: sum += k * v for every channel (the weighted form weighs RGB by k * (alpha + 1/256)).
template <bool WEIGHTED>
__device__ __forceinline__ void tap(float4 &sum, float &norm, float k, const float4 v) {
    if (WEIGHTED) {
        const float wgt = k * (v.w + (1.0f / 256.0f));
        norm += wgt;
        sum.x += wgt * v.x; sum.y += wgt * v.y; sum.z += wgt * v.z;
        sum.w += k * v.w;
    } else {
        sum.x += k * v.x; sum.y += k * v.y; sum.z += k * v.z; sum.w += k * v.w;
    }
}

template <bool WEIGHTED>
__device__ __forceinline__ float4 finish(float4 sum, float norm) {
    if (WEIGHTED) { sum.x = sum.x / norm; sum.y = sum.y / norm; sum.z = sum.z / norm; }
    return sum;
}

__device__ __forceinline__ void store_texel(const MipJob &L, size_t o, size_t dn, float4 v, const float *s_steps) {
    L.dst[o] = v.x;
    L.dst[dn + o] = v.y;
    L.dst[2 * dn + o] = v.z;
    L.dst[3 * dn + o] = v.w;
    if (L.q_out) L.q_out[o] = quantize_bgra(v.x, v.y, v.z, v.w, L.xform, s_steps);
}

constexpr int PTW = 32;    // general kernel: output tile width (one warp lane per output column)
constexpr int PTH = 16;    // general kernel: output tile height
constexpr int PMAXW = 32;  // widest window handled
constexpr int PTHREADS = 256;
constexpr int PWARPS = PTHREADS / 32;

// General kernel, any scale and window (odd sizes, 1-wide axes). One CTA per PTW x PTH output
// tile: wrap maps for the tile's source rows and columns, the wrapped source window staged once as
// float4, X taps for every window row into a (rows x PTW) plane, then the Y taps.
template <bool WEIGHTED, bool SRC_U8>
__global__ void __launch_bounds__(PTHREADS) k_poly(const MipJob *__restrict__ jobs, int njobs) {
    extern __shared__ float4 sm4[];
    __shared__ float s_kx[PTW * PMAXW], s_ky[PTH * PMAXW], s_steps[256];
    __shared__ int s_lx[PTW], s_ly[PTH];
    load_steps(jobs, s_steps);
    const MipJob &L = jobs[find_mip_job(jobs, njobs, blockIdx.x)];
    const int lu = (int)(blockIdx.x - L.first_unit);
    const int ox0 = (lu % L.tiles_x) * PTW, oy0 = (lu / L.tiles_x) * PTH;
    const int tw = min(PTW, L.w - ox0), th = min(PTH, L.h - oy0);
    const int wsx = L.wsx, wsy = L.wsy;
    const int xlo = L.lx[ox0], xhi = L.lx[ox0 + tw - 1] + wsx - 1;
    const int ylo = L.ly[oy0], yhi = L.ly[oy0 + th - 1] + wsy - 1;
    const int rx = xhi - xlo + 1, ry = yhi - ylo + 1;
    float4 *s_in = sm4;                 // ry * rx
    float4 *s_tmp = s_in + ry * rx;     // ry * PTW
    int *s_col = reinterpret_cast<int *>(s_tmp + ry * PTW);  // rx
    int *s_row = s_col + rx;                                  // ry
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < tw * wsx; i += PTHREADS) s_kx[i] = L.kx[(size_t)ox0 * wsx + i];
    for (int i = tid; i < th * wsy; i += PTHREADS) s_ky[i] = L.ky[(size_t)oy0 * wsy + i];
    if (tid < tw) s_lx[tid] = L.lx[ox0 + tid] - xlo;
    if (tid < th) s_ly[tid] = L.ly[oy0 + tid] - ylo;
    for (int i = tid; i < rx; i += PTHREADS) s_col[i] = wrap_index(xlo + i, L.W, L.wrap);
    for (int i = tid; i < ry; i += PTHREADS) s_row[i] = wrap_index(ylo + i, L.H, L.wrap);
    __syncthreads();

    const size_t sn = (size_t)L.W * L.H;
    for (int r = warp; r < ry; r += PWARPS) {
        const size_t rowoff = (size_t)s_row[r] * L.W;
        for (int x = lane; x < rx; x += 32) s_in[r * rx + x] = load_texel<SRC_U8>(L, rowoff + s_col[x], sn);
    }
    __syncthreads();

    if (lane < tw) {  // X taps: one lane per output column, warps over the window rows
        const float *k = s_kx + lane * wsx;
        const int off = s_lx[lane];
        for (int r = warp; r < ry; r += PWARPS) {
            const float4 *row = s_in + r * rx + off;
            float4 sum = make_float4(0, 0, 0, 0);
            float norm = 0;
            for (int j = 0; j < wsx; j++) tap<WEIGHTED>(sum, norm, k[j], row[j]);
            s_tmp[r * PTW + lane] = finish<WEIGHTED>(sum, norm);
        }
    }
    __syncthreads();

    if (lane < tw) {  // Y taps: one lane per output column, warps over the output rows
        const size_t dn = (size_t)L.w * L.h;
        for (int y = warp; y < th; y += PWARPS) {
            const float *k = s_ky + y * wsy;
            const float4 *col = s_tmp + s_ly[y] * PTW + lane;
            float4 sum = make_float4(0, 0, 0, 0);
            float norm = 0;
            for (int j = 0; j < wsy; j++) tap<WEIGHTED>(sum, norm, k[j], col[j * PTW]);
            store_texel(L, (size_t)(oy0 + y) * L.w + ox0 + lane, dn, finish<WEIGHTED>(sum, norm), s_steps);
        }
    }
}

// Exact 2:1 kernel (both axes halve and every output has the same taps: power-of-two chains).
// One CTA per tile of 32 output columns x TH output rows (TH = the job's `strip`): the wrapped
// source window (62 + WS columns x 2 TH - 2 + WS rows) is staged once in shared memory as float4,
// even and odd columns in separate halves so the stride-2 tap reads of a warp are consecutive;
// then every window row's X taps go to a (rows x 32) plane, then the Y taps. Every item of both
// passes is independent, sums start at 0 and take their taps in order, as applyKernelX/Y do
// (src/nvimage/FloatImage.cpp:1115-1176). The taps are the same for every output, so both
// weight vectors live in registers.
template <int WS>
struct Tile2x {
    static_assert(WS % 2 == 1, "odd windows");
    static constexpr int TW = 32;
    static constexpr int RW = 2 * (TW - 1) + WS;                       // source columns of a tile
    static constexpr int HALF = ((RW + 1) / 2 + 3) / 8 * 8 + 4;         // >= RW/2, = 4 mod 8: conflict-free stores
    static constexpr int ROW = 2 * HALF;                                // float4 per staged row
    static __host__ __device__ constexpr int rows(int th) { return 2 * (th - 1) + WS; }
    static __host__ __device__ constexpr size_t smem(int th) {
        return ((size_t)rows(th) * ROW + (size_t)rows(th) * TW) * sizeof(float4);
    }
};

// A source texel as loaded (BGRA8 word or four FP32 planes), converted to float4 when staged.
template <bool SRC_U8> struct RawTexel;
template <> struct RawTexel<true> { uint32_t v; };
template <> struct RawTexel<false> { float4 v; };

template <bool SRC_U8>
__device__ __forceinline__ void fetch_raw(const MipJob &L, size_t s, size_t sn, RawTexel<SRC_U8> &r) {
    if constexpr (SRC_U8) r.v = __ldg(L.bgra8 + s);
    else r.v = make_float4(__ldg(L.src + s), __ldg(L.src + sn + s), __ldg(L.src + 2 * sn + s), __ldg(L.src + 3 * sn + s));
}

template <int WS, bool WEIGHTED, bool SRC_U8>
__global__ void __launch_bounds__(512, 2) k_tile2x(const MipJob *__restrict__ jobs, int njobs) {
    using P = Tile2x<WS>;
    constexpr int TW = P::TW, RW = P::RW, HALF = P::HALF, ROW = P::ROW;
    extern __shared__ float4 sm4[];
    __shared__ float s_steps[256];
    __shared__ float s_lut[SRC_U8 ? 512 : 1];
    __shared__ uint8_t s_buckets[kSrgbBuckets];
    const MipJob &L = jobs[find_mip_job(jobs, njobs, blockIdx.x)];
    const int tid = threadIdx.x, nt = blockDim.x;
    const bool srgb = L.q_out && L.xform == 2;
    if (L.q_out) {
        for (int i = tid; i < 256; i += nt) s_steps[i] = __ldg(L.steps + i);
        if (srgb) {
            const uint32_t *b = reinterpret_cast<const uint32_t *>(L.steps + 256);
            for (int i = tid; i < kSrgbBuckets / 4; i += nt) reinterpret_cast<uint32_t *>(s_buckets)[i] = __ldg(b + i);
        }
    }
    if constexpr (SRC_U8)
        for (int i = tid; i < 512; i += nt) s_lut[i] = __ldg(L.lut + i);
    const int th = L.strip;
    const int rh = P::rows(th);
    const unsigned lu = (unsigned)((long long)blockIdx.x - L.first_unit), tx = (unsigned)L.tiles_x;
    const int x0 = (int)(lu % tx) * TW, y0 = (int)(lu / tx) * th;
    const int W = L.W, H = L.H, w = L.w, h = L.h, wrap = L.wrap;
    const int c0 = 2 * x0 + L.cx, r0 = 2 * y0 + L.cy;
    const bool cols_in = c0 >= 0 && c0 + RW <= W, rows_in = r0 >= 0 && r0 + rh <= H;
    const size_t sn = (size_t)W * H, dn = (size_t)w * h;
    float4 *region = sm4;                       // rh x ROW
    float4 *tmp = sm4 + (size_t)rh * ROW;       // rh x TW
    __syncthreads();

    // stage the wrapped source window: a warp per row, lanes over consecutive columns; the next
    // row's loads are in flight while this row is converted and stored
    const int lane = tid & 31, nwarps = nt >> 5;
    constexpr int CPL = (RW + 31) / 32;  // columns per lane
    auto fetch = [&](int r, RawTexel<SRC_U8> (&raw)[CPL]) {
        const size_t rowoff = (size_t)(rows_in ? r0 + r : wrap_index(r0 + r, H, wrap)) * W;
#pragma unroll
        for (int k = 0; k < CPL; k++) {
            const int c = lane + 32 * k;
            if (c < RW) fetch_raw<SRC_U8>(L, rowoff + (cols_in ? c0 + c : wrap_index(c0 + c, W, wrap)), sn, raw[k]);
        }
    };
    // rows in flight ahead of the one being stored: two for BGRA8 words, one for FP32 texels
    constexpr int AHEAD = SRC_U8 ? 2 : 1;
    RawTexel<SRC_U8> cur[CPL], nxt[CPL], nxt2[CPL];
    int r = tid >> 5;
    if (r < rh) fetch(r, cur);
    if (AHEAD > 1 && r + nwarps < rh) fetch(r + nwarps, nxt);
    for (; r < rh; r += nwarps) {
        if (AHEAD > 1) {
            if (r + 2 * nwarps < rh) fetch(r + 2 * nwarps, nxt2);
        } else if (r + nwarps < rh) {
            fetch(r + nwarps, nxt);
        }
        float4 *dst = region + r * ROW;
#pragma unroll
        for (int k = 0; k < CPL; k++) {
            const int c = lane + 32 * k;
            if (c < RW) {
                float4 v;
                if constexpr (SRC_U8) {
                    const uint32_t q = cur[k].v;
                    v = make_float4(s_lut[(q >> 16) & 255], s_lut[(q >> 8) & 255], s_lut[q & 255], s_lut[256 + (q >> 24)]);
                } else {
                    v = cur[k].v;
                }
                dst[(c & 1) * HALF + (c >> 1)] = v;
            }
        }
#pragma unroll
        for (int k = 0; k < CPL; k++) {
            cur[k] = nxt[k];
            if (AHEAD > 1) nxt[k] = nxt2[k];
        }
    }
    __syncthreads();

    // the taps (the same for every output), loaded after the staging to keep its registers free
    float kx[WS], ky[WS];
#pragma unroll
    for (int j = 0; j < WS; j++) { kx[j] = __ldg(L.kx + j); ky[j] = __ldg(L.ky + j); }

    // X taps of every window row: output column x (= lane) reads source columns 2x .. 2x + WS - 1
    // (unweighted: two channels per packed add, the same roundings as the scalar taps)
    for (int r = tid >> 5; r < rh; r += nwarps) {
        const float4 *row = region + r * ROW + lane;
        if constexpr (WEIGHTED) {
            float4 sum = make_float4(0, 0, 0, 0);
            float norm = 0;
#pragma unroll
            for (int j = 0; j < WS; j++) tap<WEIGHTED>(sum, norm, kx[j], row[(j & 1) * HALF + (j >> 1)]);
            tmp[r * TW + lane] = finish<WEIGHTED>(sum, norm);
        } else {
            F4x2 sum{0, 0};
#pragma unroll
            for (int j = 0; j < WS; j++) tap2(sum, kx[j], row[(j & 1) * HALF + (j >> 1)]);
            tmp[r * TW + lane] = f4_of(sum);
        }
    }
    __syncthreads();

    // Y taps: output row y reads window rows 2y .. 2y + WS - 1
    if (x0 + lane >= w) return;
    const int ty = min(th, h - y0);
    float *const dst = L.dst + (size_t)y0 * w + x0 + lane;
    uint32_t *const qd = L.q_out ? L.q_out + (size_t)y0 * w + x0 + lane : nullptr;
    for (int y = tid >> 5; y < ty; y += nwarps) {
        const float4 *col = tmp + (2 * y) * TW + lane;
        float4 v;
        if constexpr (WEIGHTED) {
            float4 sum = make_float4(0, 0, 0, 0);
            float norm = 0;
#pragma unroll
            for (int j = 0; j < WS; j++) tap<WEIGHTED>(sum, norm, ky[j], col[j * TW]);
            v = finish<WEIGHTED>(sum, norm);
        } else {
            F4x2 sum{0, 0};
#pragma unroll
            for (int j = 0; j < WS; j++) tap2(sum, ky[j], col[j * TW]);
            v = f4_of(sum);
        }
        float *const d = dst + (size_t)y * w;
        d[0] = v.x;
        d[dn] = v.y;
        d[2 * dn] = v.z;
        d[3 * dn] = v.w;
        if (qd) qd[(size_t)y * w] = srgb ? quantize_srgb_bgra(v, s_steps, s_buckets) : quantize_bgra(v.x, v.y, v.z, v.w, L.xform, s_steps);
    }
}

// 2:1 steps that read the BGRA8 input (the first step of a chain): a persistent kernel, one
// 1024-thread CTA per SM walking 64 x 16 output tiles with one barrier per tile. A tile's source
// window of BGRA8 words is copied into shared memory with cp.async while the previous tile is
// filtered. Each warp then takes whole source rows: it converts the row's words through the input
// table into its own scratch row, as float4 columns split by column mod 4 (a lane that computes two
// adjacent outputs then reads consecutive float4 at every tap, and each texel it loads serves both
// outputs), and writes the row's X taps to the tile's X plane. In the same phase the other warps run
// the Y taps of the previous tile from the other X plane, two output rows of one column per thread.
// Every sum starts at 0 and takes its taps in window order, as in applyKernelX/Y
// (src/nvimage/FloatImage.cpp:1115-1176), so the levels equal k_tile2x's. The input table, the
// quantiser tables and the taps are the same for every job of a launch (the host groups by them).
template <int WS>
struct TileU8 {
    static constexpr int TW = 64, TH = 16, WARPS = 32;
    static constexpr int D = WS == 3 ? 0 : 3;            // window start of output column 0, mod 4 (-5, -1, 0)
    static constexpr int RW = 2 * (TW - 1) + WS;          // source columns of a tile
    static constexpr int NC = (D + RW + 3) / 4 * 4;       // staged columns, from a multiple of 4
    static constexpr int QP = (NC / 4 + 1) / 8 * 8 + 6;   // float4 per column class of a scratch row,
                                                          // = 6 mod 8: conflict-free class-split stores
    static constexpr int ROWS = 2 * (TH - 1) + WS;        // source rows of a tile
    static constexpr size_t RAW_WORDS = (size_t)ROWS * NC;
    static constexpr size_t XPLANE = (size_t)ROWS * TW;   // float4
    static constexpr size_t smem() { return (2 * XPLANE + (size_t)WARPS * 4 * QP) * 16 + 2 * RAW_WORDS * 4; }
};

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

struct TilePos {
    const MipJob *L;
    int x0, y0;   // first output column / row
    int a0, r0;   // first staged source column (a multiple of 4) / row, before wrapping
    bool inner;   // window inside the level, rows 16-byte aligned: whole-vector copies
};

template <int WS>
__device__ __forceinline__ TilePos tile_u8_pos(const MipJob *__restrict__ jobs, int njobs, long long u) {
    using P = TileU8<WS>;
    const MipJob &L = jobs[find_mip_job(jobs, njobs, u)];
    const unsigned lu = (unsigned)(u - L.first_unit), tx = (unsigned)L.tiles_x;  // 32-bit division
    TilePos p;
    p.L = &L;
    p.x0 = (int)(lu % tx) * P::TW;
    p.y0 = (int)(lu / tx) * P::TH;
    p.a0 = 2 * p.x0 + L.cx - P::D;
    p.r0 = 2 * p.y0 + L.cy;
    p.inner = p.a0 >= 0 && p.a0 + P::NC <= L.W && p.r0 >= 0 && p.r0 + P::ROWS <= L.H && (L.W & 3) == 0 &&
              ((uintptr_t)L.bgra8 & 15) == 0;
    return p;
}

// Issues the copies of a tile's source window (ROWS x NC words, wrapped at the level's edges).
template <int WS>
__device__ __forceinline__ void tile_u8_fetch(const TilePos &p, uint32_t *raw) {
    using P = TileU8<WS>;
    const MipJob &L = *p.L;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (p.inner) {
        constexpr int CH = P::NC / 4;
        for (int i = tid; i < P::ROWS * CH; i += nt) {
            const int r = i / CH, k = i - r * CH;
            cp_async16(raw + r * P::NC + 4 * k, L.bgra8 + (size_t)(p.r0 + r) * L.W + p.a0 + 4 * k);
        }
    } else {
        for (int i = tid; i < P::ROWS * P::NC; i += nt) {
            const int r = i / P::NC, c = i - r * P::NC;
            const int sy = wrap_index(p.r0 + r, L.H, L.wrap), sx = wrap_index(p.a0 + c, L.W, L.wrap);
            cp_async4(raw + i, L.bgra8 + (size_t)sy * L.W + sx);
        }
    }
    cp_async_commit();
}

template <int WS, bool WEIGHTED>
__global__ void __launch_bounds__(1024, 1) k_tile2x_u8(const MipJob *__restrict__ jobs, int njobs, long long units) {
    using P = TileU8<WS>;
    constexpr int TW = P::TW, TH = P::TH, D = P::D, NC = P::NC, QP = P::QP, ROWS = P::ROWS;
    extern __shared__ float4 sm4[];
    __shared__ float s_steps[256];
    __shared__ float s_lut[512];
    __shared__ uint8_t s_buckets[kSrgbBuckets];
    __shared__ float s_ky[WS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float4 *const xplane0 = sm4;                                   // 2 x ROWS x TW
    float4 *const scratch = sm4 + 2 * P::XPLANE + warp * 4 * QP;   // this warp's converted row
    uint32_t *const raw0 = reinterpret_cast<uint32_t *>(sm4 + 2 * P::XPLANE + P::WARPS * 4 * QP);  // 2 x ROWS x NC
    const long long g = gridDim.x;
    if (blockDim.x != 32 * P::WARPS || (long long)blockIdx.x >= units) return;

    // tables and taps, shared by every job of the launch
    const MipJob &J0 = jobs[0];
    for (int i = tid; i < 512; i += blockDim.x) s_lut[i] = __ldg(J0.lut + i);
    if (tid < WS) s_ky[tid] = __ldg(J0.ky + tid);
    if (J0.steps) {
        for (int i = tid; i < 256; i += blockDim.x) s_steps[i] = __ldg(J0.steps + i);
        const uint32_t *b = reinterpret_cast<const uint32_t *>(J0.steps + 256);
        for (int i = tid; i < kSrgbBuckets / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(s_buckets)[i] = __ldg(b + i);
    }
    float kx[WS];
#pragma unroll
    for (int j = 0; j < WS; j++) kx[j] = __ldg(J0.kx + j);

    // iteration i converts and X-filters tile blockIdx + i g and Y-filters tile blockIdx + (i - 1) g
    const long long n = (units - blockIdx.x + g - 1) / g;
    tile_u8_fetch<WS>(tile_u8_pos<WS>(jobs, njobs, blockIdx.x), raw0);
    for (long long i = 0; i <= n; i++) {
        cp_async_wait<0>();
        __syncthreads();  // tile i's words are in; iteration i - 1 is done with raw[(i + 1) % 2] and the X planes
        if (i + 1 < n) tile_u8_fetch<WS>(tile_u8_pos<WS>(jobs, njobs, blockIdx.x + (i + 1) * g), raw0 + ((i + 1) & 1) * P::RAW_WORDS);
        const uint32_t *const raw = raw0 + (i & 1) * P::RAW_WORDS;
        float4 *const xp = xplane0 + (i & 1) * P::XPLANE;
        const float4 *const yp = xplane0 + ((i + 1) & 1) * P::XPLANE;
        const int nx = i < n ? ROWS : 0, ny = i > 0 ? TH : 0;
        for (int item = warp; item < nx + ny; item += P::WARPS) {
            if (item < nx) {
                // convert source row `item`: staged column c -> class c % 4, slot c / 4
                const int r = item;
                __syncwarp();  // the warp's previous row has been read
#pragma unroll
                for (int c = lane; c < NC; c += 32) {
                    const uint32_t q = raw[r * NC + c];
                    scratch[(c & 3) * QP + (c >> 2)] =
                        make_float4(s_lut[(q >> 16) & 255], s_lut[(q >> 8) & 255], s_lut[q & 255], s_lut[256 + (q >> 24)]);
                }
                __syncwarp();
                // X taps: lane -> output columns 2 lane, 2 lane + 1 = staged columns D + 4 lane + t,
                // t in [0, WS) and [2, WS + 2)
                if constexpr (WEIGHTED) {
                    float4 s0 = make_float4(0, 0, 0, 0), s1 = s0;
                    float n0 = 0, n1 = 0;
#pragma unroll
                    for (int t = 0; t < WS + 2; t++) {
                        const float4 v = scratch[((D + t) & 3) * QP + ((D + t) >> 2) + lane];
                        if (t < WS) tap<WEIGHTED>(s0, n0, kx[t], v);
                        if (t >= 2) tap<WEIGHTED>(s1, n1, kx[t - 2], v);
                    }
                    xp[r * TW + 2 * lane] = finish<WEIGHTED>(s0, n0);
                    xp[r * TW + 2 * lane + 1] = finish<WEIGHTED>(s1, n1);
                } else {
                    // two channels per packed add, the same roundings as the scalar taps
                    F4x2 s0{0, 0}, s1{0, 0};
#pragma unroll
                    for (int t = 0; t < WS + 2; t++) {
                        const float4 v = scratch[((D + t) & 3) * QP + ((D + t) >> 2) + lane];
                        if (t < WS) tap2(s0, kx[t], v);
                        if (t >= 2) tap2(s1, kx[t - 2], v);
                    }
                    xp[r * TW + 2 * lane] = f4_of(s0);
                    xp[r * TW + 2 * lane + 1] = f4_of(s1);
                }
            } else {
                // Y taps of tile i - 1: output rows 2 p, 2 p + 1 (p = k / 2) of column 32 (k % 2) + lane
                // read X rows 4 p + t, t in [0, WS) and [2, WS + 2)
                const int k = item - nx, p = k >> 1, x = 32 * (k & 1) + lane;
                const float4 *const col = yp + (4 * p) * TW + x;
                float4 s0 = make_float4(0, 0, 0, 0), s1 = s0;
                float n0 = 0, n1 = 0;
                if constexpr (WEIGHTED) {
#pragma unroll
                    for (int t = 0; t < WS + 2; t++) {
                        const float4 v = col[t * TW];
                        if (t < WS) tap<WEIGHTED>(s0, n0, s_ky[t], v);
                        if (t >= 2) tap<WEIGHTED>(s1, n1, s_ky[t - 2], v);
                    }
                } else {
                    F4x2 p0{0, 0}, p1{0, 0};
#pragma unroll
                    for (int t = 0; t < WS + 2; t++) {
                        const float4 v = col[t * TW];
                        if (t < WS) tap2(p0, s_ky[t], v);
                        if (t >= 2) tap2(p1, s_ky[t - 2], v);
                    }
                    s0 = f4_of(p0);
                    s1 = f4_of(p1);
                }
                const TilePos pos = tile_u8_pos<WS>(jobs, njobs, blockIdx.x + (i - 1) * g);
                const MipJob &L = *pos.L;
                const int w = L.w, h = L.h, gx = pos.x0 + x, gy = pos.y0 + 2 * p;
                if (gx >= w) continue;
                const size_t dn = (size_t)w * h;
                const bool srgb = L.q_out && L.xform == 2;
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    if (gy + e >= h) break;
                    const float4 v = e == 0 ? finish<WEIGHTED>(s0, n0) : finish<WEIGHTED>(s1, n1);
                    const size_t o = (size_t)(gy + e) * w + gx;
                    L.dst[o] = v.x;
                    L.dst[dn + o] = v.y;
                    L.dst[2 * dn + o] = v.z;
                    L.dst[3 * dn + o] = v.w;
                    if (L.q_out)
                        L.q_out[o] = srgb ? quantize_srgb_bgra(v, s_steps, s_buckets) : quantize_bgra(v.x, v.y, v.z, v.w, L.xform, s_steps);
                }
            }
        }
    }
}

// The thread that issues the FP32 tile kernel's TMA loads: lane 0 of the last warp, which has no
// filter item. It acquires a job's tensor map once, before its first load through it (`fenced`).
__device__ __forceinline__ bool tma_issuer() { return threadIdx.x == blockDim.x - 32; }

__device__ __forceinline__ void tma_tile(const MipJob &L, const MipJob *&fenced, void *dst, uint32_t bytes, int x, int y,
                                         uint64_t *bar) {
    if (fenced != &L) {
        tensormap_acquire(&L.map);
        fenced = &L;
    }
    mbar_expect_tx(bar, bytes);
    tma_load_3d(dst, &L.map, x, y, 0, bar);
}

// 2:1 steps between FP32 levels (level 2 on), unweighted: persistent like k_tile2x_u8, one
// 1024-thread CTA per SM walking 32 x TH output tiles (TH = the job's strip, at most 16) with one
// barrier per tile, the X taps of tile i beside the Y taps of tile i - 1. A tile's source window, four
// planes of ROWS x NC floats, is one TMA box of the level's 3-D tensor map (x, y, plane), loaded into
// one of NBUF buffers while the tiles before it are filtered (a third buffer, for two boxes in flight,
// measured slower: its shared memory and the extra state cost more than the hidden latency gave).
// Positions of an edge box outside the level read 0; the half-warp that filters a row first fills them
// from their wrapped positions in the same box (box_remap). Windows that cannot be remapped, and
// levels without a tensor map, are copied by the threads (cp.async) with the wrap applied, into the
// same layout. The X pass reads the planes directly: a half-warp per source row, each lane two
// adjacent outputs from NV consecutive float4 of each plane (conflict-free). Sums start at 0 and take their taps in window order as in
// applyKernelX/Y (src/nvimage/FloatImage.cpp:1115-1176), so the levels equal k_tile2x's.
template <int WS>
struct TileF32 {
    static constexpr int TW = 32, TH = 16, WARPS = 32;
    static constexpr int D = WS == 3 ? 0 : 3;                    // window start of output column 0, mod 4
    static constexpr int RW = 2 * (TW - 1) + WS;                 // source columns of a tile
    static constexpr int NC = (D + RW + 3) / 4 * 4;              // staged columns, from a multiple of 4
    static constexpr int NV = (D + WS + 1) / 4 + 1;              // float4 per plane under a lane's two outputs
    static_assert(4 * (TW / 2 - 1) + 4 * NV <= NC, "X reads stay inside the staged row");
    static constexpr int ROWS = 2 * (TH - 1) + WS;               // source rows of the tallest tile
    static constexpr int RAW = (4 * ROWS * NC + 31) / 32 * 32;   // floats per window buffer (128-byte multiple)
    static constexpr int NBUF = 2;                               // window buffers
    static constexpr int XPLANE = ROWS * TW;                     // float4
    static constexpr size_t smem() { return 128 + (size_t)NBUF * RAW * 4 + (size_t)2 * XPLANE * 16; }
    static __host__ __device__ constexpr int rows(int th) { return 2 * (th - 1) + WS; }
};

struct TileF32Pos {
    const MipJob *L;
    int x0, y0;    // first output column / row
    int a0, r0;    // first staged source column (a multiple of 4) / row, before wrapping
    int th, rows;  // output rows of the tile (its job's strip) and source rows of its window
    bool tma;      // one TMA box (the job has a tensor map, and the edges can be remapped)
    bool remap;    // tma, and the box reaches past the level's edges: edge rows fixed in place
};

template <int WS>
__device__ __forceinline__ TileF32Pos tile_f32_pos(const MipJob *__restrict__ jobs, int njobs, long long u) {
    using P = TileF32<WS>;
    const MipJob &L = jobs[find_mip_job(jobs, njobs, u)];
    const unsigned lu = (unsigned)(u - L.first_unit), tx = (unsigned)L.tiles_x;  // 32-bit division
    TileF32Pos p;
    p.L = &L;
    p.th = L.strip;
    p.rows = P::rows(p.th);
    p.x0 = (int)(lu % tx) * P::TW;
    p.y0 = (int)(lu / tx) * p.th;
    p.a0 = 2 * p.x0 + L.cx - P::D;
    p.r0 = 2 * p.y0 + L.cy;
    const bool edge = p.a0 < 0 || p.a0 + P::NC > L.W || p.r0 < 0 || p.r0 + p.rows > L.H;
    p.tma = L.tma && (!edge || (in_box(p.a0 + P::D, p.a0 + P::D + P::RW - 1, p.a0, P::NC, L.W, L.wrap) &&
                                in_box(p.r0, p.r0 + p.rows - 1, p.r0, p.rows, L.H, L.wrap)));
    p.remap = p.tma && edge;
    return p;
}

// Issues the copies of a tile's source window into `raw` (plane c, row r at (c rows + r) NC).
template <int WS>
__device__ __forceinline__ void tile_f32_fetch(const TileF32Pos &p, float *raw, uint64_t *bar, const MipJob *&fenced) {
    using P = TileF32<WS>;
    const MipJob &L = *p.L;
    if (p.tma) {
        if (tma_issuer()) tma_tile(L, fenced, raw, (uint32_t)(4 * p.rows * P::NC * 4), p.a0, p.r0, bar);
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t sn = (size_t)L.W * L.H;
    for (int row = warp; row < 4 * p.rows; row += P::WARPS) {
        const int c = row / p.rows, r = row - c * p.rows;
        const float *srow = L.src + c * sn + (size_t)wrap_index(p.r0 + r, L.H, L.wrap) * L.W;
        float *drow = raw + (size_t)row * P::NC;
        for (int k = lane; k < P::NC; k += 32) cp_async4(drow + k, srow + wrap_index(p.a0 + k, L.W, L.wrap));
    }
    cp_async_commit();
}

template <int WS>
__global__ void __launch_bounds__(1024, 1) k_tile2x_f32(const MipJob *__restrict__ jobs, int njobs, long long units) {
    using P = TileF32<WS>;
    constexpr int TW = P::TW, D = P::D, NC = P::NC, NV = P::NV;
    extern __shared__ float4 sm4[];
    __shared__ float s_steps[256];
    __shared__ uint8_t s_buckets[kSrgbBuckets];
    __shared__ float s_ky[WS];
    __shared__ uint64_t s_bar[TileF32<WS>::NBUF];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float *const raw0 = reinterpret_cast<float *>(sm4 + ((128 - (smem_u32(sm4) & 127)) & 127) / 16);  // NBUF x RAW
    float4 *const xplane0 = reinterpret_cast<float4 *>(raw0 + P::NBUF * P::RAW);                     // 2 x XPLANE
    constexpr int NB = P::NBUF;
    const long long g = gridDim.x;
    if (blockDim.x != 32 * P::WARPS || (long long)blockIdx.x >= units) return;
    const int polls = g_mip_wait_polls;
    if (tid == 0) {
        for (int k = 0; k < NB; k++) mbar_init(&s_bar[k], 1);
        fence_barrier_init();
    }

    // quantiser tables and taps, shared by every job of the launch
    const MipJob &J0 = jobs[0];
    if (tid < WS) s_ky[tid] = __ldg(J0.ky + tid);
    if (J0.steps) {
        for (int i = tid; i < 256; i += blockDim.x) s_steps[i] = __ldg(J0.steps + i);
        const uint32_t *b = reinterpret_cast<const uint32_t *>(J0.steps + 256);
        for (int i = tid; i < kSrgbBuckets / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(s_buckets)[i] = __ldg(b + i);
    }
    float kx[WS];
#pragma unroll
    for (int j = 0; j < WS; j++) kx[j] = __ldg(J0.kx + j);
    __syncthreads();  // barriers initialised before any thread waits on them

    // iteration i X-filters tile blockIdx + i g (t0, window in buffer i % NB) and Y-filters tile
    // blockIdx + (i - 1) g (prev); the boxes of the next AHEAD tiles (t1, t2) are in flight meanwhile.
    // Buffer k's barrier completes once per box loaded into it (phase bit k of ph).
    constexpr int AHEAD = NB - 1;
    const long long n = (units - blockIdx.x + g - 1) / g;
    TileF32Pos t0 = tile_f32_pos<WS>(jobs, njobs, blockIdx.x), t1 = t0, prev = t0;
    const MipJob *fenced = nullptr;
    uint32_t ph = 0;
    auto fetch = [&](const TileF32Pos &t, int k) { tile_f32_fetch<WS>(t, raw0 + k * P::RAW, &s_bar[k], fenced); };
    fetch(t0, 0);
    if (AHEAD > 1 && n > 1) {
        t1 = tile_f32_pos<WS>(jobs, njobs, blockIdx.x + g);
        fetch(t1, 1);
    }
    for (long long i = 0; i <= n; i++) {
        const int b = (int)(i % NB), bx = (int)(i & 1);
        bool ok = true;
        if (i < n) {
            cp_async_wait<0>();
            if (t0.tma) {
                // one thread polls the barrier; the others wait at the CTA barrier below, which
                // makes the box visible to them and keeps them off the issue slots meanwhile
                if (tma_issuer()) ok = mbar_wait(&s_bar[b], (ph >> b) & 1, polls);
                ph ^= 1u << b;
            }
        }
        if (!__syncthreads_and(ok)) {
            // a wait ran out: record it, let the boxes in flight (tile i, and i + 1 with two ahead)
            // land, and leave
            if (tma_issuer()) {
                atomicOr(&g_mip_status, 1u);
                mbar_wait(&s_bar[b], ((ph >> b) & 1) ^ 1, kMipWaitPolls);
                const int b1 = (int)((i + 1) % NB);
                if (AHEAD > 1 && i + 1 < n && t1.tma) mbar_wait(&s_bar[b1], (ph >> b1) & 1, kMipWaitPolls);
            }
            return;
        }
        TileF32Pos t2 = t1;
        if (i + AHEAD < n) {
            t2 = tile_f32_pos<WS>(jobs, njobs, blockIdx.x + (i + AHEAD) * g);
            fetch(t2, (int)((i + AHEAD) % NB));
        }
        const TileF32Pos &cur = t0;
        const float *const raw = raw0 + b * P::RAW;
        float4 *const xp = xplane0 + bx * P::XPLANE;
        const float4 *const yp = xplane0 + (1 - bx) * P::XPLANE;
        const int nx = i < n ? (cur.rows + 1) / 2 : 0, ny = i > 0 ? prev.th / 2 : 0;
        for (int item = warp; item < nx + ny; item += P::WARPS) {
            if (item < nx) {
                // X taps of source rows 2 item (lanes 0-15) and 2 item + 1 (lanes 16-31): lane l -> output
                // columns 2 l, 2 l + 1 = staged columns D + 4 l + t, t in [0, WS) and [2, WS + 2)
                const int r = 2 * item + (lane >> 4), l = lane & 15;
                if (cur.remap) {
                    // an edge box: the half-warp fills its row's positions outside the level from
                    // their wrapped positions (inside the level, so read-only for every lane)
                    if (r < cur.rows) {
                        const MipJob &L = *cur.L;
                        const int rr = box_remap(r, cur.r0, L.H, L.wrap);
                        const bool row_out = rr != r;
#pragma unroll 1
                        for (int c = 0; c < 4; c++) {
                            float *row = const_cast<float *>(raw) + ((size_t)c * cur.rows + r) * NC;
                            const float *from = raw + ((size_t)c * cur.rows + rr) * NC;
                            for (int k = l; k < NC; k += 16) {
                                const int sx = cur.a0 + k;
                                if (row_out || sx < 0 || sx >= L.W) {
                                    const int kk = box_remap(k, cur.a0, L.W, L.wrap);
                                    if (kk >= 0 && kk < NC) row[k] = from[kk];  // outside the box: feeds no output
                                }
                            }
                        }
                        fence_async_smem();  // a later TMA box overwrites this row
                    }
                    __syncwarp();
                }
                if (r < cur.rows) {
                    float o0[4], o1[4];
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        const float4 *src = reinterpret_cast<const float4 *>(raw + ((size_t)c * cur.rows + r) * NC) + l;
                        float v[4 * NV];
#pragma unroll
                        for (int k = 0; k < NV; k++) {
                            const float4 q = src[k];
                            v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
                        }
                        f32x2 sum = f2_pack(0.0f, 0.0f);
#pragma unroll
                        for (int t = 0; t < WS; t++) sum = f2_add(sum, f2_pack(kx[t] * v[D + t], kx[t] * v[D + 2 + t]));
                        f2_unpack(sum, o0[c], o1[c]);
                    }
                    xp[r * TW + 2 * l] = make_float4(o0[0], o0[1], o0[2], o0[3]);
                    xp[r * TW + 2 * l + 1] = make_float4(o1[0], o1[1], o1[2], o1[3]);
                }
            } else {
                // Y taps of tile i - 1: output rows 2 q, 2 q + 1 of column `lane` read X rows 4 q + t,
                // t in [0, WS) and [2, WS + 2)
                const int q = item - nx;
                const float4 *const col = yp + (4 * q) * TW + lane;
                F4x2 p0{0, 0}, p1{0, 0};
#pragma unroll
                for (int t = 0; t < WS + 2; t++) {
                    const float4 v = col[t * TW];
                    if (t < WS) tap2(p0, s_ky[t], v);
                    if (t >= 2) tap2(p1, s_ky[t - 2], v);
                }
                const MipJob &L = *prev.L;
                const int w = L.w, h = L.h, gx = prev.x0 + lane, gy = prev.y0 + 2 * q;
                if (gx >= w) continue;
                const size_t dn = (size_t)w * h;
                const bool srgb = L.q_out && L.xform == 2;
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    if (gy + e >= h) break;
                    const float4 v = f4_of(e == 0 ? p0 : p1);
                    const size_t o = (size_t)(gy + e) * w + gx;
                    L.dst[o] = v.x;
                    L.dst[dn + o] = v.y;
                    L.dst[2 * dn + o] = v.z;
                    L.dst[3 * dn + o] = v.w;
                    if (L.q_out)
                        L.q_out[o] = srgb ? quantize_srgb_bgra(v, s_steps, s_buckets) : quantize_bgra(v.x, v.y, v.z, v.w, L.xform, s_steps);
                }
            }
        }
        prev = t0;
        if (AHEAD > 1) {
            t0 = t1;
            t1 = t2;
        } else {
            t0 = t2;
        }
    }
}

// Chain tails: once a texture's level is small (at most TAIL_MAX texels), one CTA finishes every
// remaining level in shared memory, one level after the other, instead of one latency-bound
// launch per tiny level. Levels are planar FP32 in shared memory; each polyphase step runs the
// X pass over every source row into a plane, then the Y pass (applyKernelX / applyKernelY order),
// box steps use the fastDownSample formulas; every level is also written out. The jobs of a tail
// are consecutive in the list: the first carries the number of levels in tiles_x, and all carry
// the chain's index in first_unit.
constexpr int TAIL_MAX = 4096;
constexpr int TAIL_TAB = 12288;  // words of shared memory for the levels' weights and window starts

__device__ __forceinline__ float fast_box_texel(const float *src, int W, int H, unsigned w, unsigned h, unsigned t) {
    const unsigned x = t % w, y = t / w;
    if (W == 1 || H == 1) {
        const unsigned n = w * h, i = t;
        const float *s = src + 2 * (size_t)i;
        if (((unsigned)W * (unsigned)H) & 1) {
            const float scale = 1.0f / (2 * n + 1);
            const float w0 = (float)(n - i), w1 = (float)(n - 0), w2 = (float)(1 + i);
            return scale * (w0 * s[0] + w1 * s[1] + w2 * s[2]);
        }
        return 0.5f * (s[0] + s[1]);
    }
    const float *s = src + (size_t)(2 * y) * W + 2 * x;
    if ((W & 1) == 0 && (H & 1) == 0) return 0.25f * (s[0] + s[1] + s[W] + s[W + 1]);
    if ((W & 1) && (H & 1)) {
        const float scale = 1.0f / (float)((unsigned)W * (unsigned)H);
        const float v0 = (float)(h - y), v1 = (float)(h - 0), v2 = (float)(1 + y);
        const float w0 = (float)(w - x), w1 = (float)(w - 0), w2 = (float)(1 + x);
        float acc = 0.0f;
        acc += v0 * (w0 * s[0] + w1 * s[1] + w2 * s[2]);
        acc += v1 * (w0 * s[W] + w1 * s[W + 1] + w2 * s[W + 2]);
        acc += v2 * (w0 * s[2 * W] + w1 * s[2 * W + 1] + w2 * s[2 * W + 2]);
        return acc * scale;
    }
    if (W & 1) {
        const float scale = 1.0f / (float)(2 * (unsigned)W);
        const float w0 = (float)(w - x), w1 = (float)(w - 0), w2 = (float)(1 + x);
        float acc = 0.0f;
        acc += w0 * (s[0] + s[W]);
        acc += w1 * (s[1] + s[W + 1]);
        acc += w2 * (s[2] + s[W + 2]);
        return acc * scale;
    }
    const float scale = 1.0f / (float)(2 * (unsigned)H);
    const float v0 = (float)(h - y), v1 = (float)(h - 0), v2 = (float)(1 + y);
    float acc = 0.0f;
    acc += v0 * (s[0] + s[1]);
    acc += v1 * (s[W] + s[W + 1]);
    acc += v2 * (s[2 * W] + s[2 * W + 1]);
    return acc * scale;
}

size_t tail_smem_bytes() {
    return (size_t)4 * (TAIL_MAX + TAIL_MAX / 2 + TAIL_MAX / 2) * sizeof(float) + TAIL_TAB * sizeof(float);
}

template <bool WEIGHTED>
__global__ void __launch_bounds__(1024) k_mip_tail(const MipJob *__restrict__ jobs, int njobs) {
    extern __shared__ float4 sm4[];
    __shared__ float s_steps[256];
    __shared__ uint8_t s_buckets[kSrgbBuckets];
    __shared__ int s_off[16][4];  // per level: offsets of kx, ky, lx, ly in s_tab, or -1 (read from global)
    float *const lv0 = reinterpret_cast<float *>(sm4);  // levels alternate between two buffers: 4 planes of TAIL_MAX
    float *const s_t = lv0 + 4 * TAIL_MAX;              // X pass, 4 planes of up to TAIL_MAX / 2
    float *const lv1 = s_t + 2 * TAIL_MAX;              // 4 planes of up to TAIL_MAX / 2
    float *const s_tab = lv1 + 2 * TAIL_MAX;            // every level's weights and window starts
    const int tid = threadIdx.x, nt = blockDim.x;
    int j0 = 0, hi = njobs - 1;  // first job of chain blockIdx.x
    while (j0 < hi) {
        const int mid = (j0 + hi) >> 1;
        if (jobs[mid].first_unit < (long long)blockIdx.x) j0 = mid + 1;
        else hi = mid;
    }
    // the chain's job records, copied to shared memory once (every thread reads them every level)
    __shared__ MipJob s_jobs[16];
    const int count = min(jobs[j0].tiles_x, 16);
    {
        static_assert(sizeof(MipJob) % 8 == 0, "job records copy as 8-byte words");
        const unsigned long long *src = reinterpret_cast<const unsigned long long *>(jobs + j0);
        unsigned long long *dst = reinterpret_cast<unsigned long long *>(s_jobs);
        const int words = count * (int)(sizeof(MipJob) / 8);
        for (int i = tid; i < words; i += nt) dst[i] = __ldg(src + i);
    }
    __syncthreads();
    const bool quant = s_jobs[0].q_out != nullptr, srgb = quant && s_jobs[0].xform == 2;
    if (tid == 0) {  // table layout: each level's tables where they fit, in level order
        int off = 0;
        for (int k = 0; k < count; k++) {
            const MipJob &L = s_jobs[k];
            const int need = L.kx ? L.w * L.wsx + L.h * L.wsy + L.w + L.h : 0;
            const bool fit = L.kx && off + need <= TAIL_TAB;
            s_off[k][0] = fit ? off : -1;
            s_off[k][1] = fit ? off + L.w * L.wsx : -1;
            s_off[k][2] = fit ? off + L.w * L.wsx + L.h * L.wsy : -1;
            s_off[k][3] = fit ? off + L.w * L.wsx + L.h * L.wsy + L.w : -1;
            if (fit) off += need;
        }
    }
    if (quant)
        for (int i = tid; i < 256; i += nt) s_steps[i] = __ldg(s_jobs[0].steps + i);
    if (srgb)
        for (int i = tid; i < kSrgbBuckets / 4; i += nt)
            reinterpret_cast<uint32_t *>(s_buckets)[i] = __ldg(reinterpret_cast<const uint32_t *>(s_jobs[0].steps + 256) + i);
    {  // stage the chain's source level
        const MipJob &L = s_jobs[0];
        const int n = L.W * L.H;
        float *s_a = lv0;
        for (int i = tid; i < n; i += nt) {
            if (L.src) {
#pragma unroll
                for (int c = 0; c < 4; c++) s_a[c * n + i] = __ldg(L.src + (size_t)c * n + i);
            } else {
                const uint32_t q = __ldg(L.bgra8 + i);
                s_a[i] = __ldg(L.lut + ((q >> 16) & 255));
                s_a[n + i] = __ldg(L.lut + ((q >> 8) & 255));
                s_a[2 * n + i] = __ldg(L.lut + (q & 255));
                s_a[3 * n + i] = __ldg(L.lut + 256 + (q >> 24));
            }
        }
    }
    __syncthreads();
    for (int k = 0; k < count; k++) {  // all levels' tables at once: one round of global latency
        const MipJob &L = s_jobs[k];
        if (s_off[k][0] < 0) continue;
        for (int i = tid; i < L.w * L.wsx; i += nt) s_tab[s_off[k][0] + i] = __ldg(L.kx + i);
        for (int i = tid; i < L.h * L.wsy; i += nt) s_tab[s_off[k][1] + i] = __ldg(L.ky + i);
        for (int i = tid; i < L.w; i += nt) reinterpret_cast<int *>(s_tab)[s_off[k][2] + i] = __ldg(L.lx + i);
        for (int i = tid; i < L.h; i += nt) reinterpret_cast<int *>(s_tab)[s_off[k][3] + i] = __ldg(L.ly + i);
    }
    __syncthreads();
    for (int k = 0; k < count; k++) {
        const MipJob &L = s_jobs[k];
        const float *src = (k & 1) ? lv1 : lv0;
        float *dstb = (k & 1) ? lv0 : lv1;
        const int W = L.W, H = L.H, w = L.w, h = L.h, wrap = L.wrap;
        const int sn = W * H, tn = H * w, dn = w * h;
        const int wsx = L.wsx, wsy = L.wsy;
        const bool staged = s_off[k][0] >= 0;
        const float *kxs = staged ? s_tab + s_off[k][0] : L.kx;
        const float *kys = staged ? s_tab + s_off[k][1] : L.ky;
        const int *lxs = staged ? reinterpret_cast<const int *>(s_tab) + s_off[k][2] : L.lx;
        const int *lys = staged ? reinterpret_cast<const int *>(s_tab) + s_off[k][3] : L.ly;
        if (L.kx) {
            for (int i = tid; i < tn; i += nt) {  // X taps of every source row
                const int y = i / w, x = i - y * w;
                const float *kx = kxs + x * wsx;
                const int lx = lxs[x];
                const bool inside = lx >= 0 && lx + wsx <= W;
                const float *row = src + y * W;
                float4 sum = make_float4(0, 0, 0, 0);
                float norm = 0;
                for (int j = 0; j < wsx; j++) {
                    const int s = inside ? lx + j : wrap_index(lx + j, W, wrap);
                    tap<WEIGHTED>(sum, norm, kx[j], make_float4(row[s], row[sn + s], row[2 * sn + s], row[3 * sn + s]));
                }
                sum = finish<WEIGHTED>(sum, norm);
                s_t[i] = sum.x; s_t[tn + i] = sum.y; s_t[2 * tn + i] = sum.z; s_t[3 * tn + i] = sum.w;
            }
            __syncthreads();
        }
        for (int o = tid; o < dn; o += nt) {  // Y taps (or the box step), then out to the level
            float4 v;
            if (L.kx) {
                const int y = o / w, x = o - y * w;
                const float *ky = kys + y * wsy;
                const int ly = lys[y];
                const bool inside = ly >= 0 && ly + wsy <= H;
                float4 sum = make_float4(0, 0, 0, 0);
                float norm = 0;
                for (int j = 0; j < wsy; j++) {
                    const int s = (inside ? ly + j : wrap_index(ly + j, H, wrap)) * w + x;
                    tap<WEIGHTED>(sum, norm, ky[j], make_float4(s_t[s], s_t[tn + s], s_t[2 * tn + s], s_t[3 * tn + s]));
                }
                v = finish<WEIGHTED>(sum, norm);
            } else {
                v = make_float4(fast_box_texel(src, W, H, w, h, o), fast_box_texel(src + sn, W, H, w, h, o),
                                fast_box_texel(src + 2 * sn, W, H, w, h, o), fast_box_texel(src + 3 * sn, W, H, w, h, o));
            }
            dstb[o] = v.x; dstb[dn + o] = v.y; dstb[2 * dn + o] = v.z; dstb[3 * dn + o] = v.w;
            L.dst[o] = v.x;
            L.dst[dn + o] = v.y;
            L.dst[2 * dn + o] = v.z;
            L.dst[3 * dn + o] = v.w;
            if (L.q_out)
                L.q_out[o] = srgb ? quantize_srgb_bgra(v, s_steps, s_buckets) : quantize_bgra(v.x, v.y, v.z, v.w, L.xform, s_steps);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------------
// Colour transforms of RGB on a planar FP32 level, in place (Surface::toLinear / toGamma /
// toLinearFromSrgb / toSrgb, src/nvtt/Surface.cpp:1470-1592). Gamma 2.2 uses the reference's own
// table-and-quartic powf_11_5 / powf_5_11 and the sRGB curves the device's correction tables: both
// bit-exact. Other gammas call the device powf, which can differ from the host libm's in the last place.
static __device__ const uint8_t *g_to_srgb_fix_m, *g_from_srgb_fix_m;

__device__ __forceinline__ float dev_to_srgb(float f) { return to_srgb_exact(f, g_to_srgb_fix_m); }
__device__ __forceinline__ float dev_from_srgb(float f) { return from_srgb_exact(f, g_from_srgb_fix_m); }

int set_srgb_fix_mip(const uint8_t *to_srgb, const uint8_t *from_srgb) {
    if (cudaMemcpyToSymbol(g_to_srgb_fix_m, &to_srgb, sizeof to_srgb) != cudaSuccess ||
        cudaMemcpyToSymbol(g_from_srgb_fix_m, &from_srgb, sizeof from_srgb) != cudaSuccess)
        return launch_status();
    return 0;
}

// One chunk of a correction table: entries [first, first + count) (first even) of the toSrgb (which 0)
// or toLinearFromSrgb (which 1) power segment, from the host's results `host` of those entries. One
// thread per table byte (two entries); entries outside -8..7 count in *bad.
__global__ void k_srgb_fix(const float *__restrict__ host, uint32_t first, uint32_t count, int which,
                           uint8_t *__restrict__ fix, unsigned int *__restrict__ bad) {
    const uint32_t pairs = (count + 1) / 2;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < pairs; t += gridDim.x * blockDim.x) {
        uint32_t byte = 0;
        for (int j = 0; j < 2; j++) {
            const uint32_t k = 2 * t + j;
            if (k >= count) break;
            const float f = __uint_as_float((which ? kFromSrgbLo : kToSrgbLo) + first + k);
            const float y = which ? linear_pow_segment(f) : srgb_pow_segment(f);
            const int d = (int)(__float_as_uint(host[k]) - __float_as_uint(y));
            if (d < -8 || d > 7) atomicAdd(bad, 1u);
            byte |= (uint32_t)(d & 15) << (4 * j);
        }
        fix[(first >> 1) + t] = (uint8_t)byte;
    }
}


// kind: 0 toLinear(2.2), 1 toGamma(2.2), 2 toLinearFromSrgb, 3 toSrgb, 4 pow(max(0, x), p)
__global__ void k_transform(float *__restrict__ rgb, size_t n3, int kind, float p) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n3; i += (size_t)gridDim.x * blockDim.x) {
        const float x = rgb[i];
        float y;
        switch (kind) {
            case 0: y = powf_11_5(x); break;
            case 1: y = powf_5_11(x); break;
            case 2: y = dev_from_srgb(x); break;
            case 3: y = dev_to_srgb(x); break;
            default: y = powf(ic_max(0.0f, x), p); break;
        }
        rgb[i] = y;
    }
}

static int grid_for(size_t n, int threads) {
    size_t g = (n + threads - 1) / threads;
    const size_t cap = 152 * 64;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

int launch_srgb_fix(const float *host_chunk, uint32_t first, uint32_t count, int which, uint8_t *fix, unsigned int *bad,
                    cudaStream_t s) {
    if (count == 0) return 0;
    k_srgb_fix<<<grid_for((count + 1) / 2, 256), 256, 0, s>>>(host_chunk, first, count, which, fix, bad);
    return launch_status();
}

int launch_set_image(const uint32_t *bgra, size_t n, const float *lut, float *out, cudaStream_t s) {
    if (n == 0) return 0;
    k_set_image<<<grid_for(n, 256), 256, 0, s>>>(bgra, n, lut, out);
    return launch_status();
}

int launch_transform(float *rgba, size_t n, int kind, float p, cudaStream_t s) {
    if (n == 0) return 0;
    k_transform<<<grid_for(3 * n, 256), 256, 0, s>>>(rgba, 3 * n, kind, p);
    return launch_status();
}

int launch_quantize(const float *rgba, size_t n, int xform, const float *steps, uint32_t *out, cudaStream_t s) {
    if (n == 0) return 0;
    k_quantize_level<<<grid_for(n, 256), 256, 0, s>>>(rgba, n, Quant{xform, steps}, out);
    return launch_status();
}

template <bool W, bool U8>
static int launch_poly_t(const MipLaunch &m, const MipJob *jobs, cudaStream_t s) {
    static std::atomic<unsigned long long> configured{0};
    if (first_use_on_device(configured))
        cudaFuncSetAttribute(k_poly<W, U8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    k_poly<W, U8><<<(unsigned)m.units, PTHREADS, m.smem, s>>>(jobs, m.njobs);
    return launch_status();
}

template <int WS, bool W, bool U8>
static int launch_tile2x_t(const MipLaunch &m, const MipJob *jobs, cudaStream_t s) {
    static std::atomic<unsigned long long> configured{0};
    if (first_use_on_device(configured))
        cudaFuncSetAttribute(k_tile2x<WS, W, U8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    k_tile2x<WS, W, U8><<<(unsigned)m.units, m.threads, m.smem, s>>>(jobs, m.njobs);
    return launch_status();
}

template <int WS>
static int launch_tile2x_ws(const MipLaunch &m, const MipJob *jobs, cudaStream_t s) {
    if (m.weighted) return m.u8 ? launch_tile2x_t<WS, true, true>(m, jobs, s) : launch_tile2x_t<WS, true, false>(m, jobs, s);
    return m.u8 ? launch_tile2x_t<WS, false, true>(m, jobs, s) : launch_tile2x_t<WS, false, false>(m, jobs, s);
}

bool poly2x_supported(int ws) { return ws == 3 || ws == 5 || ws == 13; }

template <int WS, bool W>
static int launch_tile2x_u8_t(const MipLaunch &m, const MipJob *jobs, cudaStream_t s) {
    static std::atomic<unsigned long long> configured{0};
    static int sms = 0;
    if (first_use_on_device(configured)) {
        cudaFuncSetAttribute(k_tile2x_u8<WS, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TileU8<WS>::smem());
        int d = 0;
        cudaGetDevice(&d);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
    }
    const long long grid = std::min<long long>(m.units, sms > 0 ? sms : 152);
    k_tile2x_u8<WS, W><<<(unsigned)grid, 1024, TileU8<WS>::smem(), s>>>(jobs, m.njobs, m.units);
    return launch_status();
}

template <int WS>
static int launch_tile2x_u8_ws(const MipLaunch &m, const MipJob *jobs, cudaStream_t s) {
    return m.weighted ? launch_tile2x_u8_t<WS, true>(m, jobs, s) : launch_tile2x_u8_t<WS, false>(m, jobs, s);
}

template <int WS>
static int launch_tile2x_f32_t(const MipLaunch &m, const MipJob *jobs, cudaStream_t s) {
    static std::atomic<unsigned long long> configured{0};
    static int sms = 0;
    if (first_use_on_device(configured)) {
        cudaFuncSetAttribute(k_tile2x_f32<WS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TileF32<WS>::smem());
        int d = 0;
        cudaGetDevice(&d);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
    }
    const long long grid = std::min<long long>(m.units, sms > 0 ? sms : 152);
    k_tile2x_f32<WS><<<(unsigned)grid, 1024, TileF32<WS>::smem(), s>>>(jobs, m.njobs, m.units);
    return launch_status();
}

int tile_f32_phase(int ws) {
    if (ws == 3) return TileF32<3>::D;
    if (ws == 5) return TileF32<5>::D;
    if (ws == 13) return TileF32<13>::D;
    return -1;
}
int tile_f32_w() { return TileF32<13>::TW; }
int tile_f32_h() { return TileF32<13>::TH; }

int tile_box_cols(int ws) { return ws == 3 ? TileF32<3>::NC : ws == 5 ? TileF32<5>::NC : TileF32<13>::NC; }
int tile_box_rows(int ws, int strip) { return 2 * (strip - 1) + ws; }

int set_mip_wait_polls(int polls) {
    if (cudaMemcpyToSymbol(g_mip_wait_polls, &polls, sizeof polls) != cudaSuccess) return launch_status();
    return 0;
}

int read_mip_status(int *status) {
    unsigned int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_mip_status, sizeof v) != cudaSuccess ||
        cudaMemcpyToSymbol(g_mip_status, &zero, sizeof zero) != cudaSuccess)
        return launch_status();
    *status = (int)v;
    return 0;
}

int tile_u8_phase(int ws) {
    if (ws == 3) return TileU8<3>::D;
    if (ws == 5) return TileU8<5>::D;
    if (ws == 13) return TileU8<13>::D;
    return -1;
}
int tile_u8_w() { return TileU8<13>::TW; }
int tile_u8_h() { return TileU8<13>::TH; }

// ---------------------------------------------------------------------------------------------
// Surface::resize (src/nvtt/Surface.cpp:1152-1230) -> FloatImage::resize (src/nvimage/FloatImage.cpp:
// 761-808, and the alpha-first variant :877-925, which computes every channel the same way): the X
// pass into a w x H planar buffer, then the Y pass, taps summed in window order
// (applyKernelX/Y, :1115-1176). One thread per texel; any scale and window, so it also covers the
// ratios whose tiles would not fit the mip kernels' shared memory. Used once per texture, for the
// InputOptions resize step.
__global__ void k_resize_x(const float *__restrict__ src, int W, int H, const float *__restrict__ kx,
                           const int *__restrict__ lx, int ws, int wrap, float *__restrict__ tmp, int w) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)w * H;
    if (i >= n) return;
    const int x = (int)((unsigned)i % (unsigned)w), y = (int)((unsigned)i / (unsigned)w);
    const size_t sn = (size_t)W * H;
    const float *k = kx + (size_t)x * ws;
    const int left = lx[x];
    float4 sum = make_float4(0, 0, 0, 0);
    float norm = 0;
    for (int j = 0; j < ws; j++) {
        const size_t s = (size_t)y * W + wrap_index(left + j, W, wrap);
        tap<false>(sum, norm, __ldg(k + j), make_float4(__ldg(src + s), __ldg(src + sn + s), __ldg(src + 2 * sn + s),
                                                        __ldg(src + 3 * sn + s)));
    }
    tmp[i] = sum.x; tmp[n + i] = sum.y; tmp[2 * n + i] = sum.z; tmp[3 * n + i] = sum.w;
}

__global__ void k_resize_y(const float *__restrict__ tmp, int w, int H, const float *__restrict__ ky,
                           const int *__restrict__ ly, int ws, int wrap, float *__restrict__ dst, int h) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)w * h;
    if (o >= n) return;
    const int x = (int)((unsigned)o % (unsigned)w), y = (int)((unsigned)o / (unsigned)w);
    const size_t tn = (size_t)w * H;
    const float *k = ky + (size_t)y * ws;
    const int left = ly[y];
    float4 sum = make_float4(0, 0, 0, 0);
    float norm = 0;
    for (int j = 0; j < ws; j++) {
        const size_t s = (size_t)wrap_index(left + j, H, wrap) * w + x;
        tap<false>(sum, norm, __ldg(k + j), make_float4(__ldg(tmp + s), __ldg(tmp + tn + s), __ldg(tmp + 2 * tn + s),
                                                        __ldg(tmp + 3 * tn + s)));
    }
    dst[o] = sum.x; dst[n + o] = sum.y; dst[2 * n + o] = sum.z; dst[3 * n + o] = sum.w;
}

int launch_resize(const float *src, int W, int H, float *tmp, int w, int h, const float *kx, const int *lx, int wsx,
                  const float *ky, const int *ly, int wsy, int wrap, float *dst, cudaStream_t s) {
    const long long nt = (long long)w * H, nd = (long long)w * h;
    if (nt == 0 || nd == 0) return 0;
    k_resize_x<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(src, W, H, kx, lx, wsx, wrap, tmp, w);
    const int st = launch_status();
    if (st) return st;
    k_resize_y<<<(unsigned)((nd + 255) / 256), 256, 0, s>>>(tmp, w, H, ky, ly, wsy, wrap, dst, h);
    return launch_status();
}

size_t poly_smem_bytes(int rx_max, int ry_max) {
    return (size_t)ry_max * rx_max * sizeof(float4) + (size_t)ry_max * PTW * sizeof(float4) +
           (size_t)(rx_max + ry_max) * sizeof(int);
}

size_t poly2x_smem_bytes(int ws, int tile_h) {
    return ws == 3 ? Tile2x<3>::smem(tile_h) : ws == 5 ? Tile2x<5>::smem(tile_h) : Tile2x<13>::smem(tile_h);
}

int launch_mip(const MipLaunch &m, const MipJob *d_jobs, cudaStream_t s) {
    if (m.units <= 0 || m.njobs <= 0) return 0;
    const MipJob *jobs = d_jobs + m.first_job;
    switch (m.kernel) {
        case MIP_FAST_BOX: {
            const long long cap = 152LL * 64, g = (m.units + 255) / 256;
            k_fast_down<<<(unsigned)(g < cap ? g : cap), 256, 0, s>>>(jobs, m.njobs, m.units);
            return launch_status();
        }
        case MIP_POLY:
            if (m.smem > 200 * 1024) return 2;  // Error_UnsupportedFeature
            if (m.weighted) return m.u8 ? launch_poly_t<true, true>(m, jobs, s) : launch_poly_t<true, false>(m, jobs, s);
            return m.u8 ? launch_poly_t<false, true>(m, jobs, s) : launch_poly_t<false, false>(m, jobs, s);
        case MIP_TAIL: {
            static std::atomic<unsigned long long> configured{0};
            if (first_use_on_device(configured)) {
                cudaFuncSetAttribute(k_mip_tail<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tail_smem_bytes());
                cudaFuncSetAttribute(k_mip_tail<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tail_smem_bytes());
            }
            if (m.weighted) k_mip_tail<true><<<(unsigned)m.units, 1024, tail_smem_bytes(), s>>>(jobs, m.njobs);
            else k_mip_tail<false><<<(unsigned)m.units, 1024, tail_smem_bytes(), s>>>(jobs, m.njobs);
            return launch_status();
        }
        case MIP_TILE_U8:
            if (m.ws == 3) return launch_tile2x_u8_ws<3>(m, jobs, s);
            if (m.ws == 5) return launch_tile2x_u8_ws<5>(m, jobs, s);
            if (m.ws == 13) return launch_tile2x_u8_ws<13>(m, jobs, s);
            return 2;
        case MIP_TILE_F32:
            if (m.ws == 3) return launch_tile2x_f32_t<3>(m, jobs, s);
            if (m.ws == 5) return launch_tile2x_f32_t<5>(m, jobs, s);
            if (m.ws == 13) return launch_tile2x_f32_t<13>(m, jobs, s);
            return 2;
        case MIP_POLY2X:
            if (m.threads < 64 || m.threads > 512 || m.threads % 32 || m.smem > 200 * 1024) return 1;
            if (m.ws == 3) return launch_tile2x_ws<3>(m, jobs, s);
            if (m.ws == 5) return launch_tile2x_ws<5>(m, jobs, s);
            if (m.ws == 13) return launch_tile2x_ws<13>(m, jobs, s);
            return 2;
        default:
            return 1;
    }
}

int poly_tile_w() { return PTW; }
int poly_tile_h() { return PTH; }
int poly_max_window() { return PMAXW; }
int tail_max_texels() { return TAIL_MAX; }

NTG_DEFINE_TABLE_UPLOAD(upload_tables_mip)

}  // namespace ntg
