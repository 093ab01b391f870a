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
#include "ntg_device.cuh"
#include "ntg_internal.h"

namespace ntg {

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
// FloatImage::fastDownSample (src/nvimage/FloatImage.cpp:559-737): 2x2 box for even sizes,
// pair average for 1-D images and the three-tap polyphase box for odd sizes. One thread per
// destination texel and channel.
__global__ void k_fast_down(const float *__restrict__ src0, int W, int H, float *__restrict__ dst0,
                            uint32_t *__restrict__ q_out, Quant q) {
    __shared__ float s_steps[256];
    if (q_out && q.xform == 2)
        for (int i = threadIdx.x; i < 256; i += blockDim.x) s_steps[i] = q.steps[i];
    __syncthreads();
    const unsigned w = W / 2 > 1 ? (unsigned)W / 2 : 1u, h = H / 2 > 1 ? (unsigned)H / 2 : 1u;
    const size_t sn = (size_t)W * H, dn = (size_t)w * h;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < dn; t += (size_t)gridDim.x * blockDim.x) {
        const unsigned x = (unsigned)(t % w), y = (unsigned)(t / w);
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
            dst0[c * dn + t] = f;
        }
        if (q_out) q_out[t] = quantize_bgra(v[0], v[1], v[2], v[3], q.xform, s_steps);
    }
}

// ---------------------------------------------------------------------------------------------
// Fused separable polyphase resize: FloatImage::resize 2D (src/nvimage/FloatImage.cpp:761-808)
// = applyKernelX over every source row into a (w' x H) plane, then applyKernelY
// (:1115-1176). A CTA owns a TW x TH output tile: it stages the (wrapped) source window of the
// tile in shared memory, runs the X taps for the rows the tile's Y taps touch, then the Y taps.
// The optional weighted mode applies the alpha-weighted kernels (:1212-1281) to RGB.
struct PolyLevel {
    const float *src;        // planar FP32 source level (null when reading bgra8 + lut)
    const uint32_t *bgra8;   // BGRA8 source words (level 0 read straight from the input)
    const float *lut;        // 256-entry input transform for bgra8 RGB
    int W, H, w, h;
    int wsx, wsy;            // window sizes
    const float *kx;         // w * wsx weights
    const float *ky;         // h * wsy weights
    const int *lx;           // w left offsets
    const int *ly;           // h left offsets
    int wrap;                // 0 clamp, 1 repeat, 2 mirror (src/nvimage/FloatImage.h:298-317)
    float *dst;              // planar FP32 destination level
    uint32_t *q_out;         // optional quantised BGRA8 destination
    Quant q;
};

__device__ __forceinline__ int wrap_index(int x, int w, int wm) {
    if (wm == 0) return x < 0 ? 0 : (x > w - 1 ? w - 1 : x);
    if (wm == 1) return x >= 0 ? x % w : (x + 1) % w + w - 1;
    if (w == 1) return 0;
    x = abs(x);
    while (x >= w) x = abs(w + w - x - 2);
    return x;
}

constexpr int PTW = 32;    // output tile width (one warp lane per output column)
constexpr int PTH = 16;    // output tile height
constexpr int PMAXW = 32;  // widest window handled by the fused kernel
constexpr int PTHREADS = 256;
constexpr int PWARPS = PTHREADS / 32;

// One CTA per PTW x PTH output tile, all four channels at once (RGBA as float4 in shared memory):
//  1. wrap maps for the tile's source rows and columns (FloatImage::index, one wrap per row/column),
//  2. the wrapped source window staged once as float4 (from planar FP32 or BGRA8 + input table),
//  3. X taps for every window row into a (rows x PTW) float4 plane,
//  4. Y taps, written as four planes and, optionally, the quantised BGRA8 word.
// Channel arithmetic is the reference's, lane by lane: sum starts at 0 and adds k * v in tap order.
template <bool WEIGHTED, bool SRC_U8>
__global__ void __launch_bounds__(PTHREADS) k_poly(PolyLevel L) {
    extern __shared__ float4 sm4[];
    const int ox0 = blockIdx.x * PTW, oy0 = blockIdx.y * PTH;
    const int tw = min(PTW, L.w - ox0), th = min(PTH, L.h - oy0);
    const int xlo = L.lx[ox0], xhi = L.lx[ox0 + tw - 1] + L.wsx - 1;
    const int ylo = L.ly[oy0], yhi = L.ly[oy0 + th - 1] + L.wsy - 1;
    const int rx = xhi - xlo + 1, ry = yhi - ylo + 1;
    float4 *s_in = sm4;                 // ry * rx
    float4 *s_tmp = s_in + ry * rx;     // ry * PTW
    int *s_col = reinterpret_cast<int *>(s_tmp + ry * PTW);  // rx
    int *s_row = s_col + rx;                                  // ry
    __shared__ float s_kx[PTW * PMAXW], s_ky[PTH * PMAXW], s_steps[256], s_lut[256];
    __shared__ int s_lx[PTW], s_ly[PTH];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < tw * L.wsx; i += PTHREADS) s_kx[i] = L.kx[(size_t)ox0 * L.wsx + i];
    for (int i = tid; i < th * L.wsy; i += PTHREADS) s_ky[i] = L.ky[(size_t)oy0 * L.wsy + i];
    if (tid < tw) s_lx[tid] = L.lx[ox0 + tid] - xlo;
    if (tid < th) s_ly[tid] = L.ly[oy0 + tid] - ylo;
    for (int i = tid; i < rx; i += PTHREADS) s_col[i] = wrap_index(xlo + i, L.W, L.wrap);
    for (int i = tid; i < ry; i += PTHREADS) s_row[i] = wrap_index(ylo + i, L.H, L.wrap);
    if (L.q_out && L.q.xform == 2) for (int i = tid; i < 256; i += PTHREADS) s_steps[i] = L.q.steps[i];
    if (SRC_U8) for (int i = tid; i < 256; i += PTHREADS) s_lut[i] = L.lut[i];
    __syncthreads();

    const size_t sn = (size_t)L.W * L.H;
    for (int r = warp; r < ry; r += PWARPS) {
        const size_t rowoff = (size_t)s_row[r] * L.W;
        float4 *dst = s_in + r * rx;
        for (int x = lane; x < rx; x += 32) {
            const size_t s = rowoff + s_col[x];
            float4 v;
            if (SRC_U8) {
                const uint32_t p = L.bgra8[s];
                v = make_float4(s_lut[(p >> 16) & 255], s_lut[(p >> 8) & 255], s_lut[p & 255], (float)(p >> 24) / 255.0f);
            } else {
                v = make_float4(L.src[s], L.src[sn + s], L.src[2 * sn + s], L.src[3 * sn + s]);
            }
            dst[x] = v;
        }
    }
    __syncthreads();

    // X taps: one lane per output column, warps over the window rows
    if (lane < tw) {
        const float *k = s_kx + lane * L.wsx;
        const int off = s_lx[lane];
        for (int r = warp; r < ry; r += PWARPS) {
            const float4 *row = s_in + r * rx + off;
            float4 sum = make_float4(0, 0, 0, 0);
            if (WEIGHTED) {
                float norm = 0;
                for (int j = 0; j < L.wsx; j++) {
                    const float4 v = row[j];
                    const float kj = k[j];
                    const float wgt = kj * (v.w + (1.0f / 256.0f));
                    norm += wgt;
                    sum.x += wgt * v.x; sum.y += wgt * v.y; sum.z += wgt * v.z;
                    sum.w += kj * v.w;
                }
                sum.x = sum.x / norm; sum.y = sum.y / norm; sum.z = sum.z / norm;
            } else {
                for (int j = 0; j < L.wsx; j++) {
                    const float4 v = row[j];
                    const float kj = k[j];
                    sum.x += kj * v.x; sum.y += kj * v.y; sum.z += kj * v.z; sum.w += kj * v.w;
                }
            }
            s_tmp[r * PTW + lane] = sum;
        }
    }
    __syncthreads();

    // Y taps: one lane per output column, warps over the output rows
    if (lane < tw) {
        const size_t dn = (size_t)L.w * L.h;
        for (int y = warp; y < th; y += PWARPS) {
            const float *k = s_ky + y * L.wsy;
            const float4 *col = s_tmp + s_ly[y] * PTW + lane;
            float4 sum = make_float4(0, 0, 0, 0);
            if (WEIGHTED) {
                float norm = 0;
                for (int j = 0; j < L.wsy; j++) {
                    const float4 v = col[j * PTW];
                    const float kj = k[j];
                    const float wgt = kj * (v.w + (1.0f / 256.0f));
                    norm += wgt;
                    sum.x += wgt * v.x; sum.y += wgt * v.y; sum.z += wgt * v.z;
                    sum.w += kj * v.w;
                }
                sum.x = sum.x / norm; sum.y = sum.y / norm; sum.z = sum.z / norm;
            } else {
                for (int j = 0; j < L.wsy; j++) {
                    const float4 v = col[j * PTW];
                    const float kj = k[j];
                    sum.x += kj * v.x; sum.y += kj * v.y; sum.z += kj * v.z; sum.w += kj * v.w;
                }
            }
            const size_t o = (size_t)(oy0 + y) * L.w + ox0 + lane;
            L.dst[o] = sum.x;
            L.dst[dn + o] = sum.y;
            L.dst[2 * dn + o] = sum.z;
            L.dst[3 * dn + o] = sum.w;
            if (L.q_out) L.q_out[o] = quantize_bgra(sum.x, sum.y, sum.z, sum.w, L.q.xform, s_steps);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Colour transforms of RGB on a planar FP32 level, in place (Surface::toLinear / toGamma /
// toLinearFromSrgb / toSrgb, src/nvtt/Surface.cpp:1470-1592). Gamma 2.2 uses the reference's own
// table-and-quartic powf_11_5 / powf_5_11 and is bit-exact; the sRGB curves and other gammas call
// the device powf, which can differ from the host libm's in the last place.
__device__ __forceinline__ float dev_to_srgb(float f) {
    if (isnan(f)) return 0.0f;
    if (f <= 0.0f) return 0.0f;
    if (f <= 0.0031308f) return 12.92f * f;
    if (f <= 1.0f) return (powf(f, 0.41666f) * 1.055f) - 0.055f;
    return 1.0f;
}

__device__ __forceinline__ float dev_from_srgb(float f) {
    if (f < 0.0f) return 0.0f;
    if (f < 0.04045f) return f / 12.92f;
    if (f <= 1.0f) return powf((f + 0.055f) / 1.055f, 2.4f);
    return 1.0f;
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

int launch_fast_down(const float *src, int W, int H, float *dst, uint32_t *q_out, int xform, const float *steps,
                     cudaStream_t s) {
    const size_t dn = (size_t)(W / 2 > 1 ? W / 2 : 1) * (H / 2 > 1 ? H / 2 : 1);
    k_fast_down<<<grid_for(dn, 256), 256, 0, s>>>(src, W, H, dst, q_out, Quant{xform, steps});
    return launch_status();
}

size_t poly_smem_bytes(int rx_max, int ry_max, bool) {
    return (size_t)ry_max * rx_max * sizeof(float4) + (size_t)ry_max * PTW * sizeof(float4) +
           (size_t)(rx_max + ry_max) * sizeof(int);
}

template <bool W, bool U8>
static int launch_poly_t(const PolyLevel &L, size_t sm, cudaStream_t s) {
    static std::atomic<unsigned long long> configured{0};
    if (first_use_on_device(configured))
        cudaFuncSetAttribute(k_poly<W, U8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    dim3 grid((L.w + PTW - 1) / PTW, (L.h + PTH - 1) / PTH);
    k_poly<W, U8><<<grid, PTHREADS, sm, s>>>(L);
    return launch_status();
}

int launch_poly(const PolyArgs &a, cudaStream_t s) {
    PolyLevel L;
    L.src = a.src; L.bgra8 = a.bgra8; L.lut = a.lut;
    L.W = a.W; L.H = a.H; L.w = a.w; L.h = a.h;
    L.wsx = a.wsx; L.wsy = a.wsy; L.kx = a.kx; L.ky = a.ky; L.lx = a.lx; L.ly = a.ly;
    L.wrap = a.wrap; L.dst = a.dst; L.q_out = a.q_out; L.q = Quant{a.xform, a.steps};
    const size_t sm = poly_smem_bytes(a.rx_max, a.ry_max, a.weighted);
    if (a.wsx > PMAXW || a.wsy > PMAXW || sm > 200 * 1024) return 2;  // Error_UnsupportedFeature
    const bool u8 = a.src == nullptr;
    if (a.weighted) return u8 ? launch_poly_t<true, true>(L, sm, s) : launch_poly_t<true, false>(L, sm, s);
    return u8 ? launch_poly_t<false, true>(L, sm, s) : launch_poly_t<false, false>(L, sm, s);
}

int poly_tile_w() { return PTW; }
int poly_tile_h() { return PTH; }

NTG_DEFINE_TABLE_UPLOAD(upload_tables_mip)

}  // namespace ntg
