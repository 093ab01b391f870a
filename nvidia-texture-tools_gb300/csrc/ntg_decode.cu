// Block decode and error sums on the GPU: Surface::setImage2D with the D3D10 decoder
// (src/nvtt/Surface.cpp:908-1116, src/nvimage/BlockDXT.cpp) and nv::rmsColorError /
// rmsAlphaError (src/nvimage/ErrorMetric.cpp:13-71), so quality checks run at GPU speed.
#include "ntg_device.cuh"
#include "ntg_internal.h"

namespace ntg {

__device__ __forceinline__ void decode_alpha8(uint2 b, uint8_t out[16]) {
    const uint64_t u = (uint64_t)b.x | ((uint64_t)b.y << 32);
    int pal[8];
    alpha_palette((int)(u & 255), (int)((u >> 8) & 255), pal);
#pragma unroll
    for (int i = 0; i < 16; i++) out[i] = (uint8_t)pal[(u >> (16 + 3 * i)) & 7];
}

// One thread per block; writes the texels inside the image (1/255 scale, as setImage2D does).
__global__ void k_decode(int format, const uint8_t *__restrict__ blocks, int w, int h, float *__restrict__ rgba) {
    const int bw = (w + 3) / 4, bh = (h + 3) / 4;
    const long long nb = (long long)bw * bh;
    const long long blk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (blk >= nb) return;
    const int bx = (int)(blk % bw), by = (int)(blk / bw);
    const size_t n = (size_t)w * h;
    uint8_t r[16], g[16], b[16], a[16];
    const bool bc1 = format == 1 || format == 2;  // BC1a has BC1's block layout
    if (format == 6) {  // BlockATI1::decodeBlock (src/nvimage/BlockDXT.cpp:513-526)
        decode_alpha8(*reinterpret_cast<const uint2 *>(blocks + 8 * (size_t)blk), r);
#pragma unroll
        for (int i = 0; i < 16; i++) { g[i] = r[i]; b[i] = r[i]; a[i] = 255; }
    } else if (bc1 || format == 4) {
        const uint2 c = *reinterpret_cast<const uint2 *>(blocks + (bc1 ? 8 : 16) * (size_t)blk + (bc1 ? 0 : 8));
        const unsigned c0 = c.x & 0xFFFF, c1 = c.x >> 16;
        Pal8 p;
        palette_d3d10(c0, c1, p);
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const int k = (c.y >> (2 * i)) & 3;
            r[i] = (uint8_t)p.r[k]; g[i] = (uint8_t)p.g[k]; b[i] = (uint8_t)p.b[k];
            a[i] = (c0 <= c1 && k == 3) ? 0 : 255;
        }
        if (format == 4) decode_alpha8(*reinterpret_cast<const uint2 *>(blocks + 16 * (size_t)blk), a);
    } else {
        decode_alpha8(*reinterpret_cast<const uint2 *>(blocks + 16 * (size_t)blk), r);
        decode_alpha8(*reinterpret_cast<const uint2 *>(blocks + 16 * (size_t)blk + 8), g);
#pragma unroll
        for (int i = 0; i < 16; i++) { b[i] = 0; a[i] = 255; }
    }
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const int x = bx * 4 + (i & 3), y = by * 4 + (i >> 2);
        if (x >= w || y >= h) continue;
        const size_t s = (size_t)y * w + x;
        rgba[s] = r[i] / 255.0f;
        rgba[n + s] = g[i] / 255.0f;
        rgba[2 * n + s] = b[i] / 255.0f;
        rgba[3 * n + s] = a[i] / 255.0f;
    }
}

// Squared-error sums in double, reduced per CTA and accumulated atomically.
__global__ void k_error_sums(const float *__restrict__ ref, const float *__restrict__ img, size_t n, int alpha_mode,
                             double *__restrict__ sums) {
    double c = 0, al = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float r = ref[i] - img[i], g = ref[n + i] - img[n + i], b = ref[2 * n + i] - img[2 * n + i];
        float wgt = 1;
        if (alpha_mode == 1) wgt = ref[3 * n + i] * ref[3 * n + i];
        c += (double)((r * r) * wgt);
        c += (double)((g * g) * wgt);
        c += (double)((b * b) * wgt);
        const float da = img[3 * n + i] - ref[3 * n + i];
        al += (double)(da * da);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_down_sync(0xffffffffu, c, o);
        al += __shfl_down_sync(0xffffffffu, al, o);
    }
    __shared__ double s_c[32], s_a[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { s_c[warp] = c; s_a[warp] = al; }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        c = lane < nw ? s_c[lane] : 0.0;
        al = lane < nw ? s_a[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            c += __shfl_down_sync(0xffffffffu, c, o);
            al += __shfl_down_sync(0xffffffffu, al, o);
        }
        if (lane == 0) { atomicAdd(&sums[0], c); atomicAdd(&sums[1], al); }
    }
}

int launch_decode(int format, const uint8_t *blocks, int w, int h, float *rgba, cudaStream_t s) {
    const long long nb = (long long)((w + 3) / 4) * ((h + 3) / 4);
    if (nb == 0) return 0;
    k_decode<<<(unsigned)((nb + 127) / 128), 128, 0, s>>>(format, blocks, w, h, rgba);
    return launch_status();
}

int launch_rms(const float *ref, const float *img, int w, int h, int alpha_mode, double *sums, cudaStream_t s) {
    const size_t n = (size_t)w * h;
    if (cudaMemsetAsync(sums, 0, 2 * sizeof(double), s) != cudaSuccess) return launch_status();
    if (n == 0) return 0;
    size_t g = (n + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    k_error_sums<<<(unsigned)g, 256, 0, s>>>(ref, img, n, alpha_mode, sums);
    return launch_status();
}

NTG_DEFINE_TABLE_UPLOAD(upload_tables_decode)

}  // namespace ntg
