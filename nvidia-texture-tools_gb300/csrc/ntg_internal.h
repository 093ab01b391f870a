// Internal interfaces between the C-ABI layer (ntg_api.cu) and the kernel translation units.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

namespace ntg {

// Launcher status: 0 on success, else kLaunchErrorBase + the cudaError_t of the failed launch.
constexpr int kLaunchErrorBase = 1000;
// True the first time it is called for the current device (function attributes are per device).
inline bool first_use_on_device(std::atomic<unsigned long long> &mask) {
    int d = 0;
    cudaGetDevice(&d);
    const unsigned long long bit = 1ull << (d & 63);
    return (mask.fetch_or(bit) & bit) == 0;
}

inline int launch_status() {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : kLaunchErrorBase + (int)e;
}

// One texture level to encode. An encoder launch walks a list of jobs: thread-blocks of 4x4
// texels are numbered across all jobs and a thread finds its job by binary search over the
// running block counts (`first_block`), so one launch covers a whole mip chain or a batch of
// textures of uneven sizes.
struct EncJob {
    const float *rgba;        // planar FP32 level, or null
    const uint32_t *bgra;     // BGRA8 words, or null (used when non-null)
    const float *lut_f;       // BC1: 256-entry float table applied to the bgra bytes (RGB), or null
    const uint8_t *lut8;      // BC3/BC5: 2 x 256 byte tables (RGB, alpha) applied to bgra bytes, or null
    int w, h, bw;             // level size and width in blocks
    int alpha_mode;           // 1 = AlphaMode_Transparency
    int out_xform;            // BC1 on float input: 0 none, 1 toGamma(2.2), 2 toSrgb
    float cw[3];              // colour weights
    uint8_t *out;             // blocks, row-major
    long long first_block;    // index of this job's first block in the launch
};

int launch_bc1(const EncJob *d_jobs, int njobs, long long nblocks, int quality, cudaStream_t s);
int launch_bc3(const EncJob *d_jobs, int njobs, long long nblocks, int quality, cudaStream_t s);
int launch_bc5(const EncJob *d_jobs, int njobs, long long nblocks, int quality, cudaStream_t s);

struct PolyArgs {
    const float *src;
    const uint32_t *bgra8;
    const float *lut;
    int W, H, w, h, wsx, wsy;
    const float *kx, *ky;
    const int *lx, *ly;
    int wrap;
    float *dst;
    uint32_t *q_out;
    int xform;
    const float *steps;
    bool weighted;
    int rx_max, ry_max;  // largest source window of any output tile (host-computed)
};

int launch_set_image(const uint32_t *bgra, size_t n, const float *lut, float *out, cudaStream_t s);
int launch_quantize(const float *rgba, size_t n, int xform, const float *steps, uint32_t *out, cudaStream_t s);
int launch_transform(float *rgba, size_t n, int kind, float p, cudaStream_t s);
int launch_fast_down(const float *src, int W, int H, float *dst, uint32_t *q_out, int xform, const float *steps,
                     cudaStream_t s);
int launch_poly(const PolyArgs &a, cudaStream_t s);
int poly_tile_w();
int poly_tile_h();

int launch_decode(int format, const uint8_t *blocks, int w, int h, float *rgba, cudaStream_t s);
int launch_rms(const float *ref, const float *dec, int w, int h, int alpha_mode, double *sums, cudaStream_t s);

// Upload the constant tables of each kernel translation unit to the current device.
struct HostTables;
int upload_tables_bc1(const HostTables &t);
int upload_tables_bc3(const HostTables &t);
int upload_tables_mip(const HostTables &t);
int upload_tables_decode(const HostTables &t);

// Sets the message ntg_last_error_string() returns on this thread.
void set_last_error(const std::string &msg);

}  // namespace ntg
