// Internal interfaces between the C-ABI layer (ntg_api.cu) and the kernel translation units.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda.h>  // CUtensorMap (maps are encoded through the runtime's driver entry point)
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

// threads = blocks per CTA (one thread per 4x4 block); 0 = the default shape.
int launch_bc1(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t s);
int launch_bc3(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t s);
int launch_bc5(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t s);
int launch_bc1a(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t s);
// Counts the floats on which the fast sRGB quantiser and the step search disagree.
int launch_check_srgb(const float *steps, unsigned long long *bad, cudaStream_t s);
// Separable polyphase resize of a planar FP32 image (two launches through `tmp`, w * H * 16 bytes).
int launch_resize(const float *src, int W, int H, float *tmp, int w, int h, const float *kx, const int *lx, int wsx,
                  const float *ky, const int *ly, int wsy, int wrap, float *dst, cudaStream_t s);
int launch_bc4(const EncJob *d_jobs, int njobs, long long nblocks, int quality, int threads, cudaStream_t s);

// Learned endpoint proposal, BC1 Normal quality: the network's inputs (x [nblocks x 48]), training
// targets from encoded blocks (tg [nblocks x 8]), the pruned fit from the network's outputs
// (y [nblocks x 16]) listing the blocks that need the full fit, and the full fit over such a list.
int launch_bc1_features(const EncJob *d_jobs, int njobs, long long nblocks, float *x, cudaStream_t s);
int launch_bc1_targets(const EncJob *d_jobs, int njobs, long long nblocks, float *tg, cudaStream_t s);
int launch_bc1_learned(const EncJob *d_jobs, int njobs, long long nblocks, const float *y, int radius, float margin,
                       long long *fallback, unsigned long long *stats, cudaStream_t s);
// The same for BC3 Normal colour (squish Compress4 splits): inputs, targets, pruned fit (unit_metric:
// all colour weights 1), and the full k_bc3 over a list.
int launch_bc3_features(const EncJob *d_jobs, int njobs, long long nblocks, float *x, cudaStream_t s);
int launch_bc3_targets(const EncJob *d_jobs, int njobs, long long nblocks, float *tg, cudaStream_t s);
int launch_bc3_learned(const EncJob *d_jobs, int njobs, long long nblocks, const float *y, int radius, float margin,
                       bool unit_metric, long long *fallback, unsigned long long *stats, cudaStream_t s);
int launch_bc3_list(const EncJob *d_jobs, int njobs, const long long *list, const unsigned long long *d_count,
                    long long max_count, cudaStream_t s);
// Orderings the Level8 fit evaluates over the jobs' blocks (four-cluster, three-cluster), added to
// work[0], work[1] (measurement only).
int launch_bc1_work(const EncJob *d_jobs, int njobs, long long nblocks, unsigned long long *work, cudaStream_t s);
// The full fit over the first *d_count entries of `list` (at most max_count; no host round trip).
int launch_bc1_list(const EncJob *d_jobs, int njobs, const long long *list, const unsigned long long *d_count,
                    long long max_count, cudaStream_t s);
}  // namespace ntg
struct ntg_mlp;
struct ntg_context;
namespace ntg {
int mlp_forward_device(ntg_mlp *m, const float *d_x, long long rows, float *d_y, cudaStream_t s);

// One buildNextMipmap step (source level -> destination level) of one texture. A mip launch walks a
// list of these: its units (destination texels or tiles, depending on the kernel) are
// numbered across the jobs (`first_unit`), so one launch covers the same step of many textures.
struct MipJob {
    const float *src;        // planar FP32 source level, or null to read bgra8 through lut
    const uint32_t *bgra8;   // BGRA8 source words (level 0 read straight from the input)
    const float *lut;        // 256-entry input transform for bgra8 RGB
    int W, H, w, h;          // source and destination sizes
    int wsx, wsy;            // polyphase windows
    const float *kx, *ky;    // weights: w x wsx and h x wsy (the 2:1 kernel reads row 0 only)
    const int *lx, *ly;      // window offsets of every output column / row (general kernel)
    int cx, cy;              // 2:1 kernel: window offset of output column / row 0
    int wrap;                // 0 clamp, 1 repeat, 2 mirror
    float *dst;              // planar FP32 destination level
    uint32_t *q_out;         // optional quantised BGRA8 destination (for the BC3/BC5 encoders)
    int xform;               // output transform folded into the quantiser (0 none, 1 gamma 2.2, 2 sRGB)
    const float *steps;      // sRGB quantiser steps (xform 2)
    int tiles_x;             // units along x (tail launches: levels in the chain, on its first job)
    int strip;               // 2:1 kernel: output rows per tile
    int rx_max, ry_max;      // general kernel: widest source window of a tile (host side, for shared memory)
    long long first_unit;    // running unit count of the launch (tail launches: the chain's index)
    int tma;                 // TMA-staged FP32 tile kernel: `map` describes the source level
    CUtensorMap map;         // the source level's FP32 planes as a 3-D (x, y, plane) tensor map whose box is
                             // a tile's source window (64-byte aligned, as the TMA requires)
};

enum MipKernel { MIP_FAST_BOX = 0, MIP_POLY = 1, MIP_POLY2X = 2, MIP_TAIL = 3, MIP_TILE_U8 = 4, MIP_TILE_F32 = 5 };

// One launch over jobs [first_job, first_job + njobs) of a device job array.
struct MipLaunch {
    int kernel;              // MipKernel
    int ws;                  // 2:1 kernel: window size (3, 5 or 13)
    int weighted, u8;        // template switches: alpha-weighted taps, BGRA8 source
    int first_job, njobs;
    long long units;
    size_t smem;             // dynamic shared memory
    int threads;             // 2:1 kernel: threads per CTA (one tile per CTA)
};

int launch_set_image(const uint32_t *bgra, size_t n, const float *lut, float *out, cudaStream_t s);
int launch_quantize(const float *rgba, size_t n, int xform, const float *steps, uint32_t *out, cudaStream_t s);
int launch_transform(float *rgba, size_t n, int kind, float p, cudaStream_t s);
int launch_mip(const MipLaunch &m, const MipJob *d_jobs, cudaStream_t s);
// The sRGB curves' correction tables (ntg_device.cuh): one chunk of entries from the host's results,
// and the tables' device addresses for the kernels of each translation unit that evaluates the curves.
int launch_srgb_fix(const float *host_chunk, uint32_t first, uint32_t count, int which, uint8_t *fix, unsigned int *bad,
                    cudaStream_t s);
int set_srgb_fix_mip(const uint8_t *to_srgb, const uint8_t *from_srgb);
int set_srgb_fix_bc1(const uint8_t *to_srgb);
bool poly2x_supported(int ws);
// 2:1 steps from the BGRA8 input (persistent, cp.async-pipelined 64 x 16 tiles): the window start of
// output column 0 mod 4 that the kernel for `ws` taps is built for (-1: none), and the tile size.
int tile_u8_phase(int ws);
int tile_u8_w();
int tile_u8_h();
// 2:1 steps between FP32 levels without alpha weighting (persistent, TMA-staged 32 x strip tiles,
// strip at most tile_f32_h()): the same window phase rule and the tile width / tallest tile.
int tile_f32_phase(int ws);
int tile_f32_w();
int tile_f32_h();
// The TMA box of the FP32 tile kernel's source window: columns, and rows for a tile of `strip` output rows.
int tile_box_cols(int ws);
int tile_box_rows(int ws, int strip);
// Poll limit of the FP32 tile kernel's mbarrier waits on the current device, and the status word a
// wait that ran out sets (read and cleared by read_mip_status).
int set_mip_wait_polls(int polls);
int read_mip_status(int *status);
size_t poly_smem_bytes(int rx_max, int ry_max);
size_t poly2x_smem_bytes(int ws, int tile_h);  // dynamic shared memory of a 2:1 tile launch
int poly_tile_w();
int poly_tile_h();
int poly_max_window();
int tail_max_texels();  // largest source level a tail launch starts from

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
// Makes the context's device current (ntg_last_error_string describes a failure).
int use_context_device(ntg_context *ctx);

}  // namespace ntg
