// ntg_encode_noalloc: the level encoder of ntg_encode for callers that cannot allocate device memory.
//
// Who needs it: engines and plugins that own every byte of GPU memory through their own pools and
// forbid hidden allocations; real-time loops where cudaMalloc's implicit device synchronisation
// would stall the frame; code that runs where allocating is not allowed at all. ntg_encode itself
// allocates on first use (its job list, the quantised level of BC3/BC5 with an output transform,
// the transform tables), so those callers use this entry point instead.
//
// Its scratch is the file-scope array below, allocated by the CUDA runtime when the library's
// module loads on a GPU: every GPU that loads libntg.so holds NTG_NOALLOC_SCRATCH_BYTES of device
// memory until the process exits. Host code never passes the array's name to a kernel (on the host
// it is only a stand-in symbol): the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress and caches it, and the kernels receive that
// address. That first call should therefore come before any stream capture on the device.
//
// All calls share the one array and it keeps what the last call left there: each call rewrites the
// parts it reads (job record, quantiser steps, quantised level) before its kernels run. Calls whose
// work overlaps on the GPU (different streams, or different host threads) race on the array; issue
// them on one stream, or serialise them. The job record and the quantiser steps reach the array as
// kernel arguments (written by a one-CTA kernel), so no call reads host memory after it returns.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "ntg.h"
#include "ntg_host_tables.h"
#include "ntg_internal.h"

namespace {

// Layout of the scratch array (byte offsets).
constexpr size_t kJobOffset = 0;                         // one EncJob record
constexpr size_t kStepsOffset = 256;                     // 256 floats: sRGB quantiser steps
constexpr size_t kLevelOffset = 2048;                    // quantised BGRA8 level, 4 bytes per texel
constexpr size_t kMaxTexels = NTG_NOALLOC_MAX_TEXELS;
constexpr size_t kScratchBytes = kLevelOffset + 4 * kMaxTexels;
static_assert(kScratchBytes <= NTG_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the declared size");
static_assert(sizeof(ntg::EncJob) <= kStepsOffset - kJobOffset, "job record does not fit");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NTG_NOALLOC_SCRATCH_BYTES];

std::mutex g_mu;
unsigned char *g_scratch_ptr[256];  // device address of g_noalloc_scratch per device, once looked up

int scratch_address(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return ntg::kLaunchErrorBase + (int)e;
    if (dev < 0 || dev >= 256) return NTG_ERROR_INVALID_INPUT;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return ntg::kLaunchErrorBase + (int)e;
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[dev];
    return NTG_OK;
}

int report(int code, const std::string &msg) {
    ntg::set_last_error(msg);
    return code;
}

int report_status(int st, const char *what) {
    if (st == 0) return NTG_OK;
    if (st >= ntg::kLaunchErrorBase)
        return report(NTG_ERROR_CUDA, std::string(what) + ": " + cudaGetErrorString((cudaError_t)(st - ntg::kLaunchErrorBase)));
    return report(st, what);
}

struct StepTable {
    float v[256];
};

const StepTable &srgb_steps_host() {
    static StepTable steps;
    static std::once_flag once;
    std::call_once(once, [] { ntg::build_srgb_steps(steps.v); });
    return steps;
}

// Writes the call's job record (and, when `steps` is non-null, the sRGB quantiser steps) into the
// scratch array from the launch's own arguments.
__global__ void k_put_record(ntg::EncJob j, ntg::EncJob *d_job, StepTable t, float *steps) {
    if (threadIdx.x == 0) *d_job = j;
    if (steps) steps[threadIdx.x] = t.v[threadIdx.x];
}

}  // namespace

extern "C" int ntg_encode_noalloc(ntg_context *ctx, int format, const float *d_rgba, int w, int h, int quality,
                                  int alpha_mode, int out_xform, float gamma, const float *cw, void *d_blocks,
                                  void *stream) {
    ntg::set_last_error("");
    if (!ctx || !d_rgba || !d_blocks || w <= 0 || h <= 0) return report(NTG_ERROR_INVALID_INPUT, "bad arguments");
    if ((size_t)w * (size_t)h > kMaxTexels)
        return report(NTG_ERROR_INVALID_INPUT, "ntg_encode_noalloc: level of " + std::to_string(w) + "x" +
                                                   std::to_string(h) + " texels exceeds its scratch limit of " +
                                                   std::to_string(kMaxTexels) + " texels (use ntg_encode)");
    if (format != NTG_FORMAT_BC1 && format != NTG_FORMAT_BC1A && format != NTG_FORMAT_BC3 && format != NTG_FORMAT_BC4 &&
        format != NTG_FORMAT_BC5)
        return report(NTG_ERROR_UNSUPPORTED_FEATURE, "format not supported (BC1, BC1a, BC3, BC4, BC5)");
    if (quality < 0 || quality > 3 || out_xform < 0 || out_xform > 2)
        return report(NTG_ERROR_INVALID_INPUT, "bad quality or colour transform");
    if (format == NTG_FORMAT_BC1A && quality == NTG_QUALITY_FASTEST)
        return report(NTG_ERROR_UNSUPPORTED_FEATURE, "BC1a at Fastest quality is not supported (use Normal or above)");
    // Surface::toGamma returns early for gamma == 1 (src/nvtt/Surface.cpp:1480-1488)
    const bool unit = std::fabs(gamma - 1.0f) <= 0.0001f * std::fmax(1.0f, std::fabs(gamma));
    if (out_xform == NTG_XFORM_GAMMA && unit) out_xform = NTG_XFORM_NONE;
    if (out_xform == NTG_XFORM_GAMMA && gamma != 2.2f)
        return report(NTG_ERROR_UNSUPPORTED_FEATURE, "power-law gamma other than 2.2 is not supported on the GPU");

    // the context's tables live on its device: run there whatever device the caller has current
    int st = ntg::use_context_device(ctx);
    if (st != NTG_OK) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned char *scratch = nullptr;
    st = scratch_address(&scratch);
    if (st != NTG_OK) return report_status(st, "cudaGetSymbolAddress of the scratch array");

    ntg::EncJob j;
    std::memset(&j, 0, sizeof j);
    j.w = w; j.h = h; j.bw = (w + 3) / 4;
    j.alpha_mode = alpha_mode;
    j.out = static_cast<uint8_t *>(d_blocks);
    j.first_block = 0;
    if (cw) { j.cw[0] = cw[0]; j.cw[1] = cw[1]; j.cw[2] = cw[2]; }
    else { j.cw[0] = j.cw[1] = j.cw[2] = 1.0f; }
    ntg::EncJob *d_job = reinterpret_cast<ntg::EncJob *>(scratch + kJobOffset);
    float *d_steps = reinterpret_cast<float *>(scratch + kStepsOffset);
    const bool quantise = format != NTG_FORMAT_BC1 && out_xform != NTG_XFORM_NONE;
    if (format == NTG_FORMAT_BC1) {
        j.rgba = d_rgba;
        j.out_xform = out_xform;  // applied per texel on the device
    } else if (quantise) {
        j.bgra = reinterpret_cast<uint32_t *>(scratch + kLevelOffset);
    } else {
        j.rgba = d_rgba;
    }
    const bool steps = quantise && out_xform == NTG_XFORM_SRGB;
    k_put_record<<<1, 256, 0, s>>>(j, d_job, srgb_steps_host(), steps ? d_steps : nullptr);
    st = ntg::launch_status();
    if (st != NTG_OK) return report_status(st, "job record");
    if (quantise) {
        // ColorBlock quantises the transformed level: build that level in the scratch array
        st = ntg::launch_quantize(d_rgba, (size_t)w * h, out_xform, d_steps, const_cast<uint32_t *>(j.bgra), s);
        if (st != NTG_OK) return report_status(st, "quantise level");
    }
    const long long nblocks = (long long)((w + 3) / 4) * ((h + 3) / 4);
    st = format == NTG_FORMAT_BC1    ? ntg::launch_bc1(d_job, 1, nblocks, quality, 0, s)
         : format == NTG_FORMAT_BC3  ? ntg::launch_bc3(d_job, 1, nblocks, quality, 0, s)
         : format == NTG_FORMAT_BC1A ? ntg::launch_bc1a(d_job, 1, nblocks, quality, 0, s)
         : format == NTG_FORMAT_BC4  ? ntg::launch_bc4(d_job, 1, nblocks, quality, 0, s)
                                     : ntg::launch_bc5(d_job, 1, nblocks, quality, 0, s);
    return report_status(st, "encoder launch");
}
