// C ABI of the GB300 texture path (include/ntg.h): contexts, table caches, chain planning and the
// launch sequences. Host code only; kernels live in the .cu translation units.
#include "ntg.h"

#include <cuda_runtime.h>

#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "ntg_host_tables.h"
#include "ntg_internal.h"

using namespace ntg;

namespace {

thread_local std::string g_error;

int fail(int code, const std::string &msg) {
    g_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(NTG_ERROR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Kernel launches the library has issued (each successful launcher call through launched()).
std::atomic<unsigned long long> g_launches{0};

// Maps a launcher status (ntg_internal.h) to an nvtt error code with a message.
int launched(int status, const char *what) {
    if (status == 0) {
        g_launches.fetch_add(1, std::memory_order_relaxed);
        return NTG_OK;
    }
    if (status >= kLaunchErrorBase) return cuda_fail((cudaError_t)(status - kLaunchErrorBase), what);
    return fail(status, what);
}

#define NTG_CUDA(call)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

#define NTG_TRY(call)                         \
    do {                                      \
        int r_ = (call);                      \
        if (r_ != NTG_OK) {                   \
            if (g_error.empty()) g_error = #call; \
            return r_;                        \
        }                                     \
    } while (0)

inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

struct Level { int w, h; };

std::vector<Level> chain_levels(int w, int h, int max_levels) {
    std::vector<Level> v;
    for (;;) {
        v.push_back({w, h});
        if ((max_levels > 0 && (int)v.size() >= max_levels) || (w == 1 && h == 1)) break;
        w = std::max(1, w / 2);
        h = std::max(1, h / 2);
    }
    return v;
}

int block_bytes(int format) {
    return format == NTG_FORMAT_BC1 || format == NTG_FORMAT_BC1A || format == NTG_FORMAT_BC4 ? 8 : 16;
}
bool known_format(int f) {
    return f == NTG_FORMAT_BC1 || f == NTG_FORMAT_BC1A || f == NTG_FORMAT_BC3 || f == NTG_FORMAT_BC4 || f == NTG_FORMAT_BC5;
}
long long blocks_of(int w, int h) { return (long long)((w + 3) / 4) * ((h + 3) / 4); }

// Filter defaults of Surface::buildNextMipmap (getDefaultFilterWidthAndParams,
// src/nvtt/Surface.cpp:1121-1141).
void filter_defaults(const ntg_chain_options &o, float &width, float p[2]) {
    width = o.filter_width;
    p[0] = o.params[0];
    p[1] = o.params[1];
    if (width > 0) return;
    if (o.filter == NTG_FILTER_BOX) width = 0.5f;
    else if (o.filter == NTG_FILTER_TRIANGLE) width = 1.0f;
    else { width = 3.0f; p[0] = 4.0f; p[1] = 1.0f; }
}

// True when buildNextMipmap takes FloatImage::fastDownSample (src/nvtt/Surface.cpp:1382-1386).
bool uses_fast_box(const ntg_chain_options &o, float width) {
    return o.alpha_mode != NTG_ALPHA_TRANSPARENCY && o.filter == NTG_FILTER_BOX && width == 0.5f;
}

// Device copy of one axis' polyphase table.
struct AxisTable {
    int ws = 0;
    float *d_w = nullptr;
    int *d_left = nullptr;
    std::vector<int> left;
    bool half = false;  // exact 2:1 with every output on the same taps (left[i] = left0 + 2i, equal rows)
    int left0 = 0;
    std::vector<float> row0;  // taps of output 0
};

// Launch shape of the 2:1 mip kernel (output rows per tile, threads per CTA).
struct MipTuning {
    int strip = 16;
    int threads = 512;
    long long tail_texels = 1024;  // a chain's remaining levels go to one tail CTA from a source this small
};

// Device copy of one 256-entry table set for an (in, out, gamma) transform combination.
struct XformTables {
    float *d_in = nullptr;       // input transform of 8-bit RGB values [256], then v / 255 for alpha [256]
    float *d_comp = nullptr;     // output(input(v/255)) for the BC1 level-0 path
    uint8_t *d_comp8 = nullptr;  // quantised composition (RGB) + alpha quantiser, 512 bytes
    float *d_steps = nullptr;    // sRGB quantiser steps (256 floats), then its bucket table (kSrgbBuckets bytes)
};

}  // namespace

struct ntg_context {
    int device = 0;
    HostTables tables;
    std::mutex mu;
    std::map<std::tuple<int, float, float, float, int, int>, AxisTable> axes;
    std::map<std::tuple<int, int, float>, XformTables> xforms;
    std::vector<void *> owned;  // every cudaMalloc of the caches
    uint8_t *ws = nullptr;      // grow-only workspace (stream-ordered)
    size_t ws_bytes = 0;
    EncJob *d_jobs = nullptr;   // job list of chain encodes
    int d_jobs_cap = 0;
    MipJob *d_mipjobs = nullptr;  // job lists of chain mip launches
    int d_mipjobs_cap = 0;
    MipTuning tune;
    bool profile = false;       // record phase events in chain calls
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};

    ~ntg_context() {
        cudaSetDevice(device);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        for (void *p : owned) cudaFree(p);
        if (ws) cudaFree(ws);
        if (d_jobs) cudaFree(d_jobs);
        if (d_mipjobs) cudaFree(d_mipjobs);
        if (slots) cudaFree(slots);
        for (int i = 0; i < 2; i++) {
            if (ev_in[i]) cudaEventDestroy(ev_in[i]);
            if (ev_done[i]) cudaEventDestroy(ev_done[i]);
            if (ev_out[i]) cudaEventDestroy(ev_out[i]);
        }
        if (up) cudaStreamDestroy(up);
        if (down) cudaStreamDestroy(down);
    }

    // copy streams and slots of ntg_compress_chains_host
    cudaStream_t up = nullptr, down = nullptr;
    cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_done[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr};
    uint8_t *slots = nullptr;
    size_t slot_in = 0, slot_out = 0;

    int copy_streams() {
        if (up) return NTG_OK;
        NTG_CUDA(cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking));
        NTG_CUDA(cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking));
        for (int i = 0; i < 2; i++) {
            NTG_CUDA(cudaEventCreateWithFlags(&ev_in[i], cudaEventDisableTiming));
            NTG_CUDA(cudaEventCreateWithFlags(&ev_done[i], cudaEventDisableTiming));
            NTG_CUDA(cudaEventCreateWithFlags(&ev_out[i], cudaEventDisableTiming));
        }
        return NTG_OK;
    }

    // Two input and two output slots of at least these sizes (synchronous growth, between calls).
    int host_slots(size_t in_bytes, size_t out_bytes) {
        in_bytes = align_up(in_bytes), out_bytes = align_up(out_bytes);
        if (slots && in_bytes <= slot_in && out_bytes <= slot_out) return NTG_OK;
        if (slots) { NTG_CUDA(cudaDeviceSynchronize()); cudaFree(slots); slots = nullptr; }
        slot_in = std::max(in_bytes, slot_in);
        slot_out = std::max(out_bytes, slot_out);
        NTG_CUDA(cudaMalloc((void **)&slots, 2 * (slot_in + slot_out)));
        return NTG_OK;
    }
    static size_t align_up(size_t b) { return (b + 255) / 256 * 256; }

    int alloc(void **p, size_t bytes) {
        NTG_CUDA(cudaMalloc(p, bytes));
        owned.push_back(*p);
        return NTG_OK;
    }

    int workspace(size_t bytes, cudaStream_t s, uint8_t **out) {
        if (bytes > ws_bytes) {
            if (ws) NTG_CUDA(cudaFreeAsync(ws, s));
            ws = nullptr;
            ws_bytes = 0;
            const size_t want = std::max(bytes, ws_bytes + ws_bytes / 4);
            NTG_CUDA(cudaMallocAsync((void **)&ws, want, s));
            ws_bytes = want;
        }
        *out = ws;
        return NTG_OK;
    }

    const AxisTable *axis(int filter, float width, float p0, float p1, int src, int dst) {
        auto key = std::make_tuple(filter, width, p0, p1, src, dst);
        auto it = axes.find(key);
        if (it != axes.end()) return &it->second;
        AxisTable t;
        t.ws = polyphase_window(width, src, dst);
        std::vector<float> w((size_t)t.ws * dst);
        t.left.resize(dst);
        build_polyphase(filter, width, p0, p1, src, dst, w.data(), t.left.data());
        t.left0 = t.left[0];
        t.row0.assign(w.begin(), w.begin() + t.ws);
        t.half = src == 2 * dst;
        for (int i = 1; i < dst && t.half; i++) {
            t.half = t.left[i] == t.left0 + 2 * i &&
                     std::memcmp(&w[(size_t)i * t.ws], &w[0], (size_t)t.ws * sizeof(float)) == 0;
        }
        if (alloc((void **)&t.d_w, w.size() * sizeof(float)) != NTG_OK) return nullptr;
        if (alloc((void **)&t.d_left, t.left.size() * sizeof(int)) != NTG_OK) return nullptr;
        if (cudaMemcpy(t.d_w, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
        if (cudaMemcpy(t.d_left, t.left.data(), t.left.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
            return nullptr;
        return &(axes[key] = t);
    }

    const XformTables *xform(int in_x, int out_x, float gamma) {
        auto key = std::make_tuple(in_x, out_x, gamma);
        auto it = xforms.find(key);
        if (it != xforms.end()) return &it->second;
        XformTables t;
        float lin[512], comp[256], steps[256];  // lin: input transform of RGB, then v / 255 for alpha
        uint8_t comp8[512];
        build_input_lut(in_x, gamma, tables, lin);
        for (int v = 0; v < 256; v++) lin[256 + v] = (float)v / 255.0f;
        build_composed_lut(in_x, out_x, gamma, tables, comp);
        build_composed_lut8(in_x, out_x, gamma, tables, comp8);
        // the quantiser steps, followed by the bucket table of the fast sRGB path
        static_assert(sizeof(float) * 256 % 4 == 0, "bucket table alignment");
        std::vector<uint8_t> quant(sizeof(float) * 256 + kSrgbBuckets);
        build_srgb_steps(steps);
        if (!build_srgb_buckets(steps, quant.data() + sizeof steps)) return nullptr;
        std::memcpy(quant.data(), steps, sizeof steps);
        if (alloc((void **)&t.d_in, sizeof lin) || alloc((void **)&t.d_comp, sizeof comp) ||
            alloc((void **)&t.d_comp8, sizeof comp8) || alloc((void **)&t.d_steps, quant.size()))
            return nullptr;
        if (cudaMemcpy(t.d_in, lin, sizeof lin, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(t.d_comp, comp, sizeof comp, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(t.d_comp8, comp8, sizeof comp8, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(t.d_steps, quant.data(), quant.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return nullptr;
        return &(xforms[key] = t);
    }
};

namespace {

// Largest source window (columns) any PTW-wide run of outputs of this axis can touch.
int max_window(const AxisTable &t, int tile) {
    int m = 0;
    const int n = (int)t.left.size();
    for (int i0 = 0; i0 < n; i0 += tile) {
        const int i1 = std::min(n, i0 + tile) - 1;
        m = std::max(m, t.left[i1] + t.ws - t.left[i0]);
    }
    return m;
}

int check_opts(const ntg_chain_options *opt) {
    if (!opt) return fail(NTG_ERROR_INVALID_INPUT, "null options");
    if (!known_format(opt->format))
        return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "format not supported (BC1, BC1a, BC3, BC4, BC5)");
    if (opt->quality < 0 || opt->quality > 3) return fail(NTG_ERROR_INVALID_INPUT, "bad quality");
    // FastCompressorDXT1a (QuickCompress::compressDXT1a, src/nvtt/QuickCompressDXT.cpp:716-763)
    // computes the indices of a block with transparent texels over 16 entries of an array that
    // holds only the opaque ones: the rest is uninitialised, so there is no output to reproduce.
    if (opt->format == NTG_FORMAT_BC1A && opt->quality == NTG_QUALITY_FASTEST)
        return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "BC1a at Fastest quality is not supported (use Normal or above)");
    if (opt->filter < 0 || opt->filter > 2) return fail(NTG_ERROR_INVALID_INPUT, "bad filter");
    if (opt->wrap < 0 || opt->wrap > 2) return fail(NTG_ERROR_INVALID_INPUT, "bad wrap mode");
    if (opt->in_xform < 0 || opt->in_xform > 2 || opt->out_xform < 0 || opt->out_xform > 2)
        return fail(NTG_ERROR_INVALID_INPUT, "bad colour transform");
    return NTG_OK;
}

void colour_weights(const ntg_chain_options &o, float cw[3]) {
    if (o.cw[0] == 0 && o.cw[1] == 0 && o.cw[2] == 0) { cw[0] = cw[1] = cw[2] = 1.0f; return; }
    cw[0] = o.cw[0]; cw[1] = o.cw[1]; cw[2] = o.cw[2];
}

// Workspace plan of one chain.
struct ChainPlan {
    std::vector<Level> lv;
    std::vector<size_t> f_off;   // float level offsets (bytes) in the workspace, SIZE_MAX = none
    std::vector<size_t> q_off;   // quantised BGRA8 level offsets, SIZE_MAX = none
    size_t bytes = 0;
    bool fast_box = false;
    float width = 0, p[2] = {0, 0};
};

const size_t NONE = (size_t)-1;

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

ChainPlan plan_chain(int w, int h, const ntg_chain_options &o, bool keep_level0_float) {
    ChainPlan P;
    P.lv = chain_levels(w, h, o.max_levels);
    filter_defaults(o, P.width, P.p);
    P.fast_box = uses_fast_box(o, P.width);
    const bool need_q = o.format != NTG_FORMAT_BC1;
    size_t off = 0;
    for (size_t l = 0; l < P.lv.size(); l++) {
        const size_t n = (size_t)P.lv[l].w * P.lv[l].h;
        if (l > 0 || P.fast_box || keep_level0_float) { P.f_off.push_back(off); off = align256(off + 16 * n); }
        else P.f_off.push_back(NONE);
        if (l > 0 && need_q) { P.q_off.push_back(off); off = align256(off + 4 * n); }
        else P.q_off.push_back(NONE);
    }
    P.bytes = off;
    return P;
}

struct MipKey {
    int kernel, ws, weighted, u8;
    // the BGRA8 tile kernel loads these once per launch: its jobs must share them
    const float *lut = nullptr, *steps = nullptr;
    std::vector<float> taps;
    bool operator<(const MipKey &o) const {
        return std::tie(kernel, ws, weighted, u8, lut, steps, taps) <
               std::tie(o.kernel, o.ws, o.weighted, o.u8, o.lut, o.steps, o.taps);
    }
};

// The mip job of one buildNextMipmap step from `src` (planar FP32; null = the BGRA8 input through
// the input table `lut`) of size S into `dst` of size D, and the kernel variant that runs it:
// the box path, the 2:1 kernel when both axes halve with uniform taps, else the general kernel.
int plan_step(ntg_context *ctx, const ntg_chain_options &o, float width, const float p[2], bool fast_box,
              const float *src, const uint32_t *bgra, const float *lut, Level S, Level D, float *dst, uint32_t *q,
              const float *steps, MipJob &J, MipKey &key) {
    std::memset(&J, 0, sizeof J);
    J.src = src; J.bgra8 = src ? nullptr : bgra; J.lut = lut;
    J.W = S.w; J.H = S.h; J.w = D.w; J.h = D.h;
    J.wrap = o.wrap; J.dst = dst; J.q_out = q; J.xform = o.out_xform; J.steps = steps;
    if (fast_box) {
        if (!src) return fail(NTG_ERROR_INVALID_INPUT, "box downsample needs an FP32 source level");
        key = {MIP_FAST_BOX, 0, 0, 0};
        return NTG_OK;
    }
    const AxisTable *ax = ctx->axis(o.filter, width, p[0], p[1], S.w, D.w);
    const AxisTable *ay = ctx->axis(o.filter, width, p[0], p[1], S.h, D.h);
    if (!ax || !ay) return fail(NTG_ERROR_CUDA, "polyphase table upload failed");
    J.wsx = ax->ws; J.wsy = ay->ws; J.kx = ax->d_w; J.ky = ay->d_w; J.lx = ax->d_left; J.ly = ay->d_left;
    const int weighted = o.weighted != 0, u8 = src == nullptr;
    if (u8 && ax->half && ay->half && ax->ws == ay->ws && ((ax->left0 % 4) + 4) % 4 == tile_u8_phase(ax->ws)) {
        J.cx = ax->left0; J.cy = ay->left0;
        J.tiles_x = (D.w + tile_u8_w() - 1) / tile_u8_w();
        J.strip = tile_u8_h();
        key = {MIP_TILE_U8, ax->ws, weighted, u8, lut, steps, ax->row0};
        key.taps.insert(key.taps.end(), ay->row0.begin(), ay->row0.end());
        return NTG_OK;
    }
    if (!u8 && !weighted && ax->half && ay->half && ax->ws == ay->ws && poly2x_supported(ax->ws) &&
        ((ax->left0 % 4) + 4) % 4 == tile_f32_phase(ax->ws)) {
        J.cx = ax->left0; J.cy = ay->left0;
        J.tiles_x = (D.w + tile_f32_w() - 1) / tile_f32_w();
        J.strip = tile_f32_h();
        key = {MIP_TILE_F32, ax->ws, 0, 0, nullptr, steps, ax->row0};
        key.taps.insert(key.taps.end(), ay->row0.begin(), ay->row0.end());
        return NTG_OK;
    }
    if (ax->half && ay->half && ax->ws == ay->ws && poly2x_supported(ax->ws)) {
        J.cx = ax->left0; J.cy = ay->left0;
        J.tiles_x = (D.w + 31) / 32;
        J.strip = ctx->tune.strip;
        key = {MIP_POLY2X, ax->ws, weighted, u8};
        return NTG_OK;
    }
    if (ax->ws > poly_max_window() || ay->ws > poly_max_window())
        return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "polyphase windows wider than 32 taps are not supported");
    J.tiles_x = (D.w + poly_tile_w() - 1) / poly_tile_w();
    J.rx_max = max_window(*ax, poly_tile_w());
    J.ry_max = max_window(*ay, poly_tile_h());
    key = {MIP_POLY, 0, weighted, u8};
    return NTG_OK;
}

long long mip_units(const MipKey &k, const MipJob &J) {
    if (k.kernel == MIP_FAST_BOX) return (long long)J.w * J.h;
    if (k.kernel == MIP_POLY2X || k.kernel == MIP_TILE_U8 || k.kernel == MIP_TILE_F32)
        return (long long)J.tiles_x * ((J.h + J.strip - 1) / J.strip);
    return (long long)J.tiles_x * ((J.h + poly_tile_h() - 1) / poly_tile_h());
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against the driver
// library); null when the driver does not provide it.
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (EncodeTiledFn) nullptr;
        }
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// The tensor map of an FP32 tile job's source level, its four planes as a W x H x 4 tensor whose box
// is one tile's source window. Left unset (tma = 0: the kernel copies with its threads) when the
// level's base or rows are not 16-byte aligned, the box is too large for the TMA, or the driver
// cannot encode it.
void encode_tile_map(MipJob &J, int ws) {
    J.tma = 0;
    const EncodeTiledFn enc = encode_tiled();
    const cuuint64_t row = (cuuint64_t)J.W * 4;
    const int bw = tile_box_cols(ws), bh = tile_box_rows(ws, J.strip);
    if (!enc || !J.src || ((uintptr_t)J.src & 15) || (row & 15) || bw > 256 || bh > 256 || J.W < 1 || J.H < 1) return;
    const cuuint64_t dims[3] = {(cuuint64_t)J.W, (cuuint64_t)J.H, 4};
    const cuuint64_t strides[2] = {row, row * (cuuint64_t)J.H};
    const cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 4};
    const cuuint32_t unit[3] = {1, 1, 1};
    const CUresult r = enc(&J.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(J.src), dims, strides, box, unit,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    J.tma = r == CUDA_SUCCESS ? 1 : 0;
}

// Where the TMA-staged FP32 tile kernel is used. Measured on GB300 against the one-tile-per-CTA
// kernel (k_tile2x) on Kaiser 2:1 steps: 15% faster from a 4096 x 4096 source (54 tiles per SM),
// even from 2048 x 2048 (13.5 tiles per SM), slower below: a persistent CTA with few tiles exposes
// the box latency, and windows at the level's edges (a third of the tiles of a 512 x 512 source)
// cost extra. So it takes a job from a source of at least kTmaMinSide texels in each direction,
// and only when such jobs give a launch at least kTmaMinTilesPerSm tiles per SM; every other FP32
// 2:1 job runs on k_tile2x.
constexpr int kTmaMinSide = 2048;
constexpr long long kTmaMinTilesPerSm = 16;

// Groups the jobs of one chain depth by kernel variant into launches; appends the jobs to `all`.
void group_launches(const std::vector<std::pair<MipKey, MipJob>> &items, const MipTuning &tune, std::vector<MipJob> &all,
                    std::vector<MipLaunch> &out) {
    std::map<MipKey, std::vector<MipJob>> groups;
    for (const auto &it : items) groups[it.first].push_back(it.second);
    // FP32 2:1 jobs the TMA tile kernel does not take go to k_tile2x (same tile width and job fields)
    for (auto it = groups.begin(); it != groups.end(); ++it) {
        if (it->first.kernel != MIP_TILE_F32) continue;
        std::vector<MipJob> big, small;
        long long tiles = 0;
        for (const MipJob &J : it->second) {
            if (std::min(J.W, J.H) >= kTmaMinSide) {
                big.push_back(J);
                tiles += (long long)J.tiles_x * ((J.h + tile_f32_h() - 1) / tile_f32_h());
            } else {
                small.push_back(J);
            }
        }
        if (tiles < kTmaMinTilesPerSm * 152) {
            small.insert(small.end(), big.begin(), big.end());
            big.clear();
        }
        if (!small.empty()) {
            MipKey k{MIP_POLY2X, it->first.ws, 0, 0};
            std::vector<MipJob> &dst = groups[k];
            dst.insert(dst.end(), small.begin(), small.end());
        }
        it->second.swap(big);
    }
    for (auto &g : groups) {
        if (g.second.empty()) continue;
        MipLaunch m;
        std::memset(&m, 0, sizeof m);
        m.kernel = g.first.kernel; m.ws = g.first.ws; m.weighted = g.first.weighted; m.u8 = g.first.u8;
        m.first_job = (int)all.size();
        m.njobs = (int)g.second.size();
        m.threads = tune.threads;
        int tile_h = std::min(m.kernel == MIP_TILE_F32 ? tile_f32_h() : 32, std::max(4, tune.strip));
        if (m.kernel == MIP_POLY2X || m.kernel == MIP_TILE_F32) {
            // lower tiles for small levels, so that the launch still spreads over the SMs
            for (;;) {
                long long n = 0;
                for (const MipJob &J : g.second) n += (long long)J.tiles_x * ((J.h + tile_h - 1) / tile_h);
                if (tile_h <= 4 || n >= 2 * 152) break;
                tile_h /= 2;
            }
            for (MipJob &J : g.second) J.strip = tile_h;
        }
        long long units = 0;
        int rx = 0, ry = 0;
        for (MipJob J : g.second) {
            J.first_unit = units;
            units += mip_units(g.first, J);
            if (m.kernel == MIP_TILE_F32) encode_tile_map(J, m.ws);
            rx = std::max(rx, J.rx_max);
            ry = std::max(ry, J.ry_max);
            all.push_back(J);
        }
        m.units = units;
        m.smem = m.kernel == MIP_POLY ? poly_smem_bytes(rx, ry) : m.kernel == MIP_POLY2X ? poly2x_smem_bytes(m.ws, tile_h) : 0;
        if (m.kernel == MIP_TILE_U8 || m.kernel == MIP_TILE_F32) m.threads = 1024;  // shared memory sized inside the launcher
        out.push_back(m);
    }
}

// First destination level of a chain that its tail launch computes (lv.size() = no tail).
size_t tail_start(const ChainPlan &P, const MipTuning &tune) {
    const long long limit = std::min<long long>(tune.tail_texels, tail_max_texels());
    for (size_t l = 1; l < P.lv.size(); l++) {
        const Level &S = P.lv[l - 1];
        // the X pass plane (H x max(1, W/2)) must fit the tail's half-size buffer as well: a 1-wide
        // level keeps its height there
        if ((long long)S.w * S.h <= limit && (long long)S.h * std::max(1, S.w / 2) <= tail_max_texels() / 2)
            return P.lv.size() - l >= 2 ? l : P.lv.size();
    }
    return P.lv.size();
}

// Mip job of destination level l of a chain.
int chain_step(ntg_context *ctx, const ChainPlan &P, size_t l, const uint32_t *d_bgra, const ntg_chain_options &o,
               const XformTables *xt, uint8_t *ws, MipJob &J, MipKey &key) {
    const float *src = P.f_off[l - 1] != NONE ? (const float *)(ws + P.f_off[l - 1]) : nullptr;
    uint32_t *q = P.q_off[l] != NONE ? (uint32_t *)(ws + P.q_off[l]) : nullptr;
    return plan_step(ctx, o, P.width, P.p, P.fast_box, src, d_bgra, xt->d_in, P.lv[l - 1], P.lv[l],
                     (float *)(ws + P.f_off[l]), q, xt->d_steps, J, key);
}

// Appends the tail jobs of a chain (levels from..end) to `all` as tail chain number `chain`.
int chain_tail(ntg_context *ctx, const ChainPlan &P, size_t from, const uint32_t *d_bgra, const ntg_chain_options &o,
               const XformTables *xt, uint8_t *ws, long long chain, std::vector<MipJob> &all) {
    const size_t first = all.size();
    for (size_t l = from; l < P.lv.size(); l++) {
        MipJob J;
        MipKey key;
        NTG_TRY(chain_step(ctx, P, l, d_bgra, o, xt, ws, J, key));
        J.first_unit = chain;
        all.push_back(J);
    }
    all[first].tiles_x = (int)(P.lv.size() - from);
    return NTG_OK;
}

// The mip steps of one chain: one stage (list of launches) per destination level, then one tail
// launch for the small levels.
int chain_stages(ntg_context *ctx, const ChainPlan &P, const uint32_t *d_bgra, const ntg_chain_options &o,
                 const XformTables *xt, uint8_t *ws, std::vector<MipJob> &all,
                 std::vector<std::vector<MipLaunch>> &stages) {
    const size_t tail = tail_start(P, ctx->tune);
    for (size_t l = 1; l < tail; l++) {
        std::vector<std::pair<MipKey, MipJob>> items(1);
        NTG_TRY(chain_step(ctx, P, l, d_bgra, o, xt, ws, items[0].second, items[0].first));
        stages.emplace_back();
        group_launches(items, ctx->tune, all, stages.back());
    }
    if (tail < P.lv.size()) {
        MipLaunch m;
        std::memset(&m, 0, sizeof m);
        m.kernel = MIP_TAIL;
        m.weighted = o.weighted != 0;
        m.first_job = (int)all.size();
        NTG_TRY(chain_tail(ctx, P, tail, d_bgra, o, xt, ws, 0, all));
        m.njobs = (int)all.size() - m.first_job;
        m.units = 1;
        stages.push_back({m});
    }
    return NTG_OK;
}

int upload_mip_jobs(ntg_context *ctx, const std::vector<MipJob> &jobs, cudaStream_t s) {
    if (jobs.empty()) return NTG_OK;
    if ((int)jobs.size() > ctx->d_mipjobs_cap) {
        if (ctx->d_mipjobs) NTG_CUDA(cudaFreeAsync(ctx->d_mipjobs, s));
        ctx->d_mipjobs = nullptr;
        const int cap = std::max<int>((int)jobs.size(), 64);
        NTG_CUDA(cudaMallocAsync((void **)&ctx->d_mipjobs, cap * sizeof(MipJob), s));
        ctx->d_mipjobs_cap = cap;
    }
    NTG_CUDA(cudaMemcpyAsync(ctx->d_mipjobs, jobs.data(), jobs.size() * sizeof(MipJob), cudaMemcpyHostToDevice, s));
    return NTG_OK;
}

int run_stages(const std::vector<std::vector<MipLaunch>> &stages, const MipJob *d_jobs, cudaStream_t s) {
    for (const auto &stage : stages)
        for (const MipLaunch &m : stage) NTG_TRY(launched(launch_mip(m, d_jobs, s), "mip filter"));
    return NTG_OK;
}

// Builds the levels of a chain into the workspace. Level 0 comes straight from the BGRA8 input:
// the fast box path materialises it as FP32, the polyphase path reads the bytes through the input
// transform table.
int build_levels(ntg_context *ctx, const ChainPlan &P, const uint32_t *d_bgra, const ntg_chain_options &o,
                 const XformTables *xt, uint8_t *ws, cudaStream_t s) {
    if (P.f_off[0] != NONE) {
        NTG_TRY(launched(launch_set_image(d_bgra, (size_t)P.lv[0].w * P.lv[0].h, xt->d_in, (float *)(ws + P.f_off[0]), s), "set image"));
    }
    std::vector<MipJob> all;
    std::vector<std::vector<MipLaunch>> stages;
    NTG_TRY(chain_stages(ctx, P, d_bgra, o, xt, ws, all, stages));
    NTG_TRY(upload_mip_jobs(ctx, all, s));
    return run_stages(stages, ctx->d_mipjobs, s);
}

int upload_jobs(ntg_context *ctx, const std::vector<EncJob> &jobs, cudaStream_t s) {
    if ((int)jobs.size() > ctx->d_jobs_cap) {
        if (ctx->d_jobs) NTG_CUDA(cudaFreeAsync(ctx->d_jobs, s));
        ctx->d_jobs = nullptr;
        NTG_CUDA(cudaMallocAsync((void **)&ctx->d_jobs, jobs.size() * sizeof(EncJob), s));
        ctx->d_jobs_cap = (int)jobs.size();
    }
    // pageable source: the copy is staged before the call returns, so `jobs` may go away
    NTG_CUDA(cudaMemcpyAsync(ctx->d_jobs, jobs.data(), jobs.size() * sizeof(EncJob), cudaMemcpyHostToDevice, s));
    return NTG_OK;
}

int launch_encode(int format, const EncJob *d_jobs, int njobs, long long nblocks, int quality, cudaStream_t s,
                  int threads = 0) {
    int r = format == NTG_FORMAT_BC1    ? launch_bc1(d_jobs, njobs, nblocks, quality, threads, s)
            : format == NTG_FORMAT_BC3  ? launch_bc3(d_jobs, njobs, nblocks, quality, threads, s)
            : format == NTG_FORMAT_BC1A ? launch_bc1a(d_jobs, njobs, nblocks, quality, threads, s)
            : format == NTG_FORMAT_BC4  ? launch_bc4(d_jobs, njobs, nblocks, quality, threads, s)
                                        : launch_bc5(d_jobs, njobs, nblocks, quality, threads, s);
    return launched(r, "encoder launch");
}

// Encode jobs of a chain: level 0 from the input bytes (through the composed transform tables),
// the other levels from the workspace.
void chain_jobs(const ChainPlan &P, const uint32_t *d_bgra, const ntg_chain_options &o, const XformTables *xt,
                uint8_t *ws, uint8_t *d_blocks, std::vector<EncJob> &jobs, long long &nblocks) {
    float cw[3];
    colour_weights(o, cw);
    size_t out_off = 0;
    for (size_t l = 0; l < P.lv.size(); l++) {
        const Level &L = P.lv[l];
        EncJob j;
        std::memset(&j, 0, sizeof j);
        j.w = L.w; j.h = L.h; j.bw = (L.w + 3) / 4;
        j.alpha_mode = o.alpha_mode;
        j.out_xform = o.out_xform;
        std::memcpy(j.cw, cw, sizeof cw);
        j.out = d_blocks + out_off;
        j.first_block = nblocks;
        if (o.format == NTG_FORMAT_BC1) {
            if (l == 0) { j.bgra = d_bgra; j.lut_f = xt->d_comp; }
            else j.rgba = (const float *)(ws + P.f_off[l]);
        } else {
            if (l == 0) { j.bgra = d_bgra; j.lut8 = xt->d_comp8; }
            else j.bgra = (const uint32_t *)(ws + P.q_off[l]);
        }
        jobs.push_back(j);
        nblocks += blocks_of(L.w, L.h);
        out_off += (size_t)block_bytes(o.format) * blocks_of(L.w, L.h);
    }
}

// Surface::toLinear/toGamma return early for gamma == 1 (nv::equal, src/nvtt/Surface.cpp:1470-1488).
ntg_chain_options normalized(const ntg_chain_options &o) {
    ntg_chain_options n = o;
    const float g = o.gamma;
    const bool unit = std::fabs(g - 1.0f) <= 0.0001f * std::max(1.0f, std::max(std::fabs(g), 1.0f));
    if (unit && n.in_xform == NTG_XFORM_GAMMA) n.in_xform = NTG_XFORM_NONE;
    if (unit && n.out_xform == NTG_XFORM_GAMMA) n.out_xform = NTG_XFORM_NONE;
    return n;
}

int ensure_device(ntg_context *ctx) {
    int cur = -1;
    NTG_CUDA(cudaGetDevice(&cur));
    if (cur != ctx->device) NTG_CUDA(cudaSetDevice(ctx->device));
    return NTG_OK;
}

}  // namespace

int ntg::use_context_device(ntg_context *ctx) { return ensure_device(ctx); }

void ntg::set_last_error(const std::string &msg) { g_error = msg; }

extern "C" {

int ntg_version(void) { return NTG_VERSION; }

const char *ntg_last_error_string(void) { return g_error.c_str(); }

unsigned long long ntg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

namespace {

// The sRGB curves' correction tables (ntg_device.cuh), built once per device by the first context on
// it: the host evaluates every float of both power segments with its libm, on all its cores; a kernel
// compares each with the device's result and keeps the 4-bit difference. Kept until the process ends.
std::mutex g_fix_mu;
uint8_t *g_fix_to[64], *g_fix_from[64];

void host_segment(int which, uint32_t first, uint32_t count, float *out) {
    const unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; t++) {
        pool.emplace_back([=] {
            const uint32_t lo = which ? kFromSrgbLo : kToSrgbLo;
            for (uint32_t k = (uint32_t)((uint64_t)count * t / nt); k < (uint32_t)((uint64_t)count * (t + 1) / nt); k++) {
                const uint32_t u = lo + first + k;
                float f;
                std::memcpy(&f, &u, 4);
                out[k] = which ? host_from_srgb(f) : host_to_srgb(f);
            }
        });
    }
    for (auto &th : pool) th.join();
}

int build_srgb_fix(int device) {
    std::lock_guard<std::mutex> lk(g_fix_mu);
    if (device < 0 || device >= 64) return fail(NTG_ERROR_INVALID_INPUT, "device index out of range");
    if (g_fix_to[device]) return NTG_OK;
    const uint32_t chunk = 1u << 24;
    std::vector<float> h(chunk);
    uint8_t *fix[2] = {nullptr, nullptr};
    float *d_chunk = nullptr;
    unsigned int *d_bad = nullptr;
    unsigned int bad = 0;
    int r = NTG_OK;
    if (cudaMalloc((void **)&fix[0], (kToSrgbCount + 1) / 2) != cudaSuccess ||
        cudaMalloc((void **)&fix[1], (kFromSrgbCount + 1) / 2) != cudaSuccess ||
        cudaMalloc((void **)&d_chunk, (size_t)chunk * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&d_bad, sizeof bad) != cudaSuccess || cudaMemset(d_bad, 0, sizeof bad) != cudaSuccess)
        r = cuda_fail(cudaGetLastError(), "sRGB correction tables");
    for (int which = 0; which < 2 && r == NTG_OK; which++) {
        const uint32_t n = which ? kFromSrgbCount : kToSrgbCount;
        for (uint32_t first = 0; first < n && r == NTG_OK; first += chunk) {
            const uint32_t count = std::min(chunk, n - first);
            host_segment(which, first, count, h.data());
            if (cudaMemcpy(d_chunk, h.data(), (size_t)count * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
                r = cuda_fail(cudaGetLastError(), "sRGB correction tables");
            else
                r = launched(launch_srgb_fix(d_chunk, first, count, which, fix[which], d_bad, nullptr), "sRGB correction tables");
        }
    }
    if (r == NTG_OK && cudaMemcpy(&bad, d_bad, sizeof bad, cudaMemcpyDeviceToHost) != cudaSuccess)
        r = cuda_fail(cudaGetLastError(), "sRGB correction tables");
    if (r == NTG_OK && bad) r = fail(NTG_ERROR_CUDA, "device sRGB curve outside the correction range");
    if (r == NTG_OK && (set_srgb_fix_mip(fix[0], fix[1]) || set_srgb_fix_bc1(fix[0])))
        r = cuda_fail(cudaGetLastError(), "sRGB correction tables");
    cudaFree(d_chunk);
    cudaFree(d_bad);
    if (r != NTG_OK) {
        cudaFree(fix[0]);
        cudaFree(fix[1]);
        return r;
    }
    g_fix_to[device] = fix[0];
    g_fix_from[device] = fix[1];
    return NTG_OK;
}

}  // namespace

int ntg_create(int device, ntg_context **out) {
    g_error.clear();
    if (!out) return fail(NTG_ERROR_INVALID_INPUT, "null output");
    int count = 0;
    NTG_CUDA(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) return fail(NTG_ERROR_INVALID_INPUT, "no such CUDA device");
    NTG_CUDA(cudaSetDevice(device));
    std::unique_ptr<ntg_context> ctx(new ntg_context);
    ctx->device = device;
    build_device_tables(ctx->tables);
    NTG_TRY(upload_tables_bc1(ctx->tables));
    NTG_TRY(upload_tables_bc3(ctx->tables));
    NTG_TRY(upload_tables_mip(ctx->tables));
    NTG_TRY(upload_tables_decode(ctx->tables));
    NTG_TRY(build_srgb_fix(device));
    *out = ctx.release();
    return NTG_OK;
}

int ntg_destroy(ntg_context *ctx) {
    if (!ctx) return NTG_OK;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    delete ctx;
    return NTG_OK;
}

int ntg_chain_levels(int w, int h, int max_levels) {
    if (w <= 0 || h <= 0) return 0;
    return (int)chain_levels(w, h, max_levels).size();
}

size_t ntg_chain_bytes(int w, int h, const ntg_chain_options *opt) {
    if (!opt || w <= 0 || h <= 0) return 0;
    size_t b = 0;
    for (const Level &L : chain_levels(w, h, opt->max_levels)) b += (size_t)block_bytes(opt->format) * blocks_of(L.w, L.h);
    return b;
}

int ntg_set_image_bgra8(ntg_context *ctx, const void *d_bgra, int w, int h, int in_xform, float gamma, float *d_rgba,
                        void *stream) {
    g_error.clear();
    if (!ctx || !d_bgra || !d_rgba || w <= 0 || h <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    const XformTables *xt = ctx->xform(in_xform, NTG_XFORM_NONE, gamma);
    if (!xt) return fail(NTG_ERROR_CUDA, "table upload failed");
    return launched(launch_set_image((const uint32_t *)d_bgra, (size_t)w * h, xt->d_in, d_rgba, S(stream)), "set image");
}

int ntg_mip_level(ntg_context *ctx, const float *d_src, int w, int h, float *d_dst, int filter, float width,
                  const float *params, int wrap, int alpha_mode, int weighted, void *stream) {
    g_error.clear();
    if (!ctx || !d_src || !d_dst || w <= 0 || h <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    if (w == 1 && h == 1) return fail(NTG_ERROR_INVALID_INPUT, "no smaller level (canMakeNextMipmap)");
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    ntg_chain_options o;
    std::memset(&o, 0, sizeof o);
    o.filter = filter; o.filter_width = width;
    if (params) { o.params[0] = params[0]; o.params[1] = params[1]; }
    o.wrap = wrap; o.alpha_mode = alpha_mode; o.weighted = weighted;
    float fw, p[2];
    filter_defaults(o, fw, p);
    const int dw = std::max(1, w / 2), dh = std::max(1, h / 2);
    std::vector<std::pair<MipKey, MipJob>> items(1);
    NTG_TRY(plan_step(ctx, o, fw, p, uses_fast_box(o, fw) && !weighted, d_src, nullptr, nullptr, Level{w, h},
                      Level{dw, dh}, d_dst, nullptr, nullptr, items[0].second, items[0].first));
    std::vector<MipJob> all;
    std::vector<std::vector<MipLaunch>> stages(1);
    group_launches(items, ctx->tune, all, stages[0]);
    cudaStream_t s = S(stream);
    NTG_TRY(upload_mip_jobs(ctx, all, s));
    return run_stages(stages, ctx->d_mipjobs, s);
}

int ntg_resize(ntg_context *ctx, const float *d_src, int w, int h, float *d_dst, int dw, int dh, int filter, float width,
               const float *params, int wrap, int alpha_mode, void *stream) {
    g_error.clear();
    if (!ctx || !d_src || !d_dst || w <= 0 || h <= 0 || dw <= 0 || dh <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    if (filter < 0 || filter > 2) return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "resize filter not supported (box, triangle, kaiser)");
    if (wrap < 0 || wrap > 2 || alpha_mode < 0 || alpha_mode > 2) return fail(NTG_ERROR_INVALID_INPUT, "bad wrap or alpha mode");
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    cudaStream_t s = S(stream);
    if (dw == w && dh == h) {  // Surface::resize returns early: the image is unchanged
        if (d_dst != d_src) NTG_CUDA(cudaMemcpyAsync(d_dst, d_src, (size_t)w * h * 4 * sizeof(float), cudaMemcpyDeviceToDevice, s));
        return NTG_OK;
    }
    ntg_chain_options o;
    std::memset(&o, 0, sizeof o);
    o.filter = filter; o.filter_width = width;
    if (params) { o.params[0] = params[0]; o.params[1] = params[1]; }
    float fw, p[2];
    filter_defaults(o, fw, p);
    const AxisTable *ax = ctx->axis(filter, fw, p[0], p[1], w, dw);
    const AxisTable *ay = ctx->axis(filter, fw, p[0], p[1], h, dh);
    if (!ax || !ay) return fail(NTG_ERROR_CUDA, "polyphase table upload failed");
    uint8_t *tmp = nullptr;
    NTG_TRY(ctx->workspace((size_t)dw * h * 4 * sizeof(float), s, &tmp));
    return launched(launch_resize(d_src, w, h, (float *)tmp, dw, dh, ax->d_w, ax->d_left, ax->ws, ay->d_w, ay->d_left,
                                  ay->ws, wrap, d_dst, s), "resize");
}

int ntg_mip_set_wait_limit(ntg_context *ctx, int polls) {
    g_error.clear();
    if (!ctx) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    NTG_CUDA(cudaDeviceSynchronize());
    const int st = set_mip_wait_polls(polls < 0 ? 1 << 22 : polls);
    if (st) return cuda_fail((cudaError_t)(st - kLaunchErrorBase), "mip wait limit");
    NTG_CUDA(cudaDeviceSynchronize());
    return NTG_OK;
}

int ntg_mip_status(ntg_context *ctx, int *gave_up) {
    g_error.clear();
    if (!ctx || !gave_up) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    NTG_CUDA(cudaDeviceSynchronize());
    const int st = read_mip_status(gave_up);
    return st ? cuda_fail((cudaError_t)(st - kLaunchErrorBase), "mip status") : NTG_OK;
}

int ntg_selftest_srgb_quantizer(ntg_context *ctx, unsigned long long *mismatches) {
    g_error.clear();
    if (!ctx || !mismatches) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    const XformTables *xt = ctx->xform(NTG_XFORM_NONE, NTG_XFORM_SRGB, 2.2f);
    if (!xt) return fail(NTG_ERROR_CUDA, "table upload failed");
    unsigned long long *d = nullptr;
    NTG_CUDA(cudaMalloc((void **)&d, sizeof *d));
    int r = launched(launch_check_srgb(xt->d_steps, d, nullptr), "quantiser check");
    if (r == NTG_OK && cudaMemcpy(mismatches, d, sizeof *d, cudaMemcpyDeviceToHost) != cudaSuccess) r = cuda_fail(cudaGetLastError(), "copy");
    cudaFree(d);
    return r;
}

// nv::getTargetExtent (src/nvtt/Surface.cpp:220-326) for 2D textures, cube maps and arrays, no shape
// restriction, with the rounding helpers of src/nvtt/Surface.cpp:60-105. Its else-if chain tests
// RoundMode_ToNextMultipleOfFour twice, so RoundMode_ToNearestMultipleOfFour leaves the extents
// unchanged; kept that way.
int ntg_target_extent_ex(int w, int h, int max_extent, int round_mode, int texture_type, int *out_w, int *out_h) {
    g_error.clear();
    if (w <= 0 || h <= 0 || !out_w || !out_h || round_mode < 0 || round_mode > 6 || texture_type < 0 || texture_type > 3)
        return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    if (texture_type == 2) return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "3D textures are not supported");
    auto next_pow2 = [](unsigned x) {
        x--;
        x |= x >> 1; x |= x >> 2; x |= x >> 4; x |= x >> 8; x |= x >> 16;
        return x + 1;
    };
    auto prev_pow2 = [&](unsigned v) { return next_pow2(v + 1) / 2; };
    auto nearest_pow2 = [&](unsigned v) {
        const unsigned up = next_pow2(v), down = prev_pow2(v);
        return up - v <= v - down ? up : down;
    };
    if (round_mode != 0 && max_extent > 0) max_extent = (int)prev_pow2((unsigned)max_extent);
    const int m = std::max(w, h);
    if (max_extent > 0 && m > max_extent) {
        w = std::max((w * max_extent) / m, 1);
        h = std::max((h * max_extent) / m, 1);
    }
    if (texture_type == 1) w = h = (w + h) / 2;  // a cube map's faces are square
    if (round_mode == 1) { w = (int)next_pow2((unsigned)w); h = (int)next_pow2((unsigned)h); }
    else if (round_mode == 2) { w = (int)nearest_pow2((unsigned)w); h = (int)nearest_pow2((unsigned)h); }
    else if (round_mode == 3) { w = (int)prev_pow2((unsigned)w); h = (int)prev_pow2((unsigned)h); }
    else if (round_mode == 4) { w = (w + 3) & ~3; h = (h + 3) & ~3; }
    else if (round_mode == 6) { w &= ~3; h &= ~3; }
    *out_w = w;
    *out_h = h;
    return NTG_OK;
}

int ntg_target_extent(int w, int h, int max_extent, int round_mode, int *out_w, int *out_h) {
    return ntg_target_extent_ex(w, h, max_extent, round_mode, 0, out_w, out_h);
}

int ntg_encode(ntg_context *ctx, int format, const float *d_rgba, int w, int h, int quality, int alpha_mode,
               int out_xform, float gamma, const float *cw, void *d_blocks, void *stream) {
    g_error.clear();
    if (!ctx || !d_rgba || !d_blocks || w <= 0 || h <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    ntg_chain_options o0;
    std::memset(&o0, 0, sizeof o0);
    o0.format = format; o0.quality = quality; o0.out_xform = out_xform; o0.gamma = gamma; o0.alpha_mode = alpha_mode;
    NTG_TRY(check_opts(&o0));
    const ntg_chain_options o = normalized(o0);
    out_xform = o.out_xform;
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    cudaStream_t s = S(stream);
    uint32_t *q = nullptr;
    if (format != NTG_FORMAT_BC1 && out_xform != NTG_XFORM_NONE) {
        // the 8-bit formats quantise the transformed level first (ColorBlock::init on the toGamma'd copy)
        const XformTables *xt = ctx->xform(NTG_XFORM_NONE, out_xform, gamma);
        if (!xt) return fail(NTG_ERROR_CUDA, "table upload failed");
        if (out_xform == NTG_XFORM_GAMMA && gamma != 2.2f)
            return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "power-law gamma other than 2.2 is not supported on the GPU");
        uint8_t *ws = nullptr;
        NTG_TRY(ctx->workspace((size_t)w * h * 4, s, &ws));
        q = (uint32_t *)ws;
        NTG_TRY(launched(launch_quantize(d_rgba, (size_t)w * h, out_xform, xt->d_steps, q, s), "quantise level"));
    } else if (format == NTG_FORMAT_BC1 && out_xform == NTG_XFORM_GAMMA && gamma != 2.2f) {
        return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "power-law gamma other than 2.2 is not supported on the GPU");
    }
    EncJob j;
    std::memset(&j, 0, sizeof j);
    j.w = w; j.h = h; j.bw = (w + 3) / 4;
    j.alpha_mode = alpha_mode;
    j.out_xform = format == NTG_FORMAT_BC1 ? out_xform : NTG_XFORM_NONE;
    if (format == NTG_FORMAT_BC1) j.rgba = d_rgba;
    else if (q) j.bgra = q;
    else j.rgba = d_rgba;
    if (cw) { j.cw[0] = cw[0]; j.cw[1] = cw[1]; j.cw[2] = cw[2]; }
    else { j.cw[0] = j.cw[1] = j.cw[2] = 1.0f; }
    j.out = (uint8_t *)d_blocks;
    j.first_block = 0;
    std::vector<EncJob> jobs(1, j);
    NTG_TRY(upload_jobs(ctx, jobs, s));
    return launch_encode(format, ctx->d_jobs, 1, blocks_of(w, h), quality, s);
}

static int chain_common(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt_in,
                        void *d_blocks, float *d_levels, void *stream) {
    NTG_TRY(check_opts(opt_in));
    const ntg_chain_options norm = normalized(*opt_in);
    const ntg_chain_options *opt = &norm;
    if (!ctx || !d_bgra || w <= 0 || h <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    if ((opt->in_xform == NTG_XFORM_GAMMA || opt->out_xform == NTG_XFORM_GAMMA) && opt->gamma != 2.2f &&
        std::fabs(opt->gamma - 1.0f) > 0.0001f * std::max(1.0f, std::fabs(opt->gamma)))
        return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "power-law gamma other than 2.2 is not supported on the GPU");
    NTG_TRY(ensure_device(ctx));
    cudaStream_t s = S(stream);
    const ChainPlan P = plan_chain(w, h, *opt, d_levels != nullptr);
    const XformTables *xt = ctx->xform(opt->in_xform, opt->out_xform, opt->gamma);
    if (!xt) return fail(NTG_ERROR_CUDA, "table upload failed");
    uint8_t *ws = nullptr;
    NTG_TRY(ctx->workspace(std::max<size_t>(P.bytes, 256), s, &ws));
    if (d_levels && P.f_off[0] != NONE && !P.fast_box) {
        NTG_TRY(launched(launch_set_image((const uint32_t *)d_bgra, (size_t)w * h, xt->d_in, (float *)(ws + P.f_off[0]), s), "set image"));
    }
    // The mip levels, then one encoder launch over every level. (Encoding level 0 beside the mip
    // launches, on a lower-priority stream, measured slower: the encoder's CTAs hold nearly all of an
    // SM's registers for ~0.4 ms each, so every mip launch first waits for SMs to drain.)
    if (ctx->profile) NTG_CUDA(cudaEventRecord(ctx->ev[0], s));
    NTG_TRY(build_levels(ctx, P, (const uint32_t *)d_bgra, *opt, xt, ws, s));
    if (ctx->profile) NTG_CUDA(cudaEventRecord(ctx->ev[1], s));
    if (d_levels) {
        size_t off = 0;
        for (size_t l = 0; l < P.lv.size(); l++) {
            const size_t n = 4 * (size_t)P.lv[l].w * P.lv[l].h;
            NTG_CUDA(cudaMemcpyAsync(d_levels + off, ws + P.f_off[l], n * sizeof(float), cudaMemcpyDeviceToDevice, s));
            off += n;
        }
    }
    if (d_blocks) {
        std::vector<EncJob> jobs;
        long long nblocks = 0;
        chain_jobs(P, (const uint32_t *)d_bgra, *opt, xt, ws, (uint8_t *)d_blocks, jobs, nblocks);
        NTG_TRY(upload_jobs(ctx, jobs, s));
        NTG_TRY(launch_encode(opt->format, ctx->d_jobs, (int)jobs.size(), nblocks, opt->quality, s));
    }
    if (ctx->profile) NTG_CUDA(cudaEventRecord(ctx->ev[2], s));
    return NTG_OK;
}

// True when every job has the default colour weights (1, 1, 1): the BC3 fit then skips the metric.
static bool unit_weights(const std::vector<EncJob> &jobs) {
    for (const EncJob &j : jobs)
        if (j.cw[0] != 1.0f || j.cw[1] != 1.0f || j.cw[2] != 1.0f) return false;
    return true;
}

// The learned endpoint proposal over a chain (BC1, BC3): the network's inputs for every block of every
// level, training targets from the plain fit's blocks, or the learned encode (inputs -> network ->
// pruned fit -> full fit for the listed blocks), all on one stream without host round trips.
enum { LEARN_FEATURES = 0, LEARN_TARGETS = 1, LEARN_ENCODE = 2 };

static int chain_learned(ntg_context *ctx, ntg_mlp *mlp, const void *d_bgra, int w, int h, const ntg_chain_options *opt_in,
                         int mode, void *d_blocks, float *d_aux, int radius, float margin, unsigned long long *h_stats,
                         void *stream, const float *d_proposals = nullptr) {
    NTG_TRY(check_opts(opt_in));
    if (!ctx || !d_bgra || w <= 0 || h <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    const bool bc3 = opt_in->format == NTG_FORMAT_BC3;
    if (opt_in->format != NTG_FORMAT_BC1 && !bc3)
        return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "the learned proposal is for BC1 and BC3");
    if (mode == LEARN_ENCODE && ((!mlp && !d_proposals) || opt_in->quality != NTG_QUALITY_NORMAL || radius < 0))
        return fail(NTG_ERROR_INVALID_INPUT, "learned encode needs a network, Quality_Normal and radius >= 0");
    const ntg_chain_options norm = normalized(*opt_in);
    const ntg_chain_options *opt = &norm;
    if ((opt->in_xform == NTG_XFORM_GAMMA || opt->out_xform == NTG_XFORM_GAMMA) && opt->gamma != 2.2f)
        return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "power-law gamma other than 2.2 is not supported on the GPU");
    NTG_TRY(ensure_device(ctx));
    cudaStream_t s = S(stream);
    const ChainPlan P = plan_chain(w, h, *opt, false);
    const XformTables *xt = ctx->xform(opt->in_xform, opt->out_xform, opt->gamma);
    if (!xt) return fail(NTG_ERROR_CUDA, "table upload failed");
    long long nb = 0;
    for (const Level &L : P.lv) nb += blocks_of(L.w, L.h);
    const size_t base = align256(std::max<size_t>(P.bytes, 256));
    const size_t xoff = base, yoff = align256(xoff + (size_t)nb * 48 * 4), loff = align256(yoff + (size_t)nb * 16 * 4),
                 soff = align256(loff + (size_t)nb * 8);
    const size_t need = mode == LEARN_ENCODE ? soff + 256 : base;
    uint8_t *ws = nullptr;
    NTG_TRY(ctx->workspace(need, s, &ws));
    NTG_TRY(build_levels(ctx, P, (const uint32_t *)d_bgra, *opt, xt, ws, s));
    std::vector<EncJob> jobs;
    long long nblocks = 0;
    chain_jobs(P, (const uint32_t *)d_bgra, *opt, xt, ws, (uint8_t *)d_blocks, jobs, nblocks);
    NTG_TRY(upload_jobs(ctx, jobs, s));
    const int nj = (int)jobs.size();
    if (mode == LEARN_FEATURES)
        return launched(bc3 ? launch_bc3_features(ctx->d_jobs, nj, nblocks, d_aux, s)
                            : launch_bc1_features(ctx->d_jobs, nj, nblocks, d_aux, s), "block features");
    if (mode == LEARN_TARGETS)
        return launched(bc3 ? launch_bc3_targets(ctx->d_jobs, nj, nblocks, d_aux, s)
                            : launch_bc1_targets(ctx->d_jobs, nj, nblocks, d_aux, s), "fit targets");
    float *x = (float *)(ws + xoff), *y = (float *)(ws + yoff);
    long long *list = (long long *)(ws + loff);
    unsigned long long *stats = (unsigned long long *)(ws + soff);
    if (d_proposals) {
        y = const_cast<float *>(d_proposals);
    } else {
        NTG_TRY(launched(bc3 ? launch_bc3_features(ctx->d_jobs, nj, nblocks, x, s)
                             : launch_bc1_features(ctx->d_jobs, nj, nblocks, x, s), "block features"));
        int r = mlp_forward_device(mlp, x, nblocks, y, s);
        if (r) return fail(r, std::string("proposal network: ") + ntg_last_error_string());
    }
    NTG_CUDA(cudaMemsetAsync(stats, 0, 3 * sizeof(unsigned long long), s));
    if (bc3) {
        NTG_TRY(launched(launch_bc3_learned(ctx->d_jobs, nj, nblocks, y, radius, margin, unit_weights(jobs), list, stats, s),
                         "pruned fit"));
        NTG_TRY(launched(launch_bc3_list(ctx->d_jobs, nj, list, stats + 1, nblocks, s), "full fit of the listed blocks"));
    } else {
        NTG_TRY(launched(launch_bc1_learned(ctx->d_jobs, nj, nblocks, y, radius, margin, list, stats, s), "pruned fit"));
        NTG_TRY(launched(launch_bc1_list(ctx->d_jobs, nj, list, stats + 1, nblocks, s), "full fit of the listed blocks"));
    }
    if (h_stats) {
        NTG_CUDA(cudaMemcpyAsync(h_stats, stats, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        NTG_CUDA(cudaStreamSynchronize(s));
    }
    return NTG_OK;
}

int ntg_compress_chain_proposed(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt,
                                const float *d_proposals, int radius, float margin, void *d_blocks, unsigned long long *stats,
                                void *stream) {
    g_error.clear();
    if (!ctx || !d_blocks || !d_proposals) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return chain_learned(ctx, nullptr, d_bgra, w, h, opt, LEARN_ENCODE, d_blocks, nullptr, radius, margin, stats, stream,
                         d_proposals);
}

int ntg_chain_features(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt, float *d_x,
                       void *stream) {
    g_error.clear();
    if (!ctx || !d_x) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return chain_learned(ctx, nullptr, d_bgra, w, h, opt, LEARN_FEATURES, nullptr, d_x, 0, 0, nullptr, stream);
}

int ntg_chain_targets(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt,
                      const void *d_blocks, float *d_t, void *stream) {
    g_error.clear();
    if (!ctx || !d_blocks || !d_t) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return chain_learned(ctx, nullptr, d_bgra, w, h, opt, LEARN_TARGETS, const_cast<void *>(d_blocks), d_t, 0, 0, nullptr,
                         stream);
}

int ntg_compress_chain_learned(ntg_context *ctx, ntg_mlp *mlp, const void *d_bgra, int w, int h,
                               const ntg_chain_options *opt, int radius, float margin, void *d_blocks,
                               unsigned long long *stats, void *stream) {
    g_error.clear();
    if (!ctx || !d_blocks) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->profile) NTG_CUDA(cudaEventRecord(ctx->ev[0], S(stream)));
    int r = chain_learned(ctx, mlp, d_bgra, w, h, opt, LEARN_ENCODE, d_blocks, nullptr, radius, margin, stats, stream);
    if (r == NTG_OK && ctx->profile) {
        NTG_CUDA(cudaEventRecord(ctx->ev[1], S(stream)));
        NTG_CUDA(cudaEventRecord(ctx->ev[2], S(stream)));
    }
    return r;
}

int ntg_compress_chain(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt, void *d_blocks,
                       void *stream) {
    g_error.clear();
    if (!d_blocks) return fail(NTG_ERROR_INVALID_INPUT, "null output");
    if (!ctx) return fail(NTG_ERROR_INVALID_INPUT, "null context");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return chain_common(ctx, d_bgra, w, h, opt, d_blocks, nullptr, stream);
}

int ntg_mip_chain(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt, float *d_levels,
                  void *stream) {
    g_error.clear();
    if (!d_levels) return fail(NTG_ERROR_INVALID_INPUT, "null output");
    if (!ctx) return fail(NTG_ERROR_INVALID_INPUT, "null context");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return chain_common(ctx, d_bgra, w, h, opt, nullptr, d_levels, stream);
}

int ntg_compress_chain_host(ntg_context *ctx, const void *h_bgra, int w, int h, const ntg_chain_options *opt,
                            void *h_blocks, void *stream) {
    g_error.clear();
    if (!ctx || !h_bgra || !h_blocks || !opt || w <= 0 || h <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    NTG_TRY(check_opts(opt));
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    cudaStream_t s = S(stream);
    const size_t in_bytes = (size_t)w * h * 4, out_bytes = ntg_chain_bytes(w, h, opt);
    uint8_t *io = nullptr;
    NTG_CUDA(cudaMallocAsync((void **)&io, align256(in_bytes) + out_bytes, s));
    int r = NTG_OK;
    if (cudaMemcpyAsync(io, h_bgra, in_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) r = cuda_fail(cudaGetLastError(), "copy in");
    if (r == NTG_OK) r = chain_common(ctx, io, w, h, opt, io + align256(in_bytes), nullptr, stream);
    if (r == NTG_OK && cudaMemcpyAsync(h_blocks, io + align256(in_bytes), out_bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        r = cuda_fail(cudaGetLastError(), "copy out");
    cudaFreeAsync(io, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (r == NTG_OK && e != cudaSuccess) r = cuda_fail(e, "stream");
    return r;
}

int ntg_compress_chains_host(ntg_context *ctx, int n, const void *const *h_bgra, int w, int h,
                             const ntg_chain_options *opt, void *const *h_blocks, void *stream) {
    g_error.clear();
    if (!ctx || n < 0 || (n > 0 && (!h_bgra || !h_blocks)) || !opt || w <= 0 || h <= 0)
        return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    for (int i = 0; i < n; i++)
        if (!h_bgra[i] || !h_blocks[i]) return fail(NTG_ERROR_INVALID_INPUT, "null image or output");
    NTG_TRY(check_opts(opt));
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    NTG_TRY(ctx->copy_streams());
    const size_t in_bytes = (size_t)w * h * 4, out_bytes = ntg_chain_bytes(w, h, opt);
    NTG_TRY(ctx->host_slots(in_bytes, out_bytes));
    cudaStream_t s = S(stream);
    uint8_t *in[2] = {ctx->slots, ctx->slots + ctx->slot_in};
    uint8_t *out[2] = {ctx->slots + 2 * ctx->slot_in, ctx->slots + 2 * ctx->slot_in + ctx->slot_out};
    // the slots' previous users (an earlier call) are done: they all ended with this call's streams drained
    auto copy_in = [&](int i) -> int {
        const int k = i & 1;
        if (i >= 2) NTG_CUDA(cudaStreamWaitEvent(ctx->up, ctx->ev_done[k], 0));      // chain i-2 read in[k]
        NTG_CUDA(cudaMemcpyAsync(in[k], h_bgra[i], in_bytes, cudaMemcpyHostToDevice, ctx->up));
        NTG_CUDA(cudaEventRecord(ctx->ev_in[k], ctx->up));
        return NTG_OK;
    };
    // the next image's copy-in is issued before this chain's copy-out: a copy-out to memory the driver
    // does not treat as page-locked returns only once it is done, and must not hold back the copy-in
    if (n > 0) NTG_TRY(copy_in(0));
    for (int i = 0; i < n; i++) {
        const int k = i & 1;
        NTG_CUDA(cudaStreamWaitEvent(s, ctx->ev_in[k], 0));
        if (i >= 2) NTG_CUDA(cudaStreamWaitEvent(s, ctx->ev_out[k], 0));             // blocks of i-2 copied out
        NTG_TRY(chain_common(ctx, in[k], w, h, opt, out[k], nullptr, s));
        NTG_CUDA(cudaEventRecord(ctx->ev_done[k], s));
        if (i + 1 < n) NTG_TRY(copy_in(i + 1));
        NTG_CUDA(cudaStreamWaitEvent(ctx->down, ctx->ev_done[k], 0));
        NTG_CUDA(cudaMemcpyAsync(h_blocks[i], out[k], out_bytes, cudaMemcpyDeviceToHost, ctx->down));
        NTG_CUDA(cudaEventRecord(ctx->ev_out[k], ctx->down));
    }
    NTG_CUDA(cudaStreamSynchronize(ctx->up));
    NTG_CUDA(cudaStreamSynchronize(s));
    NTG_CUDA(cudaStreamSynchronize(ctx->down));
    return NTG_OK;
}

int ntg_host_polyphase(int filter, float width, const float *params, int src_len, int dst_len, float *weights,
                       int *lefts, int capacity) {
    const int ws = polyphase_window(width, src_len, dst_len);
    if (weights && lefts && (long long)ws * dst_len <= capacity)
        build_polyphase(filter, width, params ? params[0] : 0.0f, params ? params[1] : 0.0f, src_len, dst_len, weights, lefts);
    return ws;
}

int ntg_host_transform_tables(int in_xform, int out_xform, float gamma, float *lut_in, float *lut_composed,
                              unsigned char *lut8, float *srgb_steps) {
    HostTables t;
    build_device_tables(t);
    if (lut_in) build_input_lut(in_xform, gamma, t, lut_in);
    if (lut_composed) build_composed_lut(in_xform, out_xform, gamma, t, lut_composed);
    if (lut8) build_composed_lut8(in_xform, out_xform, gamma, t, lut8);
    if (srgb_steps) build_srgb_steps(srgb_steps);
    return NTG_OK;
}

int ntg_transform(ntg_context *ctx, float *d_rgba, int w, int h, int kind, float gamma, void *stream) {
    g_error.clear();
    if (!ctx || !d_rgba || w <= 0 || h <= 0 || kind < 0 || kind > 3) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    NTG_TRY(ensure_device(ctx));
    int k = kind;
    float p = gamma;
    if (kind <= 1) {
        // Surface::toLinear / toGamma return early for gamma == 1 (nv::equal)
        if (std::fabs(gamma - 1.0f) <= 0.0001f * std::max(1.0f, std::fabs(gamma))) return NTG_OK;
        if (gamma != 2.2f) { k = 4; p = kind == 0 ? gamma : 1.0f / gamma; }
    }
    return launched(launch_transform(d_rgba, (size_t)w * h, k, p, S(stream)), "colour transform");
}

int ntg_profile_enable(ntg_context *ctx, int enable) {
    g_error.clear();
    if (!ctx) return fail(NTG_ERROR_INVALID_INPUT, "null context");
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    for (cudaEvent_t &e : ctx->ev)
        if (!e) NTG_CUDA(cudaEventCreate(&e));
    ctx->profile = enable != 0;
    return NTG_OK;
}

int ntg_profile_read(ntg_context *ctx, float *mips_ms, float *encode_ms) {
    g_error.clear();
    if (!ctx || !ctx->ev[2]) return fail(NTG_ERROR_INVALID_INPUT, "profiling not enabled");
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_CUDA(cudaEventSynchronize(ctx->ev[2]));
    float a = 0, b = 0;
    NTG_CUDA(cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]));
    NTG_CUDA(cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]));
    if (mips_ms) *mips_ms = a;
    if (encode_ms) *encode_ms = b;
    return NTG_OK;
}

int ntg_decode(ntg_context *ctx, int format, const void *d_blocks, int w, int h, float *d_rgba, void *stream) {
    g_error.clear();
    if (!ctx || !d_blocks || !d_rgba || w <= 0 || h <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    if (!known_format(format)) return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "format not supported");
    NTG_TRY(ensure_device(ctx));
    return launched(launch_decode(format, (const uint8_t *)d_blocks, w, h, d_rgba, S(stream)), "decode");
}

int ntg_error_sums(ntg_context *ctx, const float *d_ref, const float *d_img, int w, int h, int alpha_mode, double *d_sums,
                   void *stream) {
    g_error.clear();
    if (!ctx || !d_ref || !d_img || !d_sums || w <= 0 || h <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    NTG_TRY(ensure_device(ctx));
    return launched(launch_rms(d_ref, d_img, w, h, alpha_mode, d_sums, S(stream)), "error sums");
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Batches: every texture's chain planned together, launched as one CUDA graph.

struct ntg_batch {
    ntg_context *ctx = nullptr;
    std::vector<ntg_batch_texture> tex;
    std::vector<ntg_chain_options> opts;  // normalised
    std::vector<ChainPlan> plans;
    std::vector<const XformTables *> xts;
    std::vector<size_t> base;             // workspace offset of each texture's levels
    uint8_t *d_ws = nullptr;
    MipJob *d_mip = nullptr;
    EncJob *d_enc = nullptr;
    std::vector<int> set_images;          // textures whose level 0 is materialised (box path)
    std::vector<std::vector<MipLaunch>> stages;
    struct Enc {
        int format, quality, first, njobs;
        long long nblocks;
    };
    std::vector<Enc> encodes;
    MipTuning tune;
    int enc_threads[3] = {64, 128, 128};  // blocks per CTA of the BC1, BC3 + BC1a, BC5 + BC4 encoders
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long texels = 0, blocks = 0;
    int launches = 0;
    std::string key;                      // tuning-cache key (device | batch signature)
    // learned endpoint proposals for the BC1 [0] and BC3 [1] Normal blocks (none: the full fit)
    ntg_mlp *mlp[2] = {nullptr, nullptr};
    int radius[2] = {1, 1};
    float margin[2] = {0.5f, 0.5f};
    uint8_t *d_learn[2] = {nullptr, nullptr};  // network inputs, outputs, full-fit list, statistics
    bool unit_bc3 = true;                 // every BC3 texture has the default colour weights
    // The alternate binding: the same plan over a second set of inputs and outputs, with its own job
    // lists and graph (double-buffered host copies). Both graphs use the one workspace, so they run
    // one after the other. `which` selects the binding the planning and launching helpers work on.
    std::vector<ntg_batch_texture> alt;   // empty: none bound
    MipJob *d_mip_alt = nullptr;
    EncJob *d_enc_alt = nullptr;
    cudaGraph_t graph_alt = nullptr;
    cudaGraphExec_t exec_alt = nullptr;
    int which = 0;

    const std::vector<ntg_batch_texture> &io() const { return which ? alt : tex; }
    MipJob *&dmip() { return which ? d_mip_alt : d_mip; }
    EncJob *&denc() { return which ? d_enc_alt : d_enc; }
    cudaGraph_t &gr() { return which ? graph_alt : graph; }
    cudaGraphExec_t &ex() { return which ? exec_alt : exec; }

    ~ntg_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (exec_alt) cudaGraphExecDestroy(exec_alt);
        if (graph_alt) cudaGraphDestroy(graph_alt);
        if (d_mip_alt) cudaFree(d_mip_alt);
        if (d_enc_alt) cudaFree(d_enc_alt);
        if (d_ws) cudaFree(d_ws);
        if (d_mip) cudaFree(d_mip);
        if (d_enc) cudaFree(d_enc);
        if (d_learn[0]) cudaFree(d_learn[0]);
        if (d_learn[1]) cudaFree(d_learn[1]);
    }
};

namespace {

// Encoder families sharing one launch shape: BC1 (icbc); BC3 and BC1a (squish fit in shared
// memory); BC5 and BC4 (interpolated-alpha blocks).
int enc_slot(int format) {
    return format == NTG_FORMAT_BC1 ? 0 : (format == NTG_FORMAT_BC3 || format == NTG_FORMAT_BC1A) ? 1 : 2;
}

// Byte offsets of the learned path's buffers for n blocks: x, y, list, stats.
struct LearnLayout {
    size_t x, y, list, stats, bytes;
    explicit LearnLayout(long long n) {
        x = 0;
        y = align256(x + (size_t)n * 48 * 4);
        list = align256(y + (size_t)n * 16 * 4);
        stats = align256(list + (size_t)n * 8);
        bytes = stats + 256;
    }
};

// The proposal slot of an encode group (0 BC1, 1 BC3), or -1 when it runs the plain fit.
int learned_slot(const ntg_batch *b, const ntg_batch::Enc &e) {
    if (e.quality != NTG_QUALITY_NORMAL) return -1;
    const int k = e.format == NTG_FORMAT_BC1 ? 0 : (e.format == NTG_FORMAT_BC3 ? 1 : -1);
    return k >= 0 && b->mlp[k] ? k : -1;
}
bool learned_group(const ntg_batch *b, const ntg_batch::Enc &e) { return learned_slot(b, e) >= 0; }


// Plans the mip stages and encode launches of a batch for its current tuning and uploads the job
// lists (the workspace layout does not depend on the tuning).
int batch_plan(ntg_batch *b) {
    ntg_context *ctx = b->ctx;
    const size_t n = b->tex.size();
    std::vector<MipJob> all;
    b->stages.clear();
    b->set_images.clear();
    size_t max_levels = 0;
    std::vector<size_t> tails(n);
    for (size_t t = 0; t < n; t++) {
        max_levels = std::max(max_levels, b->plans[t].lv.size());
        tails[t] = tail_start(b->plans[t], b->tune);
        if (b->plans[t].f_off[0] != NONE) b->set_images.push_back((int)t);
    }
    for (size_t l = 1; l < max_levels; l++) {
        std::vector<std::pair<MipKey, MipJob>> items;
        for (size_t t = 0; t < n; t++) {
            const ChainPlan &P = b->plans[t];
            if (l >= P.lv.size() || l >= tails[t]) continue;
            items.emplace_back();
            NTG_TRY(chain_step(ctx, P, l, (const uint32_t *)b->io()[t].d_bgra, b->opts[t], b->xts[t], b->d_ws + b->base[t],
                               items.back().second, items.back().first));
        }
        std::vector<MipLaunch> stage;
        if (!items.empty()) group_launches(items, b->tune, all, stage);
        for (int weighted = 0; weighted < 2; weighted++) {  // tails starting at this level
            MipLaunch m;
            std::memset(&m, 0, sizeof m);
            m.kernel = MIP_TAIL;
            m.weighted = weighted;
            m.first_job = (int)all.size();
            long long chains = 0;
            for (size_t t = 0; t < n; t++) {
                if (tails[t] != l || (b->opts[t].weighted != 0) != (weighted != 0)) continue;
                NTG_TRY(chain_tail(ctx, b->plans[t], l, (const uint32_t *)b->io()[t].d_bgra, b->opts[t], b->xts[t],
                                   b->d_ws + b->base[t], chains++, all));
            }
            if (chains) {
                m.njobs = (int)all.size() - m.first_job;
                m.units = chains;
                stage.push_back(m);
            }
        }
        if (!stage.empty()) b->stages.push_back(stage);
    }
    std::map<std::pair<int, int>, std::vector<size_t>> groups;
    for (size_t t = 0; t < n; t++) groups[{b->opts[t].format, b->opts[t].quality}].push_back(t);
    std::vector<EncJob> ejobs;
    b->encodes.clear();
    for (auto &g : groups) {
        ntg_batch::Enc e{g.first.first, g.first.second, (int)ejobs.size(), 0, 0};
        long long nb = 0;
        for (size_t t : g.second)
            chain_jobs(b->plans[t], (const uint32_t *)b->io()[t].d_bgra, b->opts[t], b->xts[t], b->d_ws + b->base[t],
                       (uint8_t *)b->io()[t].d_blocks, ejobs, nb);
        e.njobs = (int)ejobs.size() - e.first;
        e.nblocks = nb;
        b->encodes.push_back(e);
    }
    MipJob *&dm = b->dmip();
    EncJob *&de = b->denc();
    if (dm) cudaFree(dm);
    if (de) cudaFree(de);
    dm = nullptr;
    de = nullptr;
    if (!all.empty()) {
        NTG_CUDA(cudaMalloc((void **)&dm, all.size() * sizeof(MipJob)));
        NTG_CUDA(cudaMemcpy(dm, all.data(), all.size() * sizeof(MipJob), cudaMemcpyHostToDevice));
    }
    NTG_CUDA(cudaMalloc((void **)&de, ejobs.size() * sizeof(EncJob)));
    NTG_CUDA(cudaMemcpy(de, ejobs.data(), ejobs.size() * sizeof(EncJob), cudaMemcpyHostToDevice));
    b->launches = (int)b->set_images.size() + (int)b->encodes.size();
    for (const auto &e : b->encodes)
        if (learned_group(b, e)) b->launches += 3;  // features, network, pruned fit, full-fit list
    for (const auto &st : b->stages) b->launches += (int)st.size();
    return NTG_OK;
}

int batch_mips(ntg_batch *b, cudaStream_t s) {
    for (int t : b->set_images) {
        const ChainPlan &P = b->plans[t];
        NTG_TRY(launched(launch_set_image((const uint32_t *)b->io()[t].d_bgra, (size_t)P.lv[0].w * P.lv[0].h, b->xts[t]->d_in,
                                          (float *)(b->d_ws + b->base[t] + P.f_off[0]), s), "set image"));
    }
    return run_stages(b->stages, b->dmip(), s);
}

int batch_encodes(ntg_batch *b, cudaStream_t s, int only_slot = -1) {
    for (const auto &e : b->encodes) {
        if (only_slot >= 0 && enc_slot(e.format) != only_slot) continue;
        const int k = learned_slot(b, e);
        if (k >= 0) {
            const LearnLayout L(e.nblocks);
            uint8_t *buf = b->d_learn[k];
            float *x = (float *)(buf + L.x), *y = (float *)(buf + L.y);
            long long *list = (long long *)(buf + L.list);
            unsigned long long *stats = (unsigned long long *)(buf + L.stats);
            const EncJob *jobs = b->denc() + e.first;
            NTG_TRY(launched(k ? launch_bc3_features(jobs, e.njobs, e.nblocks, x, s)
                               : launch_bc1_features(jobs, e.njobs, e.nblocks, x, s), "block features"));
            const int r = mlp_forward_device(b->mlp[k], x, e.nblocks, y, s);
            if (r) return fail(r, std::string("proposal network: ") + ntg_last_error_string());
            NTG_CUDA(cudaMemsetAsync(stats, 0, 3 * sizeof(unsigned long long), s));
            if (k) {
                NTG_TRY(launched(launch_bc3_learned(jobs, e.njobs, e.nblocks, y, b->radius[k], b->margin[k], b->unit_bc3, list,
                                                    stats, s), "pruned fit"));
                NTG_TRY(launched(launch_bc3_list(jobs, e.njobs, list, stats + 1, e.nblocks, s), "full fit of the listed blocks"));
            } else {
                NTG_TRY(launched(launch_bc1_learned(jobs, e.njobs, e.nblocks, y, b->radius[k], b->margin[k], list, stats, s),
                                 "pruned fit"));
                NTG_TRY(launched(launch_bc1_list(jobs, e.njobs, list, stats + 1, e.nblocks, s), "full fit of the listed blocks"));
            }
            continue;
        }
        NTG_TRY(launch_encode(e.format, b->denc() + e.first, e.njobs, e.nblocks, e.quality, s, b->enc_threads[enc_slot(e.format)]));
    }
    return NTG_OK;
}

// Runs the sequence once on a private stream (first-use attributes, and the outputs), then
// captures it into a graph.
int batch_capture(ntg_batch *b) {
    if (b->ex()) { cudaGraphExecDestroy(b->ex()); b->ex() = nullptr; }
    if (b->gr()) { cudaGraphDestroy(b->gr()); b->gr() = nullptr; }
    cudaStream_t cs;
    NTG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    int r = batch_mips(b, cs);
    if (r == NTG_OK) r = batch_encodes(b, cs);
    cudaError_t e = cudaStreamSynchronize(cs);
    if (r == NTG_OK && e != cudaSuccess) r = cuda_fail(e, "batch run");
    if (r == NTG_OK) {
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) r = cuda_fail(e, "begin capture");
        else {
            r = batch_mips(b, cs);
            if (r == NTG_OK) r = batch_encodes(b, cs);
            e = cudaStreamEndCapture(cs, &b->gr());
            if (r == NTG_OK && e != cudaSuccess) r = cuda_fail(e, "end capture");
        }
    }
    if (r == NTG_OK) {
        e = cudaGraphInstantiate(&b->ex(), b->gr(), 0);
        if (e != cudaSuccess) r = cuda_fail(e, "graph instantiate");
    }
    cudaStreamDestroy(cs);
    return r;
}

// Plans and captures both bindings for the current launch shapes (the alternate one if bound),
// leaving the primary selected.
int batch_replan(ntg_batch *b) {
    if (!b->alt.empty()) {
        b->which = 1;
        int r = batch_plan(b);
        if (r == NTG_OK) r = batch_capture(b);
        b->which = 0;
        NTG_TRY(r);
    }
    NTG_TRY(batch_plan(b));
    return batch_capture(b);
}

// ---- tuning cache: a small JSON file of {"key", launch shape, timings} entries

struct TuneEntry {
    std::string key;
    int strip = 16, threads = 512, tail = 1024, bc1 = 64, bc3 = 128, bc5 = 128;
    double mip_ms = 0, encode_ms = 0;
};

std::string tune_cache_path() {
    const char *p = std::getenv("NTG_TUNE_CACHE");
    if (p && *p) return p;
    const char *home = std::getenv("HOME");
    return std::string(home && *home ? home : ".") + "/.cache/ntg_tune.json";
}

// Value after "field": in one flat JSON object (numbers, or a string without escapes).
size_t json_value(const std::string &obj, const char *field) {
    const std::string pat = std::string("\"") + field + "\"";
    size_t i = obj.find(pat);
    if (i == std::string::npos) return std::string::npos;
    i += pat.size();
    while (i < obj.size() && (obj[i] == ' ' || obj[i] == ':')) i++;
    return i;
}

double json_number(const std::string &obj, const char *field, double def) {
    const size_t i = json_value(obj, field);
    return i == std::string::npos ? def : std::atof(obj.c_str() + i);
}

std::vector<TuneEntry> tune_cache_read() {
    std::vector<TuneEntry> v;
    FILE *f = std::fopen(tune_cache_path().c_str(), "rb");
    if (!f) return v;
    std::string text;
    char buf[4096];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, k);
    std::fclose(f);
    size_t pos = 0;
    while ((pos = text.find('{', pos + 1)) != std::string::npos) {
        const size_t end = text.find('}', pos);
        if (end == std::string::npos) break;
        const std::string obj = text.substr(pos, end - pos);
        const size_t k0 = json_value(obj, "key");
        if (k0 == std::string::npos || obj[k0] != '"') continue;
        const size_t k1 = obj.find('"', k0 + 1);
        if (k1 == std::string::npos) continue;
        TuneEntry e;
        e.key = obj.substr(k0 + 1, k1 - k0 - 1);
        e.strip = (int)json_number(obj, "strip", 16);
        e.threads = (int)json_number(obj, "threads", 512);
        e.tail = (int)json_number(obj, "tail", 1024);
        e.bc1 = (int)json_number(obj, "bc1", 64);
        e.bc3 = (int)json_number(obj, "bc3", 128);
        e.bc5 = (int)json_number(obj, "bc5", 128);
        e.mip_ms = json_number(obj, "mip_ms", 0);
        e.encode_ms = json_number(obj, "encode_ms", 0);
        v.push_back(e);
    }
    return v;
}

void tune_cache_write(const std::vector<TuneEntry> &v) {
    const std::string path = tune_cache_path();
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {  // create the parent directory if it is missing (one level)
        const std::string dir = path.substr(0, slash);
        if (!dir.empty()) mkdir(dir.c_str(), 0755);
    }
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return;
    std::fprintf(f, "{\"version\": 1, \"entries\": [\n");
    for (size_t i = 0; i < v.size(); i++) {
        const TuneEntry &e = v[i];
        std::fprintf(f,
                     "  {\"key\": \"%s\", \"strip\": %d, \"threads\": %d, \"tail\": %d, \"bc1\": %d, \"bc3\": %d, \"bc5\": %d, "
                     "\"mip_ms\": %.4f, \"encode_ms\": %.4f}%s\n",
                     e.key.c_str(), e.strip, e.threads, e.tail, e.bc1, e.bc3, e.bc5, e.mip_ms, e.encode_ms,
                     i + 1 < v.size() ? "," : "");
    }
    std::fprintf(f, "]}\n");
    std::fclose(f);
}

void apply_entry(ntg_batch *b, const TuneEntry &e) {
    b->tune.strip = e.strip;
    b->tune.threads = e.threads;
    b->tune.tail_texels = e.tail;
    b->enc_threads[0] = e.bc1;
    b->enc_threads[1] = e.bc3;
    b->enc_threads[2] = e.bc5;
}

// Device name and a hash of every texture's size and options.
// Version of the tunable launch shapes (2:1 tile height and CTA size, tail size, encoder CTA sizes).
constexpr long long kTuneShapeVersion = 2;

std::string batch_key(const ntg_batch *b) {
    cudaDeviceProp prop;
    std::string dev = cudaGetDeviceProperties(&prop, b->ctx->device) == cudaSuccess ? prop.name : "device";
    for (char &c : dev)
        if (c == '"' || c == '\\') c = '_';
    unsigned long long h = 1469598103934665603ull;
    auto mix = [&](long long v) {
        for (int i = 0; i < 8; i++) { h ^= (unsigned long long)((v >> (8 * i)) & 255); h *= 1099511628211ull; }
    };
    mix(kTuneShapeVersion);  // entries written for another set of kernel shapes do not apply
    for (size_t t = 0; t < b->tex.size(); t++) {
        const ntg_chain_options &o = b->opts[t];
        mix(b->tex[t].w); mix(b->tex[t].h); mix(o.format); mix(o.quality); mix(o.filter); mix(o.alpha_mode);
        mix(o.in_xform); mix(o.out_xform); mix(o.weighted); mix(o.max_levels);
    }
    char buf[32];
    std::snprintf(buf, sizeof buf, "%016llx", h);
    return dev + "|" + buf;
}

float time_ms(cudaStream_t s, const std::function<int()> &fn, int reps, int *status) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int r = 0; r < reps && *status == NTG_OK; r++) {
        cudaEventRecord(e0, s);
        *status = fn();
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) *status = cuda_fail(cudaGetLastError(), "tuning run");
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return best;
}

}  // namespace

extern "C" {

int ntg_batch_build(ntg_context *ctx, const ntg_batch_texture *textures, int count, ntg_batch **out) {
    g_error.clear();
    if (!ctx || !textures || count <= 0 || !out) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    NTG_TRY(ensure_device(ctx));
    std::unique_ptr<ntg_batch> b(new ntg_batch);
    b->ctx = ctx;
    b->tex.assign(textures, textures + count);
    size_t off = 0;
    for (int t = 0; t < count; t++) {
        const ntg_batch_texture &T = textures[t];
        if (!T.d_bgra || !T.d_blocks || T.w <= 0 || T.h <= 0) return fail(NTG_ERROR_INVALID_INPUT, "bad texture");
        NTG_TRY(check_opts(&T.opt));
        const ntg_chain_options o = normalized(T.opt);
        if ((o.in_xform == NTG_XFORM_GAMMA || o.out_xform == NTG_XFORM_GAMMA) && o.gamma != 2.2f)
            return fail(NTG_ERROR_UNSUPPORTED_FEATURE, "power-law gamma other than 2.2 is not supported on the GPU");
        b->opts.push_back(o);
        b->plans.push_back(plan_chain(T.w, T.h, o, false));
        const XformTables *xt = ctx->xform(o.in_xform, o.out_xform, o.gamma);
        if (!xt) return fail(NTG_ERROR_CUDA, "table upload failed");
        b->xts.push_back(xt);
        b->base.push_back(off);
        off = align256(off + b->plans.back().bytes);
        for (const Level &L : b->plans.back().lv) {
            b->texels += (long long)L.w * L.h;
            b->blocks += blocks_of(L.w, L.h);
        }
    }
    NTG_CUDA(cudaMalloc((void **)&b->d_ws, std::max<size_t>(off, 256)));
    b->key = batch_key(b.get());
    for (const TuneEntry &e : tune_cache_read())
        if (e.key == b->key) apply_entry(b.get(), e);
    NTG_TRY(batch_plan(b.get()));
    NTG_TRY(batch_capture(b.get()));
    *out = b.release();
    return NTG_OK;
}

int ntg_batch_launch(ntg_batch *b, void *stream) {
    g_error.clear();
    if (!b || !b->exec) return fail(NTG_ERROR_INVALID_INPUT, "batch not built");
    NTG_TRY(ensure_device(b->ctx));
    NTG_CUDA(cudaGraphLaunch(b->exec, S(stream)));
    return NTG_OK;
}

int ntg_batch_bind_alternate(ntg_batch *b, const void *const *d_bgra, void *const *d_blocks) {
    g_error.clear();
    if (!b || !d_bgra || !d_blocks) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    for (size_t t = 0; t < b->tex.size(); t++)
        if (!d_bgra[t] || !d_blocks[t]) return fail(NTG_ERROR_INVALID_INPUT, "null input or output");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    NTG_TRY(ensure_device(b->ctx));
    b->alt = b->tex;
    for (size_t t = 0; t < b->alt.size(); t++) {
        b->alt[t].d_bgra = d_bgra[t];
        b->alt[t].d_blocks = d_blocks[t];
    }
    // the plan (stages, encode groups) is the same for both bindings; only the job lists differ
    b->which = 1;
    int r = batch_plan(b);
    if (r == NTG_OK) r = batch_capture(b);
    b->which = 0;
    return r;
}

int ntg_batch_launch_alternate(ntg_batch *b, void *stream) {
    g_error.clear();
    if (!b || !b->exec_alt) return fail(NTG_ERROR_INVALID_INPUT, "no alternate binding");
    NTG_TRY(ensure_device(b->ctx));
    NTG_CUDA(cudaGraphLaunch(b->exec_alt, S(stream)));
    return NTG_OK;
}

int ntg_batch_process_host(ntg_batch *b, int count, const void *const *const *h_bgra, void *const *const *h_blocks,
                           void *stream) {
    g_error.clear();
    if (!b || !b->exec || count < 0 || (count > 0 && (!h_bgra || !h_blocks))) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    const size_t nt = b->tex.size();
    for (int i = 0; i < count; i++) {
        if (!h_bgra[i] || !h_blocks[i]) return fail(NTG_ERROR_INVALID_INPUT, "null set");
        for (size_t t = 0; t < nt; t++)
            if (!h_bgra[i][t] || !h_blocks[i][t]) return fail(NTG_ERROR_INVALID_INPUT, "null image or output");
    }
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    ntg_context *ctx = b->ctx;
    NTG_TRY(ensure_device(ctx));
    NTG_TRY(ctx->copy_streams());
    cudaStream_t s = S(stream);
    const bool two = b->exec_alt != nullptr;
    const int lag = two ? 2 : 1;  // sets between two uses of one binding
    auto slot = [&](int i) { return two ? (i & 1) : 0; };
    // copy-in of set i on the up stream, once the graph that last read its binding's inputs is done
    auto copy_in = [&](int i) -> int {
        const int k = slot(i);
        const std::vector<ntg_batch_texture> &io = k ? b->alt : b->tex;
        if (i >= lag) NTG_CUDA(cudaStreamWaitEvent(ctx->up, ctx->ev_done[k], 0));
        for (size_t t = 0; t < nt; t++)
            NTG_CUDA(cudaMemcpyAsync(const_cast<void *>(io[t].d_bgra), h_bgra[i][t], (size_t)io[t].w * io[t].h * 4,
                                     cudaMemcpyHostToDevice, ctx->up));
        NTG_CUDA(cudaEventRecord(ctx->ev_in[k], ctx->up));
        return NTG_OK;
    };
    // graph of set i on the compute stream, once its inputs are in and the blocks of the set that last
    // used its binding are out
    auto run = [&](int i) -> int {
        const int k = slot(i);
        NTG_CUDA(cudaStreamWaitEvent(s, ctx->ev_in[k], 0));
        if (i >= lag) NTG_CUDA(cudaStreamWaitEvent(s, ctx->ev_out[k], 0));
        NTG_CUDA(cudaGraphLaunch(k ? b->exec_alt : b->exec, s));
        NTG_CUDA(cudaEventRecord(ctx->ev_done[k], s));
        return NTG_OK;
    };
    // the same events as the single-chain pipeline: their previous users ended with drained streams.
    // A copy-out to memory the driver does not treat as page-locked returns only once it is done, so
    // everything that can run beside it is issued first: the next set's copy-in, and with two bindings
    // the next set's graph too (its binding's previous blocks, set i - 1's, were copied out earlier).
    if (count > 0) {
        NTG_TRY(copy_in(0));
        NTG_TRY(run(0));
    }
    for (int i = 0; i < count; i++) {
        const int k = slot(i);
        const std::vector<ntg_batch_texture> &io = k ? b->alt : b->tex;
        if (i + 1 < count) {
            NTG_TRY(copy_in(i + 1));
            if (two) NTG_TRY(run(i + 1));
        }
        NTG_CUDA(cudaStreamWaitEvent(ctx->down, ctx->ev_done[k], 0));
        for (size_t t = 0; t < nt; t++)
            NTG_CUDA(cudaMemcpyAsync(h_blocks[i][t], io[t].d_blocks, ntg_chain_bytes(io[t].w, io[t].h, &io[t].opt),
                                     cudaMemcpyDeviceToHost, ctx->down));
        NTG_CUDA(cudaEventRecord(ctx->ev_out[k], ctx->down));
        if (!two && i + 1 < count) NTG_TRY(run(i + 1));  // one binding: after this set's blocks are out
    }
    NTG_CUDA(cudaStreamSynchronize(ctx->up));
    NTG_CUDA(cudaStreamSynchronize(s));
    NTG_CUDA(cudaStreamSynchronize(ctx->down));
    return NTG_OK;
}

int ntg_batch_autotune(ntg_batch *b, void *stream) {
    g_error.clear();
    if (!b) return fail(NTG_ERROR_INVALID_INPUT, "null batch");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    NTG_TRY(ensure_device(b->ctx));
    cudaStream_t s = S(stream);
    int status = NTG_OK;
    // mip launch shapes: rows per strip x threads per CTA x tail threshold
    const MipTuning keep = b->tune;
    MipTuning best = keep;
    float best_ms = 1e30f;
    for (int tail : {1024, 4096})
        for (int threads : {256, 512})
            for (int strip : {8, 16, 32}) {
                b->tune.strip = strip;
                b->tune.threads = threads;
                b->tune.tail_texels = tail;
                NTG_TRY(batch_plan(b));
                const float ms = time_ms(s, [&] { return batch_mips(b, s); }, 3, &status);
                NTG_TRY(status);
                if (ms < best_ms) { best_ms = ms; best = b->tune; }
            }
    b->tune = best;
    NTG_TRY(batch_plan(b));
    // encoder blocks per CTA, per format present
    float enc_total = 0;
    for (int slot = 0; slot < 3; slot++) {
        bool present = false;
        for (const auto &e : b->encodes) present = present || enc_slot(e.format) == slot;
        if (!present) continue;
        int best_t = b->enc_threads[slot];
        float best_e = 1e30f;
        for (int threads : {32, 64, 128}) {
            if (slot == 0 && threads > 64) continue;
            b->enc_threads[slot] = threads;
            const float ms = time_ms(s, [&] { return batch_encodes(b, s, slot); }, 3, &status);
            NTG_TRY(status);
            if (ms < best_e) { best_e = ms; best_t = threads; }
        }
        b->enc_threads[slot] = best_t;
        enc_total += best_e;
    }
    NTG_TRY(batch_replan(b));
    std::vector<TuneEntry> cache = tune_cache_read();
    TuneEntry e;
    e.key = b->key;
    e.strip = b->tune.strip;
    e.threads = b->tune.threads;
    e.tail = (int)b->tune.tail_texels;
    e.bc1 = b->enc_threads[0];
    e.bc3 = b->enc_threads[1];
    e.bc5 = b->enc_threads[2];
    e.mip_ms = best_ms;
    e.encode_ms = enc_total;
    cache.erase(std::remove_if(cache.begin(), cache.end(), [&](const TuneEntry &x) { return x.key == e.key; }), cache.end());
    cache.push_back(e);
    tune_cache_write(cache);
    return NTG_OK;
}

int ntg_batch_info(const ntg_batch *b, long long *texels, long long *blocks, int *launches, int shape[6]) {
    if (!b) return fail(NTG_ERROR_INVALID_INPUT, "null batch");
    if (texels) *texels = b->texels;
    if (blocks) *blocks = b->blocks;
    if (launches) *launches = b->launches;
    if (shape) {
        shape[0] = b->tune.strip;
        shape[1] = b->tune.threads;
        shape[2] = (int)b->tune.tail_texels;
        shape[3] = b->enc_threads[0];
        shape[4] = b->enc_threads[1];
        shape[5] = b->enc_threads[2];
    }
    return NTG_OK;
}

int ntg_batch_time_phases(ntg_batch *b, void *stream, float ms[4], long long blocks[3]) {
    g_error.clear();
    if (!b || !ms) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    NTG_TRY(ensure_device(b->ctx));
    cudaStream_t s = S(stream);
    int status = NTG_OK;
    ms[0] = time_ms(s, [&] { return batch_mips(b, s); }, 1, &status);
    NTG_TRY(status);
    for (int i = 0; i < 3; i++) {
        long long nb = 0;
        for (const auto &e : b->encodes)
            if (enc_slot(e.format) == i) nb += e.nblocks;
        if (blocks) blocks[i] = nb;
        ms[1 + i] = nb ? time_ms(s, [&] { return batch_encodes(b, s, i); }, 1, &status) : 0.0f;
        NTG_TRY(status);
    }
    return NTG_OK;
}

int ntg_batch_count_work(ntg_batch *b, void *stream, unsigned long long bc1_orderings[2]) {
    g_error.clear();
    if (!b || !bc1_orderings) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    NTG_TRY(ensure_device(b->ctx));
    cudaStream_t s = S(stream);
    unsigned long long *d = nullptr;
    NTG_CUDA(cudaMallocAsync((void **)&d, 2 * sizeof(unsigned long long), s));
    int status = cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), s) == cudaSuccess ? NTG_OK : NTG_ERROR_CUDA;
    for (const auto &e : b->encodes)
        if (status == NTG_OK && e.format == NTG_FORMAT_BC1 && e.quality != NTG_QUALITY_FASTEST)
            status = launched(launch_bc1_work(b->denc() + e.first, e.njobs, e.nblocks, d, s), "fit work count");
    if (status == NTG_OK && cudaMemcpyAsync(bc1_orderings, d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        status = NTG_ERROR_CUDA;
    cudaFreeAsync(d, s);
    if (status == NTG_OK && cudaStreamSynchronize(s) != cudaSuccess) status = NTG_ERROR_CUDA;
    return status == NTG_OK ? NTG_OK : fail(status, "fit work count failed");
}

int ntg_batch_set_proposal_format(ntg_batch *b, int format, ntg_mlp *mlp, int radius, float margin) {
    g_error.clear();
    if (!b || radius < 0 || (format != NTG_FORMAT_BC1 && format != NTG_FORMAT_BC3))
        return fail(NTG_ERROR_INVALID_INPUT, "bad arguments (proposals are for BC1 and BC3)");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    NTG_TRY(ensure_device(b->ctx));
    const int k = format == NTG_FORMAT_BC3 ? 1 : 0;
    b->mlp[k] = mlp;
    b->radius[k] = radius;
    b->margin[k] = margin;
    long long nb = 0;
    for (const auto &e : b->encodes)
        if (learned_slot(b, e) == k) nb = std::max(nb, e.nblocks);
    if (b->d_learn[k]) { cudaFree(b->d_learn[k]); b->d_learn[k] = nullptr; }
    if (mlp && nb > 0) NTG_CUDA(cudaMalloc((void **)&b->d_learn[k], LearnLayout(nb).bytes));
    b->unit_bc3 = true;
    for (const auto &o : b->opts)
        if (o.format == NTG_FORMAT_BC3 && !(o.cw[0] == 0 && o.cw[1] == 0 && o.cw[2] == 0) &&
            !(o.cw[0] == 1 && o.cw[1] == 1 && o.cw[2] == 1))
            b->unit_bc3 = false;
    return batch_replan(b);
}

int ntg_batch_set_proposal(ntg_batch *b, ntg_mlp *mlp, int radius, float margin) {
    return ntg_batch_set_proposal_format(b, NTG_FORMAT_BC1, mlp, radius, margin);
}

int ntg_batch_proposal_stats_format(ntg_batch *b, int format, unsigned long long stats[3]) {
    g_error.clear();
    if (!b || !stats) return fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    const int k = format == NTG_FORMAT_BC3 ? 1 : 0;
    stats[0] = stats[1] = stats[2] = 0;
    for (const auto &e : b->encodes) {
        if (learned_slot(b, e) != k) continue;
        NTG_CUDA(cudaDeviceSynchronize());
        NTG_CUDA(cudaMemcpy(stats, b->d_learn[k] + LearnLayout(e.nblocks).stats, 3 * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost));
    }
    return NTG_OK;
}

int ntg_batch_proposal_stats(ntg_batch *b, unsigned long long stats[3]) {
    return ntg_batch_proposal_stats_format(b, NTG_FORMAT_BC1, stats);
}

int ntg_batch_destroy(ntg_batch *b) {
    if (!b) return NTG_OK;
    cudaSetDevice(b->ctx->device);
    cudaDeviceSynchronize();
    delete b;
    return NTG_OK;
}

}  // extern "C"
