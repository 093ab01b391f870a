/* ntg.h -- C ABI of the GB300 (sm_103a) texture hot path.
 *
 * Drop-in boundary for NVTT 2.1.2's mip-chain + BC1/BC1a/BC3/BC4/BC5 path. Plain C types only: device
 * pointers are caller-owned CUDA allocations, host pointers are plain memory, every call takes an
 * explicit CUDA stream (cudaStream_t passed as void *; NULL = the legacy default stream) and
 * returns an int status:
 *     NTG_OK (0), or an nvtt::Error value (src/nvtt/nvtt.h:345-364):
 *     1 InvalidInput, 2 UnsupportedFeature, 3 CudaError, 6 UnsupportedOutputFormat;
 *     NTG_ERROR_UNKNOWN (100) stands in for nvtt's Error_Unknown (0).
 * ntg_last_error_string() describes the last failure on the calling thread.
 * Calls that take device pointers only enqueue work; they never synchronise. Calls that take host
 * pointers (the *_host variants) copy in, run and copy out on the given stream and return after
 * it has drained.
 *
 * Enum values are nvtt's own: Format (src/nvtt/nvtt.h:77-129), Quality (:145-151), WrapMode
 * (:217-222), MipmapFilter (:253-258), AlphaMode (:279-284).
 */
#ifndef NTG_H
#define NTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NTG_VERSION 20102      /* the NVTT release whose behaviour this reproduces */

#define NTG_OK 0
#define NTG_ERROR_INVALID_INPUT 1
#define NTG_ERROR_UNSUPPORTED_FEATURE 2
#define NTG_ERROR_CUDA 3
#define NTG_ERROR_UNSUPPORTED_OUTPUT_FORMAT 6
#define NTG_ERROR_UNKNOWN 100

/* nvtt::Format subset */
#define NTG_FORMAT_BC1 1   /* Format_DXT1 */
#define NTG_FORMAT_BC1A 2  /* Format_DXT1a: Normal quality and above (CompressorDXT1a) */
#define NTG_FORMAT_BC3 4   /* Format_DXT5 */
#define NTG_FORMAT_BC4 6   /* Format_BC4 */
#define NTG_FORMAT_BC5 7   /* Format_BC5 */
/* nvtt::Quality */
#define NTG_QUALITY_FASTEST 0
#define NTG_QUALITY_NORMAL 1
#define NTG_QUALITY_PRODUCTION 2
#define NTG_QUALITY_HIGHEST 3
/* nvtt::WrapMode */
#define NTG_WRAP_CLAMP 0
#define NTG_WRAP_REPEAT 1
#define NTG_WRAP_MIRROR 2
/* nvtt::MipmapFilter */
#define NTG_FILTER_BOX 0
#define NTG_FILTER_TRIANGLE 1
#define NTG_FILTER_KAISER 2
/* nvtt::AlphaMode */
#define NTG_ALPHA_NONE 0
#define NTG_ALPHA_TRANSPARENCY 1
/* colour transforms applied around the mip chain */
#define NTG_XFORM_NONE 0   /* linear data */
#define NTG_XFORM_GAMMA 1  /* Surface::toLinear(gamma) / toGamma(gamma) (src/nvtt/Surface.cpp:1470-1488) */
#define NTG_XFORM_SRGB 2   /* Surface::toLinearFromSrgb / toSrgb (src/nvtt/Surface.cpp:1512-1592) */

typedef struct ntg_context ntg_context;

/* Per-device state: constant tables, a grow-only scratch workspace and staging buffers.
 * Replaces the reference's CudaContext (src/nvtt/Context.cpp:81-98). The first context on a device
 * also builds that device's sRGB correction tables (about 55 MB of device memory, held until exit);
 * later contexts on the device allocate nothing until their first call that needs scratch. */
int ntg_create(int device, ntg_context **out);
int ntg_destroy(ntg_context *ctx);
const char *ntg_last_error_string(void);
int ntg_version(void);
/* Kernel launches this process has issued through the library so far (graph replays of a batch
 * are not counted here: ntg_batch_info reports a batch's launches). No reference counterpart. */
unsigned long long ntg_launch_count(void);

/* ---- single steps on device buffers ---- */

/* Surface::setImage(InputFormat_BGRA_8UB) (src/nvtt/Surface.cpp:728-760) followed by the input
 * transform of RGB. bgra: w*h BGRA8 texels. rgba: 4*w*h floats, planar. */
int ntg_set_image_bgra8(ntg_context *ctx, const void *d_bgra, int w, int h, int in_xform, float gamma,
                        float *d_rgba, void *stream);

/* Surface::resize(w, h, 1, filter, width, params) (src/nvtt/Surface.cpp:1152-1230) of a planar FP32
 * image w x h into dw x dh (FloatImage::resize, src/nvimage/FloatImage.cpp:761-808, 877-925: X pass,
 * then Y pass, any scale, up or down). filter 0 box / 1 triangle / 2 kaiser (Mitchell is not
 * supported); width 0 picks getDefaultFilterWidthAndParams (src/nvtt/Surface.cpp:1121-1141). Equal
 * extents copy the image unchanged, as Surface::resize returns early. Uses the context workspace
 * for the intermediate dw x h plane. */
int ntg_resize(ntg_context *ctx, const float *d_src, int w, int h, float *d_dst, int dw, int dh, int filter, float width,
               const float *params, int wrap, int alpha_mode, void *stream);

/* Self-test of the mip kernels' sRGB quantiser (a bucket table plus one step comparison) against the
 * plain search over the toSrgb step table, on every float bit pattern of both signs: writes the
 * number of disagreements (0 expected). No reference counterpart; synchronous. */
int ntg_selftest_srgb_quantizer(ntg_context *ctx, unsigned long long *mismatches);

/* nv::getTargetExtent (src/nvtt/Surface.cpp:220-326) for a 2D texture: the level-0 extent that
 * Compressor::process resizes to for InputOptions::setMaxExtent / setRoundMode (round_mode is an
 * nvtt::RoundMode). A result may be 0 (ToPreviousMultipleOfFour below 4), as in the reference. */
int ntg_target_extent(int w, int h, int max_extent, int round_mode, int *out_w, int *out_h);
/* The same for an nvtt::TextureType: 0 (2D) and 3 (array) as above; 1 (cube map) makes the faces
 * square at the mean of the scaled extents before rounding (src/nvtt/Surface.cpp:248-252). 3D
 * textures (2) are outside this path: NTG_ERROR_UNSUPPORTED_FEATURE. */
int ntg_target_extent_ex(int w, int h, int max_extent, int round_mode, int texture_type, int *out_w, int *out_h);

/* Surface::buildNextMipmap (src/nvtt/Surface.cpp:1344-1406): one level down from a planar FP32
 * level to max(1, w/2) x max(1, h/2). params = {kaiser alpha, kaiser stretch} (ignored otherwise).
 * weighted != 0 selects the alpha-weighted kernels of FloatImage::applyKernelX/Y
 * (src/nvimage/FloatImage.cpp:1212-1281), which the reference defines but does not call. */
int ntg_mip_level(ntg_context *ctx, const float *d_src, int w, int h, float *d_dst, int filter, float width,
                  const float *params, int wrap, int alpha_mode, int weighted, void *stream);

/* Bounded waits of the mip filter: the TMA-staged FP32 2:1 tile kernel waits on an mbarrier for each
 * tile's source window, at most `polls` polls per wait on the context's device (negative: the
 * default, 4,194,304); 0 makes every wait give up at once, with no fault. A kernel whose wait gave
 * up records it (ntg_mip_status), waits with the default limit for the copy in flight and returns
 * without writing its remaining tiles, so later calls run normally. Synchronises the device. No
 * counterpart in the reference. */
int ntg_mip_set_wait_limit(ntg_context *ctx, int polls);
/* *gave_up = 1 when a mip wait gave up since the previous call, else 0; clears the record.
 * Synchronises the device. */
int ntg_mip_status(ntg_context *ctx, int *gave_up);

/* CompressorInterface::compress (src/nvtt/Compressor.h:34-38) for one planar FP32 level, as
 * CompressorDXT1 / CompressorDXT5 / FastCompressorBC5 etc. encode it (chooseCpuCompressor,
 * src/nvtt/Context.cpp:1038-1163). out_xform / gamma apply the output transform to RGB first
 * (Compressor::Private::compress's toGamma step, src/nvtt/Context.cpp:283-289); cw = colour
 * weights (CompressionOptions::setColorWeights). Output: ((w+3)/4)*((h+3)/4) blocks of 8 (BC1)
 * or 16 (BC3, BC5) bytes in row-major block order. */
int ntg_encode(ntg_context *ctx, int format, const float *d_rgba, int w, int h, int quality, int alpha_mode,
               int out_xform, float gamma, const float *cw, void *d_blocks, void *stream);

/* ntg_encode for callers that cannot allocate device memory (engines that own all GPU memory
 * through their own pools, frame loops where cudaMalloc's implicit synchronisation would stall):
 * it calls no cudaMalloc/cudaFree and no allocating library routine. No counterpart in the
 * reference. Its scratch is a static device array of NTG_NOALLOC_SCRATCH_BYTES that every GPU
 * loading this library holds until exit; levels above NTG_NOALLOC_MAX_TEXELS texels are rejected
 * with NTG_ERROR_INVALID_INPUT. The first call on a device looks up the array's device address
 * (make it before any stream capture). All calls share the array: calls that overlap on the GPU
 * race, so issue them on one stream. The context must come from ntg_create (whose allocations, the
 * per-device sRGB tables, happen there, before any frame loop); same arguments and results as
 * ntg_encode. */
#define NTG_NOALLOC_MAX_TEXELS 1048576
#define NTG_NOALLOC_SCRATCH_BYTES (4 * NTG_NOALLOC_MAX_TEXELS + 2048)
int ntg_encode_noalloc(ntg_context *ctx, int format, const float *d_rgba, int w, int h, int quality, int alpha_mode,
                       int out_xform, float gamma, const float *cw, void *d_blocks, void *stream);

/* Surface::toLinear(gamma) / toGamma(gamma) / toLinearFromSrgb / toSrgb (src/nvtt/Surface.cpp:1470-1592)
 * on RGB of a planar FP32 level, in place. kind: 0 toLinear, 1 toGamma, 2 toLinearFromSrgb, 3 toSrgb.
 * Gamma 2.2 is bit-exact (the reference's own table-and-quartic powf), and so are the sRGB curves (the
 * device powf corrected, per input, to the host libm's result by tables built when the first context
 * on a device is created); other gammas use the device powf (may differ from the host libm in the
 * last place). */
#define NTG_TRANSFORM_TO_LINEAR 0
#define NTG_TRANSFORM_TO_GAMMA 1
#define NTG_TRANSFORM_FROM_SRGB 2
#define NTG_TRANSFORM_TO_SRGB 3
int ntg_transform(ntg_context *ctx, float *d_rgba, int w, int h, int kind, float gamma, void *stream);

/* ---- whole chains ---- */

typedef struct ntg_chain_options {
    int format;          /* NTG_FORMAT_* */
    int quality;         /* NTG_QUALITY_* */
    int filter;          /* NTG_FILTER_* */
    float filter_width;  /* 0 = nvtt default for the filter (box 0.5, triangle 1, kaiser 3) */
    float params[2];     /* kaiser alpha, stretch (defaults 4, 1 when filter_width is 0) */
    int wrap;            /* NTG_WRAP_* */
    int alpha_mode;      /* NTG_ALPHA_* */
    int in_xform;        /* NTG_XFORM_* applied after setImage */
    int out_xform;       /* NTG_XFORM_* applied to a copy of each level before encoding */
    float gamma;         /* for NTG_XFORM_GAMMA */
    int max_levels;      /* 0 = full chain down to 1x1 */
    int weighted;        /* alpha-weighted polyphase kernels (opt-in) */
    float cw[3];         /* colour weights; zeros mean 1,1,1 */
} ntg_chain_options;

/* Number of levels and encoded bytes of a chain (nvtt::countMipmaps, src/nvtt/Surface.cpp:181). */
int ntg_chain_levels(int w, int h, int max_levels);
size_t ntg_chain_bytes(int w, int h, const ntg_chain_options *opt);

/* The Surface-API loop of the reference (setImage -> input transform -> per level: copy, output
 * transform, Compressor::compress -> buildNextMipmap), src/nvtt/tests/imperativeapi.cpp:32-86 and
 * Compressor::Private::compress (src/nvtt/Context.cpp:217-346), for one BGRA8 image. All levels'
 * blocks are written back to back, largest level first. */
int ntg_compress_chain(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt,
                       void *d_blocks, void *stream);
/* Many same-shaped images from host memory with the copies overlapped: while image k is encoded on
 * `stream`, image k+1 is copied in and image k-1's blocks are copied out on two context-owned copy
 * streams (double-buffered device slots). h_bgra[i]: w*h BGRA8 texels; h_blocks[i]: ntg_chain_bytes
 * bytes; pinned host memory lets the copies run beside the kernels. Returns when every image's
 * blocks are on the host. The same loop as n calls of ntg_compress_chain_host; no reference
 * counterpart (the reference compresses one image per call). */
int ntg_compress_chains_host(ntg_context *ctx, int n, const void *const *h_bgra, int w, int h,
                             const ntg_chain_options *opt, void *const *h_blocks, void *stream);
/* Same from host memory: copies the image in, encodes, copies the blocks out, drains the stream. */
int ntg_compress_chain_host(ntg_context *ctx, const void *h_bgra, int w, int h, const ntg_chain_options *opt,
                            void *h_blocks, void *stream);

/* Mip chain only: writes every level, planar FP32 (linear, before the output transform),
 * back to back into d_levels (sum of 4*w_l*h_l floats). */
int ntg_mip_chain(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt,
                  float *d_levels, void *stream);

/* ---- batches: many textures of uneven sizes, whole chains, one CUDA graph ----
 * No counterpart in the reference, which compresses one image per Compressor::process call
 * (src/nvtt/Context.cpp:217-346); a batch runs that loop for every texture at once. Each
 * texture's chain gives the same blocks as ntg_compress_chain with the same options. The plan
 * groups the level steps of all textures by depth (one mip launch per depth and kernel variant;
 * the small last levels of all textures in one tail launch), encodes every level of every texture
 * with one launch per (format, quality), and captures the sequence in a CUDA graph. The device
 * pointers are baked into the graph: to compress new images, write them into the same input
 * buffers and launch again. A batch uses its context's tables and must be destroyed first. */
typedef struct ntg_batch ntg_batch;
typedef struct ntg_batch_texture {
    const void *d_bgra;        /* device BGRA8 level 0, w * h words */
    int w, h;
    ntg_chain_options opt;
    void *d_blocks;            /* device output, ntg_chain_bytes(w, h, &opt) bytes */
} ntg_batch_texture;

/* Plans the batch, allocates its level workspace (FP32 + BGRA8 levels of every texture), runs the
 * sequence once (this computes the outputs) and captures it. Launch shapes come from the tuning
 * cache when it holds an entry for this device and batch (file: $NTG_TUNE_CACHE, else
 * $HOME/.cache/ntg_tune.json), else defaults. */
int ntg_batch_build(ntg_context *ctx, const ntg_batch_texture *textures, int count, ntg_batch **out);
/* Replays the graph on `stream` (enqueue only). */
int ntg_batch_launch(ntg_batch *batch, void *stream);
/* Double buffering: binds a second set of inputs and outputs (d_bgra[i], d_blocks[i] for texture i,
 * same sizes and options) to the batch, with its own job lists and graph; ntg_batch_launch_alternate
 * replays that graph. While one binding's graph runs, the other's inputs can be copied in and its
 * outputs copied out. Both graphs use the batch's workspace: launch them on one stream (or order
 * them), never concurrently. Autotuning and ntg_batch_set_proposal recapture both. */
int ntg_batch_bind_alternate(ntg_batch *batch, const void *const *d_bgra, void *const *d_blocks);
int ntg_batch_launch_alternate(ntg_batch *batch, void *stream);
/* The batch over host buffers: for each of `count` sets, copies the set's images in
 * (h_bgra[set][texture], w * h words each), replays the graph and copies the blocks out
 * (h_blocks[set][texture], ntg_chain_bytes each), as Compressor::process would for each image and
 * texture. With an alternate binding the two bindings take turns, so that one set's copies run
 * beside the neighbouring sets' graphs (copy-in and copy-out on their own streams); without one the
 * sets run one after the other. Host buffers should be page-locked (cudaHostAlloc / cudaHostRegister)
 * for the copies to overlap. The batch's own device inputs and outputs (and the alternate binding's)
 * are overwritten. Returns after the last set's blocks are on the host. No counterpart in the
 * reference, which compresses one image per process() call (src/nvtt/Context.cpp:217-346). */
int ntg_batch_process_host(ntg_batch *batch, int count, const void *const *const *h_bgra, void *const *const *h_blocks,
                           void *stream);
/* Times candidate launch shapes on this batch (rows per strip and threads per CTA of the 2:1 mip
 * kernel, the tail threshold, blocks per CTA of each encoder), keeps the fastest, recaptures the
 * graph and stores the choice in the tuning cache. Synchronises `stream`. */
int ntg_batch_autotune(ntg_batch *batch, void *stream);
/* Texels of all levels, 4x4 blocks, kernel launches per replay, and the launch shapes in use:
 * shape[] = {strip, threads, tail texels, bc1 blocks/CTA, bc3 blocks/CTA, bc5 blocks/CTA}.
 * Any pointer may be NULL. */
int ntg_batch_info(const ntg_batch *batch, long long *texels, long long *blocks, int *launches, int shape[6]);
/* Runs the batch's phases once each, outside the graph, timed with CUDA events on `stream`:
 * ms[0] = every mip launch, ms[1..3] = the BC1, BC3, BC5 encoder launches (0 when absent), and
 * blocks[0..2] = the 4x4 blocks of each format. Synchronises `stream`. */
int ntg_batch_time_phases(ntg_batch *batch, void *stream, float ms[4], long long blocks[3]);
/* Measurement only: the cluster orderings the BC1 Level8 fit evaluates over the batch's BC1 blocks
 * (Normal and Production quality), four-cluster in bc1_orderings[0] and three-cluster in [1]
 * (icbc::compress_dxt1_cluster_fit, src/nvtt/icbc.h:3292-3325: four_total / three_total of each
 * block's reduced colour counts). Synchronises `stream`. */
int ntg_batch_count_work(ntg_batch *batch, void *stream, unsigned long long bc1_orderings[2]);
/* Encodes the batch's BC1 Normal-quality blocks through the learned endpoint proposal (see
 * ntg_compress_chain_learned; mlp NULL restores the full fit) and recaptures the graph; the network
 * must outlive the batch. ntg_batch_proposal_stats reads the last run's {kept, full fit, orderings}
 * (synchronises). */
int ntg_batch_set_proposal(ntg_batch *batch, struct ntg_mlp *mlp, int radius, float margin);
int ntg_batch_proposal_stats(ntg_batch *batch, unsigned long long stats[3]);
/* The same for one format: NTG_FORMAT_BC1 (as above) or NTG_FORMAT_BC3 (the BC3 Normal blocks' colour:
 * the network, trained on BC3 blocks, proposes squish Compress4's split; see ntg_compress_chain_learned).
 * Each format keeps its own network, search and margin. */
int ntg_batch_set_proposal_format(ntg_batch *batch, int format, struct ntg_mlp *mlp, int radius, float margin);
int ntg_batch_proposal_stats_format(ntg_batch *batch, int format, unsigned long long stats[3]);
int ntg_batch_destroy(ntg_batch *batch);

/* ---- the learned endpoint proposal's network ----
 * No counterpart in the reference. An MLP 48 -> 256 -> 256 -> 8 (GELU, tanh form; BF16 weights and
 * activations, FP32 accumulation) on the tcgen05 tensor cores: inputs are a 4x4 block's 16 texels
 * in the block's principal frame (centred on its weighted mean colour, divided by its RMS deviation
 * + 1/255, rotated onto the principal axis of its colours and two axes orthogonal to it, sorted
 * along the axis); outputs 0-5 are the two endpoints of the block's cluster fit in that frame,
 * output 6 the fit's error as log((SSE + 1) / (V + 1)) with V the block's weighted variance (both
 * in 8-bit, colour-weighted units), output 7 unused.
 * Parameters are one flat FP32 vector: W1 [256 x 48], b1 [256], W2 [256 x 256], b2 [256],
 * W3 [8 x 256], b3 [8] (weights row-major, out x in). Training is Adam (beta 0.9 / 0.999, eps 1e-8)
 * on the weighted mean squared error of the outputs (weights 1 for the endpoints, 0.25 for the
 * error, 0 for output 7). Device buffers: x [batch x 48], targets [batch x 8], y [batch x 16]
 * (columns 8-15 zero), all FP32 row-major; batch a multiple of 8. */
typedef struct ntg_mlp ntg_mlp;
int ntg_mlp_create(int device, unsigned long long seed, ntg_mlp **out);
int ntg_mlp_destroy(ntg_mlp *mlp);
int ntg_mlp_param_count(void);
int ntg_mlp_get_params(ntg_mlp *mlp, float *h_params);
int ntg_mlp_set_params(ntg_mlp *mlp, const float *h_params);
/* Inference: one persistent kernel per call, the weights resident in shared memory and the three
 * layers chained through TMEM; any batch size. */
int ntg_mlp_infer(ntg_mlp *mlp, const float *d_x, int batch, float *d_y, void *stream);
/* The same forward pass as three separate tensor-core products (the training path). */
int ntg_mlp_infer_unfused(ntg_mlp *mlp, const float *d_x, int batch, float *d_y, void *stream);
/* One forward + backward pass: the flat gradient (parameter layout) into d_grads (may be NULL) and
 * the loss into *h_loss (may be NULL); synchronises `stream`. */
int ntg_mlp_gradients(ntg_mlp *mlp, const float *d_x, const float *d_t, int batch, float *d_grads, float *h_loss,
                      void *stream);
/* One Adam step (enqueue only); the batch's loss into *d_loss (device, may be NULL). */
int ntg_mlp_train_step(ntg_mlp *mlp, const float *d_x, const float *d_t, int batch, float lr, float *d_loss,
                       void *stream);
/* Non-zero when a tensor-core wait of an earlier call gave up (synchronises the device). */
int ntg_mlp_status(ntg_mlp *mlp);
/* The bounded waits' limit: each tensor-core wait (mbarrier phase) of this network's kernels polls at
 * most `polls` times (negative: the default, 4,194,304) before it gives up; 0 makes every wait give
 * up at once, with no fault. A kernel whose wait gave up records it (ntg_mlp_status reports
 * NTG_ERROR_CUDA), waits with the default limit for the tensor-core work it has already issued, frees
 * its TMEM and returns, so later calls run normally. Also clears the recorded status; synchronises
 * the device. No counterpart in the reference. */
int ntg_mlp_set_wait_limit(ntg_mlp *mlp, int polls);
/* Search of the learned encode: `radius` is the half-width of the window of orderings around the
 * proposal's, in each cumulative cluster end; NTG_PROPOSAL_DESCENT | k instead runs a steepest descent
 * from the proposal's ordering (each move evaluates the orderings one step away in any end and goes to
 * the lowest error below the current one), at most k moves (BC1). */
#define NTG_PROPOSAL_DESCENT 256
/* Also with the BC1 search: after it, the block's endpoints are refitted by weighted least squares for
 * its indices (at most twice, kept only when the error drops) - a step the plain Level8 fit does not
 * take, so refitted blocks can be better than the reference's. */
#define NTG_PROPOSAL_REFIT 512
/* Learned encode of a chain (BC1 or BC3 at Normal quality; same options and output layout as
 * ntg_compress_chain). Each block's texels go through the network; its proposal seeds the cluster
 * fit's search - icbc's orderings for BC1, squish Compress4's splits for the BC3 colour block - which
 * evaluates only the orderings within `radius` (in each cumulative cluster end) of the proposal's
 * (BC1 also: a descent, NTG_PROPOSAL_DESCENT), with the full search's arithmetic and order; a block
 * whose result's error exceeds (1 + margin) x the network's estimate of the full fit's error gets the
 * full fit. BC3 alpha is the plain QuickCompress DXT5A. The network must have been trained on blocks
 * of the chain's format (ntg_chain_features / ntg_chain_targets with the same format). stats (host,
 * may be NULL; then nothing synchronises): {blocks kept from the pruned search, blocks given the full
 * fit, orderings evaluated by the pruned search}. */
int ntg_compress_chain_learned(ntg_context *ctx, ntg_mlp *mlp, const void *d_bgra, int w, int h,
                               const ntg_chain_options *opt, int radius, float margin, void *d_blocks,
                               unsigned long long *stats, void *stream);
/* The same pruned search with the proposals supplied by the caller (d_proposals [blocks x 16], the
 * network's output layout) instead of the network: seeds from other methods, for comparison. */
int ntg_compress_chain_proposed(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt,
                                const float *d_proposals, int radius, float margin, void *d_blocks, unsigned long long *stats,
                                void *stream);
/* Training data from a BC1 or BC3 chain: the network's inputs for every block of every level
 * (d_x [blocks x 48]: the block's texels as RGB in [0, 1] sorted along its principal axis, each
 * pulled towards the mean by its fit weight), and targets (d_t [blocks x 8]): the full fit's winning
 * ordering as cumulative weight fractions (BC1: three four-cluster ends, two three-cluster ends; BC3:
 * three split ends, then 1/3, 2/3), the fit's error as log((SSE + 1) / (V + 1)) in 8-bit units, 0, 0.
 * BC1 reads the fit's error from d_blocks (that chain's encoded blocks, e.g. ntg_compress_chain's
 * output); BC3 runs the search itself (d_blocks is only checked for NULL). */
int ntg_chain_features(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt, float *d_x,
                       void *stream);
int ntg_chain_targets(ntg_context *ctx, const void *d_bgra, int w, int h, const ntg_chain_options *opt,
                      const void *d_blocks, float *d_t, void *stream);
/* The network's matrix product on its own: C[M x N] (FP32) = A[M x K] * B[N x K]^T, A and B BF16
 * row-major, K a multiple of 8 (exposed for testing the tensor-core path). */
int ntg_gemm_bf16(const void *d_a, const void *d_b, int M, int N, int K, float *d_c, void *stream);

/* Phase timing of chain calls: when enabled, ntg_compress_chain records CUDA events on its stream
 * around the mip phase and the encode phase; ntg_profile_read waits for the last call's events and
 * returns the two durations in milliseconds. */
int ntg_profile_enable(ntg_context *ctx, int enable);
int ntg_profile_read(ntg_context *ctx, float *mips_ms, float *encode_ms);

/* ---- decode and error ---- */

/* Surface::setImage2D(format, Decoder_D3D10, ...) (src/nvtt/Surface.cpp:908-1116): blocks to a
 * planar FP32 image of w x h. */
int ntg_decode(ntg_context *ctx, int format, const void *d_blocks, int w, int h, float *d_rgba, void *stream);
/* nv::rmsColorError / rmsAlphaError (src/nvimage/ErrorMetric.cpp:13-71) sums in double:
 * d_sums[0] = colour squared error (alpha-weighted when alpha_mode is Transparency),
 * d_sums[1] = alpha squared error. rms = sqrt(sum / (w*h)). */
int ntg_error_sums(ntg_context *ctx, const float *d_ref, const float *d_img, int w, int h, int alpha_mode,
                   double *d_sums, void *stream);

/* ---- host-side tables (no GPU needed) ---- */

/* PolyphaseKernel weights (src/nvimage/Filter.cpp:520-566) and the window offsets
 * FloatImage::applyKernelX/Y start from (src/nvimage/FloatImage.cpp:1124-1131), as the kernels
 * receive them. Returns the window size; fills weights (dst_len * window) and lefts (dst_len)
 * when capacity allows. */
int ntg_host_polyphase(int filter, float width, const float *params, int src_len, int dst_len, float *weights,
                       int *lefts, int capacity);
/* The 8-bit transform tables of a chain: lut_in[256] = input transform of v/255; lut_composed[256]
 * = output(input(v/255)); lut8[512] = ColorBlock quantisation of lut_composed, then of v/255
 * (alpha); srgb_steps[256] = smallest float whose toSrgb code reaches k. Any pointer may be NULL. */
int ntg_host_transform_tables(int in_xform, int out_xform, float gamma, float *lut_in, float *lut_composed,
                              unsigned char *lut8, float *srgb_steps);

#ifdef __cplusplus
}
#endif
#endif /* NTG_H */
