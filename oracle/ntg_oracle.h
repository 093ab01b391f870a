/* CPU restatement of the NVTT 2.1.2 texture hot path: mip filtering and BC1/BC3/BC5 block
 * encoding, in plain C.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle the CUDA kernels are checked against, and the
 * timed CPU baseline of the benchmark. Only tests/, the smoke check and the benchmark's CPU leg
 * may load it; the product never calls it.
 *
 * Parity: pinned against the reference library compiled from its own sources
 * (oracle/ref/Makefile -> oracle/_ref/libnvtt_ref.so) by tests/test_oracle_pin.py, and against
 * the golden fixtures in tests/golden/ written by tests/golden/make_golden.py.
 *
 * Arithmetic contract: IEEE-754 single precision, every product and sum rounded separately
 * (build with -ffp-contract=off), the scalar code paths of the reference. */
#ifndef NTG_ORACLE_H
#define NTG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* nvtt enums, numerically as the reference declares them. */
enum { ORA_FMT_BC1 = 1, ORA_FMT_BC1A = 2, ORA_FMT_BC3 = 4, ORA_FMT_BC4 = 6, ORA_FMT_BC5 = 7 };
enum { ORA_Q_FASTEST = 0, ORA_Q_NORMAL = 1, ORA_Q_PRODUCTION = 2, ORA_Q_HIGHEST = 3 };
enum { ORA_WRAP_CLAMP = 0, ORA_WRAP_REPEAT = 1, ORA_WRAP_MIRROR = 2 };
enum { ORA_FILTER_BOX = 0, ORA_FILTER_TRIANGLE = 1, ORA_FILTER_KAISER = 2 };
enum { ORA_ALPHA_NONE = 0, ORA_ALPHA_TRANSPARENCY = 1 };
enum { ORA_XFORM_NONE = 0, ORA_XFORM_GAMMA = 1, ORA_XFORM_SRGB = 2 };

int ora_version(void);

/* ---- BC1 (icbc 1.05) ---- */
float ora_bc1_block(int icbc_level, const float *colors64, const float *weights16, const float *cw3,
                    int three_color_mode, int three_color_black, uint8_t *out8);
/* FloatColorCompressor over a planar FP32 image, nvtt quality -> icbc level mapping. */
void ora_bc1_image(const float *rgba, int w, int h, int alpha_mode, int quality, const float *cw3,
                   uint8_t *out, int threads);

/* ---- BC3 / BC5 / interpolated-alpha ---- */
void ora_colorblock_gather(const float *rgba, int w, int h, int x, int y, uint8_t *bgra64);
void ora_dxt5a_quick(const uint8_t *a16, uint8_t *out8);
void ora_dxt5a_optimal(const uint8_t *a16, uint8_t *out8);
void ora_dxt1_single_color(int r, int g, int b, uint8_t *out8);
void ora_quick_dxt1(const uint8_t *bgra64, uint8_t *out8);
void ora_bc3_block(const uint8_t *bgra64, int alpha_mode, int quality, const float *cw3, uint8_t *out16);
void ora_bc5_block(const uint8_t *bgra64, int quality, uint8_t *out16);
void ora_bc3_image(const float *rgba, int w, int h, int alpha_mode, int quality, const float *cw3,
                   uint8_t *out, int threads);
void ora_bc5_image(const float *rgba, int w, int h, int quality, uint8_t *out, int threads);
/* BC1a (Normal quality and above) and BC4. */
void ora_dxt1a_single_color(int r, int g, int b, uint32_t alpha_mask, uint8_t *out8);
void ora_bc1a_block(const uint8_t *bgra64, int alpha_mode, const float *cw3, uint8_t *out8);
void ora_bc4_block(const uint8_t *bgra64, int quality, uint8_t *out8);
void ora_bc1a_image(const float *rgba, int w, int h, int alpha_mode, const float *cw3, uint8_t *out, int threads);
void ora_bc4_image(const float *rgba, int w, int h, int quality, uint8_t *out, int threads);
/* Target extent of the InputOptions resize step (2D). */
void ora_target_extent(int w, int h, int max_extent, int round_mode, int *out_w, int *out_h);
/* BC3/BC5 from an already quantised BGRA8 image (ColorBlock path without the float stage). */
void ora_bc3_image_u8(const uint8_t *bgra, int w, int h, int alpha_mode, int quality, const float *cw3,
                      uint8_t *out, int threads);

/* ---- filters and mips ---- */
float ora_filter_evaluate(int filter, float width, float p0, float p1, float x);
/* Polyphase weights: returns the window size; writes dst_len*window weights when they fit. */
int ora_polyphase(int filter, float width, float p0, float p1, int src_len, int dst_len,
                  float *weights, int cap);
int ora_polyphase_left(float width_scaled, int src_len, int dst_len, int i);
void ora_fast_downsample(const float *src, int w, int h, int channels, float *dst);
void ora_resize(const float *src, int w, int h, int channels, int dw, int dh, int filter, float width,
                float p0, float p1, int wrap, float *dst);
void ora_resize_weighted(const float *src, int w, int h, int dw, int dh, int filter, float width,
                         float p0, float p1, int wrap, float *dst);
/* Surface mip chain from BGRA8, mirroring the reference Surface flow; see the .c file. */
int ora_mip_chain(const uint8_t *bgra, int w, int h, int filter, float width, float p0, float p1,
                  int wrap, int alpha_mode, int in_xform, int out_xform, float gamma, int max_levels,
                  float *linear, float *encoded);

/* ---- colour transforms ---- */
void ora_set_image_bgra8(const uint8_t *bgra, int n, float *rgba);
void ora_powf_11_5(const float *src, float *dst, int n);
void ora_powf_5_11(const float *src, float *dst, int n);
void ora_to_srgb(const float *src, float *dst, int n);
void ora_from_srgb(const float *src, float *dst, int n);

/* ---- decode and error ---- */
int ora_decode(int format, const uint8_t *blocks, int w, int h, float *rgba);
int ora_rms(int format, const float *rgba, const uint8_t *blocks, int w, int h, int alpha_mode,
            float *rms_color, float *rms_alpha);

/* Number of floats in [0, 2] where counting `steps` disagrees with toSrgb + ColorBlock quantiser. */
long long ora_count_srgb_step_mismatches(const float *steps, int threads);

#ifdef __cplusplus
}
#endif
#endif
