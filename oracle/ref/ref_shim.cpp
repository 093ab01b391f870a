// C entry points into the reference library (NVTT 2.1.2) compiled from its own sources.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled together with the reference's sources by
// oracle/ref/Makefile into oracle/_ref/libnvtt_ref.so. The tests use it to pin the C
// restatement in oracle/ntg_oracle.c and to produce the golden fixtures under tests/golden/;
// nothing in the product links or loads it.
//
// Every function goes through the reference's own public or internal API; none restates an
// algorithm.

#include "nvtt/nvtt.h"
#include "nvtt/icbc.h"
#include "nvtt/QuickCompressDXT.h"
#include "nvtt/OptimalCompressDXT.h"
#include "nvtt/CompressorDX9.h"
#include "nvtt/CompressorDX10.h"
#include "nvtt/CompressionOptions.h"
#include "nvtt/Surface.h"
#include "nvimage/ColorBlock.h"
#include "nvimage/BlockDXT.h"
#include "nvimage/Filter.h"
#include "nvimage/FloatImage.h"
#include "nvmath/Gamma.h"

#include <string.h>
#include <vector>

using namespace nvtt;

namespace {

struct MemoryOutput : public OutputHandler {
    std::vector<unsigned char> bytes;
    virtual void beginImage(int, int, int, int, int, int) {}
    virtual bool writeData(const void * data, int size) {
        const unsigned char * p = (const unsigned char *)data;
        bytes.insert(bytes.end(), p, p + size);
        return true;
    }
    virtual void endImage() {}
};

struct CountingErrors : public ErrorHandler {
    int last = -1;
    virtual void error(Error e) { last = (int)e; }
};

Compressor & compressor() {
    static Compressor * c = NULL;
    if (c == NULL) {
        c = new Compressor();
        c->enableCudaAcceleration(false);
    }
    return *c;
}

void fill_options(CompressionOptions & co, int format, int quality, const float * cw) {
    co.setFormat((Format)format);
    co.setQuality((Quality)quality);
    if (cw) co.setColorWeights(cw[0], cw[1], cw[2], cw[3]);
}

nv::Filter * make_filter(int filter, float width, float p0, float p1) {
    if (filter == 0) return new nv::BoxFilter(width);
    if (filter == 1) return new nv::TriangleFilter(width);
    nv::KaiserFilter * k = new nv::KaiserFilter(width);
    k->setParameters(p0, p1);
    return k;
}

long long copy_out(const std::vector<unsigned char> & v, unsigned char * out, long long cap) {
    if ((long long)v.size() > cap) return -1;
    if (!v.empty()) memcpy(out, v.data(), v.size());
    return (long long)v.size();
}

} // namespace

extern "C" {

int ref_version() { return NVTT_VERSION; }

// icbc::compress_dxt1 (src/nvtt/icbc.h:3592), with three-colour mode and black as
// CompressorDXT1::compressBlock passes them (src/nvtt/BlockCompressor.cpp:219-222).
float ref_icbc_compress_dxt1(int level, const float * colors64, const float * weights16,
                             const float * cw3, int three_color_mode, int three_color_black,
                             unsigned char * out8) {
    compressor();
    return icbc::compress_dxt1((icbc::Quality)level, colors64, weights16, cw3,
                               three_color_mode != 0, three_color_black != 0, out8);
}

// Compressor::compress(Surface) over a planar FP32 RGBA image (the Surface API path).
long long ref_compress_planar(const float * rgba, int w, int h, int alpha_mode, int format,
                              int quality, const float * cw4, unsigned char * out, long long cap) {
    Surface s;
    const size_t n = (size_t)w * h;
    s.setImage(InputFormat_RGBA_32F, w, h, 1, rgba, rgba + n, rgba + 2 * n, rgba + 3 * n);
    s.setAlphaMode((AlphaMode)alpha_mode);
    CompressionOptions co;
    fill_options(co, format, quality, cw4);
    MemoryOutput mem;
    OutputOptions oo;
    oo.setOutputHandler(&mem);
    oo.setOutputHeader(false);
    if (!compressor().compress(s, 0, 0, co, oo)) return -2;
    return copy_out(mem.bytes, out, cap);
}

// One BC3 block through the compressor chooseCpuCompressor picks: FastCompressorDXT5 at Fastest,
// CompressorDXT5::compressBlock (src/nvtt/CompressorDX9.cpp:145) otherwise.
void ref_bc3_block(const unsigned char * bgra64, int alpha_mode, int quality, const float * cw4,
                   unsigned char * out16) {
    nv::ColorBlock cb((const uint *)bgra64);
    CompressionOptions co;
    fill_options(co, Format_BC3, quality, cw4);
    if (quality == Quality_Fastest) {   // chooseCpuCompressor (src/nvtt/Context.cpp:1076-1084)
        nv::FastCompressorDXT5 c;
        c.compressBlock(cb, (AlphaMode)alpha_mode, co.m, out16);
        return;
    }
    nv::CompressorDXT5 c;
    c.compressBlock(cb, (AlphaMode)alpha_mode, co.m, out16);
}

// One BC5 block through FastCompressorBC5 / ProductionCompressorBC5 (src/nvtt/CompressorDX10.cpp).
void ref_bc5_block(const unsigned char * bgra64, int quality, unsigned char * out16) {
    nv::ColorBlock cb((const uint *)bgra64);
    CompressionOptions co;
    fill_options(co, Format_BC5, quality, NULL);
    if (quality == Quality_Fastest || quality == Quality_Normal) {
        nv::FastCompressorBC5 c;
        c.compressBlock(cb, AlphaMode_None, co.m, out16);
    } else {
        nv::ProductionCompressorBC5 c;
        c.compressBlock(cb, AlphaMode_None, co.m, out16);
    }
}

// One BC1a block through CompressorDXT1a::compressBlock (src/nvtt/CompressorDX9.cpp:83-111),
// the compressor chooseCpuCompressor picks above Fastest (src/nvtt/Context.cpp:1058-1066).
void ref_bc1a_block(const unsigned char * bgra64, int alpha_mode, const float * cw4, unsigned char * out8) {
    nv::ColorBlock cb((const uint *)bgra64);
    CompressionOptions co;
    fill_options(co, Format_BC1a, Quality_Normal, cw4);
    memset(out8, 0, 8);
    nv::CompressorDXT1a c;
    c.compressBlock(cb, (AlphaMode)alpha_mode, co.m, out8);
}

// One BC4 block through FastCompressorBC4 / ProductionCompressorBC4 (src/nvtt/CompressorDX10.cpp).
void ref_bc4_block(const unsigned char * bgra64, int quality, unsigned char * out8) {
    nv::ColorBlock cb((const uint *)bgra64);
    CompressionOptions co;
    fill_options(co, Format_BC4, quality, NULL);
    if (quality == Quality_Fastest || quality == Quality_Normal) {
        nv::FastCompressorBC4 c;
        c.compressBlock(cb, AlphaMode_None, co.m, out8);
    } else {
        nv::ProductionCompressorBC4 c;
        c.compressBlock(cb, AlphaMode_None, co.m, out8);
    }
}

void ref_dxt5a_quick(const unsigned char * a16, unsigned char * out8) {
    nv::AlphaBlock4x4 ab;
    for (int i = 0; i < 16; i++) { ab.alpha[i] = a16[i]; ab.weights[i] = 1.0f; }
    nv::AlphaBlockDXT5 blk;
    nv::QuickCompress::compressDXT5A(ab, &blk);
    memcpy(out8, &blk, 8);
}

void ref_dxt5a_optimal(const unsigned char * a16, unsigned char * out8) {
    nv::AlphaBlock4x4 ab;
    for (int i = 0; i < 16; i++) { ab.alpha[i] = a16[i]; ab.weights[i] = 1.0f; }
    nv::AlphaBlockDXT5 blk;
    memset(&blk, 0, sizeof(blk));
    nv::OptimalCompress::compressDXT5A(ab, &blk);
    memcpy(out8, &blk, 8);
}

void ref_dxt1_single_color(int r, int g, int b, unsigned char * out8) {
    nv::Color32 c((uint8)r, (uint8)g, (uint8)b, 255);
    nv::BlockDXT1 blk;
    nv::OptimalCompress::compressDXT1(c, &blk);
    memcpy(out8, &blk, 8);
}

void ref_quick_dxt1(const unsigned char * bgra64, unsigned char * out8) {
    nv::ColorBlock cb((const uint *)bgra64);
    nv::BlockDXT1 blk;
    nv::QuickCompress::compressDXT1(cb, &blk);
    memcpy(out8, &blk, 8);
}

// ColorBlock::init(float) gather (src/nvimage/ColorBlock.cpp:80): truncating quantiser and
// edge repetition, for a block at (x, y) of a planar FP32 image.
void ref_colorblock_init(const float * rgba, int w, int h, int x, int y, unsigned char * bgra64) {
    nv::ColorBlock cb;
    cb.init((uint)w, (uint)h, rgba, (uint)x, (uint)y);
    memcpy(bgra64, cb.colors(), 64);
}

// PolyphaseKernel weights (src/nvimage/Filter.cpp:520). Returns the window size.
int ref_polyphase(int filter, float width, float p0, float p1, int src_len, int dst_len,
                  float * weights, int cap) {
    nv::Filter * f = make_filter(filter, width, p0, p1);
    nv::PolyphaseKernel k(*f, (uint)src_len, (uint)dst_len, 32);
    const int ws = k.windowSize();
    if ((long long)ws * dst_len <= cap) {
        for (int i = 0; i < dst_len; i++)
            for (int j = 0; j < ws; j++) weights[i * ws + j] = k.valueAt(i, j);
    }
    delete f;
    return ws;
}

float ref_filter_evaluate(int filter, float width, float p0, float p1, float x) {
    nv::Filter * f = make_filter(filter, width, p0, p1);
    float v = f->evaluate(x);
    delete f;
    return v;
}

void ref_powf_11_5(const float * src, float * dst, int n) { nv::powf_11_5(src, dst, n); }
void ref_powf_5_11(const float * src, float * dst, int n) { nv::powf_5_11(src, dst, n); }

// Surface mip chain (src/nvtt/Surface.cpp:1344) from BGRA8 input.
//   in_xform:  0 none, 1 toLinear(gamma), 2 toLinearFromSrgb
//   out_xform: 0 none, 1 toGamma(gamma),  2 toSrgb
// Writes, level by level, the linear level (planar FP32) into `linear` and the level after the
// output transform into `encoded` (either may be NULL). Returns the number of levels built.
int ref_mip_chain(const unsigned char * bgra, int w, int h, int filter, float width, float p0,
                  float p1, int wrap, int alpha_mode, int in_xform, int out_xform, float gamma,
                  int max_levels, float * linear, float * encoded) {
    Surface img;
    img.setWrapMode((WrapMode)wrap);
    img.setAlphaMode((AlphaMode)alpha_mode);
    img.setImage(InputFormat_BGRA_8UB, w, h, 1, bgra);
    if (in_xform == 1) img.toLinear(gamma);
    else if (in_xform == 2) img.toLinearFromSrgb();
    size_t off = 0;
    int levels = 0;
    const float params[2] = {p0, p1};
    for (;;) {
        const size_t n = (size_t)img.width() * img.height() * 4;
        if (linear) memcpy(linear + off, img.data(), n * sizeof(float));
        if (encoded) {
            Surface tmp = img;
            if (out_xform == 1) tmp.toGamma(gamma);
            else if (out_xform == 2) tmp.toSrgb();
            memcpy(encoded + off, tmp.data(), n * sizeof(float));
        }
        off += n;
        levels++;
        if (levels >= max_levels) break;
        bool ok;
        if (filter == 2) ok = img.buildNextMipmap(MipmapFilter_Kaiser, width, params);
        else ok = img.buildNextMipmap((MipmapFilter)filter, width, params);
        if (!ok) break;
    }
    return levels;
}

// Alpha-weighted separable resize built from the reference's weighted kernels
// FloatImage::applyKernelX/Y(..., alpha, ...) (src/nvimage/FloatImage.cpp:1212-1281): the alpha
// plane is filtered with the plain kernels, the colour planes with the alpha-weighted ones
// (X pass weighted by the source alpha, Y pass by the X-filtered alpha).
void ref_resize_weighted(const float * rgba, int w, int h, int dw, int dh, int filter, float width,
                         float p0, float p1, int wrap, float * out) {
    nv::FloatImage src;
    src.allocate(4, w, h, 1);
    memcpy(src.channel(0), rgba, sizeof(float) * 4 * (size_t)w * h);
    nv::Filter * f = make_filter(filter, width, p0, p1);
    nv::PolyphaseKernel kx(*f, (uint)w, (uint)dw, 32);
    nv::PolyphaseKernel ky(*f, (uint)h, (uint)dh, 32);
    nv::FloatImage tmp;
    tmp.allocate(4, dw, h, 1);
    nv::FloatImage::WrapMode wm = (nv::FloatImage::WrapMode)wrap;
    for (int y = 0; y < h; y++) src.applyKernelX(kx, y, 0, 3, wm, tmp.channel(3) + (size_t)y * dw);
    for (int c = 0; c < 3; c++)
        for (int y = 0; y < h; y++) src.applyKernelX(kx, y, 0, c, 3, wm, tmp.channel(c) + (size_t)y * dw);
    const size_t dn = (size_t)dw * dh;
    for (int x = 0; x < dw; x++) tmp.applyKernelY(ky, x, 0, 3, wm, out + 3 * dn + x, dw);
    for (int c = 0; c < 3; c++)
        for (int x = 0; x < dw; x++) tmp.applyKernelY(ky, x, 0, c, 3, wm, out + c * dn + x, dw);
    delete f;
}

// Surface::resize(w, h, d, filter, filterWidth, params) (src/nvtt/Surface.cpp:1152-1230) of a
// planar FP32 image, with the surface's wrap and alpha modes. filter is an nvtt::ResizeFilter.
void ref_surface_resize(const float * rgba, int w, int h, int dw, int dh, int filter, float width, float p0, float p1,
                        int wrap, int alpha_mode, float * out) {
    Surface s;
    const size_t n = (size_t)w * h;
    s.setImage(InputFormat_RGBA_32F, w, h, 1, rgba, rgba + n, rgba + 2 * n, rgba + 3 * n);
    s.setWrapMode((WrapMode)wrap);
    s.setAlphaMode((AlphaMode)alpha_mode);
    const float params[2] = {p0, p1};
    s.resize(dw, dh, 1, (ResizeFilter)filter, width, params);
    memcpy(out, s.data(), sizeof(float) * 4 * (size_t)dw * dh);
}

// nv::getTargetExtent (src/nvtt/Surface.cpp:220-326) for a 2D texture.
void ref_target_extent(int w, int h, int max_extent, int round_mode, int * out_w, int * out_h) {
    int d = 1;
    nv::getTargetExtent(&w, &h, &d, max_extent, (RoundMode)round_mode, TextureType_2D);
    *out_w = w;
    *out_h = h;
}

// The same for a texture type (TextureType_2D, _Cube or _Array).
void ref_target_extent_type(int w, int h, int max_extent, int round_mode, int type, int * out_w, int * out_h) {
    int d = 1;
    nv::getTargetExtent(&w, &h, &d, max_extent, (RoundMode)round_mode, (TextureType)type);
    *out_w = w;
    *out_h = h;
}

// Decode blocks with Surface::setImage2D (src/nvtt/Surface.cpp:908) into planar FP32.
int ref_decode(int format, const unsigned char * blocks, int w, int h, float * out) {
    Surface s;
    if (!s.setImage2D((Format)format, Decoder_D3D10, w, h, blocks)) return -1;
    memcpy(out, s.data(), sizeof(float) * 4 * (size_t)w * h);
    return 0;
}

// nvtt::rmsError / rmsAlphaError (src/nvtt/Surface.cpp:3270-3280) between a planar FP32 image
// and the D3D10 decode of its blocks.
int ref_rms(int format, const float * rgba, const unsigned char * blocks, int w, int h,
            int alpha_mode, float * rms_color, float * rms_alpha) {
    Surface ref;
    const size_t n = (size_t)w * h;
    ref.setImage(InputFormat_RGBA_32F, w, h, 1, rgba, rgba + n, rgba + 2 * n, rgba + 3 * n);
    ref.setAlphaMode((AlphaMode)alpha_mode);
    Surface dec;
    if (!dec.setImage2D((Format)format, Decoder_D3D10, w, h, blocks)) return -1;
    *rms_color = rmsError(ref, dec);
    *rms_alpha = rmsAlphaError(ref, dec);
    return 0;
}

// Compressor::process (src/nvtt/Context.cpp:117): the InputOptions pipeline, DDS container
// included, from one BGRA8 image. Returns the byte count or a negative nvtt::Error - 100.
long long ref_process(const unsigned char * bgra, int w, int h, int format, int quality,
                      int mip_filter, int alpha_mode, int wrap, float in_gamma, float out_gamma,
                      int max_level, int header, unsigned char * out, long long cap) {
    InputOptions io;
    io.setTextureLayout(TextureType_2D, w, h);
    io.setMipmapData(bgra, w, h);
    io.setFormat(InputFormat_BGRA_8UB);
    io.setAlphaMode((AlphaMode)alpha_mode);
    io.setWrapMode((WrapMode)wrap);
    io.setGamma(in_gamma, out_gamma);
    io.setMipmapFilter((MipmapFilter)mip_filter);
    io.setMipmapGeneration(max_level != 0, max_level);
    CompressionOptions co;
    fill_options(co, format, quality, NULL);
    MemoryOutput mem;
    CountingErrors err;
    OutputOptions oo;
    oo.setOutputHandler(&mem);
    oo.setErrorHandler(&err);
    oo.setOutputHeader(header != 0);
    if (!compressor().process(io, co, oo)) return -100 - (err.last < 0 ? 0 : err.last);
    return copy_out(mem.bytes, out, cap);
}

// Compressor::process with the rest of the options the GPU drop-in mirrors. `data` holds, for each
// face (cube map) or layer (array), `nsrc_levels` source levels back to back (largest first) in
// `input_format` (0 BGRA8, 1 RGBA16F, 2 RGBA32F, interleaved); opts[] = {kaiser width, kaiser alpha,
// kaiser stretch, in gamma, out gamma, colour weights r, g, b, a}; flags[] = {container, srgb, user
// version, normal map, normalize mipmaps, max extent, round mode, texture type, layers}.
long long ref_process_ex(const void * data, int w, int h, int input_format, int nsrc_levels,
                         int format, int quality, int mip_filter, int alpha_mode, int wrap,
                         int max_level, int header, const float * opts, const int * flags,
                         unsigned char * out, long long cap) {
    InputOptions io;
    const TextureType type = (TextureType)flags[7];
    const int faces = type == TextureType_Cube ? 6 : (type == TextureType_Array ? flags[8] : 1);
    io.setTextureLayout(type, w, h, 1, type == TextureType_Array ? faces : 1);
    io.setFormat((InputFormat)input_format);
    const int bpp = input_format == 0 ? 4 : (input_format == 1 ? 8 : 16);
    const unsigned char * p = (const unsigned char *)data;
    for (int f = 0; f < faces; f++) {
        int lw = w, lh = h;
        for (int l = 0; l < nsrc_levels; l++) {
            io.setMipmapData(p, lw, lh, 1, f, l);
            p += (size_t)lw * lh * bpp;
            lw = lw > 1 ? lw / 2 : 1;
            lh = lh > 1 ? lh / 2 : 1;
        }
    }
    io.setAlphaMode((AlphaMode)alpha_mode);
    io.setWrapMode((WrapMode)wrap);
    io.setGamma(opts[3], opts[4]);
    io.setMipmapFilter((MipmapFilter)mip_filter);
    io.setKaiserParameters(opts[0], opts[1], opts[2]);
    io.setMipmapGeneration(max_level != 0, max_level);
    io.setNormalMap(flags[3] != 0);
    io.setNormalizeMipmaps(flags[4] != 0);
    io.setMaxExtents(flags[5]);
    io.setRoundMode((RoundMode)flags[6]);
    CompressionOptions co;
    fill_options(co, format, quality, opts + 5);
    MemoryOutput mem;
    CountingErrors err;
    OutputOptions oo;
    oo.setOutputHandler(&mem);
    oo.setErrorHandler(&err);
    oo.setOutputHeader(header != 0);
    oo.setContainer((Container)flags[0]);
    oo.setSrgbFlag(flags[1] != 0);
    oo.setUserVersion(flags[2]);
    if (!compressor().process(io, co, oo)) return -100 - (err.last < 0 ? 0 : err.last);
    return copy_out(mem.bytes, out, cap);
}

} // extern "C"
