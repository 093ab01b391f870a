// Test driver of the nvtt:: drop-in API (include/nvtt/nvtt.h), written the way an NVTT user calls
// the library (src/nvtt/tools/compress.cpp, src/nvtt/tests/imperativeapi.cpp of the reference).
//
//   nvtt_harness <mode> <input file | -> <output file | -> key=value ...
//
// modes:
//   process  InputOptions + Compressor::process (levels 0..nsrc-1 of the input file are source mipmaps,
//            for each face of a cube map (type=1) or layer of an array (type=3, layers=n) in turn)
//   estimate the same InputOptions, Compressor::estimateSize only (no GPU work): prints "estimate=<n>"
//   surface  the Surface loop: setImage, toLinear, {copy, toGamma, compress, buildNextMipmap}
//   header   Compressor::outputHeader only (no GPU work)
//   rms      BC-encode level 0, decode it with setImage2D, print rmsError / rmsAlphaError
// Prints "bytes=<n> estimate=<n>" (or "rms=<color> <alpha>") and exits 0, or prints "error=<nvtt::Error>"
// and exits 10 + the error code.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "nvtt/nvtt.h"

namespace {

struct Memory : public nvtt::OutputHandler {
    std::vector<unsigned char> bytes;
    int images = 0;
    void beginImage(int, int, int, int, int, int) override { images++; }
    bool writeData(const void *data, int size) override {
        bytes.insert(bytes.end(), (const unsigned char *)data, (const unsigned char *)data + size);
        return true;
    }
    void endImage() override {}
};

struct LastError : public nvtt::ErrorHandler {
    int last = -1;
    void error(nvtt::Error e) override { last = (int)e; }
};

std::map<std::string, std::string> g_opt;

double num(const char *key, double def) {
    auto it = g_opt.find(key);
    return it == g_opt.end() ? def : std::atof(it->second.c_str());
}

std::vector<unsigned char> read_file(const char *path) {
    std::vector<unsigned char> v;
    if (std::strcmp(path, "-") == 0) return v;
    FILE *f = std::fopen(path, "rb");
    if (!f) return v;
    unsigned char buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) v.insert(v.end(), buf, buf + n);
    std::fclose(f);
    return v;
}

int fail(const LastError &err) {
    std::printf("error=%d\n", err.last < 0 ? 0 : err.last);
    return 10 + (err.last < 0 ? 0 : err.last);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: nvtt_harness <process|estimate|surface|header|rms> <in> <out> key=value...\n");
        return 2;
    }
    const std::string mode = argv[1];
    for (int i = 4; i < argc; i++) {
        const char *eq = std::strchr(argv[i], '=');
        if (eq) g_opt[std::string(argv[i], (size_t)(eq - argv[i]))] = eq + 1;
    }
    const int w = (int)num("w", 16), h = (int)num("h", 16);
    const nvtt::InputFormat inFormat = (nvtt::InputFormat)(int)num("input_format", 0);
    const int nsrc = (int)num("nsrc", 1);
    const int maxLevel = (int)num("max_level", -1);
    const bool normal = num("normal", 0) != 0;
    const bool srgbCurve = num("srgb_xform", 0) != 0;
    const float gin = (float)num("gin", 2.2), gout = (float)num("gout", 2.2);
    const nvtt::MipmapFilter filter = (nvtt::MipmapFilter)(int)num("filter", 0);
    const float kaiser[3] = {(float)num("kw", 3.0), (float)num("ka", 4.0), (float)num("ks", 1.0)};
    std::vector<unsigned char> input = read_file(argv[2]);

    nvtt::CompressionOptions co;
    co.setFormat((nvtt::Format)(int)num("format", 1));
    co.setQuality((nvtt::Quality)(int)num("quality", 1));
    co.setColorWeights((float)num("cw_r", 1), (float)num("cw_g", 1), (float)num("cw_b", 1), (float)num("cw_a", 1));

    Memory mem;
    LastError err;
    nvtt::OutputOptions oo;
    oo.setOutputHandler(&mem);
    oo.setErrorHandler(&err);
    oo.setOutputHeader(num("header", 1) != 0);
    oo.setContainer((nvtt::Container)(int)num("container", 0));
    oo.setSrgbFlag(num("srgb", 0) != 0);
    oo.setUserVersion((int)num("version", 0));

    nvtt::Compressor compressor;
    int estimate = 0;
    int mipmapCount = 1;
    if (maxLevel != 0) {  // nvtt::countMipmaps, capped like Compressor::process
        int x = w, y = h;
        while (x != 1 || y != 1) { x = x > 1 ? x / 2 : 1; y = y > 1 ? y / 2 : 1; mipmapCount++; }
        if (maxLevel > 0 && maxLevel < mipmapCount) mipmapCount = maxLevel;
    }

    if (mode == "header") {
        const nvtt::TextureType type = (nvtt::TextureType)(int)num("type", 0);
        const int arraySize = type == nvtt::TextureType_Array ? (int)num("layers", 1) : 1;
        if (!compressor.outputHeader(type, w, h, 1, arraySize, mipmapCount, normal, co, oo)) return fail(err);
    } else if (mode == "process" || mode == "estimate") {
        // type=0 2D, 1 cube map (six faces), 3 array of `layers` images; the input holds each face's
        // (or layer's) source levels, face by face
        nvtt::InputOptions io;
        const nvtt::TextureType type = (nvtt::TextureType)(int)num("type", 0);
        const int faces = type == nvtt::TextureType_Cube ? 6 : (type == nvtt::TextureType_Array ? (int)num("layers", 1) : 1);
        io.setTextureLayout(type, w, h, 1, type == nvtt::TextureType_Array ? faces : 1);
        io.setFormat(inFormat);
        const size_t bpp = inFormat == nvtt::InputFormat_BGRA_8UB ? 4 : (inFormat == nvtt::InputFormat_RGBA_16F ? 8 : 16);
        size_t off = 0;
        for (int f = 0; f < faces; f++) {
            int lw = w, lh = h;
            for (int l = 0; l < nsrc; l++) {
                if (off + (size_t)lw * lh * bpp > input.size()) { std::fprintf(stderr, "short input\n"); return 2; }
                if (!io.setMipmapData(input.data() + off, lw, lh, 1, f, l)) { std::fprintf(stderr, "setMipmapData\n"); return 2; }
                off += (size_t)lw * lh * bpp;
                lw = lw > 1 ? lw / 2 : 1;
                lh = lh > 1 ? lh / 2 : 1;
            }
        }
        io.setAlphaMode((nvtt::AlphaMode)(int)num("alpha", 0));
        io.setWrapMode((nvtt::WrapMode)(int)num("wrap", 2));
        io.setGamma(gin, gout);
        io.setMipmapFilter(filter);
        io.setKaiserParameters(kaiser[0], kaiser[1], kaiser[2]);
        io.setMipmapGeneration(maxLevel != 0, maxLevel);
        io.setNormalMap(normal);
        io.setNormalizeMipmaps(num("normalize", 1) != 0);
        io.setMaxExtents((int)num("max_extent", 0));
        io.setRoundMode((nvtt::RoundMode)(int)num("round_mode", 0));
        estimate = compressor.estimateSize(io, co);
        if (mode == "estimate") {  // the size process() would write after the header; needs no GPU
            std::printf("estimate=%d\n", estimate);
            return 0;
        }
        if (!compressor.process(io, co, oo)) return fail(err);
    } else if (mode == "surface" || mode == "rms") {
        nvtt::Surface img;
        if (!img.setImage(inFormat, w, h, 1, input.data())) { std::fprintf(stderr, "setImage\n"); return 3; }
        img.setWrapMode((nvtt::WrapMode)(int)num("wrap", 2));
        img.setAlphaMode((nvtt::AlphaMode)(int)num("alpha", 0));
        img.setNormalMap(normal);
        if (mode == "rms") {
            oo.setOutputHeader(false);
            if (!compressor.compress(img, 0, 0, co, oo)) return fail(err);
            nvtt::Surface decoded;
            if (!decoded.setImage2D(co.format(), nvtt::Decoder_D3D10, w, h, mem.bytes.data())) return 4;
            std::printf("rms=%.9g %.9g\n", nvtt::rmsError(img, decoded), nvtt::rmsAlphaError(img, decoded));
            return 0;
        }
        if (!normal) {
            if (srgbCurve) img.toLinearFromSrgb();
            else img.toLinear(gin);
        }
        const int maxExtent = (int)num("max_extent", 0), roundMode = (int)num("round_mode", 0);
        if (maxExtent > 0 || roundMode != 0) {  // the InputOptions resize step, through the Surface API
            img.resize(maxExtent, (nvtt::RoundMode)roundMode, nvtt::ResizeFilter_Box);
            if (maxLevel != 0) {
                int x = img.width(), y = img.height();
                mipmapCount = 1;
                while (x != 1 || y != 1) { x = x > 1 ? x / 2 : 1; y = y > 1 ? y / 2 : 1; mipmapCount++; }
                if (maxLevel > 0 && maxLevel < mipmapCount) mipmapCount = maxLevel;
            }
        }
        estimate = compressor.estimateSize(img, mipmapCount, co);
        if (!compressor.outputHeader(img, mipmapCount, co, oo)) return fail(err);
        for (int m = 0; m < mipmapCount; m++) {
            nvtt::Surface tmp = img;
            if (!normal) {
                if (srgbCurve) tmp.toSrgb();
                else tmp.toGamma(gout);
            }
            if (!compressor.compress(tmp, 0, m, co, oo)) return fail(err);
            if (m + 1 < mipmapCount) {
                const bool ok = filter == nvtt::MipmapFilter_Kaiser
                                    ? img.buildNextMipmap(filter, kaiser[0], kaiser + 1)
                                    : img.buildNextMipmap(filter);
                if (!ok) { std::fprintf(stderr, "buildNextMipmap\n"); return 3; }
            }
        }
    } else {
        std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
        return 2;
    }

    if (std::strcmp(argv[3], "-") != 0) {
        FILE *f = std::fopen(argv[3], "wb");
        if (!f || std::fwrite(mem.bytes.data(), 1, mem.bytes.size(), f) != mem.bytes.size()) return 5;
        std::fclose(f);
    }
    std::printf("bytes=%zu estimate=%d images=%d\n", mem.bytes.size(), estimate, mem.images);
    return 0;
}
