/* Test driver of the plain-C interface (include/nvtt/nvtt_wrapper.h), written in C99 the way a C
 * program uses NVTT's C interface: option handles, setters, callbacks, nvttCompress.
 *
 *   nvtt_wrapper_harness <input file> <output file | -> key=value ...
 *
 * Keys (defaults): w h (16), format (1), quality (1), filter (0), alpha (0), wrap (2), max_level (-1),
 * container (0), srgb (0), header (1), normal (0), normalize (1), input_format (0), nsrc (1),
 * gin gout (2.2), kw ka ks (3 4 1), cw_r cw_g cw_b cw_a (1), max_extent (0), round_mode (0),
 * dither (0), file (write through nvttSetOutputOptionsFileName to the output path instead of the
 * output callback).
 * Prints "bytes=<n> estimate=<n> images=<n> version=<n>" and exits 0, or prints "error=<NvttError>" and
 * exits 10 + the error code. */
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nvtt/nvtt_wrapper.h"

static unsigned char *g_out;
static size_t g_len, g_cap;
static int g_images, g_error = -1;

static void on_begin(int size, int width, int height, int depth, int face, int miplevel) {
    (void)size; (void)width; (void)height; (void)depth; (void)face; (void)miplevel;
    g_images++;
}

static bool on_output(const void *data, int size) {
    if (g_len + (size_t)size > g_cap) {
        g_cap = (g_len + (size_t)size) * 2;
        g_out = (unsigned char *)realloc(g_out, g_cap);
        if (!g_out) return false;
    }
    memcpy(g_out + g_len, data, (size_t)size);
    g_len += (size_t)size;
    return true;
}

static void on_end(void) {}

static void on_error(NvttError e) { g_error = (int)e; }

static int g_argc;
static char **g_argv;

static double num(const char *key, double def) {
    size_t n = strlen(key);
    for (int i = 3; i < g_argc; i++)
        if (strncmp(g_argv[i], key, n) == 0 && g_argv[i][n] == '=') return atof(g_argv[i] + n + 1);
    return def;
}

static unsigned char *read_file(const char *path, size_t *len) {
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    unsigned char *buf = (unsigned char *)malloc(n > 0 ? (size_t)n : 1);
    *len = fread(buf, 1, (size_t)n, f);
    fclose(f);
    return buf;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: nvtt_wrapper_harness <in> <out> key=value...\n");
        return 2;
    }
    g_argc = argc;
    g_argv = argv;
    const int w = (int)num("w", 16), h = (int)num("h", 16);
    const int in_format = (int)num("input_format", 0), nsrc = (int)num("nsrc", 1);
    const int max_level = (int)num("max_level", -1);
    const bool to_file = num("file", 0) != 0;
    size_t in_len = 0;
    unsigned char *input = read_file(argv[1], &in_len);
    if (!input) return 2;

    NvttInputOptions *io = nvttCreateInputOptions();
    /* type=0 2D, 1 cube map (six faces), 3 array of `layers` images, face by face in the input */
    const NvttTextureType type = (NvttTextureType)(int)num("type", 0);
    const int faces = type == NVTT_TextureType_Cube ? 6 : (type == TextureType_Array ? (int)num("layers", 1) : 1);
    nvttSetInputOptionsTextureLayout(io, type, w, h, 1, type == TextureType_Array ? faces : 1);
    nvttSetInputOptionsFormat(io, (NvttInputFormat)in_format);
    const size_t bpp = in_format == NVTT_InputFormat_BGRA_8UB ? 4 : (in_format == NVTT_InputFormat_RGBA_16F ? 8 : 16);
    size_t off = 0;
    for (int f = 0; f < faces; f++) {
        int lw = w, lh = h;
        for (int l = 0; l < nsrc; l++) {
            if (off + (size_t)lw * lh * bpp > in_len) return 2;
            if (nvttSetInputOptionsMipmapData(io, input + off, lw, lh, 1, f, l) != NVTT_True) return 2;
            off += (size_t)lw * lh * bpp;
            lw = lw > 1 ? lw / 2 : 1;
            lh = lh > 1 ? lh / 2 : 1;
        }
    }
    nvttSetInputOptionsAlphaMode(io, (NvttAlphaMode)(int)num("alpha", 0));
    nvttSetInputOptionsWrapMode(io, (NvttWrapMode)(int)num("wrap", 2));
    nvttSetInputOptionsGamma(io, (float)num("gin", 2.2), (float)num("gout", 2.2));
    nvttSetInputOptionsMipmapFilter(io, (NvttMipmapFilter)(int)num("filter", 0));
    nvttSetInputOptionsKaiserParameters(io, (float)num("kw", 3.0), (float)num("ka", 4.0), (float)num("ks", 1.0));
    nvttSetInputOptionsMipmapGeneration(io, max_level != 0 ? NVTT_True : NVTT_False, max_level);
    nvttSetInputOptionsNormalMap(io, num("normal", 0) != 0 ? NVTT_True : NVTT_False);
    nvttSetInputOptionsNormalizeMipmaps(io, num("normalize", 1) != 0 ? NVTT_True : NVTT_False);
    nvttSetInputOptionsMaxExtents(io, (int)num("max_extent", 0));
    nvttSetInputOptionsRoundMode(io, (NvttRoundMode)(int)num("round_mode", 0));

    NvttCompressionOptions *co = nvttCreateCompressionOptions();
    nvttSetCompressionOptionsFormat(co, (NvttFormat)(int)num("format", 1));
    nvttSetCompressionOptionsQuality(co, (NvttQuality)(int)num("quality", 1));
    nvttSetCompressionOptionsColorWeights(co, (float)num("cw_r", 1), (float)num("cw_g", 1), (float)num("cw_b", 1),
                                          (float)num("cw_a", 1));
    if (num("dither", 0) != 0) nvttSetCompressionOptionsQuantization(co, NVTT_True, NVTT_False, NVTT_False, 127);

    NvttOutputOptions *oo = nvttCreateOutputOptions();
    nvttSetOutputOptionsErrorHandler(oo, on_error);
    if (to_file) nvttSetOutputOptionsFileName(oo, argv[2]);
    else nvttSetOutputOptionsOutputHandler(oo, on_begin, on_output, on_end);
    nvttSetOutputOptionsOutputHeader(oo, num("header", 1) != 0 ? NVTT_True : NVTT_False);
    nvttSetOutputOptionsContainer(oo, (NvttContainer)(int)num("container", 0));
    nvttSetOutputOptionsSrgbFlag(oo, num("srgb", 0) != 0 ? NVTT_True : NVTT_False);

    NvttCompressor *c = nvttCreateCompressor();
    nvttEnableCudaAcceleration(c, NVTT_True);
    const int estimate = nvttEstimateSize(c, io, co);
    const NvttBoolean ok = nvttCompress(c, io, co, oo);
    nvttDestroyCompressor(c);
    nvttDestroyOutputOptions(oo);
    nvttDestroyCompressionOptions(co);
    nvttDestroyInputOptions(io);
    free(input);
    if (ok != NVTT_True) {
        const int e = g_error < 0 ? 0 : g_error;
        printf("error=%d (%s)\n", e, nvttErrorString((NvttError)e));
        return 10 + e;
    }
    if (!to_file && strcmp(argv[2], "-") != 0) {
        FILE *f = fopen(argv[2], "wb");
        if (!f || fwrite(g_out, 1, g_len, f) != g_len) return 5;
        fclose(f);
    }
    printf("bytes=%zu estimate=%d images=%d version=%u\n", g_len, estimate, g_images, nvttVersion());
    free(g_out);
    return 0;
}
