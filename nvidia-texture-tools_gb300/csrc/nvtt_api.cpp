// The nvtt:: drop-in API (include/nvtt/nvtt.h) on top of the C ABI (include/ntg.h).
//
// Compressor / CompressionOptions / InputOptions / OutputOptions / Surface keep the reference's
// semantics for the mip-chain + BC1/BC3/BC5 path:
//  * Compressor::process runs the InputOptions pipeline of Compressor::Private::compress
//    (src/nvtt/Context.cpp:217-346): header, then per face setImage -> toLinear -> levels of
//    {toGamma copy -> compress} -> buildNextMipmap. When no source mipmaps are supplied it is one
//    fused ntg_compress_chain_host call per face.
//  * Surfaces hold planar FP32 pixels in GPU memory, copy-on-write. An output transform (toGamma /
//    toSrgb) is kept pending until something needs the pixels, so that a following compress() of
//    BC3/BC5 can apply it through the exact 8-bit quantiser tables; an 8-bit source that has not
//    been modified yet goes through the exact 8-bit input tables.
//  * Errors: bool results plus ErrorHandler::error with nvtt's codes, as the reference reports them.
#include "nvtt/nvtt.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "ntg.h"

namespace {

// Process-wide GPU context for Surface operations (device 0), created on first use.
ntg_context *global_ctx() {
    static ntg_context *ctx = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        if (ntg_create(0, &ctx) != NTG_OK) ctx = nullptr;
    });
    return ctx;
}

bool nv_equal(float a, float b) {
    return std::fabs(a - b) <= 0.0001f * std::max(1.0f, std::max(std::fabs(a), std::fabs(b)));
}

struct DeviceBuffer {
    void *p = nullptr;
    size_t bytes = 0;
    explicit DeviceBuffer(size_t n) : bytes(n) {
        if (cudaMalloc(&p, n) != cudaSuccess) p = nullptr;
    }
    ~DeviceBuffer() {
        if (p) cudaFree(p);
    }
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
};

using Buf = std::shared_ptr<DeviceBuffer>;

Buf make_buf(size_t bytes) {
    Buf b = std::make_shared<DeviceBuffer>(bytes);
    return b->p ? b : nullptr;
}

int block_bytes(nvtt::Format f) { return f == nvtt::Format_BC1 || f == nvtt::Format_BC1a || f == nvtt::Format_BC4 ? 8 : 16; }
long long blocks_of(int w, int h) { return (long long)((w + 3) / 4) * ((h + 3) / 4); }

int ntg_format(nvtt::Format f) {
    if (f == nvtt::Format_BC1) return NTG_FORMAT_BC1;
    if (f == nvtt::Format_BC1a) return NTG_FORMAT_BC1A;
    if (f == nvtt::Format_BC3) return NTG_FORMAT_BC3;
    if (f == nvtt::Format_BC4) return NTG_FORMAT_BC4;
    if (f == nvtt::Format_BC5) return NTG_FORMAT_BC5;
    return -1;
}

nvtt::Error to_error(int code) {
    if (code == NTG_ERROR_INVALID_INPUT) return nvtt::Error_InvalidInput;
    if (code == NTG_ERROR_UNSUPPORTED_FEATURE) return nvtt::Error_UnsupportedFeature;
    if (code == NTG_ERROR_CUDA) return nvtt::Error_CudaError;
    if (code == NTG_ERROR_UNSUPPORTED_OUTPUT_FORMAT) return nvtt::Error_UnsupportedOutputFormat;
    return nvtt::Error_Unknown;
}

// IEEE binary16 -> binary32, exact (every half is a float): the conversion of InputFormat_RGBA_16F
// (src/nvtt/Surface.cpp:763-777). Subnormal halves are renormalised; Inf/NaN keep their payload.
float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t exp = (h >> 10) & 0x1f, mant = h & 0x3ffu, bits;
    if (exp == 0x1f) {
        bits = sign | 0x7f800000u | (mant << 13);
    } else if (exp != 0) {
        bits = sign | ((exp + 112) << 23) | (mant << 13);
    } else if (mant == 0) {
        bits = sign;
    } else {
        int e = 113;  // value = mant * 2^-24: shift the leading one up to the implicit bit
        while (!(mant & 0x400u)) { mant <<= 1; e--; }
        bits = sign | ((uint32_t)e << 23) | ((mant & 0x3ffu) << 13);
    }
    float f;
    std::memcpy(&f, &bits, sizeof f);
    return f;
}

// nv::countMipmaps (src/nvtt/Surface.cpp:181-193)
int count_mipmaps(int w, int h) {
    int n = 1;
    while (w != 1 || h != 1) { w = std::max(1, w / 2); h = std::max(1, h / 2); n++; }
    return n;
}

}  // namespace

namespace nvtt {

// ------------------------------------------------------------------------------------------------
// CompressionOptions (src/nvtt/CompressionOptions.cpp:55-82 defaults)

struct CompressionOptions::Private {
    Format format = Format_DXT1;
    Quality quality = Quality_Normal;
    float colorWeight[4] = {1, 1, 1, 1};
    Decoder decoder = Decoder_D3D10;
    bool colorDithering = false, alphaDithering = false, binaryAlpha = false;
    int alphaThreshold = 127;
    PixelType pixelType = PixelType_UnsignedNorm;
    int pitchAlignment = 1;
};

CompressionOptions::CompressionOptions() : m(*new Private()) {}
CompressionOptions::~CompressionOptions() { delete &m; }
void CompressionOptions::reset() { m = Private(); }
void CompressionOptions::setFormat(Format format) { m.format = format; }
void CompressionOptions::setQuality(Quality quality) { m.quality = quality; }
void CompressionOptions::setColorWeights(float r, float g, float b, float a) {
    m.colorWeight[0] = r; m.colorWeight[1] = g; m.colorWeight[2] = b; m.colorWeight[3] = a;
}
void CompressionOptions::setTargetDecoder(Decoder decoder) { m.decoder = decoder; }
void CompressionOptions::setQuantization(bool colorDithering, bool alphaDithering, bool binaryAlpha, int alphaThreshold) {
    m.colorDithering = colorDithering; m.alphaDithering = alphaDithering;
    m.binaryAlpha = binaryAlpha; m.alphaThreshold = alphaThreshold;
}
void CompressionOptions::setPixelType(PixelType t) { m.pixelType = t; }
void CompressionOptions::setPitchAlignment(int a) { m.pitchAlignment = a; }
Format CompressionOptions::format() const { return m.format; }

// ------------------------------------------------------------------------------------------------
// InputOptions (src/nvtt/InputOptions.cpp:95-187 defaults and layout)

struct InputOptions::Private {
    WrapMode wrapMode = WrapMode_Mirror;
    TextureType textureType = TextureType_2D;
    InputFormat inputFormat = InputFormat_BGRA_8UB;
    AlphaMode alphaMode = AlphaMode_None;
    float inputGamma = 2.2f, outputGamma = 2.2f;
    bool generateMipmaps = true;
    int maxLevel = -1;
    MipmapFilter mipmapFilter = MipmapFilter_Box;
    float kaiserWidth = 3, kaiserAlpha = 4.0f, kaiserStretch = 1.0f;
    bool isNormalMap = false, normalizeMipmaps = true, convertToNormalMap = false;
    int maxExtent = 0;
    RoundMode roundMode = RoundMode_None;
    int width = 0, height = 0, depth = 0, faceCount = 0, mipmapCount = 0;
    std::vector<std::vector<unsigned char>> images;  // mipLevel * faceCount + face
};

InputOptions::InputOptions() : m(*new Private()) {}
InputOptions::~InputOptions() { delete &m; }
void InputOptions::reset() {
    std::vector<std::vector<unsigned char>> keep;
    keep.swap(m.images);
    const int w = m.width, h = m.height, d = m.depth, f = m.faceCount, mc = m.mipmapCount;
    m = Private();  // like the reference, reset() keeps the layout and images but sets TextureType_2D
    m.images.swap(keep);
    m.width = w; m.height = h; m.depth = d; m.faceCount = f; m.mipmapCount = mc;
}
void InputOptions::setTextureLayout(TextureType type, int w, int h, int d, int arraySize) {
    if (w == 0) w = 1;
    if (h == 0) h = 1;
    if (d == 0) d = 1;
    if (arraySize == 0) arraySize = 1;
    resetTextureLayout();
    m.textureType = type;
    m.width = w; m.height = h; m.depth = d;
    m.faceCount = type == TextureType_Cube ? 6 : (type == TextureType_Array ? arraySize : 1);
    int mc = 1;
    int x = w, y = h, z = d;
    while (x != 1 || y != 1 || z != 1) { x = std::max(1, x / 2); y = std::max(1, y / 2); z = std::max(1, z / 2); mc++; }
    m.mipmapCount = mc;
    m.images.assign((size_t)mc * m.faceCount, std::vector<unsigned char>());
}
void InputOptions::resetTextureLayout() {
    m.width = m.height = m.depth = 0;
    m.faceCount = m.mipmapCount = 0;
    m.images.clear();
}
bool InputOptions::setMipmapData(const void *data, int w, int h, int d, int face, int mipLevel) {
    if (face < 0 || face >= m.faceCount || mipLevel < 0 || mipLevel >= m.mipmapCount) return false;
    int ew = m.width, eh = m.height, ed = m.depth;
    for (int i = 0; i < mipLevel; i++) { ew = std::max(1, ew / 2); eh = std::max(1, eh / 2); ed = std::max(1, ed / 2); }
    if (w != ew || h != eh || d != ed) return false;
    size_t bpp = m.inputFormat == InputFormat_BGRA_8UB ? 4 : (m.inputFormat == InputFormat_RGBA_16F ? 8 : (m.inputFormat == InputFormat_RGBA_32F ? 16 : 4));
    const size_t bytes = (size_t)w * h * d * bpp;
    std::vector<unsigned char> &img = m.images[(size_t)mipLevel * m.faceCount + face];
    img.assign((const unsigned char *)data, (const unsigned char *)data + bytes);
    return true;
}
void InputOptions::setFormat(InputFormat format) { m.inputFormat = format; }
void InputOptions::setAlphaMode(AlphaMode a) { m.alphaMode = a; }
void InputOptions::setGamma(float inputGamma, float outputGamma) { m.inputGamma = inputGamma; m.outputGamma = outputGamma; }
void InputOptions::setWrapMode(WrapMode mode) { m.wrapMode = mode; }
void InputOptions::setMipmapFilter(MipmapFilter filter) { m.mipmapFilter = filter; }
void InputOptions::setMipmapGeneration(bool enabled, int maxLevel) { m.generateMipmaps = enabled; m.maxLevel = maxLevel; }
void InputOptions::setKaiserParameters(float width, float alpha, float stretch) {
    m.kaiserWidth = width; m.kaiserAlpha = alpha; m.kaiserStretch = stretch;
}
void InputOptions::setNormalMap(bool b) { m.isNormalMap = b; }
void InputOptions::setConvertToNormalMap(bool b) { m.convertToNormalMap = b; }
void InputOptions::setNormalizeMipmaps(bool b) { m.normalizeMipmaps = b; }
void InputOptions::setMaxExtents(int d) { m.maxExtent = d; }
void InputOptions::setRoundMode(RoundMode mode) { m.roundMode = mode; }

// ------------------------------------------------------------------------------------------------
// OutputOptions (src/nvtt/OutputOptions.cpp:44-177)

namespace {
struct FileOutput : public OutputHandler {
    FILE *f = nullptr;
    explicit FileOutput(const char *name) { f = std::fopen(name, "wb"); }
    ~FileOutput() override { if (f) std::fclose(f); }
    void beginImage(int, int, int, int, int, int) override {}
    bool writeData(const void *data, int size) override { return f && std::fwrite(data, 1, (size_t)size, f) == (size_t)size; }
    void endImage() override {}
};
}  // namespace

struct OutputOptions::Private {
    std::string fileName;
    OutputHandler *outputHandler = nullptr;
    ErrorHandler *errorHandler = nullptr;
    bool outputHeader = true;
    Container container = Container_DDS;
    int version = 0;
    bool srgb = false;
    std::unique_ptr<FileOutput> owned;

    bool hasValidOutputHandler() const { return fileName.empty() || outputHandler != nullptr; }
    void beginImage(int size, int w, int h, int d, int face, int mip) const {
        if (outputHandler) outputHandler->beginImage(size, w, h, d, face, mip);
    }
    bool writeData(const void *data, int size) const { return outputHandler == nullptr || outputHandler->writeData(data, size); }
    void endImage() const { if (outputHandler) outputHandler->endImage(); }
    void error(Error e) const { if (errorHandler) errorHandler->error(e); }
};

OutputOptions::OutputOptions() : m(*new Private()) {}
OutputOptions::~OutputOptions() { delete &m; }
void OutputOptions::reset() {
    m.fileName.clear();
    m.owned.reset();
    m.outputHandler = nullptr;
    m.errorHandler = nullptr;
    m.outputHeader = true;
    m.container = Container_DDS;
    m.version = 0;
    m.srgb = false;
}
void OutputOptions::setFileName(const char *fileName) {
    m.owned.reset();
    m.fileName = fileName ? fileName : "";
    m.outputHandler = nullptr;
    if (!m.fileName.empty()) {
        m.owned.reset(new FileOutput(m.fileName.c_str()));
        if (m.owned->f) m.outputHandler = m.owned.get();
    }
}
void OutputOptions::setOutputHandler(OutputHandler *h) {
    m.owned.reset();
    m.fileName.clear();
    m.outputHandler = h;
}
void OutputOptions::setErrorHandler(ErrorHandler *h) { m.errorHandler = h; }
void OutputOptions::setOutputHeader(bool b) { m.outputHeader = b; }
void OutputOptions::setContainer(Container c) { m.container = c; }
void OutputOptions::setUserVersion(int v) { m.version = v; }
void OutputOptions::setSrgbFlag(bool b) { m.srgb = b; }

// ------------------------------------------------------------------------------------------------
// Surface

struct Surface::Private {
    int w = 0, h = 0;
    WrapMode wrapMode = WrapMode_Mirror;
    AlphaMode alphaMode = AlphaMode_None;
    bool normalMap = false;
    Buf data;            // planar FP32, 4 channels
    Buf src8;            // the BGRA8 source while `data` is still exactly setImage() of it
    int pending = NTG_XFORM_NONE;  // output transform not yet applied to `data`
    float pendingGamma = 1.0f;
    mutable std::vector<float> host;
    mutable bool hostValid = false;

    size_t texels() const { return (size_t)w * h; }
    float *dev() const { return data ? static_cast<float *>(data->p) : nullptr; }

    // Makes `data` private to this surface before an in-place change (copy-on-write).
    bool unshare() {
        hostValid = false;
        if (!data || data.use_count() == 1) return true;
        Buf copy = make_buf(data->bytes);
        if (!copy) return false;
        if (cudaMemcpy(copy->p, data->p, data->bytes, cudaMemcpyDeviceToDevice) != cudaSuccess) return false;
        data = copy;
        return true;
    }

    // Applies a pending output transform to the pixels.
    bool materialize() {
        if (pending == NTG_XFORM_NONE) return true;
        if (!unshare()) return false;
        const int kind = pending == NTG_XFORM_SRGB ? NTG_TRANSFORM_TO_SRGB : NTG_TRANSFORM_TO_GAMMA;
        pending = NTG_XFORM_NONE;
        src8.reset();
        if (ntg_transform(global_ctx(), dev(), w, h, kind, pendingGamma, nullptr) != NTG_OK) return false;
        return cudaDeviceSynchronize() == cudaSuccess;
    }
};

Surface::Surface() : m(new Private()) {}
Surface::Surface(const Surface &img) : m(new Private(*img.m)) {}
Surface::~Surface() { delete m; }
void Surface::operator=(const Surface &img) {
    if (this != &img) *m = *img.m;
}

void Surface::setWrapMode(WrapMode mode) { m->wrapMode = mode; }
void Surface::setAlphaMode(AlphaMode a) { m->alphaMode = a; }
void Surface::setNormalMap(bool b) { m->normalMap = b; }
bool Surface::isNull() const { return !m->data; }
int Surface::width() const { return m->w; }
int Surface::height() const { return m->h; }
int Surface::depth() const { return m->data ? 1 : 0; }
TextureType Surface::type() const { return TextureType_2D; }
WrapMode Surface::wrapMode() const { return m->wrapMode; }
AlphaMode Surface::alphaMode() const { return m->alphaMode; }
bool Surface::isNormalMap() const { return m->normalMap; }
int Surface::countMipmaps() const { return m->data ? count_mipmaps(m->w, m->h) : 0; }
int Surface::countMipmaps(int min_size) const {
    if (!m->data) return 0;
    int w = m->w, h = m->h, n = 1;
    for (;;) {  // nv::countMipmapsWithMinSize (src/nvtt/Surface.cpp:195-207)
        const bool can = min_size == 1 ? !(w == 1 && h == 1) : !(w <= min_size || h <= min_size);
        if (!can) break;
        w = std::max(1, w / 2); h = std::max(1, h / 2); n++;
    }
    return n;
}

const float *Surface::data() const {
    if (!m->data) return nullptr;
    if (!const_cast<Private *>(m)->materialize()) return nullptr;
    if (!m->hostValid) {
        m->host.resize(4 * m->texels());
        if (cudaMemcpy(m->host.data(), m->data->p, 4 * m->texels() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
            return nullptr;
        m->hostValid = true;
    }
    return m->host.data();
}

const float *Surface::channel(int i) const {
    const float *d = data();
    return d && i >= 0 && i < 4 ? d + (size_t)i * m->texels() : nullptr;
}

bool Surface::setImage(int w, int h, int d) {
    if (w <= 0 || h <= 0 || d != 1) return false;
    Buf b = make_buf((size_t)w * h * 4 * sizeof(float));
    if (!b || cudaMemset(b->p, 0, b->bytes) != cudaSuccess) return false;
    m->w = w; m->h = h; m->data = b; m->src8.reset(); m->pending = NTG_XFORM_NONE; m->hostValid = false;
    return true;
}

// Surface::setImage (src/nvtt/Surface.cpp:728-812): BGRA8, or interleaved RGBA FP32.
bool Surface::setImage(InputFormat format, int w, int h, int d, const void *data) {
    if (w <= 0 || h <= 0 || d != 1 || !data || !global_ctx()) return false;
    const size_t n = (size_t)w * h;
    Buf b = make_buf(n * 4 * sizeof(float));
    if (!b) return false;
    if (format == InputFormat_BGRA_8UB) {
        Buf s8 = make_buf(n * 4);
        if (!s8 || cudaMemcpy(s8->p, data, n * 4, cudaMemcpyHostToDevice) != cudaSuccess) return false;
        if (ntg_set_image_bgra8(global_ctx(), s8->p, w, h, NTG_XFORM_NONE, 1.0f, (float *)b->p, nullptr) != NTG_OK) return false;
        m->src8 = s8;
    } else {
        // interleaved half / float RGBA, or a single float channel (G, B, A = 0), made planar here
        std::vector<float> planar(4 * n, 0.0f);
        if (format == InputFormat_RGBA_16F) {
            const uint16_t *src = (const uint16_t *)data;
            for (size_t i = 0; i < n; i++)
                for (int c = 0; c < 4; c++) planar[c * n + i] = half_to_float(src[4 * i + c]);
        } else if (format == InputFormat_RGBA_32F) {
            const float *src = (const float *)data;
            for (size_t i = 0; i < n; i++)
                for (int c = 0; c < 4; c++) planar[c * n + i] = src[4 * i + c];
        } else if (format == InputFormat_R_32F) {
            std::memcpy(planar.data(), data, n * sizeof(float));
        } else {
            return false;
        }
        if (cudaMemcpy(b->p, planar.data(), planar.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return false;
        m->src8.reset();
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return false;
    m->w = w; m->h = h; m->data = b; m->pending = NTG_XFORM_NONE; m->hostValid = false;
    return true;
}

bool Surface::setImage(InputFormat format, int w, int h, int d, const void *r, const void *g, const void *b, const void *a) {
    if (format != InputFormat_RGBA_32F || w <= 0 || h <= 0 || d != 1 || !r || !g || !b || !a) return false;
    const size_t n = (size_t)w * h;
    Buf buf = make_buf(n * 4 * sizeof(float));
    if (!buf) return false;
    const void *planes[4] = {r, g, b, a};
    for (int c = 0; c < 4; c++)
        if (cudaMemcpy((float *)buf->p + c * n, planes[c], n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return false;
    m->w = w; m->h = h; m->data = buf; m->src8.reset(); m->pending = NTG_XFORM_NONE; m->hostValid = false;
    return true;
}

// Surface::setImage2D (src/nvtt/Surface.cpp:908-1116), D3D10 decoder, BC1/BC3/BC4/BC5 (the
// reference refuses BC1a here).
bool Surface::setImage2D(Format format, Decoder, int w, int h, const void *data) {
    const int f = ntg_format(format);
    if (f < 0 || format == Format_BC1a || w <= 0 || h <= 0 || !data || !global_ctx()) return false;
    const size_t bytes = (size_t)blocks_of(w, h) * block_bytes(format);
    Buf blocks = make_buf(bytes), b = make_buf((size_t)w * h * 4 * sizeof(float));
    if (!blocks || !b || cudaMemcpy(blocks->p, data, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return false;
    if (ntg_decode(global_ctx(), f, blocks->p, w, h, (float *)b->p, nullptr) != NTG_OK) return false;
    if (cudaDeviceSynchronize() != cudaSuccess) return false;
    m->w = w; m->h = h; m->data = b; m->src8.reset(); m->pending = NTG_XFORM_NONE; m->hostValid = false;
    return true;
}

bool Surface::canMakeNextMipmap(int min_size) {
    if (!m->data) return false;
    if (min_size == 1) return !(m->w == 1 && m->h == 1);
    return !(m->w <= min_size || m->h <= min_size);
}

bool Surface::buildNextMipmap(MipmapFilter filter, int min_size) {
    // getDefaultFilterWidthAndParams (src/nvtt/Surface.cpp:1121-1141)
    float width = filter == MipmapFilter_Box ? 0.5f : (filter == MipmapFilter_Triangle ? 1.0f : 3.0f);
    const float params[2] = {4.0f, 1.0f};
    return buildNextMipmap(filter, width, params, min_size);
}

// Surface::buildNextMipmap (src/nvtt/Surface.cpp:1344-1406)
bool Surface::buildNextMipmap(MipmapFilter filter, float filterWidth, const float *params, int min_size) {
    if (!canMakeNextMipmap(min_size) || !global_ctx()) return false;
    if (!m->materialize()) return false;
    const int dw = std::max(1, m->w / 2), dh = std::max(1, m->h / 2);
    Buf b = make_buf((size_t)dw * dh * 4 * sizeof(float));
    if (!b) return false;
    float p[2] = {4.0f, 1.0f};
    if (filter == MipmapFilter_Kaiser && params) { p[0] = params[0]; p[1] = params[1]; }
    if (ntg_mip_level(global_ctx(), m->dev(), m->w, m->h, (float *)b->p, (int)filter, filterWidth, p, (int)m->wrapMode,
                      (int)m->alphaMode, 0, nullptr) != NTG_OK)
        return false;
    if (cudaDeviceSynchronize() != cudaSuccess) return false;
    m->w = dw; m->h = dh; m->data = b; m->src8.reset(); m->hostValid = false;
    return true;
}

// getDefaultFilterWidthAndParams (src/nvtt/Surface.cpp:1121-1141) for the resize filters.
static void resize_defaults(ResizeFilter filter, float &width, float params[2]) {
    width = filter == ResizeFilter_Box ? 0.5f : filter == ResizeFilter_Triangle ? 1.0f : filter == ResizeFilter_Kaiser ? 3.0f : 2.0f;
    params[0] = filter == ResizeFilter_Mitchell ? 1.0f / 3.0f : 4.0f;
    params[1] = filter == ResizeFilter_Mitchell ? 1.0f / 3.0f : 1.0f;
}

void Surface::resize(int w, int h, int d, ResizeFilter filter) {
    float width, params[2];
    resize_defaults(filter, width, params);
    resize(w, h, d, filter, width, params);
}

// Surface::resize(w, h, d, filter, filterWidth, params) (src/nvtt/Surface.cpp:1152-1230).
void Surface::resize(int w, int h, int d, ResizeFilter filter, float filterWidth, const float *params) {
    if (!m->data || (w == m->w && h == m->h && d == 1) || d != 1 || w <= 0 || h <= 0 || filter == ResizeFilter_Mitchell ||
        !global_ctx())
        return;
    if (!m->materialize()) return;
    Buf b = make_buf((size_t)w * h * 4 * sizeof(float));
    if (!b) return;
    float p[2] = {4.0f, 1.0f};
    if (params) { p[0] = params[0]; p[1] = params[1]; }
    if (ntg_resize(global_ctx(), m->dev(), m->w, m->h, (float *)b->p, w, h, (int)filter, filterWidth, p, (int)m->wrapMode,
                   (int)m->alphaMode, nullptr) != NTG_OK || cudaDeviceSynchronize() != cudaSuccess)
        return;
    m->w = w; m->h = h; m->data = b; m->src8.reset(); m->hostValid = false;
}

void Surface::resize(int maxExtent, RoundMode mode, ResizeFilter filter) {
    float width, params[2];
    resize_defaults(filter, width, params);
    resize(maxExtent, mode, filter, width, params);
}

void Surface::resize(int maxExtent, RoundMode mode, ResizeFilter filter, float filterWidth, const float *params) {
    if (!m->data) return;
    int w = 0, h = 0;
    if (ntg_target_extent(m->w, m->h, maxExtent, (int)mode, &w, &h) != NTG_OK) return;
    resize(w, h, 1, filter, filterWidth, params);
}

// Surface::resizeMakeSquare (src/nvtt/Surface.cpp:1220-1246): the target extent, squared to the smaller side.
void Surface::resizeMakeSquare(int maxExtent, RoundMode roundMode, ResizeFilter filter) {
    if (!m->data) return;
    float width, params[2];
    resize_defaults(filter, width, params);
    int w = 0, h = 0;
    if (ntg_target_extent(m->w, m->h, maxExtent, (int)roundMode, &w, &h) != NTG_OK) return;
    const int md = std::min(w, h);
    resize(md, md, 1, filter, width, params);
}

void Surface::toLinear(float gamma) {
    if (!m->data || nv_equal(gamma, 1.0f)) return;
    if (!m->materialize()) return;
    if (m->src8) {  // 8-bit source: the exact 256-entry table
        Buf b = make_buf(m->data->bytes);
        if (b && ntg_set_image_bgra8(global_ctx(), m->src8->p, m->w, m->h, NTG_XFORM_GAMMA, gamma, (float *)b->p, nullptr) == NTG_OK &&
            cudaDeviceSynchronize() == cudaSuccess) {
            m->data = b; m->src8.reset(); m->hostValid = false;
        }
        return;
    }
    if (!m->unshare()) return;
    ntg_transform(global_ctx(), m->dev(), m->w, m->h, NTG_TRANSFORM_TO_LINEAR, gamma, nullptr);
    cudaDeviceSynchronize();
}

void Surface::toLinearFromSrgb() {
    if (!m->data) return;
    if (!m->materialize()) return;
    if (m->src8) {
        Buf b = make_buf(m->data->bytes);
        if (b && ntg_set_image_bgra8(global_ctx(), m->src8->p, m->w, m->h, NTG_XFORM_SRGB, 1.0f, (float *)b->p, nullptr) == NTG_OK &&
            cudaDeviceSynchronize() == cudaSuccess) {
            m->data = b; m->src8.reset(); m->hostValid = false;
        }
        return;
    }
    if (!m->unshare()) return;
    ntg_transform(global_ctx(), m->dev(), m->w, m->h, NTG_TRANSFORM_FROM_SRGB, 1.0f, nullptr);
    cudaDeviceSynchronize();
}

void Surface::toGamma(float gamma) {
    if (!m->data || nv_equal(gamma, 1.0f)) return;
    if (!m->materialize()) return;
    m->pending = NTG_XFORM_GAMMA;
    m->pendingGamma = gamma;
    m->hostValid = false;
}

void Surface::toSrgb() {
    if (!m->data) return;
    if (!m->materialize()) return;
    m->pending = NTG_XFORM_SRGB;
    m->pendingGamma = 1.0f;
    m->hostValid = false;
}

// nvtt::rmsError / rmsAlphaError (src/nvtt/Surface.cpp:3270-3280)
static bool error_sums(const Surface &ref, const Surface &img, double sums[2]) {
    if (ref.isNull() || img.isNull() || ref.width() != img.width() || ref.height() != img.height()) return false;
    if (!ref.m->materialize() || !img.m->materialize()) return false;
    Buf ds = make_buf(2 * sizeof(double));
    return ds && ntg_error_sums(global_ctx(), ref.m->dev(), img.m->dev(), ref.width(), ref.height(), (int)ref.alphaMode(),
                                (double *)ds->p, nullptr) == NTG_OK &&
           cudaMemcpy(sums, ds->p, 2 * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess;
}

float rmsError(const Surface &reference, const Surface &img) {
    double s[2];
    if (!error_sums(reference, img, s)) return 3.402823466e+38F;
    return (float)std::sqrt(s[0] / ((double)reference.width() * reference.height()));
}

float rmsAlphaError(const Surface &reference, const Surface &img) {
    double s[2];
    if (!error_sums(reference, img, s)) return 3.402823466e+38F;
    return (float)std::sqrt(s[1] / ((double)reference.width() * reference.height()));
}

// ------------------------------------------------------------------------------------------------
// DDS header (src/nvtt/Context.cpp:604-869 with src/nvimage/DirectDrawSurface.cpp:574-860): the
// 128-byte DDS header, plus the 20-byte DX10 extension, as the reference writes them for BC1/3/5.

namespace {

uint32_t fourcc(char a, char b, char c, char d) {
    return (uint32_t)(uint8_t)a | ((uint32_t)(uint8_t)b << 8) | ((uint32_t)(uint8_t)c << 16) | ((uint32_t)(uint8_t)d << 24);
}

// nv::getTargetExtent (src/nvtt/Surface.cpp:220-283) for the InputOptions' layout (a cube map's faces
// square). False for a layout without a positive extent. A 3D layout takes the 2D extent here, and
// process() then refuses it as unsupported.
bool target_extent(const InputOptions::Private &io, int *w, int *h) {
    const int type = io.textureType == TextureType_3D ? (int)TextureType_2D : (int)io.textureType;
    return ntg_target_extent_ex(io.width, io.height, io.maxExtent, (int)io.roundMode, type, w, h) == NTG_OK;
}

// `type` is TextureType_2D, _Cube or _Array; `arraySize` the image count of an array (1 otherwise).
bool dds_header(Format format, TextureType type, int w, int h, int arraySize, int mipmapCount, bool isNormalMap,
                const OutputOptions::Private &oo, std::vector<uint32_t> &words) {
    enum : uint32_t {
        CAPS = 0x1, HEIGHT = 0x2, WIDTH = 0x4, PIXELFORMAT = 0x1000, MIPMAPCOUNT = 0x20000, LINEARSIZE = 0x80000,
        CAPS_COMPLEX = 0x8, CAPS_TEXTURE = 0x1000, CAPS_MIPMAP = 0x400000,
        CAPS2_CUBEMAP = 0x200, CAPS2_ALL_FACES = 0xFC00,  // +X -X +Y -Y +Z -Z
        PF_ALPHAPIXELS = 0x1, PF_FOURCC = 0x4, PF_NORMAL = 0x80000000u, PF_SRGB = 0x40000000u,
    };
    const bool cube = type == TextureType_Cube;
    words.assign(37, 0);                            // magic + 124-byte header + 20-byte DX10 extension
    words[0] = fourcc('D', 'D', 'S', ' ');
    words[1] = 124;
    uint32_t flags = CAPS | PIXELFORMAT | WIDTH | HEIGHT;
    words[3] = (uint32_t)h;
    words[4] = (uint32_t)w;
    uint32_t *reserved = &words[8];                 // 11 words
    reserved[7] = fourcc('U', 'V', 'E', 'R');
    reserved[8] = (uint32_t)oo.version;
    reserved[9] = fourcc('N', 'V', 'T', 'T');
    reserved[10] = (2u << 16) | (1u << 8) | 2u;     // the reference writes its own version, 2.1.2
    uint32_t *pf = &words[19];                      // size, flags, fourcc, bitcount, r, g, b, a masks
    pf[0] = 32;
    // a cube map is a complex surface with all six faces present, even with a single level
    uint32_t caps1 = CAPS_TEXTURE | (cube ? CAPS_COMPLEX : 0u);
    if (mipmapCount > 1) { flags |= MIPMAPCOUNT; words[7] = (uint32_t)mipmapCount; caps1 |= CAPS_COMPLEX | CAPS_MIPMAP; }
    else words[7] = 1;
    words[27] = caps1;
    words[28] = cube ? CAPS2_CUBEMAP | CAPS2_ALL_FACES : 0u;
    uint32_t *h10 = &words[32];                     // dxgiFormat, dimension, miscFlag, arraySize, reserved
    h10[1] = 3;                                     // DDS_DIMENSION_TEXTURE2D
    h10[2] = cube ? 4u : 0u;                        // DDS_RESOURCE_MISC_TEXTURECUBE
    h10[3] = type == TextureType_Array ? (uint32_t)arraySize : 1u;  // only the DX10 extension records layers
    if (oo.container == Container_DDS10) {
        pf[1] = PF_FOURCC;
        pf[2] = fourcc('D', 'X', '1', '0');
        if (format == Format_BC1 || format == Format_BC1a) {
            h10[0] = oo.srgb ? 72 : 71;
            if (format == Format_BC1a) pf[1] |= PF_ALPHAPIXELS;
            if (isNormalMap) pf[1] |= PF_NORMAL;
        }
        else if (format == Format_BC3) h10[0] = oo.srgb ? 78 : 77;
        else if (format == Format_BC4) h10[0] = 80;
        else if (format == Format_BC5) { h10[0] = 83; if (isNormalMap) pf[1] |= PF_NORMAL; }
        else return false;
    } else {
        flags |= LINEARSIZE;
        words[5] = (uint32_t)(blocks_of(w, h) * block_bytes(format));
        pf[1] = PF_FOURCC;
        if (format == Format_BC1 || format == Format_BC1a) { pf[2] = fourcc('D', 'X', 'T', '1'); if (isNormalMap) pf[1] |= PF_NORMAL; }
        else if (format == Format_BC3) pf[2] = fourcc('D', 'X', 'T', '5');
        else if (format == Format_BC4) pf[2] = fourcc('A', 'T', 'I', '1');
        else if (format == Format_BC5) {
            pf[2] = fourcc('A', 'T', 'I', '2');
            if (isNormalMap) { pf[1] |= PF_NORMAL; pf[3] = fourcc('A', '2', 'X', 'Y'); }
        } else return false;
        if (oo.srgb) pf[1] |= PF_SRGB;
        words.resize(32);
    }
    words[2] = flags;
    return true;
}

}  // namespace

// ------------------------------------------------------------------------------------------------
// Compressor

struct Compressor::Private {
    ntg_context *ctx = nullptr;
    bool cudaEnabled = true;

    bool outputHeader(TextureType type, int w, int h, int d, int arraySize, int mipmapCount, bool isNormalMap,
                      const CompressionOptions::Private &co, const OutputOptions::Private &oo) const {
        if (w <= 0 || h <= 0 || d <= 0 || arraySize <= 0 || mipmapCount <= 0) { oo.error(Error_InvalidInput); return false; }
        if (!oo.outputHeader) return true;
        // 3D textures and KTX files are outside the GPU path. The reference asserts (nvCheck) that a 2D
        // texture or a cube map has an array size of 1; here that is refused as invalid input.
        if (oo.container == Container_KTX || type == TextureType_3D || d != 1) {
            oo.error(Error_UnsupportedFeature);
            return false;
        }
        if (type != TextureType_Array && arraySize != 1) { oo.error(Error_InvalidInput); return false; }
        std::vector<uint32_t> words;
        if (!dds_header(co.format, type, w, h, arraySize, mipmapCount, isNormalMap, oo, words)) {
            oo.error(Error_UnsupportedOutputFormat);
            return false;
        }
        if (!oo.writeData(words.data(), (int)(words.size() * 4))) { oo.error(Error_FileWrite); return false; }
        return true;
    }

    // Compressor::Private::compress(alphaMode, w, h, d, face, mipmap, rgba) (src/nvtt/Context.cpp:486-516)
    bool compressLevel(const float *d_rgba, int w, int h, int face, int mip, AlphaMode alphaMode, int outXform,
                       float outGamma, const CompressionOptions::Private &co, const OutputOptions::Private &oo) const {
        const int f = ntg_format(co.format);
        const size_t bytes = f < 0 ? 0 : (size_t)blocks_of(w, h) * block_bytes(co.format);
        oo.beginImage((int)bytes, w, h, 1, face, mip);
        bool ok = true;
        if (f < 0) {
            oo.error(Error_UnsupportedFeature);
        } else {
            Buf blocks = make_buf(bytes);
            std::vector<unsigned char> host(bytes);
            const float cw[3] = {co.colorWeight[0], co.colorWeight[1], co.colorWeight[2]};
            int rc = blocks ? ntg_encode(ctx, f, d_rgba, w, h, (int)co.quality, (int)alphaMode, outXform, outGamma, cw,
                                         blocks->p, nullptr)
                            : NTG_ERROR_CUDA;
            if (rc == NTG_OK && cudaMemcpy(host.data(), blocks->p, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) rc = NTG_ERROR_CUDA;
            if (rc != NTG_OK) { oo.error(to_error(rc)); ok = false; }
            else if (!oo.writeData(host.data(), (int)bytes)) ok = false;
        }
        oo.endImage();
        return ok;
    }
};

Compressor::Compressor() : m(*new Private()) {
    if (ntg_create(0, &m.ctx) != NTG_OK) m.ctx = nullptr;
}
Compressor::~Compressor() {
    if (m.ctx) ntg_destroy(m.ctx);
    delete &m;
}
void Compressor::enableCudaAcceleration(bool enable) { m.cudaEnabled = enable; }
bool Compressor::isCudaAccelerationEnabled() const { return m.ctx != nullptr; }

int Compressor::estimateSize(int w, int h, int d, int mipmapCount, const CompressionOptions &co) const {
    if (ntg_format(co.m.format) < 0) return 0;
    int size = 0;
    for (int i = 0; i < mipmapCount; i++) {
        size += (int)(blocks_of(w, h) * block_bytes(co.m.format)) * d;
        w = std::max(1, w / 2); h = std::max(1, h / 2); d = std::max(1, d / 2);
    }
    return size;
}
int Compressor::estimateSize(const Surface &img, int mipmapCount, const CompressionOptions &co) const {
    return estimateSize(img.width(), img.height(), 1, mipmapCount, co);
}
// Compressor::estimateSize(InputOptions) (src/nvtt/Context.cpp:122-137), at the target extent.
int Compressor::estimateSize(const InputOptions &io, const CompressionOptions &co) const {
    int w = 0, h = 0;
    if (!target_extent(io.m, &w, &h) || w <= 0 || h <= 0) return 0;
    int mc = io.m.generateMipmaps ? count_mipmaps(w, h) : 1;
    if (io.m.generateMipmaps && io.m.maxLevel > 0) mc = std::min(mc, io.m.maxLevel);
    return io.m.faceCount * estimateSize(w, h, io.m.depth, mc, co);
}

bool Compressor::outputHeader(TextureType type, int w, int h, int d, int arraySize, int mipmapCount, bool isNormalMap,
                              const CompressionOptions &co, const OutputOptions &oo) const {
    return m.outputHeader(type, w, h, d, arraySize, mipmapCount, isNormalMap, co.m, oo.m);
}
bool Compressor::outputHeader(const Surface &img, int mipmapCount, const CompressionOptions &co, const OutputOptions &oo) const {
    return m.outputHeader(TextureType_2D, img.width(), img.height(), 1, 1, mipmapCount, img.isNormalMap(), co.m, oo.m);
}

bool Compressor::compress(const Surface &img, int face, int mipmap, const CompressionOptions &co, const OutputOptions &oo) const {
    if (img.isNull() || !m.ctx) { oo.m.error(m.ctx ? Error_InvalidInput : Error_CudaError); return false; }
    const Surface::Private &s = *img.m;
    return m.compressLevel(s.dev(), s.w, s.h, face, mipmap, s.alphaMode, s.pending, s.pendingGamma, co.m, oo.m);
}

bool Compressor::compress(int w, int h, int d, int face, int mipmap, const float *rgba, const CompressionOptions &co,
                          const OutputOptions &oo) const {
    if (w <= 0 || h <= 0 || d != 1 || !rgba || !m.ctx) { oo.m.error(Error_InvalidInput); return false; }
    const size_t bytes = (size_t)w * h * 4 * sizeof(float);
    Buf b = make_buf(bytes);
    if (!b || cudaMemcpy(b->p, rgba, bytes, cudaMemcpyHostToDevice) != cudaSuccess) { oo.m.error(Error_CudaError); return false; }
    return m.compressLevel((const float *)b->p, w, h, face, mipmap, AlphaMode_None, NTG_XFORM_NONE, 1.0f, co.m, oo.m);
}

// Compressor::Private::compress(InputOptions) (src/nvtt/Context.cpp:217-346), DDS containers.
bool Compressor::process(const InputOptions &inputOptions, const CompressionOptions &compressionOptions,
                         const OutputOptions &outputOptions) const {
    const InputOptions::Private &io = inputOptions.m;
    const CompressionOptions::Private &co = compressionOptions.m;
    const OutputOptions::Private &oo = outputOptions.m;
    if (!oo.hasValidOutputHandler()) { oo.error(Error_FileOpen); return false; }
    if (!m.ctx) { oo.error(Error_CudaError); return false; }
    // the InputOptions resize step: nv::getTargetExtent, then Surface::resize(box) of level 0
    int w = 0, h = 0;
    if (!target_extent(io, &w, &h)) {
        oo.error(Error_InvalidInput);
        return false;
    }
    const bool resized = w != io.width || h != io.height;
    int mipmapCount = 1;
    if (io.generateMipmaps) {
        mipmapCount = count_mipmaps(w, h);
        if (io.maxLevel > 0) mipmapCount = std::min(mipmapCount, io.maxLevel);
    }
    // an array's layers are counted in the header; cube faces and 2D images are not
    const int arraySize = io.textureType == TextureType_Array ? io.faceCount : 1;
    if (!m.outputHeader(io.textureType, w, h, io.depth, arraySize, mipmapCount, io.isNormalMap, co, oo)) return false;
    // (an extent rounded to 0, ToPreviousMultipleOfFour below 4 texels, fails in outputHeader with
    // Error_InvalidInput, as in the reference)
    // outside this path: normal-map generation / renormalisation, dithering, 3D textures
    const bool normalMips = io.isNormalMap && io.normalizeMipmaps && mipmapCount > 1;
    if (io.textureType == TextureType_3D || io.depth != 1 || io.convertToNormalMap || normalMips ||
        co.colorDithering || co.alphaDithering || co.binaryAlpha || ntg_format(co.format) < 0) {
        oo.error(Error_UnsupportedFeature);
        return false;
    }
    const bool linearIn = io.isNormalMap || nv_equal(io.inputGamma, 1.0f);
    const bool linearOut = io.isNormalMap || nv_equal(io.outputGamma, 1.0f);
    if ((!linearIn && io.inputGamma != 2.2f) || (!linearOut && io.outputGamma != 2.2f)) {
        oo.error(Error_UnsupportedFeature);  // power-law gammas other than 2.2 are not on the GPU path
        return false;
    }
    for (int f = 0; f < io.faceCount; f++) {
        const std::vector<unsigned char> &base = io.images[f];
        if (base.empty()) { oo.error(Error_InvalidInput); return false; }
        bool sourceMips = false;
        for (int l = 1; l < mipmapCount; l++) sourceMips = sourceMips || !io.images[(size_t)l * io.faceCount + f].empty();
        if (!sourceMips && !resized && io.inputFormat == InputFormat_BGRA_8UB) {
            // the whole chain in one fused call: levels stay in GPU memory, one encoder launch
            ntg_chain_options opt;
            std::memset(&opt, 0, sizeof opt);
            opt.format = ntg_format(co.format);
            opt.quality = (int)co.quality;
            opt.filter = (int)io.mipmapFilter;
            if (io.mipmapFilter == MipmapFilter_Kaiser) {
                opt.filter_width = io.kaiserWidth;
                opt.params[0] = io.kaiserAlpha;  // the DDS branch passes {alpha, stretch}
                opt.params[1] = io.kaiserStretch;
            }
            opt.wrap = (int)io.wrapMode;
            opt.alpha_mode = (int)io.alphaMode;
            opt.in_xform = linearIn ? NTG_XFORM_NONE : NTG_XFORM_GAMMA;
            opt.out_xform = linearOut ? NTG_XFORM_NONE : NTG_XFORM_GAMMA;
            opt.gamma = 2.2f;
            opt.max_levels = mipmapCount;
            opt.cw[0] = co.colorWeight[0]; opt.cw[1] = co.colorWeight[1]; opt.cw[2] = co.colorWeight[2];
            std::vector<unsigned char> out(ntg_chain_bytes(w, h, &opt));
            const int rc = ntg_compress_chain_host(m.ctx, base.data(), w, h, &opt, out.data(), nullptr);
            if (rc != NTG_OK) { oo.error(to_error(rc)); return false; }
            size_t off = 0;
            int lw = w, lh = h;
            for (int l = 0; l < mipmapCount; l++) {
                const size_t bytes = (size_t)blocks_of(lw, lh) * block_bytes(co.format);
                oo.beginImage((int)bytes, lw, lh, 1, f, l);
                const bool ok = oo.writeData(out.data() + off, (int)bytes);
                oo.endImage();
                if (!ok) return false;
                off += bytes;
                lw = std::max(1, lw / 2); lh = std::max(1, lh / 2);
            }
            continue;
        }
        // float input, source mipmaps or a resize: the reference's level loop, step by step
        Surface img;
        img.setWrapMode(io.wrapMode);
        img.setAlphaMode(io.alphaMode);
        img.setNormalMap(io.isNormalMap);
        if (!img.setImage(io.inputFormat, io.width, io.height, 1, base.data())) { oo.error(Error_CudaError); return false; }
        if (!linearIn) img.toLinear(io.inputGamma);
        if (resized) {
            img.resize(w, h, 1, ResizeFilter_Box);
            if (img.width() != w || img.height() != h) { oo.error(Error_CudaError); return false; }
        }
        bool useSource = !resized;  // source mipmaps only when the extents are unchanged
        for (int l = 0; l < mipmapCount; l++) {
            if (l > 0) {
                const std::vector<unsigned char> &src = io.images[(size_t)l * io.faceCount + f];
                useSource = useSource && !src.empty();
                if (useSource) {
                    if (!img.setImage(io.inputFormat, std::max(1, w >> l), std::max(1, h >> l), 1, src.data())) {
                        oo.error(Error_CudaError);
                        return false;
                    }
                    if (!linearIn) img.toLinear(io.inputGamma);
                } else if (io.mipmapFilter == MipmapFilter_Kaiser) {
                    const float params[2] = {io.kaiserAlpha, io.kaiserStretch};
                    img.buildNextMipmap(MipmapFilter_Kaiser, io.kaiserWidth, params);
                } else {
                    img.buildNextMipmap(io.mipmapFilter);
                }
            }
            Surface tmp = img;
            if (!linearOut) tmp.toGamma(io.outputGamma);
            if (!compress(tmp, f, l, compressionOptions, outputOptions)) return false;
        }
    }
    return true;
}

}  // namespace nvtt
