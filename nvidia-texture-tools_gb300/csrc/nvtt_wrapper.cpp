// The plain-C interface of NVTT (include/nvtt/nvtt_wrapper.h; the reference's src/nvtt/nvtt_wrapper.h:183-252)
// over the nvtt:: C++ interface of this library (include/nvtt/nvtt.h, nvtt_api.cpp).
//
// The handles are the C++ objects themselves. The C callbacks of an OutputOptions are adapted to the
// C++ OutputHandler / ErrorHandler interfaces by objects this file owns, one set per OutputOptions,
// kept in a table keyed by the handle and released with it.
#include <map>
#include <memory>
#include <mutex>

#include "nvtt/nvtt.h"
#include "nvtt/nvtt_wrapper.h"

namespace {

struct CallbackOutput : public nvtt::OutputHandler {
    nvttBeginImageHandler begin = nullptr;
    nvttOutputHandler output = nullptr;
    nvttEndImageHandler end = nullptr;
    void beginImage(int size, int width, int height, int depth, int face, int miplevel) override {
        if (begin) begin(size, width, height, depth, face, miplevel);
    }
    bool writeData(const void *data, int size) override { return output ? output(data, size) : true; }
    void endImage() override {
        if (end) end();
    }
};

struct CallbackError : public nvtt::ErrorHandler {
    nvttErrorHandler fn = nullptr;
    void error(nvtt::Error e) override {
        if (fn) fn((NvttError)e);
    }
};

struct Adapters {
    CallbackOutput out;
    CallbackError err;
};

std::mutex g_mu;
std::map<const nvtt::OutputOptions *, std::unique_ptr<Adapters>> g_adapters;

Adapters &adapters_of(nvtt::OutputOptions *o) {
    std::lock_guard<std::mutex> lk(g_mu);
    std::unique_ptr<Adapters> &a = g_adapters[o];
    if (!a) a.reset(new Adapters());
    return *a;
}

bool on(NvttBoolean b) { return b != NVTT_False; }
NvttBoolean as_bool(bool b) { return b ? NVTT_True : NVTT_False; }

}  // namespace

extern "C" {

// ---- InputOptions ----

NvttInputOptions *nvttCreateInputOptions(void) { return new nvtt::InputOptions(); }
void nvttDestroyInputOptions(NvttInputOptions *o) { delete o; }
void nvttSetInputOptionsTextureLayout(NvttInputOptions *o, NvttTextureType type, int w, int h, int d, int arraySize) {
    o->setTextureLayout((nvtt::TextureType)type, w, h, d, arraySize);
}
void nvttResetInputOptionsTextureLayout(NvttInputOptions *o) { o->resetTextureLayout(); }
NvttBoolean nvttSetInputOptionsMipmapData(NvttInputOptions *o, const void *data, int w, int h, int d, int face, int mipmap) {
    return as_bool(o->setMipmapData(data, w, h, d, face, mipmap));
}
void nvttSetInputOptionsFormat(NvttInputOptions *o, NvttInputFormat format) { o->setFormat((nvtt::InputFormat)format); }
void nvttSetInputOptionsAlphaMode(NvttInputOptions *o, NvttAlphaMode a) { o->setAlphaMode((nvtt::AlphaMode)a); }
void nvttSetInputOptionsGamma(NvttInputOptions *o, float inputGamma, float outputGamma) {
    o->setGamma(inputGamma, outputGamma);
}
void nvttSetInputOptionsWrapMode(NvttInputOptions *o, NvttWrapMode mode) { o->setWrapMode((nvtt::WrapMode)mode); }
void nvttSetInputOptionsMipmapFilter(NvttInputOptions *o, NvttMipmapFilter f) { o->setMipmapFilter((nvtt::MipmapFilter)f); }
void nvttSetInputOptionsMipmapGeneration(NvttInputOptions *o, NvttBoolean enabled, int maxLevel) {
    o->setMipmapGeneration(on(enabled), maxLevel);
}
void nvttSetInputOptionsKaiserParameters(NvttInputOptions *o, float width, float alpha, float stretch) {
    o->setKaiserParameters(width, alpha, stretch);
}
void nvttSetInputOptionsNormalMap(NvttInputOptions *o, NvttBoolean b) { o->setNormalMap(on(b)); }
void nvttSetInputOptionsConvertToNormalMap(NvttInputOptions *o, NvttBoolean convert) { o->setConvertToNormalMap(on(convert)); }
// Height evaluation and the normal filter only parametrise the conversion to a normal map, which
// compress() reports as unsupported when it is enabled: nothing to record.
void nvttSetInputOptionsHeightEvaluation(NvttInputOptions *, float, float, float, float) {}
void nvttSetInputOptionsNormalFilter(NvttInputOptions *, float, float, float, float) {}
void nvttSetInputOptionsNormalizeMipmaps(NvttInputOptions *o, NvttBoolean b) { o->setNormalizeMipmaps(on(b)); }
void nvttSetInputOptionsMaxExtents(NvttInputOptions *o, int dim) { o->setMaxExtents(dim); }
void nvttSetInputOptionsRoundMode(NvttInputOptions *o, NvttRoundMode mode) { o->setRoundMode((nvtt::RoundMode)mode); }

// ---- CompressionOptions ----

NvttCompressionOptions *nvttCreateCompressionOptions(void) { return new nvtt::CompressionOptions(); }
void nvttDestroyCompressionOptions(NvttCompressionOptions *o) { delete o; }
void nvttSetCompressionOptionsFormat(NvttCompressionOptions *o, NvttFormat format) { o->setFormat((nvtt::Format)format); }
void nvttSetCompressionOptionsQuality(NvttCompressionOptions *o, NvttQuality q) { o->setQuality((nvtt::Quality)q); }
void nvttSetCompressionOptionsColorWeights(NvttCompressionOptions *o, float r, float g, float b, float a) {
    o->setColorWeights(r, g, b, a);
}
// The pixel format describes the uncompressed RGB output (Format_RGB), which this path does not
// produce (compress() reports that format as unsupported); the block formats ignore it.
void nvttSetCompressionOptionsPixelFormat(NvttCompressionOptions *, unsigned int, unsigned int, unsigned int, unsigned int,
                                          unsigned int) {}
void nvttSetCompressionOptionsQuantization(NvttCompressionOptions *o, NvttBoolean colorDithering, NvttBoolean alphaDithering,
                                           NvttBoolean binaryAlpha, int alphaThreshold) {
    o->setQuantization(on(colorDithering), on(alphaDithering), on(binaryAlpha), alphaThreshold);
}

// ---- OutputOptions ----

NvttOutputOptions *nvttCreateOutputOptions(void) { return new nvtt::OutputOptions(); }
void nvttDestroyOutputOptions(NvttOutputOptions *o) {
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_adapters.erase(o);
    }
    delete o;
}
void nvttSetOutputOptionsFileName(NvttOutputOptions *o, const char *fileName) { o->setFileName(fileName); }
void nvttSetOutputOptionsOutputHeader(NvttOutputOptions *o, NvttBoolean b) { o->setOutputHeader(on(b)); }
void nvttSetOutputOptionsContainer(NvttOutputOptions *o, NvttContainer c) { o->setContainer((nvtt::Container)c); }
void nvttSetOutputOptionsSrgbFlag(NvttOutputOptions *o, NvttBoolean b) { o->setSrgbFlag(on(b)); }
void nvttSetOutputOptionsErrorHandler(NvttOutputOptions *o, nvttErrorHandler handler) {
    Adapters &a = adapters_of(o);
    a.err.fn = handler;
    o->setErrorHandler(handler ? &a.err : nullptr);
}
void nvttSetOutputOptionsOutputHandler(NvttOutputOptions *o, nvttBeginImageHandler begin, nvttOutputHandler output,
                                       nvttEndImageHandler end) {
    Adapters &a = adapters_of(o);
    a.out.begin = begin;
    a.out.output = output;
    a.out.end = end;
    o->setOutputHandler(begin || output || end ? &a.out : nullptr);
}

// ---- Compressor ----

NvttCompressor *nvttCreateCompressor(void) { return new nvtt::Compressor(); }
void nvttDestroyCompressor(NvttCompressor *c) { delete c; }
void nvttEnableCudaAcceleration(NvttCompressor *c, NvttBoolean b) { c->enableCudaAcceleration(on(b)); }
NvttBoolean nvttIsCudaAccelerationEnabled(const NvttCompressor *c) { return as_bool(c->isCudaAccelerationEnabled()); }
NvttBoolean nvttCompress(const NvttCompressor *c, const NvttInputOptions *io, const NvttCompressionOptions *co,
                         const NvttOutputOptions *oo) {
    return as_bool(c->process(*io, *co, *oo));
}
int nvttEstimateSize(const NvttCompressor *c, const NvttInputOptions *io, const NvttCompressionOptions *co) {
    return c->estimateSize(*io, *co);
}

// ---- global ----

const char *nvttErrorString(NvttError e) {
    switch (e) {
        case NVTT_Error_Unknown: return "unknown error";
        case NVTT_Error_InvalidInput: return "the input is not valid";
        case NVTT_Error_UnsupportedFeature: return "the requested feature is not supported";
        case NVTT_Error_CudaError: return "a CUDA call failed (or no CUDA device is available)";
        case NVTT_Error_FileOpen: return "the output file cannot be opened";
        case NVTT_Error_FileWrite: return "the output file cannot be written";
        case NVTT_Error_UnsupportedOutputFormat: return "the output format is not supported by the container";
    }
    return "invalid error code";
}

unsigned int nvttVersion(void) { return NVTT_VERSION; }

}  // extern "C"
