// nvtt.h -- drop-in C++ API of the GB300 texture path.
//
// The subset of NVTT 2.1.2's public API (src/nvtt/nvtt.h:52-444, 472-605 of the reference) that the
// mip-chain + BC1/BC1a/BC3/BC4/BC5 path needs, with the same class names, method names, argument
// meaning, enum values and error behaviour (bool results plus ErrorHandler::error), implemented on
// the sm_103a kernels behind include/ntg.h. Surfaces keep their pixels in GPU memory; Surface::data()
// and channel() mirror them to the host on demand. Compressor::process takes 2D textures, cube maps
// and texture arrays, with the InputOptions resize step (max extent, round mode).
//
// What is outside the path reports Error_UnsupportedFeature (or returns false) instead of silently
// doing something else: other formats, BC1a at Fastest quality, 3D textures, normal-map generation
// and renormalisation of normal-map mipmaps, dithering, KTX.
#ifndef NVTT_GB300_NVTT_H
#define NVTT_GB300_NVTT_H

#define NVTT_VERSION 20102

struct ntg_context;

namespace nvtt {

struct Surface;

// Same values as the reference: the format enum doubles as a wire value in DDS/KTX handling.
enum Format {
    Format_RGB,
    Format_RGBA = Format_RGB,
    Format_DXT1,
    Format_DXT1a,
    Format_DXT3,
    Format_DXT5,
    Format_DXT5n,
    Format_BC1 = Format_DXT1,
    Format_BC1a = Format_DXT1a,
    Format_BC2 = Format_DXT3,
    Format_BC3 = Format_DXT5,
    Format_BC3n = Format_DXT5n,
    Format_BC4,
    Format_BC5,
    Format_DXT1n,
    Format_CTX1,
    Format_BC6,
    Format_BC7,
    Format_BC3_RGBM,
    Format_ETC1,
    Format_ETC2_R,
    Format_ETC2_RG,
    Format_ETC2_RGB,
    Format_ETC2_RGBA,
    Format_ETC2_RGB_A1,
    Format_ETC2_RGBM,
    Format_PVR_2BPP_RGB,
    Format_PVR_4BPP_RGB,
    Format_PVR_2BPP_RGBA,
    Format_PVR_4BPP_RGBA,
    Format_Count
};

enum PixelType {
    PixelType_UnsignedNorm = 0,
    PixelType_SignedNorm = 1,
    PixelType_UnsignedInt = 2,
    PixelType_SignedInt = 3,
    PixelType_Float = 4,
    PixelType_UnsignedFloat = 5,
    PixelType_SharedExp = 6,
};

enum Quality { Quality_Fastest, Quality_Normal, Quality_Production, Quality_Highest };

enum Decoder { Decoder_D3D10, Decoder_D3D9, Decoder_NV5x };

enum WrapMode { WrapMode_Clamp, WrapMode_Repeat, WrapMode_Mirror };

enum TextureType { TextureType_2D, TextureType_Cube, TextureType_3D, TextureType_Array };

enum InputFormat { InputFormat_BGRA_8UB, InputFormat_RGBA_16F, InputFormat_RGBA_32F, InputFormat_R_32F };

enum MipmapFilter { MipmapFilter_Box, MipmapFilter_Triangle, MipmapFilter_Kaiser };

enum ResizeFilter { ResizeFilter_Box, ResizeFilter_Triangle, ResizeFilter_Kaiser, ResizeFilter_Mitchell };

enum RoundMode {
    RoundMode_None,
    RoundMode_ToNextPowerOfTwo,
    RoundMode_ToNearestPowerOfTwo,
    RoundMode_ToPreviousPowerOfTwo,
    RoundMode_ToNextMultipleOfFour,
    RoundMode_ToNearestMultipleOfFour,
    RoundMode_ToPreviousMultipleOfFour,
};

enum AlphaMode { AlphaMode_None, AlphaMode_Transparency, AlphaMode_Premultiplied };

enum Error {
    Error_Unknown,
    Error_InvalidInput,
    Error_UnsupportedFeature,
    Error_CudaError,
    Error_FileOpen,
    Error_FileWrite,
    Error_UnsupportedOutputFormat,
    Error_Count
};

enum Container { Container_DDS, Container_DDS10, Container_KTX };

// Compression settings: format, quality, colour weights, target decoder.
struct CompressionOptions {
    CompressionOptions();
    ~CompressionOptions();
    void reset();
    void setFormat(Format format);
    void setQuality(Quality quality);
    void setColorWeights(float red, float green, float blue, float alpha = 1.0f);
    void setTargetDecoder(Decoder decoder);
    void setQuantization(bool colorDithering, bool alphaDithering, bool binaryAlpha, int alphaThreshold = 127);
    void setPixelType(PixelType pixelType);
    void setPitchAlignment(int pitchAlignment);
    Format format() const;

    struct Private;
    Private &m;

private:
    CompressionOptions(const CompressionOptions &);
    void operator=(const CompressionOptions &);
};

// Input layout and pipeline settings of Compressor::process (deprecated in NVTT 2.1, still the
// path nvcompress takes).
struct InputOptions {
    InputOptions();
    ~InputOptions();
    void reset();
    void setTextureLayout(TextureType type, int w, int h, int d = 1, int arraySize = 1);
    void resetTextureLayout();
    bool setMipmapData(const void *data, int w, int h, int d = 1, int face = 0, int mipmap = 0);
    void setFormat(InputFormat format);
    void setAlphaMode(AlphaMode alphaMode);
    void setGamma(float inputGamma, float outputGamma);
    void setWrapMode(WrapMode mode);
    void setMipmapFilter(MipmapFilter filter);
    void setMipmapGeneration(bool enabled, int maxLevel = -1);
    void setKaiserParameters(float width, float alpha, float stretch);
    void setNormalMap(bool b);
    void setConvertToNormalMap(bool convert);
    void setNormalizeMipmaps(bool b);
    void setMaxExtents(int d);
    void setRoundMode(RoundMode mode);

    struct Private;
    Private &m;

private:
    InputOptions(const InputOptions &);
    void operator=(const InputOptions &);
};

struct OutputHandler {
    virtual ~OutputHandler() {}
    virtual void beginImage(int size, int width, int height, int depth, int face, int miplevel) = 0;
    virtual bool writeData(const void *data, int size) = 0;
    virtual void endImage() = 0;
};

struct ErrorHandler {
    virtual ~ErrorHandler() {}
    virtual void error(Error e) = 0;
};

struct OutputOptions {
    OutputOptions();
    ~OutputOptions();
    void reset();
    void setFileName(const char *fileName);
    void setOutputHandler(OutputHandler *outputHandler);
    void setErrorHandler(ErrorHandler *errorHandler);
    void setOutputHeader(bool outputHeader);
    void setContainer(Container container);
    void setUserVersion(int version);
    void setSrgbFlag(bool b);

    struct Private;
    Private &m;

private:
    OutputOptions(const OutputOptions &);
    void operator=(const OutputOptions &);
};

// The compression context. Owns a GPU context (device 0) for its lifetime.
struct Compressor {
    Compressor();
    ~Compressor();

    void enableCudaAcceleration(bool enable);  // the GPU path is the only path; kept for the API
    bool isCudaAccelerationEnabled() const;

    // InputOptions API
    bool process(const InputOptions &inputOptions, const CompressionOptions &compressionOptions,
                 const OutputOptions &outputOptions) const;
    int estimateSize(const InputOptions &inputOptions, const CompressionOptions &compressionOptions) const;

    // Surface API
    bool outputHeader(const Surface &img, int mipmapCount, const CompressionOptions &compressionOptions,
                      const OutputOptions &outputOptions) const;
    bool compress(const Surface &img, int face, int mipmap, const CompressionOptions &compressionOptions,
                  const OutputOptions &outputOptions) const;
    int estimateSize(const Surface &img, int mipmapCount, const CompressionOptions &compressionOptions) const;

    // Raw API
    bool outputHeader(TextureType type, int w, int h, int d, int arraySize, int mipmapCount, bool isNormalMap,
                      const CompressionOptions &compressionOptions, const OutputOptions &outputOptions) const;
    bool compress(int w, int h, int d, int face, int mipmap, const float *rgba,
                  const CompressionOptions &compressionOptions, const OutputOptions &outputOptions) const;
    int estimateSize(int w, int h, int d, int mipmapCount, const CompressionOptions &compressionOptions) const;

    struct Private;
    Private &m;

private:
    Compressor(const Compressor &);
    void operator=(const Compressor &);
};

typedef Compressor Context;

// One level of a 2D texture, four FP32 channels, held in GPU memory (copy-on-write).
struct Surface {
    Surface();
    Surface(const Surface &img);
    ~Surface();
    void operator=(const Surface &img);

    void setWrapMode(WrapMode mode);
    void setAlphaMode(AlphaMode alphaMode);
    void setNormalMap(bool isNormalMap);

    bool isNull() const;
    int width() const;
    int height() const;
    int depth() const;
    TextureType type() const;
    WrapMode wrapMode() const;
    AlphaMode alphaMode() const;
    bool isNormalMap() const;
    int countMipmaps() const;
    int countMipmaps(int min_size) const;
    const float *data() const;      // host mirror of the planar FP32 pixels
    const float *channel(int i) const;

    bool setImage(int w, int h, int d);
    bool setImage(InputFormat format, int w, int h, int d, const void *data);
    bool setImage(InputFormat format, int w, int h, int d, const void *r, const void *g, const void *b, const void *a);
    bool setImage2D(Format format, Decoder decoder, int w, int h, const void *data);

    // Resizing (Surface::resize, src/nvtt/Surface.cpp:1143-1268): box, triangle and Kaiser filters;
    // Mitchell leaves the surface unchanged and reports nothing, as there is no error channel here.
    void resize(int w, int h, int d, ResizeFilter filter);
    void resize(int w, int h, int d, ResizeFilter filter, float filterWidth, const float *params = 0);
    void resize(int maxExtent, RoundMode mode, ResizeFilter filter);
    void resize(int maxExtent, RoundMode mode, ResizeFilter filter, float filterWidth, const float *params = 0);
    void resizeMakeSquare(int maxExtent, RoundMode roundMode, ResizeFilter filter);

    bool buildNextMipmap(MipmapFilter filter, int min_size = 1);
    bool buildNextMipmap(MipmapFilter filter, float filterWidth, const float *params = 0, int min_size = 1);
    bool canMakeNextMipmap(int min_size = 1);

    void toLinear(float gamma);
    void toGamma(float gamma);
    void toSrgb();
    void toLinearFromSrgb();

    struct Private;
    Private *m;
};

// Root-mean-square errors of `img` against `reference` (nv::rmsColorError / rmsAlphaError).
float rmsError(const Surface &reference, const Surface &img);
float rmsAlphaError(const Surface &reference, const Surface &img);

}  // namespace nvtt

#endif  // NVTT_GB300_NVTT_H
