/* nvtt_wrapper.h -- the plain-C interface of NVTT 2.1.2 (src/nvtt/nvtt_wrapper.h:183-241) over this
 * library's GPU path: opaque handles for the option objects and the compressor, the same function
 * names, argument meaning and enum values, so that a C program (or a language binding over a C FFI)
 * written against NVTT's C interface recompiles against this header unchanged as long as it stays on
 * the path (BC1/BC1a/BC3/BC4/BC5, Box/Triangle/Kaiser mipmaps, 2D textures, cube maps and texture
 * arrays). Requests outside the path
 * fail the way the C++ interface reports them: nvttCompress returns NVTT_False and the error callback
 * receives NVTT_Error_UnsupportedFeature (or NVTT_Error_UnsupportedOutputFormat). Implemented in
 * nvidia-texture-tools_gb300/csrc/nvtt_wrapper.cpp over include/nvtt/nvtt.h; links with libntg.so. */
#ifndef NVTT_GB300_NVTT_WRAPPER_H
#define NVTT_GB300_NVTT_WRAPPER_H

#define NVTT_VERSION 20102

#ifdef __cplusplus
namespace nvtt {
struct InputOptions;
struct CompressionOptions;
struct OutputOptions;
struct Compressor;
}
typedef struct nvtt::InputOptions NvttInputOptions;
typedef struct nvtt::CompressionOptions NvttCompressionOptions;
typedef struct nvtt::OutputOptions NvttOutputOptions;
typedef struct nvtt::Compressor NvttCompressor;
#else
typedef struct NvttInputOptions NvttInputOptions;
typedef struct NvttCompressionOptions NvttCompressionOptions;
typedef struct NvttOutputOptions NvttOutputOptions;
typedef struct NvttCompressor NvttCompressor;
#endif

/* Enum values are NVTT's own (src/nvtt/nvtt_wrapper.h:65-181). */
typedef enum {
    NVTT_Format_RGB,
    NVTT_Format_RGBA = NVTT_Format_RGB,
    NVTT_Format_DXT1,
    NVTT_Format_DXT1a,
    NVTT_Format_DXT3,
    NVTT_Format_DXT5,
    NVTT_Format_DXT5n,
    NVTT_Format_BC1 = NVTT_Format_DXT1,
    NVTT_Format_BC1a = NVTT_Format_DXT1a,
    NVTT_Format_BC2 = NVTT_Format_DXT3,
    NVTT_Format_BC3 = NVTT_Format_DXT5,
    NVTT_Format_BC3n = NVTT_Format_DXT5n,
    NVTT_Format_BC4,
    NVTT_Format_BC5,
    NVTT_Format_DXT1n,
    NVTT_Format_CTX1,
    NVTT_Format_BC6,
    NVTT_Format_BC7,
    NVTT_Format_BC3_RGBM,
    NVTT_Format_ETC1,
    NVTT_Format_ETC2_R,
    NVTT_Format_ETC2_RG,
    NVTT_Format_ETC2_RGB,
    NVTT_Format_ETC2_RGBA,
    NVTT_Format_ETC2_RGB_A1,
    NVTT_Format_ETC2_RGBM,
    NVTT_Format_PVR_2BPP_RGB,
    NVTT_Format_PVR_4BPP_RGB,
    NVTT_Format_PVR_2BPP_RGBA,
    NVTT_Format_PVR_4BPP_RGBA
} NvttFormat;

typedef enum { NVTT_Quality_Fastest, NVTT_Quality_Normal, NVTT_Quality_Production, NVTT_Quality_Highest } NvttQuality;
typedef enum { NVTT_WrapMode_Clamp, NVTT_WrapMode_Repeat, NVTT_WrapMode_Mirror } NvttWrapMode;
typedef enum { NVTT_TextureType_2D, NVTT_TextureType_Cube, TextureType_3D, TextureType_Array } NvttTextureType;
typedef enum {
    NVTT_InputFormat_BGRA_8UB,
    NVTT_InputFormat_RGBA_16F,
    NVTT_InputFormat_RGBA_32F,
    NVTT_InputFormat_R_32F
} NvttInputFormat;
typedef enum { NVTT_MipmapFilter_Box, NVTT_MipmapFilter_Triangle, NVTT_MipmapFilter_Kaiser } NvttMipmapFilter;
typedef enum {
    NVTT_RoundMode_None,
    NVTT_RoundMode_ToNextPowerOfTwo,
    NVTT_RoundMode_ToNearestPowerOfTwo,
    NVTT_RoundMode_ToPreviousPowerOfTwo,
    NVTT_RoundMode_ToNextMultipleOfFour,
    NVTT_RoundMode_ToNearestMultipleOfFour,
    NVTT_RoundMode_ToPreviousMultipleOfFour
} NvttRoundMode;
typedef enum { NVTT_AlphaMode_None, NVTT_AlphaMode_Transparency, NVTT_AlphaMode_Premultiplied } NvttAlphaMode;
typedef enum {
    NVTT_Error_Unknown,
    NVTT_Error_InvalidInput,
    NVTT_Error_UnsupportedFeature,
    NVTT_Error_CudaError,
    NVTT_Error_FileOpen,
    NVTT_Error_FileWrite,
    NVTT_Error_UnsupportedOutputFormat
} NvttError;
typedef enum { NVTT_Container_DDS, NVTT_Container_DDS10, NVTT_Container_KTX } NvttContainer;
typedef enum { NVTT_False, NVTT_True } NvttBoolean;

#ifdef __cplusplus
extern "C" {
#endif

/* Callbacks (src/nvtt/nvtt_wrapper.h:188-191). */
typedef void (*nvttErrorHandler)(NvttError e);
typedef void (*nvttBeginImageHandler)(int size, int width, int height, int depth, int face, int miplevel);
typedef bool (*nvttOutputHandler)(const void *data, int size);
typedef void (*nvttEndImageHandler)(void);

/* InputOptions (src/nvtt/nvtt_wrapper.h:194-214). Normal-map conversion, height evaluation and the
 * normal filter are outside the path: those setters are accepted and nvttCompress reports
 * NVTT_Error_UnsupportedFeature when they are in effect. */
NvttInputOptions *nvttCreateInputOptions(void);
void nvttDestroyInputOptions(NvttInputOptions *inputOptions);
void nvttSetInputOptionsTextureLayout(NvttInputOptions *inputOptions, NvttTextureType type, int w, int h, int d,
                                      int arraySize);
void nvttResetInputOptionsTextureLayout(NvttInputOptions *inputOptions);
NvttBoolean nvttSetInputOptionsMipmapData(NvttInputOptions *inputOptions, const void *data, int w, int h, int d, int face,
                                          int mipmap);
void nvttSetInputOptionsFormat(NvttInputOptions *inputOptions, NvttInputFormat format);
void nvttSetInputOptionsAlphaMode(NvttInputOptions *inputOptions, NvttAlphaMode alphaMode);
void nvttSetInputOptionsGamma(NvttInputOptions *inputOptions, float inputGamma, float outputGamma);
void nvttSetInputOptionsWrapMode(NvttInputOptions *inputOptions, NvttWrapMode mode);
void nvttSetInputOptionsMipmapFilter(NvttInputOptions *inputOptions, NvttMipmapFilter filter);
void nvttSetInputOptionsMipmapGeneration(NvttInputOptions *inputOptions, NvttBoolean enabled, int maxLevel);
void nvttSetInputOptionsKaiserParameters(NvttInputOptions *inputOptions, float width, float alpha, float stretch);
void nvttSetInputOptionsNormalMap(NvttInputOptions *inputOptions, NvttBoolean b);
void nvttSetInputOptionsConvertToNormalMap(NvttInputOptions *inputOptions, NvttBoolean convert);
void nvttSetInputOptionsHeightEvaluation(NvttInputOptions *inputOptions, float redScale, float greenScale, float blueScale,
                                         float alphaScale);
void nvttSetInputOptionsNormalFilter(NvttInputOptions *inputOptions, float sm, float medium, float big, float large);
void nvttSetInputOptionsNormalizeMipmaps(NvttInputOptions *inputOptions, NvttBoolean b);
void nvttSetInputOptionsMaxExtents(NvttInputOptions *inputOptions, int dim);
void nvttSetInputOptionsRoundMode(NvttInputOptions *inputOptions, NvttRoundMode mode);

/* CompressionOptions (src/nvtt/nvtt_wrapper.h:217-225). Pixel formats and quantisation (dithering,
 * binary alpha) belong to the uncompressed and dithered paths, outside this one: nvttCompress reports
 * NVTT_Error_UnsupportedFeature when they are set. */
NvttCompressionOptions *nvttCreateCompressionOptions(void);
void nvttDestroyCompressionOptions(NvttCompressionOptions *compressionOptions);
void nvttSetCompressionOptionsFormat(NvttCompressionOptions *compressionOptions, NvttFormat format);
void nvttSetCompressionOptionsQuality(NvttCompressionOptions *compressionOptions, NvttQuality quality);
void nvttSetCompressionOptionsColorWeights(NvttCompressionOptions *compressionOptions, float red, float green, float blue,
                                           float alpha);
void nvttSetCompressionOptionsPixelFormat(NvttCompressionOptions *compressionOptions, unsigned int bitcount,
                                          unsigned int rmask, unsigned int gmask, unsigned int bmask, unsigned int amask);
void nvttSetCompressionOptionsQuantization(NvttCompressionOptions *compressionOptions, NvttBoolean colorDithering,
                                           NvttBoolean alphaDithering, NvttBoolean binaryAlpha, int alphaThreshold);

/* OutputOptions (src/nvtt/nvtt_wrapper.h:228-237). */
NvttOutputOptions *nvttCreateOutputOptions(void);
void nvttDestroyOutputOptions(NvttOutputOptions *outputOptions);
void nvttSetOutputOptionsFileName(NvttOutputOptions *outputOptions, const char *fileName);
void nvttSetOutputOptionsOutputHeader(NvttOutputOptions *outputOptions, NvttBoolean b);
void nvttSetOutputOptionsContainer(NvttOutputOptions *outputOptions, NvttContainer containerFormat);
void nvttSetOutputOptionsSrgbFlag(NvttOutputOptions *outputOptions, NvttBoolean b);
void nvttSetOutputOptionsErrorHandler(NvttOutputOptions *outputOptions, nvttErrorHandler errorHandler);
void nvttSetOutputOptionsOutputHandler(NvttOutputOptions *outputOptions, nvttBeginImageHandler beginImageHandler,
                                       nvttOutputHandler outputHandler, nvttEndImageHandler endImageHandler);

/* Compressor (src/nvtt/nvtt_wrapper.h:240-247). The GPU path is the only path: disabling CUDA
 * acceleration is recorded and changes nothing. */
NvttCompressor *nvttCreateCompressor(void);
void nvttDestroyCompressor(NvttCompressor *compressor);
void nvttEnableCudaAcceleration(NvttCompressor *compressor, NvttBoolean b);
NvttBoolean nvttIsCudaAccelerationEnabled(const NvttCompressor *compressor);
NvttBoolean nvttCompress(const NvttCompressor *compressor, const NvttInputOptions *inputOptions,
                         const NvttCompressionOptions *compressionOptions, const NvttOutputOptions *outputOptions);
int nvttEstimateSize(const NvttCompressor *compressor, const NvttInputOptions *inputOptions,
                     const NvttCompressionOptions *compressionOptions);

/* Global functions (src/nvtt/nvtt_wrapper.h:251-252). */
const char *nvttErrorString(NvttError e);
unsigned int nvttVersion(void);

#ifdef __cplusplus
}
#endif
#endif /* NVTT_GB300_NVTT_WRAPPER_H */
