/*
 * ORACLE (test infrastructure only) — stand-in for the OptiX SDK header, which is absent here.
 *
 * The reference's common/common_renderer_types.h reaches <optix.h> through
 * common/utils/optix_util.h only for its ray-tracing wrappers; the host-side functions the
 * known-answer programs call (PCG32RNG, the phase functions, HierarchicalImportanceMap,
 * ImageBasedEnvironmentalLight) use none of it. This header declares just enough names, as
 * opaque placeholders of this project's own, for those headers to compile in host code. Nothing
 * declared here is ever called.
 */
#pragma once
#include <cstddef>
#include <cstdint>

typedef unsigned long long OptixTraversableHandle;
typedef unsigned int OptixVisibilityMask;
typedef struct OptixDeviceContext_t* OptixDeviceContext;
typedef struct OptixModule_t* OptixModule;
typedef struct OptixProgramGroup_t* OptixProgramGroup;
typedef struct OptixPipeline_t* OptixPipeline;
typedef struct OptixDenoiser_t* OptixDenoiser;
typedef void (*OptixLogCallback)(unsigned int, const char*, const char*, void*);

enum OptixResult { OPTIX_SUCCESS = 0 };
enum OptixGeometryFlags { OPTIX_GEOMETRY_FLAG_NONE = 0 };
enum OptixPrimitiveTypeFlags { OPTIX_PRIMITIVE_TYPE_FLAGS_TRIANGLE = 0 };
enum OptixMotionFlags { OPTIX_MOTION_FLAG_NONE = 0 };
enum OptixInstanceFlags { OPTIX_INSTANCE_FLAG_NONE = 0 };
enum OptixRayFlags { OPTIX_RAY_FLAG_NONE = 0 };
enum OptixTraversableGraphFlags { OPTIX_TRAVERSABLE_GRAPH_FLAG_ALLOW_ANY = 0 };
enum OptixPayloadTypeID { OPTIX_PAYLOAD_TYPE_DEFAULT = 0 };
enum OptixPayloadSemantics { OPTIX_PAYLOAD_SEMANTICS_NONE = 0 };
enum OptixExceptionFlags { OPTIX_EXCEPTION_FLAG_NONE = 0 };
enum OptixVertexFormat { OPTIX_VERTEX_FORMAT_NONE = 0 };
enum OptixIndicesFormat { OPTIX_INDICES_FORMAT_NONE = 0, OPTIX_INDICES_FORMAT_UNSIGNED_INT3 = 1 };
enum OptixDenoiserModelKind { OPTIX_DENOISER_MODEL_KIND_HDR = 0 };
enum OptixCurveEndcapFlags { OPTIX_CURVE_ENDCAP_DEFAULT = 0 };
enum OptixCompileDebugLevel { OPTIX_COMPILE_DEBUG_LEVEL_DEFAULT = 0 };
enum OptixCompileOptimizationLevel { OPTIX_COMPILE_OPTIMIZATION_DEFAULT = 0 };
enum OptixPixelFormat { OPTIX_PIXEL_FORMAT_FLOAT4 = 0 };
enum OptixPrimitiveType { OPTIX_PRIMITIVE_TYPE_TRIANGLE = 0 };
struct OptixAccelBufferSizes { size_t outputSizeInBytes, tempSizeInBytes, tempUpdateSizeInBytes; };
struct OptixModuleCompileBoundValueEntry { size_t pipelineParamOffsetInBytes, sizeInBytes; const void* boundValuePtr; const char* annotation; };
struct OptixStackSizes { unsigned int cssRG, cssMS, cssCH, cssAH, cssIS, cssCC, dssDC; };
struct OptixPayloadType { unsigned int numPayloadValues; const unsigned int* payloadSemantics; };

#if defined(__CUDACC__)
#include <cuda.h>
// Device-side entry points referenced by the wrappers' device code (never instantiated here).
template <typename R, typename... A>
__device__ R optixDirectCall(unsigned int, A...);
template <typename R, typename... A>
__device__ R optixContinuationCall(unsigned int, A...);
template <typename... A>
__device__ void optixTrace(A...);
template <typename... A>
__device__ bool optixReportIntersection(float, unsigned int, A...);
template <typename... A>
__device__ void optixThrowException(int, A...);
__device__ CUdeviceptr optixGetSbtDataPointer();
__device__ unsigned int optixGetPrimitiveIndex();
__device__ float2 optixGetTriangleBarycentrics();
#endif
