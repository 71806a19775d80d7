// ORACLE (test infrastructure only) — known-answer kernels over the reference's own device code.
//
// The reference's path-tracing helpers are device functions (CUDA_DEVICE_FUNCTION, texture reads)
// and its radiance-cache set-up code is four CUDA kernels, so they can only be executed on a GPU.
// oracle/build_ref.sh compiles this file, with the reference checkout on the include path and
// oracle/optix_stub standing in for the absent OptiX SDK, to PTX in oracle/_ref/; the loader
// oracle/kat_device_loader.cpp (built on the GPU host) runs these kernels and the reference's own
// kernels from that PTX. tests/golden/make_golden_device.py turns the results into fixtures.
//
// Included reference translation units (read in place, never copied):
//   renderer/gpu_kernels/nrc_set_up_kernels.cu   prepareNRC, propagateRadianceValues,
//                                                shuffleTrainingData, accumulateInferredRadianceValues
//   renderer/gpu_kernels/compute_light_probs.cu  computeFirstMipOfEnvIBLImportanceMap,
//                                                computeMipOfImportanceMap
// and, through them, common/common_renderer_types.h (PCG32RNG, SchlickPhaseFunction,
// HierarchicalImportanceMap, ImageBasedEnvironmentalLight).

// renderer_kernel_common.h names Pi in a function the set-up kernels do not use.
static constexpr float Pi = 3.14159265358979323846f;

#include "renderer/gpu_kernels/nrc_set_up_kernels.cu"
#include "renderer/gpu_kernels/compute_light_probs.cu"

// ------------------------------------------------------------------------------ radiance-cache set-up
// The buffers of the four set-up kernels, given as raw device addresses by the loader.
struct KatNrcBuffers {
    int32_t imageW, imageH;
    uint32_t maxNumTrainingSuffixes;
    uint32_t nrcBufferIndex;
    uint32_t offsetToSelectUnbiasedPath;
    float radianceScale;
    uint32_t numAccumFrames;
    uint32_t pad;
    void* numTrainingData[2];
    void* trainImageSize[2];
    void* targetMinMax[2][2];
    void* targetAvg[2];
    void* inferenceRadianceQueryBuffer;
    void* inferenceTerminalInfoBuffer;
    void* trainSuffixTerminalInfoBuffer;
    void* inferredRadianceBuffer;
    unsigned long long perFrameContributionSurface;
    unsigned long long accumSurface;
    void* trainRadianceQueryBuffer[2];
    void* trainTargetBuffer[2];
    void* trainVertexInfoBuffer;
    void* dataShufflerBuffer;
};

// ------------------------------------------------------------------------------ sizes
// Byte sizes of the records the loader allocates, in the reference's own layouts.
extern "C" __global__ void kat_sizes(uint32_t* out) {
    out[0] = sizeof(StaticPipelineLaunchParameters);
    out[1] = sizeof(PerFramePipelineLaunchParameters);
    out[2] = sizeof(RadianceQuery);
    out[3] = sizeof(TerminalInfo);
    out[4] = sizeof(TrainingVertexInfo);
    out[5] = sizeof(TrainingSuffixTerminalInfo);
    out[6] = sizeof(LinearCongruentialGenerator);
    out[7] = sizeof(RGBSpectrum);
    out[8] = sizeof(RGBSpectrumAsOrderedInt);
    out[9] = sizeof(ImageBasedEnvironmentalLight);
    out[10] = sizeof(PipelineLaunchParameters);
    out[11] = offsetof(ImageBasedEnvironmentalLight, importanceMap);
    out[12] = sizeof(KatNrcBuffers);
}

// ------------------------------------------------------------------------------ PCG32RNG
// Per state: 8 raw outputs, then 8 getFloat0cTo1o values from the state the raw outputs left.
extern "C" __global__ void kat_pcg(const uint64_t* states, uint32_t n, uint32_t* raw, float* f01) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PCG32RNG rng;
    rng.setState(states[i]);
    for (int k = 0; k < 8; ++k) raw[8 * i + k] = rng();
    for (int k = 0; k < 8; ++k) f01[8 * i + k] = rng.getFloat0cTo1o();
}

// ------------------------------------------------------------------------------ Schlick phase function
// out[6 i ..]: sampled dirLocal (3), sampled density, evaluatePDF and evaluateF(r) at that direction.
extern "C" __global__ void kat_schlick(float k, const float* u, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    SchlickPhaseFunction pf(k);
    BSDFQuery query;
    BSDFSample smp(u[2 * i], u[2 * i + 1]);
    BSDFQueryResult res;
    RGBSpectrum f = pf.sampleF(query, smp, &res);
    float* o = out + 6 * i;
    o[0] = res.dirLocal.x;
    o[1] = res.dirLocal.y;
    o[2] = res.dirLocal.z;
    o[3] = res.dirPDensity;
    o[4] = pf.evaluatePDF(query, res.dirLocal);
    o[5] = pf.evaluateF(query, res.dirLocal).r;
    (void)f;
}

// ------------------------------------------------------------------------------ environment light
// Fills an ImageBasedEnvironmentalLight as the renderer's setUpDeviceData does
// (renderer_scene.h:1213-1222): image texture, importance-map texture and its full dimensions.
extern "C" __global__ void kat_env_setup(ImageBasedEnvironmentalLight* light, CUtexObject image,
                                         CUtexObject impMap, uint32_t mapW, uint32_t mapH, uint32_t imageW,
                                         uint32_t imageH) {
    light->texObj = image;
    light->importanceMap.setTexObject(impMap, make_uint2(mapW, mapH));
    light->imageWidth = imageW;
    light->imageHeight = imageH;
}

// Per sample: HierarchicalImportanceMap::sample (pixel x, y, remapped u0, u1, prob) and
// ImageBasedEnvironmentalLight::sample (phi, theta, dirPDensity, radiance rgb) from the same u,
// then ImageBasedEnvironmentalLight::evaluate at the sampled (phi, theta) (hypDirPDensity, rgb):
// 15 floats.
extern "C" __global__ void kat_env_sample(const ImageBasedEnvironmentalLight* light, const float* u, uint32_t n,
                                          float* out, float* integral) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *integral = light->importanceMap.integral();
    if (i >= n) return;
    float* o = out + 15 * i;
    float r0, r1, prob;
    const uint2 pix = light->importanceMap.sample(u[2 * i], u[2 * i + 1], &r0, &r1, &prob);
    o[0] = static_cast<float>(pix.x);
    o[1] = static_cast<float>(pix.y);
    o[2] = r0;
    o[3] = r1;
    o[4] = prob;
    float phi, theta, pdf;
    const RGBSpectrum rad = light->sample(u[2 * i], u[2 * i + 1], &phi, &theta, &pdf);
    o[5] = phi;
    o[6] = theta;
    o[7] = pdf;
    o[8] = rad.r;
    o[9] = rad.g;
    o[10] = rad.b;
    float hyp;
    const RGBSpectrum ev = light->evaluate(phi, theta, &hyp);
    o[11] = hyp;
    o[12] = ev.r;
    o[13] = ev.g;
    o[14] = ev.b;
}

// Writes the two launch-parameter blocks the set-up kernels read through `plp`.
extern "C" __global__ void kat_build_plp(const KatNrcBuffers* b, StaticPipelineLaunchParameters* s,
                                         PerFramePipelineLaunchParameters* f) {
    memset(s, 0, sizeof(*s));
    memset(f, 0, sizeof(*f));
    s->imageSize = make_int2(b->imageW, b->imageH);
    s->accumBuffer = b->accumSurface;
    s->maxNumTrainingSuffixes = b->maxNumTrainingSuffixes;
    for (int i = 0; i < 2; ++i) {
        s->numTrainingData[i] = static_cast<uint32_t*>(b->numTrainingData[i]);
        s->trainImageSize[i] = static_cast<int2*>(b->trainImageSize[i]);
        s->targetMinMax[i][0] = static_cast<RGBSpectrumAsOrderedInt*>(b->targetMinMax[i][0]);
        s->targetMinMax[i][1] = static_cast<RGBSpectrumAsOrderedInt*>(b->targetMinMax[i][1]);
        s->targetAvg[i] = static_cast<RGBSpectrum*>(b->targetAvg[i]);
        s->trainRadianceQueryBuffer[i] = static_cast<RadianceQuery*>(b->trainRadianceQueryBuffer[i]);
        s->trainTargetBuffer[i] = static_cast<RGBSpectrum*>(b->trainTargetBuffer[i]);
    }
    s->inferenceRadianceQueryBuffer = static_cast<RadianceQuery*>(b->inferenceRadianceQueryBuffer);
    s->inferenceTerminalInfoBuffer = static_cast<TerminalInfo*>(b->inferenceTerminalInfoBuffer);
    s->trainSuffixTerminalInfoBuffer = static_cast<TrainingSuffixTerminalInfo*>(b->trainSuffixTerminalInfoBuffer);
    s->inferredRadianceBuffer = static_cast<RGBSpectrum*>(b->inferredRadianceBuffer);
    s->perFrameContributionBuffer = b->perFrameContributionSurface;
    s->trainVertexInfoBuffer = static_cast<TrainingVertexInfo*>(b->trainVertexInfoBuffer);
    s->dataShufflerBuffer = static_cast<LinearCongruentialGenerator*>(b->dataShufflerBuffer);
    f->nrcBufferIndex = b->nrcBufferIndex;
    f->offsetToSelectUnbiasedPath = b->offsetToSelectUnbiasedPath;
    f->radianceScale = b->radianceScale;
    f->numAccumFrames = b->numAccumFrames;
}

// The shuffler states as the renderer seeds them (renderer_main.cpp:218-229): one LCG seeded with
// 471313181 is advanced once per slot and copied into it. (The class's constructor is host-only,
// so the seeder lives in a word of the right size.)
extern "C" __global__ void kat_seed_shufflers(LinearCongruentialGenerator* shufflers, uint32_t n) {
    uint32_t word = 0;
    LinearCongruentialGenerator& seeder = *reinterpret_cast<LinearCongruentialGenerator*>(&word);
    seeder.setState(471313181);
    for (uint32_t i = 0; i < n; ++i) {
        seeder.next();
        shufflers[i] = seeder;
    }
}

// Field-by-field views of the bit-field records, so the loader needs no layout knowledge.
extern "C" __global__ void kat_write_suffix_terminals(TrainingSuffixTerminalInfo* dst, const uint32_t* prev,
                                                      const uint32_t* has_query, const uint32_t* path_length,
                                                      const uint32_t* unbiased, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    TrainingSuffixTerminalInfo t;
    t.prevVertexDataIndex = prev[i];
    t.hasQuery = has_query[i];
    t.pathLength = path_length[i];
    t.isUnbiasedPath = unbiased[i];
    dst[i] = t;
}
extern "C" __global__ void kat_read_suffix_terminals(const TrainingSuffixTerminalInfo* src, uint32_t* prev,
                                                     uint32_t* has_query, uint32_t* path_length, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    prev[i] = src[i].prevVertexDataIndex;
    has_query[i] = src[i].hasQuery;
    path_length[i] = src[i].pathLength;
}
extern "C" __global__ void kat_write_vertices(TrainingVertexInfo* dst, const float* throughput, const uint32_t* prev,
                                              uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    TrainingVertexInfo v;
    v.localThroughput = RGBSpectrum(throughput[3 * i], throughput[3 * i + 1], throughput[3 * i + 2]);
    v.prevVertexDataIndex = prev[i];
    v.pathLength = 0;
    v.isUnbiasedPath = 0;
    dst[i] = v;
}
extern "C" __global__ void kat_write_terminals(TerminalInfo* dst, const float* throughput, const uint32_t* has_query,
                                               uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    TerminalInfo t;
    t.throughput = RGBSpectrum(throughput[3 * i], throughput[3 * i + 1], throughput[3 * i + 2]);
    t.hasQuery = has_query[i];
    t.pathLength = 0;
    dst[i] = t;
}
// Ordered-int min / max statistics back to floats (r, g, b of min, then max).
extern "C" __global__ void kat_read_minmax(const RGBSpectrumAsOrderedInt* mn, const RGBSpectrumAsOrderedInt* mx,
                                           float* out) {
    const RGBSpectrum a = static_cast<RGBSpectrum>(*mn);
    const RGBSpectrum b = static_cast<RGBSpectrum>(*mx);
    out[0] = a.r;
    out[1] = a.g;
    out[2] = a.b;
    out[3] = b.r;
    out[4] = b.g;
    out[5] = b.b;
}

// ------------------------------------------------------------------------------ surface BSDFs
// The reference's LambertBRDF and SimplePBR_BRDF (a DichromaticBRDF) built from decoded material
// values; per input: sampleF's direction (3), value (3) and density, then evaluateF (3) and
// evaluatePDF at the second direction v (11 floats).
extern "C" __global__ void kat_bsdf(int32_t kind, float br, float bg, float bb, float smoothness, float metallic,
                                    const float* q, const float* u, const float* v, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vector3D ql(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
    const Vector3D vl(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    const BSDFQuery query(ql, Normal3D(0, 0, 1));
    const BSDFSample smp(u[2 * i], u[2 * i + 1]);
    BSDFQueryResult res;
    RGBSpectrum f, fe;
    float pe;
    if (kind == 1) {
        const LambertBRDF b(RGBSpectrum(br, bg, bb));
        f = b.sampleF(query, smp, &res);
        fe = b.evaluateF(query, vl);
        pe = b.evaluatePDF(query, vl);
    } else {
        SimplePBR_BRDF b(RGBSpectrum(br, bg, bb), 0.5f, smoothness, metallic);
        f = b.sampleF(query, smp, &res);
        fe = b.evaluateF(query, vl);
        pe = b.evaluatePDF(query, vl);
    }
    float* o = out + 11 * i;
    o[0] = res.dirLocal.x;
    o[1] = res.dirLocal.y;
    o[2] = res.dirLocal.z;
    o[3] = f.r;
    o[4] = f.g;
    o[5] = f.b;
    o[6] = res.dirPDensity;
    o[7] = fe.r;
    o[8] = fe.g;
    o[9] = fe.b;
    o[10] = pe;
}

// offsetRayOrigin (common_renderer_types.h:1326-1349) for n (point, normal) pairs.
extern "C" __global__ void kat_offset(const float* pn, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Point3D p(pn[6 * i], pn[6 * i + 1], pn[6 * i + 2]);
    const Normal3D nn(pn[6 * i + 3], pn[6 * i + 4], pn[6 * i + 5]);
    const Point3D r = offsetRayOrigin(p, nn);
    out[3 * i] = r.x;
    out[3 * i + 1] = r.y;
    out[3 * i + 2] = r.z;
}
