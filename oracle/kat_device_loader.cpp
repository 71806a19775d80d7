// ORACLE (test infrastructure only) — runs the known-answer kernels of oracle/ref_kat_device.cu.
//
// Loads the PTX that oracle/build_ref.sh compiled from the reference's own device code (JIT for
// the GPU at hand), builds the textures, surfaces and buffers those kernels read exactly as the
// reference's host code does, and writes the results as raw files. Inputs and outputs are raw
// little-endian arrays in a working directory (written and read by
// tests/golden/make_golden_device.py):
//
//   kat_device_loader <ptx> <dir>
//
// The record layouts (RadianceQuery, TerminalInfo, ...) are never spelt out here: bit-field
// records are written and read through small kernels in the PTX, and byte sizes come from there.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace {

[[noreturn]] void die(const std::string& msg) {
    std::fprintf(stderr, "kat_device_loader: %s\n", msg.c_str());
    std::exit(1);
}
void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) die(std::string(what) + ": " + cudaGetErrorString(e));
}
void ckd(CUresult r, const char* what) {
    if (r != CUDA_SUCCESS) {
        const char* s = nullptr;
        cuGetErrorString(r, &s);
        die(std::string(what) + ": " + (s ? s : "driver error"));
    }
}

std::string g_dir;

template <typename T>
std::vector<T> read_vec(const std::string& name, size_t expect = 0) {
    std::ifstream f(g_dir + "/" + name, std::ios::binary | std::ios::ate);
    if (!f) die("missing input " + name);
    const size_t bytes = static_cast<size_t>(f.tellg());
    if (bytes % sizeof(T)) die("bad size of " + name);
    if (expect && bytes != expect * sizeof(T)) die("unexpected element count in " + name);
    std::vector<T> v(bytes / sizeof(T));
    f.seekg(0);
    f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(bytes));
    return v;
}
void write_raw(const std::string& name, const void* p, size_t bytes) {
    std::ofstream f(g_dir + "/" + name, std::ios::binary);
    f.write(static_cast<const char*>(p), static_cast<std::streamsize>(bytes));
    if (!f) die("cannot write " + name);
}
template <typename T>
void write_vec(const std::string& name, const std::vector<T>& v) {
    write_raw(name, v.data(), v.size() * sizeof(T));
}

struct Dev {
    void* p = nullptr;
    size_t bytes = 0;
    explicit Dev(size_t n) : bytes(n) {
        ck(cudaMalloc(&p, n ? n : 1), "cudaMalloc");
        ck(cudaMemset(p, 0, n ? n : 1), "cudaMemset");
    }
    ~Dev() { cudaFree(p); }
    template <typename T>
    void put(const std::vector<T>& v) {
        if (v.size() * sizeof(T) > bytes) die("upload larger than its buffer");
        ck(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
    }
    template <typename T>
    std::vector<T> get(size_t n) const {
        std::vector<T> v(n);
        if (n * sizeof(T) > bytes) die("download larger than its buffer");
        ck(cudaMemcpy(v.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost), "download");
        return v;
    }
    CUdeviceptr ptr() const { return reinterpret_cast<CUdeviceptr>(p); }
};

CUmodule g_mod;

void launch(const char* name, unsigned gx, unsigned gy, unsigned bx, std::vector<void*> args) {
    CUfunction f;
    ckd(cuModuleGetFunction(&f, g_mod, name), name);
    ckd(cuLaunchKernel(f, gx, gy, 1, bx, 1, 1, 0, nullptr, args.data(), nullptr), name);
    ck(cudaDeviceSynchronize(), name);
}
unsigned blocks(size_t n, unsigned b) { return static_cast<unsigned>((n + b - 1) / b); }

// A 2D CUDA array of 16-byte texels (surface load/store), as the reference's accumulation and
// per-frame contribution buffers and the environment image are.
struct Array4 {
    cudaArray_t arr = nullptr;
    cudaSurfaceObject_t surf = 0;
    int w, h;
    Array4(int width, int height) : w(width), h(height) {
        cudaChannelFormatDesc d = cudaCreateChannelDesc<float4>();
        ck(cudaMallocArray(&arr, &d, w, h, cudaArraySurfaceLoadStore), "cudaMallocArray");
        cudaResourceDesc r{};
        r.resType = cudaResourceTypeArray;
        r.res.array.array = arr;
        ck(cudaCreateSurfaceObject(&surf, &r), "cudaCreateSurfaceObject");
    }
    ~Array4() {
        cudaDestroySurfaceObject(surf);
        cudaFreeArray(arr);
    }
    void put_rgb(const std::vector<float>& rgb) {
        std::vector<float> t(4 * static_cast<size_t>(w) * h, 0.0f);
        for (size_t i = 0; i < static_cast<size_t>(w) * h; ++i)
            for (int c = 0; c < 3; ++c) t[4 * i + c] = rgb[3 * i + c];
        ck(cudaMemcpy2DToArray(arr, 0, 0, t.data(), 16 * w, 16 * w, h, cudaMemcpyHostToDevice), "to array");
    }
    std::vector<float> get_rgb() const {
        std::vector<float> t(4 * static_cast<size_t>(w) * h), rgb(3 * static_cast<size_t>(w) * h);
        ck(cudaMemcpy2DFromArray(t.data(), 16 * w, arr, 0, 0, 16 * w, h, cudaMemcpyDeviceToHost), "from array");
        for (size_t i = 0; i < static_cast<size_t>(w) * h; ++i)
            for (int c = 0; c < 3; ++c) rgb[3 * i + c] = t[4 * i + c];
        return rgb;
    }
};

std::vector<uint32_t> g_sizes;

// ------------------------------------------------------------------------------ tests
void run_sizes() {
    Dev d(64 * 4);
    void* p = d.p;
    launch("kat_sizes", 1, 1, 1, {&p});
    g_sizes = d.get<uint32_t>(16);
    write_vec("sizes.out", g_sizes);
}

void run_pcg() {
    auto st = read_vec<uint64_t>("pcg.states");
    uint32_t n = static_cast<uint32_t>(st.size());
    Dev ds(8 * n), dr(4 * 8 * n), df(4 * 8 * n);
    ds.put(st);
    void *a = ds.p, *b = dr.p, *c = df.p;
    launch("kat_pcg", blocks(n, 64), 1, 64, {&a, &n, &b, &c});
    write_vec("pcg.raw", dr.get<uint32_t>(8 * n));
    write_vec("pcg.f01", df.get<float>(8 * n));
}

void run_schlick() {
    auto ks = read_vec<float>("schlick.k");
    auto u = read_vec<float>("schlick.u");
    uint32_t n = static_cast<uint32_t>(u.size() / 2);
    Dev du(4 * u.size()), dout(4 * 6 * n);
    du.put(u);
    std::vector<float> all;
    for (float k : ks) {
        void *a = du.p, *b = dout.p;
        launch("kat_schlick", blocks(n, 64), 1, 64, {&k, &a, &n, &b});
        auto o = dout.get<float>(6 * n);
        all.insert(all.end(), o.begin(), o.end());
    }
    write_vec("schlick.out", all);
}

uint32_t next_pow2(uint32_t x) {
    uint32_t p = 1;
    while (p < x) p <<= 1;
    return p;
}
uint32_t pow2_exponent(uint32_t x) {  // exponent of the next power of two
    uint32_t e = 0;
    while ((1u << e) < x) ++e;
    return e;
}

void run_env() {
    auto dims = read_vec<uint32_t>("env.dims", 2);
    const uint32_t W = dims[0], H = dims[1];
    auto rgb = read_vec<float>("env.rgb", 3ull * W * H);
    auto u = read_vec<float>("env.u");
    uint32_t n = static_cast<uint32_t>(u.size() / 2);

    // Environment image: float4 array, surface for the importance-map kernel and a texture with
    // point filtering, wrap mode repeat and normalised coordinates (the analytic-sky environment,
    // renderer_scene.h:1264-1287).
    Array4 img(W, H);
    img.put_rgb(rgb);
    cudaResourceDesc r{};
    r.resType = cudaResourceTypeArray;
    r.res.array.array = img.arr;
    cudaTextureDesc td{};
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    cudaTextureObject_t img_tex = 0;
    ck(cudaCreateTextureObject(&img_tex, &r, &td, nullptr), "env texture");

    // Importance map: float mipmapped array of next-power-of-two size (renderer_scene.h:1194-1203,
    // 1273-1281), a surface per level, read through a texture with the Texture2D defaults
    // (linear filtering within a level, point filtering between levels, wrap mode repeat).
    const uint32_t dimX = next_pow2(W);
    const uint32_t dimY = std::max(next_pow2(H), dimX >> 1);
    const uint32_t levels = pow2_exponent(dimX) + 1;
    cudaMipmappedArray_t mm;
    cudaChannelFormatDesc d1 = cudaCreateChannelDesc<float>();
    ck(cudaMallocMipmappedArray(&mm, &d1, make_cudaExtent(dimX, dimY, 0), levels, cudaArraySurfaceLoadStore),
       "cudaMallocMipmappedArray");
    std::vector<cudaSurfaceObject_t> lsurf(levels);
    std::vector<cudaArray_t> larr(levels);
    for (uint32_t l = 0; l < levels; ++l) {
        ck(cudaGetMipmappedArrayLevel(&larr[l], mm, l), "level");
        cudaResourceDesc rl{};
        rl.resType = cudaResourceTypeArray;
        rl.res.array.array = larr[l];
        ck(cudaCreateSurfaceObject(&lsurf[l], &rl), "level surface");
    }
    cudaResourceDesc rm{};
    rm.resType = cudaResourceTypeMipmappedArray;
    rm.res.mipmap.mipmap = mm;
    cudaTextureDesc tm{};
    tm.addressMode[0] = tm.addressMode[1] = cudaAddressModeWrap;
    tm.filterMode = cudaFilterModeLinear;
    tm.mipmapFilterMode = cudaFilterModePoint;
    tm.readMode = cudaReadModeElementType;
    tm.normalizedCoords = 1;
    tm.maxMipmapLevelClamp = static_cast<float>(levels - 1);
    cudaTextureObject_t imp_tex = 0;
    ck(cudaCreateTextureObject(&imp_tex, &rm, &tm, nullptr), "importance texture");

    Dev light(g_sizes[9]);
    {
        void* lp = light.p;
        unsigned long long a = img_tex, b = imp_tex;
        uint32_t mw = dimX, mh = dimY, iw = W, ih = H;
        launch("kat_env_setup", 1, 1, 1, {&lp, &a, &b, &mw, &mh, &iw, &ih});
    }
    // The reference's own map build (renderer_scene.h:990-1060): first mip, then each level.
    CUdeviceptr imp = light.ptr() + g_sizes[11];
    {
        unsigned long long s_img = img.surf, s0 = lsurf[0];
        uint2 size = make_uint2(W, H);
        launch("computeFirstMipOfEnvIBLImportanceMap", blocks(dimX, 32), dimY, 32, {&s_img, &size, &imp, &s0});
        uint2 cur = make_uint2(dimX, dimY);
        for (uint32_t l = 1; l < levels; ++l) {
            cur = make_uint2((cur.x + 1) / 2, (cur.y + 1) / 2);
            unsigned long long src = lsurf[l - 1], dst = lsurf[l];
            uint32_t level = l;
            launch("computeMipOfImportanceMap", blocks(cur.x, 32), cur.y, 32, {&imp, &level, &src, &dst});
        }
    }
    std::vector<float> mips;
    for (uint32_t l = 0; l < levels; ++l) {
        const uint32_t lw = std::max(dimX >> l, 1u), lh = std::max(dimY >> l, 1u);
        std::vector<float> m(static_cast<size_t>(lw) * lh);
        ck(cudaMemcpy2DFromArray(m.data(), 4 * lw, larr[l], 0, 0, 4 * lw, lh, cudaMemcpyDeviceToHost), "mip");
        mips.insert(mips.end(), m.begin(), m.end());
    }
    write_vec("env.mips", mips);
    Dev du(4 * u.size()), dout(4 * 15 * n), dint(4);
    du.put(u);
    void *lp = light.p, *a = du.p, *o = dout.p, *ip = dint.p;
    launch("kat_env_sample", blocks(n, 64), 1, 64, {&lp, &a, &n, &o, &ip});
    write_vec("env.out", dout.get<float>(15 * n));
    write_vec("env.integral", dint.get<float>(1));
    for (auto s : lsurf) cudaDestroySurfaceObject(s);
    cudaDestroyTextureObject(imp_tex);
    cudaDestroyTextureObject(img_tex);
    cudaFreeMipmappedArray(mm);
}

// Mirror of KatNrcBuffers in oracle/ref_kat_device.cu (its size is checked against the PTX's).
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

void run_nrc() {
    if (g_sizes[12] != sizeof(KatNrcBuffers)) die("KatNrcBuffers layout differs from the PTX's");
    if (g_sizes[2] != 56) die("RadianceQuery is not 14 floats");
    auto prm = read_vec<uint32_t>("nrc.params", 16);
    const int W = static_cast<int>(prm[0]), H = static_cast<int>(prm[1]);
    const uint32_t maxSuffix = prm[2], buf = prm[3], offset = prm[4], newSeq = prm[5], prevCount = prm[6];
    const uint32_t prevTrainW = prm[7], prevTrainH = prm[8], accumFrames = prm[9], shuffleCount = prm[10];
    const uint32_t nVert = prm[11];
    float radianceScale;
    std::memcpy(&radianceScale, &prm[12], 4);
    const uint32_t kPerFrame = 1u << 16, kTrainBuffer = 2 * kPerFrame;
    const size_t npix = static_cast<size_t>(W) * H;
    const uint32_t q = g_sizes[2], tinfo = g_sizes[3], vinfo = g_sizes[4], sinfo = g_sizes[5], lcg = g_sizes[6];
    const uint32_t spec = g_sizes[7], oint = g_sizes[8];

    Dev numTrain0(4), numTrain1(4), trainSize0(8), trainSize1(8);
    Dev mm00(oint), mm01(oint), mm10(oint), mm11(oint), avg0(spec), avg1(spec);
    Dev inferQuery(static_cast<size_t>(q) * std::max<size_t>(npix, maxSuffix));
    Dev inferTerm(static_cast<size_t>(tinfo) * npix);
    Dev suffixTerm(static_cast<size_t>(sinfo) * maxSuffix);
    Dev inferred(static_cast<size_t>(spec) * std::max<size_t>(npix, maxSuffix));
    Dev trainQ0(static_cast<size_t>(q) * kTrainBuffer), trainQ1(static_cast<size_t>(q) * kTrainBuffer);
    Dev trainT0(static_cast<size_t>(spec) * kTrainBuffer), trainT1(static_cast<size_t>(spec) * kTrainBuffer);
    Dev vertices(static_cast<size_t>(vinfo) * kTrainBuffer), shufflers(static_cast<size_t>(lcg) * kTrainBuffer);
    Array4 contrib(W, H), accum(W, H);
    KatNrcBuffers hb{};
    hb.imageW = W;
    hb.imageH = H;
    hb.maxNumTrainingSuffixes = maxSuffix;
    hb.nrcBufferIndex = buf;
    hb.offsetToSelectUnbiasedPath = 0;
    hb.radianceScale = radianceScale;
    hb.numAccumFrames = accumFrames;
    hb.numTrainingData[0] = numTrain0.p;
    hb.numTrainingData[1] = numTrain1.p;
    hb.trainImageSize[0] = trainSize0.p;
    hb.trainImageSize[1] = trainSize1.p;
    hb.targetMinMax[0][0] = mm00.p;
    hb.targetMinMax[0][1] = mm01.p;
    hb.targetMinMax[1][0] = mm10.p;
    hb.targetMinMax[1][1] = mm11.p;
    hb.targetAvg[0] = avg0.p;
    hb.targetAvg[1] = avg1.p;
    hb.inferenceRadianceQueryBuffer = inferQuery.p;
    hb.inferenceTerminalInfoBuffer = inferTerm.p;
    hb.trainSuffixTerminalInfoBuffer = suffixTerm.p;
    hb.inferredRadianceBuffer = inferred.p;
    hb.perFrameContributionSurface = contrib.surf;
    hb.accumSurface = accum.surf;
    hb.trainRadianceQueryBuffer[0] = trainQ0.p;
    hb.trainRadianceQueryBuffer[1] = trainQ1.p;
    hb.trainTargetBuffer[0] = trainT0.p;
    hb.trainTargetBuffer[1] = trainT1.p;
    hb.trainVertexInfoBuffer = vertices.p;
    hb.dataShufflerBuffer = shufflers.p;
    Dev db(sizeof(hb)), dstatic(g_sizes[0]), dframe(g_sizes[1]);
    ck(cudaMemcpy(db.p, &hb, sizeof(hb), cudaMemcpyHostToDevice), "buffers");
    {
        void *a = db.p, *b = dstatic.p, *c = dframe.p;
        launch("kat_build_plp", 1, 1, 1, {&a, &b, &c});
    }
    CUdeviceptr plp;
    size_t plp_bytes;
    ckd(cuModuleGetGlobal(&plp, &plp_bytes, g_mod, "plp"), "plp");
    if (plp_bytes != g_sizes[10]) die("plp size");
    void* ptrs[2] = {dstatic.p, dframe.p};
    ckd(cuMemcpyHtoD(plp, ptrs, sizeof(ptrs)), "plp upload");
    auto read_minmax = [&](Dev& mn, Dev& mx) {
        Dev out(6 * 4);
        void *a = mn.p, *b = mx.p, *c = out.p;
        launch("kat_read_minmax", 1, 1, 1, {&a, &b, &c});
        return out.get<float>(6);
    };
    Dev& curNum = buf == 0 ? numTrain0 : numTrain1;
    Dev& prevNum = buf == 0 ? numTrain1 : numTrain0;
    Dev& curSize = buf == 0 ? trainSize0 : trainSize1;
    Dev& prevSize = buf == 0 ? trainSize1 : trainSize0;
    Dev& curMin = buf == 0 ? mm00 : mm10;
    Dev& curMax = buf == 0 ? mm01 : mm11;
    Dev& curAvg = buf == 0 ? avg0 : avg1;

    // ---- prepareNRC (nrc_set_up_kernels.cu:4-44)
    prevNum.put(std::vector<uint32_t>{prevCount});
    prevSize.put(std::vector<int32_t>{static_cast<int32_t>(prevTrainW), static_cast<int32_t>(prevTrainH)});
    ck(cudaMemset(suffixTerm.p, 0xFF, suffixTerm.bytes), "suffix fill");
    {
        uint32_t off = offset;
        bool ns = newSeq != 0;
        launch("prepareNRC", blocks(maxSuffix, 32), 1, 32, {&off, &ns});
    }
    {
        std::vector<int32_t> sz = curSize.get<int32_t>(2);
        std::vector<uint32_t> out = {static_cast<uint32_t>(sz[0]), static_cast<uint32_t>(sz[1]),
                                     curNum.get<uint32_t>(1)[0]};
        write_vec("prep.out", out);
        write_vec("prep.minmax", read_minmax(curMin, curMax));
        write_vec("prep.avg", curAvg.get<float>(3));
        Dev p(4 * maxSuffix), hq(4 * maxSuffix), pl(4 * maxSuffix);
        void *a = suffixTerm.p, *b = p.p, *c = hq.p, *d = pl.p;
        uint32_t n = maxSuffix;
        launch("kat_read_suffix_terminals", blocks(n, 64), 1, 64, {&a, &b, &c, &d, &n});
        auto vp = p.get<uint32_t>(n), vh = hq.get<uint32_t>(n), vl = pl.get<uint32_t>(n);
        std::vector<uint32_t> all;
        all.insert(all.end(), vp.begin(), vp.end());
        all.insert(all.end(), vh.begin(), vh.end());
        all.insert(all.end(), vl.begin(), vl.end());
        write_vec("prep.term", all);
    }

    // ---- propagateRadianceValues (:46-86)
    {
        auto term = read_vec<uint32_t>("prop.term", 3ull * maxSuffix);
        Dev p(4 * maxSuffix), hq(4 * maxSuffix), pl(4 * maxSuffix), ub(4 * maxSuffix);
        p.put(std::vector<uint32_t>(term.begin(), term.begin() + maxSuffix));
        hq.put(std::vector<uint32_t>(term.begin() + maxSuffix, term.begin() + 2 * maxSuffix));
        pl.put(std::vector<uint32_t>(term.begin() + 2 * maxSuffix, term.end()));
        uint32_t n = maxSuffix;
        void *dst = suffixTerm.p, *a = p.p, *b = hq.p, *c = pl.p, *d = ub.p;
        launch("kat_write_suffix_terminals", blocks(n, 64), 1, 64, {&dst, &a, &b, &c, &d, &n});
        inferred.put(read_vec<float>("prop.inferred", 3ull * maxSuffix));
        inferQuery.put(read_vec<float>("prop.query", 14ull * maxSuffix));
        auto vtp = read_vec<float>("prop.vtp", 3ull * nVert);
        auto vprev = read_vec<uint32_t>("prop.vprev", nVert);
        Dev dtp(4 * vtp.size()), dvp(4 * vprev.size());
        dtp.put(vtp);
        dvp.put(vprev);
        void *vd = vertices.p, *t = dtp.p, *pv = dvp.p;
        uint32_t nv = nVert;
        launch("kat_write_vertices", blocks(nv, 64), 1, 64, {&vd, &t, &pv, &nv});
        trainT0.put(read_vec<float>("prop.target0", 3ull * nVert));
        trainQ0.put(read_vec<float>("prop.query0", 14ull * nVert));
        launch("propagateRadianceValues", blocks(maxSuffix, 32), 1, 32, {});
        write_vec("prop.target_out", trainT0.get<float>(3ull * nVert));
    }

    // ---- shuffleTrainingData (:88-174), statistics reset by a prepareNRC of the same buffer
    {
        uint32_t off = offset;
        bool ns = true;
        launch("prepareNRC", blocks(maxSuffix, 32), 1, 32, {&off, &ns});
        curNum.put(std::vector<uint32_t>{shuffleCount});
        trainQ0.put(read_vec<float>("shuf.query0", 14ull * nVert));
        trainT0.put(read_vec<float>("shuf.target0", 3ull * nVert));
        void* sp = shufflers.p;
        uint32_t nsh = kPerFrame;
        launch("kat_seed_shufflers", 1, 1, 1, {&sp, &nsh});
        launch("shuffleTrainingData", kPerFrame / 32, 1, 32, {});
        write_vec("shuf.query1", trainQ1.get<float>(14ull * kPerFrame));
        write_vec("shuf.target1", trainT1.get<float>(3ull * kPerFrame));
        write_vec("shuf.minmax", read_minmax(curMin, curMax));
        write_vec("shuf.avg", curAvg.get<float>(3));
    }

    // ---- accumulateInferredRadianceValues (:176-219)
    {
        auto ttp = read_vec<float>("acc.ttp", 3 * npix);
        auto hasq = read_vec<uint32_t>("acc.hasq", npix);
        Dev dtp(4 * ttp.size()), dhq(4 * hasq.size());
        dtp.put(ttp);
        dhq.put(hasq);
        void *td = inferTerm.p, *a = dtp.p, *b = dhq.p;
        uint32_t n = static_cast<uint32_t>(npix);
        launch("kat_write_terminals", blocks(n, 64), 1, 64, {&td, &a, &b, &n});
        contrib.put_rgb(read_vec<float>("acc.contrib", 3 * npix));
        inferred.put(read_vec<float>("acc.inferred", 3 * npix));
        inferQuery.put(read_vec<float>("acc.query", 14 * npix));
        accum.put_rgb(read_vec<float>("acc.prev", 3 * npix));
        launch("accumulateInferredRadianceValues", blocks(npix, 32), 1, 32, {});
        write_vec("acc.out", accum.get_rgb());
    }
}

}  // namespace

// Surface BSDFs: bsdf.params holds 6 floats per material (kind, linear base colour, smoothness,
// metallic); every material gets the same query directions, variates and second directions.
void run_bsdf() {
    auto params = read_vec<float>("bsdf.params");
    auto q = read_vec<float>("bsdf.q");
    auto u = read_vec<float>("bsdf.u");
    auto v = read_vec<float>("bsdf.v");
    uint32_t n = static_cast<uint32_t>(q.size() / 3);
    if (u.size() != 2 * static_cast<size_t>(n) || v.size() != 3 * static_cast<size_t>(n) || params.size() % 6)
        die("bsdf inputs have inconsistent sizes");
    Dev dq(4 * q.size()), du(4 * u.size()), dv(4 * v.size()), dout(4 * 11 * static_cast<size_t>(n));
    dq.put(q);
    du.put(u);
    dv.put(v);
    std::vector<float> all;
    for (size_t m = 0; m < params.size() / 6; ++m) {
        int32_t kind = static_cast<int32_t>(params[6 * m]);
        float br = params[6 * m + 1], bg = params[6 * m + 2], bb = params[6 * m + 3];
        float sm = params[6 * m + 4], me = params[6 * m + 5];
        void *a = dq.p, *b = du.p, *c = dv.p, *o = dout.p;
        launch("kat_bsdf", blocks(n, 64), 1, 64, {&kind, &br, &bg, &bb, &sm, &me, &a, &b, &c, &n, &o});
        auto r = dout.get<float>(11 * static_cast<size_t>(n));
        all.insert(all.end(), r.begin(), r.end());
    }
    write_vec("bsdf.out", all);
}

void run_offset() {
    auto pn = read_vec<float>("offset.pn");
    uint32_t n = static_cast<uint32_t>(pn.size() / 6);
    Dev dp(4 * pn.size()), dout(4 * 3 * static_cast<size_t>(n));
    dp.put(pn);
    void *a = dp.p, *o = dout.p;
    launch("kat_offset", blocks(n, 64), 1, 64, {&a, &n, &o});
    write_vec("offset.out", dout.get<float>(3 * static_cast<size_t>(n)));
}

int main(int argc, char** argv) {
    if (argc != 3) die("usage: kat_device_loader <ptx> <dir>");
    g_dir = argv[2];
    std::ifstream f(argv[1], std::ios::binary);
    if (!f) die(std::string("cannot read ") + argv[1]);
    std::string ptx((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    ck(cudaFree(nullptr), "runtime init");
    ckd(cuModuleLoadData(&g_mod, ptx.c_str()), "cuModuleLoadData");
    run_sizes();
    run_pcg();
    run_schlick();
    run_env();
    run_nrc();
    run_bsdf();
    run_offset();
    std::printf("ok\n");
    return 0;
}
