// C ABI of the radiance-cache frame (renderer/renderer_main.cpp:1553-1637): cache buffers of a
// context, the training and render passes of the tracker, the set-up kernels, and the frame
// loop with the tcgen05 network of nrc_mlp.cu. Everything is enqueued on one stream; unlike
// the reference (renderer_main.cpp:1568-1573, 1613) no step waits for the host, because the
// training image size and the query counts stay on the device.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/rtc8_nrc.h"
#include "../../include/rtc8_vpt.h"
#include "nrc_buffers.cuh"
#include "vpt_ctx.h"
#include "vpt_tracer.cuh"

namespace {

int fail(int code, const std::string& msg) { return vpt::ctx_set_error(code, msg.c_str()); }

#define NRCP_CUDA(call)                                                                    \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) return fail(VPT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
cudaError_t alloc_zero(T** p, size_t count) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return e;
    }
    return cudaMemset(*p, 0, count * sizeof(T));
}

template <typename T>
void free_ptr(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

int ensure_nrc(VptContext* c) {
    if (c->nrc) return VPT_OK;
    auto* b = new vpt::NrcBuffers();
    c->nrc = b;
    b->width = c->width;
    b->height = c->height;
    const size_t npix = static_cast<size_t>(c->width) * c->height;
    b->max_train_suffixes = static_cast<uint32_t>(npix);
    b->infer_capacity = static_cast<uint32_t>((npix + 127) / 128 * 128);
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    chk(alloc_zero(&b->infer_query, static_cast<size_t>(b->infer_capacity) * vpt::kQueryFloats));
    chk(alloc_zero(&b->infer_terminal, npix));
    chk(alloc_zero(&b->train_suffix, npix));
    chk(alloc_zero(&b->inferred, static_cast<size_t>(b->infer_capacity) * 3));
    chk(alloc_zero(&b->frame_contribution, npix * 3));
    chk(alloc_zero(&b->infer_index, npix));
    for (int i = 0; i < 2; ++i) {
        chk(alloc_zero(&b->train_query[i], static_cast<size_t>(vpt::kTrainBufferSize) * vpt::kQueryFloats));
        chk(alloc_zero(&b->train_target[i], static_cast<size_t>(vpt::kTrainBufferSize) * 3));
    }
    chk(alloc_zero(&b->train_vertex, vpt::kTrainBufferSize));
    chk(alloc_zero(&b->train_end_query, npix * vpt::kQueryFloats));
    chk(alloc_zero(&b->train_end_inferred, npix * 3));
    chk(alloc_zero(&b->train_rng, npix));
    chk(alloc_zero(&b->shufflers, vpt::kNumTrainingDataPerFrame));
    chk(alloc_zero(&b->counters, 16));
    chk(alloc_zero(&b->stats, 18));
    if (e != cudaSuccess) {
        c->release_nrc();
        return fail(VPT_ERR_OUT_OF_MEMORY, std::string("vpt_nrc_enable: ") + cudaGetErrorString(e));
    }
    // renderer_main.cpp:218-229: shuffler i holds the LCG state after i + 1 steps from 471313181
    // (state = (state * 1103515245 + 12345) mod 2^31 in 32-bit arithmetic, renderer_shared.h:92-109).
    std::vector<uint32_t> st(vpt::kNumTrainingDataPerFrame);
    uint32_t s = 471313181u;
    for (uint32_t i = 0; i < vpt::kNumTrainingDataPerFrame; ++i) {
        s = (s * 1103515245u + 12345u) % (1u << 31);
        st[i] = s;
    }
    NRCP_CUDA(cudaMemcpy(b->shufflers, st.data(), st.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    return vpt::nrc_reseed_train_rng(c);
}

__global__ void derive_states_kernel(uint64_t* __restrict__ out, const uint64_t* __restrict__ in, uint32_t n,
                                     uint64_t mult, uint64_t plus) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = mult * in[i] + plus;
}

// radianceScale of the frame (renderer_shared.h:160); <= 0 = off.
float radiance_scale(const VptContext* c) { return c->frame.radiance_scale > 0 ? c->frame.radiance_scale : 0.0f; }

// Grows the render-pass buffers (queries, terminals, predictions, contributions) to `spp`
// sample slots per pixel. Waits for the device before freeing the old buffers.
int ensure_render_slots(VptContext* c, uint32_t spp) {
    int rc = ensure_nrc(c);
    if (rc) return rc;
    vpt::NrcBuffers& b = *c->nrc;
    if (spp <= b.render_spp) return VPT_OK;
    const size_t slots = static_cast<size_t>(c->width) * c->height * spp;
    if (slots >= (1ull << 31)) return fail(VPT_ERR_INVALID_ARGUMENT, "too many render-pass samples in one launch");
    NRCP_CUDA(cudaDeviceSynchronize());
    free_ptr(b.infer_query);
    free_ptr(b.infer_terminal);
    free_ptr(b.inferred);
    free_ptr(b.frame_contribution);
    free_ptr(b.infer_index);
    const uint32_t cap = static_cast<uint32_t>((slots + 127) / 128 * 128);
    cudaError_t e = alloc_zero(&b.infer_query, static_cast<size_t>(cap) * vpt::kQueryFloats);
    if (e == cudaSuccess) e = alloc_zero(&b.infer_terminal, slots);
    if (e == cudaSuccess) e = alloc_zero(&b.inferred, static_cast<size_t>(cap) * 3);
    if (e == cudaSuccess) e = alloc_zero(&b.frame_contribution, slots * 3);
    if (e == cudaSuccess) e = alloc_zero(&b.infer_index, slots);
    if (e != cudaSuccess) {
        c->release_nrc();
        return fail(VPT_ERR_OUT_OF_MEMORY, std::string("render-pass buffers: ") + cudaGetErrorString(e));
    }
    b.infer_capacity = cap;
    b.render_spp = spp;
    return VPT_OK;
}

// Jump of the training states of set k: 2^62 draws past the context's per-pixel states (clear
// of the render samples' streams, sample s starting s * 2^40 draws in) plus k * 2^58.
void set_jump(uint32_t k, uint64_t* mult, uint64_t* plus) {
    vpt::lcg_jump((1ull << 62) + static_cast<uint64_t>(k) * (1ull << 58), mult, plus);
}

// Training sets 0 .. n-1 of the multi-pass frame (set 0 = the cache's own training arrays) and
// their device table.
int ensure_train_sets(VptContext* c, uint32_t n) {
    vpt::NrcBuffers& b = *c->nrc;
    if (n <= b.num_sets) return VPT_OK;
    const size_t npix = static_cast<size_t>(c->width) * c->height;
    b.sets[0] = vpt::TrainSet{b.counters, b.train_rng, b.train_vertex, b.train_query[0], b.train_target[0],
                              b.train_end_query, b.train_end_inferred, b.train_suffix};
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    for (uint32_t k = b.num_sets > 1 ? b.num_sets : 1; k < n; ++k) {
        vpt::TrainSet& t = b.sets[k];
        chk(alloc_zero(&t.counters, 16));
        chk(alloc_zero(&t.rng, npix));
        chk(alloc_zero(&t.vertex, vpt::kTrainBufferSize));
        chk(alloc_zero(&t.query0, static_cast<size_t>(vpt::kTrainBufferSize) * vpt::kQueryFloats));
        chk(alloc_zero(&t.target0, static_cast<size_t>(vpt::kTrainBufferSize) * 3));
        chk(alloc_zero(&t.end_query, npix * vpt::kQueryFloats));
        chk(alloc_zero(&t.end_inferred, npix * 3));
        chk(alloc_zero(&t.suffix, npix));
        if (e == cudaSuccess) {
            uint64_t mult, plus;
            set_jump(k, &mult, &plus);
            const uint32_t np = static_cast<uint32_t>(npix);
            derive_states_kernel<<<(np + 255) / 256, 256>>>(t.rng, c->d_rng, np, mult, plus);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && !b.train_sets) e = cudaMalloc(reinterpret_cast<void**>(&b.train_sets), sizeof(b.sets));
    if (e == cudaSuccess) e = cudaMemcpy(b.train_sets, b.sets, sizeof(b.sets), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        c->release_nrc();
        return fail(VPT_ERR_OUT_OF_MEMORY, std::string("training sets: ") + cudaGetErrorString(e));
    }
    b.num_sets = n;
    return VPT_OK;
}

// The cache's buffers as the set-up kernels see them for training set k.
vpt::NrcBuffers set_view(const vpt::NrcBuffers& b, uint32_t k) {
    vpt::NrcBuffers v = b;
    const vpt::TrainSet& t = b.sets[k];
    v.counters = t.counters;
    v.train_rng = t.rng;
    v.train_vertex = t.vertex;
    v.train_query[0] = t.query0;
    v.train_target[0] = t.target0;
    v.train_end_query = t.end_query;
    v.train_end_inferred = t.end_inferred;
    v.train_suffix = t.suffix;
    return v;
}

// Launch of a radiance-cache pass of the persistent tracker: the training pass or a render pass
// of one sample per pixel on the per-pixel streams (stream_mode 0), or a render pass of `spp`
// samples per pixel on sample-parallel streams (stream_mode 1). With `index_queries` the render
// paths also list the slots of the queries they write (infer_index, counters[8]).
int launch_pass(VptContext* c, cudaStream_t s, int mode, uint32_t buf, uint32_t spp = 1, int32_t stream_mode = 0,
                bool index_queries = false, uint32_t num_sets = 0, uint32_t set_bufs = 0) {
    if (!c->surf && !c->has_volume)
        return fail(VPT_ERR_INVALID_ARGUMENT, "the radiance-cache passes need a volume or surfaces");
    int rc = ensure_nrc(c);
    if (rc) return rc;
    vpt::TraceParams tp;
    if ((rc = vpt::fill_trace_params(c, &tp))) return rc;
    // With sample-parallel render streams the training pass draws from its own per-pixel states.
    if (mode == vpt::kModeTrainNrc && c->frame.rng_stream_mode == 1) tp.rng = c->nrc->train_rng;
    tp.spp = spp;
    tp.accum_base = 0;
    tp.stream_mode = stream_mode;
    if (stream_mode == 1 && spp > 0) {  // a combined launch of training sets alone has no samples
        if ((rc = vpt::upload_sample_jumps(c, spp, s))) return rc;
        tp.sample_jumps = c->d_jumps;
    }
    tp.park_threshold = c->park_threshold;
    tp.nrc = *c->nrc;
    if (index_queries) {
        NRCP_CUDA(cudaMemsetAsync(c->nrc->counters + 8, 0, sizeof(uint32_t), s));
    } else {
        tp.nrc.infer_index = nullptr;
    }
    tp.nrc_buf = buf;
    tp.train_sets = c->nrc->train_sets;
    tp.num_train_sets = num_sets;
    tp.train_bufs = set_bufs;
    tp.nrc_density_query = c->nrc_query_density;
    tp.nrc_termination = c->nrc_termination;
    tp.nrc_train_termination = c->nrc_train_termination;
    NRCP_CUDA(cudaMemsetAsync(c->d_work, 0, sizeof(unsigned int), s));
    const int threads = c->threads > 0 ? c->threads : (c->surf ? 128 : vpt::kPlainSampleParallelThreads);
    const bool grid_maj = c->has_volume && c->frame.majorant_mode == 1;
    const bool surfaces = c->surf != nullptr;
    size_t smem = 0;
    if (grid_maj && c->mx * c->my * c->mz <= vpt::kMajSmemCells) {
        tp.maj_in_smem = 1;
        smem = static_cast<size_t>(c->mx) * c->my * c->mz * sizeof(float);
    }
    const int ctas = vpt::persistent_grid(c, threads, vpt::nrc_kernel_ptr(mode, grid_maj, surfaces), smem);
    vpt::launch_nrc_pass(tp, mode, grid_maj, surfaces, ctas, threads, smem, s);
    NRCP_CUDA(cudaGetLastError());
    if (stream_mode == 1 && spp > 0) {
        vpt::launch_frame_update(c->d_frame, spp, false, 0, s);
        c->stream_samples += spp;
    }
    return VPT_OK;
}

}  // namespace

namespace vpt {
int nrc_reseed_train_rng(VptContextImpl* c) {
    if (!c->nrc || !c->nrc->train_rng) return VPT_OK;
    // 2^62 draws ahead: disjoint from the render samples' streams (sample s starts s * 2^40
    // draws in, s < 2^22) for any realistic run.
    uint64_t mult, plus;
    lcg_jump(1ull << 62, &mult, &plus);
    const uint32_t n = static_cast<uint32_t>(c->width) * static_cast<uint32_t>(c->height);
    derive_states_kernel<<<(n + 255) / 256, 256>>>(c->nrc->train_rng, c->d_rng, n, mult, plus);
    for (uint32_t k = 1; k < c->nrc->num_sets; ++k) {
        set_jump(k, &mult, &plus);
        derive_states_kernel<<<(n + 255) / 256, 256>>>(c->nrc->sets[k].rng, c->d_rng, n, mult, plus);
    }
    NRCP_CUDA(cudaGetLastError());
    NRCP_CUDA(cudaDeviceSynchronize());
    return VPT_OK;
}

void VptContextImpl::release_nrc() {
    if (!nrc) return;
    free_ptr(nrc->train_end_query);
    free_ptr(nrc->train_end_inferred);
    free_ptr(nrc->train_rng);
    free_ptr(nrc->infer_query);
    free_ptr(nrc->infer_terminal);
    free_ptr(nrc->train_suffix);
    free_ptr(nrc->inferred);
    free_ptr(nrc->frame_contribution);
    free_ptr(nrc->infer_index);
    for (int i = 0; i < 2; ++i) {
        free_ptr(nrc->train_query[i]);
        free_ptr(nrc->train_target[i]);
    }
    free_ptr(nrc->train_vertex);
    free_ptr(nrc->shufflers);
    free_ptr(nrc->counters);
    free_ptr(nrc->stats);
    for (uint32_t k = 1; k < kMaxTrainSets; ++k) {
        TrainSet& t = nrc->sets[k];
        free_ptr(t.counters);
        free_ptr(t.rng);
        free_ptr(t.vertex);
        free_ptr(t.query0);
        free_ptr(t.target0);
        free_ptr(t.end_query);
        free_ptr(t.end_inferred);
        free_ptr(t.suffix);
    }
    free_ptr(nrc->train_sets);
    delete nrc;
    nrc = nullptr;
}
}  // namespace vpt

extern "C" {

int vpt_nrc_enable(VptContext* c) {
    if (!c) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nrc_enable: null context");
    return ensure_nrc(c);
}

int vpt_nrc_get_buffers(VptContext* c, VptNrcBuffers* out) {
    if (!c || !out) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nrc_get_buffers: null argument");
    int rc = ensure_nrc(c);
    if (rc) return rc;
    const vpt::NrcBuffers& b = *c->nrc;
    out->infer_query = b.infer_query;
    out->infer_terminal = b.infer_terminal;
    out->train_suffix = b.train_suffix;
    out->inferred = b.inferred;
    out->frame_contribution = b.frame_contribution;
    for (int i = 0; i < 2; ++i) {
        out->train_query[i] = b.train_query[i];
        out->train_target[i] = b.train_target[i];
    }
    out->train_vertex = b.train_vertex;
    out->train_end_query = b.train_end_query;
    out->train_end_inferred = b.train_end_inferred;
    out->train_rng = b.train_rng;
    out->shufflers = b.shufflers;
    out->counters = b.counters;
    out->stats = b.stats;
    out->infer_capacity = b.infer_capacity;
    out->render_spp = b.render_spp;
    out->buffer_index = c->nrc_buf_index;
    return VPT_OK;
}

int vpt_nrc_set_query_density(VptContext* c, int32_t query_density) {
    if (!c) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nrc_set_query_density: null context");
    c->nrc_query_density = query_density ? 1 : 0;
    return VPT_OK;
}

int vpt_nrc_set_termination_factor(VptContext* c, float render_factor, float train_factor) {
    if (!c || !(render_factor >= 0.0f) || !(render_factor < 1e30f) || !(train_factor >= 0.0f) ||
        !(train_factor < 1e30f))
        return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nrc_set_termination_factor: bad arguments");
    c->nrc_termination = render_factor;
    c->nrc_train_termination = train_factor;
    return VPT_OK;
}

int vpt_prepare_nrc(VptContext* c, void* stream, uint32_t buf, uint32_t offset, int32_t new_sequence) {
    if (!c || buf > 1) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_prepare_nrc: bad arguments");
    int rc = ensure_nrc(c);
    if (rc) return rc;
    vpt::nrc_prepare(*c->nrc, buf, offset, new_sequence != 0, static_cast<cudaStream_t>(stream));
    NRCP_CUDA(cudaGetLastError());
    return VPT_OK;
}

int vpt_launch_generate_training(VptContext* c, void* stream, uint32_t buf) {
    if (!c || buf > 1) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_launch_generate_training: bad arguments");
    return launch_pass(c, static_cast<cudaStream_t>(stream), vpt::kModeTrainNrc, buf);
}

int vpt_propagate(VptContext* c, void* stream) {
    if (!c) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_propagate: null context");
    int rc = ensure_nrc(c);
    if (rc) return rc;
    vpt::nrc_propagate(*c->nrc, radiance_scale(c), static_cast<cudaStream_t>(stream));
    NRCP_CUDA(cudaGetLastError());
    return VPT_OK;
}

int vpt_shuffle(VptContext* c, void* stream, uint32_t buf) {
    if (!c || buf > 1) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_shuffle: bad arguments");
    int rc = ensure_nrc(c);
    if (rc) return rc;
    vpt::nrc_shuffle(*c->nrc, buf, radiance_scale(c), static_cast<cudaStream_t>(stream));
    NRCP_CUDA(cudaGetLastError());
    return VPT_OK;
}

int vpt_launch_render_nrc(VptContext* c, void* stream) {
    if (!c) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_launch_render_nrc: null context");
    return launch_pass(c, static_cast<cudaStream_t>(stream), vpt::kModeRenderNrc, 0);
}

int vpt_accumulate_inferred(VptContext* c, void* stream, uint32_t accum_frames) {
    if (!c) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_accumulate_inferred: null context");
    int rc = ensure_nrc(c);
    if (rc) return rc;
    vpt::nrc_accumulate(*c->nrc, radiance_scale(c), accum_frames, 1, false, c->d_sum, c->d_mean, c->d_err,
                        static_cast<cudaStream_t>(stream));
    NRCP_CUDA(cudaGetLastError());
    c->accum_samples = accum_frames + 1;
    vpt::launch_frame_update(c->d_frame, 0, true, accum_frames + 1, static_cast<cudaStream_t>(stream));
    return VPT_OK;
}

int vpt_launch_render_nrc_batch(VptContext* c, void* stream, uint32_t spp) {
    if (!c || spp == 0) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_launch_render_nrc_batch: bad arguments");
    if (c->has_frame && c->frame.rng_stream_mode != 1)
        return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_launch_render_nrc_batch needs sample-parallel streams");
    int rc = ensure_render_slots(c, spp);
    if (rc) return rc;
    return launch_pass(c, static_cast<cudaStream_t>(stream), vpt::kModeRenderNrc, 0, spp, 1);
}

int vpt_accumulate_inferred_batch(VptContext* c, void* stream, uint32_t accum_frames, uint32_t spp) {
    if (!c || spp == 0) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_accumulate_inferred_batch: bad arguments");
    int rc = ensure_nrc(c);
    if (rc) return rc;
    if (spp > c->nrc->render_spp) return fail(VPT_ERR_INVALID_ARGUMENT, "more samples than render-pass slots");
    vpt::nrc_accumulate(*c->nrc, radiance_scale(c), accum_frames, spp, true, c->d_sum, c->d_mean, c->d_err,
                        static_cast<cudaStream_t>(stream));
    NRCP_CUDA(cudaGetLastError());
    c->accum_samples = accum_frames + spp;
    vpt::launch_frame_update(c->d_frame, 0, true, accum_frames + spp, static_cast<cudaStream_t>(stream));
    return VPT_OK;
}

int vpt_nrc_set_combined_pass(VptContext* c, int32_t on) {
    if (!c) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nrc_set_combined_pass: null context");
    c->nrc_combined_pass = on != 0;
    return VPT_OK;
}

int vpt_nrc_frame(VptContext* c, void* nrc, void* stream, uint32_t train_iterations, uint32_t spp,
                  int32_t new_sequence) {
    if (!c || !nrc) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nrc_frame: null argument");
    auto* net = static_cast<NrcHandle*>(nrc);
    int rc = ensure_nrc(c);
    if (rc) return rc;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t npix = static_cast<uint32_t>(c->width) * static_cast<uint32_t>(c->height);
    const bool batched = c->frame.rng_stream_mode == 1 && spp > 0;
    if (batched && (rc = ensure_render_slots(c, spp))) return rc;
    vpt::NrcBuffers& b = *c->nrc;
    const bool combo = batched && c->nrc_combined_pass;
    constexpr uint32_t kBatch = vpt::kNumTrainingDataPerFrame / 4;  // renderer_main.cpp:1595
    // Predictions for a training pass's suffix-end queries, propagation, shuffle and the four
    // training steps of one iteration (renderer_main.cpp:1578-1600) on the buffers `v`.
    auto post_pass = [&](const vpt::NrcBuffers& v, uint32_t buf) -> int {
        if (nrc_infer_device_count(net, stream, v.train_end_query, v.counters + 7, v.max_train_suffixes,
                                   v.train_end_inferred))
            return fail(VPT_ERR_CUDA, std::string("nrc_infer_device_count: ") + nrc_last_error());
        vpt::nrc_propagate(v, radiance_scale(c), s);
        vpt::nrc_shuffle(v, buf, radiance_scale(c), s);
        NRCP_CUDA(cudaGetLastError());
        for (uint32_t step = 0; step < 4; ++step) {
            const size_t first = static_cast<size_t>(step) * kBatch;
            if (nrc_train(net, stream, v.train_query[1] + first * vpt::kQueryFloats, v.train_target[1] + first * 3,
                          kBatch, nullptr))
                return fail(VPT_ERR_CUDA, std::string("nrc_train: ") + nrc_last_error());
        }
        return VPT_OK;
    };
    if (combo && train_iterations > 0) {
        // The frame's training passes are traced in the launch of its render samples (up to
        // kMaxTrainSets of them per launch, each into its own training set): no pass's path
        // needs the network, only the predictions of its suffix ends, which are inferred after
        // the training steps of the iterations before it, in order, as the sequential frame does.
        // A frame of more iterations (the first one: 8) launches groups of sets, the render
        // samples with the last group.
        const uint32_t group_max = train_iterations < vpt::kMaxTrainSets ? train_iterations : vpt::kMaxTrainSets;
        if ((rc = ensure_train_sets(c, group_max))) return rc;
        for (uint32_t it = 0; it < train_iterations;) {
            const uint32_t group = train_iterations - it < group_max ? train_iterations - it : group_max;
            const bool last = it + group == train_iterations;
            uint32_t bufs = 0;
            for (uint32_t k = 0; k < group; ++k) {
                b.set_buf[k] ^= 1u;
                bufs |= b.set_buf[k] << k;
                const uint32_t offset = static_cast<uint32_t>(c->nrc_offset_rng());
                vpt::nrc_prepare(set_view(b, k), b.set_buf[k], offset, new_sequence != 0, s);
            }
            NRCP_CUDA(cudaGetLastError());
            if ((rc = launch_pass(c, s, vpt::kModeComboNrc, 0, last ? spp : 0, 1, last, group, bufs))) return rc;
            for (uint32_t k = 0; k < group; ++k)
                if ((rc = post_pass(set_view(b, k), b.set_buf[k]))) return rc;
            it += group;
        }
        c->nrc_buf_index = b.set_buf[0];
    } else {
        for (uint32_t it = 0; it < train_iterations; ++it) {
            c->nrc_buf_index = (c->nrc_buf_index + 1) % 2;
            const uint32_t buf = c->nrc_buf_index;
            const uint32_t offset = static_cast<uint32_t>(c->nrc_offset_rng());
            if ((rc = vpt_prepare_nrc(c, stream, buf, offset, new_sequence))) return rc;
            if ((rc = vpt_launch_generate_training(c, stream, buf))) return rc;
            if ((rc = post_pass(b, buf))) return rc;
        }
    }
    if (spp == 0) return VPT_OK;
    if (batched) {
        if ((train_iterations == 0 || !combo) && (rc = launch_pass(c, s, vpt::kModeRenderNrc, 0, spp, 1, true)))
            return rc;
        // Only the slots whose paths ended with a cache query are inferred (the others are not
        // read by the accumulation).
        if (nrc_infer_indexed(net, stream, b.infer_query, b.infer_index, b.counters + 8, npix * spp, b.inferred))
            return fail(VPT_ERR_CUDA, std::string("nrc_infer_indexed: ") + nrc_last_error());
        return vpt_accumulate_inferred_batch(c, stream, c->accum_samples, spp);
    }
    for (uint32_t i = 0; i < spp; ++i) {
        if ((rc = vpt_launch_render_nrc(c, stream))) return rc;
        if (nrc_infer(net, stream, b.infer_query, npix, b.inferred))
            return fail(VPT_ERR_CUDA, std::string("nrc_infer: ") + nrc_last_error());
        if ((rc = vpt_accumulate_inferred(c, stream, c->accum_samples))) return rc;
    }
    return VPT_OK;
}

}  // extern "C"
