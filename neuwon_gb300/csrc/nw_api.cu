// C-ABI entry points of neuwon_gb300: contexts, model structure, attribute
// transfer, mechanisms, stimulus, detectors, probes and stepping dispatch.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>

#include "nw_internal.cuh"

namespace nw {

int fail(nw_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_fail(nw_ctx* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(ctx, e == cudaErrorMemoryAllocation ? NW_ERR_NOMEM : NW_ERR_CUDA, m);
}

int dev_alloc(nw_ctx* ctx, DevBuf& b, size_t bytes) {
    if (b.ptr && b.bytes == bytes) return NW_OK;
    dev_free(b);
    if (bytes == 0) return NW_OK;
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) {
        b.ptr = nullptr;
        return fail(ctx, NW_ERR_NOMEM, "cudaMalloc of " + std::to_string(bytes) +
                                       " bytes failed: " + cudaGetErrorString(e));
    }
    b.bytes = bytes;
    return NW_OK;
}

void dev_free(DevBuf& b) {
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

size_t dtype_size(int dtype) {
    switch (dtype) {
        case NW_DTYPE_F64: case NW_DTYPE_I64: return 8;
        case NW_DTYPE_F32: case NW_DTYPE_I32: case NW_DTYPE_U32: return 4;
        case NW_DTYPE_U8: return 1;
    }
    return 0;
}

static double read_as_double(const void* p, int dtype, int64_t i) {
    switch (dtype) {
        case NW_DTYPE_F64: return static_cast<const double*>(p)[i];
        case NW_DTYPE_F32: return static_cast<const float*>(p)[i];
        case NW_DTYPE_I64: return (double)static_cast<const int64_t*>(p)[i];
        case NW_DTYPE_I32: return static_cast<const int32_t*>(p)[i];
        case NW_DTYPE_U32: return static_cast<const uint32_t*>(p)[i];
        case NW_DTYPE_U8: return static_cast<const uint8_t*>(p)[i];
    }
    return 0.0;
}

static void write_from_double(void* p, int dtype, int64_t i, double v) {
    switch (dtype) {
        case NW_DTYPE_F64: static_cast<double*>(p)[i] = v; break;
        case NW_DTYPE_F32: static_cast<float*>(p)[i] = (float)v; break;
        case NW_DTYPE_I64: static_cast<int64_t*>(p)[i] = (int64_t)v; break;
        case NW_DTYPE_I32: static_cast<int32_t*>(p)[i] = (int32_t)v; break;
        case NW_DTYPE_U32: static_cast<uint32_t*>(p)[i] = (uint32_t)v; break;
        case NW_DTYPE_U8: static_cast<uint8_t*>(p)[i] = (uint8_t)(v != 0.0); break;
    }
}

// Host-side conversion, then one synchronous copy (set-up data only).
int upload_convert(nw_ctx* ctx, void* dst, int dst_dtype, const void* host, int src_dtype,
                   int64_t count) {
    if (count == 0) return NW_OK;
    size_t es = dtype_size(dst_dtype);
    if (!es || !dtype_size(src_dtype)) return fail(ctx, NW_ERR_ARG, "unknown dtype");
    if (dst_dtype == src_dtype) {
        NW_CUDA(ctx, cudaMemcpyAsync(dst, host, es * count, cudaMemcpyHostToDevice, ctx->stream));
        NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return NW_OK;
    }
    std::vector<unsigned char> tmp(es * count);
    for (int64_t i = 0; i < count; ++i)
        write_from_double(tmp.data(), dst_dtype, i, read_as_double(host, src_dtype, i));
    NW_CUDA(ctx, cudaMemcpyAsync(dst, tmp.data(), es * count, cudaMemcpyHostToDevice, ctx->stream));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NW_OK;
}

int download_convert(nw_ctx* ctx, void* host, int dst_dtype, const void* src, int src_dtype,
                     int64_t count) {
    if (count == 0) return NW_OK;
    size_t es = dtype_size(src_dtype);
    if (!es || !dtype_size(dst_dtype)) return fail(ctx, NW_ERR_ARG, "unknown dtype");
    if (dst_dtype == src_dtype) {
        NW_CUDA(ctx, cudaMemcpyAsync(host, src, es * count, cudaMemcpyDeviceToHost, ctx->stream));
        NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return NW_OK;
    }
    std::vector<unsigned char> tmp(es * count);
    NW_CUDA(ctx, cudaMemcpyAsync(tmp.data(), src, es * count, cudaMemcpyDeviceToHost, ctx->stream));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t i = 0; i < count; ++i)
        write_from_double(host, dst_dtype, i, read_as_double(tmp.data(), src_dtype, i));
    return NW_OK;
}

static int real_dtype(nw_ctx* ctx) { return ctx->precision == NW_F64 ? NW_DTYPE_F64 : NW_DTYPE_F32; }

// kI = (dt/2)/C [ms/F], kG = (dt/2 * 1e-3)/C [s/F]  (neuwon/rxd/neuron/electric.py:60-72).
template <typename real>
__global__ void k_factors(const double* cap, real* kI, real* kG, double h_ms, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double c = cap[i];
    kI[i] = (real)(h_ms / c);
    kG[i] = (real)(h_ms * 1e-3 / c);
}

static int refresh_k(nw_ctx* ctx) {
    if (!ctx->have_cap) return NW_OK;
    int64_t n = ctx->n_seg;
    int threads = 256;
    int64_t blocks = (n + threads - 1) / threads;
    double h = 0.5 * ctx->time_step;
    if (ctx->precision == NW_F64)
        k_factors<double><<<blocks, threads, 0, ctx->stream>>>(
            ctx->cap64.as<double>(), ctx->kI.as<double>(), ctx->kG.as<double>(), h, n);
    else
        k_factors<float><<<blocks, threads, 0, ctx->stream>>>(
            ctx->cap64.as<double>(), ctx->kI.as<float>(), ctx->kG.as<float>(), h, n);
    NW_CUDA(ctx, cudaGetLastError());
    return NW_OK;
}

template <typename real>
__global__ void fill_real(real* p, real v, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

static int fill(nw_ctx* ctx, DevBuf& b, double v, int64_t n) {
    if (n == 0) return NW_OK;
    int threads = 256;
    int64_t blocks = (n + threads - 1) / threads;
    if (ctx->precision == NW_F64)
        fill_real<double><<<blocks, threads, 0, ctx->stream>>>(b.as<double>(), v, n);
    else
        fill_real<float><<<blocks, threads, 0, ctx->stream>>>(b.as<float>(), (float)v, n);
    NW_CUDA(ctx, cudaGetLastError());
    return NW_OK;
}

static int64_t neuron_of(const nw_ctx* ctx, int64_t seg) {
    const auto& s = ctx->h_neuron_start;
    return (int64_t)(std::upper_bound(s.begin(), s.end(), seg) - s.begin()) - 1;
}

static void free_hh(HHState& hh) {
    for (DevBuf* b : {&hh.seg, &hh.gm, &hh.gh, &hh.gn, &hh.cna, &hh.ck, &hh.cl, &hh.seg_ptr, &hh.neuron_ptr})
        dev_free(*b);
    hh = HHState();
}

static void free_adj(AdjointState& a) {
    if (a.stream) cudaStreamSynchronize(a.stream);
    for (DevBuf* b : {&a.ckpt, &a.target, &a.loss_part, &a.tape, &a.lamV, &a.lamV2, &a.lamM, &a.lamH, &a.lamN,
                      &a.gGna, &a.gGk, &a.gGl, &a.ra_part, &a.coef})
        dev_free(*b);
    for (cudaEvent_t e : {a.rec_done, a.rev_done[0], a.rev_done[1], a.start})
        if (e) cudaEventDestroy(e);
    if (a.stream) cudaStreamDestroy(a.stream);
    a = AdjointState();
}

static void free_kin(KineticState& k) {
    for (DevBuf* b : {&k.seg, &k.state, &k.gcoef, &k.table, &k.seg_ptr, &k.neuron_ptr, &k.input}) dev_free(*b);
    k = KineticState();
}

static void free_kinetics(nw_ctx* ctx) {
    for (int q = 0; q < kMaxKinetic; ++q) free_kin(ctx->kin[q]);
    ctx->n_kin = 0;
}

// "kinetic.state" names mechanism 0; "kinetic.<q>.<post>" mechanism q's array `post`
// ("state", or "input": the instance values of a two-input table).  Returns the
// index, -1 when the name is not of that form, -2 when q is out of range.
static int kinetic_array_name(const nw_ctx* ctx, const std::string& nm, const std::string& post) {
    if (post == ".state" && nm == "kinetic.state") return ctx->n_kin > 0 ? 0 : -2;
    const std::string pre = "kinetic.";
    if (nm.size() <= pre.size() + post.size() || nm.compare(0, pre.size(), pre) != 0 ||
        nm.compare(nm.size() - post.size(), post.size(), post) != 0)
        return -1;
    const std::string mid = nm.substr(pre.size(), nm.size() - pre.size() - post.size());
    if (mid.empty() || mid.size() > 3 || mid.find_first_not_of("0123456789") != std::string::npos) return -1;
    const int q = std::stoi(mid);
    return q < ctx->n_kin ? q : -2;
}

static int kinetic_state_name(const nw_ctx* ctx, const std::string& nm) {
    return kinetic_array_name(ctx, nm, ".state");
}

void free_syn(SynState& y) {
    for (DevBuf* b : {&y.seg, &y.pre, &y.delay, &y.wa, &y.wn, &y.oa, &y.on, &y.od, &y.pulse_end, &y.events,
                      &y.last_event, &y.mats, &y.seg_ptr, &y.neuron_ptr, &y.ring})
        dev_free(*b);
    y = SynState();
}

int synapse_ring_clear(nw_ctx* ctx) {
    if (ctx->syn.n == 0) return NW_OK;
    NW_CUDA(ctx, cudaMemsetAsync(ctx->syn.ring.ptr, 0, ctx->syn.ring.bytes, ctx->stream));
    return NW_OK;
}

// HH steady state at v (nmodl_library/artificial/hh.mod:48-53, 62-94).
static void hh_steady(double v, double* m, double* h, double* n) {
    auto vtrap = [](double x, double y) {
        return std::fabs(x / y) < 1e-6 ? y * (1 - x / y / 2) : x / (std::exp(x / y) - 1);
    };
    double a = .1 * vtrap(-(v + 40), 10), b = 4 * std::exp(-(v + 65) / 18);
    *m = a / (a + b);
    a = .07 * std::exp(-(v + 65) / 20); b = 1 / (std::exp(-(v + 35) / 10) + 1);
    *h = a / (a + b);
    a = .01 * vtrap(-(v + 55), 10); b = .125 * std::exp(-(v + 65) / 80);
    *n = a / (a + b);
}

// Scatters user-order clamp amplitudes (staged as f64) into the neuron-sorted array.
template <typename real>
__global__ void stage_clamp_amps(const double* stage, const int64_t* sorted_to_user, real* amp, int64_t n) {
    int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s < n) amp[s] = (real)stage[sorted_to_user[s]];
}

}  // namespace nw

using namespace nw;

extern "C" {

int nw_version(void) { return 100; }

int nw_ctx_create(int device, int precision, nw_ctx** out) {
    if (!out) return NW_ERR_ARG;
    *out = nullptr;
    if (precision != NW_F32 && precision != NW_F64) return NW_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return NW_ERR_CUDA;
    }
    nw_ctx* ctx = new nw_ctx();
    ctx->device = device;
    ctx->precision = precision;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    int sms = 0, optin = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e != cudaSuccess) { delete ctx; return NW_ERR_CUDA; }
    ctx->num_sms = sms;
    ctx->smem_optin = (size_t)optin;
    if (dev_alloc(ctx, ctx->work_counter, 64) != NW_OK ||
        dev_alloc(ctx, ctx->status, 64) != NW_OK ||
        dev_alloc(ctx, ctx->dclock, 64) != NW_OK) { delete ctx; return NW_ERR_NOMEM; }
    cudaMemsetAsync(ctx->status.ptr, 0, 64, ctx->stream);
    *out = ctx;
    return NW_OK;
}

int nw_ctx_destroy(nw_ctx* ctx) {
    if (!ctx) return NW_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    graphs_clear(ctx);
    free_hh(ctx->hh);
    free_kinetics(ctx);
    free_syn(ctx->syn);
    free_calcium(ctx->ca);
    free_adj(ctx->adj);
    free_flux(ctx);
    free_quads(ctx);
    DevBuf* bufs[] = {&ctx->neuron_start, &ctx->parent, &ctx->V, &ctx->Vint, &ctx->Inonspec, &ctx->gcache,
                      &ctx->kI, &ctx->kG, &ctx->cap64, &ctx->res64, &ctx->p_rowptr, &ctx->p_col,
                      &ctx->p_val, &ctx->b_rowptr, &ctx->b_col, &ctx->b_val, &ctx->b_leak,
                      &ctx->clamp_seg, &ctx->clamp_amp, &ctx->clamp_first, &ctx->clamp_count,
                      &ctx->clamp_neuron_ptr, &ctx->clamp_amp_stage, &ctx->det_seg, &ctx->det_thr,
                      &ctx->ap_detected, &ctx->ap_state, &ctx->spike_count, &ctx->probe_seg,
                      &ctx->probe_neuron_ptr, &ctx->probe_slot, &ctx->trace, &ctx->neuron_order,
                      &ctx->work_counter, &ctx->status, &ctx->plain_x, &ctx->dclock,
                      &ctx->clamp_seg_ptr, &ctx->w_rowptr, &ctx->w_col, &ctx->w_val, &ctx->w_leak,
                      &ctx->wide_x2, &ctx->wide_cs2, &ctx->vstage[0], &ctx->vstage[1]};
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    for (DevBuf* b : bufs) dev_free(*b);
    for (int k = 0; k < 2; ++k) {
        if (ctx->stage_ready[k]) cudaEventDestroy(ctx->stage_ready[k]);
        if (ctx->stage_done[k]) cudaEventDestroy(ctx->stage_done[k]);
    }
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return NW_OK;
}

int nw_last_error(nw_ctx* ctx, char* buf, int len) {
    if (!buf || len <= 0) return NW_ERR_ARG;
    const char* m = ctx ? ctx->err.c_str() : "no context";
    std::strncpy(buf, m, (size_t)len - 1);
    buf[len - 1] = '\0';
    return NW_OK;
}

int nw_get_stream(nw_ctx* ctx, void** stream) {
    if (!ctx || !stream) return NW_ERR_ARG;
    *stream = (void*)ctx->stream;
    return NW_OK;
}

int nw_synchronize(nw_ctx* ctx) {
    if (!ctx) return NW_ERR_ARG;
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->copy_stream) NW_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
    if (ctx->adj.stream) NW_CUDA(ctx, cudaStreamSynchronize(ctx->adj.stream));
    return NW_OK;
}

int nw_model_init(nw_ctx* ctx, int64_t num_segments, int64_t num_neurons,
                  const int64_t* neuron_start, const int64_t* parent,
                  double time_step_ms, double celsius) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (num_segments <= 0 || num_neurons <= 0 || !neuron_start || !parent)
        return fail(ctx, NW_ERR_ARG, "nw_model_init: empty model or null arrays");
    if (!(time_step_ms > 0.0)) return fail(ctx, NW_ERR_ARG, "nw_model_init: time_step must be > 0");
    if (neuron_start[0] != 0 || neuron_start[num_neurons] != num_segments)
        return fail(ctx, NW_ERR_ARG, "nw_model_init: neuron_start must span [0, num_segments]");
    int64_t maxn = 0;
    for (int64_t k = 0; k < num_neurons; ++k) {
        int64_t a = neuron_start[k], b = neuron_start[k + 1];
        if (b <= a) return fail(ctx, NW_ERR_ARG, "nw_model_init: empty or unordered neuron range");
        maxn = std::max(maxn, b - a);
        for (int64_t i = a; i < b; ++i) {
            int64_t p = parent[i];
            if (p >= 0 && (p < a || p >= i))
                return fail(ctx, NW_ERR_ARG, "nw_model_init: parent of segment " + std::to_string(i) +
                                             " must be an earlier segment of the same neuron");
        }
    }
    // Propagator columns are 32-bit segment indices (the batched path's are
    // 16-bit within a neuron: larger neurons run on the wide path).
    if (num_segments >= INT32_MAX)
        return fail(ctx, NW_ERR_LIMIT, "nw_model_init: at most 2^31 - 2 segments");
    ctx->n_seg = num_segments;
    ctx->n_neuron = num_neurons;
    ctx->max_neuron = maxn;
    ctx->time_step = time_step_ms;
    ctx->celsius = celsius;
    ctx->h_neuron_start.assign(neuron_start, neuron_start + num_neurons + 1);
    ctx->h_parent.assign(parent, parent + num_segments);
    ctx->prop_valid = false;
    ctx->have_cap = ctx->have_res = false;
    ctx->nonspec_nonzero = false;
    ctx->g_valid = false;
    ctx->input_ticks = ctx->steps = 0;
    ctx->have_detectors = false;
    ctx->n_clamps = 0;
    ctx->n_probes = 0;
    ctx->probe_len = 0;
    cudaStreamSynchronize(ctx->stream);
    if (ctx->adj.stream) cudaStreamSynchronize(ctx->adj.stream);
    graphs_clear(ctx);
    free_hh(ctx->hh);
    free_kinetics(ctx);
    free_syn(ctx->syn);
    free_calcium(ctx->ca);
    free_adj(ctx->adj);
    free_flux(ctx);
    free_quads(ctx);
    size_t rs = (size_t)ctx->precision;
    NW_CHECK(dev_alloc(ctx, ctx->neuron_start, 8 * (num_neurons + 1)));
    NW_CHECK(dev_alloc(ctx, ctx->parent, 8 * num_segments));
    NW_CHECK(dev_alloc(ctx, ctx->V, rs * num_segments));
    NW_CHECK(dev_alloc(ctx, ctx->Vint, rs * num_segments));
    NW_CHECK(dev_alloc(ctx, ctx->gcache, 2 * rs * num_segments));
    NW_CHECK(dev_alloc(ctx, ctx->Inonspec, rs * num_segments));
    NW_CHECK(dev_alloc(ctx, ctx->kI, rs * num_segments));
    NW_CHECK(dev_alloc(ctx, ctx->kG, rs * num_segments));
    NW_CHECK(dev_alloc(ctx, ctx->cap64, 8 * num_segments));
    NW_CHECK(dev_alloc(ctx, ctx->res64, 8 * num_segments));
    NW_CHECK(dev_alloc(ctx, ctx->plain_x, rs * num_segments));
    NW_CUDA(ctx, cudaMemcpyAsync(ctx->neuron_start.ptr, neuron_start, 8 * (num_neurons + 1),
                                 cudaMemcpyHostToDevice, ctx->stream));
    NW_CUDA(ctx, cudaMemcpyAsync(ctx->parent.ptr, parent, 8 * num_segments,
                                 cudaMemcpyHostToDevice, ctx->stream));
    NW_CHECK(fill(ctx, ctx->V, -70.0, num_segments));   // rxd_model.py:12 initial_voltage
    NW_CUDA(ctx, cudaMemsetAsync(ctx->Vint.ptr, 0, rs * num_segments, ctx->stream));
    NW_CUDA(ctx, cudaMemsetAsync(ctx->Inonspec.ptr, 0, rs * num_segments, ctx->stream));
    // Default AP detectors: each neuron's first segment (its root), 20 mV (neuron.py:28, 43).
    std::vector<int64_t> dseg(num_neurons);
    std::vector<double> dthr(num_neurons, 20.0);
    for (int64_t k = 0; k < num_neurons; ++k) dseg[k] = neuron_start[k];
    NW_CHECK(nw_detectors_set(ctx, dseg.data(), dthr.data()));
    // Work order: largest neurons first (longest-processing-time-first).
    std::vector<int32_t> order(num_neurons);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        return (neuron_start[a + 1] - neuron_start[a]) > (neuron_start[b + 1] - neuron_start[b]);
    });
    NW_CHECK(dev_alloc(ctx, ctx->neuron_order, 4 * num_neurons));
    NW_CUDA(ctx, cudaMemcpyAsync(ctx->neuron_order.ptr, order.data(), 4 * num_neurons,
                                 cudaMemcpyHostToDevice, ctx->stream));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NW_OK;
}

int nw_set_data(nw_ctx* ctx, const char* name, const void* host, int dtype, int64_t count) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx || !name || (!host && count)) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    std::string nm(name);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_set_data before nw_model_init");
    auto need = [&](int64_t n) {
        return count == n ? NW_OK : fail(ctx, NW_ERR_ARG, nm + ": expected " + std::to_string(n) +
                                                           " values, got " + std::to_string(count));
    };
    int rd = real_dtype(ctx);
    if (nm == "Segment.voltage") {
        NW_CHECK(need(ctx->n_seg));
        return upload_convert(ctx, ctx->V.ptr, rd, host, dtype, count);
    }
    if (nm == "Segment.integral_voltage") {
        NW_CHECK(need(ctx->n_seg));
        return upload_convert(ctx, ctx->Vint.ptr, rd, host, dtype, count);
    }
    if (nm == "Segment.nonspecific_current") {
        NW_CHECK(need(ctx->n_seg));
        bool nz = false;
        for (int64_t i = 0; i < count && !nz; ++i) nz = read_as_double(host, dtype, i) != 0.0;
        ctx->nonspec_nonzero = nz;
        return upload_convert(ctx, ctx->Inonspec.ptr, rd, host, dtype, count);
    }
    if (nm == "Segment.capacitance" || nm == "Segment.axial_resistance") {
        NW_CHECK(need(ctx->n_seg));
        bool cap = nm == "Segment.capacitance";
        for (int64_t i = 0; i < count; ++i) {
            double v = read_as_double(host, dtype, i);
            if (!(v > 0.0) || !std::isfinite(v)) {
                if (!cap && ctx->h_parent[i] < 0) continue;   // a root's resistance is unused
                return fail(ctx, NW_ERR_ARG, nm + " must be finite and > 0 (segment " + std::to_string(i) + ")");
            }
        }
        NW_CHECK(upload_convert(ctx, cap ? ctx->cap64.ptr : ctx->res64.ptr, NW_DTYPE_F64, host, dtype, count));
        if (cap) { ctx->have_cap = true; NW_CHECK(refresh_k(ctx)); }
        else ctx->have_res = true;
        ctx->prop_valid = false;
        NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return NW_OK;
    }
    if (nm == "hh.m" || nm == "hh.h" || nm == "hh.n" ||
        nm == "hh.gna_coef" || nm == "hh.gk_coef" || nm == "hh.gl_coef") {
        NW_CHECK(need(ctx->hh.m));
        std::vector<double> sorted(count);
        for (int64_t i = 0; i < count; ++i) sorted[ctx->hh.user_to_sorted[i]] = read_as_double(host, dtype, i);
        HHState& hh = ctx->hh;
        DevBuf& b = nm == "hh.m" ? hh.gm : nm == "hh.h" ? hh.gh : nm == "hh.n" ? hh.gn :
                    nm == "hh.gna_coef" ? hh.cna : nm == "hh.gk_coef" ? hh.ck : hh.cl;
        return upload_convert(ctx, b.ptr, rd, sorted.data(), NW_DTYPE_F64, count);
    }
    if (const int q = kinetic_array_name(ctx, nm, ".input"); q != -1) {
        if (q < 0 || ctx->kin[q].ninp != 2) return fail(ctx, NW_ERR_ARG, nm + ": no two-input kinetic mechanism");
        const KineticState& K = ctx->kin[q];
        NW_CHECK(need(K.m));
        std::vector<double> sorted(count);
        for (int64_t i = 0; i < count; ++i) sorted[K.user_to_sorted[i]] = read_as_double(host, dtype, i);
        return upload_convert(ctx, K.input.ptr, rd, sorted.data(), NW_DTYPE_F64, count);
    }
    if (const int q = kinetic_state_name(ctx, nm); q != -1) {
        if (q < 0) return fail(ctx, NW_ERR_ARG, nm + ": no such kinetic mechanism");
        const KineticState& K = ctx->kin[q];
        NW_CHECK(need(K.m * K.S));
        std::vector<double> sorted((size_t)K.S * K.m);
        for (int64_t u = 0; u < K.m; ++u)
            for (int c = 0; c < K.S; ++c)
                sorted[(size_t)c * K.m + K.user_to_sorted[u]] = read_as_double(host, dtype, u * K.S + c);
        return upload_convert(ctx, K.state.ptr, rd, sorted.data(), NW_DTYPE_F64, count);
    }
    if (nm == "Synapse.ampa_open" || nm == "Synapse.nmda_open" || nm == "Synapse.nmda_desensitized") {
        SynState& Y = ctx->syn;
        NW_CHECK(need(Y.n));
        std::vector<double> sorted(count);
        for (int64_t i = 0; i < count; ++i) sorted[Y.user_to_sorted[i]] = read_as_double(host, dtype, i);
        DevBuf& b = nm == "Synapse.ampa_open" ? Y.oa : nm == "Synapse.nmda_open" ? Y.on : Y.od;
        return upload_convert(ctx, b.ptr, rd, sorted.data(), NW_DTYPE_F64, count);
    }
    if (nm == "Synapse.events" || nm == "Synapse.last_event" || nm == "Synapse.pulse_end") {
        SynState& Y = ctx->syn;
        NW_CHECK(need(Y.n));
        std::vector<double> sorted(count);
        for (int64_t i = 0; i < count; ++i) sorted[Y.user_to_sorted[i]] = read_as_double(host, dtype, i);
        DevBuf& b = nm == "Synapse.events" ? Y.events : nm == "Synapse.last_event" ? Y.last_event : Y.pulse_end;
        return upload_convert(ctx, b.ptr, nm == "Synapse.events" ? NW_DTYPE_U32 : NW_DTYPE_I32, sorted.data(),
                              NW_DTYPE_F64, count);
    }
    if (nm == "Synapse.spike_ring") {
        // Raw spike bits: ring_neurons x ring_words u32 words (steps modulo the ring length).
        NW_CHECK(need(ctx->syn.n ? ctx->syn.ring_neurons * ctx->syn.ring_words : 0));
        if (!count) return NW_OK;
        return upload_convert(ctx, ctx->syn.ring.ptr, NW_DTYPE_U32, host, dtype, count);
    }
    if (nm == "Neuron.AP_state") {
        NW_CHECK(need(ctx->n_neuron));
        return upload_convert(ctx, ctx->ap_state.ptr, NW_DTYPE_U8, host, dtype, count);
    }
    if (nm == "Neuron.AP_detected") {
        NW_CHECK(need(ctx->n_neuron));
        return upload_convert(ctx, ctx->ap_detected.ptr, NW_DTYPE_U8, host, dtype, count);
    }
    if (nm == "Neuron.spike_count") {
        NW_CHECK(need(ctx->n_neuron));
        return upload_convert(ctx, ctx->spike_count.ptr, NW_DTYPE_U32, host, dtype, count);
    }
    return fail(ctx, NW_ERR_ARG, "nw_set_data: unknown attribute " + nm);
}

int nw_get_data(nw_ctx* ctx, const char* name, void* host, int dtype, int64_t count) {
    if (!ctx || !name || (!host && count)) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    std::string nm(name);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_get_data before nw_model_init");
    auto need = [&](int64_t n) {
        return count == n ? NW_OK : fail(ctx, NW_ERR_ARG, nm + ": expected " + std::to_string(n) +
                                                           " values, got " + std::to_string(count));
    };
    int rd = real_dtype(ctx);
    if (nm == "Segment.voltage") { NW_CHECK(need(ctx->n_seg)); return download_convert(ctx, host, dtype, ctx->V.ptr, rd, count); }
    if (nm == "Segment.integral_voltage") { NW_CHECK(need(ctx->n_seg)); return download_convert(ctx, host, dtype, ctx->Vint.ptr, rd, count); }
    if (nm == "Segment.nonspecific_current") { NW_CHECK(need(ctx->n_seg)); return download_convert(ctx, host, dtype, ctx->Inonspec.ptr, rd, count); }
    if (nm == "Segment.capacitance") { NW_CHECK(need(ctx->n_seg)); return download_convert(ctx, host, dtype, ctx->cap64.ptr, NW_DTYPE_F64, count); }
    if (nm == "Segment.axial_resistance") { NW_CHECK(need(ctx->n_seg)); return download_convert(ctx, host, dtype, ctx->res64.ptr, NW_DTYPE_F64, count); }
    if (nm == "hh.m" || nm == "hh.h" || nm == "hh.n" ||
        nm == "hh.gna_coef" || nm == "hh.gk_coef" || nm == "hh.gl_coef") {
        NW_CHECK(need(ctx->hh.m));
        const HHState& hh = ctx->hh;
        const DevBuf& b = nm == "hh.m" ? hh.gm : nm == "hh.h" ? hh.gh : nm == "hh.n" ? hh.gn :
                          nm == "hh.gna_coef" ? hh.cna : nm == "hh.gk_coef" ? hh.ck : hh.cl;
        std::vector<double> sorted(count);
        NW_CHECK(download_convert(ctx, sorted.data(), NW_DTYPE_F64, b.ptr, rd, count));
        for (int64_t i = 0; i < count; ++i) write_from_double(host, dtype, i, sorted[ctx->hh.user_to_sorted[i]]);
        return NW_OK;
    }
    if (const int q = kinetic_array_name(ctx, nm, ".input"); q != -1) {
        if (q < 0 || ctx->kin[q].ninp != 2) return fail(ctx, NW_ERR_ARG, nm + ": no two-input kinetic mechanism");
        const KineticState& K = ctx->kin[q];
        NW_CHECK(need(K.m));
        std::vector<double> sorted(count);
        NW_CHECK(download_convert(ctx, sorted.data(), NW_DTYPE_F64, K.input.ptr, rd, count));
        for (int64_t i = 0; i < count; ++i) write_from_double(host, dtype, i, sorted[K.user_to_sorted[i]]);
        return NW_OK;
    }
    if (const int q = kinetic_state_name(ctx, nm); q != -1) {
        if (q < 0) return fail(ctx, NW_ERR_ARG, nm + ": no such kinetic mechanism");
        const KineticState& K = ctx->kin[q];
        NW_CHECK(need(K.m * K.S));
        std::vector<double> sorted((size_t)K.S * K.m);
        NW_CHECK(download_convert(ctx, sorted.data(), NW_DTYPE_F64, K.state.ptr, rd, count));
        for (int64_t u = 0; u < K.m; ++u)
            for (int c = 0; c < K.S; ++c)
                write_from_double(host, dtype, u * K.S + c, sorted[(size_t)c * K.m + K.user_to_sorted[u]]);
        return NW_OK;
    }
    if (nm == "Synapse.spike_ring") {
        NW_CHECK(need(ctx->syn.n ? ctx->syn.ring_neurons * ctx->syn.ring_words : 0));
        if (!count) return NW_OK;
        return download_convert(ctx, host, dtype, ctx->syn.ring.ptr, NW_DTYPE_U32, count);
    }
    if (nm.rfind("Synapse.", 0) == 0) {
        const SynState& Y = ctx->syn;
        const DevBuf* b = nullptr;
        int sd = rd;
        if (nm == "Synapse.ampa_open") b = &Y.oa;
        else if (nm == "Synapse.nmda_open") b = &Y.on;
        else if (nm == "Synapse.nmda_desensitized") b = &Y.od;
        else if (nm == "Synapse.events") { b = &Y.events; sd = NW_DTYPE_U32; }
        else if (nm == "Synapse.last_event") { b = &Y.last_event; sd = NW_DTYPE_I32; }
        else if (nm == "Synapse.pulse_end") { b = &Y.pulse_end; sd = NW_DTYPE_I32; }
        else return fail(ctx, NW_ERR_ARG, "nw_get_data: unknown attribute " + nm);
        NW_CHECK(need(Y.n));
        std::vector<double> sorted(count);
        NW_CHECK(download_convert(ctx, sorted.data(), NW_DTYPE_F64, b->ptr, sd, count));
        for (int64_t i = 0; i < count; ++i) write_from_double(host, dtype, i, sorted[Y.user_to_sorted[i]]);
        return NW_OK;
    }
    if (nm == "Neuron.AP_state") { NW_CHECK(need(ctx->n_neuron)); return download_convert(ctx, host, dtype, ctx->ap_state.ptr, NW_DTYPE_U8, count); }
    if (nm == "Neuron.AP_detected") { NW_CHECK(need(ctx->n_neuron)); return download_convert(ctx, host, dtype, ctx->ap_detected.ptr, NW_DTYPE_U8, count); }
    if (nm == "Neuron.spike_count") { NW_CHECK(need(ctx->n_neuron)); return download_convert(ctx, host, dtype, ctx->spike_count.ptr, NW_DTYPE_U32, count); }
    return fail(ctx, NW_ERR_ARG, "nw_get_data: unknown attribute " + nm);
}

int nw_propagator_build(nw_ctx* ctx, double prune_tolerance, int64_t* nnz_out) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_propagator_build before nw_model_init");
    if (!ctx->have_cap || !ctx->have_res)
        return fail(ctx, NW_ERR_STATE, "nw_propagator_build needs Segment.capacitance and Segment.axial_resistance");
    if (!(prune_tolerance >= 0.0)) return fail(ctx, NW_ERR_ARG, "prune_tolerance must be >= 0");
    NW_CHECK(propagator_build(ctx, prune_tolerance, nnz_out));
    NW_CHECK(propagator_to_batched(ctx));
    ctx->prop_valid = true;
    ctx->prop_built = !ctx->prop_lump;           // lumped rows break detailed balance
    ctx->prop_lumped = ctx->prop_lump;
    if (ctx->prop_lump && ctx->prop_format == 1) ctx->prop_format = 0;
    return NW_OK;
}

int nw_propagator_set_csr(nw_ctx* ctx, int64_t n, const int64_t* rowptr, const int64_t* col,
                          const double* val, int64_t nnz) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_propagator_set_csr before nw_model_init");
    if (n != ctx->n_seg || !rowptr || (nnz && (!col || !val)))
        return fail(ctx, NW_ERR_ARG, "nw_propagator_set_csr: shape does not match the model");
    if (rowptr[0] != 0 || rowptr[n] != nnz) return fail(ctx, NW_ERR_ARG, "nw_propagator_set_csr: bad rowptr");
    for (int64_t k = 0; k < ctx->n_neuron; ++k) {
        int64_t a = ctx->h_neuron_start[k], b = ctx->h_neuron_start[k + 1];
        for (int64_t i = a; i < b; ++i) {
            if (rowptr[i + 1] < rowptr[i]) return fail(ctx, NW_ERR_ARG, "nw_propagator_set_csr: rowptr decreases");
            for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
                if (col[e] < a || col[e] >= b)
                    return fail(ctx, NW_ERR_ARG, "nw_propagator_set_csr: entry couples two neurons (row " +
                                                 std::to_string(i) + ")");
        }
    }
    NW_CHECK(propagator_from_host(ctx, rowptr, col, val, nnz));
    NW_CHECK(propagator_to_batched(ctx));
    ctx->prop_valid = true;
    ctx->prop_built = false;
    ctx->prop_lumped = false;
    ctx->prop_format = 0;
    return NW_OK;
}

int nw_propagator_conserve(nw_ctx* ctx) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!ctx->prop_valid) return fail(ctx, NW_ERR_STATE, "nw_propagator_conserve: no propagator installed");
    NW_CHECK(propagator_conserve(ctx));
    return propagator_to_batched(ctx);
}

int nw_propagator_get_csr(nw_ctx* ctx, int64_t* rowptr, int64_t* col, double* val, int64_t* nnz_out) {
    if (!ctx) return NW_ERR_ARG;
    if (!ctx->prop_valid) return fail(ctx, NW_ERR_STATE, "no propagator installed");
    if (nnz_out) *nnz_out = ctx->nnz64;
    if (!rowptr) return NW_OK;
    NW_CUDA(ctx, cudaMemcpyAsync(rowptr, ctx->p_rowptr.ptr, 8 * (ctx->n_seg + 1), cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<int32_t> c32(ctx->nnz64);
    if (ctx->nnz64) {
        NW_CUDA(ctx, cudaMemcpyAsync(c32.data(), ctx->p_col.ptr, 4 * ctx->nnz64, cudaMemcpyDeviceToHost, ctx->stream));
        NW_CUDA(ctx, cudaMemcpyAsync(val, ctx->p_val.ptr, 8 * ctx->nnz64, cudaMemcpyDeviceToHost, ctx->stream));
    }
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t e = 0; e < ctx->nnz64; ++e) col[e] = c32[e];
    return NW_OK;
}

int nw_propagator_stats(nw_ctx* ctx, int64_t* rows, int64_t* nnz, int64_t* stored, int64_t* bytes) {
    if (!ctx) return NW_ERR_ARG;
    if (!ctx->prop_valid) return fail(ctx, NW_ERR_STATE, "no propagator installed");
    if (rows) *rows = ctx->n_seg;
    if (nnz) *nnz = ctx->nnz64;
    if (ctx->prop_format == 3 && ctx->b_ok) {
        // Windows format: per window its values and a 16-bit base (value blocks
        // padded to 4 values); per row a 16-byte descriptor and the leak.
        NW_CHECK(ensure_windows(ctx));
        const int64_t slots = ctx->win_slots;
        const int64_t windows = ctx->nwin[0] + ctx->nwin[1] + ctx->nwin[2] + ctx->nwin[3];
        if (stored) *stored = slots;
        if (bytes) *bytes = slots * ctx->precision + 2 * windows + ctx->n_seg * (16 + ctx->precision);
        return NW_OK;
    }
    if (ctx->prop_format == 2 && ctx->b_ok) {
        // Quad format: 4 value slots + a 16-bit base per quad.
        NW_CHECK(ensure_quads(ctx));
        if (stored) *stored = 4 * ctx->nq;
        if (bytes) *bytes = ctx->nq * (4 * ctx->precision + 2) + ctx->n_seg * (8 + ctx->precision);
        return NW_OK;
    }
    if (ctx->prop_format == 1 && ctx->b_ok) {
        // Pair format: stored pairs, with c_max / c_i per row besides the leak.
        NW_CHECK(ensure_flux(ctx));
        if (stored) *stored = ctx->nnz_f;
        if (bytes) *bytes = ctx->nnz_f * (2 + ctx->precision) + ctx->n_seg * (8 + 2 * ctx->precision);
        return NW_OK;
    }
    if (stored) *stored = ctx->b_ok ? ctx->nnz_b : ctx->nnz_w;
    if (bytes) *bytes = ctx->b_ok ? ctx->nnz_b * (2 + ctx->precision) + ctx->n_seg * (8 + ctx->precision)
                                  : ctx->nnz_w * (4 + ctx->precision) + ctx->n_seg * (8 + ctx->precision);
    return NW_OK;
}

// Segment-sorted (stable) layout of mechanism instances, so every segment's
// instances are contiguous and every neuron's instances form one range.
struct InstanceLayout {
    std::vector<int64_t> order;          // sorted position -> user index
    std::vector<int64_t> user_to_sorted;
    std::vector<uint32_t> seg, seg_ptr;  // [m], [n_seg+1]
    std::vector<int64_t> nptr;           // [n_neuron+1]
    bool identity = false;
};

static int layout_instances(nw_ctx* ctx, int64_t m, const int64_t* segment, const char* who,
                            InstanceLayout& L) {
    const int64_t n = ctx->n_seg;
    for (int64_t i = 0; i < m; ++i)
        if (segment[i] < 0 || segment[i] >= n)
            return fail(ctx, NW_ERR_ARG, std::string(who) + ": segment index out of range");
    L.order.resize(m);
    std::iota(L.order.begin(), L.order.end(), 0);
    std::stable_sort(L.order.begin(), L.order.end(), [&](int64_t a, int64_t b) { return segment[a] < segment[b]; });
    L.user_to_sorted.assign(m, 0);
    for (int64_t s = 0; s < m; ++s) L.user_to_sorted[L.order[s]] = s;
    L.identity = (m == n);
    for (int64_t s = 0; s < m && L.identity; ++s) L.identity = segment[L.order[s]] == s;
    L.seg.assign(m, 0);
    L.seg_ptr.assign(n + 1, 0);
    L.nptr.assign(ctx->n_neuron + 1, 0);
    for (int64_t s = 0; s < m; ++s) {
        int64_t u = L.order[s];
        L.seg[s] = (uint32_t)segment[u];
        L.seg_ptr[segment[u] + 1]++;
        L.nptr[neuron_of(ctx, segment[u]) + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) L.seg_ptr[i + 1] += L.seg_ptr[i];
    for (int64_t k = 0; k < ctx->n_neuron; ++k) L.nptr[k + 1] += L.nptr[k];
    return NW_OK;
}

static int upload_layout(nw_ctx* ctx, const InstanceLayout& L, DevBuf& seg, DevBuf& seg_ptr, DevBuf& nptr) {
    const int64_t m = (int64_t)L.seg.size();
    NW_CHECK(dev_alloc(ctx, seg, 4 * std::max<int64_t>(m, 1)));
    NW_CHECK(dev_alloc(ctx, seg_ptr, 4 * (ctx->n_seg + 1)));
    NW_CHECK(dev_alloc(ctx, nptr, 8 * (ctx->n_neuron + 1)));
    NW_CHECK(upload_convert(ctx, seg.ptr, NW_DTYPE_U32, L.seg.data(), NW_DTYPE_U32, m));
    NW_CHECK(upload_convert(ctx, seg_ptr.ptr, NW_DTYPE_U32, L.seg_ptr.data(), NW_DTYPE_U32, ctx->n_seg + 1));
    NW_CHECK(upload_convert(ctx, nptr.ptr, NW_DTYPE_I64, L.nptr.data(), NW_DTYPE_I64, ctx->n_neuron + 1));
    return NW_OK;
}

int nw_hh_register(nw_ctx* ctx, int64_t num_instances, const int64_t* segment,
                   const double* gna_coef, const double* gk_coef, const double* gl_coef,
                   double ena, double ek, double el, double v_init) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_hh_register before nw_model_init");
    if (num_instances < 0 || (num_instances && (!segment || !gna_coef || !gk_coef || !gl_coef)))
        return fail(ctx, NW_ERR_ARG, "nw_hh_register: null arrays");
    const int64_t m = num_instances;
    InstanceLayout L;
    NW_CHECK(layout_instances(ctx, m, segment, "nw_hh_register", L));
    HHState& hh = ctx->hh;
    free_hh(hh);
    hh.m = m;
    hh.ena = ena; hh.ek = ek; hh.el = el; hh.v_init = v_init;
    hh.user_to_sorted = L.user_to_sorted;
    hh.identity = L.identity;
    hh.h_neuron_ptr = L.nptr;
    std::vector<double> cna(m), ck(m), cl(m), g0(m);
    for (int64_t s = 0; s < m; ++s) {
        int64_t u = L.order[s];
        cna[s] = gna_coef[u]; ck[s] = gk_coef[u]; cl[s] = gl_coef[u];
    }
    double m0, h0, n0;
    hh_steady(v_init, &m0, &h0, &n0);
    size_t rs = (size_t)ctx->precision;
    int rd = real_dtype(ctx);
    NW_CHECK(upload_layout(ctx, L, hh.seg, hh.seg_ptr, hh.neuron_ptr));
    for (DevBuf* b : {&hh.gm, &hh.gh, &hh.gn, &hh.cna, &hh.ck, &hh.cl})
        NW_CHECK(dev_alloc(ctx, *b, rs * std::max<int64_t>(m, 1)));
    NW_CHECK(upload_convert(ctx, hh.cna.ptr, rd, cna.data(), NW_DTYPE_F64, m));
    NW_CHECK(upload_convert(ctx, hh.ck.ptr, rd, ck.data(), NW_DTYPE_F64, m));
    NW_CHECK(upload_convert(ctx, hh.cl.ptr, rd, cl.data(), NW_DTYPE_F64, m));
    std::fill(g0.begin(), g0.end(), m0);
    NW_CHECK(upload_convert(ctx, hh.gm.ptr, rd, g0.data(), NW_DTYPE_F64, m));
    std::fill(g0.begin(), g0.end(), h0);
    NW_CHECK(upload_convert(ctx, hh.gh.ptr, rd, g0.data(), NW_DTYPE_F64, m));
    std::fill(g0.begin(), g0.end(), n0);
    NW_CHECK(upload_convert(ctx, hh.gn.ptr, rd, g0.data(), NW_DTYPE_F64, m));
    ctx->g_valid = false;
    return NW_OK;
}

}  // extern "C"

namespace nw {

// Appends one kinetic mechanism (see nw_kinetic_add) and stores its index in *id_out.
static int kinetic_add(nw_ctx* ctx, const char* who, int64_t num_instances, const int64_t* segment,
                       const double* g_coef, int num_states, int num_open, const int32_t* open_states,
                       double erev, int32_t species, const double* table, int num_buckets, int num_terms,
                       double vmin, double bucket_frq, double conserve_sum, const double* init_state,
                       int32_t* id_out) {
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    const std::string w(who);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, w + " before nw_model_init");
    const int S = num_states, T = num_terms;
    if (S < 1 || S > 16 || T < 1 || T > kMaxTerms || num_buckets < 1 || num_open < 1 || num_open > kMaxOpen ||
        !open_states || !table || !init_state || !(bucket_frq > 0))
        return fail(ctx, NW_ERR_ARG, w + ": need 1<=S<=16, 1<=terms<=" + std::to_string(kMaxTerms) + ", 1.." +
                                     std::to_string(kMaxOpen) + " open states, a table and an initial state");
    for (int k = 0; k < num_open; ++k)
        if (open_states[k] < 0 || open_states[k] >= S)
            return fail(ctx, NW_ERR_ARG, w + ": open state index out of range");
    if (species >= (int32_t)ctx->species_erev.size() || species < -1)
        return fail(ctx, NW_ERR_ARG, w + ": species " + std::to_string(species) + " was not declared (nw_species_set)");
    if (ctx->n_kin >= kMaxKinetic)
        return fail(ctx, NW_ERR_LIMIT, w + ": at most " + std::to_string(kMaxKinetic) + " kinetic mechanisms");
    const int64_t m = num_instances;
    if (m < 0 || (m && (!segment || !g_coef))) return fail(ctx, NW_ERR_ARG, w + ": null arrays");
    InstanceLayout L;
    NW_CHECK(layout_instances(ctx, m, segment, who, L));
    const int q = ctx->n_kin;
    KineticState& K = ctx->kin[q];
    free_kin(K);
    K.m = m; K.S = S; K.T = T; K.nb = num_buckets; K.n_open = num_open;
    for (int k = 0; k < num_open; ++k) K.open[k] = open_states[k];
    K.identity = L.identity;
    K.species = species;
    K.erev = species >= 0 ? ctx->species_erev[species] : erev;
    K.vmin = vmin; K.frq = bucket_frq; K.conserve = conserve_sum;
    K.user_to_sorted = L.user_to_sorted;
    K.h_neuron_ptr = L.nptr;
    size_t rs = (size_t)ctx->precision;
    int rd = real_dtype(ctx);
    NW_CHECK(upload_layout(ctx, L, K.seg, K.seg_ptr, K.neuron_ptr));
    NW_CHECK(dev_alloc(ctx, K.state, rs * S * std::max<int64_t>(m, 1)));
    NW_CHECK(dev_alloc(ctx, K.gcoef, rs * std::max<int64_t>(m, 1)));
    const int64_t tsize = (int64_t)num_buckets * S * S * T;
    NW_CHECK(dev_alloc(ctx, K.table, rs * tsize));
    std::vector<double> g(m), st((size_t)S * m);
    for (int64_t s = 0; s < m; ++s) g[s] = g_coef[L.order[s]];
    for (int c = 0; c < S; ++c)
        for (int64_t s = 0; s < m; ++s) st[(size_t)c * m + s] = init_state[c];
    NW_CHECK(upload_convert(ctx, K.gcoef.ptr, rd, g.data(), NW_DTYPE_F64, m));
    NW_CHECK(upload_convert(ctx, K.state.ptr, rd, st.data(), NW_DTYPE_F64, (int64_t)S * m));
    NW_CHECK(upload_convert(ctx, K.table.ptr, rd, table, NW_DTYPE_F64, tsize));
    ctx->n_kin = q + 1;
    ctx->g_valid = false;
    if (id_out) *id_out = q;
    return NW_OK;
}

}  // namespace nw

extern "C" {

int nw_species_set(nw_ctx* ctx, int32_t count, const double* reversal_potential_mV) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx || count < 0 || (count && !reversal_potential_mV)) return NW_ERR_ARG;
    for (int32_t s = 0; s < count; ++s)
        if (!std::isfinite(reversal_potential_mV[s]))
            return fail(ctx, NW_ERR_ARG, "nw_species_set: reversal potentials must be finite");
    for (int q = 0; q < ctx->n_kin; ++q)
        if (ctx->kin[q].species >= count)
            return fail(ctx, NW_ERR_STATE, "nw_species_set: a registered kinetic mechanism feeds species " +
                                           std::to_string(ctx->kin[q].species));
    ctx->species_erev.assign(reversal_potential_mV, reversal_potential_mV + count);
    for (int q = 0; q < ctx->n_kin; ++q)
        if (ctx->kin[q].species >= 0) ctx->kin[q].erev = ctx->species_erev[ctx->kin[q].species];
    return NW_OK;
}

int nw_species_conductance(nw_ctx* ctx, int32_t species, double* conductance_out) {
    if (!ctx || !conductance_out) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_species_conductance before nw_model_init");
    if (species < 0 || species >= (int32_t)ctx->species_erev.size())
        return fail(ctx, NW_ERR_ARG, "nw_species_conductance: no such species");
    return species_conductance(ctx, species, conductance_out);
}

int nw_kinetic_clear(nw_ctx* ctx) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    free_kinetics(ctx);
    ctx->g_valid = false;
    return NW_OK;
}

int nw_kinetic_add(nw_ctx* ctx, int64_t num_instances, const int64_t* segment, const double* g_coef,
                   int num_states, int num_open, const int32_t* open_states, double erev, int32_t species,
                   const double* table, int num_buckets, int num_terms, double vmin, double bucket_frq,
                   double conserve_sum, const double* init_state, int32_t* mechanism_out) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    return kinetic_add(ctx, "nw_kinetic_add", num_instances, segment, g_coef, num_states, num_open, open_states,
                       erev, species, table, num_buckets, num_terms, vmin, bucket_frq, conserve_sum, init_state,
                       mechanism_out);
}

int nw_kinetic_inputs(nw_ctx* ctx, int32_t mechanism, int32_t kind1, int32_t num_buckets1, double minimum1,
                      double bucket_frq1, double scale1, int32_t kind2, int32_t num_buckets2, double minimum2,
                      double bucket_frq2, double scale2, int32_t num_terms, const int32_t* powers,
                      double input_initial) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (mechanism < 0 || mechanism >= ctx->n_kin)
        return fail(ctx, NW_ERR_ARG, "nw_kinetic_inputs: no such kinetic mechanism");
    KineticState& K = ctx->kin[mechanism];
    const int32_t kinds[2] = {kind1, kind2}, nbs[2] = {num_buckets1, num_buckets2};
    const double mins[2] = {minimum1, minimum2}, frqs[2] = {bucket_frq1, bucket_frq2}, scs[2] = {scale1, scale2};
    for (int d = 0; d < 2; ++d) {
        if (kinds[d] < 0 || kinds[d] > 2 || nbs[d] < 1 || !(frqs[d] > 0) || !std::isfinite(mins[d]))
            return fail(ctx, NW_ERR_ARG, "nw_kinetic_inputs: kinds 0..2, buckets >= 1, bucket_frq > 0");
        if (kinds[d] == 1 && !(mins[d] + scs[d] > 0))
            return fail(ctx, NW_ERR_ARG, "nw_kinetic_inputs: a logarithmic input needs minimum + scale > 0");
    }
    if ((int64_t)num_buckets1 * num_buckets2 != K.nb || num_terms != K.T || !powers)
        return fail(ctx, NW_ERR_ARG, "nw_kinetic_inputs: buckets1 * buckets2 and terms must match the table (" +
                                     std::to_string(K.nb) + " buckets, " + std::to_string(K.T) + " terms)");
    for (int t = 0; t < num_terms; ++t)
        if (powers[2 * t] < 0 || powers[2 * t] > 9 || powers[2 * t + 1] < 0 || powers[2 * t + 1] > 9)
            return fail(ctx, NW_ERR_ARG, "nw_kinetic_inputs: powers in 0..9");
    if (!std::isfinite(input_initial)) return fail(ctx, NW_ERR_ARG, "nw_kinetic_inputs: finite input_initial");
    cudaStreamSynchronize(ctx->stream);
    for (int d = 0; d < 2; ++d) {
        K.kind[d] = kinds[d];
        K.nbi[d] = nbs[d];
        K.offi[d] = kinds[d] == 1 ? std::log2(mins[d] + scs[d]) : mins[d];
        K.frqi[d] = frqs[d];
        K.sci[d] = scs[d];
    }
    for (int t = 0; t < kMaxTerms; ++t) {
        K.pw[t][0] = t < num_terms ? (signed char)powers[2 * t] : 0;
        K.pw[t][1] = t < num_terms ? (signed char)powers[2 * t + 1] : 0;
    }
    NW_CHECK(dev_alloc(ctx, K.input, (size_t)ctx->precision * std::max<int64_t>(K.m, 1)));
    std::vector<double> init(std::max<int64_t>(K.m, 1), input_initial);
    NW_CHECK(upload_convert(ctx, K.input.ptr, real_dtype(ctx), init.data(), NW_DTYPE_F64, K.m));
    K.ninp = 2;
    graphs_clear(ctx);
    return NW_OK;
}

int nw_kinetic_register(nw_ctx* ctx, int64_t num_instances, const int64_t* segment,
                        const double* g_coef, int num_states, int num_open, const int32_t* open_states,
                        double erev, const double* table, int num_buckets, int num_terms,
                        double vmin, double bucket_frq, double conserve_sum, const double* init_state) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    NW_CHECK(nw_kinetic_clear(ctx));
    return kinetic_add(ctx, "nw_kinetic_register", num_instances, segment, g_coef, num_states, num_open,
                       open_states, erev, -1, table, num_buckets, num_terms, vmin, bucket_frq, conserve_sum,
                       init_state, nullptr);
}

int nw_synapses_set(nw_ctx* ctx, int64_t num_synapses, const int64_t* pre_neuron, const int64_t* post_segment,
                    const double* w_ampa, const double* w_nmda, const int32_t* delay_steps,
                    const double* ampa_on, const double* ampa_off, const double* nmda_on, const double* nmda_off,
                    int32_t pulse_steps, double e_syn, double mg) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_synapses_set before nw_model_init");
    const int64_t m = num_synapses;
    if (m < 0 || (m && (!pre_neuron || !post_segment || !w_ampa || !w_nmda || !delay_steps ||
                        !ampa_on || !ampa_off || !nmda_on || !nmda_off)))
        return fail(ctx, NW_ERR_ARG, "nw_synapses_set: null arrays");
    if (m > 0 && (pulse_steps < 1 || !(mg >= 0.0) || !std::isfinite(e_syn)))
        return fail(ctx, NW_ERR_ARG, "nw_synapses_set: pulse_steps >= 1, mg >= 0, finite e_syn");
    // Presynaptic neurons index the spike ring: this model's neurons, or all
    // ranks' neurons when the network is partitioned ("spike_neurons").
    const int64_t ring_neurons = ctx->spike_neurons > 0 ? ctx->spike_neurons : ctx->n_neuron;
    if (ctx->spike_offset < 0 || ctx->spike_offset + ctx->n_neuron > ring_neurons)
        return fail(ctx, NW_ERR_ARG, "nw_synapses_set: spike_neuron_offset + neurons exceeds spike_neurons");
    int dmin = INT32_MAX, dmax = 0;
    for (int64_t k = 0; k < m; ++k) {
        if (pre_neuron[k] < 0 || pre_neuron[k] >= ring_neurons)
            return fail(ctx, NW_ERR_ARG, "nw_synapses_set: presynaptic neuron out of range");
        if (delay_steps[k] < 1 || delay_steps[k] > (1 << 20))
            return fail(ctx, NW_ERR_ARG, "nw_synapses_set: delay must be in [1, 2^20] steps");
        if (!(w_ampa[k] >= 0.0) || !(w_nmda[k] >= 0.0))
            return fail(ctx, NW_ERR_ARG, "nw_synapses_set: weights must be >= 0");
        dmin = std::min(dmin, (int)delay_steps[k]);
        dmax = std::max(dmax, (int)delay_steps[k]);
    }
    InstanceLayout L;
    NW_CHECK(layout_instances(ctx, m, post_segment, "nw_synapses_set", L));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    SynState& Y = ctx->syn;
    free_syn(Y);
    if (m == 0) return NW_OK;
    Y.n = m;
    Y.min_delay = dmin; Y.max_delay = dmax; Y.pulse_steps = pulse_steps;
    Y.e_syn = e_syn; Y.mg = mg;
    // A spike of step t is read up to max_delay steps later while its owner may
    // already have written min_delay (the most steps one launch fuses) newer ones.
    int R = 32;
    while (R < dmax + dmin + 1 || R < ctx->spike_ring_min) R *= 2;
    Y.ring_steps = R;
    Y.ring_words = R / 32;
    Y.ring_neurons = ring_neurons;
    Y.neuron_offset = ctx->spike_offset;
    Y.user_to_sorted = L.user_to_sorted;
    Y.h_neuron_ptr = L.nptr;
    NW_CHECK(upload_layout(ctx, L, Y.seg, Y.seg_ptr, Y.neuron_ptr));
    const size_t rs = (size_t)ctx->precision;
    std::vector<int32_t> pre(m), dl(m), pe(m, 0), last(m, -1);
    std::vector<double> wa(m), wn(m), zero(m, 0.0);
    for (int64_t s = 0; s < m; ++s) {
        const int64_t u = L.order[s];
        pre[s] = (int32_t)pre_neuron[u]; dl[s] = delay_steps[u];
        wa[s] = w_ampa[u]; wn[s] = w_nmda[u];
    }
    for (DevBuf* b : {&Y.pre, &Y.delay, &Y.pulse_end, &Y.last_event, &Y.events}) NW_CHECK(dev_alloc(ctx, *b, 4 * m));
    for (DevBuf* b : {&Y.wa, &Y.wn, &Y.oa, &Y.on, &Y.od}) NW_CHECK(dev_alloc(ctx, *b, rs * m));
    NW_CHECK(dev_alloc(ctx, Y.mats, rs * 26));
    NW_CHECK(dev_alloc(ctx, Y.ring, 4 * (size_t)Y.ring_words * ring_neurons));
    NW_CHECK(upload_convert(ctx, Y.pre.ptr, NW_DTYPE_I32, pre.data(), NW_DTYPE_I32, m));
    NW_CHECK(upload_convert(ctx, Y.delay.ptr, NW_DTYPE_I32, dl.data(), NW_DTYPE_I32, m));
    NW_CHECK(upload_convert(ctx, Y.pulse_end.ptr, NW_DTYPE_I32, pe.data(), NW_DTYPE_I32, m));
    NW_CHECK(upload_convert(ctx, Y.last_event.ptr, NW_DTYPE_I32, last.data(), NW_DTYPE_I32, m));
    NW_CUDA(ctx, cudaMemsetAsync(Y.events.ptr, 0, 4 * m, ctx->stream));
    const int rd = real_dtype(ctx);
    NW_CHECK(upload_convert(ctx, Y.wa.ptr, rd, wa.data(), NW_DTYPE_F64, m));
    NW_CHECK(upload_convert(ctx, Y.wn.ptr, rd, wn.data(), NW_DTYPE_F64, m));
    for (DevBuf* b : {&Y.oa, &Y.on, &Y.od}) NW_CHECK(upload_convert(ctx, b->ptr, rd, zero.data(), NW_DTYPE_F64, m));
    std::vector<double> mats(26);
    std::copy(ampa_on, ampa_on + 4, mats.begin());
    std::copy(ampa_off, ampa_off + 4, mats.begin() + 4);
    std::copy(nmda_on, nmda_on + 9, mats.begin() + 8);
    std::copy(nmda_off, nmda_off + 9, mats.begin() + 17);
    NW_CHECK(upload_convert(ctx, Y.mats.ptr, rd, mats.data(), NW_DTYPE_F64, 26));
    NW_CHECK(synapse_ring_clear(ctx));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NW_OK;
}

int nw_clamps_set(nw_ctx* ctx, int64_t count, const int64_t* segment, const double* amps,
                  const int64_t* first_tick, const int64_t* num_ticks) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_clamps_set before nw_model_init");
    if (count < 0 || (count && (!segment || !amps || !first_tick || !num_ticks)))
        return fail(ctx, NW_ERR_ARG, "nw_clamps_set: null arrays");
    std::vector<int64_t> nb(count);
    std::vector<int32_t> per(ctx->n_neuron + 1, 0);
    for (int64_t c = 0; c < count; ++c) {
        if (segment[c] < 0 || segment[c] >= ctx->n_seg || num_ticks[c] < 0)
            return fail(ctx, NW_ERR_ARG, "nw_clamps_set: bad clamp " + std::to_string(c));
        nb[c] = neuron_of(ctx, segment[c]);
        if (++per[nb[c] + 1] > kMaxClampsPerNeuron)
            return fail(ctx, NW_ERR_LIMIT, "nw_clamps_set: more than " + std::to_string(kMaxClampsPerNeuron) +
                                           " clamps on one neuron");
    }
    for (int64_t k = 0; k < ctx->n_neuron; ++k) per[k + 1] += per[k];
    std::vector<int64_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    // By segment (segments are neuron-contiguous, so also by neuron).
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return segment[a] < segment[b]; });
    std::vector<uint32_t> seg(count), seg_ptr(ctx->n_seg + 1, 0);
    for (int64_t c = 0; c < count; ++c) seg_ptr[segment[c] + 1]++;
    for (int64_t i = 0; i < ctx->n_seg; ++i) seg_ptr[i + 1] += seg_ptr[i];
    std::vector<double> amp(count);
    std::vector<int64_t> first(count), cnt(count);
    ctx->clamp_user_to_sorted.assign(count, 0);
    for (int64_t s = 0; s < count; ++s) {
        int64_t u = order[s];
        ctx->clamp_user_to_sorted[u] = s;
        seg[s] = (uint32_t)segment[u]; amp[s] = amps[u]; first[s] = first_tick[u]; cnt[s] = num_ticks[u];
    }
    size_t n1 = (size_t)std::max<int64_t>(count, 1);
    NW_CHECK(dev_alloc(ctx, ctx->clamp_seg, 4 * n1));
    NW_CHECK(dev_alloc(ctx, ctx->clamp_amp, (size_t)ctx->precision * n1));
    NW_CHECK(dev_alloc(ctx, ctx->clamp_amp_stage, 16 * n1));
    NW_CHECK(dev_alloc(ctx, ctx->clamp_first, 8 * n1));
    NW_CHECK(dev_alloc(ctx, ctx->clamp_count, 8 * n1));
    NW_CHECK(dev_alloc(ctx, ctx->clamp_neuron_ptr, 4 * (ctx->n_neuron + 1)));
    NW_CHECK(dev_alloc(ctx, ctx->clamp_seg_ptr, 4 * (ctx->n_seg + 1)));
    NW_CHECK(upload_convert(ctx, ctx->clamp_seg_ptr.ptr, NW_DTYPE_U32, seg_ptr.data(), NW_DTYPE_U32, ctx->n_seg + 1));
    NW_CHECK(upload_convert(ctx, ctx->clamp_seg.ptr, NW_DTYPE_U32, seg.data(), NW_DTYPE_U32, count));
    NW_CHECK(upload_convert(ctx, ctx->clamp_amp.ptr, real_dtype(ctx), amp.data(), NW_DTYPE_F64, count));
    NW_CHECK(upload_convert(ctx, ctx->clamp_first.ptr, NW_DTYPE_I64, first.data(), NW_DTYPE_I64, count));
    NW_CHECK(upload_convert(ctx, ctx->clamp_count.ptr, NW_DTYPE_I64, cnt.data(), NW_DTYPE_I64, count));
    NW_CHECK(upload_convert(ctx, ctx->clamp_neuron_ptr.ptr, NW_DTYPE_I32, per.data(), NW_DTYPE_I32, ctx->n_neuron + 1));
    // Second half of the staging buffer: sorted position -> user index, used by
    // nw_advance_host to scatter user-order amplitudes.
    NW_CHECK(upload_convert(ctx, (char*)ctx->clamp_amp_stage.ptr + 8 * n1, NW_DTYPE_I64, order.data(),
                            NW_DTYPE_I64, count));
    ctx->n_clamps = count;
    return NW_OK;
}

int nw_detectors_set(nw_ctx* ctx, const int64_t* segment, const double* threshold_mV) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx || !segment || !threshold_mV) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_detectors_set before nw_model_init");
    int64_t nn = ctx->n_neuron;
    std::vector<uint32_t> seg(nn);
    for (int64_t k = 0; k < nn; ++k) {
        if (segment[k] < ctx->h_neuron_start[k] || segment[k] >= ctx->h_neuron_start[k + 1])
            return fail(ctx, NW_ERR_ARG, "nw_detectors_set: detector of neuron " + std::to_string(k) +
                                         " is not one of its segments");
        seg[k] = (uint32_t)segment[k];
    }
    NW_CHECK(dev_alloc(ctx, ctx->det_seg, 4 * nn));
    NW_CHECK(dev_alloc(ctx, ctx->det_thr, (size_t)ctx->precision * nn));
    NW_CHECK(dev_alloc(ctx, ctx->ap_detected, nn));
    NW_CHECK(dev_alloc(ctx, ctx->ap_state, nn));
    NW_CHECK(dev_alloc(ctx, ctx->spike_count, 4 * nn));
    NW_CHECK(upload_convert(ctx, ctx->det_seg.ptr, NW_DTYPE_U32, seg.data(), NW_DTYPE_U32, nn));
    NW_CHECK(upload_convert(ctx, ctx->det_thr.ptr, real_dtype(ctx), threshold_mV, NW_DTYPE_F64, nn));
    NW_CUDA(ctx, cudaMemsetAsync(ctx->ap_detected.ptr, 0, nn, ctx->stream));
    NW_CUDA(ctx, cudaMemsetAsync(ctx->ap_state.ptr, 0, nn, ctx->stream));
    NW_CUDA(ctx, cudaMemsetAsync(ctx->spike_count.ptr, 0, 4 * nn, ctx->stream));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->have_detectors = true;
    return NW_OK;
}

int nw_probes_set(nw_ctx* ctx, int64_t count, const int64_t* segment, int64_t max_steps) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_probes_set before nw_model_init");
    if (count < 0 || max_steps < 0 || (count && !segment)) return fail(ctx, NW_ERR_ARG, "nw_probes_set: bad arguments");
    std::vector<int64_t> nb(count);
    std::vector<int32_t> per(ctx->n_neuron + 1, 0);
    for (int64_t p = 0; p < count; ++p) {
        if (segment[p] < 0 || segment[p] >= ctx->n_seg) return fail(ctx, NW_ERR_ARG, "nw_probes_set: bad segment");
        nb[p] = neuron_of(ctx, segment[p]);
        if (++per[nb[p] + 1] > kMaxProbesPerNeuron)
            return fail(ctx, NW_ERR_LIMIT, "nw_probes_set: more than " + std::to_string(kMaxProbesPerNeuron) +
                                           " probes on one neuron");
    }
    for (int64_t k = 0; k < ctx->n_neuron; ++k) per[k + 1] += per[k];
    std::vector<int64_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return nb[a] < nb[b]; });
    std::vector<uint32_t> seg(count), slot(count);
    for (int64_t s = 0; s < count; ++s) { seg[s] = (uint32_t)segment[order[s]]; slot[s] = (uint32_t)order[s]; }
    size_t n1 = (size_t)std::max<int64_t>(count, 1);
    NW_CHECK(dev_alloc(ctx, ctx->probe_seg, 4 * n1));
    NW_CHECK(dev_alloc(ctx, ctx->probe_slot, 4 * n1));
    NW_CHECK(dev_alloc(ctx, ctx->probe_neuron_ptr, 4 * (ctx->n_neuron + 1)));
    NW_CHECK(dev_alloc(ctx, ctx->trace, (size_t)ctx->precision * n1 * (size_t)std::max<int64_t>(max_steps, 1)));
    NW_CHECK(upload_convert(ctx, ctx->probe_seg.ptr, NW_DTYPE_U32, seg.data(), NW_DTYPE_U32, count));
    NW_CHECK(upload_convert(ctx, ctx->probe_slot.ptr, NW_DTYPE_U32, slot.data(), NW_DTYPE_U32, count));
    NW_CHECK(upload_convert(ctx, ctx->probe_neuron_ptr.ptr, NW_DTYPE_I32, per.data(), NW_DTYPE_I32, ctx->n_neuron + 1));
    ctx->n_probes = count;
    ctx->probe_cap = max_steps;
    ctx->probe_len = 0;
    return NW_OK;
}

int nw_probes_read(nw_ctx* ctx, void* host, int dtype, int64_t max_rows, int64_t* steps_out) {
    if (!ctx) return NW_ERR_ARG;
    int64_t rows = std::min(max_rows, ctx->probe_len);
    if (steps_out) *steps_out = ctx->probe_len;
    if (!host || rows <= 0 || ctx->n_probes == 0) return NW_OK;
    return download_convert(ctx, host, dtype, ctx->trace.ptr, real_dtype(ctx), rows * ctx->n_probes);
}

static int check_ready(nw_ctx* ctx, int k_steps) {
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_advance before nw_model_init");
    if (!ctx->have_cap) return fail(ctx, NW_ERR_STATE, "nw_advance: Segment.capacitance not set");
    if (!ctx->prop_valid) return fail(ctx, NW_ERR_STATE, "nw_advance: no valid propagator (build or install one)");
    if (k_steps < 0) return fail(ctx, NW_ERR_ARG, "nw_advance: negative step count");
    if (ctx->n_probes && ctx->probe_len + k_steps > ctx->probe_cap)
        return fail(ctx, NW_ERR_LIMIT, "nw_advance: probe buffer full (" + std::to_string(ctx->probe_cap) + " steps)");
    return NW_OK;
}

static int read_status(nw_ctx* ctx) {
    int st = 0;
    NW_CUDA(ctx, cudaMemcpyAsync(&st, ctx->status.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (st & kStatusWaitTimeout) {
        cudaMemsetAsync(ctx->status.ptr, 0, 4, ctx->stream);
        return fail(ctx, NW_ERR_CUDA, "batched step: a bulk copy did not complete within the wait limit");
    }
    if (st & kStatusNonFinite) {
        cudaMemsetAsync(ctx->status.ptr, 0, 4, ctx->stream);
        return fail(ctx, NW_ERR_NUMERIC, "a segment voltage became non-finite");
    }
    return NW_OK;
}

int nw_advance(nw_ctx* ctx, int32_t k_steps, int path) {
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    NW_CHECK(check_ready(ctx, k_steps));
    if (k_steps == 0) return NW_OK;
    if (path != NW_PATH_BATCHED) ctx->gc_valid = false;   // these paths do not fill the cache
    if (path == NW_PATH_BATCHED) NW_CHECK(advance_batched(ctx, k_steps));
    else if (path == NW_PATH_PLAIN) NW_CHECK(advance_plain(ctx, k_steps));
    else if (path == NW_PATH_WIDE) NW_CHECK(advance_wide(ctx, k_steps));
    else return fail(ctx, NW_ERR_ARG, "nw_advance: unknown path");
    return read_status(ctx);
}

int nw_advance_host(nw_ctx* ctx, int32_t k_steps, const double* stim_amps, void* v_out, int v_dtype) {
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    NW_CHECK(check_ready(ctx, k_steps));
    if (stim_amps && ctx->n_clamps) {
        // Staging buffer: [user-order amplitudes (f64) | sorted -> user map (i64)].
        size_t half = ctx->clamp_amp_stage.bytes / 2;
        const int64_t* s2u = (const int64_t*)((char*)ctx->clamp_amp_stage.ptr + half);
        NW_CUDA(ctx, cudaMemcpyAsync(ctx->clamp_amp_stage.ptr, stim_amps, 8 * ctx->n_clamps,
                                     cudaMemcpyHostToDevice, ctx->stream));
        int threads = 256;
        int64_t blocks = (ctx->n_clamps + threads - 1) / threads;
        if (ctx->precision == NW_F64)
            stage_clamp_amps<double><<<blocks, threads, 0, ctx->stream>>>(
                ctx->clamp_amp_stage.as<double>(), s2u, ctx->clamp_amp.as<double>(), ctx->n_clamps);
        else
            stage_clamp_amps<float><<<blocks, threads, 0, ctx->stream>>>(
                ctx->clamp_amp_stage.as<double>(), s2u, ctx->clamp_amp.as<float>(), ctx->n_clamps);
        NW_CUDA(ctx, cudaGetLastError());
    }
    if (k_steps) NW_CHECK(advance_batched(ctx, k_steps));
    if (v_out) {
        int rd = real_dtype(ctx);
        if (v_dtype == rd) {
            NW_CUDA(ctx, cudaMemcpyAsync(v_out, ctx->V.ptr, (size_t)ctx->precision * ctx->n_seg,
                                         cudaMemcpyDeviceToHost, ctx->stream));
        } else {
            NW_CHECK(download_convert(ctx, v_out, v_dtype, ctx->V.ptr, rd, ctx->n_seg));
        }
    }
    return read_status(ctx);
}

int nw_advance_host_async(nw_ctx* ctx, int32_t k_steps, const double* stim_amps, void* v_out, int v_dtype) {
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (v_out && v_dtype != real_dtype(ctx))
        return fail(ctx, NW_ERR_ARG, "nw_advance_host_async: v_dtype must be the context precision");
    NW_CHECK(check_ready(ctx, k_steps));
    if (stim_amps && ctx->n_clamps) {
        size_t half = ctx->clamp_amp_stage.bytes / 2;
        const int64_t* s2u = (const int64_t*)((char*)ctx->clamp_amp_stage.ptr + half);
        NW_CUDA(ctx, cudaMemcpyAsync(ctx->clamp_amp_stage.ptr, stim_amps, 8 * ctx->n_clamps,
                                     cudaMemcpyHostToDevice, ctx->stream));
        int threads = 256;
        int64_t blocks = (ctx->n_clamps + threads - 1) / threads;
        if (ctx->precision == NW_F64)
            stage_clamp_amps<double><<<blocks, threads, 0, ctx->stream>>>(
                ctx->clamp_amp_stage.as<double>(), s2u, ctx->clamp_amp.as<double>(), ctx->n_clamps);
        else
            stage_clamp_amps<float><<<blocks, threads, 0, ctx->stream>>>(
                ctx->clamp_amp_stage.as<double>(), s2u, ctx->clamp_amp.as<float>(), ctx->n_clamps);
        NW_CUDA(ctx, cudaGetLastError());
    }
    if (k_steps) NW_CHECK(advance_batched(ctx, k_steps));
    if (v_out) {
        if (!ctx->copy_stream) {
            NW_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
            for (int k = 0; k < 2; ++k) {
                NW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->stage_ready[k], cudaEventDisableTiming));
                NW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->stage_done[k], cudaEventDisableTiming));
            }
        }
        const size_t bytes = (size_t)ctx->precision * ctx->n_seg;
        const int b = ctx->stage_slot;
        ctx->stage_slot ^= 1;
        // The slot's previous copy to the host must be done before it is overwritten.
        if (ctx->stage_pending[b]) NW_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->stage_done[b], 0));
        NW_CHECK(dev_alloc(ctx, ctx->vstage[b], bytes));
        NW_CUDA(ctx, cudaMemcpyAsync(ctx->vstage[b].ptr, ctx->V.ptr, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        NW_CUDA(ctx, cudaEventRecord(ctx->stage_ready[b], ctx->stream));
        NW_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->stage_ready[b], 0));
        NW_CUDA(ctx, cudaMemcpyAsync(v_out, ctx->vstage[b].ptr, bytes, cudaMemcpyDeviceToHost, ctx->copy_stream));
        NW_CUDA(ctx, cudaEventRecord(ctx->stage_done[b], ctx->copy_stream));
        ctx->stage_pending[b] = true;
    }
    return NW_OK;
}

int nw_get_clock(nw_ctx* ctx, int64_t* steps, int64_t* input_ticks) {
    if (!ctx) return NW_ERR_ARG;
    if (steps) *steps = ctx->steps;
    if (input_ticks) *input_ticks = ctx->input_ticks;
    return NW_OK;
}

int nw_set_tuning(nw_ctx* ctx, int lanes_per_row, int threads, int ctas_per_sm) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    if (lanes_per_row != 0 && lanes_per_row != 4 && lanes_per_row != 8 && lanes_per_row != 16 && lanes_per_row != 32)
        return fail(ctx, NW_ERR_ARG, "lanes_per_row must be 0, 4, 8, 16 or 32");
    if (threads < 128 || threads > 1024 || threads % 32)
        return fail(ctx, NW_ERR_ARG, "threads must be a multiple of 32 in [128, 1024]");
    if (ctas_per_sm < 0 || ctas_per_sm > 32) return fail(ctx, NW_ERR_ARG, "ctas_per_sm out of range");
    ctx->lanes_per_row = lanes_per_row;
    ctx->threads = threads;
    ctx->ctas_per_sm = ctas_per_sm;
    return NW_OK;
}

int nw_set_option(nw_ctx* ctx, const char* name, int64_t value) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx || !name) return NW_ERR_ARG;
    std::string nm(name);
    if (nm == "bulk_pipeline") { ctx->use_bulk = value != 0; return NW_OK; }
    if (nm == "cuda_graph") { ctx->use_graph = value != 0; return NW_OK; }
    if (nm == "spike_neurons" || nm == "spike_neuron_offset" || nm == "spike_ring_steps") {
        // Partitioned networks: taken by the next nw_synapses_set.
        if (value < 0 || value > INT32_MAX) return fail(ctx, NW_ERR_ARG, nm + " out of range");
        if (nm == "spike_neurons") ctx->spike_neurons = value;
        else if (nm == "spike_neuron_offset") ctx->spike_offset = value;
        else ctx->spike_ring_min = (int)value;
        return NW_OK;
    }
    if (nm == "pair_shared_limit") {
        // Largest neuron whose pair sums stay in shared memory (-1: as many as fit);
        // larger ones use global memory.  The integer sums are the same either way.
        if (value < -1 || value > INT32_MAX) return fail(ctx, NW_ERR_ARG, "pair_shared_limit out of range");
        ctx->pair_shared_limit = (int)value;
        return NW_OK;
    }
    if (nm == "duplicates") {
        // 0: every instance on a segment counts; 1: the reference's fancy-index "+="
        // for nonspecific conductances (only the last-registered instance of a
        // segment counts, per mechanism kind).
        if (value < 0 || value > 1) return fail(ctx, NW_ERR_ARG, "duplicates must be 0 or 1");
        ctx->duplicates = (int)value;
        return NW_OK;
    }
    if (nm == "propagator_lump") {
        // Taken by the next propagator build: a value below the tolerance is added to
        // the nearest kept entry on the tree path towards the row's segment instead
        // of being dropped (row sums unchanged; pair format unavailable).
        ctx->prop_lump = value != 0;
        return NW_OK;
    }
    if (nm == "propagator_format") {
        // 0: rows (every P_ij stored in its row); 1: pairs (each coupling once,
        // applied to both rows through detailed balance; built propagators only);
        // 2: quads; 3: windows of 8, 4, 2 or 1 columns (rows sorted by column).
        if (value < 0 || value > 3) return fail(ctx, NW_ERR_ARG, "propagator_format must be 0, 1, 2 or 3");
        if (value == 1 && !ctx->prop_built)
            return fail(ctx, NW_ERR_STATE, "pair format needs a propagator built by nw_propagator_build");
        ctx->prop_format = (int)value;
        return NW_OK;
    }
    if (nm == "wide_fusion") { ctx->wide_fusion = value != 0; return NW_OK; }
    if (nm == "adjoint_overlap") { ctx->adjoint_overlap = value != 0; return NW_OK; }
    if (nm == "propagator_single_walk") { ctx->prop_walk_once = value != 0; return NW_OK; }
    if (nm == "rows_claimed") { ctx->rows_claimed = value != 0; return NW_OK; }
    if (nm == "propagator_pool_chunks") {
        if (value < 0) return fail(ctx, NW_ERR_ARG, "propagator_pool_chunks must be >= 0");
        ctx->prop_pool_chunks = value;
        return NW_OK;
    }
    if (nm == "lanes_split") {
        // Quad format: neurons whose mean quads per row are below this take half the
        // lanes per row of the kernel's choice (0: all neurons the same).
        if (value < 0 || value > 65535) return fail(ctx, NW_ERR_ARG, "lanes_split must be in [0, 65535]");
        ctx->lanes_split = value;
        return NW_OK;
    }
    if (nm == "fusion_depth") {
        if (value < 0 || value > (1 << 20)) return fail(ctx, NW_ERR_ARG, "fusion_depth must be in [0, 2^20]");
        ctx->fusion = (int)value;
        return NW_OK;
    }
    if (nm == "prepare_graph") {
        // Capture (without running) the graph a later nw_advance(value) will replay.
        if (value < 1 || value > INT32_MAX) return fail(ctx, NW_ERR_ARG, "prepare_graph: step count out of range");
        NW_CHECK(check_ready(ctx, (int32_t)value));
        if (!ctx->use_graph) return NW_OK;
        return prepare_graph(ctx, (int)value);
    }
    if (nm == "clear_graphs") {
        NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        graphs_clear(ctx);
        return NW_OK;
    }
    if (nm == "set_steps") {
        // Resume at a saved step: clock, input ticks (two per step) and
        // conductance validity; probes start empty.
        if (value < 0) return fail(ctx, NW_ERR_ARG, "set_steps: negative step");
        ctx->steps = value;
        ctx->input_ticks = 2 * value;
        ctx->g_valid = value > 0 && has_channel_mechanisms(ctx);
        ctx->probe_len = 0;
        return NW_OK;
    }
    if (nm == "reset_clock") {
        // Back to time 0: clock, conductance validity, detector state and probes.
        ctx->input_ticks = ctx->steps = 0;
        ctx->g_valid = false;
        ctx->probe_len = 0;
        if (ctx->have_detectors) {
            NW_CUDA(ctx, cudaMemsetAsync(ctx->ap_detected.ptr, 0, ctx->n_neuron, ctx->stream));
            NW_CUDA(ctx, cudaMemsetAsync(ctx->ap_state.ptr, 0, ctx->n_neuron, ctx->stream));
            NW_CUDA(ctx, cudaMemsetAsync(ctx->spike_count.ptr, 0, 4 * ctx->n_neuron, ctx->stream));
            NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        }
        NW_CHECK(synapse_ring_clear(ctx));
        return NW_OK;
    }
    return fail(ctx, NW_ERR_ARG, "nw_set_option: unknown option " + nm);
}

int nw_get_option(nw_ctx* ctx, const char* name, int64_t* value) {
    if (!ctx || !name || !value) return NW_ERR_ARG;
    std::string nm(name);
    if (nm == "bulk_pipeline") { *value = ctx->use_bulk ? 1 : 0; return NW_OK; }
    if (nm == "bulk_pipeline_active") { *value = uses_bulk_pipeline(ctx) ? 1 : 0; return NW_OK; }
    if (nm == "cuda_graph") { *value = ctx->use_graph ? 1 : 0; return NW_OK; }
    if (nm == "propagator_format") { *value = ctx->prop_format; return NW_OK; }
    if (nm == "propagator_lump") { *value = ctx->prop_lump ? 1 : 0; return NW_OK; }
    if (nm == "duplicates") { *value = ctx->duplicates; return NW_OK; }
    if (nm == "kinetic_mechanisms") { *value = ctx->n_kin; return NW_OK; }
    if (nm == "pair_entries") { *value = ctx->nnz_f; return NW_OK; }
    if (nm == "quads") { *value = ctx->nq; return NW_OK; }
    if (nm == "wide_quads") { *value = ctx->nwq; return NW_OK; }
    if (nm == "wide_entries") { *value = ctx->nnz_w; return NW_OK; }
    if (nm == "calcium_wide_entries") { *value = ctx->ca.on ? ctx->ca.nnz_w : 0; return NW_OK; }
    if (nm == "lanes_split") { *value = ctx->lanes_split; return NW_OK; }
    if (nm == "wide_fusion") { *value = ctx->wide_fusion ? 1 : 0; return NW_OK; }
    if (nm == "adjoint_overlap") { *value = ctx->adjoint_overlap ? 1 : 0; return NW_OK; }
    if (nm == "propagator_single_walk") { *value = ctx->prop_walk_once ? 1 : 0; return NW_OK; }
    if (nm == "propagator_walks") { *value = ctx->prop_walks; return NW_OK; }
    if (nm == "rows_claimed") { *value = ctx->rows_claimed ? 1 : 0; return NW_OK; }
    if (nm == "conductance_cache_valid") { *value = ctx->gc_valid ? 1 : 0; return NW_OK; }
    if (nm == "propagator_pool_chunks") { *value = ctx->prop_pool_chunks; return NW_OK; }
    if (nm == "narrow_neurons") {
        int64_t k = 0;
        if (ctx->q_ok && ctx->lanes_split > 0)
            for (float q : ctx->h_neuron_qpr) k += q < (float)ctx->lanes_split ? 1 : 0;
        *value = k;
        return NW_OK;
    }
    if (nm == "windows") { *value = ctx->nwin[0] + ctx->nwin[1] + ctx->nwin[2] + ctx->nwin[3]; return NW_OK; }
    if (nm == "windows_8") { *value = ctx->nwin[0]; return NW_OK; }
    if (nm == "windows_4") { *value = ctx->nwin[1]; return NW_OK; }
    if (nm == "windows_2") { *value = ctx->nwin[2]; return NW_OK; }
    if (nm == "windows_1") { *value = ctx->nwin[3]; return NW_OK; }
    if (nm == "fusion_depth") { *value = ctx->fusion; return NW_OK; }
    if (nm == "graphs_cached") { *value = (int64_t)ctx->graphs.size(); return NW_OK; }
    if (nm == "graph_captures") { *value = ctx->graph_captures; return NW_OK; }
    if (nm == "graph_replays") { *value = ctx->graph_replays; return NW_OK; }
    if (nm == "synapse_ring_words") { *value = ctx->syn.ring_words; return NW_OK; }
    if (nm == "spike_neurons") { *value = ctx->syn.n ? ctx->syn.ring_neurons : ctx->n_neuron; return NW_OK; }
    if (nm == "spike_neuron_offset") { *value = ctx->spike_offset; return NW_OK; }
    return fail(ctx, NW_ERR_ARG, "nw_get_option: unknown option " + nm);
}

int nw_adjoint_forward(nw_ctx* ctx, int64_t num_steps, int32_t checkpoint_every, const double* target,
                       double* loss_out) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    return adjoint_forward(ctx, num_steps, checkpoint_every, target, loss_out);
}

int nw_adjoint_backward(nw_ctx* ctx, double cytoplasmic_resistance, double* grad_gna, double* grad_gk,
                        double* grad_gl, double* grad_ra) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    return adjoint_backward(ctx, cytoplasmic_resistance, grad_gna, grad_gk, grad_gl, grad_ra);
}

int nw_autotune(nw_ctx* ctx, int32_t trial_steps, int32_t* lanes_per_row, int32_t* threads,
                int32_t* fusion_depth, double* ms_per_step) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    NW_CHECK(check_ready(ctx, 0));
    const int rc = autotune(ctx, trial_steps, lanes_per_row, threads, fusion_depth, ms_per_step);
    ctx->gc_valid = false;   // the trials advanced the model and then restored its state
    return rc;
}

int nw_get_tuning(nw_ctx* ctx, int* lanes_per_row, int* threads, int* ctas_per_sm) {
    if (!ctx) return NW_ERR_ARG;
    if (lanes_per_row) *lanes_per_row = ctx->lanes_per_row ? ctx->lanes_per_row : choose_lanes_per_row(ctx);
    if (threads) *threads = ctx->threads;
    if (ctas_per_sm) *ctas_per_sm = ctx->ctas_per_sm;
    return NW_OK;
}

}  // extern "C"
