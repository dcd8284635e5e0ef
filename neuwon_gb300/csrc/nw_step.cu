// Time-step kernels of neuwon_gb300.
//
// One staggered step follows neuwon/rxd/rxd_model.py:63-80:
//   species(dt/2) -> mechanisms(dt) -> species(dt/2) -> AP detector
// where species(dt/2) (rxd_model.py:91-113) gathers every segment's
// conductance / driving voltage / current, applies the exact exponential
// membrane update of neuwon/rxd/neuron/electric.py:56-76 and multiplies by
// the propagator.
//
// Batched path: a persistent kernel.  Each CTA takes whole neurons from a
// work counter (largest first) and advances one neuron through all K steps
// before taking the next, so the only synchronisation is __syncthreads():
// the propagator is block-diagonal by neuron and nothing couples neurons.
// The vector the propagator multiplies lives in shared memory; propagator
// rows are streamed from HBM as (fp32 value, u16 neuron-relative column)
// in 16-byte vectors, LPR lanes per row, with a compensated sum of
//   V_i = x_i - leak_i * x_i + sum_{j != i} P_ij (x_j - x_i),
// which equals sum_j P_ij x_j exactly when leak_i = 1 - sum_j P_ij.  The
// default storage is the quad format: windows of 4 consecutive columns (one
// 16-byte value vector and a u16 base per window).  When every conductance
// source maps one-to-one onto segments (the FUSE instances), the mid-step
// mechanism update, the new conductance and the second half step's x are one
// pass, and the conductances are cached for the next step's first half.
//
// Plain path: the reference's GPU design (neuwon/database/compute.py:360-418):
// per-neuron launches, one thread per row or per instance, 32 threads per
// block, FP64 CSR with the diagonal.
#include <algorithm>
#include <type_traits>

#include "nw_step_batched.cuh"

namespace nw {
// ------------------------------------------------------------ plain path

template <typename real>
__global__ void plain_prepare_kernel(const StepArgs<real> a, int j, int64_t base, int n, int64_t tick,
                                     int gv, int last) {
    int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n) return;
    int64_t i = base + li;
    real G, GE;
    if (gv) segment_conductance(a, i, G, GE);
    else { G = real(0); GE = real(0); }
    real I = a.has_nonspec ? a.Inonspec[i] : real(0);
    if (a.clamp_neuron_ptr) {
        for (int c = a.clamp_neuron_ptr[j]; c < a.clamp_neuron_ptr[j + 1]; ++c)
            if (a.clamp_seg[c] == (uint32_t)i && tick >= a.clamp_first[c] && tick < a.clamp_first[c] + a.clamp_count[c])
                I += a.clamp_amp[c];
    }
    a.px[i] = membrane_x(a, i, G, GE, I, last != 0);
}

template <typename real>
__global__ void plain_spmv_kernel(const StepArgs<real> a, int64_t base, int n) {
    int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n) return;
    int64_t r = base + li;
    double acc = 0.0;
    for (int64_t k = a.prow[r]; k < a.prow[r + 1]; ++k) acc += a.pval[k] * (double)a.px[a.pcol[k]];
    if (!isfinite(acc)) atomicOr(a.status, kStatusNonFinite);
    a.V[r] = (real)acc;
}

template <typename real>
__global__ void plain_hh_kernel(const StepArgs<real> a, int64_t ib, int64_t ie) {
    int64_t k = ib + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= ie) return;
    const real v = a.V[a.hh_identity ? k : (int64_t)a.hh_seg[k]];
    real m = a.gm[k], h = a.gh[k], nn = a.gn[k];
    hh_gates(v, a.dtq10, m, h, nn);
    a.gm[k] = m; a.gh[k] = h; a.gn[k] = nn;
}

template <typename real>
__global__ void plain_kinetic_kernel(const StepArgs<real> a, int q, int64_t kb, int64_t ke) {
    int64_t k = kb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= ke) return;
    const KinArgs<real>& K = a.kin[q];
    const real v = a.V[K.identity ? k : (int64_t)K.seg[k]];
    if (K.ninp == 2) kinetic_step_2d(K, k, v);
    else kinetic_step_generic(K, k, v);
}

template <typename real>
__global__ void plain_detect_kernel(const StepArgs<real> a, int64_t row) {
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j < a.n_neuron && a.has_det) {
        const bool over = a.V[a.det_seg[j]] >= a.det_thr[j];
        const bool det = over && !a.ap_state[j];
        a.ap_detected[j] = det;
        a.ap_state[j] = over;
        a.spike_count[j] += det ? 1u : 0u;
    }
    if (j < a.n_probes && a.n_probes) {
        // probe_seg/probe_slot are neuron-sorted; every probe is written once.
        a.trace[row * a.n_probes + a.probe_slot[j]] = a.V[a.probe_seg[j]];
    }
}

// ------------------------------------------------------------ host side

int choose_lanes_per_row(nw_ctx* ctx) {
    if (ctx->lanes_per_row) return ctx->lanes_per_row;
    int64_t nnz = (ctx->prop_format == 1 && ctx->f_ok) ? ctx->nnz_f : ctx->nnz_b;
    if (ctx->prop_format == 2 && ctx->q_ok) nnz = ctx->nq;   // quads per row: one per lane and load
    if (ctx->prop_format == 3 && ctx->win_ok)                // window items (halves of 8-wide windows)
        nnz = 2 * ctx->nwin[0] + ctx->nwin[1] + ctx->nwin[2] + ctx->nwin[3];
    double avg = ctx->n_seg ? (double)nnz / (double)ctx->n_seg : 0.0;
    if (avg >= 48) return 16;
    if (avg >= 20) return 8;
    return 4;
}

// The asynchronous bulk pipeline is used for FP32 state when it fits in shared
// memory next to the neuron's x vector; otherwise the register path.
static bool bulk_fits(nw_ctx* ctx) {
    const size_t xs_bytes = ((size_t)ctx->max_neuron * sizeof(float) + 127) & ~(size_t)127;
    const size_t ring = (size_t)(ctx->threads / 32) * kBulkStages * (BulkGeom<float>::kStageBytes + 8);
    return xs_bytes + ring + 4096 <= ctx->smem_optin;
}

bool uses_bulk_pipeline(nw_ctx* ctx) {
    return ctx->precision == NW_F32 && ctx->use_bulk && ctx->lanes_per_row == 0 && ctx->prop_format == 0 &&
           bulk_fits(ctx);
}

// k_steps steps as launches of ctx->fusion fused steps each, on the context's
// stream (also the body of a captured graph: no host synchronisation here).
// Steps per launch: the fusion depth, capped by the shortest axonal delay so that
// every spike a synapse reads was written by an earlier launch.
static int fusion_steps(nw_ctx* ctx, int k_steps) {
    int F = ctx->fusion > 0 ? ctx->fusion : k_steps;
    if (ctx->syn.n > 0) F = std::min(F, ctx->syn.min_delay);
    return std::max(F, 1);
}

template <typename real>
static int enqueue_batched(nw_ctx* ctx, const BatchedCfg<real>& c, const StepArgs<real>& a0, int k_steps) {
    const int F = fusion_steps(ctx, k_steps);
    for (int s_off = 0; s_off < k_steps; s_off += F) {
        StepArgs<real> a = a0;
        a.k_steps = std::min(F, k_steps - s_off);
        NW_CUDA(ctx, cudaMemsetAsync(ctx->work_counter.ptr, 0, sizeof(int), ctx->stream));
        c.kern<<<c.grid, c.threads, c.smem, ctx->stream>>>(a, c.xs_bytes, s_off);
        NW_CUDA(ctx, cudaGetLastError());
    }
    return NW_OK;
}

__global__ void set_clock_kernel(DevClock* d, DevClock v) { *d = v; }

static int push_clock(nw_ctx* ctx) {
    DevClock v;
    memset(&v, 0, sizeof(v));
    v.input_ticks = ctx->input_ticks;
    v.steps = ctx->steps;
    v.probe_len = ctx->probe_len;
    v.g_valid = ctx->g_valid ? 1 : 0;
    v.gc_valid = ctx->gc_valid ? 1 : 0;
    set_clock_kernel<<<1, 1, 0, ctx->stream>>>(ctx->dclock.as<DevClock>(), v);
    NW_CUDA(ctx, cudaGetLastError());
    return NW_OK;
}

void graphs_clear(nw_ctx* ctx) {
    for (auto& g : ctx->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        if (g.graph) cudaGraphDestroy(g.graph);
    }
    ctx->graphs.clear();
}

static void key_append(std::vector<unsigned char>& key, const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    key.insert(key.end(), b, b + n);
}

constexpr size_t kMaxGraphs = 8;

// Replays (capturing first if needed) the graph of k_steps batched steps.
// The key holds every byte that enters the captured launches, so an entry is
// reused exactly when the launches it recorded are the ones asked for.
template <typename real>
static int launch_graph(nw_ctx* ctx, const BatchedCfg<real>& c, const StepArgs<real>& a0, int k_steps,
                        bool launch = true) {
    std::vector<unsigned char> key;
    StepArgs<real> ka = a0;
    ka.tick0 = 0; ka.g_valid = 0; ka.trace_row0 = 0; ka.k_steps = 0;   // not read by the kernel
    key_append(key, &ka, sizeof(ka));
    key_append(key, &c, sizeof(c));
    key_append(key, &k_steps, sizeof(k_steps));
    const int F = fusion_steps(ctx, k_steps);
    key_append(key, &F, sizeof(F));
    key_append(key, &ctx->work_counter.ptr, sizeof(void*));
    for (auto& g : ctx->graphs) {
        if (g.key == key) {
            g.last_use = ++ctx->graph_uses;
            if (!launch) return NW_OK;
            NW_CUDA(ctx, cudaGraphLaunch(g.exec, ctx->stream));
            ctx->graph_replays++;
            return NW_OK;
        }
    }
    if (ctx->graphs.size() >= kMaxGraphs) {
        size_t lru = 0;
        for (size_t i = 1; i < ctx->graphs.size(); ++i)
            if (ctx->graphs[i].last_use < ctx->graphs[lru].last_use) lru = i;
        cudaGraphExecDestroy(ctx->graphs[lru].exec);
        cudaGraphDestroy(ctx->graphs[lru].graph);
        ctx->graphs.erase(ctx->graphs.begin() + lru);
    }
    GraphEntry e;
    e.key = std::move(key);
    NW_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_batched(ctx, c, a0, k_steps);
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &e.graph);
    if (rc != NW_OK) {
        if (e.graph) cudaGraphDestroy(e.graph);
        return rc;
    }
    NW_CUDA(ctx, ce);
    const cudaError_t ie = cudaGraphInstantiate(&e.exec, e.graph, 0);
    if (ie != cudaSuccess) {
        cudaGraphDestroy(e.graph);
        return cuda_fail(ctx, ie, "cudaGraphInstantiate");
    }
    e.last_use = ++ctx->graph_uses;
    ctx->graph_captures++;
    ctx->graphs.push_back(std::move(e));
    if (!launch) return NW_OK;
    NW_CUDA(ctx, cudaGraphLaunch(ctx->graphs.back().exec, ctx->stream));
    ctx->graph_replays++;
    return NW_OK;
}

template <typename real>
static int launch_batched(nw_ctx* ctx, int k_steps) {
    BatchedCfg<real> c;
    memset(&c, 0, sizeof(c));
    NW_CHECK(config_batched<real>(ctx, c));
    StepArgs<real> a = make_args<real>(ctx, k_steps);
    a.facc_cap = c.acc_cap;
    a.frc_smem = c.rc_smem;
    NW_CHECK(push_clock(ctx));
    if (ctx->use_graph) return launch_graph<real>(ctx, c, a, k_steps);
    return enqueue_batched<real>(ctx, c, a, k_steps);
}

template <typename real>
static int prepare_graph_t(nw_ctx* ctx, int k_steps) {
    BatchedCfg<real> c;
    memset(&c, 0, sizeof(c));
    NW_CHECK(config_batched<real>(ctx, c));
    StepArgs<real> a = make_args<real>(ctx, k_steps);
    a.facc_cap = c.acc_cap;
    a.frc_smem = c.rc_smem;
    return launch_graph<real>(ctx, c, a, k_steps, false);
}

int prepare_graph(nw_ctx* ctx, int k_steps) {
    return ctx->precision == NW_F64 ? prepare_graph_t<double>(ctx, k_steps) : prepare_graph_t<float>(ctx, k_steps);
}

static void finish_steps(nw_ctx* ctx, int k_steps) {
    ctx->input_ticks += 2 * (int64_t)k_steps;
    ctx->steps += k_steps;
    if (ctx->n_probes) ctx->probe_len += k_steps;
    if (has_channel_mechanisms(ctx)) ctx->g_valid = true;
}

int advance_batched(nw_ctx* ctx, int k_steps) {
    int rc = ctx->precision == NW_F64 ? launch_batched<double>(ctx, k_steps)
                                      : launch_batched<float>(ctx, k_steps);
    if (rc != NW_OK) {
        ctx->gc_valid = false;
        return rc;
    }
    finish_steps(ctx, k_steps);
    // The fused mechanism pass (compiled into the quad and windows kernels) ran and
    // left the cache filled from the state the next step starts from.
    if (k_steps > 0)
        ctx->gc_valid = (ctx->prop_format == 2 || ctx->prop_format == 3) && fuse_mechanisms(ctx);
    return NW_OK;
}

template <typename real>
static int plain_steps(nw_ctx* ctx, int k_steps) {
    constexpr int T = 32;   // compute.py:368: 32 threads per block
    for (int s = 0; s < k_steps; ++s) {
        StepArgs<real> a = make_args<real>(ctx, 1);
        for (int half = 0; half < 2; ++half) {
            const int64_t tick = ctx->input_ticks + half + 1;
            const int gv = (half > 0 || ctx->g_valid) ? 1 : 0;
            const int last = half == 1;
            for (int64_t j = 0; j < ctx->n_neuron; ++j) {
                int64_t base = ctx->h_neuron_start[j];
                int n = (int)(ctx->h_neuron_start[j + 1] - base);
                int blocks = (n + T - 1) / T;
                plain_prepare_kernel<real><<<blocks, T, 0, ctx->stream>>>(a, (int)j, base, n, tick, gv, last);
                plain_spmv_kernel<real><<<blocks, T, 0, ctx->stream>>>(a, base, n);
            }
            if (half == 0) {
                for (int64_t j = 0; j < ctx->n_neuron; ++j) {
                    if (ctx->hh.m > 0) {
                        const int64_t ib = ctx->hh.h_neuron_ptr[j], ie = ctx->hh.h_neuron_ptr[j + 1];
                        if (ie > ib)
                            plain_hh_kernel<real><<<(unsigned)((ie - ib + T - 1) / T), T, 0, ctx->stream>>>(a, ib, ie);
                    }
                    for (int q = 0; q < ctx->n_kin; ++q) {
                        const KineticState& K = ctx->kin[q];
                        if (K.m == 0) continue;
                        const int64_t kb = K.h_neuron_ptr[j], ke = K.h_neuron_ptr[j + 1];
                        if (ke > kb)
                            plain_kinetic_kernel<real><<<(unsigned)((ke - kb + T - 1) / T), T, 0, ctx->stream>>>(
                                a, q, kb, ke);
                    }
                }
            }
            ctx->g_valid = ctx->g_valid || has_channel_mechanisms(ctx);
        }
        int64_t cover = std::max<int64_t>(ctx->n_neuron, ctx->n_probes);
        StepArgs<real> d = make_args<real>(ctx, 1);
        plain_detect_kernel<real><<<(unsigned)((cover + 127) / 128), 128, 0, ctx->stream>>>(d, ctx->probe_len);
        NW_CUDA(ctx, cudaGetLastError());
        ctx->input_ticks += 2;
        ctx->steps += 1;
        if (ctx->n_probes) ctx->probe_len += 1;
    }
    return NW_OK;
}

int advance_plain(nw_ctx* ctx, int k_steps) {
    if (ctx->syn.n) return fail(ctx, NW_ERR_STATE, "the plain path has no synapses; use the batched path");
    if (ctx->ca.on) return fail(ctx, NW_ERR_STATE, "the plain path has no calcium; use the batched or wide path");
    return ctx->precision == NW_F64 ? plain_steps<double>(ctx, k_steps) : plain_steps<float>(ctx, k_steps);
}

}  // namespace nw
