// Autotuner of the batched step: lanes per propagator row, threads per CTA,
// the bulk-copy pipeline, and the step-fusion depth, each chosen by timing
// short runs on the model itself (state is saved before and restored after).
//
// The reference has no tuner: its GPU kernels launch with a fixed 32 threads
// per block (neuwon/database/compute.py:360-418) and its CPU kernels rely on
// numba's prange.  Here the row shape depends on the propagator's density and
// the fusion depth on launch overhead, so both are measured per model.
#include <algorithm>
#include <cstring>
#include <vector>

#include "nw_internal.cuh"

namespace nw {

namespace {

struct Saved {
    int64_t split;
    int lanes, threads, fusion, ctas;
    bool graph, bulk, g_valid;
    int64_t n_probes, input_ticks, steps, probe_len;
};

// Every device buffer a step writes (probes are switched off during trials).
std::vector<DevBuf*> stepped_buffers(nw_ctx* ctx) {
    std::vector<DevBuf*> v = {&ctx->V, &ctx->Vint, &ctx->hh.gm, &ctx->hh.gh, &ctx->hh.gn,
                              &ctx->ap_detected, &ctx->ap_state,
                              &ctx->spike_count, &ctx->status, &ctx->syn.oa, &ctx->syn.on,
                              &ctx->syn.od, &ctx->syn.pulse_end, &ctx->syn.events,
                              &ctx->syn.last_event, &ctx->syn.ring, &ctx->ca.c, &ctx->ca.dcdt,
                              &ctx->ca.state};
    for (int q = 0; q < ctx->n_kin; ++q) v.push_back(&ctx->kin[q].state);
    std::vector<DevBuf*> out;
    for (DevBuf* b : v)
        if (b->ptr && b->bytes) out.push_back(b);
    return out;
}

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
    ~Timer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

}  // namespace

int autotune(nw_ctx* ctx, int trial_steps, int32_t* lanes_out, int32_t* threads_out, int32_t* fusion_out,
             double* ms_out) {
    if (trial_steps < 1 || trial_steps > 10000) return fail(ctx, NW_ERR_ARG, "autotune: trial_steps in [1, 10000]");
    Saved sv{ctx->lanes_split, ctx->lanes_per_row, ctx->threads, ctx->fusion, ctx->ctas_per_sm, ctx->use_graph, ctx->use_bulk,
             ctx->g_valid, ctx->n_probes, ctx->input_ticks, ctx->steps, ctx->probe_len};

    // Snapshot of the stepped state.
    std::vector<DevBuf*> bufs = stepped_buffers(ctx);
    size_t total = 0;
    for (DevBuf* b : bufs) total += (b->bytes + 255) & ~(size_t)255;
    DevBuf store;
    NW_CHECK(dev_alloc(ctx, store, std::max<size_t>(total, 256)));
    auto copy_all = [&](bool save) -> int {
        size_t off = 0;
        for (DevBuf* b : bufs) {
            char* s = static_cast<char*>(store.ptr) + off;
            NW_CUDA(ctx, cudaMemcpyAsync(save ? s : b->ptr, save ? b->ptr : s, b->bytes,
                                         cudaMemcpyDeviceToDevice, ctx->stream));
            off += (b->bytes + 255) & ~(size_t)255;
        }
        return NW_OK;
    };
    auto restore_settings = [&]() {
        ctx->lanes_split = sv.split;
        ctx->lanes_per_row = sv.lanes; ctx->threads = sv.threads; ctx->fusion = sv.fusion;
        ctx->ctas_per_sm = sv.ctas; ctx->use_graph = sv.graph; ctx->use_bulk = sv.bulk;
        ctx->g_valid = sv.g_valid; ctx->n_probes = sv.n_probes; ctx->input_ticks = sv.input_ticks;
        ctx->steps = sv.steps; ctx->probe_len = sv.probe_len;
    };
    int rc = copy_all(true);
    if (rc != NW_OK) { dev_free(store); return rc; }

    Timer t;
    if (cudaEventCreate(&t.a) != cudaSuccess || cudaEventCreate(&t.b) != cudaSuccess) {
        dev_free(store);
        return fail(ctx, NW_ERR_CUDA, "autotune: cudaEventCreate failed");
    }
    ctx->n_probes = 0;          // trials record nothing
    ctx->use_graph = false;     // direct launches: the graph cache keeps the user's entries

    // One trial: a warm-up call, then `timed` steps in one call; ms per step.
    auto trial = [&](int warm, int timed, double* ms) -> int {
        NW_CHECK(advance_batched(ctx, warm));
        NW_CUDA(ctx, cudaEventRecord(t.a, ctx->stream));
        NW_CHECK(advance_batched(ctx, timed));
        NW_CUDA(ctx, cudaEventRecord(t.b, ctx->stream));
        NW_CUDA(ctx, cudaEventSynchronize(t.b));
        float el = 0.f;
        NW_CUDA(ctx, cudaEventElapsedTime(&el, t.a, t.b));
        *ms = (double)el / timed;
        return NW_OK;
    };

    struct Cand { int lanes, threads; bool bulk; double ms; };
    std::vector<Cand> cands;
    const int lane_opts[] = {4, 8, 16, 32};
    const int thread_opts[] = {512, 768, 1024};
    for (int th : thread_opts)
        for (int l : lane_opts) cands.push_back({l, th, false, 0.0});
    if (ctx->precision == NW_F32) cands.push_back({0, 1024, true, 0.0});

    // Phase 1: row shape at one launch per trial.
    int best = -1;
    ctx->fusion = trial_steps;
    ctx->lanes_split = 0;
    for (size_t i = 0; i < cands.size(); ++i) {
        ctx->lanes_per_row = cands[i].lanes;
        ctx->threads = cands[i].threads;
        ctx->use_bulk = cands[i].bulk;
        if (cands[i].bulk && !uses_bulk_pipeline(ctx)) { cands[i].ms = -1; continue; }
        double ms = 0;
        rc = trial(1, trial_steps, &ms);
        if (rc == NW_ERR_LIMIT) { cands[i].ms = -1; rc = NW_OK; continue; }   // does not fit: skip
        if (rc != NW_OK) break;
        cands[i].ms = ms;
        if (best < 0 || ms < cands[best].ms) best = (int)i;
    }
    if (rc == NW_OK && best < 0) rc = fail(ctx, NW_ERR_LIMIT, "autotune: no launch shape fits this model");

    // Phase 1b (quad format, 8 or more lanes): the row length below which a neuron's
    // rows take half the lanes, from the spread of the neurons' mean quads per row.
    int64_t best_split = 0;
    double best_ms = best >= 0 ? cands[best].ms : 0.0;
    if (rc == NW_OK && ctx->prop_format == 2 && cands[best].lanes >= 8) {
        ctx->lanes_per_row = cands[best].lanes;
        ctx->threads = cands[best].threads;
        ctx->use_bulk = cands[best].bulk;
        const int64_t lanes = cands[best].lanes;
        const int64_t split_opts[] = {lanes, 2 * lanes, 3 * lanes, 4 * lanes, 6 * lanes};
        for (int64_t sp : split_opts) {
            ctx->lanes_split = sp;
            double ms = 0;
            rc = trial(1, trial_steps, &ms);
            if (rc != NW_OK) break;
            if (ms < best_ms * 0.995) { best_ms = ms; best_split = sp; }
        }
    }
    ctx->lanes_split = best_split;

    // Phase 2: fusion depth with that row shape, over the same step count.
    int best_f = trial_steps;
    if (rc == NW_OK) {
        ctx->lanes_per_row = cands[best].lanes;
        ctx->threads = cands[best].threads;
        ctx->use_bulk = cands[best].bulk;
        const int span = 4 * trial_steps;
        const int f_opts[] = {1, 2, 5, 10, 20, 25, 50, 100, 200, 500};
        std::vector<std::pair<int, double>> fr;
        for (int F : f_opts) {
            if (F > span) break;
            ctx->fusion = F;
            double ms_f = 0;
            rc = trial(std::min(F, span), span, &ms_f);
            if (rc != NW_OK) break;
            fr.push_back({F, ms_f});
        }
        if (rc == NW_OK && !fr.empty()) {
            // The deepest fusion within 1 % of the fastest: fewer launches per call.
            double mn = fr[0].second;
            for (auto& p : fr) mn = std::min(mn, p.second);
            for (auto& p : fr)
                if (p.second <= mn * 1.01) { best_f = p.first; best_ms = p.second; }
        }
    }

    // Restore the model state and clock, keep the chosen tuning.
    const int rc2 = copy_all(false);
    cudaStreamSynchronize(ctx->stream);
    dev_free(store);
    restore_settings();
    if (rc != NW_OK) return rc;
    if (rc2 != NW_OK) return rc2;
    ctx->lanes_per_row = cands[best].lanes;
    ctx->threads = cands[best].threads;
    ctx->use_bulk = cands[best].bulk;
    ctx->lanes_split = best_split;
    ctx->fusion = best_f;
    if (lanes_out) *lanes_out = cands[best].lanes;
    if (threads_out) *threads_out = cands[best].threads;
    if (fusion_out) *fusion_out = best_f;
    if (ms_out) *ms_out = best_ms;
    return NW_OK;
}

}  // namespace nw
