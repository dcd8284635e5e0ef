// Intracellular calcium: the diffusing species of neuwon/rxd/species.py
// (_SpeciesInstance._advance, species.py:56-70: c <- max(0, c + dc/dt h), then
// c <- M c with M the diffusion propagator), with its propagator built like the
// electric one (the reference's _compute_matrix, species.py:74-83, is
// unfinished), plus the calcium pump and sodium-fraction influx as mechanisms.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "nw_internal.cuh"

namespace nw {

void free_calcium(CalciumState& c) {
    for (DevBuf* b : {&c.res, &c.vol, &c.p_rowptr, &c.p_col, &c.p_val, &c.b_rowptr, &c.b_col, &c.b_val, &c.b_leak,
                      &c.w_rowptr, &c.w_col, &c.w_val, &c.w_leak, &c.c, &c.dcdt, &c.scratch, &c.influx,
                      &c.efflux, &c.state, &c.table})
        dev_free(*b);
    c = CalciumState();
}

int calcium_ensure_wide(nw_ctx* ctx) {
    CalciumState& C = ctx->ca;
    if (C.w_ok) return NW_OK;
    NW_CHECK(csr_to_rows<int32_t>(ctx, C.p_rowptr, C.p_col, C.p_val, false, C.w_rowptr, C.w_col, C.w_val, C.w_leak,
                                  &C.nnz_w));
    NW_CHECK(dev_alloc(ctx, C.scratch, (size_t)ctx->precision * ctx->n_seg));
    C.w_ok = true;
    return NW_OK;
}

static int real_dtype_of(nw_ctx* ctx) { return ctx->precision == NW_F64 ? NW_DTYPE_F64 : NW_DTYPE_F32; }

}  // namespace nw

using namespace nw;

extern "C" {

int nw_calcium_set(nw_ctx* ctx, double diffusivity, const double* cross_area_um2, const double* length_um,
                   const double* volume_um3, double initial_mM, double prune_tolerance, int conserve,
                   int64_t* nnz_out) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "nw_calcium_set before nw_model_init");
    if (!cross_area_um2 || !length_um || !volume_um3) return fail(ctx, NW_ERR_ARG, "nw_calcium_set: null arrays");
    if (!(diffusivity > 0.0) || !(initial_mM >= 0.0) || !(prune_tolerance >= 0.0))
        return fail(ctx, NW_ERR_ARG, "nw_calcium_set: diffusivity > 0, initial >= 0, tolerance >= 0");
    const int64_t n = ctx->n_seg;
    // Diffusion between a segment and its parent through the segment's own cross
    // section over its own length (the electric builder's convention for the
    // axial resistance, electric.py:49-54): d c_i / dt = D A / (L vol_i) (c_p - c_i).
    // With "resistance" R' = 1e-3 L / (D A) and "capacity" vol, the builder's
    // coefficient h_s / (R' vol) equals h_ms D A / (L vol).
    std::vector<double> res(n), vol(n);
    for (int64_t i = 0; i < n; ++i) {
        if (!(volume_um3[i] > 0.0)) return fail(ctx, NW_ERR_ARG, "nw_calcium_set: volumes must be > 0");
        vol[i] = volume_um3[i];
        if (ctx->h_parent[i] < 0) { res[i] = 1.0; continue; }
        if (!(cross_area_um2[i] > 0.0) || !(length_um[i] > 0.0))
            return fail(ctx, NW_ERR_ARG, "nw_calcium_set: cross sections and lengths must be > 0");
        res[i] = 1e-3 * length_um[i] / (diffusivity * cross_area_um2[i]);
    }
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    graphs_clear(ctx);
    CalciumState& C = ctx->ca;
    free_calcium(C);
    C.D = diffusivity;
    C.c0 = initial_mM;
    const size_t rs = (size_t)ctx->precision;
    NW_CHECK(dev_alloc(ctx, C.res, 8 * n));
    NW_CHECK(dev_alloc(ctx, C.vol, 8 * n));
    NW_CHECK(upload_convert(ctx, C.res.ptr, NW_DTYPE_F64, res.data(), NW_DTYPE_F64, n));
    NW_CHECK(upload_convert(ctx, C.vol.ptr, NW_DTYPE_F64, vol.data(), NW_DTYPE_F64, n));
    int64_t nnz = 0;
    NW_CHECK(tree_propagator_build(ctx, C.res.as<double>(), C.vol.as<double>(), 0.5 * ctx->time_step * 1e-3,
                                   prune_tolerance, ctx->prop_lump ? 1 : 0, C.p_rowptr, C.p_col, C.p_val, &nnz));
    if (conserve) NW_CHECK(csr_conserve(ctx, C.p_rowptr, C.p_col, C.p_val));
    C.nnz64 = nnz;
    if (ctx->max_neuron <= 65535) {
        NW_CHECK(csr_to_rows<uint16_t>(ctx, C.p_rowptr, C.p_col, C.p_val, true, C.b_rowptr, C.b_col, C.b_val,
                                       C.b_leak, &C.nnz_b));
        C.b_ok = true;
    }
    std::vector<double> c0(n, initial_mM), zero(n, 0.0);
    for (DevBuf* b : {&C.c, &C.dcdt, &C.influx, &C.efflux}) NW_CHECK(dev_alloc(ctx, *b, rs * n));
    NW_CHECK(upload_convert(ctx, C.c.ptr, real_dtype_of(ctx), c0.data(), NW_DTYPE_F64, n));
    for (DevBuf* b : {&C.dcdt, &C.influx, &C.efflux})
        NW_CHECK(upload_convert(ctx, b->ptr, real_dtype_of(ctx), zero.data(), NW_DTYPE_F64, n));
    C.on = true;
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nnz_out) *nnz_out = nnz;
    return NW_OK;
}

int nw_calcium_pump_set(nw_ctx* ctx, const double* influx_coef, const double* efflux_coef, const double* table,
                        int32_t num_buckets, int32_t num_terms, double log2_min, double bucket_frq, double scale,
                        const double* initial_state) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    CalciumState& C = ctx->ca;
    if (!C.on) return fail(ctx, NW_ERR_STATE, "nw_calcium_pump_set before nw_calcium_set");
    if (!influx_coef || !efflux_coef) return fail(ctx, NW_ERR_ARG, "nw_calcium_pump_set: null arrays");
    const int64_t n = ctx->n_seg;
    const int rd = real_dtype_of(ctx);
    NW_CHECK(upload_convert(ctx, C.influx.ptr, rd, influx_coef, NW_DTYPE_F64, n));
    NW_CHECK(upload_convert(ctx, C.efflux.ptr, rd, efflux_coef, NW_DTYPE_F64, n));
    dev_free(C.state);
    dev_free(C.table);
    C.pump = false;
    if (table) {
        if (num_buckets < 1 || num_terms < 1 || num_terms > 4 || !(bucket_frq > 0.0) || !(scale > 0.0) ||
            !initial_state)
            return fail(ctx, NW_ERR_ARG, "nw_calcium_pump_set: bad table description");
        const size_t tn = (size_t)num_buckets * 9 * num_terms;
        NW_CHECK(dev_alloc(ctx, C.table, (size_t)ctx->precision * tn));
        NW_CHECK(upload_convert(ctx, C.table.ptr, rd, table, NW_DTYPE_F64, (int64_t)tn));
        std::vector<double> st((size_t)3 * n);
        for (int s = 0; s < 3; ++s) std::fill(st.begin() + (size_t)s * n, st.begin() + (size_t)(s + 1) * n, initial_state[s]);
        NW_CHECK(dev_alloc(ctx, C.state, (size_t)ctx->precision * 3 * n));
        NW_CHECK(upload_convert(ctx, C.state.ptr, rd, st.data(), NW_DTYPE_F64, 3 * n));
        C.nb = num_buckets; C.T = num_terms;
        C.log2_min = log2_min; C.frq = bucket_frq; C.scale = scale;
        C.pump = true;
    }
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NW_OK;
}

int nw_calcium_data(nw_ctx* ctx, const char* name, void* host, int dtype, int64_t count, int write) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx || !name || (!host && count)) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    CalciumState& C = ctx->ca;
    if (!C.on) return fail(ctx, NW_ERR_STATE, "calcium is not set up");
    std::string nm(name);
    const int rd = real_dtype_of(ctx);
    const int64_t n = ctx->n_seg;
    DevBuf* b = nullptr;
    int64_t want = n;
    if (nm == "Species.ca") b = &C.c;
    else if (nm == "Species.ca_derivative") b = &C.dcdt;
    else if (nm == "CaPump.state" && C.pump) { b = &C.state; want = 3 * n; }
    else return fail(ctx, NW_ERR_ARG, "nw_calcium_data: unknown attribute " + nm);
    if (count != want)
        return fail(ctx, NW_ERR_ARG, nm + ": expected " + std::to_string(want) + " values");
    if (write) {
        NW_CHECK(upload_convert(ctx, b->ptr, rd, host, dtype, count));
        NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return NW_OK;
    }
    return download_convert(ctx, host, dtype, b->ptr, rd, count);
}

}  // extern "C"
