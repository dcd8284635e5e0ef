// Kinetic-scheme tables on the GPU in FP64 (lti_sim's approximation,
// neuwon/rxd/lti_sim/approx.py:159-174 and lti_model.py:51-65): the exact
// one-step propagator expm(Q(u) dt) at every sample input u, then per bucket
// the least-squares polynomial in the in-bucket location, stored in the
// generated kernel's layout [bucket][col][row][term] (codegen.py:35-37).
//
// The matrix exponential is scaling and squaring around a degree-18 Taylor
// polynomial (Moler & Van Loan, "Nineteen dubious ways", method 3): scale by
// 2^-s until the 1-norm is at most 1/2, where the truncation term is below
// 1e-21 relative, evaluate by Horner's rule and square s times.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "nw_internal.cuh"

namespace nw {

constexpr int kLtiMaxStates = 16;
constexpr int kTaylorDegree = 18;

__device__ void mat_mul(const double* A, const double* B, double* C, int S) {
    for (int r = 0; r < S; ++r)
        for (int c = 0; c < S; ++c) {
            double acc = 0.0;
            for (int k = 0; k < S; ++k) acc = fma(A[r * S + k], B[k * S + c], acc);
            C[r * S + c] = acc;
        }
}

// One thread per sample: out = expm(Q dt), row-major S x S.
__global__ void lti_expm_kernel(const double* __restrict__ Q, int64_t count, int S, double dt,
                                double* __restrict__ out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count) return;
    double A[kLtiMaxStates * kLtiMaxStates], E[kLtiMaxStates * kLtiMaxStates], T[kLtiMaxStates * kLtiMaxStates];
    const double* q = Q + t * S * S;
    double norm = 0.0;
    for (int c = 0; c < S; ++c) {
        double col = 0.0;
        for (int r = 0; r < S; ++r) col += fabs(q[r * S + c] * dt);
        norm = fmax(norm, col);
    }
    int s = 0;
    if (norm > 0.5) s = (int)ceil(log2(norm / 0.5));
    if (s > 60) s = 60;
    const double scale = ldexp(dt, -s);
    for (int i = 0; i < S * S; ++i) A[i] = q[i] * scale;
    // Horner: E = I + A/m; E <- I + A E / k for k = m-1 .. 1.
    for (int i = 0; i < S * S; ++i) E[i] = A[i] / kTaylorDegree;
    for (int d = 0; d < S; ++d) E[d * S + d] += 1.0;
    for (int k = kTaylorDegree - 1; k >= 1; --k) {
        mat_mul(A, E, T, S);
        const double inv = 1.0 / k;
        for (int i = 0; i < S * S; ++i) E[i] = T[i] * inv;
        for (int d = 0; d < S; ++d) E[d * S + d] += 1.0;
    }
    for (int k = 0; k < s; ++k) {
        mat_mul(E, E, T, S);
        for (int i = 0; i < S * S; ++i) E[i] = T[i];
    }
    double* o = out + t * S * S;
    for (int i = 0; i < S * S; ++i) o[i] = E[i];
}

// table[b][c][r][t] = sum_s W[t][s] * P[b * spb + s][r][c], each sample's
// columns first renormalised to sum 1 (lti_model.py:51-65).
__global__ void lti_fit_kernel(const double* __restrict__ P, const double* __restrict__ W, int nb, int spb, int S,
                               int T, double* __restrict__ table) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nb * S * S) return;
    const int b = (int)(t / (S * S));
    const int c = (int)((t / S) % S);
    const int r = (int)(t % S);
    double acc[kMaxTerms];
    for (int k = 0; k < kMaxTerms; ++k) acc[k] = 0.0;
    for (int s = 0; s < spb; ++s) {
        const double* p = P + ((int64_t)b * spb + s) * S * S;
        double col = 0.0;
        for (int rr = 0; rr < S; ++rr) col += p[rr * S + c];
        const double v = p[r * S + c] / col;
        for (int k = 0; k < T; ++k) acc[k] = fma(W[k * spb + s], v, acc[k]);
    }
    for (int k = 0; k < T; ++k) table[(((int64_t)b * S + c) * S + r) * T + k] = acc[k];
}

}  // namespace nw

using namespace nw;

extern "C" {

int nw_lti_expm(nw_ctx* ctx, int32_t S, int64_t count, const double* rates, double dt, double* out) {
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (S < 1 || S > kLtiMaxStates || count < 0 || (count && (!rates || !out)) || !(dt > 0.0))
        return fail(ctx, NW_ERR_ARG, "nw_lti_expm: 1 <= S <= 16, count >= 0, dt > 0");
    if (count == 0) return NW_OK;
    const size_t bytes = (size_t)count * S * S * 8;
    DevBuf dq, dp;
    NW_CHECK(dev_alloc(ctx, dq, bytes));
    int rc = dev_alloc(ctx, dp, bytes);
    if (rc == NW_OK) {
        cudaMemcpyAsync(dq.ptr, rates, bytes, cudaMemcpyHostToDevice, ctx->stream);
        lti_expm_kernel<<<(unsigned)((count + 127) / 128), 128, 0, ctx->stream>>>(dq.as<double>(), count, S, dt,
                                                                                  dp.as<double>());
        cudaMemcpyAsync(out, dp.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "nw_lti_expm");
    }
    dev_free(dq);
    dev_free(dp);
    return rc;
}

int nw_lti_table_build(nw_ctx* ctx, int32_t S, int32_t num_buckets, int32_t samples_per_bucket, int32_t num_terms,
                       const double* rates, const double* fit, double dt, int32_t target, double* table_out) {
    if (ctx) ctx->gc_valid = false;   // the model may change: the next launch gathers G
    if (!ctx) return NW_ERR_ARG;
    cudaSetDevice(ctx->device);
    const bool kin_target = target == 1 || (target >= 16 && target < 16 + kMaxKinetic);
    if (S < 1 || S > kLtiMaxStates || num_buckets < 1 || samples_per_bucket < 1 || num_terms < 1 ||
        num_terms > kMaxTerms || !rates || !fit || !(dt > 0.0) || !(target == 0 || target == 2 || kin_target))
        return fail(ctx, NW_ERR_ARG, "nw_lti_table_build: bad arguments");
    const int64_t count = (int64_t)num_buckets * samples_per_bucket;
    const int64_t tn = (int64_t)num_buckets * S * S * num_terms;
    const int kq = target == 1 ? 0 : target - 16;
    if (kin_target && (kq >= ctx->n_kin || ctx->kin[kq].S != S || ctx->kin[kq].nb != num_buckets ||
                       ctx->kin[kq].T != num_terms))
        return fail(ctx, NW_ERR_STATE, "nw_lti_table_build: no kinetic mechanism " + std::to_string(kq) +
                                       " with a table of this shape");
    if (target == 2 && (!ctx->ca.pump || S != 3 || ctx->ca.nb != num_buckets || ctx->ca.T != num_terms))
        return fail(ctx, NW_ERR_STATE, "nw_lti_table_build: the calcium pump's table has another shape");
    DevBuf dq, dp, dw, dt_tab;
    auto cleanup = [&]() { dev_free(dq); dev_free(dp); dev_free(dw); dev_free(dt_tab); };
    int rc = NW_OK;
    do {
        if ((rc = dev_alloc(ctx, dq, (size_t)count * S * S * 8)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, dp, (size_t)count * S * S * 8)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, dw, (size_t)num_terms * samples_per_bucket * 8)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, dt_tab, (size_t)tn * 8)) != NW_OK) break;
        cudaMemcpyAsync(dq.ptr, rates, (size_t)count * S * S * 8, cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(dw.ptr, fit, (size_t)num_terms * samples_per_bucket * 8, cudaMemcpyHostToDevice, ctx->stream);
        lti_expm_kernel<<<(unsigned)((count + 127) / 128), 128, 0, ctx->stream>>>(dq.as<double>(), count, S, dt,
                                                                                  dp.as<double>());
        const int64_t cells = (int64_t)num_buckets * S * S;
        lti_fit_kernel<<<(unsigned)((cells + 127) / 128), 128, 0, ctx->stream>>>(
            dp.as<double>(), dw.as<double>(), num_buckets, samples_per_bucket, S, num_terms, dt_tab.as<double>());
        if (cudaGetLastError() != cudaSuccess) { rc = fail(ctx, NW_ERR_CUDA, "nw_lti_table_build: launch failed"); break; }
        if (target) {
            DevBuf& dst = kin_target ? ctx->kin[kq].table : ctx->ca.table;
            std::vector<double> host(tn);
            cudaMemcpyAsync(host.data(), dt_tab.ptr, (size_t)tn * 8, cudaMemcpyDeviceToHost, ctx->stream);
            cudaError_t e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "nw_lti_table_build"); break; }
            rc = upload_convert(ctx, dst.ptr, ctx->precision == NW_F64 ? NW_DTYPE_F64 : NW_DTYPE_F32, host.data(),
                                NW_DTYPE_F64, tn);
            if (rc != NW_OK) break;
        }
        if (table_out) cudaMemcpyAsync(table_out, dt_tab.ptr, (size_t)tn * 8, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "nw_lti_table_build"); break; }
    } while (0);
    cleanup();
    return rc;
}

}  // extern "C"
