// Adjoint of the staggered step: gradients of a soma-voltage trace loss with
// respect to every HH instance's conductance coefficients and the cytoplasmic
// resistivity Ra.  The reference has no differentiation; the forward it
// differentiates is the step of neuwon/rxd/rxd_model.py:63-80 as computed here.
//
// Loss: L = mean over steps s and neurons j of (V_det(j)(s+1) - target[s][j])^2,
// V_det the voltage of the neuron's detector segment (its soma by default)
// after step s.
//
// Forward (nw_adjoint_forward) advances the model, stores the state (V and the
// HH gates) every K steps and accumulates L.  Backward (nw_adjoint_backward)
// walks the checkpoint segments from last to first: it restores a checkpoint,
// recomputes the K steps while taping V at the start and middle of each step
// and the gates, then runs the reverse sweep:
//   half step  V' = P x(V, G, E):   lambda_x = P^T lambda_V' = C (P (lambda_V' / C)),
//       the transpose obtained from detailed balance C P = P^T C of the
//       exponential of the tree matrix (exact for the unpruned propagator);
//       dx/dV = alpha, dx/dE = 1 - alpha, dx/dalpha = V - E, alpha = exp(-kG G),
//       E = GE / G;
//   propagator: P = expm(A), A proportional to 1/Ra, so dP/dRa = -(1/Ra) A P and
//       lambda . dV'/dRa = -(1/Ra) sum over edges (child c, parent p) of
//       h (V'_p - V'_c) (lambda_c / C_c - lambda_p / C_p) / R_c;
//   HH gates: Jacobian-vector products of the exact gate update by forward-mode
//       dual numbers through the same device code as the forward.
// Parameter gradients accumulate in FP64, one thread per instance and one
// fixed-order block reduction for Ra, so results are deterministic.
#include <algorithm>
#include <cmath>

#include "nw_step_common.cuh"

namespace nw {

constexpr int kTapeSlots = 5;   // V at step start, V at mid step, m, h, n at step start

template <typename real>
struct AdjArgs {
    StepArgs<real> a;
    int64_t n_seg;
    real* tape;                 // [(k+1)][kTapeSlots][n_seg], or null (forward only)
    const real* target;         // [total_steps][n_neuron], or null
    int64_t step0;              // global index of the first step of this launch
    double* loss_part;          // [n_neuron]
    int update_detectors;
    // reverse sweep
    real* lamV; real* lamV2; real* lamM; real* lamH; real* lamN;
    // Density gradients as compensated sums: sum at [0, n_seg), compensation at
    // [n_seg, 2 n_seg) of each (true value = sum - compensation).
    real* gGna; real* gGk; real* gGl;
    double* ra_part;            // [n_neuron]: sums of flow * d(lambda / C), scaled on the host
    const int64_t* parent;
    const double* res;
    const double* cap;
    // 1/C, C and 1/R per segment in the state precision (the reverse sweep's
    // per-segment arithmetic stays off the FP64 pipe).
    const real* inv_cap; const real* cap_r; const real* inv_res;
    double loss_scale;          // 2 / (total_steps * n_neuron)
    double inv_ra;
    double h_s;                 // half step in seconds
    int g_valid_first;          // conductances valid at global step 0
};

template <typename real>
__device__ __forceinline__ real* tape_slot(const AdjArgs<real>& A, int s, int slot) {
    return A.tape + ((int64_t)s * kTapeSlots + slot) * A.n_seg;
}

// V_r-like sums of one neuron's rows applied to xs in the row format or, when the
// model stores it, the quad format (the same entries); fin(r, row, xi, y).
// Quad rows are claimed by the warps from the CTA's counters ctr[0..1], which
// alternate from call to call (phase, the same in every thread): the call resets the
// other counter, which no warp reads before the barrier that ends this call's phase.
template <typename real, int LPR, bool QUAD, typename Fin>
__device__ __forceinline__ void propagate_adj(const StepArgs<real>& a, int64_t base, int n, const real* xs, Fin fin,
                                              int* ctr, int& phase) {
    if constexpr (QUAD) {
        if (threadIdx.x == 0) ctr[(phase + 1) & 1] = 0;
        propagate_quads_claimed<real, LPR>(a, base, n, xs, fin, ctr + (phase & 1));
        ++phase;
    } else {
        propagate_rows<real, LPR>(a, base, n, xs, fin);
    }
}

// Quad windows of a neuron of fewer than 4 segments reach past it: zeros there.
template <typename real, bool QUAD>
__device__ __forceinline__ void pad_quad_x(real* xs, int n) {
    if (QUAD)
        for (int li = n + threadIdx.x; li < 4; li += blockDim.x) xs[li] = real(0);
}

// Forward steps of one neuron per CTA (HH, one instance per segment), with an
// optional tape and the loss; the arithmetic is that of the batched path.
template <typename real, int LPR, bool QUAD>
__global__ void __launch_bounds__(1024) adjoint_forward_kernel(const AdjArgs<real> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    real* xs = reinterpret_cast<real*>(smem_raw);
    __shared__ int s_job;
    __shared__ int s_ctr[2];
    if (threadIdx.x == 0) { s_ctr[0] = 0; s_ctr[1] = 0; }
    int phase = 0;
    __shared__ int s_nclamp;
    __shared__ uint32_t s_cseg[kMaxClampsPerNeuron];
    __shared__ real s_camp[kMaxClampsPerNeuron];
    __shared__ int64_t s_cfirst[kMaxClampsPerNeuron], s_cend[kMaxClampsPerNeuron];
    const StepArgs<real>& a = A.a;
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (;;) {
        if (tid == 0) s_job = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int job = s_job;
        if (job >= a.n_neuron) break;
        const int j = a.neuron_order[job];
        const int64_t base = a.neuron_start[j];
        const int n = (int)(a.neuron_start[j + 1] - base);
        pad_quad_x<real, QUAD>(xs, n);
        if (tid == 0) {
            const int c0 = a.clamp_neuron_ptr ? a.clamp_neuron_ptr[j] : 0;
            const int c1 = a.clamp_neuron_ptr ? a.clamp_neuron_ptr[j + 1] : 0;
            s_nclamp = c1 - c0;
            for (int c = 0; c < c1 - c0; ++c) {
                s_cseg[c] = a.clamp_seg[c0 + c];
                s_camp[c] = a.clamp_amp[c0 + c];
                s_cfirst[c] = a.clamp_first[c0 + c];
                s_cend[c] = a.clamp_first[c0 + c] + a.clamp_count[c0 + c];
            }
        }
        __syncthreads();
        const int nclamp = s_nclamp;
        bool ap_state = false, ap_det = false;
        uint32_t spikes = 0;
        double loss = 0.0;
        if (tid == 0 && A.update_detectors && a.has_det) {
            ap_state = a.ap_state[j] != 0;
            ap_det = a.ap_detected[j] != 0;
            spikes = a.spike_count[j];
        }
        for (int s = 0; s < a.k_steps; ++s) {
            if (A.tape) {
                for (int li = tid; li < n; li += nthr) {
                    const int64_t i = base + li;
                    tape_slot(A, s, 0)[i] = a.V[i];
                    tape_slot(A, s, 2)[i] = a.gm[i];
                    tape_slot(A, s, 3)[i] = a.gh[i];
                    tape_slot(A, s, 4)[i] = a.gn[i];
                }
            }
#pragma unroll 1
            for (int half = 0; half < 2; ++half) {
                const int64_t tick = a.tick0 + 2 * s + half + 1;
                const bool gv = (s > 0) || (half > 0) || a.g_valid;
                const bool last = (s == a.k_steps - 1) && (half == 1);
                for (int li = tid; li < n; li += nthr) {
                    const int64_t i = base + li;
                    real G, GE;
                    if (gv) segment_conductance(a, i, G, GE);
                    else { G = real(0); GE = real(0); }
                    real I = a.has_nonspec ? a.Inonspec[i] : real(0);
                    for (int c = 0; c < nclamp; ++c)
                        if (s_cseg[c] == (uint32_t)i && tick >= s_cfirst[c] && tick < s_cend[c]) I += s_camp[c];
                    xs[li] = membrane_x(a, i, G, GE, I, last);
                }
                __syncthreads();
                propagate_adj<real, LPR, QUAD>(a, base, n, xs, [&](int64_t r, int, real, real vnew) {
                    if (!isfinite(vnew)) atomicOr(a.status, kStatusNonFinite);
                    a.V[r] = vnew;
                }, s_ctr, phase);
                __syncthreads();
                if (half == 0) {
                    for (int li = tid; li < n; li += nthr) {
                        const int64_t k = base + li;
                        const real v = a.V[k];
                        if (A.tape) tape_slot(A, s, 1)[k] = v;
                        real m = a.gm[k], h = a.gh[k], nn = a.gn[k];
                        hh_gates(v, a.dtq10, m, h, nn);
                        a.gm[k] = m; a.gh[k] = h; a.gn[k] = nn;
                    }
                }
            }
            if (tid == 0) {
                const real vd = a.V[a.det_seg[j]];
                if (A.target) {
                    const double d = (double)vd - (double)A.target[(A.step0 + s) * a.n_neuron + j];
                    loss += d * d;
                }
                if (A.update_detectors && a.has_det) {
                    const bool over = vd >= a.det_thr[j];
                    ap_det = over && !ap_state;
                    ap_state = over;
                    spikes += ap_det ? 1u : 0u;
                }
            }
        }
        if (A.tape) {
            for (int li = tid; li < n; li += nthr) {
                const int64_t i = base + li;
                tape_slot(A, a.k_steps, 0)[i] = a.V[i];
                tape_slot(A, a.k_steps, 2)[i] = a.gm[i];
                tape_slot(A, a.k_steps, 3)[i] = a.gh[i];
                tape_slot(A, a.k_steps, 4)[i] = a.gn[i];
            }
        }
        if (tid == 0) {
            if (A.target) A.loss_part[j] += loss;
            if (A.update_detectors && a.has_det) {
                a.ap_state[j] = ap_state;
                a.ap_detected[j] = ap_det;
                a.spike_count[j] = spikes;
            }
        }
        __syncthreads();
    }
}

// Reverse sweep of one half step of segment i's neuron (called by all threads).
// lam_out holds lambda of the half step's output voltage, lam_in receives lambda
// of its input voltage; the gate adjoints of `gates` accumulate in lamM/H/N.
// The dP/dRa term of the half step (electric.py's coefficients scale with 1/Ra)
// accumulates flow_i * (lambda_i / C_i - lambda_p / C_p) per segment with a parent,
// into the thread's compensated sum (ra_s, ra_c); the factor -h / Ra is applied
// once per neuron.  Density gradients accumulate in compensated sums per segment.
template <typename real, int LPR, bool QUAD>
__device__ __forceinline__ void half_step_reverse(const AdjArgs<real>& A, int64_t base, int n, real* xs,
                                                  const real* V_in, const real* V_out, const real* gm,
                                                  const real* gh, const real* gn, const real* lam_out,
                                                  real* lam_in, bool gv, real& ra_s, real& ra_c, int* ctr,
                                                  int& phase) {
    const StepArgs<real>& a = A.a;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int64_t ns = A.n_seg;
    for (int li = tid; li < n; li += nthr) {
        const int64_t i = base + li;
        xs[li] = lam_out[i] * A.inv_cap[i];
    }
    __syncthreads();
    // The rows leave lambda of x (C P^T applied) in lam_in; the membrane update's
    // adjoint follows per segment below, with every lane of the CTA.
    propagate_adj<real, LPR, QUAD>(a, base, n, xs, [&](int64_t r, int, real, real nu) { lam_in[r] = nu * A.cap_r[r]; },
                                   ctr, phase);
    // xs still holds lambda / C of every segment of the neuron (the rows only read it).
    for (int li = tid; li < n; li += nthr) {
        const int64_t i = base + li;
        const int64_t p = A.parent[i];
        if (p >= 0) {
            const real flow = (V_out[p] - V_out[i]) * A.inv_res[i];
            kahan_add(ra_s, ra_c, flow * (xs[li] - xs[p - base]));
        }
    }
    __syncthreads();
    if (!gv) return;                     // G = 0: x = V, no parameter dependence
    for (int li = tid; li < n; li += nthr) {
        const int64_t r = base + li;
        const real lx = lam_in[r];
        const real m = gm[r], h = gh[r], nn = gn[r];
        const real M = m * m * m * h, N4 = nn * nn * nn * nn;
        const real gna = a.cna[r] * M, gk = a.ck[r] * N4, gl = a.cl[r];
        const real G = (gna + gk) + gl;
        const real GE = (gna * a.ena + gk * a.ek) + gl * a.el;
        const real E = GE / G;
        const real alpha = d_exp(-a.kG[r] * G);
        lam_in[r] = alpha * lx;
        const real lE = (real(1) - alpha) * lx;
        const real lalpha = (V_in[r] - E) * lx;
        const real lG = -a.kG[r] * alpha * lalpha - (E / G) * lE;
        const real lGE = lE / G;
        const real wna = lG + lGE * a.ena, wk = lG + lGE * a.ek, wl = lG + lGE * a.el;
        auto acc = [&](real* g, real term) {
            real sg = g[r], cg = g[ns + r];
            kahan_add(sg, cg, term);
            g[r] = sg;
            g[ns + r] = cg;
        };
        acc(A.gGna, wna * M);
        acc(A.gGk, wk * N4);
        acc(A.gGl, wl);
        const real lM = wna * a.cna[r], lN4 = wk * a.ck[r];
        A.lamM[r] += lM * real(3) * m * m * h;
        A.lamH[r] += lM * m * m * m;
        A.lamN[r] += lN4 * real(4) * nn * nn * nn;
    }
    __syncthreads();
}

// FP32: bounds (1024, 2), so two neurons share an SM (32 registers, a few spilled
// bytes; every neuron of the 256-neuron differentiation batch in one wave, twice
// the warps in flight: 0.40 -> 0.34 ms per backward step); FP64 keeps one.
template <typename real, int LPR, bool QUAD>
__global__ void __launch_bounds__(1024, sizeof(real) == 4 ? 2 : 1) adjoint_reverse_kernel(const AdjArgs<real> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    real* xs = reinterpret_cast<real*>(smem_raw);
    __shared__ int s_job;
    __shared__ double s_red[1024];
    __shared__ int s_ctr[2];
    if (threadIdx.x == 0) { s_ctr[0] = 0; s_ctr[1] = 0; }
    int phase = 0;
    const StepArgs<real>& a = A.a;
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (;;) {
        if (tid == 0) s_job = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int job = s_job;
        if (job >= a.n_neuron) break;
        const int j = a.neuron_order[job];
        const int64_t base = a.neuron_start[j];
        const int n = (int)(a.neuron_start[j + 1] - base);
        pad_quad_x<real, QUAD>(xs, n);
        real ra_s = real(0), ra_c = real(0);
        for (int s = a.k_steps - 1; s >= 0; --s) {
            const int64_t gs = A.step0 + s;
            if (tid == 0 && A.target) {
                const int64_t d = a.det_seg[j];
                const real vd = tape_slot(A, s + 1, 0)[d];
                A.lamV[d] += (real)(A.loss_scale * ((double)vd - (double)A.target[gs * a.n_neuron + j]));
            }
            __syncthreads();
            // Second half step: V_mid, gates(s+1) -> V(s+1).
            half_step_reverse<real, LPR, QUAD>(A, base, n, xs, tape_slot(A, s, 1), tape_slot(A, s + 1, 0),
                                         tape_slot(A, s + 1, 2), tape_slot(A, s + 1, 3), tape_slot(A, s + 1, 4),
                                         A.lamV, A.lamV2, true, ra_s, ra_c, s_ctr, phase);
            // Mechanisms: gates(s+1) = f(gates(s), V_mid).
            for (int li = tid; li < n; li += nthr) {
                const int64_t i = base + li;
                const real v = tape_slot(A, s, 1)[i];
                const real m0 = tape_slot(A, s, 2)[i], h0 = tape_slot(A, s, 3)[i], n0 = tape_slot(A, s, 4)[i];
                // d gates(s+1) / d V_mid in the dual parts; d gate(s+1) / d gate(s) is
                // each gate's decay factor exp(-dt/xtau), the value parts of em, eh, en.
                Dual<real> dv(v, real(1)), dm(m0), dh(h0), dn(n0), dq(a.dtq10), em, eh, en;
                hh_gates_decay(dv, dq, dm, dh, dn, em, eh, en);
                const real lm = A.lamM[i], lh = A.lamH[i], ln = A.lamN[i];
                A.lamV2[i] += dm.d * lm + dh.d * lh + dn.d * ln;
                A.lamM[i] = em.v * lm;
                A.lamH[i] = eh.v * lh;
                A.lamN[i] = en.v * ln;
            }
            __syncthreads();
            // First half step: V(s), gates(s) -> V_mid.
            const bool gv = (gs > 0) || A.g_valid_first;
            half_step_reverse<real, LPR, QUAD>(A, base, n, xs, tape_slot(A, s, 0), tape_slot(A, s, 1),
                                         tape_slot(A, s, 2), tape_slot(A, s, 3), tape_slot(A, s, 4),
                                         A.lamV2, A.lamV, gv, ra_s, ra_c, s_ctr, phase);
        }
        // Fixed-order reduction of the Ra partial sums, scaled by -h / Ra.
        s_red[tid] = (double)ra_s - (double)ra_c;
        __syncthreads();
        if (tid == 0) {
            double r = 0.0;
            for (int t = 0; t < nthr; ++t) r += s_red[t];
            A.ra_part[j] += -A.inv_ra * A.h_s * r;
        }
        __syncthreads();
    }
}

// 1/C, C and 1/R of every segment in the state precision (1/R = 0 for a root).
template <typename real>
__global__ void adj_coef_kernel(int64_t n, const double* __restrict__ cap, const double* __restrict__ res,
                                real* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = (real)(1.0 / cap[i]);
    out[n + i] = (real)cap[i];
    out[2 * n + i] = res[i] > 0.0 ? (real)(1.0 / res[i]) : real(0);
}

// ---------------------------------------------------------------- host

template <typename real>
static AdjArgs<real> adj_args(nw_ctx* ctx) {
    AdjArgs<real> A{};
    A.a = make_args<real>(ctx, 1);
    A.n_seg = ctx->n_seg;
    A.loss_part = ctx->adj.loss_part.as<double>();
    A.target = ctx->adj.target.as<real>();
    A.parent = ctx->parent.as<int64_t>();
    A.res = ctx->res64.as<double>();
    A.cap = ctx->cap64.as<double>();
    A.h_s = 0.5 * ctx->time_step * 1e-3;
    A.g_valid_first = ctx->adj.g_valid0 ? 1 : 0;
    A.loss_scale = 2.0 / ((double)ctx->adj.total_steps * (double)ctx->n_neuron);
    return A;
}

static int adj_lpr(nw_ctx* ctx) {
    int l = choose_lanes_per_row(ctx);
    return l >= 16 ? 16 : (l >= 8 ? 8 : 4);
}

// x of the largest neuron (at least 4 entries: quad windows of smaller neurons
// reach past them).
template <typename real>
static size_t adj_smem(const nw_ctx* ctx) {
    return ((size_t)std::max<int64_t>(ctx->max_neuron, 4) * sizeof(real) + 15) & ~(size_t)15;
}

template <typename real, int LPR, bool QUAD>
static int launch_forward_cfg(nw_ctx* ctx, AdjArgs<real>& A, cudaStream_t st) {
    auto kern = adjoint_forward_kernel<real, LPR, QUAD>;
    const size_t smem = adj_smem<real>(ctx);
    NW_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    NW_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, ctx->threads, smem));
    if (occ < 1) return fail(ctx, NW_ERR_LIMIT, "adjoint forward kernel does not fit on an SM");
    const int64_t grid = std::min<int64_t>(ctx->n_neuron, (int64_t)occ * ctx->num_sms);
    NW_CUDA(ctx, cudaMemsetAsync(A.a.work_counter, 0, sizeof(int), st));
    kern<<<(unsigned)grid, ctx->threads, smem, st>>>(A);
    NW_CUDA(ctx, cudaGetLastError());
    return NW_OK;
}

template <typename real, int LPR, bool QUAD>
static int launch_reverse_cfg(nw_ctx* ctx, AdjArgs<real>& A, cudaStream_t st) {
    auto kern = adjoint_reverse_kernel<real, LPR, QUAD>;
    const size_t smem = adj_smem<real>(ctx);
    NW_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    NW_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, ctx->threads, smem));
    if (occ < 1) return fail(ctx, NW_ERR_LIMIT, "adjoint reverse kernel does not fit on an SM");
    const int64_t grid = std::min<int64_t>(ctx->n_neuron, (int64_t)occ * ctx->num_sms);
    NW_CUDA(ctx, cudaMemsetAsync(A.a.work_counter, 0, sizeof(int), st));
    kern<<<(unsigned)grid, ctx->threads, smem, st>>>(A);
    NW_CUDA(ctx, cudaGetLastError());
    return NW_OK;
}

// The quad format when the model stores its propagator that way (the same entries
// as the rows, fewer bytes), else the row format.
static bool adj_quads(const nw_ctx* ctx) { return ctx->prop_format == 2 && ctx->q_ok; }

template <typename real>
static int launch_forward(nw_ctx* ctx, AdjArgs<real>& A, cudaStream_t st) {
    const bool q = adj_quads(ctx);
    switch (adj_lpr(ctx)) {
        case 4: return q ? launch_forward_cfg<real, 4, true>(ctx, A, st) : launch_forward_cfg<real, 4, false>(ctx, A, st);
        case 8: return q ? launch_forward_cfg<real, 8, true>(ctx, A, st) : launch_forward_cfg<real, 8, false>(ctx, A, st);
        default: return q ? launch_forward_cfg<real, 16, true>(ctx, A, st) : launch_forward_cfg<real, 16, false>(ctx, A, st);
    }
}

template <typename real>
static int launch_reverse(nw_ctx* ctx, AdjArgs<real>& A, cudaStream_t st) {
    const bool q = adj_quads(ctx);
    switch (adj_lpr(ctx)) {
        case 4: return q ? launch_reverse_cfg<real, 4, true>(ctx, A, st) : launch_reverse_cfg<real, 4, false>(ctx, A, st);
        case 8: return q ? launch_reverse_cfg<real, 8, true>(ctx, A, st) : launch_reverse_cfg<real, 8, false>(ctx, A, st);
        default: return q ? launch_reverse_cfg<real, 16, true>(ctx, A, st) : launch_reverse_cfg<real, 16, false>(ctx, A, st);
    }
}

// State copied at checkpoints: V, m, h, n.
static int copy_state(nw_ctx* ctx, char* dst, bool to_ckpt, cudaStream_t st) {
    const size_t b = (size_t)ctx->precision * ctx->n_seg;
    void* arrs[4] = {ctx->V.ptr, ctx->hh.gm.ptr, ctx->hh.gh.ptr, ctx->hh.gn.ptr};
    for (int k = 0; k < 4; ++k) {
        if (to_ckpt) NW_CUDA(ctx, cudaMemcpyAsync(dst + k * b, arrs[k], b, cudaMemcpyDeviceToDevice, st));
        else NW_CUDA(ctx, cudaMemcpyAsync(arrs[k], dst + k * b, b, cudaMemcpyDeviceToDevice, st));
    }
    return NW_OK;
}

template <typename real>
static int adjoint_forward_impl(nw_ctx* ctx, int64_t T, int K, const double* target, double* loss_out) {
    AdjointState& S = ctx->adj;
    const int64_t nn = ctx->n_neuron, n = ctx->n_seg;
    const int64_t nseg = (T + K - 1) / K;
    const size_t b = (size_t)ctx->precision * n;
    NW_CHECK(dev_alloc(ctx, S.ckpt, 4 * b * (size_t)(nseg + 1)));
    NW_CHECK(dev_alloc(ctx, S.target, (size_t)ctx->precision * T * nn));
    NW_CHECK(dev_alloc(ctx, S.loss_part, 8 * nn));
    NW_CHECK(upload_convert(ctx, S.target.ptr, ctx->precision == NW_F64 ? NW_DTYPE_F64 : NW_DTYPE_F32, target,
                            NW_DTYPE_F64, T * nn));
    NW_CUDA(ctx, cudaMemsetAsync(S.loss_part.ptr, 0, 8 * nn, ctx->stream));
    S.K = K; S.total_steps = T; S.tick0 = ctx->input_ticks; S.g_valid0 = ctx->g_valid;
    for (int64_t sg = 0; sg < nseg; ++sg) {
        NW_CHECK(copy_state(ctx, S.ckpt.as<char>() + 4 * b * sg, true, ctx->stream));
        const int k = (int)std::min<int64_t>(K, T - sg * K);
        AdjArgs<real> A = adj_args<real>(ctx);
        A.a.k_steps = k;
        A.a.tick0 = ctx->input_ticks;
        A.a.g_valid = ctx->g_valid ? 1 : 0;
        A.step0 = sg * K;
        A.update_detectors = 1;
        NW_CHECK(launch_forward(ctx, A, ctx->stream));
        ctx->input_ticks += 2 * (int64_t)k;
        ctx->steps += k;
        ctx->g_valid = true;
    }
    NW_CHECK(copy_state(ctx, S.ckpt.as<char>() + 4 * b * nseg, true, ctx->stream));
    std::vector<double> lp(nn);
    NW_CUDA(ctx, cudaMemcpyAsync(lp.data(), S.loss_part.ptr, 8 * nn, cudaMemcpyDeviceToHost, ctx->stream));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double loss = 0.0;
    for (int64_t k = 0; k < nn; ++k) loss += lp[k];
    S.loss = loss / ((double)T * (double)nn);
    S.ready = true;
    if (loss_out) *loss_out = S.loss;
    return NW_OK;
}

template <typename real>
static int adjoint_backward_impl(nw_ctx* ctx, double Ra, double* g_gna, double* g_gk, double* g_gl,
                                 double* g_ra) {
    AdjointState& S = ctx->adj;
    const int64_t nn = ctx->n_neuron, n = ctx->n_seg, T = S.total_steps;
    const int K = S.K;
    const int64_t nseg = (T + K - 1) / K;
    const size_t b = (size_t)ctx->precision * n;
    // Two tapes (by the parity of the checkpoint segment) when the recompute of
    // segment k-1 runs beside the reverse sweep of segment k, else one.
    const bool overlap = ctx->adjoint_overlap && nseg > 1;
    const size_t tape_elems = (size_t)n * kTapeSlots * (size_t)(K + 1);
    NW_CHECK(dev_alloc(ctx, S.tape, (size_t)ctx->precision * tape_elems * (overlap ? 2 : 1)));
    if (overlap && !S.stream) {
        NW_CUDA(ctx, cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
        for (cudaEvent_t* e : {&S.rec_done, &S.rev_done[0], &S.rev_done[1], &S.start})
            NW_CUDA(ctx, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    // Recompute and reverse sweep count their neurons on separate counters.
    int* const wc_rec = ctx->work_counter.as<int>();
    int* const wc_rev = overlap ? wc_rec + 4 : wc_rec;
    const cudaStream_t rs = overlap ? S.stream : ctx->stream;
    for (DevBuf* buf : {&S.lamV, &S.lamV2, &S.lamM, &S.lamH, &S.lamN}) {
        NW_CHECK(dev_alloc(ctx, *buf, b));
        NW_CUDA(ctx, cudaMemsetAsync(buf->ptr, 0, b, ctx->stream));
    }
    for (DevBuf* buf : {&S.gGna, &S.gGk, &S.gGl}) {
        NW_CHECK(dev_alloc(ctx, *buf, 2 * b));
        NW_CUDA(ctx, cudaMemsetAsync(buf->ptr, 0, 2 * b, ctx->stream));
    }
    NW_CHECK(dev_alloc(ctx, S.coef, 3 * b));
    adj_coef_kernel<real><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
        n, ctx->cap64.as<double>(), ctx->res64.as<double>(), S.coef.as<real>());
    NW_CUDA(ctx, cudaGetLastError());
    NW_CHECK(dev_alloc(ctx, S.ra_part, 8 * nn));
    NW_CUDA(ctx, cudaMemsetAsync(S.ra_part.ptr, 0, 8 * nn, ctx->stream));
    if (overlap) {
        NW_CUDA(ctx, cudaEventRecord(S.start, ctx->stream));
        NW_CUDA(ctx, cudaStreamWaitEvent(rs, S.start, 0));
    }
    for (int64_t sg = nseg - 1; sg >= 0; --sg) {
        const int k = (int)std::min<int64_t>(K, T - sg * K);
        const int par = overlap ? (int)(sg & 1) : 0;
        // This tape was last read by the reverse sweep of segment sg + 2.
        if (overlap && sg + 2 <= nseg - 1) NW_CUDA(ctx, cudaStreamWaitEvent(rs, S.rev_done[par], 0));
        NW_CHECK(copy_state(ctx, S.ckpt.as<char>() + 4 * b * sg, false, rs));
        AdjArgs<real> A = adj_args<real>(ctx);
        A.a.k_steps = k;
        A.a.tick0 = S.tick0 + 2 * sg * (int64_t)K;
        A.a.g_valid = (sg == 0) ? (S.g_valid0 ? 1 : 0) : 1;
        A.a.work_counter = wc_rec;
        A.step0 = sg * K;
        A.tape = S.tape.as<real>() + (size_t)par * tape_elems;
        A.target = nullptr;
        A.update_detectors = 0;
        NW_CHECK(launch_forward(ctx, A, rs));
        if (overlap) {
            NW_CUDA(ctx, cudaEventRecord(S.rec_done, rs));
            NW_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, S.rec_done, 0));
        }
        A.a.work_counter = wc_rev;
        A.target = S.target.as<real>();
        A.lamV = S.lamV.as<real>(); A.lamV2 = S.lamV2.as<real>();
        A.lamM = S.lamM.as<real>(); A.lamH = S.lamH.as<real>(); A.lamN = S.lamN.as<real>();
        A.gGna = S.gGna.as<real>(); A.gGk = S.gGk.as<real>(); A.gGl = S.gGl.as<real>();
        A.inv_cap = S.coef.as<real>(); A.cap_r = A.inv_cap + n; A.inv_res = A.inv_cap + 2 * n;
        A.ra_part = S.ra_part.as<double>();
        A.inv_ra = 1.0 / Ra;
        NW_CHECK(launch_reverse(ctx, A, ctx->stream));
        if (overlap) NW_CUDA(ctx, cudaEventRecord(S.rev_done[par], ctx->stream));
    }
    // Every recompute precedes a reverse sweep that the context's stream waited for.
    NW_CHECK(copy_state(ctx, S.ckpt.as<char>() + 4 * b * nseg, false, ctx->stream));
    std::vector<real> gsum[3] = {std::vector<real>(2 * n), std::vector<real>(2 * n), std::vector<real>(2 * n)};
    std::vector<double> rp(nn);
    DevBuf* gbuf[3] = {&S.gGna, &S.gGk, &S.gGl};
    for (int k = 0; k < 3; ++k)
        NW_CUDA(ctx, cudaMemcpyAsync(gsum[k].data(), gbuf[k]->ptr, 2 * b, cudaMemcpyDeviceToHost, ctx->stream));
    NW_CUDA(ctx, cudaMemcpyAsync(rp.data(), S.ra_part.ptr, 8 * nn, cudaMemcpyDeviceToHost, ctx->stream));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<double> gna(n), gk(n), gl(n);
    for (int64_t i = 0; i < n; ++i) {
        gna[i] = (double)gsum[0][i] - (double)gsum[0][n + i];
        gk[i] = (double)gsum[1][i] - (double)gsum[1][n + i];
        gl[i] = (double)gsum[2][i] - (double)gsum[2][n + i];
    }
    const std::vector<int64_t>& u2s = ctx->hh.user_to_sorted;
    for (int64_t u = 0; u < ctx->hh.m; ++u) {
        if (g_gna) g_gna[u] = gna[u2s[u]];
        if (g_gk) g_gk[u] = gk[u2s[u]];
        if (g_gl) g_gl[u] = gl[u2s[u]];
    }
    if (g_ra) {
        double r = 0.0;
        for (int64_t k = 0; k < nn; ++k) r += rp[k];
        *g_ra = r;
    }
    return NW_OK;
}

static int adjoint_check(nw_ctx* ctx) {
    if (ctx->n_seg == 0) return fail(ctx, NW_ERR_STATE, "adjoint before nw_model_init");
    if (!ctx->prop_valid) return fail(ctx, NW_ERR_STATE, "adjoint: no propagator installed");
    if (ctx->prop_lumped)
        return fail(ctx, NW_ERR_STATE, "adjoint: a lumped propagator has no detailed-balance transpose");
    if (!ctx->have_cap || !ctx->have_res) return fail(ctx, NW_ERR_STATE, "adjoint: capacitance/resistance not set");
    if (ctx->hh.m == 0 || !ctx->hh.identity)
        return fail(ctx, NW_ERR_STATE, "adjoint: needs exactly one HH instance on every segment");
    if (kinetic_instances(ctx) != 0) return fail(ctx, NW_ERR_STATE, "adjoint: kinetic mechanisms are not differentiated");
    if (ctx->syn.n != 0) return fail(ctx, NW_ERR_STATE, "adjoint: synapses are not differentiated");
    if (ctx->ca.on) return fail(ctx, NW_ERR_STATE, "adjoint: calcium is not differentiated");
    if (!ctx->b_ok) return fail(ctx, NW_ERR_LIMIT, "adjoint: a neuron has more than 65,535 segments");
    if (ctx->nonspec_nonzero) return fail(ctx, NW_ERR_STATE, "adjoint: nonspecific currents are not supported");
    if (ctx->prop_format == 2) NW_CHECK(ensure_quads(ctx));
    return NW_OK;
}

// A backward that stopped on an error may have left recomputes queued on the
// second stream; nothing it reads is reallocated before they finish.
static int adjoint_quiesce(nw_ctx* ctx) {
    if (ctx->adj.stream) NW_CUDA(ctx, cudaStreamSynchronize(ctx->adj.stream));
    return NW_OK;
}

int adjoint_forward(nw_ctx* ctx, int64_t T, int K, const double* target, double* loss_out) {
    NW_CHECK(adjoint_quiesce(ctx));
    NW_CHECK(adjoint_check(ctx));
    if (T <= 0 || K <= 0 || !target) return fail(ctx, NW_ERR_ARG, "nw_adjoint_forward: bad steps or target");
    return ctx->precision == NW_F64 ? adjoint_forward_impl<double>(ctx, T, K, target, loss_out)
                                    : adjoint_forward_impl<float>(ctx, T, K, target, loss_out);
}

int adjoint_backward(nw_ctx* ctx, double Ra, double* g_gna, double* g_gk, double* g_gl, double* g_ra) {
    NW_CHECK(adjoint_quiesce(ctx));
    NW_CHECK(adjoint_check(ctx));
    if (!ctx->adj.ready) return fail(ctx, NW_ERR_STATE, "nw_adjoint_backward before nw_adjoint_forward");
    if (!(Ra > 0)) return fail(ctx, NW_ERR_ARG, "nw_adjoint_backward: Ra must be > 0");
    const int rc = ctx->precision == NW_F64 ? adjoint_backward_impl<double>(ctx, Ra, g_gna, g_gk, g_gl, g_ra)
                                            : adjoint_backward_impl<float>(ctx, Ra, g_gna, g_gk, g_gl, g_ra);
    // On an error nothing stays queued on the second stream.
    if (rc != NW_OK && ctx->adj.stream) cudaStreamSynchronize(ctx->adj.stream);
    return rc;
}

}  // namespace nw
