// Wide path: the staggered step (neuwon/rxd/rxd_model.py:63-80) as whole-model
// launches, one per phase, so a neuron of any size spreads over every SM.
//
//   membrane x (all segments) -> propagator rows (all rows, x from L2) ->
//   mechanisms (HH, kinetic, synapses; first half only) -> ... -> AP detector
//
// The propagator is the same difference form as the batched path with global
// int32 columns.  Launch sequences of up to kWideGraphSteps steps are captured
// as CUDA graphs; the step offset within the sequence is a launch argument and
// the clock is the device word written before each replay.
#include <algorithm>
#include <cstring>

#include "nw_step_common.cuh"

namespace nw {

constexpr int kWideGraphSteps = 32;
constexpr int kWideThreads = 256;

template <typename real>
__global__ void __launch_bounds__(kWideThreads)
wide_membrane_kernel(const StepArgs<real> a, const int s_off, const int half, const int last) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= a.neuron_start[a.n_neuron]) return;
    const int64_t tick = a.clk->input_ticks + 2 * (int64_t)s_off + half + 1;
    const bool gv = s_off > 0 || half > 0 || a.clk->g_valid != 0;
    real G = real(0), GE = real(0);
    if (gv) segment_conductance(a, i, G, GE);
    real I = a.has_nonspec ? a.Inonspec[i] : real(0);
    if (a.clamp_seg_ptr) {
        for (uint32_t c = a.clamp_seg_ptr[i]; c < a.clamp_seg_ptr[i + 1]; ++c)
            if (tick >= a.clamp_first[c] && tick < a.clamp_first[c] + a.clamp_count[c]) I += a.clamp_amp[c];
    }
    a.px[i] = membrane_x(a, i, G, GE, I, last != 0);
    // species._advance (species.py:56-70), first part: c + dc/dt h into the scratch
    // the calcium rows multiply (the same launch: independent of x).
    if (a.ca_on) a.ca_scratch[i] = fmax(real(0), a.ca_c[i] + a.ca_dcdt[i] * a.h_ms);
}

// V_i = x_i - leak_i x_i + sum_j P_ij (x_j - x_i), LPR lanes per row, 4-entry
// vectors with the evict-first hint, Kahan-compensated lane sums.
// gt: the thread's index in the launch's part for these rows (LPR threads per row).
template <typename real, int LPR>
__device__ __forceinline__ void rows_body(const int64_t gt, const int64_t* __restrict__ rowptr,
                                          const int32_t* __restrict__ col, const real* __restrict__ val,
                                          const real* __restrict__ leak, const real* __restrict__ x,
                                          real* __restrict__ y, const int64_t n, int* status) {
    const int64_t g = gt / LPR;
    const int l = threadIdx.x % LPR;
    const bool valid = g < n;
    real s = real(0), c = real(0), xi = real(0);
    if (valid) {
        xi = __ldg(x + g);
        const int64_t beg = rowptr[g], end = rowptr[g + 1];
        // Two 4-entry vectors per lane in flight.
        for (int64_t k0 = beg + 4 * l; k0 < end; k0 += 8 * LPR) {
            real v[2][4];
            int4 cc[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int64_t k = k0 + 4 * LPR * u;
                if (k < end) {
                    Vec4Loader<real>::load(val + k, v[u]);
                    cc[u] = __ldcs(reinterpret_cast<const int4*>(col + k));
                } else {
                    v[u][0] = v[u][1] = v[u][2] = v[u][3] = real(0);
                    cc[u] = make_int4(g, g, g, g);     // zero weights on x_i
                }
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const real p = v[u][0] * (__ldg(x + cc[u].x) - xi) + v[u][1] * (__ldg(x + cc[u].y) - xi);
                const real q = v[u][2] * (__ldg(x + cc[u].z) - xi) + v[u][3] * (__ldg(x + cc[u].w) - xi);
                kahan_add(s, c, p + q);
            }
        }
    }
    real t = s - c;
#pragma unroll
    for (int off = LPR / 2; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off, LPR);
    if (valid && l == 0) {
        const real vnew = (xi - leak[g] * xi) + t;
        if (!isfinite(vnew)) atomicOr(status, kStatusNonFinite);
        y[g] = vnew;
    }
}

template <typename real, int LPR>
__global__ void __launch_bounds__(kWideThreads)
wide_rows_kernel(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                 const real* __restrict__ val, const real* __restrict__ leak, const real* __restrict__ x,
                 real* __restrict__ y, const int64_t n, int* status) {
    rows_body<real, LPR>(blockIdx.x * (int64_t)blockDim.x + threadIdx.x, rowptr, col, val, leak, x, y, n, status);
}

// Quad format with global bases: each window's four x are consecutive in memory
// (one or two cache sectors instead of four).
template <typename real, int LPR>
__device__ __forceinline__ void quads_body(const int64_t gt, const int64_t* __restrict__ qrow,
                                           const int32_t* __restrict__ qbase, const real* __restrict__ qval,
                                           const real* __restrict__ leak, const real* __restrict__ x,
                                           real* __restrict__ y, const int64_t n, int* status) {
    const int64_t g = gt / LPR;
    const int l = threadIdx.x % LPR;
    const bool valid = g < n;
    real s = real(0), c = real(0), xi = real(0);
    if (valid) {
        xi = __ldg(x + g);
        const int64_t beg = qrow[g], end = qrow[g + 1];
        // Four FP32 windows per lane in flight (FP64: two; more only costs registers
        // on that slower path).
        constexpr int UNROLL = sizeof(real) == 4 ? 4 : 2;
        for (int64_t k0 = beg + l; k0 < end; k0 += UNROLL * LPR) {
            real v[UNROLL][4];
            int32_t b[UNROLL];
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                const int64_t k = k0 + LPR * u;
                if (k < end) {
                    Vec4Loader<real>::load(qval + 4 * k, v[u]);
                    b[u] = __ldcs(qbase + k);
                } else {
                    v[u][0] = v[u][1] = v[u][2] = v[u][3] = real(0);
                    b[u] = 0;                 // zero weights on x[0..3] (n >= 4)
                }
            }
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                const real* xb = x + b[u];
                const real p = v[u][0] * (__ldg(xb) - xi) + v[u][1] * (__ldg(xb + 1) - xi);
                const real q = v[u][2] * (__ldg(xb + 2) - xi) + v[u][3] * (__ldg(xb + 3) - xi);
                kahan_add(s, c, p + q);
            }
        }
    }
    real t = s - c;
#pragma unroll
    for (int off = LPR / 2; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off, LPR);
    if (valid && l == 0) {
        const real vnew = (xi - leak[g] * xi) + t;
        if (!isfinite(vnew)) atomicOr(status, kStatusNonFinite);
        y[g] = vnew;
    }
}

template <typename real, int LPR>
__global__ void __launch_bounds__(kWideThreads)
wide_quads_kernel(const int64_t* __restrict__ qrow, const int32_t* __restrict__ qbase,
                  const real* __restrict__ qval, const real* __restrict__ leak, const real* __restrict__ x,
                  real* __restrict__ y, const int64_t n, int* status) {
    quads_body<real, LPR>(blockIdx.x * (int64_t)blockDim.x + threadIdx.x, qrow, qbase, qval, leak, x, y, n, status);
}

// The voltage rows (quad format, LPR lanes per row) and the calcium rows (row
// format, 4 lanes per row) of one half step in one launch: blocks below
// `vblocks` take voltage rows, the others calcium rows (the two read different x
// and write different outputs).
template <typename real, int LPR>
__global__ void __launch_bounds__(kWideThreads)
wide_quads_calcium_kernel(const StepArgs<real> a, const int64_t* __restrict__ qrow, const int32_t* __restrict__ qbase,
                          const real* __restrict__ qval, const real* __restrict__ leak, const int64_t vblocks) {
    const int64_t n = a.neuron_start[a.n_neuron];
    if (blockIdx.x < vblocks)
        quads_body<real, LPR>(blockIdx.x * (int64_t)blockDim.x + threadIdx.x, qrow, qbase, qval, leak, a.px, a.V, n,
                              a.status);
    else
        rows_body<real, 4>((blockIdx.x - vblocks) * (int64_t)blockDim.x + threadIdx.x, a.ca_wrow, a.ca_wcol,
                           a.ca_wval, a.ca_wleak, a.ca_scratch, a.ca_c, a.ca_n, a.status);
}

template <typename real>
__global__ void __launch_bounds__(kWideThreads)
wide_mechanism_kernel(const StepArgs<real> a, const int s_off, const int64_t n_hh, const int64_t n_kin,
                      const int64_t n_syn) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n_hh) {
        const real v = a.V[a.hh_identity ? k : (int64_t)a.hh_seg[k]];
        real m = a.gm[k], h = a.gh[k], nn = a.gn[k];
        hh_gates(v, a.dtq10, m, h, nn);
        a.gm[k] = m; a.gh[k] = h; a.gn[k] = nn;
        return;
    }
    k -= n_hh;
    if (k < n_kin) {
        // n_kin counts the instances of all kinetic mechanisms, in registration order.
        int q = 0;
        while (k >= a.kin[q].m) { k -= a.kin[q].m; ++q; }
        const KinArgs<real>& K = a.kin[q];
        kinetic_step(K, k, a.V[K.identity ? k : (int64_t)K.seg[k]]);
        return;
    }
    k -= n_kin;
    if (k < n_syn) synapse_step(a, k, a.clk->steps + s_off);
}

template <typename real>
__global__ void __launch_bounds__(kWideThreads)
wide_calcium_mechanism_kernel(const StepArgs<real> a) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= a.ca_n) return;
    calcium_mechanisms(a, i);
}

// HH gates (one instance per segment, in segment order) and the calcium mechanisms
// of each segment in one launch: a thread updates segment i's gates, then its
// calcium, which reads the new gates for the sodium influx (the order of the two
// launches this replaces).
template <typename real>
__global__ void __launch_bounds__(kWideThreads)
wide_hh_calcium_kernel(const StepArgs<real> a) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= a.ca_n) return;
    if (a.hh_on) {
        const real v = a.V[i];
        real m = a.gm[i], h = a.gh[i], nn = a.gn[i];
        hh_gates(v, a.dtq10, m, h, nn);
        a.gm[i] = m; a.gh[i] = h; a.gn[i] = nn;
    }
    calcium_mechanisms(a, i);
}

template <typename real>
__global__ void wide_detect_kernel(const StepArgs<real> a, const int s_off) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t s_abs = a.clk->steps + s_off;
    if (j < a.n_neuron && a.has_det) {
        const bool over = a.V[a.det_seg[j]] >= a.det_thr[j];
        const bool det = over && !a.ap_state[j];
        a.ap_detected[j] = det;
        a.ap_state[j] = over;
        a.spike_count[j] += det ? 1u : 0u;
        if (a.syn_on) spike_ring_write(a, j, s_abs, det);
    }
    if (j < a.n_probes)
        a.trace[(a.clk->probe_len + s_off) * a.n_probes + a.probe_slot[j]] = a.V[a.probe_seg[j]];
}

// ------------------------------------------------------------ fused half step
//
// When every conductance source maps one-to-one onto segments (HH and kinetic
// instances in segment order, no synapses), a half step is one launch: each warp
// applies the propagator to 32 consecutive rows (LPR lanes per row, the row
// format's or the quad format's sums as in wide_rows_kernel / wide_quads_kernel,
// reading x from x_in; the 32 row pointers and x_i come in one coalesced load
// each, and every lane has UNROLL windows in flight before it sums any), parks
// the 32 results in shared memory, and then each lane
// finishes its own segment i: V_i, the calcium row i (one lane per row, reading
// the scratch cs_in), and, after the first half, the mechanisms at the mid-step
// voltage (HH, kinetic, calcium, rxd_model.py:115-123), the new conductance and
// the second half's x_i and calcium scratch; after the second half (when the
// launch sequence goes on), the next step's first-half x_i and scratch.  The next
// x goes to x_out (other rows of this launch still read x_in).  Per step: two
// launches and the detector launch, instead of up to ten.
template <typename real, int LPR, bool QUAD>
__global__ void __launch_bounds__(kWideThreads)
wide_fused_kernel(const StepArgs<real> a, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colidx,
                  const real* __restrict__ val, const real* __restrict__ leak, const real* __restrict__ x_in,
                  real* __restrict__ x_out, const real* __restrict__ cs_in, real* __restrict__ cs_out,
                  const int s_off, const int phase, const int last, const int next) {
    __shared__ real vnew_s[kWideThreads];
    constexpr int GPW = 32 / LPR;
    constexpr int UNROLL = 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t n = a.neuron_start[a.n_neuron];
    const int64_t r0 = ((int64_t)blockIdx.x * (kWideThreads / 32) + warp) * 32;
    if (r0 >= n) return;                                  // the whole warp leaves
    const int q = lane / LPR, l = lane % LPR;
    // Row starts and x of the warp's 32 rows, one coalesced load each (lane k holds
    // row r0 + k), handed to the row groups by shuffles: no row waits for its own
    // row pointer before its propagator loads.
    const int64_t rk = r0 + lane;
    const int64_t beg_k = rowptr[rk < n ? rk : n];
    const int64_t end_32 = rowptr[r0 + 32 < n ? r0 + 32 : n];
    const real x_k = rk < n ? __ldg(x_in + rk) : real(0);
    real* vb = vnew_s + warp * 32;
    for (int g = 0; g < 32; g += GPW) {
        const int64_t r = r0 + g + q;
        const bool valid = r < n;
        const int64_t beg = __shfl_sync(0xffffffffu, beg_k, g + q);
        const int64_t nxt = __shfl_sync(0xffffffffu, beg_k, (g + q + 1) & 31);
        const int64_t end = g + q + 1 < 32 ? nxt : end_32;
        const real xi = __shfl_sync(0xffffffffu, x_k, g + q);
        real s = real(0), c = real(0);
        // UNROLL windows (quads) or 4-entry vectors (rows) per lane are loaded before
        // any is used.
        if (QUAD) {
            for (int64_t k0 = beg + l; k0 < end; k0 += LPR * UNROLL) {
                real v[UNROLL][4];
                int32_t b[UNROLL];
#pragma unroll
                for (int u = 0; u < UNROLL; ++u) {
                    const int64_t k = k0 + LPR * u;
                    if (k < end) {
                        Vec4Loader<real>::load(val + 4 * k, v[u]);
                        b[u] = __ldcs(colidx + k);
                    } else {
                        v[u][0] = v[u][1] = v[u][2] = v[u][3] = real(0);
                        b[u] = 0;
                    }
                }
#pragma unroll
                for (int u = 0; u < UNROLL; ++u) {
                    const real* xb = x_in + b[u];
                    const real p = v[u][0] * (__ldg(xb) - xi) + v[u][1] * (__ldg(xb + 1) - xi);
                    const real t = v[u][2] * (__ldg(xb + 2) - xi) + v[u][3] * (__ldg(xb + 3) - xi);
                    kahan_add(s, c, p + t);
                }
            }
        } else {
            for (int64_t k0 = beg + 4 * l; k0 < end; k0 += 4 * LPR * UNROLL) {
                real v[UNROLL][4];
                int4 cc[UNROLL];
#pragma unroll
                for (int u = 0; u < UNROLL; ++u) {
                    const int64_t k = k0 + 4 * LPR * u;
                    if (k < end) {
                        Vec4Loader<real>::load(val + k, v[u]);
                        cc[u] = __ldcs(reinterpret_cast<const int4*>(colidx + k));
                    } else {
                        v[u][0] = v[u][1] = v[u][2] = v[u][3] = real(0);
                        cc[u] = make_int4(0, 0, 0, 0);
                    }
                }
#pragma unroll
                for (int u = 0; u < UNROLL; ++u) {
                    const real p = v[u][0] * (__ldg(x_in + cc[u].x) - xi) + v[u][1] * (__ldg(x_in + cc[u].y) - xi);
                    const real t = v[u][2] * (__ldg(x_in + cc[u].z) - xi) + v[u][3] * (__ldg(x_in + cc[u].w) - xi);
                    kahan_add(s, c, p + t);
                }
            }
        }
        real t = s - c;
#pragma unroll
        for (int off = LPR / 2; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off, LPR);
        if (l == 0) vb[g + q] = valid ? (xi - leak[r] * xi) + t : real(0);
    }
    __syncwarp();
    const int64_t i = r0 + lane;
    if (i >= n) return;
    const real v = vb[lane];
    if (!isfinite(v)) atomicOr(a.status, kStatusNonFinite);
    a.V[i] = v;
    real cnew = real(0);
    if (a.ca_on) {
        const real si = __ldg(cs_in + i);
        real s = real(0), c = real(0);
        for (int64_t k = a.ca_wrow[i]; k < a.ca_wrow[i + 1]; k += 4) {
            real w[4];
            Vec4Loader<real>::load(a.ca_wval + k, w);
            const int4 cc = __ldcs(reinterpret_cast<const int4*>(a.ca_wcol + k));
            const real p = w[0] * (__ldg(cs_in + cc.x) - si) + w[1] * (__ldg(cs_in + cc.y) - si);
            const real t = w[2] * (__ldg(cs_in + cc.z) - si) + w[3] * (__ldg(cs_in + cc.w) - si);
            kahan_add(s, c, p + t);
        }
        cnew = (si - a.ca_wleak[i] * si) + (s - c);
        if (!isfinite(cnew)) atomicOr(a.status, kStatusNonFinite);
        a.ca_c[i] = cnew;
    }
    if (phase == 0) {
        if (a.hh_on) {
            real m = a.gm[i], h = a.gh[i], nn = a.gn[i];
            hh_gates(v, a.dtq10, m, h, nn);
            a.gm[i] = m; a.gh[i] = h; a.gn[i] = nn;
        }
        for (int qq = 0; qq < a.n_kin; ++qq) kinetic_step(a.kin[qq], i, v);
        if (a.ca_on) calcium_mechanisms(a, i);
    }
    if (phase == 0 || next) {
        // The next half step's x_i: after the first half, the second half of this
        // step; after the second, the first half of the next step.
        const int64_t tick = a.clk->input_ticks + 2 * (int64_t)s_off + (phase == 0 ? 2 : 3);
        real I = a.has_nonspec ? a.Inonspec[i] : real(0);
        if (a.clamp_seg_ptr) {
            for (uint32_t cc = a.clamp_seg_ptr[i]; cc < a.clamp_seg_ptr[i + 1]; ++cc)
                if (tick >= a.clamp_first[cc] && tick < a.clamp_first[cc] + a.clamp_count[cc]) I += a.clamp_amp[cc];
        }
        real G, GE;
        segment_conductance(a, i, G, GE);
        x_out[i] = membrane_x_of(a, i, v, a.kG[i], a.kI[i], G, GE, I, phase == 0 && last != 0);
        if (a.ca_on) cs_out[i] = fmax(real(0), cnew + a.ca_dcdt[i] * a.h_ms);
    }
}

// ------------------------------------------------------------ host side

// The fused half step applies: every conductance source maps one-to-one onto
// segments (HH and kinetic instances in segment order) and there are no synapses.
static bool wide_fusable(const nw_ctx* ctx) {
    if (!ctx->wide_fusion || ctx->syn.n != 0 || (ctx->hh.m != 0 && !ctx->hh.identity)) return false;
    for (int q = 0; q < ctx->n_kin; ++q)
        if (!ctx->kin[q].identity) return false;
    return true;
}

static int wide_lanes(nw_ctx* ctx) {
    if (ctx->lanes_per_row) return ctx->lanes_per_row;
    const double avg = ctx->n_seg ? (double)ctx->nnz_w / (double)ctx->n_seg : 0.0;
    if (avg >= 48) return 16;
    if (avg >= 20) return 8;
    return 4;
}

template <typename real>
static int launch_rows(nw_ctx* ctx, int lanes, const int64_t* R, const int32_t* C, const real* V, const real* L,
                       const real* x, real* y, int* status) {
    const int64_t n = ctx->n_seg;
    const unsigned blocks = (unsigned)((n * lanes + kWideThreads - 1) / kWideThreads);
    switch (lanes) {
        case 4: wide_rows_kernel<real, 4><<<blocks, kWideThreads, 0, ctx->stream>>>(R, C, V, L, x, y, n, status); break;
        case 8: wide_rows_kernel<real, 8><<<blocks, kWideThreads, 0, ctx->stream>>>(R, C, V, L, x, y, n, status); break;
        case 16: wide_rows_kernel<real, 16><<<blocks, kWideThreads, 0, ctx->stream>>>(R, C, V, L, x, y, n, status); break;
        default: wide_rows_kernel<real, 32><<<blocks, kWideThreads, 0, ctx->stream>>>(R, C, V, L, x, y, n, status); break;
    }
    NW_CUDA(ctx, cudaGetLastError());
    return NW_OK;
}

template <typename real>
static int launch_quads(nw_ctx* ctx, const StepArgs<real>& a) {
    const int64_t n = ctx->n_seg;
    const double avg = n ? (double)ctx->nwq / (double)n : 0.0;
    // About 2-4 windows per lane: one round of the kernel's four loads per row.
    const int lanes = ctx->lanes_per_row ? ctx->lanes_per_row : (avg > 32 ? 16 : avg > 12 ? 8 : 4);
    const unsigned blocks = (unsigned)((n * lanes + kWideThreads - 1) / kWideThreads);
    const int64_t* R = ctx->wq_rowptr.as<int64_t>();
    const int32_t* B = ctx->wq_base.as<int32_t>();
    const real* V = ctx->wq_val.as<real>();
    const real* L = ctx->w_leak.as<real>();
    if (a.ca_on) {
        // The calcium rows in the same launch (4 lanes per row, blocks after the voltage rows').
        const unsigned cb = (unsigned)((a.ca_n * 4 + kWideThreads - 1) / kWideThreads);
        switch (lanes) {
            case 4: wide_quads_calcium_kernel<real, 4><<<blocks + cb, kWideThreads, 0, ctx->stream>>>(a, R, B, V, L, blocks); break;
            case 8: wide_quads_calcium_kernel<real, 8><<<blocks + cb, kWideThreads, 0, ctx->stream>>>(a, R, B, V, L, blocks); break;
            case 16: wide_quads_calcium_kernel<real, 16><<<blocks + cb, kWideThreads, 0, ctx->stream>>>(a, R, B, V, L, blocks); break;
            default: wide_quads_calcium_kernel<real, 32><<<blocks + cb, kWideThreads, 0, ctx->stream>>>(a, R, B, V, L, blocks); break;
        }
        NW_CUDA(ctx, cudaGetLastError());
        return NW_OK;
    }
    switch (lanes) {
        case 4: wide_quads_kernel<real, 4><<<blocks, kWideThreads, 0, ctx->stream>>>(R, B, V, L, a.px, a.V, n, a.status); break;
        case 8: wide_quads_kernel<real, 8><<<blocks, kWideThreads, 0, ctx->stream>>>(R, B, V, L, a.px, a.V, n, a.status); break;
        case 16: wide_quads_kernel<real, 16><<<blocks, kWideThreads, 0, ctx->stream>>>(R, B, V, L, a.px, a.V, n, a.status); break;
        default: wide_quads_kernel<real, 32><<<blocks, kWideThreads, 0, ctx->stream>>>(R, B, V, L, a.px, a.V, n, a.status); break;
    }
    NW_CUDA(ctx, cudaGetLastError());
    return NW_OK;
}

template <typename real, int LPR>
static void launch_fused_lpr(nw_ctx* ctx, const StepArgs<real>& a, bool quad, const real* x_in, real* x_out,
                             const real* cs_in, real* cs_out, int s, int phase, int last, int next) {
    const unsigned blocks = (unsigned)((ctx->n_seg + kWideThreads - 1) / kWideThreads);
    if (quad)
        wide_fused_kernel<real, LPR, true><<<blocks, kWideThreads, 0, ctx->stream>>>(
            a, ctx->wq_rowptr.as<int64_t>(), ctx->wq_base.as<int32_t>(), ctx->wq_val.as<real>(),
            ctx->w_leak.as<real>(), x_in, x_out, cs_in, cs_out, s, phase, last, next);
    else
        wide_fused_kernel<real, LPR, false><<<blocks, kWideThreads, 0, ctx->stream>>>(
            a, a.wrow, a.wcol, a.wval, a.wleak, x_in, x_out, cs_in, cs_out, s, phase, last, next);
}

// The fused sequence: the first half's x (and calcium scratch) of the first step
// by the phase kernels, then per step the two fused half steps (x and scratch
// alternating between two buffers) and the detector launch.
template <typename real>
static int enqueue_wide_fused(nw_ctx* ctx, const StepArgs<real>& a, int steps) {
    const int64_t n = ctx->n_seg;
    const unsigned seg_blocks = (unsigned)((n + kWideThreads - 1) / kWideThreads);
    const int64_t cover = std::max<int64_t>(ctx->n_neuron, ctx->n_probes);
    const bool quad = ctx->prop_format == 2 && ctx->wq_ok;
    // Lanes per row by the mean windows (or 4-entry vectors) per row: about 2-4 per
    // lane, so one round of UNROLL loads covers most rows.
    const double avg = n ? (double)(quad ? ctx->nwq : ctx->nnz_w / 4) / (double)n : 0.0;
    const int lanes = ctx->lanes_per_row ? ctx->lanes_per_row : (avg > 32 ? 16 : avg > 12 ? 8 : 4);
    real* x0 = a.px;
    real* x1 = ctx->wide_x2.as<real>();
    real* c0 = a.ca_scratch;
    real* c1 = ctx->wide_cs2.as<real>();
    wide_membrane_kernel<real><<<seg_blocks, kWideThreads, 0, ctx->stream>>>(a, 0, 0, 0);   // x and calcium scratch
    NW_CUDA(ctx, cudaGetLastError());
    for (int s = 0; s < steps; ++s) {
        const int last = s == steps - 1 ? 1 : 0;
        for (int phase = 0; phase < 2; ++phase) {
            const real* xi = phase == 0 ? x0 : x1;
            real* xo = phase == 0 ? x1 : x0;
            const real* ci = phase == 0 ? c0 : c1;
            real* co = phase == 0 ? c1 : c0;
            if (lanes >= 16) launch_fused_lpr<real, 16>(ctx, a, quad, xi, xo, ci, co, s, phase, last, !last);
            else if (lanes == 8) launch_fused_lpr<real, 8>(ctx, a, quad, xi, xo, ci, co, s, phase, last, !last);
            else launch_fused_lpr<real, 4>(ctx, a, quad, xi, xo, ci, co, s, phase, last, !last);
            NW_CUDA(ctx, cudaGetLastError());
        }
        wide_detect_kernel<real><<<(unsigned)((cover + 127) / 128), 128, 0, ctx->stream>>>(a, s);
        NW_CUDA(ctx, cudaGetLastError());
    }
    return NW_OK;
}

// The launches of `steps` steps (no host synchronisation: also a graph body).
template <typename real>
static int enqueue_wide(nw_ctx* ctx, const StepArgs<real>& a, int steps, int lanes) {
    if (wide_fusable(ctx)) return enqueue_wide_fused<real>(ctx, a, steps);
    const int64_t n = ctx->n_seg;
    const unsigned seg_blocks = (unsigned)((n + kWideThreads - 1) / kWideThreads);
    const int64_t n_hh = ctx->hh.m, n_kin = kinetic_instances(ctx), n_syn = ctx->syn.n;
    const int64_t n_mech = n_hh + n_kin + n_syn;
    const int64_t cover = std::max<int64_t>(ctx->n_neuron, ctx->n_probes);
    // HH (one instance per segment) and calcium as the only mechanisms: one launch.
    const bool hh_calcium = a.ca_on && n_kin == 0 && n_syn == 0 && (n_hh == 0 || ctx->hh.identity);
    for (int s = 0; s < steps; ++s) {
        for (int half = 0; half < 2; ++half) {
            const int last = (s == steps - 1 && half == 1) ? 1 : 0;
            // x of every segment and, with calcium, its scratch c + dc/dt h.
            wide_membrane_kernel<real><<<seg_blocks, kWideThreads, 0, ctx->stream>>>(a, s, half, last);
            NW_CUDA(ctx, cudaGetLastError());
            if (ctx->prop_format == 2 && ctx->wq_ok) NW_CHECK(launch_quads<real>(ctx, a));   // + calcium rows
            else NW_CHECK(launch_rows<real>(ctx, lanes, a.wrow, a.wcol, a.wval, a.wleak, a.px, a.V, a.status));
            if (a.ca_on && !(ctx->prop_format == 2 && ctx->wq_ok))
                NW_CHECK(launch_rows<real>(ctx, 4, a.ca_wrow, a.ca_wcol, a.ca_wval, a.ca_wleak, a.ca_scratch, a.ca_c,
                                           a.status));
            if (half == 0 && hh_calcium) {
                wide_hh_calcium_kernel<real><<<seg_blocks, kWideThreads, 0, ctx->stream>>>(a);
                NW_CUDA(ctx, cudaGetLastError());
            } else if (half == 0) {
                if (n_mech > 0) {
                    wide_mechanism_kernel<real><<<(unsigned)((n_mech + kWideThreads - 1) / kWideThreads),
                                                  kWideThreads, 0, ctx->stream>>>(a, s, n_hh, n_kin, n_syn);
                    NW_CUDA(ctx, cudaGetLastError());
                }
                if (a.ca_on) {
                    wide_calcium_mechanism_kernel<real><<<seg_blocks, kWideThreads, 0, ctx->stream>>>(a);
                    NW_CUDA(ctx, cudaGetLastError());
                }
            }
        }
        wide_detect_kernel<real><<<(unsigned)((cover + 127) / 128), 128, 0, ctx->stream>>>(a, s);
        NW_CUDA(ctx, cudaGetLastError());
    }
    return NW_OK;
}

__global__ void wide_set_clock_kernel(DevClock* d, DevClock v) { *d = v; }

static int push_clock_wide(nw_ctx* ctx) {
    DevClock v;
    memset(&v, 0, sizeof(v));
    v.input_ticks = ctx->input_ticks;
    v.steps = ctx->steps;
    v.probe_len = ctx->probe_len;
    v.g_valid = ctx->g_valid ? 1 : 0;
    wide_set_clock_kernel<<<1, 1, 0, ctx->stream>>>(ctx->dclock.as<DevClock>(), v);
    NW_CUDA(ctx, cudaGetLastError());
    return NW_OK;
}

static void key_bytes(std::vector<unsigned char>& key, const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    key.insert(key.end(), b, b + n);
}

// Replays (capturing on first use) the graph of `steps` wide steps.
template <typename real>
static int wide_graph(nw_ctx* ctx, const StepArgs<real>& a0, int steps, int lanes) {
    std::vector<unsigned char> key;
    StepArgs<real> ka = a0;
    ka.tick0 = 0; ka.g_valid = 0; ka.trace_row0 = 0; ka.k_steps = 0;
    const int tag = 0x57494445;   // distinguishes wide-path entries in the shared cache
    key_bytes(key, &tag, sizeof(tag));
    key_bytes(key, &ka, sizeof(ka));
    key_bytes(key, &steps, sizeof(steps));
    key_bytes(key, &lanes, sizeof(lanes));
    key_bytes(key, &ctx->n_seg, sizeof(ctx->n_seg));
    key_bytes(key, &ctx->hh.m, sizeof(ctx->hh.m));
    const int64_t n_kin = kinetic_instances(ctx);
    key_bytes(key, &n_kin, sizeof(n_kin));
    key_bytes(key, &ctx->syn.n, sizeof(ctx->syn.n));
    key_bytes(key, &ctx->ca.on, sizeof(ctx->ca.on));
    key_bytes(key, &ctx->prop_format, sizeof(ctx->prop_format));
    key_bytes(key, &ctx->wq_ok, sizeof(ctx->wq_ok));
    key_bytes(key, &ctx->wq_rowptr.ptr, sizeof(void*));
    key_bytes(key, &ctx->wq_base.ptr, sizeof(void*));
    key_bytes(key, &ctx->wq_val.ptr, sizeof(void*));
    key_bytes(key, &ctx->nwq, sizeof(ctx->nwq));
    const int fused = wide_fusable(ctx) ? 1 : 0;
    key_bytes(key, &fused, sizeof(fused));
    key_bytes(key, &ctx->wide_x2.ptr, sizeof(void*));
    key_bytes(key, &ctx->wide_cs2.ptr, sizeof(void*));
    for (auto& g : ctx->graphs) {
        if (g.key == key) {
            g.last_use = ++ctx->graph_uses;
            NW_CUDA(ctx, cudaGraphLaunch(g.exec, ctx->stream));
            ctx->graph_replays++;
            return NW_OK;
        }
    }
    if (ctx->graphs.size() >= 8) {
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
    const int rc = enqueue_wide<real>(ctx, a0, steps, lanes);
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
    NW_CUDA(ctx, cudaGraphLaunch(ctx->graphs.back().exec, ctx->stream));
    ctx->graph_replays++;
    return NW_OK;
}

template <typename real>
static int wide_steps(nw_ctx* ctx, int k_steps) {
    NW_CHECK(ensure_wide(ctx));
    if (ctx->prop_format == 2 && ctx->n_seg >= 4) NW_CHECK(ensure_wide_quads(ctx));
    if (ctx->ca.on) NW_CHECK(calcium_ensure_wide(ctx));
    if (wide_fusable(ctx)) {
        NW_CHECK(dev_alloc(ctx, ctx->wide_x2, (size_t)ctx->precision * std::max<int64_t>(ctx->n_seg, 1)));
        if (ctx->ca.on)
            NW_CHECK(dev_alloc(ctx, ctx->wide_cs2, (size_t)ctx->precision * std::max<int64_t>(ctx->n_seg, 1)));
    }
    const int lanes = wide_lanes(ctx);
    // Every phase is its own launch, so a spike written by one step's detector
    // launch is visible to every later mechanism launch: no cap by the delays.
    const int G = kWideGraphSteps;
    int done = 0;
    while (done < k_steps) {
        const int steps = std::min(G, k_steps - done);
        const StepArgs<real> a = make_args<real>(ctx, steps);
        NW_CHECK(push_clock_wide(ctx));
        if (ctx->use_graph) NW_CHECK(wide_graph<real>(ctx, a, steps, lanes));
        else NW_CHECK(enqueue_wide<real>(ctx, a, steps, lanes));
        ctx->input_ticks += 2 * (int64_t)steps;
        ctx->steps += steps;
        if (ctx->n_probes) ctx->probe_len += steps;
        if (has_channel_mechanisms(ctx)) ctx->g_valid = true;
        done += steps;
    }
    return NW_OK;
}

int advance_wide(nw_ctx* ctx, int k_steps) {
    return ctx->precision == NW_F64 ? wide_steps<double>(ctx, k_steps) : wide_steps<float>(ctx, k_steps);
}

// Per segment, the summed conductance (S) of the kinetic mechanisms feeding
// `species` at their present state: the species' conductance accumulator as a
// mechanism phase leaves it (neuwon/rxd/species.py:129-133, 155-160).
template <typename real>
__global__ void species_conductance_kernel(const StepArgs<real> a, int32_t species, int32_t feeds_mask,
                                           double* out, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double g = 0.0;
    for (int q = 0; q < a.n_kin; ++q)
        if ((feeds_mask >> q) & 1) g += (double)kinetic_conductance(a.kin[q], i);
    out[i] = g;
}

template <typename real>
static int species_conductance_t(nw_ctx* ctx, int32_t species, double* host) {
    const StepArgs<real> a = make_args<real>(ctx, 1);
    int32_t mask = 0;
    for (int q = 0; q < ctx->n_kin; ++q)
        if (ctx->kin[q].species == species) mask |= 1 << q;
    DevBuf out;
    NW_CHECK(dev_alloc(ctx, out, 8 * ctx->n_seg));
    species_conductance_kernel<real><<<(unsigned)((ctx->n_seg + 255) / 256), 256, 0, ctx->stream>>>(
        a, species, mask, out.as<double>(), ctx->n_seg);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, out.ptr, 8 * ctx->n_seg, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(out);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "nw_species_conductance");
    return NW_OK;
}

int species_conductance(nw_ctx* ctx, int32_t species, double* host_out) {
    return ctx->precision == NW_F64 ? species_conductance_t<double>(ctx, species, host_out)
                                    : species_conductance_t<float>(ctx, species, host_out);
}

}  // namespace nw
