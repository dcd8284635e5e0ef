// Batched step kernel of neuwon_gb300 and its launch configuration.
//
// The kernel templates are instantiated only by config_batched<real>, which
// nw_step_f32.cu and nw_step_f64.cu compile in parallel; nw_step.cu launches the
// kernel through the function pointer config_batched returns.
#pragma once
#include <algorithm>
#include <type_traits>

#include "nw_step_common.cuh"

namespace nw {
// ----------------------------------------------------------------------------
// Asynchronous bulk-copy pipeline for the propagator stream (FP32 path).
//
// The rows of a neuron are split among the warps of the CTA into contiguous
// ranges holding about equal numbers of entries, so each warp's part of the
// propagator is one contiguous stream.  Each warp owns a ring of kBulkStages
// shared-memory stages; lane 0 copies the stream in chunks of kBulkChunk
// entries (values, then u16 columns) with cp.async.bulk, completing on the
// stage's mbarrier, kBulkStages chunks ahead of the consumer.  All lanes wait
// on the barrier and consume a chunk row segment by row segment; row ends come
// from a 32-row window of row pointers held one per lane.  Rows are padded to
// multiples of 8 entries, so every copy starts on a 16-byte boundary and moves
// a multiple of 16 bytes, and no 4-entry vector straddles two rows.  Waits are
// bounded: on timeout the kernel records kStatusWaitTimeout and stops.
constexpr int kBulkChunk = 128;
constexpr int kBulkStages = 4;
constexpr uint32_t kWaitLimit = 1u << 20;

template <typename real>
struct BulkGeom {
    static constexpr int kValBytes = kBulkChunk * (int)sizeof(real);
    static constexpr int kStageBytes = kValBytes + kBulkChunk * 2;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

struct BulkRing {
    unsigned char* stages;   // this warp's kBulkStages stages
    uint64_t* bar;           // this warp's kBulkStages mbarriers
    uint32_t seq;            // chunks consumed by this warp since the kernel started
};

// This warp's rows [row_lo, row_hi) and their entries [e0, e1) in one neuron.
struct WarpSlice {
    int row_lo, row_hi;
    int64_t e0, e1;
};

// Entry-balanced split of the neuron's rows among the warps (once per neuron).
template <typename real>
__device__ __forceinline__ WarpSlice warp_slice(const StepArgs<real>& a, int64_t base, int n) {
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int64_t E0 = a.rowptr[base], total = a.rowptr[base + n] - E0;
    auto split = [&](int w) -> int {
        if (w <= 0) return 0;
        if (w >= nw) return n;
        const int64_t target = E0 + (total * w) / nw;
        int lo = 0, hi = n;                     // first row whose start is >= target
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (a.rowptr[base + mid] < target) lo = mid + 1; else hi = mid;
        }
        return lo;
    };
    WarpSlice ws;
    ws.row_lo = split(warp);
    ws.row_hi = split(warp + 1);
    ws.e0 = a.rowptr[base + ws.row_lo];
    ws.e1 = a.rowptr[base + ws.row_hi];
    return ws;
}

template <typename real>
__device__ __forceinline__ void bulk_issue(const StepArgs<real>& a, BulkRing& R, uint32_t seq,
                                           int64_t off, int64_t end) {
    const int stage = (int)(seq % kBulkStages);
    const int len = (int)((end - off) < (int64_t)kBulkChunk ? (end - off) : (int64_t)kBulkChunk);
    unsigned char* dst = R.stages + stage * BulkGeom<real>::kStageBytes;
    const uint32_t bv = (uint32_t)len * (uint32_t)sizeof(real), bc = (uint32_t)len * 2u;
    const uint32_t bar = smem_u32(R.bar + stage);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(bar), "r"(bv + bc) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_u32(dst)), "l"(a.val + off), "r"(bv), "r"(bar) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_u32(dst + BulkGeom<real>::kValBytes)), "l"(a.col + off), "r"(bc), "r"(bar)
                 : "memory");
}

// Lane 0 starts the copies of the first kBulkStages chunks of the warp's stream.
template <typename real>
__device__ __forceinline__ void bulk_prologue(const StepArgs<real>& a, BulkRing& R, const WarpSlice& ws) {
    if ((threadIdx.x & 31) != 0) return;
    uint32_t seq = R.seq;
    for (int k = 0; k < kBulkStages; ++k) {
        const int64_t off = ws.e0 + (int64_t)k * kBulkChunk;
        if (off >= ws.e1) break;
        bulk_issue(a, R, seq++, off, ws.e1);
    }
}

__device__ __forceinline__ bool bulk_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          int* status) {
    const uint32_t b = smem_u32(bar);
    for (uint32_t it = 0; it < kWaitLimit; ++it) {
        uint32_t ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok) : "r"(b), "r"(parity) : "memory");
        if (ok) return true;
        if (*abort_flag) return false;
    }
    atomicOr(status, kStatusWaitTimeout);
    *abort_flag = 1;
    return false;
}

// V_i <- propagator row i applied to xs for the rows of this warp's slice.
template <typename real>
__device__ __forceinline__ void propagate_neuron_bulk(const StepArgs<real>& a, int64_t base,
                                                      const real* __restrict__ xs, BulkRing& R,
                                                      const WarpSlice& ws, volatile int* abort_flag) {
    const int lane = threadIdx.x & 31;
    // Row-end window: lane k holds the end of row win + k.
    int win = ws.row_lo;
    int64_t wend = (win + lane < ws.row_hi) ? a.rowptr[base + win + lane + 1] : ws.e1;
    int row = ws.row_lo;
    int64_t row_end = __shfl_sync(0xffffffffu, wend, 0);
    real s = real(0), c = real(0);
    // Finishes `row` (all of its entries have been summed) and moves to the next one.
    auto finish_row = [&]() {
        real t = s - c;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) {
            const int64_t r = base + row;
            const real xi = xs[row];
            const real vnew = (xi - a.leak[r] * xi) + t;
            if (!isfinite(vnew)) atomicOr(a.status, kStatusNonFinite);
            a.V[r] = vnew;
        }
        s = real(0); c = real(0);
        ++row;
        if (row < ws.row_hi) {
            if (row - win == 32) {
                win = row;
                wend = (win + lane < ws.row_hi) ? a.rowptr[base + win + lane + 1] : ws.e1;
            }
            row_end = __shfl_sync(0xffffffffu, wend, row - win);
        }
    };
    uint32_t seq = R.seq;
    // Rows without off-diagonal entries before the first chunk.
    while (row < ws.row_hi && row_end == ws.e0) finish_row();
    for (int64_t c0 = ws.e0; c0 < ws.e1; c0 += kBulkChunk) {
        const int64_t c1 = (ws.e1 - c0) < (int64_t)kBulkChunk ? ws.e1 : c0 + kBulkChunk;
        const int stage = (int)(seq % kBulkStages);
        // Every lane waits (the barrier's acquire covers its own reads); the vote
        // keeps the warp uniform if a bounded wait gave up in some lanes only.
        const bool ok = __all_sync(0xffffffffu, bulk_wait(R.bar + stage, (seq / kBulkStages) & 1u,
                                                          abort_flag, a.status));
        if (!ok) {
            *abort_flag = 1;
            R.seq = seq;
            return;
        }
        const real* vals = reinterpret_cast<const real*>(R.stages + stage * BulkGeom<real>::kStageBytes);
        const uint16_t* cols = reinterpret_cast<const uint16_t*>(
            R.stages + stage * BulkGeom<real>::kStageBytes + BulkGeom<real>::kValBytes);
        int64_t pos = c0;
        while (pos < c1) {
            const int64_t seg_end = row_end < c1 ? row_end : c1;
            const real xi = xs[row];
            for (int q = (int)(pos - c0) + 4 * lane; q < (int)(seg_end - c0); q += 128) {
                real v[4];
                if (sizeof(real) == 4) {
                    const float4 f = *reinterpret_cast<const float4*>(vals + q);
                    v[0] = f.x; v[1] = f.y; v[2] = f.z; v[3] = f.w;
                } else {
                    v[0] = vals[q]; v[1] = vals[q + 1]; v[2] = vals[q + 2]; v[3] = vals[q + 3];
                }
                const ushort4 cc = *reinterpret_cast<const ushort4*>(cols + q);
                kahan_add(s, c, quad_sum(v, cc, xs, xi));
            }
            pos = seg_end;
            if (pos == row_end) {
                finish_row();
                while (row < ws.row_hi && row_end == pos) finish_row();   // empty rows
            }
        }
        __syncwarp();
        if (lane == 0) {
            const int64_t nxt = c0 + (int64_t)kBulkStages * kBulkChunk;
            if (nxt < ws.e1) bulk_issue(a, R, seq + kBulkStages, nxt, ws.e1);
        }
        ++seq;
    }
    R.seq = seq;
}

// ------------------------------------------------------------ pair format

// Every stored pair (i, j) of a neuron adds t = w (x_j - x_i) to row i and
// subtracts it from row j (w = c_i P_ij / c_max; detailed balance c_i P_ij =
// c_j P_ji), so each coupling is read from HBM once instead of twice.  The
// contributions are summed per segment in fixed point, in mV (scaled by
// c_max / c of the receiving segment), so integer atomic adds give the same
// bits in any order.  FP32 state: 32-bit sums with 2^-22 mV resolution (range
// +-512 mV, checked); FP64 state: 64-bit sums with 2^-40 mV resolution.
template <typename real> struct PairSum;
template <> struct PairSum<float> {
    using acc_t = unsigned int;
    static constexpr float kScale = (float)kPairScaleF32;
    static constexpr float kLimit = 400.0f;                   // |x| beyond this could overflow a sum
    static __device__ __forceinline__ acc_t fix_scaled(float t) { return (acc_t)__float2int_rn(t); }
    static __device__ __forceinline__ float unfix(acc_t q) { return (float)(int)q * (1.0f / kScale); }
};
template <> struct PairSum<double> {
    using acc_t = unsigned long long;
    static constexpr double kScale = kPairScaleF64;
    static constexpr double kLimit = 1e6;
    static __device__ __forceinline__ acc_t fix_scaled(double t) { return (acc_t)__double2ll_rn(t); }
    static __device__ __forceinline__ double unfix(acc_t q) { return (double)(long long)q * (1.0 / kScale); }
};

template <typename real, int LPR>
__device__ __forceinline__ void propagate_flux(const StepArgs<real>& a, int64_t base, int n,
                                               const real* __restrict__ xs, const real* __restrict__ rcs,
                                               typename PairSum<real>::acc_t* acc) {
    using PS = PairSum<real>;
    constexpr int UNROLL = 2;
    constexpr int GPW = 32 / LPR;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int q = lane / LPR, l = lane % LPR;
    for (int rb = warp * GPW; rb < n; rb += nwarps * GPW) {
        const int row = rb + q;
        const bool valid = row < n;
        real s = real(0), c = real(0), xi = real(0);
        if (valid) {
            const int64_t r = base + row;
            const int64_t beg = a.frow[r], end = a.frow[r + 1];
            xi = xs[row];
            for (int64_t k0 = beg + 4 * l; k0 < end; k0 += 4 * LPR * UNROLL) {
                real v[UNROLL][4];
                ushort4 cc[UNROLL];
#pragma unroll
                for (int u = 0; u < UNROLL; ++u) {
                    const int64_t k = k0 + 4 * LPR * u;
                    if (k < end) {
                        Vec4Loader<real>::load(a.fval + k, v[u]);
                        cc[u] = __ldcs(reinterpret_cast<const ushort4*>(a.fcol + k));
                    } else {
                        v[u][0] = v[u][1] = v[u][2] = v[u][3] = real(0);
                        cc[u] = make_ushort4((unsigned short)row, (unsigned short)row, (unsigned short)row,
                                             (unsigned short)row);
                    }
                }
#pragma unroll
                for (int u = 0; u < UNROLL; ++u) {
                    const real t0 = v[u][0] * (xs[cc[u].x] - xi), t1 = v[u][1] * (xs[cc[u].y] - xi);
                    const real t2 = v[u][2] * (xs[cc[u].z] - xi), t3 = v[u][3] * (xs[cc[u].w] - xi);
                    kahan_add(s, c, (t0 + t1) + (t2 + t3));
                    // Padding (w = 0, column = the row) adds zero to the row's own sum.
                    atomicAdd(acc + cc[u].x, PS::fix_scaled(-t0 * rcs[cc[u].x]));
                    atomicAdd(acc + cc[u].y, PS::fix_scaled(-t1 * rcs[cc[u].y]));
                    atomicAdd(acc + cc[u].z, PS::fix_scaled(-t2 * rcs[cc[u].z]));
                    atomicAdd(acc + cc[u].w, PS::fix_scaled(-t3 * rcs[cc[u].w]));
                }
            }
        }
        real t = s - c;
#pragma unroll
        for (int off = LPR / 2; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        if (valid && l == 0) atomicAdd(acc + row, PS::fix_scaled(t * rcs[row]));
    }
}

// V_i = x_i - leak_i x_i + (sum of the pair terms reaching i); resets the sums.
template <typename real>
__device__ __forceinline__ void flux_finalize(const StepArgs<real>& a, int64_t base, int n, const real* xs,
                                              typename PairSum<real>::acc_t* acc) {
    for (int li = threadIdx.x; li < n; li += blockDim.x) {
        const int64_t i = base + li;
        const real xi = xs[li];
        const typename PairSum<real>::acc_t q = acc[li];
        acc[li] = 0;
        const real vnew = (xi - a.fleak[i] * xi) + PairSum<real>::unfix(q);
        if (!isfinite(vnew) || !(fabs(xi) < PairSum<real>::kLimit)) atomicOr(a.status, kStatusNonFinite);
        a.V[i] = vnew;
    }
}

// ------------------------------------------------------------ fused mechanism pass

// The fused pass's register form applies: no kinetic mechanism, or one of 8
// states, 2 terms and one input.
template <typename real>
__device__ __forceinline__ bool fused_fast_form(const StepArgs<real>& a) {
    return a.n_kin == 0 || (a.n_kin == 1 && a.kin[0].S == 8 && a.kin[0].T == 2 && a.kin[0].ninp == 1);
}

// One segment of the fused mechanism pass (instances in segment order): the
// mechanisms at the mid-step voltage v (rxd_model.py:115-123), the segment's
// conductance and G*E (cached for the next step's first half when `keep`), and
// the second half step's x, which it returns (I = the segment's stimulus then).
// Register form: every input of the segment is loaded before the first store,
// and the conductances come from registers through the helpers
// segment_conductance uses, in its order, so the same bits as the general form.
template <typename real>
__device__ __forceinline__ real fused_segment_fast(const StepArgs<real>& a, int64_t i, real v, real I, bool keep,
                                                   bool last1) {
    const KinArgs<real>& K = a.kin[0];
    const bool kin_on = a.n_kin > 0;
    const real kGi = a.kG[i], kIi = a.kI[i];
    real m = real(0), h = real(0), nn = real(0);
    real cna = real(0), ck = real(0), cl = real(0), gco = real(0);
    real st[8];
    if (a.hh_on) {
        m = a.gm[i]; h = a.gh[i]; nn = a.gn[i];
        cna = a.cna[i]; ck = a.ck[i]; cl = a.cl[i];
    }
    if (kin_on) {
#pragma unroll
        for (int c = 0; c < 8; ++c) st[c] = K.state[(int64_t)c * K.m + i];
        gco = K.gcoef[i];
    }
    real G = real(0), GE = real(0);
    if (a.hh_on) {
        hh_gates(v, a.dtq10, m, h, nn);
        real gna = real(0), gk = real(0), gl = real(0);
        hh_conductance_add(cna, ck, cl, m, h, nn, gna, gk, gl);
        hh_conductance_total(a, gna, gk, gl, G, GE);
    }
    if (kin_on) {
        kinetic_advance<real, 8, 2>(K, v, st);
        const real open = kinetic_open(K, [&](int c) {
            real x = st[0];
#pragma unroll
            for (int q = 1; q < 8; ++q) x = (c == q) ? st[q] : x;
            return x;
        });
        real gkin = real(0);
        gkin += gco * open;
        G += gkin;
        GE += gkin * K.erev;
    }
    if (a.hh_on) { a.gm[i] = m; a.gh[i] = h; a.gn[i] = nn; }
    if (kin_on) {
#pragma unroll
        for (int c = 0; c < 8; ++c) K.state[(int64_t)c * K.m + i] = st[c];
    }
    if (keep) { a.gc[i] = G; a.gc[a.gc_n + i] = GE; }
    return membrane_x_of(a, i, v, kGi, kIi, G, GE, I, last1);
}

// The same for any set of one-to-one mechanisms (state through memory).
template <typename real>
__device__ __forceinline__ real fused_segment_general(const StepArgs<real>& a, int64_t i, real v, real I, bool keep,
                                                      bool last1) {
    if (a.hh_on) {
        real m = a.gm[i], h = a.gh[i], nn = a.gn[i];
        hh_gates(v, a.dtq10, m, h, nn);
        a.gm[i] = m; a.gh[i] = h; a.gn[i] = nn;
    }
    for (int q = 0; q < a.n_kin; ++q) kinetic_step(a.kin[q], i, v);
    real G, GE;
    segment_conductance(a, i, G, GE);
    if (keep) { a.gc[i] = G; a.gc[a.gc_n + i] = GE; }
    return membrane_x_of(a, i, v, a.kG[i], a.kI[i], G, GE, I, last1);
}

template <typename real, int LPR, bool BULK, bool FLUX, bool QUAD = false, bool FUSE = false, bool WIN = false>
__global__ void __launch_bounds__(1024)
batched_advance_kernel(const StepArgs<real> a, const int xs_bytes, const int s_off) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    real* xs = reinterpret_cast<real*>(smem_raw);
    // Steps s_off .. s_off + k_steps - 1 of the sequence that starts at the clock.
    const int64_t tick_base = a.clk->input_ticks + 2 * (int64_t)s_off;
    const int64_t row_base = a.clk->probe_len + s_off;
    const int64_t step_base = a.clk->steps + s_off;
    const bool g_valid0 = s_off > 0 || a.clk->g_valid != 0;
    // The fused pass leaves G, G*E in the cache at every step, the last one of a
    // launch included, so a launch's first step reads them too unless the host
    // changed the model since.
    const bool gc_in0 = s_off > 0 || a.clk->gc_valid != 0;
    __shared__ int s_job;
    __shared__ int s_abort;
    BulkRing ring;
    WarpSlice slice;
    if (BULK) {
        const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5;
        unsigned char* rings = smem_raw + xs_bytes;
        uint64_t* bars = reinterpret_cast<uint64_t*>(rings + nw * kBulkStages * BulkGeom<real>::kStageBytes);
        ring.stages = rings + warp * kBulkStages * BulkGeom<real>::kStageBytes;
        ring.bar = bars + warp * kBulkStages;
        ring.seq = 0;
        slice.row_lo = slice.row_hi = 0; slice.e0 = slice.e1 = 0;
        if (threadIdx.x < nw * kBulkStages)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(bars + threadIdx.x)) : "memory");
        if (threadIdx.x == 0) s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        __syncthreads();
    }
    __shared__ int s_nclamp;
    __shared__ int s_rowctr[2];          // quad rows claimed, one counter per half step
    if (QUAD && threadIdx.x == 0) { s_rowctr[0] = 0; s_rowctr[1] = 0; }
    __shared__ uint32_t s_cseg[kMaxClampsPerNeuron];
    __shared__ real s_camp[kMaxClampsPerNeuron];
    __shared__ int64_t s_cfirst[kMaxClampsPerNeuron], s_cend[kMaxClampsPerNeuron];
    const int tid = threadIdx.x, nthr = blockDim.x;

    for (;;) {
        if (tid == 0) s_job = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int job = s_job;
        if (job >= a.n_neuron || (BULK && s_abort)) break;
        const int j = a.neuron_order[job];
        const int64_t base = a.neuron_start[j];
        const int n = (int)(a.neuron_start[j + 1] - base);
        if (QUAD && n < 4) {
            // Quad windows of a neuron of fewer than 4 segments reach past it: zeros there.
            for (int li = n + threadIdx.x; li < 4; li += blockDim.x) xs[li] = real(0);
        }
        if (WIN) {
            // Windows reach up to 7 columns past the neuron's last segment: zeros there.
            for (int li = n + threadIdx.x; li < n + 8; li += blockDim.x) xs[li] = real(0);
        }
        if (FLUX) {
            // c_max / c of the neuron's segments next to x; sums start at zero (the
            // finalize pass leaves them at zero for the next half step).
            using acc_t = typename PairSum<real>::acc_t;
            if (a.frc_smem) {
                // c_max / c times the fixed-point scale: one multiply per pair term.
                real* rc = reinterpret_cast<real*>(smem_raw + xs_bytes);
                for (int li = threadIdx.x; li < n; li += blockDim.x) rc[li] = a.frc[base + li];
            }
            if (n <= a.facc_cap) {
                acc_t* z = reinterpret_cast<acc_t*>(smem_raw + (a.frc_smem ? 2 : 1) * xs_bytes);
                for (int li = threadIdx.x; li < n; li += blockDim.x) z[li] = 0;
            } else {
                acc_t* z = reinterpret_cast<acc_t*>(a.facc) + base;
                for (int li = threadIdx.x; li < n; li += blockDim.x) z[li] = 0;
            }
        }
        if (tid == 0) {
            int c0 = a.clamp_neuron_ptr ? a.clamp_neuron_ptr[j] : 0;
            int c1 = a.clamp_neuron_ptr ? a.clamp_neuron_ptr[j + 1] : 0;
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
        if (BULK) slice = warp_slice(a, base, n);
        // Pair-format accumulators: in shared memory behind x when the neuron fits,
        // else the neuron's slice of a global array (each branch keeps its address
        // space known to the compiler).
        using acc_t = typename PairSum<real>::acc_t;
        const bool acc_in_smem = n <= a.facc_cap;
        const real* const rcs = a.frc_smem ? reinterpret_cast<const real*>(smem_raw + xs_bytes) : a.frc + base;
        acc_t* const sacc = reinterpret_cast<acc_t*>(smem_raw + (a.frc_smem ? 2 : 1) * xs_bytes);
        acc_t* const gacc = reinterpret_cast<acc_t*>(a.facc) + base;
        // Mechanism instance ranges of this neuron (kinetic ones per mechanism, below).
        int64_t ib = 0, ie = 0, yb = 0, ye = 0;
        if (a.syn_on) { yb = a.syn_neuron_ptr[j]; ye = a.syn_neuron_ptr[j + 1]; }
        if (a.hh_on) {
            if (a.hh_identity) { ib = base; ie = base + n; }
            else { ib = a.hh_neuron_ptr[j]; ie = a.hh_neuron_ptr[j + 1]; }
        }
        // With one instance per segment the thread that updates a segment's
        // instances is the one that gathers them next; otherwise synchronise.
        bool mech_sync = (a.hh_on && !a.hh_identity) || ye > yb;
        for (int q = 0; q < a.n_kin; ++q) mech_sync = mech_sync || !a.kin[q].identity;
        // The fused mechanism pass is compiled only into the FUSE instances, so the
        // kernels for synapses, calcium or scattered instances keep their own code.
        const bool fuse = FUSE && !BULK && a.fuse_mech;
        // Stimulus of segment i at a tick: nonspecific current plus the clamps playing.
        auto stim = [&](int64_t i, int64_t tick) {
            real I = a.has_nonspec ? a.Inonspec[i] : real(0);
            for (int c = 0; c < nclamp; ++c)
                if (s_cseg[c] == (uint32_t)i && tick >= s_cfirst[c] && tick < s_cend[c]) I += s_camp[c];
            return I;
        };
        // AP detector state lives in thread 0's registers across the K steps.
        bool ap_state = false, ap_det = false;
        uint32_t spikes = 0;
        if (tid == 0 && a.has_det) {
            ap_state = a.ap_state[j] != 0;
            ap_det = a.ap_detected[j] != 0;
            spikes = a.spike_count[j];
        }
        int pb = 0, pe = 0;
        if (a.n_probes) { pb = a.probe_neuron_ptr[j]; pe = a.probe_neuron_ptr[j + 1]; }

        for (int s = 0; s < a.k_steps; ++s) {
#pragma unroll 1
            for (int half = 0; half < 2; ++half) {
                const int64_t tick = tick_base + 2 * s + half + 1;
                const bool gv = (s > 0) || (half > 0) || g_valid0;
                const bool last = (s == a.k_steps - 1) && (half == 1);
                // The propagator does not depend on x: start streaming it now.
                if (BULK) bulk_prologue(a, ring, slice);
                // With fused mechanisms the second half's x comes from the mechanism
                // pass, and later steps' first halves take G from the cache (the
                // state it was computed from does not change in between).
                if (!(fuse && half == 1)) {
                    for (int li = tid; li < n; li += nthr) {
                        const int64_t i = base + li;
                        real G, GE;
                        if (fuse && (s > 0 || gc_in0)) { G = a.gc[i]; GE = a.gc[a.gc_n + i]; }
                        else if (gv) segment_conductance(a, i, G, GE);
                        else { G = real(0); GE = real(0); }
                        xs[li] = membrane_x(a, i, G, GE, stim(i, tick), last);
                    }
                }
                __syncthreads();
                if (FLUX) {
                    if (acc_in_smem) {
                        propagate_flux<real, LPR>(a, base, n, xs, rcs, sacc);
                        __syncthreads();
                        flux_finalize(a, base, n, xs, sacc);
                    } else {
                        propagate_flux<real, LPR>(a, base, n, xs, rcs, gacc);
                        __syncthreads();
                        flux_finalize(a, base, n, xs, gacc);
                    }
                } else if (QUAD) {
                    auto store = [&](int64_t r, int, real, real vnew) {
                        if (!isfinite(vnew)) atomicOr(a.status, kStatusNonFinite);
                        a.V[r] = vnew;
                    };
                    // Neurons of short rows (mean quads per row below the tuned split)
                    // take half the lanes per row, the others the kernel's LPR.
                    if (a.rows_claimed && !(LPR >= 8 && a.neuron_narrow && a.neuron_narrow[j])) {
                        // This half step's counter starts at zero; the other half's is
                        // reset for its next use (no warp reads it before a barrier).
                        if (tid == 0) s_rowctr[half ^ 1] = 0;
                        propagate_quads_claimed<real, LPR>(a, base, n, xs, store, &s_rowctr[half]);
                    } else if (LPR >= 8 && a.neuron_narrow && a.neuron_narrow[j])
                        propagate_quads<real, (LPR >= 8 ? LPR / 2 : LPR)>(a, base, n, xs, store);
                    else
                        propagate_quads<real, LPR>(a, base, n, xs, store);
                } else if (WIN) {
                    propagate_windows<real, LPR>(a, base, n, xs, [&](int64_t r, int, real, real vnew) {
                        if (!isfinite(vnew)) atomicOr(a.status, kStatusNonFinite);
                        a.V[r] = vnew;
                    });
                } else if (BULK) propagate_neuron_bulk(a, base, xs, ring, slice, &s_abort);
                else propagate_neuron<real, LPR>(a, base, n, xs);
                __syncthreads();
                if (BULK && s_abort) break;
                if (a.ca_on) {
                    // species._advance (species.py:56-70): c <- max(0, c + dcdt h), then diffusion.
                    for (int li = tid; li < n; li += nthr) {
                        const int64_t i = base + li;
                        xs[li] = fmax(real(0), a.ca_c[i] + a.ca_dcdt[i] * a.h_ms);
                    }
                    __syncthreads();
                    propagate_rows_of<real, 4>(a.ca_brow, a.ca_bcol, a.ca_bval, a.ca_bleak, base, n, xs,
                                               [&](int64_t r, int, real, real cnew) { a.ca_c[r] = cnew; });
                    __syncthreads();
                }
                if (half == 0 && fuse) {
                    // Mechanisms (rxd_model.py:115-123) at the mid-step voltage, then
                    // the segment's conductance and the second half's x, in one pass.
                    const bool last1 = s == a.k_steps - 1;
                    const bool keep = true;
                    if (fused_fast_form(a)) {
                        for (int li = tid; li < n; li += nthr) {
                            const int64_t i = base + li;
                            const real v = a.V[i];
                            xs[li] = fused_segment_fast(a, i, v, stim(i, tick + 1), keep, last1);
                        }
                    } else {
                        for (int li = tid; li < n; li += nthr) {
                            const int64_t i = base + li;
                            const real v = a.V[i];
                            xs[li] = fused_segment_general(a, i, v, stim(i, tick + 1), keep, last1);
                        }
                    }
                    __syncthreads();
                } else if (half == 0) {
                    // Mechanisms (rxd_model.py:115-123) at the mid-step voltage.
                    if (a.hh_on) {
                        for (int64_t k = ib + tid; k < ie; k += nthr) {
                            const real v = a.V[a.hh_identity ? k : (int64_t)a.hh_seg[k]];
                            real m = a.gm[k], h = a.gh[k], nn = a.gn[k];
                            hh_gates(v, a.dtq10, m, h, nn);
                            a.gm[k] = m; a.gh[k] = h; a.gn[k] = nn;
                        }
                    }
                    for (int q = 0; q < a.n_kin; ++q) {
                        const KinArgs<real>& K = a.kin[q];
                        const int64_t kb = K.identity ? base : K.neuron_ptr[j];
                        const int64_t ke = K.identity ? base + n : K.neuron_ptr[j + 1];
                        for (int64_t k = kb + tid; k < ke; k += nthr)
                            kinetic_step(K, k, a.V[K.identity ? k : (int64_t)K.seg[k]]);
                    }
                    for (int64_t k = yb + tid; k < ye; k += nthr) synapse_step(a, k, step_base + s);
                    if (mech_sync) __syncthreads();
                    if (a.ca_on) {
                        for (int li = tid; li < n; li += nthr) calcium_mechanisms(a, base + li);
                        __syncthreads();
                    }
                }
            }
            if (BULK && s_abort) break;
            // AP detector (neuron.py:72-75) and probes after the full step.
            if (tid == 0 && a.has_det) {
                const bool over = a.V[a.det_seg[j]] >= a.det_thr[j];
                ap_det = over && !ap_state;
                ap_state = over;
                spikes += ap_det ? 1u : 0u;
                if (a.syn_on) spike_ring_write(a, j, step_base + s, ap_det);
            }
            for (int p = pb + tid; p < pe; p += nthr)
                a.trace[(row_base + s) * a.n_probes + a.probe_slot[p]] = a.V[a.probe_seg[p]];
        }
        if (tid == 0 && a.has_det) {
            a.ap_state[j] = ap_state;
            a.ap_detected[j] = ap_det;
            a.spike_count[j] = spikes;
        }
        __syncthreads();
    }
}

// Launch shape of the batched kernel for the context's current tuning.
template <typename real>
struct BatchedCfg {
    void (*kern)(const StepArgs<real>, int, int);
    unsigned grid;
    int threads;
    size_t smem;
    int xs_bytes;
    int acc_cap;      // pair format: largest neuron whose accumulators fit in shared memory
    int rc_smem;      // pair format: c_max / c staged in shared memory
};

template <typename real, int LPR, bool BULK, bool FLUX, bool QUAD = false, bool FUSE = false, bool WIN = false>
static int config_batched_lpr(nw_ctx* ctx, BatchedCfg<real>& c) {
    auto kern = batched_advance_kernel<real, LPR, BULK, FLUX, QUAD, FUSE, WIN>;
    const size_t xs_bytes = ((size_t)(ctx->max_neuron + (WIN ? 8 : 0)) * sizeof(real) + 127) & ~(size_t)127;
    const int threads = ctx->threads;
    size_t smem = xs_bytes;
    if (BULK) smem += (size_t)(threads / 32) * kBulkStages * (BulkGeom<real>::kStageBytes + 8);
    const size_t static_smem = 4096;
    int acc_cap = 0;
    int rc_smem = 0;
    if (FLUX) {
        // x | c_max / c (when it fits) | pair sums (as many neurons' sums as fit;
        // larger ones use global memory)
        if (2 * xs_bytes + static_smem <= ctx->smem_optin) { smem += xs_bytes; rc_smem = 1; }
        const size_t acc_bytes = sizeof(typename PairSum<real>::acc_t);
        if (smem + static_smem < ctx->smem_optin)
            acc_cap = (int)std::min<int64_t>(ctx->max_neuron, (int64_t)((ctx->smem_optin - static_smem - smem) / acc_bytes));
        if (ctx->pair_shared_limit >= 0) acc_cap = std::min(acc_cap, ctx->pair_shared_limit);
        smem += (size_t)acc_cap * acc_bytes;
    }
    if (smem + static_smem > ctx->smem_optin)
        return fail(ctx, NW_ERR_LIMIT, "batched path: a neuron of " + std::to_string(ctx->max_neuron) +
                                       " segments does not fit in shared memory at this precision");
    NW_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    NW_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem));
    if (occ < 1) return fail(ctx, NW_ERR_LIMIT, "batched path: kernel does not fit on an SM");
    int per_sm = ctx->ctas_per_sm ? std::min(ctx->ctas_per_sm, occ) : occ;
    c.kern = kern;
    c.grid = (unsigned)std::min<int64_t>(ctx->n_neuron, (int64_t)per_sm * ctx->num_sms);
    c.threads = threads;
    c.smem = smem;
    c.xs_bytes = (int)xs_bytes;
    c.acc_cap = acc_cap;
    c.rc_smem = rc_smem;
    return NW_OK;
}

template <typename real>
int config_batched(nw_ctx* ctx, BatchedCfg<real>& c) {
    if (!ctx->b_ok || (ctx->ca.on && !ctx->ca.b_ok))
        return fail(ctx, NW_ERR_LIMIT, "batched path: a neuron has more than 65,535 segments (use the wide path)");
    if (ctx->prop_format == 3) {
        NW_CHECK(ensure_windows(ctx));
        // 16 lanes per row only: the format is kept as a measured alternative (on the
        // bench batch it moves 12 % fewer bytes than quads but issues a third more
        // instructions, and runs slower), so it carries no lane variants.
        return fuse_mechanisms(ctx) ? config_batched_lpr<real, 16, false, false, false, true, true>(ctx, c)
                                    : config_batched_lpr<real, 16, false, false, false, false, true>(ctx, c);
    }
    if (ctx->prop_format == 2) {
        NW_CHECK(ensure_quads(ctx));
        NW_CHECK(ensure_narrow(ctx));
        if (fuse_mechanisms(ctx)) {
            switch (choose_lanes_per_row(ctx)) {
                case 4: return config_batched_lpr<real, 4, false, false, true, true>(ctx, c);
                case 8: return config_batched_lpr<real, 8, false, false, true, true>(ctx, c);
                case 16: return config_batched_lpr<real, 16, false, false, true, true>(ctx, c);
                default: return config_batched_lpr<real, 32, false, false, true, true>(ctx, c);
            }
        }
        switch (choose_lanes_per_row(ctx)) {
            case 4: return config_batched_lpr<real, 4, false, false, true>(ctx, c);
            case 8: return config_batched_lpr<real, 8, false, false, true>(ctx, c);
            case 16: return config_batched_lpr<real, 16, false, false, true>(ctx, c);
            default: return config_batched_lpr<real, 32, false, false, true>(ctx, c);
        }
    }
    if (ctx->prop_format == 1) {
        NW_CHECK(ensure_flux(ctx));
        switch (choose_lanes_per_row(ctx)) {
            case 4: return config_batched_lpr<real, 4, false, true>(ctx, c);
            case 8: return config_batched_lpr<real, 8, false, true>(ctx, c);
            case 16: return config_batched_lpr<real, 16, false, true>(ctx, c);
            default: return config_batched_lpr<real, 32, false, true>(ctx, c);
        }
    }
    if constexpr (std::is_same<real, float>::value) {
        if (uses_bulk_pipeline(ctx)) return config_batched_lpr<float, 32, true, false>(ctx, c);
    }
    switch (choose_lanes_per_row(ctx)) {
        case 4: return config_batched_lpr<real, 4, false, false>(ctx, c);
        case 8: return config_batched_lpr<real, 8, false, false>(ctx, c);
        case 16: return config_batched_lpr<real, 16, false, false>(ctx, c);
        default: return config_batched_lpr<real, 32, false, false>(ctx, c);
    }
}

extern template int config_batched<float>(nw_ctx*, BatchedCfg<float>&);
extern template int config_batched<double>(nw_ctx*, BatchedCfg<double>&);

}  // namespace nw
