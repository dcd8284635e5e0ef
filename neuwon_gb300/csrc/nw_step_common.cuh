// Device building blocks of the time step shared by the forward kernels
// (nw_step.cu) and the adjoint kernels (nw_adjoint.cu).
#pragma once

#include <cstring>
#include <type_traits>

#include "nw_internal.cuh"

namespace nw {

template <typename real> __device__ __forceinline__ real d_exp(real x);
template <> __device__ __forceinline__ float d_exp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double d_exp<double>(double x) { return exp(x); }
template <typename real> __device__ __forceinline__ real d_expm1(real x);
template <> __device__ __forceinline__ float d_expm1<float>(float x) { return expm1f(x); }
template <> __device__ __forceinline__ double d_expm1<double>(double x) { return expm1(x); }

// Forward-mode dual numbers: running the templated mechanism code on Dual<T>
// gives Jacobian-vector products for the adjoint.
template <typename T>
struct Dual {
    T v, d;
    __device__ __forceinline__ Dual() : v(0), d(0) {}
    __device__ __forceinline__ Dual(T x) : v(x), d(0) {}
    __device__ __forceinline__ Dual(T x, T dx) : v(x), d(dx) {}
    __device__ __forceinline__ explicit Dual(double x, int) : v((T)x), d(0) {}
};
template <typename T> __device__ __forceinline__ Dual<T> operator+(Dual<T> a, Dual<T> b) { return Dual<T>(a.v + b.v, a.d + b.d); }
template <typename T> __device__ __forceinline__ Dual<T> operator-(Dual<T> a, Dual<T> b) { return Dual<T>(a.v - b.v, a.d - b.d); }
template <typename T> __device__ __forceinline__ Dual<T> operator-(Dual<T> a) { return Dual<T>(-a.v, -a.d); }
template <typename T> __device__ __forceinline__ Dual<T> operator*(Dual<T> a, Dual<T> b) { return Dual<T>(a.v * b.v, a.d * b.v + a.v * b.d); }
template <typename T> __device__ __forceinline__ Dual<T> operator/(Dual<T> a, Dual<T> b) {
    const T q = a.v / b.v;
    return Dual<T>(q, (a.d - q * b.d) / b.v);
}
template <typename T> __device__ __forceinline__ bool operator<(Dual<T> a, Dual<T> b) { return a.v < b.v; }
__device__ __forceinline__ float d_abs(float a) { return fabsf(a); }
__device__ __forceinline__ double d_abs(double a) { return ::fabs(a); }
template <typename T> __device__ __forceinline__ Dual<T> d_abs(Dual<T> a) { return a.v < T(0) ? -a : a; }
template <typename T> __device__ __forceinline__ Dual<T> d_exp(Dual<T> a) {
    const T e = d_exp(a.v);
    return Dual<T>(e, e * a.d);
}
template <typename T> __device__ __forceinline__ Dual<T> d_expm1(Dual<T> a) {
    return Dual<T>(d_expm1(a.v), d_exp(a.v) * a.d);
}

// FUNCTION vtrap (nmodl_library/artificial/hh.mod:88-94).  x/(exp(x/y)-1) is
// evaluated as x/expm1(x/y), the same quantity without cancellation.
template <typename real>
__device__ __forceinline__ real vtrap(real x, real y) {
    real r = x / y;
    if (d_abs(r) < real(1e-6)) return y * (real(1) - r / real(2));
    return x / d_expm1(r);
}

// rates(v) and the exact gate update x <- xinf + (x - xinf) exp(-dt/xtau)
// (hh.mod:55-86, nmodl/solver.py:48-55); dtq10 = dt * q10, so
// dt/xtau = dtq10 * (alpha + beta).
// Also returns each gate's decay factor exp(-dt/xtau), which is d gate_new /
// d gate_old (the adjoint's Jacobian).
template <typename real>
__device__ __forceinline__ void hh_gates_decay(real v, real dtq10, real& m, real& h, real& n, real& em, real& eh,
                                               real& en) {
    real a = real(0.1) * vtrap(-(v + real(40)), real(10));
    real b = real(4) * d_exp(-(v + real(65)) / real(18));
    real s = a + b, inf = a / s;
    em = d_exp(-dtq10 * s);
    m = inf + (m - inf) * em;
    a = real(0.07) * d_exp(-(v + real(65)) / real(20));
    b = real(1) / (d_exp(-(v + real(35)) / real(10)) + real(1));
    s = a + b; inf = a / s;
    eh = d_exp(-dtq10 * s);
    h = inf + (h - inf) * eh;
    a = real(0.01) * vtrap(-(v + real(55)), real(10));
    b = real(0.125) * d_exp(-(v + real(65)) / real(80));
    s = a + b; inf = a / s;
    en = d_exp(-dtq10 * s);
    n = inf + (n - inf) * en;
}

template <typename real>
__device__ __forceinline__ void hh_gates(real v, real dtq10, real& m, real& h, real& n) {
    real em, eh, en;
    hh_gates_decay(v, dtq10, m, h, n, em, eh, en);
}

// One kinetic mechanism (lti_sim scheme) as the step kernels see it.
template <typename real>
struct KinArgs {
    int identity, S, T, nb, nopen, dup_last;
    int open[kMaxOpen];
    int64_t m;
    const uint32_t* seg_ptr; const int64_t* neuron_ptr; const uint32_t* seg;
    real* state; const real* gcoef; const real* table;
    real vmin, frq, cs, erev;
    // two-input tables (ninp 2): per input kind (0 voltage, 1 instance value on a
    // log2 scale, 2 instance value), buckets, offset, buckets per unit, log scale;
    // term powers; instance values
    int ninp;
    int kind[2], nbi[2];
    real offi[2], frqi[2], sci[2];
    signed char pw[kMaxTerms][2];
    const real* input;
};

template <typename real>
struct StepArgs {
    int64_t n_neuron;
    const int64_t* neuron_start;
    const int32_t* neuron_order;
    int* work_counter;
    int* status;
    real* V; real* Vint;
    const real* kI; const real* kG; const real* Inonspec; int has_nonspec;
    // batched propagator
    const int64_t* rowptr; const uint16_t* col; const real* val; const real* leak;
    // plain propagator
    const int64_t* prow; const int32_t* pcol; const double* pval; real* px;
    // quad propagator: windows of 4 consecutive columns
    const int64_t* qrow; const uint16_t* qbase; const real* qval;
    const uint8_t* neuron_narrow;     // quad rows of these neurons take half the lanes (null: none)
    int rows_claimed;                 // quad rows taken by the warps from a shared counter
    // windows propagator: per row a descriptor {value block / 4, first base,
    // n8 | n4 << 16, n2 | n1 << 16}, the u16 bases and the values
    const uint4* wnrow; const uint16_t* wnbase; const real* wnval;
    // pair ("flux") propagator: rows of owned pairs, leak, c_max / c_i, global accumulators
    const int64_t* frow; const uint16_t* fcol; const real* fval; const real* fleak; const real* frc;
    unsigned long long* facc; int facc_cap; int frc_smem;
    // wide propagator (global int32 columns)
    const int64_t* wrow; const int32_t* wcol; const real* wval; const real* wleak;
    // hh (hh_dup_last: only the last instance of a segment counts, the reference's
    // fancy-index "+=" for nonspecific conductances)
    int hh_on, hh_identity, hh_dup_last;
    const uint32_t* hh_seg_ptr; const int64_t* hh_neuron_ptr; const uint32_t* hh_seg;
    real* gm; real* gh; real* gn; const real* cna; const real* ck; const real* cl;
    real ena, ek, el, dtq10;
    // kinetic schemes (lti_sim), in registration order
    int n_kin;
    KinArgs<real> kin[kMaxKinetic];
    // synapses
    int syn_on, syn_ring_words, syn_ring_mask, syn_pulse;
    const uint32_t* syn_seg_ptr; const int64_t* syn_neuron_ptr;
    const int32_t* syn_pre; const int32_t* syn_delay;
    const real* syn_wa; const real* syn_wn; real* syn_oa; real* syn_on_; real* syn_od;
    int32_t* syn_pulse_end; uint32_t* syn_events; int32_t* syn_last; const real* syn_mats;
    uint32_t* syn_ring; int64_t syn_ring_offset;
    real syn_e, syn_mg357;
    // calcium
    int ca_on, ca_pump, ca_nb, ca_T;
    real* ca_c; real* ca_dcdt; real* ca_scratch; const real* ca_influx; const real* ca_efflux;
    real* ca_state; const real* ca_table;
    const int64_t* ca_brow; const uint16_t* ca_bcol; const real* ca_bval; const real* ca_bleak;
    const int64_t* ca_wrow; const int32_t* ca_wcol; const real* ca_wval; const real* ca_wleak;
    int64_t ca_n;
    real ca_log2min, ca_frq, ca_scale, h_ms;
    // Conductance cache of the batched kernel (G at gc, G*E at gc + n): written by the
    // fused mechanism pass of step s, read by the first half of step s + 1 in the
    // same launch; fuse_mech when every conductance source maps one-to-one onto
    // segments (HH and kinetic instances in segment order, no synapses or calcium).
    real* gc; int64_t gc_n; int fuse_mech;
    // clamps (sorted by segment)
    const uint32_t* clamp_seg_ptr;
    const int32_t* clamp_neuron_ptr; const uint32_t* clamp_seg; const real* clamp_amp;
    const int64_t* clamp_first; const int64_t* clamp_count;
    // detectors
    int has_det;
    const uint32_t* det_seg; const real* det_thr;
    uint8_t* ap_detected; uint8_t* ap_state; uint32_t* spike_count;
    // probes
    const int32_t* probe_neuron_ptr; const uint32_t* probe_seg; const uint32_t* probe_slot;
    real* trace; int64_t n_probes; int64_t trace_row0;
    // time: the batched kernel reads the clock from clk (device), the
    // plain and adjoint kernels from tick0 / g_valid / trace_row0
    const DevClock* clk;
    int64_t tick0; int k_steps; int g_valid; real h_s;
};

// Sum of a segment's mechanism conductances and conductance-weighted reversal
// potentials (species.py:256-260 scatter, done here as a gather over the
// segment's instances in registration order: deterministic, no atomics).
// One HH instance's conductances added to the segment's running sums.
template <typename real>
__device__ __forceinline__ void hh_conductance_add(real cna, real ck, real cl, real m, real h, real n,
                                                   real& gna, real& gk, real& gl) {
    gna += cna * m * m * m * h;
    gk += ck * n * n * n * n;
    gl += cl;
}

// Sum of the conductances and conductance-weighted reversal potentials of HH.
template <typename real>
__device__ __forceinline__ void hh_conductance_total(const StepArgs<real>& a, real gna, real gk, real gl,
                                                     real& G, real& GE) {
    G = (gna + gk) + gl;
    GE = (gna * a.ena + gk * a.ek) + gl * a.el;
}

// A kinetic instance's open probability: its open states summed in list order.
template <typename real, typename Get>
__device__ __forceinline__ real kinetic_open(const KinArgs<real>& K, Get state) {
    real open = real(0);
    for (int o = 0; o < K.nopen; ++o) open += state(K.open[o]);
    return open;
}

// The conductance (S) of kinetic mechanism K's instances on segment i.
template <typename real>
__device__ __forceinline__ real kinetic_conductance(const KinArgs<real>& K, int64_t i) {
    real gkin = real(0);
    auto add = [&](int64_t k) {
        const real open = kinetic_open(K, [&](int s) { return K.state[(int64_t)s * K.m + k]; });
        gkin += K.gcoef[k] * open;
    };
    if (K.identity) add(i);
    else {
        const int64_t b = K.seg_ptr[i], e = K.seg_ptr[i + 1];
        if (K.dup_last) { if (e > b) add(e - 1); }
        else for (int64_t k = b; k < e; ++k) add(k);
    }
    return gkin;
}

template <typename real>
__device__ __forceinline__ void segment_conductance(const StepArgs<real>& a, int64_t i, real& G, real& GE) {
    G = real(0); GE = real(0);
    if (a.hh_on) {
        real gna = real(0), gk = real(0), gl = real(0);
        if (a.hh_identity) {
            hh_conductance_add(a.cna[i], a.ck[i], a.cl[i], a.gm[i], a.gh[i], a.gn[i], gna, gk, gl);
        } else {
            const int64_t e = a.hh_seg_ptr[i + 1];
            const int64_t b = a.hh_dup_last && e > a.hh_seg_ptr[i] ? e - 1 : a.hh_seg_ptr[i];
            for (int64_t k = b; k < e; ++k)
                hh_conductance_add(a.cna[k], a.ck[k], a.cl[k], a.gm[k], a.gh[k], a.gn[k], gna, gk, gl);
        }
        hh_conductance_total(a, gna, gk, gl, G, GE);
    }
    for (int q = 0; q < a.n_kin; ++q) {
        const real gkin = kinetic_conductance(a.kin[q], i);
        G += gkin;
        GE += gkin * a.kin[q].erev;
    }
    if (a.syn_on) {
        const uint32_t b = a.syn_seg_ptr[i], e = a.syn_seg_ptr[i + 1];
        if (b < e) {
            // NMDA magnesium block at the segment's present voltage (Jahr & Stevens 1990).
            const real block = real(1) / (real(1) + d_exp(real(-0.062) * a.V[i]) * a.syn_mg357);
            real gs = real(0);
            for (uint32_t k = b; k < e; ++k) gs += a.syn_wa[k] * a.syn_oa[k] + a.syn_wn[k] * a.syn_on_[k] * block;
            G += gs;
            GE += gs * a.syn_e;
        }
    }
}

// One synapse through step s_abs: a spike of its presynaptic neuron at step
// s_abs - delay (read from that neuron's spike ring) arrives now and keeps
// transmitter present for syn_pulse steps; then the exact per-step update of the
// AMPA (C, O) and NMDA (C, O, D) schemes with the transmitter present or absent.
template <typename real>
__device__ __forceinline__ void synapse_step(const StepArgs<real>& a, int64_t k, int64_t s_abs) {
    const int64_t src = s_abs - a.syn_delay[k];
    bool arrive = false;
    if (src >= 0) {
        const uint32_t slot = (uint32_t)(src & a.syn_ring_mask);
        const uint32_t w = __ldcg(a.syn_ring + (int64_t)a.syn_pre[k] * a.syn_ring_words + (slot >> 5));
        arrive = ((w >> (slot & 31u)) & 1u) != 0u;
    }
    int32_t pe = a.syn_pulse_end[k];
    if (arrive) {
        pe = (int32_t)(s_abs + a.syn_pulse);
        a.syn_pulse_end[k] = pe;
        a.syn_events[k] += 1u;
        a.syn_last[k] = (int32_t)s_abs;
    }
    const bool on = s_abs < (int64_t)pe;
    const real* Ma = a.syn_mats + (on ? 0 : 4);
    const real oa = a.syn_oa[k];
    a.syn_oa[k] = Ma[2] * (real(1) - oa) + Ma[3] * oa;
    const real* Mn = a.syn_mats + 8 + (on ? 0 : 9);
    const real o = a.syn_on_[k], d = a.syn_od[k];
    const real c = (real(1) - o) - d;
    a.syn_on_[k] = Mn[3] * c + Mn[4] * o + Mn[5] * d;
    a.syn_od[k] = Mn[6] * c + Mn[7] * o + Mn[8] * d;
}

template <typename real> __device__ __forceinline__ real d_log2(real x);
template <> __device__ __forceinline__ float d_log2<float>(float x) { return log2f(x); }
template <> __device__ __forceinline__ double d_log2<double>(double x) { return log2(x); }

// Calcium of segment i through the mechanism phase: the pump's 3 states advance
// one step at the present concentration (table over log2(c + scale), bucket and
// in-bucket location as lti_sim's LogarithmicInput and codegen compute them,
// neuwon/rxd/lti_sim/inputs.py:85-109, codegen.py:43-106, then renormalised),
// and the concentration's rate of change for this step: influx = a fraction of
// the segment's HH sodium current, efflux = transport from the bound state.
template <typename real>
__device__ __forceinline__ void calcium_mechanisms(const StepArgs<real>& a, int64_t i) {
    const real v = a.V[i];
    real d = real(0);
    if (a.hh_on) {
        int64_t b, e;
        if (a.hh_identity) { b = i; e = i + 1; }
        else { b = a.hh_seg_ptr[i]; e = a.hh_seg_ptr[i + 1]; }
        real ina = real(0);
        for (int64_t k = b; k < e; ++k) {
            const real m = a.gm[k], h = a.gh[k];
            ina += a.cna[k] * m * m * m * h * (v - a.ena);
        }
        d = -a.ca_influx[i] * ina;
    }
    if (a.ca_pump) {
        const real c = a.ca_c[i];
        real x = (d_log2(c + a.ca_scale) - a.ca_log2min) * a.ca_frq;
        int b = (int)x;
        real loc = x - (real)b;
        if (b > a.ca_nb - 1) { b = a.ca_nb - 1; loc = real(1); }
        if (b < 0 || !(x == x)) { b = 0; loc = real(0); }
        const int T = a.ca_T;
        const real* tb = a.ca_table + (int64_t)b * 9 * T;
        const int64_t n = a.ca_n;
        real st[3] = {a.ca_state[i], a.ca_state[n + i], a.ca_state[2 * n + i]};
        real out[3] = {real(0), real(0), real(0)};
        for (int col = 0; col < 3; ++col) {
            for (int row = 0; row < 3; ++row) {
                const real* t = tb + (col * 3 + row) * T;
                real poly = t[T - 1];
                for (int k = T - 2; k >= 0; --k) poly = poly * loc + t[k];
                out[row] += poly * st[col];
            }
        }
        const real inv = real(1) / ((out[0] + out[1]) + out[2]);
        a.ca_state[i] = out[0] * inv;
        a.ca_state[n + i] = out[1] * inv;
        a.ca_state[2 * n + i] = out[2] * inv;
        d -= a.ca_efflux[i] * (out[1] * inv);
    }
    a.ca_dcdt[i] = d;
}

// The AP detector's output for step s_abs into the neuron's spike ring (the
// neuron's own CTA is the only writer of its words).
template <typename real>
__device__ __forceinline__ void spike_ring_write(const StepArgs<real>& a, int64_t j, int64_t s_abs, bool spike) {
    const uint32_t slot = (uint32_t)(s_abs & a.syn_ring_mask);
    uint32_t* wp = a.syn_ring + (j + a.syn_ring_offset) * a.syn_ring_words + (slot >> 5);
    const uint32_t bit = 1u << (slot & 31u);
    const uint32_t w = __ldcg(wp);
    *wp = spike ? (w | bit) : (w & ~bit);
}

// Voltage -> (bucket, location within it) as the generated lti_sim kernel
// computes them (codegen.py:43-59): bucket = trunc((v - vmin) * frq), clamped to
// the table, location 1 above it and 0 below it.  Non-finite voltages land in bucket 0.
template <typename real>
__device__ __forceinline__ int kinetic_locate(const KinArgs<real>& K, real v, real& loc) {
    real x = (v - K.vmin) * K.frq;
    if (!(x > real(-2))) x = real(-2);
    if (x > real(K.nb + 1)) x = real(K.nb + 1);
    int b = (int)x;
    if (b > K.nb - 1) { b = K.nb - 1; loc = real(1); }
    else if (b < 0) { b = 0; loc = real(0); }
    else loc = x - real(b);
    return b;
}

// One exact-integration step of a kinetic instance (codegen.py:60-106): the
// polynomial approximation of the column-normalised propagator, evaluated per
// (col, row) as table[bucket][col][row][term], times the state, then CONSERVE.
// FP32 linear tables with an even number of states are read as 16-byte vectors
// (two rows' terms per load; the same arithmetic in the same order).
template <typename real, int S, int T>
__device__ __forceinline__ void kinetic_advance(const KinArgs<real>& K, real v, real (&st)[S]) {
    real loc;
    const int b = kinetic_locate(K, v, loc);
    real basis[T];
    basis[0] = real(1);
#pragma unroll
    for (int t = 1; t < T; ++t) basis[t] = basis[t - 1] * loc;
    const real* __restrict__ tb = K.table + (int64_t)b * (S * S * T);
    real out[S];
#pragma unroll
    for (int c = 0; c < S; ++c) out[c] = real(0);
    if constexpr (std::is_same<real, float>::value && T == 2 && S % 2 == 0) {
#pragma unroll
        for (int col = 0; col < S; ++col) {
#pragma unroll
            for (int row = 0; row < S; row += 2) {
                const float4 q = __ldg(reinterpret_cast<const float4*>(tb + (col * S + row) * 2));
                real p0 = real(0) + q.x;
                p0 += basis[1] * q.y;
                out[row] += p0 * st[col];
                real p1 = real(0) + q.z;
                p1 += basis[1] * q.w;
                out[row + 1] += p1 * st[col];
            }
        }
    } else {
#pragma unroll
        for (int col = 0; col < S; ++col) {
#pragma unroll
            for (int row = 0; row < S; ++row) {
                const real* p = tb + (col * S + row) * T;
                real poly = real(0) + __ldg(p);
#pragma unroll
                for (int t = 1; t < T; ++t) poly += basis[t] * __ldg(p + t);
                out[row] += poly * st[col];
            }
        }
    }
    if (K.cs > real(0)) {
        real sum = out[0];
#pragma unroll
        for (int c = 1; c < S; ++c) sum += out[c];
        const real f = K.cs / sum;
#pragma unroll
        for (int c = 0; c < S; ++c) out[c] *= f;
    }
#pragma unroll
    for (int c = 0; c < S; ++c) st[c] = out[c];
}

template <typename real, int S, int T>
__device__ __forceinline__ void kinetic_step_fixed(const KinArgs<real>& K, int64_t k, real v) {
    real st[S];
#pragma unroll
    for (int c = 0; c < S; ++c) st[c] = K.state[(int64_t)c * K.m + k];
    kinetic_advance<real, S, T>(K, v, st);
#pragma unroll
    for (int c = 0; c < S; ++c) K.state[(int64_t)c * K.m + k] = st[c];
}

// Same step for any S <= 16 and T <= 4.
template <typename real>
__device__ __noinline__ void kinetic_step_generic(const KinArgs<real>& K, int64_t k, real v) {
    const int S = K.S, T = K.T;
    real loc;
    const int b = kinetic_locate(K, v, loc);
    real basis[kMaxTerms];
    basis[0] = real(1);
    for (int t = 1; t < T; ++t) basis[t] = basis[t - 1] * loc;
    const real* tb = K.table + (int64_t)b * (S * S * T);
    real st[16], out[16];
    for (int c = 0; c < S; ++c) { st[c] = K.state[(int64_t)c * K.m + k]; out[c] = real(0); }
    for (int col = 0; col < S; ++col)
        for (int row = 0; row < S; ++row) {
            const real* p = tb + (col * S + row) * T;
            real poly = real(0) + p[0];
            for (int t = 1; t < T; ++t) poly += basis[t] * p[t];
            out[row] += poly * st[col];
        }
    if (K.cs > real(0)) {
        real sum = out[0];
        for (int c = 1; c < S; ++c) sum += out[c];
        const real f = K.cs / sum;
        for (int c = 0; c < S; ++c) out[c] *= f;
    }
    for (int c = 0; c < S; ++c) K.state[(int64_t)c * K.m + k] = out[c];
}

// One input of a two-input table -> (bucket, location), as the generated lti_sim
// kernel locates it (codegen.py:43-59): LinearInput (value - minimum) * frq,
// LogarithmicInput (log2(value + scale) - log2(minimum + scale)) * frq; clamped
// to the table like the voltage (location 1 above it, 0 below it).
template <typename real>
__device__ __forceinline__ int kinetic_locate_input(const KinArgs<real>& K, int d, real value, real& loc) {
    real x = K.kind[d] == 1 ? (d_log2(value + K.sci[d]) - K.offi[d]) * K.frqi[d] : (value - K.offi[d]) * K.frqi[d];
    const int nb = K.nbi[d];
    if (!(x > real(-2))) x = real(-2);
    if (x > real(nb + 1)) x = real(nb + 1);
    int b = (int)x;
    if (b > nb - 1) { b = nb - 1; loc = real(1); }
    else if (b < 0) { b = 0; loc = real(0); }
    else loc = x - real(b);
    return b;
}

// One step of an instance of a two-input table (lti_sim's Approx2D,
// neuwon/rxd/lti_sim/approx.py:242-337, run as codegen.py:60-106 runs it): table
// [b1][b2][col][row][term], term t = loc1^pw[t][0] * loc2^pw[t][1] (products taken
// factor by factor, as the generated code writes them).
template <typename real>
__device__ __noinline__ void kinetic_step_2d(const KinArgs<real>& K, int64_t k, real v) {
    const int S = K.S, T = K.T;
    const real u = K.input[k];
    real loc[2];
    int b[2];
    for (int d = 0; d < 2; ++d) b[d] = kinetic_locate_input(K, d, K.kind[d] == 0 ? v : u, loc[d]);
    real basis[kMaxTerms];
    for (int t = 0; t < T; ++t) {
        real x = real(1);
        for (int p = 0; p < K.pw[t][0]; ++p) x = p == 0 ? loc[0] : x * loc[0];
        for (int p = 0; p < K.pw[t][1]; ++p) x = (p == 0 && K.pw[t][0] == 0) ? loc[1] : x * loc[1];
        basis[t] = x;
    }
    const real* tb = K.table + ((int64_t)b[0] * K.nbi[1] + b[1]) * (S * S * T);
    real st[16], out[16];
    for (int c = 0; c < S; ++c) { st[c] = K.state[(int64_t)c * K.m + k]; out[c] = real(0); }
    for (int col = 0; col < S; ++col)
        for (int row = 0; row < S; ++row) {
            const real* p = tb + (col * S + row) * T;
            real poly = real(0);
            for (int t = 0; t < T; ++t) poly += (K.pw[t][0] == 0 && K.pw[t][1] == 0) ? p[t] : basis[t] * p[t];
            out[row] += poly * st[col];
        }
    if (K.cs > real(0)) {
        real sum = out[0];
        for (int c = 1; c < S; ++c) sum += out[c];
        const real f = K.cs / sum;
        for (int c = 0; c < S; ++c) out[c] *= f;
    }
    for (int c = 0; c < S; ++c) K.state[(int64_t)c * K.m + k] = out[c];
}

// Unrolled instances for the shapes of the schemes this package defines
// (8-state sodium, 6-state Nav1.1 / Kv1.1 with linear tables); others generic.
template <typename real>
__device__ __forceinline__ void kinetic_step(const KinArgs<real>& K, int64_t k, real v) {
    if (K.ninp == 2) kinetic_step_2d(K, k, v);
    else if (K.S == 8 && K.T == 2) kinetic_step_fixed<real, 8, 2>(K, k, v);
    else if (K.S == 6 && K.T == 2) kinetic_step_fixed<real, 6, 2>(K, k, v);
    else kinetic_step_generic(K, k, v);
}

// Exact exponential membrane update of one segment (electric.py:60-76).
template <typename real>
__device__ __forceinline__ real membrane_x_of(const StepArgs<real>& a, int64_t i, real v, real kG, real kI,
                                              real G, real GE, real I, bool store_integral) {
    real E = (G != real(0)) ? GE / G : real(0);          // nan_to_num(GE/G), rxd_model.py:106-109
    real expo = -kG * G;
    real alpha = d_exp(expo);
    real dv = kI * I;
    real diff = E - v;
    real x = E - diff * alpha + dv;
    if (store_integral) a.Vint[i] = a.h_s * E - expo * diff * alpha + real(0.5) * a.h_s * dv;
    return x;
}

template <typename real>
__device__ __forceinline__ real membrane_x(const StepArgs<real>& a, int64_t i, real G, real GE, real I,
                                           bool store_integral) {
    return membrane_x_of(a, i, a.V[i], a.kG[i], a.kI[i], G, GE, I, store_integral);
}

// Propagator entries are streamed once per half step and do not fit in L2, so
// they are loaded with the evict-first (streaming) cache hint.
template <typename real> struct Vec4Loader;
template <> struct Vec4Loader<float> {
    static __device__ __forceinline__ void load(const float* p, float (&v)[4]) {
        float4 q = __ldcs(reinterpret_cast<const float4*>(p));
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    }
};
template <> struct Vec4Loader<double> {
    static __device__ __forceinline__ void load(const double* p, double (&v)[4]) {
        double2 q0 = __ldcs(reinterpret_cast<const double2*>(p));
        double2 q1 = __ldcs(reinterpret_cast<const double2*>(p) + 1);
        v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
    }
};

template <typename real> struct Vec2Loader;
template <> struct Vec2Loader<float> {
    static __device__ __forceinline__ void load(const float* p, float (&v)[2]) {
        float2 q = __ldcs(reinterpret_cast<const float2*>(p));
        v[0] = q.x; v[1] = q.y;
    }
};
template <> struct Vec2Loader<double> {
    static __device__ __forceinline__ void load(const double* p, double (&v)[2]) {
        double2 q = __ldcs(reinterpret_cast<const double2*>(p));
        v[0] = q.x; v[1] = q.y;
    }
};

template <typename real>
__device__ __forceinline__ void kahan_add(real& s, real& c, real term) {
    real y = term - c;
    real t = s + y;
    c = (t - s) - y;
    s = t;
}

// Four entries of a row: sum of P_ij (x_j - x_i), added pairwise; the running
// row sum around it is compensated (kahan_add), so the dependent chain per lane
// is one compensated add per 4 entries.
template <typename real>
__device__ __forceinline__ real quad_sum(const real (&v)[4], const ushort4 cc, const real* __restrict__ xs,
                                         real xi) {
    const real a = v[0] * (xs[cc.x] - xi) + v[1] * (xs[cc.y] - xi);
    const real b = v[2] * (xs[cc.z] - xi) + v[3] * (xs[cc.w] - xi);
    return a + b;
}

// Row i of the propagator applied to xs for every row of one neuron; fin(r, row, xi, y)
// receives y = sum_j P_ij xs_j for the global row r.
template <typename real, int LPR, int UNROLL = (LPR >= 16 ? 4 : 2), typename Fin>
__device__ __forceinline__ void propagate_rows_of(const int64_t* __restrict__ rowptr, const uint16_t* __restrict__ col,
                                                  const real* __restrict__ val, const real* __restrict__ leak,
                                                  int64_t base, int n, const real* __restrict__ xs, Fin fin) {
    constexpr int GPW = 32 / LPR;                  // row groups per warp
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
            const int64_t beg = rowptr[r], end = rowptr[r + 1];
            xi = xs[row];
            // UNROLL chunks of 4 entries per lane are loaded before any is consumed,
            // to keep enough bytes in flight per SM for HBM latency.
            for (int64_t k0 = beg + 4 * l; k0 < end; k0 += 4 * LPR * UNROLL) {
                real v[UNROLL][4];
                ushort4 cc[UNROLL];
#pragma unroll
                for (int u = 0; u < UNROLL; ++u) {
                    const int64_t k = k0 + 4 * LPR * u;
                    if (k < end) {
                        Vec4Loader<real>::load(val + k, v[u]);
                        cc[u] = __ldcs(reinterpret_cast<const ushort4*>(col + k));
                    } else {
                        v[u][0] = v[u][1] = v[u][2] = v[u][3] = real(0);
                        cc[u] = make_ushort4(0, 0, 0, 0);
                    }
                }
#pragma unroll
                for (int u = 0; u < UNROLL; ++u)
                    kahan_add(s, c, quad_sum(v[u], cc[u], xs, xi));
            }
        }
        real t = s - c;
#pragma unroll
        for (int off = LPR / 2; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        if (valid && l == 0) {
            const int64_t r = base + row;
            fin(r, row, xi, (xi - leak[r] * xi) + t);
        }
    }
}

template <typename real, int LPR, int UNROLL = (LPR >= 16 ? 4 : 2), typename Fin>
__device__ __forceinline__ void propagate_rows(const StepArgs<real>& a, int64_t base, int n,
                                               const real* __restrict__ xs, Fin fin) {
    propagate_rows_of<real, LPR, UNROLL>(a.rowptr, a.col, a.val, a.leak, base, n, xs, fin);
}

// Quad format: row i is a list of windows (base b, values v0..v3 for columns
// b..b+3); the window's four x are consecutive in shared memory (neurons of
// fewer than 4 segments keep zeros in x[n..3]).
//
// One row r of a row group of LPR lanes (lane l of the group; every lane of the
// warp calls this, valid or not): sum over the row's windows of P_ij (x_j - x_i),
// each lane taking every LPR-th window with UNROLL windows loaded before any is
// used, compensated lane sums reduced over the group, so every lane of the
// group returns the row's sum.
template <typename real, int LPR, int UNROLL>
__device__ __forceinline__ real quad_row_sum(const StepArgs<real>& a, bool valid, int64_t r, int l,
                                             const real* __restrict__ xs, real xi) {
    real s = real(0), c = real(0);
    if (valid) {
        const int64_t beg = a.qrow[r], end = a.qrow[r + 1];
        for (int64_t k0 = beg + l; k0 < end; k0 += LPR * UNROLL) {
            real v[UNROLL][4];
            int b[UNROLL];
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                const int64_t k = k0 + LPR * u;
                if (k < end) {
                    Vec4Loader<real>::load(a.qval + 4 * k, v[u]);
                    b[u] = __ldcs(a.qbase + k);
                } else {
                    v[u][0] = v[u][1] = v[u][2] = v[u][3] = real(0);
                    b[u] = 0;                         // zero weights on x[0..3]
                }
            }
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                const real* x = xs + b[u];
                const real p = v[u][0] * (x[0] - xi) + v[u][1] * (x[1] - xi);
                const real t = v[u][2] * (x[2] - xi) + v[u][3] * (x[3] - xi);
                kahan_add(s, c, p + t);
            }
        }
    }
    real t = s - c;
#pragma unroll
    for (int off = LPR / 2; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    return t;
}

// Rows of a neuron taken by the warps from a shared counter (ctr, zero at the
// phase's start) in chunks of kRowChunk row groups, each warp claiming its next
// chunk before it works on the current one; a row's sum is the same whichever
// warp computes it.
constexpr int kRowChunk = 2;
template <typename real, int LPR, int UNROLL = (LPR >= 16 ? 4 : 2), typename Fin>
__device__ __forceinline__ void propagate_quads_claimed(const StepArgs<real>& a, int64_t base, int n,
                                                        const real* __restrict__ xs, Fin fin, int* ctr) {
    constexpr int GPW = 32 / LPR;
    const int lane = threadIdx.x & 31;
    const int q = lane / LPR, l = lane % LPR;
    int next = 0;
    if (lane == 0) next = atomicAdd(ctr, kRowChunk * GPW);
    next = __shfl_sync(0xffffffffu, next, 0);
    while (next < n) {
        const int cur = next;
        if (lane == 0) next = atomicAdd(ctr, kRowChunk * GPW);
#pragma unroll 1
        for (int c = 0; c < kRowChunk; ++c) {
            const int row = cur + c * GPW + q;
            const bool valid = row < n;
            const int64_t r = base + row;
            const real xi = valid ? xs[row] : real(0);
            const real t = quad_row_sum<real, LPR, UNROLL>(a, valid, r, l, xs, xi);
            if (valid && l == 0) fin(r, row, xi, (xi - a.leak[r] * xi) + t);
        }
        next = __shfl_sync(0xffffffffu, next, 0);
    }
}

template <typename real, int LPR, int UNROLL = (LPR >= 16 ? 4 : 2), typename Fin>
__device__ __forceinline__ void propagate_quads(const StepArgs<real>& a, int64_t base, int n,
                                                const real* __restrict__ xs, Fin fin) {
    constexpr int GPW = 32 / LPR;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int q = lane / LPR, l = lane % LPR;
    for (int rb = warp * GPW; rb < n; rb += nwarps * GPW) {
        const int row = rb + q;
        const bool valid = row < n;
        const int64_t r = base + row;
        const real xi = valid ? xs[row] : real(0);
        const real t = quad_row_sum<real, LPR, UNROLL>(a, valid, r, l, xs, xi);
        if (valid && l == 0) fin(r, row, xi, (xi - a.leak[r] * xi) + t);
    }
}

// Windows format: row i is a list of windows of widths 8, 4, 2 and 1 (base b,
// values for columns b..b+w-1), stored as one contiguous block of values and one
// of bases.  The row's windows form one list of items of at most 4 values: an
// 8-wide window is two items (its halves), the others one each, so items t < e4
// are 4 values at 4t in the block; the row's lanes take consecutive items, UNROLL
// items per lane loaded before any is used (as in the quad format), and every item
// is summed as a 4-column window with zero weights past its width.  Windows may
// reach 7 columns past the neuron's last segment, where x holds zeros.
template <typename real, int LPR, int UNROLL = (LPR >= 16 ? 4 : 2), typename Fin>
__device__ __forceinline__ void propagate_windows(const StepArgs<real>& a, int64_t base, int n,
                                                  const real* __restrict__ xs, Fin fin) {
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
            const uint4 d = __ldg(a.wnrow + r);
            const real* __restrict__ vb = a.wnval + 4 * (int64_t)d.x;
            const uint16_t* __restrict__ bb = a.wnbase + d.y;
            const uint32_t n8 = d.z & 0xffffu;
            const uint32_t e8 = 2 * n8, e4 = e8 + (d.z >> 16), e2 = e4 + (d.w & 0xffffu), e1 = e2 + (d.w >> 16);
            xi = xs[row];
            for (uint32_t t0 = l; t0 < e1; t0 += LPR * UNROLL) {
                real v[UNROLL][4];
                int b[UNROLL];
#pragma unroll
                for (int u = 0; u < UNROLL; ++u) {
                    const uint32_t t = t0 + LPR * u;
                    v[u][0] = v[u][1] = v[u][2] = v[u][3] = real(0);
                    b[u] = 0;                                 // zero weights on x[0..3]
                    if (t < e4) {
                        Vec4Loader<real>::load(vb + 4 * t, v[u]);
                        b[u] = t < e8 ? __ldcs(bb + (t >> 1)) + 4 * (int)(t & 1) : __ldcs(bb + (t - n8));
                    } else if (t < e2) {
                        real w2[2];
                        Vec2Loader<real>::load(vb + 4 * e4 + 2 * (t - e4), w2);
                        v[u][0] = w2[0]; v[u][1] = w2[1];
                        b[u] = __ldcs(bb + (t - n8));
                    } else if (t < e1) {
                        v[u][0] = __ldcs(vb + 4 * e4 + 2 * (e2 - e4) + (t - e2));
                        b[u] = __ldcs(bb + (t - n8));
                    }
                }
#pragma unroll
                for (int u = 0; u < UNROLL; ++u) {
                    const real* x = xs + b[u];
                    const real p = v[u][0] * (x[0] - xi) + v[u][1] * (x[1] - xi);
                    const real t = v[u][2] * (x[2] - xi) + v[u][3] * (x[3] - xi);
                    kahan_add(s, c, p + t);
                }
            }
        }
        real t = s - c;
#pragma unroll
        for (int off = LPR / 2; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        if (valid && l == 0) {
            const int64_t r = base + row;
            fin(r, row, xi, (xi - a.leak[r] * xi) + t);
        }
    }
}

// V_i <- propagator row i applied to xs, for every row of one neuron.
template <typename real, int LPR>
__device__ __forceinline__ void propagate_neuron(const StepArgs<real>& a, int64_t base, int n,
                                                 const real* __restrict__ xs) {
    propagate_rows<real, LPR>(a, base, n, xs, [&](int64_t r, int, real, real vnew) {
        if (!isfinite(vnew)) atomicOr(a.status, kStatusNonFinite);
        a.V[r] = vnew;
    });
}


// The batched kernel's fused mechanism pass applies: every conductance source maps
// one-to-one onto segments (HH and kinetic instances in segment order, no synapses,
// no calcium) and the conductance cache exists.
inline bool fuse_mechanisms(const nw_ctx* ctx) {
    if (!ctx->gcache.ptr || ctx->syn.n != 0 || ctx->ca.on || (ctx->hh.m != 0 && !ctx->hh.identity)) return false;
    for (int q = 0; q < ctx->n_kin; ++q)
        if (!ctx->kin[q].identity) return false;
    return true;
}

template <typename real>
inline StepArgs<real> make_args(nw_ctx* ctx, int k_steps) {
    StepArgs<real> a;
    memset(&a, 0, sizeof(a));      // padding bytes too: the struct is a graph-cache key
    a.n_neuron = ctx->n_neuron;
    a.neuron_start = ctx->neuron_start.as<int64_t>();
    a.neuron_order = ctx->neuron_order.as<int32_t>();
    a.work_counter = ctx->work_counter.as<int>();
    a.status = ctx->status.as<int>();
    a.V = ctx->V.as<real>(); a.Vint = ctx->Vint.as<real>();
    a.kI = ctx->kI.as<real>(); a.kG = ctx->kG.as<real>();
    a.Inonspec = ctx->Inonspec.as<real>(); a.has_nonspec = ctx->nonspec_nonzero ? 1 : 0;
    a.rowptr = ctx->b_rowptr.as<int64_t>(); a.col = ctx->b_col.as<uint16_t>();
    a.val = ctx->b_val.as<real>(); a.leak = ctx->b_leak.as<real>();
    a.prow = ctx->p_rowptr.as<int64_t>(); a.pcol = ctx->p_col.as<int32_t>(); a.pval = ctx->p_val.as<double>();
    a.px = ctx->plain_x.as<real>();
    a.qrow = ctx->q_rowptr.as<int64_t>(); a.qbase = ctx->q_base.as<uint16_t>(); a.qval = ctx->q_val.as<real>();
    a.neuron_narrow = (ctx->lanes_split > 0 && ctx->narrow_for == ctx->lanes_split)
                          ? ctx->neuron_narrow.as<uint8_t>() : nullptr;
    a.rows_claimed = ctx->rows_claimed ? 1 : 0;
    if (ctx->win_ok) {
        a.wnrow = ctx->win_row.as<uint4>();
        a.wnbase = ctx->win_base.as<uint16_t>(); a.wnval = ctx->win_val.as<real>();
    }
    a.frow = ctx->f_rowptr.as<int64_t>(); a.fcol = ctx->f_col.as<uint16_t>();
    a.fval = ctx->f_val.as<real>(); a.fleak = ctx->f_leak.as<real>(); a.frc = ctx->f_rc.as<real>();
    a.facc = ctx->f_acc.as<unsigned long long>();
    a.wrow = ctx->w_rowptr.as<int64_t>(); a.wcol = ctx->w_col.as<int32_t>();
    a.wval = ctx->w_val.as<real>(); a.wleak = ctx->w_leak.as<real>();
    const HHState& hh = ctx->hh;
    a.hh_on = hh.m > 0 ? 1 : 0;
    a.hh_identity = hh.identity ? 1 : 0;
    a.hh_seg_ptr = hh.seg_ptr.as<uint32_t>(); a.hh_neuron_ptr = hh.neuron_ptr.as<int64_t>();
    a.hh_seg = hh.seg.as<uint32_t>();
    a.gm = hh.gm.as<real>(); a.gh = hh.gh.as<real>(); a.gn = hh.gn.as<real>();
    a.cna = hh.cna.as<real>(); a.ck = hh.ck.as<real>(); a.cl = hh.cl.as<real>();
    a.ena = (real)hh.ena; a.ek = (real)hh.ek; a.el = (real)hh.el;
    a.hh_dup_last = ctx->duplicates == 1 ? 1 : 0;
    a.n_kin = ctx->n_kin;
    for (int q = 0; q < ctx->n_kin; ++q) {
        const KineticState& K = ctx->kin[q];
        KinArgs<real>& k = a.kin[q];
        k.identity = K.identity ? 1 : 0;
        k.dup_last = (ctx->duplicates == 1 && K.species < 0) ? 1 : 0;
        k.S = K.S; k.T = K.T; k.nb = K.nb; k.nopen = K.n_open;
        for (int o = 0; o < kMaxOpen; ++o) k.open[o] = K.open[o];
        k.m = K.m;
        k.seg_ptr = K.seg_ptr.as<uint32_t>(); k.neuron_ptr = K.neuron_ptr.as<int64_t>();
        k.seg = K.seg.as<uint32_t>();
        k.state = K.state.as<real>(); k.gcoef = K.gcoef.as<real>(); k.table = K.table.as<real>();
        k.vmin = (real)K.vmin; k.frq = (real)K.frq; k.cs = (real)K.conserve; k.erev = (real)K.erev;
        k.ninp = K.ninp;
        for (int d = 0; d < 2; ++d) {
            k.kind[d] = K.kind[d]; k.nbi[d] = K.nbi[d];
            k.offi[d] = (real)K.offi[d]; k.frqi[d] = (real)K.frqi[d]; k.sci[d] = (real)K.sci[d];
        }
        for (int t = 0; t < kMaxTerms; ++t) { k.pw[t][0] = K.pw[t][0]; k.pw[t][1] = K.pw[t][1]; }
        k.input = K.ninp == 2 ? K.input.as<real>() : nullptr;
    }
    const CalciumState& Ca = ctx->ca;
    a.ca_on = Ca.on ? 1 : 0;
    a.gc = ctx->gcache.as<real>(); a.gc_n = ctx->n_seg;
    a.fuse_mech = fuse_mechanisms(ctx) ? 1 : 0;
    a.h_ms = (real)(0.5 * ctx->time_step);
    if (Ca.on) {
        a.ca_pump = Ca.pump ? 1 : 0; a.ca_nb = Ca.nb; a.ca_T = Ca.T;
        a.ca_c = Ca.c.as<real>(); a.ca_dcdt = Ca.dcdt.as<real>(); a.ca_scratch = Ca.scratch.as<real>();
        a.ca_influx = Ca.influx.as<real>(); a.ca_efflux = Ca.efflux.as<real>();
        a.ca_state = Ca.state.as<real>(); a.ca_table = Ca.table.as<real>();
        a.ca_brow = Ca.b_rowptr.as<int64_t>(); a.ca_bcol = Ca.b_col.as<uint16_t>();
        a.ca_bval = Ca.b_val.as<real>(); a.ca_bleak = Ca.b_leak.as<real>();
        a.ca_wrow = Ca.w_rowptr.as<int64_t>(); a.ca_wcol = Ca.w_col.as<int32_t>();
        a.ca_wval = Ca.w_val.as<real>(); a.ca_wleak = Ca.w_leak.as<real>();
        a.ca_log2min = (real)Ca.log2_min; a.ca_frq = (real)Ca.frq; a.ca_scale = (real)Ca.scale;
        a.ca_n = ctx->n_seg;
    }
    const SynState& Y = ctx->syn;
    a.syn_on = Y.n > 0 ? 1 : 0;
    if (Y.n > 0) {
        a.syn_ring_words = Y.ring_words; a.syn_ring_mask = Y.ring_steps - 1; a.syn_pulse = Y.pulse_steps;
        a.syn_seg_ptr = Y.seg_ptr.as<uint32_t>(); a.syn_neuron_ptr = Y.neuron_ptr.as<int64_t>();
        a.syn_pre = Y.pre.as<int32_t>(); a.syn_delay = Y.delay.as<int32_t>();
        a.syn_wa = Y.wa.as<real>(); a.syn_wn = Y.wn.as<real>();
        a.syn_oa = Y.oa.as<real>(); a.syn_on_ = Y.on.as<real>(); a.syn_od = Y.od.as<real>();
        a.syn_pulse_end = Y.pulse_end.as<int32_t>(); a.syn_events = Y.events.as<uint32_t>();
        a.syn_last = Y.last_event.as<int32_t>(); a.syn_mats = Y.mats.as<real>();
        a.syn_ring = Y.ring.as<uint32_t>(); a.syn_ring_offset = Y.neuron_offset;
        a.syn_e = (real)Y.e_syn; a.syn_mg357 = (real)(Y.mg / 3.57);
    }
    const double q10 = pow(3.0, (ctx->celsius - 6.3) / 10.0);      // hh.mod:67
    a.dtq10 = (real)(ctx->time_step * q10);
    if (ctx->n_clamps) {
        a.clamp_neuron_ptr = ctx->clamp_neuron_ptr.as<int32_t>();
        a.clamp_seg_ptr = ctx->clamp_seg_ptr.as<uint32_t>();
        a.clamp_seg = ctx->clamp_seg.as<uint32_t>(); a.clamp_amp = ctx->clamp_amp.as<real>();
        a.clamp_first = ctx->clamp_first.as<int64_t>(); a.clamp_count = ctx->clamp_count.as<int64_t>();
    }
    a.has_det = ctx->have_detectors ? 1 : 0;
    a.det_seg = ctx->det_seg.as<uint32_t>(); a.det_thr = ctx->det_thr.as<real>();
    a.ap_detected = ctx->ap_detected.as<uint8_t>(); a.ap_state = ctx->ap_state.as<uint8_t>();
    a.spike_count = ctx->spike_count.as<uint32_t>();
    a.n_probes = ctx->n_probes;
    if (ctx->n_probes) {
        a.probe_neuron_ptr = ctx->probe_neuron_ptr.as<int32_t>();
        a.probe_seg = ctx->probe_seg.as<uint32_t>(); a.probe_slot = ctx->probe_slot.as<uint32_t>();
        a.trace = ctx->trace.as<real>(); a.trace_row0 = ctx->probe_len;
    }
    a.clk = ctx->dclock.as<DevClock>();
    a.tick0 = ctx->input_ticks;
    a.k_steps = k_steps;
    a.g_valid = ctx->g_valid ? 1 : 0;
    a.h_s = (real)(0.5 * ctx->time_step * 1e-3);
    return a;
}

// Lanes per propagator row (measured on GB300 with ~490 entries/row: 16 lanes and
// 1,024 threads beat 32 lanes; 8 lanes is too few for such rows).

}  // namespace nw
