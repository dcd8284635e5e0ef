// Internal declarations shared by the neuwon_gb300 translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/neuwon_gb300.h"

namespace nw {

// One device allocation owned by a context.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    template <typename T> T* as() const { return static_cast<T*>(ptr); }
};

// Largest neuron the batched path keeps in shared memory, per precision,
// and the most clamps one neuron may carry on that path.
constexpr int kMaxClampsPerNeuron = 16;
constexpr int kMaxProbesPerNeuron = 64;

// Fixed-point scales of the pair format's per-segment sums (mV): 2^22 with FP32
// state (32-bit sums), 2^40 with FP64 state (64-bit sums).
constexpr double kPairScaleF32 = 4194304.0;
constexpr double kPairScaleF64 = 1099511627776.0;

// Status bits written by kernels into the context's status word.
constexpr int kStatusNonFinite = 1;
constexpr int kStatusWaitTimeout = 16;   // a bounded wait on an mbarrier gave up

// Simulation clock as the step kernels see it.  The host keeps the
// authoritative copy and writes this one (by value, in stream order) before
// every batched launch sequence, so a captured CUDA graph replays unchanged.
struct DevClock {
    int64_t input_ticks;        // half-step input clock before the sequence
    int64_t steps;              // completed steps before the sequence
    int64_t probe_len;          // probe rows already recorded
    int32_t g_valid;            // mechanism conductances valid at the first half step
    int32_t gc_valid;           // the conductance cache holds G, G*E of the mechanism state
};

// One instantiated CUDA graph of a batched launch sequence, keyed by every
// byte that enters its launches (arguments, launch shape, step count, fusion).
struct GraphEntry {
    std::vector<unsigned char> key;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t last_use = 0;
};

struct HHState {
    int64_t m = 0;              // instances
    bool identity = false;      // instance i sits on segment i for every i
    double ena = 0, ek = 0, el = 0, v_init = -70.0;
    DevBuf seg;                 // u32 [m], segment-sorted order
    DevBuf gm, gh, gn;          // real [m] gates
    DevBuf cna, ck, cl;         // real [m] conductance coefficients (S)
    DevBuf seg_ptr;             // u32 [n_seg+1] instance range of each segment
    DevBuf neuron_ptr;          // i64 [n_neuron+1] instance range of each neuron
    std::vector<int64_t> user_to_sorted;  // registration order -> device order
    std::vector<int64_t> h_neuron_ptr;    // host copy of neuron_ptr
};

// Most kinetic mechanisms (kinds, each with its own scheme, table and instances)
// and most open states per scheme a model may have.
constexpr int kMaxKinetic = 8;
constexpr int kMaxOpen = 8;
constexpr int kMaxTerms = 10;      // polynomial terms of a kinetic table

struct KineticState {
    int64_t m = 0;
    int S = 0, T = 0, nb = 0, n_open = 0;
    int open[kMaxOpen] = {0, 0, 0, 0, 0, 0, 0, 0};
    bool identity = false;
    int species = -1;           // electric species its conductance feeds (-1: nonspecific, own erev)
    double erev = 0, vmin = 0, frq = 0, conserve = 0;
    // Two-input tables (nw_kinetic_inputs): per input its kind (0 voltage, linear;
    // 1 instance value, logarithmic; 2 instance value, linear), buckets, offset
    // (minimum, or log2(minimum + scale)), buckets per unit and log scale; the
    // terms' powers; the instance values.
    int ninp = 1;
    int kind[2] = {0, 0}, nbi[2] = {0, 0};
    double offi[2] = {0, 0}, frqi[2] = {0, 0}, sci[2] = {0, 0};
    signed char pw[kMaxTerms][2] = {};
    DevBuf input;               // real [m] (sorted order)
    DevBuf seg;                 // u32 [m] segment-sorted
    DevBuf state;               // real [S][m]
    DevBuf gcoef;               // real [m]
    DevBuf table;               // real [nb][S][S][T]
    DevBuf seg_ptr;             // u32 [n_seg+1]
    DevBuf neuron_ptr;          // i64 [n_neuron+1]
    std::vector<int64_t> user_to_sorted;
    std::vector<int64_t> h_neuron_ptr;
};

// Synapses with AMPA (C, O) and NMDA (C, O, D) kinetics, driven by spikes of
// their presynaptic neuron after an axonal delay of whole steps.  Spikes are
// kept per neuron in a bit ring of the last ring_steps steps; a synapse pulls
// its arrival from the ring (step - delay), so delivery order cannot vary.
struct SynState {
    int64_t n = 0;
    // Spike-ring partition: the ring covers `ring_neurons` neurons (all ranks' when
    // neurons are split across GPUs) and this model's neuron j is ring entry
    // j + `neuron_offset`; `ring_steps_min` forces a common ring length.
    int64_t ring_neurons = 0, neuron_offset = 0;
    int ring_steps_min = 0;
    int min_delay = 0, max_delay = 0, pulse_steps = 0, ring_steps = 0, ring_words = 0;
    double e_syn = 0, mg = 1.0;
    DevBuf seg;                 // u32 [n] post segment, segment-sorted order
    DevBuf pre;                 // i32 [n] presynaptic neuron
    DevBuf delay;               // i32 [n] steps, >= 1
    DevBuf wa, wn;              // real [n] AMPA / NMDA weights (S)
    DevBuf oa, on, od;          // real [n] AMPA open, NMDA open, NMDA desensitised
    DevBuf pulse_end;           // i32 [n] first step without transmitter
    DevBuf events;              // u32 [n] deliveries so far
    DevBuf last_event;          // i32 [n] step of the last delivery (-1: none)
    DevBuf mats;                // real [26]: AMPA on, off (2x2), NMDA on, off (3x3), row-major
    DevBuf seg_ptr;             // u32 [n_seg+1]
    DevBuf neuron_ptr;          // i64 [n_neuron+1] synapse range of each post neuron
    DevBuf ring;                // u32 [n_neuron][ring_words] spike bits by step mod ring_steps
    std::vector<int64_t> user_to_sorted;
    std::vector<int64_t> h_neuron_ptr;
};

// Intracellular calcium (one diffusing species): concentration per segment,
// its diffusion propagator (same tree builder, same row formats as the
// electric one), a 3-state pump on every segment advanced through a table over
// log2(c + scale), and an influx that is a fraction of the segment's HH sodium
// current.
struct CalciumState {
    bool on = false, pump = false;
    double D = 0, c0 = 0;
    int64_t nnz64 = 0, nnz_b = 0, nnz_w = 0;
    bool b_ok = false, w_ok = false;
    DevBuf res, vol;                            // f64 [n_seg]: 1e-3 L / (D A) and volume (um3)
    DevBuf p_rowptr, p_col, p_val;              // FP64 CSR
    DevBuf b_rowptr, b_col, b_val, b_leak;      // batched format
    DevBuf w_rowptr, w_col, w_val, w_leak;      // wide format
    DevBuf c, dcdt, scratch;                    // real [n_seg]: mM, mM/ms, wide-path scratch
    DevBuf influx, efflux;                      // real [n_seg]: mM/ms per A of Na current, per bound pump fraction
    DevBuf state;                               // real [3][n_seg] pump states (E1, E1Ca, E2)
    DevBuf table;                               // real [nb][3][3][T] ([bucket][col][row][term])
    int nb = 0, T = 0;
    double log2_min = 0, frq = 0, scale = 0;
};

struct AdjointState {
    bool ready = false, g_valid0 = false;
    int K = 0;
    int64_t total_steps = 0, tick0 = 0;
    double loss = 0.0;
    DevBuf ckpt, target, loss_part, tape;
    DevBuf lamV, lamV2, lamM, lamH, lamN;
    DevBuf gGna, gGk, gGl, ra_part;
    DevBuf coef;                // 1/C, C and 1/R per segment in the state precision
    // Backward: the recompute of checkpoint segment k-1 runs on `stream` while the
    // reverse sweep of segment k runs on the context's stream; two tapes by parity.
    cudaStream_t stream = nullptr;
    cudaEvent_t rec_done = nullptr, rev_done[2] = {nullptr, nullptr}, start = nullptr;
};

}  // namespace nw

struct nw_ctx {
    int device = 0;
    int precision = NW_F32;     // bytes per real
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    // nw_advance_host_async: voltages staged on the device (two slots) and copied to
    // the host on a second stream while the next step runs.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t stage_ready[2] = {nullptr, nullptr}, stage_done[2] = {nullptr, nullptr};
    nw::DevBuf vstage[2];
    bool stage_pending[2] = {false, false};
    int stage_slot = 0;

    // Topology.
    int64_t n_seg = 0, n_neuron = 0, max_neuron = 0;
    double time_step = 0.1, celsius = 6.3;
    std::vector<int64_t> h_neuron_start, h_parent;
    nw::DevBuf neuron_start;    // i64 [n_neuron+1]
    nw::DevBuf parent;          // i64 [n_seg]

    // Electric state (context precision) and FP64 passive properties.
    nw::DevBuf V, Vint, Inonspec, kI, kG;
    nw::DevBuf gcache;          // 2 x n_seg reals: G and G*E cached between the steps of one launch
    nw::DevBuf cap64, res64;    // f64 [n_seg]
    bool have_cap = false, have_res = false, nonspec_nonzero = false;

    // Propagator: FP64 CSR with the diagonal (plain path, readback) and the
    // batched difference form (off-diagonal entries, u16 neuron-relative
    // columns, rows padded to 4 entries, per-row leak = 1 - row sum).
    bool prop_valid = false;
    bool prop_built = false;    // built here (detailed balance holds): the pair format may be used
    bool prop_lump = false;     // next build moves dropped values to the nearest kept node (option "propagator_lump")
    bool prop_lumped = false;   // the installed propagator was built with lumping (no detailed balance)
    bool b_ok = false;          // batched format present (every neuron <= 65,535 segments)
    bool w_ok = false;          // wide format present (built on first use of the wide path)
    int64_t nnz64 = 0, nnz_b = 0, nnz_w = 0;
    nw::DevBuf p_rowptr, p_col, p_val;          // i64, i32, f64
    nw::DevBuf b_rowptr, b_col, b_val, b_leak;  // i64, u16, real, real
    nw::DevBuf w_rowptr, w_col, w_val, w_leak;  // i64, i32 (global columns), real, real
    // Pair ("flux") format of the batched path: each coupled pair (i, j) stored
    // once, in the row of the member with the smaller capacitance (the larger
    // P), as w = c_i P_ij / c_max(neuron); both rows receive w (x_j - x_i).
    bool f_ok = false;
    int64_t nnz_f = 0;
    nw::DevBuf f_rowptr, f_col, f_val, f_leak, f_rc;   // i64, u16, real, real, real (c_max / c_i)
    nw::DevBuf f_acc;                                  // i64 [n_seg] accumulators of neurons too large for shared memory
    // Quad format of the batched path: each row's off-diagonal entries covered by
    // windows of 4 consecutive columns (base column + 4 values, zero where a
    // column is not kept); rows with depth-first numbering form long runs.
    bool q_ok = false;
    int64_t nq = 0;
    // Lane count by row length: neurons whose mean quads per row are below
    // lanes_split take half the kernel's lanes per row (0: every neuron the same).
    std::vector<float> h_neuron_qpr;                   // mean quads per row, per neuron
    int64_t lanes_split = 0;
    // The conductance cache (gcache) holds G and G*E of the present mechanism state:
    // set by a batched advance whose kernel ran the fused mechanism pass, cleared by
    // every other entry point that can change the model (its next launch gathers).
    bool gc_valid = false;
    bool rows_claimed = true;   // batched quad rows: warps claim row chunks from a shared counter
    bool prop_walk_once = true;  // tree propagator build: one walk per row into a pool when it fits
    int prop_walks = 0;          // walks per row of the last tree propagator build
    int64_t prop_pool_chunks = 0;   // cap on the pool's chunks (0: a quarter of free memory)
    int64_t narrow_for = -1;                           // lanes_split the flags were made for
    nw::DevBuf neuron_narrow;                          // u8 per neuron
    nw::DevBuf q_rowptr, q_base, q_val;                // i64 (in quads), u16 (neuron-relative), real x 4
    bool wq_ok = false;                                // wide path: global 32-bit bases
    int64_t nwq = 0;
    nw::DevBuf wq_rowptr, wq_base, wq_val;
    // Windows format of the batched path: each row's off-diagonal entries covered
    // by windows of 8, 4, 2 or 1 consecutive columns (u16 neuron-relative base +
    // the window's values).  Per row one block of values (its 8-, 4-, 2- then 1-wide
    // windows' values; blocks start on 4-value boundaries) and one block of bases in
    // the same order; win_row holds per row {value block / 4, first base, n8 | n4 << 16,
    // n2 | n1 << 16}.
    bool win_ok = false;
    int64_t nwin[4] = {0, 0, 0, 0};                    // windows of width 8, 4, 2, 1
    int64_t win_slots = 0;                             // value slots, block padding included
    nw::DevBuf win_row, win_base, win_val;
    int prop_format = 0;                               // 0: rows, 1: pairs, 2: quads, 3: windows
    int pair_shared_limit = -1;                        // cap on neurons with shared-memory sums (-1: none)

    // Mechanisms.  Kinetic mechanisms are kept in registration order; their
    // conductances are summed per segment in that order.
    nw::HHState hh;
    nw::KineticState kin[nw::kMaxKinetic];
    int n_kin = 0;
    // Electric species (neuwon/rxd/species.py:90-142 with a constant reversal
    // potential): a kinetic mechanism's conductance feeds one of them or is
    // nonspecific.
    std::vector<double> species_erev;
    // Duplicate instances on one segment: 0 = all summed, 1 = the reference's
    // fancy-index "+=" for nonspecific conductances (species.py:256-260): only the
    // last-registered instance of a segment counts.
    int duplicates = 0;
    nw::SynState syn;
    int64_t spike_neurons = 0, spike_offset = 0;   // partition settings applied by nw_synapses_set
    int spike_ring_min = 0;
    nw::CalciumState ca;
    nw::AdjointState adj;
    bool g_valid = false;       // conductances computed by a mechanism step

    // Clamps (sorted by neuron, stable).
    int64_t n_clamps = 0;
    std::vector<int64_t> clamp_user_to_sorted;
    nw::DevBuf clamp_seg, clamp_amp, clamp_first, clamp_count, clamp_neuron_ptr;
    nw::DevBuf clamp_seg_ptr;    // u32 [n_seg+1]: clamps are sorted by segment
    nw::DevBuf clamp_amp_stage;  // f64 staging for nw_advance_host

    // Detectors (one per neuron).
    bool have_detectors = false;
    nw::DevBuf det_seg, det_thr, ap_detected, ap_state, spike_count;

    // Probes (sorted by neuron, stable).
    int64_t n_probes = 0, probe_cap = 0, probe_len = 0;
    std::vector<int64_t> probe_user_to_sorted;
    nw::DevBuf probe_seg, probe_neuron_ptr, probe_slot, trace;

    // Batched-path schedule and scratch.
    nw::DevBuf neuron_order;    // i32 [n_neuron], descending work
    nw::DevBuf work_counter;    // i32 [1]
    nw::DevBuf status;          // i32 [1]
    nw::DevBuf plain_x;         // real [n_seg] scratch of the plain path (the wide path's x)
    nw::DevBuf wide_x2, wide_cs2;   // real [n_seg]: the fused wide path's second x / calcium scratch
    bool wide_fusion = false;   // wide path: one launch per half step when mechanisms allow it
    bool adjoint_overlap = true; // backward: recompute of segment k-1 beside the reverse sweep of k
    int lanes_per_row = 0, threads = 1024, ctas_per_sm = 0;
    int fusion = 50;            // steps fused per launch (0: one launch per call)
    bool use_bulk = false;      // asynchronous bulk-copy pipeline (FP32 batched path)
    bool use_graph = true;      // replay batched launch sequences as CUDA graphs
    nw::DevBuf dclock;          // nw::DevClock
    std::vector<nw::GraphEntry> graphs;
    uint64_t graph_uses = 0;
    int64_t graph_captures = 0, graph_replays = 0;

    // Clock.
    int64_t input_ticks = 0, steps = 0;
};

namespace nw {

// Any HH or kinetic instance: after a mechanism phase the conductances are valid.
inline bool has_channel_mechanisms(const nw_ctx* ctx) {
    if (ctx->hh.m > 0) return true;
    for (int q = 0; q < ctx->n_kin; ++q)
        if (ctx->kin[q].m > 0) return true;
    return false;
}

inline int64_t kinetic_instances(const nw_ctx* ctx) {
    int64_t m = 0;
    for (int q = 0; q < ctx->n_kin; ++q) m += ctx->kin[q].m;
    return m;
}

int fail(nw_ctx* ctx, int code, const std::string& msg);
int cuda_fail(nw_ctx* ctx, cudaError_t e, const char* what);
int dev_alloc(nw_ctx* ctx, DevBuf& b, size_t bytes);
void dev_free(DevBuf& b);
size_t dtype_size(int dtype);

// Propagator (nw_propagator.cu).
int propagator_build(nw_ctx* ctx, double tol, int64_t* nnz_out);
int propagator_from_host(nw_ctx* ctx, const int64_t* rowptr, const int64_t* col,
                         const double* val, int64_t nnz);
int propagator_to_batched(nw_ctx* ctx);
int propagator_conserve(nw_ctx* ctx);
int tree_propagator_build(nw_ctx* ctx, const double* d_res, const double* d_cap, double h_s, double tol, int lump,
                          DevBuf& out_rowptr, DevBuf& out_col, DevBuf& out_val, int64_t* nnz_out);
int csr_conserve(nw_ctx* ctx, DevBuf& rowptr, DevBuf& col, DevBuf& val);
template <typename CT>
int csr_to_rows(nw_ctx* ctx, const DevBuf& src_row, const DevBuf& src_col, const DevBuf& src_val, bool relative,
                DevBuf& R, DevBuf& C, DevBuf& V, DevBuf& L, int64_t* nnz_out);

// Stepping (nw_step.cu).
int advance_batched(nw_ctx* ctx, int k_steps);
int advance_plain(nw_ctx* ctx, int k_steps);
int advance_wide(nw_ctx* ctx, int k_steps);
int species_conductance(nw_ctx* ctx, int32_t species, double* host_out);
int ensure_wide(nw_ctx* ctx);
int ensure_flux(nw_ctx* ctx);
int ensure_quads(nw_ctx* ctx);
int ensure_wide_quads(nw_ctx* ctx);
int ensure_windows(nw_ctx* ctx);
int ensure_narrow(nw_ctx* ctx);
void free_quads(nw_ctx* ctx);
void free_flux(nw_ctx* ctx);
void free_wide(nw_ctx* ctx);
int choose_lanes_per_row(nw_ctx* ctx);
bool uses_bulk_pipeline(nw_ctx* ctx);
void graphs_clear(nw_ctx* ctx);
void free_syn(SynState& s);
void free_calcium(CalciumState& c);
int calcium_ensure_wide(nw_ctx* ctx);
int synapse_ring_clear(nw_ctx* ctx);
int prepare_graph(nw_ctx* ctx, int k_steps);
int autotune(nw_ctx* ctx, int trial_steps, int32_t* lanes, int32_t* threads, int32_t* fusion,
             double* ms_per_step);

// Adjoint (nw_adjoint.cu).
int adjoint_forward(nw_ctx* ctx, int64_t T, int K, const double* target, double* loss_out);
int adjoint_backward(nw_ctx* ctx, double Ra, double* g_gna, double* g_gk, double* g_gl, double* g_ra);

// Device conversions (nw_api.cu).
int upload_convert(nw_ctx* ctx, void* dst, int dst_dtype, const void* host, int src_dtype,
                   int64_t count);
int download_convert(nw_ctx* ctx, void* host, int dst_dtype, const void* src, int src_dtype,
                     int64_t count);

}  // namespace nw

#define NW_CUDA(ctx, call)                                              \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return nw::cuda_fail((ctx), e_, #call);  \
    } while (0)

#define NW_CHECK(expr)                  \
    do {                                \
        int rc_ = (expr);               \
        if (rc_ != NW_OK) return rc_;   \
    } while (0)
