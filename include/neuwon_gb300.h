/*
 * neuwon_gb300 -- C ABI of the GB300 (sm_103a) implementation of NEUWON's
 * per-time-step hot path, the staggered Model.advance().
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and
 * returns an int status: NW_OK (0) or a negative NW_ERR_* code.  After an
 * error, nw_last_error() gives a one-line description.  A context owns one
 * CUDA device, one stream and the device mirror of the model's
 * structure-of-arrays; calls on one context are not thread-safe (the
 * reference is single-threaded too).  Host pointers passed in are only read
 * during the call unless stated otherwise.
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the reference project).
 */
#ifndef NEUWON_GB300_H
#define NEUWON_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nw_ctx nw_ctx;

/* Status codes. */
#define NW_OK            0
#define NW_ERR_ARG      -1   /* bad argument (size, name, range)             */
#define NW_ERR_CUDA     -2   /* CUDA runtime error                           */
#define NW_ERR_STATE    -3   /* call made in the wrong order                 */
#define NW_ERR_NOMEM    -4   /* device allocation failed                     */
#define NW_ERR_NUMERIC  -5   /* a kernel flagged a non-finite voltage        */
#define NW_ERR_LIMIT    -6   /* a size exceeds what the library supports    */

/* Arithmetic precision of a context's state and step kernels. */
#define NW_F32 4
#define NW_F64 8

/* Element types for nw_set_data / nw_get_data. */
#define NW_DTYPE_F64 1
#define NW_DTYPE_F32 2
#define NW_DTYPE_I64 3
#define NW_DTYPE_I32 4
#define NW_DTYPE_U32 5
#define NW_DTYPE_U8  6

/* Step implementations for nw_advance. */
#define NW_PATH_BATCHED 0   /* persistent fused K-step kernel, one CTA per neuron */
#define NW_PATH_PLAIN   1   /* per-neuron launches, one thread per row/instance  */
#define NW_PATH_WIDE    2   /* whole-model launches per half step, rows spread over all
                               SMs: neurons of any size (no shared-memory or 65,535 limit) */

/* ---- context -------------------------------------------------------- */

/* Replaces the reference's memory-space switch (neuwon/database/memory_spaces.py:14-35,
 * Database.using_memory_space database.py:122-154): one device, one stream. */
int nw_ctx_create(int device, int precision, nw_ctx** out);
int nw_ctx_destroy(nw_ctx* ctx);
/* Copies the last error message (NUL-terminated, truncated to len). */
int nw_last_error(nw_ctx* ctx, char* buf, int len);
/* Version of this library (major*10000 + minor*100 + patch). */
int nw_version(void);
/* The context's CUDA stream, as a cudaStream_t stored into *stream. */
int nw_get_stream(nw_ctx* ctx, void** stream);
int nw_synchronize(nw_ctx* ctx);

/* ---- model structure ------------------------------------------------ */

/* Segment tree of all neurons (neuwon/rxd/neuron/segment.py:11-25 "parent",
 * neuron.py:11-12 sort_key='neuron').  Segments are in the reference's sorted
 * order: neurons contiguous, neuron k owning [neuron_start[k], neuron_start[k+1]).
 * parent[i] is a global segment index or -1 for a root; parents precede children.
 * time_step is the model dt in ms (rxd_model.py:9); the electric half step is dt/2. */
int nw_model_init(nw_ctx* ctx, int64_t num_segments, int64_t num_neurons,
                  const int64_t* neuron_start, const int64_t* parent,
                  double time_step_ms, double celsius);

/* Replaces Database.get_data / set_data (database.py, data_components.py:318-333)
 * for the device-resident attributes.  name is "Class.attribute":
 *   Segment.voltage, Segment.integral_voltage, Segment.capacitance,
 *   Segment.axial_resistance, Segment.nonspecific_current,
 *   hh.m, hh.h, hh.n, hh.gna_coef, hh.gk_coef, hh.gl_coef (instance order as registered),
 *   kinetic.<q>.state (kinetic mechanism q: num_instances * S values,
 *   [instance][state], registration order; "kinetic.state" is mechanism 0),
 *   Neuron.AP_detected, Neuron.spike_count.
 * Values are converted between dtype and the context precision. */
int nw_set_data(nw_ctx* ctx, const char* name, const void* host, int dtype, int64_t count);
int nw_get_data(nw_ctx* ctx, const char* name, void* host, int dtype, int64_t count);

/* ---- propagator ----------------------------------------------------- */

/* Replaces Segment._compute_propagator_matrix (neuwon/rxd/neuron/electric.py:78-117):
 * builds expm(coef * dt/2) for every neuron in FP64 on the GPU from the device copies
 * of parent, axial_resistance and capacitance, prunes |p| < prune_tolerance (the
 * reference hard-codes machine epsilon, electric.py:114), and stores it for both
 * step paths.  *nnz_out receives the number of kept entries (diagonal included). */
int nw_propagator_build(nw_ctx* ctx, double prune_tolerance, int64_t* nnz_out);

/* Replaces DB_Class "electric_propagator_matrix" set_data (data_components.py:611-622):
 * install an FP64 CSR propagator computed elsewhere (global indices, n x n). */
int nw_propagator_set_csr(nw_ctx* ctx, int64_t n, const int64_t* rowptr,
                          const int64_t* col, const double* val, int64_t nnz);

/* Charge-conserving pruning: returns the pruned mass of every row of the installed
 * propagator to its diagonal, so each row sums to 1 again.  The unpruned matrix has
 * unit row sums (the reference tests this charge conservation,
 * neuwon/rxd/tests/test_electric.py:84-85); pruning without this correction
 * (the reference's own behaviour, electric.py:114-115) leaks voltage toward 0 mV
 * at coarse tolerances.  Requires a stored diagonal entry in every row. */
int nw_propagator_conserve(nw_ctx* ctx);

/* Reads the FP64 propagator back as CSR (rowptr[n+1], col[nnz], val[nnz]);
 * pass NULL arrays to query *nnz_out only. */
int nw_propagator_get_csr(nw_ctx* ctx, int64_t* rowptr, int64_t* col, double* val,
                          int64_t* nnz_out);

/* ---- mechanisms ----------------------------------------------------- */

/* Registers the instances of the Hodgkin-Huxley mechanism
 * (nmodl_library/artificial/hh.mod as compiled by neuwon/rxd/nmodl/__init__.py:28-63,
 * Mechanism API neuwon/rxd/mechanisms.py:4-54).  segment[i] is instance i's segment;
 * g*_coef[i] are its conductance coefficients in siemens (gbar[S/cm2] * 1e-8 *
 * magnitude[um2], nmodl/__init__.py:99-107, 404-406); e* are the reversal potentials
 * of the three nonspecific conductances (mV).  Gates start at their steady state at
 * v_init, as the INITIAL block does. */
int nw_hh_register(nw_ctx* ctx, int64_t num_instances, const int64_t* segment,
                   const double* gna_coef, const double* gk_coef, const double* gl_coef,
                   double ena, double ek, double el, double v_init);

/* Electric species with a constant reversal potential: replaces the accumulators of
 * _SpeciesType (neuwon/rxd/species.py:85-142, 155-160), whose per-segment
 * {name}_conductance sums feed the segment's total conductance and
 * conductance-weighted driving voltage with the species' reversal potential.
 * Species are numbered 0..count-1 in the order given; kinetic mechanisms name the
 * species their conductance feeds (nw_kinetic_add).  Calling it again replaces the
 * reversal potentials (mechanisms already registered take the new values). */
int nw_species_set(nw_ctx* ctx, int32_t count, const double* reversal_potential_mV);

/* A species' {name}_conductance accumulator (species.py:129-133) as the last mechanism
 * phase leaves it: per segment (device order, n_seg values, S), the summed
 * conductance of the kinetic mechanisms that feed the species. */
int nw_species_conductance(nw_ctx* ctx, int32_t species, double* conductance_out);

/* Appends one linear kinetic mechanism solved by exact integration with a voltage
 * table (lti_sim: neuwon/rxd/lti_sim/lti_model.py:5-65, approx.py:159-174,
 * codegen.py:29-106; NMODL "SOLVE ... METHOD sparse", nmodl/__init__.py:298-306), one
 * of the mechanisms _advance_mechanisms advances (neuwon/rxd/rxd_model.py:115-123);
 * a model holds up to 8, advanced and summed per segment in the order added.
 *   num_states S (1..16), open_states: 1..8 indices whose sum is the open probability;
 *   g_coef[i]: instance i's maximal conductance in siemens (gbar * 1e-8 * magnitude);
 *   species: the electric species (nw_species_set) whose conductance accumulator it
 *   writes (USEION, nmodl/__init__.py:168-208), or -1 for a nonspecific conductance
 *   with reversal potential erev (mV; ignored when species >= 0);
 *   table: [num_buckets][S (col)][S (row)][num_terms] polynomial coefficients, the
 *   layout of codegen.py:35-37; the voltage v falls in bucket trunc((v - vmin) * bucket_frq)
 *   clamped as in codegen.py:43-59;
 *   conserve_sum: states are rescaled to this sum after each step (<= 0: no CONSERVE);
 *   init_state: S initial occupancies for every instance.
 * *mechanism_out (may be NULL) receives the mechanism's index q: its states read and
 * write as "kinetic.<q>.state", its table is nw_lti_table_build target 16 + q. */
int nw_kinetic_add(nw_ctx* ctx, int64_t num_instances, const int64_t* segment, const double* g_coef,
                   int num_states, int num_open, const int32_t* open_states, double erev, int32_t species,
                   const double* table, int num_buckets, int num_terms, double vmin, double bucket_frq,
                   double conserve_sum, const double* init_state, int32_t* mechanism_out);

/* Removes every kinetic mechanism (before registering a new set). */
int nw_kinetic_clear(nw_ctx* ctx);

/* Replaces the voltage input of kinetic mechanism `mechanism` by two inputs: lti_sim's
 * two-input tables (Approx2D, neuwon/rxd/lti_sim/approx.py:242-337, indexed as the
 * generated kernel indexes them, codegen.py:43-70; the reference's NMODL front end
 * makes them for KINETIC blocks that read the voltage and a POINTER, e.g.
 * nmodl_library/kinetic/NMDA.mod with its glutamate concentration C, and sorts the
 * inputs by name, lti_model.py:8).  The table given to nw_kinetic_add is then
 * [b1][b2][col][row][term] with num_buckets = num_buckets1 * num_buckets2 and
 * num_terms terms, term t = loc1^powers[2t] * loc2^powers[2t+1] (loc_d the location
 * of input d within its bucket).  Input kinds: 0 = the segment voltage,
 * LinearInput: bucket value (v - minimum) * bucket_frq; 1 = the instance value
 * "kinetic.<q>.input", LogarithmicInput: (log2(x + scale) - log2(minimum + scale)) *
 * bucket_frq; 2 = the instance value, linear.  Instance values start at
 * input_initial (real, per instance, read and written through nw_get_data /
 * nw_set_data). */
int nw_kinetic_inputs(nw_ctx* ctx, int32_t mechanism, int32_t kind1, int32_t num_buckets1, double minimum1,
                      double bucket_frq1, double scale1, int32_t kind2, int32_t num_buckets2, double minimum2,
                      double bucket_frq2, double scale2, int32_t num_terms, const int32_t* powers,
                      double input_initial);

/* nw_kinetic_clear followed by nw_kinetic_add of one nonspecific mechanism (index 0). */
int nw_kinetic_register(nw_ctx* ctx, int64_t num_instances, const int64_t* segment,
                        const double* g_coef, int num_states, int num_open, const int32_t* open_states,
                        double erev, const double* table, int num_buckets, int num_terms,
                        double vmin, double bucket_frq, double conserve_sum, const double* init_state);

/* ---- kinetic-scheme tables (GPU, FP64) ------------------------------ */

/* lti_sim's table generation (neuwon/rxd/lti_sim/approx.py:159-174, lti_model.py:51-65)
 * on the GPU: the exact one-step propagators expm(Q dt) of the num_buckets *
 * samples_per_bucket rate matrices `rates` (row-major S x S each, bucket-major,
 * S <= 16; FP64 scaling and squaring), then per bucket the polynomial fit
 * table[b][col][row][t] = sum_s fit[t][s] * P[b, s][row][col] (fit = the
 * least-squares pseudo-inverse of the in-bucket sample locations, the same for
 * every bucket; 1 <= num_terms <= 10).  target 16 + q installs the table as kinetic mechanism q's (1 is
 * the same as 16: mechanism 0), 2 as the calcium pump's (shapes must match what is
 * registered), 0 only returns it; table_out (may be NULL) receives it in FP64. */
int nw_lti_table_build(nw_ctx* ctx, int32_t S, int32_t num_buckets, int32_t samples_per_bucket,
                       int32_t num_terms, const double* rates, const double* fit, double dt,
                       int32_t target, double* table_out);

/* expm(Q dt) of `count` row-major S x S matrices (the same FP64 routine). */
int nw_lti_expm(nw_ctx* ctx, int32_t S, int64_t count, const double* rates, double dt, double* out);

/* ---- intracellular calcium ----------------------------------------- */

/* One diffusing intracellular species (calcium), as neuwon/rxd/species.py advances
 * one (_SpeciesInstance._advance, species.py:56-70): after each electric half step,
 * c <- max(0, c + dc/dt * dt/2), then c <- M c with M = expm of the diffusion operator
 * over dt/2.  The reference's builder of M (_compute_matrix, species.py:74-83) is
 * unfinished; here M comes from the same tree builder as the electric propagator:
 * d c_i / dt = D A_i / (L_i vol_i) (c_parent - c_i) through segment i's own cross
 * section A_i and length L_i (D in um^2/ms, um, um^3), pruned at prune_tolerance
 * (conserve != 0: pruned mass returned to the diagonal).  Starts at initial_mM
 * everywhere with dc/dt = 0.  "Species.ca" (mM) and "Species.ca_derivative" read and
 * write through nw_calcium_data. */
int nw_calcium_set(nw_ctx* ctx, double diffusivity, const double* cross_area_um2,
                   const double* length_um, const double* volume_um3, double initial_mM,
                   double prune_tolerance, int conserve, int64_t* nnz_out);

/* Calcium mechanisms, run in the mechanism phase after the others (no counterpart in
 * the reference library): dc_i/dt = -influx_coef_i * I_Na,i - efflux_coef_i * E1Ca_i,
 * I_Na the segment's HH sodium current (A) and E1Ca the bound state of a 3-state pump
 * (E1, E1Ca, E2) on every segment.  The pump advances one step at the present c by a
 * table in lti_sim's layout [bucket][col][row][term] over a logarithmic input
 * (neuwon/rxd/lti_sim/inputs.py:85-109: location = (log2(c + scale) - log2_min) *
 * bucket_frq), then is renormalised to sum 1.  table may be NULL: influx only. */
int nw_calcium_pump_set(nw_ctx* ctx, const double* influx_coef, const double* efflux_coef,
                        const double* table, int32_t num_buckets, int32_t num_terms, double log2_min,
                        double bucket_frq, double scale, const double* initial_state);

/* Read (write = 0) or write "Species.ca", "Species.ca_derivative" (n_seg values) or
 * "CaPump.state" (3 * n_seg, state-major) in device order and the given dtype. */
int nw_calcium_data(nw_ctx* ctx, const char* name, void* host, int dtype, int64_t count, int write);

/* ---- synapses and spike events ------------------------------------ */

/* No counterpart in the reference: its neuwon/rxd/synapses.py grows synapse
 * geometry only, and no mechanism has a NET_RECEIVE block.  Spikes are the AP
 * detector's output (neuwon/rxd/neuron/neuron.py:72-75, one detector per neuron,
 * nw_detectors_set).  A spike of neuron pre_neuron[k] at step t arrives at synapse k
 * at step t + delay_steps[k] (>= 1), and keeps transmitter present for the
 * mechanism updates of pulse_steps steps.  Each synapse holds a 2-state AMPA scheme
 * (C, O) and a 3-state NMDA scheme (C, O, D) advanced exactly per step by the given
 * transition matrices (row-major, new state from old; *_on with transmitter, *_off
 * without; 2x2 and 3x3).  Conductance into post_segment[k]:
 * w_ampa O_ampa + w_nmda O_nmda B(V), B(V) = 1 / (1 + exp(-0.062 V) mg / 3.57) (S, mV,
 * mM), reversal e_syn (mV).  The batched path fuses at most min(delay) steps per
 * launch.  Replaces any previous synapse set; states start closed. Readable:
 * "Synapse.ampa_open", "Synapse.nmda_open", "Synapse.nmda_desensitized" (settable),
 * "Synapse.events" (deliveries), "Synapse.last_event", "Synapse.pulse_end" (steps). */
int nw_synapses_set(nw_ctx* ctx, int64_t num_synapses, const int64_t* pre_neuron,
                    const int64_t* post_segment, const double* w_ampa, const double* w_nmda,
                    const int32_t* delay_steps, const double* ampa_on, const double* ampa_off,
                    const double* nmda_on, const double* nmda_off, int32_t pulse_steps,
                    double e_syn, double mg);

/* ---- stimulus, detection, recording --------------------------------- */

/* Current clamps: replaces Segment.inject_current + TimeSeries.play on the
 * half-step input clock (electric.py:119-125, database/time.py:245-302).
 * Clamp k adds amps[k] (A) to its segment's sum_current on input ticks
 * first_tick[k] <= t < first_tick[k] + num_ticks[k] (tick 1 = first half step). */
int nw_clamps_set(nw_ctx* ctx, int64_t count, const int64_t* segment, const double* amps,
                  const int64_t* first_tick, const int64_t* num_ticks);

/* AP detectors, one per neuron (neuwon/rxd/neuron/neuron.py:27-33, 65-75). */
int nw_detectors_set(nw_ctx* ctx, const int64_t* segment, const double* threshold_mV);

/* Voltage probes: replaces TimeSeries.record of Segment.voltage after each
 * advance (database/time.py:189-231).  Up to max_steps samples are kept. */
int nw_probes_set(nw_ctx* ctx, int64_t count, const int64_t* segment, int64_t max_steps);
/* Copies the recorded samples, row-major [steps][count]; *steps_out gets the row count. */
int nw_probes_read(nw_ctx* ctx, void* host, int dtype, int64_t max_rows, int64_t* steps_out);

/* ---- time stepping -------------------------------------------------- */

/* Replaces RxD_Model.advance (neuwon/rxd/rxd_model.py:63-80) called k_steps times:
 * species(dt/2) -> mechanisms(dt) -> species(dt/2) -> AP detector, per step.
 * path selects NW_PATH_BATCHED (fused persistent kernel), NW_PATH_WIDE (neurons of any
 * size; one launch per phase, replayed as CUDA graphs of up to 32 steps) or
 * NW_PATH_PLAIN.  The
 * batched path runs the k_steps as launches of "fusion_depth" fused steps, captured
 * once per distinct call shape in a CUDA graph and replayed (option "cuda_graph"). */
int nw_advance(nw_ctx* ctx, int32_t k_steps, int path);

/* End-to-end step with host buffers: copies stim_amps (one value per clamp, A, or
 * NULL to keep the clamps' amplitudes) from host, advances k_steps, and copies all
 * segment voltages (context precision as dtype) back into v_out (may be NULL). */
int nw_advance_host(nw_ctx* ctx, int32_t k_steps, const double* stim_amps,
                    void* v_out, int v_dtype);

/* The same step without waiting for it: the voltages are copied on the device into
 * one of two staging buffers, then to v_out on a second stream while the next call's
 * step runs, so a loop of calls keeps the GPU busy.  Returns after enqueueing.
 * stim_amps and v_out must stay valid and unmodified until nw_synchronize() (which
 * waits for both streams) has returned; give each call in flight its own v_out
 * (alternating two buffers is enough when the caller synchronises every two calls, or
 * once at the end).  Pinned host memory makes the copies asynchronous.  v_dtype must
 * be the context precision.  A non-finite voltage is reported by the next nw_advance
 * or nw_advance_host call. */
int nw_advance_host_async(nw_ctx* ctx, int32_t k_steps, const double* stim_amps,
                          void* v_out, int v_dtype);

/* Simulation clock (rxd_model.py:22-23): completed steps and input ticks. */
int nw_get_clock(nw_ctx* ctx, int64_t* steps, int64_t* input_ticks);

/* Tuning of the batched path: lanes per propagator row (4, 8, 16 or 32, 0 = auto),
 * threads per CTA (128..1024, default 1024), CTAs per SM (0 = occupancy maximum). */
int nw_set_tuning(nw_ctx* ctx, int lanes_per_row, int threads, int ctas_per_sm);
int nw_get_tuning(nw_ctx* ctx, int* lanes_per_row, int* threads, int* ctas_per_sm);

/* Autotuner of the batched path (replaces the fixed 32-threads-per-block launch of
 * the reference's GPU kernels, neuwon/database/compute.py:360-418): times short runs
 * of this model over lanes per row {4, 8, 16, 32} x threads {512, 768, 1024} (plus the
 * bulk-copy pipeline for FP32), then (quad format, 8 or more lanes) the row-length
 * split "lanes_split" over {1, 2, 3, 4, 6} x lanes quads per row (kept only when 0.5 %
 * faster than none), then the fusion depth over {1, 2, 5, ..., 500} steps
 * up to 4 x trial_steps, and keeps the fastest (ties within 1 % go to deeper fusion).
 * The model's state, clock and probes are restored afterwards.  Outputs may be NULL;
 * lanes_per_row 0 means the bulk pipeline was chosen. */
int nw_autotune(nw_ctx* ctx, int32_t trial_steps, int32_t* lanes_per_row, int32_t* threads,
                int32_t* fusion_depth, double* ms_per_step);

/* ---- differentiation ----------------------------------------------- */

/* No counterpart in the reference (it has no autodiff): the forward half of a
 * gradient computation.  Advances num_steps steps like nw_advance (HH models with
 * one instance per segment), keeping the state every checkpoint_every steps, and
 * returns loss = mean over steps s and neurons j of (V_det(j) after step s -
 * target[s * num_neurons + j])^2, V_det the neuron's AP-detector segment. */
int nw_adjoint_forward(nw_ctx* ctx, int64_t num_steps, int32_t checkpoint_every, const double* target,
                       double* loss_out);

/* The reverse half: d loss / d (every HH instance's gna/gk/gl coefficient, S) in
 * registration order, and d loss / d Ra (cytoplasmic resistivity, ohm cm; pass its
 * current value).  Recomputes each checkpoint interval, taping V and the gates, and
 * sweeps it backwards (transposed propagator, gate Jacobians); leaves the model in
 * the state nw_adjoint_forward ended in.  Any output pointer may be NULL. */
int nw_adjoint_backward(nw_ctx* ctx, double cytoplasmic_resistance, double* grad_gna, double* grad_gk,
                        double* grad_gl, double* grad_ra);

/* Named options.  "reset_clock" (any value): back to time 0 (clock, detector state,
 * probes; conductances count as not yet computed) without touching V or gates.
 * "propagator_format" (default 0): 0 = every P_ij in its row; 2 = quads: each row as
 * windows of 4 consecutive columns (a 16-bit base and 4 values, zeros where a column
 * is not kept; fewer bytes when segments are numbered depth-first, so a row's
 * columns form runs); 1 = pairs: each
 * coupling (i, j) stored once, in the row of the segment with the smaller
 * capacitance, and applied to both rows through detailed balance c_i P_ij = c_j P_ji
 * (propagators from nw_propagator_build only; kept when the other row pruned it, so
 * a pair survives if either P_ij or P_ji reaches the tolerance); 3 = windows: each
 * row's entries covered by windows of 8, 4, 2 or 1 consecutive columns (a 16-bit
 * base and the window's values, zeros where a column is not kept), each window the
 * width of fewest bytes per entry it covers; needs rows sorted by column (the
 * batched step returns NW_ERR_STATE otherwise); nw_get_option("windows") reports
 * the window count.
 * "spike_neurons" (N), "spike_neuron_offset" (o), "spike_ring_steps" (R): for a network
 * split across ranks, taken by the next nw_synapses_set: presynaptic ids are global
 * (< N), the spike ring covers all N neurons with this model's neuron j at o + j, and
 * its length is at least R steps (a common value for all ranks); the ranks sum their
 * rings (own neurons only) after every epoch of at most the shortest delay.
 * "duplicates" (default 0): several instances of one mechanism on one segment all
 * count; 1 = the reference's behaviour for nonspecific conductances (HH and kinetic
 * mechanisms without a species), whose fancy-index "+=" keeps only the last
 * instance's value (neuwon/rxd/species.py:256-260): only the last-registered
 * instance of each segment counts (all of them still advance).
 * "propagator_lump" (default 0), taken by the next nw_propagator_build / nw_calcium_set:
 * an entry below the tolerance is added to the nearest kept entry on the tree path
 * from its segment towards the row's segment instead of being dropped (row sums are
 * kept; far lower error than dropping at the same tolerance, so fewer entries for
 * the same accuracy); the row's own entry is always kept; unvisited remainders still
 * need nw_propagator_conserve.  A lumped propagator has no detailed balance: the pair
 * format falls back to rows and the adjoint refuses it.
 * "set_steps" (k): resume at step k (clock, input ticks 2k, conductances valid when
 * k > 0 and mechanisms exist; probes start empty), for restoring a checkpoint.
 * "lanes_split" (default 0; set by nw_autotune): with the quad format, neurons whose
 * mean quads per row are below this value take half the kernel's lanes per row (the
 * SpMV shape chosen by row length); nw_get_option("narrow_neurons") counts them.
 * "fusion_depth" (default 50, 0 = the whole call in one launch): steps per launch of
 * the batched kernel.  "cuda_graph" (default 1): replay batched launch sequences as
 * CUDA graphs; "prepare_graph" (k) captures, without running, the graph that a later
 * nw_advance(k) replays; "clear_graphs" drops the cached graphs; nw_get_option also reports
 * "graphs_cached", "graph_captures", "graph_replays" and "synapse_ring_words" (u32 words
 * per neuron of the spike ring read and written as "Synapse.spike_ring"). 
 * "bulk_pipeline" (default 0): stream the propagator of the FP32
 * batched path through shared memory with cp.async.bulk copies (needs lanes_per_row
 * 0 in nw_set_tuning); nw_get_option("bulk_pipeline_active") tells whether the next
 * batched launch will use it.
 * "wide_fusion" (default 0): the wide path runs one launch per half step when the
 * mechanisms map one-to-one onto segments (each warp's 32 rows, then their segments'
 * mechanisms and next x) instead of one launch per phase; on a GB300 the phase
 * launches are faster from 2,000 to 1,000,000 segments (more rows in flight per SM).
 * "adjoint_overlap" (default 1): nw_adjoint_backward recomputes checkpoint segment
 * k-1 on a second stream while the reverse sweep of segment k runs (two tapes on the
 * device instead of one); the gradients are the same bit for bit with 0.
 * "propagator_single_walk" (default 1): nw_propagator_build walks each row once,
 * writing its entries into 64-entry chunks of a pool of at most a quarter of the free
 * device memory ("propagator_pool_chunks" > 0 caps its chunks), then packs them into
 * the CSR; with 0, or when the pool fills up, a counting walk and a filling walk.
 * The CSR is the same bit for bit; nw_get_option("propagator_walks") tells which
 * (1 or 2) the last build used.
 * "rows_claimed" (default 1): in the batched quad-format step the warps of a neuron's
 * CTA take its rows from a shared counter, two row groups at a time, each claiming its
 * next chunk before it works on the current one, instead of a fixed share each; a row
 * is summed by the same lanes in the same order either way (same bits).
 * "pair_shared_limit" (default -1): pair format, the largest neuron whose integer
 * pair sums stay in shared memory (-1: as many as fit); larger ones use global
 * memory, with the same sums.
 * nw_get_option also reports "wide_quads", "wide_entries" and
 * "calcium_wide_entries" (stored windows / entries of the wide path's voltage and
 * calcium propagators, once built), "quads" (stored quad windows of the batched
 * path), "windows_8", "windows_4", "windows_2", "windows_1" (windows of each width
 * in the windows format), "pair_entries" (couplings of the pair format),
 * "kinetic_mechanisms" (kinetic mechanisms registered) and
 * "conductance_cache_valid" (1 when the next batched launch reads its first step's
 * conductances from the cache the last fused launch left; every entry point that
 * can change the model clears it). */
int nw_set_option(nw_ctx* ctx, const char* name, int64_t value);
int nw_get_option(nw_ctx* ctx, const char* name, int64_t* value);

/* Statistics of the installed propagator: rows, kept entries (with diagonal),
 * stored off-diagonal entries including padding, bytes of the batched format (of
 * the pair format when "propagator_format" is 1: stored pairs, bytes with the
 * per-row c_max / c_i; quads (2) and windows (3): value slots, bytes with bases and
 * row offsets). */
int nw_propagator_stats(nw_ctx* ctx, int64_t* rows, int64_t* nnz, int64_t* stored,
                        int64_t* bytes);

/* ---- allocation-free half step --------------------------------------- */

/* Largest num_segments accepted by nw_electric_half_step_noalloc. */
#define NW_NOALLOC_MAX_SEGMENTS (1 << 20)

/* No counterpart in the reference.  One electric half step on arrays the caller
 * allocated, for callers that cannot call cudaMalloc: a host application whose
 * device memory must all come from its own pool allocator (a library's own
 * cudaMalloc would escape the pool's accounting or fail under its limit), or a
 * time loop that must not allocate between steps.  Per segment i, with
 * h = half_step_ms:
 *   x_i    = E_i - (E_i - V_i) exp(-h 1e-3 G_i / C_i) + h I_i / C_i
 *   V      = P x                                   (CSR matrix-vector product)
 *   Vint_i = h 1e-3 E_i + (h 1e-3 G_i / C_i)(E_i - V_i) exp(-h 1e-3 G_i / C_i)
 *            + 0.5 h 1e-3 (h I_i / C_i)            (V_i before the update)
 * Nothing is allocated by the call: the scratch vector x is a static device
 * array of NW_NOALLOC_MAX_SEGMENTS doubles (8 MiB).  The CUDA runtime creates it
 * on a GPU when this library's device code is loaded there -- with lazy module
 * loading (the default) at the first call on that GPU, at library load with
 * CUDA_MODULE_LOADING=EAGER -- and keeps it until the process exits.
 *   rowptr/col/val: the propagator P in CSR, FP64, diagonal included (n x n);
 *   voltage V (mV): read, then overwritten with the result;
 *   capacitance C (F), sum_conductance G (S), driving_voltage E (mV),
 *   sum_current I (A): inputs;
 *   integral_voltage Vint (mV s, may be NULL: not written): output;
 *   half_step_ms: the length of this half step (dt/2, ms);
 *   stream: cudaStream_t to launch on (NULL = default stream); the call returns
 *   after enqueueing, without synchronising.
 * All device pointers must be on the current device.  Returns NW_ERR_LIMIT when
 * num_segments > NW_NOALLOC_MAX_SEGMENTS, NW_ERR_ARG for null pointers or a
 * non-positive step, NW_ERR_CUDA when a CUDA error is pending before the call
 * (it is left pending) or a launch fails.  The first call in each CUDA context
 * looks up the scratch array's device address (cudaGetSymbolAddress) and keeps
 * it for that context; make that first call before any stream capture.  Every
 * call shares the one scratch array, so calls that overlap on the GPU
 * (different streams, or different threads) race; each call overwrites the
 * part it uses before reading it, so nothing needs clearing. */
int nw_electric_half_step_noalloc(int64_t num_segments, const int64_t* rowptr, const int32_t* col,
                                  const double* val, double* voltage, const double* capacitance,
                                  const double* sum_conductance, const double* driving_voltage,
                                  const double* sum_current, double* integral_voltage, double half_step_ms,
                                  void* stream);

#ifdef __cplusplus
}
#endif
#endif /* NEUWON_GB300_H */
