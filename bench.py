"""Benchmark: batched FP32 Model.advance() on one GB300 (segment-steps/s).

Workload (neuwon_gb300.workloads.batched): 1,024 seeded neurons, log-uniform
500-20,000 segments (5.59 M segments), HH on every segment, one soma current
per neuron, dt = 0.1 ms, propagator pruned at --tol.  A "step" is one
Model.advance() of the whole batch.  The propagator (about 10+ GB) is far
larger than L2, so no L2 flush is needed between timed steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  Under torchrun each rank advances its own 1,024-neuron
batch (seeds offset by rank; weak scaling) and rank 0 prints; the reference
arm runs on rank 0 only.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "segment-steps/s on 1 GB300: batched FP32 vs plain, <=0.1 mV err; adjoint ms/step"

# DRAM bytes (read + write) per segment-step of batched_advance_kernel, from ncu
# captures of full-size launches (1,024 neurons, 5,593,190 segments), keyed by
# (propagator format, tolerance, lumped): quads lumped at 3e-7 464.9 GB per 25-step
# launch (mean of the four timed launches), quads at 1e-8 charge-conserving 742.6 GB
# per 25-step launch, rows at 1e-8 1,741.6 GB per 50-step launch.  Commands and
# figures: profiles/batched_advance_kernel_lumped_quads.md, _quads_1e-8.md, _rows_1e-8.md.
NCU_TRAFFIC_PER_SEGMENT_STEP = {("quads", 3e-7, 1): 3324.7, ("quads", 1e-8, 0): 5310.6, ("rows", 1e-8, 0): 6227.5}
NCU_TRAFFIC_SEGMENTS = 5593190


def algorithmic_bytes_per_segment_step(r, s_total=11, p_seg=5):
    """B = 2(8r + 4) + 4(2 + 2 S_total + P_seg + 1): two propagator passes (4 B value +
    4 B column per entry, 4 B row pointer), V read+write, every state read+write
    (HH 3 + na8 8), per-segment parameters (C, three HH gbar, na8 gbar), one stimulus read."""
    return 2 * (8 * r + 4) + 4 * (2 + 2 * s_total + p_seg + 1)


def format_bytes_per_segment_step(prop_bytes_per_row, prec=4):
    """Compulsory HBM bytes of this implementation's layout per segment-step: per
    half step the stored propagator bytes of one row (nw_propagator_stats: values,
    16-bit columns or window bases, row offsets, the leak; pairs also c_max / c_i),
    V read + write, kI and kG, HH gates (3) and coefficients (3), the na8 open
    state and coefficient; per step the mechanism update reads V and reads + writes
    3 HH gates and 8 na8 states."""
    per_half = prop_bytes_per_row + 2 * prec + 2 * prec + 6 * prec + 2 * prec
    mech = prec + 2 * (3 + 8) * prec
    return 2 * per_half + mech


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    def __init__(self, device):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


class CpuSample:
    """The C oracle (FP64, OpenMP, all host threads) on a sample of the batch: its first
    neurons of at most max_neuron segments, up to target_segments segments, with the
    same mechanisms (HH + na8), soma clamps, detectors and propagator pruning as the
    batch (lumped at the bench tolerance: oracle_lump in C, the walk of the GPU build;
    else charge-conserving).  Everything is built on the CPU (scipy expm per neuron,
    host lti_sim table): no GPU and none of this package's kernels are involved."""

    def __init__(self, trees, currents, tol, lump=True, max_neuron=3000, target_segments=20000):
        from neuwon_gb300.kinetic import Kinetic, LTITable, na8
        from neuwon_gb300.morphology import geometry, passive_electric
        from neuwon_gb300.workloads import CELSIUS, HH_PARAMS, TIME_STEP
        from oracle.cpu_oracle import CpuOracle, lump as c_lump
        from oracle.reference_step import propagator
        import scipy.sparse
        sample, idx, segs = [], [], 0
        for k, t in enumerate(trees):
            if len(t) <= max_neuron:
                sample.append(t)
                idx.append(k)
                segs += len(t)
                if segs >= target_segments:
                    break
        t0 = time.perf_counter()
        blocks, roots, area, C, off = [], [], [], [], 0
        for t in sample:
            g = geometry(t)
            r, c = passive_electric(g)
            P = propagator(t.parent, r, c, 0.5 * TIME_STEP, prune=0.0).toarray()
            if lump:
                P = c_lump(P, t.parent, tol)
            else:
                P[np.abs(P) < tol] = 0.0
                P[np.diag_indices(len(t))] += 1.0 - P.sum(axis=1)        # charge-conserving
            blocks.append(scipy.sparse.csr_matrix(P))
            roots.append(off); area.append(g["surface_area"]); C.append(c)
            off += len(t)
        P = scipy.sparse.block_diag(blocks, format="csr")
        P.sort_indices()
        area, C = np.concatenate(area), np.concatenate(C)
        n = off
        seg = np.arange(n)
        hh = dict(segment=seg, gna=HH_PARAMS["gnabar"] * 1e-8 * area, gk=HH_PARAMS["gkbar"] * 1e-8 * area,
                  gl=HH_PARAMS["glbar"] * 1e-8 * area, ena=HH_PARAMS["ena"], ek=HH_PARAMS["ek"], el=HH_PARAMS["el"])
        sch = na8()
        tbl = LTITable(sch, TIME_STEP, CELSIUS)
        kin = dict(segment=seg, gcoef=Kinetic.gbar * 1e-8 * area, table=tbl.layout, vmin=tbl.vmin,
                   bucket_frq=tbl.bucket_frq, open=sch.open_states, erev=Kinetic.erev, conserve=sch.conserve_sum,
                   init=sch.steady_state(-70.0, CELSIUS))
        clamps = [(r, float(currents[k]) * 1e-9, 1, 1 << 40) for r, k in zip(roots, idx)]
        self.co = CpuOracle(P.indptr, P.indices.astype(np.int32), P.data, C, time_step=TIME_STEP, celsius=CELSIUS,
                            hh=hh, clamps=clamps, detectors=[(r, 20.0) for r in roots], kinetic=kin)
        self.build_s = time.perf_counter() - t0
        self.n, self.neurons, self.entries_per_row = n, len(sample), P.nnz / n
        self.max_neuron, self.lump, self.tol = max_neuron, lump, tol

    def describe(self, steps):
        pruning = "lumped" if self.lump else "charge-conserving"
        return (f"{self.neurons} neurons of the batch of <= {self.max_neuron} segments ({self.n} segments, "
                f"{self.entries_per_row:.0f} propagator entries/row, {pruning} at {self.tol:g}), HH + na8, {steps} "
                f"steps, FP64 C restatement (oracle/cpu_step.c) with OpenMP, built on the CPU in {self.build_s:.0f} s")

    def steps_for(self, seconds):
        """Steps that take about `seconds`, from calls of 1, 2, 4, ... steps until one
        takes 0.5 s (multi-step calls, as timed, so the per-call thread start-up is
        not charged to every step; advances the model)."""
        k = 1
        while True:
            t0 = time.perf_counter()
            self.co.advance(k)
            dt = time.perf_counter() - t0
            if dt >= 0.5:
                return max(1, int(k * seconds / dt))
            k *= 2


def cpu_sample(trees, currents, tol, lump=True, time_budget_s=15.0, warmup=2):
    """Segment-steps/s of the C oracle on the batch sample over about time_budget_s
    seconds of CPU work (after `warmup` untimed steps)."""
    cs = CpuSample(trees, currents, tol, lump)
    cs.co.advance(max(warmup, 1))                 # untimed
    k = cs.steps_for(time_budget_s)
    t0 = time.perf_counter()
    cs.co.advance(k)
    dt = time.perf_counter() - t0
    return {"value": cs.n * k / dt, "unit": "segment-steps/s", "cores": cs.co.threads(), "kind": "port",
            "sample": cs.describe(k), "entries_per_row": cs.entries_per_row, "seconds": dt}


def workload_name(neurons, lo, hi):
    """The bench workload as both arms name it in config.workload."""
    return (f"batched: {neurons} neurons, log-uniform {lo}-{hi} segments, HH + 8-state Markov Na on every "
            "segment, soma current U(0.05,0.5) nA, dt 0.1 ms, FP32 state, FP64-built propagator")


def run_reference(args, rank):
    """The reference arm: the CPU path restated in C (the reference's own numba path
    cannot run here: numba is absent) on the batch sample, all host threads.  A step
    is a bounded chunk of that sample: max(0.5 s, 10 s / K) of CPU work, so the K
    timed steps always cover at least 10 s whatever K is; W chunks warm up first."""
    from neuwon_gb300.workloads import batched_currents, batched_trees
    lo, hi = (int(x) for x in args.size_range.split(","))
    trees = batched_trees(args.neurons, first=0, count=64, processes=8, lo=lo, hi=hi)
    currents = batched_currents(args.neurons)
    cs = CpuSample(trees, currents, args.tol, bool(args.lump))
    K = max(1, args.steps)
    chunk = cs.steps_for(max(0.5, 11.0 / K))
    for _ in range(max(args.warmup, 1)):
        cs.co.advance(chunk)
    t0 = time.perf_counter()
    for _ in range(K):
        cs.co.advance(chunk)
    dt = time.perf_counter() - t0
    value = cs.n * chunk * K / dt
    res = {"value": value, "unit": "segment-steps/s", "cores": cs.co.threads(), "kind": "port",
           "sample": cs.describe(chunk * K) + f"; one step = {chunk} sample steps", "seconds": dt,
           "entries_per_row": cs.entries_per_row}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "segment-steps/s",
            "n_gpus": args.gpus, "steps": K, "warmup": args.warmup, "ms_per_step": 1e3 * dt / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": workload_name(args.neurons, lo, hi),
                                            "sample": res["sample"], "propagator_tolerance": args.tol,
                                            "propagator_pruning": "lumped" if args.lump else "charge-conserving"},
            "cpu_baseline": res,
            "e2e": {"value": value, "unit": "segment-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def accuracy(trees, currents, tol, device, steps, ref_tol, fmt="rows", lump=False, label="sample"):
    """FP32 batched at the bench tolerance and pruning against FP64 with a propagator
    pruned at ref_tol (charge-conserving); the FP64 reference runs on the wide path,
    which spreads the sample neurons over every SM.  Max |dV| at every soma after every
    step and at every segment every 50 steps (also per 100 ms of simulated time)."""
    from neuwon_gb300 import Segment, TimeSeries
    from neuwon_gb300.workloads import build_model
    t0 = time.perf_counter()
    ref, nref = build_model(trees, currents, precision="f64", tolerance=ref_tol, conserve=True, device=device,
                            path="wide")
    test, ntest = build_model(trees, currents, precision="f32", tolerance=tol, conserve=True, device=device, fmt=fmt,
                              lump=lump)
    probes = []
    for m, ns in ((ref, nref), (test, ntest)):
        probes.append([TimeSeries().record(nr.root, "voltage") for nr in ns])
    ref._sync(); test._sync()
    log(f"accuracy models built in {time.perf_counter() - t0:.1f} s "
        f"(reference {ref.propagator_nnz / ref._n:.0f} entries/row)")
    t0 = time.perf_counter()
    worst_all, chunk = 0.0, 50
    by_period, period = [], 1000                       # max error over all segments per 100 ms
    for k in range(steps // chunk):
        ref.advance(chunk); test.advance(chunk)
        err = float(np.abs(ref.get_data("Segment.voltage") - test.get_data("Segment.voltage")).max())
        worst_all = max(worst_all, err)
        if (k * chunk) % period == 0:
            by_period.append(err)
        else:
            by_period[-1] = max(by_period[-1], err)
    log(f"accuracy run of {steps} steps in {time.perf_counter() - t0:.1f} s")
    soma_ref = np.array([p.get_data() for p in probes[0]])
    soma_test = np.array([p.get_data() for p in probes[1]])
    soma_err = np.abs(soma_ref - soma_test)
    sp_ref = ref.get_data("Neuron.spike_count"); sp_test = test.get_data("Neuron.spike_count")
    n = ref._n
    ref.close(); test.close()
    return {"max_err_mV": max(worst_all, float(soma_err.max())),
            "max_err_soma_every_step_mV": float(soma_err.max()),
            "max_err_soma_per_neuron_mV": [float(x) for x in soma_err.max(axis=1)],
            "max_err_all_segments_every_50_steps_mV": worst_all,
            "max_err_all_segments_per_100ms_mV": by_period,
            "spikes_equal": bool(np.array_equal(sp_ref, sp_test)), "spikes_total": int(sp_ref.sum()),
            "steps": steps,
            "against": f"FP64 GPU (wide path), propagator pruned at {ref_tol:g} (charge-conserving)",
            "sample": f"{label} ({len(trees)} neurons of {min(len(t) for t in trees)}-{max(len(t) for t in trees)} "
                      f"segments, {n} segments)"}


def epsilon_gap(trees, currents, device, steps, ref_tol):
    """How far the accuracy reference (FP64, pruned at ref_tol, charge-conserving) is from
    the reference's own pruning at machine epsilon, on neurons of at most 2,000 segments."""
    from neuwon_gb300.morphology import EPSILON
    from neuwon_gb300.workloads import build_model
    models = []
    for tol, conserve in ((EPSILON, False), (ref_tol, True)):
        m, _ = build_model(trees, currents, precision="f64", tolerance=tol, conserve=conserve, device=device,
                           path="wide")
        m._sync()
        models.append(m)
    worst, chunk = 0.0, 50
    for _ in range(steps // chunk):
        for m in models:
            m.advance(chunk)
        worst = max(worst, float(np.abs(models[0].get_data("Segment.voltage") -
                                        models[1].get_data("Segment.voltage")).max()))
    spikes = [int(m.get_data("Neuron.spike_count").sum()) for m in models]
    out = {"max_dV_mV": worst, "steps": steps, "spikes": spikes,
           "entries_per_row": [m.propagator_nnz / m._n for m in models],
           "sample": f"{len(trees)} neurons of the batch of <= 2,000 segments ({models[0]._n} segments)",
           "compared": f"FP64 at machine epsilon (the reference's pruning) vs FP64 at {ref_tol:g} charge-conserving"}
    for m in models:
        m.close()
    return out


def cpu_baseline_config1(device, steps=1000):
    """The single-neuron configuration (one seeded 2,000-segment HH tree, 0.2 nA soma
    clamp 5-80 ms, dt 0.1 ms for 100 ms, FP64, propagator pruned at machine epsilon as
    the reference prunes it): the reference's own path as it runs without numba (scipy
    CSR SpMV + numpy mechanisms, restated in the oracle: rxd_model.py:63-80,
    electric.py:56-76) timed on one host core, and this package's batched and wide
    paths on the GPU over the same 1,000 steps, with each one's max voltage difference
    from the oracle's at the end and its spike count."""
    import neuwon_gb300 as nw
    from neuwon_gb300.morphology import geometry, passive_electric, random_tree
    from oracle.reference_step import HHInstances, OracleModel, clamp_ticks
    tree = random_tree(2000, seed=0)
    hh_kw = dict(ena=50.0, ek=-77.0, el=-54.3)
    g = geometry(tree)
    R, C = passive_electric(g)
    n = len(tree)
    f, c = clamp_ticks(5.0, 75.0, 0.1)
    t0 = time.perf_counter()
    om = OracleModel(tree.parent, R, C, time_step=0.1, celsius=6.3,
                     hh=HHInstances(np.arange(n), g["surface_area"], celsius=6.3, **hh_kw),
                     clamps=[(0, 0.2e-9, f, c)], detectors=[(0, 20.0)])
    build_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(steps):
        om.advance()
    ref_s = time.perf_counter() - t0
    out = {"config": "one 2,000-segment HH tree (seed 0), 0.2 nA soma clamp 5-80 ms, dt 0.1 ms, "
                     f"{steps} steps, propagator at machine epsilon ({om.P.nnz / n:.0f} entries/row)",
           "reference_path": {"value": n * steps / ref_s, "unit": "segment-steps/s", "ms_per_step": ref_s / steps * 1e3,
                              "cores": 1, "kind": "port",
                              "sample": "the reference's numba-less path restated (oracle/reference_step.py: "
                                        "scipy CSR SpMV + numpy HH), FP64, all 1,000 steps",
                              "build_s": build_s, "spikes": int(om.spike_count[0])}}
    for precision, path in (("f64", "batched"), ("f64", "wide"), ("f32", "batched"), ("f32", "wide")):
        m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision=precision, path=path, device=device,
                         mechanisms=[nw.HH.configure(**hh_kw)])
        nr = m.add_tree(tree)
        m.insert_everywhere("hh")
        m._sync()
        m._ctx.call("nw_synchronize")
        # The first 50 steps (untimed) also build the row formats and capture the
        # launch graph; the clamp starts at 5 ms; the other steps are timed as
        # calls of 50 steps each.
        t0 = time.perf_counter()
        m.advance(50)
        m._ctx.call("nw_synchronize")
        first_s = time.perf_counter() - t0
        nr.root.inject_current(0.2, 75.0)
        t0 = time.perf_counter()
        for _ in range(steps // 50 - 1):
            m.advance(50)
        m._ctx.call("nw_synchronize")
        dt = time.perf_counter() - t0
        timed = 50 * (steps // 50 - 1)
        out[f"gpu_{precision}_{path}"] = {
            "value": n * timed / dt, "unit": "segment-steps/s", "ms_per_step": dt / timed * 1e3,
            "first_50_steps_s": first_s,
            "max_err_mV": float(np.abs(m.get_data("Segment.voltage") - om.voltage).max()),
            "spikes": int(m.get_data("Neuron.spike_count")[0])}
        m.close()
    return out


def plain_timing(trees, currents, tol, device, steps=10):
    """The plain per-neuron FP64 path (reference GPU design) on a subset of the batch."""
    from neuwon_gb300.workloads import build_model
    m, _ = build_model(trees, currents, precision="f64", tolerance=tol, conserve=True, path="plain",
                       device=device)
    m._sync()
    m.advance(1)
    m._ctx.call("nw_synchronize")
    t0 = time.perf_counter()
    m.advance(steps)
    m._ctx.call("nw_synchronize")
    dt = time.perf_counter() - t0
    n = m._n
    m.close()
    return {"value": n * steps / dt, "unit": "segment-steps/s", "ms_per_step": 1e3 * dt / steps,
            "sample": f"first {len(trees)} neurons ({n} segments), {steps} steps, per-neuron launches, "
                      "32 threads/block, FP64 CSR, same propagator tolerance"}


def adjoint_build(trees, precision, device, ra=100.0, amps=None):
    """The differentiation configuration's model: HH on every segment of the given
    trees, dt 0.025 ms, a constant soma clamp per neuron (0.3 nA unless amps gives
    one per tree), propagator pruned at 1e-8 (charge-conserving)."""
    from neuwon_gb300 import HH, RxD_Model
    from neuwon_gb300.workloads import HH_PARAMS
    m = RxD_Model(time_step=0.025, temperature=6.3, precision=precision, device=device,
                  propagator_tolerance=1e-8, propagator_conserve=True, cytoplasmic_resistance=ra,
                  mechanisms=[HH.configure(**HH_PARAMS)])
    ns = [m.add_tree(t) for t in trees]
    m.insert_everywhere("hh")
    for k, nr in enumerate(ns):
        nr.root.inject_current(0.3 if amps is None or amps[k] is None else amps[k], 1e9)
    m._sync()
    return m


def adjoint_target(trees, steps, device, seed=4):
    """FP64 soma traces of the same neurons with densities drawn +-30 % around the defaults."""
    from neuwon_gb300.workloads import HH_PARAMS
    rng = np.random.default_rng(seed)
    k = sum(len(t) for t in trees)
    m64 = adjoint_build(trees, "f64", device)
    m64.set_hh_densities(*(rng.uniform(0.7, 1.3, k) * HH_PARAMS[g] for g in ("gnabar", "gkbar", "glbar")))
    m64.reset_state()
    roots = np.array(m64._neuron_root, dtype=np.int64)
    m64._ctx.call("nw_probes_set", len(trees), _lib_ptr(roots), steps)
    m64._ctx.advance(steps)
    target = np.empty((steps, len(trees)))
    s_out = ctypes.c_int64()
    m64._ctx.call("nw_probes_read", _lib_ptr(target), 1, steps, ctypes.byref(s_out))
    m64.close()
    return target


def diff_check(args, device):
    """The differentiation configuration as specified: 256 HH neurons of 2,000 segments,
    dt 0.025 ms, --diff-steps steps (8,000 = 200 ms), checkpoint every 100; FP32 adjoint
    gradients (and the FP64 adjoint) against FP64 central differences (h = 1e-4 relative)
    on 31 random per-segment densities (gNa / gK / gL) and Ra, relative error per parameter."""
    from neuwon_gb300.adjoint import central_differences, loss_and_gradients
    from neuwon_gb300.morphology import random_tree
    steps, neurons, size = args.diff_steps, args.diff_neurons, 2000
    trees = [random_tree(size, seed=5000 + k) for k in range(neurons)]
    t0 = time.perf_counter()
    target = adjoint_target(trees, steps, device)
    log(f"diff check: target in {time.perf_counter() - t0:.1f} s")
    rng = np.random.default_rng(11)
    kinds = rng.choice(["gna", "gk", "gl"], 31)
    params = [(str(kd), int(rng.integers(neurons)), int(rng.integers(size))) for kd in kinds]
    params[0] = ("gna", params[0][1], 0)                      # a soma
    params.append(("ra",))
    res = {}
    for precision in ("f32", "f64"):
        t0 = time.perf_counter()
        m = adjoint_build(trees, precision, device)
        loss, gna, gk, gl, gra = loss_and_gradients(m, steps, target, checkpoint_every=100)
        m.close()
        g = {"gna": gna, "gk": gk, "gl": gl}
        res[precision] = [gra if p[0] == "ra" else float(g[p[0]][p[1] * size + p[2]]) for p in params]
        res[precision + "_loss"] = loss
        log(f"diff check: {precision} adjoint in {time.perf_counter() - t0:.1f} s, loss {loss}")
    t0 = time.perf_counter()
    fd = central_differences(lambda ts, prec, ra, amps: adjoint_build(ts, prec, device, ra, amps),
                             trees, steps, target, params)
    log(f"diff check: central differences in {time.perf_counter() - t0:.1f} s")
    rel = lambda a, b: abs(a - b) / max(abs(b), 1e-300)
    rows = [{"param": (p[0] if p[0] == "ra" else f"{p[0]}[neuron {p[1]}, segment {p[2]}]"), "fd_f64": f,
             "adjoint_f32": a32, "adjoint_f64": a64, "rel_err_f32": rel(a32, f), "rel_err_f64": rel(a64, f)}
            for p, f, a32, a64 in zip(params, fd, res["f32"], res["f64"])]
    # Parameters whose derivative is below 1e-3 of the largest one are reported but
    # not in the maxima: their relative error measures cancellation in the differences.
    big = max(abs(r["fd_f64"]) for r in rows)
    sig = [r for r in rows if abs(r["fd_f64"]) >= 1e-3 * big]
    out = {"metric": "adjoint check: FP32 / FP64 adjoint gradients vs FP64 central differences",
           "config": {"workload": f"{neurons} HH neurons x {size} segments, dt 0.025 ms, {steps} steps, checkpoint "
                                  "every 100, propagator 1e-8 (charge-conserving), targets from FP64 runs with "
                                  "densities +-30 %", "parameters": len(params), "h_rel": 1e-4},
           "loss_f32": res["f32_loss"], "loss_f64": res["f64_loss"],
           "max_rel_err_f32": max(r["rel_err_f32"] for r in sig), "max_rel_err_f64": max(r["rel_err_f64"] for r in sig),
           "median_rel_err_f32": float(np.median([r["rel_err_f32"] for r in sig])),
           "parameters_in_maxima": len(sig), "rows": rows}
    print(json.dumps(out), flush=True)


def adjoint_leg(device, steps, checkpoint_every=100, neurons=256, size=2000, threads=0, overlap=1, lanes=0):
    """Config 4 shape: 256 HH neurons of 2,000 segments, dt 0.025 ms, FP32, targets = FP64
    soma traces of the same neurons with densities drawn +-30 % around the defaults;
    gradients of the soma MSE w.r.t. per-segment gNa/gK/gL and Ra (checkpoint every 100)."""
    import torch
    from neuwon_gb300.adjoint import _backward, _forward
    from neuwon_gb300.morphology import random_tree
    trees = [random_tree(size, seed=5000 + k) for k in range(neurons)]
    k = neurons * size
    target = adjoint_target(trees, steps, device)
    m = adjoint_build(trees, "f32", device)
    if threads or lanes:
        m._ctx.call("nw_set_tuning", lanes, threads or 1024, 0)
    m._ctx.set_option("adjoint_overlap", overlap)
    m.reset_state()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = _forward(m, steps, target, checkpoint_every)
    t1 = time.perf_counter()
    gna, gk, gl, gra = _backward(m)
    t2 = time.perf_counter()
    m.close()
    return {"ms_per_step": 1e3 * (t2 - t0) / steps, "forward_ms_per_step": 1e3 * (t1 - t0) / steps,
            "backward_ms_per_step": 1e3 * (t2 - t1) / steps, "steps": steps,
            "checkpoint_every": checkpoint_every, "threads": threads or "context default",
            "lanes_per_row": lanes or "by quads per row",
            "recompute_beside_reverse": bool(overlap), "loss_mV2": loss,
            "grad_norm": float(np.sqrt((gna ** 2).sum() + (gk ** 2).sum() + (gl ** 2).sum())),
            "grad_ra": gra, "parameters": 3 * k + 1,
            "config": f"{neurons} HH neurons x {size} segments, dt 0.025 ms, FP32, propagator 1e-8 "
                      "(charge-conserving), targets from FP64 runs with densities +-30 %"}


def network_leg(device, steps, neurons=4096, synapses=2_000_000):
    """Config 5 shape: 4,096 seeded neurons of 200-5,000 segments (log-uniform), HH on every
    segment, 2 M synapses (AMPA + NMDA with Mg block), lognormal weights (mu -1, sigma 0.5,
    nS), delays U(1, 20) ms, FP32, dt 0.1 ms, autotuned fusion depth (capped at the shortest
    delay), a bounded sample of the 2 s run."""
    from neuwon_gb300.synapses import random_network
    from neuwon_gb300.workloads import batched_currents, batched_trees, build_model
    t0 = time.perf_counter()
    trees = batched_trees(neurons, seed=7, processes=min(16, os.cpu_count() or 1), lo=200, hi=5000)
    currents = batched_currents(neurons, seed=7)
    m, _ = build_model(trees, currents, precision="f32", tolerance=1e-8, conserve=True, device=device,
                       kinetic=False, fmt="quads")
    net = random_network([len(t) for t in trees], synapses, 7)
    offs = np.cumsum([0] + [len(t) for t in trees])[:-1]
    m.add_synapses(net["pre"], offs[net["post_neuron"]] + net["post_local"], net["weight_nS"], net["weight_nS"],
                   net["delay_steps"] * 0.1)
    m._sync()
    build_s = time.perf_counter() - t0
    tuned = m.autotune(5)
    m.advance(20)
    m._ctx.call("nw_synchronize")
    ev0 = int(m.get_data("Synapse.events").sum())
    sp0 = int(m.get_data("Neuron.spike_count").sum())
    t0 = time.perf_counter()
    m.advance(steps)
    m._ctx.call("nw_synchronize")
    dt = time.perf_counter() - t0
    n = m._n
    out = {"ms_per_step": 1e3 * dt / steps, "segment_steps_per_s": n * steps / dt, "segments": n,
           "synapses": synapses, "steps": steps, "build_s": build_s,
           "events_delivered": int(m.get_data("Synapse.events").sum()) - ev0,
           "spikes": int(m.get_data("Neuron.spike_count").sum()) - sp0,
           "fusion_depth": min(tuned["fusion_depth"], int(net["delay_steps"].min())), "autotune": tuned,
           "config": f"{neurons} HH neurons, log-uniform 200-5000 segments, {synapses} AMPA+NMDA synapses, "
                     "delays U(1, 20) ms, FP32, dt 0.1 ms, propagator 1e-8 (charge-conserving), quad format"}
    m.close()
    return out


def wide_bytes_per_segment_step(windows_per_row, ca_entries_per_row, calcium=True, prec=4):
    """Compulsory HBM bytes of one step of the wide path per segment (FP32): per
    half step the voltage propagator's quad windows (16 B of values and a 4 B base
    each), its row pointer (8 B) and leak, x read, kG and kI read, the next x and V
    written; with calcium the same for its propagator (entries in 4-entry vectors of
    4 B values and 4 B columns), scratch read and written and c written; per step
    the HH gates (read and written) and their conductance coefficients, and with
    calcium the pump states (read and written), dc/dt and the influx and efflux
    coefficients."""
    half = 20 * windows_per_row + 8 + prec + 3 * prec + 2 * prec
    if calcium:
        half += 2 * prec * ca_entries_per_row + 8 + prec + 3 * prec
    step = 2 * half + 2 * 3 * prec + 3 * prec
    if calcium:
        step += 2 * 3 * prec + 3 * prec
    return step


def wide_leg(device, segments, tol, steps, variants=((0, 0),)):
    """The precision configuration's step on the wide path, timed: one seeded tree
    (same length and diameter laws), HH + calcium (diffusion, pump, Na influx),
    FP32, dt 0.025 ms, propagators pruned at `tol` (charge/mass-conserving), 10 nA
    soma clamp.  For each (wide_fusion, lanes per row; 0 = by row length) variant:
    64 untimed steps (formats built, graphs captured), then `steps` steps timed
    with CUDA events on the library's stream."""
    import torch
    import neuwon_gb300 as nw
    from neuwon_gb300.morphology import random_tree
    tree = random_tree(segments, seed=3)
    m = nw.RxD_Model(time_step=0.025, temperature=6.3, precision="f32", path="wide", species=[nw.Calcium()],
                     propagator_tolerance=tol, propagator_conserve=True, device=device,
                     mechanisms=[nw.HH.configure(ena=50.0, ek=-77.0, el=-54.3)])
    nr = m.add_tree(tree)
    m.insert_everywhere("hh")
    nr.root.inject_current(10.0, 1e9)
    m._sync()
    ctx = m._ctx
    sptr = ctypes.c_void_p()
    ctx.call("nw_get_stream", ctypes.byref(sptr))
    stream = torch.cuda.ExternalStream(sptr.value, device=torch.device("cuda", device))
    peak, src = 6800.0, "fallback"
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    runs = []
    for wide_fusion, lanes in variants:
        ctx.call("nw_set_tuning", lanes, 1024, 0)
        ctx.set_option("wide_fusion", wide_fusion)
        m.advance(64)
        ctx.call("nw_synchronize")
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        m.advance(steps)
        ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1) / steps
        n = m._n
        wpr = ctx.get_option("wide_quads") / n
        epr = ctx.get_option("calcium_wide_entries") / n
        B = wide_bytes_per_segment_step(wpr, epr)
        achieved = B * n / (ms * 1e-3) / 1e9
        runs.append({"wide_fusion": wide_fusion, "lanes_per_row": lanes or "by row length", "ms_per_step": ms,
                     "segment_steps_per_s": n * 1e3 / ms,
                     "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                  "frac": achieved / peak, "peak_source": src}})
        log(f"wide leg {runs[-1]}")
    spikes = int(m.get_data("Neuron.spike_count")[0])
    m.close()
    return {"segments": n, "steps": steps, "tolerance": tol, "windows_per_row": wpr, "calcium_entries_per_row": epr,
            "bytes_per_segment_step": B, "runs": runs, "spikes": spikes,
            "config": f"one tree of {n} segments, HH + calcium, FP32, dt 0.025 ms, propagators {tol:g} "
                      "(charge/mass-conserving), quad format, 10 nA soma clamp"}


def run_leg(args, rank, local):
    """One side leg alone (rank 0), at its configuration's shape or a smaller case."""
    if rank != 0:
        return
    if args.leg == "plain":
        from neuwon_gb300.workloads import batched_currents, batched_trees
        k = args.leg_neurons or 64
        lo, hi = (int(x) for x in args.size_range.split(","))
        trees = batched_trees(args.neurons, first=0, count=k, processes=min(16, os.cpu_count() or 1), lo=lo, hi=hi)
        currents = batched_currents(args.neurons)[:k]
    import torch
    torch.cuda.set_device(local)
    if args.leg == "adjoint":
        out = adjoint_leg(local, args.adjoint_steps, neurons=args.leg_neurons or 256, size=args.leg_size or 2000,
                          threads=args.adjoint_threads, overlap=args.adjoint_overlap, lanes=args.adjoint_lanes)
    elif args.leg == "wide":
        variants = [tuple(int(x) for x in v.split(":")) for v in args.wide_variants.split(",")]
        out = wide_leg(local, args.study_segments, args.wide_tol, args.wide_steps, variants)
    elif args.leg == "network":
        out = network_leg(local, args.network_steps, neurons=args.leg_neurons or 4096,
                          synapses=args.leg_synapses or 2_000_000)
    else:
        out = plain_timing(trees, currents, args.tol, local)
    print(json.dumps({"leg": args.leg, **out}), flush=True)


def _lib_ptr(a):
    from neuwon_gb300 import _lib
    return _lib.ptr(a)


def precision_study(args, device):
    """The 1 M-segment precision configuration: one seeded tree (same length and
    diameter laws), HH + intracellular calcium (D 0.6 um2/ms, pump, Na-fraction
    influx), dt 0.025 ms for 500 ms on the wide path; FP32 + compensated sums vs
    FP64 (both on the GPU, run in lockstep), propagators pruned at 1e-6 and 1e-9
    (charge- and mass-conserving).  Reports max |dV| and max relative d[Ca]."""
    import neuwon_gb300 as nw
    from neuwon_gb300.morphology import random_tree
    steps, chunk = args.study_steps, 500
    t0 = time.perf_counter()
    tree = random_tree(args.study_segments, seed=3)
    log(f"precision study: tree of {len(tree)} segments in {time.perf_counter() - t0:.1f} s")
    out = {"metric": "precision study: FP32 vs FP64, max |dV| (mV) and max relative d[Ca]",
           "config": {"workload": f"one tree of {len(tree)} segments, HH + calcium (diffusion 0.6 um2/ms, 3-state "
                                  f"pump, 0.5 % of the Na current as Ca), {args.study_current:g} nA soma clamp, dt 0.025 ms",
                      "steps": steps, "path": "wide", "pruning": "charge/mass-conserving",
                      "wide_fusion": args.wide_fusion},
           "results": []}
    for tol in (1e-6, 1e-9):
        models = {}
        for precision in ("f64", "f32"):
            t0 = time.perf_counter()
            m = nw.RxD_Model(time_step=0.025, temperature=6.3, precision=precision, path="wide", species=[nw.Calcium()],
                             propagator_tolerance=tol, propagator_conserve=True, device=device,
                             mechanisms=[nw.HH.configure(ena=50.0, ek=-77.0, el=-54.3)])
            nr = m.add_tree(tree)
            m.insert_everywhere("hh")
            nr.root.inject_current(args.study_current, 1e9)
            m._sync()
            m._ctx.set_option("wide_fusion", args.wide_fusion)
            m._ctx.call("nw_synchronize")
            models[precision] = (m, time.perf_counter() - t0)
        dv = dca = 0.0
        # Step times leave out the first chunk (wide formats built, graphs captured)
        # when there is more than one.
        times = {"f64": 0.0, "f32": 0.0}
        done = timed = 0
        while done < steps:
            k = min(chunk, steps - done)
            for precision, (m, _) in models.items():
                m._ctx.call("nw_synchronize")
                t0 = time.perf_counter()
                m.advance(k)
                m._ctx.call("nw_synchronize")
                if done > 0 or steps <= chunk:
                    times[precision] += time.perf_counter() - t0
            if done > 0 or steps <= chunk:
                timed += k
            done += k
            v64, v32 = (models[p][0].get_data("Segment.voltage") for p in ("f64", "f32"))
            c64, c32 = (models[p][0].get_data("Species.ca") for p in ("f64", "f32"))
            dv = max(dv, float(np.abs(v64 - v32).max()))
            dca = max(dca, float((np.abs(c64 - c32) / c64).max()))
        spikes = {p: int(models[p][0].get_data("Neuron.spike_count")[0]) for p in models}
        nnz = models["f32"][0].propagator_nnz / len(tree)
        res = {"tolerance": tol, "max_abs_dV_mV": dv, "max_rel_dCa": dca, "spikes": spikes,
               "entries_per_row": nnz, "calcium_entries_per_row": models["f32"][0].calcium_nnz / len(tree),
               "ms_per_step": {p: 1e3 * times[p] / timed for p in times}, "timed_steps": timed,
               "build_s": {p: models[p][1] for p in models}}
        log(f"precision study {res}")
        out["results"].append(res)
        for m, _ in models.values():
            m.close()
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--neurons", type=int, default=1024)
    ap.add_argument("--tol", type=float, default=3e-7)
    ap.add_argument("--ref-tol", type=float, default=1e-10,
                    help="pruning of the FP64 accuracy reference (machine epsilon makes rows dense)")
    ap.add_argument("--size-range", default="500,20000", help="neuron size range (segments)")
    ap.add_argument("--acc-neurons", type=int, default=32,
                    help="accuracy sample: the batch's largest half and its first other half")
    ap.add_argument("--acc-steps", type=int, default=10000, help="accuracy run (10,000 steps = the full 1 s)")
    ap.add_argument("--fusion", type=int, default=50, help="steps fused per kernel launch (without --autotune)")
    ap.add_argument("--autotune", type=int, default=10,
                    help="trial steps of the autotuner (lanes, threads, fusion depth); 0 = use the flags")
    ap.add_argument("--lump", type=int, default=1, choices=[0, 1],
                    help="lumped pruning (pruned entries moved to the nearest kept entry on the tree path)")
    ap.add_argument("--format", default="quads", choices=["rows", "pairs", "quads", "windows"],
                    help="propagator storage: every P_ij in its row; windows of 4 consecutive columns; "
                         "or each coupling once (detailed balance)")
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--threads", type=int, default=1024)
    ap.add_argument("--bulk", type=int, default=0, help="cp.async.bulk propagator stream (FP32)")
    ap.add_argument("--quick", action="store_true", help="skip accuracy/plain/cpu/adjoint legs")
    ap.add_argument("--adjoint-steps", type=int, default=800)
    ap.add_argument("--adjoint-threads", type=int, default=0, help="threads per CTA of the adjoint kernels (0: default)")
    ap.add_argument("--adjoint-lanes", type=int, default=0, help="lanes per row of the adjoint kernels (0: by quads per row)")
    ap.add_argument("--adjoint-overlap", type=int, default=1,
                    help="1: the backward recomputes segment k-1 on a second stream beside the reverse sweep of k")
    ap.add_argument("--network-steps", type=int, default=200,
                    help="steps of the 4,096-neuron, 2 M-synapse network leg (0 = skip)")
    ap.add_argument("--precision-study", action="store_true",
                    help="run only the 1 M-segment FP32-vs-FP64 calcium precision study")
    ap.add_argument("--study-segments", type=int, default=1_000_000)
    ap.add_argument("--study-steps", type=int, default=20000)
    ap.add_argument("--study-current", type=float, default=10.0, help="soma clamp of the precision study (nA)")
    ap.add_argument("--wide-fusion", type=int, default=0, choices=[0, 1],
                    help="precision study: one launch per half step (1) or one per phase (0)")
    ap.add_argument("--diff-check", action="store_true",
                    help="differentiation configuration: FP32/FP64 adjoint vs FP64 central differences (own JSON line)")
    ap.add_argument("--diff-steps", type=int, default=8000)
    ap.add_argument("--diff-neurons", type=int, default=256)
    ap.add_argument("--wide-tol", type=float, default=1e-9, help="propagator tolerance of the wide leg")
    ap.add_argument("--wide-steps", type=int, default=320, help="timed steps of the wide leg")
    ap.add_argument("--wide-variants", default="0:0",
                    help="wide leg: comma-separated wide_fusion:lanes_per_row (0 = by row length)")
    ap.add_argument("--leg", choices=["adjoint", "network", "plain", "wide"],
                    help="run one side leg alone and print its JSON line (a small case with --leg-neurons, "
                         "--leg-size, --leg-synapses, --adjoint-steps / --network-steps)")
    ap.add_argument("--leg-neurons", type=int, default=0)
    ap.add_argument("--leg-size", type=int, default=0, help="segments per neuron (adjoint leg)")
    ap.add_argument("--leg-synapses", type=int, default=0)
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, rank)
        return
    if args.precision_study:
        import torch
        torch.cuda.set_device(local)
        if rank == 0:
            precision_study(args, local)
        return
    if args.diff_check:
        import torch
        torch.cuda.set_device(local)
        if rank == 0:
            diff_check(args, local)
        return
    if args.leg:
        run_leg(args, rank, local)
        return

    from neuwon_gb300.workloads import batched_currents, batched_trees, build_model
    # Trees are generated in a spawned pool before any CUDA work.
    t_setup = time.perf_counter()
    lo, hi = (int(x) for x in args.size_range.split(","))
    from neuwon_gb300.replicas import replica_seed
    trees = batched_trees(args.neurons, seed=replica_seed(rank), processes=min(16, os.cpu_count() or 1), lo=lo, hi=hi)
    currents = batched_currents(args.neurons, seed=rank)
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    log(f"trees ready ({sum(len(t) for t in trees)} segments) in {time.perf_counter() - t_setup:.1f} s")
    extra = {}
    if not args.quick and rank == 0:
        # The sample: the batch's largest neurons and its first others, half each.
        k = args.acc_neurons
        sizes = np.array([len(t) for t in trees])
        largest = [int(i) for i in np.argsort(-sizes, kind="stable")[:k // 2]]
        pick = largest + [i for i in range(len(trees)) if i not in largest][:k - len(largest)]
        extra["accuracy"] = accuracy([trees[i] for i in pick], [currents[i] for i in pick], args.tol, local,
                                     args.acc_steps, args.ref_tol, args.format, bool(args.lump),
                                     label=f"the batch's {len(largest)} largest neurons and its first "
                                           f"{len(pick) - len(largest)} others")
        log(f"accuracy: {extra['accuracy']}")
        small = [i for i in range(len(trees)) if sizes[i] <= 2000][:4]
        extra["accuracy"]["reference_gap"] = epsilon_gap([trees[i] for i in small], [currents[i] for i in small],
                                                         local, 2000, args.ref_tol)
        log(f"epsilon gap: {extra['accuracy']['reference_gap']}")
        extra["plain_fp64"] = plain_timing(trees[:64], currents[:64], args.tol, local)
        log(f"plain: {extra['plain_fp64']}")

    from neuwon_gb300 import _lib
    if not args.quick and rank == 0 and args.adjoint_steps > 0:
        extra["adjoint"] = adjoint_leg(local, args.adjoint_steps, overlap=args.adjoint_overlap)
        log(f"adjoint: {extra['adjoint']}")
    if not args.quick and rank == 0 and args.network_steps > 0:
        extra["network"] = network_leg(local, args.network_steps)
        log(f"network: {extra['network']}")
    if not args.quick and rank == 0 and args.wide_steps > 0:
        extra["wide"] = wide_leg(local, args.study_segments, args.wide_tol, args.wide_steps)
        log(f"wide: {extra['wide']}")
    t_build = time.perf_counter()
    model, neurons = build_model(trees, currents, precision="f32", tolerance=args.tol, conserve=True,
                                 device=local, fmt=args.format, lump=bool(args.lump))
    log(f"host model built in {time.perf_counter() - t_build:.1f} s")
    model._sync()
    ctx = model._ctx
    ctx.call("nw_set_tuning", args.lanes, args.threads, 0)
    ctx.call("nw_set_option", b"bulk_pipeline", args.bulk)
    ctx.set_option("fusion_depth", max(1, min(args.fusion, args.steps)))
    ctx.call("nw_synchronize")
    build_s = time.perf_counter() - t_build
    log(f"device model + propagator in {build_s:.1f} s")
    tuned = None
    if args.autotune > 0:
        t0 = time.perf_counter()
        tuned = ctx.autotune(args.autotune)
        tuned["seconds"] = time.perf_counter() - t0
        log(f"autotune: {tuned}")
    rows, nnz, stored, pbytes = (ctypes.c_int64() for _ in range(4))
    ctx.call("nw_propagator_stats", ctypes.byref(rows), ctypes.byref(nnz), ctypes.byref(stored), ctypes.byref(pbytes))
    n = model._n
    r_kept = nnz.value / n
    r_stored = stored.value / n
    windows_per_row = ({w: ctx.get_option(f"windows_{w}") / n for w in (8, 4, 2, 1)}
                       if args.format == "windows" else None)
    bulk_active = ctypes.c_int64()
    ctx.call("nw_get_option", b"bulk_pipeline_active", ctypes.byref(bulk_active))
    lanes = ctypes.c_int(); thr = ctypes.c_int(); cps = ctypes.c_int()
    ctx.call("nw_get_tuning", ctypes.byref(lanes), ctypes.byref(thr), ctypes.byref(cps))
    sptr = ctypes.c_void_p()
    ctx.call("nw_get_stream", ctypes.byref(sptr))
    stream = torch.cuda.ExternalStream(sptr.value, device=torch.device("cuda", local))

    F = ctx.get_option("fusion_depth") or args.steps
    # Warm-up.
    w = args.warmup
    while w > 0:
        k = min(F, w)
        model.advance(k)
        w -= k
    ctx.call("nw_synchronize")

    # Timed device-resident region: the K steps are one nw_advance call, which
    # replays one CUDA graph of ceil(K / F) launches of F fused steps.  The graph
    # is captured (not run) beforehand.
    K = args.steps
    ctx.set_option("prepare_graph", K)
    n_launch = -(-K // F)
    replays0 = ctx.get_option("graph_replays")
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    ctx.call("nw_synchronize")
    with ClockSampler(local) as clocks:
        with torch.cuda.stream(stream):
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            ctx.advance(K, _lib.PATH_BATCHED)
            ev1.record(stream)
        ev1.synchronize()
    graph_replayed = ctx.get_option("graph_replays") - replays0 == 1
    model.input_hook.ticks += 2 * K
    model.advance_hook.ticks += K
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    from neuwon_gb300.replicas import aggregate
    agg = aggregate(ev0.elapsed_time(ev1), n, K, dist, device=f"cuda:{local}")
    ms, n_total, value = agg["ms"], agg["segments"], agg["value"]
    # Average launch of the batched kernel, per fused step (the region holds the
    # n_launch kernels plus one clock write and n_launch 4-byte memsets).
    per_step_launch_ms = ms / K

    # End to end through the C ABI with host buffers: per step, the clamp currents
    # go host->device and every segment voltage comes back device->host.
    # nw_advance_host_async: each step's voltages are staged on the device and copied
    # to one of two pinned buffers on a second stream while the next step runs; the
    # timed region ends when both streams are done.  nw_advance_host (one step per
    # call, synchronous) is timed beside it.
    stim = torch.empty(len(neurons), dtype=torch.float64, pin_memory=True)
    stim.copy_(torch.from_numpy(np.asarray(currents, dtype=np.float64) * 1e-9))
    vouts = [torch.empty(n, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    E = max(10, min(K, 200))
    sp = ctypes.c_void_p(stim.data_ptr())
    vp = [ctypes.c_void_p(v.data_ptr()) for v in vouts]
    ctx.call("nw_advance_host_async", 1, sp, vp[0], 2)
    ctx.call("nw_advance_host", 1, sp, vp[1], 2)
    ctx.call("nw_synchronize")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(E):
        ctx.call("nw_advance_host_async", 1, sp, vp[k % 2], 2)
    ctx.call("nw_synchronize")
    e2e_s = time.perf_counter() - t0
    vcheck = vouts[(E - 1) % 2].numpy().copy()
    vdev = model.get_data("Segment.voltage")
    finite = bool(np.all(np.isfinite(vcheck)))
    last_step_read = bool(np.array_equal(np.sort(vcheck), np.sort(vdev.astype(np.float32))))
    t0 = time.perf_counter()
    for _ in range(E):
        ctx.call("nw_advance_host", 1, sp, vp[0], 2)
    e2e_sync_s = time.perf_counter() - t0
    model.input_hook.ticks += 2 * (2 * E + 2)
    model.advance_hook.ticks += 2 * E + 2
    e2e_value = aggregate(e2e_s * 1e3, n, E, dist, device=f"cuda:{local}")["value"]
    e2e_sync_value = aggregate(e2e_sync_s * 1e3, n, E, dist, device=f"cuda:{local}")["value"]

    from neuwon_gb300.morphology import EPSILON  # noqa: F401
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    B_alg = algorithmic_bytes_per_segment_step(r_kept)
    B_fmt = format_bytes_per_segment_step(pbytes.value / n)
    achieved = B_alg * n / (per_step_launch_ms * 1e-3) / 1e9
    achieved_fmt = B_fmt * n / (per_step_launch_ms * 1e-3) / 1e9

    log(f"timed: {ms / K:.3f} ms/step; e2e {e2e_s / E * 1e3:.3f} ms/step")
    cpu = None
    if not args.quick and rank == 0:
        cpu = cpu_sample(trees, currents, args.tol, bool(args.lump), time_budget_s=15.0)
        cpu["config1"] = cpu_baseline_config1(local)
        log(f"config 1: {cpu['config1']}")
    spikes = model.get_data("Neuron.spike_count")
    model.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "segment-steps/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded trees; no dataset involved)",
        "config": {"workload": workload_name(len(neurons), lo, hi),
                   "segments": n_total, "segments_rank0": n, "neurons": len(neurons) * world,
                   "propagator_tolerance": args.tol,
                   "propagator_pruning": ("lumped (each pruned entry moved to the nearest kept entry on the tree "
                                          "path to the row's segment; unvisited remainder to the diagonal)"
                                          if args.lump else "charge-conserving (pruned mass returned to the diagonal)"),
                   "propagator_format": args.format,
                   "propagator_entries_per_row": r_kept, "stored_entries_per_row": r_stored,
                   **({"windows_per_row": windows_per_row} if windows_per_row else {}),
                   "propagator_build_s": build_s, "steps_per_launch": F, "lanes_per_row": lanes.value,
                   "autotune": tuned, "cuda_graph": {"replayed": graph_replayed, "launches_in_graph": n_launch},
                   "propagator_stream": "cp.async.bulk ring (4 x 256 entries per warp)" if bulk_active.value
                   else "register loads",
                   "threads": thr.value, "l2": "inputs larger than L2 (propagator "
                   f"{pbytes.value / 1e9:.1f} GB), no flush", "mechanisms": ["hh", "na8 (8-state Markov Na, LTI voltage table 1600 x 0.1 mV, linear)"],
                   "parallelism": f"replicas x{world}"},
        # achieved / frac: the compulsory bytes of the stored layout (quads: 18 B per
        # window of 4 column slots, no diagonal) per launch over the launch time, the
        # bytes the kernel must move (ncu traffic is 1.00x of them); the formula of
        # 8 B per kept entry (value + int32 column, diagonal included) is kept as
        # achieved_alg / frac_alg: the compressed layout moves fewer bytes than it
        # counts, so frac_alg can exceed 1.
        "roofline": {"bound": "hbm", "achieved": achieved_fmt, "peak": peak, "unit": "GB/s",
                     "frac": achieved_fmt / peak,
                     "traffic": (NCU_TRAFFIC_PER_SEGMENT_STEP[(args.format, args.tol, args.lump)] * n * F
                                 if n == NCU_TRAFFIC_SEGMENTS
                                 and (args.format, args.tol, args.lump) in NCU_TRAFFIC_PER_SEGMENT_STEP else None),
                     "traffic_unit": f"bytes per launch of {F} steps (ncu dram__bytes_read+write)",
                     "algorithmic_bytes_per_launch": B_fmt * n * F,
                     "peak_source": peak_src,
                     "bytes_per_segment_step": B_fmt,
                     "achieved_alg": achieved, "frac_alg": achieved / peak,
                     "alg_bytes_per_segment_step": B_alg, "alg_bytes_per_launch": B_alg * n * F,
                     "kernel": "batched_advance_kernel", "launch_ms_per_step": per_step_launch_ms},
        "clocks": clocks.summary(),
        "e2e": {"value": e2e_value, "unit": "segment-steps/s", "steps": E,
                "h2d_bytes_per_step": int(stim.numel() * 8), "d2h_bytes_per_step": int(vouts[0].numel() * 4),
                "api": "nw_advance_host_async (C ABI), one step per call: clamp currents in and every voltage "
                       "out each step, the copy out overlapping the next step; both streams synchronised at the end",
                "finite": finite, "last_step_read": last_step_read,
                "sync_call": {"value": e2e_sync_value, "api": "nw_advance_host, one step per call, synchronous"}},
        "gpu_launches": n_launch + 1,
        "cpu_baseline": cpu,
        "spikes_total": int(spikes.sum()),
        "setup_s": time.perf_counter() - t_setup,
    }
    line.update(extra)
    if "plain_fp64" in extra:
        line["batched_over_plain"] = value / world / extra["plain_fp64"]["value"]
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
