/*
 * CPU restatement of NEUWON's staggered Model.advance() -- TEST ORACLE and
 * CPU baseline only (never linked into the product library).
 *
 * FP64, OpenMP over segments / instances.  Follows:
 *   neuwon/rxd/rxd_model.py:63-80     advance: species(dt/2), mechanisms, species(dt/2), AP
 *   neuwon/rxd/rxd_model.py:91-113    accumulators, input clock tick, driving voltage
 *   neuwon/rxd/species.py:256-260     nonspecific conductance scatter (summed here)
 *   neuwon/rxd/neuron/electric.py:56-76  exact membrane update and V <- P x
 *   nmodl_library/artificial/hh.mod + neuwon/rxd/nmodl/solver.py:48-55  HH gates
 *   neuwon/rxd/neuron/neuron.py:72-75  AP detector
 *   neuwon/database/time.py:287-302   current clamps on the half-step clock
 *   neuwon/rxd/lti_sim/codegen.py:39-106  kinetic scheme: voltage bucket, polynomial
 *                                     table [bucket][col][row][term], CONSERVE renormalisation
 *
 * Build: see oracle/Makefile (gcc -O3 -fopenmp -shared).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int64_t n_seg;
    /* propagator, CSR with the diagonal, global column indices */
    const int64_t* rowptr; const int32_t* col; const double* val;
    /* electric state */
    double* V; double* Vint; const double* C; const double* Inonspec;
    double time_step;              /* ms */
    /* hh instances sorted by segment; inst range of segment i: [seg_ptr[i], seg_ptr[i+1]) */
    int64_t m; const int64_t* hh_seg_ptr; const int64_t* hh_seg;
    double* gm; double* gh; double* gn; const double* cna; const double* ck; const double* cl;
    double ena, ek, el, celsius;
    /* clamps grouped by segment: [clamp_ptr[i], clamp_ptr[i+1]) */
    const int64_t* clamp_ptr; const double* clamp_amp; const int64_t* clamp_first; const int64_t* clamp_count;
    /* detectors */
    int64_t n_neuron; const int64_t* det_seg; const double* det_thr;
    uint8_t* ap_state; uint8_t* ap_detected; int64_t* spike_count;
    /* scratch [n_seg] and clock */
    double* x;
    int64_t input_ticks;
    int g_valid;
    /* kinetic instances sorted by segment; states state-major [S][km] */
    int64_t km; const int64_t* kin_seg_ptr; const int64_t* kin_seg;
    double* kstate; const double* kgcoef; const double* ktable;
    int64_t kS, kT, knb, knopen; const int64_t* kopen;
    double kvmin, kfrq, kcs, kerev;
} oracle_model;

static double vtrap(double x, double y) {
    if (fabs(x / y) < 1e-6) return y * (1 - x / y / 2);
    return x / (exp(x / y) - 1);
}

static void half_step(oracle_model* m) {
    const double h = 0.5 * m->time_step, h_s = h * 1e-3;
    const int64_t tick = ++m->input_ticks;
    const int gv = m->g_valid;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m->n_seg; ++i) {
        double gna = 0, gk = 0, gl = 0;
        if (gv && m->m) {
            for (int64_t k = m->hh_seg_ptr[i]; k < m->hh_seg_ptr[i + 1]; ++k) {
                double mm = m->gm[k], hh = m->gh[k], nn = m->gn[k];
                gna += m->cna[k] * mm * mm * mm * hh;
                gk += m->ck[k] * nn * nn * nn * nn;
                gl += m->cl[k];
            }
        }
        double G = (gna + gk) + gl;
        double GE = (gna * m->ena + gk * m->ek) + gl * m->el;
        if (gv && m->km) {
            double gkin = 0.0;
            for (int64_t k = m->kin_seg_ptr[i]; k < m->kin_seg_ptr[i + 1]; ++k) {
                double open = 0.0;
                for (int64_t o = 0; o < m->knopen; ++o) open += m->kstate[m->kopen[o] * m->km + k];
                gkin += m->kgcoef[k] * open;
            }
            G += gkin;
            GE += gkin * m->kerev;
        }
        double I = m->Inonspec ? m->Inonspec[i] : 0.0;
        if (m->clamp_ptr)
            for (int64_t c = m->clamp_ptr[i]; c < m->clamp_ptr[i + 1]; ++c)
                if (tick >= m->clamp_first[c] && tick < m->clamp_first[c] + m->clamp_count[c]) I += m->clamp_amp[c];
        double E = GE / G;
        if (isnan(E)) E = 0.0;
        double dv = h * I / m->C[i];
        double expo = -h_s * G / m->C[i];
        double alpha = exp(expo);
        double diff = E - m->V[i];
        m->x[i] = E - diff * alpha + dv;
        m->Vint[i] = h_s * E - expo * diff * alpha + (.5 * h_s * dv);
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < m->n_seg; ++i) {
        double acc = 0.0;
        for (int64_t k = m->rowptr[i]; k < m->rowptr[i + 1]; ++k) acc += m->val[k] * m->x[m->col[k]];
        m->V[i] = acc;
    }
}

static void mechanisms(oracle_model* m) {
    const double q10 = pow(3.0, (m->celsius - 6.3) / 10.0);
    const double dt = m->time_step;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m->n_seg; ++i) {
        for (int64_t k = m->hh_seg_ptr[i]; k < m->hh_seg_ptr[i + 1]; ++k) {
            double v = m->V[m->hh_seg[k]];
            double a = .1 * vtrap(-(v + 40), 10), b = 4 * exp(-(v + 65) / 18);
            double mtau = 1 / (q10 * (a + b)), minf = a / (a + b);
            a = .07 * exp(-(v + 65) / 20); b = 1 / (exp(-(v + 35) / 10) + 1);
            double htau = 1 / (q10 * (a + b)), hinf = a / (a + b);
            a = .01 * vtrap(-(v + 55), 10); b = .125 * exp(-(v + 65) / 80);
            double ntau = 1 / (q10 * (a + b)), ninf = a / (a + b);
            m->gm[k] = minf + (m->gm[k] - minf) * exp(-dt / mtau);
            m->gh[k] = hinf + (m->gh[k] - hinf) * exp(-dt / htau);
            m->gn[k] = ninf + (m->gn[k] - ninf) * exp(-dt / ntau);
        }
    }
}

static void kinetic(oracle_model* m) {
    const int64_t S = m->kS, T = m->kT;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < m->km; ++k) {
        double x = (m->V[m->kin_seg[k]] - m->kvmin) * m->kfrq;
        int64_t b = (int64_t)trunc(x);
        double loc = x - (double)b;
        if (b > m->knb - 1) { b = m->knb - 1; loc = 1.0; }
        if (b < 0) { b = 0; loc = 0.0; }
        double s_old[16], s_new[16];
        for (int64_t c = 0; c < S; ++c) { s_old[c] = m->kstate[c * m->km + k]; s_new[c] = 0.0; }
        const double* tb = m->ktable + b * S * S * T;
        for (int64_t c = 0; c < S; ++c)
            for (int64_t r = 0; r < S; ++r) {
                const double* t = tb + (c * S + r) * T;
                double poly = 0.0, p = 1.0;
                for (int64_t u = 0; u < T; ++u) { poly += t[u] * p; p *= loc; }
                s_new[r] += poly * s_old[c];
            }
        double sum = 0.0;
        for (int64_t r = 0; r < S; ++r) sum += s_new[r];
        const double f = m->kcs > 0 ? m->kcs / sum : 1.0;
        for (int64_t r = 0; r < S; ++r) m->kstate[r * m->km + k] = s_new[r] * f;
    }
}

int oracle_advance(oracle_model* m, int k_steps) {
    for (int s = 0; s < k_steps; ++s) {
        half_step(m);
        if (m->m) mechanisms(m);
        if (m->km) kinetic(m);
        if (m->m || m->km) m->g_valid = 1;
        half_step(m);
        for (int64_t j = 0; j < m->n_neuron; ++j) {
            int over = m->V[m->det_seg[j]] >= m->det_thr[j];
            int det = over && !m->ap_state[j];
            m->ap_detected[j] = (uint8_t)det;
            m->ap_state[j] = (uint8_t)over;
            m->spike_count[j] += det;
        }
    }
    return 0;
}

int oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/*
 * Lumped pruning of one neuron's dense propagator P (n x n, row-major; parent[i]
 * = parent within the neuron or -1), the restatement in
 * oracle/reference_step.py: lump_and_conserve in C: walking the tree outward
 * from row i's segment, expanding nodes whose |P_iu| reaches tol *
 * explore_factor, a visited entry below tol is added to the nearest kept entry
 * on the path back to i; what the walk never reaches goes to the diagonal.
 * Neighbours are pushed children first (creation order), then the parent, and
 * popped last-in first-out, as the restatement does.  out (n x n) is
 * overwritten.  Returns 0, or -1 when a scratch allocation fails.
 */
int oracle_lump(const double* P, const int64_t* parent, int64_t n, double tol, double explore_factor,
                double* out) {
    int64_t* child_ptr = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    int64_t* child = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    if (!child_ptr || !child) { free(child_ptr); free(child); return -1; }
    for (int64_t c = 0; c < n; ++c)
        if (parent[c] >= 0) child_ptr[parent[c] + 1]++;
    for (int64_t u = 0; u < n; ++u) child_ptr[u + 1] += child_ptr[u];
    {
        int64_t* fill = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
        if (!fill) { free(child_ptr); free(child); return -1; }
        for (int64_t u = 0; u < n; ++u) fill[u] = child_ptr[u];
        for (int64_t c = 0; c < n; ++c)
            if (parent[c] >= 0) child[fill[parent[c]]++] = c;
        free(fill);
    }
    const double explore = tol * explore_factor;
    int failed = 0;
#pragma omp parallel
    {
        /* (node, came from, nearest kept toward i); a tree node is reached once per row. */
        int64_t* stack = (int64_t*)malloc((size_t)3 * (size_t)(n > 0 ? n : 1) * sizeof(int64_t));
        if (!stack) {
#pragma omp atomic write
            failed = 1;
        }
#pragma omp for schedule(dynamic, 16)
        for (int64_t i = 0; i < n; ++i) {
            if (!stack) continue;
            const double* row = P + i * n;
            double* o = out + i * n;
            double total = 0.0, kept = 0.0;
            for (int64_t u = 0; u < n; ++u) { total += row[u]; o[u] = 0.0; }
            int64_t top = 0;
            stack[0] = i; stack[1] = -1; stack[2] = i; top = 1;
            while (top > 0) {
                --top;
                const int64_t u = stack[3 * top], w = stack[3 * top + 1];
                int64_t t = stack[3 * top + 2];
                const double v = row[u];
                if (fabs(v) >= tol || u == i) { o[u] += v; t = u; }
                else o[t] += v;
                if (fabs(v) < explore && u != i) continue;
                for (int64_t k = child_ptr[u]; k < child_ptr[u + 1]; ++k) {
                    const int64_t x = child[k];
                    if (x != w) { stack[3 * top] = x; stack[3 * top + 1] = u; stack[3 * top + 2] = t; ++top; }
                }
                const int64_t p = parent[u];
                if (p >= 0 && p != w) { stack[3 * top] = p; stack[3 * top + 1] = u; stack[3 * top + 2] = t; ++top; }
            }
            for (int64_t u = 0; u < n; ++u) kept += o[u];
            o[i] += total - kept;
        }
        free(stack);
    }
    free(child_ptr);
    free(child);
    return failed ? -1 : 0;
}
