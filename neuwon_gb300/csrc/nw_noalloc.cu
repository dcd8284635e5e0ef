// Electric half step on caller-owned device arrays, with no device allocation.
//
// Some callers cannot call cudaMalloc: a host application whose device memory
// is owned by its own pool allocator (every byte must come from that pool, and
// a foreign cudaMalloc would bypass its accounting or fail under its limit),
// or a simulation loop that must not allocate between steps.  This entry
// point lets them run the membrane update and propagator multiply of one half
// step (neuwon/rxd/neuron/electric.py:56-76) on arrays they allocated.  The
// vector the propagator multiplies is scratch; it lives in the file-scope
// array below, which the CUDA runtime creates on a GPU when this file's
// device code is loaded there (with lazy module loading, the default, at the
// first call on that device) and keeps until the process exits.
#include <mutex>
#include <vector>

#include <cuda.h>

#include "nw_internal.cuh"

namespace {

// NW_NOALLOC_MAX_SEGMENTS doubles = 8 MiB on every GPU that loads the library.
static __device__ __align__(256) double g_noalloc_x[NW_NOALLOC_MAX_SEGMENTS];

// The scratch array's device address, looked up once per CUDA context.  The
// name g_noalloc_x is only a host-side stand-in, so the address must come from
// cudaGetSymbolAddress with the context current; a context is identified by
// its process-unique id (cuCtxGetId), so a context created after a device reset
// or a non-primary context gets its own lookup.
struct ScratchEntry {
    unsigned long long ctx_id;
    double* ptr;
};
std::mutex g_setup_mutex;
std::vector<ScratchEntry> g_scratch;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Id of the current context (0 when none is current yet: the runtime then
// makes the device's primary context current in cudaGetSymbolAddress).
int current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return NW_ERR_CUDA;
        get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS) return NW_ERR_CUDA;
    *id = 0;
    if (c && get_id(c, id) != CUDA_SUCCESS) return NW_ERR_CUDA;
    return NW_OK;
}

int scratch_in_current_context(double** out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc != NW_OK) return rc;
    if (id != 0) {
        for (const ScratchEntry& e : g_scratch)
            if (e.ctx_id == id) {
                *out = e.ptr;
                return NW_OK;
            }
    }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_x) != cudaSuccess || p == nullptr) return NW_ERR_CUDA;
    if (id == 0) {                                  // the lookup made the primary context current
        rc = current_context_id(&id);
        if (rc != NW_OK) return rc;
    }
    g_scratch.push_back(ScratchEntry{id, static_cast<double*>(p)});
    *out = static_cast<double*>(p);
    return NW_OK;
}

// x = E - (E - V) exp(-dt G / C) + (dt/2) I / C, and the integral of V over the
// half step, as electric.py:60-76 computes them.
__global__ void noalloc_membrane_kernel(int64_t n, const double* __restrict__ V,
                                        const double* __restrict__ C, const double* __restrict__ G,
                                        const double* __restrict__ E, const double* __restrict__ I,
                                        double half_step_ms, double* __restrict__ x,
                                        double* __restrict__ Vint) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = half_step_ms * 1e-3;
    const double dv_currents = half_step_ms * I[i] / C[i];
    const double exponent = -dt * G[i] / C[i];
    const double alpha = exp(exponent);
    const double diff_v = E[i] - V[i];
    x[i] = E[i] - diff_v * alpha + dv_currents;
    if (Vint) Vint[i] = dt * E[i] - exponent * diff_v * alpha + 0.5 * dt * dv_currents;
}

// V = P x with P in CSR (diagonal included), one thread per row.
__global__ void noalloc_propagate_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                         const int32_t* __restrict__ col, const double* __restrict__ val,
                                         const double* __restrict__ x, double* __restrict__ V) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    double acc = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) acc += val[k] * x[col[k]];
    V[r] = acc;
}

}  // namespace

extern "C" int nw_electric_half_step_noalloc(int64_t num_segments, const int64_t* rowptr,
                                             const int32_t* col, const double* val, double* voltage,
                                             const double* capacitance, const double* sum_conductance,
                                             const double* driving_voltage, const double* sum_current,
                                             double* integral_voltage, double half_step_ms, void* stream) {
    if (num_segments < 0) return NW_ERR_ARG;
    if (num_segments > NW_NOALLOC_MAX_SEGMENTS) return NW_ERR_LIMIT;
    if (num_segments == 0) return NW_OK;
    if (!rowptr || !col || !val || !voltage || !capacitance || !sum_conductance || !driving_voltage ||
        !sum_current || !(half_step_ms > 0.0))
        return NW_ERR_ARG;
    // An error left by the caller's earlier work is reported, not consumed.
    if (cudaPeekAtLastError() != cudaSuccess) return NW_ERR_CUDA;
    double* x = nullptr;
    int rc = scratch_in_current_context(&x);
    if (rc != NW_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int threads = 256;
    const unsigned blocks = (unsigned)((num_segments + threads - 1) / threads);
    // The whole scratch range [0, num_segments) is written before it is read,
    // so nothing has to be cleared between calls.
    noalloc_membrane_kernel<<<blocks, threads, 0, s>>>(num_segments, voltage, capacitance, sum_conductance,
                                                     driving_voltage, sum_current, half_step_ms, x,
                                                     integral_voltage);
    if (cudaGetLastError() != cudaSuccess) return NW_ERR_CUDA;
    noalloc_propagate_kernel<<<blocks, threads, 0, s>>>(num_segments, rowptr, col, val, x, voltage);
    if (cudaGetLastError() != cudaSuccess) return NW_ERR_CUDA;
    return NW_OK;
}
