// Electric half step on caller-owned device arrays, with no device allocation.
//
// Some callers cannot call cudaMalloc: a host application whose device memory
// is owned by its own pool allocator (every byte must come from that pool, and
// a foreign cudaMalloc would bypass its accounting or fail under its limit),
// or a simulation loop that must not allocate between steps.  This entry
// point lets them run the membrane update and propagator multiply of one half
// step (neuwon/rxd/neuron/electric.py:56-76) on arrays they allocated.  The
// vector the propagator multiplies is scratch; it lives in the file-scope
// array below, which the CUDA runtime creates once per GPU when this library's
// device code is loaded and keeps until the process exits.
#include <mutex>

#include "nw_internal.cuh"

namespace {

// NW_NOALLOC_MAX_SEGMENTS doubles = 8 MiB on every GPU that loads the library.
static __device__ __align__(256) double g_noalloc_x[NW_NOALLOC_MAX_SEGMENTS];

constexpr int kMaxDevices = 256;
std::mutex g_setup_mutex;
double* g_scratch[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device.  The name
// g_noalloc_x is only a host-side stand-in, so the address must come from
// cudaGetSymbolAddress, once per device with that device current.
int scratch_on_current_device(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return NW_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return NW_ERR_LIMIT;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch[dev] == nullptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_x);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return NW_ERR_CUDA;
        }
        g_scratch[dev] = static_cast<double*>(p);
    }
    *out = g_scratch[dev];
    return NW_OK;
}

// x = E - (E - V) exp(-dt G / C) + (dt/2) I / C, as electric.py:70-75 computes it.
__global__ void noalloc_membrane_kernel(int64_t n, const double* __restrict__ V,
                                        const double* __restrict__ C, const double* __restrict__ G,
                                        const double* __restrict__ E, const double* __restrict__ I,
                                        double half_step_ms, double* __restrict__ x) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = half_step_ms * 1e-3;
    const double dv_currents = half_step_ms * I[i] / C[i];
    const double exponent = -dt * G[i] / C[i];
    const double alpha = exp(exponent);
    const double diff_v = E[i] - V[i];
    x[i] = E[i] - diff_v * alpha + dv_currents;
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
                                             double half_step_ms, void* stream) {
    if (num_segments < 0) return NW_ERR_ARG;
    if (num_segments > NW_NOALLOC_MAX_SEGMENTS) return NW_ERR_LIMIT;
    if (num_segments == 0) return NW_OK;
    if (!rowptr || !col || !val || !voltage || !capacitance || !sum_conductance || !driving_voltage ||
        !sum_current || !(half_step_ms > 0.0))
        return NW_ERR_ARG;
    double* x = nullptr;
    int rc = scratch_on_current_device(&x);
    if (rc != NW_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int threads = 256;
    const unsigned blocks = (unsigned)((num_segments + threads - 1) / threads);
    // The whole scratch range [0, num_segments) is written before it is read,
    // so nothing has to be cleared between calls.
    noalloc_membrane_kernel<<<blocks, threads, 0, s>>>(num_segments, voltage, capacitance, sum_conductance,
                                                     driving_voltage, sum_current, half_step_ms, x);
    noalloc_propagate_kernel<<<blocks, threads, 0, s>>>(num_segments, rowptr, col, val, x, voltage);
    return cudaGetLastError() == cudaSuccess ? NW_OK : NW_ERR_CUDA;
}
