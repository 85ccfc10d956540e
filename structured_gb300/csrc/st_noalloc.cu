// Allocation-free variant of the residual L2-norm reduction.
//
// Some callers cannot allocate device memory once they are running: a host
// application that has reserved the whole device for its own memory pool, or
// a time-stepping loop that must not pay the device-wide synchronisation that
// cudaMalloc / cudaFree can impose.  st_norms_noalloc serves them: the caller
// passes the residual and the output on the device, and the per-block partial
// sums live in a fixed array in this file instead of a context buffer.
#include <cuda_runtime.h>

#include <cmath>

#include "st_context.h"

namespace {

constexpr int NA_MAX_COMPONENTS = 8;   // largest nq accepted
constexpr int NA_MAX_BLOCKS = 1024;    // partial sums per component
constexpr int NA_THREADS = 256;

// Scratch for the partial sums: NA_MAX_BLOCKS x NA_MAX_COMPONENTS doubles
// (64 KiB).  Every device that loads this library holds one copy until the
// process exits.  All calls share it, so calls that overlap on the GPU (on
// different streams, or from different host threads) race on it.
static __device__ __align__(256) double g_norm_scratch[NA_MAX_BLOCKS * NA_MAX_COMPONENTS];

// Device address of g_norm_scratch in the current device's copy of this
// module.  The host-side symbol is only a stand-in; kernels must receive the
// address that cudaGetSymbolAddress returns.  It is looked up on every call
// (a table lookup in the runtime, no allocation) rather than cached, so the
// address stays valid after cudaDeviceReset or when the runtime reloads the
// module in a new primary context.  The first lookup on a device loads the
// module there; make that first call outside any stream capture.
int scratch_address(double** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_norm_scratch);
    if (e != cudaSuccess) return stx::cuda_fail(e, "st_norms_noalloc: cudaGetSymbolAddress");
    *out = static_cast<double*>(p);
    return ST_OK;
}

__global__ void __launch_bounds__(NA_THREADS) k_norm_partial_na(const double* __restrict__ r, size_t ncell, int nq,
                                                                double* __restrict__ part) {
    // fully unrolled with a guard on nq, so acc stays in registers
    double acc[NA_MAX_COMPONENTS];
#pragma unroll
    for (int k = 0; k < NA_MAX_COMPONENTS; k++) acc[k] = 0.0;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < ncell; idx += (size_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < NA_MAX_COMPONENTS; k++)
            if (k < nq) {
                const double x = r[idx * nq + k];
                acc[k] = fma(x, x, acc[k]);
            }
    __shared__ double sm[NA_THREADS / 32][NA_MAX_COMPONENTS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NA_MAX_COMPONENTS; k++) {
        if (k >= nq) break;
        double x = acc[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sm[wid][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < nq) {
        double s = 0.0;
        for (int w = 0; w < NA_THREADS / 32; w++) s += sm[w][threadIdx.x];
        part[blockIdx.x * NA_MAX_COMPONENTS + threadIdx.x] = s;
    }
}

__global__ void k_norm_final_na(const double* __restrict__ part, int nblocks, int nq, double* __restrict__ out) {
    if (threadIdx.x < nq) {
        double s = 0.0;
        for (int b = 0; b < nblocks; b++) s += part[b * NA_MAX_COMPONENTS + threadIdx.x];
        out[threadIdx.x] = sqrt(s);
    }
}

}  // namespace

extern "C" {

int st_norms_noalloc(const double* rhs_dev, long long ncell, int nq, double* out_dev, void* stream) {
    if (!rhs_dev || !out_dev) return stx::fail(ST_ERR_ARG, "st_norms_noalloc: null pointer");
    if (nq < 1 || nq > NA_MAX_COMPONENTS)
        return stx::fail(ST_ERR_ARG, "st_norms_noalloc: nq must be in [1, 8] (scratch holds 8 components)");
    if (ncell < 1) return stx::fail(ST_ERR_ARG, "st_norms_noalloc: ncell must be positive");
    double* part = nullptr;
    int rc = scratch_address(&part);
    if (rc) return rc;
    long long want = (ncell + NA_THREADS - 1) / NA_THREADS;
    const int nblocks = (int)(want < NA_MAX_BLOCKS ? want : NA_MAX_BLOCKS);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // every partial slot that the final pass reads is rewritten by this call
    k_norm_partial_na<<<nblocks, NA_THREADS, 0, s>>>(rhs_dev, (size_t)ncell, nq, part);
    k_norm_final_na<<<1, 32, 0, s>>>(part, nblocks, nq, out_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return stx::cuda_fail(e, "st_norms_noalloc launch");
    return ST_OK;
}

}  // extern "C"
