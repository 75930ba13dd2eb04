// suli_noalloc.cu -- divergence and max|div| (the check CONMASSA makes after
// every step) for callers that may not allocate device memory.
//
// Who needs this: a host program that owns every device buffer through its
// own allocator -- for example a Fortran code whose arrays live in CUDA
// Fortran or OpenACC data regions, or an application that runs the GPU under
// a fixed memory budget -- cannot let a library call cudaMalloc behind its
// back: cudaMalloc can synchronise the device, takes memory outside the
// caller's pool and can fail at an arbitrary point of a run.  This entry point
// works on buffers the caller already owns and allocates nothing.
//
// The reduction needs a little scratch (one partial maximum per z-plane and
// an arrival counter).  It lives in a file-scope static __device__ array of
// SULI_NOALLOC_MAX_PLANES + 1 doubles (32 KiB + 8 bytes), which every GPU that
// loads the library holds until the process exits.  Host code cannot use the
// array's name as a device address, so the first call on each device looks
// the address up with cudaGetSymbolAddress (with that device current) and
// caches it; that first call should therefore come before any stream capture.
// All calls share the one array: calls whose work overlaps on the GPU race on
// it and must be serialised by the caller (one stream, or events).
#include "../../include/suli_gpu.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#define SULI_NOALLOC_MAX_PLANES 4096
#define SULI_NOALLOC_MAX_DEVICES 64

// [0, MAX_PLANES): per-plane partial maxima; [MAX_PLANES]: arrival counter
static __device__ __align__(256) double g_noalloc_scratch[SULI_NOALLOC_MAX_PLANES + 1];

namespace {

std::mutex g_mu;
double *g_scratch_addr[SULI_NOALLOC_MAX_DEVICES] = {nullptr};

// one block per z-plane k; reference layout (column-major, Fortran bounds):
// u(0:nx+2,0:ny+1,0:nz+1), v(0:nx+1,0:ny+2,0:nz+1), w(0:nx+1,0:ny+1,0:nz+2),
// div(1:nx,1:ny,1:nz)
__global__ void k_conmassa_noalloc(const double *__restrict__ u, const double *__restrict__ v,
                                   const double *__restrict__ w, int nx, int ny, int nz, double dx, double dy,
                                   double dz, double *__restrict__ div, double *__restrict__ maxdiv,
                                   double *__restrict__ scratch)
{
    const int k = blockIdx.x + 1;
    const long long su1 = nx + 3, su2 = su1 * (ny + 2);
    const long long sv1 = nx + 2, sv2 = sv1 * (ny + 3);
    const long long sw1 = nx + 2, sw2 = sw1 * (ny + 2);
    const long long sd1 = nx, sd2 = (long long)nx * ny;
    double m = 0.0;
    for (int t = threadIdx.x; t < nx * ny; t += blockDim.x) {
        const int i = 1 + t % nx, j = 1 + t / nx;
        const double d = (u[(i + 1) + su1 * j + su2 * k] - u[i + su1 * j + su2 * k]) / dx +
                         (v[i + sv1 * (j + 1) + sv2 * k] - v[i + sv1 * j + sv2 * k]) / dy +
                         (w[i + sw1 * j + sw2 * (k + 1)] - w[i + sw1 * j + sw2 * k]) / dz;
        div[(i - 1) + sd1 * (j - 1) + sd2 * (k - 1)] = d;
        m = fmax(m, fabs(d));
    }
    // block maximum
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int q = 0; q < (int)(blockDim.x + 31) / 32; ++q) b = fmax(b, sh[q]);
        scratch[blockIdx.x] = b;
        __threadfence();
        const double prev = atomicAdd(&scratch[SULI_NOALLOC_MAX_PLANES], 1.0);
        last = (prev == (double)(gridDim.x - 1));
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double g = 0.0;
    for (int q = 0; q < nz; ++q) g = fmax(g, __ldcg(&scratch[q]));
    *maxdiv = g;
    scratch[SULI_NOALLOC_MAX_PLANES] = 0.0;   // leave the counter cleared
}

}  // namespace

extern "C" int suli_conmassa_noalloc(const double *u, const double *v, const double *w, int32_t nx, int32_t ny,
                                     int32_t nz, double dx, double dy, double dz, double *div, double *maxdiv,
                                     void *stream)
{
    if (!u || !v || !w || !div || !maxdiv) return SULI_BAD_ARG;
    if (nx < 1 || ny < 1 || nz < 1) return SULI_BAD_ARG;
    if (nz > SULI_NOALLOC_MAX_PLANES) {
        std::fprintf(stderr, "suli_conmassa_noalloc: nz = %d exceeds the %d z-planes of its built-in scratch\n",
                     (int)nz, SULI_NOALLOC_MAX_PLANES);
        return SULI_BAD_ARG;
    }
    if ((long long)nx * ny > (1LL << 31) - 1) return SULI_BAD_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= SULI_NOALLOC_MAX_DEVICES) {
        cudaGetLastError();
        return SULI_NO_DEVICE;
    }
    double *scratch;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_addr[dev]) {
            // set-up, once per device, with that device current
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return SULI_CUDA_ERROR;
            }
            g_scratch_addr[dev] = (double *)p;
        }
        scratch = g_scratch_addr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    // the arrival counter must start at zero
    if (cudaMemsetAsync(scratch + SULI_NOALLOC_MAX_PLANES, 0, sizeof(double), s) != cudaSuccess) {
        cudaGetLastError();
        return SULI_CUDA_ERROR;
    }
    k_conmassa_noalloc<<<nz, 256, 0, s>>>(u, v, w, nx, ny, nz, dx, dy, dz, div, maxdiv, scratch);
    if (cudaGetLastError() != cudaSuccess) return SULI_CUDA_ERROR;
    return SULI_OK;
}
