// Component (de)interleaving for the Fortran-style push and pull of one array
// holding all components, component fastest (poisson_solver_push.f:8-140,
// poisson_solver_pull.f:8-485). The host moves the field's box out of or
// into the caller's array (with its ghost offsets) as one pitched 3D copy of
// a packed [nz][ny][nx][ncomp] buffer; these kernels split it into, or build
// it from, the solver's separate component arrays, coalesced on both sides.
#include <cuda_runtime.h>

#include "ps_types.hpp"

namespace ps {

namespace {

__global__ void k_deinterleave(const double *__restrict__ packed, int ncomp, long long n, double *o0, double *o1,
                               double *o2)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const double *p = packed + q * ncomp;
        o0[q] = p[0];
        if (ncomp > 1) o1[q] = p[1];
        if (ncomp > 2) o2[q] = p[2];
    }
}

__global__ void k_interleave(const double *i0, const double *i1, const double *i2, int ncomp, long long n,
                             double *__restrict__ packed)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        double *p = packed + q * ncomp;
        p[0] = i0 ? i0[q] : 0.0;
        if (ncomp > 1) p[1] = i1 ? i1[q] : 0.0;
        if (ncomp > 2) p[2] = i2 ? i2[q] : 0.0;
    }
}

unsigned grid_of(long long n)
{
    long long g = (n + 255) / 256;
    if (g > 152LL * 32) g = 152LL * 32;
    return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace

cudaError_t launch_deinterleave(const double *packed, int ncomp, long long n, double *const out[3], cudaStream_t st)
{
    if (ncomp < 1 || ncomp > 3 || !out[0] || (ncomp > 1 && !out[1]) || (ncomp > 2 && !out[2]))
        return cudaErrorInvalidValue;
    k_deinterleave<<<grid_of(n), 256, 0, st>>>(packed, ncomp, n, out[0], out[1], out[2]);
    return cudaGetLastError();
}

cudaError_t launch_interleave(const double *const in[3], int ncomp, long long n, double *packed, cudaStream_t st)
{
    if (ncomp < 1 || ncomp > 3) return cudaErrorInvalidValue;
    k_interleave<<<grid_of(n), 256, 0, st>>>(in[0], in[1], in[2], ncomp, n, packed);
    return cudaGetLastError();
}

}  // namespace ps
