// Shared pieces of the wide FP32 kernels: L = 256, 512, 1024 or 2048 and 32
// elements per thread, so a length-1024 line is two radix-32 stages. The
// first stage of every transform reads its inputs straight from global memory
// into registers (zero padding: rows past the data are never loaded) and the
// last stage writes straight to global memory (crop: rows past the output are
// never stored); shared memory carries only the exchanges between stages.
// Relative to the length-specialised kernels this removes a shared-memory
// round trip at each end of every transform.
//
// Shared layout: line-major, one pad slot per 32 elements (sk(n) = n + n/32),
// lines `pitch` elements apart. The banks serve an 8-byte access one half-warp
// at a time (16 lanes, 16 eight-byte banks), so each half-warp's 16 addresses
// must fall in 16 different banks:
//   column passes (y, z) are lane-fast over the B lines (a warp's global
//     accesses are B adjacent columns of 32/B rows); a half-warp holds B lines
//     x 16/B positions, conflict-free when pitch = 16/B (mod 16);
//   row passes (x) are lane-fast along the line (global rows contiguous); a
//     half-warp holds 16/TPL lines when TPL = L/32 < 16, conflict-free when
//     pitch = TPL (mod 16).
// A bank model of every stage's reads and writes (first-stage writes
// n = 32t + r, later reads t + r NBF, writes r M + t) gives one wavefront per
// half-warp for L = 256..2048 and B = 1..16 with these pitches.
#pragma once
#include <cuda_runtime.h>

#include "ps_fft_p2.cuh"
#include "ps_types.hpp"

namespace ps {
namespace wide {

using p2::ilog2;

template <int L> using WP = p2::Plan<L, 32>;

__device__ __forceinline__ int skw(int n) { return n + (n >> 5); }

__host__ __device__ constexpr int pitch_to(int L, int target)
{
    const int base = L + L / 32;
    return base + (((target - base) % 16) + 16) % 16;
}
// lines of a column pass (lane-fast over the B lines)
__host__ __device__ constexpr int pitch_col(int L, int B) { return pitch_to(L, (16 / B) % 16); }
// lines of a row pass (lane-fast along the line)
__host__ __device__ constexpr int pitch_row(int L) { return pitch_to(L, (L / 32) % 16); }

// Stage S of the length-L plan: butterfly bf = t + u TPL reads positions
// bf + r NBF and writes (q R + r) M + j, j = bf mod M, q = bf / M.
template <int L, int S> struct St {
    using PL = WP<L>;
    static constexpr int R = PL::radix(S), M = PL::mm(S), NBF = L / R, U = 32 / R, TPL = PL::TPL;
    static constexpr int LM = ilog2(M), TWO = PL::tw(S);
    static constexpr bool LAST = S == PL::NST - 1;
    __device__ __forceinline__ static int in_pos(int t, int u, int r) { return t + u * TPL + r * NBF; }
    __device__ __forceinline__ static int out_pos(int t, int u, int r)
    {
        const int bf = t + u * TPL;
        return ((bf >> LM) * R + r) * M + (bf & (M - 1));
    }
};

template <int L, int S, bool INV, typename C>
__device__ __forceinline__ void twiddle_dft(C (&v)[St<L, S>::U][St<L, S>::R], const C *tws, int t)
{
    using T = St<L, S>;
#pragma unroll
    for (int u = 0; u < T::U; ++u) {
        if constexpr (T::M > 1) {
            const int j = (t + u * T::TPL) & (T::M - 1);
            const C *w = tws + T::TWO + j * (T::R - 1);
#pragma unroll
            for (int r = 1; r < T::R; ++r) v[u][r] = INV ? cmulc(v[u][r], w[r - 1]) : cmul(v[u][r], w[r - 1]);
        }
        dft<T::R, INV>(v[u]);
    }
}

template <int L, int S, typename C>
__device__ __forceinline__ void read_line(const C *line, int t, C (&v)[St<L, S>::U][St<L, S>::R])
{
    using T = St<L, S>;
#pragma unroll
    for (int u = 0; u < T::U; ++u)
#pragma unroll
        for (int r = 0; r < T::R; ++r) v[u][r] = line[skw(T::in_pos(t, u, r))];
}

template <int L, int S, typename C>
__device__ __forceinline__ void write_line(C *line, int t, const C (&v)[St<L, S>::U][St<L, S>::R])
{
    using T = St<L, S>;
#pragma unroll
    for (int u = 0; u < T::U; ++u)
#pragma unroll
        for (int r = 0; r < T::R; ++r) line[skw(T::out_pos(t, u, r))] = v[u][r];
}

// Barrier between the exchanges of a line: the CTA's, or (WARP) the warp's
// when all threads of the line are one warp's.
template <bool WARP> __device__ __forceinline__ void line_sync()
{
    if constexpr (WARP) __syncwarp();
    else __syncthreads();
}

// Shared-memory stages from S up to (excluding) the last, in place: read,
// barrier, write, barrier. nsets line sets cstride elements apart.
template <int L, int S, bool INV, bool WARP = false, typename C>
__device__ __forceinline__ void middle_stages(C *line, const C *tws, int t, int nsets, int cstride)
{
    if constexpr (S < WP<L>::NST - 1) {
        using T = St<L, S>;
        for (int c = 0; c < nsets; ++c) {
            C v[T::U][T::R];
            read_line<L, S>(line + c * cstride, t, v);
            twiddle_dft<L, S, INV>(v, tws, t);
            line_sync<WARP>();
            write_line<L, S>(line + c * cstride, t, v);
        }
        line_sync<WARP>();
        middle_stages<L, S + 1, INV, WARP>(line, tws, t, nsets, cstride);
    }
}

template <typename C, int NTW> __device__ __forceinline__ void load_twiddles(C *TW, const void *table)
{
    const C *g = reinterpret_cast<const C *>(table);
    for (int i = threadIdx.x; i < NTW; i += blockDim.x) TW[i] = __ldg(&g[i]);
}

__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }

template <typename T> __device__ __forceinline__ T wavenumber(int k, int P, T c, bool derivative)
{
    const int m = (2 * k < P) ? k : k - P;
    if (derivative && 2 * k == P) return (T)0;
    return (T)m * c;
}

}  // namespace wide
}  // namespace ps
