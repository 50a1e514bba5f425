// Compile-time FFT core for power-of-two lengths (the hot path).
//
// Same Stockham stages as ps_fft.cuh, but the length L and the per-thread
// element budget EM are template parameters, so every radix, sub-transform
// size, twiddle offset and shared-memory stride is a constant: the butterfly
// addresses fold into immediate offsets from one base per butterfly.
//
// Layout: line-major with a skew. Element n of a line sits at
// sk(n) = n + n / W, W = 128 bytes / sizeof(complex), i.e. one padding slot
// per 128 bytes. Threads of a line are t-fast (tid = line * TPL + t), so a warp
// reads or writes consecutive (or R-strided, skew-spread) elements of one
// line: conflict-free for every stage. Lines are LDP elements apart, LDP
// chosen so that the coalesced column loads (B lanes per row, 32/B rows per
// warp) also hit distinct banks.
//
// Stages: log2(L)/log2(EM) radix-EM stages, then one radix 2^rem stage.
#pragma once
#include <cuda_runtime.h>

#include "ps_fft.cuh"

namespace ps {
namespace p2 {

__host__ __device__ constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }

template <int L, int EM> struct Plan {
    static constexpr int LL = ilog2(L), LE = ilog2(EM);
    static constexpr int NFULL = LL / LE, REM = LL - NFULL * LE;
    static constexpr int NST = NFULL + (REM ? 1 : 0);
    static constexpr int TPL = L / EM;
    __host__ __device__ static constexpr int radix(int s) { return s < NFULL ? EM : (1 << REM); }
    __host__ __device__ static constexpr int mm(int s)
    {
        int m = 1;
        for (int i = 0; i < s; ++i) m *= radix(i);
        return m;
    }
    __host__ __device__ static constexpr int tw(int s)
    {
        int o = 0;
        for (int i = 0; i < s; ++i) o += mm(i) * (radix(i) - 1);
        return o;
    }
    static constexpr int NTW = tw(NST);
    static_assert(L >= EM && (L & (L - 1)) == 0 && (EM & (EM - 1)) == 0, "power-of-two lengths >= EM");
};

// skew: one padding slot per 128 bytes
template <typename C> struct Skew {
    static constexpr int LW = sizeof(C) == 16 ? 3 : 4;
    static constexpr int W = 1 << LW;
};
template <typename C> __device__ __forceinline__ int sk(int n) { return n + (n >> Skew<C>::LW); }
template <typename C> __host__ __device__ constexpr int sk_const(int n) { return n + (n >> (sizeof(C) == 16 ? 3 : 4)); }

// Line pitch: the skewed length padded so that pitch = 32/B (mod W), which
// spreads the B lines of one row over the banks in the coalesced load/store
// phases.
template <typename C> __host__ __device__ inline int line_pitch(int L, int B)
{
    const int W = sizeof(C) == 16 ? 8 : 16;
    const int base = L + L / W;
    const int target = (32 / B) % W;
    return base + (((target - base) % W) + W) % W;
}

// Stage S as two halves: butterflies read (and computed) into registers, and
// their results written back. Separate halves let several line sets share the
// barriers of one stage.
template <int L, int EM, int S, bool INV, typename C>
__device__ __forceinline__ void stage_read(const C *line, const C *tws, int t, C (&v)[EM / Plan<L, EM>::radix(S)][Plan<L, EM>::radix(S)])
{
    using PL = Plan<L, EM>;
    constexpr int R = PL::radix(S), M = PL::mm(S), NBF = L / R, U = EM / R, TPL = PL::TPL;
    constexpr int W = Skew<C>::W;
    const C *tw = tws + PL::tw(S);
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int bf = t + u * TPL;
        if constexpr (NBF % W == 0) {
            const C *src = line + sk<C>(bf);
#pragma unroll
            for (int r = 0; r < R; ++r) v[u][r] = src[r * (NBF + NBF / W)];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) v[u][r] = line[sk<C>(bf + r * NBF)];
        }
        if constexpr (M > 1) {
            const int j = bf & (M - 1);
            const C *w = tw + j * (R - 1);
#pragma unroll
            for (int r = 1; r < R; ++r) v[u][r] = INV ? cmulc(v[u][r], w[r - 1]) : cmul(v[u][r], w[r - 1]);
        }
        dft<R, INV>(v[u]);
    }
}

template <int L, int EM, int S, typename C>
__device__ __forceinline__ void stage_write(C *line, int t, const C (&v)[EM / Plan<L, EM>::radix(S)][Plan<L, EM>::radix(S)])
{
    using PL = Plan<L, EM>;
    constexpr int R = PL::radix(S), M = PL::mm(S), U = EM / R, TPL = PL::TPL;
    constexpr int LW = Skew<C>::LW, W = Skew<C>::W, LM = ilog2(M);
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int bf = t + u * TPL;
        const int j = bf & (M - 1), q = bf >> LM;
        if constexpr (M % W == 0) {
            C *dst = line + sk<C>(q * R * M + j);
#pragma unroll
            for (int r = 0; r < R; ++r) dst[r * (M + M / W)] = v[u][r];
        } else if constexpr ((R * M) % W == 0 && W % M == 0) {
            // n = q R M + r M + j with j < M | W: the skew of r M + j is that of r M
            C *dst = line + q * R * M + ((q * R * M) >> LW) + j;
#pragma unroll
            for (int r = 0; r < R; ++r) dst[r * M + ((r * M) >> LW)] = v[u][r];
        } else {
            const int n0 = q * R * M + j;
#pragma unroll
            for (int r = 0; r < R; ++r) line[sk<C>(n0 + r * M)] = v[u][r];
        }
    }
}

// One stage over ncomp line sets (cstride elements apart), pipelined: the
// results of set c are written while set c+1 is read (different buffers),
// so the stage costs ncomp + 1 barriers instead of 2 ncomp.
template <int L, int EM, int S, bool INV, typename C>
__device__ __forceinline__ void stage_sets(C *line, const C *tws, int t, int ncomp, int cstride)
{
    constexpr int R = Plan<L, EM>::radix(S), U = EM / R;
    C v[U][R];
    stage_read<L, EM, S, INV>(line, tws, t, v);
    __syncthreads();
    for (int c = 1; c < ncomp; ++c) {
        C w[U][R];
        stage_read<L, EM, S, INV>(line + c * cstride, tws, t, w);
        stage_write<L, EM, S>(line + (c - 1) * cstride, t, v);
        __syncthreads();
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int r = 0; r < R; ++r) v[u][r] = w[u][r];
    }
    stage_write<L, EM, S>(line + (ncomp - 1) * cstride, t, v);
    __syncthreads();
}

// Stages S .. SEND-1 over ncomp line sets.
template <int L, int EM, bool INV, typename C, int S = 0, int SEND = Plan<L, EM>::NST>
__device__ __forceinline__ void run(C *line, const C *tws, int t, int ncomp = 1, int cstride = 0)
{
    if constexpr (S < SEND) {
        stage_sets<L, EM, S, INV>(line, tws, t, ncomp, cstride);
        run<L, EM, INV, C, S + 1, SEND>(line, tws, t, ncomp, cstride);
    }
}

// Stage 0 of a transform whose inputs n >= L/2 are zero (the padded half of an
// unbounded axis): a radix-16 stage (bf + r NBF, M = 1) reads r < 8 and runs
// the half-input DFT; the zero half is never read, so it need not be stored.
template <int L, int EM, bool INV, typename C> __device__ __forceinline__ void stage0_half(C *line, int t)
{
    using PL = Plan<L, EM>;
    constexpr int R = PL::radix(0), U = EM / R, NBF = L / R, TPL = PL::TPL;
    static_assert(R == 16, "a radix-16 first stage");
    C v[U][R];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int bf = t + u * TPL;
#pragma unroll
        for (int r = 0; r < R / 2; ++r) v[u][r] = line[sk<C>(bf + r * NBF)];
        dft16_half<INV>(v[u]);
    }
    __syncthreads();
    stage_write<L, EM, 0>(line, t, v);
    __syncthreads();
}

// The last stage of a transform whose outputs n >= L/2 are cropped: it writes
// positions r M + bf (bf < M = L / R) for r < R/2 only; the other outputs of
// its DFT are dead code.
template <int L, int EM, bool INV, typename C>
__device__ __forceinline__ void last_stage_half(C *line, const C *tws, int t)
{
    using PL = Plan<L, EM>;
    constexpr int S = PL::NST - 1, R = PL::radix(S), M = PL::mm(S), U = EM / R, TPL = PL::TPL;
    static_assert(M * R == L, "the last stage");
    C v[U][R];
    stage_read<L, EM, S, INV>(line, tws, t, v);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int bf = t + u * TPL;
#pragma unroll
        for (int r = 0; r < R / 2; ++r) line[sk<C>(r * M + bf)] = v[u][r];
    }
    __syncthreads();
}

}  // namespace p2
}  // namespace ps
