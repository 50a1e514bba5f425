// Pieces shared by the fused z kernels that keep the spectra of a column in
// registers and tensor memory (ps_kernels_ztm.cu, ps_kernels_zq.cu): the
// adjoint stages of the inverse transform, the per-thread TMEM slots and the
// spectral operation.
#pragma once
#include "ps_tmem.cuh"
#include "ps_wide.cuh"

namespace ps {
namespace wide {

// Adjoint of stage S on registers gathered from its output positions:
// inverse DFT, then conjugate twiddles.
template <int L, int S, typename C>
__device__ __forceinline__ void adjoint_dft(C (&v)[St<L, S>::U][St<L, S>::R], const C *tws, int t)
{
    using T = St<L, S>;
#pragma unroll
    for (int u = 0; u < T::U; ++u) {
        dft<T::R, true>(v[u]);
        if constexpr (T::M > 1) {
            // keep the twiddle loads behind the DFT: hoisted above it they
            // would hold R - 1 more complex values in registers
            asm volatile("" ::: "memory");
            const int j = (t + u * T::TPL) & (T::M - 1);
            const C *w = tws + T::TWO + j * (T::R - 1);
#pragma unroll
            for (int r = 1; r < T::R; ++r) v[u][r] = cmulc(v[u][r], w[r - 1]);
        }
    }
}

template <int L, int S, typename C>
__device__ __forceinline__ void read_out(const C *line, int t, C (&v)[St<L, S>::U][St<L, S>::R])
{
    using T = St<L, S>;
#pragma unroll
    for (int u = 0; u < T::U; ++u)
#pragma unroll
        for (int r = 0; r < T::R; ++r) v[u][r] = line[skw(T::out_pos(t, u, r))];
}

template <int L, int S, typename C>
__device__ __forceinline__ void write_in(C *line, int t, const C (&v)[St<L, S>::U][St<L, S>::R])
{
    using T = St<L, S>;
#pragma unroll
    for (int u = 0; u < T::U; ++u)
#pragma unroll
        for (int r = 0; r < T::R; ++r) line[skw(T::in_pos(t, u, r))] = v[u][r];
}

// Adjoint middle stages S = from .. 1, in place on one line. WARP: the
// line's threads are one warp's (a warp barrier between exchanges).
template <int L, int S, bool WARP = false, typename C>
__device__ __forceinline__ void adjoint_middle(C *line, const C *tws, int t)
{
    if constexpr (S >= 1) {
        using T = St<L, S>;
        C v[T::U][T::R];
        read_out<L, S>(line, t, v);
        adjoint_dft<L, S>(v, tws, t);
        line_sync<WARP>();
        write_in<L, S>(line, t, v);
        line_sync<WARP>();
        adjoint_middle<L, S - 1, WARP>(line, tws, t);
    }
}

// 32 values <-> 4 x 16 columns of the thread's TMEM row.
template <int U, int R>
__device__ __forceinline__ void stash(uint32_t taddr, const float2 (&v)[U][R])
{
    static_assert(U * R == 32, "32 values per thread");
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
        uint32_t w[16];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int i = ch * 8 + e;
            w[2 * e] = __float_as_uint(v[i / R][i % R].x);
            w[2 * e + 1] = __float_as_uint(v[i / R][i % R].y);
        }
        tmem::st16(taddr + 16 * ch, w);
    }
}

template <int U, int R>
__device__ __forceinline__ void unstash(uint32_t taddr, float2 (&v)[U][R])
{
    uint32_t w[4][16];
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) tmem::ld16(taddr + 16 * ch, w[ch]);
    tmem::wait_ld16x2(w[0], w[1]);
    tmem::wait_ld16x2(w[2], w[3]);
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i / R][i % R] = float2{__uint_as_float(w[i / 8][2 * (i % 8)]), __uint_as_float(w[i / 8][2 * (i % 8) + 1])};
}

constexpr int SLOT_COLUMNS = 64;  // 32 complex values

// Spectral operation on the 32 values a thread holds after its last forward
// stage (positions n = out_pos(t, u, r) of z-column kx in y-row ky):
// components 0 .. nin-2 come from the TMEM slots at tbase, the last from cur;
// outputs 0 .. nout-2 go back to the slots, the last to cur. gk(m) returns
// the column's kernel value at octant row m = min(n, Pz - n).
template <int L, int OP, typename GK>
__device__ __forceinline__ void spectral_op(const ZArgs &a, float2 (&cur)[St<L, WP<L>::NST - 1>::U][St<L, WP<L>::NST - 1>::R],
                                            uint32_t tbase, int ky, int kx, int t, GK gk)
{
    using C = float2;
    using T = float;
    using TL = St<L, WP<L>::NST - 1>;
    const T kyv = wavenumber<T>(ky, a.Py, (T)a.kyc, true);
    const T kxv = wavenumber<T>(kx, a.Px, (T)a.kxc, true);
    const T kzc = (T)a.kzc;
    const int nslot_in = a.nin - 1;
    T gall[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
        const int n = TL::out_pos(t, i / TL::R, i % TL::R);
        gall[i] = gk(imin(n, a.Pz - n));
    }
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
        T g[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) g[e] = gall[ch * 8 + e];
        uint32_t s0[16], s1[16];
        if (nslot_in > 0) tmem::ld16(tbase + 16 * ch, s0);
        if (nslot_in > 1) tmem::ld16(tbase + SLOT_COLUMNS + 16 * ch, s1);
        if (nslot_in > 0) tmem::wait_ld16x2(s0, s1);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int i = ch * 8 + e, u = i / TL::R, r = i % TL::R;
            const int n = TL::out_pos(t, u, r);
            const T kzv = wavenumber<T>(n, a.Pz, kzc, true);
            const C ic = cur[u][r];
            const C i0 = C{__uint_as_float(s0[2 * e]), __uint_as_float(s0[2 * e + 1])};
            const C i1 = C{__uint_as_float(s1[2 * e]), __uint_as_float(s1[2 * e + 1])};
            const T gi = g[e];
            C o0{0.f, 0.f}, o1{0.f, 0.f}, o2;
            if constexpr (OP == OP_NONE) {
                o0 = cscale(i0, gi);
                o1 = cscale(i1, gi);
                o2 = cscale(ic, gi);
            } else if constexpr (OP == OP_GRAD) {
                // nin = 1: every output from the one input; nin = 3: output d from input d
                const C a0 = a.nin > 1 ? i0 : ic, a1 = a.nin > 1 ? i1 : ic;
                const T gx = gi * kxv, gy = gi * kyv, gz = gi * kzv;
                o0 = C{-gx * a0.y, gx * a0.x};
                o1 = C{-gy * a1.y, gy * a1.x};
                o2 = C{-gz * ic.y, gz * ic.x};
            } else if constexpr (OP == OP_DIV) {
                const C s = C{kxv * i0.x + kyv * i1.x + kzv * ic.x, kxv * i0.y + kyv * i1.y + kzv * ic.y};
                o2 = C{-gi * s.y, gi * s.x};
            } else {  // OP_CURL
                const C c0 = C{kyv * ic.x - kzv * i1.x, kyv * ic.y - kzv * i1.y};
                const C c1 = C{kzv * i0.x - kxv * ic.x, kzv * i0.y - kxv * ic.y};
                const C c2 = C{kxv * i1.x - kyv * i0.x, kxv * i1.y - kyv * i0.y};
                o0 = C{-gi * c0.y, gi * c0.x};
                o1 = C{-gi * c1.y, gi * c1.x};
                o2 = C{-gi * c2.y, gi * c2.x};
            }
            s0[2 * e] = __float_as_uint(o0.x);
            s0[2 * e + 1] = __float_as_uint(o0.y);
            s1[2 * e] = __float_as_uint(o1.x);
            s1[2 * e + 1] = __float_as_uint(o1.y);
            cur[u][r] = o2;
        }
        if (a.nout > 1) tmem::st16(tbase + 16 * ch, s0);
        if (a.nout > 2) tmem::st16(tbase + SLOT_COLUMNS + 16 * ch, s1);
    }
    tmem::wait_st();
}

}  // namespace wide
}  // namespace ps
