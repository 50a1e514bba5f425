// Wide FP32 pass kernels: column passes (y), the fused z pass and the x
// passes, on the stages and layout of ps_wide.cuh.
#include <cuda_runtime.h>

#include "ps_wide.cuh"

namespace ps {
namespace wide {

// ---------------------------------------------------------------------------
// y pass: strided columns, in place.
// HALF: the y axis is unbounded. Forward: n_in = L / 2, so the first stage
// (one radix-32 butterfly a thread over n = t + r L/32) has data only for
// r < 16. Inverse: n_out = L / 2, so the last stage writes only its first
// R/2 outputs (positions r M + bf < L / 2).
template <int L, bool INV, bool HALF>
__global__ void __launch_bounds__(MAX_THREADS) k_col(const ColArgs a)
{
    using C = float2;
    using PL = WP<L>;
    constexpr int LAST = PL::NST - 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, LDP = pitch_col(L, B);
    C *TW = S + B * LDP;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    const int lb = __ffs(B) - 1;
    const int b = threadIdx.x & (B - 1), t = threadIdx.x >> lb;
    const int x0 = blockIdx.x * B;
    const bool active = b < imin(B, a.Mx - x0);
    C *col = reinterpret_cast<C *>(pick3(a.data, blockIdx.z)) + (long long)blockIdx.y * a.outer_stride + x0 + b;
    const long long as = a.axis_stride;
    C *line = S + b * LDP;

    {   // first stage from global
        using T0 = St<L, 0>;
        C v[T0::U][T0::R];
        if constexpr (HALF && !INV) {
            static_assert(T0::U == 1 && T0::R == 32, "one radix-32 butterfly a thread in the first stage");
#pragma unroll
            for (int r = 0; r < 16; ++r) v[0][r] = active ? col[T0::in_pos(t, 0, r) * as] : C{0.f, 0.f};
            dft32_half<INV>(v[0]);
        } else {
            const int n_in = active ? a.n_in : 0;
#pragma unroll
            for (int u = 0; u < T0::U; ++u)
#pragma unroll
                for (int r = 0; r < T0::R; ++r) {
                    const int n = T0::in_pos(t, u, r);
                    v[u][r] = n < n_in ? col[n * as] : C{0.f, 0.f};
                }
            twiddle_dft<L, 0, INV>(v, TW, t);
        }
        write_line<L, 0>(line, t, v);
    }
    __syncthreads();
    middle_stages<L, 1, INV>(line, TW, t, 1, 0);
    {   // last stage to global
        using TL = St<L, LAST>;
        C v[TL::U][TL::R];
        read_line<L, LAST>(line, t, v);
        twiddle_dft<L, LAST, INV>(v, TW, t);
        if (active) {
            // HALF inverse: out_pos = r M + bf with bf < M = L / R, so r < R/2 is the cropped half
            constexpr int RW = (HALF && INV) ? TL::R / 2 : TL::R;
#pragma unroll
            for (int u = 0; u < TL::U; ++u)
#pragma unroll
                for (int r = 0; r < RW; ++r) {
                    const int n = TL::out_pos(t, u, r);
                    if ((HALF && INV) || n < a.n_out) col[n * as] = v[u][r];
                }
        }
    }
}

// ---------------------------------------------------------------------------
// Fused z pass.
template <int L, int OP>
__global__ void __launch_bounds__(Z_MAX_THREADS) k_z(const ZArgs a)
{
    using C = float2;
    using T = float;
    using PL = WP<L>;
    constexpr int LAST = PL::NST - 1;
    using TL = St<L, LAST>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, LDP = pitch_col(L, B), CS = B * LDP;
    const int nbuf = a.nin > a.nout ? a.nin : a.nout;
    C *TW = S + nbuf * CS;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    const int lb = __ffs(B) - 1;
    const int b = threadIdx.x & (B - 1), t = threadIdx.x >> lb;
    const int x0 = blockIdx.x * B;
    const int ky = a.ky0 + blockIdx.y;
    const bool active = b < imin(B, a.Mx - x0);
    const long long off = (long long)ky * a.row_stride + x0 + b;
    const long long as = a.axis_stride;
    C *line = S + b * LDP;

    // forward: first stage of every input component from global
    for (int c = 0; c < a.nin; ++c) {
        using T0 = St<L, 0>;
        const C *col = reinterpret_cast<const C *>(pick3(a.in, c)) + off;
        C v[T0::U][T0::R];
        const int n_in = active ? a.n_in : 0;
#pragma unroll
        for (int u = 0; u < T0::U; ++u)
#pragma unroll
            for (int r = 0; r < T0::R; ++r) {
                const int n = T0::in_pos(t, u, r);
                v[u][r] = n < n_in ? col[n * as] : C{0.f, 0.f};
            }
        twiddle_dft<L, 0, false>(v, TW, t);
        write_line<L, 0>(line + c * CS, t, v);
    }
    __syncthreads();
    middle_stages<L, 1, false>(line, TW, t, a.nin, CS);
    // last forward stage: in place on the thread's own positions
    for (int c = 0; c < a.nin; ++c) {
        C v[TL::U][TL::R];
        read_line<L, LAST>(line + c * CS, t, v);
        twiddle_dft<L, LAST, false>(v, TW, t);
        write_line<L, LAST>(line + c * CS, t, v);
    }

    // spectral operation on the positions this thread owns (no barrier:
    // the same thread wrote them)
    {
        const int oy = imin(ky, a.Py - ky);
        const int kx = x0 + b;
        const T *Kc = reinterpret_cast<const T *>(a.kern) + (long long)oy * a.Mx + (active ? kx : 0);
        const long long kzs = (long long)a.oct_y * a.Mx;
        const T kyv = wavenumber<T>(ky, a.Py, (T)a.kyc, true);
        const T kxv = wavenumber<T>(kx, a.Px, (T)a.kxc, true);
        const T kzc = (T)a.kzc;
        C *S0 = line, *S1 = line + CS, *S2 = line + 2 * CS;
#pragma unroll 4
        for (int i = 0; i < TL::U * TL::R; ++i) {
            const int n = TL::out_pos(t, i / TL::R, i % TL::R);
            const int e = skw(n);
            const int oz = imin(n, a.Pz - n);
            const T g = active ? Kc[oz * kzs] : (T)0;
            const T kzv = wavenumber<T>(n, a.Pz, kzc, true);
            if constexpr (OP == OP_NONE) {
                S0[e] = cscale(S0[e], g);
                if (a.nin > 1) S1[e] = cscale(S1[e], g);
                if (a.nin > 2) S2[e] = cscale(S2[e], g);
            } else if constexpr (OP == OP_GRAD) {
                const C i0 = S0[e];
                const C i1 = a.nin > 1 ? S1[e] : i0;
                const C i2 = a.nin > 2 ? S2[e] : i0;
                const T gx = g * kxv, gy = g * kyv, gz = g * kzv;
                S0[e] = C{-gx * i0.y, gx * i0.x};
                S1[e] = C{-gy * i1.y, gy * i1.x};
                S2[e] = C{-gz * i2.y, gz * i2.x};
            } else if constexpr (OP == OP_DIV) {
                const C i0 = S0[e], i1 = S1[e], i2 = S2[e];
                const C s = C{kxv * i0.x + kyv * i1.x + kzv * i2.x, kxv * i0.y + kyv * i1.y + kzv * i2.y};
                S0[e] = C{-g * s.y, g * s.x};
            } else if constexpr (OP == OP_CURL) {
                const C i0 = S0[e], i1 = S1[e], i2 = S2[e];
                const C c0 = C{kyv * i2.x - kzv * i1.x, kyv * i2.y - kzv * i1.y};
                const C c1 = C{kzv * i0.x - kxv * i2.x, kzv * i0.y - kxv * i2.y};
                const C c2 = C{kxv * i1.x - kyv * i0.x, kxv * i1.y - kyv * i0.y};
                S0[e] = C{-g * c0.y, g * c0.x};
                S1[e] = C{-g * c1.y, g * c1.x};
                S2[e] = C{-g * c2.y, g * c2.x};
            }
        }
    }
    __syncthreads();

    // inverse: first stage in place (read, barrier, write), middle stages,
    // last stage to global
    for (int c = 0; c < a.nout; ++c) {
        using T0 = St<L, 0>;
        C v[T0::U][T0::R];
        read_line<L, 0>(line + c * CS, t, v);
        twiddle_dft<L, 0, true>(v, TW, t);
        __syncthreads();
        write_line<L, 0>(line + c * CS, t, v);
    }
    __syncthreads();
    middle_stages<L, 1, true>(line, TW, t, a.nout, CS);
    for (int c = 0; c < a.nout; ++c) {
        C *col0 = reinterpret_cast<C *>(pick3(a.out, c));
        C v[TL::U][TL::R];
        read_line<L, LAST>(line + c * CS, t, v);
        twiddle_dft<L, LAST, true>(v, TW, t);
        if (active && col0) {
            C *col = col0 + off;
#pragma unroll
            for (int u = 0; u < TL::U; ++u)
#pragma unroll
                for (int r = 0; r < TL::R; ++r) {
                    const int n = TL::out_pos(t, u, r);
                    if (n < a.n_out) col[n * as] = v[u][r];
                }
        }
    }
}

// ---------------------------------------------------------------------------
// x forward: threads run along the line; line l carries rows 2l and 2l+1.
template <int L>
__global__ void __launch_bounds__(MAX_THREADS) k_xfwd(const XFwdArgs a)
{
    using C = float2;
    using PL = WP<L>;
    constexpr int LAST = PL::NST - 1, TPL = PL::TPL, LT = ilog2(TPL);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, LDP = pitch_row(L);
    C *TW = S + B * LDP;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    const int b = threadIdx.x >> LT, t = threadIdx.x & (TPL - 1);
    const int comp = blockIdx.y;
    const double *in = pick3(a.in, comp);
    C *out = reinterpret_cast<C *>(pick3(a.out, comp));
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long ra = (long long)blockIdx.x * 2 * B + 2 * b, rb = ra + 1;
    __shared__ long long rofs[2 * MAX_LINES];
    row_offsets(rofs, (long long)blockIdx.x * 2 * B, 2 * B, rows, a.rows_y, a.out_y, a.ld);
    C *line = S + b * LDP;
    {
        using T0 = St<L, 0>;
        C v[T0::U][T0::R];
        const bool va = ra < rows, vb = rb < rows;
        const int ja = (int)(ra % a.rows_y), ka = (int)(ra / a.rows_y);
        const int jb = (int)(rb % a.rows_y), kb = (int)(rb / a.rows_y);
#pragma unroll
        for (int u = 0; u < T0::U; ++u)
#pragma unroll
            for (int r = 0; r < T0::R; ++r) {
                const int n = T0::in_pos(t, u, r);
                double xa = 0.0, xb = 0.0;
                if (n < a.n_in) {
                    if (!a.mirror) {
                        if (va) xa = in[ra * a.in_stride + n];
                        if (vb) xb = in[rb * a.in_stride + n];
                    } else {
                        const int nn = imin(n, L - n);
                        if (va)
                            xa = in[((long long)imin(ka, a.Pz - ka) * a.oct_y + imin(ja, a.Py - ja)) * a.oct_x + nn];
                        if (vb)
                            xb = in[((long long)imin(kb, a.Pz - kb) * a.oct_y + imin(jb, a.Py - jb)) * a.oct_x + nn];
                    }
                }
                v[u][r] = C{(float)xa, (float)xb};
            }
        twiddle_dft<L, 0, false>(v, TW, t);
        write_line<L, 0>(line, t, v);
    }
    __syncthreads();
    middle_stages<L, 1, false>(line, TW, t, 1, 0);
    {
        using TL = St<L, LAST>;
        C v[TL::U][TL::R];
        read_line<L, LAST>(line, t, v);
        twiddle_dft<L, LAST, false>(v, TW, t);
        write_line<L, LAST>(line, t, v);
    }
    __syncthreads();
    // separate the half spectra of rows a and b
    constexpr int Mx = L / 2 + 1;
    const int nt = blockDim.x;
    for (int idx = threadIdx.x; idx < B * Mx; idx += nt) {
        const int l = idx / Mx, k = idx - l * Mx;
        const long long oa = rofs[2 * l], ob = rofs[2 * l + 1];
        if (oa < 0) continue;
        const C *ln = S + l * LDP;
        const C z = ln[skw(k)], w = ln[skw((L - k) & (L - 1))];
        out[oa + k] = C{0.5f * (z.x + w.x), 0.5f * (z.y - w.y)};
        if (ob >= 0) out[ob + k] = C{0.5f * (z.y + w.y), 0.5f * (w.x - z.x)};
    }
}

// x inverse: rebuild Z = Xa + i Xb, transform back, Re -> row a, Im -> row b.
template <int L>
__global__ void __launch_bounds__(MAX_THREADS) k_xinv(const XInvArgs a)
{
    using C = float2;
    using PL = WP<L>;
    constexpr int LAST = PL::NST - 1, TPL = PL::TPL, LT = ilog2(TPL);
    constexpr int Mx = L / 2 + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, LDP = pitch_row(L);
    C *TW = S + B * LDP;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    const int comp = blockIdx.y;
    const C *in = reinterpret_cast<const C *>(pick3(a.in, comp));
    double *out = pick3(a.out, comp);
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long row0 = (long long)blockIdx.x * 2 * B;
    const int nt = blockDim.x;
    __shared__ long long rofs[2 * MAX_LINES];
    row_offsets(rofs, row0, 2 * B, rows, a.rows_y, a.in_y, a.ld);
    __syncthreads();
    for (int idx = threadIdx.x; idx < B * Mx; idx += nt) {
        const int l = idx / Mx, k = idx - l * Mx;
        const long long oa = rofs[2 * l], ob = rofs[2 * l + 1];
        C xa = C{0.f, 0.f}, xb = C{0.f, 0.f};
        if (oa >= 0) xa = in[oa + k];
        if (ob >= 0) xb = in[ob + k];
        C *ln = S + l * LDP;
        ln[skw(k)] = C{xa.x - xb.y, xa.y + xb.x};
        if (k >= 1 && k <= L - Mx) ln[skw(L - k)] = C{xa.x + xb.y, xb.x - xa.y};
    }
    __syncthreads();
    const int b = threadIdx.x >> LT, t = threadIdx.x & (TPL - 1);
    C *line = S + b * LDP;
    {
        using T0 = St<L, 0>;
        C v[T0::U][T0::R];
        read_line<L, 0>(line, t, v);
        twiddle_dft<L, 0, true>(v, TW, t);
        __syncthreads();
        write_line<L, 0>(line, t, v);
    }
    __syncthreads();
    middle_stages<L, 1, true>(line, TW, t, 1, 0);
    {
        using TL = St<L, LAST>;
        C v[TL::U][TL::R];
        read_line<L, LAST>(line, t, v);
        twiddle_dft<L, LAST, true>(v, TW, t);
        const long long ra = row0 + 2 * b, rb = ra + 1;
#pragma unroll
        for (int u = 0; u < TL::U; ++u)
#pragma unroll
            for (int r = 0; r < TL::R; ++r) {
                const int n = TL::out_pos(t, u, r);
                if (n < a.n_out) {
                    if (ra < rows) out[ra * a.out_stride + n] = (double)v[u][r].x;
                    if (rb < rows) out[rb * a.out_stride + n] = (double)v[u][r].y;
                }
            }
    }
}

// ---------------------------------------------------------------------------
template <typename K> cudaError_t prep(K kernel, size_t smem)
{
    // Always: the 48 KB a launch gets without it includes the kernel's static
    // shared memory, so a request just under 48 KB can already be too large.
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

#define PS_WIDE_LENGTHS(X) X(256) X(512) X(1024) X(2048)

bool supported(int prec, int L) { return prec == PREC_FP32 && (L == 256 || L == 512 || L == 1024 || L == 2048); }

size_t smem_lines(int L, int B, int nbuf, int ntw_entries, bool column)
{
    const int ldp = column ? pitch_col(L, B) : pitch_row(L);
    return sizeof(float2) * ((size_t)nbuf * B * ldp + ntw_entries);
}

cudaError_t launch_xfwd(const XFwdArgs &a, cudaStream_t st)
{
    if (a.B > MAX_LINES) return cudaErrorInvalidConfiguration;  // row-offset table size
    const long long rows = (long long)a.rows_y * a.rows_z;
    dim3 grid((unsigned)(((rows + 1) / 2 + a.B - 1) / a.B), a.ncomp);
    const size_t sm = smem_lines(a.L, a.B, 1, a.plan.ntw, false);
    const int nt = a.B * (a.L / 32);
    cudaError_t e;
    switch (a.L) {
#define X(LV)                                                            \
    case LV:                                                             \
        if ((e = prep(k_xfwd<LV>, sm)) != cudaSuccess) return e;         \
        k_xfwd<LV><<<grid, nt, sm, st>>>(a);                             \
        break;
        PS_WIDE_LENGTHS(X)
#undef X
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int L, bool INV, bool HALF>
static cudaError_t launch_col_t(const ColArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    const cudaError_t e = prep(k_col<L, INV, HALF>, sm);
    if (e != cudaSuccess) return e;
    k_col<L, INV, HALF><<<grid, nt, sm, st>>>(a);
    return cudaGetLastError();
}

template <int L> static cudaError_t launch_col_len(int inverse, const ColArgs &a, dim3 grid, int nt, size_t sm,
                                                   cudaStream_t st)
{
    // the zero-padded half of an unbounded axis: forward input, inverse output
    if (inverse)
        return 2 * a.n_out == L ? launch_col_t<L, true, true>(a, grid, nt, sm, st)
                                : launch_col_t<L, true, false>(a, grid, nt, sm, st);
    return 2 * a.n_in == L ? launch_col_t<L, false, true>(a, grid, nt, sm, st)
                           : launch_col_t<L, false, false>(a, grid, nt, sm, st);
}

cudaError_t launch_col(int inverse, const ColArgs &a, int outer, cudaStream_t st)
{
    dim3 grid((unsigned)((a.Mx + a.B - 1) / a.B), outer, a.ncomp);
    const size_t sm = smem_lines(a.L, a.B, 1, a.plan.ntw, true);
    const int nt = a.B * (a.L / 32);
    switch (a.L) {
#define X(LV) \
    case LV: return launch_col_len<LV>(inverse, a, grid, nt, sm, st);
        PS_WIDE_LENGTHS(X)
#undef X
    default: return cudaErrorInvalidValue;
    }
}

template <int L> cudaError_t launch_z_len(const ZArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    cudaError_t e;
    switch (a.op) {
#define Z(OPV)                                                           \
    case OPV:                                                            \
        if ((e = prep(k_z<L, OPV>, sm)) != cudaSuccess) return e;        \
        k_z<L, OPV><<<grid, nt, sm, st>>>(a);                            \
        break;
        Z(OP_NONE)
        Z(OP_GRAD)
        Z(OP_DIV)
        Z(OP_CURL)
#undef Z
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_z(const ZArgs &a, int ny, cudaStream_t st)
{
    if (a.B * (a.L / 32) > Z_MAX_THREADS) return cudaErrorInvalidConfiguration;
    dim3 grid((unsigned)((a.Mx + a.B - 1) / a.B), ny);
    const int nbuf = a.nin > a.nout ? a.nin : a.nout;
    const size_t sm = smem_lines(a.L, a.B, nbuf, a.plan.ntw, true);
    const int nt = a.B * (a.L / 32);
    switch (a.L) {
#define X(LV) \
    case LV: return launch_z_len<LV>(a, grid, nt, sm, st);
        PS_WIDE_LENGTHS(X)
#undef X
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_xinv(const XInvArgs &a, cudaStream_t st)
{
    if (a.B > MAX_LINES) return cudaErrorInvalidConfiguration;  // row-offset table size
    const long long rows = (long long)a.rows_y * a.rows_z;
    dim3 grid((unsigned)(((rows + 1) / 2 + a.B - 1) / a.B), a.ncomp);
    const size_t sm = smem_lines(a.L, a.B, 1, a.plan.ntw, false);
    const int nt = a.B * (a.L / 32);
    cudaError_t e;
    switch (a.L) {
#define X(LV)                                                            \
    case LV:                                                             \
        if ((e = prep(k_xinv<LV>, sm)) != cudaSuccess) return e;         \
        k_xinv<LV><<<grid, nt, sm, st>>>(a);                             \
        break;
        PS_WIDE_LENGTHS(X)
#undef X
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace wide
}  // namespace ps
