// Pass kernels specialised on power-of-two transform lengths (FP32 hot path):
// the same five passes as ps_kernels_body.cuh, built on the compile-time FFT core of
// ps_fft_p2.cuh. The host uses them for FP32 and 64 <= L <= 2048 and falls
// back to the run-time kernels otherwise (p2::supported).
#include <cuda_runtime.h>

#include "ps_fft_p2.cuh"
#include "ps_types.hpp"

namespace ps {
namespace p2 {

namespace {

__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }

template <typename C, int NTW> __device__ __forceinline__ void load_twiddles(C *TW, const void *table)
{
    const C *g = reinterpret_cast<const C *>(table);
    for (int i = threadIdx.x; i < NTW; i += blockDim.x) TW[i] = __ldg(&g[i]);
}

template <typename T> __device__ __forceinline__ T wavenumber(int k, int P, T c, bool derivative)
{
    const int m = (2 * k < P) ? k : k - P;
    if (derivative && 2 * k == P) return (T)0;
    return (T)m * c;
}

}  // namespace

// ---------------------------------------------------------------------------
// x forward: line l = rows 2l (re) and 2l+1 (im), then the two half spectra.
// BL lines a CTA is a template parameter, so the thread count NT = BL TPL is
// a constant and the load, separation and store loops address global memory
// as one row base plus immediate offsets.
// HALF: the x axis is unbounded (n_in = L / 2): the padded half is neither
// stored nor read (stage0_half).
template <typename T, int L, int EM, int BL, bool HALF>
__global__ void __launch_bounds__(BL *(L / EM)) k_xfwd(const XFwdArgs a)
{
    using C = typename CxT<T>::type;
    using PL = Plan<L, EM>;
    constexpr int TPL = PL::TPL, LT = ilog2(TPL), NT = BL * TPL, PER = L / NT;
    static_assert(PER * NT == L, "a CTA's threads divide the line");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int LDP = line_pitch<C>(L, BL);
    C *TW = S + BL * LDP;
    const int tid = threadIdx.x;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    const int comp = blockIdx.y;
    const double *in = pick3(a.in, comp);
    C *out = reinterpret_cast<C *>(pick3(a.out, comp));
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long row0 = (long long)blockIdx.x * 2 * BL;
    __shared__ long long rofs[2 * BL];
    row_offsets(rofs, row0, 2 * BL, rows, a.rows_y, a.out_y, a.ld);

    // line l = (row 2l, row 2l+1) as (re, im); zero past n_in and past the last row
    if (!a.mirror) {
        // every load of the thread issued before the first shared-memory store
        constexpr int JN = HALF ? PER / 2 : PER;  // HALF: n < L/2 = n_in exactly
        C v[BL][JN];
#pragma unroll
        for (int l = 0; l < BL; ++l) {
            const long long ra = row0 + 2 * l;
            const double *pa = in + ra * a.in_stride + tid, *pb = pa + a.in_stride;
            const bool va = ra < rows, vb = ra + 1 < rows;
#pragma unroll
            for (int j = 0; j < JN; ++j) {
                const bool live = HALF || tid + j * NT < a.n_in;
                v[l][j] = C{(live && va) ? (T)pa[j * NT] : (T)0, (live && vb) ? (T)pb[j * NT] : (T)0};
            }
        }
#pragma unroll
        for (int l = 0; l < BL; ++l)
#pragma unroll
            for (int j = 0; j < JN; ++j) S[l * LDP + sk<C>(tid + j * NT)] = v[l][j];
    } else {
        // rows of the kernel octant, mirrored: (z, y) -> (min(z, Pz-z), min(y, Py-y)), n -> min(n, L-n)
        for (int line = 0; line < BL; ++line) {
            const long long ra = row0 + 2 * line;
            const bool va = ra < rows, vb = ra + 1 < rows;
            long long oa = 0, ob = 0;
            if (va) {
                const int j = (int)(ra % a.rows_y), k = (int)(ra / a.rows_y);
                oa = ((long long)imin(k, a.Pz - k) * a.oct_y + imin(j, a.Py - j)) * a.oct_x;
            }
            if (vb) {
                const int j = (int)((ra + 1) % a.rows_y), k = (int)((ra + 1) / a.rows_y);
                ob = ((long long)imin(k, a.Pz - k) * a.oct_y + imin(j, a.Py - j)) * a.oct_x;
            }
            C *ln = S + line * LDP;
            for (int n = tid; n < L; n += NT) {
                T xa = (T)0, xb = (T)0;
                if (n < a.n_in) {
                    const int nn = imin(n, L - n);
                    if (va) xa = (T)in[oa + nn];
                    if (vb) xb = (T)in[ob + nn];
                }
                ln[sk<C>(n)] = C{xa, xb};
            }
        }
    }
    __syncthreads();
    if constexpr (HALF) {
        // the mirrored kernel rows (a.mirror) are never HALF: the launcher checks
        stage0_half<L, EM, false>(S + (tid >> LT) * LDP, tid & (TPL - 1));
        run<L, EM, false, C, 1>(S + (tid >> LT) * LDP, TW, tid & (TPL - 1));
    } else {
        run<L, EM, false>(S + (tid >> LT) * LDP, TW, tid & (TPL - 1));
    }

    constexpr int Mx = L / 2 + 1, KPER = (Mx + NT - 1) / NT;
#pragma unroll
    for (int line = 0; line < BL; ++line) {
        const long long oa = rofs[2 * line], ob = rofs[2 * line + 1];
        if (oa < 0) break;
        const C *ln = S + line * LDP;
        C *outa = out + oa + tid, *outb = out + ob + tid;
#pragma unroll
        for (int j = 0; j < KPER; ++j) {
            const int k = tid + j * NT;
            if (k < Mx) {
                const C z = ln[sk<C>(k)], w = ln[sk<C>((L - k) & (L - 1))];
                const T h = (T)0.5;
                outa[j * NT] = C{h * (z.x + w.x), h * (z.y - w.y)};
                if (ob >= 0) outb[j * NT] = C{h * (z.y + w.y), h * (w.x - z.x)};
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Strided column transforms, in place.
template <typename T, int L, int EM, bool INV>
__global__ void __launch_bounds__(MAX_THREADS) k_col(const ColArgs a)
{
    using C = typename CxT<T>::type;
    using PL = Plan<L, EM>;
    constexpr int TPL = PL::TPL, LT = ilog2(TPL);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, LDP = line_pitch<C>(L, B);
    C *TW = S + B * LDP;
    const int nt = blockDim.x, tid = threadIdx.x;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    const int lb = __ffs(B) - 1;
    const int x0 = blockIdx.x * B;
    const int nb = imin(B, a.Mx - x0);
    C *base = reinterpret_cast<C *>(pick3(a.data, blockIdx.z)) + (long long)blockIdx.y * a.outer_stride + x0;

    // coalesced phases: lane -> (column bl, row nl); each thread moves EM rows,
    // all of its loads in flight before the first shared-memory write
    const int bl = tid & (B - 1), nl = tid >> lb, rstep = nt >> lb;
    const long long gstep = (long long)rstep * a.axis_stride;
    {
        const C *src = base + (long long)nl * a.axis_stride + bl;
        const int n_in = bl < nb ? a.n_in : 0;
        C *dst = S + bl * LDP;
        C v[EM];
#pragma unroll
        for (int i = 0; i < EM; ++i) {
            const int n = nl + i * rstep;
            v[i] = n < n_in ? src[i * gstep] : C{0, 0};
        }
#pragma unroll
        for (int i = 0; i < EM; ++i) dst[sk<C>(nl + i * rstep)] = v[i];
    }
    __syncthreads();
    run<L, EM, INV>(S + (tid >> LT) * LDP, TW, tid & (TPL - 1));
    if (bl < nb) {
        C *dst = base + (long long)nl * a.axis_stride + bl;
        const C *src = S + bl * LDP;
#pragma unroll 4
        for (int n = nl; n < a.n_out; n += rstep, dst += gstep) *dst = src[sk<C>(n)];
    }
}

// ---------------------------------------------------------------------------
// Fused z pass (operators none/grad/div/curl).
template <typename T, int L, int EM, int OP>
__global__ void __launch_bounds__(MAX_THREADS) k_z(const ZArgs a)
{
    using C = typename CxT<T>::type;
    using PL = Plan<L, EM>;
    constexpr int TPL = PL::TPL, LT = ilog2(TPL);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, LDP = line_pitch<C>(L, B), CS = B * LDP;
    const int nbuf = a.nin > a.nout ? a.nin : a.nout;
    C *TW = S + nbuf * CS;
    const int nt = blockDim.x, tid = threadIdx.x;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    const int lb = __ffs(B) - 1;
    const int x0 = blockIdx.x * B;
    const int ky = a.ky0 + blockIdx.y;
    const int nb = imin(B, a.Mx - x0);
    const long long off = (long long)ky * a.row_stride + x0;
    const int bl = tid & (B - 1), nl = tid >> lb, rstep = nt >> lb;
    const long long gstep = (long long)rstep * a.axis_stride;
    const int n_in = bl < nb ? a.n_in : 0;

    for (int c = 0; c < a.nin; ++c) {
        // every thread moves EM rows of each component, a component's loads
        // all in flight before its shared-memory writes
        const C *src = reinterpret_cast<const C *>(pick3(a.in, c)) + off + (long long)nl * a.axis_stride + bl;
        C *dst = S + c * CS + bl * LDP;
        C v[EM];
#pragma unroll
        for (int i = 0; i < EM; ++i) {
            const int n = nl + i * rstep;
            v[i] = n < n_in ? src[i * gstep] : C{0, 0};
        }
#pragma unroll
        for (int i = 0; i < EM; ++i) dst[sk<C>(nl + i * rstep)] = v[i];
    }
    __syncthreads();
    C *myline = S + (tid >> LT) * LDP;
    const int t = tid & (TPL - 1);
    run<L, EM, false>(myline, TW, t, a.nin, CS);

    {
        const int oy = imin(ky, a.Py - ky);
        const int kx = x0 + bl;
        const T *Kc = reinterpret_cast<const T *>(a.kern) + (long long)oy * a.Mx + kx;
        const long long kzs = (long long)a.oct_y * a.Mx;
        const T kyv = wavenumber<T>(ky, a.Py, (T)a.kyc, true);
        const T kxv = wavenumber<T>(kx, a.Px, (T)a.kxc, true);
        const T kzc = (T)a.kzc;
        C *S0 = S + bl * LDP, *S1 = S0 + CS, *S2 = S1 + CS;
        for (int n = nl; n < (bl < nb ? L : 0); n += rstep) {
            const int e = sk<C>(n);
            const int oz = imin(n, a.Pz - n);
            const T g = Kc[oz * kzs];
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
    run<L, EM, true>(myline, TW, t, a.nout, CS);

    if (bl < nb) {
        for (int c = 0; c < a.nout; ++c) {
            C *dst0 = reinterpret_cast<C *>(pick3(a.out, c));
            if (dst0 == nullptr) continue;
            C *dst = dst0 + off + (long long)nl * a.axis_stride + bl;
            const C *src = S + c * CS + bl * LDP;
#pragma unroll 4
            for (int n = nl; n < a.n_out; n += rstep, dst += gstep) *dst = src[sk<C>(n)];
        }
    }
}

// ---------------------------------------------------------------------------
// x inverse: half spectra of row pairs -> real rows, cropped.
// HALF: n_out = L / 2 (unbounded x): the last stage writes only the kept half.
template <typename T, int L, int EM, int BL, bool HALF>
__global__ void __launch_bounds__(BL *(L / EM)) k_xinv(const XInvArgs a)
{
    using C = typename CxT<T>::type;
    using PL = Plan<L, EM>;
    constexpr int TPL = PL::TPL, LT = ilog2(TPL), NT = BL * TPL;
    constexpr int Mx = L / 2 + 1, KPER = (Mx + NT - 1) / NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int LDP = line_pitch<C>(L, BL);
    C *TW = S + BL * LDP;
    const int tid = threadIdx.x;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    const int comp = blockIdx.y;
    const C *in = reinterpret_cast<const C *>(pick3(a.in, comp));
    double *out = pick3(a.out, comp);
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long row0 = (long long)blockIdx.x * 2 * BL;
    __shared__ long long rofs[2 * BL];
    row_offsets(rofs, row0, 2 * BL, rows, a.rows_y, a.in_y, a.ld);
    __syncthreads();

    // Z = Xa + i Xb over the full line from the two half spectra
    {
        C va[BL][KPER], vb[BL][KPER];
#pragma unroll
        for (int l = 0; l < BL; ++l) {
            const long long oa = rofs[2 * l], ob = rofs[2 * l + 1];
            const C *ia = in + oa + tid, *ib = in + ob + tid;
#pragma unroll
            for (int j = 0; j < KPER; ++j) {
                const bool live = tid + j * NT < Mx;
                va[l][j] = (live && oa >= 0) ? ia[j * NT] : C{0, 0};
                vb[l][j] = (live && ob >= 0) ? ib[j * NT] : C{0, 0};
            }
        }
#pragma unroll
        for (int l = 0; l < BL; ++l) {
            C *ln = S + l * LDP;
#pragma unroll
            for (int j = 0; j < KPER; ++j) {
                const int k = tid + j * NT;
                if (k < Mx) {
                    const C xa = va[l][j], xb = vb[l][j];
                    ln[sk<C>(k)] = C{xa.x - xb.y, xa.y + xb.x};
                    if (k >= 1 && k <= L - Mx) ln[sk<C>(L - k)] = C{xa.x + xb.y, xb.x - xa.y};
                }
            }
        }
    }
    __syncthreads();
    if constexpr (HALF) {
        run<L, EM, true, C, 0, Plan<L, EM>::NST - 1>(S + (tid >> LT) * LDP, TW, tid & (TPL - 1));
        last_stage_half<L, EM, true>(S + (tid >> LT) * LDP, TW, tid & (TPL - 1));
    } else {
        run<L, EM, true>(S + (tid >> LT) * LDP, TW, tid & (TPL - 1));
    }

    // line l -> rows 2l (real parts) and 2l+1 (imaginary parts), n < n_out
    const int no = a.n_out;
    constexpr int NPER = (L + NT - 1) / NT;
#pragma unroll
    for (int line = 0; line < BL; ++line) {
        const long long ra = row0 + 2 * line;
        if (ra >= rows) break;
        const bool vb = ra + 1 < rows;
        double *oa = out + ra * a.out_stride + tid, *ob = oa + a.out_stride;
        const C *ln = S + line * LDP;
#pragma unroll
        for (int j = 0; j < NPER; ++j) {
            if (tid + j * NT < no) {
                const C v = ln[sk<C>(tid + j * NT)];
                oa[j * NT] = (double)v.x;
                if (vb) ob[j * NT] = (double)v.y;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Launchers

template <typename K> cudaError_t prep(K kernel, size_t smem)
{
    // Always: the 48 KB a launch gets without it includes the kernel's static
    // shared memory, so a request just under 48 KB can already be too large.
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int L, int EM> constexpr size_t ntw() { return Plan<L, EM>::NTW; }

#define PS_P2_LENGTHS(X) X(64) X(128) X(256) X(512) X(1024) X(2048)

bool supported(int prec, int L) { return prec == PREC_FP32 && L >= 64 && L <= 2048 && (L & (L - 1)) == 0; }

size_t smem_lines(int prec, int L, int B, int nbuf, int ntw_entries)
{
    const size_t c = prec == PREC_FP64 ? 16 : 8;
    const int ldp = prec == PREC_FP64 ? line_pitch<double2>(L, B) : line_pitch<float2>(L, B);
    return c * ((size_t)nbuf * B * ldp + ntw_entries);
}

// The x kernels are compiled for 1, 2, 4 or 8 lines a CTA.
template <int L, int BL, bool HALF>
cudaError_t launch_xfwd_h(const XFwdArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    const cudaError_t e = prep(k_xfwd<float, L, 16, BL, HALF>, sm);
    if (e != cudaSuccess) return e;
    k_xfwd<float, L, 16, BL, HALF><<<grid, nt, sm, st>>>(a);
    return cudaGetLastError();
}

template <int L, int BL> cudaError_t launch_xfwd_t(const XFwdArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    // the zero-padded half of an unbounded axis (never for mirrored kernel rows)
    if (!a.mirror && 2 * a.n_in == L && L >= 256) return launch_xfwd_h<L, BL, true>(a, grid, nt, sm, st);
    return launch_xfwd_h<L, BL, false>(a, grid, nt, sm, st);
}

template <int L, int BL, bool HALF>
cudaError_t launch_xinv_h(const XInvArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    const cudaError_t e = prep(k_xinv<float, L, 16, BL, HALF>, sm);
    if (e != cudaSuccess) return e;
    k_xinv<float, L, 16, BL, HALF><<<grid, nt, sm, st>>>(a);
    return cudaGetLastError();
}

template <int L, int BL> cudaError_t launch_xinv_t(const XInvArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    if (2 * a.n_out == L && L >= 256) return launch_xinv_h<L, BL, true>(a, grid, nt, sm, st);
    return launch_xinv_h<L, BL, false>(a, grid, nt, sm, st);
}

template <int L> cudaError_t launch_xfwd_len(const XFwdArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    switch (a.B) {
    case 1: return launch_xfwd_t<L, 1>(a, grid, nt, sm, st);
    case 2: return launch_xfwd_t<L, 2>(a, grid, nt, sm, st);
    case 4: return launch_xfwd_t<L, 4>(a, grid, nt, sm, st);
    case 8: return launch_xfwd_t<L, 8>(a, grid, nt, sm, st);
    default: return cudaErrorInvalidConfiguration;
    }
}

template <int L> cudaError_t launch_xinv_len(const XInvArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    switch (a.B) {
    case 1: return launch_xinv_t<L, 1>(a, grid, nt, sm, st);
    case 2: return launch_xinv_t<L, 2>(a, grid, nt, sm, st);
    case 4: return launch_xinv_t<L, 4>(a, grid, nt, sm, st);
    case 8: return launch_xinv_t<L, 8>(a, grid, nt, sm, st);
    default: return cudaErrorInvalidConfiguration;
    }
}

cudaError_t launch_xfwd(const XFwdArgs &a, cudaStream_t st)
{
    const long long rows = (long long)a.rows_y * a.rows_z;
    dim3 grid((unsigned)(((rows + 1) / 2 + a.B - 1) / a.B), a.ncomp);
    const size_t sm = smem_lines(PREC_FP32, a.L, a.B, 1, a.plan.ntw);
    const int nt = a.B * (a.L / e_max(PREC_FP32));
    switch (a.L) {
#define X(LV) \
    case LV: return launch_xfwd_len<LV>(a, grid, nt, sm, st);
        PS_P2_LENGTHS(X)
#undef X
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_col(int inverse, const ColArgs &a, int outer, cudaStream_t st)
{
    dim3 grid((unsigned)((a.Mx + a.B - 1) / a.B), outer, a.ncomp);
    const size_t sm = smem_lines(PREC_FP32, a.L, a.B, 1, a.plan.ntw);
    const int nt = a.B * (a.L / e_max(PREC_FP32));
    cudaError_t e;
    switch (a.L) {
#define X(LV)                                                                            \
    case LV:                                                                             \
        if (inverse) {                                                                   \
            if ((e = prep(k_col<float, LV, 16, true>, sm)) != cudaSuccess) return e;     \
            k_col<float, LV, 16, true><<<grid, nt, sm, st>>>(a);                         \
        } else {                                                                         \
            if ((e = prep(k_col<float, LV, 16, false>, sm)) != cudaSuccess) return e;    \
            k_col<float, LV, 16, false><<<grid, nt, sm, st>>>(a);                        \
        }                                                                                \
        break;
        PS_P2_LENGTHS(X)
#undef X
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int L, int EM>
cudaError_t launch_z_len(const ZArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    cudaError_t e;
    switch (a.op) {
#define Z(OPV)                                                                     \
    case OPV:                                                                      \
        if ((e = prep(k_z<float, L, EM, OPV>, sm)) != cudaSuccess) return e;       \
        k_z<float, L, EM, OPV><<<grid, nt, sm, st>>>(a);                           \
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

bool supports_op(int op) { return op == OP_NONE || op == OP_GRAD || op == OP_DIV || op == OP_CURL; }

cudaError_t launch_z(const ZArgs &a, int ny, int em, cudaStream_t st)
{
    dim3 grid((unsigned)((a.Mx + a.B - 1) / a.B), ny);
    const int nbuf = a.nin > a.nout ? a.nin : a.nout;
    const size_t sm = smem_lines(PREC_FP32, a.L, a.B, nbuf, a.plan.ntw);
    const int nt = a.B * (a.L / em);
    switch (a.L) {
#define X(LV)                                                                         \
    case LV:                                                                          \
        return em == 8 ? launch_z_len<LV, 8>(a, grid, nt, sm, st)                     \
                       : launch_z_len<LV, 16>(a, grid, nt, sm, st);
        PS_P2_LENGTHS(X)
#undef X
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_xinv(const XInvArgs &a, cudaStream_t st)
{
    const long long rows = (long long)a.rows_y * a.rows_z;
    dim3 grid((unsigned)(((rows + 1) / 2 + a.B - 1) / a.B), a.ncomp);
    const size_t sm = smem_lines(PREC_FP32, a.L, a.B, 1, a.plan.ntw);
    const int nt = a.B * (a.L / e_max(PREC_FP32));
    switch (a.L) {
#define X(LV) \
    case LV: return launch_xinv_len<LV>(a, grid, nt, sm, st);
        PS_P2_LENGTHS(X)
#undef X
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace p2
}  // namespace ps
