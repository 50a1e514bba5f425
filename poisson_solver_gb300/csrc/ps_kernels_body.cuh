// Pass kernels of the 3D solve with run-time transform plans (any length):
// x forward (real-to-half-spectrum, zero-pad fused), y column transforms, the
// fused z pass (forward, spectral kernel and derivative operator, inverse),
// and x inverse (half-spectrum-to-real, crop fused). Each CTA stages its
// lines in shared memory and runs the Stockham stages of ps_fft.cuh on them;
// global traffic is coalesced along x. Templated on the pass precision T
// (double, float or dfloat); ps_kernels.cu instantiates the first two and
// ps_kernels_df.cu the third, each through the typed launches (namespace rt)
// at the end of this file.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "ps_fft.cuh"
#include "ps_types.hpp"

namespace ps {

namespace {

template <typename T> struct Cplx { using type = typename CxT<T>::type; };

__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }

// element budget per thread: x and y passes, and the fused z pass
template <typename T> constexpr int EMX = e_max(sizeof(T) == 8 ? PREC_FP64 : PREC_FP32);
template <typename T> constexpr int EMZ = e_max_z(sizeof(T) == 8 ? PREC_FP64 : PREC_FP32);

}  // namespace

// ---------------------------------------------------------------------------
// x forward. Line l of the CTA carries rows 2l (real part) and 2l+1 (imag
// part); after the complex transform Z the two half spectra are
// Xa[k] = (Z[k] + conj Z[L-k]) / 2 and Xb[k] = (Z[k] - conj Z[L-k]) / 2i.
//
// The pass bodies take the CTA's tile coordinates and its working thread count
// nt explicitly, so the same code serves the per-problem launches and the
// batched ones (one launch over the tiles of many problems, where a CTA may
// have more threads than the problem of its tile uses). Threads tid >= nt only
// join the barriers: their line-thread index is set to L, past every
// butterfly, and the load/store loops skip them.
template <typename T, bool RAD = false>
__device__ __forceinline__ void xfwd_body(const XFwdArgs &a, int bx, int comp, int nt)
{
    using C = typename Cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, L = a.L, ld = a.plan.L + 1;  // lines as long as the plan's working length
    C *W = a.plan.generic ? S + B * ld : nullptr;
    const FftPlanDev &plan = a.plan;
    const C *tws = stage_twiddles(plan, S + B * ld * (a.plan.generic ? 2 : 1));
    __shared__ StageInfo si;
    load_stages(si, a.plan);
    const double *in = pick3(a.in, comp);
    C *out = reinterpret_cast<C *>(pick3(a.out, comp));
    const int tid = threadIdx.x;
    const bool live = tid < nt;
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long row0 = (long long)bx * 2 * B;
    __shared__ long long rofs[2 * MAX_LINES];
    row_offsets(rofs, row0, 2 * B, rows, a.rows_y, a.out_y, a.ld);

    // line l = (row 2l, row 2l+1) as (re, im); zero past n_in and past the last
    // row. With the mirror flag the rows are those of the kernel octant,
    // (z, y) -> (min(z, Pz-z), min(y, Py-y)), and n -> min(n, L-n).
    for (int line = 0; line < B; ++line) {
        const long long ra = row0 + 2 * line;
        const bool va = ra < rows, vb = ra + 1 < rows;
        long long oa = ra * a.in_stride, ob = oa + a.in_stride;
        if (a.mirror) {
            if (va) {
                const int j = (int)(ra % a.rows_y), k = (int)(ra / a.rows_y);
                oa = ((long long)imin(k, a.Pz - k) * a.oct_y + imin(j, a.Py - j)) * a.oct_x;
            }
            if (vb) {
                const int j = (int)((ra + 1) % a.rows_y), k = (int)((ra + 1) / a.rows_y);
                ob = ((long long)imin(k, a.Pz - k) * a.oct_y + imin(j, a.Py - j)) * a.oct_x;
            }
        }
        C *ln = S + line * ld;
        for (int n = live ? tid : L; n < L; n += nt) {
            T xa = (T)0, xb = (T)0;
            if (n < a.n_in) {
                const int nn = a.mirror ? imin(n, L - n) : n;
                if (va) xa = (T)in[oa + nn];
                if (vb) xb = (T)in[ob + nn];
            }
            ln[n] = C{xa, xb};
        }
    }
    __syncthreads();
    fft_lines<false, EMX<T>, RAD>(S, W, 1, ld, tid % B, live ? tid / B : IDLE_T, plan, tws, si);

    // separate the two half spectra and store
    const int Mx = a.Mx;
    for (int line = 0; line < B; ++line) {
        const long long oa = rofs[2 * line], ob = rofs[2 * line + 1];
        if (oa < 0) break;
        for (int k = live ? tid : Mx; k < Mx; k += nt) {
            const C z = S[line * ld + k], w = S[line * ld + (k == 0 ? 0 : L - k)];
            const T h = (T)0.5;
            out[oa + k] = C{h * (z.x + w.x), h * (z.y - w.y)};
            if (ob >= 0) out[ob + k] = C{h * (z.y + w.y), h * (w.x - z.x)};
        }
    }
}

template <typename T, bool RAD = false> __global__ void __launch_bounds__(MAX_THREADS) k_xfwd(const XFwdArgs a)
{
    xfwd_body<T, RAD>(a, blockIdx.x, blockIdx.y, blockDim.x);
}

// ---------------------------------------------------------------------------
// Column transforms along a strided axis, in place: the CTA takes B adjacent
// columns (one 128-byte row segment per sample for the default B) of one slab.
template <typename T, bool INV, bool RAD = false>
__device__ __forceinline__ void col_body(const ColArgs &a, int bx, int slab, int comp, int nt)
{
    using C = typename Cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, L = a.L, Lw = a.plan.L;  // Lw: the plan's working length
    C *W = a.plan.generic ? S + Lw * B : nullptr;
    const int lb = __ffs(B) - 1;
    const FftPlanDev &plan = a.plan;
    const C *tws = stage_twiddles(plan, S + Lw * B * (a.plan.generic ? 2 : 1));
    __shared__ StageInfo si;
    load_stages(si, a.plan);
    const int x0 = bx * B;
    const int nb = imin(B, a.Mx - x0);
    C *base = reinterpret_cast<C *>(pick3(a.data, comp)) + (long long)slab * a.outer_stride + x0;
    const int tid = threadIdx.x;

    // each thread keeps one column b and walks rows n = t, t + nt/B, ...
    const int b = tid & (B - 1), t = tid < nt ? tid >> lb : IDLE_T, rstep = nt >> lb;
    const long long gstep = (long long)rstep * a.axis_stride;
    {
        const C *src = base + (long long)t * a.axis_stride + b;
        const int n_in = b < nb ? a.n_in : 0;
#pragma unroll 4
        for (int n = t; n < L; n += rstep, src += gstep) {
            C v = C{0, 0};
            if (n < n_in) v = *src;
            S[n * B + b] = v;
        }
    }
    __syncthreads();
    fft_lines<INV, EMX<T>, RAD>(S, W, B, 1, b, t, plan, tws, si);
    if (b < nb) {
        C *dst = base + (long long)t * a.axis_stride + b;
#pragma unroll 4
        for (int n = t; n < a.n_out; n += rstep, dst += gstep) *dst = S[n * B + b];
    }
}

template <typename T, bool INV, bool RAD = false> __global__ void __launch_bounds__(MAX_THREADS) k_col(const ColArgs a)
{
    col_body<T, INV, RAD>(a, blockIdx.x, blockIdx.y, blockIdx.z, blockDim.x);
}

// ---------------------------------------------------------------------------
// Fused z pass.
template <typename T>
__device__ __forceinline__ T wavenumber(int k, int P, T c, bool derivative)
{
    // k in [0, P): signed index wrapped at P/2; the derivative drops the
    // unpaired Nyquist mode (its Hermitian part vanishes in the real output).
    // Computed in the pass precision (FP64 arithmetic is slow on this GPU).
    const int m = (2 * k < P) ? k : k - P;
    if (derivative && 2 * k == P) return (T)0;
    return (T)m * c;
}

// OPT: the spectral operation, or -1 to take it from a.op at run time (the
// batched pass); a fixed OPT folds every test on op away.
template <typename T, int OPT, bool RAD = false>
__device__ __forceinline__ void z_body(const ZArgs &a, int bx, int by, int nt)
{
    const int op = OPT >= 0 ? OPT : a.op;
    using C = typename Cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, L = a.L, LB = a.plan.L * B;  // buffers as long as the plan's working length
    const int nbuf = a.nin > a.nout ? a.nin : a.nout;
    C *W = a.plan.generic ? S + nbuf * LB : nullptr;
    const int lb = __ffs(B) - 1;
    const int x0 = bx * B;
    const int ky = a.ky0 + by;
    const int nb = imin(B, a.Mx - x0);
    const long long off = (long long)ky * a.row_stride + x0;
    const int tid = threadIdx.x;
    const int b = tid & (B - 1), t = tid < nt ? tid >> lb : IDLE_T;
    const FftPlanDev &plan = a.plan;
    const C *tws = stage_twiddles(plan, S + (nbuf + (a.plan.generic ? 1 : 0)) * LB);
    __shared__ StageInfo si;
    load_stages(si, a.plan);

    const int rstep = nt >> lb;
    const long long gstep = (long long)rstep * a.axis_stride;
    const int n_in = b < nb ? a.n_in : 0;
    for (int c = 0; c < a.nin; ++c) {
        const C *src = reinterpret_cast<const C *>(pick3(a.in, c)) + off + (long long)t * a.axis_stride + b;
        C *buf = S + c * LB + b;
#pragma unroll 4
        for (int n = t; n < L; n += rstep, src += gstep) {
            C v = C{0, 0};
            if (n < n_in) v = *src;
            buf[n * B] = v;
        }
    }
    __syncthreads();
    fft_lines<false, EMZ<T>, RAD>(S, W, B, 1, b, t, plan, tws, si, a.nin, LB);

    if (op != OP_FORWARD) {
        // the thread's column kx is fixed; it walks kz = t, t + nt/B, ...
        const int oy = imin(ky, a.Py - ky);
        const int kx = x0 + b;
        const T *Kc = reinterpret_cast<const T *>(a.kern) + (long long)oy * a.Mx + kx;
        const long long kzs = (long long)a.oct_y * a.Mx;
        const T kyv = wavenumber<T>(ky, a.Py, (T)a.kyc, true);
        const T kxv = wavenumber<T>(kx, a.Px, (T)a.kxc, true);
        const T kzc = (T)a.kzc;
        for (int n = t; n < (b < nb ? L : 0); n += rstep) {
            const int idx = n * B + b;
            const int oz = imin(n, a.Pz - n);
            const T g = Kc[oz * kzs];
            const T kzv = wavenumber<T>(n, a.Pz, kzc, true);
            if (op == OP_NONE) {
                for (int c = 0; c < a.nin; ++c) S[c * LB + idx] = cscale(S[c * LB + idx], g);
            } else if (op == OP_GRAD) {
                // out_d = i k_d K in_d; in_d falls back to component x
                const C i0 = S[idx];
                const C i1 = a.nin > 1 ? S[LB + idx] : i0;
                const C i2 = a.nin > 2 ? S[2 * LB + idx] : i0;
                const T gx = g * kxv, gy = g * kyv, gz = g * kzv;
                S[idx] = C{-gx * i0.y, gx * i0.x};
                S[LB + idx] = C{-gy * i1.y, gy * i1.x};
                S[2 * LB + idx] = C{-gz * i2.y, gz * i2.x};
            } else if (op == OP_DIV) {
                const C i0 = S[idx], i1 = S[LB + idx], i2 = S[2 * LB + idx];
                const C s = C{kxv * i0.x + kyv * i1.x + kzv * i2.x, kxv * i0.y + kyv * i1.y + kzv * i2.y};
                S[idx] = C{-g * s.y, g * s.x};
            } else if (op == OP_CURL) {
                const C i0 = S[idx], i1 = S[LB + idx], i2 = S[2 * LB + idx];
                const C c0 = C{kyv * i2.x - kzv * i1.x, kyv * i2.y - kzv * i1.y};
                const C c1 = C{kzv * i0.x - kxv * i2.x, kzv * i0.y - kxv * i2.y};
                const C c2 = C{kxv * i1.x - kyv * i0.x, kxv * i1.y - kyv * i0.y};
                S[idx] = C{-g * c0.y, g * c0.x};
                S[LB + idx] = C{-g * c1.y, g * c1.x};
                S[2 * LB + idx] = C{-g * c2.y, g * c2.x};
            } else if (op == OP_FILTER) {
                const T z = (reinterpret_cast<const T *>(a.zeta) + (long long)oy * a.Mx + kx)[oz * kzs];
                if (a.reproject && a.nin == 3) {
                    // r'_c = z r_c - K sum_d k_c k_d r_d. A product k_c k_d is
                    // even under k -> -k (and survives in the real output)
                    // unless exactly one of the two axes sits on its Nyquist
                    // mode, where the unpaired wavenumber makes it odd.
                    const T kf[3] = {wavenumber<T>(kx, a.Px, (T)a.kxc, false),
                                     wavenumber<T>(ky, a.Py, (T)a.kyc, false), wavenumber<T>(n, a.Pz, kzc, false)};
                    const bool nq[3] = {2 * kx == a.Px, 2 * ky == a.Py, 2 * n == a.Pz};
                    const C in3[3] = {S[idx], S[LB + idx], S[2 * LB + idx]};
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        C acc = C{0, 0};
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            const T kk = nq[c] == nq[d] ? kf[c] * kf[d] : (T)0;
                            acc.x += kk * in3[d].x;
                            acc.y += kk * in3[d].y;
                        }
                        S[c * LB + idx] = C{z * in3[c].x - g * acc.x, z * in3[c].y - g * acc.y};
                    }
                } else {
                    for (int c = 0; c < a.nin; ++c) S[c * LB + idx] = cscale(S[c * LB + idx], z);
                }
            }
        }
        __syncthreads();
        fft_lines<true, EMZ<T>, RAD>(S, W, B, 1, b, t, plan, tws, si, a.nout, LB);
    }

    if (b < nb) {
        for (int c = 0; c < a.nout; ++c) {
            C *dst0 = reinterpret_cast<C *>(pick3(a.out, c));
            if (dst0 == nullptr) continue;
            C *dst = dst0 + off + (long long)t * a.axis_stride + b;
            const C *buf = S + c * LB + b;
#pragma unroll 4
            for (int n = t; n < a.n_out; n += rstep, dst += gstep) *dst = buf[n * B];
        }
    }
}

template <typename T, int OP, bool RAD = false> __global__ void __launch_bounds__(MAX_THREADS) k_z(const ZArgs a)
{
    z_body<T, OP, RAD>(a, blockIdx.x, blockIdx.y, blockDim.x);
}

// ---------------------------------------------------------------------------
// x inverse. Line l rebuilds Z = Xa + i Xb over the full length from the two
// half spectra (Z[L-k] = conj Xa[k] + i conj Xb[k]), transforms back and
// writes Re -> row 2l, Im -> row 2l+1, first n_out samples only.
template <typename T, bool RAD = false>
__device__ __forceinline__ void xinv_body(const XInvArgs &a, int bx, int comp, int nt)
{
    using C = typename Cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    const int B = a.B, L = a.L, ld = a.plan.L + 1, Mx = a.Mx;
    C *W = a.plan.generic ? S + B * ld : nullptr;
    const FftPlanDev &plan = a.plan;
    const C *tws = stage_twiddles(plan, S + B * ld * (a.plan.generic ? 2 : 1));
    __shared__ StageInfo si;
    load_stages(si, a.plan);
    const C *in = reinterpret_cast<const C *>(pick3(a.in, comp));
    double *out = pick3(a.out, comp);
    const int tid = threadIdx.x;
    const bool live = tid < nt;
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long row0 = (long long)bx * 2 * B;
    __shared__ long long rofs[2 * MAX_LINES];
    row_offsets(rofs, row0, 2 * B, rows, a.rows_y, a.in_y, a.ld);
    __syncthreads();

    for (int line = 0; line < B; ++line) {
        const long long oa = rofs[2 * line], ob = rofs[2 * line + 1];
        for (int k = live ? tid : Mx; k < Mx; k += nt) {
            C xa = C{0, 0}, xb = C{0, 0};
            if (oa >= 0) xa = in[oa + k];
            if (ob >= 0) xb = in[ob + k];
            S[line * ld + k] = C{xa.x - xb.y, xa.y + xb.x};
            if (k >= 1 && k <= L - Mx) S[line * ld + L - k] = C{xa.x + xb.y, xb.x - xa.y};
        }
    }
    __syncthreads();
    fft_lines<true, EMX<T>, RAD>(S, W, 1, ld, tid % B, live ? tid / B : IDLE_T, plan, tws, si);

    // line l -> rows 2l (real parts) and 2l+1 (imaginary parts), n < n_out
    const int no = a.n_out;
    for (int line = 0; line < B; ++line) {
        const long long ra = row0 + 2 * line;
        if (ra >= rows) break;
        const bool vb = ra + 1 < rows;
        double *oa = out + ra * a.out_stride, *ob = oa + a.out_stride;
        const C *ln = S + line * ld;
        for (int n = live ? tid : no; n < no; n += nt) {
            const C v = ln[n];
            oa[n] = (double)v.x;
            if (vb) ob[n] = (double)v.y;
        }
    }
}

template <typename T, bool RAD = false> __global__ void __launch_bounds__(MAX_THREADS) k_xinv(const XInvArgs a)
{
    xinv_body<T, RAD>(a, blockIdx.x, blockIdx.y, blockDim.x);
}

// ---------------------------------------------------------------------------
// Batched passes: one launch runs a pass of many independent problems. CTA i
// takes tile i of the tile list, copies the arguments of its tile's problem
// into shared memory and runs the pass body with that problem's thread count
// (the launch's block size is the largest of them). One tile a CTA, not a
// persistent CTA walking the list: with the pass body inside a tile loop
// ptxas kept these kernels at 128 registers and spilled 1.7-3.7 KB a thread
// (255 registers still spilled 1.1-1.8 KB), where one tile a CTA compiles to
// 48-76 registers without spills.
template <typename Args> __device__ __forceinline__ void load_args(Args &dst, const Args *src)
{
    static_assert(sizeof(Args) % sizeof(int) == 0, "argument blocks are whole words");
    const int *s = reinterpret_cast<const int *>(src);
    int *d = reinterpret_cast<int *>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(Args) / sizeof(int)); i += blockDim.x) d[i] = s[i];
}

template <typename T, bool RAD = false>
__global__ void __launch_bounds__(BATCH_MAX_THREADS) k_xfwd_batch(const XFwdArgs *args, const BatchTile *tiles, int ntiles)
{
    __shared__ XFwdArgs a;
    if ((int)blockIdx.x < ntiles) {
        const BatchTile tl = tiles[blockIdx.x];
        load_args(a, args + tl.p);
        __syncthreads();
        xfwd_body<T, RAD>(a, tl.bx, tl.by, a.B * a.plan.tpl);
    }
}

template <typename T, bool INV, bool RAD = false>
__global__ void __launch_bounds__(BATCH_MAX_THREADS) k_col_batch(const ColArgs *args, const BatchTile *tiles, int ntiles)
{
    __shared__ ColArgs a;
    if ((int)blockIdx.x < ntiles) {
        const BatchTile tl = tiles[blockIdx.x];
        load_args(a, args + tl.p);
        __syncthreads();
        col_body<T, INV, RAD>(a, tl.bx, tl.by, tl.bz, a.B * a.plan.tpl);
    }
}

template <typename T, bool RAD = false>
__global__ void __launch_bounds__(BATCH_MAX_THREADS) k_z_batch(const ZArgs *args, const BatchTile *tiles, int ntiles)
{
    __shared__ ZArgs a;
    if ((int)blockIdx.x < ntiles) {
        const BatchTile tl = tiles[blockIdx.x];
        load_args(a, args + tl.p);
        __syncthreads();
        z_body<T, -1, RAD>(a, tl.bx, tl.by, a.B * a.plan.tpl);
    }
}

template <typename T, bool RAD = false>
__global__ void __launch_bounds__(BATCH_MAX_THREADS) k_xinv_batch(const XInvArgs *args, const BatchTile *tiles, int ntiles)
{
    __shared__ XInvArgs a;
    if ((int)blockIdx.x < ntiles) {
        const BatchTile tl = tiles[blockIdx.x];
        load_args(a, args + tl.p);
        __syncthreads();
        xinv_body<T, RAD>(a, tl.bx, tl.by, a.B * a.plan.tpl);
    }
}

// ---------------------------------------------------------------------------
// Typed launches: grid, block and shared-memory sizes come from the public
// launchers (ps_kernels.cu), which dispatch on the precision.
namespace rt {

template <typename K> inline cudaError_t prep(K kernel, size_t smem)
{
    // Always: the 48 KB a launch gets without it includes the kernel's static
    // shared memory, so a request just under 48 KB can already be too large.
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <typename K, typename A> inline cudaError_t run(K kernel, dim3 grid, int nt, size_t sm, cudaStream_t st, const A &a)
{
    cudaError_t e = prep(kernel, sm);
    if (e != cudaSuccess) return e;
    kernel<<<grid, nt, sm, st>>>(a);
    return cudaGetLastError();
}

// Rader plans (an FP32 plan variant) run on their own instantiations, in
// ps_kernels_rader.cu (a translation unit of its own, compiled in parallel).
template <typename T> constexpr bool HAS_RAD = std::is_same<T, float>::value;
cudaError_t xfwd_rader(const XFwdArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st);
cudaError_t col_rader(int inverse, const ColArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st);
cudaError_t z_rader(const ZArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st);
cudaError_t xinv_rader(const XInvArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st);
cudaError_t xfwd_batch_rader(const XFwdArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                             cudaStream_t st);
cudaError_t col_batch_rader(int inverse, const ColArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                            cudaStream_t st);
cudaError_t z_batch_rader(const ZArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem, cudaStream_t st);
cudaError_t xinv_batch_rader(const XInvArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                             cudaStream_t st);

template <typename T> inline cudaError_t xfwd(const XFwdArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    if constexpr (HAS_RAD<T>)
        if (a.plan.rader) return xfwd_rader(a, grid, nt, sm, st);
    return run(k_xfwd<T>, grid, nt, sm, st, a);
}

template <typename T>
inline cudaError_t col(int inverse, const ColArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    if constexpr (HAS_RAD<T>)
        if (a.plan.rader) return col_rader(inverse, a, grid, nt, sm, st);
    return inverse ? run(k_col<T, true>, grid, nt, sm, st, a) : run(k_col<T, false>, grid, nt, sm, st, a);
}

template <typename T> inline cudaError_t z(const ZArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    if constexpr (HAS_RAD<T>)
        if (a.plan.rader) return z_rader(a, grid, nt, sm, st);
    switch (a.op) {
    case OP_NONE: return run(k_z<T, OP_NONE>, grid, nt, sm, st, a);
    case OP_GRAD: return run(k_z<T, OP_GRAD>, grid, nt, sm, st, a);
    case OP_DIV: return run(k_z<T, OP_DIV>, grid, nt, sm, st, a);
    case OP_CURL: return run(k_z<T, OP_CURL>, grid, nt, sm, st, a);
    case OP_FILTER: return run(k_z<T, OP_FILTER>, grid, nt, sm, st, a);
    case OP_FORWARD: return run(k_z<T, OP_FORWARD>, grid, nt, sm, st, a);
    default: return cudaErrorInvalidValue;
    }
}

// one kernel for every spectral operation, read from a.op at run time
template <typename T> inline cudaError_t z_any_op(const ZArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    return run(k_z<T, -1>, grid, nt, sm, st, a);
}

template <typename T> inline cudaError_t xinv(const XInvArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    if constexpr (HAS_RAD<T>)
        if (a.plan.rader) return xinv_rader(a, grid, nt, sm, st);
    return run(k_xinv<T>, grid, nt, sm, st, a);
}

// Batched launches: nt threads and smem bytes a CTA (the largest over the
// batch's problems), one CTA a tile; a configuration no SM can hold is an
// error here rather than at the launch.
template <typename K> inline cudaError_t tile_grid(K kernel, int ntiles, int nt, size_t smem, int &grid)
{
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nt, smem)) != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    grid = ntiles;
    return cudaSuccess;
}

template <typename K, typename A>
inline cudaError_t run_tiles(K kernel, const A *args, const BatchTile *tiles, int ntiles, int nt, size_t smem, cudaStream_t st)
{
    int grid = 0;
    cudaError_t e = tile_grid(kernel, ntiles, nt, smem, grid);
    if (e != cudaSuccess) return e;
    kernel<<<grid, nt, smem, st>>>(args, tiles, ntiles);
    return cudaGetLastError();
}

// rader: some problem of the launch has a Rader plan on this pass (FP32)
template <typename T>
inline cudaError_t xfwd_batch(const XFwdArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem, bool rader,
                              cudaStream_t st)
{
    if constexpr (HAS_RAD<T>)
        if (rader) return xfwd_batch_rader(args, tiles, ntiles, nt, smem, st);
    return run_tiles(k_xfwd_batch<T>, args, tiles, ntiles, nt, smem, st);
}

template <typename T>
inline cudaError_t col_batch(int inverse, const ColArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                             bool rader, cudaStream_t st)
{
    if constexpr (HAS_RAD<T>)
        if (rader) return col_batch_rader(inverse, args, tiles, ntiles, nt, smem, st);
    return inverse ? run_tiles(k_col_batch<T, true>, args, tiles, ntiles, nt, smem, st)
                   : run_tiles(k_col_batch<T, false>, args, tiles, ntiles, nt, smem, st);
}

template <typename T>
inline cudaError_t z_batch(const ZArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem, bool rader,
                           cudaStream_t st)
{
    if constexpr (HAS_RAD<T>)
        if (rader) return z_batch_rader(args, tiles, ntiles, nt, smem, st);
    return run_tiles(k_z_batch<T>, args, tiles, ntiles, nt, smem, st);
}

template <typename T>
inline cudaError_t xinv_batch(const XInvArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem, bool rader,
                              cudaStream_t st)
{
    if constexpr (HAS_RAD<T>)
        if (rader) return xinv_batch_rader(args, tiles, ntiles, nt, smem, st);
    return run_tiles(k_xinv_batch<T>, args, tiles, ntiles, nt, smem, st);
}

// the double-float instantiations (ps_kernels_df.cu): single problems only,
// the z pass with its spectral operation read at run time
cudaError_t xfwd_df(const XFwdArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st);
cudaError_t col_df(int inverse, const ColArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st);
cudaError_t z_df(const ZArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st);
cudaError_t xinv_df(const XInvArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st);

}  // namespace rt

}  // namespace ps
