// x passes with a warp per line group (FP32; L = 256, 512, 1024).
//
// A line is a pair of real rows packed as one complex line (row 2l the real
// part, row 2l + 1 the imaginary part). Its L/32 threads are consecutive
// lanes of one warp (L = 1024: one warp; 512: half; 256: a quarter), each
// holding 32 elements, so a line is two radix-32 stages with one exchange
// through the line's padded shared buffer, and every synchronisation is a
// warp barrier: the warps of a CTA run independently, with no CTA barrier
// after the twiddle table is loaded. Global memory is read and written
// straight from registers along the rows (a warp instruction covers 32
// consecutive elements of a row, 256 contiguous bytes):
//   forward: the first stage loads its 32 (HALF: 16, the rest is the zero
//     padding) FP64 samples of each row, the last stage's outputs are split
//     into the two half spectra on the way out, each beside its mirror
//     fetched from another lane by a warp shuffle;
//   inverse: the two half spectra are combined into the first stage's
//     inputs in registers (mirrors by warp shuffles), the last stage stores
//     Re and Im of its outputs (HALF: the kept half) to the two FP64 rows.
// Against the length-specialised kernels (16 elements a thread, three stages
// through shared memory, CTA barriers) this halves the shared-memory passes.
#include "ps_wide.cuh"

namespace ps {
namespace wide {

namespace {

constexpr int XQ_THREADS = 256;

template <int L> struct Xq {
    static constexpr int TPL = L / 32;          // threads a line
    static constexpr int NL = XQ_THREADS / TPL;  // lines a CTA
    static constexpr int LDP = pitch_row(L);
    static constexpr int Mx = L / 2 + 1;
    static constexpr int KPER = (Mx + TPL - 1) / TPL;  // half-spectrum elements a thread
    static size_t bytes(int ntw) { return sizeof(float2) * ((size_t)NL * LDP + (size_t)ntw); }
};

// Output (or input) offset of spectrum row r = k rows_y + j: (k ny + j) ld; -1 past the rows.
__device__ __forceinline__ long long spec_row(long long r, long long rows, int rows_y, int ny, int ld)
{
    if (r >= rows) return -1;
    const long long k = r / rows_y;
    return (k * ny + (r - k * rows_y)) * ld;
}

template <int L, bool HALF>
__global__ void __launch_bounds__(XQ_THREADS, 2) k_xfq(const XFwdArgs a)
{
    using C = float2;
    using PL = WP<L>;
    using Q = Xq<L>;
    constexpr int LAST = PL::NST - 1;
    using T0 = St<L, 0>;
    using TL = St<L, LAST>;
    static_assert(PL::NST == 2 && T0::U == 1 && T0::R == 32, "two stages, one radix-32 butterfly first");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    C *TW = S + Q::NL * Q::LDP;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    __syncthreads();

    const int l = threadIdx.x / Q::TPL, t = threadIdx.x % Q::TPL;
    C *line = S + l * Q::LDP;
    const double *in = pick3(a.in, blockIdx.y);
    C *out = reinterpret_cast<C *>(pick3(a.out, blockIdx.y));
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long ra = 2 * ((long long)blockIdx.x * Q::NL + l), rb = ra + 1;
    const bool va = ra < rows, vb = rb < rows;
    {
        const double *pa = in + ra * a.in_stride + t, *pb = pa + a.in_stride;
        constexpr int RN = HALF ? 16 : 32;  // HALF: n_in = L/2 exactly
        C v[1][32];
#pragma unroll
        for (int r = 0; r < RN; ++r) {
            const bool live = HALF || t + r * Q::TPL < a.n_in;
            v[0][r] = C{(va && live) ? (float)pa[r * Q::TPL] : 0.f, (vb && live) ? (float)pb[r * Q::TPL] : 0.f};
        }
        if constexpr (HALF) {
            dft32_half<false>(v[0]);
        } else {
            dft<32, false>(v[0]);  // the first stage has no twiddles (m = 1)
        }
        write_line<L, 0>(line, t, v);
    }
    __syncwarp();
    C v[TL::U][TL::R];
    read_line<L, LAST>(line, t, v);
    twiddle_dft<L, LAST, false>(v, TW, t);
    // Separate the half spectra of rows a and b straight from the registers:
    // this thread holds Z[k], k = t + TPL u + 32 r, and the mirror Z[L - k]
    // sits in lane TPL - t of the line at (U - 1 - u, R - 1 - r), or for
    // t = 0 in this thread ((0, R - r mod R) for u = 0, else (U - u, R - 1 - r));
    // one warp shuffle a value, for the k < L/2 this thread stores.
    constexpr int U = TL::U, R = TL::R;
    const long long oa = spec_row(ra, rows, a.rows_y, a.out_y, a.ld), ob = spec_row(rb, rows, a.rows_y, a.out_y, a.ld);
    C *outa = out + (oa >= 0 ? oa : 0), *outb = out + (ob >= 0 ? ob : 0);
    const int lane = threadIdx.x & 31;
    const int src = (lane & ~(Q::TPL - 1)) | ((Q::TPL - t) & (Q::TPL - 1));
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
        for (int r = 0; r < R / 2; ++r) {
            const C z = v[u][r], p = v[U - 1 - u][R - 1 - r];
            C w = C{__shfl_sync(0xffffffffu, p.x, src), __shfl_sync(0xffffffffu, p.y, src)};
            if (t == 0) w = v[u == 0 ? 0 : U - u][u == 0 ? (R - r) % R : R - 1 - r];
            const int k = t + Q::TPL * u + 32 * r;
            if (oa >= 0) outa[k] = C{0.5f * (z.x + w.x), 0.5f * (z.y - w.y)};
            if (ob >= 0) outb[k] = C{0.5f * (z.y + w.y), 0.5f * (w.x - z.x)};
        }
    if (t == 0) {  // k = L/2 is its own mirror
        const C z = v[0][R / 2];
        if (oa >= 0) outa[L / 2] = C{0.5f * (z.x + z.x), 0.5f * (z.y - z.y)};
        if (ob >= 0) outb[L / 2] = C{0.5f * (z.y + z.y), 0.5f * (z.x - z.x)};
    }
}

template <int L, bool HALF>
__global__ void __launch_bounds__(XQ_THREADS, 2) k_xiq(const XInvArgs a)
{
    using C = float2;
    using PL = WP<L>;
    using Q = Xq<L>;
    constexpr int LAST = PL::NST - 1;
    using T0 = St<L, 0>;
    using TL = St<L, LAST>;
    static_assert(PL::NST == 2 && T0::U == 1 && T0::R == 32, "two stages, one radix-32 butterfly first");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *S = reinterpret_cast<C *>(smem_raw);
    C *TW = S + Q::NL * Q::LDP;
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    __syncthreads();

    const int l = threadIdx.x / Q::TPL, t = threadIdx.x % Q::TPL;
    C *line = S + l * Q::LDP;
    const C *in = reinterpret_cast<const C *>(pick3(a.in, blockIdx.y));
    double *out = pick3(a.out, blockIdx.y);
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long ra = 2 * ((long long)blockIdx.x * Q::NL + l), rb = ra + 1;
    {
        // Z = Xa + i Xb over the full line from the two half spectra
        const long long ia = spec_row(ra, rows, a.rows_y, a.in_y, a.ld), ib = spec_row(rb, rows, a.rows_y, a.in_y, a.ld);
        const C *pa = in + (ia >= 0 ? ia : 0) + t, *pb = in + (ib >= 0 ? ib : 0) + t;
        C xa[Q::KPER], xb[Q::KPER];
#pragma unroll
        for (int j = 0; j < Q::KPER; ++j) {
            const bool live = t + j * Q::TPL < Q::Mx;
            xa[j] = (live && ia >= 0) ? pa[j * Q::TPL] : C{0.f, 0.f};
            xb[j] = (live && ib >= 0) ? pb[j * Q::TPL] : C{0.f, 0.f};
        }
        // The first stage's inputs Z[t + TPL r], r < 32, from the registers:
        // Z[k] = Xa[k] + i Xb[k] for r < 16 (k < L/2); above, the mirror
        // conj(Xa[k']) + i conj(Xb[k']) of k' = L - k, loaded by lane TPL - t
        // of the line at j = 31 - r (one warp shuffle), or for t = 0 by this
        // thread (Z[L/2] directly at j = 16, then the mirrors of j = 32 - r).
        // j runs down so the loaded values die as they are used.
        static_assert(Q::KPER == 17, "16 values below L/2 a thread, and L/2 itself");
        const int lane = threadIdx.x & 31;
        const int src = (lane & ~(Q::TPL - 1)) | ((Q::TPL - t) & (Q::TPL - 1));
        C v0[1][32];
        C own = C{xa[16].x - xb[16].y, xa[16].y + xb[16].x};  // t = 0: Z[L/2]
#pragma unroll
        for (int j = 15; j >= 0; --j) {
            v0[0][j] = C{xa[j].x - xb[j].y, xa[j].y + xb[j].x};
            const C m = C{xa[j].x + xb[j].y, xb[j].x - xa[j].y};
            const C got = C{__shfl_sync(0xffffffffu, m.x, src), __shfl_sync(0xffffffffu, m.y, src)};
            v0[0][31 - j] = t == 0 ? own : got;
            own = m;
        }
        dft<32, true>(v0[0]);  // the first stage has no twiddles (m = 1)
        write_line<L, 0>(line, t, v0);
    }
    __syncwarp();
    C v[TL::U][TL::R];
    read_line<L, LAST>(line, t, v);
    twiddle_dft<L, LAST, true>(v, TW, t);
    if (ra >= rows) return;
    // Re -> row a, Im -> row b; HALF: out_pos = r M + bf with bf < M, so r < R/2 is the kept half
    double *pa = out + ra * a.out_stride, *pb = pa + a.out_stride;
    const bool vb = rb < rows;
    constexpr int RW = HALF ? TL::R / 2 : TL::R;
#pragma unroll
    for (int u = 0; u < TL::U; ++u)
#pragma unroll
        for (int r = 0; r < RW; ++r) {
            const int n = TL::out_pos(t, u, r);
            if (HALF || n < a.n_out) {
                pa[n] = (double)v[u][r].x;
                if (vb) pb[n] = (double)v[u][r].y;
            }
        }
}

template <typename K> cudaError_t prep_q(K kernel, size_t sm)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
}

template <int L, bool HALF> cudaError_t launch_xfq_t(const XFwdArgs &a, cudaStream_t st)
{
    using Q = Xq<L>;
    const long long pairs = ((long long)a.rows_y * a.rows_z + 1) / 2;
    const dim3 grid((unsigned)((pairs + Q::NL - 1) / Q::NL), a.ncomp);
    const size_t sm = Q::bytes(a.plan.ntw);
    const cudaError_t e = prep_q(k_xfq<L, HALF>, sm);
    if (e != cudaSuccess) return e;
    k_xfq<L, HALF><<<grid, XQ_THREADS, sm, st>>>(a);
    return cudaGetLastError();
}

template <int L, bool HALF> cudaError_t launch_xiq_t(const XInvArgs &a, cudaStream_t st)
{
    using Q = Xq<L>;
    const long long pairs = ((long long)a.rows_y * a.rows_z + 1) / 2;
    const dim3 grid((unsigned)((pairs + Q::NL - 1) / Q::NL), a.ncomp);
    const size_t sm = Q::bytes(a.plan.ntw);
    const cudaError_t e = prep_q(k_xiq<L, HALF>, sm);
    if (e != cudaSuccess) return e;
    k_xiq<L, HALF><<<grid, XQ_THREADS, sm, st>>>(a);
    return cudaGetLastError();
}

}  // namespace

bool xq_supported(int prec, int inverse, int L, int n, int mirror)
{
    return prec == PREC_FP32 && !mirror && (L == 256 || L == 512 || L == 1024) && n >= 1 && n <= L &&
           (!inverse || n <= L);
}

int xq_lines(int L) { return L >= 32 ? XQ_THREADS / (L / 32) : 0; }

size_t smem_lines_xq(int L, int ntw_entries)
{
    switch (L) {
    case 256: return Xq<256>::bytes(ntw_entries);
    case 512: return Xq<512>::bytes(ntw_entries);
    case 1024: return Xq<1024>::bytes(ntw_entries);
    default: return 0;
    }
}

cudaError_t launch_xfq(const XFwdArgs &a, cudaStream_t st)
{
    if (a.B != xq_lines(a.L) || !xq_supported(PREC_FP32, 0, a.L, a.n_in, a.mirror)) return cudaErrorInvalidConfiguration;
    const bool half = 2 * a.n_in == a.L;
    switch (a.L) {
    case 256: return half ? launch_xfq_t<256, true>(a, st) : launch_xfq_t<256, false>(a, st);
    case 512: return half ? launch_xfq_t<512, true>(a, st) : launch_xfq_t<512, false>(a, st);
    case 1024: return half ? launch_xfq_t<1024, true>(a, st) : launch_xfq_t<1024, false>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_xiq(const XInvArgs &a, cudaStream_t st)
{
    if (a.B != xq_lines(a.L) || !xq_supported(PREC_FP32, 1, a.L, a.n_out, 0)) return cudaErrorInvalidConfiguration;
    const bool half = 2 * a.n_out == a.L;
    switch (a.L) {
    case 256: return half ? launch_xiq_t<256, true>(a, st) : launch_xiq_t<256, false>(a, st);
    case 512: return half ? launch_xiq_t<512, true>(a, st) : launch_xiq_t<512, false>(a, st);
    case 1024: return half ? launch_xiq_t<1024, true>(a, st) : launch_xiq_t<1024, false>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace wide
}  // namespace ps
