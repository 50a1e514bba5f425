// Solve entry point that allocates nothing (ps_solve3d_device_noalloc).
//
// Who needs it: callers that must not call cudaMalloc/cudaFree once their
// run is under way -- a time-stepping flow code that solves the Poisson
// problem every step inside a device-memory budget it reserved up front (or
// that another framework's pool owns), where an allocation in the loop could
// fail late or stall every stream, since cudaMalloc and cudaFree may
// synchronise the device. ps_solve3d_device grows the handle's spectral work
// buffers on first use; this variant instead works in fixed memory compiled
// into the library:
//
//   g_noalloc_scratch   32 MiB of spectra (complex FP64)
//   g_noalloc_twiddles   1 MiB of FFT twiddle factors, recomputed on the
//                        device in the call's stream by every call
//
// Both are file-scope __device__ arrays, so every GPU that loads this part of
// the library holds them until the process exits. The kernel octant comes
// from the handle (ps_setup3d built it), so a call needs only a set-up
// handle, device inputs and device outputs.
//
// Limits and rules:
//   * Transforms are FP64, whatever PS_OPT_PRECISION says, with the plans
//     the handle's own FP64 solve uses (Bluestein for lengths with a prime
//     factor of 17 or more).
//   * The problem must fit: (components in use) x Nz x Py x (Px/2+1) x 16
//     bytes <= 32 MiB (e.g. a 64^3 unbounded 3-component curl solve needs
//     25.6 MiB). Larger problems fail with PS_ERR_UNSUPPORTED and say why.
//   * The first call on a device resolves the arrays' device addresses
//     (cudaGetSymbolAddress, once per device, with that device current) and
//     may load this part of the library's device code; make that first call
//     before any stream capture.
//   * All calls in the process share the two arrays. Calls whose GPU work
//     overlaps -- different streams, different handles, different host
//     threads -- race on them; serialise them on one stream. Nothing in the
//     scratch needs to start at zero: every element a call reads was written
//     earlier in the same call.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <mutex>
#include <string>

#include "poisson_solver_gb300.h"
#include "ps_solver.hpp"
#include "ps_types.hpp"

namespace ps {

namespace {

constexpr size_t kScratchBytes = size_t(32) << 20;
constexpr size_t kTwiddleBytes = size_t(1) << 20;
constexpr size_t kScratchElems = kScratchBytes / sizeof(double2);
constexpr size_t kTwiddleElems = kTwiddleBytes / sizeof(double2);
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double2 g_noalloc_scratch[kScratchElems];
static __device__ __align__(256) double2 g_noalloc_twiddles[kTwiddleElems];

// Device addresses of the two arrays, resolved once per device.
struct Symbols {
    double2 *scratch = nullptr;
    double2 *twiddles = nullptr;
};
std::mutex g_mu;
Symbols g_symbols[kMaxDevices];

Symbols device_symbols()
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) throw Error(PS_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) throw Error(PS_ERR_UNSUPPORTED, "device ordinal above 63");
    Symbols &s = g_symbols[dev];
    if (!s.scratch) {
        void *p = nullptr, *q = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            throw Error(PS_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        e = cudaGetSymbolAddress(&q, g_noalloc_twiddles);
        if (e != cudaSuccess)
            throw Error(PS_ERR_CUDA, std::string("cudaGetSymbolAddress(twiddles): ") + cudaGetErrorString(e));
        s.twiddles = static_cast<double2 *>(q);
        s.scratch = static_cast<double2 *>(p);
    }
    return s;
}

// The twiddle tables are computed on the device, in the call's stream, as
// runs ("segments") of one of four kinds:
//   SEG_STAGE  e^{-2 pi i j r / (m R)} for j < m, r = 1..R-1 (a stage's twiddles)
//   SEG_ROOTS  e^{-2 pi i q / R} for q < R (a direct prime-radix stage)
//   SEG_CHIRP  c[k] = e^{-i pi k^2 / Lt} for k < Lt (Bluestein chirp)
//   SEG_KSPEC  K[k] = DFT_M(conj c wrapped onto M points)[k] / M for k < M
enum SegKind { SEG_STAGE = 0, SEG_ROOTS = 1, SEG_CHIRP = 2, SEG_KSPEC = 3 };
struct Seg {
    int kind;
    int off;    // first table entry
    int count;  // entries
    int a, b;   // STAGE: m, R; ROOTS: -, R; CHIRP: Lt, -; KSPEC: Lt, M
};
constexpr int kMaxSegs = 3 * (2 * MAX_STAGES + 2);
struct FillArgs {
    Seg seg[kMaxSegs];
    int nseg;
    double2 *table;
};

// e^{-2 pi i e / N} from the exactly reduced fraction e / N (angle in (-pi, pi]).
__device__ double2 na_root(long long e, long long N)
{
    e %= N;
    if (e < 0) e += N;
    if (2 * e > N) e -= N;
    double sn, cs;
    sincospi(2.0 * (double)e / (double)N, &sn, &cs);
    return make_double2(cs, -sn);
}

__global__ void k_noalloc_twiddles(const __grid_constant__ FillArgs a)
{
    const Seg sg = a.seg[blockIdx.y];
    double2 *out = a.table + sg.off;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < sg.count; i += gridDim.x * blockDim.x) {
        double2 v;
        if (sg.kind == SEG_STAGE) {
            const int j = i / (sg.b - 1), r = i % (sg.b - 1) + 1;
            v = na_root((long long)j * r, (long long)sg.a * sg.b);
        } else if (sg.kind == SEG_ROOTS) {
            v = na_root(i, sg.b);
        } else if (sg.kind == SEG_CHIRP) {
            const long long Lt = sg.a;
            v = na_root(((long long)i * i) % (2 * Lt), 2 * Lt);
        } else {
            // conj c[n] sits at n and (n > 0) at M - n; their two DFT terms
            // add to 2 cos(2 pi n k / M) conj c[n].
            const long long Lt = sg.a, M = sg.b;
            double re = 0.0, im = 0.0;
            for (long long n = 0; n < Lt; ++n) {
                const double2 c = na_root(-((n * n) % (2 * Lt)), 2 * Lt);  // conj c[n]
                const double w = n == 0 ? 1.0 : 2.0 * na_root((n * i) % M, M).x;
                re += w * c.x;
                im += w * c.y;
            }
            v = make_double2(re / (double)M, im / (double)M);
        }
        out[i] = v;
    }
}

// Stage order of the FP64 plans (Solver::plan with radices up to 8): primes
// above 7 (direct DFT stages), 7s, 5s, 3s, 8s, then one 4 or 2.
void factor_fp64(int L, int rad[MAX_STAGES], int &nr)
{
    nr = 0;
    auto push = [&](int r) {
        if (nr == MAX_STAGES) throw Error(PS_ERR_UNSUPPORTED, "transform length has too many factors");
        rad[nr++] = r;
    };
    int x = L, p2 = 0;
    int big[MAX_STAGES], nbig = 0, odd[3] = {0, 0, 0};
    while (x > 1 && x % 2 == 0) { x /= 2; ++p2; }
    const int small_primes[3] = {3, 5, 7};
    for (int i = 0; i < 3; ++i)
        while (x % small_primes[i] == 0) { ++odd[i]; x /= small_primes[i]; }
    for (int p = 11; (long long)p * p <= x; p += 2)
        while (x % p == 0) {
            if (nbig == MAX_STAGES) throw Error(PS_ERR_UNSUPPORTED, "transform length has too many factors");
            big[nbig++] = p;
            x /= p;
        }
    if (x > 1) big[nbig++] = x;
    for (int i = 0; i < nbig; ++i) push(big[i]);
    for (int i = 2; i >= 0; --i)
        for (int k = 0; k < odd[i]; ++k) push(small_primes[i]);
    while (p2 >= 3) { push(8); p2 -= 3; }
    if (p2 == 2) push(4);
    if (p2 == 1) push(2);
}

int largest_prime(int x)
{
    int f = 1;
    for (int p = 2; (long long)p * p <= x; ++p)
        while (x % p == 0) {
            f = p;
            x /= p;
        }
    return x > 1 ? (x > f ? x : f) : f;
}

// FP64 plan of transform length Lt laid out in the fixed twiddle array: the
// plan Solver::plan builds for PREC_FP64 (same radix order, table layout and
// Bluestein switch for lengths above 16 with a prime factor of 17 or more),
// with the table entries described as segments for k_noalloc_twiddles
// instead of being computed on the host.
void describe_fp64_plan(int Lt, FftPlanDev &d, size_t &used, FillArgs &fill, const double2 *dev_table)
{
    d = FftPlanDev{};
    const bool blue = Lt > 16 && largest_prime(Lt) >= 17 && !getenv("PS_NO_BLUESTEIN");
    int L = Lt;
    if (blue) {
        L = 1;
        while (L < 2 * Lt - 1) L <<= 1;
    }
    d.L = L;
    d.blue = blue ? 1 : 0;
    d.lb = Lt;
    int rad[MAX_STAGES], nr = 0;
    if (L > 1) factor_fp64(L, rad, nr);

    const size_t base = used;
    auto segment = [&](int kind, int count, int a, int b) {
        if (count <= 0) return;
        if (used + (size_t)count > kTwiddleElems)
            throw Error(PS_ERR_UNSUPPORTED, "twiddle tables exceed the 1 MiB of the no-allocation solve");
        if (fill.nseg == kMaxSegs) throw Error(PS_ERR_UNSUPPORTED, "too many twiddle segments");
        fill.seg[fill.nseg++] = Seg{kind, (int)used, count, a, b};
        used += (size_t)count;
    };
    const int emax = e_max(PREC_FP64);
    int m = 1, tpl = 1;
    d.nstages = nr;
    for (int s = 0; s < nr; ++s) {
        const int R = rad[s];
        d.radix[s] = R;
        d.m[s] = m;
        d.lm[s] = (m & (m - 1)) == 0 ? __builtin_ctz((unsigned)m) : -1;
        d.tw[s] = (int)(used - base);
        segment(SEG_STAGE, m * (R - 1), m, R);
        const int nbf = L / R;
        const bool fixed = R == 2 || R == 3 || R == 4 || R == 5 || R == 7 || R == 8;
        if (fixed) {
            const int U = emax / R;
            tpl = tpl > (nbf + U - 1) / U ? tpl : (nbf + U - 1) / U;
            d.gw[s] = 0;
        } else {
            d.generic = 1;
            d.gw[s] = (int)(used - base);
            segment(SEG_ROOTS, R, 0, R);
            const int g = L < 64 ? L : 64;  // the direct DFT spreads a line's L outputs over its threads
            tpl = tpl > g ? tpl : g;
        }
        m *= R;
    }
    d.tpl = tpl;
    d.ntw = (int)(used - base);  // the part the kernels stage in shared memory
    if (blue) {
        d.chirp = (int)(used - base);
        segment(SEG_CHIRP, Lt, Lt, 0);
        d.kspec = (int)(used - base);
        segment(SEG_KSPEC, L, Lt, L);
    }
    if (tpl > MAX_THREADS) throw Error(PS_ERR_UNSUPPORTED, "transform length too large");
    d.table = dev_table + base;
}

template <typename F> int lines_per_cta(int tpl, F smem)
{
    const int limit = max_smem_per_block() - 1024;
    int B = 8;
    while (B > 1 && (B * tpl > MAX_THREADS || smem(B) > (size_t)limit)) B >>= 1;
    if (B * tpl > MAX_THREADS || smem(B) > (size_t)limit)
        throw Error(PS_ERR_UNSUPPORTED, "transform length too large for one CTA");
    return B;
}

#define PS_NA_CK(expr)                                                                                         \
    do {                                                                                                       \
        cudaError_t e_ = (expr);                                                                               \
        if (e_ != cudaSuccess) throw Error(PS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

// The five-pass FP64 solve of Solver::solve, with the spectra in
// g_noalloc_scratch and the twiddles in g_noalloc_twiddles.
int solve_noalloc(Solver &s, const double *const Bin[3], double *const Aout[3])
{
    if (!s.is_setup) throw Error(PS_ERR_STATE, "setup3d has not been called");
    if (s.dims != 3) throw Error(PS_ERR_STATE, "the no-allocation solve is 3D only");
    int in_mask = 0;
    for (int c = 0; c < 3; ++c)
        if (Bin[c]) in_mask |= 1 << c;
    if (!in_mask) throw Error(PS_ERR_STATE, "no right-hand side component given");
    const int out_mask = s.output_mask(in_mask);
    const int op = s.opt_grad ? OP_GRAD : s.opt_div ? OP_DIV : s.opt_curl ? OP_CURL : OP_NONE;
    int write_mask = 0;
    for (int c = 0; c < 3; ++c)
        if ((out_mask >> c & 1) && Aout[c]) write_mask |= 1 << c;

    const int *n = s.n, *P = s.P;
    const int Mx = s.Mx;
    const size_t slab = (size_t)n[2] * P[1] * Mx;
    int nslots = 0;
    for (int c = 0; c < 3; ++c)
        if ((in_mask | out_mask) >> c & 1) ++nslots;
    const size_t need = (size_t)nslots * slab * sizeof(double2);
    if (need > kScratchBytes)
        throw Error(PS_ERR_UNSUPPORTED, "the no-allocation solve holds " + std::to_string(kScratchBytes) +
                                            " bytes of scratch; this problem needs " + std::to_string(need));

    std::lock_guard<std::mutex> lock(g_mu);
    const Symbols sym = device_symbols();
    double2 *work[3] = {nullptr, nullptr, nullptr};
    for (int c = 0, k = 0; c < 3; ++c)
        if ((in_mask | out_mask) >> c & 1) work[c] = sym.scratch + (size_t)(k++) * slab;

    FftPlanDev px, py, pz;
    size_t used = 0;
    FillArgs fill{};
    fill.table = sym.twiddles;
    describe_fp64_plan(P[0], px, used, fill, sym.twiddles);
    describe_fp64_plan(P[1], py, used, fill, sym.twiddles);
    describe_fp64_plan(P[2], pz, used, fill, sym.twiddles);
    if (fill.nseg) {
        k_noalloc_twiddles<<<dim3(8, fill.nseg), 256, 0, s.stream>>>(fill);
        PS_NA_CK(cudaGetLastError());
    }
    const int prec = PREC_FP64;

    XFwdArgs xa{};
    for (int c = 0; c < 3; ++c)
        if (in_mask >> c & 1) {
            xa.in[xa.ncomp] = Bin[c];
            xa.out[xa.ncomp] = work[c];
            ++xa.ncomp;
        }
    xa.L = P[0];
    xa.n_in = n[0];
    xa.in_stride = n[0];
    xa.rows_y = n[1];
    xa.rows_z = n[2];
    xa.out_y = P[1];
    xa.Mx = Mx;
    xa.ld = Mx;  // the scratch spectra are unpadded
    xa.plan = px;
    xa.B = lines_per_cta(px.tpl, [&](int B) { return smem_x(prec, px, B); });
    PS_NA_CK(launch_xfwd(prec, xa, s.stream));

    ColArgs ya{};
    for (int c = 0; c < 3; ++c)
        if (in_mask >> c & 1) ya.data[ya.ncomp++] = work[c];
    ya.L = P[1];
    ya.n_in = n[1];
    ya.n_out = P[1];
    ya.Mx = Mx;
    ya.axis_stride = Mx;
    ya.outer_stride = (long long)P[1] * Mx;
    ya.plan = py;
    ya.B = lines_per_cta(py.tpl, [&](int B) { return smem_col(prec, py, B); });
    PS_NA_CK(launch_col(prec, 0, ya, n[2], s.stream));

    ZArgs za{};
    if (op == OP_GRAD) {
        if (in_mask == 1) {
            za.nin = 1;
            za.in[0] = work[0];
        } else {
            za.nin = 3;
            for (int d = 0; d < 3; ++d) za.in[d] = work[(in_mask >> d & 1) ? d : 0];
        }
        for (int d = 0; d < 3; ++d) za.out[za.nout++] = (write_mask >> d & 1) ? work[d] : nullptr;
    } else if (op == OP_DIV || op == OP_CURL) {
        za.nin = 3;
        for (int d = 0; d < 3; ++d) za.in[d] = work[d];
        za.nout = op == OP_DIV ? 1 : 3;
        for (int d = 0; d < za.nout; ++d) za.out[d] = (write_mask >> d & 1) ? work[d] : nullptr;
    } else {
        for (int c = 0; c < 3; ++c)
            if (in_mask >> c & 1) {
                za.in[za.nin] = work[c];
                za.out[za.nin] = (write_mask >> c & 1) ? work[c] : nullptr;
                ++za.nin;
            }
        za.nout = za.nin;
    }
    za.L = P[2];
    za.n_in = n[2];
    za.n_out = n[2];
    za.Mx = Mx;
    za.axis_stride = (long long)P[1] * Mx;
    za.row_stride = Mx;
    za.op = op;
    za.kern = s.kern64.p;
    za.oct_y = s.oy;
    za.Px = P[0];
    za.Py = P[1];
    za.Pz = P[2];
    za.kxc = 2.0 * M_PI / ((double)P[0] * s.dx[0]);
    za.kyc = 2.0 * M_PI / ((double)P[1] * s.dx[1]);
    za.kzc = 2.0 * M_PI / ((double)P[2] * s.dx[2]);
    za.plan = pz;
    const int nbuf = za.nin > za.nout ? za.nin : za.nout;
    za.B = lines_per_cta(pz.tpl, [&](int B) { return smem_z(prec, pz, B, nbuf); });
    PS_NA_CK(launch_z(prec, za, P[1], s.stream));

    if (write_mask) {
        ColArgs yi{};
        for (int c = 0; c < 3; ++c)
            if (write_mask >> c & 1) yi.data[yi.ncomp++] = work[c];
        yi.L = P[1];
        yi.n_in = P[1];
        yi.n_out = n[1];
        yi.Mx = Mx;
        yi.axis_stride = Mx;
        yi.outer_stride = (long long)P[1] * Mx;
        yi.plan = py;
        yi.B = ya.B;
        PS_NA_CK(launch_col(prec, 1, yi, n[2], s.stream));

        XInvArgs xi{};
        for (int c = 0; c < 3; ++c)
            if (write_mask >> c & 1) {
                xi.in[xi.ncomp] = work[c];
                xi.out[xi.ncomp] = Aout[c];
                ++xi.ncomp;
            }
        xi.L = P[0];
        xi.n_out = n[0];
        xi.Mx = Mx;
        xi.ld = Mx;
        xi.rows_y = n[1];
        xi.rows_z = n[2];
        xi.in_y = P[1];
        xi.out_stride = n[0];
        xi.plan = px;
        xi.B = xa.B;
        PS_NA_CK(launch_xinv(prec, xi, s.stream));
    }
    return write_mask;
}

}  // namespace ps
