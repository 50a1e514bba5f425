// Host orchestration of the 3D solve: transform plans, device buffers, the
// kernel build and the five-launch pipeline
//   x forward (R2C, zero-pad) -> y forward -> z (forward, kernel x operator,
//   inverse) -> y inverse -> x inverse (C2R, crop)
// that replaces the reference's pencil FFTs and MPI remaps (solve3d.cpp:8-635).
#include "ps_solver.hpp"

#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <mutex>
#include <sstream>
#include <vector>

#include "poisson_solver_gb300.h"

namespace ps {

#define PS_CK(expr)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (expr);                                                                      \
        if (e_ != cudaSuccess) throw Error(PS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

static constexpr long double PI_L = 3.141592653589793238462643383279502884L;

// ---------------------------------------------------------------------------
void DevBuf::ensure(size_t n)
{
    if (p && n <= bytes) return;
    release();
    if (n == 0) return;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
        p = nullptr;
        bytes = 0;
        cudaGetLastError();
        throw Error(PS_ERR_MEMORY, "device allocation of " + std::to_string(n) + " bytes failed: " +
                                       cudaGetErrorString(e));
    }
    bytes = n;
}

void DevBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

Solver::Solver() { PS_CK(cudaGetDevice(&device)); }

Solver::~Solver()
{
    for (auto *v : {&ev_pending, &ev_pool})
        for (auto &set : *v)
            for (cudaEvent_t e : set) cudaEventDestroy(e);
}

void Solver::drain_timing()
{
    for (auto &set : ev_pending) {
        PS_CK(cudaEventSynchronize(set[NPASS]));
        for (int i = 0; i < NPASS; ++i) {
            float ms = 0.f;
            PS_CK(cudaEventElapsedTime(&ms, set[i], set[i + 1]));
            pass_ms[i] += ms;
        }
        ++timed_solves;
        ev_pool.push_back(set);
    }
    ev_pending.clear();
}

// ---------------------------------------------------------------------------
// Transform plans. Stage order (which fft_lines relies on): primes above 7
// (direct DFT stages), 7s, 5s, 3s, 16s (FP32 only), 8s, then one 4 or 2.
static std::vector<int> factorize(int L, int max_radix)
{
    std::vector<int> big, small;
    int x = L;
    int p2 = 0;
    while (x % 2 == 0) { x /= 2; ++p2; }
    std::vector<int> odd;
    for (int p : {3, 5, 7})
        while (x % p == 0) { odd.push_back(p); x /= p; }
    for (int p = 11; (long long)p * p <= x; p += 2)
        while (x % p == 0) { big.push_back(p); x /= p; }
    if (x > 1) big.push_back(x);
    std::vector<int> r(big.begin(), big.end());
    for (int p : {7, 5, 3})
        for (int q : odd)
            if (q == p) r.push_back(p);
    if (max_radix >= 32)
        while (p2 >= 5) { r.push_back(32); p2 -= 5; }
    if (max_radix >= 16)
        while (p2 >= 4) { r.push_back(16); p2 -= 4; }
    while (p2 >= 3) { r.push_back(8); p2 -= 3; }
    if (p2 == 2) r.push_back(4);
    if (p2 == 1) r.push_back(2);
    return r;
}

static bool fixed_radix(int R)
{
    return R == 2 || R == 3 || R == 4 || R == 5 || R == 7 || R == 8 || R == 16 || R == 32;
}

// e^{-2 pi i e / N}, from the exactly reduced fraction e/N in extended precision
static std::complex<long double> root(long long e, long long N)
{
    e %= N;
    const long double a = 2.0L * PI_L * (long double)e / (long double)N;
    return {cosl(a), -sinl(a)};
}

static int largest_prime_factor(int x)
{
    int f = 1;
    for (int p = 2; (long long)p * p <= x; ++p)
        while (x % p == 0) {
            f = p;
            x /= p;
        }
    return x > 1 ? std::max(f, x) : f;
}

// In-place DFT (e^{-2 pi i nk / M}) of a power-of-two length in extended
// precision: the Bluestein kernel spectrum.
static void host_fft_pow2(std::vector<std::complex<long double>> &a)
{
    const size_t M = a.size();
    for (size_t i = 1, j = 0; i < M; ++i) {
        size_t bit = M >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= M; len <<= 1) {
        for (size_t i = 0; i < M; i += len)
            for (size_t k = 0; k < len / 2; ++k) {
                const std::complex<long double> w = root((long long)k, (long long)len);
                const std::complex<long double> u = a[i + k], v = a[i + k + len / 2] * w;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
            }
    }
}

// In-place DFT (e^{-2 pi i nk / M}) in extended precision, by recursive
// decimation in time over the smallest prime factor (O(M * sum of the prime
// factors)): the spectrum of a Bluestein kernel on a smooth convolution
// length, and the convolution spectrum of a Rader stage.
static void host_fft_smooth(std::vector<std::complex<long double>> &a)
{
    const size_t M = a.size();
    if (M <= 1) return;
    size_t R = 2;
    while (M % R != 0) ++R;
    const size_t m = M / R;
    std::vector<std::vector<std::complex<long double>>> sub(R, std::vector<std::complex<long double>>(m));
    for (size_t n = 0; n < m; ++n)
        for (size_t r = 0; r < R; ++r) sub[r][n] = a[n * R + r];
    for (auto &s : sub) host_fft_smooth(s);
    for (size_t k = 0; k < M; ++k) {
        std::complex<long double> acc = 0.0L;
        for (size_t r = 0; r < R; ++r) acc += sub[r][k % m] * root((long long)(r * k % M), (long long)M);
        a[k] = acc;
    }
}

// Lengths with a prime factor of at least this take Bluestein's algorithm
// (two FFTs of M >= 2L - 1 points) instead of a direct prime-radix stage
// (about R complex products an element).
constexpr int BLUESTEIN_MIN_PRIME = 17;

static int next_pow2(int n)
{
    int m = 1;
    while (m < n) m <<= 1;
    return m;
}

// least 2^a 3^b 5^c >= n
static int next_smooth(int n)
{
    for (int m = n;; ++m) {
        int x = m;
        for (int p : {2, 3, 5})
            while (x % p == 0) x /= p;
        if (x == 1) return m;
    }
}

static bool bluestein_length(int L)
{
    return L > 16 && largest_prime_factor(L) >= BLUESTEIN_MIN_PRIME && !getenv("PS_NO_BLUESTEIN");
}

// Threads a line of length Ls needs for the stages rs with emax register
// elements a thread: a fixed radix R takes emax / R butterflies a thread, a
// direct-DFT stage spreads the line's outputs over up to 64 threads.
static int stage_threads(const std::vector<int> &rs, int Ls, int emax)
{
    int tp = 1;
    for (int R : rs) tp = std::max(tp, fixed_radix(R) ? (Ls / R + emax / R - 1) / (emax / R) : std::min(Ls, 64));
    return tp;
}

// Rader's algorithm applies to a Bluestein length L whose largest prime p
// divides it once, whose cofactor L / p and p - 1 have no prime factor above
// 13 (their stages are the fixed radices and the direct radix-11/13 stages),
// whose sub-transforms all run at once on at most 256 threads a line, and
// whose stage count (the Rader stage, the cofactor's stages and those of
// p - 1) fits the stage table.
static bool rader_length(int L, int max_radix, int emax)
{
    if (!bluestein_length(L)) return false;
    const int p = largest_prime_factor(L), c = L / p;
    if (c % p == 0 || largest_prime_factor(c) > 13 || largest_prime_factor(p - 1) > 13) return false;
    const std::vector<int> sub = factorize(p - 1, max_radix);
    if (stage_threads(sub, p - 1, emax) * c > 256) return false;
    return 1 + (int)factorize(c, max_radix).size() + (int)sub.size() <= MAX_STAGES;
}

// smallest primitive root of the prime p
static int primitive_root(int p)
{
    std::vector<int> f;
    for (int x = p - 1, q = 2; x > 1; ++q)
        if (x % q == 0) {
            f.push_back(q);
            while (x % q == 0) x /= q;
        }
    for (int g = 2;; ++g) {
        bool ok = true;
        for (int q : f) {
            long long r = 1, b = g;
            for (int e = (p - 1) / q; e > 0; e >>= 1, b = b * b % p)
                if (e & 1) r = r * b % p;
            if (r == 1) ok = false;
        }
        if (ok) return g;
    }
}

const Plan &Solver::plan(int L, int prec, int emax, int pv)
{
    if (emax <= 0) emax = e_max(prec);
    if (prec != PREC_FP32) pv = 0;  // FP64 results do not depend on tuning
    const int Lt = L;  // the transform length
    if (emax < 16) pv &= ~PV_HALF_RADIX;
    const int rmax = (pv & PV_HALF_RADIX) ? emax / 2 : emax;  // the radix cap of the stages
    if (!rader_length(Lt, rmax, emax)) pv &= ~PV_RADER;
    const bool rader = (pv & PV_RADER) != 0;
    const bool blue = bluestein_length(Lt) && !rader;
    if (!blue) pv &= ~PV_SMOOTH_M;
    const auto key = std::make_tuple(L, prec, emax, pv);
    auto it = plans.find(key);
    if (it != plans.end()) return *it->second;
    auto pl = std::make_unique<Plan>();
    FftPlanDev &d = pl->dev;
    if (blue) {
        L = next_pow2(2 * Lt - 1);
        if (pv & PV_SMOOTH_M) L = std::min(L, next_smooth(2 * Lt - 1));
    }
    d.L = L;
    d.blue = blue ? 1 : 0;
    d.lb = Lt;
    const int rp = rader ? largest_prime_factor(Lt) : 0;  // the Rader stage's prime
    std::vector<int> rad = L > 1 ? factorize(rader ? L / rp : L, rmax) : std::vector<int>{};
    if (rader) rad.insert(rad.begin(), rp);
    if ((int)rad.size() > MAX_STAGES) throw Error(PS_ERR_UNSUPPORTED, "transform length has too many factors");
    d.nstages = (int)rad.size();
    std::vector<std::complex<long double>> tab;
    // stages s0.. of a transform of length Ls from table slot `slot`: radices,
    // sub-transform sizes, twiddles (the table entries) and the threads a line
    // they need; a Rader stage (slot 0 of a Rader plan) has no table entries
    auto add_stages = [&](const std::vector<int> &rs, int Ls, int slot, bool skip_first) {
        int m = 1, tp = 1;
        for (size_t i = 0; i < rs.size(); ++i, ++slot) {
            const int R = rs[i];
            d.radix[slot] = R;
            d.m[slot] = m;
            d.lm[slot] = (m & (m - 1)) == 0 ? __builtin_ctz((unsigned)m) : -1;
            d.tw[slot] = (int)tab.size();
            d.gw[slot] = 0;
            if (!(skip_first && i == 0)) {
                for (int j = 0; j < m; ++j)
                    for (int r = 1; r < R; ++r) tab.push_back(root((long long)j * r, (long long)m * R));
                const int nbf = Ls / R;
                if (fixed_radix(R)) {
                    const int U = emax / R;
                    tp = std::max(tp, (nbf + U - 1) / U);
                } else {
                    d.generic = 1;
                    d.gw[slot] = (int)tab.size();
                    for (int q = 0; q < R; ++q) tab.push_back(root(q, R));
                    // the direct DFT spreads a line's L outputs over its threads
                    tp = std::max(tp, std::min(Ls, 64));
                }
            }
            m *= R;
        }
        return tp;
    };
    int tpl = add_stages(rad, L, 0, rader);
    if (rader) {
        // sub-transforms of p - 1 points in the stage slots after the plan's
        const std::vector<int> sub = factorize(rp - 1, rmax);
        d.rader = 1;
        d.generic = 1;  // the scratch line stages the gather and the outputs
        d.rq = rp - 1;
        d.rs0 = d.nstages;
        d.rns = (int)sub.size();
        d.rtpl = add_stages(sub, rp - 1, d.rs0, false);
        // every sub-line at once (rader_length keeps this within 256 threads);
        // the DC terms of the sub-transforms are held by line threads 0 .. L / p - 1
        const int nbf = L / rp;
        tpl = std::max({tpl, d.rtpl * nbf, nbf});
        d.rinv_p = (float)(1.0 / rp);
        d.rinv_q = (float)(1.0 / (rp - 1));
    }
    d.tpl = tpl;
    d.ntw = (int)tab.size();  // the part copied to shared memory
    std::vector<int> itab;
    if (rader) {
        // the convolution spectra FFT(beta) / (p - 1), beta[m] = w^(g^m),
        // forward (w = e^{-2 pi i / p}) then inverse (its conjugate), and the
        // index tables: g^-j mod p, then log_g k at k - 1
        const int p = rp, q1 = p - 1, g = primitive_root(p);
        std::vector<long long> gp(q1);
        gp[0] = 1;
        for (int j = 1; j < q1; ++j) gp[j] = gp[j - 1] * g % p;
        for (int inv = 0; inv < 2; ++inv) {
            std::vector<std::complex<long double>> bt(q1);
            for (int j = 0; j < q1; ++j) bt[j] = inv ? std::conj(root(gp[j], p)) : root(gp[j], p);
            host_fft_smooth(bt);
            if (inv == 0) d.rbh = (int)tab.size();
            for (int j = 0; j < q1; ++j) tab.push_back(bt[j] / (long double)q1);
        }
        itab.resize(2 * q1);
        for (int j = 0; j < q1; ++j) itab[j] = (int)gp[(q1 - j) % q1];  // g^-j
        for (int q = 0; q < q1; ++q) itab[q1 + gp[q] - 1] = q;          // log_g (g^q)
    }
    if (blue) {
        // chirp c[n] = e^{-i pi n^2 / Lt} and the spectrum of its conjugate
        // wrapped onto M = L points, scaled by 1/M; staged in shared memory
        // with the twiddles when the two take at most 16 KB (the kernels read
        // each entry once a line), else read through the cache
        d.chirp = (int)tab.size();
        for (long long k = 0; k < Lt; ++k) tab.push_back(root((k * k) % (2LL * Lt), 2LL * Lt));
        std::vector<std::complex<long double>> b(L, {0.0L, 0.0L});
        for (int k = 0; k < Lt; ++k) {
            const std::complex<long double> cc = std::conj(tab[d.chirp + k]);
            b[k] = cc;
            if (k > 0) b[L - k] = cc;
        }
        if ((L & (L - 1)) == 0) host_fft_pow2(b);
        else host_fft_smooth(b);
        d.kspec = (int)tab.size();
        for (int k = 0; k < L; ++k) tab.push_back(b[k] / (long double)L);
        const size_t elem = prec == PREC_FP32 ? 8 : 16;
        if ((size_t)(Lt + L) * elem <= 16384) {
            d.ntw = (int)tab.size();
            d.bsh = 1;
        }
        // the kernels' compile-time stage sequence of a power-of-two M (64 ..
        // 1024): radix-emax stages, then one stage of the remaining power of
        // two, M / emax threads a line
        bool ct = (L & (L - 1)) == 0 && L >= 64 && L <= 1024 && d.tpl == L / emax;
        for (int s = 0, lg = __builtin_ctz((unsigned)L), le = __builtin_ctz((unsigned)emax); ct && s < d.nstages; ++s)
            ct = d.radix[s] == (s < lg / le ? emax : 1 << (lg % le)) && d.nstages == lg / le + (lg % le ? 1 : 0);
        if (ct) d.ctm = L;
    }
    if (tpl > MAX_THREADS) throw Error(PS_ERR_UNSUPPORTED, "transform length " + std::to_string(Lt) + " too large");
    if (!tab.empty()) {
        if (prec == PREC_FP64) {
            std::vector<double2> h(tab.size());
            for (size_t i = 0; i < tab.size(); ++i) h[i] = make_double2((double)tab[i].real(), (double)tab[i].imag());
            pl->table.ensure(h.size() * sizeof(double2));
            PS_CK(cudaMemcpy(pl->table.p, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice));
        } else if (prec == PREC_DF64) {
            // (re hi, re lo, im hi, im lo), each part rounded from the extended-precision value
            std::vector<float4> h(tab.size());
            auto split = [](long double v, float &hi, float &lo) {
                hi = (float)v;
                lo = (float)(v - (long double)hi);
            };
            for (size_t i = 0; i < tab.size(); ++i) {
                split(tab[i].real(), h[i].x, h[i].y);
                split(tab[i].imag(), h[i].z, h[i].w);
            }
            pl->table.ensure(h.size() * sizeof(float4));
            PS_CK(cudaMemcpy(pl->table.p, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice));
        } else {
            std::vector<float2> h(tab.size());
            for (size_t i = 0; i < tab.size(); ++i) h[i] = make_float2((float)tab[i].real(), (float)tab[i].imag());
            pl->table.ensure(h.size() * sizeof(float2));
            PS_CK(cudaMemcpy(pl->table.p, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice));
        }
    }
    d.table = pl->table.p;
    if (!itab.empty()) {
        pl->itable.ensure(itab.size() * sizeof(int));
        PS_CK(cudaMemcpy(pl->itable.p, itab.data(), itab.size() * sizeof(int), cudaMemcpyHostToDevice));
        d.itab = static_cast<const int *>(pl->itable.p);
    }
    Plan &ref = *pl;
    plans[key] = std::move(pl);
    return ref;
}

// Lines per CTA: the 128-byte row default (or the power of two named by the
// environment variable `env`, e.g. PS_LINES_Z=4), halved until threads and
// shared memory fit.
static int pick_lines(int prec, int tpl, const std::function<size_t(int)> &smem, const char *env = nullptr,
                      int pref = 0, int max_threads = MAX_THREADS)
{
    static const int limit = max_smem_per_block() - 1024;  // room for the static stage table
    int B = pref > 0 ? pref : (prec == PREC_FP32 ? 16 : 8);
    if (const char *v = env ? getenv(env) : nullptr) {
        const int want = atoi(v);
        if (want >= 1 && want <= 64 && (want & (want - 1)) == 0) B = want;
    }
    while (B > 1 && (B * tpl > max_threads || smem(B) > (size_t)limit)) B >>= 1;
    if (B * tpl > max_threads || smem(B) > (size_t)limit)
        throw Error(PS_ERR_UNSUPPORTED, "transform length too large for one CTA");
    return B;
}

// ---------------------------------------------------------------------------
void Solver::check_setup() const
{
    if (!is_setup) throw Error(PS_ERR_STATE, "setup3d has not been called");
}

void Solver::setup3d(const int ncell[3], const int bcs[3], const double dxs[3], int reg_order)
{
    for (int d = 0; d < 3; ++d) {
        if (ncell[d] < 1) throw Error(PS_ERR_ARGUMENT, "ncell must be positive");
        if (!(dxs[d] > 0.0) || !std::isfinite(dxs[d])) throw Error(PS_ERR_ARGUMENT, "dx must be positive and finite");
        if (bcs[d] != 0 && bcs[d] != 1) throw Error(PS_ERR_BOUNDARY, "boundary condition must be 0 (unbounded) or 1 (periodic)");
    }
    if (reg_order < 0) throw Error(PS_ERR_ARGUMENT, "reg_order must be >= 0");
    const int b0 = bcs[0], b1 = bcs[1], b2 = bcs[2];
    const bool ok = (b0 == 0 && b1 == 0 && b2 == 0) || (b0 == 1 && b1 == 1 && b2 == 0) ||
                    (b0 == 0 && b1 == 0 && b2 == 1) || (b0 == 1 && b1 == 1 && b2 == 1);
    if (!ok) {
        // the reference's three diagnostics (greens3d.cpp:522-541)
        const int sum = b0 + b1 + b2;
        if (sum == 1)
            throw Error(PS_ERR_BOUNDARY, "for unbounded-unbounded-periodic domains the z-direction must be the periodic direction");
        if (sum == 2)
            throw Error(PS_ERR_BOUNDARY, "for unbounded-periodic-periodic domains the z-direction must be the unbounded direction");
        throw Error(PS_ERR_BOUNDARY, "boundary condition configuration unknown");
    }
    for (int d = 0; d < 3; ++d) {
        const long long p = (bcs[d] == 0 ? 2LL : 1LL) * ncell[d];
        if (p > 8192) throw Error(PS_ERR_UNSUPPORTED, "padded transform length above 8192");
    }
    is_setup = false;
    dims = 3;
    for (int d = 0; d < 3; ++d) {
        n[d] = ncell[d];
        bc[d] = bcs[d];
        dx[d] = dxs[d];
        P[d] = (bcs[d] == 0 ? 2 : 1) * ncell[d];
    }
    reg = reg_order;
    finish_setup();
}

// setup2d (setup2d.cpp:8-71, greens2d.cpp:9-443): every (x, y) boundary
// combination. The problem is held as one periodic z-plane: n[2] = P[2] = 1
// (kz = 0 only) and dx[2] = min(dx, dy), so the filter width h = max(dx, dy)
// as greens2d.cpp:55 takes it.
void Solver::setup2d(const int ncell[2], const int bcs[2], const double dxs[2], int reg_order)
{
    for (int d = 0; d < 2; ++d) {
        if (ncell[d] < 1) throw Error(PS_ERR_ARGUMENT, "ncell must be positive");
        if (!(dxs[d] > 0.0) || !std::isfinite(dxs[d])) throw Error(PS_ERR_ARGUMENT, "dx must be positive and finite");
        if (bcs[d] != 0 && bcs[d] != 1) throw Error(PS_ERR_BOUNDARY, "boundary condition must be 0 (unbounded) or 1 (periodic)");
        if ((bcs[d] == 0 ? 2LL : 1LL) * ncell[d] > 8192) throw Error(PS_ERR_UNSUPPORTED, "padded transform length above 8192");
    }
    if (reg_order < 0) throw Error(PS_ERR_ARGUMENT, "reg_order must be >= 0");
    is_setup = false;
    dims = 2;
    for (int d = 0; d < 2; ++d) {
        n[d] = ncell[d];
        bc[d] = bcs[d];
        dx[d] = dxs[d];
        P[d] = (bcs[d] == 0 ? 2 : 1) * ncell[d];
    }
    n[2] = 1;
    bc[2] = 1;
    dx[2] = std::min(dxs[0], dxs[1]);
    P[2] = 1;
    reg = reg_order;
    finish_setup();
}

void Solver::finish_setup()
{
    Mx = P[0] / 2 + 1;
    ldx = (Mx + 1) & ~1;  // even: rows of the spectra are whole 16-byte units
    oy = P[1] / 2 + 1;
    oz = P[2] / 2 + 1;
    // z pitch of the fast-axis kernel copy: the fused pass runs along z (3D) or y (2D)
    kzp = ((dims == 2 ? oy : oz) + 3) & ~3;
    pushed = produced = rhs_ready = 0;
    kern32.release();
    kern_df.release();
    kernzf32.release();
    zeta64.release();
    zeta32.release();
    zeta_df.release();
    smooth64.release();
    smooth32.release();
    smooth_df.release();
    smooth_s = -1.0;
    stage.release();
    for (int c = 0; c < 3; ++c) {
        work[c].release();
        fb[c].release();
        fa[c].release();
        fr[c].release();
    }
    build_kernel();
    if (!status.p) {
        status.ensure(4 * sizeof(int));  // [0] error bits, [1] tile counter of the bulk-copy kernels
        PS_CK(cudaMemsetAsync(status.p, 0, 4 * sizeof(int), stream));
        PS_CK(cudaStreamSynchronize(stream));
    }
    is_setup = true;
}

void Solver::set_option(int option, int value)
{
    switch (option) {
    case PS_OPT_GRAD: opt_grad = value != 0; break;
    case PS_OPT_DIV: opt_div = value != 0; break;
    case PS_OPT_CURL: opt_curl = value != 0; break;
    case PS_OPT_REPROJECT: opt_reproject = value != 0; rhs_ready = 0; break;
    case PS_OPT_PASS_TIMING: opt_timing = value != 0; break;
    case PS_OPT_PRECISION:
        if (value != PS_PREC_FP64 && value != PS_PREC_FP32 && value != PS_PREC_DF64)
            throw Error(PS_ERR_ARGUMENT, "unknown precision");
        precision = value == PS_PREC_FP64 ? PREC_FP64 : value == PS_PREC_FP32 ? PREC_FP32 : PREC_DF64;
        rhs_ready = 0;
        break;
    default: throw Error(PS_ERR_ARGUMENT, "unknown option");
    }
}

void Solver::set_kernel(int family, double width)
{
    if (family != PS_KERNEL_SPECTRAL && family != PS_KERNEL_GAUSSIAN) throw Error(PS_ERR_ARGUMENT, "unknown kernel family");
    if (!(width >= 0.0) || !std::isfinite(width)) throw Error(PS_ERR_ARGUMENT, "kernel width must be finite and >= 0");
    kernel_family = family;
    gauss_width = width;
    if (is_setup) {
        is_setup = false;
        finish_setup();
    }
}

GaussFamily Solver::gauss_family() const
{
    GaussFamily g{0, 0.0};
    if (kernel_family != PS_KERNEL_GAUSSIAN) return g;
    const int r = (reg % 2 != 0) ? reg + 1 : reg;
    g.gm = std::max(1, r / 2);
    g.gs = gauss_width > 0.0 ? gauss_width : 2.0 * std::max(std::max(dx[0], dx[1]), dx[2]);
    return g;
}

int Solver::get_option(int option) const
{
    switch (option) {
    case PS_OPT_GRAD: return opt_grad;
    case PS_OPT_DIV: return opt_div;
    case PS_OPT_CURL: return opt_curl;
    case PS_OPT_REPROJECT: return opt_reproject;
    case PS_OPT_PRECISION:
        return precision == PREC_FP64 ? PS_PREC_FP64 : precision == PREC_FP32 ? PS_PREC_FP32 : PS_PREC_DF64;
    case PS_OPT_PASS_TIMING: return opt_timing;
    default: throw Error(PS_ERR_ARGUMENT, "unknown option");
    }
}

// ---------------------------------------------------------------------------
// Kernel build (greens3d.cpp:9-547), FP64 on the GPU.
void Solver::build_kernel()
{
    const int prec = PREC_FP64;
    const size_t nk = (size_t)Mx * oy * oz;
    kern64.ensure(nk * sizeof(double));
    if (const Solver *k = kernel_from) {
        bool same = k->is_setup && k->kern64.p && k->dims == dims && k->reg == reg &&
                    k->kernel_family == kernel_family && k->gauss_width == gauss_width;
        for (int d = 0; d < 3 && same; ++d) same = k->P[d] == P[d] && k->bc[d] == bc[d] && k->dx[d] == dx[d];
        if (same) {
            PS_CK(cudaMemcpyAsync(kern64.p, k->kern64.p, nk * sizeof(double), cudaMemcpyDeviceToDevice, stream));
            PS_CK(cudaStreamSynchronize(stream));
            return;
        }
    }
    ++kernel_builds;
    KernelFillArgs fa{};
    fa.kern = (double *)kern64.p;
    fa.Mx = Mx;
    fa.oy = oy;
    fa.oz = oz;
    for (int d = 0; d < 3; ++d) {
        fa.P[d] = P[d];
        fa.dx[d] = dx[d];
    }
    fa.reg = reg;
    fa.norm = (double)P[0] * (double)P[1] * (double)P[2];
    fa.gauss = gauss_family();
    const int b0 = bc[0], b1 = bc[1], b2 = bc[2];
    if (dims == 3)
        fa.kind = (b0 == 0 && b1 == 0 && b2 == 0) ? 0 : (b0 == 1 && b1 == 1 && b2 == 0) ? 1 : (b2 == 1 && b0 == 0) ? 2 : 3;
    else  // 2D on one kz = 0 plane: unbounded = the 2D kernel plane, periodic, or one mixed line
        fa.kind = (b0 == 0 && b1 == 0) ? 2 : (b0 == 1 && b1 == 1) ? 3 : (b0 == 1) ? 4 : 5;

    DevBuf oct, spec, line;
    const int ox = P[0] / 2 + 1;
    const Plan &px = plan(P[0], prec);
    const Plan &py = plan(P[1], prec);
    if (fa.kind == 0 || fa.kind == 2) {
        const bool three = fa.kind == 0;
        const int pz = three ? P[2] : 1;
        const int ozs = three ? oz : 1;
        oct.ensure((size_t)ox * oy * ozs * sizeof(double));
        if (three) {
            const int oext[3] = {ox, oy, oz};
            PS_CK(launch_sample_unbounded3d((double *)oct.p, oext, P, dx, fa.gauss, stream));
        } else {
            const int oext[2] = {ox, oy}, P2[2] = {P[0], P[1]};
            const double dx2[2] = {dx[0], dx[1]};
            PS_CK(launch_sample_unbounded2d((double *)oct.p, oext, P2, dx2, fa.gauss, stream));
        }
        spec.ensure((size_t)pz * P[1] * Mx * sizeof(double2));
        XFwdArgs xa{};
        xa.in[0] = (const double *)oct.p;
        xa.out[0] = spec.p;
        xa.ncomp = 1;
        xa.L = P[0];
        xa.n_in = P[0];
        xa.in_stride = 0;
        xa.rows_y = P[1];
        xa.rows_z = pz;
        xa.out_y = P[1];
        xa.Mx = Mx;
        xa.ld = Mx;  // the kernel-build spectrum is unpadded
        xa.mirror = 1;
        xa.oct_x = ox;
        xa.oct_y = oy;
        xa.Py = P[1];
        xa.Pz = pz;
        xa.plan = px.dev;
        xa.B = pick_lines(prec, px.dev.tpl, [&](int B) { return smem_x(prec, px.dev, B); });
        PS_CK(launch_xfwd(prec, xa, stream));
        ColArgs ya{};
        ya.data[0] = spec.p;
        ya.ncomp = 1;
        ya.L = P[1];
        ya.n_in = P[1];
        ya.n_out = oy;
        ya.Mx = Mx;
        ya.axis_stride = Mx;
        ya.outer_stride = (long long)P[1] * Mx;
        ya.plan = py.dev;
        ya.B = pick_lines(prec, py.dev.tpl, [&](int B) { return smem_col(prec, py.dev, B); });
        PS_CK(launch_col(prec, 0, ya, pz, stream));
        if (three) {
            const Plan &pzp = plan(P[2], prec, e_max_z(prec));
            ZArgs za{};
            za.in[0] = spec.p;
            za.out[0] = spec.p;
            za.nin = za.nout = 1;
            za.L = P[2];
            za.n_in = P[2];
            za.n_out = oz;
            za.Mx = Mx;
            za.axis_stride = (long long)P[1] * Mx;
            za.row_stride = Mx;
            za.op = OP_FORWARD;
            za.plan = pzp.dev;
            za.B = pick_lines(prec, pzp.dev.tpl, [&](int B) { return smem_z(prec, pzp.dev, B, 1); });
            PS_CK(launch_z(prec, za, oy, stream));
            fa.spec = (const double2 *)spec.p;
        } else {
            fa.plane = (const double2 *)spec.p;
        }
    } else if (fa.kind == 1 || fa.kind == 4 || fa.kind == 5) {
        // the 1D kernel along the unbounded axis: z (3D periodic-periodic-
        // unbounded), y (2D x-periodic) or x (2D y-periodic)
        const int u = fa.kind == 1 ? 2 : fa.kind == 4 ? 1 : 0;
        line.ensure((size_t)(P[u] / 2 + 1) * sizeof(double));
        PS_CK(launch_line_ppf((double *)line.p, P[u], dx[u], fa.gauss, stream));
        fa.line = (const double *)line.p;
    }
    PS_CK(launch_kernel_fill(fa, stream));
    PS_CK(cudaStreamSynchronize(stream));
}

void Solver::ensure_kernel(int prec)
{
    if (prec == PREC_FP64) return;
    const size_t nk = (size_t)Mx * oy * oz;
    if (prec == PREC_DF64) {
        if (!kern_df.p) {
            kern_df.ensure(nk * sizeof(float2));
            PS_CK(launch_to_df((const double *)kern64.p, (float2 *)kern_df.p, nk, stream));
        }
        return;
    }
    if (!kern32.p) {
        kern32.ensure(nk * sizeof(float));
        PS_CK(launch_to_fp32((const double *)kern64.p, (float *)kern32.p, nk, stream));
    }
    // the fast-axis copy for the bulk-copy fused kernel, on the extents it
    // runs: z in 3D; y in 2D, where the kernel [oy][Mx] is read as [oy][1][Mx]
    const int fa_axis = dims == 2 ? 1 : 2;
    const int Lf = P[fa_axis];
    if (!kernzf32.p && bc[fa_axis] == 0 && (Lf == 256 || Lf == 512 || Lf == 1024)) {
        const int rows = dims == 2 ? 1 : oy, planes = dims == 2 ? oy : oz;
        kernzf32.ensure((size_t)Mx * rows * kzp * sizeof(float));
        PS_CK(launch_kernel_zfast((const double *)kern64.p, (float *)kernzf32.p, Mx, rows, planes, kzp, stream));
    }
}

void Solver::ensure_zeta(int prec)
{
    const size_t nk = (size_t)Mx * oy * oz;
    if (!zeta64.p) {
        zeta64.ensure(nk * sizeof(double));
        KernelFillArgs fa{};
        fa.zeta_out = (double *)zeta64.p;
        fa.Mx = Mx;
        fa.oy = oy;
        fa.oz = oz;
        for (int d = 0; d < 3; ++d) {
            fa.P[d] = P[d];
            fa.dx[d] = dx[d];
        }
        fa.reg = reg;
        fa.norm = (double)P[0] * (double)P[1] * (double)P[2];
        fa.gauss = gauss_family();
        PS_CK(launch_kernel_fill(fa, stream));
    }
    if (prec == PREC_FP32 && !zeta32.p) {
        zeta32.ensure(nk * sizeof(float));
        PS_CK(launch_to_fp32((const double *)zeta64.p, (float *)zeta32.p, nk, stream));
    }
    if (prec == PREC_DF64 && !zeta_df.p) {
        zeta_df.ensure(nk * sizeof(float2));
        PS_CK(launch_to_df((const double *)zeta64.p, (float2 *)zeta_df.p, nk, stream));
    }
}

// ---------------------------------------------------------------------------
int Solver::output_mask(int in_mask) const
{
    if (dims == 2) {
        // solve2d.cpp:43-103: grad of X -> X, Y; div of X, Y -> X; curl of Z -> X, Y
        if (opt_grad) {
            if (!(in_mask & 1)) throw Error(PS_ERR_COMPONENTS, "rhs fields have not been pushed correctly for grad option");
            return 3;
        }
        if (opt_div) {
            if ((in_mask & 3) != 3) throw Error(PS_ERR_COMPONENTS, "rhs fields have not been pushed correctly for div option");
            return 1;
        }
        if (opt_curl) {
            if (!(in_mask & 4)) throw Error(PS_ERR_COMPONENTS, "rhs fields have not been pushed correctly for curl option");
            return 3;
        }
        return in_mask;
    }
    if (opt_grad) {
        if (!(in_mask & 1)) throw Error(PS_ERR_COMPONENTS, "rhs fields have not been pushed correctly for grad option");
        return 7;
    }
    if (opt_div) {
        if (in_mask != 7) throw Error(PS_ERR_COMPONENTS, "rhs fields have not been pushed correctly for div option");
        return 1;
    }
    if (opt_curl) {
        if (in_mask != 7) throw Error(PS_ERR_COMPONENTS, "rhs fields have not been pushed correctly for curl option");
        return 7;
    }
    return in_mask;
}

int Solver::prepare(const double *const Bin[3], double *const Aout[3], bool filter_only, PassArgs &pa)
{
    check_setup();
    int in_mask = 0;
    for (int c = 0; c < 3; ++c)
        if (Bin[c]) in_mask |= 1 << c;
    if (!in_mask) throw Error(PS_ERR_STATE, "no right-hand side component given");
    int op, out_mask;
    if (filter_only) {
        op = OP_FILTER;
        out_mask = in_mask;
        if (filter_source == 1 && !smooth64.p) throw Error(PS_ERR_STATE, "smoothing filter not built");
    } else {
        out_mask = output_mask(in_mask);
        op = opt_grad ? OP_GRAD : opt_div ? OP_DIV : opt_curl ? OP_CURL : OP_NONE;
    }
    int write_mask = 0;
    for (int c = 0; c < 3; ++c)
        if ((out_mask >> c & 1) && Aout[c]) write_mask |= 1 << c;

    const int prec = precision;
    const size_t csz = prec == PREC_FP32 ? sizeof(float2) : sizeof(double2);  // double-float complex: 16 bytes
    ensure_kernel(prec);
    if (op == OP_FILTER && filter_source == 0) ensure_zeta(prec);
    if (op == OP_FILTER && filter_source == 1 && prec == PREC_FP32 && !smooth32.p) {
        smooth32.ensure((size_t)Mx * oy * oz * sizeof(float));
        PS_CK(launch_to_fp32((const double *)smooth64.p, (float *)smooth32.p, (size_t)Mx * oy * oz, stream));
    }
    if (op == OP_FILTER && filter_source == 1 && prec == PREC_DF64 && !smooth_df.p) {
        smooth_df.ensure((size_t)Mx * oy * oz * sizeof(float2));
        PS_CK(launch_to_df((const double *)smooth64.p, (float2 *)smooth_df.p, (size_t)Mx * oy * oz, stream));
    }
    for (int c = 0; c < 3; ++c)
        if ((in_mask | out_mask) >> c & 1) work[c].ensure(work_elems() * csz);
    pa = PassArgs{};
    pa.write_mask = write_mask;

    // x forward over the pushed components
    XFwdArgs &xa = pa.x;
    for (int c = 0; c < 3; ++c)
        if (in_mask >> c & 1) {
            xa.in[xa.ncomp] = Bin[c];
            xa.out[xa.ncomp] = work[c].p;
            ++xa.ncomp;
        }
    xa.L = P[0];
    xa.n_in = n[0];
    xa.in_stride = n[0];
    xa.rows_y = n[1];
    xa.rows_z = n[2];
    xa.out_y = P[1];
    xa.Mx = Mx;
    xa.ld = ldx;

    // y forward (zero-padded from Ny to Py)
    ColArgs &ya = pa.y;
    for (int c = 0; c < 3; ++c)
        if (in_mask >> c & 1) ya.data[ya.ncomp++] = work[c].p;
    ya.L = P[1];
    ya.n_in = n[1];
    ya.n_out = P[1];
    ya.Mx = Mx;
    ya.axis_stride = ldx;
    ya.outer_stride = (long long)P[1] * ldx;

    // z: forward (zero-padded from Nz to Pz), spectral operation, inverse (cropped)
    ZArgs &za = pa.z;
    if (op == OP_GRAD) {
        if (in_mask == 1) {
            za.nin = 1;
            za.in[0] = work[0].p;
        } else {
            za.nin = 3;
            for (int d = 0; d < 3; ++d) za.in[d] = work[(in_mask >> d & 1) ? d : 0].p;
        }
        za.nout = 0;
        for (int d = 0; d < 3; ++d) za.out[za.nout++] = (write_mask >> d & 1) ? work[d].p : nullptr;
    } else if (op == OP_DIV || op == OP_CURL) {
        za.nin = 3;
        for (int d = 0; d < 3; ++d) za.in[d] = work[d].p;
        za.nout = op == OP_DIV ? 1 : 3;
        for (int d = 0; d < za.nout; ++d) za.out[d] = (write_mask >> d & 1) ? work[d].p : nullptr;
    } else {
        for (int c = 0; c < 3; ++c)
            if (in_mask >> c & 1) {
                za.in[za.nin] = work[c].p;
                za.out[za.nin] = (write_mask >> c & 1) ? work[c].p : nullptr;
                ++za.nin;
            }
        za.nout = za.nin;
    }
    za.L = P[2];
    za.n_in = n[2];
    za.n_out = n[2];
    za.Mx = Mx;
    za.axis_stride = (long long)P[1] * ldx;
    za.row_stride = ldx;
    za.op = op;
    za.reproject = op == OP_FILTER && filter_source == 0 && opt_reproject && in_mask == 7;
    za.kern = prec == PREC_FP64 ? kern64.p : prec == PREC_FP32 ? kern32.p : kern_df.p;
    za.zeta = nullptr;
    if (op == OP_FILTER)
        za.zeta = filter_source == 1 ? (prec == PREC_FP64 ? smooth64.p : prec == PREC_FP32 ? smooth32.p : smooth_df.p)
                                     : (prec == PREC_FP64 ? zeta64.p : prec == PREC_FP32 ? zeta32.p : zeta_df.p);
    za.oct_y = oy;
    za.kern_zf = prec == PREC_FP32 ? static_cast<const float *>(kernzf32.p) : nullptr;
    za.kzp = kzp;
    za.Px = P[0];
    za.Py = P[1];
    za.Pz = P[2];
    za.kxc = 2.0 * M_PI / ((double)P[0] * dx[0]);
    za.kyc = 2.0 * M_PI / ((double)P[1] * dx[1]);
    za.kzc = 2.0 * M_PI / ((double)P[2] * dx[2]);
    if (dims == 2) {
        // The fused pass runs along y over one row of x columns: its transform
        // axis ("z") is y, its row axis has one entry (ky = 0 there), and the
        // kernel [oy][Mx] is its [oz][1][Mx] octant. The 2D outputs
        // (solve2d.cpp:292-325) from the 3D operations with k = (kx, 0, ky):
        // grad X -> (X, -, Y); div (X, -, Y); curl of Z = (ky, -kx) K Z is the
        // gradient with kx negated, written (Y, -, X).
        za.L = P[1];
        za.n_in = n[1];
        za.n_out = n[1];
        za.axis_stride = ldx;
        za.row_stride = ldx;
        za.oct_y = 1;
        za.Py = 1;
        za.Pz = P[1];
        za.kyc = 0.0;
        za.kzc = 2.0 * M_PI / ((double)P[1] * dx[1]);
        za.reproject = 0;
        void *wX = (write_mask & 1) ? work[0].p : nullptr, *wY = (write_mask & 2) ? work[1].p : nullptr;
        if (op == OP_GRAD || op == OP_CURL) {
            const bool curl = op == OP_CURL;
            za.op = OP_GRAD;
            za.nin = 1;
            za.in[0] = work[curl ? 2 : 0].p;
            za.in[1] = za.in[2] = nullptr;
            za.nout = 3;
            za.out[0] = curl ? wY : wX;
            za.out[1] = nullptr;
            za.out[2] = curl ? wX : wY;
            if (curl) za.kxc = -za.kxc;
        } else if (op == OP_DIV) {
            za.nin = 3;
            za.in[0] = work[0].p;
            za.in[1] = work[0].p;  // weighted by ky = 0
            za.in[2] = work[1].p;
            za.nout = 1;
            za.out[0] = wX;
            za.out[1] = za.out[2] = nullptr;
        }
    }

    // y inverse (cropped to Ny) and x inverse (cropped to Nx) of the written outputs
    ColArgs &yi = pa.yi;
    for (int c = 0; c < 3; ++c)
        if (write_mask >> c & 1) yi.data[yi.ncomp++] = work[c].p;
    yi.L = P[1];
    yi.n_in = P[1];
    yi.n_out = n[1];
    yi.Mx = Mx;
    yi.axis_stride = ldx;
    yi.outer_stride = (long long)P[1] * ldx;

    XInvArgs &xi = pa.xi;
    for (int c = 0; c < 3; ++c)
        if (write_mask >> c & 1) {
            xi.in[xi.ncomp] = work[c].p;
            xi.out[xi.ncomp] = Aout[c];
            ++xi.ncomp;
        }
    xi.L = P[0];
    xi.n_out = n[0];
    xi.Mx = Mx;
    xi.ld = ldx;
    xi.rows_y = n[1];
    xi.rows_z = n[2];
    xi.in_y = P[1];
    xi.out_stride = n[0];
    return write_mask;
}

// ---------------------------------------------------------------------------
// Kernel family and lines per CTA of each pass.
//
// Families: 'r' run-time kernels (any length, FP64 and FP32), 'p' length-
// specialised FP32 kernels (powers of two 64..2048), 'w' wide FP32 kernels
// (256..2048; for z the shared-memory fused kernel), 't' the fused z kernel
// with tensor-memory staging (z only), 'q' a warp per line or column group
// (x and y: L = 256..1024; z: unbounded axes of 256..1024 points; y and z
// fed by tiled bulk copies), 'c' the fused z kernel with its DFT stages on
// the tensor cores (unbounded z of 1024 points; only when PS_KERNELS_Z=tc).
// Defaults, measured at 512^3 (FP32 curl): the 'q' kernels where they apply
// (x: a warp per line; y, z: bulk copies), else x forward p2 with 2 lines a
// CTA (2.3 against 3.4 ms for wide), x inverse p2 with 4, y wide with 8 and
// z tensor-memory with 8.
// PS_KERNELS, PS_KERNELS_X/_Y/_Z (= tma, tc, tmem, wide, p2 or runtime),
// PS_LINES_X/_XI/_Y/_Z and PS_Z_EM override the defaults; ps_autotune
// replaces them for one configuration.

static int axis_of(int pass) { return pass == 0 || pass == 4 ? 0 : pass == 2 ? 2 : 1; }

int Solver::pass_len(int pass) const { return dims == 2 && pass == 2 ? P[1] : P[axis_of(pass)]; }

bool Solver::family_ok(int pass, char fam, const PassArgs &pa) const
{
    const int prec = precision, L = pass_len(pass), op = pa.z.op;
    switch (fam) {
    case 'r': return true;
    case 'p': return p2::supported(prec, L) && (pass != 2 || p2::supports_op(op));
    case 'w': return wide::supported(prec, L) && (pass != 2 || p2::supports_op(op));
    case 't': return pass == 2 && wide::zt_supported(prec, L, op, pa.z.nin, pa.z.nout);
    case 'q':
        if (pass == 0) return wide::xq_supported(prec, 0, L, pa.x.n_in, pa.x.mirror);
        if (pass == 4) return wide::xq_supported(prec, 1, L, pa.xi.n_out, 0);
        if (pass == 1 || pass == 3) {
            const ColArgs &c = pass == 1 ? pa.y : pa.yi;
            return wide::yq_supported(prec, pass == 3, L, c.n_in, c.n_out);
        }
        return pass == 2 && pa.z.kern_zf && wide::zq_supported(prec, L, op, pa.z.nin, pa.z.nout, pa.z.n_in, pa.z.n_out);
    case 'c':
        return pass == 2 && dims == 3 && pa.z.kern_zf &&
               tc::ztc_supported(prec, L, op, pa.z.nin, pa.z.nout, pa.z.n_in, pa.z.n_out);
    default: return false;
    }
}

int Solver::family_emax(int pass, char fam) const
{
    if (fam == 'w' || fam == 't' || fam == 'q' || fam == 'c') return 32;
    if (pass == 2) {
        if (fam == 'p') {
            const char *v = getenv("PS_Z_EM");  // 16 measured faster than 8 (13.4 vs 15.4 ms at 512^3)
            return v && atoi(v) == 8 ? 8 : 16;
        }
        return e_max_z(precision);
    }
    return e_max(precision);
}

// Shared memory of a CTA of B lines and the largest B the family allows.
size_t Solver::pass_smem(int pass, char fam, int B, const PassArgs &pa, const Plan &pl) const
{
    const int prec = precision, L = pl.dev.L, ntw = pl.dev.ntw;
    const int nbuf = std::max(pa.z.nin, pa.z.nout);
    if (pass == 2) {
        if (fam == 't') return wide::smem_lines_zt(L, B, ntw);
        if (fam == 'q') return wide::smem_lines_zq(L, ntw);
        if (fam == 'c') return tc::smem_ztc();
        if (fam == 'w') return wide::smem_lines(L, B, nbuf, ntw, true);
        if (fam == 'p') return p2::smem_lines(prec, L, B, nbuf, ntw);
        return smem_z(prec, pl.dev, B, nbuf);
    }
    const bool x = pass == 0 || pass == 4;
    if (fam == 'q') {
        if (x) return wide::smem_lines_xq(L, ntw);
        const ColArgs &c = pass == 1 ? pa.y : pa.yi;
        return wide::smem_lines_yq(pass == 3, L, c.n_in, c.n_out, ntw);
    }
    if (fam == 'w') return wide::smem_lines(L, B, 1, ntw, !x);
    if (fam == 'p') return p2::smem_lines(prec, L, B, 1, ntw);
    return x ? smem_x(prec, pl.dev, B) : smem_col(prec, pl.dev, B);
}

bool Solver::pass_fits(int pass, char fam, int B, const PassArgs &pa, const Plan &pl) const
{
    static const int limit = max_smem_per_block() - 1024;  // room for static shared data
    const int tpl = pl.dev.tpl, nt = B * tpl;
    int max_threads = MAX_THREADS;
    if (pass == 2 && fam == 't') max_threads = wide::ZT_MAX_THREADS;
    if (pass == 2 && fam == 'w') max_threads = wide::Z_MAX_THREADS;
    if ((pass == 0 || pass == 4) && fam == 'p' && B > 8) return false;  // compiled for 1, 2, 4, 8 lines
    if ((pass == 0 || pass == 4) && B > MAX_LINES) return false;
    if (pass == 2 && fam == 't' && nt % 32 != 0) return false;           // whole warps
    if (fam == 'c') return B == tc::ZTC_LINES && pass_smem(pass, fam, B, pa, pl) <= (size_t)max_smem_per_block();
    if (fam == 'q')  // fixed lines per length; no static shared memory
        return B == (pass == 2 ? wide::zq_lines(pl.dev.L) : axis_of(pass) == 0 ? wide::xq_lines(pl.dev.L) : wide::yq_lines(pl.dev.L)) &&
               pass_smem(pass, fam, B, pa, pl) <= (size_t)max_smem_per_block();
    return nt <= max_threads && pass_smem(pass, fam, B, pa, pl) <= (size_t)limit;
}

PassChoice Solver::default_choice(int pass, const PassArgs &pa)
{
    static const char *fam_env[3] = {"PS_KERNELS_X", "PS_KERNELS_Y", "PS_KERNELS_Z"};
    static const char *line_env[5] = {"PS_LINES_X", "PS_LINES_Y", "PS_LINES_Z", "PS_LINES_Y", "PS_LINES_XI"};
    const int axis = axis_of(pass);
    const char *f = getenv(fam_env[axis]);
    if (!f) f = getenv("PS_KERNELS");
    char fam;
    if (f && strcmp(f, "runtime") == 0) fam = 'r';
    else if (f && strcmp(f, "p2") == 0) fam = family_ok(pass, 'p', pa) ? 'p' : 'r';
    else if (f && strcmp(f, "wide") == 0)
        fam = family_ok(pass, 'w', pa) ? 'w' : family_ok(pass, 'p', pa) ? 'p' : 'r';
    else if (f && strcmp(f, "tmem") == 0 && family_ok(pass, 't', pa)) fam = 't';
    else if (f && strcmp(f, "tma") == 0 && family_ok(pass, 'q', pa)) fam = 'q';
    else if (f && strcmp(f, "tc") == 0 && family_ok(pass, 'c', pa)) fam = 'c';
    // 'q' at 512^3: z 6.0 against 7.7 ms for 't'; y 1.67 / 2.01 against 2.51 / 2.31 ms for 'w';
    // x 1.25 / 1.20 against 1.33 / 1.45 ms for 'p'
    else if (family_ok(pass, 'q', pa)) fam = 'q';
    else if (pass == 2 && family_ok(pass, 't', pa)) fam = 't';
    else if (axis > 0 && family_ok(pass, 'w', pa)) fam = 'w';
    else fam = family_ok(pass, 'p', pa) ? 'p' : 'r';

    int pref = precision == PREC_FP32 ? 16 : 8;
    if (fam == 'w') pref = pass == 0 || pass == 4 ? 4 : 8;
    if (fam == 't') pref = 8;  // 64-byte rows: 8.7 against 10.0 ms with 4 for the 512^3 curl pass
    if (fam == 'p' && pass == 0) pref = 2;
    if (fam == 'p' && pass == 4) pref = 4;  // 1.47 against 1.53 ms with 2 at 512^3
    if (const char *v = getenv(line_env[pass])) {
        const int want = atoi(v);
        if (want >= 1 && want <= 64 && (want & (want - 1)) == 0) pref = want;
    }
    // PS_PLAN_X/_Y/_Z: the run-time family's plan variant (PV_* bits, FP32)
    static const char *plan_env[3] = {"PS_PLAN_X", "PS_PLAN_Y", "PS_PLAN_Z"};
    int pv = 0;
    if (fam == 'r')
        if (const char *v = getenv(plan_env[axis])) pv = atoi(v) & plan_variants(pass);
    const Plan &pl = plan(pass_len(pass), precision, family_emax(pass, fam), pv);
    if (fam == 'c') pref = tc::ZTC_LINES;
    if (fam == 'q')  // fixed by the length
        pref = pass == 2 ? wide::zq_lines(pl.dev.L) : axis == 0 ? wide::xq_lines(pl.dev.L) : wide::yq_lines(pl.dev.L);
    int B = pref;
    while (B > 1 && !pass_fits(pass, fam, B, pa, pl)) B >>= 1;
    if (fam == 't')
        while (B * pl.dev.tpl < 32 && pass_fits(pass, fam, 2 * B, pa, pl)) B *= 2;
    if (!pass_fits(pass, fam, B, pa, pl)) throw Error(PS_ERR_UNSUPPORTED, "transform length too large for one CTA");
    return PassChoice{fam, B, pv};
}

const Plan &Solver::pass_plan(int pass, const PassChoice &c)
{
    return plan(pass_len(pass), precision, family_emax(pass, c.fam), c.fam == 'r' ? c.pv : 0);
}

// The plan variants that change the run-time family's plan of a pass (FP32
// only): a radix cap below an element budget of 16, a smooth Bluestein
// length that is shorter than the power of two, and a Rader stage in place of
// Bluestein's algorithm.
int Solver::plan_variants(int pass) const
{
    if (precision != PREC_FP32) return 0;
    const int L = pass_len(pass);
    int v = 0;
    if (family_emax(pass, 'r') >= 16 && L > 1) v |= PV_HALF_RADIX;
    if (bluestein_length(L) && next_smooth(2 * L - 1) < next_pow2(2 * L - 1)) v |= PV_SMOOTH_M;
    if (rader_length(L, family_emax(pass, 'r'), family_emax(pass, 'r'))) v |= PV_RADER;
    return v;
}

void Solver::launch_pass(int pass, const PassChoice &c, PassArgs &pa)
{
    const int prec = precision;
    const Plan &pl = pass_plan(pass, c);
    switch (pass) {
    case 0: {
        XFwdArgs &a = pa.x;
        a.plan = pl.dev;
        a.B = c.B;
        if (c.fam == 'q') PS_CK(wide::launch_xfq(a, stream));
        else if (c.fam == 'w') PS_CK(wide::launch_xfwd(a, stream));
        else if (c.fam == 'p') PS_CK(p2::launch_xfwd(a, stream));
        else PS_CK(launch_xfwd(prec, a, stream));
        break;
    }
    case 1:
    case 3: {
        ColArgs &a = pass == 1 ? pa.y : pa.yi;
        const int inv = pass == 3;
        a.plan = pl.dev;
        a.B = c.B;
        if (c.fam == 'q') PS_CK(wide::launch_yq(inv, a, n[2], static_cast<int *>(status.p), stream));
        else if (c.fam == 'w') PS_CK(wide::launch_col(inv, a, n[2], stream));
        else if (c.fam == 'p') PS_CK(p2::launch_col(inv, a, n[2], stream));
        else PS_CK(launch_col(prec, inv, a, n[2], stream));
        break;
    }
    case 2: {
        ZArgs &a = pa.z;
        a.plan = pl.dev;
        a.B = c.B;
        const int ny = dims == 2 ? 1 : P[1];  // rows of columns (2D: one row of x columns)
        if (c.fam == 'q') PS_CK(wide::launch_zq(a, ny, static_cast<int *>(status.p), stream));
        else if (c.fam == 'c') PS_CK(tc::launch_ztc(a, ny, static_cast<int *>(status.p), stream));
        else if (c.fam == 't') PS_CK(wide::launch_zt(a, ny, stream));
        else if (c.fam == 'w') PS_CK(wide::launch_z(a, ny, stream));
        else if (c.fam == 'p') PS_CK(p2::launch_z(a, ny, family_emax(2, 'p'), stream));
        else PS_CK(launch_z(prec, a, ny, stream));
        break;
    }
    default: {
        XInvArgs &a = pa.xi;
        a.plan = pl.dev;
        a.B = c.B;
        if (c.fam == 'q') PS_CK(wide::launch_xiq(a, stream));
        else if (c.fam == 'w') PS_CK(wide::launch_xinv(a, stream));
        else if (c.fam == 'p') PS_CK(p2::launch_xinv(a, stream));
        else PS_CK(launch_xinv(prec, a, stream));
        break;
    }
    }
}

// ---------------------------------------------------------------------------
// Tuned choices: in memory for the process, and in a text file (one
// "key family lines variant" line a pass; files without the variant field
// read as variant 0) at $PS_TUNE_CACHE, else
// $XDG_CACHE_HOME/poisson_solver_gb300/tune.txt or
// $HOME/.cache/poisson_solver_gb300/tune.txt; PS_TUNE_CACHE="" keeps them in
// memory only.
namespace {

std::mutex tune_mu;
std::map<std::string, PassChoice> tune_table;
bool tune_loaded = false;

std::string tune_path()
{
    if (const char *p = getenv("PS_TUNE_CACHE")) return p;
    std::string base;
    if (const char *x = getenv("XDG_CACHE_HOME")) base = x;
    else if (const char *h = getenv("HOME")) base = std::string(h) + "/.cache";
    else return "";
    return base + "/poisson_solver_gb300/tune.txt";
}

void tune_load_locked()
{
    if (tune_loaded) return;
    tune_loaded = true;
    const std::string path = tune_path();
    if (path.empty()) return;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream in(line);
        std::string key, fam;
        int B = 0, pv = 0;
        if (!(in >> key >> fam >> B)) continue;
        if (!(in >> pv)) pv = 0;
        if (fam.size() == 1 && B >= 1 && B <= 64 && pv >= 0 && pv <= 7) tune_table[key] = PassChoice{fam[0], B, pv};
    }
}

void tune_store_locked(const std::string &key, const PassChoice &c)
{
    tune_table[key] = c;
    const std::string path = tune_path();
    if (path.empty()) return;
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {
        // create the directory chain (best effort)
        for (size_t i = 1; i <= slash; ++i)
            if (path[i] == '/' || i == slash) mkdir(path.substr(0, i == slash ? slash : i).c_str(), 0755);
    }
    std::ofstream f(path, std::ios::app);
    if (f) f << key << ' ' << c.fam << ' ' << c.B << ' ' << c.pv << '\n';
}

}  // namespace

std::string Solver::tune_key(int pass, const PassArgs &pa)
{
    if (device_tag.empty()) {
        cudaDeviceProp prop{};
        PS_CK(cudaGetDeviceProperties(&prop, device));
        std::ostringstream d;
        for (const char *c = prop.name; *c; ++c) d << (*c == ' ' ? '_' : *c);
        d << ":sm" << prop.multiProcessorCount;
        device_tag = d.str();
    }
    std::ostringstream k;
    k << device_tag << ":" << (precision == PREC_FP64 ? "fp64" : precision == PREC_FP32 ? "fp32" : "df64") << ":" << dims << "d:N" << n[0] << 'x'
      << n[1] << 'x' << n[2] << ":P" << P[0] << 'x' << P[1] << 'x' << P[2] << ":op" << pa.z.op << ":in" << pa.x.ncomp
      << ":out" << pa.xi.ncomp << ":z" << pa.z.nin << pa.z.nout << ":pass" << pass;
    return k.str();
}

// Any PS_KERNELS* or PS_LINES* setting bypasses the tuned choices.
static bool env_override()
{
    for (const char *v : {"PS_KERNELS", "PS_KERNELS_X", "PS_KERNELS_Y", "PS_KERNELS_Z", "PS_LINES_X", "PS_LINES_XI",
                          "PS_LINES_Y", "PS_LINES_Z", "PS_PLAN_X", "PS_PLAN_Y", "PS_PLAN_Z"})
        if (getenv(v)) return true;
    return false;
}

PassChoice Solver::choice(int pass, const PassArgs &pa)
{
    if (!env_override()) {
        std::lock_guard<std::mutex> lock(tune_mu);
        tune_load_locked();
        auto it = tune_table.find(tune_key(pass, pa));
        if (it != tune_table.end() && family_ok(pass, it->second.fam, pa) &&
            (it->second.pv & ~plan_variants(pass)) == 0) {
            const Plan &pl = pass_plan(pass, it->second);
            if (pass_fits(pass, it->second.fam, it->second.B, pa, pl)) return it->second;
        }
    }
    return default_choice(pass, pa);
}

int Solver::solve(const double *const Bin[3], double *const Aout[3], bool filter_only)
{
    PassArgs pa;
    const int write_mask = prepare(Bin, Aout, filter_only, pa);

    std::array<cudaEvent_t, NPASS + 1> ev{};
    if (opt_timing) {
        if (ev_pool.empty()) {
            for (auto &e : ev) PS_CK(cudaEventCreate(&e));
        } else {
            ev = ev_pool.back();
            ev_pool.pop_back();
        }
        ev_pending.push_back(ev);
    }
    auto mark = [&](int i) {
        if (opt_timing) PS_CK(cudaEventRecord(ev[i], stream));
    };
    mark(0);
    // x forward, y forward, z (forward, spectral operation, inverse), then
    // y inverse and x inverse of the written outputs
    for (int pass = 0; pass < NPASS; ++pass) {
        if ((pass < 3 || write_mask) && !(dims == 2 && (pass == 1 || pass == 3))) {
            // 2D: the fused pass transforms y itself
            launch_pass(pass, choice(pass, pa), pa);
        }
        mark(pass + 1);
    }
    return write_mask;
}

void Solver::autotune(int in_mask)
{
    check_setup();
    if (in_mask <= 0 || in_mask > 7) throw Error(PS_ERR_ARGUMENT, "component mask must be 1..7");
    const int out_mask = output_mask(in_mask);
    // zero-filled scratch fields: the tuning runs leave every buffer at zero
    DevBuf tb[3], ta[3];
    const size_t bytes = field_elems() * sizeof(double);
    const double *Bin[3];
    double *Aout[3];
    for (int c = 0; c < 3; ++c) {
        Bin[c] = nullptr;
        Aout[c] = nullptr;
        if (in_mask >> c & 1) {
            tb[c].ensure(bytes);
            PS_CK(cudaMemsetAsync(tb[c].p, 0, bytes, stream));
            Bin[c] = (const double *)tb[c].p;
        }
        if (out_mask >> c & 1) {
            ta[c].ensure(bytes);
            Aout[c] = (double *)ta[c].p;
        }
    }
    PassArgs pa;
    const int write_mask = prepare(Bin, Aout, false, pa);
    for (int c = 0; c < 3; ++c)
        if (work[c].p) PS_CK(cudaMemsetAsync(work[c].p, 0, work[c].bytes, stream));
    cudaEvent_t e0, e1;
    PS_CK(cudaEventCreate(&e0));
    PS_CK(cudaEventCreate(&e1));
    try {
        for (int pass = 0; pass < NPASS; ++pass) {
            if (pass >= 3 && !write_mask) continue;
            if (dims == 2 && (pass == 1 || pass == 3)) continue;  // the fused pass transforms y
            // candidates: every family, plan variant (run-time family, FP32)
            // and line count that fits
            std::vector<PassChoice> cands;
            for (char fam : {'q', 't', 'w', 'p', 'r'}) {
                if (!family_ok(pass, fam, pa)) continue;
                const int pvs = fam == 'r' ? plan_variants(pass) : 0;
                for (int pv = 0; pv <= 7; ++pv) {
                    if ((pv & ~pvs) != 0) continue;
                    const Plan &pl = pass_plan(pass, PassChoice{fam, 1, pv});
                    for (int B = 1; B <= 64; B *= 2)
                        if (pass_fits(pass, fam, B, pa, pl)) cands.push_back(PassChoice{fam, B, pv});
                }
            }
            PassChoice best{0, 0};
            float best_ms = 0.f;
            for (const PassChoice &c : cands) {
                PassArgs run = pa;
                try {
                    launch_pass(pass, c, run);  // warm-up (and the one-time attribute setup)
                } catch (const Error &err) {
                    throw Error(err.status, std::string(err.what()) + " (tuning pass " + std::to_string(pass) +
                                                ", family " + c.fam + ", " + std::to_string(c.B) + " lines, plan variant " +
                                                std::to_string(c.pv) + ")");
                }
                PS_CK(cudaEventRecord(e0, stream));
                const int reps = 3;
                for (int r = 0; r < reps; ++r) launch_pass(pass, c, run);
                PS_CK(cudaEventRecord(e1, stream));
                PS_CK(cudaEventSynchronize(e1));
                float ms = 0.f;
                PS_CK(cudaEventElapsedTime(&ms, e0, e1));
                ms /= reps;
                if (!best.fam || ms < best_ms) {
                    best = c;
                    best_ms = ms;
                }
            }
            if (best.fam) {
                std::lock_guard<std::mutex> lock(tune_mu);
                tune_load_locked();
                tune_store_locked(tune_key(pass, pa), best);
            }
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    synchronize();
}

PassChoice Solver::current_choice(int pass, int in_mask)
{
    check_setup();
    if (pass < 0 || pass >= NPASS) throw Error(PS_ERR_ARGUMENT, "pass must be 0..4");
    const int out_mask = output_mask(in_mask);
    // arguments only: no buffer is touched (pointers are placeholders)
    const double *Bin[3];
    double *Aout[3];
    for (int c = 0; c < 3; ++c) {
        Bin[c] = (in_mask >> c & 1) ? reinterpret_cast<const double *>(16) : nullptr;
        Aout[c] = (out_mask >> c & 1) ? reinterpret_cast<double *>(16) : nullptr;
    }
    PassArgs pa;
    prepare(Bin, Aout, false, pa);
    return choice(pass, pa);
}

const FftPlanDev &Solver::current_plan(int pass, int in_mask)
{
    return pass_plan(pass, current_choice(pass, in_mask)).dev;
}

// ---------------------------------------------------------------------------
// push / solve3d / pull on handle-owned field buffers.
void Solver::push(const double *const B[3], cudaMemcpyKind kind)
{
    check_setup();
    const size_t bytes = field_elems() * sizeof(double);
    int mask = 0;
    for (int c = 0; c < 3; ++c)
        if (B[c]) {
            fb[c].ensure(bytes);
            PS_CK(cudaMemcpyAsync(fb[c].p, B[c], bytes, kind, stream));
            mask |= 1 << c;
        }
    PS_CK(cudaStreamSynchronize(stream));
    pushed = mask;
    rhs_ready = 0;
}

void Solver::solve_internal(int want_dims)
{
    check_setup();
    if (want_dims != dims)
        throw Error(PS_ERR_STATE, dims == 2 ? "handle set up by setup2d: call solve2d" : "handle set up by setup3d: call solve3d");
    if (!pushed) throw Error(PS_ERR_STATE, "solve3d called before push");
    const int out_mask = output_mask(pushed);
    const double *Bin[3];
    double *Aout[3];
    for (int c = 0; c < 3; ++c) {
        Bin[c] = (pushed >> c & 1) ? (const double *)fb[c].p : nullptr;
        Aout[c] = nullptr;
        if (out_mask >> c & 1) {
            fa[c].ensure(field_elems() * sizeof(double));
            Aout[c] = (double *)fa[c].p;
        }
    }
    produced = solve(Bin, Aout);
    rhs_ready = 0;
}

void Solver::returned_rhs(const double *out[3])
{
    // the reference returns B after its forward/inverse round trip, i.e.
    // B itself unless the regulariser or the reprojection changed it (the
    // Gaussian family always filters)
    const size_t bytes = field_elems() * sizeof(double);
    const bool filtered = reg > 0 || kernel_family == PS_KERNEL_GAUSSIAN || (opt_reproject && pushed == 7 && dims == 3);
    if (filtered && !rhs_ready) {
        const double *Bin[3];
        double *Rout[3];
        for (int c = 0; c < 3; ++c) {
            Bin[c] = (pushed >> c & 1) ? (const double *)fb[c].p : nullptr;
            Rout[c] = nullptr;
            if (pushed >> c & 1) {
                fr[c].ensure(bytes);
                Rout[c] = (double *)fr[c].p;
            }
        }
        solve(Bin, Rout, true);
        rhs_ready = 1;
    }
    for (int c = 0; c < 3; ++c)
        out[c] = (pushed >> c & 1) ? (const double *)(filtered ? fr[c].p : fb[c].p) : nullptr;
}

void Solver::pull(double *const A[3], double *const RB[3], cudaMemcpyKind kind)
{
    check_setup();
    const size_t bytes = field_elems() * sizeof(double);
    for (int c = 0; c < 3; ++c)
        if (A[c] && (produced >> c & 1)) PS_CK(cudaMemcpyAsync(A[c], fa[c].p, bytes, kind, stream));
    bool want_rhs = false;
    for (int c = 0; c < 3; ++c)
        if (RB[c] && (pushed >> c & 1)) want_rhs = true;
    if (want_rhs) {
        const double *src[3];
        returned_rhs(src);
        for (int c = 0; c < 3; ++c)
            if (RB[c] && src[c]) PS_CK(cudaMemcpyAsync(RB[c], src[c], bytes, kind, stream));
    }
    synchronize();
}

// Fortran-style arrays (poisson_solver_push.f:8-140, poisson_solver_pull.f:8-485):
// element (c, i, j, k) of the field at ((k + o2) e1 + (j + o1)) e0 + (i + o0))
// ncomp + c. The field box moves as one pitched 3D copy to or from a packed
// device buffer, which the (de)interleave kernels split or build.
static cudaMemcpy3DParms box_copy(const int n[3], int ncomp)
{
    cudaMemcpy3DParms p{};
    p.extent = make_cudaExtent((size_t)n[0] * ncomp * sizeof(double), (size_t)n[1], (size_t)n[2]);
    return p;
}

static void check_box(const int n[3], int ncomp, const int ext[3], const int off[3])
{
    if (ncomp < 1 || ncomp > 3) throw Error(PS_ERR_ARGUMENT, "an interleaved array holds 1 to 3 components");
    for (int d = 0; d < 3; ++d)
        if (off[d] < 0 || ext[d] < off[d] + n[d])
            throw Error(PS_ERR_ARGUMENT, "array extents must hold the field at its offset");
}

void Solver::push_interleaved(const double *b, int ncomp, const int ext[3], const int off[3], cudaMemcpyKind kind)
{
    check_setup();
    if (!b) throw Error(PS_ERR_ARGUMENT, "null array");
    check_box(n, ncomp, ext, off);
    const size_t elems = field_elems();
    stage.ensure(elems * ncomp * sizeof(double));
    cudaMemcpy3DParms p = box_copy(n, ncomp);
    p.srcPtr = make_cudaPitchedPtr(const_cast<double *>(b), (size_t)ext[0] * ncomp * sizeof(double),
                                   (size_t)ext[0] * ncomp, (size_t)ext[1]);
    p.srcPos = make_cudaPos((size_t)off[0] * ncomp * sizeof(double), (size_t)off[1], (size_t)off[2]);
    p.dstPtr = make_cudaPitchedPtr(stage.p, (size_t)n[0] * ncomp * sizeof(double), (size_t)n[0] * ncomp, (size_t)n[1]);
    p.kind = kind;
    PS_CK(cudaMemcpy3DAsync(&p, stream));
    double *dst[3] = {nullptr, nullptr, nullptr};
    for (int c = 0; c < ncomp; ++c) {
        fb[c].ensure(elems * sizeof(double));
        dst[c] = (double *)fb[c].p;
    }
    PS_CK(launch_deinterleave((const double *)stage.p, ncomp, (long long)elems, dst, stream));
    PS_CK(cudaStreamSynchronize(stream));
    pushed = (1 << ncomp) - 1;  // X; X, Y; or X, Y, Z as the array's first extent says
    rhs_ready = 0;
}

void Solver::pull_interleaved(double *a, int ncomp_a, double *b, int ncomp_b, const int ext[3], const int off[3],
                              cudaMemcpyKind kind)
{
    check_setup();
    const size_t elems = field_elems();
    // both arrays are checked before either is written
    if (a) check_box(n, ncomp_a, ext, off);
    if (b) check_box(n, ncomp_b, ext, off);
    for (int which = 0; which < 2; ++which) {
        double *arr = which == 0 ? a : b;
        const int ncomp = which == 0 ? ncomp_a : ncomp_b;
        if (!arr) continue;
        // solution components the solve produced, or the returned right-hand
        // side; components not there are written as zero (pull.f:340-365)
        const double *src[3] = {nullptr, nullptr, nullptr};
        if (which == 0) {
            for (int c = 0; c < 3; ++c) src[c] = (produced >> c & 1) ? (const double *)fa[c].p : nullptr;
        } else {
            returned_rhs(src);
        }
        stage.ensure(elems * ncomp * sizeof(double));
        PS_CK(launch_interleave(src, ncomp, (long long)elems, (double *)stage.p, stream));
        cudaMemcpy3DParms p = box_copy(n, ncomp);
        p.srcPtr = make_cudaPitchedPtr(stage.p, (size_t)n[0] * ncomp * sizeof(double), (size_t)n[0] * ncomp, (size_t)n[1]);
        p.dstPtr = make_cudaPitchedPtr(arr, (size_t)ext[0] * ncomp * sizeof(double), (size_t)ext[0] * ncomp, (size_t)ext[1]);
        p.dstPos = make_cudaPos((size_t)off[0] * ncomp * sizeof(double), (size_t)off[1], (size_t)off[2]);
        p.kind = kind;
        PS_CK(cudaMemcpy3DAsync(&p, stream));
        PS_CK(cudaStreamSynchronize(stream));  // the stage is reused by the next array
    }
    synchronize();
}

// smooth3d (poisson_solver_smooth3d.f): the pushed fields, zero-padded on
// unbounded axes, transformed, multiplied by exp(-s^2 |k|^2 / 2) with the
// solver's wavenumbers, transformed back and cropped, in place. It runs the
// filter pass of the pipeline with the Gaussian octant.
void Solver::smooth3d(double s)
{
    check_setup();
    if (dims != 3) throw Error(PS_ERR_STATE, "smooth3d is for 3D handles");
    if (!(s >= 0.0) || !std::isfinite(s)) throw Error(PS_ERR_ARGUMENT, "smoothing width must be finite and >= 0");
    if (!pushed) throw Error(PS_ERR_STATE, "smooth3d called before push");
    const size_t nk = (size_t)Mx * oy * oz;
    if (smooth_s != s) {
        smooth64.ensure(nk * sizeof(double));
        smooth32.release();
        smooth_df.release();
        KernelFillArgs fa{};
        fa.zeta_out = (double *)smooth64.p;
        fa.Mx = Mx;
        fa.oy = oy;
        fa.oz = oz;
        for (int d = 0; d < 3; ++d) {
            fa.P[d] = P[d];
            fa.dx[d] = dx[d];
        }
        fa.norm = (double)P[0] * (double)P[1] * (double)P[2];
        fa.smooth = 1;
        fa.smooth_sigma = s;
        PS_CK(launch_kernel_fill(fa, stream));
        smooth_s = s;
    }
    const double *Bin[3];
    double *Aout[3];
    for (int c = 0; c < 3; ++c) {
        Bin[c] = (pushed >> c & 1) ? (const double *)fb[c].p : nullptr;
        Aout[c] = (pushed >> c & 1) ? (double *)fb[c].p : nullptr;
    }
    filter_source = 1;
    try {
        solve(Bin, Aout, true);
    } catch (...) {
        filter_source = 0;
        throw;
    }
    filter_source = 0;
    rhs_ready = 0;
}

void Solver::synchronize()
{
    PS_CK(cudaStreamSynchronize(stream));
    check_status();
}

void Solver::check_status()
{
    if (!status.p) return;
    int word = 0;
    PS_CK(cudaMemcpyAsync(&word, status.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    PS_CK(cudaStreamSynchronize(stream));
    if (word) {
        PS_CK(cudaMemsetAsync(status.p, 0, sizeof(int), stream));
        PS_CK(cudaStreamSynchronize(stream));
        throw Error(PS_ERR_TIMEOUT, "a pass kernel's wait for an asynchronous copy timed out; results are invalid");
    }
}

size_t Solver::device_bytes() const
{
    size_t s = kern64.bytes + kern32.bytes + kern_df.bytes + kernzf32.bytes + zeta64.bytes + zeta32.bytes +
               zeta_df.bytes + smooth64.bytes + smooth32.bytes + smooth_df.bytes;
    for (int c = 0; c < 3; ++c) s += work[c].bytes + fb[c].bytes + fa[c].bytes + fr[c].bytes;
    for (auto &kv : plans) s += kv.second->table.bytes;
    return s;
}

void Solver::copy_kernel(double *host, long long capacity) const
{
    check_setup();
    const size_t nk = (size_t)Mx * oy * oz;
    if (capacity < (long long)nk) throw Error(PS_ERR_ARGUMENT, "kernel buffer too small");
    PS_CK(cudaMemcpy(host, kern64.p, nk * sizeof(double), cudaMemcpyDeviceToHost));
}

}  // namespace ps
