/*
 * CPU oracle: plain-C restatement of the reference 3D Poisson solve
 * (mmhej/poissonsolver, c++/source). TEST INFRASTRUCTURE ONLY -- the tests,
 * the smoke check and the benchmark's CPU-baseline leg use it as the checker;
 * the product never links it.
 *
 * Every step follows the reference single-rank data flow and operation order
 * (C99 complex arithmetic lowers to the same compiler builtins as
 * std::complex<double>), so on the same machine its results agree with the
 * reference built from source to rounding level; tests/test_oracle.py checks
 * that and the golden fixtures the reference build wrote.
 *
 * One deliberate difference: the periodic-periodic-unbounded kernel samples
 * its 1D free-space Green's function at z = -(Pz/2) dz + k dz and stores it
 * at index k. The reference (greens3d.cpp:361-370) writes pen.X[j] with j
 * uninitialised and reads an uninitialised xmin[2]; the restatement does
 * what that code evidently intends. Only sources with a non-zero x-y mean see
 * the difference.
 *
 * A second: for grad with fewer than three pushed components the reference
 * dereferences NULL (solve3d.cpp:350-352); here a missing component d uses
 * component x, so a scalar push gives the gradient of the scalar solution.
 */
#define _POSIX_C_SOURCE 199309L
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "ps_oracle.h"

#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* Threads: pencils (and kernel samples) are shared out over OpenMP threads.
 * Each pencil's arithmetic is the same whichever thread runs it, so results
 * do not depend on the thread count; the reference spreads the same pencils
 * over MPI ranks. */
void oracle_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
#else
    (void)n;
#endif
}

int oracle_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static const double PI = 3.1415926535897932;
static const double EULER_GAMMA = 0.5772156649015329;

/* ------------------------------------------------------------------------ */
/* 1D transform: Glassman's general-N FFT (W. E. Ferguson, "A simple
 * derivation of Glassman's general N fast Fourier transform", Comp. & Math.
 * with Appls. 1982), as class_pencil::fft (pencil/fft.cpp:33-197) and ::ifft
 * (pencil/ifft.cpp, delta with +sin) apply it: each stage takes the smallest
 * prime factor c of the remaining length b, evaluates the c-point sums by
 * Horner's rule in the running twiddle omega, and advances omega by the
 * recurrence omega <- delta * omega. Data ping-pong between x and work. */
static void glassman(cplx *x, cplx *work, int n, int inverse)
{
    int a = 1, b = n, c = 1;
    cplx *u = x, *v = work;
    int in_x = 1;
    while (b > 1) {
        a = c * a;
        for (c = 2; c <= b; ++c)
            if (b % c == 0) break;
        b = b / c;
        double angle = 2.0 * PI / (double)(a * c);
        cplx delta = inverse ? CMPLX(cos(angle), sin(angle)) : CMPLX(cos(angle), -sin(angle));
        cplx omega = CMPLX(1.0, 0.0);
        for (int ic = 0; ic < c; ++ic) {
            for (int ia = 0; ia < a; ++ia) {
                const cplx *src = u + (size_t)b * c * ia;
                for (int ib = 0; ib < b; ++ib) {
                    cplx sum = src[ib + b * (c - 1)];
                    for (int jc = c - 2; jc >= 0; --jc) sum = src[ib + b * jc] + omega * sum;
                    v[ib + b * ia + b * a * ic] = sum;
                }
                omega = delta * omega;
            }
        }
        cplx *t = u; u = v; v = t;
        in_x = !in_x;
    }
    if (!in_x) memcpy(x, u, sizeof(cplx) * (size_t)n);
}

/* Swap halves (pencil/fft_shift.cpp:9-72); only applied to even lengths. */
static void fft_shift(cplx *x, int n)
{
    int h = n / 2;
    for (int i = 0; i < h; ++i) {
        cplx t = x[i];
        x[i] = x[i + h];
        x[i + h] = t;
    }
}

int oracle_fft(int n, int dir, double *data)
{
    if (n < 1) return 1;
    cplx *x = malloc(sizeof(cplx) * (size_t)n), *w = malloc(sizeof(cplx) * (size_t)n);
    if (!x || !w) { free(x); free(w); return 4; }
    for (int i = 0; i < n; ++i) x[i] = CMPLX(data[2 * i], data[2 * i + 1]);
    glassman(x, w, n, dir > 0);
    for (int i = 0; i < n; ++i) { data[2 * i] = creal(x[i]); data[2 * i + 1] = cimag(x[i]); }
    free(x); free(w);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Sine integral by the method of Numerical Recipes' cisi (Press et al., 2nd
 * ed.): for t > 2 the continued fraction of E1(it) by the modified Lentz
 * method, else the interleaved power series of Si and Ci, both stopped at
 * relative change 1e-10 -- the rules special_functions.cpp:238-352 uses. */
double oracle_sine_int(double x)
{
    const double eps = 1.0e-10, fpmin = 1.0e-30, fpmax = 1.0e30, tmin = 2.0;
    const int maxit = 1000;
    double t = fabs(x), ans;
    if (t == 0.0) return 0.0;
    if (t > tmin) {
        cplx b = CMPLX(1.0, t);
        cplx c = CMPLX(fpmax, 0.0);
        cplx d = 1.0 / b;
        cplx h = d;
        int i = 2;
        double err = 1.0;
        while (i < maxit && err > eps) {
            double a = -pow((double)(i - 1), 2.0);
            b = b + 2.0;
            d = 1.0 / (a * d + b);
            c = b + a / c;
            cplx del = c * d;
            h = h * del;
            err = fabs(creal(del - 1.0)) + fabs(cimag(del - 1.0));
            ++i;
        }
        cplx g = CMPLX(cos(t), -sin(t));
        h = g * h;
        ans = 0.5 * PI + cimag(h);
    } else {
        double sums;
        if (t < sqrt(fpmin)) {
            sums = t;
        } else {
            double sum = 0.0, sumc = 0.0, sign = 1.0, fact = 1.0, err = 1.0;
            int odd = 1, k = 1;
            sums = 0.0;
            while (k <= maxit && err > eps) {
                fact = fact * t / k;
                double term = fact / k;
                sum = sum + sign * term;
                err = term / fabs(sum);
                if (odd) { sign = -sign; sums = sum; sum = sumc; }
                else { sumc = sum; sum = sums; }
                odd = !odd;
                ++k;
            }
        }
        ans = sums;
    }
    return x < 0.0 ? -ans : ans;
}

/* Integral of (1 - J0(t))/t over [0, x] from the Chebyshev expansions of
 * Y. L. Luke, "Mathematical functions and their approximations" (1975),
 * Table 9.3: an even series in T_2n(x/8) for x < 8 and a complex series in
 * T_n(10/x - 1) times the asymptotic phase for x >= 8 -- the form
 * special_functions.cpp:115-229 evaluates. */
static const double LUKE_JI0_SMALL[18] = {
    1.35105091918187636388,  0.83791030734868376979, -0.35047963978529462711,
    0.12777415867753198659, -0.02981035698255560990,  0.00455219841169387328,
   -0.00048408621967185359,  0.00003780202859916883, -0.00000225886908506771,
    0.00000010664609068423, -0.00000000408005443149,  0.00000000012909996251,
   -0.00000000000343577839,  0.00000000000007799552, -0.00000000000000152842,
    0.00000000000000002612, -0.00000000000000000039,  0.00000000000000000001};
static const double LUKE_JI0_LARGE[39][2] = {
    { 0.95360150809738558095, -0.13917925930200001236}, {-0.05860838853872331670, -0.12902065726135067062},
    {-0.01020283575659856676,  0.01103004348109535741}, { 0.00196012704043622581,  0.00051817180856880364},
    {-0.00009574977697756219, -0.00030928210173975681}, {-0.00003570479477043714,  0.00004647098443047525},
    { 0.00001169677960430223, -0.00000008198845340928}, {-0.00000164386246452682, -0.00000191888381006925},
    {-0.00000007415845751760,  0.00000057813667761104}, { 0.00000011434387527717, -0.00000008448997773317},
    {-0.00000003600903214141, -0.00000000525612161520}, { 0.00000000601257386446,  0.00000000763257790924},
    { 0.00000000019124656215, -0.00000000268643963177}, {-0.00000000054892028385,  0.00000000054279949860},
    { 0.00000000022740445656, -0.00000000001744365343}, {-0.00000000005671490865, -0.00000000003975692920},
    { 0.00000000000607510983,  0.00000000002069683990}, { 0.00000000000252060520, -0.00000000000639623674},
    {-0.00000000000191255246,  0.00000000000116359235}, { 0.00000000000074056501,  0.00000000000006759603},
    {-0.00000000000018950214, -0.00000000000016557337}, { 0.00000000000002021389,  0.00000000000008425597},
    { 0.00000000000001103617, -0.00000000000002824474}, {-0.00000000000000889993,  0.00000000000000607698},
    { 0.00000000000000388558, -0.00000000000000003171}, {-0.00000000000000119200, -0.00000000000000077237},
    { 0.00000000000000021456,  0.00000000000000048022}, { 0.00000000000000002915, -0.00000000000000019502},
    {-0.00000000000000004877,  0.00000000000000005671}, { 0.00000000000000002737, -0.00000000000000000862},
    {-0.00000000000000001080, -0.00000000000000000269}, { 0.00000000000000000308,  0.00000000000000000309},
    {-0.00000000000000000042, -0.00000000000000000167}, {-0.00000000000000000020,  0.00000000000000000066},
    { 0.00000000000000000020, -0.00000000000000000019}, {-0.00000000000000000011,  0.00000000000000000003},
    { 0.00000000000000000004,  0.00000000000000000001}, {-0.00000000000000000001, -0.00000000000000000001},
    { 0.00000000000000000000,  0.00000000000000000001}};

double oracle_bessel_int_J0(double x)
{
    double x8 = 0.125 * x;
    double x5sh = 2.0 * 5.0 / x - 1.0;
    double t0, t1, t2, ans;
    if (x < 8.0) {
        t0 = 1.0;
        t1 = x8;
        ans = t0 * LUKE_JI0_SMALL[0];
        for (int i = 2; i < 36; ++i) {
            t2 = 2 * x8 * t1 - t0;
            if (i % 2 == 0) ans += LUKE_JI0_SMALL[i / 2] * t2;
            t0 = t1;
            t1 = t2;
        }
    } else {
        t0 = 1.0;
        t1 = x5sh;
        cplx sum = CMPLX(LUKE_JI0_LARGE[0][0], LUKE_JI0_LARGE[0][1]) * t0;
        sum += CMPLX(LUKE_JI0_LARGE[1][0], LUKE_JI0_LARGE[1][1]) * t1;
        for (int i = 2; i < 39; ++i) {
            t2 = 2.0 * x5sh * t1 - t0;
            t0 = t1;
            t1 = t2;
            sum += CMPLX(LUKE_JI0_LARGE[i][0], LUKE_JI0_LARGE[i][1]) * t2;
        }
        double fac = cos(x + 0.25 * PI) * creal(sum) - sin(x + 0.25 * PI) * cimag(sum);
        ans = sqrt(2.0 / (PI * x)) / x * fac + EULER_GAMMA + log(0.5 * x);
    }
    return ans;
}

/* ------------------------------------------------------------------------ */
/* Spectral kernel (greens3d.cpp:9-547). */
typedef struct {
    int n[3], bc[3], p[3], reg;
    int gm;        /* Gaussian family of order 2 gm (0: the reference's kernels) */
    double gs;     /* its width */
    double dx[3];
    cplx *ik[3];   /* spectral derivative vectors, lengths p[d] */
    double *zeta;  /* [p2][p1][p0] or NULL */
    cplx *G;       /* [p2][p1][p0] */
} kernel_t;

static void kernel_free(kernel_t *K)
{
    for (int d = 0; d < 3; ++d) free(K->ik[d]);
    free(K->zeta);
    free(K->G);
    memset(K, 0, sizeof(*K));
}

/* In-place transforms of a [p2][p1][p0] complex array along one axis, with an
 * optional half swap first (the fft_shift the kernel build applies). */
static void transform_axis(cplx *a, const int p[3], int axis, int shift, int inverse)
{
    int n = p[axis];
    size_t stride = axis == 0 ? 1 : axis == 1 ? (size_t)p[0] : (size_t)p[0] * p[1];
    int o1 = axis == 0 ? p[1] : p[0];
    int o2 = axis == 2 ? p[1] : p[2];
#pragma omp parallel
    {
        cplx *pen = malloc(sizeof(cplx) * (size_t)n), *w = malloc(sizeof(cplx) * (size_t)n);
#pragma omp for collapse(2) schedule(static)
        for (int b = 0; b < o2; ++b) {
            for (int q = 0; q < o1; ++q) {
                size_t base;
                if (axis == 0) base = ((size_t)b * p[1] + q) * p[0];
                else if (axis == 1) base = (size_t)b * p[1] * p[0] + q;
                else base = (size_t)b * p[0] + q;
                for (int m = 0; m < n; ++m) pen[m] = a[base + m * stride];
                if (shift) fft_shift(pen, n);
                glassman(pen, w, n, inverse);
                for (int m = 0; m < n; ++m) a[base + m * stride] = pen[m];
            }
        }
        free(pen); free(w);
    }
}

/* ------------------------------------------------------------------------ */
/* Gaussian-regularised family (an extension; the reference has no such
 * kernels): spectrum zeta_m(s|k|)/|k|^2, zeta_m(k) = e^{-a} sum_{n<m} a^n/n!,
 * a = s^2 k^2 / 2. In d dimensions G = G_0 + sum_{n=1}^{m-1} G_n with G_0 the
 * potential of a unit Gaussian of width s (zero added constant: G_0 tends to
 * the free-space kernel) and
 *   G_n(r) = s^{2-d} / (2 (2 pi)^{d/2}) e^{-u} L^{(d/2-1)}_{n-1}(u) / n,
 * u = r^2/(2 s^2). The functions below evaluate it by other means than the
 * GPU build does (explicit Laguerre sums, a backward continued fraction), so
 * the two check each other; tests/test_oracle.py pins them to quadratures of
 * the spectrum. */

/* L^{(alpha)}_n(u) = sum_{i<=n} (-1)^i binom(n+alpha, n-i) u^i / i! */
static double laguerre(int n, double alpha, double u)
{
    double sum = 0.0;
    for (int i = 0; i <= n; ++i) {
        double b = 1.0, f = 1.0;
        for (int t = 1; t <= n - i; ++t) b *= (alpha + (double)i + (double)t) / (double)t;
        for (int t = 1; t <= i; ++t) f *= u / (double)t;
        sum += ((i & 1) ? -1.0 : 1.0) * b * f;
    }
    return sum;
}

/* ln r + E1(u)/2, u = r^2/(2 s^2): the series of E1 below u = 1 with ln r
 * cancelled analytically; above, E1(u) = e^{-u}/(u+ 1/(1+ 1/(u+ 2/(1+ 2/(u+ ...)))))
 * evaluated backward from a fixed depth. */
static double log_e1_half(double r, double s)
{
    double u = 0.5 * (r / s) * (r / s);
    if (u <= 1.0) {
        double term = 1.0, sum = 0.0;
        for (int k = 1; k < 100; ++k) {
            term *= -u / (double)k;
            sum += term / (double)k;
        }
        return 0.5 * (log(2.0 * s * s) - EULER_GAMMA - sum);
    }
    double t = u;
    for (int n = 2000; n >= 1; --n) t = u + (double)n / (1.0 + (double)n / t);
    return log(r) + 0.5 * exp(-u) / t;
}

double oracle_gauss_green(int dim, int m, double s, double r)
{
    double u = 0.5 * (r / s) * (r / s), tail = 0.0, g0;
    for (int n = 1; n <= m - 1; ++n) tail += laguerre(n - 1, 0.5 * (double)dim - 1.0, u) / (double)n;
    double kappa = pow(s, 2.0 - (double)dim) / (2.0 * pow(2.0 * PI, 0.5 * (double)dim));
    if (dim == 3) g0 = r > 0.0 ? erf(r / (sqrt(2.0) * s)) / (4.0 * PI * r) : 1.0 / (pow(2.0 * PI, 1.5) * s);
    else if (dim == 2) g0 = -log_e1_half(r, s) / (2.0 * PI);
    else g0 = -0.5 * fabs(r) * erf(fabs(r) / (sqrt(2.0) * s)) - s / sqrt(2.0 * PI) * exp(-u);
    return g0 + kappa * exp(-u) * tail;
}

/* two_d: the 2D kernel (greens2d.cpp:9-443) on a grid of one periodic
 * z-plane (ncell[2] = 1, bc[2] = 1, dx[2] <= dx[0], dx[1] so that the filter
 * width h = max(dx, dy) as greens2d.cpp:55 takes it); all four (x, y)
 * boundary combinations are allowed. */
/* gauss_width >= 0 builds the Gaussian family instead (width 0: 2h); its
 * zeta is the family's filter and its G already carries the regularisation,
 * so the solve applies zeta to the returned right-hand side only. */
static int kernel_build(kernel_t *K, const int ncell[3], const int bc[3], const double dx[3], int reg, int two_d,
                        double gauss_width)
{
    memset(K, 0, sizeof(*K));
    for (int d = 0; d < 3; ++d) {
        K->n[d] = ncell[d];
        K->bc[d] = bc[d];
        K->dx[d] = dx[d];
    }
    int b0 = bc[0], b1 = bc[1], b2 = bc[2];
    int ok = (b0 == 0 && b1 == 0 && b2 == 0) || (b0 == 1 && b1 == 1 && b2 == 0) ||
             (b0 == 0 && b1 == 0 && b2 == 1) || (b0 == 1 && b1 == 1 && b2 == 1);
    if (two_d) ok = b2 == 1 && ncell[2] == 1 && (b0 == 0 || b0 == 1) && (b1 == 0 || b1 == 1);
    if (!ok) return 2;
    for (int d = 0; d < 3; ++d) K->p[d] = (bc[d] == 0 ? 2 : 1) * ncell[d];
    K->reg = reg;
    const int *p = K->p;
    size_t np = (size_t)p[0] * p[1] * p[2];
    double h = fmax(fmax(dx[0], dx[1]), dx[2]);

    /* ik vectors (greens3d.cpp:73-118): i 2 pi m / (P dx), m wrapped at P/2. */
    for (int d = 0; d < 3; ++d) {
        K->ik[d] = malloc(sizeof(cplx) * (size_t)p[d]);
        double dk = 1.0 / ((double)p[d] * dx[d]);
        for (int m = 0; m < p[d]; ++m) {
            int mm = (2 * m < p[d]) ? m : m - p[d];
            K->ik[d][m] = CMPLX(0.0, 2.0 * PI * (double)mm * dk);
        }
    }

    /* Regularisation filter (greens3d.cpp:123-159): zeta = e^{-a} sum_{n<m/2} a^n/n!,
     * a = sigma^2 |k|^2 / 2, sigma = 2h, m = reg rounded up to even. The
     * reference allocates m/2 - 1 coefficients and writes m/2 of them; this
     * keeps all m/2. */
    if (reg > 0 || gauss_width >= 0.0) {
        int r = reg % 2 != 0 ? reg + 1 : reg;
        double sigma = 2.0 * h;
        int nc = r / 2;
        if (gauss_width >= 0.0) {
            if (nc < 1) nc = 1;
            if (gauss_width > 0.0) sigma = gauss_width;
            K->gm = nc;
            K->gs = sigma;
        }
        double *c = malloc(sizeof(double) * (size_t)nc);
        c[0] = 1.0;
        for (int n = 1; n <= nc - 1; ++n) c[n] = c[n - 1] * 1.0 / (double)n;
        K->zeta = malloc(sizeof(double) * np);
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < p[2]; ++k)
            for (int j = 0; j < p[1]; ++j)
                for (int i = 0; i < p[0]; ++i) {
                    double arg = 0.5 * pow(sigma, 2.0) *
                                 (pow(cimag(K->ik[0][i]), 2.0) + pow(cimag(K->ik[1][j]), 2.0) +
                                  pow(cimag(K->ik[2][k]), 2.0));
                    double sum = 0.0;
                    for (int n = 0; n <= nc - 1; ++n) sum += c[n] * pow(arg, (double)n);
                    K->zeta[((size_t)k * p[1] + j) * p[0] + i] = sum * exp(-arg);
                }
        free(c);
    }

    K->G = malloc(sizeof(cplx) * np);
    cplx *G = K->G;
    if (b0 == 0 && b1 == 0 && b2 == 0) {
        /* Unbounded (greens3d.cpp:167-332): spectrally truncated kernel
         * Si(r/sigma)/(2 pi^2 r) dV, sigma = h/pi, sampled at
         * x = -(P/2) dx + i dx, then half-swapped and transformed along x, y, z. */
        const double c_1_2pi2 = 0.5 / pow(PI, 2.0);
        double sigma = h / PI;
        double xmin[3];
        for (int d = 0; d < 3; ++d) xmin[d] = -(0.5 * (double)p[d]) * dx[d];
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
        for (int k = 0; k < p[2]; ++k) {
            for (int j = 0; j < p[1]; ++j) {
                double z = xmin[2] + (double)k * dx[2];
                double y = xmin[1] + (double)j * dx[1];
                for (int i = 0; i < p[0]; ++i) {
                    double x = xmin[0] + (double)i * dx[0];
                    double r = sqrt(x * x + y * y + z * z);
                    double rho = r / sigma;
                    double g;
                    if (K->gm) g = oracle_gauss_green(3, K->gm, K->gs, r) * dx[0] * dx[1] * dx[2];
                    else if (r > 0.25 * dx[0]) g = c_1_2pi2 * oracle_sine_int(rho) / r * dx[0] * dx[1] * dx[2];
                    else g = c_1_2pi2 / sigma * dx[0] * dx[1] * dx[2];
                    G[((size_t)k * p[1] + j) * p[0] + i] = CMPLX(g, 0.0);
                }
            }
        }
        transform_axis(G, p, 0, 1, 0);
        transform_axis(G, p, 1, 1, 0);
        transform_axis(G, p, 2, 1, 0);
    } else if (b0 == 1 && b1 == 1 && b2 == 0) {
        /* Periodic-periodic-unbounded (greens3d.cpp:336-403): the kx = ky = 0
         * line is the transform of the 1D kernel -(sigma/pi)(rho Si(rho) + cos rho) dz,
         * sigma = dz/pi; every other mode is 1/|k|^2. */
        int n = p[2];
        cplx *pen = malloc(sizeof(cplx) * (size_t)n), *w = malloc(sizeof(cplx) * (size_t)n);
        double sigma = dx[2] / PI, C1 = sigma / PI;
        double zmin = -(0.5 * (double)n) * dx[2];
        for (int k = 0; k < n; ++k) {
            double z = zmin + (double)k * dx[2];
            double rho = fabs(z) / sigma;
            pen[k] = CMPLX(K->gm ? oracle_gauss_green(1, K->gm, K->gs, z) * dx[2]
                                 : -C1 * (oracle_sine_int(rho) * rho + cos(rho)) * dx[2], 0.0);
        }
        fft_shift(pen, n);
        glassman(pen, w, n, 0);
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < p[2]; ++k)
            for (int j = 0; j < p[1]; ++j)
                for (int i = 0; i < p[0]; ++i) {
                    size_t q = ((size_t)k * p[1] + j) * p[0] + i;
                    if (i == 0 && j == 0) G[q] = pen[k];
                    else G[q] = -(K->gm ? K->zeta[q] : 1.0) /
                                 (K->ik[0][i] * K->ik[0][i] + K->ik[1][j] * K->ik[1][j] + K->ik[2][k] * K->ik[2][k]);
                }
        free(pen); free(w);
    } else if (b0 == 0 && b1 == 0 && b2 == 1) {
        /* Unbounded-unbounded-periodic (greens3d.cpp:407-474 with the 2D
         * unbounded kernel of greens2d.cpp:157-264): the kz = 0 plane is the 2D
         * transform of -(1/2pi)(Ji0(rho) + ln(2 sigma) - gamma) dx dy,
         * sigma = max(dx, dy)/pi; every other mode is 1/|k|^2. */
        int p2[3] = {p[0], p[1], 1};
        size_t n2 = (size_t)p[0] * p[1];
        cplx *G2 = malloc(sizeof(cplx) * n2);
        const double c_1_2pi = 0.5 / PI;
        double h2 = fmax(dx[0], dx[1]);
        double sigma = h2 / PI;
        double C2 = log(2.0 * sigma) - EULER_GAMMA;
        double xmin0 = -(0.5 * (double)p[0]) * dx[0], xmin1 = -(0.5 * (double)p[1]) * dx[1];
#pragma omp parallel for schedule(dynamic, 4)
        for (int j = 0; j < p[1]; ++j) {
            double y = xmin1 + (double)j * dx[1];
            for (int i = 0; i < p[0]; ++i) {
                double x = xmin0 + (double)i * dx[0];
                double r = sqrt(x * x + y * y);
                double rho = r / sigma;
                G2[(size_t)j * p[0] + i] = CMPLX(K->gm ? oracle_gauss_green(2, K->gm, K->gs, r) * dx[0] * dx[1]
                                                       : -c_1_2pi * (oracle_bessel_int_J0(rho) + C2) * dx[0] * dx[1], 0.0);
            }
        }
        transform_axis(G2, p2, 0, 1, 0);
        transform_axis(G2, p2, 1, 1, 0);
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < p[2]; ++k)
            for (int j = 0; j < p[1]; ++j)
                for (int i = 0; i < p[0]; ++i) {
                    size_t q = ((size_t)k * p[1] + j) * p[0] + i;
                    if (k == 0) G[q] = G2[(size_t)j * p[0] + i];
                    else G[q] = -(K->gm ? K->zeta[q] : 1.0) /
                                 (K->ik[0][i] * K->ik[0][i] + K->ik[1][j] * K->ik[1][j] + K->ik[2][k] * K->ik[2][k]);
                }
        free(G2);
    } else if (b0 != b1) {
        /* 2D mixed (greens2d.cpp:316-440): along the unbounded axis u the line
         * of zero wavenumber on the periodic axis is the transform of the 1D
         * kernel -(sigma/pi)(rho Si(rho) + cos rho) du, sigma = du/pi, sampled
         * at -(P_u/2) du + m du and half-swapped; every other mode is 1/|k|^2.
         * For the x-unbounded case the reference stores the samples at an index
         * it never sets (greens2d.cpp:400); the samples go to their own index. */
        const int u = b0 == 0 ? 0 : 1;
        int n = p[u];
        cplx *pen = malloc(sizeof(cplx) * (size_t)n), *w = malloc(sizeof(cplx) * (size_t)n);
        double sigma = dx[u] / PI, C1 = sigma / PI;
        double umin = -(0.5 * (double)n) * dx[u];
        for (int m = 0; m < n; ++m) {
            double s = umin + (double)m * dx[u];
            double rho = fabs(s) / sigma;
            pen[m] = CMPLX(K->gm ? oracle_gauss_green(1, K->gm, K->gs, s) * dx[u]
                                 : -C1 * (oracle_sine_int(rho) * rho + cos(rho)) * dx[u], 0.0);
        }
        fft_shift(pen, n);
        glassman(pen, w, n, 0);
        for (int j = 0; j < p[1]; ++j)
            for (int i = 0; i < p[0]; ++i) {
                size_t q = (size_t)j * p[0] + i;
                if (u == 1 ? i == 0 : j == 0) G[q] = pen[u == 1 ? j : i];
                else G[q] = -(K->gm ? K->zeta[q] : 1.0) / (K->ik[0][i] * K->ik[0][i] + K->ik[1][j] * K->ik[1][j]);
            }
        free(pen); free(w);
    } else {
        /* Periodic (greens3d.cpp:478-521): 1/|k|^2 with the zero mode removed. */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < p[2]; ++k)
            for (int j = 0; j < p[1]; ++j)
                for (int i = 0; i < p[0]; ++i) {
                    size_t q = ((size_t)k * p[1] + j) * p[0] + i;
                    if (i == 0 && j == 0 && k == 0) G[q] = CMPLX(0.0, 0.0);
                    else G[q] = -(K->gm ? K->zeta[q] : 1.0) /
                                 (K->ik[0][i] * K->ik[0][i] + K->ik[1][j] * K->ik[1][j] + K->ik[2][k] * K->ik[2][k]);
                }
    }
    return 0;
}

int oracle_greens3d(const int ncell[3], const int bc[3], const double dx[3], int reg,
                    double *g_re, double *g_im, double *zeta, int pext[3])
{
    kernel_t K;
    int st = kernel_build(&K, ncell, bc, dx, reg, 0, -1.0);
    if (st) { kernel_free(&K); return st; }
    size_t np = (size_t)K.p[0] * K.p[1] * K.p[2];
    for (int d = 0; d < 3; ++d) pext[d] = K.p[d];
    for (size_t q = 0; q < np; ++q) {
        if (g_re) g_re[q] = creal(K.G[q]);
        if (g_im) g_im[q] = cimag(K.G[q]);
        if (zeta && reg > 0) zeta[q] = K.zeta[q];
    }
    kernel_free(&K);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* setup3d + push + solve3d + pull on one rank. */
static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int oracle_solve3d(const int ncell[3], const int bc[3], const double dx[3], int reg,
                   int grad, int div, int curl, int reproject,
                   const double *bx, const double *by, const double *bz,
                   double *ax, double *ay, double *az,
                   double *rbx, double *rby, double *rbz)
{
    return oracle_solve3d_timed(ncell, bc, dx, reg, grad, div, curl, reproject, bx, by, bz, ax, ay, az,
                                rbx, rby, rbz, NULL);
}

/* setup3d/push/solve3d/pull, or with two_d setup2d/push/solve2d/pull on a
 * grid of one periodic z-plane (see kernel_build): the z transforms are then
 * of length one and ikZ = 0, so the 3D data flow is the 2D one
 * (solve2d.cpp:8-475); only the output selection differs. */
static int solve_core(const int ncell[3], const int bc[3], const double dx[3], int reg, double gauss_width,
                      int grad, int div, int curl, int reproject, int two_d,
                      const double *bx, const double *by, const double *bz,
                      double *ax, double *ay, double *az,
                      double *rbx, double *rby, double *rbz, double seconds[3])
{
    double t0 = now_s();
    const double *B[3] = {bx, by, bz};
    double *A[3] = {ax, ay, az};
    double *RB[3] = {rbx, rby, rbz};
    int r[3] = {bx != NULL, by != NULL, bz != NULL};
    int l[3] = {0, 0, 0};

    if (!two_d) {
        /* Output selection (solve3d.cpp:43-107). */
        if (grad) {
            if (!r[0]) return 3;
            l[0] = l[1] = l[2] = 1;
        } else if (div) {
            if (!(r[0] && r[1] && r[2])) return 3;
            l[0] = 1;
        } else if (curl) {
            if (!(r[0] && r[1] && r[2])) return 3;
            l[0] = l[1] = l[2] = 1;
        } else {
            for (int c = 0; c < 3; ++c) l[c] = r[c];
        }
    } else {
        /* 2D (solve2d.cpp:43-103): grad of X -> (X, Y); div of (X, Y) -> X;
         * curl of Z -> (X, Y) = (d/dy, -d/dx); no reprojection. */
        reproject = 0;
        if (grad) {
            if (!r[0]) return 3;
            l[0] = l[1] = 1;
        } else if (div) {
            if (!(r[0] && r[1])) return 3;
            l[0] = 1;
        } else if (curl) {
            if (!r[2]) return 3;
            l[0] = l[1] = 1;
        } else {
            for (int c = 0; c < 3; ++c) l[c] = r[c];
        }
    }

    kernel_t K;
    int st = kernel_build(&K, ncell, bc, dx, reg, two_d, gauss_width);
    if (st) { kernel_free(&K); return st; }
    double t1 = now_s();

    const int nx = ncell[0], ny = ncell[1], nz = ncell[2];
    const int px = K.p[0], py = K.p[1];
    const int nfft = bc[2] == 0 ? 2 * nz : nz;
    const size_t nyp = (size_t)nz * py * px;   /* y-pencil arrays [Nz][Py][Px] */
    cplx *rhs[3] = {NULL, NULL, NULL}, *lhs[3] = {NULL, NULL, NULL};
    for (int c = 0; c < 3; ++c) {
        if (r[c]) rhs[c] = calloc(nyp, sizeof(cplx));
        if (l[c]) lhs[c] = calloc(nyp, sizeof(cplx));
    }
    int lmax = px > py ? px : py;
    if (nfft > lmax) lmax = nfft;

    /* push (push.cpp:284-368): real input, x zero-padded to Px; rows j >= Ny
     * stay zero, as the x-to-y pencil map leaves them (map.cpp:376-384). */
    for (int c = 0; c < 3; ++c) {
        if (!r[c]) continue;
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    rhs[c][((size_t)k * py + j) * px + i] = CMPLX(B[c][((size_t)k * ny + j) * nx + i], 0.0);
    }

#pragma omp parallel
    {
        cplx *pen = malloc(sizeof(cplx) * (size_t)lmax), *w = malloc(sizeof(cplx) * (size_t)lmax);
        cplx *pr[3], *pl[3];
        for (int c = 0; c < 3; ++c) {
            pr[c] = malloc(sizeof(cplx) * (size_t)nfft);
            pl[c] = malloc(sizeof(cplx) * (size_t)nfft);
        }

        /* x forward (solve3d.cpp:118-173), rows j < Ny. */
        for (int c = 0; c < 3; ++c) {
            if (!r[c]) continue;
#pragma omp for collapse(2) schedule(static)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j) glassman(rhs[c] + ((size_t)k * py + j) * px, w, px, 0);
        }
        /* y forward (solve3d.cpp:183-237). */
        for (int c = 0; c < 3; ++c) {
            if (!r[c]) continue;
#pragma omp for collapse(2) schedule(static)
            for (int k = 0; k < nz; ++k)
                for (int i = 0; i < px; ++i) {
                    cplx *base = rhs[c] + (size_t)k * py * px + i;
                    for (int j = 0; j < py; ++j) pen[j] = base[(size_t)j * px];
                    glassman(pen, w, py, 0);
                    for (int j = 0; j < py; ++j) base[(size_t)j * px] = pen[j];
                }
        }

        /* z forward, spectral operation, z inverse (solve3d.cpp:243-440). */
        const cplx *ikX = K.ik[0], *ikY = K.ik[1], *ikZ = K.ik[2];
#pragma omp for collapse(2) schedule(static)
        for (int i = 0; i < px; ++i) {
            for (int j = 0; j < py; ++j) {
                for (int c = 0; c < 3; ++c) {
                    if (!r[c]) continue;
                    for (int k = 0; k < nz; ++k) pr[c][k] = rhs[c][((size_t)k * py + j) * px + i];
                    for (int k = nz; k < nfft; ++k) pr[c][k] = CMPLX(0.0, 0.0);
                    glassman(pr[c], w, nfft, 0);
                }
                /* grad reads component d, or component x where d was not pushed
                 * (2D: always x, solve2d.cpp:298-299) */
                const cplx *gY = (r[1] && !two_d) ? pr[1] : pr[0], *gZ = r[2] ? pr[2] : pr[0];
                for (int k = 0; k < nfft; ++k) {
                    size_t q = ((size_t)k * py + j) * px + i;
                    if (K.zeta && !K.gm)
                        for (int c = 0; c < 3; ++c)
                            if (r[c]) pr[c][k] *= K.zeta[q];
                    cplx G = K.G[q];
                    if (two_d) {
                        /* solve2d.cpp:292-325 */
                        if (grad) {
                            pl[0][k] = ikX[i] * G * pr[0][k];
                            pl[1][k] = ikY[j] * G * pr[0][k];
                        } else if (div) {
                            pl[0][k] = G * (ikX[i] * pr[0][k] + ikY[j] * pr[1][k]);
                        } else if (curl) {
                            pl[0][k] = ikY[j] * G * pr[2][k];
                            pl[1][k] = -ikX[i] * G * pr[2][k];
                        } else {
                            for (int c = 0; c < 3; ++c)
                                if (l[c]) pl[c][k] = G * pr[c][k];
                        }
                    } else if (grad) {
                        pl[0][k] = ikX[i] * G * pr[0][k];
                        pl[1][k] = ikY[j] * G * gY[k];
                        pl[2][k] = ikZ[k] * G * gZ[k];
                    } else if (div) {
                        pl[0][k] = G * (ikX[i] * pr[0][k] + ikY[j] * pr[1][k] + ikZ[k] * pr[2][k]);
                    } else if (curl) {
                        pl[0][k] = G * (ikY[j] * pr[2][k] - ikZ[k] * pr[1][k]);
                        pl[1][k] = G * (ikZ[k] * pr[0][k] - ikX[i] * pr[2][k]);
                        pl[2][k] = G * (ikX[i] * pr[1][k] - ikY[j] * pr[0][k]);
                    } else {
                        for (int c = 0; c < 3; ++c)
                            if (l[c]) pl[c][k] = G * pr[c][k];
                    }
                    /* the Gaussian family filters the returned right-hand side after
                     * the kernel has acted on the unfiltered one */
                    const int rp = reproject && r[0] && r[1] && r[2];
                    cplx div_psi = rp ? G * (ikX[i] * pr[0][k] + ikY[j] * pr[1][k] + ikZ[k] * pr[2][k]) : 0.0;
                    if (K.gm)
                        for (int c = 0; c < 3; ++c)
                            if (r[c]) pr[c][k] *= K.zeta[q];
                    if (rp) {
                        pr[0][k] += ikX[i] * div_psi;
                        pr[1][k] += ikY[j] * div_psi;
                        pr[2][k] += ikZ[k] * div_psi;
                    }
                }
                for (int c = 0; c < 3; ++c) {
                    if (r[c]) glassman(pr[c], w, nfft, 1);
                    if (l[c]) glassman(pl[c], w, nfft, 1);
                }
                for (int k = 0; k < nz; ++k) {
                    size_t q = ((size_t)k * py + j) * px + i;
                    for (int c = 0; c < 3; ++c) {
                        if (r[c]) rhs[c][q] = pr[c][k] / (double)nfft;
                        if (l[c]) lhs[c][q] = pl[c][k] / (double)nfft;
                    }
                }
            }
        }

        /* y inverse (solve3d.cpp:447-530). */
        for (int f = 0; f < 6; ++f) {
            cplx *a = f < 3 ? rhs[f] : lhs[f - 3];
            if (!a) continue;
#pragma omp for collapse(2) schedule(static)
            for (int k = 0; k < nz; ++k)
                for (int i = 0; i < px; ++i) {
                    cplx *base = a + (size_t)k * py * px + i;
                    for (int j = 0; j < py; ++j) pen[j] = base[(size_t)j * px];
                    glassman(pen, w, py, 1);
                    for (int j = 0; j < py; ++j) base[(size_t)j * px] = pen[j] / (double)py;
                }
        }
        /* y-to-x pencil map keeps rows j < Ny; x inverse (solve3d.cpp:541-629). */
        for (int f = 0; f < 6; ++f) {
            cplx *a = f < 3 ? rhs[f] : lhs[f - 3];
            if (!a) continue;
#pragma omp for collapse(2) schedule(static)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j) {
                    cplx *row = a + ((size_t)k * py + j) * px;
                    glassman(row, w, px, 1);
                    for (int i = 0; i < px; ++i) row[i] = row[i] / (double)px;
                }
        }
        for (int c = 0; c < 3; ++c) {
            free(pr[c]); free(pl[c]);
        }
        free(pen); free(w);
    }

    double t2 = now_s();

    /* pull (pull.cpp:327-451): real part, x cropped to Nx. */
    for (int f = 0; f < 6; ++f) {
        cplx *a = f < 3 ? lhs[f] : rhs[f - 3];
        double *out = f < 3 ? A[f] : RB[f - 3];
        if (!a || !out) continue;
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    out[((size_t)k * ny + j) * nx + i] = creal(a[((size_t)k * py + j) * px + i]);
    }

    for (int c = 0; c < 3; ++c) {
        free(rhs[c]); free(lhs[c]);
    }
    kernel_free(&K);
    if (seconds) {
        seconds[0] = t1 - t0;        /* setup3d: kernel build */
        seconds[1] = t2 - t1;        /* push + solve3d */
        seconds[2] = now_s() - t2;   /* pull */
    }
    return 0;
}

int oracle_solve3d_timed(const int ncell[3], const int bc[3], const double dx[3], int reg,
                         int grad, int div, int curl, int reproject,
                         const double *bx, const double *by, const double *bz,
                         double *ax, double *ay, double *az,
                         double *rbx, double *rby, double *rbz, double seconds[3])
{
    return solve_core(ncell, bc, dx, reg, -1.0, grad, div, curl, reproject, 0, bx, by, bz, ax, ay, az, rbx, rby, rbz,
                      seconds);
}

int oracle_solve3d_gauss(const int ncell[3], const int bc[3], const double dx[3], int reg, double width,
                         int grad, int div, int curl, int reproject,
                         const double *bx, const double *by, const double *bz,
                         double *ax, double *ay, double *az,
                         double *rbx, double *rby, double *rbz)
{
    if (!(width >= 0.0)) return 1;
    return solve_core(ncell, bc, dx, reg, width, grad, div, curl, reproject, 0, bx, by, bz, ax, ay, az, rbx, rby,
                      rbz, NULL);
}

int oracle_solve2d(const int ncell[2], const int bc[2], const double dx[2], int reg,
                   int grad, int div, int curl,
                   const double *bx, const double *by, const double *bz,
                   double *ax, double *ay, double *az,
                   double *rbx, double *rby, double *rbz)
{
    const int nc3[3] = {ncell[0], ncell[1], 1};
    const int bc3[3] = {bc[0], bc[1], 1};
    const double dx3[3] = {dx[0], dx[1], fmin(dx[0], dx[1])};
    return solve_core(nc3, bc3, dx3, reg, -1.0, grad, div, curl, 0, 1, bx, by, bz, ax, ay, az, rbx, rby, rbz, NULL);
}

int oracle_solve2d_gauss(const int ncell[2], const int bc[2], const double dx[2], int reg, double width,
                         int grad, int div, int curl,
                         const double *bx, const double *by, const double *bz,
                         double *ax, double *ay, double *az,
                         double *rbx, double *rby, double *rbz)
{
    const int nc3[3] = {ncell[0], ncell[1], 1};
    const int bc3[3] = {bc[0], bc[1], 1};
    const double dx3[3] = {dx[0], dx[1], fmin(dx[0], dx[1])};
    if (!(width >= 0.0)) return 1;
    return solve_core(nc3, bc3, dx3, reg, width, grad, div, curl, 0, 1, bx, by, bz, ax, ay, az, rbx, rby, rbz, NULL);
}

/* ------------------------------------------------------------------------ */
/* smooth3d (fortran/source/poisson_solver/poisson_solver_smooth3d.f): each
 * field zero-padded on unbounded axes, transformed along x, y, z, multiplied
 * by exp(-s^2 |k|^2 / 2) with the ik wavenumbers of greens3d.cpp:73-118,
 * transformed back, normalised by the padded size and cropped. */
int oracle_smooth3d(const int ncell[3], const int bc[3], const double dx[3], double s,
                    const double *bx, const double *by, const double *bz,
                    double *ox, double *oy, double *oz)
{
    const double *B[3] = {bx, by, bz};
    double *O[3] = {ox, oy, oz};
    int p[3];
    for (int d = 0; d < 3; ++d) {
        if (bc[d] != 0 && bc[d] != 1) return 2;
        p[d] = (bc[d] == 0 ? 2 : 1) * ncell[d];
    }
    double *k2[3];
    for (int d = 0; d < 3; ++d) {
        k2[d] = malloc(sizeof(double) * (size_t)p[d]);
        double dk = 1.0 / ((double)p[d] * dx[d]);
        for (int m = 0; m < p[d]; ++m) {
            int mm = (2 * m < p[d]) ? m : m - p[d];
            double k = 2.0 * PI * (double)mm * dk;
            k2[d][m] = k * k;
        }
    }
    size_t np = (size_t)p[0] * p[1] * p[2];
    cplx *a = malloc(sizeof(cplx) * np);
    for (int c = 0; c < 3; ++c) {
        if (!B[c] || !O[c]) continue;
        for (size_t q = 0; q < np; ++q) a[q] = CMPLX(0.0, 0.0);
        for (int k = 0; k < ncell[2]; ++k)
            for (int j = 0; j < ncell[1]; ++j)
                for (int i = 0; i < ncell[0]; ++i)
                    a[((size_t)k * p[1] + j) * p[0] + i] = CMPLX(B[c][((size_t)k * ncell[1] + j) * ncell[0] + i], 0.0);
        transform_axis(a, p, 0, 0, 0);
        transform_axis(a, p, 1, 0, 0);
        transform_axis(a, p, 2, 0, 0);
        for (int k = 0; k < p[2]; ++k)
            for (int j = 0; j < p[1]; ++j)
                for (int i = 0; i < p[0]; ++i)
                    a[((size_t)k * p[1] + j) * p[0] + i] *= exp(-0.5 * s * s * (k2[0][i] + k2[1][j] + k2[2][k]));
        transform_axis(a, p, 2, 0, 1);
        transform_axis(a, p, 1, 0, 1);
        transform_axis(a, p, 0, 0, 1);
        for (int k = 0; k < ncell[2]; ++k)
            for (int j = 0; j < ncell[1]; ++j)
                for (int i = 0; i < ncell[0]; ++i)
                    O[c][((size_t)k * ncell[1] + j) * ncell[0] + i] =
                        creal(a[((size_t)k * p[1] + j) * p[0] + i]) / (double)np;
    }
    free(a);
    for (int d = 0; d < 3; ++d) free(k2[d]);
    return 0;
}
