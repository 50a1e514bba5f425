// Green's-kernel construction on the GPU, all in FP64. The solver samples the
// real-space kernel of the domain on one octant of the padded grid (the
// kernel is even in every axis), transforms it with the same pass kernels as
// the solve, and folds the regularisation filter and the inverse-transform
// normalisation into one real octant K = G zeta / (Px Py Pz).
#include <cuda_runtime.h>
#include <math.h>

#include "ps_types.hpp"

namespace ps {

namespace {

constexpr double PI = 3.1415926535897932;
constexpr double EULER_GAMMA = 0.5772156649015329;

struct cd { double x, y; };
__device__ __forceinline__ cd cd_add(cd a, cd b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cd cd_mul(cd a, cd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
// complex quotient by Smith's method
__device__ __forceinline__ cd cd_div(cd a, cd b)
{
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, den = b.x + b.y * r;
        return {(a.x + a.y * r) / den, (a.y - a.x * r) / den};
    }
    const double r = b.x / b.y, den = b.x * r + b.y;
    return {(a.x * r + a.y) / den, (a.y * r - a.x) / den};
}

// Sine integral by the method of Numerical Recipes' cisi (Press et al., 2nd
// ed.): modified-Lentz continued fraction of E1(it) for t > 2, interleaved
// Si/Ci power series below, both stopped at relative change 1e-10 (the
// tolerance and switch point of the reference, special_functions.cpp:238-352,
// so the kernel carries the same truncation).
__device__ double sine_int(double x)
{
    const double eps = 1.0e-10, fpmin = 1.0e-30, fpmax = 1.0e30, tmin = 2.0;
    const int maxit = 1000;
    const double t = fabs(x);
    double ans;
    if (t == 0.0) return 0.0;
    if (t > tmin) {
        cd b = {1.0, t}, c = {fpmax, 0.0};
        cd d = cd_div({1.0, 0.0}, b), h = d;
        double err = 1.0;
        for (int i = 2; i < maxit && err > eps; ++i) {
            const double a = -(double)(i - 1) * (double)(i - 1);
            b.x += 2.0;
            d = cd_div({1.0, 0.0}, cd_add({a * d.x, a * d.y}, b));
            c = cd_add(b, cd_div({a, 0.0}, c));
            const cd del = cd_mul(c, d);
            h = cd_mul(h, del);
            err = fabs(del.x - 1.0) + fabs(del.y);
        }
        double s, co;
        sincos(t, &s, &co);
        h = cd_mul({co, -s}, h);
        ans = 0.5 * PI + h.y;
    } else {
        double sums = 0.0;
        if (t < sqrt(fpmin)) {
            sums = t;
        } else {
            double sum = 0.0, sumc = 0.0, sign = 1.0, fact = 1.0, err = 1.0;
            bool odd = true;
            for (int k = 1; k <= maxit && err > eps; ++k) {
                fact = fact * t / k;
                const double term = fact / k;
                sum = sum + sign * term;
                err = term / fabs(sum);
                if (odd) { sign = -sign; sums = sum; sum = sumc; }
                else { sumc = sum; sum = sums; }
                odd = !odd;
            }
        }
        ans = sums;
    }
    return x < 0.0 ? -ans : ans;
}

// Integral of (1 - J0(t))/t over [0, x]: Chebyshev expansions of Y. L. Luke,
// "Mathematical functions and their approximations" (1975), Table 9.3 -- an
// even series in T_2n(x/8) below 8 and a complex series in T_n(10/x - 1)
// times the asymptotic phase above (the form special_functions.cpp:115-229
// evaluates). The coefficients are Luke's published values.
__constant__ double c_luke_small[18] = {
    1.35105091918187636388,  0.83791030734868376979, -0.35047963978529462711,
    0.12777415867753198659, -0.02981035698255560990,  0.00455219841169387328,
   -0.00048408621967185359,  0.00003780202859916883, -0.00000225886908506771,
    0.00000010664609068423, -0.00000000408005443149,  0.00000000012909996251,
   -0.00000000000343577839,  0.00000000000007799552, -0.00000000000000152842,
    0.00000000000000002612, -0.00000000000000000039,  0.00000000000000000001};
__constant__ double c_luke_large[39][2] = {
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

__device__ double bessel_int_j0(double x)
{
    if (x < 8.0) {
        const double x8 = 0.125 * x;
        double t0 = 1.0, t1 = x8, ans = c_luke_small[0];
        for (int i = 2; i < 36; ++i) {
            const double t2 = 2.0 * x8 * t1 - t0;
            if ((i & 1) == 0) ans += c_luke_small[i / 2] * t2;
            t0 = t1;
            t1 = t2;
        }
        return ans;
    }
    const double u = 10.0 / x - 1.0;
    double t0 = 1.0, t1 = u;
    double sr = c_luke_large[0][0] + c_luke_large[1][0] * t1;
    double si = c_luke_large[0][1] + c_luke_large[1][1] * t1;
    for (int i = 2; i < 39; ++i) {
        const double t2 = 2.0 * u * t1 - t0;
        t0 = t1;
        t1 = t2;
        sr += c_luke_large[i][0] * t2;
        si += c_luke_large[i][1] * t2;
    }
    const double ph = x + 0.25 * PI;
    const double fac = cos(ph) * sr - sin(ph) * si;
    return sqrt(2.0 / (PI * x)) / x * fac + EULER_GAMMA + log(0.5 * x);
}

// ---------------------------------------------------------------------------
// Gaussian-regularised family of order 2m and width s (an extension with no
// counterpart in the reference). Its spectrum is zeta_m(s|k|)/|k|^2 with the
// reference's filter zeta_m(k) = e^{-a} sum_{n<m} a^n/n!, a = s^2 k^2/2, so
// in d dimensions G = G_0 + sum_{n=1}^{m-1} G_n, where G_0 is the potential of
// a unit Gaussian of width s and, with u = r^2/(2 s^2),
//   G_n(r) = s^{2-d} / (2 (2 pi)^{d/2}) e^{-u} L^{(d/2-1)}_{n-1}(u) / n
// (generalised Laguerre polynomials). G_0 is erf(r/(sqrt2 s))/(4 pi r) in 3D,
// -(ln r + E1(u)/2)/(2 pi) in 2D and -|z| erf(|z|/(sqrt2 s))/2 -
// s e^{-u}/sqrt(2 pi) in 1D, each tending to the free-space kernel at
// infinity with no added constant.

// sum_{n=1}^{m-1} L^{(alpha)}_{n-1}(u) / n by the three-term recurrence
// (k+1) L_{k+1} = (2k+1+alpha-u) L_k - (k+alpha) L_{k-1}.
__device__ double laguerre_tail(int m, double alpha, double u)
{
    double s = 0.0, lp = 0.0, l = 1.0;
    for (int n = 1; n <= m - 1; ++n) {
        s += l / (double)n;
        const double k = (double)(n - 1);
        const double nx = ((2.0 * k + 1.0 + alpha - u) * l - (k + alpha) * lp) / (k + 1.0);
        lp = l;
        l = nx;
    }
    return s;
}

// sum_{k>=1} (-u)^k / (k k!), the power series of -gamma - ln u - E1(u).
__device__ double e1_series(double u)
{
    double term = 1.0, sum = 0.0;
    for (int k = 1; k < 80; ++k) {
        term *= -u / (double)k;
        const double d = term / (double)k;
        sum += d;
        if (fabs(d) <= 1e-17 * fabs(sum)) break;
    }
    return sum;
}

// ln r + E1(r^2/(2 s^2))/2. For u <= 1 by the series, written so that ln r
// cancels analytically (the value at r = 0 is (ln(2 s^2) - gamma)/2); above,
// E1 by the continued fraction e^{-u}/(u+1- 1/(u+3- 4/(u+5- ...))) evaluated
// with the modified Lentz method.
__device__ double log_e1_half(double r, double s)
{
    const double u = 0.5 * (r / s) * (r / s);
    if (u <= 1.0) return 0.5 * (log(2.0 * s * s) - EULER_GAMMA - e1_series(u));
    double b = u + 1.0, c = 1.0e300, d = 1.0 / b, h = d;
    for (int i = 1; i < 300; ++i) {
        const double an = -(double)i * (double)i;
        b += 2.0;
        d = 1.0 / (an * d + b);
        c = b + an / c;
        const double del = c * d;
        h *= del;
        if (fabs(del - 1.0) < 1e-16) break;
    }
    return log(r) + 0.5 * h * exp(-u);
}

__device__ double gauss_green3(double r, int m, double s)
{
    const double u = 0.5 * (r / s) * (r / s);
    const double inv_2pi_32 = 1.0 / ((2.0 * PI) * sqrt(2.0 * PI));
    const double g0 = r > 0.0 ? erf(r / (sqrt(2.0) * s)) / (4.0 * PI * r) : inv_2pi_32 / s;
    return g0 + 0.5 * inv_2pi_32 / s * exp(-u) * laguerre_tail(m, 0.5, u);
}

__device__ double gauss_green2(double r, int m, double s)
{
    const double u = 0.5 * (r / s) * (r / s);
    return -log_e1_half(r, s) / (2.0 * PI) + exp(-u) * laguerre_tail(m, 0.0, u) / (4.0 * PI);
}

__device__ double gauss_green1(double z, int m, double s)
{
    const double a = fabs(z), u = 0.5 * (a / s) * (a / s);
    const double c = s / sqrt(2.0 * PI);
    return -0.5 * a * erf(a / (sqrt(2.0) * s)) - c * exp(-u) + 0.5 * c * exp(-u) * laguerre_tail(m, -0.5, u);
}

// 3D unbounded kernel, spectrally truncated: G(r) = Si(r/sigma)/(2 pi^2 r) dV,
// sigma = h/pi, h = max dx; 1/(2 pi^2 sigma) dV at the origin
// (greens3d.cpp:193-225). Octant index i' is the half-swapped grid index, so
// the sample sits at x = -(P/2) dx + (i' + P/2) dx as the reference forms it.
// With gf.gm >= 1 the samples are the Gaussian family's gauss_green3 dV.
__global__ void k_sample_unbounded3d(double *oct, int ox, int oy, int oz, int P0, int P1, int P2,
                                     double dx0, double dx1, double dx2, GaussFamily gf)
{
    const long long n = (long long)ox * oy * oz;
    const double h = fmax(fmax(dx0, dx1), dx2);
    const double sigma = h / PI;
    const double c = 0.5 / (PI * PI);
    const double xmin0 = -(0.5 * (double)P0) * dx0, xmin1 = -(0.5 * (double)P1) * dx1,
                 xmin2 = -(0.5 * (double)P2) * dx2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % ox), j = (int)((q / ox) % oy), k = (int)(q / ((long long)ox * oy));
        const double x = xmin0 + (double)(i + P0 / 2) * dx0;
        const double y = xmin1 + (double)(j + P1 / 2) * dx1;
        const double z = xmin2 + (double)(k + P2 / 2) * dx2;
        const double r = sqrt(x * x + y * y + z * z);
        double g;
        if (gf.gm > 0) g = gauss_green3(r, gf.gm, gf.gs) * dx0 * dx1 * dx2;
        else if (r > 0.25 * dx0) g = c * sine_int(r / sigma) / r * dx0 * dx1 * dx2;
        else g = c / sigma * dx0 * dx1 * dx2;
        oct[q] = g;
    }
}

// 2D unbounded kernel -(1/2 pi)(Ji0(r/sigma) + ln(2 sigma) - gamma) dx dy,
// sigma = max(dx, dy)/pi (greens2d.cpp:157-202); with gf.gm >= 1 the
// Gaussian family's gauss_green2 dx dy.
__global__ void k_sample_unbounded2d(double *oct, int ox, int oy, int P0, int P1, double dx0, double dx1,
                                     GaussFamily gf)
{
    const long long n = (long long)ox * oy;
    const double sigma = fmax(dx0, dx1) / PI;
    const double C2 = log(2.0 * sigma) - EULER_GAMMA;
    const double c = 0.5 / PI;
    const double xmin0 = -(0.5 * (double)P0) * dx0, xmin1 = -(0.5 * (double)P1) * dx1;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % ox), j = (int)(q / ox);
        const double x = xmin0 + (double)(i + P0 / 2) * dx0;
        const double y = xmin1 + (double)(j + P1 / 2) * dx1;
        const double r = sqrt(x * x + y * y);
        oct[q] = gf.gm > 0 ? gauss_green2(r, gf.gm, gf.gs) * dx0 * dx1 : -c * (bessel_int_j0(r / sigma) + C2) * dx0 * dx1;
    }
}

// Spectrum of the 1D free-space kernel of the periodic-periodic-unbounded
// domain, -(sigma/pi)(rho Si(rho) + cos rho) dz with rho = |z|/sigma,
// sigma = dz/pi (greens3d.cpp:361-373), sampled at z = -(Pz/2) dz + k dz and
// half-swapped. The samples are even, so the transform is the real cosine sum
// G1[k] = g0 + (-1)^k g_{P/2} + 2 sum_{0<m<P/2} g_m cos(2 pi k m / P).
// With gf.gm >= 1 the samples are the Gaussian family's gauss_green1 dz.
__global__ void k_line_ppf(double *line, int P, double dz, GaussFamily gf)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > P / 2) return;
    const double sigma = dz / PI, C1 = sigma / PI;
    const double zmin = -(0.5 * (double)P) * dz;
    auto g = [&](int m) {
        const double z = zmin + (double)(m + P / 2) * dz;
        if (gf.gm > 0) return gauss_green1(z, gf.gm, gf.gs) * dz;
        const double rho = fabs(z) / sigma;
        return -C1 * (sine_int(rho) * rho + cos(rho)) * dz;
    };
    double acc = g(0) + ((k & 1) ? -1.0 : 1.0) * g(P / 2);
    for (int m = 1; m < P / 2; ++m) {
        const long long e = ((long long)k * m) % P;
        acc += 2.0 * g(m) * cospi(2.0 * (double)e / (double)P);
    }
    line[k] = acc;
}

__device__ __forceinline__ double wn(int m, int P, double dx)
{
    // signed wavenumber as greens3d.cpp:78-118 forms it: 2 pi m / (P dx), m wrapped at P/2
    const int mm = (2 * m < P) ? m : m - P;
    const double dk = 1.0 / ((double)P * dx);
    return 2.0 * PI * (double)mm * dk;
}

__global__ void k_kernel_fill(const KernelFillArgs a)
{
    const long long n = (long long)a.Mx * a.oy * a.oz;
    const double h = fmax(fmax(a.dx[0], a.dx[1]), a.dx[2]);
    const double sigma = 2.0 * h;
    const int r = (a.reg % 2 != 0) ? a.reg + 1 : a.reg;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int kx = (int)(q % a.Mx), ky = (int)((q / a.Mx) % a.oy), kz = (int)(q / ((long long)a.Mx * a.oy));
        const double fx = wn(kx, a.P[0], a.dx[0]), fy = wn(ky, a.P[1], a.dx[1]), fz = wn(kz, a.P[2], a.dx[2]);
        const double k2 = fx * fx + fy * fy + fz * fz;
        // zeta_m(s |k|) of the Gaussian family: the spectral part of its kernel and its RHS filter
        double zg = 1.0;
        if (a.gauss.gm > 0) {
            const double arg = 0.5 * a.gauss.gs * a.gauss.gs * k2;
            double t = 1.0, sum = 1.0;
            for (int m = 1; m <= a.gauss.gm - 1; ++m) {
                t *= arg / (double)m;
                sum += t;
            }
            zg = sum * exp(-arg);
        }
        const double inv = zg / k2;
        double g = 0.0;
        if (a.kern) {
            switch (a.kind) {
            case 0: g = a.spec[((long long)kz * a.P[1] + ky) * a.Mx + kx].x; break;
            case 1: g = (kx == 0 && ky == 0) ? a.line[kz] : inv; break;
            case 2: g = (kz == 0) ? a.plane[(long long)ky * a.Mx + kx].x : inv; break;
            // 2D mixed (greens2d.cpp:316-440): the zero-wavenumber line of the periodic axis
            case 4: g = (kx == 0) ? a.line[ky] : inv; break;  // x periodic, y unbounded
            case 5: g = (ky == 0) ? a.line[kx] : inv; break;  // x unbounded, y periodic
            default: g = (kx == 0 && ky == 0 && kz == 0) ? 0.0 : inv; break;
            }
        }
        // zeta = e^{-a} sum_{n < r/2} a^n / n!, a = sigma^2 |k|^2 / 2 (greens3d.cpp:123-159);
        // the smooth3d filter e^{-s^2 |k|^2 / 2} (poisson_solver_smooth3d.f:205-212)
        double zeta = 1.0;
        if (a.smooth) {
            zeta = exp(-0.5 * a.smooth_sigma * a.smooth_sigma * k2);
        } else if (a.gauss.gm > 0) {
            // the family's kernel carries its regularisation; zeta filters the returned RHS
            if (a.kern) a.kern[q] = g / a.norm;
            if (a.zeta_out) a.zeta_out[q] = zg / a.norm;
            continue;
        } else if (a.reg > 0) {
            const double arg = 0.5 * sigma * sigma * k2;
            double c = 1.0, p = 1.0, sum = 1.0;
            for (int m = 1; m <= r / 2 - 1; ++m) {
                c = c * 1.0 / (double)m;
                p = p * arg;
                sum += c * p;
            }
            zeta = sum * exp(-arg);
        }
        if (a.kern) a.kern[q] = g * zeta / a.norm;
        if (a.zeta_out) a.zeta_out[q] = zeta / a.norm;
    }
}

__global__ void k_to_fp32(const double *in, float *out, size_t n)
{
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        out[q] = (float)in[q];
}

// double -> double-float (hi, lo) pairs: hi = fl(x), lo = fl(x - hi)
__global__ void k_to_df(const double *in, float2 *out, size_t n)
{
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const double x = in[q];
        const float hi = __double2float_rn(x);
        out[q] = make_float2(hi, __double2float_rn(x - (double)hi));
    }
}

unsigned grid_for(long long n, int threads)
{
    long long g = (n + threads - 1) / threads;
    if (g > 152LL * 64) g = 152LL * 64;
    return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace

cudaError_t launch_sample_unbounded3d(double *oct, const int oext[3], const int P[3], const double dx[3],
                                      GaussFamily gf, cudaStream_t st)
{
    const long long n = (long long)oext[0] * oext[1] * oext[2];
    k_sample_unbounded3d<<<grid_for(n, 256), 256, 0, st>>>(oct, oext[0], oext[1], oext[2], P[0], P[1], P[2], dx[0],
                                                             dx[1], dx[2], gf);
    return cudaGetLastError();
}

cudaError_t launch_sample_unbounded2d(double *oct, const int oext[2], const int P[2], const double dx[2],
                                      GaussFamily gf, cudaStream_t st)
{
    const long long n = (long long)oext[0] * oext[1];
    k_sample_unbounded2d<<<grid_for(n, 256), 256, 0, st>>>(oct, oext[0], oext[1], P[0], P[1], dx[0], dx[1], gf);
    return cudaGetLastError();
}

cudaError_t launch_line_ppf(double *line, int P, double dz, GaussFamily gf, cudaStream_t st)
{
    const int n = P / 2 + 1;
    k_line_ppf<<<(n + 127) / 128, 128, 0, st>>>(line, P, dz, gf);
    return cudaGetLastError();
}

cudaError_t launch_kernel_fill(const KernelFillArgs &a, cudaStream_t st)
{
    const long long n = (long long)a.Mx * a.oy * a.oz;
    k_kernel_fill<<<grid_for(n, 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_to_fp32(const double *in, float *out, size_t n, cudaStream_t st)
{
    k_to_fp32<<<grid_for((long long)n, 256), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_to_df(const double *in, float2 *out, size_t n, cudaStream_t st)
{
    k_to_df<<<grid_for((long long)n, 256), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

// 32 x 32 (x, z) tiles of one y row through shared memory: reads along x,
// writes along z, both coalesced.
__global__ void k_kernel_zfast(const double *__restrict__ kern, float *__restrict__ out, int Mx, int oy, int oz,
                               int kzp)
{
    __shared__ float tile[32][33];
    const int y = blockIdx.z, x0 = blockIdx.x * 32, z0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int z = z0 + r, x = x0 + threadIdx.x;
        tile[r][threadIdx.x] = (z < oz && x < Mx) ? (float)kern[((long long)z * oy + y) * Mx + x] : 0.f;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int x = x0 + r, z = z0 + threadIdx.x;
        if (x < Mx && z < kzp) out[((long long)y * Mx + x) * kzp + z] = tile[threadIdx.x][r];
    }
}

cudaError_t launch_kernel_zfast(const double *kern, float *out, int Mx, int oy, int oz, int kzp, cudaStream_t st)
{
    const dim3 grid((unsigned)((Mx + 31) / 32), (unsigned)((kzp + 31) / 32), (unsigned)oy);
    k_kernel_zfast<<<grid, dim3(32, 8), 0, st>>>(kern, out, Mx, oy, oz, kzp);
    return cudaGetLastError();
}

}  // namespace ps
