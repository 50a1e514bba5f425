/*
 * CPU oracle for the 3D Green's-function FFT Poisson solve: a plain-C
 * restatement of the reference algorithm (mmhej/poissonsolver, c++/source).
 *
 * TEST INFRASTRUCTURE ONLY. The tests, the smoke check and the CPU-baseline
 * leg of the benchmark call it as the checker; the product never links it.
 *
 * Parity pin: tests/test_oracle.py checks it against the reference built from
 * its own sources (oracle/_ref/libpsref.so, where the reference is present)
 * and against the golden fixtures in tests/golden/, which that build wrote.
 */
#ifndef PS_ORACLE_H
#define PS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Unnormalised general-N transform of n interleaved (re, im) pairs, in place;
 * dir < 0 forward (e^{-2 pi i jk/n}), dir > 0 inverse. */
int oracle_fft(int n, int dir, double *data);

/* OpenMP threads the solves and kernel builds share their pencils over
 * (n <= 0: one a core); results do not depend on it. */
void oracle_set_threads(int n);
int oracle_threads(void);

/* Sine integral Si(x) and the integral of (1 - J0(t))/t from 0 to x, as the
 * reference evaluates them. */
double oracle_sine_int(double x);
double oracle_bessel_int_J0(double x);

/* Spectral kernel G and filter zeta on the padded grid [Pz][Py][Px]
 * (x fastest). Returns 0, or 2 for an unsupported boundary-condition
 * combination. pext receives (Px, Py, Pz). zeta is written when reg > 0. */
int oracle_greens3d(const int ncell[3], const int bc[3], const double dx[3], int reg,
                    double *g_re, double *g_im, double *zeta, int pext[3]);

/* Full setup3d / push / solve3d / pull. Real fields are [Nz][Ny][Nx], x
 * fastest. NULL inputs are absent components; NULL outputs are not written;
 * outputs for components the solve does not produce are left untouched.
 * Returns 0, 2 (boundary conditions) or 3 (components missing for the
 * requested output option, as the reference rejects them). */
int oracle_solve3d(const int ncell[3], const int bc[3], const double dx[3], int reg,
                   int grad, int div, int curl, int reproject,
                   const double *bx, const double *by, const double *bz,
                   double *ax, double *ay, double *az,
                   double *rbx, double *rby, double *rbz);

/* As oracle_solve3d, also returning wall seconds of the kernel build
 * (seconds[0]), push + solve (seconds[1]) and pull (seconds[2]). */
int oracle_solve3d_timed(const int ncell[3], const int bc[3], const double dx[3], int reg,
                         int grad, int div, int curl, int reproject,
                         const double *bx, const double *by, const double *bz,
                         double *ax, double *ay, double *az,
                         double *rbx, double *rby, double *rbz, double seconds[3]);

/* Full setup2d / push / solve2d / pull (solve2d.cpp:8-475). Real fields are
 * [Ny][Nx], x fastest; X, Y, Z as in the reference (grad of X -> X, Y; div
 * of X, Y -> X; curl of Z -> X, Y). Returns 0, 2 or 3 as oracle_solve3d. */
int oracle_solve2d(const int ncell[2], const int bc[2], const double dx[2], int reg,
                   int grad, int div, int curl,
                   const double *bx, const double *by, const double *bz,
                   double *ax, double *ay, double *az,
                   double *rbx, double *rby, double *rbz);

/* Gaussian smoothing of up to three fields [Nz][Ny][Nx] by
 * exp(-s^2 |k|^2 / 2) on the (zero-padded) solver grid. */
int oracle_smooth3d(const int ncell[3], const int bc[3], const double dx[3], double s,
                    const double *bx, const double *by, const double *bz,
                    double *ox, double *oy, double *oz);

/* Gaussian-regularised kernel family (an extension with no reference
 * counterpart): the d-dimensional (dim = 1, 2, 3) free-space kernel of order
 * 2m and width s at distance r, whose spectrum is zeta_m(s|k|)/|k|^2. */
double oracle_gauss_green(int dim, int m, double s, double r);

/* oracle_solve3d / oracle_solve2d with the Gaussian family of order
 * max(2, reg rounded up to even) and width `width` (0: twice the largest cell
 * size); the returned right-hand side is filtered by zeta_m. Returns 1 for a
 * negative width, else as oracle_solve3d. */
int oracle_solve3d_gauss(const int ncell[3], const int bc[3], const double dx[3], int reg, double width,
                         int grad, int div, int curl, int reproject,
                         const double *bx, const double *by, const double *bz,
                         double *ax, double *ay, double *az,
                         double *rbx, double *rby, double *rbz);
int oracle_solve2d_gauss(const int ncell[2], const int bc[2], const double dx[2], int reg, double width,
                         int grad, int div, int curl,
                         const double *bx, const double *by, const double *bz,
                         double *ax, double *ay, double *az,
                         double *rbx, double *rby, double *rbz);

#ifdef __cplusplus
}
#endif

#endif
