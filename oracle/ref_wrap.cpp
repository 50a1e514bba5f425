/*
 * C entry points over the UNMODIFIED reference C++ solver (mmhej/poissonsolver,
 * c++/source), compiled single-rank against oracle/mpi_stub/mpi.h by
 * oracle/Makefile into oracle/_ref/libpsref.so.
 *
 * Test infrastructure only. It is used here to pin the oracle restatement
 * (oracle/ps_oracle.c) and to write the golden fixtures under tests/golden/.
 * Nothing in the product links or loads it.
 *
 * The reference keeps its spectral kernel in private members
 * (poisson_solver.hpp:74-82); ref_greens3d reads them by widening access for
 * this translation unit only, which changes no code of the reference.
 */
#include <cstring>
#include <complex>
#include <vector>
#include <iostream>
#include <iomanip>
#include <fstream>
#include <string>
#include "mpi.h"
#define private public
#include "poisson_solver.hpp"
#undef private

double sine_int(double);         /* special_functions.cpp:238 */
double bessel_int_J0(double);    /* special_functions.cpp:115 */

extern "C" {

/* One setup3d/push/solve3d/pull sequence (setup3d.cpp:8, push.cpp:9,
 * solve3d.cpp:8, pull.cpp:8). NULL input pointers mean "component absent";
 * NULL output pointers are not pulled. */
int ref_solve3d(const int ncell[3], const int bc[3], const double dx[3], int reg,
                int grad, int div, int curl, int reproject,
                const double *bx, const double *by, const double *bz,
                double *ax, double *ay, double *az,
                double *rbx, double *rby, double *rbz)
{
    int nc[3] = {ncell[0], ncell[1], ncell[2]};
    int b[3] = {bc[0], bc[1], bc[2]};
    double d[3] = {dx[0], dx[1], dx[2]};
    poisson_solver ps;
    ps.setup3d(nc, b, d, reg);
    if (ps.G3D == NULL) return 2;
    ps.set_return_grad(grad != 0);
    ps.set_return_div(div != 0);
    ps.set_return_curl(curl != 0);
    ps.set_reprojection(reproject != 0);
    ps.push(const_cast<double *>(bx), const_cast<double *>(by), const_cast<double *>(bz));
    ps.solve3d();
    ps.pull(ax, ay, az, rbx, rby, rbz);
    return 0;
}

/* One setup2d/push/solve2d/pull sequence (setup2d.cpp:8, push.cpp:9,
 * solve2d.cpp:8, pull.cpp:8); fields [Ny][Nx]. */
int ref_solve2d(const int ncell[2], const int bc[2], const double dx[2], int reg,
                int grad, int div, int curl,
                const double *bx, const double *by, const double *bz,
                double *ax, double *ay, double *az,
                double *rbx, double *rby, double *rbz)
{
    int nc[2] = {ncell[0], ncell[1]};
    int b[2] = {bc[0], bc[1]};
    double d[2] = {dx[0], dx[1]};
    poisson_solver ps;
    ps.setup2d(nc, b, d, reg);
    if (ps.G2D == NULL) return 2;
    ps.set_return_grad(grad != 0);
    ps.set_return_div(div != 0);
    ps.set_return_curl(curl != 0);
    ps.push(const_cast<double *>(bx), const_cast<double *>(by), const_cast<double *>(bz));
    ps.solve2d();
    ps.pull(ax, ay, az, rbx, rby, rbz);
    return 0;
}

double ref_sine_int(double x) { return sine_int(x); }
double ref_bessel_int_J0(double x) { return bessel_int_J0(x); }

/* Spectral kernel and regularisation filter as built by greens3d
 * (greens3d.cpp:9-547). Layout [Pz][Py][Px], x fastest; Pd = 2 Nd on
 * unbounded axes. zeta is written only when reg > 0. Returns the three
 * padded extents in pext. */
int ref_greens3d(const int ncell[3], const int bc[3], const double dx[3], int reg,
                 double *g_re, double *g_im, double *zeta, int pext[3])
{
    int nc[3] = {ncell[0], ncell[1], ncell[2]};
    int b[3] = {bc[0], bc[1], bc[2]};
    double d[3] = {dx[0], dx[1], dx[2]};
    poisson_solver ps;
    ps.setup3d(nc, b, d, reg);
    if (ps.G3D == NULL) return 2;
    int px = (b[0] == 0 ? 2 : 1) * nc[0];
    int py = (b[1] == 0 ? 2 : 1) * nc[1];
    int pz = (b[2] == 0 ? 2 : 1) * nc[2];
    pext[0] = px; pext[1] = py; pext[2] = pz;
    size_t n = (size_t)px * py * pz;
    for (size_t q = 0; q < n; ++q) {
        if (g_re) g_re[q] = ps.G3D[q].real();
        if (g_im) g_im[q] = ps.G3D[q].imag();
        if (zeta && reg > 0) zeta[q] = ps.zeta[q];
    }
    return 0;
}

/* One pencil transform (pencil/fft.cpp:11, pencil/ifft.cpp:11): unnormalised,
 * forward e^{-2 pi i jk/n} when dir < 0, inverse otherwise. data holds n
 * interleaved (re, im) pairs and is transformed in place. */
int ref_fft(int n, int dir, double *data)
{
    class_pencil pen(true, false, false);
    pen.resize(n);
    for (int i = 0; i < n; ++i) pen.X[i] = std::complex<double>(data[2 * i], data[2 * i + 1]);
    if (dir < 0) pen.fft(); else pen.ifft();
    for (int i = 0; i < n; ++i) { data[2 * i] = pen.X[i].real(); data[2 * i + 1] = pen.X[i].imag(); }
    return 0;
}

}  /* extern "C" */
