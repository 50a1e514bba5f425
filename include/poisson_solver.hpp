/*
 * poisson_solver.hpp -- drop-in for the reference solver class
 * (mmhej/poissonsolver, c++/source/poisson_solver.hpp:39-124 and
 * class_partition.hpp:29-43), implemented header-only over the C ABI in
 * poisson_solver_gb300.h.
 *
 * Client code written against the reference (construct, setup3d,
 * set_return_*, push, solve3d, pull, read partition[rank]) compiles unchanged
 * and links against libps_gb300.so instead of libpoissonsolver.a. As in the
 * reference, errors are reported on std::cerr and the call returns; the
 * status of the last call is also available from last_status().
 *
 * Differences a client can observe:
 *   - One GPU holds the whole grid: `partition` has one entry (icell = 0).
 *     Client code that indexes partition[rank] with rank 0 works as before.
 *   - No MPI is needed or used. Clients that call MPI themselves keep doing so.
 */
#ifndef GB300_POISSON_SOLVER_HPP
#define GB300_POISSON_SOLVER_HPP

#include <stdlib.h>

#include <cmath>
#include <complex>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "poisson_solver_gb300.h"

class class_partition
{
public:
    int ncell[3];
    int icell[3];
    double dx[3];
};

class poisson_solver
{
private:
    ps_solver *h_ = NULL;
    int status_ = PS_OK;

    bool report(int st, const char *where)
    {
        status_ = st;
        if (st != PS_OK) {
            const char *msg = h_ ? ps_last_error(h_) : ps_status_string(st);
            std::cerr << " [poisson_solver." << where << "]: " << (msg && *msg ? msg : ps_status_string(st))
                      << std::endl;
            return false;
        }
        return true;
    }

    void fill_partition()
    {
        const int n = ps_partition_count(h_);
        for (int i = 0; i < n; ++i) {
            class_partition p;
            ps_partition(h_, i, p.ncell, p.icell, p.dx);
            partition.push_back(p);
        }
    }

public:
    std::vector<class_partition> partition;

    poisson_solver(void) { report(ps_create(&h_), "constructor"); }
    ~poisson_solver(void)
    {
        if (h_) ps_destroy(h_);
    }
    poisson_solver(const poisson_solver &) = delete;
    poisson_solver &operator=(const poisson_solver &) = delete;

    void setup2d(int ncell[2], int bc[2], double dx[2], int reg_order = 0)
    {
        partition.clear();
        if (!report(ps_setup2d(h_, ncell, bc, dx, reg_order), "setup2d")) return;
        fill_partition();
    }

    void setup3d(int ncell[3], int bc[3], double dx[3], int reg_order = 0)
    {
        partition.clear();
        if (!report(ps_setup3d(h_, ncell, bc, dx, reg_order), "setup3d")) return;
        fill_partition();
    }

    void set_return_grad(bool toggle) { report(ps_set_option(h_, PS_OPT_GRAD, toggle ? 1 : 0), "set_return_grad"); }
    void set_return_div(bool toggle) { report(ps_set_option(h_, PS_OPT_DIV, toggle ? 1 : 0), "set_return_div"); }
    void set_return_curl(bool toggle) { report(ps_set_option(h_, PS_OPT_CURL, toggle ? 1 : 0), "set_return_curl"); }
    void set_reprojection(bool toggle)
    {
        report(ps_set_option(h_, PS_OPT_REPROJECT, toggle ? 1 : 0), "set_reprojection");
    }

    void solve2d() { report(ps_solve2d(h_), "solve2d"); }
    void solve3d() { report(ps_solve3d(h_), "solve3d"); }

    void push(double *bx, double *by, double *bz) { report(ps_push(h_, bx, by, bz), "push"); }
    void pull(double *ax, double *ay, double *az, double *bx = NULL, double *by = NULL, double *bz = NULL)
    {
        report(ps_pull(h_, ax, ay, az, bx, by, bz), "pull");
    }

    /* Extensions beyond the reference interface. */
    void set_precision(int precision) { report(ps_set_option(h_, PS_OPT_PRECISION, precision), "set_precision"); }
    void set_kernel(int family, double width = 0.0) { report(ps_set_kernel(h_, family, width), "set_kernel"); }
    void smooth3d(double width) { report(ps_smooth3d(h_, width), "smooth3d"); }
    /* One array holding ncomp components interleaved (component fastest),
     * allocated extents ext[3] (x, y, z), field box at offset[3]
     * (poisson_solver_push.f / poisson_solver_pull.f). */
    void push_interleaved(const double *b, int ncomp, const int ext[3], const int offset[3])
    {
        report(ps_push_interleaved(h_, b, ncomp, ext, offset), "push_interleaved");
    }
    void pull_interleaved(double *a, int ncomp_a, double *b, int ncomp_b, const int ext[3], const int offset[3])
    {
        report(ps_pull_interleaved(h_, a, ncomp_a, b, ncomp_b, ext, offset), "pull_interleaved");
    }
    int last_status() const { return status_; }
    ps_solver *handle() { return h_; }
};

#endif
