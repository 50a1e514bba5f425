// C ABI (include/poisson_solver_gb300.h) over ps::Solver. Every entry point
// catches the solver's exceptions and turns them into a status code plus the
// handle's last-error message; nothing propagates across the ABI.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>

#include "poisson_solver_gb300.h"
#include "ps_solver.hpp"

struct ps_solver {
    ps::Solver s;
};

namespace {

template <typename F> int guarded(ps_solver *h, F &&f)
{
    if (!h) return PS_ERR_ARGUMENT;
    try {
        ps::DeviceScope scope(h->s.device);
        f(h->s);
        h->s.last_error.clear();
        return PS_OK;
    } catch (const ps::Error &e) {
        h->s.last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc &) {
        h->s.last_error = "host allocation failed";
        return PS_ERR_MEMORY;
    } catch (const std::exception &e) {
        h->s.last_error = e.what();
        return PS_ERR_CUDA;
    }
}

}  // namespace

extern "C" {

int ps_create(ps_solver **out)
{
    if (!out) return PS_ERR_ARGUMENT;
    *out = nullptr;
    try {
        *out = new ps_solver();
    } catch (const ps::Error &e) {
        return e.status;
    } catch (...) {
        return PS_ERR_MEMORY;
    }
    return PS_OK;
}

int ps_destroy(ps_solver *h)
{
    if (!h) return PS_OK;
    ps::DeviceScope scope(h->s.device);
    if (h->s.stream) cudaStreamSynchronize(h->s.stream);
    delete h;
    return PS_OK;
}

int ps_setup3d(ps_solver *h, const int ncell[3], const int bc[3], const double dx[3], int reg_order)
{
    if (!ncell || !bc || !dx) return h ? (h->s.last_error = "NULL argument", PS_ERR_ARGUMENT) : PS_ERR_ARGUMENT;
    return guarded(h, [&](ps::Solver &s) { s.setup3d(ncell, bc, dx, reg_order); });
}

int ps_set_option(ps_solver *h, int option, int value)
{
    return guarded(h, [&](ps::Solver &s) { s.set_option(option, value); });
}

int ps_get_option(const ps_solver *h, int option, int *value)
{
    if (!value) return PS_ERR_ARGUMENT;
    return guarded(const_cast<ps_solver *>(h), [&](ps::Solver &s) { *value = s.get_option(option); });
}

int ps_push(ps_solver *h, const double *bx, const double *by, const double *bz)
{
    const double *B[3] = {bx, by, bz};
    return guarded(h, [&](ps::Solver &s) { s.push(B, cudaMemcpyHostToDevice); });
}

int ps_push_device(ps_solver *h, const double *bx, const double *by, const double *bz)
{
    const double *B[3] = {bx, by, bz};
    return guarded(h, [&](ps::Solver &s) { s.push(B, cudaMemcpyDeviceToDevice); });
}

int ps_solve3d(ps_solver *h)
{
    return guarded(h, [&](ps::Solver &s) { s.solve_internal(3); });
}

int ps_pull(ps_solver *h, double *ax, double *ay, double *az, double *bx, double *by, double *bz)
{
    double *A[3] = {ax, ay, az}, *RB[3] = {bx, by, bz};
    return guarded(h, [&](ps::Solver &s) { s.pull(A, RB, cudaMemcpyDeviceToHost); });
}

int ps_pull_device(ps_solver *h, double *ax, double *ay, double *az, double *bx, double *by, double *bz)
{
    double *A[3] = {ax, ay, az}, *RB[3] = {bx, by, bz};
    return guarded(h, [&](ps::Solver &s) { s.pull(A, RB, cudaMemcpyDeviceToDevice); });
}

int ps_solve3d_device(ps_solver *h, const double *bx, const double *by, const double *bz,
                      double *ax, double *ay, double *az)
{
    const double *B[3] = {bx, by, bz};
    double *A[3] = {ax, ay, az};
    return guarded(h, [&](ps::Solver &s) { s.solve(B, A); });
}

int ps_solve3d_device_noalloc(ps_solver *h, const double *bx, const double *by, const double *bz,
                              double *ax, double *ay, double *az)
{
    const double *B[3] = {bx, by, bz};
    double *A[3] = {ax, ay, az};
    return guarded(h, [&](ps::Solver &s) { ps::solve_noalloc(s, B, A); });
}

int ps_partition_count(const ps_solver *h) { return (h && h->s.is_setup) ? 1 : 0; }

int ps_partition(const ps_solver *h, int index, int ncell[3], int icell[3], double dx[3])
{
    if (!h) return PS_ERR_ARGUMENT;
    if (!h->s.is_setup) return PS_ERR_STATE;
    if (index != 0) return PS_ERR_ARGUMENT;
    for (int d = 0; d < 3; ++d) {
        if (ncell) ncell[d] = h->s.n[d];
        if (icell) icell[d] = 0;
        if (dx) dx[d] = h->s.dx[d];
    }
    return PS_OK;
}

int ps_setup2d(ps_solver *h, const int ncell[2], const int bc[2], const double dx[2], int reg_order)
{
    if (!ncell || !bc || !dx) return PS_ERR_ARGUMENT;
    return guarded(h, [&](ps::Solver &s) { s.setup2d(ncell, bc, dx, reg_order); });
}

int ps_solve2d(ps_solver *h)
{
    return guarded(h, [&](ps::Solver &s) { s.solve_internal(2); });
}

int ps_push_interleaved(ps_solver *h, const double *b, int ncomp, const int ext[3], const int offset[3])
{
    if (!ext || !offset) return PS_ERR_ARGUMENT;
    return guarded(h, [&](ps::Solver &s) { s.push_interleaved(b, ncomp, ext, offset, cudaMemcpyHostToDevice); });
}

int ps_pull_interleaved(ps_solver *h, double *a, int ncomp_a, double *b, int ncomp_b, const int ext[3],
                        const int offset[3])
{
    if (!ext || !offset) return PS_ERR_ARGUMENT;
    return guarded(h, [&](ps::Solver &s) {
        s.pull_interleaved(a, ncomp_a, b, ncomp_b, ext, offset, cudaMemcpyDeviceToHost);
    });
}

int ps_smooth3d(ps_solver *h, double width)
{
    return guarded(h, [&](ps::Solver &s) { s.smooth3d(width); });
}

int ps_set_kernel(ps_solver *h, int family, double width)
{
    return guarded(h, [&](ps::Solver &s) { s.set_kernel(family, width); });
}

int ps_set_stream(ps_solver *h, void *stream)
{
    return guarded(h, [&](ps::Solver &s) { s.stream = (cudaStream_t)stream; });
}

int ps_synchronize(ps_solver *h)
{
    return guarded(h, [&](ps::Solver &s) { s.synchronize(); });
}

const char *ps_last_error(const ps_solver *h) { return h ? h->s.last_error.c_str() : "NULL handle"; }

const char *ps_status_string(int status)
{
    switch (status) {
    case PS_OK: return "ok";
    case PS_ERR_ARGUMENT: return "invalid argument";
    case PS_ERR_BOUNDARY: return "unsupported boundary conditions";
    case PS_ERR_COMPONENTS: return "pushed components do not fit the output option";
    case PS_ERR_MEMORY: return "out of memory";
    case PS_ERR_CUDA: return "CUDA error";
    case PS_ERR_STATE: return "call out of order";
    case PS_ERR_UNSUPPORTED: return "unsupported";
    case PS_ERR_TIMEOUT: return "a kernel's wait for an asynchronous copy timed out";
    default: return "unknown status";
    }
}

int ps_get_info(const ps_solver *h, int what, double *value)
{
    if (!h || !value) return PS_ERR_ARGUMENT;
    const ps::Solver &s = h->s;
    switch (what) {
    case PS_INFO_PADDED_X: *value = s.P[0]; break;
    case PS_INFO_PADDED_Y: *value = s.P[1]; break;
    case PS_INFO_PADDED_Z: *value = s.P[2]; break;
    case PS_INFO_LAUNCHES_PER_SOLVE: *value = s.dims == 2 ? 3 : 5; break;
    case PS_INFO_DEVICE_BYTES: *value = (double)s.device_bytes(); break;
    case PS_INFO_KERNEL_OCTANT: *value = (double)s.Mx * s.oy * s.oz; break;
    default: return PS_ERR_ARGUMENT;
    }
    return PS_OK;
}

int ps_get_pass_times(ps_solver *h, double ms[5], int *nsolves, int reset)
{
    if (!ms) return PS_ERR_ARGUMENT;
    return guarded(h, [&](ps::Solver &s) {
        s.drain_timing();
        for (int i = 0; i < ps::Solver::NPASS; ++i) ms[i] = s.pass_ms[i];
        if (nsolves) *nsolves = s.timed_solves;
        if (reset) {
            for (double &v : s.pass_ms) v = 0.0;
            s.timed_solves = 0;
        }
    });
}

int ps_autotune(ps_solver *h, int component_mask)
{
    return guarded(h, [&](ps::Solver &s) { s.autotune(component_mask); });
}

int ps_get_pass_config(ps_solver *h, int pass, int component_mask, int *family, int *lines)
{
    if (!family || !lines) return PS_ERR_ARGUMENT;
    return guarded(h, [&](ps::Solver &s) {
        const ps::PassChoice c = s.current_choice(pass, component_mask);
        *family = c.fam == 'p'   ? PS_FAMILY_P2
                  : c.fam == 'w' ? PS_FAMILY_WIDE
                  : c.fam == 't' ? PS_FAMILY_TMEM
                  : c.fam == 'q' ? PS_FAMILY_TMA
                  : c.fam == 'c' ? PS_FAMILY_TC
                                 : PS_FAMILY_RUNTIME;
        *lines = c.B;
    });
}

int ps_get_pass_plan(ps_solver *h, int pass, int component_mask, int *radices, int capacity, int *nstages,
                     int *conv_length)
{
    if (!nstages || !conv_length || capacity < 0 || (capacity > 0 && !radices)) return PS_ERR_ARGUMENT;
    return guarded(h, [&](ps::Solver &s) {
        const ps::FftPlanDev &d = s.current_plan(pass, component_mask);
        *nstages = d.nstages;
        for (int i = 0; i < d.nstages && i < capacity; ++i) radices[i] = d.radix[i];
        *conv_length = d.blue ? d.L : d.rader ? d.rq : 0;
    });
}

int ps_get_kernel(const ps_solver *h, double *out, long long capacity)
{
    if (!out) return PS_ERR_ARGUMENT;
    return guarded(const_cast<ps_solver *>(h), [&](ps::Solver &s) { s.copy_kernel(out, capacity); });
}

}  // extern "C"
