/*
 * poisson_solver_gb300.h -- C ABI of the GB300-native Green's-function FFT
 * Poisson solver (solves lap(A) = -B on 3D unbounded, periodic and mixed
 * unbounded/periodic domains, optionally returning grad, div or curl of A).
 *
 * The entry points replace the public C++ interface of the reference solver
 * (mmhej/poissonsolver, c++/source/poisson_solver.hpp:107-122); each one names
 * the member it stands for. include/poisson_solver.hpp re-creates that class
 * on top of this ABI so existing client code compiles unchanged.
 *
 * Conventions
 *   - Plain pointers and sizes only. Real fields are double arrays of
 *     Nx*Ny*Nz values laid out [Nz][Ny][Nx] (x fastest), index (k*Ny + j)*Nx + i,
 *     exactly as the reference's push/pull take them.
 *   - Boundary conditions per axis: 0 = unbounded (free space), 1 = periodic.
 *     Supported combinations, as in the reference: (0,0,0), (1,1,1),
 *     (1,1,0) and (0,0,1).
 *   - Every call returns a PS_* status; ps_last_error() gives the message of
 *     the last failure on a handle. No call exits the process.
 *   - A handle is not thread-safe; use one handle per host thread.
 *   - All GPU work runs on the handle's stream (default: the legacy stream).
 */
#ifndef POISSON_SOLVER_GB300_H
#define POISSON_SOLVER_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ps_solver ps_solver;

/* Status codes. */
enum {
    PS_OK = 0,
    PS_ERR_ARGUMENT = 1,    /* bad pointer, size or option value */
    PS_ERR_BOUNDARY = 2,    /* unsupported boundary-condition combination */
    PS_ERR_COMPONENTS = 3,  /* pushed components do not fit the output option */
    PS_ERR_MEMORY = 4,      /* device or host allocation failed */
    PS_ERR_CUDA = 5,        /* a CUDA call failed */
    PS_ERR_STATE = 6,       /* call out of order (e.g. solve before setup/push) */
    PS_ERR_UNSUPPORTED = 7, /* outside what the library implements (e.g. a padded
                               transform length above 8192) */
    PS_ERR_TIMEOUT = 8      /* a kernel's bounded wait for an asynchronous copy ran
                               out (reported by the next synchronising call:
                               ps_pull, ps_pull_device, ps_synchronize) */
};

/* Options for ps_set_option. */
enum {
    PS_OPT_GRAD = 0,       /* value 0/1: return grad A   (set_return_grad, settings.cpp:9)  */
    PS_OPT_DIV = 1,        /* value 0/1: return div A    (set_return_div, settings.cpp:15)  */
    PS_OPT_CURL = 2,       /* value 0/1: return curl A   (set_return_curl, settings.cpp:21) */
    PS_OPT_REPROJECT = 3,  /* value 0/1: reproject the returned B (set_reprojection, settings.cpp:26) */
    PS_OPT_PRECISION = 4,  /* PS_PREC_FP64 (default), PS_PREC_FP32 or PS_PREC_DF64 transforms */
    PS_OPT_PASS_TIMING = 5 /* value 0/1: time each pass of every solve with CUDA events */
};

enum {
    PS_PREC_FP64 = 0,  /* all transforms and the spectral operation in FP64 */
    PS_PREC_FP32 = 1,  /* FP64 kernel build, FP32 transforms, FP64 field I/O */
    PS_PREC_DF64 = 2   /* FP64 kernel build, transforms in double-float arithmetic (pairs of FP32
                          numbers, about 48 bits: FP64-class accuracy, FP32's exponent range), FP64
                          field I/O; no reference counterpart */
};

/* Kernel families for ps_set_kernel. */
enum {
    PS_KERNEL_SPECTRAL = 0, /* the reference's kernels (greens3d.cpp, greens2d.cpp):
                               spectrally truncated free-space parts, times the
                               regularisation filter zeta of reg_order */
    PS_KERNEL_GAUSSIAN = 1  /* extension: Gaussian-regularised kernels whose
                               spectrum is zeta_m(s |k|) / |k|^2 exactly, sampled in
                               real space on unbounded axes (erf in 3D, E1 in 2D,
                               erf in 1D, plus Laguerre terms for m > 1) */
};

/* Constructor / destructor: poisson_solver::poisson_solver / ~poisson_solver
 * (poisson_solver.hpp:107-108). ps_create binds the handle to the current
 * CUDA device. */
int ps_create(ps_solver **out);
int ps_destroy(ps_solver *h);

/* poisson_solver::setup3d(int ncell[3], int bc[3], double dx[3], int reg_order)
 * (poisson_solver.hpp:111, setup3d.cpp:8-71): grid of ncell cells of size dx,
 * boundary conditions bc, regularisation order reg_order (0 = none; odd orders
 * round up to the next even one). Builds the spectral kernel on the GPU. */
int ps_setup3d(ps_solver *h, const int ncell[3], const int bc[3], const double dx[3], int reg_order);

/* set_return_grad / set_return_div / set_return_curl / set_reprojection
 * (poisson_solver.hpp:113-116), plus the transform precision. */
int ps_set_option(ps_solver *h, int option, int value);
int ps_get_option(const ps_solver *h, int option, int *value);

/* poisson_solver::push(double*, double*, double*) (poisson_solver.hpp:121,
 * push.cpp:9-397): copy the right-hand side B from HOST arrays; a NULL
 * pointer means the component is absent. */
int ps_push(ps_solver *h, const double *bx, const double *by, const double *bz);

/* poisson_solver::solve3d() (poisson_solver.hpp:119, solve3d.cpp:8-635).
 * Fails with PS_ERR_COMPONENTS where the reference prints its "rhs fields
 * have not been pushed correctly" error: grad needs B_x, div and curl need all
 * three components. grad with fewer than three components differentiates
 * B_x along the missing directions (the reference dereferences NULL there). */
int ps_solve3d(ps_solver *h);

/* poisson_solver::pull(Ax, Ay, Az, Bx, By, Bz) (poisson_solver.hpp:122,
 * pull.cpp:8-469): copy the solution (A, or its grad/div/curl) and,
 * when Bx/By/Bz are non-NULL, the right-hand side as the solve used it
 * (regularised and, if enabled, reprojected) into HOST arrays. Arrays of
 * components the last solve did not produce are left untouched. */
int ps_pull(ps_solver *h, double *ax, double *ay, double *az, double *bx, double *by, double *bz);

/* Device-pointer forms of push and pull (same semantics; pointers are CUDA
 * device memory of the handle's device). */
int ps_push_device(ps_solver *h, const double *bx, const double *by, const double *bz);
int ps_pull_device(ps_solver *h, double *ax, double *ay, double *az, double *bx, double *by, double *bz);

/* Device-resident solve in one call: B in device memory -> A in device
 * memory, no copies through the handle's own field buffers. NULL B pointers
 * are absent components; NULL A pointers are outputs not written. Equivalent
 * to push_device + solve3d + pull_device of A. */
int ps_solve3d_device(ps_solver *h, const double *bx, const double *by, const double *bz,
                      double *ax, double *ay, double *az);

/* Device-resident solve that allocates no memory: no reference counterpart
 * (the reference allocates its arrays in every push and solve). For callers
 * that may not call cudaMalloc/cudaFree while their run is under way, e.g. a
 * time-stepping code solving inside a device-memory budget reserved up front
 * or owned by another framework's pool, where an allocation could fail late
 * or synchronise the device. Same arguments and result as ps_solve3d_device
 * on a handle set up with ps_setup3d, but always with FP64 transforms and
 * with its spectra in 32 MiB of scratch compiled into the library: problems
 * needing more -- (components in use) x Nz x Py x (Px/2+1) x 16 bytes, e.g.
 * a 64^3 unbounded 3-component curl solve needs 25.6 MiB -- fail with
 * PS_ERR_UNSUPPORTED. Every GPU that loads this part of the library holds the
 * scratch until exit. The first call on a device resolves the scratch
 * address; make it before any stream capture. All calls share the scratch:
 * calls whose GPU work overlaps (other streams, handles or threads) race. */
int ps_solve3d_device_noalloc(ps_solver *h, const double *bx, const double *by, const double *bz,
                              double *ax, double *ay, double *az);

/* The public member `std::vector<class_partition> partition`
 * (poisson_solver.hpp:102, class_partition.hpp:29-43): one GPU holds the
 * whole grid, so there is exactly one partition: ncell = the grid, icell = 0. */
int ps_partition_count(const ps_solver *h);
int ps_partition(const ps_solver *h, int index, int ncell[3], int icell[3], double dx[3]);

/* setup2d / solve2d (poisson_solver.hpp:110, 118; setup2d.cpp:8,
 * greens2d.cpp:9, solve2d.cpp:8). Boundary conditions per axis 0 (unbounded)
 * or 1 (periodic), all four combinations. Fields are [Ny][Nx], x fastest,
 * pushed and pulled with ps_push / ps_pull (X, Y and the out-of-plane Z as
 * the reference: grad of X -> X, Y; div of X, Y -> X; curl of Z -> X, Y =
 * (dZ/dy, -dZ/dx) of the solution). A handle set up by setup2d solves with
 * ps_solve2d (ps_solve3d returns PS_ERR_STATE, and the reverse);
 * ps_solve3d_device runs whichever solve the handle is set up for. */
int ps_setup2d(ps_solver *h, const int ncell[2], const int bc[2], const double dx[2], int reg_order);
int ps_solve2d(ps_solver *h);

/* Fortran-style fields (poisson_solver_push.f:8, poisson_solver_pull.f:8):
 * one HOST array holding ncomp = 1..3 components interleaved, component
 * fastest, then x, y, z, with allocated extents ext[3] (ghost layers
 * included); the field's cell (i, j, k) is element
 * ((k + offset[2]) ext[1] + (j + offset[1])) ext[0] + (i + offset[0]),
 * times ncomp, plus the component. push_interleaved pushes X (ncomp 1),
 * X, Y (2) or X, Y, Z (3). pull_interleaved writes the first ncomp_a solution
 * components to a and the first ncomp_b returned right-hand-side components
 * to b (either may be NULL); components the solve did not produce are
 * written as zero, and elements outside the field box are left untouched. */
int ps_push_interleaved(ps_solver *h, const double *b, int ncomp, const int ext[3], const int offset[3]);
int ps_pull_interleaved(ps_solver *h, double *a, int ncomp_a, double *b, int ncomp_b, const int ext[3],
                        const int offset[3]);

/* Gaussian smoothing of the pushed fields in place (poisson_solver_smooth3d.f):
 * each is zero-padded on unbounded axes, transformed, multiplied by
 * exp(-width^2 |k|^2 / 2) with the solver's wavenumbers, transformed back and
 * cropped; a later solve3d or pull of the right-hand side sees the smoothed
 * fields. 3D handles only. */
int ps_smooth3d(ps_solver *h, double width);

/* Extension with no reference counterpart: select the kernel family.
 * PS_KERNEL_GAUSSIAN uses order 2m = max(2, reg_order rounded up to even) and
 * width s = width (0: twice the largest cell size, the width of the
 * reference's filter); its returned right-hand side is filtered by
 * zeta_m(s |k|). Applies to the next setup; on a set-up handle the kernel is
 * rebuilt at once, as a new setup (pushed fields are dropped). */
int ps_set_kernel(ps_solver *h, int family, double width);

/* Stream the handle launches on (a cudaStream_t; NULL = legacy default). */
int ps_set_stream(ps_solver *h, void *stream);
/* Wait for the handle's stream. */
int ps_synchronize(ps_solver *h);

/* Message of the last failed call on h ("" when none); static text for a
 * status code. */
const char *ps_last_error(const ps_solver *h);
const char *ps_status_string(int status);

/* Introspection used by tests and benchmarks. */
enum {
    PS_INFO_PADDED_X = 0, PS_INFO_PADDED_Y = 1, PS_INFO_PADDED_Z = 2, /* transform lengths */
    PS_INFO_LAUNCHES_PER_SOLVE = 3,  /* kernels one solve launches */
    PS_INFO_DEVICE_BYTES = 4,        /* device memory the handle holds */
    PS_INFO_KERNEL_OCTANT = 5        /* elements of the stored kernel octant */
};
int ps_get_info(const ps_solver *h, int what, double *value);

/* Per-pass device times accumulated since the last reset while
 * PS_OPT_PASS_TIMING is on, measured with CUDA events on the handle's stream:
 * ms[0] x forward, ms[1] y forward, ms[2] fused z pass, ms[3] y inverse,
 * ms[4] x inverse. *nsolves receives the number of solves summed. Waits for
 * the timed work to finish; reset != 0 clears the sums afterwards. */
enum { PS_NUM_PASSES = 5 };
int ps_get_pass_times(ps_solver *h, double ms[5], int *nsolves, int reset);

/* Autotuning (no reference counterpart: the reference has one FFT code path).
 * Each pass of a solve -- x forward, y forward, fused z, y inverse, x inverse
 * -- can run one of several kernel families with a choice of lines per CTA.
 * ps_autotune times every choice that fits each pass for the handle's grid,
 * boundary conditions, precision and output option, with the components of
 * component_mask (bit c = component c) pushed, on zero-filled scratch buffers
 * (pushed fields are not touched), and keeps the fastest. Tuned choices are
 * kept for the process and appended to a text cache file ($PS_TUNE_CACHE,
 * else $XDG_CACHE_HOME or $HOME/.cache, poisson_solver_gb300/tune.txt;
 * PS_TUNE_CACHE="" disables the file), so later handles and runs of the same
 * configuration on the same GPU model reuse them. Without tuning a measured
 * default is used. ps_get_pass_config reports the family and lines a solve
 * with component_mask would run for pass 0..4. */
enum { PS_FAMILY_RUNTIME = 0, PS_FAMILY_P2 = 1, PS_FAMILY_WIDE = 2, PS_FAMILY_TMEM = 3, PS_FAMILY_TMA = 4, PS_FAMILY_TC = 5 };
int ps_autotune(ps_solver *h, int component_mask);
int ps_get_pass_config(ps_solver *h, int pass, int component_mask, int *family, int *lines);

/* The transform plan the same solve runs on pass 0..4: its stage radices in
 * order (the first `capacity` of *nstages written to radices) and, for a
 * length transformed by Bluestein's algorithm, the convolution length the
 * stages run on (*conv_length; 0 otherwise). With FP32 transforms the
 * run-time kernels have plan variants that ps_autotune times beside the
 * families and lines: the power-of-two part in radix 16 or radix 8,
 * Bluestein's convolution length as the least power of two or the least
 * 2^a 3^b 5^c >= 2 L - 1, and, for a length whose largest prime p divides it
 * once with p - 1 and the cofactor free of primes above 13, Rader's algorithm
 * in place of Bluestein's: the first stage has radix p and runs each p-point
 * DFT as a cyclic convolution of p - 1 points (then *conv_length is p - 1).
 * PS_PLAN_X/_Y/_Z (bit 0: radix 8, bit 1: smooth length, bit 2: Rader) set
 * them for the run-time family and bypass tuned choices. FP64 transforms
 * always take the default plan. No reference counterpart. */
int ps_get_pass_plan(ps_solver *h, int pass, int component_mask, int *radices, int capacity, int *nstages,
                     int *conv_length);

/* Copy the FP64 kernel octant K = G * zeta / (Px Py Pz), layout
 * [Pz/2+1][Py/2+1][Px/2+1] (x fastest), to a HOST array. */
int ps_get_kernel(const ps_solver *h, double *out, long long capacity);

/* ---------------------------------------------------------------------------
 * Batched solves. No reference counterpart as one call: the reference solves
 * many problems by holding one poisson_solver object per problem and calling
 * setup3d / push / solve3d / pull on each (c++/test/<case>/sources/main.cpp
 * drive one object each). A batch holds many independent problems -- any grid,
 * boundary conditions, regularisation order, components and output option
 * each -- and solves them all with one kernel launch per pass (five launches
 * in all, whatever the number of problems), replayed through a CUDA graph
 * that is captured on the first solve and again after any change to the set
 * of problems, their options or their pushed components.
 *
 *   ps_batch_create(&b, PS_PREC_FP64 or PS_PREC_FP32)   one precision a batch
 *   ps_batch_add(b, ncell, bc, dx, reg, &i)             setup3d of problem i
 *   ps_batch_set_option(b, i, PS_OPT_GRAD/DIV/CURL/REPROJECT, 0/1)
 *   ps_batch_push(b, i, bx, by, bz)                     push of problem i
 *   ps_batch_solve(b)                                   solve3d of every problem
 *   ps_batch_pull(b, i, ax, ay, az)                     pull of problem i's A
 *
 * Same field layout, components and errors as the single-problem calls; a
 * solve fails with PS_ERR_STATE if a problem has nothing pushed. The batched
 * launches run the run-time transform kernels (any length); FP32 passes over
 * power-of-two lengths that a compiled family covers run as the problem's
 * own launch right after them. Many right-hand sides of one problem are
 * problems added with the same setup: they share its kernel build.
 * ps_batch_solve runs asynchronously on the batch's stream; pulls wait. */
typedef struct ps_batch ps_batch;
int ps_batch_create(ps_batch **out, int precision);
int ps_batch_destroy(ps_batch *b);
int ps_batch_add(ps_batch *b, const int ncell[3], const int bc[3], const double dx[3], int reg_order, int *index);
int ps_batch_count(const ps_batch *b, int *count);
int ps_batch_set_option(ps_batch *b, int index, int option, int value);
/* ps_set_kernel for problem index (its kernel is rebuilt as a new setup:
 * push its fields after this call). */
int ps_batch_set_kernel(ps_batch *b, int index, int family, double width);
int ps_batch_push(ps_batch *b, int index, const double *bx, const double *by, const double *bz);
int ps_batch_push_device(ps_batch *b, int index, const double *bx, const double *by, const double *bz);
int ps_batch_solve(ps_batch *b);
/* Tune the batch (no reference counterpart): for the x, y and z launches in
 * turn, time the plan variants of every problem's transforms (FP32 batches
 * only; see ps_get_pass_plan), then the bound on a CTA's threads (64, 128,
 * 256) and the lines a CTA each problem starts from (2 .. 32) on the pushed
 * problems, and keep the fastest for this batch. Every problem must have been
 * pushed. FP64 results do not change (each line's arithmetic is the same
 * whatever the shape); FP32 results change at rounding level when a plan
 * variant is taken. The pushed fields are kept, the outputs and work buffers
 * are overwritten. Later solves, and rebuilds after adds, options or pushes,
 * use the tuned settings. ps_batch_get_tuning reports them for axis 0..2
 * (x, y, z): the CTA thread bound, the starting lines and the plan variant
 * (bit 0: radix 8, bit 1: smooth Bluestein length, bit 2: Rader's algorithm;
 * see ps_get_pass_plan). ps_batch_set_tuning sets them (a thread bound that
 * is a multiple of 32 up to 256, starting lines a power of two up to 64, a
 * variant 0..7; bits a length does not use are ignored), for instance to
 * reuse settings tuned earlier; the next solve rebuilds the batch. */
int ps_batch_autotune(ps_batch *b);
int ps_batch_get_tuning(const ps_batch *b, int axis, int *max_threads, int *start_lines, int *plan_variant);
int ps_batch_set_tuning(ps_batch *b, int axis, int max_threads, int start_lines, int plan_variant);
int ps_batch_pull(ps_batch *b, int index, double *ax, double *ay, double *az);
int ps_batch_pull_device(ps_batch *b, int index, double *ax, double *ay, double *az);
int ps_batch_set_stream(ps_batch *b, void *stream);
int ps_batch_synchronize(ps_batch *b);
enum {
    PS_BATCH_INFO_LAUNCHES_PER_SOLVE = 0, /* kernels one batched solve launches: the batched launches with
                                             tiles, plus the passes of FP32 problems routed to their own
                                             kernel family (power-of-two lengths the compiled families cover) */
    PS_BATCH_INFO_TILES_PER_SOLVE = 1,    /* CTA tiles of the last captured solve, all passes */
    PS_BATCH_INFO_POINTS = 2,             /* grid points over all problems */
    PS_BATCH_INFO_KERNEL_BUILDS = 3       /* Green's-kernel octants computed for the batch's problems: a
                                             problem added with the grid, boundary conditions, spacing and
                                             regularisation of an earlier one (another right-hand side)
                                             copies that one's octant instead */
};
int ps_batch_get_info(const ps_batch *b, int what, double *value);
const char *ps_batch_last_error(const ps_batch *b);

#ifdef __cplusplus
}
#endif

#endif
