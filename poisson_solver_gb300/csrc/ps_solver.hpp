// Host-side solver state and orchestration (C++). One handle = one problem
// (grid, boundary conditions, spacing, regularisation) on one GPU.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <map>
#include <tuple>
#include <vector>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>

#include "ps_types.hpp"

namespace ps {

// Failure carried to the C ABI as (status, message).
struct Error : std::runtime_error {
    int status;
    Error(int st, const std::string &msg) : std::runtime_error(msg), status(st) {}
};

// Makes a handle's device current for one ABI call and gives the calling
// thread back its own current device afterwards.
struct DeviceScope {
    int saved = -1;
    explicit DeviceScope(int device)
    {
        if (cudaGetDevice(&saved) != cudaSuccess) {
            cudaGetLastError();
            saved = -1;
        }
        if (saved != device) cudaSetDevice(device);
        else saved = -1;  // nothing to restore
    }
    ~DeviceScope()
    {
        if (saved >= 0) cudaSetDevice(saved);
    }
    DeviceScope(const DeviceScope &) = delete;
    DeviceScope &operator=(const DeviceScope &) = delete;
};

// Grow-only device allocation.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    void ensure(size_t n);
    void release();
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
};

struct Plan {
    FftPlanDev dev{};
    DevBuf table;
    DevBuf itable;  // index tables of a Rader plan
};

// Plan variants of the run-time family, tuned for FP32 transforms (FP64
// always takes the default plan, so FP64 results do not depend on tuning):
// PV_HALF_RADIX runs the power-of-two part of a length in radices of half the
// element budget (radix 8 instead of 16: one stage more, two butterflies a
// thread); PV_SMOOTH_M takes Bluestein's convolution length as the least
// 2^a 3^b 5^c >= 2 lb - 1 instead of the least power of two; PV_RADER
// replaces Bluestein's algorithm by a Rader stage for the largest prime p
// where p - 1 and the cofactor are 13-smooth (a cyclic convolution of p - 1
// points in place of two transforms of at least 2 L - 1).
enum { PV_HALF_RADIX = 1, PV_SMOOTH_M = 2, PV_RADER = 4 };

// Kernel family and lines per CTA of one pass: 'r' run-time, 'p' length-
// specialised, 'w' wide, 't' tensor-memory fused z, 'q' a warp per line or
// column group (y and z fed by tiled bulk copies), 'c' fused z with its DFT
// stages on the tensor cores; pv the plan variant ('r' only).
struct PassChoice {
    char fam;
    int B;
    int pv = 0;
};

// Arguments of the five passes of one solve, all but the plans and the lines
// per CTA (which depend on the kernel family that runs each pass).
struct PassArgs {
    XFwdArgs x{};
    ColArgs y{};
    ZArgs z{};
    ColArgs yi{};
    XInvArgs xi{};
    int write_mask = 0;  // outputs written; 0 skips the inverse y and x passes
};

struct Solver {
    int device = 0;
    cudaStream_t stream = nullptr;

    bool is_setup = false;
    // 2: set up by setup2d. The 2D problem is held as one periodic z-plane
    // (n[2] = P[2] = 1); its solve is the x pass, one fused pass along y
    // (forward, spectral operation, inverse) and the x inverse.
    int dims = 3;
    int n[3] = {0, 0, 0}, bc[3] = {0, 0, 0}, P[3] = {0, 0, 0};
    double dx[3] = {0, 0, 0};
    int reg = 0;
    // Kernel family: PS_KERNEL_SPECTRAL (the reference's) or PS_KERNEL_GAUSSIAN
    // of order max(2, reg rounded up to even) and width gauss_width (0: twice
    // the largest cell size, the width of the reference's filter).
    int kernel_family = 0;
    double gauss_width = 0.0;
    int Mx = 0, oy = 0, oz = 0;  // half-spectrum length and kernel octant extents
    int ldx = 0;                 // row pitch of the spectra work[c] (Mx rounded up to even)
    int kzp = 0;                 // z pitch of kernzf32 (oz rounded up to a multiple of 4)

    int opt_grad = 0, opt_div = 0, opt_curl = 0, opt_reproject = 0;
    int precision = PREC_FP64;

    DevBuf kern64, kern32, kern_df;  // octant K = G zeta / (Px Py Pz); kern_df: double-float pairs
    // A handle whose FP64 kernel octant the next build copies instead of
    // computing, when it was built from the same inputs (the batch sets it
    // for a problem added with the setup of an earlier one); kernel_builds
    // counts the octants computed, not copied.
    const Solver *kernel_from = nullptr;
    int kernel_builds = 0;
    DevBuf kernzf32;        // FP32 K with z fastest, [oy][Mx][kzp] (unbounded z of 256..1024 points)
    DevBuf zeta64, zeta32, zeta_df;  // octant zeta / (Px Py Pz), built on first use
    DevBuf smooth64, smooth32, smooth_df;  // octant exp(-s^2 |k|^2 / 2) / (Px Py Pz) of smooth3d(s)
    double smooth_s = -1.0;     // s the smooth octants hold (-1: none)
    int filter_source = 0;      // the filter pass multiplies by zeta (0) or the smooth octant (1)
    DevBuf stage;               // packed interleaved fields for push/pull_interleaved
    DevBuf work[3];         // per-component spectra [Nz][Py][Mx], pass precision
    DevBuf fb[3], fa[3], fr[3];  // handle-owned fields: pushed B, solution A, returned B
    DevBuf status;               // int[4]: [0] bit 0 set by a kernel whose bounded wait timed out,
                                 // [1] tile counter of the dynamically scheduled kernels

    int pushed = 0;    // component mask held in fb
    int produced = 0;  // component mask of fa from the last solve
    int rhs_ready = 0; // fr holds the returned right-hand side of the pushed fb

    std::map<std::tuple<int, int, int, int>, std::unique_ptr<Plan>> plans;  // (length, precision, element budget, variant)

    // Optional per-pass timing: one set of boundary events per timed solve.
    static constexpr int NPASS = 5;
    int opt_timing = 0;
    std::vector<std::array<cudaEvent_t, NPASS + 1>> ev_pending, ev_pool;
    double pass_ms[NPASS] = {0, 0, 0, 0, 0};
    int timed_solves = 0;
    void drain_timing();
    std::string last_error;

    Solver();
    ~Solver();

    void setup3d(const int ncell[3], const int bcs[3], const double dxs[3], int reg_order);
    void setup2d(const int ncell[2], const int bcs[2], const double dxs[2], int reg_order);
    void finish_setup();  // buffers and the kernel once n, bc, dx, P, reg are set
    void set_option(int option, int value);
    int get_option(int option) const;
    // Select the kernel family; on a set-up handle the kernel is rebuilt
    // (as a new setup: pushed fields are dropped).
    void set_kernel(int family, double width);
    // The family's order m (zeta_m) and width for the current setup; m = 0
    // for the spectral family.
    GaussFamily gauss_family() const;

    // Device-pointer pipeline. B: input components (NULL = absent); A: outputs.
    // Returns the mask of components written to A.
    int solve(const double *const Bin[3], double *const Aout[3], bool filter_only = false);
    // The pass arguments of that solve (buffers and the kernel ensured);
    // returns the mask of components written.
    int prepare(const double *const Bin[3], double *const Aout[3], bool filter_only, PassArgs &pa);
    // Mask of outputs a solve produces for the given input mask (throws on a
    // combination the options reject).
    int output_mask(int in_mask) const;

    void push(const double *const B[3], cudaMemcpyKind kind);
    void solve_internal(int want_dims = 3);
    void pull(double *const A[3], double *const RB[3], cudaMemcpyKind kind);
    // The returned right-hand side of the pushed fields (device pointers,
    // null where not pushed): B itself unless the regulariser or the
    // reprojection changed it, else the filtered copy (built on demand).
    void returned_rhs(const double *out[3]);
    // Fortran-style push/pull of one array with interleaved components
    // (component fastest, then x, y, z; extents ext, field box at offset).
    void push_interleaved(const double *b, int ncomp, const int ext[3], const int offset[3], cudaMemcpyKind kind);
    void pull_interleaved(double *a, int ncomp_a, double *b, int ncomp_b, const int ext[3], const int offset[3],
                          cudaMemcpyKind kind);
    // Gaussian smoothing of the pushed fields, exp(-s^2 |k|^2 / 2), in place.
    void smooth3d(double s);
    // After the stream has drained: throws PS_ERR_TIMEOUT (and clears the
    // word) if a kernel reported a timed-out wait.
    void check_status();
    void synchronize();

    // Time every kernel family and line count that fits each pass of this
    // configuration (options + in_mask) on zero-filled scratch buffers and
    // keep the fastest (tuned choices outlive the handle; see ps_solver.cpp).
    void autotune(int in_mask);
    // The family and lines a solve of in_mask would run on a pass, and the
    // transform plan it runs with.
    PassChoice current_choice(int pass, int in_mask);
    const FftPlanDev &current_plan(int pass, int in_mask);
    // For the batched solve: the choice for prepared pass arguments, and one
    // pass launched on another stream (the batch's capture stream).
    PassChoice pass_choice(int pass, const PassArgs &pa) { return choice(pass, pa); }
    void launch_on(int pass, const PassChoice &c, PassArgs &pa, cudaStream_t st)
    {
        cudaStream_t saved = stream;
        stream = st;
        try {
            launch_pass(pass, c, pa);
        } catch (...) {
            stream = saved;
            throw;
        }
        stream = saved;
    }

    size_t device_bytes() const;
    void copy_kernel(double *host, long long capacity) const;

    const Plan &plan(int L, int prec, int emax = 0, int pv = 0);  // emax 0: e_max(prec); pv: PV_* bits
    void ensure_kernel(int prec);
    void ensure_zeta(int prec);

    // length of the transform a pass runs (the fused pass runs along y in 2D)
    int pass_len(int pass) const;

private:
    bool family_ok(int pass, char fam, const PassArgs &pa) const;
    int family_emax(int pass, char fam) const;
    size_t pass_smem(int pass, char fam, int B, const PassArgs &pa, const Plan &pl) const;
    bool pass_fits(int pass, char fam, int B, const PassArgs &pa, const Plan &pl) const;
    PassChoice default_choice(int pass, const PassArgs &pa);
    PassChoice choice(int pass, const PassArgs &pa);
    std::string tune_key(int pass, const PassArgs &pa);
    std::string device_tag;  // device name and SM count, for the tuning key
    void launch_pass(int pass, const PassChoice &c, PassArgs &pa);
    const Plan &pass_plan(int pass, const PassChoice &c);
    int plan_variants(int pass) const;  // PV_* bits that change the run-time family's plan of this pass
    void build_kernel();
    void check_setup() const;
    size_t field_elems() const { return (size_t)n[0] * n[1] * n[2]; }
    size_t work_elems() const { return (size_t)n[2] * P[1] * ldx; }
};

// The FP64 solve in fixed, library-owned device memory (ps_noalloc.cu).
int solve_noalloc(Solver &s, const double *const Bin[3], double *const Aout[3]);

}  // namespace ps
