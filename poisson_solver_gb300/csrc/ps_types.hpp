// Types shared by the host orchestration (C++) and the CUDA pass kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ps {

constexpr int MAX_STAGES = 16;
constexpr int MAX_THREADS = 512;  // CTA size bound of the pass kernels (<= 128 registers a thread)
constexpr int MAX_LINES = 64;     // lines a CTA of any pass kernel (the x passes keep 2 row offsets a line)

// Pass precision: FP64, FP32, or double-float (pairs of FP32 numbers, about
// 48 significant bits: ps_dfloat.cuh).
enum Precision { PREC_FP64 = 0, PREC_FP32 = 1, PREC_DF64 = 2 };

// Register elements a thread holds per FFT stage, which also caps the radix:
// 8 complex doubles or double-floats (radix <= 8) or 16 complex floats
// (radix <= 16). The fused z pass holds three components in shared memory,
// so its FP32 variant uses 8 to double the threads per line at the same
// footprint.
__host__ __device__ constexpr int e_max(int prec) { return prec == PREC_FP32 ? 16 : 8; }
__host__ __device__ constexpr int e_max_z(int /*prec*/) { return 8; }

// One 1D transform length as the kernels see it (see ps_fft.cuh).
struct FftPlanDev {
    int L;
    int nstages;
    int tpl;      // threads per line
    int generic;  // a stage has a prime radix above 7 (needs scratch shared memory)
    int radix[MAX_STAGES];
    int m[MAX_STAGES];
    int tw[MAX_STAGES];
    int gw[MAX_STAGES];
    int lm[MAX_STAGES];  // log2(m) when m is a power of two, else -1
    int ntw;             // complex entries in the table
    const void *table;   // complex twiddles in the pass precision (copied to shared memory per CTA)
    // Bluestein plans (a prime factor of the transform length of 17 or more):
    // the stages above transform length L = M, a power of two >= 2 lb - 1,
    // and the length-lb DFT is chirp x FFT_M^-1(K FFT_M(chirp x)).
    int blue;   // 1 for a Bluestein plan
    int lb;     // the transform length (L for other plans)
    int chirp;  // table offset of c[n] = e^{-i pi n^2 / lb}, n < lb
    int kspec;  // table offset of K[k] = FFT_M(conj c, wrapped)[k] / M, k < M
    int bsh;    // 1: chirp and K lie in the part of the table staged in shared memory
    int ctm;    // M when the convolution stages are the compile-time sequence of M (64..1024), else 0
    // Rader plans (FP32 plan variant): stage 0 has a prime radix p >= 17 and
    // m = 1, and each of its L / p butterflies is computed by Rader's
    // algorithm, a cyclic convolution of p - 1 points run by the sub-transform
    // stages rs0 .. rs0 + rns - 1 of the stage table (their twiddles in the
    // shared table, like the plan's own).
    int rader;   // 1 for a Rader plan
    int rq;      // p - 1, the sub-transform length
    int rtpl;    // threads a sub-transform
    int rs0;     // first sub-transform stage in the stage table
    int rns;     // sub-transform stages
    int rbh;     // table offset of the convolution spectra: forward (p - 1 entries), then inverse
    const int *itab;  // g^-j mod p for j < p - 1, then log_g k for k = 1 .. p - 1 (g a primitive root)
    float rinv_p, rinv_q;  // 1 / p and 1 / (p - 1), for exact index division in FP32
};

// Spectral operation of the fused z pass.
enum Op {
    OP_NONE = 0,     // out_c = K in_c
    OP_GRAD = 1,     // out_d = i k_d K in_d (component x where d was not pushed)
    OP_DIV = 2,      // out_x = i K (k . in)
    OP_CURL = 3,     // out = i K (k x in)
    OP_FILTER = 4,   // out_c = Z in_c  [- K k_c (k . in) when reprojecting]
    OP_FORWARD = 5,  // kernel build: forward transform only, spectrum stored
};

// x forward: pairs of real rows -> half spectra (real-to-complex by packing
// row 2l as the real and row 2l+1 as the imaginary part of one complex line).
struct XFwdArgs {
    const double *in[3];
    void *out[3];
    int ncomp;
    int L;               // Px
    int n_in;            // leading non-zero samples per row (Nx, or Px)
    long long in_stride; // row stride of the input rows
    int rows_y, rows_z;  // row r = k * rows_y + j
    int out_y;           // y extent of the output array
    int Mx;              // L/2 + 1
    int ld;              // row pitch of the output array (>= Mx)
    int mirror;          // input is the octant of an even function
    int oct_x, oct_y;    // octant extents (x, y) when mirrored
    int Py, Pz;          // full extents the octant is reflected onto
    int B;               // lines per CTA
    FftPlanDev plan;
};

// Strided column pass (the y pass), in place.
struct ColArgs {
    void *data[3];
    int ncomp;
    int L, n_in, n_out;
    int Mx;                  // number of columns (contiguous dimension)
    long long axis_stride;   // elements between consecutive transform samples
    long long outer_stride;  // elements between consecutive outer slabs
    int B;
    FftPlanDev plan;
};

// Fused z pass: forward transform of every input component, spectral
// operation, inverse transform of every output component.
struct ZArgs {
    const void *in[3];
    void *out[3];
    int nin, nout;
    int L, n_in, n_out;
    int Mx;
    long long axis_stride;  // Py * Mx
    long long row_stride;   // Mx (between consecutive y rows)
    int ky0;                // first y row handled (blockIdx.y offset)
    int op;
    int reproject;
    const void *kern;  // octant K = G zeta / (Px Py Pz), [oz][oy][Mx]
    const void *zeta;  // octant zeta / (Px Py Pz) for OP_FILTER
    int oct_y;         // Py/2 + 1
    const float *kern_zf;  // FP32 octant of K with z fastest, [oy][Mx][kzp] (null if not built)
    int kzp;               // z pitch of kern_zf: Pz/2 + 1 rounded up to a multiple of 4
    int Px, Py, Pz;
    double kxc, kyc, kzc;  // 2 pi / (P dx) per axis
    int B;
    FftPlanDev plan;
};

// x inverse: half spectra of row pairs -> real rows, cropped to n_out.
struct XInvArgs {
    const void *in[3];
    double *out[3];
    int ncomp;
    int L;
    int n_out;            // Nx
    int Mx;
    int rows_y, rows_z;
    int in_y;             // y extent of the input array
    int ld;               // row pitch of the input array (>= Mx)
    long long out_stride; // row stride of the output rows
    int B;
    FftPlanDev plan;
};

// Launchers of the run-time kernels (ps_kernels.cu; bodies in
// ps_kernels_body.cuh). They return the launch status.
cudaError_t launch_xfwd(int prec, const XFwdArgs &a, cudaStream_t st);
cudaError_t launch_col(int prec, int inverse, const ColArgs &a, int outer, cudaStream_t st);
cudaError_t launch_z(int prec, const ZArgs &a, int ny, cudaStream_t st);
cudaError_t launch_xinv(int prec, const XInvArgs &a, cudaStream_t st);

// Batched passes (ps_kernels.cu; FP64 and FP32): one launch runs the tiles of many problems.
// Tile = (problem, bx, by, bz): x passes (line block, component); y passes
// (column block, z slab, component); z pass (column block, ky row).
struct BatchTile {
    int p, bx, by, bz;
};
// rader: some problem of the launch has a Rader plan on the pass (the
// launch then runs the kernels instantiated for them).
constexpr int BATCH_MAX_THREADS = 256;  // CTA size bound of the batched passes
cudaError_t launch_xfwd_batch(int prec, const XFwdArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                              bool rader, cudaStream_t st);
cudaError_t launch_col_batch(int prec, int inverse, const ColArgs *args, const BatchTile *tiles, int ntiles, int nt,
                             size_t smem, bool rader, cudaStream_t st);
cudaError_t launch_z_batch(int prec, const ZArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                           bool rader, cudaStream_t st);
cudaError_t launch_xinv_batch(int prec, const XInvArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                              bool rader, cudaStream_t st);

// Shared-memory bytes each pass needs for a given line count (data, scratch
// for direct-DFT stages, twiddle table).
size_t smem_x(int prec, const FftPlanDev &p, int B);
size_t smem_col(int prec, const FftPlanDev &p, int B);
size_t smem_z(int prec, const FftPlanDev &p, int B, int nbuf);
int max_smem_per_block();

// Power-of-two specialised passes (ps_kernels_p2.cu): FP32, 64 <= L <= 2048.
namespace p2 {
bool supported(int prec, int L);
bool supports_op(int op);
size_t smem_lines(int prec, int L, int B, int nbuf, int ntw_entries);
cudaError_t launch_xfwd(const XFwdArgs &a, cudaStream_t st);
cudaError_t launch_col(int inverse, const ColArgs &a, int outer, cudaStream_t st);
cudaError_t launch_z(const ZArgs &a, int ny, int em, cudaStream_t st);
cudaError_t launch_xinv(const XInvArgs &a, cudaStream_t st);
}  // namespace p2

// Wide passes (ps_kernels_wide.cu): FP32, L = 256, 512, 1024, 2048, 32
// elements per thread, first and last stages fused with global memory.
namespace wide {
// threads per CTA of the fused z kernel: its 32-element stages need ~220
// registers a thread
constexpr int Z_MAX_THREADS = 256;
bool supported(int prec, int L);
// column = true for the y and z passes (lanes across lines), false for x
size_t smem_lines(int L, int B, int nbuf, int ntw_entries, bool column);
cudaError_t launch_xfwd(const XFwdArgs &a, cudaStream_t st);
cudaError_t launch_col(int inverse, const ColArgs &a, int outer, cudaStream_t st);
cudaError_t launch_z(const ZArgs &a, int ny, cudaStream_t st);
cudaError_t launch_xinv(const XInvArgs &a, cudaStream_t st);
// fused z pass with the components parked in tensor memory (ps_kernels_ztm.cu)
constexpr int ZT_MAX_THREADS = 256;
bool zt_supported(int prec, int L, int op, int nin, int nout);
size_t smem_lines_zt(int L, int B, int ntw_entries);
cudaError_t launch_zt(const ZArgs &a, int ny, cudaStream_t st);
// fused z pass, a warp per column group, tiled bulk copies in and out
// (ps_kernels_zq.cu): unbounded z (n_in = n_out = L / 2), L = 256..1024, a
// persistent CTA per SM of ZQ_THREADS threads holding zq_lines(L) columns.
// A wait that times out sets bit 0 of *status.
constexpr int ZQ_THREADS = 256;
bool zq_supported(int prec, int L, int op, int nin, int nout, int n_in, int n_out);
int zq_lines(int L);
size_t smem_lines_zq(int L, int ntw_entries);
cudaError_t launch_zq(const ZArgs &a, int ny, int *status, cudaStream_t st);
// y passes, a warp per column group, tiled bulk copies (ps_kernels_yq.cu):
// unbounded y (forward n_in = L / 2, inverse n_out = L / 2) or periodic y
// (n_in = n_out = L), L = 256..1024, a
// persistent CTA per SM holding yq_lines(L) columns, tiles handed out by a
// counter at status[1] (reset by the launch). A wait that times out sets bit
// 0 of status[0].
bool yq_supported(int prec, int inverse, int L, int n_in, int n_out);
int yq_lines(int L);
size_t smem_lines_yq(int inverse, int L, int n_in, int n_out, int ntw_entries);
cudaError_t launch_yq(int inverse, const ColArgs &a, int nplanes, int *status, cudaStream_t st);
// x passes, a warp per line group (ps_kernels_xq.cu): L = 256..1024, not
// mirrored; xq_lines(L) lines a CTA. n = n_in (forward) or n_out (inverse).
bool xq_supported(int prec, int inverse, int L, int n, int mirror);
int xq_lines(int L);
size_t smem_lines_xq(int L, int ntw_entries);
cudaError_t launch_xfq(const XFwdArgs &a, cudaStream_t st);
cudaError_t launch_xiq(const XInvArgs &a, cudaStream_t st);
}  // namespace wide

// Fused z pass with the DFT stages on the tensor cores (ps_kernels_ztc.cu):
// FP32 spectra, unbounded z of L = 1024 (n_in = n_out = 512), 8 columns a
// tile, one persistent CTA per SM. A wait that times out sets bit 0 of
// *status.
namespace tc {
constexpr int ZTC_LINES = 8;
bool ztc_supported(int prec, int L, int op, int nin, int nout, int n_in, int n_out);
size_t smem_ztc();
cudaError_t launch_ztc(const ZArgs &a, int ny, int *status, cudaStream_t st);
}  // namespace tc

// Kernel-build helpers (ps_greens.cu), all FP64.
// Kernel family of the build: gm = 0 is the reference's spectrally truncated
// kernel (Si, Ji0) with the zeta filter; gm >= 1 is the Gaussian-regularised
// family of order 2 gm and width gs, whose spectrum is zeta_gm(gs |k|) / |k|^2.
struct GaussFamily {
    int gm;
    double gs;
};
cudaError_t launch_sample_unbounded3d(double *oct, const int oext[3], const int P[3], const double dx[3],
                                      GaussFamily gf, cudaStream_t st);
cudaError_t launch_sample_unbounded2d(double *oct, const int oext[2], const int P[2], const double dx[2],
                                      GaussFamily gf, cudaStream_t st);
// Spectrum G1[k], k <= P/2, of the 1D kernel along an unbounded axis whose
// cross-section is periodic.
cudaError_t launch_line_ppf(double *line, int P, double dz, GaussFamily gf, cudaStream_t st);
// Octant of K = G zeta / norm from the kernel spectrum (kind 0), or from
// 1/|k|^2 with the plane/line overrides of the mixed domains.
struct KernelFillArgs {
    double *kern;          // out: [oz][oy][Mx] FP64
    double *zeta_out;      // out (optional): zeta / norm
    const double2 *spec;   // kind 0: spectrum [oz][Py][Mx] (real part used)
    const double2 *plane;  // kind 2 (kz = 0 plane): spectrum [oy][Mx]
    const double *line;    // kinds 1, 4, 5: 1D kernel spectrum along the unbounded axis (z, y, x)
    int kind;              // 0 unbounded, 1 ppf, 2 ffp (and 2D unbounded), 3 periodic,
                           // 4 2D x-periodic y-unbounded, 5 2D x-unbounded y-periodic
    int Mx, oy, oz;
    int P[3];
    double dx[3];
    int reg;
    double norm;
    int smooth;           // zeta_out = exp(-smooth_sigma^2 |k|^2 / 2) / norm (the smooth3d
    double smooth_sigma;  // filter) in place of the regularisation filter
    GaussFamily gauss;    // gm >= 1: the Gaussian-regularised family (kern = its spectrum,
                          // zeta_out = zeta_gm(gs |k|) / norm)
};
cudaError_t launch_kernel_fill(const KernelFillArgs &a, cudaStream_t st);
// Fields with interleaved components (ps_fields.cu): packed [nz][ny][nx][ncomp]
// <-> ncomp separate [nz][ny][nx] arrays (absent = zero on the way out).
cudaError_t launch_deinterleave(const double *packed, int ncomp, long long n, double *const out[3], cudaStream_t st);
cudaError_t launch_interleave(const double *const in[3], int ncomp, long long n, double *packed, cudaStream_t st);
cudaError_t launch_to_fp32(const double *in, float *out, size_t n, cudaStream_t st);
cudaError_t launch_to_df(const double *in, float2 *out, size_t n, cudaStream_t st);  // (hi, lo) pairs
// FP32 copy of the octant [oz][oy][Mx] with z fastest: out[(y Mx + x) kzp + z],
// zero for oz <= z < kzp (each column a whole number of 16-byte units).
cudaError_t launch_kernel_zfast(const double *kern, float *out, int Mx, int oy, int oz, int kzp, cudaStream_t st);

}  // namespace ps
