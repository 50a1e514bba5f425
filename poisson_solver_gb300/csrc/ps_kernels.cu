// Public launchers of the run-time pass kernels (ps_kernels_body.cuh):
// grid, block and shared-memory sizes, and the dispatch on the pass
// precision (FP64 and FP32 instantiated here, double-float in
// ps_kernels_df.cu).
#include "ps_kernels_body.cuh"

namespace ps {

static int threads_for(const FftPlanDev &p, int B) { return B * p.tpl; }

// bytes of a complex element of the pass precision
static size_t cplx_bytes(int prec) { return prec == PREC_FP32 ? 8 : 16; }

size_t smem_x(int prec, const FftPlanDev &p, int B)
{
    return cplx_bytes(prec) * ((size_t)B * (p.L + 1) * (p.generic ? 2 : 1) + p.ntw);
}
size_t smem_col(int prec, const FftPlanDev &p, int B)
{
    return cplx_bytes(prec) * ((size_t)B * p.L * (p.generic ? 2 : 1) + p.ntw);
}
size_t smem_z(int prec, const FftPlanDev &p, int B, int nbuf)
{
    return cplx_bytes(prec) * ((size_t)B * p.L * (nbuf + (p.generic ? 1 : 0)) + p.ntw);
}

int max_smem_per_block()
{
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

cudaError_t launch_xfwd(int prec, const XFwdArgs &a, cudaStream_t st)
{
    if (a.B > MAX_LINES) return cudaErrorInvalidConfiguration;  // row-offset table size
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long lines = (rows + 1) / 2;
    dim3 grid((unsigned)((lines + a.B - 1) / a.B), a.ncomp);
    const int nt = threads_for(a.plan, a.B);
    const size_t sm = smem_x(prec, a.plan, a.B);
    if (prec == PREC_FP64) return rt::xfwd<double>(a, grid, nt, sm, st);
    if (prec == PREC_FP32) return rt::xfwd<float>(a, grid, nt, sm, st);
    if (prec == PREC_DF64) return rt::xfwd_df(a, grid, nt, sm, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_col(int prec, int inverse, const ColArgs &a, int outer, cudaStream_t st)
{
    dim3 grid((unsigned)((a.Mx + a.B - 1) / a.B), outer, a.ncomp);
    const int nt = threads_for(a.plan, a.B);
    const size_t sm = smem_col(prec, a.plan, a.B);
    if (prec == PREC_FP64) return rt::col<double>(inverse, a, grid, nt, sm, st);
    if (prec == PREC_FP32) return rt::col<float>(inverse, a, grid, nt, sm, st);
    if (prec == PREC_DF64) return rt::col_df(inverse, a, grid, nt, sm, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_z(int prec, const ZArgs &a, int ny, cudaStream_t st)
{
    dim3 grid((unsigned)((a.Mx + a.B - 1) / a.B), ny);
    const int nt = threads_for(a.plan, a.B);
    const int nbuf = a.nin > a.nout ? a.nin : a.nout;
    const size_t sm = smem_z(prec, a.plan, a.B, nbuf);
    if (prec == PREC_FP64) return rt::z<double>(a, grid, nt, sm, st);
    if (prec == PREC_FP32) return rt::z<float>(a, grid, nt, sm, st);
    if (prec == PREC_DF64) return rt::z_df(a, grid, nt, sm, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_xinv(int prec, const XInvArgs &a, cudaStream_t st)
{
    if (a.B > MAX_LINES) return cudaErrorInvalidConfiguration;  // row-offset table size
    const long long rows = (long long)a.rows_y * a.rows_z;
    const long long lines = (rows + 1) / 2;
    dim3 grid((unsigned)((lines + a.B - 1) / a.B), a.ncomp);
    const int nt = threads_for(a.plan, a.B);
    const size_t sm = smem_x(prec, a.plan, a.B);
    if (prec == PREC_FP64) return rt::xinv<double>(a, grid, nt, sm, st);
    if (prec == PREC_FP32) return rt::xinv<float>(a, grid, nt, sm, st);
    if (prec == PREC_DF64) return rt::xinv_df(a, grid, nt, sm, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_xfwd_batch(int prec, const XFwdArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                              bool rader, cudaStream_t st)
{
    if (ntiles <= 0) return cudaSuccess;
    if (prec == PREC_FP64) return rt::xfwd_batch<double>(args, tiles, ntiles, nt, smem, rader, st);
    if (prec == PREC_FP32) return rt::xfwd_batch<float>(args, tiles, ntiles, nt, smem, rader, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_col_batch(int prec, int inverse, const ColArgs *args, const BatchTile *tiles, int ntiles, int nt,
                             size_t smem, bool rader, cudaStream_t st)
{
    if (ntiles <= 0) return cudaSuccess;
    if (prec == PREC_FP64) return rt::col_batch<double>(inverse, args, tiles, ntiles, nt, smem, rader, st);
    if (prec == PREC_FP32) return rt::col_batch<float>(inverse, args, tiles, ntiles, nt, smem, rader, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_z_batch(int prec, const ZArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                           bool rader, cudaStream_t st)
{
    if (ntiles <= 0) return cudaSuccess;
    if (prec == PREC_FP64) return rt::z_batch<double>(args, tiles, ntiles, nt, smem, rader, st);
    if (prec == PREC_FP32) return rt::z_batch<float>(args, tiles, ntiles, nt, smem, rader, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_xinv_batch(int prec, const XInvArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                              bool rader, cudaStream_t st)
{
    if (ntiles <= 0) return cudaSuccess;
    if (prec == PREC_FP64) return rt::xinv_batch<double>(args, tiles, ntiles, nt, smem, rader, st);
    if (prec == PREC_FP32) return rt::xinv_batch<float>(args, tiles, ntiles, nt, smem, rader, st);
    return cudaErrorInvalidValue;
}

}  // namespace ps
