// The run-time pass kernels (ps_kernels_body.cuh) instantiated for Rader
// plans (FP32, plan variant PV_RADER): stage 0 of a transform runs each of
// its p-point DFTs as a cyclic convolution of p - 1 points (rader_lines in
// ps_fft.cuh). Kernels of their own, so that the Rader path's registers do
// not count against the kernels of the other plans, and a translation unit
// of its own, so that they compile beside the other instantiations. The z
// pass takes its spectral operation at run time.
#include "ps_kernels_body.cuh"

namespace ps {
namespace rt {

cudaError_t xfwd_rader(const XFwdArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    return run(k_xfwd<float, true>, grid, nt, sm, st, a);
}
cudaError_t col_rader(int inverse, const ColArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    return inverse ? run(k_col<float, true, true>, grid, nt, sm, st, a)
                   : run(k_col<float, false, true>, grid, nt, sm, st, a);
}
cudaError_t z_rader(const ZArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    return run(k_z<float, -1, true>, grid, nt, sm, st, a);
}
cudaError_t xinv_rader(const XInvArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    return run(k_xinv<float, true>, grid, nt, sm, st, a);
}
cudaError_t xfwd_batch_rader(const XFwdArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                             cudaStream_t st)
{
    return run_tiles(k_xfwd_batch<float, true>, args, tiles, ntiles, nt, smem, st);
}
cudaError_t col_batch_rader(int inverse, const ColArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                            cudaStream_t st)
{
    return inverse ? run_tiles(k_col_batch<float, true, true>, args, tiles, ntiles, nt, smem, st)
                   : run_tiles(k_col_batch<float, false, true>, args, tiles, ntiles, nt, smem, st);
}
cudaError_t z_batch_rader(const ZArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem, cudaStream_t st)
{
    return run_tiles(k_z_batch<float, true>, args, tiles, ntiles, nt, smem, st);
}
cudaError_t xinv_batch_rader(const XInvArgs *args, const BatchTile *tiles, int ntiles, int nt, size_t smem,
                             cudaStream_t st)
{
    return run_tiles(k_xinv_batch<float, true>, args, tiles, ntiles, nt, smem, st);
}

}  // namespace rt
}  // namespace ps
