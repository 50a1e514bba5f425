// The run-time pass kernels (ps_kernels_body.cuh) in double-float
// arithmetic (ps_dfloat.cuh): FP64-class accuracy on the FP32 pipes. A
// translation unit of its own so it compiles beside the FP64 and FP32
// instantiations; five kernels (the z pass takes its spectral operation at
// run time), single problems only.
#include "ps_kernels_body.cuh"

namespace ps {
namespace rt {

cudaError_t xfwd_df(const XFwdArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    return xfwd<dfloat>(a, grid, nt, sm, st);
}
cudaError_t col_df(int inverse, const ColArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    return col<dfloat>(inverse, a, grid, nt, sm, st);
}
cudaError_t z_df(const ZArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    return z_any_op<dfloat>(a, grid, nt, sm, st);
}
cudaError_t xinv_df(const XInvArgs &a, dim3 grid, int nt, size_t sm, cudaStream_t st)
{
    return xinv<dfloat>(a, grid, nt, sm, st);
}

}  // namespace rt
}  // namespace ps
