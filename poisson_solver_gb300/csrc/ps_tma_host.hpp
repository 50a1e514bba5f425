// Host side of the tiled bulk copies: tensor maps over the half spectra.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>

namespace ps {
namespace tma {

// cuTensorMapEncodeTiled from the driver, looked up once (null if absent).
inline PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
    });
    return fn;
}

// A spectrum array [planes][rows][pitch] of complex floats seen as floats:
// x extent 2 mx (the pitch padding lies outside the tensor), rows and
// planes `row_bytes` and `plane_bytes` apart (multiples of 16). Boxes of 8
// complex columns (64 bytes) x box_rows x box_planes, 64-byte swizzle;
// reads past the tensor fill zeros.
inline bool encode_spectrum(CUtensorMap *m, const void *p, int mx, int rows, int planes, long long row_bytes,
                            long long plane_bytes, int box_rows, int box_planes)
{
    const auto fn = encode_fn();
    if (!fn || !p || (reinterpret_cast<uintptr_t>(p) & 15) || row_bytes % 16 || plane_bytes % 16) return false;
    cuuint64_t dims[3] = {(cuuint64_t)(2 * mx), (cuuint64_t)rows, (cuuint64_t)planes};
    cuuint64_t strides[2] = {(cuuint64_t)row_bytes, (cuuint64_t)plane_bytes};
    cuuint32_t box[3] = {16, (cuuint32_t)box_rows, (cuuint32_t)box_planes};
    cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(p), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// SM count of the current device, cached per device ordinal (a process may
// hold handles on GPUs of different models).
inline int sm_count()
{
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cache[kMaxDevices];  // 0: not yet read
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        cudaGetLastError();
        return 1;
    }
    if (dev < kMaxDevices) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int v = 0;
    const bool ok = cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0;
    cudaGetLastError();
    if (!ok) return 1;
    if (dev < kMaxDevices) cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

}  // namespace tma
}  // namespace ps
