// Fused z pass with tensor-memory staging (FP32, L = 256, 512, 1024, 2048).
//
// One CTA transforms B z-columns of every component: forward FFT, spectral
// operation, inverse FFT. After its last forward stage a thread holds the 32
// spectral values of its own positions n = out_pos(t, u, r) in registers. The
// components other than the last are parked in the thread's private row of
// tensor memory (two slots of 64 columns), so the spectral operation runs in
// registers on all three components at once, and the inverse transform
// starts from the same registers: it is the adjoint of the forward stages
// taken in reverse order (gather from a stage's output positions, inverse
// radix-R DFT, conjugate twiddles, scatter to its input positions), so its
// first stage needs the values of exactly the positions the thread owns.
//
// Shared memory carries only the exchanges inside each transform, through
// two line buffers used in turn (a transform writes one buffer, barrier,
// reads it; the next transform writes the other), one barrier per exchange.
// Against the wide fused kernel, which keeps all components in shared memory,
// this removes four of the eight shared-memory passes per component line and
// two of the three component buffers.
#include <map>
#include <mutex>
#include <tuple>

#include "ps_zt.cuh"

namespace ps {
namespace wide {

// HALF: the z axis is unbounded (n_in = n_out = L / 2). The first forward
// stage (one radix-32 butterfly a thread over n = t + r L/32) then has data
// only for r < 16, and the last inverse stage writes only r < 16: the loads,
// stores and the zero half of the DFT arithmetic drop out.
template <int L, int OP, bool HALF>
__global__ void __launch_bounds__(ZT_MAX_THREADS) k_zt(const ZArgs a, const int tm_cols)
{
    using C = float2;
    using T = float;
    using PL = WP<L>;
    constexpr int LAST = PL::NST - 1;
    using T0 = St<L, 0>;
    using TL = St<L, LAST>;
    static_assert(TL::U * TL::R == 32, "32 values per thread");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem_raw);
    C *TW = reinterpret_cast<C *>(smem_raw + 16);
    C *S = TW + PL::NTW;
    const int B = a.B, LDP = pitch_col(L, B), CS = B * LDP;
    const int warp = threadIdx.x >> 5;
    if (warp == 0) {
        tmem::alloc(tslot, tm_cols);
        tmem::relinquish();
    }
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    tmem::fence_before_sync();
    __syncthreads();
    tmem::fence_after_sync();
    const uint32_t tbase = *tslot + tmem::lane_base(warp) + (uint32_t)((warp >> 2) * 2 * SLOT_COLUMNS);

    const int lb = __ffs(B) - 1;
    const int b = threadIdx.x & (B - 1), t = threadIdx.x >> lb;
    const int x0 = blockIdx.x * B;
    const int ky = a.ky0 + blockIdx.y;
    const bool active = b < imin(B, a.Mx - x0);
    const long long off = (long long)ky * a.row_stride + x0 + b;
    const long long as = a.axis_stride;
    const int n_in = active ? a.n_in : 0;
    int ph = 0;  // transforms done: buffer ph & 1 is the next one

    // forward transform of input component c, ending in v (own positions)
    auto forward = [&](int c, C(&v)[TL::U][TL::R]) {
        C *line = S + (ph & 1) * CS + b * LDP;
        {
            const C *col = reinterpret_cast<const C *>(pick3(a.in, c)) + off;
            C v0[T0::U][T0::R];
            if constexpr (HALF) {
                static_assert(T0::U == 1 && T0::R == 32, "one radix-32 butterfly a thread in the first stage");
#pragma unroll
                for (int r = 0; r < 16; ++r) v0[0][r] = active ? col[T0::in_pos(t, 0, r) * as] : C{0.f, 0.f};
                dft32_half<false>(v0[0]);
            } else {
#pragma unroll
                for (int u = 0; u < T0::U; ++u)
#pragma unroll
                    for (int r = 0; r < T0::R; ++r) {
                        const int n = T0::in_pos(t, u, r);
                        v0[u][r] = n < n_in ? col[n * as] : C{0.f, 0.f};
                    }
                twiddle_dft<L, 0, false>(v0, TW, t);
            }
            write_line<L, 0>(line, t, v0);
        }
        __syncthreads();
        middle_stages<L, 1, false>(line, TW, t, 1, 0);
        read_line<L, LAST>(line, t, v);
        twiddle_dft<L, LAST, false>(v, TW, t);
        ++ph;
    };

    C cur[TL::U][TL::R];
    for (int c = 0; c + 1 < a.nin; ++c) {
        forward(c, cur);
        stash(tbase + c * SLOT_COLUMNS, cur);
    }
    forward(a.nin - 1, cur);
    if (a.nin > 1) tmem::wait_st();

    {
        // kernel octant [oz][oy][Mx]: column kx of row min(ky, Py - ky)
        const int kx = x0 + b;
        const T *Kc = reinterpret_cast<const T *>(a.kern) + (long long)imin(ky, a.Py - ky) * a.Mx + (active ? kx : 0);
        const long long kzs = (long long)a.oct_y * a.Mx;
        spectral_op<L, OP>(a, cur, tbase, ky, kx, t, [&](int m) { return active ? __ldg(&Kc[m * kzs]) : (T)0; });
    }

    // inverse transforms: output nout-1 from cur, then nout-2 .. 0 from TMEM
    for (int oc = a.nout - 1; oc >= 0; --oc) {
        C *col0 = reinterpret_cast<C *>(pick3(a.out, oc));
        if (!col0) continue;  // uniform over the CTA
        if (oc < a.nout - 1) unstash(tbase + oc * SLOT_COLUMNS, cur);
        C *line = S + (ph & 1) * CS + b * LDP;
        adjoint_dft<L, LAST>(cur, TW, t);
        write_in<L, LAST>(line, t, cur);
        __syncthreads();
        adjoint_middle<L, LAST - 1>(line, TW, t);
        C v0[T0::U][T0::R];
        read_out<L, 0>(line, t, v0);
        adjoint_dft<L, 0>(v0, TW, t);
        if (active) {
            C *col = col0 + off;
            if constexpr (HALF) {
#pragma unroll
                for (int r = 0; r < 16; ++r) col[T0::in_pos(t, 0, r) * as] = v0[0][r];
            } else {
#pragma unroll
                for (int u = 0; u < T0::U; ++u)
#pragma unroll
                    for (int r = 0; r < T0::R; ++r) {
                        const int n = T0::in_pos(t, u, r);
                        if (n < a.n_out) col[n * as] = v0[u][r];
                    }
            }
        }
        ++ph;
    }

    tmem::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tmem::fence_after_sync();
        tmem::dealloc(*tslot, tm_cols);
    }
}

// ---------------------------------------------------------------------------
namespace {

size_t smem_zt(int L, int B, int ntw) { return 16 + sizeof(float2) * ((size_t)ntw + 2 * (size_t)B * pitch_col(L, B)); }

// TMEM columns of one CTA: two 64-column slots per thread, warps w and w + 4
// on disjoint columns.
int columns_zt(int threads)
{
    const int warps = (threads + 31) / 32, rows = (warps + 3) / 4;
    int cols = 32;
    while (cols < rows * 2 * SLOT_COLUMNS) cols *= 2;
    return cols;
}

// Dynamic shared memory for a launch such that (resident CTAs per SM) x
// (TMEM columns per CTA) <= 512: a CTA's tcgen05.alloc then never waits for
// another CTA's columns. Returns 0 if no size achieves it.
template <typename K> size_t smem_for_columns(K kernel, int threads, size_t sm, int cols)
{
    static std::mutex mu;
    static std::map<std::tuple<const void *, int, size_t, int>, size_t> cache;
    const auto key = std::make_tuple((const void *)kernel, threads, sm, cols);
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    const int cap = tmem::COLUMNS_PER_SM / cols;
    int dev = 0, per_sm = 0, per_block = 0;
    size_t out = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&per_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess) {
        for (int attempt = 0; attempt < 2 && !out; ++attempt) {
            if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) break;
            int occ = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, sm) != cudaSuccess) break;
            if (occ >= 1 && occ <= cap) out = sm;
            else if (occ > cap) sm = std::max(sm, (size_t)per_sm / (cap + 1) + 1);
            if (sm > (size_t)per_block) break;
        }
    }
    cudaGetLastError();
    cache[key] = out;
    return out;
}

template <int L, int OP, bool HALF> cudaError_t launch_zt_half(const ZArgs &a, dim3 grid, int nt, cudaStream_t st)
{
    const int cols = columns_zt(nt);
    const size_t sm = smem_for_columns(k_zt<L, OP, HALF>, nt, smem_zt(L, a.B, a.plan.ntw), cols);
    if (!sm) return cudaErrorInvalidConfiguration;
    // the attribute is per kernel: another configuration may have lowered it
    const cudaError_t e =
        cudaFuncSetAttribute(k_zt<L, OP, HALF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_zt<L, OP, HALF><<<grid, nt, sm, st>>>(a, cols);
    return cudaGetLastError();
}

template <int L, int OP> cudaError_t launch_zt_op(const ZArgs &a, dim3 grid, int nt, cudaStream_t st)
{
    if (2 * a.n_in == L && 2 * a.n_out == L) return launch_zt_half<L, OP, true>(a, grid, nt, st);
    return launch_zt_half<L, OP, false>(a, grid, nt, st);
}

template <int L> cudaError_t launch_zt_len(const ZArgs &a, dim3 grid, int nt, cudaStream_t st)
{
    switch (a.op) {
    case OP_NONE: return launch_zt_op<L, OP_NONE>(a, grid, nt, st);
    case OP_GRAD: return launch_zt_op<L, OP_GRAD>(a, grid, nt, st);
    case OP_DIV: return launch_zt_op<L, OP_DIV>(a, grid, nt, st);
    case OP_CURL: return launch_zt_op<L, OP_CURL>(a, grid, nt, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool zt_supported(int prec, int L, int op, int nin, int nout)
{
    return prec == PREC_FP32 && (L == 256 || L == 512 || L == 1024 || L == 2048) &&
           (op == OP_NONE || op == OP_GRAD || op == OP_DIV || op == OP_CURL) && nin >= 1 && nin <= 3 && nout >= 1 &&
           nout <= 3;
}

size_t smem_lines_zt(int L, int B, int ntw_entries) { return smem_zt(L, B, ntw_entries); }

cudaError_t launch_zt(const ZArgs &a, int ny, cudaStream_t st)
{
    const int nt = a.B * (a.L / 32);
    // whole warps only: the tcgen05 instructions are warp-collective
    if (nt > ZT_MAX_THREADS || nt % 32 != 0) return cudaErrorInvalidConfiguration;
    dim3 grid((unsigned)((a.Mx + a.B - 1) / a.B), ny);
    switch (a.L) {
    case 256: return launch_zt_len<256>(a, grid, nt, st);
    case 512: return launch_zt_len<512>(a, grid, nt, st);
    case 1024: return launch_zt_len<1024>(a, grid, nt, st);
    case 2048: return launch_zt_len<2048>(a, grid, nt, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace wide
}  // namespace ps
