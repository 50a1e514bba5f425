// y passes, one warp per column group, fed by tiled bulk copies (FP32;
// L = 256, 512, 1024; on an unbounded y axis the forward pass reads L/2
// rows and writes L, the inverse reads L and writes L/2; on a periodic one
// both read and write L).
//
// A tile is one z plane x 8 (32 / TPL) columns x one component. A column's
// L/32 threads are consecutive lanes of one warp, so the exchange between the
// two radix-32 stages needs only a warp barrier and the eight compute warps
// run independently. Global memory is moved in boxes of 8 columns (64-byte
// rows, 64-byte swizzle) x up to 256 y rows by two producer warps:
//   * the load warp keeps the next tiles' inputs in flight (full/empty
//     mbarriers over the input staging);
//   * the store warp waits until every compute thread has written a tile's
//     outputs into the output staging, starts the tiled stores and releases
//     the staging once the copies have read it.
// Inputs are double-buffered. The unbounded forward pass exchanges between
// its stages through padded line buffers and single-buffers its (full-size)
// output. Where the input holds all L rows (the unbounded inverse, both
// periodic passes) the pass exchanges inside its own input staging, whose
// column of L rows is free once the column's first stage has read them
// (positions p held at row p ^ ((p >> 5) & 7), two-way bank conflicts),
// which leaves room to double-buffer the full-size input that the loads must
// keep ahead of. Either way the shared memory of one CTA per SM is full.
// The CTAs are persistent, one per SM, and
// take tiles from a global counter in order: the CTAs then work on
// neighbouring tiles at any time (the same y rows of adjacent column groups),
// where a fixed round-robin assignment drifts apart over hundreds of tiles
// and loses DRAM page locality (3.7 against 2.5 ms for the 512^3 forward
// pass). The load warp draws the tiles and passes each tile's index along
// with its data; the compute warps pass it on to the store warp.
//
// Every mbarrier wait is bounded; a warp whose wait runs out stops and sets
// bit 0 of status[0], the load warp waits for its copies in flight, and the
// other warps' waits run out in turn. status[1] is the tile counter.
#include <cstring>

#include "ps_async.cuh"
#include "ps_tma_host.hpp"
#include "ps_wide.cuh"

namespace ps {
namespace wide {

namespace {

using namespace async;

constexpr int YQ_COMPUTE = 256;                // compute threads (8 warps)
constexpr int YQ_THREADS = YQ_COMPUTE + 64;     // + load warp + store warp
constexpr int LOAD_WARP = YQ_COMPUTE / 32, STORE_WARP = LOAD_WARP + 1;

// HALF: the y axis is unbounded (forward n_in = L/2, inverse n_out = L/2);
// else periodic (n_in = n_out = L).
template <int L, bool INV, bool HALF> struct Yq {
    static constexpr int TPL = L / 32;          // threads a column
    static constexpr int B = YQ_COMPUTE / TPL;  // columns a CTA
    static constexpr int G = B / 8;             // 64-byte column groups
    static constexpr int IN_ROWS = (HALF && !INV) ? L / 2 : L, OUT_ROWS = (HALF && INV) ? L / 2 : L;
    static constexpr bool XIN = IN_ROWS == L;     // exchange inside the input staging (no line buffers)
    static constexpr int NIN = 2, NOUT = OUT_ROWS == L ? 1 : 2;  // staging buffers
    static constexpr int NBI = IN_ROWS > 256 ? IN_ROWS / 256 : 1, BI = IN_ROWS / NBI;
    static constexpr int NBO = OUT_ROWS > 256 ? OUT_ROWS / 256 : 1, BO = OUT_ROWS / NBO;
    static constexpr int IN_GROUP = IN_ROWS * 64, OUT_GROUP = OUT_ROWS * 64;
    static constexpr int IN_BYTES = G * IN_GROUP, OUT_BYTES = G * OUT_GROUP;
    static constexpr int LDP = pitch_row(L);
    // byte offsets from the 1024-aligned base
    static constexpr int IN0 = 0, OUT0 = NIN * IN_BYTES, LINES = OUT0 + NOUT * OUT_BYTES;
    static constexpr int TWO = LINES + (XIN ? 0 : B * LDP * 8);
    __host__ __device__ static constexpr int bars(int ntw) { return (TWO + ntw * 8 + 15) & ~15; }
    __host__ __device__ static constexpr int bytes(int ntw) { return bars(ntw) + 8 * 8 + 16 + 1024; }  // + alignment slack
    static_assert(G >= 1 && G * 8 == B, "whole 64-byte column groups");
    static_assert(IN_GROUP % 1024 == 0 && OUT_GROUP % 1024 == 0 && (BI * 64) % 1024 == 0 && (BO * 64) % 1024 == 0,
                  "boxes keep the swizzle phase");
};

struct YqMaps {
    CUtensorMap in[3];
    CUtensorMap out[3];
};

__device__ __forceinline__ bool warp_ok(bool ok) { return __all_sync(0xffffffffu, ok); }

template <int L, bool INV, bool HALF>
__global__ void __launch_bounds__(YQ_THREADS, 1)
    k_yq(const ColArgs a, const __grid_constant__ YqMaps maps, const int nxt, const int nplanes, const int ntiles,
         int *status)
{
    using C = float2;
    using PL = WP<L>;
    using Q = Yq<L, INV, HALF>;
    constexpr int LAST = PL::NST - 1;
    using T0 = St<L, 0>;
    using TL = St<L, LAST>;
    static_assert(T0::U == 1 && T0::R == 32, "one radix-32 butterfly a thread in the first stage");
    static_assert(PL::NST == 2, "two stages: one exchange");
    // staged rows t + r NBF (first stage) and out_pos(t, u, r) = r M + t + u TPL
    // (last stage) are congruent to t modulo 8: one swizzle term a thread
    static_assert(T0::NBF % 8 == 0 && TL::M % 8 == 0 && TL::TPL % 8 == 0 && TL::U * TL::TPL <= TL::M,
                  "staged rows share t's swizzle term");

    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const uint32_t sb = smem_u32(base);
    C *TW = reinterpret_cast<C *>(base + Q::TWO);
    const uint32_t full0 = sb + Q::bars(PL::NTW), empty0 = full0 + 16, ofull0 = full0 + 32, oempty0 = full0 + 48;
    // tile index of each input buffer (written by the load warp) and output
    // buffer (by compute thread 0); -1 marks the end
    volatile int *itile = reinterpret_cast<volatile int *>(base + Q::bars(PL::NTW) + 64);
    volatile int *otile = itile + 2;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, YQ_COMPUTE);
            mbar_init(ofull0 + 8 * s, YQ_COMPUTE);
            mbar_init(oempty0 + 8 * s, 1);
        }
        fence_mbar_init();
    }
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    __syncthreads();

    // tile j -> component, z plane, first column (columns fastest)
    auto tile = [&](int j, int &c, int &z, int &x0) {
        x0 = (j % nxt) * Q::B;
        const int r = j / nxt;
        z = r % nplanes;
        c = r / nplanes;
    };
    bool ok = true;

    if (warp == LOAD_WARP) {
        if (lane == 0) {
            int last[2] = {-1, -1};  // newest load of each buffer not yet known to be complete
            // the next tile index is drawn one tile ahead: the atomic's round
            // trip overlaps the wait for a free buffer
            int jn = atomicAdd(status + 1, 1);
            for (int q = 0;; ++q) {
                const int s = q % Q::NIN;
                if (q >= Q::NIN && !mbar_wait(empty0 + 8 * s, ((q / Q::NIN) - 1) & 1)) {
                    ok = false;
                    break;
                }
                last[s] = -1;  // every compute thread has read it
                const int j = jn;
                if (j >= ntiles) {  // end of the tiles: a marker in place of data
                    itile[s] = -1;
                    mbar_arrive(full0 + 8 * s);
                    break;
                }
                itile[s] = j;
                int c, z, x0;
                tile(j, c, z, x0);
                mbar_arrive_expect_tx(full0 + 8 * s, Q::IN_BYTES);
                for (int g = 0; g < Q::G; ++g)
                    for (int bz = 0; bz < Q::NBI; ++bz)
                        tma_load_3d(sb + Q::IN0 + s * Q::IN_BYTES + g * Q::IN_GROUP + bz * Q::BI * 64, &maps.in[c],
                                    2 * (x0 + 8 * g), bz * Q::BI, z, full0 + 8 * s);
                last[s] = q;
                jn = atomicAdd(status + 1, 1);
            }
            // no copy may outlive the CTA
            for (int s = 0; s < Q::NIN; ++s)
                if (last[s] >= 0) mbar_wait(full0 + 8 * s, (last[s] / Q::NIN) & 1);
        }
    } else if (warp == STORE_WARP) {
        if (lane == 0) {
            for (int q = 0;; ++q) {
                const int so = q % Q::NOUT;
                if (!mbar_wait(ofull0 + 8 * so, (q / Q::NOUT) & 1)) {
                    ok = false;
                    break;
                }
                const int j = otile[so];
                if (j < 0) break;
                int c, z, x0;
                tile(j, c, z, x0);
                for (int g = 0; g < Q::G; ++g) {
                    if (x0 + 8 * g >= a.Mx) break;
                    for (int bz = 0; bz < Q::NBO; ++bz)
                        tma_store_3d(&maps.out[c], 2 * (x0 + 8 * g), bz * Q::BO, z,
                                     sb + Q::OUT0 + so * Q::OUT_BYTES + g * Q::OUT_GROUP + bz * Q::BO * 64);
                }
                bulk_commit();
                bulk_wait_read<Q::NOUT - 1>();  // store q - NOUT + 1 has read its staging: release it
                if (q + 1 >= Q::NOUT) mbar_arrive(oempty0 + 8 * ((q + 1 - Q::NOUT) % Q::NOUT));
            }
            bulk_wait_all();
        }
    } else {
        const int b = tid / Q::TPL, t = tid % Q::TPL;
        C *line = reinterpret_cast<C *>(base + Q::LINES) + b * Q::LDP;  // forward only
        const int c8 = b & 7, sw = swizzle64_col(t, c8);
        int q = 0;
        for (;; ++q) {
            const int s = q % Q::NIN;
            ok = warp_ok(mbar_wait(full0 + 8 * s, (q / Q::NIN) & 1));
            if (!ok) break;
            const int j = itile[s];
            if (j < 0) break;
            unsigned char *stg = base + Q::IN0 + s * Q::IN_BYTES + (b >> 3) * Q::IN_GROUP;
            C v[TL::U][TL::R];
            if constexpr (!Q::XIN) {
                C v0[1][32];
                // rows >= L/2 are the zero padding
#pragma unroll
                for (int r = 0; r < 16; ++r)
                    v0[0][r] = *reinterpret_cast<const C *>(stg + sw + T0::in_pos(t, 0, r) * 64);
                mbar_arrive(empty0 + 8 * s);
                dft32_half<false>(v0[0]);
                write_line<L, 0>(line, t, v0);
                __syncwarp();
                read_line<L, LAST>(line, t, v);
                twiddle_dft<L, LAST, false>(v, TW, t);
                __syncwarp();  // the next tile rewrites the line
            } else {
                // exchange through this column's rows of the staging
                auto slot = [&](int p) { return reinterpret_cast<C *>(stg + swizzle64(p ^ ((p >> 5) & 7), c8)); };
                C v0[1][32];
#pragma unroll
                for (int r = 0; r < 32; ++r)
                    v0[0][r] = *reinterpret_cast<const C *>(stg + sw + T0::in_pos(t, 0, r) * 64);
                twiddle_dft<L, 0, INV>(v0, TW, t);
                __syncwarp();  // the column's lanes have read its rows
#pragma unroll
                for (int r = 0; r < 32; ++r) *slot(T0::out_pos(t, 0, r)) = v0[0][r];
                __syncwarp();
#pragma unroll
                for (int u = 0; u < TL::U; ++u)
#pragma unroll
                    for (int r = 0; r < TL::R; ++r) v[u][r] = *slot(TL::in_pos(t, u, r));
                mbar_arrive(empty0 + 8 * s);
                twiddle_dft<L, LAST, INV>(v, TW, t);
            }

            const int so = q % Q::NOUT;
            if (q >= Q::NOUT) {
                ok = warp_ok(mbar_wait(oempty0 + 8 * so, ((q / Q::NOUT) - 1) & 1));
                if (!ok) break;
            }
            unsigned char *ostg = base + Q::OUT0 + so * Q::OUT_BYTES + (b >> 3) * Q::OUT_GROUP;
            // unbounded inverse: out_pos = r M + bf with bf < M = L / R, so r < R/2 is the kept half
            constexpr int RW = Q::OUT_ROWS < L ? TL::R / 2 : TL::R;
#pragma unroll
            for (int u = 0; u < TL::U; ++u)
#pragma unroll
                for (int r = 0; r < RW; ++r)
                    *reinterpret_cast<C *>(ostg + sw + TL::out_pos(t, u, r) * 64) = v[u][r];
            if (tid == 0) otile[so] = j;
            fence_proxy_async_smem();
            mbar_arrive(ofull0 + 8 * so);
        }
        if (ok) {  // end marker for the store warp
            const int so = q % Q::NOUT;
            if (q >= Q::NOUT) ok = warp_ok(mbar_wait(oempty0 + 8 * so, ((q / Q::NOUT) - 1) & 1));
            if (ok) {
                if (tid == 0) otile[so] = -1;
                mbar_arrive(ofull0 + 8 * so);
            }
        }
    }
    if (!ok && lane == 0) atomicOr(status, 1);
}

template <int L, bool INV, bool HALF> cudaError_t launch_yq_t(const ColArgs &a, int nplanes, int *status, cudaStream_t st)
{
    using Q = Yq<L, INV, HALF>;
    YqMaps maps;
    memset(&maps, 0, sizeof(maps));
    for (int c = 0; c < a.ncomp; ++c) {
        if (!tma::encode_spectrum(&maps.in[c], a.data[c], a.Mx, L, nplanes, a.axis_stride * 8, a.outer_stride * 8,
                                  Q::BI, 1) ||
            !tma::encode_spectrum(&maps.out[c], a.data[c], a.Mx, L, nplanes, a.axis_stride * 8, a.outer_stride * 8,
                                  Q::BO, 1))
            return cudaErrorInvalidValue;
    }
    const int nxt = (a.Mx + Q::B - 1) / Q::B, ntiles = nxt * nplanes * a.ncomp;
    if (ntiles <= 0) return cudaSuccess;
    const int grid = ntiles < tma::sm_count() ? ntiles : tma::sm_count();
    const size_t sm = Q::bytes(a.plan.ntw);
    cudaError_t e = cudaFuncSetAttribute(k_yq<L, INV, HALF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(status + 1, 0, sizeof(int), st)) != cudaSuccess) return e;  // tile counter
    k_yq<L, INV, HALF><<<grid, YQ_THREADS, sm, st>>>(a, maps, nxt, nplanes, ntiles, status);
    return cudaGetLastError();
}

template <int L> size_t yq_bytes(int inverse, int half, int ntw)
{
    if (half) return inverse ? Yq<L, true, true>::bytes(ntw) : Yq<L, false, true>::bytes(ntw);
    return inverse ? Yq<L, true, false>::bytes(ntw) : Yq<L, false, false>::bytes(ntw);
}

template <int L> cudaError_t launch_yq_len(int inverse, int half, const ColArgs &a, int nplanes, int *status, cudaStream_t st)
{
    if (half) return inverse ? launch_yq_t<L, true, true>(a, nplanes, status, st) : launch_yq_t<L, false, true>(a, nplanes, status, st);
    return inverse ? launch_yq_t<L, true, false>(a, nplanes, status, st) : launch_yq_t<L, false, false>(a, nplanes, status, st);
}

// unbounded (the zero-padded half pruned) or periodic
int yq_half(int inverse, int L, int n_in, int n_out)
{
    if (inverse ? (n_in == L && 2 * n_out == L) : (2 * n_in == L && n_out == L)) return 1;
    if (n_in == L && n_out == L) return 0;
    return -1;
}


}  // namespace

bool yq_supported(int prec, int inverse, int L, int n_in, int n_out)
{
    return prec == PREC_FP32 && (L == 256 || L == 512 || L == 1024) && yq_half(inverse, L, n_in, n_out) >= 0 &&
           tma::encode_fn() != nullptr;
}

int yq_lines(int L) { return L >= 32 ? YQ_COMPUTE / (L / 32) : 0; }

size_t smem_lines_yq(int inverse, int L, int n_in, int n_out, int ntw_entries)
{
    const int half = yq_half(inverse, L, n_in, n_out);
    if (half < 0) return 0;
    switch (L) {
    case 256: return yq_bytes<256>(inverse, half, ntw_entries);
    case 512: return yq_bytes<512>(inverse, half, ntw_entries);
    case 1024: return yq_bytes<1024>(inverse, half, ntw_entries);
    default: return 0;
    }
}

cudaError_t launch_yq(int inverse, const ColArgs &a, int nplanes, int *status, cudaStream_t st)
{
    if (!status || a.B != yq_lines(a.L) || a.ncomp < 1 || a.ncomp > 3 ||
        !yq_supported(PREC_FP32, inverse, a.L, a.n_in, a.n_out))
        return cudaErrorInvalidConfiguration;
    const int half = yq_half(inverse, a.L, a.n_in, a.n_out);
    switch (a.L) {
    case 256: return launch_yq_len<256>(inverse, half, a, nplanes, status, st);
    case 512: return launch_yq_len<512>(inverse, half, a, nplanes, status, st);
    case 1024: return launch_yq_len<1024>(inverse, half, a, nplanes, status, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace wide
}  // namespace ps
