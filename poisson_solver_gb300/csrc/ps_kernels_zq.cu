// Fused z pass, one warp per z-column group, fed by tiled bulk copies (FP32;
// L = 256, 512, 1024 with an unbounded z axis: n_in = n_out = L / 2).
//
// Why: the CTA-wide fused kernels (ps_kernels_ztm.cu) spread each column's
// L/32 threads over all warps, for coalesced global accesses, so every
// exchange between stages is a CTA barrier; at 255 registers a thread one
// CTA of 8 warps fills the SM and each barrier (about 25 a tile) drains it,
// while each component's loads stall every warp at once.
//
// Here a column's threads are consecutive (L = 1024: one warp; 512: half a
// warp; 256: a quarter), so the exchanges need only warp barriers and the
// warps run independently. Global traffic goes through shared memory in
// boxes of 8 columns (64-byte rows) x the z rows, moved by the tensor-copy
// unit:
//   * inputs: thread 0 keeps two component loads in flight (double-buffered
//     staging, full/empty mbarriers); a warp reads its columns from the
//     swizzled box and releases the buffer;
//   * outputs: each warp writes its columns of the inverse transform into one
//     of two staging boxes; thread 0 waits for all of them (an mbarrier),
//     starts the tiled store and releases the box once the copy has read it;
//   * kernel values: lane 0 of each warp copies its columns of the z-fastest
//     kernel octant (one contiguous run a column) into the warp's own buffer
//     for the next tile as soon as the spectral operation has used them.
// One persistent CTA per SM walks the tiles (y row, 8 x (32 / TPL) columns);
// loads of the next tile overlap the current one's transforms.
//
// Every mbarrier wait is bounded; on a timeout the warp stops, the CTA drains
// its copies, frees its tensor memory and sets bit 0 of *status.
#include <cstdlib>
#include <cstring>

#include "ps_async.cuh"
#include "ps_tma_host.hpp"
#include "ps_zt.cuh"

namespace ps {
namespace wide {

namespace {

using namespace async;

// Geometry of a length-L CTA.
template <int L> struct Zq {
    static constexpr int TPL = L / 32;                 // threads a column
    static constexpr int B = ZQ_THREADS / TPL;          // columns a CTA
    static constexpr int G = B / 8;                     // 64-byte column groups (one box wide)
    static constexpr int SR = L / 2;                    // staged z rows
    static constexpr int NBOX = SR > 256 ? SR / 256 : 1;  // boxes along z (at most 256 rows a box)
    static constexpr int BOXZ = SR / NBOX;
    static constexpr int GROUP_BYTES = SR * 64;
    static constexpr int STAGE_BYTES = G * GROUP_BYTES;
    static constexpr int LDP = pitch_row(L);
    static constexpr int CPW = 32 / TPL;                // columns a warp
    static constexpr int KP = (L / 2 + 1 + 3) & ~3;     // z pitch of the z-fastest kernel octant
    // byte offsets from the 1024-aligned base: in staging 0/1, out staging
    // 0/1, lines, kernel columns, twiddles, mbarriers (full, empty, out-full,
    // out-empty pairs; one a warp for its kernel columns; the test probe),
    // TMEM address slot
    static constexpr int IN0 = 0, OUT0 = 2 * STAGE_BYTES, LINES = 4 * STAGE_BYTES;
    static constexpr int GBUF = LINES + B * LDP * 8;
    static constexpr int TWO = GBUF + B * KP * 4;
    __host__ __device__ static constexpr int bars(int ntw) { return (TWO + ntw * 8 + 15) & ~15; }
    __host__ __device__ static constexpr int bytes(int ntw) { return bars(ntw) + 24 * 8 + 16 + 1024; }  // + alignment slack
    static_assert(G >= 1 && G * 8 == B, "whole 64-byte column groups");
    static_assert(GROUP_BYTES % 1024 == 0 && (BOXZ * 64) % 1024 == 0, "boxes keep the swizzle phase");
};

constexpr int ZQ_TMEM_COLUMNS = 256;  // 8 warps: two 64-column slots a thread, warps w and w + 4 apart

struct ZqMaps {
    CUtensorMap in[3];
    CUtensorMap out[3];
};

// Warp-uniform success: a warp continues only if every lane's wait succeeded.
__device__ __forceinline__ bool warp_ok(bool ok) { return __all_sync(0xffffffffu, ok); }

template <int L, int OP>
__global__ void __launch_bounds__(ZQ_THREADS, 1)
    k_zq(const ZArgs a, const __grid_constant__ ZqMaps maps, const int nxt, const int ntiles, int *status, const int probe)
{
    using C = float2;
    using PL = WP<L>;
    using Q = Zq<L>;
    constexpr int LAST = PL::NST - 1;
    using T0 = St<L, 0>;
    using TL = St<L, LAST>;
    static_assert(T0::U == 1 && T0::R == 32, "one radix-32 butterfly a thread in the first stage");
    static_assert(TL::U * TL::R == 32, "32 values per thread");
    static_assert(T0::NBF % 8 == 0, "staged rows t + r NBF share t's swizzle term");

    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const uint32_t sb = smem_u32(base);
    C *TW = reinterpret_cast<C *>(base + Q::TWO);
    const int boff = Q::bars(PL::NTW);
    const uint32_t full0 = sb + boff, empty0 = full0 + 16, ofull0 = full0 + 32, oempty0 = full0 + 48;
    const uint32_t probe_bar = full0 + 128;  // never arrived at
    uint32_t *tslot = reinterpret_cast<uint32_t *>(base + boff + 192);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t gbar = full0 + 64 + 8 * warp;  // this warp's kernel-column barrier
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, ZQ_THREADS);
            mbar_init(ofull0 + 8 * s, ZQ_THREADS);
            mbar_init(oempty0 + 8 * s, 1);
        }
        for (int w = 0; w < ZQ_THREADS / 32; ++w) mbar_init(full0 + 64 + 8 * w, 1);
        mbar_init(probe_bar, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem::alloc(tslot, ZQ_TMEM_COLUMNS);
        tmem::relinquish();
    }
    load_twiddles<C, PL::NTW>(TW, a.plan.table);
    tmem::fence_before_sync();
    __syncthreads();
    tmem::fence_after_sync();
    const uint32_t tbase = *tslot + tmem::lane_base(warp) + (uint32_t)((warp >> 2) * 2 * SLOT_COLUMNS);

    const int b = tid / Q::TPL, t = tid % Q::TPL;  // column of the CTA, thread of the column
    C *line = reinterpret_cast<C *>(base + Q::LINES) + b * Q::LDP;
    const int goff = (b >> 3) * Q::GROUP_BYTES + swizzle64_col(t, b & 7);
    const int nin = a.nin;
    const int nloc = (int)blockIdx.x < ntiles ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    const int nq = nloc * nin;  // component loads of this CTA

    // thread 0: start load q (tile q / nin, component q % nin) into buffer q & 1
    // once load q - 2 has been read by every thread (it is called while load
    // q - 2 is being transformed, so a load has about two transforms to land)
    int issued = 0;
    auto issue = [&](int q) -> bool {
        const int s = q & 1;
        if (q >= 2 && !mbar_wait(empty0 + 8 * s, ((q >> 1) - 1) & 1)) return false;
        const int j = (int)blockIdx.x + (q / nin) * (int)gridDim.x, c = q % nin;
        const int ky = a.ky0 + j / nxt, x0 = (j % nxt) * Q::B;
        mbar_arrive_expect_tx(full0 + 8 * s, Q::STAGE_BYTES);
        for (int g = 0; g < Q::G; ++g)
            for (int bz = 0; bz < Q::NBOX; ++bz)
                tma_load_3d(sb + Q::IN0 + s * Q::STAGE_BYTES + g * Q::GROUP_BYTES + bz * Q::BOXZ * 64, &maps.in[c],
                            2 * (x0 + 8 * g), ky, bz * Q::BOXZ, full0 + 8 * s);
        issued = q + 1;
        return true;
    };
    if (tid == 0)
        for (int q = 0; q < 2 && q < nq; ++q) issue(q);

    // lane 0: copy the kernel columns of this warp for local tile i
    const float *gsm = reinterpret_cast<const float *>(base + Q::GBUF) + b * Q::KP;
    int g_issued = 0, g_waited = 0;
    auto issue_g = [&](int i) {
        const int j = (int)blockIdx.x + i * (int)gridDim.x;
        const int ky = a.ky0 + j / nxt, x0 = (j % nxt) * Q::B;
        const int oyr = imin(ky, a.Py - ky), kx0 = x0 + warp * Q::CPW;
        const int ncol = imin(Q::CPW, a.Mx - kx0);
        mbar_arrive_expect_tx(gbar, ncol > 0 ? ncol * Q::KP * 4 : 0);
        for (int cw = 0; cw < ncol; ++cw)
            bulk_load(sb + Q::GBUF + (warp * Q::CPW + cw) * Q::KP * 4,
                      a.kern_zf + ((long long)oyr * a.Mx + kx0 + cw) * Q::KP, Q::KP * 4, gbar);
        g_issued = i + 1;
    };
    if (lane == 0 && nloc > 0) issue_g(0);

    // test hook: a wait on a barrier nothing arrives at runs out, and the
    // kernel winds down as after any timed-out wait
    bool ok = !probe || mbar_wait(probe_bar, 0);
    int qo = 0;        // output boxes of this CTA so far
    int consumed = 0;  // loads thread 0 has waited for
    for (int i = 0; i < nloc && ok; ++i) {
        const int j = (int)blockIdx.x + i * (int)gridDim.x;
        const int ky = a.ky0 + j / nxt, x0 = (j % nxt) * Q::B;
        const int kx = x0 + b;
        const bool active = kx < a.Mx;
        C cur[TL::U][TL::R];

        // forward transforms; components 0 .. nin-2 parked in TMEM
        for (int c = 0; c < nin; ++c) {
            const int q = i * nin + c, s = q & 1;
            ok = warp_ok(ok && mbar_wait(full0 + 8 * s, (q >> 1) & 1));
            if (!ok) break;
            if (tid == 0) consumed = q + 1;
            const unsigned char *stg = base + Q::IN0 + s * Q::STAGE_BYTES + goff;
            C v0[1][32];
#pragma unroll
            for (int r = 0; r < 16; ++r) v0[0][r] = *reinterpret_cast<const C *>(stg + T0::in_pos(t, 0, r) * 64);
            mbar_arrive(empty0 + 8 * s);
            dft32_half<false>(v0[0]);
            // refill this buffer with load q + 2 once every thread has read it
            if (tid == 0 && q + 2 < nq) ok = issue(q + 2);
            ok = warp_ok(ok);
            if (!ok) break;
            write_line<L, 0>(line, t, v0);
            __syncwarp();
            middle_stages<L, 1, false, true>(line, TW, t, 1, 0);
            read_line<L, LAST>(line, t, cur);
            twiddle_dft<L, LAST, false>(cur, TW, t);
            __syncwarp();  // the next transform rewrites the line
            if (c + 1 < nin) stash(tbase + c * SLOT_COLUMNS, cur);
        }
        if (!ok) break;
        if (nin > 1) tmem::wait_st();

        ok = warp_ok(mbar_wait(gbar, i & 1));
        if (!ok) break;
        g_waited = i + 1;
        spectral_op<L, OP>(a, cur, tbase, ky, kx, t, [&](int m) { return active ? gsm[m] : 0.f; });
        __syncwarp();  // every lane has read the kernel columns
        if (lane == 0 && i + 1 < nloc) issue_g(i + 1);

        // inverse transforms: output nout-1 from cur, then nout-2 .. 0 from TMEM
        for (int oc = a.nout - 1; oc >= 0; --oc) {
            if (!a.out[oc]) continue;  // uniform over the CTA
            if (oc < a.nout - 1) unstash(tbase + oc * SLOT_COLUMNS, cur);
            adjoint_dft<L, LAST>(cur, TW, t);
            write_in<L, LAST>(line, t, cur);
            __syncwarp();
            adjoint_middle<L, LAST - 1, true>(line, TW, t);
            C v0[T0::U][T0::R];
            read_out<L, 0>(line, t, v0);
            adjoint_dft<L, 0>(v0, TW, t);
            __syncwarp();

            const int so = qo & 1;
            if (qo >= 2) ok = warp_ok(mbar_wait(oempty0 + 8 * so, ((qo >> 1) - 1) & 1));
            if (!ok) break;
            unsigned char *ostg = base + Q::OUT0 + so * Q::STAGE_BYTES + goff;
            // rows < L / 2 (the cropped half is dropped)
#pragma unroll
            for (int r = 0; r < 16; ++r) *reinterpret_cast<C *>(ostg + T0::in_pos(t, 0, r) * 64) = v0[0][r];
            fence_proxy_async_smem();
            mbar_arrive(ofull0 + 8 * so);
            if (tid == 0) {
                ok = mbar_wait(ofull0 + 8 * so, (qo >> 1) & 1);
                if (ok) {
                    for (int g = 0; g < Q::G; ++g) {
                        if (x0 + 8 * g >= a.Mx) break;
                        for (int bz = 0; bz < Q::NBOX; ++bz)
                            tma_store_3d(&maps.out[oc], 2 * (x0 + 8 * g), ky, bz * Q::BOXZ,
                                         sb + Q::OUT0 + so * Q::STAGE_BYTES + g * Q::GROUP_BYTES + bz * Q::BOXZ * 64);
                    }
                    bulk_commit();
                    bulk_wait_read<1>();  // the previous box has been read: release it
                    if (qo >= 1) mbar_arrive(oempty0 + 8 * ((qo - 1) & 1));
                }
            }
            ok = warp_ok(ok);
            if (!ok) break;
            ++qo;
        }
    }

    if (!ok && (tid & 31) == 0) atomicOr(status, 1);
    if (tid == 0) {
        // loads started but never waited for (only after a failure), then the stores
        for (int q = consumed; q < issued; ++q) mbar_wait(full0 + 8 * (q & 1), (q >> 1) & 1);
        bulk_wait_all();
    }
    if (lane == 0 && g_waited < g_issued) mbar_wait(gbar, (g_issued - 1) & 1);
    tmem::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tmem::fence_after_sync();
        tmem::dealloc(*tslot, ZQ_TMEM_COLUMNS);
    }
}

template <int L, int OP> cudaError_t launch_zq_op(const ZArgs &a, int ny, int *status, cudaStream_t st)
{
    using Q = Zq<L>;
    if (!a.kern_zf || a.kzp != Q::KP || (reinterpret_cast<uintptr_t>(a.kern_zf) & 15)) return cudaErrorInvalidValue;
    ZqMaps maps;
    memset(&maps, 0, sizeof(maps));
    // [n_in z][Py y][ld x]: boxes of 8 columns x 1 y row x BOXZ planes
    auto map = [&](CUtensorMap *m, const void *p) {
        return tma::encode_spectrum(m, p, a.Mx, a.Py, a.n_in, a.row_stride * 8, a.axis_stride * 8, 1, Q::BOXZ);
    };
    for (int c = 0; c < a.nin; ++c)
        if (!map(&maps.in[c], a.in[c])) return cudaErrorInvalidValue;
    for (int c = 0; c < a.nout; ++c)
        if (a.out[c] && !map(&maps.out[c], a.out[c])) return cudaErrorInvalidValue;
    const int nxt = (a.Mx + Q::B - 1) / Q::B, ntiles = nxt * ny;
    if (ntiles <= 0) return cudaSuccess;
    const int grid = ntiles < tma::sm_count() ? ntiles : tma::sm_count();
    const size_t sm = Q::bytes(a.plan.ntw);
    cudaError_t e = cudaFuncSetAttribute(k_zq<L, OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    // PS_TEST_WAIT_TIMEOUT=1: every warp's first wait runs out (failure-path test)
    const char *probe = getenv("PS_TEST_WAIT_TIMEOUT");
    k_zq<L, OP><<<grid, ZQ_THREADS, sm, st>>>(a, maps, nxt, ntiles, status, probe && atoi(probe) == 1);
    return cudaGetLastError();
}

template <int L> cudaError_t launch_zq_len(const ZArgs &a, int ny, int *status, cudaStream_t st)
{
    switch (a.op) {
    case OP_NONE: return launch_zq_op<L, OP_NONE>(a, ny, status, st);
    case OP_GRAD: return launch_zq_op<L, OP_GRAD>(a, ny, status, st);
    case OP_DIV: return launch_zq_op<L, OP_DIV>(a, ny, status, st);
    case OP_CURL: return launch_zq_op<L, OP_CURL>(a, ny, status, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool zq_supported(int prec, int L, int op, int nin, int nout, int n_in, int n_out)
{
    return prec == PREC_FP32 && (L == 256 || L == 512 || L == 1024) && 2 * n_in == L && 2 * n_out == L &&
           (op == OP_NONE || op == OP_GRAD || op == OP_DIV || op == OP_CURL) && nin >= 1 && nin <= 3 && nout >= 1 &&
           nout <= 3 && tma::encode_fn() != nullptr;
}

int zq_lines(int L) { return L >= 32 ? ZQ_THREADS / (L / 32) : 0; }

size_t smem_lines_zq(int L, int ntw_entries)
{
    switch (L) {
    case 256: return Zq<256>::bytes(ntw_entries);
    case 512: return Zq<512>::bytes(ntw_entries);
    case 1024: return Zq<1024>::bytes(ntw_entries);
    default: return 0;
    }
}

cudaError_t launch_zq(const ZArgs &a, int ny, int *status, cudaStream_t st)
{
    if (!status || a.B != zq_lines(a.L) || !zq_supported(PREC_FP32, a.L, a.op, a.nin, a.nout, a.n_in, a.n_out))
        return cudaErrorInvalidConfiguration;
    switch (a.L) {
    case 256: return launch_zq_len<256>(a, ny, status, st);
    case 512: return launch_zq_len<512>(a, ny, status, st);
    case 1024: return launch_zq_len<1024>(a, ny, status, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace wide
}  // namespace ps
