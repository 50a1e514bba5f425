// Fused z pass, one warp per z-column, fed by tiled bulk copies, with the
// transforms in packed pair arithmetic, two CTAs a SM (FP32; L = 1024 along an
// unbounded z axis: n_in = n_out = 512).
//
// The data flow is k_zq's (ps_kernels_zq.cu) for L = 1024: a thread holds 32
// values of its column, a transform is two radix-32 stages with one exchange
// through shared memory, the spectral operation works on the values the
// thread holds after the forward stages (the other components parked in
// tensor memory), and the inverse is the adjoint. Two things differ.
//
// 1. A thread holds its 32 values as 16 pairs (ps_fftp.cuh): the even and
//    odd inputs of each 32-point DFT, (v[2i], v[2i+1]), on the way in, the
//    halves (V[k], V[k+16]) on the way out. A packed FP32 instruction holds
//    the FMA pipe for two cycles, so this saves issue slots, not pipe time;
//    what it buys is registers: the kernel fits in 128 a thread without
//    spilling (the complex-layout kernel spills about 1 KB a thread there).
// 2. That allows two CTAs of 8 warps a SM, 4 warps a scheduler instead of 2,
//    which is what the complex-layout kernel lacks: its FMA pipe is busy only
//    half the time, the rest being dependency and barrier stalls that two
//    warps a scheduler cannot cover. Two CTAs fit in shared memory with one
//    staging buffer a CTA, used in turn by the component loads and the output
//    stores (the other CTA on the SM runs while one waits for a copy), and
//    with the kernel column fetched into the warp's own line buffer, which is
//    idle between the last forward exchange and the first inverse one.
//
// Staging buffer order in a tile: load c, read by all, load c + 1, ..., read
// of the last component, then for each output: write by all (after the last
// read, or after the previous store has been read out), tiled store, read-out
// wait; then the next tile's first load. Thread 0 starts every copy; lane 0
// of each warp fetches its kernel column. Every mbarrier wait is bounded and a
// warp decides with a vote whether to go on; on a timeout the CTA drains its
// copies, frees its tensor memory and sets bit 0 of *status.
#include <cstdlib>
#include <cstring>

#include "ps_async.cuh"
#include "ps_fftp.cuh"
#include "ps_tma_host.hpp"
#include "ps_tmem.cuh"
#include "ps_types.hpp"
#include "ps_zt.cuh"

namespace ps {
namespace wide {

namespace {

using namespace async;
using pk::P2;

namespace zp {
constexpr int L = 1024, NZ = 512;
constexpr int NT = 256;                             // 8 warps
constexpr int B = NT / 32;                          // 8 columns a tile: one 64-byte box group
constexpr int STAGE = B * NZ * 8;                   // one component of a tile
constexpr int KP = (L / 2 + 1 + 3) & ~3;            // z pitch of the z-fastest kernel octant
constexpr int TMEM_COLUMNS = 256;                   // two 64-column slots a thread, warps w and w + 4 apart
constexpr int LINE_BYTES = pk::LINE_RECORDS * 16;   // a column's line; its first KP floats take the kernel column
constexpr int S0 = 0, LINES = STAGE;
constexpr int TWS = LINES + B * LINE_BYTES;         // stage-1 twiddles, [pair i][lane t] {wr a, wr b, wi a, wi b}
constexpr int ROT = TWS + 32 * 16 * 16;             // the 16-point DFT's rotation constants, 12 floats
constexpr int BARS = (ROT + 48 + 15) & ~15;         // full, empty, out-full, out-empty, 8 kernel-column barriers
constexpr int BYTES = BARS + 12 * 8 + 16 + 1024;    // + TMEM address slot, alignment slack
static_assert(KP * 4 <= LINE_BYTES && LINE_BYTES % 16 == 0, "kernel column fits a line");
static_assert(2 * (BYTES + 1024) <= 233472, "two CTAs a SM");
}  // namespace zp

struct ZqpMaps {
    CUtensorMap in[3];
    CUtensorMap out[3];
};

__device__ __forceinline__ bool warp_okp(bool ok) { return __all_sync(0xffffffffu, ok); }

// 16 pairs <-> 64 columns of the thread's TMEM row
__device__ __forceinline__ void stash_p(uint32_t taddr, const P2 (&v)[16])
{
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
        uint32_t w[16];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const P2 &p = v[4 * ch + e];
            w[4 * e] = __float_as_uint(p.r.x);
            w[4 * e + 1] = __float_as_uint(p.r.y);
            w[4 * e + 2] = __float_as_uint(p.i.x);
            w[4 * e + 3] = __float_as_uint(p.i.y);
        }
        tmem::st16(taddr + 16 * ch, w);
    }
}

__device__ __forceinline__ void unstash_p(uint32_t taddr, P2 (&v)[16])
{
    uint32_t w[4][16];
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) tmem::ld16(taddr + 16 * ch, w[ch]);
    tmem::wait_ld16x2(w[0], w[1]);
    tmem::wait_ld16x2(w[2], w[3]);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const uint32_t *s = &w[k / 4][4 * (k % 4)];
        v[k].r = make_float2(__uint_as_float(s[0]), __uint_as_float(s[1]));
        v[k].i = make_float2(__uint_as_float(s[2]), __uint_as_float(s[3]));
    }
}

template <int OP>
__global__ void __launch_bounds__(zp::NT, 2)
    k_zqp(const ZArgs a, const __grid_constant__ ZqpMaps maps, const int nxt, const int ntiles, int *status)
{
    using namespace zp;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const uint32_t sb = smem_u32(base);
    const float4 *TW = reinterpret_cast<const float4 *>(base + TWS);
    const uint32_t full = sb + BARS, empty = full + 8, ofull = full + 16, oempty = full + 24;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(base + BARS + 12 * 8);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int b = warp, t = lane;  // a warp a column
    const uint32_t gbar = full + 32 + 8 * warp;
    if (tid == 0) {
        mbar_init(full, 1);
        mbar_init(empty, NT);
        mbar_init(ofull, NT);
        mbar_init(oempty, 1);
        for (int w = 0; w < B; ++w) mbar_init(full + 32 + 8 * w, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem::alloc(tslot, TMEM_COLUMNS);
        tmem::relinquish();
    }
    // stage-1 twiddles from the plan's table (radix 32, 32: stage 1 at entry
    // 31, W1024^(j r) at 31 + 31 j + r - 1), as pairs of r = 2i, 2i + 1
    {
        const float2 *g = reinterpret_cast<const float2 *>(a.plan.table) + 31;
        float4 *tw = reinterpret_cast<float4 *>(base + TWS);
        for (int e = tid; e < 32 * 16; e += NT) {
            const int i = e >> 5, j = e & 31;
            const float2 wa = i == 0 ? make_float2(1.f, 0.f) : __ldg(&g[j * 31 + 2 * i - 1]);
            const float2 wb = __ldg(&g[j * 31 + 2 * i]);
            tw[e] = make_float4(wa.x, wb.x, wa.y, wb.y);
        }
        if (tid == 0) pk::store_rot_consts(reinterpret_cast<float *>(base + ROT));
    }
    tmem::fence_before_sync();
    __syncthreads();
    tmem::fence_after_sync();
    const pk::RotConsts rk = pk::load_rot_consts(reinterpret_cast<const float *>(base + ROT));
    const uint32_t tbase = *tslot + tmem::lane_base(warp) + (uint32_t)((warp >> 2) * 128);

    float *line = reinterpret_cast<float *>(base + LINES) + b * pk::LINE_RECORDS * 4;
    const uint32_t line_s = sb + LINES + b * LINE_BYTES;
    const float *gsm = line;                // the kernel column, between the forward and inverse exchanges
    const int goff = swizzle64_col(t, b);  // rows t + 32 m share t's swizzle term
    const int nin = a.nin;
    int nst = 0;  // outputs stored a tile (uniform)
    for (int oc = 0; oc < a.nout; ++oc) nst += a.out[oc] != nullptr;
    const int nloc = (int)blockIdx.x < ntiles ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;

    // thread 0: start load q (tile q / nin, component q % nin); the caller
    // has made sure the staging buffer is free
    int issued = 0;
    auto issue = [&](int q) {
        const int j = (int)blockIdx.x + (q / nin) * (int)gridDim.x, c = q % nin;
        const int ky = a.ky0 + j / nxt, x0 = (j % nxt) * B;
        mbar_arrive_expect_tx(full, STAGE);
        for (int bz = 0; bz < 2; ++bz)
            tma_load_3d(sb + S0 + bz * 256 * 64, &maps.in[c], 2 * x0, ky, bz * 256, full);
        issued = q + 1;
    };
    if (tid == 0 && nloc > 0) issue(0);

    // lane 0: copy this warp's kernel column of local tile i into its line
    int g_issued = 0, g_waited = 0;
    auto issue_g = [&](int i) {
        const int j = (int)blockIdx.x + i * (int)gridDim.x;
        const int ky = a.ky0 + j / nxt, x0 = (j % nxt) * B;
        const int oyr = imin(ky, a.Py - ky), kx = x0 + b;
        const bool on = kx < a.Mx;
        mbar_arrive_expect_tx(gbar, on ? KP * 4 : 0);
        if (on) bulk_load(line_s, a.kern_zf + ((long long)oyr * a.Mx + kx) * KP, KP * 4, gbar);
        g_issued = i + 1;
    };

    bool ok = true;
    int consumed = 0;  // loads thread 0 has waited for
    int so = 0;        // stores of this CTA so far
    for (int i = 0; i < nloc && ok; ++i) {
        const int j = (int)blockIdx.x + i * (int)gridDim.x;
        const int ky = a.ky0 + j / nxt, x0 = (j % nxt) * B;
        const int kx = x0 + b;
        const bool active = kx < a.Mx;
        P2 cur[16];

        // forward transforms; components 0 .. nin-2 parked in TMEM
        for (int c = 0; c < nin; ++c) {
            const int q = i * nin + c;
            ok = warp_okp(ok && mbar_wait(full, q & 1));
            if (!ok) break;
            if (tid == 0) consumed = q + 1;
            const unsigned char *stg = base + S0 + goff;
            // stage 0: pairs (v[2i], v[2i+1]) = rows t + 64 i, t + 64 i + 32; rows >= 512 are zero
#pragma unroll
            for (int ii = 0; ii < 8; ++ii) {
                const float2 va = *reinterpret_cast<const float2 *>(stg + (t + 64 * ii) * 64);
                const float2 vb = *reinterpret_cast<const float2 *>(stg + (t + 64 * ii + 32) * 64);
                cur[ii].r = make_float2(va.x, vb.x);
                cur[ii].i = make_float2(va.y, vb.y);
            }
            mbar_arrive(empty);
            // the tile's next component once every thread has read this one
            if (tid == 0 && c + 1 < nin) {
                ok = mbar_wait(empty, q & 1);
                if (ok) issue(q + 1);
            }
            ok = warp_okp(ok);
            if (!ok) break;
            pk::pdft32_half<false>(cur, rk);
            pk::line_write_halves(line, t, cur);
            __syncwarp();
            pk::line_read_records(line, t, cur);
            // the line is read: the next transform, or the kernel column's copy, may rewrite it
            if (c + 1 == nin) fence_proxy_async_smem();
            __syncwarp();
            if (c + 1 == nin && lane == 0) issue_g(i);
            pk::line_twiddle<false>(cur, TW, t);
            pk::pdft32<false>(cur, rk);  // cur[k] = (X[t + 32 k], X[t + 32 k + 512])
            if (c + 1 < nin) stash_p(tbase + 64 * c, cur);
        }
        if (!ok) break;
        if (nin > 1) tmem::wait_st();

        ok = warp_okp(mbar_wait(gbar, i & 1));
        if (!ok) break;
        g_waited = i + 1;

        // spectral operation on pairs (kz = t + 32 k, t + 32 k + 512)
        {
            const float kyv = wavenumber<float>(ky, a.Py, (float)a.kyc, true);
            const float kxv = wavenumber<float>(kx, a.Px, (float)a.kxc, true);
            const float kzc = (float)a.kzc;
            const float2 kx2 = pk::dup(kxv), ky2 = pk::dup(kyv);
#pragma unroll
            for (int ch = 0; ch < 4; ++ch) {
                uint32_t w0[16], w1[16];
                if (nin > 1) tmem::ld16(tbase + 16 * ch, w0);
                if (nin > 2) tmem::ld16(tbase + 64 + 16 * ch, w1);
                if (nin > 1) tmem::wait_ld16x2(w0, w1);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int k = 4 * ch + e;
                    const int za = t + 32 * k, zb = za + 512;
                    const float2 g = active ? make_float2(gsm[za], gsm[L - zb]) : make_float2(0.f, 0.f);
                    const float2 kz2 = make_float2(wavenumber<float>(za, a.Pz, kzc, true), wavenumber<float>(zb, a.Pz, kzc, true));
                    const P2 ic = cur[k];
                    const P2 i0{make_float2(__uint_as_float(w0[4 * e]), __uint_as_float(w0[4 * e + 1])),
                                make_float2(__uint_as_float(w0[4 * e + 2]), __uint_as_float(w0[4 * e + 3]))};
                    const P2 i1{make_float2(__uint_as_float(w1[4 * e]), __uint_as_float(w1[4 * e + 1])),
                                make_float2(__uint_as_float(w1[4 * e + 2]), __uint_as_float(w1[4 * e + 3]))};
                    const float2 ng = make_float2(-g.x, -g.y);
                    P2 o0{}, o1{}, o2;
                    // i (g f) for a pair f: (-g f.i, g f.r)
                    auto ig = [&](float2 gg, float2 ngg, const P2 &f) { return P2{pk::mul2(ngg, f.i), pk::mul2(gg, f.r)}; };
                    if constexpr (OP == OP_NONE) {
                        o0 = pk::pscale(i0, g);
                        o1 = pk::pscale(i1, g);
                        o2 = pk::pscale(ic, g);
                    } else if constexpr (OP == OP_GRAD) {
                        // nin = 1: every output from the one input; nin = 3: output d from input d
                        const P2 a0 = a.nin > 1 ? i0 : ic, a1 = a.nin > 1 ? i1 : ic;
                        const float2 gx = pk::mul2(g, kx2), gy = pk::mul2(g, ky2), gz = pk::mul2(g, kz2);
                        o0 = ig(gx, make_float2(-gx.x, -gx.y), a0);
                        o1 = ig(gy, make_float2(-gy.x, -gy.y), a1);
                        o2 = ig(gz, make_float2(-gz.x, -gz.y), ic);
                    } else if constexpr (OP == OP_DIV) {
                        const P2 d{pk::fma2(kz2, ic.r, pk::fma2(ky2, i1.r, pk::mul2(kx2, i0.r))),
                                   pk::fma2(kz2, ic.i, pk::fma2(ky2, i1.i, pk::mul2(kx2, i0.i)))};
                        o2 = ig(g, ng, d);
                    } else {  // OP_CURL
                        const P2 c0{pk::sub2(pk::mul2(ky2, ic.r), pk::mul2(kz2, i1.r)),
                                    pk::sub2(pk::mul2(ky2, ic.i), pk::mul2(kz2, i1.i))};
                        const P2 c1{pk::sub2(pk::mul2(kz2, i0.r), pk::mul2(kx2, ic.r)),
                                    pk::sub2(pk::mul2(kz2, i0.i), pk::mul2(kx2, ic.i))};
                        const P2 c2{pk::sub2(pk::mul2(kx2, i1.r), pk::mul2(ky2, i0.r)),
                                    pk::sub2(pk::mul2(kx2, i1.i), pk::mul2(ky2, i0.i))};
                        o0 = ig(g, ng, c0);
                        o1 = ig(g, ng, c1);
                        o2 = ig(g, ng, c2);
                    }
                    w0[4 * e] = __float_as_uint(o0.r.x);
                    w0[4 * e + 1] = __float_as_uint(o0.r.y);
                    w0[4 * e + 2] = __float_as_uint(o0.i.x);
                    w0[4 * e + 3] = __float_as_uint(o0.i.y);
                    w1[4 * e] = __float_as_uint(o1.r.x);
                    w1[4 * e + 1] = __float_as_uint(o1.r.y);
                    w1[4 * e + 2] = __float_as_uint(o1.i.x);
                    w1[4 * e + 3] = __float_as_uint(o1.i.y);
                    cur[k] = o2;
                }
                if (a.nout > 1) tmem::st16(tbase + 16 * ch, w0);
                if (a.nout > 2) tmem::st16(tbase + 64 + 16 * ch, w1);
            }
            if (a.nout > 1) tmem::wait_st();
        }
        __syncwarp();  // every lane has read the kernel column: the inverse may rewrite the line

        // inverse transforms: output nout-1 from cur, then nout-2 .. 0 from TMEM
        int st = 0;  // stores of this tile so far
        for (int oc = a.nout - 1; oc >= 0; --oc) {
            if (!a.out[oc]) continue;  // uniform over the CTA
            if (oc < a.nout - 1) unstash_p(tbase + 64 * oc, cur);
            // adjoint of stage 1: inverse DFT of (X[t + 32 k], X[t + 32 k + 512]), conjugate twiddles
            pk::pdft32_from_halves<true>(cur, rk);
            pk::line_twiddle<true>(cur, TW, t);
            pk::line_write_records(line, t, cur);
            __syncwarp();
            // adjoint of stage 0
            pk::line_read_halves(line, t, cur);
            pk::pdft32_from_halves<true>(cur, rk);  // cur[i] = rows (t + 64 i, t + 64 i + 32); i < 8 kept
            __syncwarp();

            // the staging buffer is free once every thread has read the tile's
            // last component (first store) or the previous store has been read out
            ok = warp_okp(st == 0 ? mbar_wait(empty, (i * nin + nin - 1) & 1) : mbar_wait(oempty, (so - 1) & 1));
            if (!ok) break;
            unsigned char *ostg = base + S0 + goff;
#pragma unroll
            for (int ii = 0; ii < 8; ++ii) {
                *reinterpret_cast<float2 *>(ostg + (t + 64 * ii) * 64) = make_float2(cur[ii].r.x, cur[ii].i.x);
                *reinterpret_cast<float2 *>(ostg + (t + 64 * ii + 32) * 64) = make_float2(cur[ii].r.y, cur[ii].i.y);
            }
            fence_proxy_async_smem();
            mbar_arrive(ofull);
            if (tid == 0) {
                ok = mbar_wait(ofull, so & 1);
                if (ok) {
                    for (int bz = 0; bz < 2; ++bz)
                        tma_store_3d(&maps.out[oc], 2 * x0, ky, bz * 256, sb + S0 + bz * 256 * 64);
                    bulk_commit();
                    bulk_wait_read<0>();  // read out: the buffer is free
                    mbar_arrive(oempty);
                }
            }
            ok = warp_okp(ok);
            if (!ok) break;
            ++so;
            ++st;
        }
        if (!ok) break;
        // the next tile's first component: the buffer is free once the last
        // store has been read out (thread 0 waited for it) or, with nothing
        // stored, once every thread has read the last component
        if (tid == 0 && i + 1 < nloc) {
            ok = nst > 0 || mbar_wait(empty, (i * nin + nin - 1) & 1);
            if (ok) issue((i + 1) * nin);
        }
        ok = warp_okp(ok);
    }

    if (!ok && lane == 0) atomicOr(status, 1);
    if (tid == 0) {
        for (int q = consumed; q < issued; ++q) mbar_wait(full, q & 1);
        bulk_wait_all();
    }
    if (lane == 0 && g_waited < g_issued) mbar_wait(gbar, (g_issued - 1) & 1);
    tmem::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tmem::fence_after_sync();
        tmem::dealloc(*tslot, TMEM_COLUMNS);
    }
}

template <int OP> cudaError_t launch_zqp_op(const ZArgs &a, int ny, int *status, cudaStream_t st)
{
    using namespace zp;
    if (!a.kern_zf || a.kzp != KP || (reinterpret_cast<uintptr_t>(a.kern_zf) & 15) || a.plan.ntw != 31 + 32 * 31 ||
        a.plan.nstages != 2 || a.plan.radix[0] != 32 || a.plan.radix[1] != 32)
        return cudaErrorInvalidValue;
    ZqpMaps maps;
    memset(&maps, 0, sizeof(maps));
    // [n_in z][Py y][ld x]: boxes of 8 columns x 1 y row x 256 planes
    auto map = [&](CUtensorMap *m, const void *p) {
        return tma::encode_spectrum(m, p, a.Mx, a.Py, a.n_in, a.row_stride * 8, a.axis_stride * 8, 1, 256);
    };
    for (int c = 0; c < a.nin; ++c)
        if (!map(&maps.in[c], a.in[c])) return cudaErrorInvalidValue;
    for (int c = 0; c < a.nout; ++c)
        if (a.out[c] && !map(&maps.out[c], a.out[c])) return cudaErrorInvalidValue;
    const int nxt = (a.Mx + B - 1) / B, ntiles = nxt * ny;
    if (ntiles <= 0) return cudaSuccess;
    const int grid = ntiles < 2 * tma::sm_count() ? ntiles : 2 * tma::sm_count();  // two CTAs a SM
    cudaError_t e = cudaFuncSetAttribute(k_zqp<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_zqp<OP>, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    k_zqp<OP><<<grid, NT, BYTES, st>>>(a, maps, nxt, ntiles, status);
    return cudaGetLastError();
}

}  // namespace

bool zqp_supported(int prec, int L, int op, int nin, int nout, int n_in, int n_out)
{
    return prec == PREC_FP32 && L == zp::L && n_in == zp::NZ && n_out == zp::NZ &&
           (op == OP_NONE || op == OP_GRAD || op == OP_DIV || op == OP_CURL) && nin >= 1 && nin <= 3 && nout >= 1 &&
           nout <= 3 && tma::encode_fn() != nullptr;
}

size_t smem_zqp() { return zp::BYTES; }

cudaError_t launch_zqp(const ZArgs &a, int ny, int *status, cudaStream_t st)
{
    if (!status || a.B != ZQP_LINES || !zqp_supported(PREC_FP32, a.L, a.op, a.nin, a.nout, a.n_in, a.n_out))
        return cudaErrorInvalidConfiguration;
    switch (a.op) {
    case OP_NONE: return launch_zqp_op<OP_NONE>(a, ny, status, st);
    case OP_GRAD: return launch_zqp_op<OP_GRAD>(a, ny, status, st);
    case OP_DIV: return launch_zqp_op<OP_DIV>(a, ny, status, st);
    case OP_CURL: return launch_zqp_op<OP_CURL>(a, ny, status, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace wide
}  // namespace ps
