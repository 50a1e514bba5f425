// Fused z pass with two warps a column, fed by tiled bulk copies (FP32; L =
// 1024 along an unbounded z axis: n_in = n_out = 512).
//
// Why: the one-warp-a-column kernel (ps_kernels_zq.cu, k_zq) holds 32
// values a thread for two radix-32 stages; at about 245 registers a thread
// its CTA of 8 warps fills the SM, and with two warps a scheduler the pass is
// bound by instruction latency (half the issue slots go unused). Here a
// column's 64 threads (two consecutive warps) hold 16 values each and run
// the transform as radix 16, 16, 4: twice the warps on the SM at no more than
// 128 registers, at the price of a second exchange through shared memory and
// a second twiddle step per transform. The two warps of a column synchronise
// with a 64-thread named barrier.
//
// Stages (t < 64 the thread of the column):
//   0: R = 16, M = 1,   reads t + 64 r,  writes 16 t + r
//   1: R = 16, M = 16,  reads t + 64 r,  twiddle (t mod 16), writes ((t/16) 16 + r) 16 + t mod 16
//   2: R = 4,  M = 256, four butterflies bf = t + 64 u: reads bf + 256 r, twiddle bf, outputs kz = 256 r + bf
// The forward stage 0 reads the input staging (rows z < 512 only: the
// zero-padded half is never loaded, r < 8); stage 2's outputs stay in
// registers for the spectral operation. The inverse is the adjoint, stage 2
// first on the values the thread holds, and its stage 0 writes rows z < 512
// to the output staging.
//
// Copies, tile order, staging and failure handling follow k_zq: thread 0
// keeps two component loads in flight, the first lane of each column fetches
// its kernel values, thread 0 starts the tiled stores; every mbarrier wait is
// bounded, a column's two warps decide together (an AND vote on their named
// barrier) whether to go on, and a failure drains the copies, frees the
// tensor memory and sets bit 0 of *status.
#include <cstdlib>
#include <cstring>

#include "ps_async.cuh"
#include "ps_fft_p2.cuh"
#include "ps_tma_host.hpp"
#include "ps_tmem.cuh"
#include "ps_types.hpp"
#include "ps_wide.cuh"

namespace ps {
namespace wide {

namespace {

using namespace async;

namespace z2 {
constexpr int L = 1024, NZ = 512;
constexpr int TPL = 64;                      // threads a column
constexpr int NT = 512;                      // 16 warps
constexpr int B = NT / TPL;                  // 8 columns a CTA: one 64-byte box group
constexpr int STAGE = B * NZ * 8;            // one component of a tile
constexpr int LDP = L + L / 16;              // line pitch: one skew slot per 16 values
constexpr int KP = (L / 2 + 1 + 3) & ~3;     // z pitch of the z-fastest kernel octant
constexpr int NTW = 15 + 16 * 15 + 256 * 3;  // twiddles of radices 16, 16, 4
constexpr int TMEM_COLUMNS = 256;            // 4 warps a lane quarter x 2 slots of 32 columns
constexpr int IN0 = 0, OUT0 = 2 * STAGE, LINES = 4 * STAGE;
constexpr int GBUF = LINES + B * LDP * 8;
constexpr int TWO = GBUF + B * KP * 4;
constexpr int BARS = (TWO + NTW * 8 + 15) & ~15;
constexpr int BYTES = BARS + 32 * 8 + 16 + 1024;  // + alignment slack
static_assert(BYTES <= 232448, "fits one SM");
}  // namespace z2

struct Zq2Maps {
    CUtensorMap in[3];
    CUtensorMap out[3];
};

__device__ __forceinline__ int sk16(int n) { return n + (n >> 4); }

__device__ __forceinline__ void col_sync(int b) { asm volatile("bar.sync %0, 64;" ::"r"(1 + b) : "memory"); }

// Column-uniform success: the two warps of a column share named barriers, so
// they go on only if every thread of the column's waits succeeded (a
// 64-thread barrier with an AND vote; the warp is reconverged first).
__device__ __forceinline__ bool col_ok(int b, bool v)
{
    uint32_t r;
    __syncwarp();
    asm volatile(
        "{\n\t.reg .pred pi, po;\n\tsetp.ne.u32 pi, %1, 0;\n\t"
        "bar.red.and.pred po, %2, 64, pi;\n\tselp.u32 %0, 1, 0, po;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + b)
        : "memory");
    return r != 0;
}

// 16 values <-> 32 columns of the thread's TMEM row.
__device__ __forceinline__ void stash16(uint32_t taddr, const float2 (&v)[16])
{
#pragma unroll
    for (int ch = 0; ch < 2; ++ch) {
        uint32_t w[16];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            w[2 * e] = __float_as_uint(v[ch * 8 + e].x);
            w[2 * e + 1] = __float_as_uint(v[ch * 8 + e].y);
        }
        tmem::st16(taddr + 16 * ch, w);
    }
}

__device__ __forceinline__ void unstash16(uint32_t taddr, float2 (&v)[16])
{
    uint32_t w[2][16];
    tmem::ld16(taddr, w[0]);
    tmem::ld16(taddr + 16, w[1]);
    tmem::wait_ld16x2(w[0], w[1]);
#pragma unroll
    for (int i = 0; i < 16; ++i)
        v[i] = make_float2(__uint_as_float(w[i / 8][2 * (i % 8)]), __uint_as_float(w[i / 8][2 * (i % 8) + 1]));
}

// Value i = 4 u + r of the stage-2 layout sits at kz = 256 r + t + 64 u.
__device__ __forceinline__ int kz_of(int t, int i) { return 256 * (i & 3) + t + 64 * (i >> 2); }

// Stages 1 and 2 of the forward transform of the column whose stage-0
// outputs are in the line: v[4 u + r] at kz = 256 r + t + 64 u.
__device__ __forceinline__ void forward_rest(float2 *line, const float2 *tw, int t, int b, float2 (&v)[16])
{
    float2 x[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) x[r] = line[sk16(t + 64 * r)];
    {
        const float2 *w = tw + 15 + (t & 15) * 15;
#pragma unroll
        for (int r = 1; r < 16; ++r) x[r] = cmul(x[r], w[r - 1]);
    }
    dft16<false>(x);
    col_sync(b);
    {
        const int o = (t >> 4) * 256 + (t & 15);
#pragma unroll
        for (int r = 0; r < 16; ++r) line[sk16(o + 16 * r)] = x[r];
    }
    col_sync(b);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int bf = t + 64 * u;
        float2 *q = &v[4 * u];
#pragma unroll
        for (int r = 0; r < 4; ++r) q[r] = line[sk16(bf + 256 * r)];
        const float2 *w = tw + 255 + bf * 3;
#pragma unroll
        for (int r = 1; r < 4; ++r) q[r] = cmul(q[r], w[r - 1]);
        dft4<false>(q[0], q[1], q[2], q[3]);
    }
}

// Inverse (adjoint) transform of v[4 u + r] (kz = 256 r + t + 64 u) to the
// column's rows z = t + 64 r, r < 8, in y[r].
__device__ __forceinline__ void inverse(float2 (&v)[16], float2 *line, const float2 *tw, int t, int b, float2 (&y)[8])
{
    col_sync(b);  // the previous transform's reads of the line are done
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int bf = t + 64 * u;
        float2 *q = &v[4 * u];
        dft4<true>(q[0], q[1], q[2], q[3]);
        const float2 *w = tw + 255 + bf * 3;
#pragma unroll
        for (int r = 1; r < 4; ++r) q[r] = cmulc(q[r], w[r - 1]);
#pragma unroll
        for (int r = 0; r < 4; ++r) line[sk16(bf + 256 * r)] = q[r];
    }
    col_sync(b);
    float2 x[16];
    {
        const int o = (t >> 4) * 256 + (t & 15);
#pragma unroll
        for (int r = 0; r < 16; ++r) x[r] = line[sk16(o + 16 * r)];
    }
    dft16<true>(x);
    {
        const float2 *w = tw + 15 + (t & 15) * 15;
#pragma unroll
        for (int r = 1; r < 16; ++r) x[r] = cmulc(x[r], w[r - 1]);
    }
    col_sync(b);
#pragma unroll
    for (int r = 0; r < 16; ++r) line[sk16(t + 64 * r)] = x[r];
    col_sync(b);
#pragma unroll
    for (int r = 0; r < 16; ++r) x[r] = line[sk16(16 * t + r)];
    dft16<true>(x);
#pragma unroll
    for (int r = 0; r < 8; ++r) y[r] = x[r];
}

template <int OP>
__global__ void __launch_bounds__(z2::NT, 1)
    k_zq2(const ZArgs a, const __grid_constant__ Zq2Maps maps, const int nxt, const int ntiles, int *status)
{
    using namespace z2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const uint32_t sb = smem_u32(base);
    float2 *TW = reinterpret_cast<float2 *>(base + TWO);
    const uint32_t full0 = sb + BARS, empty0 = full0 + 16, ofull0 = full0 + 32, oempty0 = full0 + 48;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(base + BARS + 8 * 24);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int b = tid / TPL, t = tid % TPL;  // column of the CTA, thread of the column
    // the column's kernel-value barrier (one a column, 8 in all)
    const uint32_t gbar = full0 + 64 + 8 * b;
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, NT);
            mbar_init(ofull0 + 8 * s, NT);
            mbar_init(oempty0 + 8 * s, 1);
        }
        for (int c = 0; c < B; ++c) mbar_init(full0 + 64 + 8 * c, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem::alloc(tslot, TMEM_COLUMNS);
        tmem::relinquish();
    }
    load_twiddles<float2, NTW>(TW, a.plan.table);
    tmem::fence_before_sync();
    __syncthreads();
    tmem::fence_after_sync();
    // lanes of this warp's quarter; warps w, w + 4, w + 8, w + 12 share them
    // and take 64 columns each (two component slots of 32)
    const uint32_t tbase = *tslot + tmem::lane_base(warp) + (uint32_t)((warp >> 2) * 64);

    float2 *line = reinterpret_cast<float2 *>(base + LINES) + b * LDP;
    const int nin = a.nin;
    const int nloc = (int)blockIdx.x < ntiles ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    const int nq = nloc * nin;

    int issued = 0;
    auto issue = [&](int q) -> bool {
        const int s = q & 1;
        if (q >= 2 && !mbar_wait(empty0 + 8 * s, ((q >> 1) - 1) & 1)) return false;
        const int j = (int)blockIdx.x + (q / nin) * (int)gridDim.x, c = q % nin;
        const int ky = a.ky0 + j / nxt, x0 = (j % nxt) * B;
        mbar_arrive_expect_tx(full0 + 8 * s, STAGE);
        for (int bz = 0; bz < 2; ++bz)
            tma_load_3d(sb + IN0 + s * STAGE + bz * 256 * 64, &maps.in[c], 2 * x0, ky, bz * 256, full0 + 8 * s);
        issued = q + 1;
        return true;
    };
    if (tid == 0)
        for (int q = 0; q < 2 && q < nq; ++q) issue(q);

    // thread 0 of the column: copy its kernel column for local tile i
    const float *gsm = reinterpret_cast<const float *>(base + GBUF) + b * KP;
    const bool gissuer = t == 0;
    int g_issued = 0, g_waited = 0;
    auto issue_g = [&](int i) {
        const int j = (int)blockIdx.x + i * (int)gridDim.x;
        const int ky = a.ky0 + j / nxt, x0 = (j % nxt) * B;
        const int oyr = imin(ky, a.Py - ky), kx = x0 + b;
        const bool on = kx < a.Mx;
        mbar_arrive_expect_tx(gbar, on ? KP * 4 : 0);
        if (on) bulk_load(sb + GBUF + b * KP * 4, a.kern_zf + ((long long)oyr * a.Mx + kx) * KP, KP * 4, gbar);
        g_issued = i + 1;
    };
    if (gissuer && nloc > 0) issue_g(0);

    bool ok = true;
    int qo = 0, consumed = 0;
    for (int i = 0; i < nloc && ok; ++i) {
        const int j = (int)blockIdx.x + i * (int)gridDim.x;
        const int ky = a.ky0 + j / nxt, x0 = (j % nxt) * B;
        const int kx = x0 + b;
        const bool active = kx < a.Mx;
        float2 cur[16];

        // forward transforms; components 0 .. nin-2 parked in TMEM
        for (int c = 0; c < nin; ++c) {
            const int q = i * nin + c, s = q & 1;
            ok = col_ok(b, ok && mbar_wait(full0 + 8 * s, (q >> 1) & 1));
            if (!ok) break;
            if (tid == 0) consumed = q + 1;
            const unsigned char *stg = base + IN0 + s * STAGE;
            float2 x[16];
#pragma unroll
            for (int r = 0; r < 8; ++r) x[r] = *reinterpret_cast<const float2 *>(stg + swizzle64(t + 64 * r, b));
            mbar_arrive(empty0 + 8 * s);
            if (tid == 0 && q + 2 < nq) ok = issue(q + 2);
            ok = col_ok(b, ok);
            if (!ok) break;
            dft16_half<false>(x);  // stage 0
            col_sync(b);           // the previous transform's reads of the line are done
#pragma unroll
            for (int r = 0; r < 16; ++r) line[sk16(16 * t + r)] = x[r];
            col_sync(b);
            forward_rest(line, TW, t, b, cur);
            if (c + 1 < nin) stash16(tbase + 32 * c, cur);
        }
        if (!ok) break;
        if (nin > 1) tmem::wait_st();

        ok = col_ok(b, mbar_wait(gbar, i & 1));
        if (!ok) break;
        if (gissuer) g_waited = i + 1;

        // spectral operation on the 16 values of every component: the last
        // component in cur, the others in the TMEM slots, eight at a time
        {
            const float kyv = wavenumber<float>(ky, a.Py, (float)a.kyc, true);
            const float kxv = wavenumber<float>(kx, a.Px, (float)a.kxc, true);
            const float kzc = (float)a.kzc;
#pragma unroll
            for (int ch = 0; ch < 2; ++ch) {
                uint32_t w0[16] = {}, w1[16] = {};
                if (nin > 1) tmem::ld16(tbase + 16 * ch, w0);
                if (nin > 2) tmem::ld16(tbase + 32 + 16 * ch, w1);
                if (nin > 1) tmem::wait_ld16x2(w0, w1);
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int k = 8 * ch + e;
                    const int kz = kz_of(t, k);
                    const float gi = active ? gsm[imin(kz, L - kz)] : 0.f;
                    const float kzv = wavenumber<float>(kz, L, kzc, true);
                    const float2 ic = cur[k];
                    const float2 i0 = make_float2(__uint_as_float(w0[2 * e]), __uint_as_float(w0[2 * e + 1]));
                    const float2 i1 = make_float2(__uint_as_float(w1[2 * e]), __uint_as_float(w1[2 * e + 1]));
                    float2 o0 = make_float2(0.f, 0.f), o1 = o0, o2;
                    if constexpr (OP == OP_NONE) {
                        o0 = cscale(i0, gi);
                        o1 = cscale(i1, gi);
                        o2 = cscale(ic, gi);
                    } else if constexpr (OP == OP_GRAD) {
                        // nin = 1: every output from the one input; nin = 3: output d from input d
                        const float2 a0 = a.nin > 1 ? i0 : ic, a1 = a.nin > 1 ? i1 : ic;
                        const float gx = gi * kxv, gy = gi * kyv, gz = gi * kzv;
                        o0 = make_float2(-gx * a0.y, gx * a0.x);
                        o1 = make_float2(-gy * a1.y, gy * a1.x);
                        o2 = make_float2(-gz * ic.y, gz * ic.x);
                    } else if constexpr (OP == OP_DIV) {
                        const float2 d = make_float2(kxv * i0.x + kyv * i1.x + kzv * ic.x, kxv * i0.y + kyv * i1.y + kzv * ic.y);
                        o2 = make_float2(-gi * d.y, gi * d.x);
                    } else {  // OP_CURL
                        const float2 c0 = make_float2(kyv * ic.x - kzv * i1.x, kyv * ic.y - kzv * i1.y);
                        const float2 c1 = make_float2(kzv * i0.x - kxv * ic.x, kzv * i0.y - kxv * ic.y);
                        const float2 c2 = make_float2(kxv * i1.x - kyv * i0.x, kxv * i1.y - kyv * i0.y);
                        o0 = make_float2(-gi * c0.y, gi * c0.x);
                        o1 = make_float2(-gi * c1.y, gi * c1.x);
                        o2 = make_float2(-gi * c2.y, gi * c2.x);
                    }
                    w0[2 * e] = __float_as_uint(o0.x);
                    w0[2 * e + 1] = __float_as_uint(o0.y);
                    w1[2 * e] = __float_as_uint(o1.x);
                    w1[2 * e + 1] = __float_as_uint(o1.y);
                    cur[k] = o2;
                }
                if (a.nout > 1) tmem::st16(tbase + 16 * ch, w0);
                if (a.nout > 2) tmem::st16(tbase + 32 + 16 * ch, w1);
            }
            if (a.nout > 1) tmem::wait_st();
        }
        col_sync(b);  // both warps of the column have read its kernel values
        if (gissuer && i + 1 < nloc) issue_g(i + 1);

        // inverse transforms: output nout-1 from cur, then nout-2 .. 0 from TMEM
        for (int oc = a.nout - 1; oc >= 0; --oc) {
            if (!a.out[oc]) continue;  // uniform over the CTA
            if (oc < a.nout - 1) unstash16(tbase + 32 * oc, cur);
            float2 y[8];
            inverse(cur, line, TW, t, b, y);

            const int so = qo & 1;
            if (qo >= 2) ok = col_ok(b, mbar_wait(oempty0 + 8 * so, ((qo >> 1) - 1) & 1));
            if (!ok) break;
            unsigned char *ostg = base + OUT0 + so * STAGE;
#pragma unroll
            for (int r = 0; r < 8; ++r) *reinterpret_cast<float2 *>(ostg + swizzle64(t + 64 * r, b)) = y[r];
            fence_proxy_async_smem();
            mbar_arrive(ofull0 + 8 * so);
            if (tid == 0) {
                ok = mbar_wait(ofull0 + 8 * so, (qo >> 1) & 1);
                if (ok) {
                    for (int bz = 0; bz < 2; ++bz)
                        tma_store_3d(&maps.out[oc], 2 * x0, ky, bz * 256, sb + OUT0 + so * STAGE + bz * 256 * 64);
                    bulk_commit();
                    bulk_wait_read<1>();  // the previous box has been read: release it
                    if (qo >= 1) mbar_arrive(oempty0 + 8 * ((qo - 1) & 1));
                }
            }
            ok = col_ok(b, ok);
            if (!ok) break;
            ++qo;
        }
    }

    if (!ok && lane == 0) atomicOr(status, 1);
    if (tid == 0) {
        for (int q = consumed; q < issued; ++q) mbar_wait(full0 + 8 * (q & 1), (q >> 1) & 1);
        bulk_wait_all();
    }
    if (gissuer && g_waited < g_issued) mbar_wait(gbar, (g_issued - 1) & 1);
    tmem::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tmem::fence_after_sync();
        tmem::dealloc(*tslot, TMEM_COLUMNS);
    }
}

template <int OP> cudaError_t launch_zq2_op(const ZArgs &a, int ny, int *status, cudaStream_t st)
{
    using namespace z2;
    if (!a.kern_zf || a.kzp != KP || (reinterpret_cast<uintptr_t>(a.kern_zf) & 15) || a.plan.ntw != NTW)
        return cudaErrorInvalidValue;
    Zq2Maps maps;
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
    const int grid = ntiles < tma::sm_count() ? ntiles : tma::sm_count();
    cudaError_t e = cudaFuncSetAttribute(k_zq2<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, BYTES);
    if (e != cudaSuccess) return e;
    k_zq2<OP><<<grid, NT, BYTES, st>>>(a, maps, nxt, ntiles, status);
    return cudaGetLastError();
}

}  // namespace

bool zq2_supported(int prec, int L, int op, int nin, int nout, int n_in, int n_out)
{
    return prec == PREC_FP32 && L == z2::L && n_in == z2::NZ && n_out == z2::NZ &&
           (op == OP_NONE || op == OP_GRAD || op == OP_DIV || op == OP_CURL) && nin >= 1 && nin <= 3 && nout >= 1 &&
           nout <= 3 && tma::encode_fn() != nullptr;
}

size_t smem_zq2() { return z2::BYTES; }

cudaError_t launch_zq2(const ZArgs &a, int ny, int *status, cudaStream_t st)
{
    if (!status || a.B != ZQ2_LINES || !zq2_supported(PREC_FP32, a.L, a.op, a.nin, a.nout, a.n_in, a.n_out))
        return cudaErrorInvalidConfiguration;
    switch (a.op) {
    case OP_NONE: return launch_zq2_op<OP_NONE>(a, ny, status, st);
    case OP_GRAD: return launch_zq2_op<OP_GRAD>(a, ny, status, st);
    case OP_DIV: return launch_zq2_op<OP_DIV>(a, ny, status, st);
    case OP_CURL: return launch_zq2_op<OP_CURL>(a, ny, status, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace wide
}  // namespace ps
