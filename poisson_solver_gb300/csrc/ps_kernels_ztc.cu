// Fused z pass with the DFT stages on the tensor cores (FP32 spectra in and
// out; L = 1024 along an unbounded z axis: n_in = n_out = 512).
//
// A length-1024 transform is two radix-32 stages, z = 32 n1 + n2,
// kz = k1 + 32 k2:
//   X[k1 + 32 k2] = sum_n2 W32^(n2 k2) W1024^(n2 k1) sum_n1 W32^(n1 k1) x[32 n1 + n2]
// Each stage is a product with the 32-point DFT matrix, taken as a real
// 64 x 64 matrix on interleaved (re, im) pairs. Per tile of 8 z-columns and
// per component, the rows of a stage's operand A are (column, the index kept)
// and its K index is the one summed, so one stage of 4 columns is
//     D[128 x 64] = A[128 x 64] B^T,  B = the DFT matrix
// issued as tcgen05.mma (kind::f16, M = 128, K = 16 a step, FP32
// accumulators in tensor memory) by one thread of the 4 warps that own the
// 4 columns. The inverse is the forward transform of the conjugate.
//
// Precision: every operand is split into FP16 hi + lo parts (x = hi + lo to
// about 2^-22 relative) and a stage accumulates hi*lo + lo*hi + hi*hi in
// FP32. Before each split the column is scaled by a power of two so that its
// largest part sits in [2^13, 2^14): the FP16 range holds it, and parts too
// small for normal FP16 numbers lie below 2^-27 of the column's largest. The
// DFT matrix is stored scaled by 2^14 for the same reason. The first stage of
// each transform takes the scale from the column's largest value; the
// second uses a fixed one, since a 32-point DFT of a column (with twiddles
// of modulus 1) keeps its largest value within a factor of 32 above and
// sqrt(32) below (Parseval), which the FP16 range covers. The scales are exact
// and undone in FP32 (the spectra for the spectral operation, the output when
// it is stored).
//
// Data flow per column (thread = TMEM lane = one row of the MMA):
//   forward  stage A: row (column, n2), K = n1 < 16 (the zero-padded half of
//            z is never staged): A from the input staging -> D in TMEM;
//            twiddle W1024^(n2 k1); transpose through shared memory;
//            stage B: row (column, k1), K = n2 -> spectrum in TMEM;
//   spectral operation on the spectra of all components (rows (column, k1),
//            kz = k1 + 32 k2), written back in place;
//   inverse  of the conjugate: stage 1 row (column, k1), K = k2; twiddle,
//            transpose; stage 2 row (column, n2), K = k1, only n1 < 16 (the
//            crop) -> the output staging.
// Operand A of every stage is written to tensor memory by the thread that
// owns its row (tcgen05.st); operand B (the DFT matrix) sits in shared
// memory, K-major without swizzle.
//
// Threads: warps 0-15 compute. Warps 8h .. 8h+7 are half h (columns 4h ..
// 4h+3, TMEM columns 256h .. 256h+255); warp w serves column 4h + (w & 3)
// (TMEM lanes 32 (w & 3) ..) and part (w >> 2) & 1 of each row: half of the
// row's values, so two warps share a row and a column's transposes (a
// 64-thread barrier a column). Warp 16 issues the loads (input components by
// tiled bulk copy, double-buffered; the tile's kernel columns by bulk copy),
// warp 17 the output stores. One persistent CTA per SM.
//
// Failure handling: every mbarrier wait is bounded; a half decides together
// (bar.red.and over its 256 threads) whether to go on, so no named barrier
// is left waiting; on a failure the CTA drains its copies and MMAs, frees its
// tensor memory and sets bit 0 of *status.
#include <cuda_fp16.h>

#include <cstdlib>
#include <cstring>

#include "ps_async.cuh"
#include "ps_tma_host.hpp"
#include "ps_tmem.cuh"
#include "ps_types.hpp"
#include "ps_wide.cuh"

namespace ps {
namespace tc {

namespace {

using namespace async;

constexpr int LZ = 1024;        // transform length
constexpr int NZ = 512;         // stored z rows (the other half is padding)
constexpr int COLS = 8;         // z-columns a tile: one 64-byte box column group
constexpr int NCOMPUTE = 512;   // two halves of eight warps
constexpr int NTHREADS = NCOMPUTE + 64;
constexpr int W_LOAD = NCOMPUTE / 32, W_STORE = W_LOAD + 1;
constexpr int TMEM_COLS = 512;  // per half: 3 spectra x 64 + operand A (hi 32 + lo 32)
constexpr int HALF_TCOLS = 256;
constexpr int SPEC = 64;        // TMEM columns of one component's spectrum row
constexpr int A_HI = 192, A_LO = 224;
constexpr int KP = 516;         // z pitch of the z-fastest kernel octant: 513 rounded up to 4
constexpr float BSCALE = 16384.f;  // the DFT matrix is stored times 2^14
// fixed scales of the second stage's input: the first stage's output is at
// most 16 (forward, 16 nonzero inputs) or 32 (inverse) times 2^14 x 2^14,
// and its column's largest value at least 1/sqrt(32) of that of its input
constexpr float S_MID_FWD = 1.f / 262144.f;  // 2^-18
constexpr float S_MID_INV = 1.f / 524288.f;  // 2^-19

// shared memory (byte offsets from a 1024-aligned base)
constexpr int STAGE = COLS * NZ * 8;  // one component of a tile: 8 columns x 512 rows of complex floats
constexpr int IN0 = 0;                // two input stages
constexpr int OUT0 = IN0 + 2 * STAGE;
constexpr int XP_PITCH = 32 * 8 + 16;  // transpose rows: 32 complex values + 16 bytes of skew
constexpr int XP_BYTES = 32 * XP_PITCH;
constexpr int XP0 = OUT0 + STAGE;      // one 32 x 32 transpose buffer a warp
constexpr int BM_BYTES = 4 * 64 * 16 * 2;  // DFT matrix [4 K-chunks][64 rows][16 K] of FP16
constexpr int BM0 = XP0 + COLS * XP_BYTES;  // hi, then lo
constexpr int TW0 = BM0 + 2 * BM_BYTES;     // W1024^(j k) S_MID_FWD, then W1024^(j k) S_MID_INV: [2][32][32] complex floats
constexpr int G0 = TW0 + 2 * 32 * 32 * 8;   // the tile's kernel columns, [8][KP] floats
constexpr int MX0 = G0 + COLS * KP * 4;     // column maxima of the two parts, [8][2][4] floats
constexpr int BAR0 = MX0 + COLS * 2 * 4 * 4;
constexpr int SMEM_BYTES = BAR0 + 16 * 8 + 16 + 1024;  // + alignment slack
static_assert(BM0 % 1024 == 0 || BM0 % 16 == 0, "matrix descriptors need 16-byte alignment");
static_assert(BAR0 % 8 == 0, "mbarriers are 8-byte aligned");
static_assert(SMEM_BYTES <= 232448, "fits one SM");

// barrier slots (8 bytes each from BAR0)
enum { B_FULL = 0, B_EMPTY = 2, B_OFULL = 4, B_OEMPTY = 5, B_GFULL = 6, B_GEMPTY = 7, B_MMA = 8, B_SLOT = 16 };

// ---------------------------------------------------------------------------
// tensor-core pieces

// Shared-memory matrix descriptor: K-major, no swizzle; lbo = byte stride
// between core matrices along K, sbo = between 8-row groups.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16: FP16 A and B (both K-major), FP32 D, M = 128, N.
__host__ __device__ constexpr uint32_t idesc_f16(int n) { return (1u << 4) | ((uint32_t)(n >> 3) << 17) | (8u << 24); }

// D (tmem) (+)= A (tmem) x B (smem)^T, one K-step of 16.
__device__ __forceinline__ void mma_ts(uint32_t d, uint32_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
        "r"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

// Arrive on an mbarrier once every MMA this thread issued has completed.
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// One stage: hi*lo + lo*hi + hi*hi over nk K-steps into D (tmem address d).
// The small cross terms go first: each MMA rounds its sum into the FP32
// accumulator, and rounding steps taken while the accumulator holds only the
// small terms cost nothing at the scale of the result, so the result sees
// nk roundings instead of 3 nk.
__device__ __forceinline__ void mma_stage(uint32_t d, uint32_t a_hi, uint32_t a_lo, uint32_t bm, int nk, int n)
{
    const uint32_t id = idesc_f16(n);
#pragma unroll 1
    for (int p = 0; p < 3; ++p) {
        const uint32_t a = p == 1 ? a_lo : a_hi;
        const uint32_t bsm = p == 0 ? bm + BM_BYTES : bm;
#pragma unroll 1
        for (int j = 0; j < nk; ++j) mma_ts(d, a + 8 * j, sdesc(bsm + j * 2048, 128, 256), id, (p | j) != 0);
    }
}

// Named barrier over one half's 256 threads with an AND vote (the warp is
// reconverged first: bounded waits can leave its lanes apart).
__device__ __forceinline__ bool half_and(int h, bool v)
{
    uint32_t r;
    __syncwarp();
    asm volatile(
        "{\n\t.reg .pred pi, po;\n\tsetp.ne.u32 pi, %1, 0;\n\t"
        "bar.red.and.pred po, %2, 256, pi;\n\tselp.u32 %0, 1, 0, po;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + h)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ uint32_t h2u(__half2 h) { return *reinterpret_cast<uint32_t *>(&h); }

// (a.x b.x, a.y b.y) as one packed instruction (mul.rn.f32x2)
__device__ __forceinline__ float2 cmul2(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mul.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

// 2^e with max * 2^e in [2^13, 2^14) (1 for a zero or subnormal max).
__device__ __forceinline__ float scale_for(float m)
{
    const int eb = (__float_as_int(m) >> 23) & 0xff;
    if (eb == 0) return 1.f;
    int e = 267 - eb;
    e = e < 1 ? 1 : e > 254 ? 254 : e;
    return __int_as_float(e << 23);
}

__device__ __forceinline__ float warp_max(float m)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

template <int NV> __device__ __forceinline__ float abs_max(const float2 (&v)[NV])
{
    float m = 0.f;
#pragma unroll
    for (int i = 0; i < NV; ++i) m = fmaxf(m, fmaxf(fabsf(v[i].x), fabsf(v[i].y)));
    return m;
}

// The two warps of a column (64 threads).
__device__ __forceinline__ void column_sync(int b)
{
    asm volatile("bar.sync %0, 64;" ::"r"(3 + b) : "memory");
}

__device__ __forceinline__ void st8(uint32_t taddr, const uint32_t (&v)[8])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}

// Operand A of this thread's part of its row: NV complex values (K = 2 n +
// (0 re, 1 im) for n = k0 .. k0 + NV - 1) times (sr, si) (si = -sr
// conjugates), split into FP16 hi and lo, packed two to a column.
template <int NV, bool SCALE = true>
__device__ __forceinline__ void put_a(uint32_t trow, int k0, const float2 (&v)[NV], float sr = 1.f, float si = 1.f)
{
    static_assert(NV == 8 || NV == 16, "8 or 16 values");
    uint32_t hi[NV], lo[NV];
#pragma unroll
    for (int e = 0; e < NV; ++e) {
        const float2 x = SCALE ? cmul2(v[e], make_float2(sr, si)) : v[e];
        const __half2 hh = __floats2half2_rn(x.x, x.y);
        const float2 r = csub(x, __half22float2(hh));
        hi[e] = h2u(hh);
        lo[e] = h2u(__floats2half2_rn(r.x, r.y));
    }
    if constexpr (NV == 16) {
        tmem::st16(trow + A_HI + k0, hi);
        tmem::st16(trow + A_LO + k0, lo);
    } else {
        st8(trow + A_HI + k0, hi);
        st8(trow + A_LO + k0, lo);
    }
}

// NV complex values (2 NV columns) of this thread's TMEM row from taddr.
template <int NV> __device__ __forceinline__ void get_d(uint32_t taddr, float2 (&v)[NV])
{
    static_assert(NV == 8 || NV == 16, "8 or 16 values");
    uint32_t w[2][16];
    tmem::ld16(taddr, w[0]);
    if constexpr (NV == 16) tmem::ld16(taddr + 16, w[1]);
    tmem::wait_ld16x2(w[0], w[1]);
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = make_float2(__uint_as_float(w[i / 8][2 * (i % 8)]), __uint_as_float(w[i / 8][2 * (i % 8) + 1]));
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// v[j] *= TW[r0 + j][lane] = W1024^((r0 + j) lane)
__device__ __forceinline__ void twiddle(float2 (&v)[16], const float2 *tw, int r0, int lane)
{
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = cmul(v[j], tw[(r0 + j) * 32 + lane]);
}

// 32 x 32 transpose over the two warps of a column: the value v[j] of row
// r0 + j in lane l becomes value j of row l in the part starting at r0 of
// the reading warp (both warps of the column take part).
__device__ __forceinline__ void transpose(float2 (&v)[16], unsigned char *xp, int r0, int lane, int b)
{
#pragma unroll
    for (int j = 0; j < 16; ++j) *reinterpret_cast<float2 *>(xp + (r0 + j) * XP_PITCH + lane * 8) = v[j];
    column_sync(b);
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
        const float4 q = *reinterpret_cast<const float4 *>(xp + lane * XP_PITCH + (r0 + j) * 8);
        v[j] = make_float2(q.x, q.y);
        v[j + 1] = make_float2(q.z, q.w);
    }
}

// The 32-point DFT matrix as the real 64 x 64 operand B (row N = 2 k + t, K =
// 2 n + s; W = e^{-2 pi i n k / 32}), times 2^14, split into FP16 hi and lo,
// and the twiddles W1024^(j k) with the fixed scale of the second stage's
// input folded in: computed in FP64 from exact fractions.
__device__ void build_tables(unsigned char *base, int tid)
{
    __half *bh = reinterpret_cast<__half *>(base + BM0), *bl = reinterpret_cast<__half *>(base + BM0 + BM_BYTES);
    for (int i = tid; i < 64 * 64; i += NTHREADS) {
        const int N = i >> 6, K = i & 63, k = N >> 1, t = N & 1, n = K >> 1, s = K & 1;
        double sn, cs;
        sincospi((double)((n * k) & 31) / 16.0, &sn, &cs);
        // re out: re in cos + im in sin; im out: -re in sin + im in cos
        const double v = (t == 0 ? (s == 0 ? cs : sn) : (s == 0 ? -sn : cs)) * (double)BSCALE;
        const __half hi = __double2half(v);
        const __half lo = __double2half(v - (double)__half2float(hi));
        const int off = (K >> 4) * 1024 + (N >> 3) * 128 + ((K & 15) >> 3) * 64 + (N & 7) * 8 + (K & 7);  // in halves
        bh[off] = hi;
        bl[off] = lo;
    }
    float2 *tw = reinterpret_cast<float2 *>(base + TW0);
    for (int i = tid; i < 32 * 32; i += NTHREADS) {
        const int j = i >> 5, k = i & 31;
        double sn, cs;
        sincospi(-(double)((j * k) & 1023) / 512.0, &sn, &cs);
        tw[i] = make_float2((float)cs * S_MID_FWD, (float)sn * S_MID_FWD);  // exact: powers of two
        tw[1024 + i] = make_float2((float)cs * S_MID_INV, (float)sn * S_MID_INV);
    }
}

struct TcMaps {
    CUtensorMap in[3];
    CUtensorMap out[3];
};

template <int OP>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_ztc(const ZArgs a, const __grid_constant__ TcMaps maps, const int nxt, const int ntiles, int *status)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const uint32_t sb = smem_u32(base);
    const uint32_t bar = sb + BAR0;
    auto B = [&](int slot) { return bar + 8 * slot; };
    uint32_t *tslot = reinterpret_cast<uint32_t *>(base + BAR0 + 8 * B_SLOT);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nin = a.nin, nout = a.nout;
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(B(B_FULL + s), 1);
            mbar_init(B(B_EMPTY + s), NCOMPUTE);
            mbar_init(B(B_MMA + s), 1);
        }
        mbar_init(B(B_OFULL), NCOMPUTE);
        mbar_init(B(B_OEMPTY), 1);
        mbar_init(B(B_GFULL), 1);
        mbar_init(B(B_GEMPTY), NCOMPUTE);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem::alloc(tslot, TMEM_COLS);
        tmem::relinquish();
    }
    build_tables(base, tid);
    fence_proxy_async_smem();  // the DFT matrix is read by the tensor cores
    tmem::fence_before_sync();
    __syncthreads();
    tmem::fence_after_sync();
    const uint32_t tbase = *tslot;

    const int nloc = (int)blockIdx.x < ntiles ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    auto tile = [&](int i, int &ky, int &x0) {
        const int j = (int)blockIdx.x + i * (int)gridDim.x;
        ky = a.ky0 + j / nxt;
        x0 = (j % nxt) * COLS;
    };
    bool ok = true;

    if (warp == W_LOAD) {
        // ---- loads: the tile's kernel columns, then its input components
        int issued = 0;
        if (lane == 0) {
            for (int i = 0; i < nloc && ok; ++i) {
                int ky, x0;
                tile(i, ky, x0);
                if (i >= 1) ok = mbar_wait(B(B_GEMPTY), (i - 1) & 1);
                if (!ok) break;
                const int oyr = ky < a.Py - ky ? ky : a.Py - ky;
                const int ncol = a.Mx - x0 < COLS ? a.Mx - x0 : COLS;
                mbar_arrive_expect_tx(B(B_GFULL), (uint32_t)(ncol * KP * 4));
                bulk_load(sb + G0, a.kern_zf + ((long long)oyr * a.Mx + x0) * KP, (uint32_t)(ncol * KP * 4), B(B_GFULL));
                for (int c = 0; c < nin; ++c) {
                    const int q = i * nin + c, s = q & 1;
                    if (q >= 2) ok = mbar_wait(B(B_EMPTY + s), ((q >> 1) - 1) & 1);
                    if (!ok) break;
                    mbar_arrive_expect_tx(B(B_FULL + s), STAGE);
                    for (int bz = 0; bz < 2; ++bz)
                        tma_load_3d(sb + IN0 + s * STAGE + bz * 256 * 64, &maps.in[c], 2 * x0, ky, bz * 256, B(B_FULL + s));
                    issued = q + 1;
                }
            }
            // after a failure: let the copies already started land before the CTA exits
            if (!ok)
                for (int q = issued - 2 > 0 ? issued - 2 : 0; q < issued; ++q) mbar_wait(B(B_FULL + (q & 1)), (q >> 1) & 1);
        }
    } else if (warp == W_STORE) {
        // ---- stores: one box a finished output component
        if (lane == 0) {
            int qo = 0;
            for (int i = 0; i < nloc && ok; ++i) {
                int ky, x0;
                tile(i, ky, x0);
                for (int oc = 0; oc < nout && ok; ++oc) {
                    if (!a.out[oc]) continue;
                    ok = mbar_wait(B(B_OFULL), qo & 1);
                    if (!ok) break;
                    for (int bz = 0; bz < 2; ++bz)
                        tma_store_3d(&maps.out[oc], 2 * x0, ky, bz * 256, sb + OUT0 + bz * 256 * 64);
                    bulk_commit();
                    bulk_wait_read<0>();
                    mbar_arrive(B(B_OEMPTY));
                    ++qo;
                }
            }
            bulk_wait_all();
        }
    } else {
        // ---- compute: half h, column b, part p (values 16 p .. 16 p + 15 of a row)
        const int h = warp >> 3, b = 4 * h + (warp & 3), p = (warp >> 2) & 1;
        const uint32_t td = tbase + (uint32_t)(HALF_TCOLS * h);  // MMA addresses (lane 0)
        const uint32_t trow = td + tmem::lane_base(warp);         // this thread's row
        const bool issuer = (warp & 7) == 0 && lane == 0;
        const uint32_t mbar = B(B_MMA + h);
        int mma_n = 0;  // commits of this half so far
        unsigned char *xp = base + XP0 + b * XP_BYTES;
        const float2 *tw = reinterpret_cast<const float2 *>(base + TW0);
        const float *gcol = reinterpret_cast<const float *>(base + G0) + b * KP;
        float *mx = reinterpret_cast<float *>(base + MX0) + b * 8;  // [part][4]
        const int r0 = 16 * p;                                     // this part's first value of a row

        // all 256 threads have written A: one thread issues the stage, all
        // wait. A wait that runs out leaves ok false in that thread only; the
        // code up to the next vote is safe with stale data, and every break
        // follows a vote, so the half leaves its loops together
        auto run = [&](int dcol, int nk, int n) {
            tmem::wait_st();
            tmem::fence_before_sync();
            ok = half_and(h, ok);
            if (!ok) return;
            if (issuer) {
                tmem::fence_after_sync();
                mma_stage(td + dcol, td + A_HI, td + A_LO, sb + BM0, nk, n);
                mma_commit(mbar);
            }
            ok = mbar_wait(mbar, mma_n & 1);
            ++mma_n;
            tmem::fence_after_sync();
        };

        int qo = 0;
        for (int i = 0; i < nloc; ++i) {
            int ky, x0;
            tile(i, ky, x0);
            const int kx = x0 + b;
            const bool active = kx < a.Mx;
            float inv0 = 1.f, inv1 = 1.f, inv2 = 1.f;  // scales of the input spectra

            // forward transforms of the input components
            for (int c = 0; c < nin; ++c) {
                const int q = i * nin + c, s = q & 1;
                ok = half_and(h, ok && mbar_wait(B(B_FULL + s), (q >> 1) & 1));
                if (!ok) break;
                float2 v[16];
                const unsigned char *stg = base + IN0 + s * STAGE;
#pragma unroll
                for (int n1 = 0; n1 < 16; ++n1)
                    v[n1] = *reinterpret_cast<const float2 *>(stg + swizzle64(32 * n1 + lane, b));
                mbar_arrive(B(B_EMPTY + s));
                const float sA = scale_for(warp_max(abs_max(v)));  // both parts see the whole column
                float2 x[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) x[j] = p ? v[8 + j] : v[j];
                put_a<8>(trow, 8 * p, x, sA, sA);
                run(SPEC * c, 2, 64);  // stage A: K = n1 < 16
                get_d<16>(trow + SPEC * c + 2 * r0, v);  // Y[k1], k1 = r0 + j, lane = n2
                twiddle(v, tw, r0, lane);  // and the fixed scale
                transpose(v, xp, r0, lane, b);  // lane = k1, v[j] = value n2 = r0 + j
                put_a<16, false>(trow, r0, v);
                run(SPEC * c, 4, 64);  // stage B -> spectrum
                const float inv = __frcp_rn(sA) * (1.f / (S_MID_FWD * BSCALE * BSCALE));
                inv0 = c == 0 ? inv : inv0;
                inv1 = c == 1 ? inv : inv1;
                inv2 = c == 2 ? inv : inv2;
            }

            // spectral operation, in place on the spectra (row (b, k1): kz = lane + 32 k2)
            ok = half_and(h, ok && mbar_wait(B(B_GFULL), i & 1));
            if (!ok) break;
            float om0 = 0.f, om1 = 0.f, om2 = 0.f;  // largest output parts
            {
                const float kxv = wide::wavenumber<float>(kx, a.Px, (float)a.kxc, true);
                const float kyv = wide::wavenumber<float>(ky, a.Py, (float)a.kyc, true);
                const float kzc = (float)a.kzc;
#pragma unroll 1
                for (int ch = 2 * p; ch < 2 * p + 2; ++ch) {
                    uint32_t s0[16], s1[16] = {}, s2[16] = {};
                    tmem::ld16(trow + 16 * ch, s0);
                    if (nin > 1) tmem::ld16(trow + SPEC + 16 * ch, s1);
                    if (nin > 2) tmem::ld16(trow + 2 * SPEC + 16 * ch, s2);
                    tmem::wait_ld16x2(s0, s1);
                    tmem::wait_ld16(s2);
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int kz = lane + 32 * (8 * ch + e);
                        const float kzv = wide::wavenumber<float>(kz, LZ, kzc, true);
                        const float g = active ? gcol[kz < LZ - kz ? kz : LZ - kz] : 0.f;
                        const float2 i0 = make_float2(__uint_as_float(s0[2 * e]) * inv0, __uint_as_float(s0[2 * e + 1]) * inv0);
                        const float2 i1 = make_float2(__uint_as_float(s1[2 * e]) * inv1, __uint_as_float(s1[2 * e + 1]) * inv1);
                        const float2 i2 = make_float2(__uint_as_float(s2[2 * e]) * inv2, __uint_as_float(s2[2 * e + 1]) * inv2);
                        float2 o0 = make_float2(0.f, 0.f), o1 = o0, o2 = o0;
                        if constexpr (OP == OP_NONE) {
                            o0 = make_float2(g * i0.x, g * i0.y);
                            o1 = make_float2(g * i1.x, g * i1.y);
                            o2 = make_float2(g * i2.x, g * i2.y);
                        } else if constexpr (OP == OP_GRAD) {
                            // nin = 1: every output from the one input; nin = 3: output d from input d
                            const float2 a1 = nin > 1 ? i1 : i0, a2 = nin > 1 ? i2 : i0;
                            const float gx = g * kxv, gy = g * kyv, gz = g * kzv;
                            o0 = make_float2(-gx * i0.y, gx * i0.x);
                            o1 = make_float2(-gy * a1.y, gy * a1.x);
                            o2 = make_float2(-gz * a2.y, gz * a2.x);
                        } else if constexpr (OP == OP_DIV) {
                            const float2 d = make_float2(kxv * i0.x + kyv * i1.x + kzv * i2.x, kxv * i0.y + kyv * i1.y + kzv * i2.y);
                            o0 = make_float2(-g * d.y, g * d.x);
                        } else {  // OP_CURL
                            const float2 c0 = make_float2(kyv * i2.x - kzv * i1.x, kyv * i2.y - kzv * i1.y);
                            const float2 c1 = make_float2(kzv * i0.x - kxv * i2.x, kzv * i0.y - kxv * i2.y);
                            const float2 c2 = make_float2(kxv * i1.x - kyv * i0.x, kxv * i1.y - kyv * i0.y);
                            o0 = make_float2(-g * c0.y, g * c0.x);
                            o1 = make_float2(-g * c1.y, g * c1.x);
                            o2 = make_float2(-g * c2.y, g * c2.x);
                        }
                        s0[2 * e] = __float_as_uint(o0.x);
                        s0[2 * e + 1] = __float_as_uint(o0.y);
                        s1[2 * e] = __float_as_uint(o1.x);
                        s1[2 * e + 1] = __float_as_uint(o1.y);
                        s2[2 * e] = __float_as_uint(o2.x);
                        s2[2 * e + 1] = __float_as_uint(o2.y);
                        om0 = fmaxf(om0, fmaxf(fabsf(o0.x), fabsf(o0.y)));
                        om1 = fmaxf(om1, fmaxf(fabsf(o1.x), fabsf(o1.y)));
                        om2 = fmaxf(om2, fmaxf(fabsf(o2.x), fabsf(o2.y)));
                    }
                    tmem::st16(trow + 16 * ch, s0);
                    if (nout > 1) tmem::st16(trow + SPEC + 16 * ch, s1);
                    if (nout > 2) tmem::st16(trow + 2 * SPEC + 16 * ch, s2);
                }
                tmem::wait_st();
            }
            mbar_arrive(B(B_GEMPTY));
            // the column's largest output values, over both parts
            om0 = warp_max(om0);
            om1 = warp_max(om1);
            om2 = warp_max(om2);
            if (lane == 0) {
                mx[4 * p] = om0;
                mx[4 * p + 1] = om1;
                mx[4 * p + 2] = om2;
            }
            column_sync(b);

            // inverse transforms (of the conjugates) of the written outputs
            for (int oc = 0; oc < nout; ++oc) {
                if (!a.out[oc]) continue;  // uniform over the CTA
                float2 v[16];
                const float s1 = scale_for(fmaxf(mx[oc], mx[4 + oc]));
                get_d<16>(trow + SPEC * oc + 2 * r0, v);  // X'[k1 + 32 k2], k2 = r0 + j, lane = k1
                put_a<16>(trow, r0, v, s1, -s1);
                run(SPEC * oc, 4, 64);  // stage 1: K = k2
                get_d<16>(trow + SPEC * oc + 2 * r0, v);  // V[k1][r], r = r0 + j, lane = k1
                twiddle(v, tw + 1024, r0, lane);  // and the fixed scale
                transpose(v, xp, r0, lane, b);  // lane = r, v[j] = value k1 = r0 + j
                put_a<16, false>(trow, r0, v);
                run(SPEC * oc, 4, 32);  // stage 2: K = k1, N = q < 16 (the crop)
                float2 w[8];
                get_d<8>(trow + SPEC * oc + 16 * p, w);  // conj x[r + 32 q], q = 8 p + j, lane = r
                const float u = __frcp_rn(s1) * (1.f / (S_MID_INV * BSCALE * BSCALE));
                if (qo >= 1) ok = ok && mbar_wait(B(B_OEMPTY), (qo - 1) & 1);
                ok = half_and(h, ok);
                if (!ok) break;
                unsigned char *ostg = base + OUT0;
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    *reinterpret_cast<float2 *>(ostg + swizzle64(32 * (8 * p + j) + lane, b)) =
                        make_float2(w[j].x * u, -w[j].y * u);
                fence_proxy_async_smem();
                mbar_arrive(B(B_OFULL));
                ++qo;
            }
            if (!ok) break;
        }
        // MMAs of this half still running after a failure complete before the TMEM is freed
        if (issuer && !ok) {
            mma_commit(mbar);
            mbar_wait(mbar, mma_n & 1);
        }
    }

    if (!ok && lane == 0) atomicOr(status, 1);
    tmem::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tmem::fence_after_sync();
        tmem::dealloc(tbase, TMEM_COLS);
    }
}

template <int OP> cudaError_t launch_op(const ZArgs &a, int ny, int *status, cudaStream_t st)
{
    if (!a.kern_zf || a.kzp != KP || (reinterpret_cast<uintptr_t>(a.kern_zf) & 15)) return cudaErrorInvalidValue;
    TcMaps maps;
    memset(&maps, 0, sizeof(maps));
    // [n_in z][Py y][ld x]: boxes of 8 columns x 1 y row x 256 planes
    auto map = [&](CUtensorMap *m, const void *p) {
        return tma::encode_spectrum(m, p, a.Mx, a.Py, a.n_in, a.row_stride * 8, a.axis_stride * 8, 1, 256);
    };
    for (int c = 0; c < a.nin; ++c)
        if (!map(&maps.in[c], a.in[c])) return cudaErrorInvalidValue;
    for (int c = 0; c < a.nout; ++c)
        if (a.out[c] && !map(&maps.out[c], a.out[c])) return cudaErrorInvalidValue;
    const int nxt = (a.Mx + COLS - 1) / COLS, ntiles = nxt * ny;
    if (ntiles <= 0) return cudaSuccess;
    const int grid = ntiles < tma::sm_count() ? ntiles : tma::sm_count();
    cudaError_t e = cudaFuncSetAttribute(k_ztc<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    k_ztc<OP><<<grid, NTHREADS, SMEM_BYTES, st>>>(a, maps, nxt, ntiles, status);
    return cudaGetLastError();
}

}  // namespace

bool ztc_supported(int prec, int L, int op, int nin, int nout, int n_in, int n_out)
{
    return prec == PREC_FP32 && L == LZ && n_in == NZ && n_out == NZ &&
           (op == OP_NONE || op == OP_GRAD || op == OP_DIV || op == OP_CURL) && nin >= 1 && nin <= 3 && nout >= 1 &&
           nout <= 3 && (op != OP_DIV && op != OP_CURL ? true : nin == 3) && tma::encode_fn() != nullptr;
}

size_t smem_ztc() { return SMEM_BYTES; }

cudaError_t launch_ztc(const ZArgs &a, int ny, int *status, cudaStream_t st)
{
    if (!status || !ztc_supported(PREC_FP32, a.L, a.op, a.nin, a.nout, a.n_in, a.n_out))
        return cudaErrorInvalidConfiguration;
    switch (a.op) {
    case OP_NONE: return launch_op<OP_NONE>(a, ny, status, st);
    case OP_GRAD: return launch_op<OP_GRAD>(a, ny, status, st);
    case OP_DIV: return launch_op<OP_DIV>(a, ny, status, st);
    case OP_CURL: return launch_op<OP_CURL>(a, ny, status, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace tc
}  // namespace ps
