// Device FFT core: Stockham autosort stages over lines held in shared memory.
//
// A CTA owns B "lines" (independent transforms of length L). Thread
// tid = t * B + b works on line b; the TPL threads of a line split each
// stage's L/R butterflies between them. Every stage reads its butterfly
// inputs into registers, synchronises, and writes the outputs back in
// place, so one shared buffer per line suffices (prime radices above 7 use a
// second, scratch buffer). The shared address of element n of line b is
// n * sn + b * sb: strided passes use sn = B, sb = 1 (a row of B adjacent
// columns, 128 bytes for the default B); the contiguous x pass uses sn = 1,
// sb = L + 1 (padded rows, so the B lines of one n fall in distinct banks).
//
// Stage s with radix R and sub-transform size m (the product of the radices
// before it) is the radix-R Stockham step: butterfly q*m + j reads
// x[q*m + j + r*L/R], multiplies by w_{mR}^{r j}, applies the R-point DFT and
// writes y[(q*R + r)*m + j]. After the last stage the line is in natural
// order. Forward uses e^{-2 pi i/N}; INV flips every sign.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "ps_dfloat.cuh"
#include "ps_types.hpp"

namespace ps {

template <typename T> struct CxT;
template <> struct CxT<double> { using type = double2; };
template <> struct CxT<float> { using type = float2; };
template <> struct CxT<dfloat> { using type = dfloat2; };

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return C{a.x + b.x, a.y + b.y}; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return C{a.x - b.x, a.y - b.y}; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b)
{
    return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b)
{
    return C{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
template <typename C, typename S> __device__ __forceinline__ C cscale(C a, S s) { return C{a.x * s, a.y * s}; }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename C> __device__ __forceinline__ C rot(C a)
{
    return INV ? C{-a.y, a.x} : C{a.y, -a.x};
}
// a + rot(b) and a - rot(b), the rotation folded into the additions
template <bool INV, typename C> __device__ __forceinline__ C addrot(C a, C b)
{
    return INV ? C{a.x - b.y, a.y + b.x} : C{a.x + b.y, a.y - b.x};
}
template <bool INV, typename C> __device__ __forceinline__ C subrot(C a, C b)
{
    return INV ? C{a.x + b.y, a.y - b.x} : C{a.x - b.y, a.y + b.x};
}

// FP32 complex addition and subtraction as one packed instruction each
// (add/sub.rn.f32x2, sm_100 and later): both lanes round to nearest like
// two scalar operations, so results are unchanged; the butterflies of the
// FFT stages issue half the instructions.
__device__ __forceinline__ float2 cadd(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 csub(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
// multiply by w = (c, -s) forward or (c, s) inverse, i.e. e^{-+ i theta}
template <bool INV, typename C, typename S> __device__ __forceinline__ C crot(C a, S c, S s)
{
    return INV ? C{a.x * c - a.y * s, a.x * s + a.y * c} : C{a.x * c + a.y * s, a.y * c - a.x * s};
}

// ---------------------------------------------------------------------------
// Small DFTs on register arrays (forward e^{-2 pi i/R}; INV conjugates).

template <bool INV, typename C> __device__ __forceinline__ void dft2(C &a, C &b)
{
    C t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV, typename C> __device__ __forceinline__ void dft4(C &x0, C &x1, C &x2, C &x3)
{
    const C t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), d = csub(x1, x3);
    x0 = cadd(t0, t2);
    x2 = csub(t0, t2);
    x1 = addrot<INV>(t1, d);
    x3 = subrot<INV>(t1, d);
}

// dft4 of (x0, x1, rot(x2), x3): x2 holds the third input before its
// rotation, which is folded into the first additions
template <bool INV, typename C> __device__ __forceinline__ void dft4_rot2(C &x0, C &x1, C &x2, C &x3)
{
    const C t0 = addrot<INV>(x0, x2), t1 = subrot<INV>(x0, x2), t2 = cadd(x1, x3), d = csub(x1, x3);
    x0 = cadd(t0, t2);
    x2 = csub(t0, t2);
    x1 = addrot<INV>(t1, d);
    x3 = subrot<INV>(t1, d);
}

template <bool INV, typename C> __device__ __forceinline__ void dft8(C *x)
{
    using S = decltype(x[0].x);
    const S h = (S)0.70710678118654752440;
    dft4<INV>(x[0], x[2], x[4], x[6]);
    dft4<INV>(x[1], x[3], x[5], x[7]);
    // twiddles w8^k on the odd half: w8^1, w8^2 = rot (folded into the
    // additions), w8^3 = rot w8^1 (folded into the constants)
    x[3] = crot<INV>(x[3], h, h);
    x[7] = crot<INV>(x[7], -h, h);
    C y[8];
    y[0] = cadd(x[0], x[1]); y[4] = csub(x[0], x[1]);
    y[1] = cadd(x[2], x[3]); y[5] = csub(x[2], x[3]);
    y[2] = addrot<INV>(x[4], x[5]); y[6] = subrot<INV>(x[4], x[5]);
    y[3] = cadd(x[6], x[7]); y[7] = csub(x[6], x[7]);
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = y[i];
}

// The twiddles and second layer of the 16-point DFT (after the first layer of
// four 4-point DFTs over n2, n = 4 n2 + n1).
template <bool INV, typename C> __device__ __forceinline__ void dft16_layer2(C *x);

template <bool INV, typename C> __device__ __forceinline__ void dft16(C *x)
{
    // n = 4 n2 + n1: four 4-point DFTs over n2 for each n1
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) dft4<INV>(x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]);
    dft16_layer2<INV>(x);
}

// The 16-point DFT of an input whose upper half x[8..15] is zero: the first
// layer's 4-point DFTs see (x[n1], x[n1 + 4], 0, 0).
template <bool INV, typename C> __device__ __forceinline__ void dft16_half(C *x)
{
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) {
        const C a = x[n1], b = x[n1 + 4];
        x[n1] = cadd(a, b);
        x[n1 + 8] = csub(a, b);
        x[n1 + 4] = addrot<INV>(a, b);
        x[n1 + 12] = subrot<INV>(a, b);
    }
    dft16_layer2<INV>(x);
}

template <bool INV, typename C> __device__ __forceinline__ void dft16_layer2(C *x)
{
    using S = decltype(x[0].x);
    const S c1 = (S)0.92387953251128675613, s1 = (S)0.38268343236508977173;
    const S h = (S)0.70710678118654752440;
    // x[n1 + 4 k1] now holds A[n1][k1]; multiply by w16^{n1 k1}. w^4 = rot is
    // folded into the k1 = 2 DFT, rot w^2 = w^6 and -w^1 = w^9 into the
    // constants.
    x[5] = crot<INV>(x[5], c1, s1);                // w^1
    x[9] = crot<INV>(x[9], h, h);                  // w^2
    x[13] = crot<INV>(x[13], s1, c1);              // w^3
    x[6] = crot<INV>(x[6], h, h);                  // w^2
    x[14] = crot<INV>(x[14], -h, h);               // w^6
    x[7] = crot<INV>(x[7], s1, c1);                // w^3
    x[11] = crot<INV>(x[11], -h, h);               // w^6
    x[15] = crot<INV>(x[15], -c1, -s1);            // w^9
    // X[k1 + 4 k2] = DFT4 over n1 of A[n1][k1]
    C y[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        C a0 = x[4 * k1], a1 = x[4 * k1 + 1], a2 = x[4 * k1 + 2], a3 = x[4 * k1 + 3];
        if (k1 == 2) dft4_rot2<INV>(a0, a1, a2, a3);  // a2 = A[2][2] w^4
        else dft4<INV>(a0, a1, a2, a3);
        y[k1] = a0; y[k1 + 4] = a1; y[k1 + 8] = a2; y[k1 + 12] = a3;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = y[i];
}

template <bool INV, typename C> __device__ __forceinline__ void dft3(C *x)
{
    using S = decltype(x[0].x);
    const S s3 = (S)0.86602540378443864676;
    C t1 = cadd(x[1], x[2]), t2 = cscale(csub(x[1], x[2]), s3);
    C a = C{x[0].x - (S)0.5 * t1.x, x[0].y - (S)0.5 * t1.y};
    x[0] = cadd(x[0], t1);
    x[1] = addrot<INV>(a, t2);
    x[2] = subrot<INV>(a, t2);
}

// Odd prime R with cosines c[k-1] = cos(2 pi k/R), sines s[k-1] = sin(2 pi k/R):
// y_k = x0 + sum_n c_{nk}(x_n + x_{R-n}) -/+ i sum_n s_{nk}(x_n - x_{R-n}).
template <bool INV, int R, typename C, typename S>
__device__ __forceinline__ void dft_odd(C *x, const S *c, const S *s)
{
    constexpr int H = (R - 1) / 2;
    C p[H], q[H];
#pragma unroll
    for (int n = 1; n <= H; ++n) {
        p[n - 1] = cadd(x[n], x[R - n]);
        q[n - 1] = csub(x[n], x[R - n]);
    }
    C y0 = x[0];
#pragma unroll
    for (int n = 0; n < H; ++n) y0 = cadd(y0, p[n]);
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        C a = x[0], b = C{0, 0};
#pragma unroll
        for (int n = 1; n <= H; ++n) {
            const int e = (n * k) % R;  // cos(2 pi e/R), sin(2 pi e/R)
            const S cc = e <= H ? c[e - 1] : c[R - e - 1];
            const S ss = e <= H ? s[e - 1] : -s[R - e - 1];
            a = C{a.x + cc * p[n - 1].x, a.y + cc * p[n - 1].y};
            b = C{b.x + ss * q[n - 1].x, b.y + ss * q[n - 1].y};
        }
        x[k] = addrot<INV>(a, b);
        x[R - k] = subrot<INV>(a, b);
    }
    x[0] = y0;
}

template <bool INV, typename C> __device__ __forceinline__ void dft5(C *x)
{
    using S = decltype(x[0].x);
    const S c[2] = {(S)0.30901699437494742410, (S)-0.80901699437494742410};
    const S s[2] = {(S)0.95105651629515357212, (S)0.58778525229247312917};
    dft_odd<INV, 5>(x, c, s);
}

template <bool INV, typename C> __device__ __forceinline__ void dft7(C *x)
{
    using S = decltype(x[0].x);
    const S c[3] = {(S)0.62348980185873353053, (S)-0.22252093395631440429, (S)-0.90096886790241912624};
    const S s[3] = {(S)0.78183148246802980871, (S)0.97492791218182360702, (S)0.43388373911755812048};
    dft_odd<INV, 7>(x, c, s);
}

// 32 = 2 x 16: X[k] = E[k] + w32^k O[k], X[k+16] = E[k] - w32^k O[k].
template <bool INV, typename C> __device__ __forceinline__ void dft32(C *x)
{
    using S = decltype(x[0].x);
    C e[16], o[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        e[i] = x[2 * i];
        o[i] = x[2 * i + 1];
    }
    dft16<INV>(e);
    dft16<INV>(o);
    const S c[8] = {(S)1.0, (S)0.98078528040323044913, (S)0.92387953251128675613, (S)0.83146961230254523708,
                    (S)0.70710678118654752440, (S)0.55557023301960222474, (S)0.38268343236508977173,
                    (S)0.19509032201612826785};
    // w32^k: k < 8 from the table; w32^8 = rot, folded into the additions;
    // w32^k = rot w32^(k-8) for k > 8, folded into the constants
#pragma unroll
    for (int k = 1; k < 16; ++k) {
        if (k < 8) o[k] = crot<INV>(o[k], c[k], c[8 - k]);
        else if (k > 8) o[k] = crot<INV>(o[k], -c[16 - k], c[k - 8]);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        if (k == 8) {
            x[k] = addrot<INV>(e[k], o[k]);
            x[k + 16] = subrot<INV>(e[k], o[k]);
        } else {
            x[k] = cadd(e[k], o[k]);
            x[k + 16] = csub(e[k], o[k]);
        }
    }
}

// The 32-point DFT of an input whose upper half x[16..31] is zero (the
// zero-padded half of an unbounded axis): both 16-point halves are half zero.
template <bool INV, typename C> __device__ __forceinline__ void dft32_half(C *x)
{
    using S = decltype(x[0].x);
    C e[16], o[16];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        e[i] = x[2 * i];
        o[i] = x[2 * i + 1];
    }
    dft16_half<INV>(e);
    dft16_half<INV>(o);
    const S c[8] = {(S)1.0, (S)0.98078528040323044913, (S)0.92387953251128675613, (S)0.83146961230254523708,
                    (S)0.70710678118654752440, (S)0.55557023301960222474, (S)0.38268343236508977173,
                    (S)0.19509032201612826785};
    // w32^k: k < 8 from the table; w32^8 = rot, folded into the additions;
    // w32^k = rot w32^(k-8) for k > 8, folded into the constants
#pragma unroll
    for (int k = 1; k < 16; ++k) {
        if (k < 8) o[k] = crot<INV>(o[k], c[k], c[8 - k]);
        else if (k > 8) o[k] = crot<INV>(o[k], -c[16 - k], c[k - 8]);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        if (k == 8) {
            x[k] = addrot<INV>(e[k], o[k]);
            x[k + 16] = subrot<INV>(e[k], o[k]);
        } else {
            x[k] = cadd(e[k], o[k]);
            x[k + 16] = csub(e[k], o[k]);
        }
    }
}

template <int R, bool INV, typename C> __device__ __forceinline__ void dft(C *x)
{
    if constexpr (R == 2) dft2<INV>(x[0], x[1]);
    else if constexpr (R == 3) dft3<INV>(x);
    else if constexpr (R == 4) dft4<INV>(x[0], x[1], x[2], x[3]);
    else if constexpr (R == 5) dft5<INV>(x);
    else if constexpr (R == 7) dft7<INV>(x);
    else if constexpr (R == 8) dft8<INV>(x);
    else if constexpr (R == 16) dft16<INV>(x);
    else if constexpr (R == 32) dft32<INV>(x);
}

// ---------------------------------------------------------------------------
// Per-stage descriptors, copied from the plan into shared memory at kernel
// start (indexing the plan's arrays in the kernel parameters at run time
// would force a local-memory copy of the whole parameter block).
struct StageInfo {
    int4 st[MAX_STAGES];       // radix, m, twiddle offset, generic-table offset
    int lm[MAX_STAGES];        // log2(m) or -1
    unsigned mg[MAX_STAGES];   // floor(2^32 / m) + 1 when m is not a power of two (split_index)
};

// One stage a thread (the caller synchronises before the first use).
__device__ __forceinline__ void load_stages(StageInfo &si, const FftPlanDev &P)
{
    const int i = threadIdx.x;
    if (i < MAX_STAGES) {
        si.st[i] = make_int4(P.radix[i], P.m[i], P.tw[i], P.gw[i]);
        si.lm[i] = P.lm[i];
        si.mg[i] = P.lm[i] < 0 && P.m[i] > 1 ? 0xFFFFFFFFu / (unsigned)P.m[i] + 1u : 0u;
    }
}

// Copy the plan's twiddle table to shared memory and return the copy, which
// the stages read (the caller synchronises before the first stage).
template <typename C> __device__ __forceinline__ const C *stage_twiddles(const FftPlanDev &P, C *TW)
{
    const C *g = reinterpret_cast<const C *>(P.table);
    for (int i = threadIdx.x; i < P.ntw; i += blockDim.x) TW[i] = __ldg(&g[i]);
    return TW;
}

// Division of n < 2^16 by a run-time d < 2^16 without a divide: q = n / d is
// the high word of n * div_magic(d) (the multiplier argument of split_index
// below); d = 1 gives n.
__device__ __forceinline__ unsigned div_magic(int d) { return d > 1 ? 0xFFFFFFFFu / (unsigned)d + 1u : 0u; }
__device__ __forceinline__ int div_by(int n, int d, unsigned mg) { return d > 1 ? (int)__umulhi((unsigned)n, mg) : n; }

// j = bf mod m and q = bf / m, by shifts when m is a power of two, else by
// the multiplier mg = floor(2^32 / m) + 1: with mg m = 2^32 + e, 0 < e <= m,
// floor(bf mg / 2^32) = floor(bf / m) whenever bf e < 2^32, which bf, m < 2^16
// (butterfly counts and sub-transform sizes of any plan) guarantee.
__device__ __forceinline__ void split_index(int bf, int m, int lm, unsigned mg, int &j, int &q)
{
    if (lm >= 0) {
        j = bf & (m - 1);
        q = bf >> lm;
    } else {
        q = (int)__umulhi((unsigned)bf, mg);
        j = bf - q * m;
    }
}

// One in-place Stockham stage with a compile-time radix.
template <int EM, int R, bool INV, typename C, typename PL>
__device__ __forceinline__ void stage(C *S, int sn, int sb, int b, int t, const PL &P, const C *tws, int4 sd, int lm,
                                      unsigned mg = 0u)
{
    constexpr int U = EM / R;
    const int L = P.L, m = sd.y, nbf = L / R, tpl = P.tpl;
    const C *tw = tws + sd.z;
    C *Sb = S + b * sb;
    const int rstride = nbf * sn;
    C v[U][R];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int bf = t + u * tpl;
        if (bf < nbf) {
            int j, q;
            split_index(bf, m, lm, mg, j, q);
            const C *src = Sb + bf * sn;
#pragma unroll
            for (int r = 0; r < R; ++r) v[u][r] = src[r * rstride];
            if (m > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    const C w = tw[j * (R - 1) + r - 1];
                    v[u][r] = INV ? cmulc(v[u][r], w) : cmul(v[u][r], w);
                }
            }
            dft<R, INV>(v[u]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int bf = t + u * tpl;
        if (bf < nbf) {
            int j, q;
            split_index(bf, m, lm, mg, j, q);
            C *dst = Sb + (q * R * m + j) * sn;
            const int mstride = m * sn;
#pragma unroll
            for (int r = 0; r < R; ++r) dst[r * mstride] = v[u][r];
        }
    }
    __syncthreads();
}

// A stage with a prime radix above 7 (no unrolled butterfly): a direct
// R-point DFT for every butterfly, out of place into W, then copied back. The
// L outputs of a line (butterfly bf = o mod nbf, output k = o / nbf) are
// spread over the line's threads, so the stage runs L R complex products on
// tpl threads however few butterflies it has (a length-194 line has 2).
// Twiddles are applied to the inputs in place first; each output then sums
// R twiddled inputs in the order r = 0 .. R-1.
template <bool INV, typename C, typename PL>
__device__ void stage_generic(C *S, C *W, int sn, int sb, int b, int t, const PL &P, const C *tws, int4 sd)
{
    const int L = P.L, R = sd.x, m = sd.y, nbf = L / R, tpl = P.tpl;
    const C *tw = tws + sd.z;
    const C *gw = tws + sd.w;
    C *Sb = S + b * sb, *Wb = W + b * sb;
    const unsigned mgn = div_magic(nbf), mgm = div_magic(m);  // index divisions by nbf and m
    if (m > 1) {
        for (int e = t; e < L; e += tpl) {
            const int r = div_by(e, nbf, mgn), bf = e - r * nbf;
            if (r > 0) {
                const C w = tw[(bf - div_by(bf, m, mgm) * m) * (R - 1) + r - 1];
                Sb[e * sn] = INV ? cmulc(Sb[e * sn], w) : cmul(Sb[e * sn], w);
            }
        }
        __syncthreads();
    }
    for (int o = t; o < L; o += tpl) {
        const int k = div_by(o, nbf, mgn), bf = o - k * nbf;
        const int q = div_by(bf, m, mgm), j = bf - q * m;
        C acc = C{0, 0};
        int idx = 0;  // (r k) mod R
        for (int r = 0; r < R; ++r) {
            const C x = Sb[(bf + r * nbf) * sn];
            const C g = gw[idx];
            acc = cadd(acc, INV ? cmulc(x, g) : cmul(x, g));
            idx += k;
            if (idx >= R) idx -= R;
        }
        Wb[(q * R * m + j + k * m) * sn] = acc;
    }
    __syncthreads();
    for (int e = t; e < L; e += tpl) Sb[e * sn] = Wb[e * sn];
    __syncthreads();
}

// Stages s .. ns-1 of the stage table over lines of P.L elements with P.tpl
// threads a line (P the plan for its own stages, a LineGeom for the
// sub-transforms of a Rader plan), for ncomp line sets cstride elements apart. EM is the register
// elements a thread holds per stage (and the largest radix); the plan's
// threads-per-line was computed for the same EM.
// Thread t of a line takes butterflies t, t + tpl, ...: a caller passes t = L
// for a thread that must only join the barriers (every butterfly index it
// would take is then past the stage's count).
// The plan orders its stages as prime radices above 7, then 7s, 5s, 3s, 16s
// (FP32 only), 8s, and at most one 4 or 2; each radix runs in its own loop,
// with the line sets innermost, so that the register arrays of different
// radices never share a live range (a radix switch inside one stage loop, or
// the stage loops inside a component loop, made the register allocator keep
// them all live and spill).
// Radices without an unrolled butterfly: primes above 7 (11 and 13 included).
__device__ __forceinline__ bool is_generic_radix(int R) { return R > 8 && R != 16; }

template <bool INV, int EM, typename C, typename PL>
__device__ __forceinline__ void run_stages(C *S, C *W, int sn, int sb, int b, int t, const PL &P, int s, int ns,
                                           const C *tws, const StageInfo &si, int ncomp, int cstride)
{
    for (; s < ns && is_generic_radix(si.st[s].x); ++s)
        for (int c = 0; c < ncomp; ++c) stage_generic<INV>(S + c * cstride, W, sn, sb, b, t, P, tws, si.st[s]);
    for (; s < ns && si.st[s].x == 7; ++s)
        for (int c = 0; c < ncomp; ++c) stage<EM, 7, INV>(S + c * cstride, sn, sb, b, t, P, tws, si.st[s], si.lm[s], si.mg[s]);
    for (; s < ns && si.st[s].x == 5; ++s)
        for (int c = 0; c < ncomp; ++c) stage<EM, 5, INV>(S + c * cstride, sn, sb, b, t, P, tws, si.st[s], si.lm[s], si.mg[s]);
    for (; s < ns && si.st[s].x == 3; ++s)
        for (int c = 0; c < ncomp; ++c) stage<EM, 3, INV>(S + c * cstride, sn, sb, b, t, P, tws, si.st[s], si.lm[s], si.mg[s]);
    if constexpr (EM >= 16)
        for (; s < ns && si.st[s].x == 16; ++s)
            for (int c = 0; c < ncomp; ++c) stage<EM, 16, INV>(S + c * cstride, sn, sb, b, t, P, tws, si.st[s], si.lm[s], si.mg[s]);
    for (; s < ns && si.st[s].x == 8; ++s)
        for (int c = 0; c < ncomp; ++c) stage<EM, 8, INV>(S + c * cstride, sn, sb, b, t, P, tws, si.st[s], si.lm[s], si.mg[s]);
    if (s < ns && si.st[s].x == 4) {
        for (int c = 0; c < ncomp; ++c) stage<EM, 4, INV>(S + c * cstride, sn, sb, b, t, P, tws, si.st[s], si.lm[s], si.mg[s]);
        ++s;
    }
    if (s < ns && si.st[s].x == 2) {
        for (int c = 0; c < ncomp; ++c) stage<EM, 2, INV>(S + c * cstride, sn, sb, b, t, P, tws, si.st[s], si.lm[s], si.mg[s]);
        ++s;
    }
}

template <bool INV, int EM, typename C>
__device__ __forceinline__ void fft_stages(C *S, C *W, int sn, int sb, int b, int t, const FftPlanDev &P,
                                           const C *tws, const StageInfo &si, int ncomp, int cstride)
{
    run_stages<INV, EM>(S, W, sn, sb, b, t, P, 0, P.nstages, tws, si, ncomp, cstride);
}

// Line-thread index of a thread that must only join the barriers: past every
// butterfly and every element of any plan.
constexpr int IDLE_T = 1 << 28;

// Compile-time stage sequence of a power-of-two length M with EM elements a
// thread: radix-EM stages, then one radix 2^rem stage (the order the host's
// factorisation gives such a length), with M / EM threads a line. Every
// radix, sub-transform size, twiddle offset and loop bound is a constant, so
// the index arithmetic of the run-time stage loop folds away. The host marks
// the Bluestein plans whose convolution stages are exactly these (ctm = M).
__host__ __device__ constexpr int ct_log2(int x) { return x <= 1 ? 0 : 1 + ct_log2(x >> 1); }

template <int M, int EM> struct CtPlan {
    static constexpr int LM = ct_log2(M), LE = ct_log2(EM);
    static constexpr int NFULL = LM / LE, REM = LM - NFULL * LE, NST = NFULL + (REM ? 1 : 0);
    static constexpr int L = M, tpl = M / EM;
    __host__ __device__ static constexpr int radix(int s) { return s < NFULL ? EM : (1 << REM); }
    __host__ __device__ static constexpr int mm(int s) { return s == 0 ? 1 : mm(s - 1) * radix(s - 1); }
    __host__ __device__ static constexpr int tw(int s) { return s == 0 ? 0 : tw(s - 1) + mm(s - 1) * (radix(s - 1) - 1); }
};

template <bool INV, int EM, int M, int S = 0, typename C>
__device__ __forceinline__ void ct_stages(C *Sl, int sn, int sb, int b, int t, const C *tws, int ncomp, int cstride)
{
    using PL = CtPlan<M, EM>;
    if constexpr (S < PL::NST) {
        constexpr int R = PL::radix(S), m = PL::mm(S);
        for (int c = 0; c < ncomp; ++c)
            stage<EM, R, INV>(Sl + c * cstride, sn, sb, b, t, PL{}, tws, make_int4(R, m, PL::tw(S), 0), ct_log2(m));
        ct_stages<INV, EM, M, S + 1>(Sl, sn, sb, b, t, tws, ncomp, cstride);
    }
}

// The convolution transforms of a Bluestein plan: compile-time stages for
// the marked power-of-two lengths in FP32 and FP64, the run-time stage loop
// otherwise (double-float transforms included: unrolled, their arithmetic
// made the compile of their instantiations several times longer).
template <bool INV, int EM, typename C>
__device__ __forceinline__ void blue_stages(C *S, C *W, int sn, int sb, int b, int t, const FftPlanDev &P,
                                            const C *tws, const StageInfo &si, int ncomp, int cstride)
{
    if constexpr (std::is_same<C, float2>::value || std::is_same<C, double2>::value) {
        switch (P.ctm) {
        case 64: ct_stages<INV, EM, 64>(S, sn, sb, b, t, tws, ncomp, cstride); return;
        case 128: ct_stages<INV, EM, 128>(S, sn, sb, b, t, tws, ncomp, cstride); return;
        case 256: ct_stages<INV, EM, 256>(S, sn, sb, b, t, tws, ncomp, cstride); return;
        case 512: ct_stages<INV, EM, 512>(S, sn, sb, b, t, tws, ncomp, cstride); return;
        case 1024: ct_stages<INV, EM, 1024>(S, sn, sb, b, t, tws, ncomp, cstride); return;
        default: break;
        }
    }
    fft_stages<INV, EM>(S, W, sn, sb, b, t, P, tws, si, ncomp, cstride);
}

// Bluestein's algorithm for a length lb with a large prime factor, on lines
// of M = P.L >= 2 lb - 1 elements (a power of two, or 2^a 3^b 5^c): with
// c[n] = e^{-i pi n^2 / lb}, X[k] = c[k] sum_n (x[n] c[n]) conj(c[k - n]), a
// circular convolution of length M done by the plan's stages (forward, times the precomputed
// spectrum K of the wrapped conj(c) scaled by 1/M, unnormalised inverse). The
// inverse DFT conjugates the chirp and reads K at -k, which is the spectrum of
// the wrapped c. The chirp and K are read from the shared copy of the table
// when the plan stages them there (bsh), else from the plan's global table
// (each entry once a line); the stage twiddles always from shared memory.
template <bool INV, int EM, typename C>
__device__ __forceinline__ void bluestein_lines(C *S, C *W, int sn, int sb, int b, int t, const FftPlanDev &P,
                                                const C *tws, const StageInfo &si, int ncomp, int cstride)
{
    const int M = P.L, Lb = P.lb, tpl = P.tpl;
    const C *g = P.bsh ? tws : reinterpret_cast<const C *>(P.table);
    const C *ch = g + P.chirp, *K = g + P.kspec;
    for (int c = 0; c < ncomp; ++c) {
        C *Sb = S + c * cstride + b * sb;
        for (int n = t; n < M; n += tpl) {
            C v = C{0, 0};
            if (n < Lb) v = INV ? cmulc(Sb[n * sn], ch[n]) : cmul(Sb[n * sn], ch[n]);
            Sb[n * sn] = v;
        }
    }
    __syncthreads();
    blue_stages<false, EM>(S, W, sn, sb, b, t, P, tws, si, ncomp, cstride);
    for (int c = 0; c < ncomp; ++c) {
        C *Sb = S + c * cstride + b * sb;
        for (int k = t; k < M; k += tpl) {
            const int km = k == 0 ? 0 : M - k;
            const C kk = INV ? C{K[km].x, -K[km].y} : K[k];
            Sb[k * sn] = cmul(Sb[k * sn], kk);
        }
    }
    __syncthreads();
    blue_stages<true, EM>(S, W, sn, sb, b, t, P, tws, si, ncomp, cstride);
    for (int c = 0; c < ncomp; ++c) {
        C *Sb = S + c * cstride + b * sb;
        for (int k = t; k < Lb; k += tpl) Sb[k * sn] = INV ? cmulc(Sb[k * sn], ch[k]) : cmul(Sb[k * sn], ch[k]);
    }
    __syncthreads();
}

// The line geometry the stage functions read (a plan's, or a Rader plan's
// sub-transforms').
struct LineGeom {
    int L, tpl;
};

// What a Rader stage reads of its plan, gathered once.
template <typename C> struct RaderGeom {
    int L, tpl, ns;            // line length, threads a line, stages of the plan
    int q1, rtpl, rs0, rns;    // sub-transform length p - 1, its threads, its stages
    float ip, iq;              // 1 / p and 1 / (p - 1)
    const int *itab;           // g^-j mod p (j < p - 1), then log_g k at k - 1
    const C *bh;               // FFT(beta) / (p - 1): forward, then inverse
};

template <typename C> __device__ __forceinline__ RaderGeom<C> rader_geom(const FftPlanDev &P)
{
    return RaderGeom<C>{P.L, P.tpl, P.nstages, P.rq, P.rtpl, P.rs0, P.rns, P.rinv_p, P.rinv_q, P.itab,
                        reinterpret_cast<const C *>(P.table) + P.rbh};
}

// The sub-transforms of a Rader stage: the L / p sub-lines of p - 1 points of
// every line set at once, sub-line bf on line threads [bf rtpl, (bf + 1) rtpl)
// (the plan's threads a line cover them all). No loop over sub-lines: with
// the stages inside one, ptxas spilled.
template <bool INV, int EM, typename C>
__device__ __forceinline__ void rader_sub(C *S, C *W, int sn, int sb, int b, int t, const RaderGeom<C> &g,
                                          const C *tws, const StageInfo &si, int ncomp, int cstride)
{
    const int q1 = g.q1, nbf = g.L / (q1 + 1), tps = g.rtpl;
    const int bf = t < g.tpl ? t / tps : nbf;
    const bool on = bf < nbf;
    const int off = on ? bf * q1 * sn : 0;
    run_stages<INV, EM>(S + off, W + off, sn, sb, b, on ? t - bf * tps : IDLE_T, LineGeom{q1, tps}, g.rs0,
                        g.rs0 + g.rns, tws, si, ncomp, cstride);
}

// Rader's algorithm for stage 0 of a Rader plan, then the plan's other
// stages. Stage 0 has a prime radix p and m = 1: butterfly bf < nbf = L / p
// is the p-point DFT of x[bf + r nbf], written to y[bf p + k]. With g a
// primitive root mod p, a[j] = x[bf + g^-j nbf] (j < p - 1) and
// beta[m] = w^(g^m), w = e^{-+2 pi i / p}:
//   y[bf p + g^q] = x[bf] + (a (*) beta)[q],  y[bf p] = x[bf] + sum_j a[j],
// a cyclic convolution of p - 1 points, computed as the sub-transform of a,
// times the precomputed spectrum FFT(beta) / (p - 1), and the unnormalised
// inverse sub-transform. In each line the sub-line of butterfly bf takes
// elements [bf (p - 1), (bf + 1)(p - 1)) and x[bf] the spare element
// nbf (p - 1) + bf; sum_j a[j] (the sub-transform's DC term) is kept in a
// register by line thread bf (nbf <= tpl, since tpl EM >= L). The scratch
// line W (one for all line sets) stages the gather and the outputs, and is
// the scratch of direct-DFT sub-stages (radix 11 or 13) in between.
// Index division by p and p - 1 runs in FP32: (e + 1/2) / q lies at least
// 1 / (2 q) from an integer, far above the rounding error for any line length.
template <bool INV, int EM, typename C>
__device__ __forceinline__ void rader_lines(C *S, C *W, int sn, int sb, int b, int t, const RaderGeom<C> &g,
                                            const C *tws, const StageInfo &si, int ncomp, int cstride)
{
    const int L = g.L, tpl = g.tpl, q1 = g.q1, p = q1 + 1, nbf = L / p, nq = nbf * q1;
    const int *perm = g.itab, *qlog = g.itab + q1;
    const C *bh = g.bh + (INV ? q1 : 0);
    C *Wb = W + b * sb;
    // gather: sub-line entries a[j] and x[bf] at the spare elements
    for (int c = 0; c < ncomp; ++c) {
        C *Sb = S + c * cstride + b * sb;
        for (int e = t; e < L; e += tpl) Wb[e * sn] = Sb[e * sn];
        __syncthreads();
        for (int e = t; e < L; e += tpl) {
            int src = e - nq;
            if (e < nq) {
                const int bf = (int)(((float)e + 0.5f) * g.iq), j = e - bf * q1;
                src = bf + __ldg(&perm[j]) * nbf;
            }
            Sb[e * sn] = Wb[src * sn];
        }
        __syncthreads();
    }
    rader_sub<false, EM>(S, W, sn, sb, b, t, g, tws, si, ncomp, cstride);
    // keep the DC terms, then multiply by the convolution spectrum
    C a0[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        a0[c] = C{0, 0};
        if (c < ncomp && t < nbf) a0[c] = S[c * cstride + b * sb + t * q1 * sn];
    }
    __syncthreads();
    for (int c = 0; c < ncomp; ++c) {
        C *Sb = S + c * cstride + b * sb;
        for (int e = t; e < nq; e += tpl) {
            const int bf = (int)(((float)e + 0.5f) * g.iq), j = e - bf * q1;
            Sb[e * sn] = cmul(Sb[e * sn], bh[j]);
        }
    }
    __syncthreads();
    rader_sub<true, EM>(S, W, sn, sb, b, t, g, tws, si, ncomp, cstride);
    // outputs into W (k > 0 from the convolution, k = 0 by line thread bf), then back
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (c >= ncomp) break;  // ncomp is the same on every thread
        C *Sb = S + c * cstride + b * sb;
        for (int e = t; e < L; e += tpl) {
            const int bf = (int)(((float)e + 0.5f) * g.ip), k = e - bf * p;
            if (k > 0) Wb[e * sn] = cadd(Sb[(nq + bf) * sn], Sb[(bf * q1 + __ldg(&qlog[k - 1])) * sn]);
        }
        if (t < nbf) Wb[t * p * sn] = cadd(Sb[(nq + t) * sn], a0[c]);
        __syncthreads();
        for (int e = t; e < L; e += tpl) Sb[e * sn] = Wb[e * sn];
        __syncthreads();
    }
    run_stages<INV, EM>(S, W, sn, sb, b, t, LineGeom{L, tpl}, 1, g.ns, tws, si, ncomp, cstride);
}

// The transform of a plan. RAD: the kernel runs Rader plans too (separate
// instantiations, so that the registers of the Rader path do not count
// against the kernels of the other plans).
template <bool INV, int EM, bool RAD = false, typename C>
__device__ __forceinline__ void fft_lines(C *S, C *W, int sn, int sb, int b, int t, const FftPlanDev &P, const C *tws,
                                          const StageInfo &si, int ncomp = 1, int cstride = 0)
{
    if (P.blue) {
        bluestein_lines<INV, EM>(S, W, sn, sb, b, t, P, tws, si, ncomp, cstride);
        return;
    }
    if constexpr (RAD) {
        if (P.rader) {
            const RaderGeom<C> g = rader_geom<C>(P);
            rader_lines<INV, EM>(S, W, sn, sb, b, t, g, tws, si, ncomp, cstride);
            return;
        }
    }
    fft_stages<INV, EM>(S, W, sn, sb, b, t, P, tws, si, ncomp, cstride);
}

// Component c of a three-entry parameter array, read with constant indices.
template <typename T> __device__ __forceinline__ T pick3(const T (&a)[3], int c)
{
    return c == 0 ? a[0] : (c == 1 ? a[1] : a[2]);
}

// Element offsets of the rows row0 .. row0 + nrows - 1 of a [rows_z][ystride][ld]
// half-spectrum array (row r = (z, y) with y = r mod rows_y), -1 past the last
// row. The x passes compute them once per CTA instead of dividing per element.
__device__ __forceinline__ void row_offsets(long long *ofs, long long row0, int nrows, long long rows, int rows_y,
                                            int ystride, int ld)
{
    for (int i = threadIdx.x; i < nrows; i += blockDim.x) {
        const long long r = row0 + i;
        ofs[i] = r < rows ? ((r / rows_y) * ystride + r % rows_y) * ld : -1;
    }
}

}  // namespace ps
