// Packed ("pair") FP32 FFT arithmetic: two complex values a, b held as a
// pair of real parts (a.re, b.re) and a pair of imaginary parts (a.im, b.im),
// so that every operation both take with the same constant -- additions,
// rotations by +-i, multiplications by a root of unity -- runs on the two
// lanes of one packed instruction (add/sub/mul/fma.rn.f32x2, sm_100 and
// later). Against the complex-as-(re, im) layout this halves the
// multiplications and makes the rotations by +-i free (the real and
// imaginary pairs swap roles in the following addition); the price is that
// combining the two values with each other takes scalar operations.
//
// The 32-point DFT here takes its inputs as pairs (x[2i], x[2i+1]): both
// 16-point halves of the radix-2 split run at once, one a lane, and the
// outputs come out as pairs (X[k], X[k+16]).
#pragma once
#include <cuda_runtime.h>

namespace ps {
namespace pk {

struct P2 {
    float2 r;  // real parts of the two values
    float2 i;  // imaginary parts
};

__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mul.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
// a * b + c
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pc, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mov.b64 pc, {%6, %7};\n\tfma.rn.f32x2 pr, pa, pb, pc;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}
__device__ __forceinline__ float2 dup(float s) { return make_float2(s, s); }

__device__ __forceinline__ P2 padd(P2 a, P2 b) { return P2{add2(a.r, b.r), add2(a.i, b.i)}; }
__device__ __forceinline__ P2 psub(P2 a, P2 b) { return P2{sub2(a.r, b.r), sub2(a.i, b.i)}; }
// a + rot(b) and a - rot(b), rot = multiply by -i (forward) or +i (inverse)
template <bool INV> __device__ __forceinline__ P2 paddrot(P2 a, P2 b)
{
    return INV ? P2{sub2(a.r, b.i), add2(a.i, b.r)} : P2{add2(a.r, b.i), sub2(a.i, b.r)};
}
template <bool INV> __device__ __forceinline__ P2 psubrot(P2 a, P2 b)
{
    return INV ? P2{add2(a.r, b.i), sub2(a.i, b.r)} : P2{sub2(a.r, b.i), add2(a.i, b.r)};
}
// multiply both values by (c, -s) forward or (c, s) inverse, i.e. e^{-+ i theta},
// with cc = (c, c), ss = (s, s), ns = (-s, -s)
template <bool INV> __device__ __forceinline__ P2 pcrot(P2 a, float2 cc, float2 ss, float2 ns)
{
    return INV ? P2{fma2(a.i, ns, mul2(a.r, cc)), fma2(a.r, ss, mul2(a.i, cc))}
               : P2{fma2(a.i, ss, mul2(a.r, cc)), fma2(a.r, ns, mul2(a.i, cc))};
}

// The rotation constants of the 16-point DFT as pairs: c1 = cos(pi / 8),
// s1 = sin(pi / 8), h = cos(pi / 4), and their negatives. A packed
// instruction takes no immediate operand, so a constant pair written in
// place is rebuilt at every use; a kernel reads these once from memory
// (load_rot_consts) and keeps them in registers.
struct RotConsts {
    float2 c1, s1, h, nc1, ns1, nh;
};
constexpr float ROT_C1 = 0.92387953251128675613f, ROT_S1 = 0.38268343236508977173f, ROT_H = 0.70710678118654752440f;

// 12 floats: c1, c1, s1, s1, h, h, -c1, -c1, -s1, -s1, -h, -h
__device__ __forceinline__ void store_rot_consts(float *dst)
{
    const float v[6] = {ROT_C1, ROT_S1, ROT_H, -ROT_C1, -ROT_S1, -ROT_H};
    for (int i = 0; i < 12; ++i) dst[i] = v[i / 2];
}
__device__ __forceinline__ RotConsts load_rot_consts(const float *src)
{
    const float2 *p = reinterpret_cast<const float2 *>(src);
    return RotConsts{p[0], p[1], p[2], p[3], p[4], p[5]};
}
// multiply lane by lane by w = (wr, wi) (forward) or by conj(w) (inverse)
template <bool INV> __device__ __forceinline__ P2 ptwiddle(P2 a, float2 wr, float2 wi)
{
    return INV ? P2{fma2(a.i, wi, mul2(a.r, wr)), sub2(mul2(a.i, wr), mul2(a.r, wi))}
               : P2{sub2(mul2(a.r, wr), mul2(a.i, wi)), fma2(a.r, wi, mul2(a.i, wr))};
}
__device__ __forceinline__ P2 pscale(P2 a, float2 s) { return P2{mul2(a.r, s), mul2(a.i, s)}; }

// the 4-point DFT of (x0, x1, x2, x3), each a pair
template <bool INV> __device__ __forceinline__ void pdft4(P2 &x0, P2 &x1, P2 &x2, P2 &x3)
{
    const P2 t0 = padd(x0, x2), t1 = psub(x0, x2), t2 = padd(x1, x3), d = psub(x1, x3);
    x0 = padd(t0, t2);
    x2 = psub(t0, t2);
    x1 = paddrot<INV>(t1, d);
    x3 = psubrot<INV>(t1, d);
}

// pdft4 of (x0, x1, rot(x2), x3), the rotation folded into the additions
template <bool INV> __device__ __forceinline__ void pdft4_rot2(P2 &x0, P2 &x1, P2 &x2, P2 &x3)
{
    const P2 t0 = paddrot<INV>(x0, x2), t1 = psubrot<INV>(x0, x2), t2 = padd(x1, x3), d = psub(x1, x3);
    x0 = padd(t0, t2);
    x2 = psub(t0, t2);
    x1 = paddrot<INV>(t1, d);
    x3 = psubrot<INV>(t1, d);
}

// Twiddles and second layer of the 16-point DFT (after four 4-point DFTs over
// n2, n = 4 n2 + n1): the radix-4 x 4 split of the complex-layout dft16.
template <bool INV> __device__ __forceinline__ void pdft16_layer2(P2 *x, const RotConsts &k)
{
    // rotations by (c, s): x5 (c1, s1), x9 and x6 (h, h), x13 and x7 (s1, c1),
    // x14 and x11 (-h, h), x15 (-c1, -s1)
    x[5] = pcrot<INV>(x[5], k.c1, k.s1, k.ns1);
    x[9] = pcrot<INV>(x[9], k.h, k.h, k.nh);
    x[13] = pcrot<INV>(x[13], k.s1, k.c1, k.nc1);
    x[6] = pcrot<INV>(x[6], k.h, k.h, k.nh);
    x[14] = pcrot<INV>(x[14], k.nh, k.h, k.nh);
    x[7] = pcrot<INV>(x[7], k.s1, k.c1, k.nc1);
    x[11] = pcrot<INV>(x[11], k.nh, k.h, k.nh);
    x[15] = pcrot<INV>(x[15], k.nc1, k.ns1, k.s1);
    P2 y[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        P2 a0 = x[4 * k1], a1 = x[4 * k1 + 1], a2 = x[4 * k1 + 2], a3 = x[4 * k1 + 3];
        if (k1 == 2) pdft4_rot2<INV>(a0, a1, a2, a3);
        else pdft4<INV>(a0, a1, a2, a3);
        y[k1] = a0;
        y[k1 + 4] = a1;
        y[k1 + 8] = a2;
        y[k1 + 12] = a3;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = y[i];
}

template <bool INV> __device__ __forceinline__ void pdft16(P2 *x, const RotConsts &k)
{
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) pdft4<INV>(x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]);
    pdft16_layer2<INV>(x, k);
}

// inputs x[8..15] zero
template <bool INV> __device__ __forceinline__ void pdft16_half(P2 *x, const RotConsts &k)
{
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) {
        const P2 a = x[n1], b = x[n1 + 4];
        x[n1] = padd(a, b);
        x[n1 + 8] = psub(a, b);
        x[n1 + 4] = paddrot<INV>(a, b);
        x[n1 + 12] = psubrot<INV>(a, b);
    }
    pdft16_layer2<INV>(x, k);
}

// cos and sin of 2 pi m / 32, m = 0..7
__device__ __forceinline__ float c32(int m)
{
    const float c[8] = {1.0f, 0.98078528040323044913f, 0.92387953251128675613f, 0.83146961230254523708f,
                        0.70710678118654752440f, 0.55557023301960222474f, 0.38268343236508977173f,
                        0.19509032201612826785f};
    return c[m];
}

// X[k] = E[k] + w32^k O[k], X[k+16] = E[k] - w32^k O[k] for the pair
// (E[k], O[k]) in x[k]: the second lane's twiddle, then the butterfly across
// the lanes, in scalar operations; the result is the pair (X[k], X[k+16]).
template <bool INV> __device__ __forceinline__ void combine32(P2 *x)
{
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const float er = x[k].r.x, ei = x[k].i.x;
        float orr = x[k].r.y, oi = x[k].i.y;
        if (k == 8) {
            // w32^8 = rot: X[8] = E + rot(O), X[24] = E - rot(O)
            const float rr = INV ? -oi : oi, ri = INV ? orr : -orr;
            x[k].r = make_float2(er + rr, er - rr);
            x[k].i = make_float2(ei + ri, ei - ri);
            continue;
        }
        if (k != 0) {
            // w32^k = (c, -s) forward; k > 8 folds the rotation into the constants
            const float c = k < 8 ? c32(k) : -c32(16 - k), s = k < 8 ? c32(8 - k) : c32(k - 8);
            const float tr = INV ? orr * c - oi * s : orr * c + oi * s;
            const float ti = INV ? orr * s + oi * c : oi * c - orr * s;
            orr = tr;
            oi = ti;
        }
        x[k].r = make_float2(er + orr, er - orr);
        x[k].i = make_float2(ei + oi, ei - oi);
    }
}

// 32-point DFT: x[i] = (v[2i], v[2i+1]) in, x[k] = (V[k], V[k+16]) out.
template <bool INV> __device__ __forceinline__ void pdft32(P2 *x, const RotConsts &k)
{
    pdft16<INV>(x, k);
    combine32<INV>(x);
}

// the same with v[16..31] zero (x[8..15] unused)
template <bool INV> __device__ __forceinline__ void pdft32_half(P2 *x, const RotConsts &k)
{
    pdft16_half<INV>(x, k);
    combine32<INV>(x);
}

// Inverse of the split: from x[k] = (V[k], V[k+16]) (the spectrum), the pairs
// (V[k] + V[k+16], (V[k] - V[k+16]) w32^{-+k}), then both 16-point inverse
// DFTs at once: x[i] = (v[2i], v[2i+1]) of the 32-point DFT with the sign of
// INV (INV = true: the unnormalised inverse of pdft32<false>).
template <bool INV> __device__ __forceinline__ void pdft32_from_halves(P2 *x, const RotConsts &rk)
{
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const float ar = x[k].r.x, ai = x[k].i.x, br = x[k].r.y, bi = x[k].i.y;
        const float er = ar + br, ei = ai + bi;
        float dr = ar - br, di = ai - bi;
        if (k == 8) {
            const float rr = INV ? -di : di, ri = INV ? dr : -dr;
            dr = rr;
            di = ri;
        } else if (k != 0) {
            const float c = k < 8 ? c32(k) : -c32(16 - k), s = k < 8 ? c32(8 - k) : c32(k - 8);
            const float tr = INV ? dr * c - di * s : dr * c + di * s;
            const float ti = INV ? dr * s + di * c : di * c - dr * s;
            dr = tr;
            di = ti;
        }
        x[k].r = make_float2(er, dr);
        x[k].i = make_float2(ei, di);
    }
    pdft16<INV>(x, rk);
}

// ---- The line buffer of a 1024-point transform in two radix-32 stages ----
//
// Stage 0 of lane t turns x[t + 32 m] (m < 32) into Y_t[k], k < 32, stored
// at position 32 t + k; stage 1 of lane t reads Y_m[t] (position 32 m + t),
// twiddles it by W1024^(m t) and gives X[t + 32 k]. The line holds records
// of two positions p and p + 32 (p mod 64 < 32): stage 1 reads whole records
// (its pair (Y_2i[t], Y_2i+1[t]) is positions t + 64 i and t + 64 i + 32,
// record t + 32 i), stage 0 writes half records (its pair (Y_t[k],
// Y_t[k+16]) goes to positions 32 t + k and 32 t + k + 16, whose partners
// belong to lane t ^ 1). The adjoint runs the same accesses the other way.
//
// Record q = 32 j + (p mod 32) of group j = p / 64 sits at float 4 (q + j / 2)
// and holds {re p, re p+32, im p, im p+32} for even j, {im p, im p+32, re p,
// re p+32} for odd j. A half-record access of lane t = 2 j' + h (fixed k)
// then lands on bank 4 k + 4 (j' / 2) + 2 (j' & 1) + h (+ 2, mod 4, for the
// other part): 32 different banks. Whole-record accesses are 32 consecutive
// records: conflict-free for any skew.
constexpr int LINE_RECORDS = 512 + 8;  // records of a line, skew included

__device__ __forceinline__ int line_rec(int q) { return q + (q >> 6); }

// Stage-0 outputs (V[k], V[k+16]) of lane t into the line.
__device__ __forceinline__ void line_write_halves(float *line, int t, const P2 (&v)[16])
{
    const int j = t >> 1, h = t & 1, q0 = 32 * j;
    const int ore = 2 * (j & 1) + h, oim = ore ^ 2;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        float *ra = line + 4 * line_rec(q0 + k), *rb = line + 4 * line_rec(q0 + k + 16);
        ra[ore] = v[k].r.x;
        ra[oim] = v[k].i.x;
        rb[ore] = v[k].r.y;
        rb[oim] = v[k].i.y;
    }
}

// The adjoint: pairs (V[k], V[k+16]) of lane t from the line.
__device__ __forceinline__ void line_read_halves(const float *line, int t, P2 (&v)[16])
{
    const int j = t >> 1, h = t & 1, q0 = 32 * j;
    const int ore = 2 * (j & 1) + h, oim = ore ^ 2;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const float *ra = line + 4 * line_rec(q0 + k), *rb = line + 4 * line_rec(q0 + k + 16);
        v[k].r = make_float2(ra[ore], rb[ore]);
        v[k].i = make_float2(ra[oim], rb[oim]);
    }
}

// Stage-1 inputs of lane t: pair i = whole record t + 32 i (group i).
__device__ __forceinline__ void line_read_records(const float *line, int t, P2 (&v)[16])
{
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const float4 q = *reinterpret_cast<const float4 *>(line + 4 * line_rec(t + 32 * i));
        const float2 lo = make_float2(q.x, q.y), hi = make_float2(q.z, q.w);
        v[i].r = (i & 1) ? hi : lo;
        v[i].i = (i & 1) ? lo : hi;
    }
}

__device__ __forceinline__ void line_write_records(float *line, int t, const P2 (&v)[16])
{
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const float2 lo = (i & 1) ? v[i].i : v[i].r, hi = (i & 1) ? v[i].r : v[i].i;
        *reinterpret_cast<float4 *>(line + 4 * line_rec(t + 32 * i)) = make_float4(lo.x, lo.y, hi.x, hi.y);
    }
}

// Stage-1 twiddles of lane t, W1024^(t m) for m = 2 i, 2 i + 1 (forward) or
// their conjugates, from tw[32 i + t] = {re m=2i, re m=2i+1, im m=2i, im m=2i+1}
// (lane-fast, so the 32 lanes read consecutive entries).
template <bool INV> __device__ __forceinline__ void line_twiddle(P2 (&v)[16], const float4 *tw, int t)
{
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const float4 w = tw[32 * i + t];
        v[i] = ptwiddle<INV>(v[i], make_float2(w.x, w.y), make_float2(w.z, w.w));
    }
}

}  // namespace pk
}  // namespace ps
