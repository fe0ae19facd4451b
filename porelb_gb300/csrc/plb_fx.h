/*
 * plb_fx.h - FP64-accurate BGK collision on the integer pipes.
 *
 * GB300 issues about 2 FP64 operations per clock per SM, so an FP64
 * collision (~150 FP64 instructions per node) caps the step near 20% of the
 * HBM roofline.  This file restates the collision of porelb.c:318-365 in
 * Q60 fixed point (int64 holding value * 2^60): the distributions are
 * converted exactly from their FP64 bits, the moments are exact integer
 * sums, products are 64x64 -> (128 >> 60) built from three 32-bit wide
 * multiply-adds (error <= 1 * 2^-60 each, zero mean), and the results are
 * rounded back to FP64.  Against the reference's FP64 arithmetic the
 * per-step difference is a fraction of an FP64 ulp of the weights, the same
 * order as the reference's own rounding.
 *
 * The update is the reference's f' = (1-w) f + (w + a_j) feq_j with
 * a_j = 3 (1 - w/2) F (e_jx - u), written with rho = 1 + delta, j = rho u
 * (J_x including the half-force shift of porelb.c:347-348) and the
 * deviations D_j = f_j - w_j as
 *
 *   f'_j = (1 - w) D_j + w_j + W_j + T_j q_j
 *   W_j  = w_j [ w delta + c (e_jx rho - J_x) ]
 *   T_j  = w_j (w + c e_jx - c u_x)
 *   q_j  = 3 e_j.J + 4.5 (e_j.J)(e_j.u) - 1.5 J.u
 *
 * with c = 3 (1 - w/2) F, u = J/rho and w_j the lattice weights.  Every
 * term is exact algebra of the reference's expression; rho = sum_j D_j +
 * sum_j w_j and J = sum_j e_j D_j (the weights of opposite directions are
 * equal).
 *
 * Range: every f_j, in and out, must stay in the binade of its weight:
 * f_0 in [1/4, 1/2), f_1..6 in [1/32, 1/16), f_7..18 in [1/64, 1/32), i.e.
 * deviations within -25%..+50% and -43%..+12.5% of the weights, so that
 * D_j is the difference of the FP64 bit patterns shifted by a constant and
 * every conversion is a constant shift.  A node outside the range is
 * flagged and the caller recomputes it in native FP64.
 *
 * The functions are host+device so that a CPU build of the same code checks
 * the integer algorithm bit for bit against the GPU.
 */
#ifndef PLB_FX_H_
#define PLB_FX_H_

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define FX_HD __host__ __device__ __forceinline__
#else
#define FX_HD static inline
#endif

namespace plb {
namespace fx {

constexpr int64_t kOne = (int64_t)1 << 60;

/* a = h * 2^30 + l with 0 <= l < 2^30 (|h| < 2^31 for |a| < 2^61) */
struct Sp {
    int32_t h;
    int32_t l;
};

FX_HD Sp split(int64_t a)
{
    Sp s;
#if defined(__CUDA_ARCH__)
    /* t = bits 30-31 of the low word; h = 4 hi + t and l = lo - t 2^30 as
     * two integer multiply-adds: the GPU's ALU pipe is the busier one in
     * the collision, the multiply-add pipe has room (and the compiler's own
     * form of the 64-bit shift and mask costs more instructions). */
    const uint32_t lo = (uint32_t)a, hi = (uint32_t)((uint64_t)a >> 32);
    const uint32_t t = lo >> 30;
    int32_t h, l;
    asm("mad.lo.s32 %0, %1, 4, %2;" : "=r"(h) : "r"(hi), "r"(t));
    asm("mad.lo.s32 %0, %1, -1073741824, %2;" : "=r"(l) : "r"(t), "r"(lo));
    s.h = h;
    s.l = l;
#else
    s.h = (int32_t)(a >> 30);
    s.l = (int32_t)((uint32_t)a & 0x3fffffffu);
#endif
    return s;
}

FX_HD int64_t wmul(int32_t a, int32_t b) { return (int64_t)a * (int64_t)b; }

/* a * b / 2^60 for |a|, |b| < 2^61 (values of magnitude < 2), from three
 * 32x32 -> 64 multiply-adds:
 *   a*b / 2^60 = ah bh + (ah bl + al bh) / 2^30 + al bl / 2^60.
 * The last term (in [0, 1)) is replaced by its mean 1/4 and the middle one
 * rounded to nearest, which is the constant 3*2^28 added before the shift:
 * |error| <= 1 unit of 2^-60, zero on average. */
FX_HD int64_t mul(Sp a, Sp b)
{
    const int64_t mid = wmul(a.h, b.l) + wmul(a.l, b.h) + ((int64_t)3 << 28);
    return wmul(a.h, b.h) + (mid >> 30);
}

FX_HD int64_t mul(int64_t a, int64_t b) { return mul(split(a), split(b)); }

/* a * b + c * d (all Q60, magnitudes < 2) with one shared shift: the four
 * middle products are summed before the shift (|sum| < 2^63), and the
 * constant 2^30 is the rounding half plus the means (1/4 each) of the two
 * dropped low x low terms.  |error| <= 1 unit of 2^-60. */
FX_HD int64_t mul2(Sp a, Sp b, Sp c, Sp d)
{
    const int64_t mid = wmul(a.h, b.l) + wmul(a.l, b.h) + wmul(c.h, d.l) + wmul(c.l, d.h) +
                        ((int64_t)1 << 30);
    return wmul(a.h, b.h) + wmul(c.h, d.h) + (mid >> 30);
}

FX_HD uint32_t f2u(float x)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

/* floor(log2(x)) + 127 for x >= 1 (the biased exponent of x as a float
 * rounded toward zero); 0 for x == 0. */
FX_HD uint32_t log2_biased(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(__uint2float_rz(x)) >> 23;
#else
    return x ? 158u - (uint32_t)__builtin_clz(x) : 0u;
#endif
}

/* FP64 bits of a Q60 value F in [2^52, 2^63) (value in [2^-8, 8)), rounded
 * to nearest (ties up).  r = bits dropped; the caller checks the running
 * maximum of r against 10 (values outside the range give r > 10). */
FX_HD uint64_t to_bits(int64_t F, uint32_t &rmax_seen)
{
    const uint64_t u = (uint64_t)F;
    const uint32_t ef = log2_biased((uint32_t)(u >> 32));
    const uint32_t r = ef - 147u; /* bit length - 53 */
    rmax_seen = rmax_seen > r ? rmax_seen : r;
    const uint32_t rr = r & 15u;
    const uint64_t q = (u + ((1u << rr) >> 1)) >> rr; /* [2^52, 2^53] */
    return ((uint64_t)(ef + 867u) << 52) + q;
}

/* The weight classes: 1/3 (rest), 1/18 (axes), 1/36 (diagonals) as the
 * reference's doubles (porelb.h:36-42).  kE: biased FP64 exponent of the
 * weight; kS = kE - 1015: the shift from mantissa units to Q60; kWBits: the
 * FP64 bits; kW: the exact Q60 value. */
FX_HD constexpr uint32_t kE(int c) { return c == 0 ? 1021u : (c == 1 ? 1018u : 1017u); }
FX_HD constexpr uint32_t kS(int c) { return kE(c) - 1015u; }
FX_HD constexpr uint64_t kWBits(int c)
{
    return c == 0 ? 0x3fd5555555555555ull : (c == 1 ? 0x3fac71c71c71c71cull : 0x3f9c71c71c71c71cull);
}
FX_HD constexpr int64_t kW(int c)
{
    return (int64_t)(((kWBits(c) & 0xfffffffffffffull) | 0x10000000000000ull) << kS(c));
}
/* sum of the 19 weights in Q60 (2^60 - 64: the doubles sum to just below 1) */
constexpr int64_t kWSum = kW(0) + 6 * kW(1) + 12 * kW(2);

/* D = f - w_c in Q60, exactly, from the FP64 bits of f: inside the weight's
 * binade the exponent fields cancel.  A value outside it (or negative) sets
 * a bit at or above bit 20 of *chk (sign and exponent field XOR their
 * expected value: one three-input logic operation); bits 0..19 of *chk
 * carry mantissa bits and mean nothing. */
template <int C>
FX_HD int64_t dev_bits(uint64_t b, uint32_t &chk)
{
    chk |= (uint32_t)(b >> 32) ^ (kE(C) << 20);
    return (int64_t)((b - kWBits(C)) << kS(C));
}

/* FP64 bits of a class-C result whose Q60 value F already includes half a
 * unit of the dropped bits (so the shift rounds to nearest, ties up).  A
 * result outside the weight's binade sets a bit at or above bit 20 of
 * *chk. */
template <int C>
FX_HD uint64_t out_bits(int64_t F, uint32_t &chk)
{
    const uint64_t q = (uint64_t)F >> kS(C); /* [2^52, 2^53) if in range */
    chk |= (uint32_t)(q >> 32) ^ (1u << 20);
    return ((uint64_t)(kE(C) - 1u) << 52) + q;
}

/* Q60 of a positive normal float in [2^-8, 4) */
FX_HD int64_t from_float(float x)
{
    const uint32_t b = f2u(x);
    const uint32_t sh = ((b >> 23) - 127u + 37u) & 63u;
    const uint64_t m = (uint64_t)((b & 0x7fffffu) | 0x800000u);
    return (int64_t)(m << sh);
}

/* Per-run constants (host-computed from the FP64 parameters). */
struct Consts {
    Sp om1;             /* 1 - omega */
    Sp kw;              /* w_1 omega (w_1 = 1/18) */
    Sp kc;              /* w_1 c, c = 3 (1 - omega/2) F */
    int64_t kwv, kcv;   /* the same two, unsplit */
    int64_t wout[3];    /* per class: w_c + half a unit of the bits dropped */
    int64_t half_force; /* 0.5 F */
    int64_t rho_hi;     /* density guard bounds 1.2 and 0.5 */
    int64_t rho_lo;
};

/* Host: constants from the FP64 parameters.  omega = 1/tau and the weights
 * are the reference's doubles (porelb.c:88, porelb.h:36-42). */
static inline Consts make_consts(double tau, double force)
{
    Consts k;
    const double omega = 1.0 / tau;
    const int64_t om = (int64_t)llround(ldexp(omega, 60));
    const int64_t cf = (int64_t)llround(ldexp((1.0 - 0.5 * omega) * 3.0 * force, 60));
    k.om1 = split(kOne - om);
    k.kwv = mul(kW(1), om);
    k.kcv = mul(kW(1), cf);
    k.kw = split(k.kwv);
    k.kc = split(k.kcv);
    for (int c = 0; c < 3; c++) k.wout[c] = kW(c) + ((int64_t)1 << (kS(c) - 1));
    k.half_force = (int64_t)llround(ldexp(0.5 * force, 60));
    k.rho_hi = (int64_t)llround(ldexp(1.2, 60));
    k.rho_lo = (int64_t)llround(ldexp(0.5, 60));
    return k;
}

/* Result flags */
enum { kBad = 1u, kDensity = 2u };

struct Moments {
    int64_t R, Jx, Jy, Jz, inv;
};

/* D3Q19 table helpers (reference order, porelb.h:10-50) */
FX_HD constexpr int fex(int j)
{
    return (j == 1 || j == 12 || j == 14 || j == 16 || j == 18) ? 1
         : (j == 2 || j == 11 || j == 13 || j == 15 || j == 17) ? -1 : 0;
}
FX_HD constexpr int fey(int j)
{
    return (j == 3 || j == 7 || j == 10 || j == 15 || j == 18) ? 1
         : (j == 4 || j == 8 || j == 9 || j == 16 || j == 17) ? -1 : 0;
}
FX_HD constexpr int fez(int j)
{
    return (j == 5 || j == 7 || j == 9 || j == 12 || j == 13) ? 1
         : (j == 6 || j == 8 || j == 10 || j == 11 || j == 14) ? -1 : 0;
}
FX_HD constexpr int fcls(int j) { return j == 0 ? 0 : (j <= 6 ? 1 : 2); }

FX_HD float rcp_rn(float x)
{
#if defined(__CUDA_ARCH__)
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}

/*
 * One collision.  bits[19]: post-stream FP64 values (in), post-collision
 * FP64 values (out).  Returns kBad if the node must be recomputed in native
 * FP64, kDensity if the density guard trips.  mom receives rho*2^60, the
 * shifted momentum and 1/rho for the macro output.
 */
FX_HD uint32_t collide(uint64_t (&bits)[19], const Consts &k, bool it_pos,
                       Moments &mom)
{
    uint32_t chk = 0;
    int64_t D[19];
    D[0] = dev_bits<0>(bits[0], chk);
#pragma unroll
    for (int j = 1; j < 19; j++)
        D[j] = j <= 6 ? dev_bits<1>(bits[j], chk) : dev_bits<2>(bits[j], chk);

    /* exact moments: rho and J from pair sums / differences */
    int64_t R = D[0] + kWSum, Jx = 0, Jy = 0, Jz = 0;
#pragma unroll
    for (int J = 1; J < 19; J += 2) {
        const int64_t s = D[J] + D[J + 1];
        const int64_t d = D[J] - D[J + 1];
        R += s;
        if (fex(J) > 0) Jx += d; else if (fex(J) < 0) Jx -= d;
        if (fey(J) > 0) Jy += d; else if (fey(J) < 0) Jy -= d;
        if (fez(J) > 0) Jz += d; else if (fez(J) < 0) Jz -= d;
    }
    uint32_t flags = 0;
    if (R > k.rho_hi || R < k.rho_lo) flags |= kDensity;
    if (it_pos) Jx += k.half_force;

    /* 1/rho: FP32 reciprocal refined by one Newton step in Q60 */
    const Sp Rs = split(R);
    const float rf = (float)(int32_t)(R >> 30) * 9.313225746154785e-10f; /* 2^-30 */
    const float r0 = rcp_rn(rf > 0.25f ? rf : 0.25f);
    const Sp R0 = split(from_float(r0));
    const int64_t E = 2 * kOne - mul(Rs, R0);
    const int64_t INV = mul(R0, split(E));
    const Sp INVs = split(INV);
    mom.R = R;
    mom.Jx = Jx;
    mom.Jy = Jy;
    mom.Jz = Jz;
    mom.inv = INV;

    /* u = J / rho.  (e.J)^2 / rho = sum_ab e_a e_b J_a u_b, and J_a u_b =
     * rho u_a u_b = J_b u_a, so the quadratic terms of all 18 directions
     * come from six products: the diagonal P_aa (whose sum is J.J / rho) and
     * the off-diagonal P_xy, P_xz, P_yz counted twice. */
    const Sp Jxs = split(Jx), Jys = split(Jy), Jzs = split(Jz);
    const int64_t ux = mul(Jxs, INVs), uy = mul(Jys, INVs), uz = mul(Jzs, INVs);
    const Sp uxs = split(ux), uys = split(uy), uzs = split(uz);
    const int64_t Pxx = mul(Jxs, uxs), Pyy = mul(Jys, uys), Pzz = mul(Jzs, uzs);
    const int64_t Pxy2 = mul(Jxs, uys) * 2, Pxz2 = mul(Jxs, uzs) * 2,
                  Pyz2 = mul(Jys, uzs) * 2;
    const int64_t Ju = Pxx + Pyy + Pzz;
    const int64_t Ju15 = Ju + (Ju >> 1);

    /* T = w_c (w + c e_x - c u_x) and W = w_c (w delta + c (e_x rho - J_x))
     * for the 1/18 class from the per-run products w_1 w and w_1 c; the
     * reference's 1/36 is exactly half its 1/18, and its 1/3 is 6 * 1/18 to
     * within 2^-54.  Each W also carries the class's weight and rounding
     * half (wout), so a result is one shift away from its FP64 bits. */
    const int64_t T10v = k.kwv - mul(k.kc, uxs);
    const int64_t T1pv = T10v + k.kcv, T1mv = T10v - k.kcv;
    const Sp T10 = split(T10v), T1p = split(T1pv), T1m = split(T1mv);
    const Sp T20 = split(T10v >> 1), T2p = split(T1pv >> 1), T2m = split(T1mv >> 1);
    const Sp T00 = split(T10v * 6);
    const int64_t Wv = mul(k.kw, split(R - kOne)) - mul(k.kc, Jxs);
    const int64_t KR = mul(k.kc, Rs);
    const int64_t W10 = Wv + k.wout[1], W1p = Wv + KR + k.wout[1], W1m = Wv - KR + k.wout[1];
    const int64_t W20 = (Wv >> 1) + k.wout[2], W2p = ((Wv + KR) >> 1) + k.wout[2],
                  W2m = ((Wv - KR) >> 1) + k.wout[2];
    const int64_t W00 = Wv * 6 + k.wout[0];

    /* rest direction: e.J = 0 */
    bits[0] = out_bits<0>(mul2(k.om1, split(D[0]), T00, split(-Ju15)) + W00, chk);
#pragma unroll
    for (int J = 1; J < 19; J += 2) {
        const int K = J + 1;
        int64_t ej = 0, e2 = 0; /* e.J and (e.J)^2 / rho */
        if (fex(J) > 0) ej += Jx; else if (fex(J) < 0) ej -= Jx;
        if (fey(J) > 0) ej += Jy; else if (fey(J) < 0) ej -= Jy;
        if (fez(J) > 0) ej += Jz; else if (fez(J) < 0) ej -= Jz;
        if (fex(J) != 0) e2 += Pxx;
        if (fey(J) != 0) e2 += Pyy;
        if (fez(J) != 0) e2 += Pzz;
        if (fex(J) * fey(J) > 0) e2 += Pxy2; else if (fex(J) * fey(J) < 0) e2 -= Pxy2;
        if (fex(J) * fez(J) > 0) e2 += Pxz2; else if (fex(J) * fez(J) < 0) e2 -= Pxz2;
        if (fey(J) * fez(J) > 0) e2 += Pyz2; else if (fey(J) * fez(J) < 0) e2 -= Pyz2;
        const int64_t qd = e2 * 4 + (e2 >> 1) - Ju15; /* (4.5 (e.J)^2 - 1.5 J.J)/rho */
        const int64_t t3 = ej * 3;
        const int c = fcls(J);
        const int eJ = fex(J), eK = fex(K);
        const int64_t WJ = c == 1 ? (eJ > 0 ? W1p : eJ < 0 ? W1m : W10)
                                  : (eJ > 0 ? W2p : eJ < 0 ? W2m : W20);
        const int64_t WK = c == 1 ? (eK > 0 ? W1p : eK < 0 ? W1m : W10)
                                  : (eK > 0 ? W2p : eK < 0 ? W2m : W20);
        const Sp TJ = c == 1 ? (eJ > 0 ? T1p : eJ < 0 ? T1m : T10)
                             : (eJ > 0 ? T2p : eJ < 0 ? T2m : T20);
        const Sp TK = c == 1 ? (eK > 0 ? T1p : eK < 0 ? T1m : T10)
                             : (eK > 0 ? T2p : eK < 0 ? T2m : T20);
        const int64_t FnJ = mul2(k.om1, split(D[J]), TJ, split(qd + t3)) + WJ;
        const int64_t FnK = mul2(k.om1, split(D[K]), TK, split(qd - t3)) + WK;
        if (c == 1) {
            bits[J] = out_bits<1>(FnJ, chk);
            bits[K] = out_bits<1>(FnK, chk);
        } else {
            bits[J] = out_bits<2>(FnJ, chk);
            bits[K] = out_bits<2>(FnK, chk);
        }
    }
    return flags | ((chk >> 20) != 0u ? kBad : 0u);
}

}  // namespace fx
}  // namespace plb

#endif
