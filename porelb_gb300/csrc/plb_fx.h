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
 * a_j = 3 (1 - w/2) F (e_jx - u), written with rho = 1 + delta and
 * j = rho u (J_x including the half-force shift of porelb.c:347-348) as
 *
 *   f'_j = f_j - w (f_j - w_j) + G_j
 *   G_j  = w_j [ w delta + c (e_jx rho - J_x)
 *                + (w + c e_jx - c u_x) (3 e_j.J + 4.5 (e_j.J)(e_j.u) - 1.5 J.u) ]
 *
 * with c = 3 (1 - w/2) F, u = J/rho and w_j the lattice weights.  Every
 * term is exact algebra of the reference's expression.
 *
 * Range: collide<false> requires f_0 in [2^-8, 1) and f_j in [2^-8, 1/4)
 * for j > 0, rho in [0.5, 1.2], and results in [2^-8, 8); collide<true>
 * (constant shifts) requires every f_j, in and out, to stay in the binade of
 * its weight: f_0 in [1/4, 1/2), f_1..6 in [1/32, 1/16), f_7..18 in
 * [1/64, 1/32), i.e. deviations within -25%..+50% and -43%..+12.5% of the
 * weights.  A node outside the range is flagged and the caller recomputes it
 * in native FP64.
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
    s.h = (int32_t)(a >> 30);
    s.l = (int32_t)((uint32_t)a & 0x3fffffffu);
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

FX_HD uint32_t clz32(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return (uint32_t)__clz((int)x);
#else
    return x ? (uint32_t)__builtin_clz(x) : 32u;
#endif
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

/* Exact Q60 value of a positive FP64 number given as bits.  The shift
 * s = (biased exponent - 1015) must lie in [0, smax] for f in [2^-8,
 * 2^(smax-7)); the caller checks the running maximum of s (a sign bit, zero,
 * NaN or a value out of range gives a large s). */
FX_HD int64_t from_bits(uint64_t b, uint32_t &smax_seen)
{
    const uint32_t hi = (uint32_t)(b >> 32);
    const uint32_t lo = (uint32_t)b;
    const uint32_t s = (hi >> 20) - 1015u;
    smax_seen = smax_seen > s ? smax_seen : s;
    const uint32_t mh = (hi & 0xfffffu) | 0x100000u;
    const uint32_t sh = s & 15u;
#if defined(__CUDA_ARCH__)
    const uint32_t oh = __funnelshift_l(lo, mh, sh);
    const uint32_t ol = lo << sh;
    return (int64_t)(((uint64_t)oh << 32) | ol);
#else
    return (int64_t)((((uint64_t)mh << 32) | lo) << sh);
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

/* Fixed-binade forms: the value's biased FP64 exponent is E, the exponent
 * of its lattice weight (1/3 -> 1021, 1/18 -> 1018, 1/36 -> 1017), so every
 * shift is a constant.  A value outside that binade (input or result) sets a
 * bit at or above bit 20 of *bad (sign and exponent field XOR their expected
 * value; one three-input logic operation per value) and the whole node is
 * recomputed by the caller; bits 0..19 of *bad carry mantissa bits and mean
 * nothing. */
template <uint32_t E>
FX_HD int64_t from_bits_fixed(uint64_t b, uint32_t &bad)
{
    bad |= (uint32_t)(b >> 32) ^ (E << 20);
    const uint64_t m = (b & 0xfffffffffffffull) | 0x10000000000000ull;
    return (int64_t)(m << (E - 1015u));
}

template <uint32_t E>
FX_HD uint64_t to_bits_fixed(int64_t F, uint32_t &bad)
{
    constexpr uint32_t r = E - 1015u; /* bits below the 53-bit mantissa */
    const uint64_t u = (uint64_t)F;
    const uint64_t q = (u + ((uint64_t)1 << r >> 1)) >> r; /* [2^52, 2^53) if in range */
    bad |= (uint32_t)(q >> 32) ^ (1u << 20);
    return ((uint64_t)(E - 1u) << 52) + q;
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
    int64_t tp[3];      /* weights 1/3, 1/18, 1/36 as the reference's doubles */
    int64_t om;         /* omega */
    int64_t cf;         /* c = 3 (1 - omega/2) F */
    int64_t half_force; /* 0.5 F */
    int64_t rho_hi;     /* density guard bounds 1.2 and 0.5 */
    int64_t rho_lo;
};

/* Host: constants from the FP64 parameters.  omega = 1/tau and the weights
 * are the reference's doubles (porelb.c:88, porelb.h:36-42); each is an exact
 * multiple of 2^-60, so their Q60 images are exact. */
static inline Consts make_consts(double tau, double force)
{
    Consts k;
    const double w[3] = {1.0 / 3, 1.0 / 18, 1.0 / 36};
    for (int c = 0; c < 3; c++) k.tp[c] = (int64_t)ldexp(w[c], 60);
    const double omega = 1.0 / tau;
    k.om = (int64_t)llround(ldexp(omega, 60));
    k.cf = (int64_t)llround(ldexp((1.0 - 0.5 * omega) * 3.0 * force, 60));
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
template <bool FIXED>
FX_HD uint32_t collide(uint64_t (&bits)[19], const Consts &k, bool it_pos,
                       Moments &mom)
{
    uint32_t s0 = 0, s12 = 0, rmax = 0, fbad = 0;
    int64_t F[19];
    if (FIXED) {
        F[0] = from_bits_fixed<1021u>(bits[0], fbad);
#pragma unroll
        for (int j = 1; j < 19; j++)
            F[j] = j <= 6 ? from_bits_fixed<1018u>(bits[j], fbad)
                          : from_bits_fixed<1017u>(bits[j], fbad);
    } else {
        F[0] = from_bits(bits[0], s0);
#pragma unroll
        for (int j = 1; j < 19; j++) F[j] = from_bits(bits[j], s12);
    }

    /* exact moments: rho and J from pair sums / differences */
    int64_t R = F[0], Jx = 0, Jy = 0, Jz = 0;
#pragma unroll
    for (int J = 1; J < 19; J += 2) {
        const int64_t s = F[J] + F[J + 1];
        const int64_t d = F[J] - F[J + 1];
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
    const Sp oms = split(k.om), cfs = split(k.cf);
    const int64_t cux = mul(cfs, uxs);
    const int64_t A0 = k.om - cux, Ap = A0 + k.cf, Am = A0 - k.cf;
    const int64_t cJx = mul(cfs, Jxs), cR = mul(cfs, Rs);
    const int64_t B0 = mul(oms, split(R - kOne)) - cJx, Bp = B0 + cR, Bm = B0 - cR;
    /* W = w_c * (w delta + c (e_x rho - J_x)),  T = w_c * A(e_x).  The
     * reference's 1/36 is exactly half its 1/18, and its 1/3 is 6 * 1/18 to
     * within 2^-54, so only the 1/18 products are formed. */
    const Sp t1 = split(k.tp[1]);
    const int64_t W10 = mul(t1, split(B0)), W1p = mul(t1, split(Bp)), W1m = mul(t1, split(Bm));
    const int64_t W20 = W10 >> 1, W2p = W1p >> 1, W2m = W1m >> 1;
    const int64_t W00 = W10 * 6;
    const int64_t T10v = mul(t1, split(A0)), T1pv = mul(t1, split(Ap)), T1mv = mul(t1, split(Am));
    const Sp T10 = split(T10v), T1p = split(T1pv), T1m = split(T1mv);
    const Sp T20 = split(T10v >> 1), T2p = split(T1pv >> 1), T2m = split(T1mv >> 1);
    const Sp T00 = split(T10v * 6);

    /* rest direction: e.J = 0 */
    {
        const int64_t qd = -Ju15;
        const int64_t G = W00 + mul(T00, split(qd));
        const int64_t Fn = F[0] - mul(oms, split(F[0] - k.tp[0])) + G;
        bits[0] = FIXED ? to_bits_fixed<1021u>(Fn, fbad) : to_bits(Fn, rmax);
    }
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
        const int64_t tpc = c == 1 ? k.tp[1] : k.tp[2];
        const int eJ = fex(J), eK = fex(K);
        const int64_t WJ = c == 1 ? (eJ > 0 ? W1p : eJ < 0 ? W1m : W10)
                                  : (eJ > 0 ? W2p : eJ < 0 ? W2m : W20);
        const int64_t WK = c == 1 ? (eK > 0 ? W1p : eK < 0 ? W1m : W10)
                                  : (eK > 0 ? W2p : eK < 0 ? W2m : W20);
        const Sp TJ = c == 1 ? (eJ > 0 ? T1p : eJ < 0 ? T1m : T10)
                             : (eJ > 0 ? T2p : eJ < 0 ? T2m : T20);
        const Sp TK = c == 1 ? (eK > 0 ? T1p : eK < 0 ? T1m : T10)
                             : (eK > 0 ? T2p : eK < 0 ? T2m : T20);
        const int64_t GJ = WJ + mul(TJ, split(qd + t3));
        const int64_t GK = WK + mul(TK, split(qd - t3));
        const int64_t FnJ = F[J] - mul(oms, split(F[J] - tpc)) + GJ;
        const int64_t FnK = F[K] - mul(oms, split(F[K] - tpc)) + GK;
        if (FIXED) {
            if (c == 1) {
                bits[J] = to_bits_fixed<1018u>(FnJ, fbad);
                bits[K] = to_bits_fixed<1018u>(FnK, fbad);
            } else {
                bits[J] = to_bits_fixed<1017u>(FnJ, fbad);
                bits[K] = to_bits_fixed<1017u>(FnK, fbad);
            }
        } else {
            bits[J] = to_bits(FnJ, rmax);
            bits[K] = to_bits(FnK, rmax);
        }
    }
    const bool bad = (s0 > 7u) | (s12 > 5u) | (rmax > 10u) | ((fbad >> 20) != 0u);
    return flags | (bad ? kBad : 0u);
}

}  // namespace fx
}  // namespace plb

#endif
