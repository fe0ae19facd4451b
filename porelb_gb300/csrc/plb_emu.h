/*
 * plb_emu.h - IEEE-754 double multiply, round to nearest even, on the
 * integer pipes.
 *
 * The bit-exact FP64 collision spends its time on GB300's FP64 pipe (about
 * 2 operations per clock per SM).  Part of its multiplies run here instead,
 * on the integer multiply-add pipe, and return the same bits as the FP64
 * pipe: the 106-bit product of the two 53-bit significands is formed
 * exactly and rounded once, to nearest, ties to even.  (An add done the same
 * way cost the integer pipes more than it saved the FP64 pipe.)
 *
 * Domain of the integer path: finite normal operands whose product is a
 * normal number, or a zero times a finite operand (a zero of the product's
 * sign).  The collision's values (distributions, densities, velocities,
 * their squares and the run constants) lie in it whenever the node's
 * values and density and the run constants are zero or of magnitude in
 * [2^-64, 2^64) (outside_node_range): then every product of the collision
 * lies in [2^-944, 2^602].  The collision checks that once per node and
 * multiplies with dmul_bits_fast, which checks nothing; a node outside the
 * range is computed with the native multiply, so the bits are the IEEE
 * product's everywhere and a diverging run carries its infinities and
 * NaNs forward.  A check in every product cost the integer pipes too much:
 * with a branch to the native multiply in each of the 84 products of a
 * node the step ran 1.77 GLUPS, with a flag per product 1.91, against 2.68
 * without checks.  dmul_bits gives the IEEE product for any operands
 * (dmul_bits_dom reports the operands outside the domain).
 *
 * Host+device, so a CPU build checks it against the host's multiply.
 */
#ifndef PLB_EMU_H_
#define PLB_EMU_H_

#include <stdint.h>

#if defined(__CUDACC__)
#define EMU_HD __host__ __device__ __forceinline__
#else
#define EMU_HD static inline
#endif

namespace plb {
namespace emu {

constexpr uint64_t kM52 = 0xfffffffffffffull;
constexpr uint64_t kH53 = 0x10000000000000ull;

EMU_HD uint64_t umulhi(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

/* the native product, bits in and out */
EMU_HD uint64_t dmul_native(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(
        __dmul_rn(__longlong_as_double((long long)a), __longlong_as_double((long long)b)));
#else
    double x, y;
    __builtin_memcpy(&x, &a, 8);
    __builtin_memcpy(&y, &b, 8);
    volatile double p = x * y;
    double q = p;
    uint64_t r;
    __builtin_memcpy(&r, &q, 8);
    return r;
#endif
}

/* Bits of a * b for operands in the integer path's domain (given as bits);
 * sets `outside` (and returns unspecified bits) for operands outside it. */
EMU_HD uint64_t dmul_bits_dom(uint64_t a, uint64_t b, uint32_t &outside)
{
    const uint64_t sign = (a ^ b) & 0x8000000000000000ull;
    const uint32_t ea = (uint32_t)(a >> 52) & 0x7ffu;
    const uint32_t eb = (uint32_t)(b >> 52) & 0x7ffu;
    /* a zero times a finite value */
    if (((a << 1) == 0ull && eb != 0x7ffu) || ((b << 1) == 0ull && ea != 0x7ffu))
        return sign;
    /* normal operands with a normal product: 1 <= ea, eb <= 2046 and the
     * biased result exponent ea + eb - 1023 (+1 for a significand product
     * >= 2, +1 more for a rounding carry) within [1, 2046] */
    outside |= (uint32_t)(ea - 1u >= 2046u) | (uint32_t)(eb - 1u >= 2046u) |
               (uint32_t)(ea + eb - 1024u > 2043u);
    const uint64_t ma = (a & kM52) | kH53, mb = (b & kM52) | kH53;
    const uint64_t hi = umulhi(ma, mb), lo = ma * mb; /* product in [2^104, 2^106) */
    const uint32_t top = (uint32_t)(hi >> 41) & 1u;   /* bit 105 */
    const uint32_t sh = 52u + top;
    uint64_t m = (hi << (64u - sh)) | (lo >> sh);     /* [2^52, 2^53) */
    const uint64_t rem = lo & ((1ull << sh) - 1ull);
    const uint64_t half = 1ull << (sh - 1u);
    m += (uint64_t)((rem > half) | ((rem == half) & (uint32_t)(m & 1u)));
    uint32_t e = ea + eb - 1023u + top;
    if (m >> 53) { /* rounded up to 2^53 */
        m >>= 1;
        e += 1u;
    }
    return sign | ((uint64_t)e << 52) | (m & kM52);
}

/* Bits of a * b for operands known to lie in the domain, or zero (given as
 * bits). */
EMU_HD uint64_t dmul_bits_fast(uint64_t a, uint64_t b)
{
    const uint64_t sign = (a ^ b) & 0x8000000000000000ull;
    const uint32_t ea = (uint32_t)(a >> 52) & 0x7ffu;
    const uint32_t eb = (uint32_t)(b >> 52) & 0x7ffu;
    if (ea == 0u || eb == 0u) return sign;
    const uint64_t ma = (a & kM52) | kH53, mb = (b & kM52) | kH53;
    const uint64_t hi = umulhi(ma, mb), lo = ma * mb; /* product in [2^104, 2^106) */
    const uint32_t top = (uint32_t)(hi >> 41) & 1u;   /* bit 105 */
    const uint32_t sh = 52u + top;
    uint64_t m = (hi << (64u - sh)) | (lo >> sh);     /* [2^52, 2^53) */
    const uint64_t rem = lo & ((1ull << sh) - 1ull);
    const uint64_t half = 1ull << (sh - 1u);
    m += (uint64_t)((rem > half) | ((rem == half) & (uint32_t)(m & 1u)));
    uint32_t e = ea + eb - 1023u + top;
    if (m >> 53) { /* rounded up to 2^53 */
        m >>= 1;
        e += 1u;
    }
    return sign | ((uint64_t)e << 52) | (m & kM52);
}

/* 1 unless x (given as bits) is a zero or of magnitude in [2^-64, 2^64):
 * the range of the node values, densities and run constants for which the
 * bit-exact collision's products stay in the domain of dmul_bits_fast. */
EMU_HD uint32_t outside_node_range(uint64_t x)
{
    const uint32_t e = (uint32_t)(x >> 52) & 0x7ffu;
    return (uint32_t)((x << 1) != 0ull) & (uint32_t)(e - (1023u - 64u) >= 128u);
}

/* Bits of a * b, both given as bits: the IEEE product for any operands. */
EMU_HD uint64_t dmul_bits(uint64_t a, uint64_t b)
{
    uint32_t outside = 0;
    const uint64_t r = dmul_bits_dom(a, b, outside);
    return outside ? dmul_native(a, b) : r;
}

}  // namespace emu
}  // namespace plb

#endif
