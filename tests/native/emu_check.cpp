/*
 * emu_check.cpp - the integer-pipe double multiply (plb_emu.h) built for
 * the CPU and checked against the host's IEEE multiply, for tests.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <random>

#include "../../porelb_gb300/csrc/plb_emu.h"

static uint64_t bits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static double dbl(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }

/* Checks n random products of each kind; returns the number of mismatches. */
extern "C" long emu_check(long n, unsigned long long seed)
{
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    long bad = 0;
    auto check = [&](double a, double b) {
        volatile double p = a * b;
        if (plb::emu::dmul_bits(bits(a), bits(b)) != bits(p)) bad++;
    };
    for (long k = 0; k < n; k++) {
        /* wide range of magnitudes and both signs */
        check(U(g) * ldexp(1.0, (int)(g() % 40) - 30), U(g) * ldexp(1.0, (int)(g() % 40) - 30));
        /* x * 1.5: a tie whenever x's significand is odd */
        check(U(g), 1.5);
        /* short significands: exact products */
        const uint64_t ma = (1ull << 52) | ((g() & 0x3ffull) << (42 - (g() % 20)));
        const uint64_t mb = (1ull << 52) | ((g() & 0x3ffull) << (42 - (g() % 20)));
        check(dbl(ma | ((uint64_t)(1023 - (g() % 8)) << 52) | ((g() & 1) << 63)),
              dbl(mb | ((uint64_t)(1023 - (g() % 8)) << 52)));
        /* the collision's products: weights x density, omega terms, velocities */
        check(1.0 / 36 * (1 + 0.1 * U(g)), 1.25 + 0.3 * U(g));
        check(4.5, U(g) * 1e-3);
    }
    /* signed zeros */
    const double z[] = {0.0, -0.0, 1.0, -1.0, 1.0 / 3};
    for (double p : z)
        for (double q : z) check(p, q);
    /* outside the integer path: infinities, NaNs, subnormals, products that
     * overflow or underflow, and the edges of the normal range */
    const double sp[] = {INFINITY, -INFINITY, NAN, -NAN, 0.0, -0.0, 1.0, -2.5,
                         ldexp(1.0, -1074), ldexp(-3.0, -1060), ldexp(1.0, -1022),
                         ldexp(1.5, -1022), ldexp(1.0, 1023), ldexp(-1.9, 1023),
                         ldexp(1.0, 512), ldexp(1.0, -512), ldexp(1.7, 511),
                         ldexp(1.3, -511), 1e-300, -1e300, 1.0 / 3};
    for (double p : sp)
        for (double q : sp) check(p, q);
    for (long k = 0; k < n / 10; k++) {
        /* exponents spread over the whole range, both signs */
        const int xa = (int)(g() % 2200) - 1100, xb = (int)(g() % 2200) - 1100;
        check(U(g) * ldexp(1.0, xa), U(g) * ldexp(1.0, xb));
        /* products at the edges of the normal range */
        const int t = (int)(g() % 8);
        check(U(g) * ldexp(1.0, -511 - t), U(g) * ldexp(1.0, -511 + (int)(g() % 8)));
        check(U(g) * ldexp(1.0, 511 + t), U(g) * ldexp(1.0, 512 - (int)(g() % 8)));
    }
    return bad;
}
