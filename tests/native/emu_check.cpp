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
    return bad;
}
