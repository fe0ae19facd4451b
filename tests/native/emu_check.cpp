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

/* The bit-exact collision's operations (plb_step.cu, collide_fp64_exact),
 * restated with each of its integer-path products checked: the number of
 * products whose operands leave dmul_bits_fast's domain.  Sums and the FP64
 * products run on the host in the same order. */
static long node_outside(const double f[19], double omega, double om1, double k3,
                         double force, double half_force, int it)
{
    static const int ex[19] = {0, 1, -1, 0, 0, 0, 0, 0, 0, 0, 0, -1, 1, -1, 1, -1, 1, -1, 1};
    static const int ey[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, -1, 1};
    static const int ez[19] = {0, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1, 0, 0, 0, 0};
    long out = 0;
    auto imul = [&](double a, double b) {
        uint32_t o = 0;
        plb::emu::dmul_bits_dom(bits(a), bits(b), o);
        out += o;
        volatile double p = a * b;
        return (double)p;
    };
    double rho = f[0];
    for (int j = 1; j < 19; j++) rho = rho + f[j];
    double mom[3] = {0, 0, 0};
    const int *e3[3] = {ex, ey, ez};
    for (int c = 0; c < 3; c++)
        for (int j = 0; j < 19; j++)
            if (e3[c][j]) mom[c] = e3[c][j] > 0 ? mom[c] + f[j] : mom[c] - f[j];
    if (it > 0) mom[0] = mom[0] + half_force;
    const double u = mom[0] / rho, v = mom[1] / rho, w = mom[2] / rho;
    const double uv15 = 1.5 * ((u * u + v * v) + w * w);
    const double h[3] = {1.0 / 3 * rho, 1.0 / 18 * rho, 1.0 / 36 * rho};
    const double am = omega + (k3 * (-1.0 - u)) * force;
    const double a0 = omega + (k3 * (0.0 - u)) * force;
    const double ap = omega + (k3 * (1.0 - u)) * force;
    imul(om1, f[0]);
    imul(a0, imul(h[0], 1.0 - uv15));
    for (int J = 1; J < 19; J += 2) {
        double eu = 0.0;
        if (ex[J]) eu = ex[J] > 0 ? u : -u;
        if (ey[J]) eu = ey[J] > 0 ? eu + v : eu - v;
        if (ez[J]) eu = ez[J] > 0 ? eu + w : eu - w;
        const double t3 = imul(3.0, eu);
        const double c2 = imul(imul(4.5, eu), eu);
        const double hh = J <= 6 ? h[1] : h[2];
        const double fJ = imul(hh, ((1.0 + t3) + c2) - uv15);
        const double fK = imul(hh, ((1.0 - t3) + c2) - uv15);
        const double AJ = ex[J] > 0 ? ap : (ex[J] < 0 ? am : a0);
        const double AK = ex[J] > 0 ? am : (ex[J] < 0 ? ap : a0);
        imul(om1, f[J]);
        imul(AJ, fJ);
        imul(om1, f[J + 1]);
        imul(AK, fK);
    }
    return out;
}

/* Nodes that pass the collision's range check (values and density zero or
 * in [2^-64, 2^64), run constants too): random values over the whole
 * range, values at its ends, and densities nearly cancelled so that the
 * velocities reach their extremes.  Returns how many of their
 * integer-path products left the multiply's domain (0 expected), and
 * stores the number of nodes checked in *checked. */
extern "C" long node_range_check(long n, unsigned long long seed, long *checked)
{
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> U(1.0, 2.0);
    long out = 0, cnt = 0;
    const double taus[] = {0.5000001, 0.51, 0.8, 1.0, 1.7, 1e6, ldexp(1.0, 60)};
    const double forces[] = {0.0, 1e-6, 5e-7, ldexp(1.0, -63), ldexp(1.0, 63), -3e-4};
    for (long k = 0; k < n; k++) {
        double f[19];
        const int mode = (int)(g() % 4);
        for (int j = 0; j < 19; j++) {
            const int ex2 = mode == 1 ? (g() & 1 ? -64 : 63) : (int)(g() % 128) - 64;
            f[j] = (g() % 11 == 0) ? 0.0 : ((g() & 1) ? -1.0 : 1.0) * U(g) * ldexp(1.0, ex2);
            if (fabs(f[j]) >= ldexp(1.0, 64)) f[j] = ldexp(1.0, 63);
        }
        if (mode >= 2) {
            /* density nearly cancelled: f0 balances the others */
            double s = 0.0;
            for (int j = 1; j < 19; j++) s = s + f[j];
            f[0] = -s + ((g() & 1) ? 1.0 : -1.0) * U(g) * ldexp(1.0, -64 + (int)(g() % 4));
        }
        bool pass = true;
        double rho = f[0];
        for (int j = 1; j < 19; j++) rho = rho + f[j];
        for (int j = 0; j < 19; j++) pass = pass && !plb::emu::outside_node_range(bits(f[j]));
        pass = pass && !plb::emu::outside_node_range(bits(rho)) && rho != 0.0;
        const double tau = taus[g() % 7], force = forces[g() % 6];
        const double omega = 1.0 / tau, om1 = 1.0 - omega, k3 = (1.0 - 0.5 * omega) * 3.0;
        const double half_force = 0.5 * force;
        const double cs[5] = {omega, om1, k3, force, half_force};
        for (double c : cs) pass = pass && !plb::emu::outside_node_range(bits(c));
        if (!pass) continue;
        cnt++;
        out += node_outside(f, omega, om1, k3, force, half_force, (int)(g() % 2));
    }
    *checked = cnt;
    return out;
}

/* dmul_bits_fast against the host's multiply on in-domain operands, and
 * outside_node_range at the ends of its range; returns mismatches. */
extern "C" long fast_check(long n, unsigned long long seed)
{
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    long bad = 0;
    for (long k = 0; k < n; k++) {
        const double a = U(g) * ldexp(1.0, (int)(g() % 400) - 200);
        const double b = U(g) * ldexp(1.0, (int)(g() % 400) - 200);
        volatile double p = a * b;
        if (plb::emu::dmul_bits_fast(bits(a), bits(b)) != bits(p)) bad++;
        volatile double q = a * 0.0;
        if (plb::emu::dmul_bits_fast(bits(a), bits(0.0)) != bits(q)) bad++;
    }
    const double inside[] = {0.0, -0.0, ldexp(1.0, -64), -ldexp(1.0, -64), 1.0,
                             nextafter(ldexp(1.0, 64), 0.0), -nextafter(ldexp(1.0, 64), 0.0)};
    const double outside[] = {ldexp(1.0, 64), nextafter(ldexp(1.0, -64), 0.0), INFINITY,
                              -INFINITY, NAN, ldexp(1.0, -1074), ldexp(1.0, -1022), 1e300};
    for (double x : inside) bad += plb::emu::outside_node_range(bits(x)) != 0;
    for (double x : outside) bad += plb::emu::outside_node_range(bits(x)) != 1;
    return bad;
}
