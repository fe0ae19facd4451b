/*
 * fx_twin.cpp - CPU build of the integer-pipe FP64 collision (plb_fx.h) with
 * the pull stream, for tests: the same integer algorithm the GPU runs,
 * checked against the oracle on the CPU.
 */
#include <stdint.h>
#include <string.h>

#include "../../porelb_gb300/csrc/plb_fx.h"

static const int OPP[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};

/* One pull-stream + collide step on AoS arrays (reference order), pull table
 * from the oracle (kind 0 pull src, 1 bounce, 2 untouched).  Returns the
 * number of nodes that left the fixed-point range (those nodes are left
 * with their streamed values), -1 on a density-guard trip. */
extern "C" int fx_twin_step(const uint8_t *kind, const uint32_t *src, int N,
                            const double *f0, double *f1, double *fout,
                            double *mac, double tau, double force, int it)
{
    const plb::fx::Consts k = plb::fx::make_consts(tau, force);
    int nbad = 0, dens = 0;
    for (int i = 0; i < N; i++) {
        f1[(size_t)i * 19] = f0[(size_t)i * 19];
        for (int j = 1; j < 19; j++) {
            const uint8_t kd = kind[(size_t)i * 18 + j - 1];
            if (kd == 0) f1[(size_t)i * 19 + j] = f0[(size_t)src[(size_t)i * 18 + j - 1] * 19 + j];
            else if (kd == 1) f1[(size_t)i * 19 + j] = f0[(size_t)i * 19 + OPP[j]];
        }
        uint64_t b[19];
        memcpy(b, f1 + (size_t)i * 19, sizeof(b));
        plb::fx::Moments m;
        uint32_t fl = plb::fx::collide(b, k, it > 0, m);
        if ((fl & plb::fx::kDensity) && !(fl & plb::fx::kBad)) dens = 1;
        if (fl & plb::fx::kBad) {
            nbad++;
            memcpy(fout + (size_t)i * 19, f1 + (size_t)i * 19, sizeof(b));
        } else {
            memcpy(fout + (size_t)i * 19, b, sizeof(b));
        }
        if (mac) {
            uint32_t ign = 0;
            const uint64_t rb = plb::fx::to_bits(m.R, ign);
            memcpy(&mac[i], &rb, 8);
            mac[N + i] = ldexp((double)plb::fx::mul(m.Jx, m.inv), -60);
            mac[2 * N + i] = ldexp((double)plb::fx::mul(m.Jy, m.inv), -60);
            mac[3 * N + i] = ldexp((double)plb::fx::mul(m.Jz, m.inv), -60);
        }
    }
    return dens ? -1 : nbad;
}
