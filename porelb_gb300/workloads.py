"""Synthetic workloads of the benchmark configurations.

The reference reads its geometry (flag.bin) from outside; these seeded
generators stand in for it.  Every random draw comes from splitmix64
(Steele, Lea & Flood 2014) so the streams are the same on every host.

* plain:   one periodic sphere pack (plb_sphere_pack).
* batched: 64 samples, seed 3.  Cube edge lognormal with median 80 and
           sigma 0.5 (log space), clipped to [32, 192]; porosity U[0.10,
           0.50]; sphere radius U[3, 8]; tau U[0.6, 1.5]; force 1e-6; FP32;
           tolerance 1e-7.
* serving: 2000 requests, seed 4, Poisson arrivals.  Edge lognormal with
           median 100 and sigma 0.5, clipped to [48, 256]; porosity U[0.15,
           0.45]; radius U[3, 10]; tau U[0.6, 1.2]; tolerance 1e-6 or 1e-7
           (equal odds); force 1e-6.
"""
import math
from dataclasses import dataclass


class SplitMix64:
    MASK = (1 << 64) - 1

    def __init__(self, seed):
        self.s = seed & self.MASK

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & self.MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next() >> 11) * 2.0 ** -53)

    def normal(self):
        # Box-Muller
        u1 = max(self.uniform(), 2.0 ** -53)
        u2 = self.uniform()
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)

    def lognormal_edge(self, median, sigma, lo, hi):
        e = int(round(median * math.exp(sigma * self.normal())))
        return min(hi, max(lo, e))


@dataclass
class Sample:
    index: int
    edge: int
    porosity: float
    rmin: float
    rmax: float
    tau: float
    force: float
    tol: float
    seed: int          # geometry seed (sphere pack)
    arrival: float = 0.0


def batched_samples(n=64, seed=3):
    g = SplitMix64(seed)
    out = []
    for i in range(n):
        edge = g.lognormal_edge(80, 0.5, 32, 192)
        phi = g.uniform(0.10, 0.50)
        r = g.uniform(3.0, 8.0)
        tau = g.uniform(0.6, 1.5)
        out.append(Sample(i, edge, phi, r, r, tau, 1e-6, 1e-7, g.next()))
    return out


def serving_requests(n=2000, seed=4, rate=20.0):
    """n requests with Poisson arrivals at `rate` per second."""
    g = SplitMix64(seed)
    out = []
    t = 0.0
    for i in range(n):
        t += -math.log(max(g.uniform(), 2.0 ** -53)) / rate
        edge = g.lognormal_edge(100, 0.5, 48, 256)
        phi = g.uniform(0.15, 0.45)
        r = g.uniform(3.0, 10.0)
        tau = g.uniform(0.6, 1.2)
        tol = 1e-6 if g.next() & 1 else 1e-7
        out.append(Sample(i, edge, phi, r, r, tau, 1e-6, tol, g.next(), t))
    return out
