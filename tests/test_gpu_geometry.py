"""Device geometry: the sphere pack and the table built from a flag grid are
the host builder's, bit for bit."""
import numpy as np
import pytest

import porelb_gb300 as P

from helpers import noise_flag

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [(0, (64, 64, 64), 6.0, 6.0, 0.40),
                                  (1, (96, 80, 72), 4.0, 10.0, 0.35),
                                  (7, (24, 20, 16), 2.5, 4.0, 0.45),
                                  (3, (16, 16, 16), 5.0, 5.0, 0.97)])
def test_device_sphere_pack_matches_host(case):
    seed, dims, rmin, rmax, phi = case
    a, na, pa = P.sphere_pack(seed, *dims, rmin, rmax, phi)
    b, nb, pb = P.sphere_pack_device(seed, *dims, rmin, rmax, phi)
    assert na == nb and pa == pb
    assert (a == b).all()


@pytest.mark.parametrize("ordering", ["morton", "reference"])
@pytest.mark.parametrize("case", [((12, 10, 8), 0.3, 1, 1), ((9, 7, 12), 0.4, 2, 3),
                                  ((2, 2, 2), 0.2, 3, 1), ((17, 5, 9), 0.5, 4, 1)])
def test_table_from_flag_equals_table_from_V(case, ordering):
    dims, p_solid, seed, num_p = case
    flag = noise_flag(dims, p_solid, seed)
    V, vs = P.build_table(flag, *dims, num_p)
    a = P.Simulation(V, *dims, vs, tau=0.7, force=2e-3, ordering=ordering)
    b = P.Simulation.from_flag(flag, *dims, num_p=num_p, tau=0.7, force=2e-3,
                               ordering=ordering)
    assert a.N == b.N
    for s in (a, b):
        s.init_dist_macro()
        s.step(12)
    assert (a.get_f() == b.get_f()).all()
    assert (a.macros() == b.macros()).all()
    a.close()
    b.close()


def test_packed_equals_host_pipeline():
    dims = (40, 36, 32)
    flag, ns, phi = P.sphere_pack(5, *dims, 3.0, 5.0, 0.4)
    V, vs = P.build_table(flag, *dims, 1)
    a = P.Simulation(V, *dims, vs, tau=0.9, force=1e-4, precision="fp64")
    b = P.Simulation.packed(5, *dims, 3.0, 5.0, 0.4, tau=0.9, force=1e-4,
                            precision="fp64")
    assert b.num_spheres == ns and b.porosity == phi and b.N == len(V)
    for s in (a, b):
        s.init_dist_macro()
        s.step(20)
    assert (a.get_f() == b.get_f()).all()
    a.close()
    b.close()


def test_from_flag_rejects_bad_values():
    flag = np.ones(27, np.uint8)
    flag[4] = 2
    with pytest.raises(P.PorelbError):
        P.Simulation.from_flag(flag, 3, 3, 3)
    with pytest.raises(P.PorelbError):
        P.Simulation.from_flag(np.ones(4 * 4 * 6, np.uint8), 4, 4, 6, num_p=4)
