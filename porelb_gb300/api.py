"""Python host mirror of porelb's solver interface over the C ABI.

The reference exposes its hot path as the SIMULATION function set of one C
program (porelb.h:127-165): alloc_memory / check_V / init_para /
build_send_recv_info / init_dist_macro, the step loop (stream, halo, collide)
and save_data.  ``Simulation`` maps those onto libporelb_gpu: construction
covers alloc_memory..build_send_recv_info, ``init_dist_macro`` and ``step``
keep the reference's names and iteration numbering, and errors raise
``PorelbError`` carrying the reference's exit code where it has one
(-6 for the density guard, porelb.c:338-342).
"""
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import NODE_DTYPE, Q

PRECISIONS = {"fp64_exact": _lib.FP64_EXACT, "fp64": _lib.FP64,
              "fp32": _lib.FP32, "fp16dev": _lib.FP16DEV,
              "bf16dev": _lib.BF16DEV, "fp64_fma": _lib.FP64_FMA}
ORDERINGS = {"morton": _lib.ORDER_MORTON, "reference": _lib.ORDER_REFERENCE,
             "auto": _lib.ORDER_AUTO}
HALOS = {"auto": _lib.HALO_AUTO, "single": _lib.HALO_SINGLE,
         "remote_wins": _lib.HALO_REMOTE_WINS}
BOUNDARIES = {"reference": _lib.BOUNDARY_REFERENCE,
              "halfway": _lib.BOUNDARY_HALFWAY}


class PorelbError(RuntimeError):
    def __init__(self, status, what=""):
        lib = _lib.load()
        msg = lib.plb_status_string(status).decode()
        super().__init__(f"{what}: {msg} (status {status})" if what else msg)
        self.status = status


def _check(status, what):
    if status != _lib.OK:
        raise PorelbError(status, what)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


# ------------------------------------------------------------------ tables

def build_table(flag, nx, ny, nz, num_p=1):
    """preprocess's build_V (preprocess.c:29-164) -> (V, v_sub_start)."""
    lib = _lib.load()
    flag = np.ascontiguousarray(flag, dtype=np.uint8).reshape(-1)
    if flag.size != nx * ny * nz:
        raise ValueError("flag size does not match nx*ny*nz")
    n = ctypes.c_int(0)
    vs = np.zeros(num_p, dtype=np.int32)
    _check(lib.plb_build_table(_ptr(flag), nx, ny, nz, num_p, None,
                               ctypes.byref(n), _iptr(vs)), "build_table")
    V = np.zeros(n.value, dtype=NODE_DTYPE)
    _check(lib.plb_build_table(_ptr(flag), nx, ny, nz, num_p, _ptr(V),
                               ctypes.byref(n), _iptr(vs)), "build_table")
    return V, vs


def check_table(V, nx, ny, nz, v_sub_start):
    lib = _lib.load()
    vs = np.ascontiguousarray(v_sub_start, dtype=np.int32)
    return lib.plb_check_table(_ptr(V), len(V), nx, ny, nz, len(vs), _iptr(vs))


def write_vbin(path, V, v_sub_start, nx, ny, nz):
    """preprocess's save_V (preprocess.c:166-193)."""
    lib = _lib.load()
    vs = np.ascontiguousarray(v_sub_start, dtype=np.int32)
    V = np.ascontiguousarray(V, dtype=NODE_DTYPE)
    _check(lib.plb_write_vbin(os.fsencode(path), _ptr(V), len(V), len(vs),
                              nx, ny, nz, _iptr(vs)), "write_vbin")


def read_vbin(path):
    """V.bin reader of alloc_memory (porelb.c:15-81), all ranks.

    Returns (V, v_sub_start, (nx, ny, nz))."""
    lib = _lib.load()
    h = [ctypes.c_int(0) for _ in range(5)]
    _check(lib.plb_read_vbin_header(os.fsencode(path),
                                    *[ctypes.byref(x) for x in h]),
           "read_vbin_header")
    n, num_p, nx, ny, nz = (x.value for x in h)
    V = np.zeros(n, dtype=NODE_DTYPE)
    vs = np.zeros(num_p, dtype=np.int32)
    _check(lib.plb_read_vbin(os.fsencode(path), _ptr(V), _iptr(vs)),
           "read_vbin")
    return V, vs, (nx, ny, nz)


def sphere_pack(seed, nx, ny, nz, rmin, rmax, porosity):
    """Deterministic periodic sphere pack -> (flag, num_spheres, porosity)."""
    lib = _lib.load()
    flag = np.zeros(nx * ny * nz, dtype=np.uint8)
    ns = ctypes.c_int(0)
    phi = ctypes.c_double(0.0)
    _check(lib.plb_sphere_pack(ctypes.c_uint64(seed), nx, ny, nz, rmin, rmax,
                               porosity, _ptr(flag), ctypes.byref(ns),
                               ctypes.byref(phi)), "sphere_pack")
    return flag, ns.value, phi.value


def sphere_pack_device(seed, nx, ny, nz, rmin, rmax, porosity, device=0):
    """sphere_pack on the GPU (bit-identical flag)."""
    lib = _lib.load()
    flag = np.zeros(nx * ny * nz, dtype=np.uint8)
    ns = ctypes.c_int(0)
    phi = ctypes.c_double(0.0)
    _check(lib.plb_sphere_pack_device(ctypes.c_uint64(seed), nx, ny, nz, rmin,
                                      rmax, porosity, device, _ptr(flag),
                                      ctypes.byref(ns), ctypes.byref(phi)),
           "sphere_pack_device")
    return flag, ns.value, phi.value


def _params(tau, force, precision, ordering, halo, block_size, device,
            boundary="reference", kernel_variant=0, prefetch=None):
    lib = _lib.load()
    p = _lib.Params()
    lib.plb_default_params(ctypes.byref(p))
    p.tau, p.force_x = float(tau), float(force)
    p.precision = PRECISIONS[precision]
    p.ordering = ORDERINGS[ordering]
    p.halo = HALOS[halo]
    p.block_size = block_size
    p.device = device
    p.boundary = BOUNDARIES[boundary]
    p.kernel_variant = kernel_variant
    p.l2_prefetch = 0 if prefetch is None else (1 if prefetch else -1)
    return p


def auto_ordering(num_node, nz, precision, device=0):
    """The node order PLB_ORDER_AUTO picks for this domain and form:
    "reference" (row order) when three z-planes of its nodes fit in 60% of
    the L2, else "morton"."""
    elem = {"fp64_exact": 8, "fp64": 8, "fp64_fma": 8, "fp32": 4, "fp16dev": 2,
            "bf16dev": 2}[precision]
    o = _lib.load().plb_auto_ordering(int(num_node), int(nz), elem, device)
    return "reference" if o == _lib.ORDER_REFERENCE else "morton"


def _tuned(precision, n, boundary):
    from . import tune
    c = tune.best(precision, n, boundary)
    return c["block_size"], c["ordering"], c["kernel_variant"]


# ------------------------------------------------------------------ solver

class Simulation:
    """One solver instance on one GPU (a SIMULATION of porelb.h:79-117)."""

    def __init__(self, V, nx, ny, nz, v_sub_start=None, tau=0.8,
                 force=1e-3, precision="fp64_exact", ordering="auto",
                 halo="auto", block_size=0, device=0, boundary="reference",
                 kernel_variant=0, prefetch=None, tuned=False):
        """tuned: take block size, ordering and register budget from the
        launch tuner's cached choice for this form and size (tune.tune)."""
        self._lib = _lib.load()
        self.V = np.ascontiguousarray(V, dtype=NODE_DTYPE)
        if tuned:
            block_size, ordering, kernel_variant = _tuned(precision, len(self.V), boundary)
        self.nx, self.ny, self.nz = nx, ny, nz
        vs = np.zeros(1, np.int32) if v_sub_start is None else v_sub_start
        self.v_sub_start = np.ascontiguousarray(vs, dtype=np.int32)
        self.num_p = len(self.v_sub_start)
        self.tau, self.force = float(tau), float(force)
        self.precision = precision
        p = _params(tau, force, precision, ordering, halo, block_size, device,
                    boundary, kernel_variant, prefetch)
        h = ctypes.c_void_p()
        _check(self._lib.plb_create(_ptr(self.V), len(self.V), nx, ny, nz,
                                    self.num_p, _iptr(self.v_sub_start),
                                    ctypes.byref(p), ctypes.byref(h)),
               "plb_create")
        self._h = h
        self.N = len(self.V)
        self.it = 0

    # reference names -------------------------------------------------
    def init_dist_macro(self):
        """init_dist_macro (porelb.c:224-238): rho=1, u=0, f = feq."""
        _check(self._lib.plb_init_equilibrium(self._h), "init_dist_macro")
        self.it = 0

    def step(self, nsteps=1, it_begin=None):
        """Run iterations it..it+nsteps-1 of main's loop (porelb.c:426-437)."""
        it0 = self.it if it_begin is None else it_begin
        _check(self._lib.plb_step(self._h, it0, nsteps), "step")
        self.it = it0 + nsteps

    def step_async(self, nsteps=1, it_begin=None):
        it0 = self.it if it_begin is None else it_begin
        _check(self._lib.plb_step_async(self._h, it0, nsteps), "step_async")
        self.it = it0 + nsteps

    def sync(self):
        _check(self._lib.plb_sync(self._h), "sync")

    def macros(self, out=None):
        """(Rho, Ux, Uy, Uz) of the last step in reference node order, into
        `out` (a C-contiguous float64 array of shape (4, N), e.g. in pinned
        host memory) when given."""
        if out is None:
            out = np.empty((4, self.N), dtype=np.float64)
        elif (out.dtype != np.float64 or out.shape != (4, self.N) or
              not out.flags.c_contiguous):
            raise ValueError("out must be a C-contiguous float64 (4, N) array")
        _check(self._lib.plb_get_macros(self._h, _ptr(out[0]), _ptr(out[1]),
                                        _ptr(out[2]), _ptr(out[3])),
               "get_macros")
        return out

    def save_data(self, directory=".", tag=None):
        """save_data (porelb.c:375-391) for every rank of the table."""
        t = self.it if tag is None else tag
        _check(self._lib.plb_save_parts(self._h, os.fsencode(directory), t),
               "save_data")

    def get_f(self):
        """f0 as the reference's AoS f[i*19+j] in reference node order."""
        out = np.empty(self.N * Q, dtype=np.float64)
        _check(self._lib.plb_get_f(self._h, _ptr(out)), "get_f")
        return out

    def get_f_streamed(self):
        """The distributions the next step collides, after its stream (the
        reference's f1 after the next stream), AoS in reference order."""
        out = np.empty(self.N * Q, dtype=np.float64)
        _check(self._lib.plb_get_f_streamed(self._h, _ptr(out)), "get_f_streamed")
        return out

    def set_f(self, f_aos):
        a = np.ascontiguousarray(f_aos, dtype=np.float64).reshape(-1)
        if a.size != self.N * Q:
            raise ValueError("f has the wrong size")
        _check(self._lib.plb_set_f(self._h, _ptr(a)), "set_f")

    def reduce(self):
        su, m = ctypes.c_double(), ctypes.c_double()
        _check(self._lib.plb_reduce(self._h, ctypes.byref(su),
                                    ctypes.byref(m)), "reduce")
        return su.value, m.value

    def permeability(self):
        kd, ki = ctypes.c_double(), ctypes.c_double()
        _check(self._lib.plb_permeability(self._h, ctypes.byref(kd),
                                          ctypes.byref(ki)), "permeability")
        return kd.value, ki.value

    def last_error(self):
        v = [ctypes.c_int(-1) for _ in range(5)]
        r = ctypes.c_double()
        st = self._lib.plb_last_error(self._h, *[ctypes.byref(x) for x in v],
                                      ctypes.byref(r))
        if st == _lib.OK:
            return None
        return dict(it=v[0].value, node=v[1].value, x=v[2].value,
                    y=v[3].value, z=v[4].value, rho=r.value)

    def kernel_flags(self):
        """PLB_FLAG_* bits the step kernel reported since init (2: nodes
        recomputed in native FP64 by the fixed-point form)."""
        f = ctypes.c_uint(0)
        _check(self._lib.plb_kernel_flags(self._h, ctypes.byref(f)), "kernel_flags")
        return f.value

    def info(self):
        n, npad, prec = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        b = ctypes.c_size_t()
        _check(self._lib.plb_info(self._h, ctypes.byref(n), ctypes.byref(npad),
                                  ctypes.byref(prec), ctypes.byref(b)), "info")
        return dict(num_node=n.value, npad=npad.value, precision=prec.value,
                    device_bytes=b.value)

    @classmethod
    def _from_handle(cls, h, nx, ny, nz, tau, force, precision):
        self = cls.__new__(cls)
        self._lib = _lib.load()
        self._h = h
        self.nx, self.ny, self.nz = nx, ny, nz
        self.tau, self.force, self.precision = float(tau), float(force), precision
        self.N = self.info()["num_node"]
        self.V = None
        self.it = 0
        return self

    @classmethod
    def from_flag(cls, flag, nx, ny, nz, num_p=1, tau=0.8, force=1e-3,
                  precision="fp64_exact", ordering="auto", halo="auto",
                  block_size=0, device=0, boundary="reference",
                  kernel_variant=0, prefetch=None, tuned=False):
        """build_V + create on the device from a 0/1 flag grid."""
        lib = _lib.load()
        flag = np.ascontiguousarray(flag, dtype=np.uint8).reshape(-1)
        if flag.size != nx * ny * nz:
            raise ValueError("flag size does not match nx*ny*nz")
        if tuned:
            block_size, ordering, kernel_variant = _tuned(
                precision, int(np.count_nonzero(flag == 1)), boundary)
        p = _params(tau, force, precision, ordering, halo, block_size, device,
                    boundary, kernel_variant, prefetch)
        h = ctypes.c_void_p()
        _check(lib.plb_create_from_flag(_ptr(flag), nx, ny, nz, num_p,
                                        ctypes.byref(p), ctypes.byref(h)),
               "plb_create_from_flag")
        return cls._from_handle(h, nx, ny, nz, tau, force, precision)

    @classmethod
    def packed(cls, seed, nx, ny, nz, rmin, rmax, porosity, num_p=1, tau=0.8,
               force=1e-3, precision="fp64", ordering="auto", halo="auto",
               block_size=0, device=0, boundary="reference", kernel_variant=0,
               prefetch=None):
        """Sphere pack, table and handle, all built on the device."""
        lib = _lib.load()
        p = _params(tau, force, precision, ordering, halo, block_size, device,
                    boundary, kernel_variant, prefetch)
        h = ctypes.c_void_p()
        ns = ctypes.c_int(0)
        phi = ctypes.c_double(0.0)
        _check(lib.plb_create_packed(ctypes.c_uint64(seed), nx, ny, nz, rmin,
                                     rmax, porosity, num_p, ctypes.byref(p),
                                     ctypes.byref(h), ctypes.byref(ns),
                                     ctypes.byref(phi)), "plb_create_packed")
        sim = cls._from_handle(h, nx, ny, nz, tau, force, precision)
        sim.num_spheres, sim.porosity = ns.value, phi.value
        return sim

    @property
    def stream(self):
        return self._lib.plb_stream(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.plb_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
