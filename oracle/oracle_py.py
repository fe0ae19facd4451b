"""ctypes bindings of the test oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.

* ``liborc.so``   - the CPU restatement of the reference path
  (porelb_oracle.c), built by oracle/Makefile on any host.
* ``_ref/*.so``   - the reference itself, compiled from its own sources by
  oracle/Makefile where the reference tree is present (this container, not
  the GPU machine).  ``ref_available()`` says whether it was built.
"""
import ctypes
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_PATH = os.path.join(HERE, "liborc.so")
REF_SOLVER_PATH = os.path.join(HERE, "_ref", "libref_porelb.so")
REF_PRE_PATH = os.path.join(HERE, "_ref", "libref_pre.so")
REF_POST_PATH = os.path.join(HERE, "_ref", "libref_post.so")

Q = 19
NB_DTYPE = np.dtype([("node_type", "u1"), ("pad_", "u1"),
                     ("node_pid", "<u2"), ("node_id", "<u4")])
NODE_DTYPE = np.dtype([("x", "<u2"), ("y", "<u2"), ("z", "<u2"),
                       ("pad_", "<u2"), ("nb_info", NB_DTYPE, (Q - 1,))])

_orc = None
_ref = None
_pre = None

_V = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_IP = ctypes.POINTER(ctypes.c_int)


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def orc():
    global _orc
    if _orc is None:
        if not os.path.exists(ORC_PATH):
            raise ImportError(f"{ORC_PATH} not built (make -C oracle)")
        lib = ctypes.CDLL(ORC_PATH)
        lib.orc_build_v.restype = _I
        lib.orc_build_v.argtypes = [_V, _I, _I, _I, _I, _V, _IP, _IP]
        lib.orc_create.restype = _V
        lib.orc_create.argtypes = [_V, _I, _I, _I, _I, _I, _IP, _D, _D]
        lib.orc_destroy.argtypes = [_V]
        lib.orc_init.argtypes = [_V]
        lib.orc_run.restype = _I
        lib.orc_run.argtypes = [_V, _I, _I, _I, _IP, _IP]
        lib.orc_stream.argtypes = [_V]
        lib.orc_collide.restype = _I
        lib.orc_collide.argtypes = [_V, _I, _IP]
        for name in ("orc_f0", "orc_f1"):
            getattr(lib, name).restype = ctypes.POINTER(ctypes.c_double)
            getattr(lib, name).argtypes = [_V]
        lib.orc_macro.restype = ctypes.POINTER(ctypes.c_double)
        lib.orc_macro.argtypes = [_V, _I]
        lib.orc_num_node.restype = _I
        lib.orc_num_node.argtypes = [_V]
        lib.orc_pull_table.argtypes = [_V, _I, _I, _IP, _I, _V, _V]
        lib.orc_pull_table_rule.argtypes = [_V, _I, _I, _IP, _I, _I, _V, _V]
        lib.orc_pull_step.restype = _I
        lib.orc_pull_step.argtypes = [_V, _V, _I, _V, _V, _V, _V, _V, _V, _D,
                                      _D, _I, _IP]
        lib.orc_reduce.argtypes = [_V, ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(ctypes.c_double)]
        lib.orc_sphere_pack.restype = _I
        lib.orc_sphere_pack.argtypes = [ctypes.c_uint64, _I, _I, _I, _D, _D,
                                        _D, _V, _IP,
                                        ctypes.POINTER(ctypes.c_double)]
        _orc = lib
    return _orc


def ref_available():
    return os.path.exists(REF_SOLVER_PATH) and os.path.exists(REF_PRE_PATH)


def _ref_libs():
    global _ref, _pre
    if _ref is None:
        if not ref_available():
            raise ImportError("oracle/_ref not built (reference tree absent)")
        _ref = ctypes.CDLL(REF_SOLVER_PATH)
        _ref.ref_run.restype = _I
        _ref.ref_run.argtypes = [ctypes.c_char_p, _I, _I, _D, _D, _I, _I, _V,
                                 _V, _V, ctypes.POINTER(ctypes.c_double)]
        _pre = ctypes.CDLL(REF_PRE_PATH)
        _pre.ref_build_v.restype = _I
        _pre.ref_build_v.argtypes = [ctypes.c_char_p, _I, _I, _I, _I, _V, _IP]
        _pre.ref_build_and_save_v.restype = _I
        _pre.ref_build_and_save_v.argtypes = [ctypes.c_char_p, _I, _I, _I, _I,
                                              ctypes.c_char_p]
    return _ref, _pre


# ----------------------------------------------------------- restatement

def sphere_pack(seed, nx, ny, nz, rmin, rmax, porosity):
    """The synthetic geometry generator -> (flag, spheres, porosity); flag
    is nx*ny*nz uint8, x fastest."""
    lib = orc()
    flag = np.empty(nx * ny * nz, np.uint8)
    ns = ctypes.c_int()
    phi = ctypes.c_double()
    st = lib.orc_sphere_pack(seed, nx, ny, nz, rmin, rmax, porosity, _p(flag),
                             ctypes.byref(ns), ctypes.byref(phi))
    if st != 0:
        raise ValueError(f"orc_sphere_pack status {st}")
    return flag, ns.value, phi.value


def build_v(flag, nx, ny, nz, num_p=1):
    lib = orc()
    flag = np.ascontiguousarray(flag, dtype=np.uint8).reshape(-1)
    n = ctypes.c_int()
    vs = np.zeros(num_p, np.int32)
    st = lib.orc_build_v(_p(flag), nx, ny, nz, num_p, None, ctypes.byref(n),
                         vs.ctypes.data_as(_IP))
    if st != 0:
        raise ValueError(f"orc_build_v status {st}")
    V = np.zeros(n.value, NODE_DTYPE)
    lib.orc_build_v(_p(flag), nx, ny, nz, num_p, _p(V), ctypes.byref(n),
                    vs.ctypes.data_as(_IP))
    return V, vs


class OracleSim:
    """Push-form CPU solver over the whole table (all rank slabs)."""

    def __init__(self, V, nx, ny, nz, v_sub_start, tau, force):
        self.lib = orc()
        self.V = np.ascontiguousarray(V, dtype=NODE_DTYPE)
        self.vs = np.ascontiguousarray(v_sub_start, dtype=np.int32)
        self.N = len(V)
        self.h = self.lib.orc_create(_p(self.V), self.N, nx, ny, nz,
                                     len(self.vs), self.vs.ctypes.data_as(_IP),
                                     tau, force)
        self.it = 0

    def init(self):
        self.lib.orc_init(self.h)
        self.it = 0

    def run(self, nsteps, threads=1, it_begin=None):
        it0 = self.it if it_begin is None else it_begin
        bi, bn = ctypes.c_int(), ctypes.c_int()
        st = self.lib.orc_run(self.h, it0, nsteps, threads, ctypes.byref(bi),
                              ctypes.byref(bn))
        self.it = it0 + nsteps
        return st, bi.value, bn.value

    def f0(self):
        return np.ctypeslib.as_array(self.lib.orc_f0(self.h),
                                     (self.N * Q,)).copy()

    def f1(self):
        return np.ctypeslib.as_array(self.lib.orc_f1(self.h),
                                     (self.N * Q,)).copy()

    def macros(self):
        return np.stack([np.ctypeslib.as_array(self.lib.orc_macro(self.h, c),
                                               (self.N,)).copy()
                         for c in range(4)])

    def reduce(self):
        a, m = ctypes.c_double(), ctypes.c_double()
        self.lib.orc_reduce(self.h, ctypes.byref(a), ctypes.byref(m))
        return a.value, m.value

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pull_table(V, v_sub_start, remote_wins=False, halfway=False):
    lib = orc()
    V = np.ascontiguousarray(V, dtype=NODE_DTYPE)
    vs = np.ascontiguousarray(v_sub_start, dtype=np.int32)
    kind = np.zeros(len(V) * 18, np.uint8)
    src = np.zeros(len(V) * 18, np.uint32)
    lib.orc_pull_table_rule(_p(V), len(V), len(vs), vs.ctypes.data_as(_IP),
                            int(remote_wins), int(halfway), _p(kind), _p(src))
    return kind, src


def pull_run(V, v_sub_start, tau, force, nsteps, remote_wins=False,
             halfway=False):
    """Pull-form restatement from rest: returns (f0, f1, macros)."""
    lib = orc()
    kind, src = pull_table(V, v_sub_start, remote_wins, halfway)
    N = len(V)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    f0 = np.tile(w, N).astype(np.float64)
    f1 = f0.copy()
    mac = np.zeros((4, N))
    mac[0] = 1.0
    bad = ctypes.c_int()
    for it in range(nsteps):
        st = lib.orc_pull_step(_p(kind), _p(src), N, _p(f0), _p(f1),
                               _p(mac[0]), _p(mac[1]), _p(mac[2]), _p(mac[3]),
                               tau, force, it, ctypes.byref(bad))
        if st != 0:
            raise RuntimeError(f"density guard at it={it} node={bad.value}")
    return f0, f1, mac


# ------------------------------------------------------------- reference

def ref_build_v(flag, nx, ny, nz, num_p=1):
    """The reference's build_V on this flag field -> (V, v_sub_start)."""
    _, pre = _ref_libs()
    flag = np.ascontiguousarray(flag, dtype=np.uint8).reshape(-1)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "flag.bin")
        flag.tofile(path)
        n = pre.ref_build_v(path.encode(), nx, ny, nz, num_p, None, None)
        V = np.zeros(n, NODE_DTYPE)
        vs = np.zeros(num_p, np.int32)
        pre.ref_build_v(path.encode(), nx, ny, nz, num_p, _p(V),
                        vs.ctypes.data_as(_IP))
    return V, vs


def ref_write_vbin(flag, nx, ny, nz, num_p, path):
    """The reference's build_V + save_V writing V.bin at path."""
    _, pre = _ref_libs()
    flag = np.ascontiguousarray(flag, dtype=np.uint8).reshape(-1)
    with tempfile.TemporaryDirectory() as d:
        fp = os.path.join(d, "flag.bin")
        flag.tofile(fp)
        return pre.ref_build_and_save_v(fp.encode(), nx, ny, nz, num_p,
                                        os.fsencode(path))


def ref_postprocess(workdir, args):
    """The reference postprocess main in workdir with argv args."""
    if not os.path.exists(REF_POST_PATH):
        raise ImportError("oracle/_ref/libref_post.so not built")
    lib = ctypes.CDLL(REF_POST_PATH)
    lib.ref_postprocess.restype = _I
    lib.ref_postprocess.argtypes = [ctypes.c_char_p, _I,
                                    ctypes.POINTER(ctypes.c_char_p)]
    argv = ["postprocess.x"] + [str(a) for a in args]
    arr = (ctypes.c_char_p * len(argv))(*[a.encode() for a in argv])
    return lib.ref_postprocess(os.fsencode(workdir), len(argv), arr)


def ref_run(workdir, num_ranks, it_max, tau=float("nan"),
            force=float("nan"), save=False, save_every=0, num_f=None):
    """Run the reference solver on workdir/V.bin with num_ranks ranks.

    Returns (f0, f1, macros, elapsed) in V.bin order."""
    ref, _ = _ref_libs()
    if num_f is None:
        num_f = int(np.fromfile(os.path.join(workdir, "V.bin"), np.int32, 1)[0])
    f0 = np.zeros(num_f * Q)
    f1 = np.zeros(num_f * Q)
    mac = np.zeros((4, num_f))
    el = ctypes.c_double()
    st = ref.ref_run(os.fsencode(workdir), num_ranks, it_max, tau, force,
                     int(save), save_every, _p(f0), _p(f1), _p(mac),
                     ctypes.byref(el))
    if st != 0:
        raise RuntimeError(f"ref_run failed in {workdir}")
    return f0, f1, mac, el.value
