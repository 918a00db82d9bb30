"""TEST INFRASTRUCTURE ONLY -- ctypes front end of the CPU oracle.

Two interchangeable back ends with the same calls:
  * ``Oracle``    -- the C restatement in oracle/oracle_ewald.c
                     (oracle/liboracle.so, built by ``build_oracle()``);
  * ``Reference`` -- the reference library itself, compiled from its sources
                     by oracle/Makefile.ref into oracle/_ref/libstokes_ref.so
                     (only where the reference checkout is present).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  The product (libstokes_gb300) never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libstokes_ref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build_oracle(force: bool = False) -> str:
    """Compile oracle/oracle_ewald.c, oracle_bd.c, oracle_adjoint.cpp and
    oracle_lub.c into liboracle.so."""
    srcs = [os.path.join(HERE, f) for f in ("oracle_ewald.c", "oracle_bd.c", "oracle_adjoint.cpp",
                                            "oracle_lub.c")
            if os.path.exists(os.path.join(HERE, f))]
    if (not force and os.path.exists(ORACLE_SO)
            and all(os.path.getmtime(ORACLE_SO) >= os.path.getmtime(s) for s in srcs)):
        return ORACLE_SO
    objs = []
    for src in srcs:
        obj = ORACLE_SO + "." + os.path.basename(src) + ".o"
        cc = "g++" if src.endswith(".cpp") else "gcc"
        std = ["-std=c++17"] if src.endswith(".cpp") else []
        # no contraction of a * b + c into FMA: the same bits on x86 and Arm
        subprocess.check_call([cc, "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off"] + std
                              + ["-c", src, "-o", obj])
        objs.append(obj)
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", ORACLE_SO] + objs + ["-lm"])
    for obj in objs:
        os.remove(obj)
    return ORACLE_SO


def build_reference(ref_root: str | None = None) -> str | None:
    """Compile the reference's own sources into oracle/_ref.  ref_root: the
    libstokes checkout (default: $LIBSTOKES_REF); None when there is none."""
    ref_root = ref_root or os.environ.get("LIBSTOKES_REF")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "src")):
        return None
    repo = os.path.dirname(HERE)
    subprocess.check_call(["make", "-s", "-f", os.path.join("oracle", "Makefile.ref"),
                           f"REF={ref_root}", f"-j{os.cpu_count() or 4}"], cwd=repo)
    return REF_SO


def _d(a):
    return a.ctypes.data_as(_dp)


def ncomp(version: int) -> int:
    return (3, 6, 11)[version]


class _Backend:
    prefix = ""
    so_path = ""
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = C.CDLL(cls.so_path)
            p = cls.prefix
            sig = {
                "new": (C.c_void_p, [C.c_int, C.c_int, _dp, C.c_double, C.c_double, C.c_double]),
                "free": (None, [C.c_void_p]),
                "set_pos": (None, [C.c_void_p, _dp]),
                "set_split": (None, [C.c_void_p, C.c_double, C.c_double]),
                "set_cube": (None, [C.c_void_p, C.c_int, C.c_int]),
                "set_radius": (None, [C.c_void_p, _dp]),
                "set_slip": (None, [C.c_void_p, _dp]),
                "set_misc": (None, [C.c_void_p, C.c_double, C.c_int, C.c_double]),
                "get_split": (None, [C.c_void_p, _dp]),
                "get_table": (None, [C.c_void_p, _dp, _ip]),
                "atimes": (None, [C.c_void_p, _dp, _dp]),
                "matrix": (None, [C.c_void_p, _dp]),
                "matvec": (None, [C.c_int, C.c_int, _dp, _dp, _dp]),
                "atimes_nonewald": (None, [C.c_void_p, _dp, _dp]),
                "matrix_nonewald": (None, [C.c_void_p, _dp]),
            }
            for name, (res, args) in sig.items():
                f = getattr(lib, p + name)
                f.restype = res
                f.argtypes = args
            cls._lib = lib
        return cls._lib

    def __init__(self, version, pos, box):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.version = int(version)
        self.np = pos.shape[0]
        self.box = tuple(float(b) for b in box)
        self._L = self.lib()
        self._f = lambda name: getattr(self._L, self.prefix + name)
        self.h = self._f("new")(self.version, self.np, _d(pos), *self.box)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self._f("free")(h)
            self.h = None

    @property
    def n(self):
        return ncomp(self.version) * self.np

    def set_pos(self, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self._f("set_pos")(self.h, _d(pos))

    def set_split(self, xi, eps):
        self._f("set_split")(self.h, float(xi), float(eps))

    def set_cube(self, nr_shell, nk_shell):
        self._f("set_cube")(self.h, int(nr_shell), int(nk_shell))

    def set_radius(self, a):
        if a is None:
            self._f("set_radius")(self.h, None)
        else:
            a = np.ascontiguousarray(a, dtype=np.float64)
            self._f("set_radius")(self.h, _d(a))

    def set_slip(self, g):
        if g is None:
            self._f("set_slip")(self.h, None)
        else:
            g = np.ascontiguousarray(g, dtype=np.float64)
            self._f("set_slip")(self.h, _d(g))

    def set_misc(self, rmin=0.0, shear_mode=0, shear_shift=0.0):
        self._f("set_misc")(self.h, float(rmin), int(shear_mode), float(shear_shift))

    def split(self):
        out = np.zeros(9)
        self._f("get_split")(self.h, _d(out))
        return dict(xi=out[0], rmax2=out[1], kmax=out[2], self_a=out[3],
                    self_c=out[4], self_m=out[5], pivol=out[6], nr=int(out[7]),
                    kmaxxyz=(int(out[8]) // 10000, int(out[8]) // 100 % 100,
                             int(out[8]) % 100))

    def table(self):
        nr = self.split()["nr"]
        rl = np.zeros((nr, 3))
        rm = np.zeros((nr, 3), dtype=np.int32)
        self._f("get_table")(self.h, _d(rl), rm.ctypes.data_as(_ip))
        return rl, rm

    def atimes(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        self._f("atimes")(self.h, _d(x), _d(y))
        return y

    def vjp(self, pos, g, f, rmin=0.0):
        """(L, dL/dr, dL/dbox) of L = g . M f (oracle/oracle_adjoint.cpp), on
        this system's split and image table (F, FT; equal spheres, no shear)."""
        sp = self.split()
        rl, rm = self.table()
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        g = np.ascontiguousarray(g, dtype=np.float64)
        f = np.ascontiguousarray(f, dtype=np.float64)
        dr = np.zeros(3 * self.np)
        db = np.zeros(3)
        L = C.c_double()
        kx, ky, kz = sp["kmaxxyz"]
        lib = Oracle.lib()
        lib.oracle_vjp(self.version, self.np, _d(pos), *self.box, sp["xi"], sp["rmax2"],
                       float(rmin), sp["nr"], _d(np.ascontiguousarray(rl)),
                       np.ascontiguousarray(rm).ctypes.data_as(_ip), kx, ky, kz, sp["kmax"],
                       sp["self_a"], sp["self_c"], _d(g), _d(f), _d(dr), _d(db), C.byref(L))
        return L.value, dr, db

    def matrix(self):
        m = np.zeros((self.n, self.n))
        self._f("matrix")(self.h, _d(m))
        return m

    def atimes_nonewald(self, x):
        """y = M x of the free-space operator (no periodic images)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        self._f("atimes_nonewald")(self.h, _d(x), _d(y))
        return y

    def matrix_nonewald(self):
        m = np.zeros((self.n, self.n))
        self._f("matrix_nonewald")(self.h, _d(m))
        return m

    def matvec(self, mat, x):
        mat = np.ascontiguousarray(mat, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        self._f("matvec")(self.version, self.np, _d(mat), _d(x), _d(y))
        return y


class Oracle(_Backend):
    """C restatement of the reference's FP64 algorithm (oracle/oracle_ewald.c)."""
    prefix = "oracle_"
    so_path = ORACLE_SO

    @classmethod
    def lib(cls):
        if cls._lib is None:
            build_oracle()
            lib = super().lib()
            lib.oracle_set_threads.argtypes = [C.c_void_p, C.c_int]
            lib.oracle_vjp.restype = None
            lib.oracle_vjp.argtypes = ([C.c_int, C.c_int, _dp] + [C.c_double] * 6
                                       + [C.c_int, _dp, _ip, C.c_int, C.c_int, C.c_int,
                                          C.c_double, C.c_double, C.c_double, _dp, _dp, _dp,
                                          _dp, C.POINTER(C.c_double)])
            lib.oracle_atimes_part.argtypes = [C.c_void_p, _dp, _dp, C.c_int]
            lib.oracle_atimes_rows.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_int]
            lib.oracle_set_open.argtypes = [C.c_void_p, C.c_int]
            lib.oracle_count_real_terms.restype = C.c_longlong
            lib.oracle_count_real_terms.argtypes = [C.c_void_p]
            lib.oracle_count_k.restype = C.c_int
            lib.oracle_count_k.argtypes = [C.c_void_p]
            lib.oracle_xi_by_tratio.restype = C.c_double
            lib.oracle_xi_by_tratio.argtypes = [C.c_double] * 4
            lib.oracle_cheb_eval.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_double,
                                             C.c_double, _dp, _dp]
            lib.oracle_bd_step.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                                           C.c_double, C.c_double, C.c_double, C.c_int, _dp,
                                           C.c_double, C.c_double, _dp, _dp, C.c_double,
                                           C.c_double, _dp, _dp]
            lib.oracle_bd_step_ex.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double,
                                              C.c_double, C.c_double, C.c_double, C.c_double,
                                              C.c_int, _dp, C.c_double, C.c_double, _dp, _dp,
                                              C.c_double, C.c_double, C.c_int, _dp, _dp]
        return cls._lib

    def set_threads(self, n):
        self._L.oracle_set_threads(self.h, int(n))

    def atimes_part(self, x, part):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        self._L.oracle_atimes_part(self.h, _d(x), _d(y), int(part))
        return y

    def atimes_rows(self, x, i0, i1):
        """Output rows [i0, i1) of the product (other rows are zero)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        self._L.oracle_atimes_rows(self.h, _d(x), _d(y), int(i0), int(i1))
        return y

    def cheb_eval(self, a, e0, e1, y):
        """z = sum_k a_k T_k(M~) y by Clenshaw (src/chebyshev.c:163-228)."""
        a = np.ascontiguousarray(a, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        z = np.zeros(self.n)
        self._L.oracle_cheb_eval(self.h, self.n, len(a), _d(a), float(e0), float(e1), _d(y),
                                 _d(z))
        return z

    def set_open(self, open_=True):
        """Make atimes / cheb_eval / bd_step use the free-space operator (an
        open system, periodic = 0)."""
        self._open = bool(open_)
        self._L.oracle_set_open(self.h, 1 if open_ else 0)

    def bd_step(self, x, dt, peclet, a, e0, e1, y, F=None, lj_e=0.0, lj_r0=2.0, lj_image=False):
        """One mid-point step from positions x with noise y; returns (x_new, z).
        lj_image: EV_LJ along the nearest-image vector (this library's BD
        engine) instead of the reference's primary-cell vector.  An open
        system (set_open) takes the plain pair vector."""
        x = np.array(x, dtype=np.float64).reshape(-1).copy()
        a = np.ascontiguousarray(a, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        Fp = None if F is None else np.ascontiguousarray(F, dtype=np.float64)
        z = np.zeros(self.n)
        self._L.oracle_bd_step_ex(self.h, self.version, self.np, *self.box, float(dt),
                                  float(peclet), len(a), _d(a), float(e0), float(e1), _d(y),
                                  None if Fp is None else _d(Fp), float(lj_e), float(lj_r0),
                                  2 if getattr(self, "_open", False) else (1 if lj_image else 0),
                                  _d(x), _d(z))
        return x, z

    def count_real_terms(self):
        return int(self._L.oracle_count_real_terms(self.h))

    def count_k(self):
        return int(self._L.oracle_count_k(self.h))

    def xi_by_tratio(self, tratio):
        return float(self._L.oracle_xi_by_tratio(*self.box, float(tratio)))


def lub_res2b(s):
    """The 22 lubrication-form resistance functions at distance s
    (oracle/oracle_lub.c, src/two-body-res.c:31)."""
    L = Oracle.lib()
    out = np.zeros(22)
    L.oracle_lub_res2b.argtypes = [C.c_double, _dp]
    L.oracle_lub_res2b(float(s), _d(out))
    return out


def lub_minv(version, s):
    """(M^inf)^-1 of two spheres at distance s: F 4 values, FT 10, FTS 22."""
    L = Oracle.lib()
    out = np.zeros(22)
    L.oracle_lub_minv.argtypes = [C.c_int, C.c_double, _dp]
    L.oracle_lub_minv(int(version), float(s), _d(out))
    return out[:(4, 10, 22)[version]]


def calc_lub(version, pos, box=None, u=None, lubmin2=0.0, lubmax=0.0, shear_mode=0,
             shear_shift=0.0):
    """f = L u for equal spheres (src/lub.c:164-575); box None: an open
    system."""
    L = Oracle.lib()
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    np_ = pos.shape[0]
    c = (3, 6, 11)[version]
    u = np.ascontiguousarray(u, dtype=np.float64)
    f = np.zeros(c * np_)
    periodic = box is not None
    lx, ly, lz = box if periodic else (0.0, 0.0, 0.0)
    L.oracle_calc_lub.argtypes = ([C.c_int, C.c_int, _dp, C.c_int] + [C.c_double] * 3
                                  + [C.c_int] + [C.c_double] * 3 + [_dp, _dp])
    L.oracle_calc_lub(int(version), np_, _d(pos), 1 if periodic else 0, float(lx), float(ly),
                      float(lz), int(shear_mode), float(shear_shift), float(lubmin2),
                      float(lubmax), _d(u), _d(f))
    return f


class Reference(_Backend):
    """The reference library compiled from its own sources (oracle/_ref)."""
    prefix = "ref_"
    so_path = REF_SO

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(REF_SO)

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = super().lib()
            lib.ref_xi_by_tratio.restype = C.c_double
            lib.ref_xi_by_tratio.argtypes = [C.c_void_p, C.c_double]
            lib.ref_atimes_notbl.argtypes = [C.c_void_p, _dp, _dp]
            lib.ref_matrix_notbl.argtypes = [C.c_void_p, _dp]
            lib.ref_cpu_times.argtypes = [C.c_void_p, _dp]
            lib.ref_cheb_coef.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp]
            lib.ref_cheb_eval.restype = C.c_double
            lib.ref_cheb_eval.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_double]
            lib.ref_cheb_eval_dense.argtypes = [C.c_int, _dp, C.c_int, _dp, _dp, _dp,
                                                C.c_double, C.c_double, _dp]
            lib.ref_cheb_eval_ewald.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp,
                                                C.c_double, C.c_double, _dp]
        return cls._lib

    def xi_by_tratio(self, tratio):
        return float(self._L.ref_xi_by_tratio(self.h, float(tratio)))

    def atimes_notbl(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        self._L.ref_atimes_notbl(self.h, _d(x), _d(y))
        return y

    def matrix_notbl(self):
        m = np.zeros((self.n, self.n))
        self._L.ref_matrix_notbl(self.h, _d(m))
        return m

    def cpu_times(self):
        out = np.zeros(3)
        self._L.ref_cpu_times(self.h, _d(out))
        return out
