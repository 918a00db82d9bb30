"""ctypes mirror of the libstokes_gb300 C ABI (include/stokes_abi.h,
include/stokes_gpu.h).

``StokesStruct`` is the Python image of ``struct stokes`` (src/stokes.h:27-154
of libstokes); ``System`` wraps one struct the way a libstokes caller would:
``stokes_init`` / ``stokes_set_np`` / ``stokes_set_l`` / ``stokes_set_xi`` and
direct member writes, then ``atimes_ewald_3all`` / ``make_matrix_mob_ewald_3all``.

There is no fallback: if libstokes_gb300.so is missing or fails to load, an
ImportError is raised.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib",
                        "libstokes_gb300.so")

STOKES_GPU_OK = 0
STOKES_GPU_EINVAL = 1
STOKES_GPU_ENOTPERIODIC = 2
STOKES_GPU_ECUDA = 3
STOKES_GPU_ENOMEM = 4
STOKES_GPU_ETIMEOUT = 5
STOKES_GPU_EACCURACY = 6
STOKES_GPU_ETOOBIG = 7
FP64 = 0
MIXED = 1
SOLVE_RES = 0
SOLVE_MOB_FTS = 1
SOLVE_MOB_LUB = 2


class TrajFrame(C.Structure):
    """struct stokes_traj_frame (include/stokes_traj.h)."""
    _fields_ = [("time", C.c_double), ("shear_shift", C.c_double)] + [
        (k, _dp) for k in ("x", "u", "o", "e", "f", "t", "s", "q", "xf")] + [
        ("rng", C.c_void_p)]


TRAJ_X, TRAJ_U, TRAJ_O, TRAJ_E, TRAJ_F, TRAJ_T, TRAJ_S, TRAJ_Q, TRAJ_XF, TRAJ_RNG = (
    1, 2, 4, 8, 16, 32, 64, 128, 256, 512)


class IterStruct(C.Structure):
    """struct iter (include/stokes_iter.h)."""
    _fields_ = [("solver", C.c_char_p), ("max", C.c_int), ("restart", C.c_int),
                ("eps", C.c_double), ("n", C.c_int), ("guess", _dp), ("flag_guess", C.c_int),
                ("debug", C.c_int), ("out", C.c_void_p), ("niter", C.c_int),
                ("res", C.c_double)]


class StokesStruct(C.Structure):
    """Byte-for-byte image of libstokes' struct stokes."""
    _fields_ = [
        ("version", C.c_int),
        ("np", C.c_int),
        ("nm", C.c_int),
        ("pos", _dp),
        ("a", _dp),
        ("rmin", C.c_double),
        ("twobody_nmax", C.c_int),
        ("twobody_lub", C.c_int),
        ("poly_table", _ip),
        ("twobody_f_list", C.c_void_p),
        ("slip", _dp),
        ("slip_a", _dp),
        ("slip_G32", _dp),
        ("slip_G30", _dp),
        ("slip_G52", _dp),
        ("slip_table", _ip),
        ("twobody_slip_f_list", C.c_void_p),
        ("Ui", C.c_double * 3),
        ("Oi", C.c_double * 3),
        ("Ei", C.c_double * 5),
        ("shear_mode", C.c_int),
        ("shear_rate", C.c_double),
        ("shear_shift", C.c_double),
        ("periodic", C.c_int),
        ("ewald_eps", C.c_double),
        ("rmax2", C.c_double),
        ("rmaxx", C.c_int), ("rmaxy", C.c_int), ("rmaxz", C.c_int),
        ("kmax", C.c_double),
        ("kmaxx", C.c_int), ("kmaxy", C.c_int), ("kmaxz", C.c_int),
        ("xi", C.c_double), ("xi2", C.c_double), ("xiaspi", C.c_double),
        ("xia2", C.c_double),
        ("pivol", C.c_double),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("ilx", C.c_int * 27), ("ily", C.c_int * 27), ("ilz", C.c_int * 27),
        ("self_a", C.c_double), ("self_c", C.c_double), ("self_m", C.c_double),
        ("flag_table", C.c_int),
        ("nr", C.c_int),
        ("rlx", _dp), ("rly", _dp), ("rlz", _dp),
        ("rmx", _ip), ("rmy", _ip), ("rmz", _ip),
        ("nk", C.c_int),
        ("ex", _dp), ("ey", _dp), ("ez", _dp),
        ("k", _dp), ("k1", _dp), ("k2", _dp), ("k3", _dp),
        ("ya", _dp), ("yb", _dp), ("yc", _dp), ("yg", _dp), ("yh", _dp),
        ("ym", _dp),
        ("lubmin2", C.c_double),
        ("lubmax", C.c_double),
        ("cpu1", C.c_double), ("cpu2", C.c_double), ("cpu3", C.c_double),
        ("it", C.c_void_p),
    ]


class BDParams(C.Structure):
    """struct stokes_gpu_bd_params (include/stokes_bd.h)."""
    _fields_ = [("peclet", C.c_double), ("dt", C.c_double), ("n_cheb", C.c_int),
                ("n_lanczos", C.c_int), ("cheb_eps", C.c_double), ("check_every", C.c_int),
                ("lj_e", C.c_double), ("lj_r0", C.c_double), ("seed", C.c_ulonglong),
                ("precision", C.c_int)]


class KIrandStruct(C.Structure):
    _fields_ = [("mt", C.c_ulong * 624), ("mti", C.c_int), ("Gaussian_has_saved", C.c_int),
                ("Gaussian_saved", C.c_double)]


class EVLJStruct(C.Structure):
    """struct EV_LJ (src/ev-LJ.h:26-51)."""
    _fields_ = [("n", C.c_int), ("flag", C.POINTER(C.c_int)), ("e", _dp), ("r0", _dp)]


class BDStruct(C.Structure):
    """struct BD_params (src/brownian.h:28-96)."""
    _fields_ = [("sys", C.c_void_p), ("rng", C.POINTER(KIrandStruct)), ("F", _dp), ("T", _dp),
                ("E", _dp), ("uf", _dp), ("of", _dp), ("ef", _dp), ("flag_noHI", C.c_int),
                ("flag_mat", C.c_int), ("flag_lub", C.c_int), ("flag_lub_B", C.c_int),
                ("t0", C.c_double), ("s0", C.c_double), ("st", C.c_double),
                ("br", C.c_void_p), ("bonds", C.c_void_p), ("groups", C.c_void_p),
                ("gamma", C.c_double), ("ev", C.c_void_p), ("ang", C.c_void_p),
                ("ev_dh", C.c_void_p), ("ev_LJ", C.POINTER(EVLJStruct)), ("cf", C.c_void_p),
                ("flag_Q", C.c_int), ("peclet", C.c_double), ("eps", C.c_double),
                ("n_minv", C.c_int), ("eig_minv", C.c_double * 2), ("a_minv", _dp),
                ("n_lub", C.c_int), ("eig_lub", C.c_double * 2), ("a_lub", _dp),
                ("scheme", C.c_int), ("BB_n", C.c_double), ("rmin", C.c_double),
                ("dt_lim", C.c_double)]


_SP = C.POINTER(StokesStruct)
ATIMES = C.CFUNCTYPE(None, C.c_int, _dp, _dp, C.c_void_p)
FUNC1 = C.CFUNCTYPE(C.c_double, C.c_double)

_SIGS = {
    # set-up
    "stokes_init": (_SP, []),
    "stokes_free": (None, [_SP]),
    "stokes_set_np": (None, [_SP, C.c_int, C.c_int]),
    "stokes_set_Ui": (None, [_SP, C.c_double, C.c_double, C.c_double]),
    "stokes_set_Oi": (None, [_SP, C.c_double, C.c_double, C.c_double]),
    "stokes_set_Ei": (None, [_SP] + [C.c_double] * 5),
    "stokes_set_shear": (None, [_SP, C.c_int, C.c_double]),
    "stokes_get_shear_shift": (C.c_double, [_SP, C.c_double, C.c_double, C.c_double]),
    "stokes_set_shear_shift": (None, [_SP, C.c_double, C.c_double, C.c_double]),
    "stokes_set_l": (None, [_SP, C.c_double, C.c_double, C.c_double]),
    "stokes_set_xi": (None, [_SP, C.c_double, C.c_double]),
    "xi_by_tratio": (C.c_double, [_SP, C.c_double]),
    "stokes_set_pos": (None, [_SP, _dp]),
    "stokes_set_pos_mobile": (None, [_SP, _dp]),
    "stokes_set_pos_fixed": (None, [_SP, _dp]),
    "stokes_set_radius": (None, [_SP, _dp]),
    "stokes_unset_radius": (None, [_SP]),
    "stokes_set_slip": (None, [_SP, _dp]),
    "stokes_unset_slip": (None, [_SP]),
    # operators
    "atimes_ewald_3all": (None, [C.c_int, _dp, _dp, C.c_void_p]),
    "atimes_ewald_3all_notbl": (None, [C.c_int, _dp, _dp, C.c_void_p]),
    "atimes_3all": (None, [C.c_int, _dp, _dp, C.c_void_p]),
    "atimes_nonewald_3all": (None, [C.c_int, _dp, _dp, C.c_void_p]),
    "make_matrix_mob_nonewald_3all": (None, [_SP, _dp]),
    "atimes_nonewald_3all_matrix": (None, [C.c_int, _dp, _dp, C.c_void_p]),
    "make_matrix_mob_ewald_3all": (None, [_SP, _dp]),
    "make_matrix_mob_ewald_3all_notbl": (None, [_SP, _dp]),
    "make_matrix_mob_3all": (None, [_SP, _dp]),
    "atimes_3all_matrix": (None, [C.c_int, _dp, _dp, C.c_void_p]),
    "atimes_ewald_3all_matrix_notbl": (None, [C.c_int, _dp, _dp, C.c_void_p]),
    "dot_prod_matrix": (None, [_dp, C.c_int, C.c_int, _dp, _dp]),
    "multiply_extmat_with_extvec_3fts": (None, [C.c_int, _dp, _dp, _dp]),
    # Chebyshev
    "chebyshev_coef": (None, [C.c_int, FUNC1, C.c_double, C.c_double, _dp]),
    "chebyshev_eval": (C.c_double, [C.c_int, _dp, C.c_double, C.c_double, C.c_double]),
    "chebyshev_eval_": (C.c_double, [C.c_int, _dp, C.c_double, C.c_double, C.c_double]),
    "chebyshev_eval_atimes": (None, [C.c_int, _dp, C.c_int, _dp, _dp, C.c_double,
                                     C.c_double, C.c_void_p, C.c_void_p]),
    "chebyshev_error_minvsqrt": (C.c_double, [C.c_int, _dp, _dp, C.c_void_p, C.c_void_p]),
    "chebyshev_error_Rsqrt": (C.c_double, [C.c_int, _dp, _dp, C.c_void_p, C.c_void_p]),
    # additive GPU API
    "stokes_gpu_last_error": (C.c_int, []),
    "stokes_gpu_last_error_message": (C.c_char_p, []),
    "stokes_gpu_set_error_mode": (None, [C.c_int]),
    "stokes_gpu_set_precision": (C.c_int, [_SP, C.c_int]),
    "stokes_gpu_get_precision": (C.c_int, [_SP, _ip]),
    "stokes_gpu_release": (C.c_int, [_SP]),
    "stokes_gpu_note_split": (None, [_SP]),
    "stokes_gpu_count_real_terms_dense": (C.c_int, [_SP, C.POINTER(C.c_longlong)]),
    "stokes_gpu_atimes": (C.c_int, [_SP, _dp, _dp]),
    # trajectory files (include/stokes_traj.h)
    "stokes_traj_create": (C.c_void_p, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "stokes_traj_open": (C.c_void_p, [C.c_char_p]),
    "stokes_traj_close": (None, [C.c_void_p]),
    "stokes_traj_append": (C.c_int, [C.c_void_p, C.c_void_p]),
    "stokes_traj_read": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "stokes_traj_nframes": (C.c_int, [C.c_void_p]),
    "stokes_traj_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_int), _dp, _dp, _dp]),
    # iterative solves (include/stokes_iter.h)
    "iter_init": (C.c_void_p, [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_int, _dp, C.c_int,
                               C.c_int, C.c_void_p]),
    "iter_free": (None, [C.c_void_p]),
    "stokes_set_iter": (None, [_SP, C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_int,
                               C.c_void_p]),
    "solve_iter": (None, [C.c_int, _dp, _dp, C.c_void_p, C.c_void_p, C.c_void_p]),
    "solve_mob_3fts_0": (None, [_SP, C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]),
    "stokes_gpu_solve": (C.c_int, [_SP, C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_double,
                                   C.POINTER(C.c_int), _dp]),
    "stokes_gpu_atimes_dev": (C.c_int, [_SP, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "stokes_gpu_atimes_noalloc": (C.c_int, [_SP, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p]),
    "stokes_gpu_matrix": (C.c_int, [_SP, _dp]),
    "stokes_gpu_matrix_dev": (C.c_int, [_SP, C.c_void_p, C.c_void_p, C.c_void_p]),
    "stokes_gpu_matvec_dev": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p]),
    "stokes_gpu_last_times": (C.c_int, [_SP, _dp]),
    "stokes_gpu_last_launches": (C.c_int, [_SP, _ip]),
    "stokes_gpu_profile_begin": (C.c_int, [_SP, C.c_int]),
    "stokes_gpu_kprof_begin": (C.c_int, [_SP, C.c_int]),
    "stokes_gpu_kprof_end": (C.c_int, [_SP, C.c_int, C.c_char_p, _dp, _ip, _ip]),
    "stokes_gpu_profile_end": (C.c_int, [_SP, _dp, _ip]),
    "stokes_gpu_count_real_terms": (C.c_int, [_SP, C.POINTER(C.c_longlong)]),
    "stokes_gpu_count_mixed_real_terms": (C.c_int, [_SP, C.POINTER(C.c_longlong)]),
    "stokes_gpu_peak_fma": (C.c_int, [C.c_int, _dp]),
    "stokes_gpu_test_stall_waits": (C.c_int, [C.c_int, C.c_longlong]),
    "stokes_gpu_mixed_split": (C.c_int, [_SP, _dp]),
    "stokes_gpu_selftest_tensor": (C.c_int, [_dp]),
    "stokes_gpu_selftest_tma": (C.c_int, [_dp]),
    # Brownian dynamics
    "KIrand_init": (C.POINTER(KIrandStruct), []),
    "KIrand_free": (None, [C.POINTER(KIrandStruct)]),
    "KIrand_init_genrand": (None, [C.POINTER(KIrandStruct), C.c_ulong]),
    "KIrand_genrand_int32": (C.c_ulong, [C.POINTER(KIrandStruct)]),
    "KIrand_genrand_res53": (C.c_double, [C.POINTER(KIrandStruct)]),
    "KIrand_genrand_real2": (C.c_double, [C.POINTER(KIrandStruct)]),
    "KIrand_Gaussian": (C.c_double, [C.POINTER(KIrandStruct)]),
    "stokes_gpu_bd_create": (C.c_int, [_SP, C.POINTER(BDParams), C.POINTER(C.c_void_p)]),
    "stokes_gpu_bd_destroy": (C.c_int, [C.c_void_p]),
    "stokes_gpu_bd_set_positions": (C.c_int, [C.c_void_p, _dp]),
    "stokes_gpu_bd_get_positions": (C.c_int, [C.c_void_p, _dp]),
    "stokes_gpu_bd_set_force": (C.c_int, [C.c_void_p, _dp, _dp]),
    "stokes_gpu_bd_estimate_bounds": (C.c_int, [C.c_void_p, _dp]),
    "stokes_gpu_bd_set_bounds": (C.c_int, [C.c_void_p, _dp]),
    "stokes_gpu_bd_noise": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "stokes_gpu_bd_step_noise": (C.c_int, [C.c_void_p, C.c_double, _dp]),
    "stokes_gpu_bd_run": (C.c_int, [C.c_void_p, C.c_double, C.c_int]),
    "stokes_gpu_bd_stats": (C.c_int, [C.c_void_p, _dp]),
    # batches
    "stokes_gpu_batch_create": (C.c_int, [C.POINTER(_SP), C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "stokes_gpu_batch_destroy": (C.c_int, [C.c_void_p]),
    "stokes_gpu_batch_size": (C.c_int, [C.c_void_p, _ip, _ip]),
    "stokes_gpu_batch_offsets": (C.c_int, [C.c_void_p, _ip, _ip]),
    "stokes_gpu_batch_set_positions": (C.c_int, [C.c_void_p, _dp]),
    "stokes_gpu_batch_atimes": (C.c_int, [C.c_void_p, _dp, _dp]),
    "stokes_gpu_batch_stats": (C.c_int, [C.c_void_p, _dp]),
    "stokes_gpu_batch_split": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp]),
    "stokes_gpu_lub": (C.c_int, [_SP, C.c_int, _dp, _dp]),
    "stokes_gpu_lub_dev": (C.c_int, [_SP, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p]),
    "stokes_gpu_lub_coefficients": (C.c_int, [_dp]),
    "calc_lub_3f": (None, [_SP, _dp, _dp]),
    "calc_lub_3ft": (None, [_SP, _dp, _dp]),
    "calc_lub_3fts": (None, [_SP, _dp, _dp]),
    "make_matrix_lub_3f": (None, [_SP, _dp]),
    "make_matrix_lub_3ft": (None, [_SP, _dp]),
    "make_matrix_lub_3fts": (None, [_SP, _dp]),
    "stokes_gpu_lub_matrix": (C.c_int, [_SP, C.c_int, _dp]),
    "stokes_gpu_lub_matrix_dev": (C.c_int, [_SP, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "stokes_gpu_batch_bd": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_int, _dp,
                                      _dp, C.c_ulonglong, C.c_int, _dp]),
    "stokes_gpu_vjp": (C.c_int, [_SP, _dp, _dp, _dp, _dp, _dp]),
    # libstokes' BD routines
    "EV_LJ_init": (C.POINTER(EVLJStruct), [C.c_int]),
    "EV_LJ_free": (None, [C.POINTER(EVLJStruct)]),
    "EV_LJ_scale": (None, [C.POINTER(EVLJStruct), C.c_double]),
    "BD_params_init": (C.POINTER(BDStruct),
                       [_SP, C.c_ulong, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int,
                        C.c_double, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                        C.c_void_p, C.POINTER(EVLJStruct), C.c_void_p, C.c_int, C.c_double,
                        C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                        C.c_double]),
    "BD_params_free": (None, [C.POINTER(BDStruct)]),
    "BD_params_get_fact": (C.c_double, [C.POINTER(BDStruct), C.c_double]),
    "BD_get_n": (C.c_int, [_SP]),
    "BD_calc_FB": (None, [C.POINTER(BDStruct), _dp]),
    "BD_evolve_mid": (C.c_double, [C.c_double, C.POINTER(BDStruct), _dp, _dp, C.c_double]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libstokes_gb300.so (raises ImportError when it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"libstokes_gb300: {path} is missing; run "
                          "`python -m libstokes_gb300.build` first")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def declared_symbols():
    """Names of every function the public headers declare."""
    return sorted(_SIGS)


def _d(a):
    return a.ctypes.data_as(_dp)


def ncomp(version: int) -> int:
    return (3, 6, 11)[version]


def kernel_profile(lib, sp, max_kernels: int = 16) -> dict:
    """Close the kernel profiling window of a system: {name: (ms, launches)}."""
    names = C.create_string_buffer(32 * max_kernels)
    ms = np.zeros(max_kernels)
    cnt = np.zeros(max_kernels, dtype=np.int32)
    nk = C.c_int()
    check(lib.stokes_gpu_kprof_end(sp, max_kernels, names, ms.ctypes.data_as(_dp),
                                   cnt.ctypes.data_as(_ip), C.byref(nk)))
    raw = names.raw
    out = {}
    for k in range(nk.value):
        nm = raw[32 * k:32 * k + 32].split(b"\0", 1)[0].decode()
        out[nm] = (float(ms[k]), int(cnt[k]))
    return out


class GPUError(RuntimeError):
    pass


def raise_if_failed():
    """After a drop-in (void) call in error mode 1: raise with the reason."""
    lib = load()
    rc = lib.stokes_gpu_last_error()
    if rc != STOKES_GPU_OK:
        raise GPUError(f"libstokes_gb300 status {rc}: "
                       f"{lib.stokes_gpu_last_error_message().decode()}")


def check(rc: int):
    if rc != STOKES_GPU_OK:
        lib = load()
        raise GPUError(f"libstokes_gb300 status {rc}: "
                       f"{lib.stokes_gpu_last_error_message().decode()}")


class System:
    """One struct stokes built through the library's own set-up calls."""

    def __init__(self, version: int, pos, box=None, xi=None, eps=1e-12, tratio=1.0,
                 periodic=True):
        """periodic=False builds an open system (src/stokes.c:339: the
        default of stokes_init) with neither a box nor a split."""
        self.lib = load()
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.version = int(version)
        self.np = pos.shape[0]
        self.sp = self.lib.stokes_init()
        s = self.sp.contents
        s.version = self.version
        self.lib.stokes_set_np(self.sp, self.np, self.np)
        self.lib.stokes_set_pos(self.sp, _d(pos))
        self._keep = []
        if not periodic:
            s.periodic = 0
            return
        s.periodic = 1
        self.lib.stokes_set_l(self.sp, *[float(b) for b in box])
        if xi is None:
            xi = self.lib.xi_by_tratio(self.sp, float(tratio))
        self.lib.stokes_set_xi(self.sp, float(xi), float(eps))

    def close(self):
        if getattr(self, "sp", None):
            # hand the library back the tables it allocated before it frees them
            self.restore_table()
            self.lib.stokes_free(self.sp)
            self.sp = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def s(self) -> StokesStruct:
        return self.sp.contents

    @property
    def n(self) -> int:
        return ncomp(self.version) * self.np

    def set_pos(self, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.lib.stokes_set_pos(self.sp, _d(pos))

    def set_radius(self, a):
        if a is None:
            self.lib.stokes_unset_radius(self.sp)
        else:
            a = np.ascontiguousarray(a, dtype=np.float64)
            self.lib.stokes_set_radius(self.sp, _d(a))

    def set_slip(self, g):
        if g is None:
            self.lib.stokes_unset_slip(self.sp)
        else:
            g = np.ascontiguousarray(g, dtype=np.float64)
            self.lib.stokes_set_slip(self.sp, _d(g))

    def set_misc(self, rmin=0.0, shear_mode=0, shear_shift=0.0):
        s = self.s
        s.rmin = float(rmin)
        s.shear_mode = int(shear_mode)
        s.shear_shift = float(shear_shift)

    def set_cube(self, nr_shell: int, nk_shell: int):
        """Full image cube |m| <= nr_shell (every image taken) and full k cube
        |m| <= nk_shell (kmax = 0): the 5-shell configuration of the N=64
        workload.  Arrays stay owned by this object."""
        s = self.s
        side = 2 * nr_shell + 1
        m = np.arange(-nr_shell, nr_shell + 1)
        m1, m2, m3 = [a.ravel() for a in np.meshgrid(m, m, m, indexing="ij")]
        rl = [np.ascontiguousarray(m1 * s.lx, dtype=np.float64),
              np.ascontiguousarray(m2 * s.ly, dtype=np.float64),
              np.ascontiguousarray(m3 * s.lz, dtype=np.float64)]
        rm = [np.ascontiguousarray(a, dtype=np.int32) for a in (m1, m2, m3)]
        self._keep = rl + rm
        # the library owns (and will free) the arrays it allocated: swap them
        # out and restore them before freeing
        # (addresses as integers: a pointer read from a ctypes Structure
        # aliases the member and would follow the reassignment below)
        self._orig = (s.nr,) + tuple(C.cast(p, C.c_void_p).value
                                     for p in (s.rlx, s.rly, s.rlz, s.rmx, s.rmy, s.rmz))
        s.nr = side ** 3
        s.rlx, s.rly, s.rlz = [_d(a) for a in rl]
        s.rmx, s.rmy, s.rmz = [a.ctypes.data_as(_ip) for a in rm]
        s.rmax2 = math.inf
        s.kmaxx = s.kmaxy = s.kmaxz = int(nk_shell)
        s.kmax = 0.0

    def restore_table(self):
        if getattr(self, "_orig", None):
            s = self.s
            nr, ax, ay, az, mx, my, mz = self._orig
            s.nr = nr
            s.rlx, s.rly, s.rlz = [C.cast(v, _dp) for v in (ax, ay, az)]
            s.rmx, s.rmy, s.rmz = [C.cast(v, _ip) for v in (mx, my, mz)]
            self._orig = None

    def set_precision(self, mode: int):
        check(self.lib.stokes_gpu_set_precision(self.sp, int(mode)))

    def atimes(self, x, notbl=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        f = self.lib.atimes_ewald_3all_notbl if notbl else self.lib.atimes_ewald_3all
        f(self.n, _d(x), _d(y), C.cast(self.sp, C.c_void_p))
        raise_if_failed()
        return y

    def atimes_checked(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        check(self.lib.stokes_gpu_atimes(self.sp, _d(x), _d(y)))
        return y

    def matrix(self, notbl=False):
        m = np.empty((self.n, self.n))
        f = (self.lib.make_matrix_mob_ewald_3all_notbl if notbl
             else self.lib.make_matrix_mob_ewald_3all)
        f(self.sp, _d(m))
        raise_if_failed()
        return m

    def atimes_matrix(self, x, notbl=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        f = (self.lib.atimes_ewald_3all_matrix_notbl if notbl
             else self.lib.atimes_3all_matrix)
        f(self.n, _d(x), _d(y), C.cast(self.sp, C.c_void_p))
        raise_if_failed()
        return y

    # the dispatchers (src/ewald.c:433-505) and the free-space operator
    # (src/non-ewald.c:330-706)
    def atimes_3all(self, x):
        return self._vec(self.lib.atimes_3all, x)

    def atimes_3all_matrix(self, x):
        return self._vec(self.lib.atimes_3all_matrix, x)

    def matrix_3all(self):
        return self._mat(self.lib.make_matrix_mob_3all)

    def atimes_nonewald(self, x):
        return self._vec(self.lib.atimes_nonewald_3all, x)

    def atimes_nonewald_matrix(self, x):
        return self._vec(self.lib.atimes_nonewald_3all_matrix, x)

    def matrix_nonewald(self):
        return self._mat(self.lib.make_matrix_mob_nonewald_3all)

    def _vec(self, f, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        f(self.n, _d(x), _d(y), C.cast(self.sp, C.c_void_p))
        raise_if_failed()
        return y

    def _mat(self, f):
        m = np.empty((self.n, self.n))
        f(self.sp, _d(m))
        raise_if_failed()
        return m

    def times(self):
        out = np.zeros(3)
        check(self.lib.stokes_gpu_last_times(self.sp, _d(out)))
        return out

    def close_table_override(self):
        self.restore_table()
