"""Generate the golden fixtures of tests/golden/ from the reference library.

Runs only where the reference checkout exists (it compiles the reference's
own sources with oracle/Makefile.ref into oracle/_ref/ and calls them through
oracle/ref_driver.c).  The fixtures it writes are small .npz/.json files that
travel with the repository, so the tests never need the reference itself:

  struct_stokes_layout.json  member offsets / size of libstokes' struct stokes
  setup.npz                  Ewald split, cutoffs and image tables
  products.npz               atimes_ewald_3all / make_matrix_mob_ewald_3all
                             outputs (F, FT, FTS; equal, unequal radii, slip,
                             both shear modes, rmin clamp, _notbl variants,
                             the 8-sphere simple-cubic test of
                             test/check-ewald.c, the N=64 5-shell workload)
  chebyshev.npz              chebyshev_coef / chebyshev_eval /
                             chebyshev_eval_atimes outputs
  bd.npz                     BD_calc_FB noise and BD_evolve_mid trajectories
                             (F and FT, EV_LJ, quaternions, shear, dt halving)
                             of the reference's own brownian.c

    python tests/golden/make_golden.py [/path/to/libstokes]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference, build_reference  # noqa: E402
from libstokes_gb300.workloads import rsa_positions  # noqa: E402

STRUCT_FIELDS = [
    "version", "np", "nm", "pos", "a", "rmin", "twobody_nmax", "twobody_lub",
    "poly_table", "twobody_f_list", "slip", "slip_a", "slip_G32", "slip_G30",
    "slip_G52", "slip_table", "twobody_slip_f_list", "Ui", "Oi", "Ei",
    "shear_mode", "shear_rate", "shear_shift", "periodic", "ewald_eps", "rmax2",
    "rmaxx", "rmaxy", "rmaxz", "kmax", "kmaxx", "kmaxy", "kmaxz", "xi", "xi2",
    "xiaspi", "xia2", "pivol", "lx", "ly", "lz", "ilx", "ily", "ilz", "self_a",
    "self_c", "self_m", "flag_table", "nr", "rlx", "rly", "rlz", "rmx", "rmy",
    "rmz", "nk", "ex", "ey", "ez", "k", "k1", "k2", "k3", "ya", "yb", "yc", "yg",
    "yh", "ym", "lubmin2", "lubmax", "cpu1", "cpu2", "cpu3", "it",
]


def layout(ref_root: str) -> dict:
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "stokes.h"',
           "int main(void){", 'printf("{\\"sizeof\\": %zu", sizeof(struct stokes));']
    for f in STRUCT_FIELDS:
        src.append(f'printf(", \\"{f}\\": %zu", offsetof(struct stokes, {f}));')
    src += ['printf("}\\n");', "return 0;}"]
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "lay.c")
        exe = os.path.join(d, "lay")
        open(c, "w").write("\n".join(src))
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "oracle", "ref_stubs", "inc"),
                               "-I", os.path.join(ref_root, "src"), c, "-o", exe])
        return json.loads(subprocess.check_output([exe]).decode())


BD_FIELDS = ["sys", "rng", "F", "T", "E", "uf", "of", "ef", "flag_noHI", "flag_mat",
             "flag_lub", "flag_lub_B", "t0", "s0", "st", "br", "bonds", "groups", "gamma", "ev",
             "ang", "ev_dh", "ev_LJ", "cf", "flag_Q", "peclet", "eps", "n_minv", "eig_minv",
             "a_minv", "n_lub", "eig_lub", "a_lub", "scheme", "BB_n", "rmin", "dt_lim"]


def bd_layouts(ref_root: str) -> dict:
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "stokes.h"',
           '#include "KIrand.h"', '#include "ev-LJ.h"', '#include "brownian.h"',
           "int main(void){", 'printf("{");']
    items = [("BD_params", f) for f in BD_FIELDS]
    items += [("KIrand", f) for f in ("mt", "mti", "Gaussian_has_saved", "Gaussian_saved")]
    items += [("EV_LJ", f) for f in ("n", "flag", "e", "r0")]
    for k, (st, f) in enumerate(items):
        sep = "" if k == 0 else ", "
        src.append(f'printf("{sep}\\"{st}.{f}\\": %zu", offsetof(struct {st}, {f}));')
    for st in ("BD_params", "KIrand", "EV_LJ"):
        src.append(f'printf(", \\"{st}.sizeof\\": %zu", sizeof(struct {st}));')
    src += ['printf("}\\n");', "return 0;}"]
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "lay.c")
        exe = os.path.join(d, "lay")
        open(c, "w").write("\n".join(src))
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "oracle", "ref_stubs", "inc"),
                               "-I", os.path.join(ref_root, "src"), c, "-o", exe])
        return json.loads(subprocess.check_output([exe]).decode())


def mk(version, pos, box, tratio=1.0, eps=1e-12, a=None, slip=None, shear=(0, 0.0),
       rmin=0.0, cube=None):
    r = Reference(version, pos, box)
    if a is not None:
        r.set_radius(a)
    if slip is not None:
        r.set_slip(slip)
    r.set_split(r.xi_by_tratio(tratio), eps)
    if cube is not None:
        r.set_cube(*cube)
    r.set_misc(rmin, shear[0], shear[1])
    return r


BD_CASES = [
    # name, version, N, phi, pos seed, rng seed, Pe, dt, steps, n_minv,
    # LJ (e, r0) or None, BD->rmin, dt_lim, shear (mode, rate), with F/T, with q
    ("f_lj", 0, 27, 0.20, 3, 42, 1.0, 1e-3, 3, 20, (1.0, 2.0), 0.0, 1e-12, (0, 0.0), False, False),
    ("f_halving", 0, 27, 0.20, 5, 43, 1.0, 1e-2, 3, 20, (1.0, 2.0), 0.9, 1e-4, (0, 0.0), True, False),
    ("ft_q", 1, 20, 0.15, 6, 44, 2.0, 1e-3, 2, 24, (0.5, 2.0), 0.0, 1e-12, (0, 0.0), True, True),
    ("f_shear", 0, 24, 0.20, 7, 45, 1.0, 1e-3, 2, 20, None, 0.0, 1e-12, (1, 2.0), False, False),
]
# open systems (periodic = 0, src/brownian.c:336 and src/ev-LJ.c:234): the
# free-space operator, no images in EV_LJ or in the overlap check
BD_OPEN_CASES = [
    ("open_f_lj", 0, 27, 0.20, 3, 46, 1.0, 1e-3, 3, 20, (1.0, 2.0), 0.0, 1e-12, (0, 0.0), True, False),
    ("open_ft_halving", 1, 20, 0.25, 9, 47, 1.0, 2e-2, 3, 24, (1.0, 2.0), 0.9, 1e-4, (0, 0.0), True, False),
]


def bd_fixtures(cases=None, periodic=True) -> dict:
    """BD_calc_FB / BD_evolve_mid of the reference on small periodic systems.
    ARPACK is absent, so the bounds are the extreme eigenvalues of the
    reference's dense mobility matrix widened by (0.8, 1.05); BD->eps = 10
    keeps the re-estimate branch off."""
    import ctypes as C
    so = os.path.join(ROOT, "oracle", "_ref", "libstokes_ref_bd.so")
    lib = C.CDLL(so)
    dp = C.POINTER(C.c_double)
    d = lambda a: None if a is None else a.ctypes.data_as(dp)  # noqa: E731
    lib.ref_new.restype = C.c_void_p
    lib.ref_new.argtypes = [C.c_int, C.c_int, dp, C.c_double, C.c_double, C.c_double]
    lib.ref_free.argtypes = [C.c_void_p]
    lib.ref_xi_by_tratio.restype = C.c_double
    lib.ref_xi_by_tratio.argtypes = [C.c_void_p, C.c_double]
    lib.ref_set_split.argtypes = [C.c_void_p, C.c_double, C.c_double]
    lib.ref_matrix.argtypes = [C.c_void_p, dp]
    lib.ref_matrix_nonewald.argtypes = [C.c_void_p, dp]
    lib.ref_set_periodic.argtypes = [C.c_void_p, C.c_int]
    lib.refbd_set_shear.argtypes = [C.c_void_p, C.c_int, C.c_double]
    lib.refbd_calc_fb.argtypes = [C.c_void_p, C.c_ulong, C.c_double, C.c_int, C.c_double,
                                  C.c_double, C.c_double, dp]
    lib.refbd_run.argtypes = [C.c_void_p, C.c_ulong, C.c_double, C.c_double, C.c_int, C.c_int,
                              C.c_double, C.c_double, C.c_double, dp, dp, C.c_int, C.c_double,
                              C.c_double, C.c_double, C.c_double, dp, dp, dp, dp, dp, dp]
    out = {}
    for (name, ver, n, phi, pseed, rseed, pe, dt, steps, nminv, lj, bdrmin, dtlim, shear,
         with_ft, with_q) in (BD_CASES if cases is None else cases):
        pos, L = rsa_positions(n, phi, seed=pseed)
        c = (3, 6, 11)[ver]
        h = lib.ref_new(ver, n, d(pos), L, L, L)
        lib.ref_set_split(h, lib.ref_xi_by_tratio(h, 1.0), 1e-12)
        if shear[0]:
            lib.refbd_set_shear(h, shear[0], shear[1])
        M = np.zeros((c * n, c * n))
        if periodic:
            lib.ref_matrix(h, d(M))
        else:
            lib.ref_set_periodic(h, 0)
            lib.ref_matrix_nonewald(h, d(M))
        ev = np.linalg.eigvalsh(0.5 * (M + M.T))
        eig = np.array([0.8 * ev[0], 1.05 * ev[-1]])
        rng = np.random.default_rng(pseed + 1000)
        F = 0.3 * rng.standard_normal(3 * n) if with_ft else None
        T = 0.3 * rng.standard_normal(3 * n) if (with_ft and ver > 0) else None
        q = None
        if with_q:
            q = rng.standard_normal((n, 4))
            q /= np.linalg.norm(q, axis=1, keepdims=True)
            q = q.ravel().copy()
        lje = lj0 = None
        if lj is not None:
            lje = np.full(n, lj[0])
            lj0 = np.full(n, lj[1])
        nb = (3 if ver == 0 else 6) * n
        z = np.zeros(nb)
        lib.refbd_calc_fb(h, rseed + 100, pe, nminv, eig[0], eig[1], 10.0, d(z))
        x = pos.ravel().copy()
        traj = np.zeros((steps, 3 * n))
        dts = np.zeros(steps)
        q0 = None if q is None else q.copy()
        lib.refbd_run(h, rseed, pe, dt, steps, nminv, eig[0], eig[1], 10.0, d(lje), d(lj0), 1,
                      bdrmin, dtlim, 0.0, 0.0, d(F), d(T), d(x), d(q), d(traj), d(dts))
        lib.ref_free(h)
        rec = dict(version=ver, pos=pos.ravel(), box=L, eig=eig, z_fb=z, fb_seed=rseed + 100,
                   seed=rseed, peclet=pe, dt=dt, n_minv=nminv, bd_rmin=bdrmin, dt_lim=dtlim,
                   shear=np.array(shear, float), traj=traj, dts=dts, periodic=int(periodic),
                   lj=np.array(lj if lj is not None else (0.0, 0.0)))
        if F is not None:
            rec["F"] = F
        if T is not None:
            rec["T"] = T
        if q is not None:
            rec["q0"] = q0
            rec["q1"] = q
        for k, v in rec.items():
            out[f"{name}:{k}"] = np.asarray(v)
        print(f"bd {name}: dts {dts}, max displacement {np.abs(traj[-1] - pos.ravel()).max():.3e}")
    return out


def nonewald_fixtures() -> dict:
    """The free-space operator (src/non-ewald.c): products and dense
    matrices of the reference for every branch, the two-sphere layout of
    test/check-minv.c:412-515 and a larger product."""
    out = {}
    rng = np.random.default_rng(2025)
    N = 12
    pos = rng.uniform(0.0, 1.0, (N, 3)) * np.array([8.0, 9.0, 10.0])
    arad = rng.uniform(0.5, 1.5, N)
    aslip_r = rng.uniform(0.7, 1.3, N)
    gslip = rng.uniform(0.0, 0.5, N)
    cases = {"mono": {}, "poly": dict(a=arad), "slip": dict(a=aslip_r, slip=gslip),
             "slipmono": dict(slip=gslip), "rmin": dict(rmin=1.5)}
    for v in (0, 1, 2):
        for cname, kw in cases.items():
            name = f"r12_v{v}_{cname}"
            r = mk(v, pos, (8.0, 9.0, 10.0), **kw)
            out[f"{name}/meta"] = np.array([v, kw.get("rmin", 0.0)])
            out[f"{name}/pos"] = pos
            if "a" in kw:
                out[f"{name}/a"] = kw["a"]
            if "slip" in kw:
                out[f"{name}/slip"] = kw["slip"]
            x = rng.standard_normal(r.n)
            out[f"{name}/x"] = x
            out[f"{name}/y"] = r.atimes_nonewald(x)
            out[f"{name}/mat"] = r.matrix_nonewald()
    # two spheres on the z axis at r = 2.5 (test/test-all.c:114,128)
    pair = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.5]])
    r = mk(2, pair, (8.0, 9.0, 10.0))
    out["pair_ez/meta"] = np.array([2, 0.0])
    out["pair_ez/pos"] = pair
    out["pair_ez/mat"] = r.matrix_nonewald()
    # a larger FTS product (N=200 non-overlapping spheres, phi 0.2 packing)
    pos200, _ = rsa_positions(200, 0.20, seed=11)
    r = mk(2, pos200, (8.0, 9.0, 10.0))
    x = rng.standard_normal(r.n)
    out["n200_v2_mono/meta"] = np.array([2, 0.0])
    out["n200_v2_mono/pos"] = pos200
    out["n200_v2_mono/x"] = x
    out["n200_v2_mono/y"] = r.atimes_nonewald(x)
    return out


# (name, version, n, phi, position seed, periodic, lubmin2, lubmax, shear (mode, shift))
LUB_CASES = [
    ("lub_f_periodic", 0, 40, 0.30, 61, True, 2.0001 ** 2, 3.0, (0, 0.0)),
    ("lub_ft_periodic", 1, 30, 0.30, 62, True, 2.0001 ** 2, 3.5, (0, 0.0)),
    ("lub_f_open", 0, 25, 0.25, 63, False, 0.0, 4.0, (0, 0.0)),
    ("lub_ft_open", 1, 20, 0.25, 64, False, 2.001 ** 2, 3.2, (0, 0.0)),
    ("lub_ft_nolimit", 1, 12, 0.20, 65, True, 0.0, 0.0, (0, 0.0)),
    ("lub_f_small_box", 0, 6, 0.25, 66, True, 0.0, 3.0, (0, 0.0)),
    ("lub_f_shear1", 0, 30, 0.30, 67, True, 2.0001 ** 2, 3.0, (1, 2.3)),
    ("lub_ft_shear2", 1, 20, 0.30, 68, True, 2.0001 ** 2, 3.0, (2, -1.7)),
    ("lub_fts_periodic", 2, 24, 0.30, 69, True, 2.0001 ** 2, 3.0, (0, 0.0)),
    ("lub_fts_open", 2, 15, 0.25, 70, False, 2.001 ** 2, 3.5, (0, 0.0)),
    ("lub_fts_shear1", 2, 16, 0.30, 71, True, 2.0001 ** 2, 3.0, (1, 1.9)),
]


# BD_calc_FB with the lubrication noise (flag_lub_B = 1, Chebyshev form):
# (name, version, N, phi, placement seed, lubmin2, lubmax, n_minv, n_lub, rng seed)
LUBNOISE_CASES = [
    ("lubnoise_f", 0, 30, 0.30, 91, 2.0001 ** 2, 3.0, 20, 20, 93),
    ("lubnoise_ft", 1, 24, 0.30, 92, 2.0001 ** 2, 3.0, 20, 24, 94),
]


# the reference's dense lubrication matrices (src/lub-matrix.c):
# (name, version, N, phi, placement seed, periodic, lubmin2, lubmax, shear)
LUBMAT_CASES = [
    ("lubmat_f_periodic", 0, 14, 0.30, 101, True, 2.0001 ** 2, 3.0, (0, 0.0)),
    ("lubmat_ft_shear1", 1, 12, 0.30, 102, True, 2.0001 ** 2, 3.0, (1, 1.3)),
    ("lubmat_ft_nolimit", 1, 8, 0.20, 106, True, 2.0001 ** 2, 0.0, (0, 0.0)),
    ("lubmat_fts_periodic", 2, 10, 0.30, 103, True, 2.0001 ** 2, 3.0, (0, 0.0)),
    ("lubmat_fts_open", 2, 10, 0.25, 104, False, 2.001 ** 2, 3.5, (0, 0.0)),
    ("lubmat_fts_shear2", 2, 8, 0.30, 105, True, 2.0001 ** 2, 3.0, (2, -0.7)),
]


def lub_fixtures() -> dict:
    """The reference's lubrication correction f = L u (src/lub.c:164-575,
    equal spheres) on small systems, its two-body functions
    (src/two-body-res.c:31, src/f.c:183, src/ft.c:414) on a grid of s, the
    lubrication noise of BD_calc_FB and the dense lubrication matrices
    (src/lub-matrix.c)."""
    import ctypes as C
    so = os.path.join(ROOT, "oracle", "_ref", "libstokes_ref_bd.so")
    lib = C.CDLL(so)
    dp = C.POINTER(C.c_double)
    d = lambda a: None if a is None else a.ctypes.data_as(dp)  # noqa: E731
    lib.ref_new.restype = C.c_void_p
    lib.ref_new.argtypes = [C.c_int, C.c_int, dp, C.c_double, C.c_double, C.c_double]
    lib.ref_free.argtypes = [C.c_void_p]
    lib.ref_set_periodic.argtypes = [C.c_void_p, C.c_int]
    lib.ref_set_misc.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_double]
    lib.refbd_calc_lub.argtypes = [C.c_void_p, C.c_double, C.c_double, dp, dp]
    lib.ref_res2b.argtypes = [C.c_double, dp]
    lib.ref_minv.argtypes = [C.c_int, C.c_double, dp]
    out = {}
    grid = np.concatenate([2.0 + np.logspace(-6, 0, 25), np.linspace(3.05, 12.0, 20)])
    res = np.zeros((len(grid), 22))
    minv = np.zeros((2, len(grid), 22))
    for q, sv in enumerate(grid):
        lib.ref_res2b(float(sv), d(res[q]))
        for v in (0, 1):
            lib.ref_minv(v, float(sv), d(minv[v, q]))
    minv_fts = np.zeros((len(grid), 22))
    for q, sv in enumerate(grid):
        lib.ref_minv(2, float(sv), d(minv_fts[q]))
    out["grid_s"] = grid
    out["grid_res2b"] = res
    out["grid_minv_f"] = minv[0, :, :4]
    out["grid_minv_ft"] = minv[1, :, :10]
    out["grid_minv_fts"] = minv_fts
    for name, ver, n, phi, pseed, periodic, lubmin2, lubmax, shear in LUB_CASES:
        pos, L = rsa_positions(n, phi, seed=pseed)
        c = (3, 6, 11)[ver]
        u = np.random.default_rng(pseed + 1000).standard_normal(c * n)
        h = lib.ref_new(ver, n, d(pos), L, L, L)
        if not periodic:
            lib.ref_set_periodic(h, 0)
        if shear[0]:
            lib.ref_set_misc(h, 0.0, shear[0], shear[1])
        f = np.zeros(c * n)
        lib.refbd_calc_lub(h, lubmin2, lubmax, d(u), d(f))
        lib.ref_free(h)
        out[f"{name}_meta"] = np.array([ver, n, L, 1.0 if periodic else 0.0, lubmin2, lubmax,
                                        shear[0], shear[1]])
        out[f"{name}_pos"] = pos
        out[f"{name}_u"] = u
        out[f"{name}_f"] = f
    # the lubrication noise of BD_calc_FB: bounds of M and L from their dense
    # matrices (ARPACK is absent), widened by (0.8, 1.05); BD->eps = 10 keeps
    # the re-estimates off
    lib.ref_xi_by_tratio.restype = C.c_double
    lib.ref_xi_by_tratio.argtypes = [C.c_void_p, C.c_double]
    lib.ref_set_split.argtypes = [C.c_void_p, C.c_double, C.c_double]
    lib.ref_matrix.argtypes = [C.c_void_p, dp]
    lib.refbd_calc_fb_lub.argtypes = [C.c_void_p, C.c_ulong, C.c_double, C.c_int, C.c_double,
                                      C.c_double, C.c_int, C.c_double, C.c_double, C.c_double,
                                      C.c_double, C.c_double, dp]
    for name, ver, n, phi, pseed, lubmin2, lubmax, nminv, nlub, rseed in LUBNOISE_CASES:
        pos, L = rsa_positions(n, phi, seed=pseed)
        c = (3, 6)[ver]
        h = lib.ref_new(ver, n, d(pos), L, L, L)
        lib.ref_set_split(h, lib.ref_xi_by_tratio(h, 1.0), 1e-12)
        M = np.zeros((c * n, c * n))
        lib.ref_matrix(h, d(M))
        ev = np.linalg.eigvalsh(0.5 * (M + M.T))
        eig = np.array([0.8 * ev[0], 1.05 * ev[-1]])
        Lm = np.zeros((c * n, c * n))
        for k in range(c * n):
            e = np.zeros(c * n)
            e[k] = 1.0
            col = np.zeros(c * n)
            lib.refbd_calc_lub(h, lubmin2, lubmax, d(e), d(col))
            Lm[:, k] = col
        evl = np.linalg.eigvalsh(0.5 * (Lm + Lm.T))
        eigl = np.array([0.8 * max(evl[0], 0.0), 1.05 * evl[-1]])
        z = np.zeros(c * n)
        lib.refbd_calc_fb_lub(h, rseed, 1.0, nminv, eig[0], eig[1], nlub, eigl[0], eigl[1], 10.0,
                              lubmin2, lubmax, d(z))
        lib.ref_free(h)
        out[f"{name}_meta"] = np.array([ver, n, L, lubmin2, lubmax, nminv, nlub, rseed])
        out[f"{name}_pos"] = pos
        out[f"{name}_eig"] = eig
        out[f"{name}_eigl"] = eigl
        out[f"{name}_z"] = z
        out[f"{name}_lev"] = np.array([evl[0], evl[-1]])
    lib.refbd_matrix_lub.argtypes = [C.c_void_p, C.c_double, C.c_double, dp]
    for name, ver, n, phi, pseed, periodic, lubmin2, lubmax, shear in LUBMAT_CASES:
        pos, L = rsa_positions(n, phi, seed=pseed)
        c = (3, 6, 11)[ver]
        h = lib.ref_new(ver, n, d(pos), L, L, L)
        if not periodic:
            lib.ref_set_periodic(h, 0)
        if shear[0]:
            lib.ref_set_misc(h, 0.0, shear[0], shear[1])
        mat = np.zeros((c * n, c * n))
        lib.refbd_matrix_lub(h, lubmin2, lubmax, d(mat))
        lib.ref_free(h)
        out[f"{name}_meta"] = np.array([ver, n, L, 1.0 if periodic else 0.0, lubmin2, lubmax,
                                        shear[0], shear[1]])
        out[f"{name}_pos"] = pos
        out[f"{name}_mat"] = mat
    return out


def write_lub(ref_root: str | None = None):
    """Only the lubrication fixtures (tests/golden/lub.npz)."""
    ref_root = ref_root or os.environ.get("LIBSTOKES_REF")
    if not ref_root or build_reference(ref_root) is None:
        raise SystemExit("usage: make_golden.py <libstokes checkout> (or set LIBSTOKES_REF)")
    np.savez_compressed(os.path.join(HERE, "lub.npz"), **lub_fixtures())


def main(ref_root: str | None = None):
    """ref_root: the libstokes checkout (argument or $LIBSTOKES_REF)."""
    ref_root = ref_root or os.environ.get("LIBSTOKES_REF")
    if not ref_root:
        raise SystemExit("usage: make_golden.py <libstokes checkout> (or set LIBSTOKES_REF)")
    if build_reference(ref_root) is None:
        raise SystemExit(f"reference checkout not found under {ref_root}")
    json.dump(layout(ref_root), open(os.path.join(HERE, "struct_stokes_layout.json"), "w"),
              indent=1)

    # ---- set-up: splits and image tables --------------------------------
    setup = {}
    boxes = [((5.0, 5.0, 5.0), 1.0, 1e-12), ((8.0, 9.0, 10.0), 1.0, 1e-12),
             ((24.07, 24.07, 24.07), 1.0, 1e-12), ((10.0, 5.0, 5.0), 4.0, 1e-10),
             ((6.0, 6.0, 12.0), 0.5, 1e-6)]
    for q, (box, tr, eps) in enumerate(boxes):
        r = mk(0, np.zeros((1, 3)), box, tratio=tr, eps=eps)
        sp = r.split()
        rl, rm = r.table()
        setup[f"c{q}_box"] = np.array(box)
        setup[f"c{q}_tr_eps"] = np.array([tr, eps])
        setup[f"c{q}_split"] = np.array([sp["xi"], sp["rmax2"], sp["kmax"], sp["self_a"],
                                         sp["self_c"], sp["self_m"], sp["pivol"], sp["nr"]]
                                        + list(sp["kmaxxyz"]))
        setup[f"c{q}_rl"] = rl
        setup[f"c{q}_rm"] = rm
    np.savez_compressed(os.path.join(HERE, "setup.npz"), **setup)

    # ---- products --------------------------------------------------------
    prod = {}
    rng = np.random.default_rng(2024)

    def record(name, r, x, with_matrix=True, notbl=False):
        prod[f"{name}/x"] = x
        prod[f"{name}/y"] = r.atimes(x)
        if with_matrix:
            prod[f"{name}/mat"] = r.matrix()
        if notbl:
            prod[f"{name}/y_notbl"] = r.atimes_notbl(x)
            if with_matrix:
                prod[f"{name}/mat_notbl"] = r.matrix_notbl()

    # simple-cubic 8 spheres of test/check-ewald.c:46-195 (phi 0.2, tr 1, eps 1e-12)
    phi = 0.2
    l = (np.pi / 0.75 / phi) ** (1.0 / 3.0)
    sc = np.array([[0, 0, 0], [l, 0, 0], [0, l, 0], [0, 0, l], [l, l, 0], [l, 0, l],
                   [0, l, l], [l, l, l]], dtype=float)
    for v in (0, 1, 2):
        name = f"sc8_v{v}"
        r = mk(v, sc, (2 * l,) * 3)
        prod[f"{name}/meta"] = np.array([v, 2 * l, 2 * l, 2 * l, 1.0, 1e-12, 0, 0.0, 0.0])
        prod[f"{name}/pos"] = sc
        record(name, r, np.ones(r.n))

    # random 12 spheres in a rectangular box: every branch
    N = 12
    box = (8.0, 9.0, 10.0)
    pos = rng.uniform(0.0, 1.0, (N, 3)) * np.array(box)
    arad = rng.uniform(0.5, 1.5, N)
    aslip_r = rng.uniform(0.7, 1.3, N)
    gslip = rng.uniform(0.0, 0.5, N)
    cases = {
        "mono": {}, "poly": dict(a=arad), "slip": dict(a=aslip_r, slip=gslip),
        "slipmono": dict(slip=gslip), "shear1": dict(shear=(1, 1.7)),
        "shear2": dict(shear=(2, -2.3)), "rmin": dict(rmin=1.5),
    }
    for v in (0, 1, 2):
        for cname, kw in cases.items():
            name = f"r12_v{v}_{cname}"
            r = mk(v, pos, box, **kw)
            sh = kw.get("shear", (0, 0.0))
            prod[f"{name}/meta"] = np.array([v, *box, 1.0, 1e-12, sh[0], sh[1],
                                             kw.get("rmin", 0.0)])
            prod[f"{name}/pos"] = pos
            if "a" in kw:
                prod[f"{name}/a"] = kw["a"]
            if "slip" in kw:
                prod[f"{name}/slip"] = kw["slip"]
            record(name, r, rng.standard_normal(r.n), notbl=True)

    # the 5-shell N=64 F workload (phi 0.10, xi = sqrt(pi)/L)
    pos64, L64 = rsa_positions(64, 0.10, seed=42)
    r = mk(0, pos64, (L64,) * 3, cube=(5, 5))
    name = "n64_5shell_v0"
    prod[f"{name}/meta"] = np.array([0, L64, L64, L64, 1.0, 1e-12, 0, 0.0, 0.0])
    prod[f"{name}/pos"] = pos64
    prod[f"{name}/cube"] = np.array([5, 5])
    record(name, r, np.random.default_rng(7).standard_normal(r.n), with_matrix=False)

    # a larger FTS case (N=40, phi 0.3) for the product only
    pos40, L40 = rsa_positions(40, 0.30, seed=5)
    r = mk(2, pos40, (L40,) * 3)
    name = "n40_fts_phi0.30"
    prod[f"{name}/meta"] = np.array([2, L40, L40, L40, 1.0, 1e-12, 0, 0.0, 0.0])
    prod[f"{name}/pos"] = pos40
    record(name, r, rng.standard_normal(r.n), with_matrix=False)
    np.savez_compressed(os.path.join(HERE, "products.npz"), **prod)

    # ---- Chebyshev -------------------------------------------------------
    lib = Reference.lib()
    import ctypes as C
    dp = C.POINTER(C.c_double)
    ch = {}
    for q, (nc, which, x0, x1) in enumerate([(30, 0, 0.05, 2.0), (50, 0, 0.1, 10.0),
                                             (20, 1, 0.5, 3.0), (100, 0, 0.01, 1.0)]):
        a = np.zeros(nc)
        lib.ref_cheb_coef(nc, which, x0, x1, a.ctypes.data_as(dp))
        xs = np.linspace(x0, x1, 17)
        ev = np.array([lib.ref_cheb_eval(nc, a.ctypes.data_as(dp), x0, x1, float(t)) for t in xs])
        ch[f"c{q}_args"] = np.array([nc, which, x0, x1])
        ch[f"c{q}_a"] = a
        ch[f"c{q}_xs"] = xs
        ch[f"c{q}_eval"] = ev
    # Chebyshev M^{-1/2} y on a dense SPD matrix
    n = 24
    A = rng.standard_normal((n, n))
    M = A @ A.T / n + np.eye(n)
    w = np.linalg.eigvalsh(M)
    e0, e1 = w[0] * 0.95, w[-1] * 1.05
    nc = 40
    a = np.zeros(nc)
    lib.ref_cheb_coef(nc, 0, e0, e1, a.ctypes.data_as(dp))
    y = rng.standard_normal(n)
    z = np.zeros(n)
    err = np.zeros(1)
    Mc = np.ascontiguousarray(M)
    lib.ref_cheb_eval_dense(nc, a.ctypes.data_as(dp), n, Mc.ctypes.data_as(dp),
                            y.ctypes.data_as(dp), z.ctypes.data_as(dp), e0, e1,
                            err.ctypes.data_as(dp))
    ch.update(dense_M=M, dense_y=y, dense_z=z, dense_err=err.copy(), dense_a=a,
              dense_e=np.array([e0, e1]))
    # Chebyshev on the reference's own Ewald operator (F, 20 non-overlapping
    # spheres, so that M is positive definite)
    pos, L20 = rsa_positions(20, 0.2, seed=9)
    box = (L20,) * 3
    r = mk(0, pos, box)
    Mfull = r.matrix()
    w = np.linalg.eigvalsh(0.5 * (Mfull + Mfull.T))
    e0, e1 = w[0] * 0.9, w[-1] * 1.1
    nc = 30
    a = np.zeros(nc)
    lib.ref_cheb_coef(nc, 0, e0, e1, a.ctypes.data_as(dp))
    y = rng.standard_normal(r.n)
    z = np.zeros(r.n)
    lib.ref_cheb_eval_ewald(C.c_void_p(r.h), nc, a.ctypes.data_as(dp), y.ctypes.data_as(dp),
                            z.ctypes.data_as(dp), e0, e1, err.ctypes.data_as(dp))
    ch.update(ewald_pos=pos, ewald_box=np.array(box), ewald_y=y, ewald_z=z,
              ewald_err=err.copy(), ewald_a=a, ewald_e=np.array([e0, e1]))
    np.savez_compressed(os.path.join(HERE, "chebyshev.npz"), **ch)

    # ---- KIrand (MT19937 + polar Box-Muller) ------------------------------
    ki = {}
    for seed in (1, 1234, 4357):
        st = lib.KIrand_init
        st.restype = C.c_void_p
        r = C.c_void_p(st())
        lib.KIrand_init_genrand.argtypes = [C.c_void_p, C.c_ulong]
        lib.KIrand_genrand_int32.argtypes = [C.c_void_p]
        lib.KIrand_genrand_int32.restype = C.c_ulong
        lib.KIrand_genrand_res53.argtypes = [C.c_void_p]
        lib.KIrand_genrand_res53.restype = C.c_double
        lib.KIrand_Gaussian.argtypes = [C.c_void_p]
        lib.KIrand_Gaussian.restype = C.c_double
        lib.KIrand_init_genrand(r, seed)
        ki[f"s{seed}_int32"] = np.array([lib.KIrand_genrand_int32(r) for _ in range(700)],
                                        dtype=np.uint64)
        ki[f"s{seed}_res53"] = np.array([lib.KIrand_genrand_res53(r) for _ in range(50)])
        ki[f"s{seed}_gauss"] = np.array([lib.KIrand_Gaussian(r) for _ in range(101)])
    np.savez_compressed(os.path.join(HERE, "kirand.npz"), **ki)

    # ---- the free-space operator (the reference's non-ewald.c) -----------
    np.savez_compressed(os.path.join(HERE, "nonewald.npz"), **nonewald_fixtures())

    # ---- Brownian dynamics (the reference's brownian.c) -------------------
    np.savez_compressed(os.path.join(HERE, "bd.npz"),
                        **bd_fixtures(), **bd_fixtures(BD_OPEN_CASES, periodic=False))

    # ---- lubrication (the reference's lub.c and two-body functions) -------
    np.savez_compressed(os.path.join(HERE, "lub.npz"), **lub_fixtures())

    # ---- struct layouts of the Brownian-dynamics interface ---------------
    json.dump(bd_layouts(ref_root), open(os.path.join(HERE, "bd_layouts.json"), "w"), indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(*sys.argv[1:])
