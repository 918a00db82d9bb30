"""libstokes' own BD entry points (BD_calc_FB, BD_evolve_mid) on the GPU
against the reference's brownian.c on identical inputs (tests/golden/bd.npz):
F with EV_LJ, F with overlap-driven dt halving (1st- and 2nd-stage redo),
FT with constant force/torque and quaternions, F under simple shear, and
open systems (periodic = 0: the free-space operator, EV_LJ and the
overlap check without images; F with EV_LJ, FT with dt halving).  The
noise comes from the same KIrand stream, the bounds and coefficients are
preset as in the fixtures.  FP64 path: positions to 1e-9; mixed path: the
displacement to 1e-5 relative."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
CASES = ["f_lj", "f_halving", "ft_q", "f_shear", "open_f_lj", "open_ft_halving"]


def bd_case(name):
    d = np.load(os.path.join(GOLDEN, "bd.npz"))
    return {k.split(":", 1)[1]: d[k] for k in d.files if k.startswith(name + ":")}


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class Run:
    """A struct stokes + struct BD_params set up like the fixture."""

    def __init__(self, lib, r, seed, precision):
        from libstokes_gb300 import System
        from libstokes_gb300.abi import FUNC1
        self.lib = lib
        ver = int(r["version"])
        self.n = len(r["pos"]) // 3
        L = float(r["box"])
        self.s = System(ver, r["pos"], (L, L, L))
        if "periodic" in r and int(r["periodic"]) == 0:
            self.s.s.periodic = 0
        if r["shear"][0]:
            lib.stokes_set_shear(self.s.sp, int(r["shear"][0]), float(r["shear"][1]))
        self.s.set_precision(precision)
        n = self.n
        self.F = r["F"].copy() if "F" in r else np.zeros(3 * n)
        self.T = r["T"].copy() if "T" in r else np.zeros(3 * n)
        self.E = np.zeros(5 * n)
        self.lj = None
        if r["lj"][0] != 0.0:
            self.lj = lib.EV_LJ_init(n)
            for i in range(n):
                self.lj.contents.flag[i] = 1
                self.lj.contents.e[i] = float(r["lj"][0])
                self.lj.contents.r0[i] = float(r["lj"][1])
        nm = int(r["n_minv"])
        self.bd = lib.BD_params_init(self.s.sp, int(seed), _dp(self.F), _dp(self.T), _dp(self.E),
                                     None, None, None, 0, 0, 0, 0.0, None, None, 1.0, None,
                                     None, None, self.lj, None, 0, float(r["peclet"]), 10.0, nm,
                                     0, 0, 0.0, float(r["bd_rmin"]), float(r["dt_lim"]))
        self.bd.contents.eig_minv[0] = float(r["eig"][0])
        self.bd.contents.eig_minv[1] = float(r["eig"][1])
        self._f = FUNC1(lambda v: 1.0 / np.sqrt(v))
        lib.chebyshev_coef(nm, self._f, float(r["eig"][0]), float(r["eig"][1]),
                           self.bd.contents.a_minv)

    def close(self):
        self.lib.BD_params_free(self.bd)
        if self.lj:
            self.lib.EV_LJ_free(self.lj)
        self.s.close()


@pytest.mark.parametrize("name", CASES)
def test_calc_fb_matches_reference(lib, name):
    from libstokes_gb300 import FP64
    r = bd_case(name)
    run = Run(lib, r, int(r["fb_seed"]), FP64)
    z = np.zeros(lib.BD_get_n(run.s.sp))
    lib.BD_calc_FB(run.bd, _dp(z))
    err = np.linalg.norm(z - r["z_fb"]) / np.linalg.norm(r["z_fb"])
    assert err < 1e-10, err
    run.close()


@pytest.mark.parametrize("name", CASES)
def test_evolve_mid_matches_reference(lib, name):
    from libstokes_gb300 import FP64
    r = bd_case(name)
    run = Run(lib, r, int(r["seed"]), FP64)
    x = r["pos"].copy()
    q = r["q0"].copy() if "q0" in r else None
    t = 0.0
    for s in range(len(r["dts"])):
        dt_done = lib.BD_evolve_mid(t, run.bd, _dp(x), _dp(q), float(r["dt"]))
        assert dt_done == r["dts"][s], (s, dt_done, r["dts"][s])
        t += dt_done
        assert np.abs(x - r["traj"][s]).max() < 1e-9, s
    if q is not None:
        assert np.abs(q - r["q1"]).max() < 1e-9
    run.close()


def test_evolve_mid_mixed_precision(lib):
    from libstokes_gb300 import MIXED
    r = bd_case("f_lj")
    run = Run(lib, r, int(r["seed"]), MIXED)
    x = r["pos"].copy()
    t = 0.0
    for s in range(len(r["dts"])):
        t += lib.BD_evolve_mid(t, run.bd, _dp(x), None, float(r["dt"]))
    disp_ref = r["traj"][-1] - r["pos"]
    err = np.linalg.norm((x - r["pos"]) - disp_ref) / np.linalg.norm(disp_ref)
    assert err < 1e-5, err
    run.close()


def test_get_fact_and_n(lib):
    from libstokes_gb300 import System
    r = bd_case("ft_q")
    run = Run(lib, r, 1, 0)
    assert lib.BD_get_n(run.s.sp) == 6 * run.n
    assert abs(lib.BD_params_get_fact(run.bd, 1e-3) - np.sqrt(2.0 / (2.0 * 1e-3))) < 1e-15
    run.close()


def test_resume_from_checkpoint(lib, tmp_path):
    """A run stopped after two steps and resumed from its checkpoint file
    (positions, time and the generator state, include/stokes_traj.h)
    continues exactly as the uninterrupted run."""
    from libstokes_gb300 import FP64
    from libstokes_gb300.abi import TrajFrame, _d
    r = bd_case("f_lj")
    run = Run(lib, r, int(r["seed"]), FP64)
    x = r["pos"].copy()
    t = 0.0
    path = str(tmp_path / "bd.traj").encode()
    tr = lib.stokes_traj_create(path, run.n, 0, 1 | 512, run.s.sp)
    for _ in range(2):
        t += lib.BD_evolve_mid(t, run.bd, _dp(x), None, float(r["dt"]))
    fr = TrajFrame()
    fr.time = t
    fr.x = _d(x)
    fr.rng = C.cast(run.bd.contents.rng, C.c_void_p)
    assert lib.stokes_traj_append(tr, C.byref(fr)) == 0
    lib.stokes_traj_close(tr)
    for _ in range(2):
        t += lib.BD_evolve_mid(t, run.bd, _dp(x), None, float(r["dt"]))
    run.close()

    run2 = Run(lib, r, 12345, FP64)        # another seed: the file sets the state
    tr = lib.stokes_traj_open(path)
    x2 = np.zeros(3 * run2.n)
    rd = TrajFrame()
    rd.x = _d(x2)
    rd.rng = C.cast(run2.bd.contents.rng, C.c_void_p)
    assert lib.stokes_traj_read(tr, 0, C.byref(rd)) == 0
    lib.stokes_traj_close(tr)
    t2 = rd.time
    for _ in range(2):
        t2 += lib.BD_evolve_mid(t2, run2.bd, _dp(x2), None, float(r["dt"]))
    assert t2 == t
    np.testing.assert_array_equal(x2, x)
    run2.close()
