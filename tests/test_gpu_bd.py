"""Device Brownian dynamics against the CPU oracle on identical inputs.

FP64 engine vs oracle (same noise y, bounds and Chebyshev coefficients):
relative error 1e-10 on the Chebyshev noise and on the step's displacement
(thirty FP64 products in sequence).  Mixed engine vs FP64 engine: 1e-5 on
the displacement."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _engine(lib, version, pos, L, precision, lj_e=1.0, n_cheb=20):
    from libstokes_gb300 import System, check
    from libstokes_gb300.abi import BDParams
    s = System(version, pos, (L, L, L))
    p = BDParams(peclet=1.0, dt=1e-3, n_cheb=n_cheb, n_lanczos=20, cheb_eps=1e-2,
                 check_every=1, lj_e=lj_e, lj_r0=2.0, seed=5, precision=precision)
    h = C.c_void_p()
    check(lib.stokes_gpu_bd_create(s.sp, C.byref(p), C.byref(h)))
    return s, h


def _oracle(version, pos, L):
    from oracle.oracle import Oracle
    o = Oracle(version, pos, (L, L, L))
    o.set_split(o.xi_by_tratio(1.0), 1e-12)
    return o


@pytest.mark.parametrize("version", [0, 1])
def test_noise_and_step_match_oracle(lib, version):
    from libstokes_gb300 import FP64, check
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(40, 0.2, seed=3)
    s, h = _engine(lib, version, pos, L, FP64)
    eig = np.zeros(2)
    check(lib.stokes_gpu_bd_estimate_bounds(h, _d(eig)))
    n = (3, 6)[version] * 40
    y = np.random.default_rng(4).standard_normal(n)
    z = np.zeros(n)
    err = C.c_double()
    check(lib.stokes_gpu_bd_noise(h, _d(y), _d(z), C.byref(err)))
    a = np.zeros(20)
    from libstokes_gb300.abi import FUNC1
    f = FUNC1(lambda t: 1.0 / np.sqrt(t))
    lib.chebyshev_coef(20, f, eig[0], eig[1], _d(a))
    o = _oracle(version, pos, L)
    zo = o.cheb_eval(a, eig[0], eig[1], y)
    assert rel_l2(z, zo) < 1e-10
    assert 0.0 <= err.value < 1.0
    # one step with the same noise
    check(lib.stokes_gpu_bd_step_noise(h, 0.0, _d(y)))
    x1 = np.zeros(3 * 40)
    check(lib.stokes_gpu_bd_get_positions(h, _d(x1)))
    xo, _ = o.bd_step(pos, 1e-3, 1.0, a, eig[0], eig[1], y, lj_e=1.0, lj_r0=2.0, lj_image=True)
    d_gpu = x1 - pos.reshape(-1)
    d_ora = xo - pos.reshape(-1)
    assert rel_l2(d_gpu, d_ora) < 1e-10
    check(lib.stokes_gpu_bd_destroy(h))
    s.close()


def _boundary_pair(n, seed):
    """RSA spheres with particles 0 and 1 moved to overlap slightly (r = 1.95)
    across the x boundary of the box, clear of every other sphere"""
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(n, 0.15, seed=seed)
    p = pos.reshape(-1, 3).copy()
    rest = p[2:]

    def clear(q):
        d = rest - q
        d -= L * np.rint(d / L)
        return np.min(np.linalg.norm(d, axis=1)) > 2.2

    for y in np.linspace(1.0, L - 1.0, 25):
        for z in np.linspace(1.0, L - 1.0, 25):
            a, b = np.array([0.2, y, z]), np.array([L - 1.75, y, z])
            if clear(a) and clear(b):
                p[0], p[1] = a, b
                return p.reshape(-1), L
    pytest.skip("no clear spot for the boundary pair")


def test_engine_lj_uses_the_image_vector(lib):
    """The device engine's EV_LJ acts along the nearest-image vector: with a
    pair overlapping across the periodic boundary the step matches the oracle
    with that convention at 1e-10, and differs measurably from the
    reference's primary-cell vector (about L/r times the force), which the
    drop-in BD_evolve_mid keeps."""
    from libstokes_gb300 import FP64, check
    from libstokes_gb300.abi import _d, FUNC1
    pos, L = _boundary_pair(40, 7)
    s, h = _engine(lib, 0, pos, L, FP64)
    # rmin = 1: the mobility of the overlapping pair at contact distance
    s.set_misc(rmin=1.0)
    eig = np.zeros(2)
    check(lib.stokes_gpu_bd_estimate_bounds(h, _d(eig)))
    y = np.random.default_rng(8).standard_normal(3 * 40)
    a = np.zeros(20)
    lib.chebyshev_coef(20, FUNC1(lambda t: 1.0 / np.sqrt(t)), eig[0], eig[1], _d(a))
    check(lib.stokes_gpu_bd_set_bounds(h, _d(eig)))
    check(lib.stokes_gpu_bd_step_noise(h, 0.0, _d(y)))
    x1 = np.zeros(3 * 40)
    check(lib.stokes_gpu_bd_get_positions(h, _d(x1)))
    o = _oracle(0, pos, L)
    o.set_misc(rmin=1.0)
    xo, _ = o.bd_step(pos, 1e-3, 1.0, a, eig[0], eig[1], y, lj_e=1.0, lj_r0=2.0, lj_image=True)
    xr, _ = o.bd_step(pos, 1e-3, 1.0, a, eig[0], eig[1], y, lj_e=1.0, lj_r0=2.0, lj_image=False)
    d_gpu, d_img, d_ref = x1 - pos, xo - pos, xr - pos
    assert rel_l2(d_gpu, d_img) < 1e-10
    assert rel_l2(d_ref, d_img) > 1e-3
    check(lib.stokes_gpu_bd_destroy(h))
    s.close()


def test_engine_on_an_open_system(lib):
    """The device engine on an open system (periodic = 0): the free-space
    operator in the noise and both products, EV_LJ on the plain pair vector.
    One step with a given noise vector against the oracle at 1e-10."""
    from libstokes_gb300 import FP64, check
    from libstokes_gb300.abi import _d, FUNC1
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(40, 0.3, seed=12)
    p = pos.reshape(-1, 3).copy()
    p[1] = p[0] + np.array([1.9, 0.0, 0.0])    # one overlapping pair for EV_LJ
    keep = np.linalg.norm(p[2:] - p[1], axis=1) > 2.5
    p = np.vstack([p[:2], p[2:][keep]])
    n = len(p)
    s, h = _engine(lib, 1, p, L, FP64)
    s.s.periodic = 0
    s.set_misc(rmin=1.0)
    check(lib.stokes_gpu_bd_destroy(h))
    from libstokes_gb300.abi import BDParams
    prm = BDParams(peclet=1.0, dt=1e-3, n_cheb=20, n_lanczos=20, cheb_eps=1e-2, check_every=1,
                   lj_e=1.0, lj_r0=2.0, seed=5, precision=FP64)
    h = C.c_void_p()
    check(lib.stokes_gpu_bd_create(s.sp, C.byref(prm), C.byref(h)))
    eig = np.zeros(2)
    check(lib.stokes_gpu_bd_estimate_bounds(h, _d(eig)))
    y = np.random.default_rng(9).standard_normal(6 * n)
    a = np.zeros(20)
    lib.chebyshev_coef(20, FUNC1(lambda t: 1.0 / np.sqrt(t)), eig[0], eig[1], _d(a))
    check(lib.stokes_gpu_bd_step_noise(h, 0.0, _d(y)))
    x1 = np.zeros(3 * n)
    check(lib.stokes_gpu_bd_get_positions(h, _d(x1)))
    o = _oracle(1, p, L)
    o.set_misc(rmin=1.0)
    o.set_open(True)
    xo, _ = o.bd_step(p, 1e-3, 1.0, a, eig[0], eig[1], y, lj_e=1.0, lj_r0=2.0)
    assert rel_l2(x1 - p.reshape(-1), xo - p.reshape(-1)) < 1e-10
    check(lib.stokes_gpu_bd_destroy(h))
    s.close()


def test_lanczos_bounds_bracket_the_spectrum(lib):
    from libstokes_gb300 import FP64, check
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(30, 0.2, seed=6)
    s, h = _engine(lib, 0, pos, L, FP64)
    eig = np.zeros(2)
    check(lib.stokes_gpu_bd_estimate_bounds(h, _d(eig)))
    m = s.matrix()
    w = np.linalg.eigvalsh(0.5 * (m + m.T))
    assert eig[0] <= w[0] and eig[1] >= w[-1]
    assert eig[0] > 0.3 * w[0] and eig[1] < 1.2 * w[-1]
    check(lib.stokes_gpu_bd_destroy(h))
    s.close()


def test_mixed_step_close_to_fp64(lib):
    from libstokes_gb300 import FP64, MIXED, check
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(300, 0.2, seed=7)
    y = np.random.default_rng(8).standard_normal(900)
    out = {}
    for prec in (FP64, MIXED):
        s, h = _engine(lib, 0, pos, L, prec)
        eig = np.array([0.05, 2.0])
        check(lib.stokes_gpu_bd_set_bounds(h, _d(eig)))
        check(lib.stokes_gpu_bd_step_noise(h, 0.0, _d(y)))
        x1 = np.zeros(900)
        check(lib.stokes_gpu_bd_get_positions(h, _d(x1)))
        out[prec] = x1 - pos.reshape(-1)
        check(lib.stokes_gpu_bd_destroy(h))
        s.close()
    assert rel_l2(out[MIXED], out[FP64]) < 1e-5


def test_device_noise_run(lib):
    from libstokes_gb300 import MIXED, check
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(200, 0.2, seed=9)
    s, h = _engine(lib, 0, pos, L, MIXED, n_cheb=30)
    check(lib.stokes_gpu_bd_run(h, 0.0, 4))
    st = np.zeros(4)
    check(lib.stokes_gpu_bd_stats(h, _d(st)))
    assert st[3] == 4
    # 30 Chebyshev + 1 check + 2 solves per step, plus 20 Lanczos products
    assert st[0] >= 4 * 33 + 20
    x = np.zeros(600)
    check(lib.stokes_gpu_bd_get_positions(h, _d(x)))
    assert np.isfinite(x).all()
    disp = np.linalg.norm(x - pos.reshape(-1)) / np.sqrt(200)
    assert 1e-3 < disp < 1.0
    check(lib.stokes_gpu_bd_destroy(h))
    s.close()
