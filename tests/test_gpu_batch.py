"""Batches of independent periodic systems (stokes_gpu_batch_*): every
system's slice of the packed product against that system's own product,
FP64 at 1e-12, mixed at the mixed-path tolerance 1e-6."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _systems(lib, nsys, seed, shear=False, nmax=80):
    from libstokes_gb300 import System
    from libstokes_gb300.workloads import rsa_positions
    rng = np.random.default_rng(seed)
    out = []
    for s in range(nsys):
        n = int(rng.integers(16, nmax + 1))
        phi = float(rng.uniform(0.05, 0.35))
        ver = s % 2
        pos, L = rsa_positions(n, phi, seed=seed * 100 + s)
        sy = System(ver, pos, (L, L, L))
        if shear and s % 3 == 2:
            sy.set_misc(0.0, 1, 0.37 * L)
        out.append(sy)
    return out


def _batch(lib, systems, precision):
    arr = (C.POINTER(type(systems[0].s)) * len(systems))(*[s.sp for s in systems])
    h = C.c_void_p()
    rc = lib.stokes_gpu_batch_create(arr, len(systems), precision, C.byref(h))
    assert rc == 0, lib.stokes_gpu_last_error_message()
    npt, nt = C.c_int(), C.c_int()
    lib.stokes_gpu_batch_size(h, C.byref(npt), C.byref(nt))
    xo = np.zeros(len(systems), dtype=np.int32)
    lib.stokes_gpu_batch_offsets(h, None, xo.ctypes.data_as(C.POINTER(C.c_int)))
    return h, nt.value, xo


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)])
def test_batch_matches_single_products(lib, precision, tol):
    from libstokes_gb300 import FP64
    systems = _systems(lib, 12, seed=3, shear=True)
    h, nt, xo = _batch(lib, systems, precision)
    x = np.random.default_rng(4).standard_normal(nt)
    y = np.zeros(nt)
    assert lib.stokes_gpu_batch_atimes(h, _dp(x), _dp(y)) == 0, lib.stokes_gpu_last_error_message()
    for s, sy in enumerate(systems):
        n = sy.n
        sy.set_precision(FP64)
        ref = sy.atimes(x[xo[s]:xo[s] + n])
        assert rel_l2(y[xo[s]:xo[s] + n], ref) < tol, (s, rel_l2(y[xo[s]:xo[s] + n], ref))
    lib.stokes_gpu_batch_destroy(h)
    for sy in systems:
        sy.close()


def test_batch_positions_and_stats(lib):
    from libstokes_gb300 import FP64
    systems = _systems(lib, 8, seed=7)
    h, nt, xo = _batch(lib, systems, 1)
    x = np.random.default_rng(8).standard_normal(nt)
    y = np.zeros(nt)
    assert lib.stokes_gpu_batch_atimes(h, _dp(x), _dp(y)) == 0
    st = np.zeros(4)
    lib.stokes_gpu_batch_stats(h, _dp(st))
    assert st[0] > 0 and st[1] in (1, 2, 4) and st[2] in (4, 8) and st[3] > 0
    # move every particle a little and compare again
    po = np.zeros(len(systems), dtype=np.int32)
    lib.stokes_gpu_batch_offsets(h, po.ctypes.data_as(C.POINTER(C.c_int)), None)
    pos = np.concatenate([np.ctypeslib.as_array(sy.s.pos, (3 * sy.s.np,)).copy() for sy in systems])
    pos += 0.05 * np.random.default_rng(9).standard_normal(pos.shape)
    assert lib.stokes_gpu_batch_set_positions(h, _dp(pos)) == 0
    assert lib.stokes_gpu_batch_atimes(h, _dp(x), _dp(y)) == 0
    for s, sy in enumerate(systems):
        n = sy.n
        sy.set_precision(FP64)
        ref = sy.atimes(x[xo[s]:xo[s] + n])
        assert rel_l2(y[xo[s]:xo[s] + n], ref) < 1e-6
    lib.stokes_gpu_batch_destroy(h)
    for sy in systems:
        sy.close()


@pytest.mark.parametrize("precision,tol", [(0, 1e-9), (1, 1e-4)])
def test_batch_bd_step_matches_oracle(lib, precision, tol):
    """One mid-point step of every system with the same noise and bounds as
    the CPU oracle's oracle_bd_step (products of the reference split in
    FP64); mixed batches to 1e-4 of the displacement."""
    from libstokes_gb300.abi import FUNC1
    from oracle.oracle import Oracle
    systems = _systems(lib, 4, seed=21, nmax=40)
    h, nt, xo = _batch(lib, systems, precision)
    po = np.zeros(len(systems), dtype=np.int32)
    lib.stokes_gpu_batch_offsets(h, po.ctypes.data_as(C.POINTER(C.c_int)), None)
    ncheb, dt, pe = 16, 1e-3, 1.0
    eig = np.zeros(2 * len(systems))
    oracles, pos0 = [], []
    for s, sy in enumerate(systems):
        L = sy.s.lx
        p = np.ctypeslib.as_array(sy.s.pos, (3 * sy.s.np,)).copy()
        pos0.append(p)
        o = Oracle(sy.s.version, p, (L, L, L))
        o.set_split(o.xi_by_tratio(1.0), 1e-12)
        ev = np.linalg.eigvalsh(0.5 * (o.matrix() + o.matrix().T))
        eig[2 * s], eig[2 * s + 1] = 0.8 * ev[0], 1.05 * ev[-1]
        oracles.append(o)
    y = np.random.default_rng(22).standard_normal(nt)
    out = np.zeros(3 * sum(sy.s.np for sy in systems))
    rc = lib.stokes_gpu_batch_bd(h, pe, dt, ncheb, 20, _dp(eig), _dp(y), 0, 1, _dp(out))
    assert rc == 0, lib.stokes_gpu_last_error_message()
    f = FUNC1(lambda v: 1.0 / np.sqrt(v))
    for s, sy in enumerate(systems):
        a = np.zeros(ncheb)
        lib.chebyshev_coef(ncheb, f, eig[2 * s], eig[2 * s + 1], _dp(a))
        n = sy.n
        xo_new, _ = oracles[s].bd_step(pos0[s], dt, pe, a, eig[2 * s], eig[2 * s + 1],
                                       y[xo[s]:xo[s] + n])
        got = out[3 * po[s]:3 * po[s] + 3 * sy.s.np]
        disp = xo_new - pos0[s]
        assert np.abs(got - xo_new).max() < tol * max(1e-3, np.abs(disp).max()) + 1e-12, s
    lib.stokes_gpu_batch_destroy(h)
    for sy in systems:
        sy.close()


def test_batch_bd_run_lanczos(lib):
    """Ten steps with device noise and Lanczos bounds: finite, moving."""
    systems = _systems(lib, 16, seed=31, nmax=120)
    h, nt, xo = _batch(lib, systems, 1)
    npt = sum(sy.s.np for sy in systems)
    pos0 = np.concatenate([np.ctypeslib.as_array(sy.s.pos, (3 * sy.s.np,)).copy() for sy in systems])
    out = np.zeros(3 * npt)
    rc = lib.stokes_gpu_batch_bd(h, 1.0, 1e-3, 30, 20, None, None, 7, 10, _dp(out))
    assert rc == 0, lib.stokes_gpu_last_error_message()
    d = out - pos0
    assert np.all(np.isfinite(out))
    rms = np.sqrt(np.mean(d ** 2))
    # free diffusion over 10 steps of dt 1e-3 at Pe 1: sqrt(2 D t) ~ 0.14 per axis
    assert 0.02 < rms < 1.0, rms
    lib.stokes_gpu_batch_destroy(h)
    for sy in systems:
        sy.close()
