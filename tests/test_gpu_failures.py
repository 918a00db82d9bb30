"""Failure detection without a GPU fault.

  * bounded device waits: a forced run-out of the tensor-core GEMMs' mbarrier
    wait (the MMA lane first waits on an mbarrier that nothing arrives at)
    and of the GMRES grid barrier (a spin limit of one poll) must end the
    kernels, come back as STOKES_GPU_ETIMEOUT, and leave the context usable:
    the next product / solve is correct;
  * host-side injections: non-finite positions, an invalid version, and a
    Chebyshev error above its bound, which must re-estimate the eigenvalue
    bounds (src/brownian.c:1710-1727)."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture
def unstall(lib):
    yield
    lib.stokes_gpu_test_stall_waits(0, 0)


def test_tensor_core_wait_runs_out(lib, unstall):
    from libstokes_gb300 import FP64, MIXED, System, abi
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(300, 0.3, seed=3)
    s = System(2, pos, (L, L, L))
    x = np.random.default_rng(4).standard_normal(s.n)
    y64 = s.atimes(x)
    s.set_precision(MIXED)
    y = np.zeros(s.n)
    assert lib.stokes_gpu_atimes(s.sp, _d(x), _d(y)) == abi.STOKES_GPU_OK
    assert rel_l2(y, y64) < 1e-6
    # the MMA lane waits 4 polls (about 80 us) on a barrier nobody arrives at
    assert lib.stokes_gpu_test_stall_waits(4, 0) == abi.STOKES_GPU_OK
    rc = lib.stokes_gpu_atimes(s.sp, _d(x), _d(y))
    assert rc == abi.STOKES_GPU_ETIMEOUT, rc
    assert b"ran out" in lib.stokes_gpu_last_error_message()
    lib.stokes_gpu_test_stall_waits(0, 0)
    # the context stays usable: the next product is right again
    y[:] = 0.0
    assert lib.stokes_gpu_atimes(s.sp, _d(x), _d(y)) == abi.STOKES_GPU_OK
    assert rel_l2(y, y64) < 1e-6
    s.set_precision(FP64)
    s.close()


def test_gmres_barrier_runs_out(lib, unstall):
    from libstokes_gb300 import System, abi
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(60, 0.2, seed=5)
    s = System(1, pos, (L, L, L))
    b = np.random.default_rng(6).standard_normal(s.n)
    it, res = C.c_int(), C.c_double()
    x = np.zeros(s.n)
    assert lib.stokes_gpu_test_stall_waits(0, 1) == abi.STOKES_GPU_OK
    rc = lib.stokes_gpu_solve(s.sp, 0, _d(b), _d(x), 20, 200, 1e-10, C.byref(it), C.byref(res))
    assert rc == abi.STOKES_GPU_ETIMEOUT, rc
    assert b"barrier" in lib.stokes_gpu_last_error_message()
    lib.stokes_gpu_test_stall_waits(0, 0)
    x[:] = 0.0
    rc = lib.stokes_gpu_solve(s.sp, 0, _d(b), _d(x), 20, 200, 1e-10, C.byref(it), C.byref(res))
    assert rc == abi.STOKES_GPU_OK and res.value <= 1e-10
    assert rel_l2(s.atimes(x), b) < 1e-9
    s.close()


def test_non_finite_positions_are_refused(lib):
    from libstokes_gb300 import MIXED, System, abi
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(40, 0.2, seed=7)
    for prec in (None, MIXED):
        s = System(0, pos, (L, L, L))
        if prec is not None:
            s.set_precision(prec)
        bad = pos.copy()
        bad[17, 1] = np.nan
        s.set_pos(bad)
        x = np.ones(s.n)
        y = np.zeros(s.n)
        assert lib.stokes_gpu_atimes(s.sp, _d(x), _d(y)) == abi.STOKES_GPU_EINVAL
        assert b"particle 17" in lib.stokes_gpu_last_error_message()
        bad[17, 1] = np.inf
        s.set_pos(bad)
        m = np.zeros((s.n, s.n))
        assert lib.stokes_gpu_matrix(s.sp, _d(m)) == abi.STOKES_GPU_EINVAL
        s.set_pos(pos)                     # the system works again once repaired
        assert lib.stokes_gpu_atimes(s.sp, _d(x), _d(y)) == abi.STOKES_GPU_OK
        assert np.isfinite(y).all()
        s.close()


def test_invalid_version_is_refused(lib):
    from libstokes_gb300 import System, abi
    from libstokes_gb300.abi import _d
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(20, 0.2, seed=8)
    s = System(0, pos, (L, L, L))
    s.s.version = 5
    x = np.ones(3 * 20)
    y = np.zeros(3 * 20)
    assert lib.stokes_gpu_atimes(s.sp, _d(x), _d(y)) == abi.STOKES_GPU_EINVAL
    assert b"version" in lib.stokes_gpu_last_error_message()
    s.s.version = 0
    assert lib.stokes_gpu_atimes(s.sp, _d(x), _d(y)) == abi.STOKES_GPU_OK
    s.close()


def test_chebyshev_error_above_bound_reestimates(lib):
    """Engine: with cheb_eps below any reachable error every checked step
    re-estimates the bounds.  Drop-in BD_calc_FB: bounds preset far too
    narrow and BD->eps tiny -- the call replaces them by Lanczos bounds."""
    from libstokes_gb300 import FP64, System, abi
    from libstokes_gb300.abi import FUNC1
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(64, 0.2, seed=9)
    s = System(0, pos, (L, L, L))
    p = abi.BDParams(peclet=1.0, dt=1e-3, n_cheb=20, n_lanczos=20, cheb_eps=1e-30,
                     check_every=1, lj_e=0.0, lj_r0=2.0, seed=3, precision=FP64)
    h = C.c_void_p()
    abi.check(lib.stokes_gpu_bd_create(s.sp, C.byref(p), C.byref(h)))
    abi.check(lib.stokes_gpu_bd_run(h, 0.0, 3))
    st = np.zeros(4)
    abi.check(lib.stokes_gpu_bd_stats(h, st.ctypes.data_as(abi._dp)))
    assert st[1] >= 4, st            # the first estimate plus one per checked step
    assert st[2] < 1e-2, st          # the re-estimated bounds give a small error
    abi.check(lib.stokes_gpu_bd_destroy(h))
    s.close()

    s = System(0, pos, (L, L, L))
    n = s.n
    F, T, E = np.zeros(n), np.zeros(n), np.zeros(5 * 64)
    dp = abi._dp
    bd = lib.BD_params_init(s.sp, 7, F.ctypes.data_as(dp), T.ctypes.data_as(dp),
                            E.ctypes.data_as(dp), None, None, None, 0, 0, 0, 0.0, None, None, 1.0,
                            None, None, None, None, None, 0, 1.0, 1e-30, 20, 0, 0, 0.0, 0.0,
                            1e-12)
    bd.contents.eig_minv[0], bd.contents.eig_minv[1] = 0.50, 0.51
    f = FUNC1(lambda v: 1.0 / np.sqrt(v))
    lib.chebyshev_coef(20, f, 0.50, 0.51, bd.contents.a_minv)
    z = np.zeros(n)
    lib.BD_calc_FB(bd, z.ctypes.data_as(dp))
    abi.raise_if_failed()
    e0, e1 = bd.contents.eig_minv[0], bd.contents.eig_minv[1]
    # replaced by Lanczos bounds, which the preset narrow interval is not
    assert (e0, e1) != (0.50, 0.51) and 0.0 < e0 < e1 and e1 - e0 > 0.05, (e0, e1)
    assert np.isfinite(z).all()
    lib.BD_params_free(bd)
    s.close()
