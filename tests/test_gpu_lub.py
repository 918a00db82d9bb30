"""The lubrication correction on the GPU (calc_lub_3f / 3ft / 3fts,
src/lub.c:164-768, equal spheres) against the reference's own outputs
(tests/golden/lub.npz: periodic, open, sheared, small-box and
unlimited-range systems) and against the oracle on larger systems; the
refusals (unequal radii, a bad version, an image cube too large); and the
lubricated mobility problem (I + M L) u = M f solved on the device against
a dense solve."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["lub_f_periodic", "lub_ft_periodic", "lub_f_open", "lub_ft_open", "lub_ft_nolimit",
         "lub_f_small_box", "lub_f_shear1", "lub_ft_shear2", "lub_fts_periodic", "lub_fts_open",
         "lub_fts_shear1"]


@pytest.fixture(scope="module")
def lub():
    return np.load(os.path.join(HERE, "golden", "lub.npz"))


def _system(ver, pos, L, periodic, lubmin2, lubmax, mode=0, shift=0.0):
    from libstokes_gb300 import System
    s = System(ver, pos, (L, L, L)) if periodic else System(ver, pos, periodic=False)
    if mode:
        s.set_misc(0.0, mode, shift)
    s.s.lubmin2 = float(lubmin2)
    s.s.lubmax = float(lubmax)
    return s


def _calc(lib, s, ver, u):
    from libstokes_gb300 import abi
    f = np.zeros_like(u)
    rc = lib.stokes_gpu_lub(s.sp, ver, u.ctypes.data_as(abi._dp), f.ctypes.data_as(abi._dp))
    assert rc == abi.STOKES_GPU_OK, lib.stokes_gpu_last_error_message()
    return f


@pytest.mark.parametrize("name", CASES)
def test_lub_against_reference(lib, lub, name):
    ver, n, L, periodic, lubmin2, lubmax, mode, shift = lub[f"{name}_meta"]
    ver = int(ver)
    s = _system(ver, lub[f"{name}_pos"], L, periodic, lubmin2, lubmax, int(mode), shift)
    f = _calc(lib, s, ver, np.ascontiguousarray(lub[f"{name}_u"]))
    assert rel_l2(f, lub[f"{name}_f"]) < 1e-12, rel_l2(f, lub[f"{name}_f"])
    # the drop-in entry point gives the same numbers
    from libstokes_gb300 import abi
    u = np.ascontiguousarray(lub[f"{name}_u"])
    g = np.zeros_like(u)
    (lib.calc_lub_3f, lib.calc_lub_3ft, lib.calc_lub_3fts)[ver](s.sp, u.ctypes.data_as(abi._dp),
                                                               g.ctypes.data_as(abi._dp))
    assert np.array_equal(f, g)
    s.close()


@pytest.mark.parametrize("ver", [0, 1, 2])
def test_lub_large_against_oracle(lib, ver):
    from libstokes_gb300.workloads import rsa_positions
    from oracle.oracle import calc_lub
    pos, L = rsa_positions(1000, 0.35, seed=71 + ver)
    c = (3, 6, 11)[ver]
    u = np.random.default_rng(72).standard_normal(c * 1000)
    s = _system(ver, pos, L, True, 2.0001 ** 2, 3.0)
    f = _calc(lib, s, ver, u)
    fo = calc_lub(ver, pos, (L, L, L), u, lubmin2=2.0001 ** 2, lubmax=3.0)
    assert np.count_nonzero(fo) > 0
    assert rel_l2(f, fo) < 1e-12, rel_l2(f, fo)
    s.close()


def test_lub_refusals(lib):
    from libstokes_gb300 import abi
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(20, 0.2, seed=5)
    s = _system(0, pos, L, True, 0.0, 3.0)
    u = np.ones(60)
    f = np.zeros(60)
    s.set_radius(np.ones(20))
    assert lib.stokes_gpu_lub(s.sp, 0, u.ctypes.data_as(abi._dp),
                              f.ctypes.data_as(abi._dp)) == abi.STOKES_GPU_EINVAL
    assert b"equal spheres" in lib.stokes_gpu_last_error_message()
    s.close()
    s = _system(2, pos, L, True, 0.0, 3.0)
    u = np.ones(220)
    f = np.zeros(220)
    assert lib.stokes_gpu_lub(s.sp, 3, u.ctypes.data_as(abi._dp),
                              f.ctypes.data_as(abi._dp)) == abi.STOKES_GPU_EINVAL
    s.s.lubmax = 1e6                    # an image cube too large to walk
    assert lib.stokes_gpu_lub(s.sp, 2, u.ctypes.data_as(abi._dp),
                              f.ctypes.data_as(abi._dp)) == abi.STOKES_GPU_EINVAL
    assert b"boxes" in lib.stokes_gpu_last_error_message()
    s.close()


@pytest.mark.parametrize("ver", [0, 1])
def test_lubricated_mobility_solve(lib, ver):
    """(I + M L) u = M f on the device (STOKES_GPU_SOLVE_MOB_LUB) against the
    dense solve of the same operator assembled from the GPU's M and L."""
    from libstokes_gb300 import abi
    from libstokes_gb300.workloads import rsa_positions
    n = 60
    c = (3, 6)[ver]
    pos, L = rsa_positions(n, 0.3, seed=81 + ver)
    s = _system(ver, pos, L, True, 2.0001 ** 2, 3.5)
    N = c * n
    M = s.matrix()
    Lm = np.zeros((N, N))
    for k in range(N):
        e = np.zeros(N)
        e[k] = 1.0
        Lm[:, k] = _calc(lib, s, ver, e)
    fvec = np.random.default_rng(3).standard_normal(N)
    b = M @ fvec
    u_dense = np.linalg.solve(np.eye(N) + M @ Lm, b)
    x = np.zeros(N)
    it, res = C.c_int(), C.c_double()
    rc = lib.stokes_gpu_solve(s.sp, abi.SOLVE_MOB_LUB, b.ctypes.data_as(abi._dp),
                              x.ctypes.data_as(abi._dp), 30, 2000, 1e-12, C.byref(it),
                              C.byref(res))
    assert rc == abi.STOKES_GPU_OK, lib.stokes_gpu_last_error_message()
    assert rel_l2(x, u_dense) < 1e-9, rel_l2(x, u_dense)
    s.close()
