"""The allocation-free entry point, stokes_gpu_atimes_noalloc.

It exists for callers that may not allocate device memory while they run;
its scratch is one fixed device array per GPU.  Its output must equal the
regular FP64 device entry point's (stokes_gpu_atimes_dev) within the FP64
tolerance of the other tests, on two calls in a row (the second call finds
the first call's leftovers in the shared array).  This file is collected
last so that a run stopping at the first failure has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _dev(a, torch):
    return torch.tensor(a, dtype=torch.float64, device="cuda:0").contiguous()


@pytest.mark.parametrize("version,n,phi,poly,extra", [
    (2, 120, 0.3, False, None), (0, 400, 0.2, False, None), (1, 64, 0.2, True, None),
    (1, 80, 0.2, False, "shear1"), (2, 60, 0.2, False, "shear2"), (1, 50, 0.15, True, "slip")])
def test_noalloc_matches_regular_entry_point(lib, version, n, phi, poly, extra):
    import torch
    from libstokes_gb300 import System, check
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(n, phi, seed=21)
    c = (3, 6, 11)[version]
    rng = np.random.default_rng(22)
    s = System(version, pos, (L, L, L))
    if poly:
        s.set_radius(rng.uniform(0.8, 1.2, n))
    if extra == "shear1":
        s.set_misc(shear_mode=1, shear_shift=0.37 * L)   # the image and k tables fold in the shift
    elif extra == "shear2":
        s.set_misc(shear_mode=2, shear_shift=-0.21 * L)
    elif extra == "slip":
        s.set_slip(rng.uniform(0.2, 2.0, n))              # slip lengths: slip radii and factors
    d_pos = _dev(pos, torch)
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    for call in range(2):
        x = rng.standard_normal(c * n)
        d_x = _dev(x, torch)
        y_ref = torch.empty_like(d_x)
        y_na = torch.full_like(d_x, float("nan"))
        check(lib.stokes_gpu_atimes_dev(s.sp, C.c_void_p(d_pos.data_ptr()),
                                        C.c_void_p(d_x.data_ptr()),
                                        C.c_void_p(y_ref.data_ptr()), sp))
        check(lib.stokes_gpu_atimes_noalloc(s.sp, C.c_void_p(d_pos.data_ptr()),
                                            C.c_void_p(d_x.data_ptr()),
                                            C.c_void_p(y_na.data_ptr()), sp))
        stream.synchronize()
        a, b = y_na.cpu().numpy(), y_ref.cpu().numpy()
        assert np.isfinite(a).all(), call
        assert rel_l2(a, b) < TOL, (call, rel_l2(a, b))
    s.close()


def test_noalloc_rejects_systems_above_its_capacity(lib):
    import torch
    from libstokes_gb300 import System, abi
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(600, 0.1, seed=3)
    s = System(0, pos, (L, L, L))
    d_pos = _dev(pos, torch)
    d_x = torch.zeros(3 * 600, dtype=torch.float64, device="cuda:0")
    d_y = torch.zeros_like(d_x)
    rc = lib.stokes_gpu_atimes_noalloc(s.sp, C.c_void_p(d_pos.data_ptr()),
                                       C.c_void_p(d_x.data_ptr()), C.c_void_p(d_y.data_ptr()),
                                       None)
    assert rc == abi.STOKES_GPU_ETOOBIG
    assert b"at most 512" in lib.stokes_gpu_last_error_message()
    s.close()


def test_noalloc_rejects_too_many_reciprocal_vectors(lib):
    import torch
    from libstokes_gb300 import System, abi
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(40, 0.1, seed=4)
    s = System(0, pos, (L, L, L))
    st = s.s
    st.kmaxx = st.kmaxy = st.kmaxz = 6        # the full 13^3 cube: 2196 vectors
    st.kmax = 0.0
    d_pos = _dev(pos, torch)
    d_x = torch.zeros(3 * 40, dtype=torch.float64, device="cuda:0")
    d_y = torch.zeros_like(d_x)
    rc = lib.stokes_gpu_atimes_noalloc(s.sp, C.c_void_p(d_pos.data_ptr()),
                                       C.c_void_p(d_x.data_ptr()), C.c_void_p(d_y.data_ptr()),
                                       None)
    assert rc == abi.STOKES_GPU_ETOOBIG
    assert b"reciprocal vectors" in lib.stokes_gpu_last_error_message()
    s.close()


def test_noalloc_refuses_unset_split_and_capture(lib):
    import torch
    from libstokes_gb300 import System, abi
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(30, 0.1, seed=5)
    s = System(0, pos, (L, L, L))
    d_pos = _dev(pos, torch)
    d_x = torch.ones(3 * 30, dtype=torch.float64, device="cuda:0")
    d_y = torch.zeros_like(d_x)
    args = (s.sp, C.c_void_p(d_pos.data_ptr()), C.c_void_p(d_x.data_ptr()),
            C.c_void_p(d_y.data_ptr()))
    xi = s.s.xi
    s.s.xi = 0.0                              # a split that was never set
    assert lib.stokes_gpu_atimes_noalloc(*args, None) == abi.STOKES_GPU_EINVAL
    assert b"xi" in lib.stokes_gpu_last_error_message()
    s.s.xi = xi
    # a stream under capture: refused before anything is enqueued on it
    g = torch.cuda.CUDAGraph()
    stream = torch.cuda.Stream()
    rcs = []
    with torch.cuda.graph(g, stream=stream):
        rcs.append(lib.stokes_gpu_atimes_noalloc(*args, C.c_void_p(stream.cuda_stream)))
        d_y.add_(1.0)                         # something for the graph to hold
    assert rcs == [abi.STOKES_GPU_EINVAL]
    assert b"captured" in lib.stokes_gpu_last_error_message()
    s.close()
