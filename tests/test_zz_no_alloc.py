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


@pytest.mark.parametrize("version,n,phi,poly", [(2, 120, 0.3, False), (0, 400, 0.2, False),
                                                (1, 64, 0.2, True)])
def test_noalloc_matches_regular_entry_point(lib, version, n, phi, poly):
    import torch
    from libstokes_gb300 import System, check
    from libstokes_gb300.workloads import rsa_positions
    pos, L = rsa_positions(n, phi, seed=21)
    c = (3, 6, 11)[version]
    rng = np.random.default_rng(22)
    s = System(version, pos, (L, L, L))
    if poly:
        s.set_radius(rng.uniform(0.8, 1.2, n))
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
