"""The CPU oracle of the adjoint (oracle/oracle_adjoint.cpp, direct pair sums
with dual numbers) against central differences of the oracle product, whose
values are pinned to the reference at 1e-12: L = g . M(r, box) f, dL/dr and
dL/dl at fixed images, k set and xi."""
import numpy as np
import pytest

from conftest import rel_l2


def _fd_grad(o, pos, g, f, h=1e-5):
    fd = np.zeros(pos.size)
    for k in range(pos.size):
        p = pos.reshape(-1).copy()
        p[k] += h
        o.set_pos(p)
        a = g @ o.atimes(f)
        p[k] -= 2 * h
        o.set_pos(p)
        b = g @ o.atimes(f)
        fd[k] = (a - b) / (2 * h)
    o.set_pos(pos)
    return fd


@pytest.mark.parametrize("version", [0, 1])
def test_oracle_vjp_matches_finite_differences(version):
    from oracle.oracle import Oracle
    from libstokes_gb300.workloads import rsa_positions
    n = 12
    pos, L = rsa_positions(n, 0.2, seed=3 + version)
    c = (3, 6)[version]
    rng = np.random.default_rng(5)
    g = rng.standard_normal(c * n)
    f = rng.standard_normal(c * n)
    o = Oracle(version, pos, (L, L, L))
    o.set_split(o.xi_by_tratio(1.0), 1e-12)
    Lv, dr, db = o.vjp(pos, g, f)
    assert abs(Lv - g @ o.atimes(f)) < 1e-12 * abs(Lv) + 1e-14
    assert rel_l2(dr, _fd_grad(o, pos, g, f)) < 1e-8
    xi = o.split()["xi"]
    for a in range(3):
        vals = []
        for s in (1.0, -1.0):
            box = [L, L, L]
            box[a] += s * 1e-5
            o2 = Oracle(version, pos, tuple(box))
            o2.set_split(xi, 1e-12)
            vals.append(g @ o2.atimes(f))
        fd = (vals[0] - vals[1]) / 2e-5
        assert abs(db[a] - fd) < 1e-7 * max(1.0, abs(fd)), (a, db[a], fd)
