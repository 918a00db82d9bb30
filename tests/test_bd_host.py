"""Host-side pieces of the Brownian-dynamics path, no GPU needed:
the KIrand generator against the reference's own stream, the struct
layouts of the BD interface against the reference headers, and the CPU
oracle's mid-point step against the reference's own BD_evolve_mid."""
import json
import os
import subprocess

import numpy as np

from conftest import GOLDEN, ROOT


def test_kirand_matches_reference_stream(lib):
    g = np.load(os.path.join(GOLDEN, "kirand.npz"))
    for seed in (1, 1234, 4357):
        r = lib.KIrand_init()
        lib.KIrand_init_genrand(r, seed)
        ints = np.array([lib.KIrand_genrand_int32(r) for _ in range(700)], dtype=np.uint64)
        np.testing.assert_array_equal(ints, g[f"s{seed}_int32"])
        res = np.array([lib.KIrand_genrand_res53(r) for _ in range(50)])
        np.testing.assert_array_equal(res, g[f"s{seed}_res53"])
        gs = np.array([lib.KIrand_Gaussian(r) for _ in range(101)])
        np.testing.assert_array_equal(gs, g[f"s{seed}_gauss"])
        lib.KIrand_free(r)


def test_unseeded_kirand_uses_default_seed(lib):
    a = lib.KIrand_init()
    b = lib.KIrand_init()
    lib.KIrand_init_genrand(b, 5489)
    assert [lib.KIrand_genrand_int32(a) for _ in range(5)] == \
        [lib.KIrand_genrand_int32(b) for _ in range(5)]
    lib.KIrand_free(a)
    lib.KIrand_free(b)


def test_bd_struct_layouts(tmp_path):
    ref = json.load(open(os.path.join(GOLDEN, "bd_layouts.json")))
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "stokes_bd.h"',
           'int main(void){']
    keys = sorted(ref)
    for k in keys:
        st, f = k.split(".")
        if f == "sizeof":
            src.append(f'printf("%zu\\n", sizeof(struct {st}));')
        else:
            src.append(f'printf("%zu\\n", offsetof(struct {st}, {f}));')
    src.append("return 0;}")
    c = tmp_path / "lay.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "lay"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)])
    out = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    for k, v in zip(keys, out):
        assert v == ref[k], k


def bd_case(name):
    d = np.load(os.path.join(GOLDEN, "bd.npz"))
    return {k.split(":", 1)[1]: d[k] for k in d.files if k.startswith(name + ":")}


def test_ctypes_bd_structs_match_reference_layout():
    import ctypes as C
    from libstokes_gb300.abi import BDStruct, EVLJStruct, KIrandStruct
    ref = json.load(open(os.path.join(GOLDEN, "bd_layouts.json")))
    cls = {"BD_params": BDStruct, "EV_LJ": EVLJStruct, "KIrand": KIrandStruct}
    checked = 0
    for k, v in ref.items():
        st, f = k.split(".")
        if st not in cls:
            continue
        got = C.sizeof(cls[st]) if f == "sizeof" else getattr(cls[st], f).offset
        assert got == v, k
        checked += 1
    assert checked > 40


def test_oracle_bd_step_matches_reference_trajectory(lib):
    """oracle_bd_step (C restatement) reproduces three steps of the
    reference's BD_evolve_mid (F, N=27, EV_LJ, no overlap checks), with the
    noise drawn from KIrand in the reference's order."""
    import ctypes as C
    from libstokes_gb300.abi import FUNC1
    from oracle.oracle import Oracle
    r = bd_case("f_lj")
    n = len(r["pos"]) // 3
    L = float(r["box"])
    o = Oracle(0, r["pos"], (L, L, L))
    o.set_split(o.xi_by_tratio(1.0), 1e-12)
    nm = int(r["n_minv"])
    a = np.zeros(nm)
    f = FUNC1(lambda v: 1.0 / np.sqrt(v))
    lib.chebyshev_coef(nm, f, float(r["eig"][0]), float(r["eig"][1]),
                       a.ctypes.data_as(C.POINTER(C.c_double)))
    rng = lib.KIrand_init()
    lib.KIrand_init_genrand(rng, int(r["seed"]))
    x = r["pos"].copy()
    for s in range(len(r["dts"])):
        y = np.array([lib.KIrand_Gaussian(rng) for _ in range(3 * n)])
        x, _ = o.bd_step(x, float(r["dt"]), float(r["peclet"]), a, r["eig"][0], r["eig"][1], y,
                         lj_e=float(r["lj"][0]), lj_r0=float(r["lj"][1]))
        assert np.abs(x - r["traj"][s]).max() < 1e-10, s
    lib.KIrand_free(rng)
