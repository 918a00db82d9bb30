"""Host-side pieces of the Brownian-dynamics path, no GPU needed:
the KIrand generator against the reference's own stream, and the struct
layouts of the BD interface against the reference headers."""
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
