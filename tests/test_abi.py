"""The C ABI without a GPU: struct layout, exported symbols, set-up code.

* struct stokes must be byte-identical to libstokes' (member offsets from the
  reference header, tests/golden/struct_stokes_layout.json);
* every function the public headers declare must be exported by the .so;
* the set-up functions (host C, no device calls) must reproduce the
  reference's Ewald split, cutoffs and image table exactly.
"""
import ctypes as C
import json
import os
import re

import numpy as np

from conftest import GOLDEN, ROOT


def test_struct_layout(lib):
    from libstokes_gb300.abi import StokesStruct
    ref = json.load(open(os.path.join(GOLDEN, "struct_stokes_layout.json")))
    assert C.sizeof(StokesStruct) == ref["sizeof"]
    for name, _ in StokesStruct._fields_:
        assert getattr(StokesStruct, name).offset == ref[name], name


def test_header_layout_compiles_to_same_offsets(tmp_path):
    """include/stokes_abi.h, compiled by the C compiler, has the same
    offsets as the reference header."""
    import subprocess
    ref = json.load(open(os.path.join(GOLDEN, "struct_stokes_layout.json")))
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "stokes_abi.h"',
           'int main(void){', 'printf("%zu\\n", sizeof(struct stokes));']
    fields = [k for k in ref if k != "sizeof"]
    for f in fields:
        src.append(f'printf("%zu\\n", offsetof(struct stokes, {f}));')
    src.append("return 0;}")
    c = tmp_path / "lay.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "lay"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)])
    out = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    assert out[0] == ref["sizeof"]
    for f, v in zip(fields, out[1:]):
        assert v == ref[f], f


def _declared_functions():
    names = set()
    for h in sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt):
            nm = m.group(1)
            if nm in ("if", "sizeof", "return", "defined") or nm.isupper():
                continue
            names.add(nm)
    # function-pointer parameter names that the regex also catches
    names -= {"atimes", "func", "void", "double", "int", "char"}
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = _declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_setup_matches_reference(lib, setup_golden):
    from libstokes_gb300 import System
    g = setup_golden
    q = 0
    while f"c{q}_box" in g.files:
        box = tuple(g[f"c{q}_box"])
        tr, eps = g[f"c{q}_tr_eps"]
        s = System(0, np.zeros((1, 3)), box, tratio=tr, eps=eps)
        st = s.s
        got = np.array([st.xi, st.rmax2, st.kmax, st.self_a, st.self_c, st.self_m, st.pivol,
                        st.nr, st.kmaxx, st.kmaxy, st.kmaxz])
        np.testing.assert_array_equal(got, g[f"c{q}_split"])
        nr = st.nr
        rl = np.stack([np.ctypeslib.as_array(st.rlx, (nr,)), np.ctypeslib.as_array(st.rly, (nr,)),
                       np.ctypeslib.as_array(st.rlz, (nr,))], axis=1)
        rm = np.stack([np.ctypeslib.as_array(st.rmx, (nr,)), np.ctypeslib.as_array(st.rmy, (nr,)),
                       np.ctypeslib.as_array(st.rmz, (nr,))], axis=1)
        np.testing.assert_array_equal(rl, g[f"c{q}_rl"])
        np.testing.assert_array_equal(rm, g[f"c{q}_rm"])
        s.close()
        q += 1


def test_setters(lib):
    from libstokes_gb300 import System
    s = System(1, np.zeros((2, 3)), (10.0, 5.0, 5.0))
    lib.stokes_set_shear(s.sp, 1, 2.0)
    assert s.s.Oi[2] == -1.0 and s.s.Ei[1] == 1.0
    s.s.periodic = 1
    # shift folded into [-lx/2, lx/2) (src/stokes.c:554-589)
    sh = lib.stokes_get_shear_shift(s.sp, 3.0, 0.0, 0.0)
    assert -5.0 <= sh < 5.0
    assert abs((5.0 * 2.0 * 3.0 - sh) / 10.0 - round((5.0 * 2.0 * 3.0 - sh) / 10.0)) < 1e-12
    g = np.array([0.1, 0.2])
    s.set_slip(g)
    np.testing.assert_allclose(np.ctypeslib.as_array(s.s.slip_a, (2,)), 1.0 / np.sqrt(1 + 2 * g))
    np.testing.assert_allclose(np.ctypeslib.as_array(s.s.slip_G32, (2,)), (1 + 3 * g) / (1 + 2 * g))
    s.set_slip(None)
    assert not s.s.slip
    s.close()


def test_cube_override_and_free(lib):
    """The 5-shell override swaps in caller-owned tables; closing must give
    the library its own tables back before stokes_free."""
    from libstokes_gb300 import System
    s = System(0, np.zeros((2, 3)), (6.0, 6.0, 6.0))
    nr0 = s.s.nr
    s.set_cube(5, 5)
    assert s.s.nr == 11 ** 3 and s.s.kmax == 0.0 and s.s.kmaxx == 5
    s.close()
    s = System(0, np.zeros((2, 3)), (6.0, 6.0, 6.0))
    s.set_cube(2, 2)
    s.restore_table()
    assert s.s.nr == nr0
    s.close()
