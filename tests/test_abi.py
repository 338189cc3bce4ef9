"""C ABI checks that need no GPU: the library loads, exports every entry point
that include/msx.h declares, and its host-only pieces agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import msx
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="session", autouse=True)
def built():
    import build
    build.build()


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "msx.h")).read()
    return sorted(set(re.findall(r"\b(msx_[a-z_0-9]+)\s*\(", src)))


def test_header_and_binding_agree():
    assert sorted(msx.SYMBOLS) == declared_symbols()


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(msx.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


@pytest.mark.parametrize("n", [1, 3, 7])
def test_cube_generator_matches_oracle(n):
    X, conn = msx.mesh_cube(n, seed=99, jitter=0.1)
    m = O.cube_mesh(n, seed=99, jitter=0.1)
    assert np.array_equal(X, m.X) and np.array_equal(conn, m.conn)


def test_cube_generator_matches_golden_mesh():
    d = np.load(os.path.join(ROOT, "tests", "golden", "cube10_cnh_S.npz"))
    X, conn = msx.mesh_cube(10)
    assert np.array_equal(X, d["X"]) and np.array_equal(conn, d["conn"])


def test_cube_bcs_match_oracle_recipe():
    assert msx.cube_bcs(4, 0.01) == O.cube_bcs(4, 0.01)
    assert msx.cube_bcs(3, 0.5, msx.BC_INST) == O.cube_bcs(3, 0.5, O.BC_INST)


def test_bad_arguments_are_reported_not_fatal():
    L = msx.load()
    st = L.msx_mesh_cube(0, 1, 0.1, None, None)
    assert st == 1 and b"cube" in L.msx_last_error()
    h = C.c_void_p()
    st = L.msx_create(None, None, 0, None, 0, None, C.byref(h))
    assert st == 1 and not h.value
