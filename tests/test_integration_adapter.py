"""The reference-side binding compiles, links and maps decks as the reference reads them.

v.1.1_gb300/integration/solverExplicitGPU.h is the `solvers` plugin a
maintainer adds to MuPhiSim (solvers.h:98-101).  This test compiles it with the
reference's own headers and flags (-std=c++11, the shim standing in for PETSc
and MPI), instantiates it, and links it with the reference's objects built
from its sources here (oracle/Makefile `ref`) and with libmsx: every reference
accessor and every msx_* entry point the adapter calls must resolve.  The
binary is then run in its link-check mode (it returns before building
anything: there is no GPU here).  Skipped where the reference's sources are
not mounted."""
import glob
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.environ.get("MSX_REFERENCE_SRC", "/root/reference/src")
ORACLE = os.path.join(ROOT, "oracle")
CUDA_LIB = "/usr/local/cuda/lib64"

MAIN = r"""
#include "solverExplicitGPU.h"
int main(int argc, char **argv)
{
    if (argc < 1000) return 0;   // link check: nothing below runs
    vector<classNodes *> nod;
    vector<classDirichlet *> dnod;
    classOutputs *outputs = nullptr;
    classPrintForces *forces = nullptr;
    vector<int> none;
    string petsc_solver, petsc_precon;
    vector<double> para_AV = {0.06, 1.2};
    solvers *s = new classSolverExplicitGPU(nod, 3, 0, dnod, 0.5, outputs, 0.0, 1.0, "EXPLICIT", none, none, none,
                                            1, para_AV, forces, false, petsc_solver, petsc_precon, false,
                                            MSX_PREC_FP64);
    vector<classNeumannBCs *> loads;
    vector<classGPs *> gps;
    vector<classElements *> elem, geo;
    vector<constitutiveModels *> laws;
    s->calculate(loads, gps, 0, nod, elem, none, none, none, none, none, geo, laws, none, 0, 0);
    delete s;
    return 0;
}
"""


def _link(tmp_path, src, exe):
    """g++ with the reference's flags, its headers, our shim, include/ and the
    adapter; linked with the reference's objects and libmsx."""
    import build as msx_build
    lib = msx_build.build()
    import oracle
    oracle.build_reference()
    objs = [o for o in glob.glob(os.path.join(ORACLE, "_ref", "obj", "**", "*.o"), recursive=True)
            if os.sep + "harness" + os.sep not in o]
    assert objs, "reference objects missing"
    dirs = [REF_SRC] + [os.path.join(REF_SRC, d) for d in
                        ("IO", "constitutiveModels", "mathematics", "solvers", "spatialDiscretisation")]
    libdir = os.path.dirname(lib)
    cmd = (["g++", "-std=c++11", "-O1", "-w", "-DNDEBUG", "-I" + os.path.join(ORACLE, "shim"),
            "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "v.1.1_gb300", "integration")] +
           ["-I" + d for d in dirs] + [str(src)] + objs +
           ["-L" + libdir, "-lmsx", "-Wl,-rpath," + libdir, "-L" + CUDA_LIB, "-Wl,-rpath-link," + CUDA_LIB,
            "-Wl,-rpath," + CUDA_LIB, "-lm", "-o", str(exe)])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


needs_ref = pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not mounted")


@needs_ref
def test_adapter_compiles_and_links_against_the_reference(tmp_path):
    src = tmp_path / "adapter_main.cpp"
    src.write_text(MAIN)
    exe = _link(tmp_path, src, tmp_path / "adapter_main")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr


@pytest.fixture(scope="module")
def dump_exe(tmp_path_factory):
    if not os.path.isdir(REF_SRC):
        pytest.skip("reference sources not mounted")
    d = tmp_path_factory.mktemp("adapter_dump")
    return _link(d, os.path.join(ROOT, "tests", "adapter_dump.cpp"), d / "adapter_dump")


def _parse_loads(text):
    """The L / LE / LF lines of the dump: [(kind, face, t0, tf, values, elems, forces)]."""
    blocks = []
    for line in text.splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "L":
            blocks.append([int(f[2]), int(f[3]), float(f[4]), float(f[5]), tuple(float(x) for x in f[6:9]), [], []])
        elif f[0] == "LE":
            blocks[int(f[1])][5].append(int(f[2]))
        elif f[0] == "LF":
            blocks[int(f[1])][6].append((int(f[2]), float(f[3]), float(f[4]), float(f[5])))
    return blocks


def _expected_blocks(items, nn):
    """msx_load_block contents for the deck's load items, as the deck reader
    builds them (force entries: dof = node + comp * nn, value = F_comp * Ff)."""
    kinds = {"force": 0, "gravity": 1, "traction_inst": 2, "traction_ramp": 3, "pressure_inst": 4, "pressure_ramp": 5}
    out = []
    for it in items:
        if it[0] == "force":
            _, t0, tf, Ff, rows = it
            forces = [(node + c * nn, t0, tf, F[c] * Ff) for node, *F in rows for c in range(3)]
            out.append([0, 0, 0.0, 0.0, (0.0, 0.0, 0.0), [], forces])
        elif it[0] == "gravity":
            out.append([1, 0, 0.0, 0.0, (float(it[1]), 0.0, 0.0), [], []])
        else:
            kind, t0, tf, val, S, elems = it
            vals = (float(val), 0.0, 0.0) if kind.startswith("pressure") else tuple(float(x) for x in val)
            out.append([kinds[kind], S, t0, tf, vals, list(elems), []])
    return out


LOAD_DECKS = ["cube3_cnh_traction_pressure", "cube3_nh_loads_mixed", "cube3_cnh_force_gravity",
              "cube3_nh_gravity_force", "cube4_stvk_pressure_ramp"]


def _write_load_deck(tmp_path, name):
    import numpy as np
    import oracle as O
    from golden_cases import load, load_loads
    mesh, mats, solvers, _, _ = load(name)
    mat_elems = None
    if mesh.elem_mat is not None:
        mat_elems = [np.nonzero(mesh.elem_mat == k)[0] for k in range(len(mats))]
    items = load_loads(name).items
    O.write_deck(str(tmp_path / "deck.inp"), mesh, mats, solvers, mat_elems, load_loads(name))
    (tmp_path / "out").mkdir()
    return mesh, items


@needs_ref
@pytest.mark.parametrize("name", LOAD_DECKS)
def test_adapter_maps_the_reference_loads(tmp_path, dump_exe, name):
    """Neumann loads through the plugin: with the deck read by the reference's
    own readers (one classNeumannBCs per block), the plugin's load blocks --
    read from the same file by the library and checked against each reference
    object's class, node ids, face count and amount at tf -- are the deck's
    blocks in deck order, bit for bit what msx_deck hands to
    msx_set_load_blocks (boundaryConditions.cpp:75-138 applies them in that
    order)."""
    mesh, items = _write_load_deck(tmp_path, name)
    r = subprocess.run([str(dump_exe), "-input", "deck.inp", "-inputDir", ".", "-outputDir", "out"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.stdout[-1000:], r.stderr[-2000:])
    got = _parse_loads(r.stdout)
    want = _expected_blocks(items, mesh.nn)
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert g[0] == w[0] and g[5] == w[5] and g[6] == w[6], (g[:5], w[:5])
        if w[0] >= 2:           # surface loads: face, t0, tf, values
            assert (g[1], g[2], g[3], g[4]) == (w[1], w[2], w[3], w[4])
        if w[0] == 1:
            assert g[4][0] == w[4][0]
    # the front end's own view of the same file
    import build as msx_build
    deck = os.path.join(os.path.dirname(msx_build.LIB), "msx_deck")
    p = subprocess.run([deck, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True, timeout=60)
    assert p.returncode == 0, p.stderr
    import json
    d = json.loads(p.stdout)
    assert [(b["kind"], b["elements"], b["entries"]) for b in d["loads"]] == \
        [({0: "FORCE", 1: "GRAVITY", 2: "TRACTION INST", 3: "TRACTION RAMP", 4: "PRESSURE INST",
           5: "PRESSURE RAMP"}[g[0]], len(g[5]), len(g[6])) for g in got]


@needs_ref
def test_adapter_refuses_a_deck_that_does_not_match_the_model(tmp_path, dump_exe):
    """If the reference's load objects and the deck file disagree (here: one
    object fewer), the plugin stops the block instead of loading the deck."""
    _write_load_deck(tmp_path, "cube3_nh_loads_mixed")
    r = subprocess.run([str(dump_exe), "-input", "deck.inp", "-inputDir", ".", "-outputDir", "out",
                        "-drop-last-load"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 4
    assert "Neumann blocks, the model" in r.stdout


def _parse_dump(text):
    X, C, M, A, S, B = {}, {}, {}, {}, [], {}
    for line in text.splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "X":
            X[int(f[1])] = [float(v) for v in f[2:5]]
        elif f[0] == "C":
            C[int(f[1])] = [int(v) for v in f[2:6]]
        elif f[0] == "M":
            M[int(f[1])] = (int(f[2]), float(f[3]), float(f[4]), float(f[5]))
        elif f[0] == "A":
            A[int(f[1])] = float(f[2])
        elif f[0] == "S":
            S.append((float(f[2]), float(f[3]), float(f[4])))
        elif f[0] == "B":
            B.setdefault(int(f[1]), []).append((int(f[2]), int(f[3]), float(f[4])))
    return X, C, M, A, S, B


@needs_ref
@pytest.mark.parametrize("name", ["tet12_stvk", "cube2_two_materials", "cube3_cnh_chain", "cube3_cnh_inst",
                                  "cube2_le_cnh", "cube3_stvk_activation", "cube3_le_activation_chain",
                                  "cube4_nh_ramp"])
def test_adapter_maps_the_reference_deck(tmp_path, dump_exe, name):
    """What the plugin hands to msx_create, read from the reference's own
    objects for a golden deck, is that deck's mesh, laws and BCs: coordinates
    and 0-based connectivity exactly, each element's law and E, nu, rho
    exactly, the *INITINTVARS activation times, and per solver block the
    Dirichlet entries (instantaneous: U; ramp: the rate U / (tf - t0) the
    reference stores, bit for bit the library's own division)."""
    import numpy as np
    import oracle as O
    from golden_cases import load
    mesh, mats, solvers, _, _ = load(name)
    mat_elems = None
    if mesh.elem_mat is not None:
        mat_elems = [np.nonzero(mesh.elem_mat == k)[0] for k in range(len(mats))]
    O.write_deck(str(tmp_path / "deck.inp"), mesh, mats, solvers, mat_elems)
    (tmp_path / "out").mkdir()
    r = subprocess.run([str(dump_exe), "-input", "deck.inp", "-inputDir", ".", "-outputDir", "out"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    X, C, M, A, S, B = _parse_dump(r.stdout)
    assert np.array_equal(np.array([X[i] for i in range(mesh.nn)]).T, mesh.X)
    assert np.array_equal(np.array([C[e] for e in range(mesh.ne)]), mesh.conn)
    em = mesh.elem_mat if mesh.elem_mat is not None else np.zeros(mesh.ne, int)
    for e in range(mesh.ne):
        m = mats[int(em[e])]
        assert M[e] == (m.law, m.young, m.nu, m.rho), (e, M[e], m)
        if getattr(mesh, "act_time", None) is not None and m.law >= O.STVK:
            assert A[e] == float(mesh.act_time[e]), e
    assert len(S) == len(solvers)
    for k, s in enumerate(solvers):
        assert S[k] == (s.t0, s.tf, s.scale_factor)
        want = sorted((dof, 1 if mode == O.BC_INST else 3, value if mode == O.BC_INST else value / (s.tf - s.t0))
                      for dof, mode, value, _ in s.bcs)
        assert sorted(B.get(k, [])) == want, k
