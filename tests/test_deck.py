"""The deck front end (msx_deck) reads the reference's keyword subset.
CPU: parse summaries of decks written the way the reference reads them.
GPU: running the golden decks through msx_deck reproduces the reference."""
import json
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from golden_cases import load, names

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECK = os.path.join(ROOT, "v.1.1_gb300", "_build", "msx_deck")


@pytest.fixture(scope="module", autouse=True)
def built():
    import build
    build.build()


def write(tmp_path, name):
    mesh, mats, solvers, ref, steps = load(name)
    mat_elems = None
    if mesh.elem_mat is not None:
        mat_elems = [np.nonzero(mesh.elem_mat == k)[0] for k in range(len(mats))]
    O.write_deck(str(tmp_path / "deck.inp"), mesh, mats, solvers, mat_elems)
    return mesh, mats, solvers, ref, steps


@pytest.mark.parametrize("name", ["cube3_cnh_chain", "cube2_two_materials", "cube3_cnh_inst", "tet12_stvk"])
def test_parse_summary(tmp_path, name):
    mesh, mats, solvers, _, _ = write(tmp_path, name)
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True, check=True)
    d = json.loads(r.stdout)
    assert d["nodes"] == mesh.nn and d["elements"] == mesh.ne
    assert d["materials"] == len(mats) and d["solvers"] == len(solvers)
    for blk, s in zip(d["blocks"], solvers):
        assert (blk["t0"], blk["tf"], blk["sf"], blk["bcs"]) == (s.t0, s.tf, s.scale_factor, len(s.bcs))


def test_rejects_out_of_scope_keywords(tmp_path):
    mesh, mats, solvers, _, _ = write(tmp_path, "cube3_cnh_ramp")
    p = tmp_path / "deck.inp"
    p.write_text(p.read_text().replace("*SOLVER, EXPLICIT", "*SOLVER, IMPLICIT STATIC"))
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "EXPLICIT" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", names())
def test_deck_run_matches_reference(tmp_path, name):
    mesh, mats, solvers, (u, v, a), steps = write(tmp_path, name)
    out = tmp_path / "final.bin"
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-precision", "exact",
                        "-dump", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert ("total %d steps" % steps) in r.stdout
    d = np.fromfile(out, dtype=np.float64).reshape(3, -1)
    assert np.linalg.norm(d[0] - u) <= 1e-12 * np.linalg.norm(u)
