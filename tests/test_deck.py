"""The deck front end (msx_deck) reads the reference's keyword subset.
CPU: parse summaries of decks written the way the reference reads them.
GPU: running the golden decks through msx_deck reproduces the reference."""
import json
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from golden_cases import load, load_extractions, load_force_files, load_loads, names

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
    O.write_deck(str(tmp_path / "deck.inp"), mesh, mats, solvers, mat_elems, load_loads(name),
                 load_extractions(name)[0])
    return mesh, mats, solvers, ref, steps


@pytest.mark.parametrize("name", ["cube3_cnh_chain", "cube2_two_materials", "cube3_cnh_inst", "tet12_stvk",
                                  "cube3_cnh_force_gravity", "cube3_nh_gravity_force"])
def test_parse_summary(tmp_path, name):
    mesh, mats, solvers, _, _ = write(tmp_path, name)
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True, check=True)
    d = json.loads(r.stdout)
    assert d["nodes"] == mesh.nn and d["elements"] == mesh.ne
    assert d["materials"] == len(mats) and d["solvers"] == len(solvers)
    L = load_loads(name)
    assert d["forces"] == (len(L.force_entries(mesh.nn)) if L else 0)
    assert d["gravity"] == (L.gravity() if L else 0.0)
    assert d["gravity_first"] == (L.gravity_first() if L else 0)
    for blk, s in zip(d["blocks"], solvers):
        assert (blk["t0"], blk["tf"], blk["sf"], blk["bcs"]) == (s.t0, s.tf, s.scale_factor, len(s.bcs))


@pytest.mark.parametrize("name", ["cube3_cnh_traction_pressure", "cube3_nh_loads_mixed", "cube4_stvk_pressure_ramp"])
def test_parse_surface_load_blocks(tmp_path, name):
    mesh, _, _, _, _ = write(tmp_path, name)
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True, check=True)
    d = json.loads(r.stdout)
    items = load_loads(name).items
    assert [b["kind"] for b in d["loads"]] == [it[0].replace("_", " ").upper() for it in items]
    for b, it in zip(d["loads"], items):
        if it[0] in ("traction_inst", "traction_ramp", "pressure_inst", "pressure_ramp"):
            assert b["face"] == it[4] and b["elements"] == len(it[5])
        elif it[0] == "force":
            assert b["entries"] == 3 * len(it[4])


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


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cube3_cnh_ramp", "cube3_cnh_chain", "cube10_stvk_S", "cube3_stvk_activation"])
def test_deck_outputs_follow_reference_cadence(tmp_path, name):
    """VTK outputs at the reference's *Outputs cadence, final fields as the
    reference's own VTK file (6 digits there)."""
    mesh, mats, solvers, ref, steps = write(tmp_path, name)
    d = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    outdir = tmp_path / "out"
    outdir.mkdir()
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-outputDir", str(outdir),
                        "-precision", "exact"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    outs = O.read_vtk_outputs(str(outdir))
    times = np.array([o[0] for o in outs])
    assert len(times) == len(d["vtk_times"])
    assert np.allclose(times, d["vtk_times"], rtol=1e-5, atol=1e-12)
    _, cau, E, vms = outs[-1]
    for mine, refv in ((cau, d["vtk_cauchy"]), (E, d["vtk_E"]), (vms, d["vtk_vms"])):
        scale = max(np.abs(refv).max(), 1e-300)
        assert np.all(np.abs(mine - refv) <= 6e-6 * np.abs(refv) + 1e-6 * scale)


@pytest.mark.parametrize("param,c1,cl", [("0.5, 2", 0.5, 2.0), ("3", 0.06, 3.0), ("", 0.06, 1.2)])
def test_parse_viscosity_keywords(tmp_path, param, c1, cl):
    """*Bulk viscosity in the first of two solver blocks: the reader keeps it on
    in the second (the reference never resets its flag) and reads "c1, cl" as
    the reference's character scan does (a lone number is cl; defaults
    0.06, 1.2)."""
    write(tmp_path, "cube3_cnh_bulk_viscosity")
    text = (tmp_path / "deck.inp").read_text()
    first = text.index("*Bulk viscosity")
    second = text.index("*Bulk viscosity", first + 1)
    end = text.index("\n", text.index("\n", second) + 1) + 1
    text = text[:second] + text[end:]                         # only the first block names it
    text = text.replace("*Bulk viscosity\n0.5, 2\n", "*Bulk viscosity\n%s\n" % param)
    (tmp_path / "deck.inp").write_text(text)
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True, check=True)
    blocks = json.loads(r.stdout)["blocks"]
    assert [(b["visc"], b["visc_c1"], b["visc_cl"]) for b in blocks] == [(1, c1, cl)] * 2


def test_parse_node_extractions(tmp_path):
    write(tmp_path, "cube3_cnh_extraction")
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True, check=True)
    d = json.loads(r.stdout)
    ex, files = load_extractions("cube3_cnh_extraction")
    assert sorted(e["name"] + ".csv" for e in d["extractions"]) == sorted(files)
    assert [e["nodes"] for e in d["extractions"]] == [len(x[4]) for x in ex]


ELEMENT_CASES = ["cube3_cnh_element_extraction", "cube2_two_materials_element_extraction", "cube4_le_ramp",
                 "cube3_stvk_activation"]


@pytest.mark.parametrize("name", ELEMENT_CASES)
def test_parse_element_extractions(tmp_path, name):
    """One extraction per file the reference wrote: All_<TYPE>_<op> or
    <name>_<TYPE>_<op>, the first block of a name kept."""
    write(tmp_path, name)
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True, check=True)
    d = json.loads(r.stdout)
    _, files = load_extractions(name)
    assert sorted(e["name"] + ".csv" for e in d["extractions"]) == sorted(files)
    mid = [e for e in d["extractions"] if e["name"] == "mid_SVM_Max"]
    assert not mid or mid[0]["elements"] == 40


@pytest.mark.parametrize("block,message", [("all,SVM,Rough\nAll", "Rough"), ("v,VOLUME,Mean\nAll", "VOLUME"),
                                           ("x,STRAIN,Max\nAll", "STRAIN"), ("x,SVM,Max\n999", "out of range")])
def test_element_extraction_refusals(tmp_path, block, message):
    write(tmp_path, "cube3_cnh_ramp")
    p = tmp_path / "deck.inp"
    p.write_text(p.read_text().replace("*END\n", "*EXTRACTION, ELEMENT\n" + block + "\n*END\n"))
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and message in r.stderr


def test_element_extraction_all_and_list_in_one_block(tmp_path):
    write(tmp_path, "cube3_cnh_ramp")
    p = tmp_path / "deck.inp"
    p.write_text(p.read_text().replace("*END\n", "*EXTRACTION, ELEMENT\nsome,KVM,Max\nAll\n3\n5\n*END\n"))
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True, check=True)
    ex = json.loads(r.stdout)["extractions"]
    assert ex == [{"name": "All_KVM_Max", "elements": "All"}, {"name": "some_KVM_Max", "elements": 2}]


def _csv(text):
    lines = text.strip().splitlines()
    return lines[0], np.array([[float(x) for x in ln.split(",")] for ln in lines[1:]])


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("exact", 1e-12), ("fp64", 1e-9)])
def test_node_extraction_matches_reference_files(tmp_path, precision, tol):
    """*EXTRACTION, NODE: the files the reference writes every step, same names,
    headers, rows (times and values at %.16g)."""
    write(tmp_path, "cube3_cnh_extraction")
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-precision", precision,
                        "-outputDir", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _, files = load_extractions("cube3_cnh_extraction")
    for fname, ref_text in files.items():
        got = (out / fname).read_text()
        h_ref, v_ref = _csv(ref_text)
        h_got, v_got = _csv(got)
        assert h_got == h_ref and v_got.shape == v_ref.shape, fname
        scale = max(np.abs(v_ref[:, 1:]).max(), 1e-300)
        assert np.allclose(v_got[:, 0], v_ref[:, 0], rtol=tol, atol=0), fname
        assert np.abs(v_got[:, 1:] - v_ref[:, 1:]).max() <= tol * scale, fname


@pytest.mark.gpu
@pytest.mark.parametrize("name", ELEMENT_CASES)
@pytest.mark.parametrize("precision,tol", [("exact", 1e-12), ("fp64", 1e-9), ("mixed", 1e-4)])
def test_element_extraction_matches_reference_files(tmp_path, name, precision, tol):
    """*EXTRACTION, ELEMENT: the files the reference writes every step, same
    names, headers and rows; values within tol of the file's largest value."""
    write(tmp_path, name)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-precision", precision,
                        "-outputDir", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _, files = load_extractions(name)
    assert sorted(f.name for f in out.glob("*.csv")) == sorted(files)
    for fname, ref_text in files.items():
        h_ref, v_ref = _csv(ref_text)
        h_got, v_got = _csv((out / fname).read_text())
        assert h_got == h_ref and v_got.shape == v_ref.shape, fname
        assert np.allclose(v_got[:, 0], v_ref[:, 0], rtol=1e-12 if precision != "mixed" else 1e-6, atol=0), fname
        scale = max(np.abs(v_ref[:, 1]).max(), 1e-300)
        assert np.abs(v_got[:, 1] - v_ref[:, 1]).max() <= tol * scale, (fname, np.abs(v_got[:, 1] - v_ref[:, 1]).max())


def test_parse_print_forces(tmp_path):
    mesh, _, solvers, _, _ = write(tmp_path, "cube3_cnh_print_forces")
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-parse-only"],
                       capture_output=True, text=True, check=True)
    blocks = json.loads(r.stdout)["blocks"]
    assert [(b["force_freq"], b["force_out"]) for b in blocks] == [(s.forces_out[0], len(s.forces_out[1]))
                                                                   for s in solvers]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("exact", 0.0), ("fp64", 1e-9), ("dword", 1e-9), ("mixed", 1e-4)])
def test_print_forces_match_reference_files(tmp_path, precision, tol):
    """*Forces: the reference's externalForces<t0>-<tf>.csv files, same rows; the
    forces within the printed 6 decimals (one unit of the last digit, or tol of
    the file's largest force)."""
    write(tmp_path, "cube3_cnh_print_forces")
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-precision", precision,
                        "-outputDir", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for fname, ref_text in load_force_files("cube3_cnh_print_forces").items():
        got = (out / fname).read_text().strip().split("\n")
        ref = ref_text.strip().split("\n")
        assert got[0] == ref[0] and len(got) == len(ref), fname
        g = np.array([[float(x) for x in ln.split(",")[:4]] for ln in got[1:]])
        e = np.array([[float(x) for x in ln.split(",")[:4]] for ln in ref[1:]])
        assert np.array_equal(g[:, :2], e[:, :2]) and np.abs(g[:, 3] - e[:, 3]).max() <= 1.01e-6, fname
        scale = np.abs(e[:, 2]).max()
        assert np.abs(g[:, 2] - e[:, 2]).max() <= 1.01e-6 + tol * scale, fname


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("exact", 1e-12), ("fp64", 1e-9), ("dword", 1e-9)])
def test_all_outputs_in_one_chain(tmp_path, precision, tol):
    """A two-block chain with VTK outputs, node and element extraction, *Forces
    and surface loads: the same files as the reference (names, headers, rows),
    the VTK outputs at its times."""
    name = "cube3_cnh_all_outputs"
    write(tmp_path, name)
    d = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([DECK, "-input", "deck.inp", "-inputDir", str(tmp_path), "-outputDir", str(out),
                        "-precision", precision], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    times = np.array([o[0] for o in O.read_vtk_outputs(str(out))])
    assert len(times) == len(d["vtk_times"]) and np.allclose(times, d["vtk_times"], rtol=1e-5, atol=1e-12)
    _, files = load_extractions(name)
    assert sorted(f.name for f in out.glob("*.csv")) == sorted(files)
    for fname, ref_text in files.items():
        ref = ref_text.strip().split("\n")
        got = (out / fname).read_text().strip().split("\n")
        assert got[0] == ref[0] and len(got) == len(ref), fname
        g = np.array([[float(x) for x in ln.rstrip(",").split(",")] for ln in got[1:]])
        e = np.array([[float(x) for x in ln.rstrip(",").split(",")] for ln in ref[1:]])
        if fname.startswith("externalForces"):   # %f: six decimals
            assert np.array_equal(g[:, :2], e[:, :2]) and np.abs(g[:, 3] - e[:, 3]).max() <= 1.01e-6, fname
            assert np.abs(g[:, 2] - e[:, 2]).max() <= 1.01e-6 + tol * np.abs(e[:, 2]).max(), fname
        else:                                     # %.16g
            assert np.allclose(g[:, 0], e[:, 0], rtol=1e-12, atol=0), fname
            assert np.abs(g[:, 1:] - e[:, 1:]).max() <= tol * max(np.abs(e[:, 1:]).max(), 1e-300), fname
