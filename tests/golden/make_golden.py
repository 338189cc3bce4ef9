"""Generate the golden fixtures in this folder from the reference MuPhiSim.

Run in a container where the reference sources are mounted:
    python tests/golden/make_golden.py [case ...]
It compiles the reference in place behind our PETSc/MPI shim (oracle/Makefile),
runs each case below through the reference's own input-deck reader and
explicit solver, and stores the inputs and the reference's final u, v, a
(float64, exact bits) as <case>.npz.  The GPU tests and the oracle tests
compare against these files; nothing here is needed at test time.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402


def tet12_mesh(ref_src):
    """Nodes and C3D4 connectivity of applications/examples/3Dcube.inp."""
    path = os.path.join(ref_src, "..", "applications", "examples", "3Dcube.inp")
    nodes, elems, mode = [], [], None
    for line in open(path):
        s = line.strip()
        if s.startswith("*"):
            mode = "n" if s.startswith("*Node") else ("e" if s.startswith("*Element") else None)
            continue
        if mode == "n":
            nodes.append([float(x) for x in s.split(",")[1:]])
        elif mode == "e":
            elems.append([int(x) - 1 for x in s.split(",")[1:]])
    X = np.ascontiguousarray(np.array(nodes).T)
    return O.Mesh(X, np.array(elems, np.int32))


def tet_face(c, S):
    """Nodes of face S (1..4) of a tet, as classLinearTetrahedra::getSubElement orders them."""
    if S == 1:
        return (c[0], c[1], c[2])
    if S in (2, 3):
        return (c[S - 2], c[3], c[S - 1])
    return (c[0], c[2], c[S - 1])


def plane_faces(mesh, coord, value):
    """[(S, [elems])] of the tet faces lying on the plane X[coord] == value, by face index."""
    out = {}
    for e in range(mesh.ne):
        for S in range(1, 5):
            if all(abs(mesh.X[coord, n] - value) < 1e-12 for n in tet_face(mesh.conn[e], S)):
                out.setdefault(S, []).append(e)
    return sorted(out.items())


def cases(ref_src):
    cnh, nh, stvk = O.COMPRESSIBLE_NH, O.NEO_HOOKEAN, O.STVK
    out = {}
    m3 = O.cube_mesh(3)
    out["cube3_cnh_ramp"] = (m3, [O.Material(cnh)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.002))])
    m4 = O.cube_mesh(4)
    out["cube4_nh_ramp"] = (m4, [O.Material(nh)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(4, 0.002))])
    out["cube4_stvk_ramp"] = (m4, [O.Material(stvk)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(4, 0.002))])
    out["cube3_cnh_inst"] = (m3, [O.Material(cnh)],
                             [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.001, O.BC_INST))])
    out["cube3_cnh_chain"] = (m3, [O.Material(cnh)],
                              [O.Solver(0.0, 0.01, 0.5, O.cube_bcs(3, 0.001)),
                               O.Solver(0.01, 0.02, 0.4, O.cube_bcs(3, 0.003))])
    m2 = O.cube_mesh(2)
    m2.elem_mat = (np.arange(m2.ne) % 2).astype(np.int32)
    out["cube2_two_materials"] = (m2, [O.Material(nh, 1e6, 0.3, 1000.0), O.Material(stvk, 3e6, 0.25, 2000.0)],
                                  [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(2, 0.002))])
    t12 = tet12_mesh(ref_src)
    nn = t12.nn
    bcs = [(node + c * nn, O.BC_RAMP, (-0.5 if (node, c) == (3, 1) else 0.0), 0)
           for node in (0, 3, 6, 7) for c in range(3)]
    out["tet12_stvk"] = (t12, [O.Material(stvk, 1e9, 0.3, 1000.0)], [O.Solver(0.0, 0.05, 0.1, bcs)])
    top = [i + 4 * j + 16 * 3 for j in range(4) for i in range(4)]
    forces = ("force", 0.0, 0.015, 2.5, [(nd, 0.1 * k, -0.2, 0.3) for k, nd in enumerate(top[:6])])
    out["cube3_cnh_force_gravity"] = (m3, [O.Material(cnh)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.0))],
                                      O.Loads([forces, ("gravity", 9.81)]))
    out["cube3_nh_gravity_force"] = (m3, [O.Material(nh)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.0))],
                                     O.Loads([("gravity", 9.81), forces]))
    # surface loads: traction on the top face, pressure on the x = 1 face
    top3, side3 = plane_faces(m3, 2, 1.0), plane_faces(m3, 0, 1.0)
    out["cube3_cnh_traction_pressure"] = (
        m3, [O.Material(cnh)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.0))],
        O.Loads([("traction_ramp", 0.0, 0.015, (1e3, -2e3, 4e3), S, el) for S, el in top3] +
                [("pressure_inst", 0.0, 0.02, 5e3, S, el) for S, el in side3]))
    out["cube3_nh_loads_mixed"] = (
        m3, [O.Material(nh)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.0))],
        O.Loads([("gravity", 9.81)] + [("pressure_ramp", 0.0, 0.02, 5e3, S, el) for S, el in side3] +
                [forces] + [("traction_inst", 0.002, 0.012, (0.0, 0.0, -2e3), S, el) for S, el in top3]))
    # node data extraction (*EXTRACTION, NODE): every node datatype and operation
    node_on = lambda mesh, c, v: [i for i in range(mesh.nn) if abs(mesh.X[c, i] - v) < 1e-12]
    topn, siden, botn = node_on(m3, 2, 1.0), node_on(m3, 0, 1.0), node_on(m3, 2, 0.0)
    out["cube3_cnh_extraction"] = (
        m3, [O.Material(cnh)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.0))],
        O.Loads([("traction_ramp", 0.0, 0.015, (1e3, -2e3, 4e3), S, el) for S, el in top3] +
                [("pressure_inst", 0.0, 0.02, 5e3, S, el) for S, el in side3] + [("gravity", 9.81)]),
        [("top", "Unknown", "Mean", 2, topn), ("top", "Unknown", "Rough", 2, topn[:5]),
         ("side", "ExternalForce", "Sum", 0, siden), ("side", "ExternalForce", "Rough", 2, siden[:4]),
         ("bottom", "InternalForce", "Max", 2, botn), ("mid", "InternalForce", "Min", 1, list(range(20, 40))),
         ("mid", "Unknown", "Max", 0, list(range(20, 40)))])
    # element data extraction (*EXTRACTION, ELEMENT): every quantity kind and
    # operation over All and over element lists (one given in reverse order, one
    # with repeats, and a second block of an existing name, which the reference drops)
    every = lambda t, op: ("element", "all", t, op, None)
    mid = list(range(40, 80))
    out["cube3_cnh_element_extraction"] = (
        m3, [O.Material(cnh)], [O.Solver(0.0, 0.04, 0.5, O.cube_bcs(3, 0.002))],
        O.Loads([("traction_ramp", 0.0, 0.015, (1e3, -2e3, 4e3), S, el) for S, el in top3] +
                [("pressure_inst", 0.0, 0.02, 5e3, S, el) for S, el in side3] + [("gravity", 9.81), forces]),
        [every(t, op) for t in ("DEFO_ENERGY", "KIN_ENERGY") for op in ("Sum", "Mean", "Max", "Min")] +
        [every("EXTERNAL_ENERGY", "Sum"), every("VOLUME", "Sum"), every("VOLUME", "Max"), every("VOLUME", "Min"),
         every("FXX", "Mean"), every("FYZ", "Sum"), every("FZZ", "Max"), every("FZX", "Min"),
         every("PXX", "Mean"), every("PZZ", "Sum"), every("PXY", "Max"), every("PYZ", "Min"),
         every("SVM", "Max"), every("SVM", "Mean"), every("KVM", "Sum"), every("INVAR1", "Mean"),
         ("element", "mid", "FZZ", "Mean", mid), ("element", "mid", "PZZ", "Sum", mid[::-1]),
         ("element", "mid", "SVM", "Max", mid), ("element", "mid", "SVM", "Max", [0, 1, 2]),
         ("element", "mid", "DEFO_ENERGY", "Sum", mid), ("element", "mid", "KIN_ENERGY", "Mean", mid),
         ("element", "mid", "VOLUME", "Min", mid), ("element", "dup", "PZZ", "Sum", mid + mid[:5])])
    out["cube2_two_materials_element_extraction"] = (
        m2, [O.Material(nh, 1e6, 0.3, 1000.0), O.Material(stvk, 3e6, 0.25, 2000.0)],
        [O.Solver(0.0, 0.04, 0.5, O.cube_bcs(2, 0.002))], None,
        [every("DEFO_ENERGY", "Sum"), every("DEFO_ENERGY", "Max"), every("KIN_ENERGY", "Sum"),
         every("SVM", "Mean"), every("SVM", "Max"), every("KVM", "Max"), every("PXX", "Mean"),
         every("FXX", "Min"), every("VOLUME", "Sum"), every("EXTERNAL_ENERGY", "Sum"),
         ("element", "nh", "DEFO_ENERGY", "Mean", list(range(0, m2.ne, 2))),
         ("element", "stvk", "DEFO_ENERGY", "Mean", list(range(1, m2.ne, 2)))])
    # *Forces output (internal force of listed node DOFs at a frequency): two
    # chained blocks, one slower than the step (period 1/500 s), one faster (every step)
    botn3 = node_on(m3, 2, 0.0)
    out["cube3_cnh_print_forces"] = (
        m3, [O.Material(cnh)],
        [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.002),
                  forces_out=(500.0, [(nd, 2) for nd in botn3[:6]] + [(21, 0), (22, 1), (42, 2)])),
         O.Solver(0.02, 0.03, 0.4, O.cube_bcs(3, 0.003), forces_out=(1e5, [(botn3[0], 2), (30, 1)]))])
    # the linear-elastic law (*Linear-Elastic): alone with element extraction, and
    # beside the compressible neo-Hookean law on a two-material mesh
    le = O.LINEAR_ELASTIC
    out["cube4_le_ramp"] = (
        m4, [O.Material(le)], [O.Solver(0.0, 0.03, 0.5, O.cube_bcs(4, 0.002))], None,
        [every("DEFO_ENERGY", "Sum"), every("DEFO_ENERGY", "Max"), every("SVM", "Max"), every("PZZ", "Mean"),
         every("KVM", "Min"), every("VOLUME", "Sum")])
    m2b = O.cube_mesh(2)
    m2b.elem_mat = (np.arange(m2b.ne) % 2).astype(np.int32)
    out["cube2_le_cnh"] = (m2b, [O.Material(le, 2e6, 0.28, 1200.0), O.Material(cnh, 1e6, 0.3, 1000.0)],
                           [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(2, 0.002))])
    # every output of the explicit solver at once in a two-block chain: VTK at the
    # *Outputs cadence, node and element extraction, *Forces, with surface loads
    out["cube3_cnh_all_outputs"] = (
        m3, [O.Material(cnh)],
        [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.002), forces_out=(300.0, [(nd, 2) for nd in botn3[:4]]),
                  outputs=4),
         O.Solver(0.02, 0.035, 0.45, O.cube_bcs(3, 0.003), forces_out=(1e4, [(21, 0), (42, 2)]), outputs=3)],
        O.Loads([("traction_ramp", 0.0, 0.015, (1e3, -2e3, 4e3), S, el) for S, el in top3] + [("gravity", 9.81)]),
        [("top", "Unknown", "Mean", 2, topn), ("bottom", "InternalForce", "Sum", 2, botn),
         every("DEFO_ENERGY", "Sum"), every("KIN_ENERGY", "Max"), every("EXTERNAL_ENERGY", "Sum"),
         ("element", "mid", "SVM", "Mean", mid)])
    # element birth (*ACTIVATION with activation times from *INITINTVARS): the upper
    # elements of a St-Venant-Kirchhoff cube come alive at two later times; a
    # linear-elastic chain whose second block runs with every element alive
    m3a = O.cube_mesh(3)
    zc = np.array([m3a.X[2, m3a.conn[e]].mean() for e in range(m3a.ne)])
    m3a.act_time = np.where(zc > 0.7, 0.009, np.where(zc > 0.4, 0.004, 0.0))
    out["cube3_stvk_activation"] = (
        m3a, [O.Material(stvk)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.002), activation=True, outputs=2)],
        O.Loads([("gravity", 9.81)]),
        [every("DEFO_ENERGY", "Sum"), every("KIN_ENERGY", "Sum"), every("VOLUME", "Sum"), every("FZZ", "Mean"),
         every("SVM", "Max"), every("DEFO_ENERGY", "Min"), ("element", "upper", "PZZ", "Mean", [int(e) for e in np.nonzero(zc > 0.7)[0]])])
    m3b = O.cube_mesh(3)
    m3b.act_time = np.where(zc > 0.5, 0.006, 0.0)
    out["cube3_le_activation_chain"] = (
        m3b, [O.Material(le)],
        [O.Solver(0.0, 0.01, 0.5, O.cube_bcs(3, 0.001), activation=True),
         O.Solver(0.01, 0.02, 0.5, O.cube_bcs(3, 0.002), activation=True)])
    side4 = plane_faces(m4, 0, 1.0)
    out["cube4_stvk_pressure_ramp"] = (
        m4, [O.Material(stvk)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(4, 0.001))],
        O.Loads([("pressure_ramp", 0.0, 0.02, 8e3, S, el) for S, el in side4]))
    # artificial viscosity: *Bulk viscosity in the first of two blocks (the reader
    # keeps it on in the second) and *Dev viscosity; the reference runs them with
    # its never-assigned element size and c0, which are 0 in its builds
    bulk = (O.VISC_BULK, 0.5, 2.0, 0.0, 0.0)
    out["cube3_cnh_bulk_viscosity"] = (
        m3, [O.Material(cnh)], [O.Solver(0.0, 0.01, 0.5, O.cube_bcs(3, 0.002), viscosity=bulk),
                                O.Solver(0.01, 0.02, 0.45, O.cube_bcs(3, 0.004), viscosity=bulk)])
    out["cube3_stvk_dev_viscosity"] = (
        m3, [O.Material(stvk)], [O.Solver(0.0, 0.02, 0.5, O.cube_bcs(3, 0.002),
                                          viscosity=(O.VISC_DEV, 1.0, 0.5, 0.0, 0.0))])
    m10 = O.cube_mesh(10)
    for name, law in (("cnh", cnh), ("nh", nh), ("stvk", stvk)):
        out["cube10_%s_S" % name] = (m10, [O.Material(law)], [O.Solver(0.0, 0.5, 0.5, O.cube_bcs(10, 0.05))])
    return out


def pack(mesh, mats, solvers, ref, orc, loads=None, extractions=()):
    outs = O.read_vtk_outputs(ref[5])
    t_last, cau, E, vms = outs[-1]
    d = {"X": mesh.X, "conn": mesh.conn,
         # the reference's own VTK output of the final state (6 significant digits)
         "vtk_times": np.array([o[0] for o in outs]), "vtk_cauchy": cau, "vtk_E": E, "vtk_vms": vms,
         "mats": np.array([[m.law, m.young, m.nu, m.rho] for m in mats]),
         "solvers": np.array([[s.t0, s.tf, s.scale_factor, len(s.bcs)] for s in solvers]),
         "bcs": np.array([[b[0], b[1], b[2], b[3]] for s in solvers for b in s.bcs], dtype=np.float64),
         "u": ref[0], "v": ref[1], "a": ref[2], "steps": np.array(orc.steps)}
    if mesh.elem_mat is not None:
        d["elem_mat"] = mesh.elem_mat
    if mesh.act_time is not None:
        d["act_time"] = np.asarray(mesh.act_time, np.float64)
    if any(s.activation for s in solvers):
        d["activation"] = np.array([int(s.activation) for s in solvers])
    if any(s.outputs != 1 for s in solvers):
        d["outputs"] = np.array([s.outputs for s in solvers])
    if any(s.viscosity for s in solvers):
        d["viscosity"] = np.array([s.viscosity or (0, 0.0, 0.0, 0.0, 0.0) for s in solvers], dtype=np.float64)
    if any(s.forces_out for s in solvers):
        import json
        d["forces_out_json"] = np.array(json.dumps([s.forces_out for s in solvers]))
        files = sorted(f for f in os.listdir(ref[5]) if f.startswith("externalForces"))
        d["force_files_json"] = np.array(json.dumps({f: open(os.path.join(ref[5], f)).read() for f in files}))
    if loads is not None:
        import json
        d["loads_json"] = np.array(json.dumps(loads.items))
    if extractions:
        import json
        # the extraction blocks and the reference's own CSV files they produced
        d["extractions_json"] = np.array(json.dumps([list(x) for x in extractions]))
        files = sorted(f for f in os.listdir(ref[5]) if f.endswith(".csv"))
        d["extract_files_json"] = np.array(json.dumps({f: open(os.path.join(ref[5], f)).read() for f in files}))
    return d


def main():
    ref_src = os.environ.get("MSX_REFERENCE_SRC", "/root/reference/src")
    O.build()
    if O.build_reference() is None:
        raise SystemExit("reference sources not found at " + ref_src)
    only = set(sys.argv[1:])   # optional case names: regenerate just those
    for name, case in cases(ref_src).items():
        if only and name not in only:
            continue
        mesh, mats, solvers = case[:3]
        loads = case[3] if len(case) > 3 else None
        extractions = case[4] if len(case) > 4 else ()
        ref = O.run_reference(mesh, mats, solvers, loads=loads, extractions=extractions)
        orc = O.run(mesh, mats, solvers, loads=loads)
        same = all(np.array_equal(x, y) for x, y in zip((orc.u, orc.v, orc.a), ref[:3]))
        print("%-22s steps %5d  oracle==reference bitwise: %s  ref solve %.2fs" % (name, orc.steps, same, ref[3]))
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            **pack(mesh, mats, solvers, ref, orc, loads, extractions))


if __name__ == "__main__":
    main()
