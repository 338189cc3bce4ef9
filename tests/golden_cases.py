"""Loader for the golden fixtures made by tests/golden/make_golden.py."""
import glob
import os

import numpy as np

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    mesh = O.Mesh(d["X"], d["conn"].astype(np.int32),
                  d["elem_mat"].astype(np.int32) if "elem_mat" in d else None)
    mats = [O.Material(int(m[0]), float(m[1]), float(m[2]), float(m[3])) for m in d["mats"]]
    solvers, k = [], 0
    for t0, tf, sf, nb in d["solvers"]:
        nb = int(nb)
        bcs = [(int(b[0]), int(b[1]), float(b[2]), int(b[3])) for b in d["bcs"][k:k + nb]]
        k += nb
        solvers.append(O.Solver(float(t0), float(tf), float(sf), bcs))
    if "act_time" in d:
        mesh.act_time = d["act_time"]
    if "activation" in d:
        for s, k in zip(solvers, d["activation"]):
            s.activation = bool(k)
    if "outputs" in d:
        for s, k in zip(solvers, d["outputs"]):
            s.outputs = int(k)
    if "viscosity" in d:
        for s, v in zip(solvers, d["viscosity"]):
            s.viscosity = (int(v[0]),) + tuple(float(x) for x in v[1:]) if int(v[0]) else None
    if "forces_out_json" in d:
        import json
        for s, fo in zip(solvers, json.loads(str(d["forces_out_json"]))):
            s.forces_out = None if fo is None else (fo[0], [tuple(x) for x in fo[1]])
    return mesh, mats, solvers, (d["u"], d["v"], d["a"]), int(d["steps"])


def load_force_files(name):
    """{file name: the reference's *Forces CSV text} of a case, or {}."""
    import json
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return json.loads(str(d["force_files_json"])) if "force_files_json" in d else {}


def load_loads(name):
    """The Neumann loads of a case (oracle.Loads) or None."""
    import json
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    if "loads_json" not in d:
        return None
    return O.Loads([_item(it) for it in json.loads(str(d["loads_json"]))])


def _item(it):
    if it[0] == "gravity":
        return tuple(it)
    if it[0] == "force":
        return (it[0], it[1], it[2], it[3], [tuple(r) for r in it[4]])
    kind, t0, tf, val, S, elems = it
    return (kind, t0, tf, val if kind.startswith("pressure") else tuple(val), int(S), [int(e) for e in elems])


def load_extractions(name):
    """(extraction blocks, {file name: the reference's CSV text}) of a case, or ((), {})."""
    import json
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    if "extractions_json" not in d:
        return (), {}
    ex = [tuple(x) for x in json.loads(str(d["extractions_json"]))]
    return ex, json.loads(str(d["extract_files_json"]))
