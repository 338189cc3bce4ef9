"""Python access to the oracle (TEST INFRASTRUCTURE ONLY).

Two checkers live here:
  * the C restatement of MuPhiSim v1.1's explicit C3D4 step (msx_oracle.c,
    built into _build/liboracle.so), and
  * the reference MuPhiSim itself, compiled in place from its own sources
    behind our PETSc/MPI shim (_ref/muphisim_ref, see Makefile), driven through
    Abaqus-style decks written by `write_deck`.

Only tests/, the smoke check and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "muphisim_ref")

NEO_HOOKEAN, COMPRESSIBLE_NH, STVK, LINEAR_ELASTIC = 0, 1, 2, 3
LAW_NAMES = {NEO_HOOKEAN: "Neo-Hookean", COMPRESSIBLE_NH: "3D-Compressible-Neo-Hookean",
             STVK: "St-Venant-Kirchhoff"}
BC_RAMP, BC_INST, BC_VEL_RAMP = 0, 1, 2
VISC_NONE, VISC_BULK, VISC_DEV = 0, 1, 2


class _Mat(C.Structure):
    _fields_ = [("law", C.c_int32), ("young", C.c_double), ("nu", C.c_double), ("rho", C.c_double)]


class _Force(C.Structure):
    _fields_ = [("dof", C.c_int64), ("t0", C.c_double), ("tf", C.c_double), ("value", C.c_double)]


class _Load(C.Structure):
    _fields_ = [("kind", C.c_int32), ("face", C.c_int32), ("t0", C.c_double), ("tf", C.c_double),
                ("value", C.c_double * 3), ("elems", C.c_void_p), ("nelems", C.c_int64),
                ("forces", C.c_void_p), ("nforces", C.c_int64)]


LOAD_FORCE, LOAD_GRAVITY, LOAD_TRACTION_INST, LOAD_TRACTION_RAMP, LOAD_PRESSURE_INST, LOAD_PRESSURE_RAMP = range(6)
_SURFACE_KINDS = {"traction_inst": LOAD_TRACTION_INST, "traction_ramp": LOAD_TRACTION_RAMP,
                  "pressure_inst": LOAD_PRESSURE_INST, "pressure_ramp": LOAD_PRESSURE_RAMP}


class _BC(C.Structure):
    _fields_ = [("dof", C.c_int64), ("mode", C.c_int32), ("ramp_steps", C.c_int32), ("value", C.c_double)]


class _Problem(C.Structure):
    _fields_ = [("nn", C.c_int64), ("ne", C.c_int64), ("X", C.c_void_p), ("conn", C.c_void_p),
                ("elem_mat", C.c_void_p), ("mats", C.c_void_p), ("nmat", C.c_int32),
                ("bcs", C.c_void_p), ("nbc", C.c_int64), ("t0", C.c_double), ("tf", C.c_double),
                ("scale_factor", C.c_double), ("max_steps", C.c_int64),
                ("first_step_zero_uK", C.c_int32), ("nthreads", C.c_int32),
                ("forces", C.c_void_p), ("nforces", C.c_int64), ("gravity", C.c_double),
                ("gravity_first", C.c_int32), ("loads", C.c_void_p), ("nloads", C.c_int64),
                ("act_time", C.c_void_p), ("activation", C.c_int32), ("time", C.c_double),
                ("viscosity", C.c_int32), ("visc_c1", C.c_double), ("visc_cl", C.c_double),
                ("visc_h", C.c_double), ("visc_c0", C.c_double), ("F_prev", C.c_void_p)]


class _Result(C.Structure):
    _fields_ = [("steps", C.c_int64), ("t", C.c_double), ("dt_last", C.c_double),
                ("dt_init", C.c_double), ("status", C.c_int32), ("loop_seconds", C.c_double)]


_lib = None


def build() -> str:
    """Compile the C restatement (make lib)."""
    subprocess.run(["make", "-s", "-C", HERE, "lib"], check=True)
    return LIB_PATH


def build_reference() -> str | None:
    """Compile the reference behind the shim when its sources are mounted."""
    src = os.environ.get("MSX_REFERENCE_SRC", "/root/reference/src")
    if not os.path.isdir(src):
        return None
    subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REF_SRC={src}"], check=True)
    return REF_BIN


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.orc_run.argtypes = [C.POINTER(_Problem), C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_int64, C.POINTER(_Result)]
        _lib.orc_external_force.argtypes = [C.POINTER(_Problem), C.c_void_p, C.c_double, C.c_void_p]
        _lib.orc_cube_mesh.argtypes = [C.c_int32, C.c_uint64, C.c_double, C.c_void_p, C.c_void_p]
        _lib.orc_precompute.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_lumped_mass.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_stress.argtypes = [C.POINTER(_Mat), C.c_void_p, C.c_void_p]
        _lib.orc_sound_speed.argtypes = [C.POINTER(_Mat)]
        _lib.orc_sound_speed.restype = C.c_double
        _lib.orc_char_length.argtypes = [C.c_void_p]
        _lib.orc_char_length.restype = C.c_double
        _lib.orc_element_fields.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_element_values.argtypes = [C.POINTER(_Problem), C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                            C.c_int64, C.c_void_p]
        _lib.orc_element_reduce.argtypes = [C.POINTER(_Problem), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                            C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_double)]
        _lib.orc_internal_force.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_int]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


@dataclass
class Material:
    law: int = COMPRESSIBLE_NH
    young: float = 1e6
    nu: float = 0.3
    rho: float = 1000.0


@dataclass
class Loads:
    """Neumann loads of a deck, in deck order: ("force", t0, tf, Ff, [(node, Fx, Fy, Fz), ...])
    for *BOUNDARY, TYPE=FORCE, ("gravity", g) for *GRAVITY,
    ("traction_inst" | "traction_ramp", t0, tf, (Tx, Ty, Tz), S, [elem, ...]) and
    ("pressure_inst" | "pressure_ramp", t0, tf, P, S, [elem, ...]) for *BOUNDARY,
    TYPE=TRACTION/PRESSURE INST/RAMP on face S (1..4) of the listed tets (0-based)."""
    items: list = field(default_factory=list)

    def blocks(self, nn):
        """ctypes blocks in deck order, plus the arrays they point into (keep alive)."""
        keep, out = [], []
        for it in self.items:
            L = _Load()
            if it[0] == "force":
                _, t0, tf, Ff, rows = it
                ents = [(node + k * nn, t0, tf, F[k] * Ff) for node, *F in rows for k in range(3)]
                arr = (_Force * max(1, len(ents)))(*[_Force(*e) for e in ents])
                keep.append(arr)
                L.kind, L.forces, L.nforces = LOAD_FORCE, C.cast(arr, C.c_void_p), len(ents)
            elif it[0] == "gravity":
                L.kind = LOAD_GRAVITY
                L.value[0] = it[1]
            else:
                kind, t0, tf, val, S, elems = it
                L.kind, L.t0, L.tf, L.face = _SURFACE_KINDS[kind], t0, tf, S
                vals = (val,) if kind.startswith("pressure") else tuple(val)
                for i, x in enumerate(vals):
                    L.value[i] = x
                e = np.ascontiguousarray(elems, dtype=np.int32)
                keep.append(e)
                L.elems, L.nelems = e.ctypes.data, len(e)
            out.append(L)
        arr = (_Load * max(1, len(out)))(*out)
        keep.append(arr)
        return arr, len(out), keep

    def force_entries(self, nn):
        out = []
        for it in self.items:
            if it[0] == "force":
                _, t0, tf, Ff, rows = it
                for node, *F in rows:
                    for k in range(3):
                        out.append((node + k * nn, t0, tf, F[k] * Ff))
        return out

    def gravity(self):
        g = [it[1] for it in self.items if it[0] == "gravity"]
        return g[-1] if g else 0.0

    def gravity_first(self):
        kinds = [it[0] for it in self.items]
        return 1 if kinds and kinds[0] == "gravity" else 0


@dataclass
class Mesh:
    X: np.ndarray          # (3, nn) float64
    conn: np.ndarray       # (ne, 4) int32, 0-based
    elem_mat: np.ndarray | None = None
    act_time: np.ndarray | None = None   # (ne,) activation times (*INITINTVARS position 1), or None (0)

    @property
    def nn(self):
        return self.X.shape[1]

    @property
    def ne(self):
        return self.conn.shape[0]


@dataclass
class Solver:
    """One *SOLVER, EXPLICIT block."""
    t0: float
    tf: float
    scale_factor: float
    bcs: list = field(default_factory=list)   # (dof, mode, value, ramp_steps)
    max_steps: int = 0
    forces_out: tuple = None                  # *Forces: (frequency, [(node, direction), ...])
    outputs: int = 1                          # *Outputs: number of VTK outputs of the block
    activation: bool = False                  # *ACTIVATION: element birth at the activation times
    # artificial viscosity (kind, c1, cl, h, c0): kind VISC_BULK (*Bulk viscosity) or VISC_DEV
    # (*Dev viscosity); h and c0 stand for solvers::_elementSize and _c0, 0 in the reference
    viscosity: tuple = None


def cube_mesh(n: int, seed: int = 1234, jitter: float = 0.1) -> Mesh:
    nn, ne = (n + 1) ** 3, 6 * n ** 3
    X = np.zeros((3, nn))
    conn = np.zeros((ne, 4), np.int32)
    rc = lib().orc_cube_mesh(n, seed, jitter, _p(X), _p(conn))
    assert rc == 0
    return Mesh(X, conn)


def cube_bcs(n: int, top_value: float, mode: int = BC_RAMP, ramp_steps: int = 0):
    """Bottom face z=0: all DOFs held at zero; top face z=1: z DOF driven.
    The bottom uses the top's mode when that is INST, since the reference
    reads one displacement *BOUNDARY block per solver."""
    m = n + 1
    nn = m ** 3
    bcs = []
    bottom = BC_INST if mode == BC_INST else BC_RAMP
    for j in range(m):
        for i in range(m):
            node = i + m * j
            for c in range(3):
                bcs.append((node + c * nn, bottom, 0.0, 0))
    for j in range(m):
        for i in range(m):
            node = i + m * j + m * m * n
            bcs.append((node + 2 * nn, mode, top_value, ramp_steps))
    return bcs


def precompute(mesh: Mesh):
    ne = mesh.ne
    dphi = np.zeros((ne, 12))
    wJ = np.zeros(ne)
    Lref = np.zeros(ne)
    X = np.ascontiguousarray(mesh.X)
    conn = np.ascontiguousarray(mesh.conn)
    rc = lib().orc_precompute(mesh.nn, ne, _p(X), _p(conn), _p(dphi), _p(wJ), _p(Lref))
    assert rc == 0
    return dphi, wJ, Lref


def _mats_array(mats):
    arr = (_Mat * len(mats))()
    for k, m in enumerate(mats):
        arr[k] = _Mat(m.law, m.young, m.nu, m.rho)
    return arr


def lumped_mass(mesh: Mesh, mats, wJ):
    out = np.zeros(mesh.nn)
    arr = _mats_array(mats)
    em = None if mesh.elem_mat is None else np.ascontiguousarray(mesh.elem_mat, np.int32)
    lib().orc_lumped_mass(mesh.nn, mesh.ne, _p(np.ascontiguousarray(mesh.conn)), _p(wJ), _p(em),
                          C.cast(arr, C.c_void_p), _p(out))
    return out


def stress(mat: Material, F: np.ndarray) -> np.ndarray:
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(9)
    P = np.zeros(9)
    m = _Mat(mat.law, mat.young, mat.nu, mat.rho)
    lib().orc_stress(C.byref(m), _p(F), _p(P))
    return P.reshape(3, 3)


def sound_speed(mat: Material) -> float:
    m = _Mat(mat.law, mat.young, mat.nu, mat.rho)
    return lib().orc_sound_speed(C.byref(m))


def char_length(x: np.ndarray) -> float:
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(12)
    return lib().orc_char_length(_p(x))


def external_force(mesh: Mesh, mats, loads: Loads, u: np.ndarray, t: float) -> np.ndarray:
    """All Neumann blocks at displacement u and time t (3*nn)."""
    nn = mesh.nn
    larr, nl, _keep = loads.blocks(nn)
    X = np.ascontiguousarray(mesh.X)
    conn = np.ascontiguousarray(mesh.conn)
    em = None if mesh.elem_mat is None else np.ascontiguousarray(mesh.elem_mat, np.int32)
    marr = _mats_array(mats)
    prob = _Problem(nn, mesh.ne, _p(X), _p(conn), _p(em), C.cast(marr, C.c_void_p), len(mats),
                    None, 0, 0.0, 1.0, 0.5, 0, 0, 1, None, 0, 0.0, 0, C.cast(larr, C.c_void_p), nl, None, 0, 0.0)
    f = np.zeros(3 * nn)
    u = np.ascontiguousarray(u, dtype=np.float64)
    lib().orc_external_force(C.byref(prob), _p(u), C.c_double(t), _p(f))
    return f


# Element data extraction (*EXTRACTION, ELEMENT): quantity names and numbers as
# the reference's ExtractData::ElementDataType, operations as ExtractData::Operation
# (src/solvers/dataExtraction.h:23-29).
ELEMENT_QUANTITIES = (["F" + a + b for a in "XYZ" for b in "XYZ"] + ["P" + a + b for a in "XYZ" for b in "XYZ"] +
                      ["SVM", "KVM"] + ["INVAR%d" % k for k in range(1, 7)] +
                      ["DEFO_ENERGY", "EXTERNAL_ENERGY", "KIN_ENERGY", "VOLUME"])
ELEMENT_QUANTITY = {name: k + 1 for k, name in enumerate(ELEMENT_QUANTITIES)}
ELEMENT_OPS = {"Mean": 1, "Min": 2, "Max": 3, "Sum": 4}


def _plain_problem(mesh: Mesh, mats, keep: list, activation=False, t=0.0):
    X = np.ascontiguousarray(mesh.X)
    conn = np.ascontiguousarray(mesh.conn)
    em = None if mesh.elem_mat is None else np.ascontiguousarray(mesh.elem_mat, np.int32)
    marr = _mats_array(mats)
    keep += [X, conn, em, marr]
    act = None if mesh.act_time is None else np.ascontiguousarray(mesh.act_time, np.float64)
    keep.append(act)
    return _Problem(mesh.nn, mesh.ne, _p(X), _p(conn), _p(em), C.cast(marr, C.c_void_p), len(mats),
                    None, 0, 0.0, 1.0, 0.5, 0, 0, 1, None, 0, 0.0, 0, None, 0,
                    _p(act), 1 if activation else 0, float(t))


def active_elements(mesh: Mesh, mats, activation: bool, t: float) -> np.ndarray:
    """Elements active at time t under the *ACTIVATION option (the laws with an
    activation time: St-Venant-Kirchhoff and linear elastic)."""
    if not activation or mesh.act_time is None:
        return np.ones(mesh.ne, bool)
    laws = np.array([mats[k].law for k in (mesh.elem_mat if mesh.elem_mat is not None else np.zeros(mesh.ne, int))])
    return ~np.isin(laws, [STVK, LINEAR_ELASTIC]) | (np.asarray(mesh.act_time) <= t)


def element_values(mesh: Mesh, mats, quantity: str, u, v, elems=None, activation=False, t=0.0) -> np.ndarray:
    """Per-element value of an element-extraction quantity at the state u, v."""
    keep = []
    prob = _plain_problem(mesh, mats, keep, activation, t)
    el = None if elems is None else np.ascontiguousarray(elems, np.int32)
    out = np.zeros(mesh.ne if el is None else len(el))
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    lib().orc_element_values(C.byref(prob), _p(u), _p(v), ELEMENT_QUANTITY[quantity], _p(el),
                             0 if el is None else len(el), _p(out))
    return out


def element_reduce(mesh: Mesh, mats, quantity: str, op: str, u, v, elems=None, fext=None, activation=False,
                   t=0.0) -> float:
    """The value one *EXTRACTION, ELEMENT row holds at the state u, v (fext: the
    external force of that step, for EXTERNAL_ENERGY)."""
    keep = []
    prob = _plain_problem(mesh, mats, keep, activation, t)
    el = None if elems is None else np.ascontiguousarray(elems, np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    f = np.zeros(3 * mesh.nn) if fext is None else np.ascontiguousarray(fext, dtype=np.float64)
    out = C.c_double(0.0)
    lib().orc_element_reduce(C.byref(prob), _p(u), _p(v), _p(f), ELEMENT_QUANTITY[quantity], ELEMENT_OPS[op],
                             _p(el), 0 if el is None else len(el), C.byref(out))
    return out.value


def internal_force(mesh: Mesh, mats, u: np.ndarray, nthreads: int = 1):
    dphi, wJ, _ = precompute(mesh)
    nn, ne = mesh.nn, mesh.ne
    f = np.zeros(3 * nn)
    F = np.zeros((ne, 9))
    P = np.zeros((ne, 9))
    arr = _mats_array(mats)
    em = None if mesh.elem_mat is None else np.ascontiguousarray(mesh.elem_mat, np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64)
    lib().orc_internal_force(nn, ne, _p(np.ascontiguousarray(mesh.conn)), _p(dphi), _p(wJ), _p(em),
                             C.cast(arr, C.c_void_p), _p(u), _p(f), _p(F), _p(P), nthreads)
    return f, F, P


def element_fields(mesh: Mesh, mats, u: np.ndarray):
    """Cauchy (ne,3,3), Green-Lagrange (ne,3,3), von Mises (ne,) of displacement u."""
    dphi, _, _ = precompute(mesh)
    ne = mesh.ne
    c, g, v = np.zeros(9 * ne), np.zeros(9 * ne), np.zeros(ne)
    arr = _mats_array(mats)
    em = None if mesh.elem_mat is None else np.ascontiguousarray(mesh.elem_mat, np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64)
    lib().orc_element_fields(mesh.nn, ne, _p(np.ascontiguousarray(mesh.conn)), _p(dphi), _p(em),
                             C.cast(arr, C.c_void_p), _p(u), _p(c), _p(g), _p(v))
    return c.reshape(-1, 3, 3), g.reshape(-1, 3, 3), v


def read_vtk_outputs(outdir: str):
    """The reference's VTK outputs: list of (time, Cauchy (ne,9), E (ne,9), VMS (ne,))
    read from allOutputs_0.vtk.series and MuPhiSimOutputs_0_.<k>.vtk (6 digits)."""
    import json
    series = json.load(open(os.path.join(outdir, "allOutputs_0.vtk.series")))
    out = []
    for item in series["files"]:
        toks = open(os.path.join(outdir, item["name"])).read().split()
        ne = int(toks[toks.index("CELL_DATA") + 1])

        def block(kind, tag, width, skip):
            i = next(k for k in range(len(toks) - 1) if toks[k] == kind and toks[k + 1] == tag)
            start = i + skip
            return np.array(toks[start:start + ne * width], dtype=np.float64).reshape(ne, width)
        cau = block("TENSORS", "Cauchy", 9, 3)
        E = block("TENSORS", "E", 9, 3)
        vms = block("SCALARS", "VMS", 1, 5)[:, 0]
        out.append((float(item["time"]), cau, E, vms))
    return out


@dataclass
class RunResult:
    u: np.ndarray
    v: np.ndarray
    a: np.ndarray
    steps: int
    t: float
    dt_init: float
    dt_last: float
    status: int
    dt_hist: np.ndarray
    loop_seconds: float = 0.0


def run(mesh: Mesh, mats, solvers, nthreads: int = 1, state=None, max_hist: int = 0, loads: Loads = None) -> RunResult:
    """Run a chain of explicit solver blocks as the reference's main does."""
    nn = mesh.nn
    if state is None:
        u, v, a = np.zeros(3 * nn), np.zeros(3 * nn), np.zeros(3 * nn)
    else:
        u, v, a = (np.array(s, dtype=np.float64, copy=True) for s in state)
    X = np.ascontiguousarray(mesh.X)
    conn = np.ascontiguousarray(mesh.conn)
    em = None if mesh.elem_mat is None else np.ascontiguousarray(mesh.elem_mat, np.int32)
    marr = _mats_array(mats)
    total = 0
    loop_s = 0.0
    res = _Result()
    hist_all = []
    fl = loads.force_entries(nn) if loads else []
    farr = (_Force * max(1, len(fl)))()
    for i, f in enumerate(fl):
        farr[i] = _Force(*f)
    larr, nl, _keep = loads.blocks(nn) if loads else (None, 0, None)
    act = None if mesh.act_time is None else np.ascontiguousarray(mesh.act_time, np.float64)
    F_prev = None
    for k, s in enumerate(solvers):
        visc = s.viscosity if s.viscosity and s.viscosity[0] in (VISC_BULK, VISC_DEV) else None
        if visc is None:
            F_prev = None
        elif F_prev is None:
            # the Gauss points' previous F: that of the current state (F = I from rest)
            F_prev, f_scratch = np.zeros(9 * mesh.ne), np.zeros(3 * nn)
            dphi, wJ, _ = precompute(mesh)
            lib().orc_internal_force(nn, mesh.ne, _p(conn), _p(dphi), _p(wJ), _p(em), C.cast(marr, C.c_void_p),
                                     _p(u), _p(f_scratch), _p(F_prev), None, 1)
        barr = (_BC * max(1, len(s.bcs)))()
        for i, (dof, mode, value, ramp) in enumerate(s.bcs):
            barr[i] = _BC(dof, mode, ramp, value)
        prob = _Problem(nn, mesh.ne, _p(X), _p(conn), _p(em), C.cast(marr, C.c_void_p), len(mats),
                        C.cast(barr, C.c_void_p), len(s.bcs), s.t0, s.tf, s.scale_factor, s.max_steps,
                        0, nthreads, C.cast(farr, C.c_void_p), len(fl),
                        loads.gravity() if loads else 0.0, loads.gravity_first() if loads else 0,
                        C.cast(larr, C.c_void_p) if nl else None, nl,
                        _p(act), 1 if s.activation else 0, 0.0,
                        visc[0] if visc else 0, *(visc[1:5] if visc else (0.0, 0.0, 0.0, 0.0)), _p(F_prev))
        hist = np.zeros(max(1, max_hist))
        rc = lib().orc_run(C.byref(prob), _p(u), _p(v), _p(a), _p(hist), max_hist, C.byref(res))
        total += res.steps
        loop_s += res.loop_seconds
        hist_all.append(hist[: min(res.steps, max_hist)])
        if rc != 0:
            break
    return RunResult(u, v, a, total, res.t, res.dt_init, res.dt_last, res.status,
                     np.concatenate(hist_all) if hist_all else np.zeros(0), loop_s)


# ---------------------------------------------------------------- the reference
def write_deck(path: str, mesh: Mesh, mats, solvers, mat_elems=None, loads: Loads = None, extractions=()):
    """Abaqus-style deck in the keyword subset the reference parses
    (src/IO/inputFile.cpp: nodes :20-108, C3D4 elements :118-323, materials
    :838-1029, solver blocks :2253-2831, displacement BCs :2960-3218)."""
    X, conn = mesh.X, mesh.conn
    lines = ["*Node"]
    for i in range(mesh.nn):
        lines.append("%d, %.17g, %.17g, %.17g" % (i + 1, X[0, i], X[1, i], X[2, i]))
    lines.append("*Element, type=C3D4")
    for e in range(mesh.ne):
        c = conn[e] + 1
        lines.append("%d, %d, %d, %d, %d" % (e + 1, c[0], c[1], c[2], c[3]))
    lines += ["*FEM Nodes", "All", "*FEM Elements", "All"]
    nn = mesh.nn
    # Neumann loads (src/IO/inputFile.cpp:4705-4735 and 2841-2945), in deck order
    for it in (loads.items if loads else []):
        if it[0] == "force":
            _, t0, tf, Ff, rows = it
            lines += ["*BOUNDARY, TYPE=FORCE", "%.17g, %.17g, %.17g" % (t0, tf, Ff)]
            lines += ["%d, %.17g, %.17g, %.17g" % (node + 1, F0, F1, F2) for node, F0, F1, F2 in rows]
        elif it[0] == "gravity":
            lines += ["*GRAVITY", "%.17g" % it[1]]
        else:
            kind, t0, tf, val, S, elems = it
            name = kind.split("_")[0].upper() + " " + kind.split("_")[1].upper()
            vals = (val,) if kind.startswith("pressure") else tuple(val)
            lines += ["*BOUNDARY, TYPE=" + name,
                      ", ".join("%.17g" % x for x in (t0, tf) + vals) + ", %d" % S]
            lines += ["%d" % (int(e) + 1) for e in elems]
    # node data extraction (src/IO/inputFile.cpp:4950-5026): the header is sliced at the
    # commas without trimming, so it is written without spaces
    # element data extraction (:5028-5111): "name,type,operation", then "All" or
    # one element per line
    for ex in extractions:
        if ex[0] == "element":
            _, name, dtype, op, elems = ex
            lines += ["*EXTRACTION, ELEMENT", "%s,%s,%s" % (name, dtype, op)]
            lines += ["All"] if elems is None else ["%d" % (int(e) + 1) for e in elems]
            continue
        name, dtype, op, comp, nodes = ex
        lines += ["*EXTRACTION, NODE", "%s,%s,%s,%d" % (name, dtype, op, comp)]
        lines += ["%d" % (int(nd) + 1) for nd in nodes]
    visc_seen = False
    for s in solvers:
        if any(b[1] == BC_VEL_RAMP for b in s.bcs):
            raise ValueError("the reference has no velocity-ramp boundary condition")
        modes = {b[1] for b in s.bcs}
        if len(modes) > 1:
            raise ValueError("one *BOUNDARY block per solver: a single mode only")
        mode = modes.pop() if modes else BC_RAMP
        lines += ["*SOLVER, EXPLICIT"] + (["*ACTIVATION"] if s.activation else [])
        if s.viscosity:
            # the reader has no element size or c0 for these (solvers.h:53-54)
            kind, c1, cl, h, c0 = s.viscosity
            if h != 0 or c0 != 0:
                raise ValueError("the reference has no element size or c0 for its artificial viscosity")
            lines += ["*Bulk viscosity" if kind == VISC_BULK else "*Dev viscosity", "%.17g, %.17g" % (c1, cl)]
        elif visc_seen:
            raise ValueError("the reference keeps artificial viscosity on in later solver blocks")
        visc_seen = visc_seen or bool(s.viscosity)
        lines += ["*Scale Factor", "%.17g" % s.scale_factor,
                  "*Outputs", "%d" % s.outputs, "*Time", "%.17g, %.17g" % (s.t0, s.tf),
                  "*BOUNDARY, TYPE=DISPLACEMENT " + ("INST" if mode == BC_INST else "RAMP")]
        for dof, _, value, _ in s.bcs:
            lines.append("%d,%d,%.17g" % (dof % nn + 1, dof // nn, value))
        if s.forces_out:
            # *Forces (src/IO/inputFile.cpp:4830-4886): the reader slices each line
            # between its first two commas, so the direction is followed by one
            freq, pairs = s.forces_out
            lines += ["*Forces", "%.17g" % freq] + ["%d,%d," % (int(nd) + 1, int(c)) for nd, c in pairs]
        lines.append("*END SOLVER")
    if mat_elems is None:
        mat_elems = [None] * len(mats)
    for k, m in enumerate(mats):
        lines += ["*MATERIAL, name=Region%d" % (k + 1), "*Density", "%.17g" % m.rho,
                  ("*Linear-Elastic" if m.law == LINEAR_ELASTIC else "*HyperElastic, " + LAW_NAMES[m.law]),
                  "%.17g, %.17g" % (m.young, m.nu)]
        if mat_elems[k] is None:
            lines += ["*List of Elements", "All"]
        else:
            # the reader takes one element per *List of Elements keyword
            # (src/IO/inputFile.cpp:2010-2053)
            for e in mat_elems[k]:
                lines += ["*List of Elements", str(int(e) + 1)]
        # activation times as the first internal variable (src/IO/inputFile.cpp:2055-2111),
        # after the element list the reader checks them against
        if mesh.act_time is not None:
            own = range(mesh.ne) if mat_elems[k] is None else mat_elems[k]
            rows = ["%d, 1, %.17g" % (int(e) + 1, mesh.act_time[int(e)]) for e in own if mesh.act_time[int(e)] != 0.0]
            if rows:
                lines += ["*INITINTVARS"] + rows
    lines.append("*END")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def run_reference(mesh: Mesh, mats, solvers, workdir: str | None = None, timeout: float = 3600,
                  loads: Loads = None, extractions=()):
    """Run the shim-built reference on a deck; returns (u, v, a, solve_wall_s)."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError("reference binary not built: make -C oracle ref")
    own = workdir is None
    wd = tempfile.mkdtemp(prefix="msxref_") if own else workdir
    os.makedirs(os.path.join(wd, "out"), exist_ok=True)
    mat_elems = None
    if mesh.elem_mat is not None:
        mat_elems = [np.nonzero(mesh.elem_mat == k)[0] for k in range(len(mats))]
    write_deck(os.path.join(wd, "deck.inp"), mesh, mats, solvers, mat_elems, loads, extractions)
    dump, timing = os.path.join(wd, "final.bin"), os.path.join(wd, "timing.txt")
    r = subprocess.run([REF_BIN, "-input", "deck.inp", "-inputDir", ".", "-outputDir", "out",
                        "-dump", dump, "-timing", timing], cwd=wd, capture_output=True, text=True,
                       timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("reference failed (%d): %s" % (r.returncode, (r.stderr or r.stdout)[-2000:]))
    data = np.fromfile(dump, dtype=np.float64)
    n = 3 * mesh.nn
    wall = float(open(timing).read())
    return data[:n], data[n:2 * n], data[2 * n:3 * n], wall, r.stdout, os.path.join(wd, "out")
