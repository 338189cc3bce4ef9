"""ctypes binding of libmsx (include/msx.h) for Python callers, tests and bench.

The product is the C ABI; this module only marshals arrays into it.  It loads
the in-tree v.1.1_gb300/_build/libmsx.so and raises if that library is missing
or if no GB300 is present: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmsx.so")

OK = 0
ERR = {0: "OK", 1: "ARG", 2: "CUDA", 3: "NEG_JACOBIAN", 4: "NAN", 5: "OOM", 6: "STATE",
       7: "NO_DEVICE", 8: "TIMEOUT", 9: "BUSY"}
NEO_HOOKEAN, COMPRESSIBLE_NH, STVK, LINEAR_ELASTIC = 0, 1, 2, 3
VISC_NONE, VISC_BULK, VISC_DEV = 0, 1, 2
BC_RAMP, BC_INST, BC_VEL_RAMP, BC_RAMP_RATE = 0, 1, 2, 3
FP64, FP64_EXACT, MIXED, DOUBLE_WORD = 0, 1, 2, 3


class MsxError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("msx error %s (%d): %s" % (ERR.get(status, "?"), status, msg))
        self.status = status


class Mesh_(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("num_elems", C.c_int64), ("X", C.c_void_p),
                ("conn", C.c_void_p), ("elem_material", C.c_void_p)]


class Material_(C.Structure):
    _fields_ = [("law", C.c_int32), ("reserved", C.c_int32), ("young", C.c_double),
                ("nu", C.c_double), ("rho", C.c_double)]


class BC_(C.Structure):
    _fields_ = [("dof", C.c_int64), ("mode", C.c_int32), ("ramp_steps", C.c_int32), ("value", C.c_double)]


FIELD_DISPLACEMENT, FIELD_EXTERNAL_FORCE, FIELD_INTERNAL_FORCE = 0, 1, 2
# element data extraction: quantity names numbered as the reference's
# ExtractData::ElementDataType, operations as ExtractData::Operation
ELEMENT_QUANTITIES = (["F" + a + b for a in "XYZ" for b in "XYZ"] + ["P" + a + b for a in "XYZ" for b in "XYZ"] +
                      ["SVM", "KVM"] + ["INVAR%d" % k for k in range(1, 7)] +
                      ["DEFO_ENERGY", "EXTERNAL_ENERGY", "KIN_ENERGY", "VOLUME"])
ELEM = {name: k + 1 for k, name in enumerate(ELEMENT_QUANTITIES)}
OP_MEAN, OP_MIN, OP_MAX, OP_SUM = 1, 2, 3, 4
OPS = {"Mean": OP_MEAN, "Min": OP_MIN, "Max": OP_MAX, "Sum": OP_SUM}
LOAD_FORCE, LOAD_GRAVITY, LOAD_TRACTION_INST, LOAD_TRACTION_RAMP, LOAD_PRESSURE_INST, LOAD_PRESSURE_RAMP = range(6)


class LoadBlock_(C.Structure):
    _fields_ = [("kind", C.c_int32), ("face", C.c_int32), ("t0", C.c_double), ("tf", C.c_double),
                ("value", C.c_double * 3), ("elems", C.c_void_p), ("num_elems", C.c_int64),
                ("forces", C.c_void_p), ("num_forces", C.c_int64)]


class Force_(C.Structure):
    _fields_ = [("dof", C.c_int64), ("t0", C.c_double), ("tf", C.c_double), ("value", C.c_double)]


class Opts_(C.Structure):
    _fields_ = [("t0", C.c_double), ("tf", C.c_double), ("scale_factor", C.c_double),
                ("max_steps", C.c_int64), ("precision", C.c_int32), ("steps_per_graph", C.c_int32)]


class Report_(C.Structure):
    _fields_ = [("steps", C.c_int64), ("total_steps", C.c_int64), ("t", C.c_double), ("dt", C.c_double),
                ("dt_init", C.c_double), ("status", C.c_int32), ("reserved", C.c_int32),
                ("device_ms", C.c_double), ("kernel_launches", C.c_int64)]


class Profile_(C.Structure):
    _fields_ = [("element_ms", C.c_double), ("node_ms", C.c_double), ("element_launches", C.c_int64),
                ("node_launches", C.c_int64), ("element_alg_bytes", C.c_double), ("node_alg_bytes", C.c_double)]


class PoolOpts_(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_slots", C.c_int32), ("precision", C.c_int32),
                ("elems_per_block", C.c_int32), ("steps_per_launch", C.c_int32), ("tune_cache", C.c_char_p)]


class PoolStats_(C.Structure):
    _fields_ = [("active", C.c_int32), ("finished_unfetched", C.c_int32), ("threads", C.c_int32),
                ("tile_elems", C.c_int32), ("ctas_per_sm", C.c_int32), ("steps_per_launch", C.c_int32),
                ("element_steps", C.c_int64), ("used_bytes", C.c_int64), ("budget_bytes", C.c_int64)]


class PoolResult_(C.Structure):
    _fields_ = [("ticket", C.c_int64), ("status", C.c_int32), ("reserved", C.c_int32), ("steps", C.c_int64),
                ("t", C.c_double), ("submit_to_done_ms", C.c_double)]


# every entry point declared in include/msx.h
SYMBOLS = ["msx_create", "msx_run", "msx_get_state", "msx_set_state", "msx_next_solver", "msx_destroy",
           "msx_last_error", "msx_internal_force", "msx_get_element_data", "msx_profile", "msx_mesh_cube",
           "msx_stream", "msx_set_device", "msx_pool_create", "msx_pool_submit", "msx_pool_step", "msx_pool_serve",
           "msx_pool_poll", "msx_pool_fetch", "msx_pool_wait", "msx_pool_destroy", "msx_pool_stats_get",
           "msx_internal_force_noalloc", "msx_initial_dt", "msx_element_fields", "msx_set_loads",
           "msx_set_load_blocks", "msx_node_values", "msx_element_values", "msx_element_reduce",
           "msx_set_activation", "msx_pool_inject_alloc_failures", "msx_deck_read_loads", "msx_deck_loads_blocks",
           "msx_deck_loads_free", "msx_set_viscosity"]

_lib = None


def load(path: str = LIB_PATH):
    """Load libmsx.so; raise if it is absent (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError("libmsx.so not built: run python v.1.1_gb300/build.py (%s)" % path)
    L = C.CDLL(path)
    vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int32
    sig = {
        "msx_create": [C.POINTER(Mesh_), vp, i32, vp, i64, C.POINTER(Opts_), C.POINTER(vp)],
        "msx_run": [vp, i64, C.POINTER(Report_)],
        "msx_get_state": [vp, vp, vp, vp],
        "msx_set_state": [vp, vp, vp, vp],
        "msx_next_solver": [vp, vp, i64, C.POINTER(Opts_)],
        "msx_destroy": [vp],
        "msx_internal_force": [vp, vp, vp],
        "msx_get_element_data": [vp, vp, vp, vp, vp],
        "msx_profile": [vp, i64, C.POINTER(Profile_)],
        "msx_mesh_cube": [i32, C.c_uint64, C.c_double, vp, vp],
        "msx_stream": [vp],
        "msx_set_device": [i32],
        "msx_initial_dt": [vp, C.POINTER(C.c_double)],
        "msx_element_fields": [vp, vp, vp, vp],
        "msx_set_loads": [vp, vp, i64, C.c_double, i32],
        "msx_set_load_blocks": [vp, vp, i64],
        "msx_node_values": [vp, i32, i32, vp, i64, vp],
        "msx_element_values": [vp, i32, vp, i64, vp],
        "msx_set_activation": [vp, vp, i32],
        "msx_element_reduce": [vp, i32, i32, vp, i64, vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.msx_last_error.restype = C.c_char_p
    L.msx_stream.restype = vp
    _lib = L
    return L


def set_device(device: int):
    _check(load().msx_set_device(int(device)))


def _check(st):
    if st != OK:
        raise MsxError(st, load().msx_last_error().decode())


def _p(a):
    return None if a is None else a.ctypes.data


def mesh_cube(n: int, seed: int = 1234, jitter: float = 0.1):
    """Seeded cube mesh from the library: X (3, nn), conn (ne, 4)."""
    nn, ne = (n + 1) ** 3, 6 * n ** 3
    X = np.zeros((3, nn))
    conn = np.zeros((ne, 4), np.int32)
    _check(load().msx_mesh_cube(n, seed, jitter, _p(X), _p(conn)))
    return X, conn


def cube_bcs(n: int, top_value: float, mode: int = BC_RAMP, ramp_steps: int = 0):
    """Bottom face held at zero, top face z DOF driven (same recipe as the fixtures)."""
    m = n + 1
    nn = m ** 3
    bottom = BC_INST if mode == BC_INST else BC_RAMP
    ij = np.arange(m * m)
    dof_b = (ij[:, None] + nn * np.arange(3)[None, :]).ravel()
    dof_t = ij + m * m * n + 2 * nn
    return ([(d, bottom, 0.0, 0) for d in dof_b.tolist()] +
            [(d, mode, top_value, ramp_steps) for d in dof_t.tolist()])


_BC_DTYPE = np.dtype({"names": [f for f, _ in BC_._fields_], "formats": ["<i8", "<i4", "<i4", "<f8"],
                      "offsets": [getattr(BC_, f).offset for f, _ in BC_._fields_], "itemsize": C.sizeof(BC_)})


def bc_array(bcs):
    """(dof, mode, value, ramp_steps) rows as an msx_bc array.  Solver,
    next_solver and Pool.submit take such an array in place of the rows."""
    if isinstance(bcs, np.ndarray) and bcs.dtype == _BC_DTYPE:
        return bcs
    out = np.zeros(len(bcs), _BC_DTYPE)
    if len(bcs):
        rows = np.array(bcs, dtype=[("dof", "<i8"), ("mode", "<i4"), ("value", "<f8"), ("ramp", "<i4")])
        out["dof"][:] = rows["dof"]
        out["mode"][:] = rows["mode"]
        out["ramp_steps"][:] = rows["ramp"]
        out["value"][:] = rows["value"]
    return out


def _opts(t0, tf, sf, max_steps, precision, spg):
    return Opts_(t0, tf, sf, max_steps, precision, spg)


@dataclass
class Report:
    steps: int
    total_steps: int
    t: float
    dt: float
    dt_init: float
    status: int
    device_ms: float
    kernel_launches: int


class Solver:
    """One device-resident explicit solve (mesh + materials + solver blocks)."""

    def __init__(self, X, conn, materials, bcs, t0, tf, scale_factor, max_steps=0,
                 precision=FP64, elem_material=None, steps_per_graph=0):
        L = load()
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.int32)
        self.nn, self.ne = self.X.shape[1], self.conn.shape[0]
        em = None if elem_material is None else np.ascontiguousarray(elem_material, np.int32)
        mesh = Mesh_(self.nn, self.ne, _p(self.X), _p(self.conn), _p(em))
        mats = (Material_ * len(materials))()
        for k, m in enumerate(materials):
            law, E, nu, rho = m
            mats[k] = Material_(int(law), 0, float(E), float(nu), float(rho))
        barr = bc_array(bcs)
        opts = _opts(t0, tf, scale_factor, max_steps, precision, steps_per_graph)
        h = C.c_void_p()
        _check(L.msx_create(C.byref(mesh), C.cast(mats, C.c_void_p), len(materials),
                            _p(barr), len(barr), C.byref(opts), C.byref(h)))
        self.h = h

    def run(self, max_steps: int = 0) -> Report:
        r = Report_()
        st = load().msx_run(self.h, max_steps, C.byref(r))
        rep = Report(r.steps, r.total_steps, r.t, r.dt, r.dt_init, r.status, r.device_ms, r.kernel_launches)
        self.last_report = rep
        _check(st)
        return rep

    def next_solver(self, bcs, t0, tf, scale_factor, max_steps=0, precision=FP64, steps_per_graph=0):
        barr = bc_array(bcs)
        opts = _opts(t0, tf, scale_factor, max_steps, precision, steps_per_graph)
        _check(load().msx_next_solver(self.h, _p(barr), len(barr), C.byref(opts)))

    def state(self, out=None):
        """u, v, a of the last step, into `out` (three contiguous float64 arrays
        of 3*nn, e.g. in page-locked memory) when given."""
        if out is None:
            out = tuple(np.zeros(3 * self.nn) for _ in range(3))
        for x in out:
            if x.dtype != np.float64 or x.size != 3 * self.nn or not x.flags.c_contiguous:
                raise ValueError("state buffers must be contiguous float64 arrays of 3*nn")
        u, v, a = out
        _check(load().msx_get_state(self.h, _p(u), _p(v), _p(a)))
        return u, v, a

    def set_state(self, u=None, v=None, a=None):
        conv = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, a)]
        _check(load().msx_set_state(self.h, *[_p(x) for x in conv]))

    def internal_force(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        f = np.zeros(3 * self.nn)
        _check(load().msx_internal_force(self.h, _p(u), _p(f)))
        return f

    def set_loads(self, forces=(), gravity=0.0, gravity_first=False):
        """forces: (dof, t0, tf, value) per nodal-force DOF in deck order."""
        arr = (Force_ * max(1, len(forces)))()
        for i, f in enumerate(forces):
            arr[i] = Force_(*f)
        _check(load().msx_set_loads(self.h, C.cast(arr, C.c_void_p), len(forces), float(gravity),
                                    1 if gravity_first else 0))

    def set_load_blocks(self, items):
        """All Neumann loads in deck order, items as
        ("force", t0, tf, Ff, [(node, Fx, Fy, Fz), ...]), ("gravity", g),
        ("traction_inst" | "traction_ramp", t0, tf, (Tx, Ty, Tz), S, [tet, ...]),
        ("pressure_inst" | "pressure_ramp", t0, tf, P, S, [tet, ...]) (S = face 1..4)."""
        kinds = {"force": LOAD_FORCE, "gravity": LOAD_GRAVITY, "traction_inst": LOAD_TRACTION_INST,
                 "traction_ramp": LOAD_TRACTION_RAMP, "pressure_inst": LOAD_PRESSURE_INST,
                 "pressure_ramp": LOAD_PRESSURE_RAMP}
        keep, blocks = [], []
        for it in items:
            B = LoadBlock_()
            B.kind = kinds[it[0]]
            if it[0] == "force":
                _, t0, tf, Ff, rows = it
                ents = [(int(node) + k * self.nn, t0, tf, F[k] * Ff) for node, *F in rows for k in range(3)]
                arr = (Force_ * max(1, len(ents)))(*[Force_(*e) for e in ents])
                keep.append(arr)
                B.forces, B.num_forces = C.cast(arr, C.c_void_p), len(ents)
            elif it[0] == "gravity":
                B.value[0] = it[1]
            else:
                _, t0, tf, val, S, elems = it
                B.t0, B.tf, B.face = t0, tf, S
                vals = (val,) if it[0].startswith("pressure") else tuple(val)
                for i, x in enumerate(vals):
                    B.value[i] = x
                e = np.ascontiguousarray(elems, dtype=np.int32)
                keep.append(e)
                B.elems, B.num_elems = e.ctypes.data, len(e)
            blocks.append(B)
        arr = (LoadBlock_ * max(1, len(blocks)))(*blocks)
        _check(load().msx_set_load_blocks(self.h, C.cast(arr, C.c_void_p), len(blocks)))

    def set_viscosity(self, kind, c1=0.06, cl=1.2, element_size=0.0, c0=0.0):
        """Artificial viscosity (VISC_NONE, VISC_BULK, VISC_DEV); element_size and c0 are
        the reference's never-set solvers::_elementSize and _c0 (0 there)."""
        load().msx_set_viscosity.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double,
                                             C.c_double]
        _check(load().msx_set_viscosity(self.h, int(kind), float(c1), float(cl), float(element_size), float(c0)))

    def node_values(self, field, comp, nodes):
        """Component comp of FIELD_DISPLACEMENT / FIELD_EXTERNAL_FORCE /
        FIELD_INTERNAL_FORCE at the listed nodes for the current state."""
        n = np.ascontiguousarray(nodes, dtype=np.int32)
        out = np.zeros(len(n))
        _check(load().msx_node_values(self.h, int(field), int(comp), _p(n), len(n), _p(out)))
        return out

    def set_activation(self, activation_time=None, enabled=True):
        """Element birth (*ACTIVATION): per-element activation times (None keeps the
        current ones) and whether the current and later blocks use them."""
        t = None if activation_time is None else np.ascontiguousarray(activation_time, dtype=np.float64)
        if t is not None and t.shape != (self.ne,):
            raise ValueError("one activation time per element")
        _check(load().msx_set_activation(self.h, _p(t), 1 if enabled else 0))

    def element_values(self, quantity, elems=None):
        """Per-element value of an element-extraction quantity (a name of
        ELEMENT_QUANTITIES or its number) for the listed elements (None: all)."""
        q = ELEM[quantity] if isinstance(quantity, str) else int(quantity)
        e = None if elems is None else np.ascontiguousarray(elems, dtype=np.int32)
        out = np.zeros(self.ne if e is None else len(e))
        _check(load().msx_element_values(self.h, q, _p(e), 0 if e is None else len(e), _p(out)))
        return out

    def element_reduce(self, quantity, op, elems=None):
        """The value one *EXTRACTION, ELEMENT row holds: quantity as for
        element_values, op "Mean", "Min", "Max", "Sum" or OP_*."""
        q = ELEM[quantity] if isinstance(quantity, str) else int(quantity)
        o = OPS[op] if isinstance(op, str) else int(op)
        e = None if elems is None else np.ascontiguousarray(elems, dtype=np.int32)
        out = np.zeros(1)
        _check(load().msx_element_reduce(self.h, q, o, _p(e), 0 if e is None else len(e), _p(out)))
        return float(out[0])

    def initial_dt(self):
        d = C.c_double()
        _check(load().msx_initial_dt(self.h, C.byref(d)))
        return d.value

    def element_fields(self):
        """Cauchy (ne, 3, 3), Green-Lagrange (ne, 3, 3), von Mises (ne,) of the current state."""
        c, g, v = np.zeros(9 * self.ne), np.zeros(9 * self.ne), np.zeros(self.ne)
        _check(load().msx_element_fields(self.h, _p(c), _p(g), _p(v)))
        return c.reshape(-1, 3, 3), g.reshape(-1, 3, 3), v

    def von_mises(self):
        """Von Mises stress (ne,) of the current state (the other fields are not copied)."""
        v = np.zeros(self.ne)
        _check(load().msx_element_fields(self.h, None, None, _p(v)))
        return v

    def element_data(self):
        G, wJ, L, m = np.zeros(9 * self.ne), np.zeros(self.ne), np.zeros(self.ne), np.zeros(self.nn)
        _check(load().msx_get_element_data(self.h, _p(G), _p(wJ), _p(L), _p(m)))
        return G.reshape(9, self.ne), wJ, L, m

    def profile(self, steps: int):
        r = Profile_()
        _check(load().msx_profile(self.h, steps, C.byref(r)))
        return r

    def close(self):
        if getattr(self, "h", None):
            load().msx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pool:
    """Batched / serving pool: independent solves resident on the device and
    stepped together (include/msx.h msx_pool_*)."""

    def __init__(self, max_slots=256, precision=MIXED, hbm_budget_bytes=0, elems_per_block=0,
                 steps_per_launch=0, tune_cache=None):
        L = load()
        for name, args in (("msx_pool_create", [C.POINTER(PoolOpts_), C.POINTER(C.c_void_p)]),
                           ("msx_pool_submit", [C.c_void_p, C.POINTER(Mesh_), C.POINTER(Material_), C.c_void_p,
                                                C.c_int64, C.POINTER(Opts_), C.POINTER(C.c_int64)]),
                           ("msx_pool_step", [C.c_void_p, C.c_int64]),
                           ("msx_pool_serve", [C.c_void_p, C.c_int32]),
                           ("msx_pool_poll", [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
                           ("msx_pool_fetch", [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
                           ("msx_pool_wait", [C.c_void_p, C.c_int64, C.c_void_p]),
                           ("msx_pool_destroy", [C.c_void_p]),
                           ("msx_pool_stats_get", [C.c_void_p, C.POINTER(PoolStats_)]),
                           ("msx_pool_inject_alloc_failures", [C.c_void_p, C.c_int32])):
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        self._cache = tune_cache.encode() if tune_cache else None
        o = PoolOpts_(hbm_budget_bytes, max_slots, precision, elems_per_block, steps_per_launch, self._cache)
        h = C.c_void_p()
        _check(L.msx_pool_create(C.byref(o), C.byref(h)))
        self.h = h
        self.sizes = {}
        self._keep = {}

    def submit(self, X, conn, material, bcs, max_steps, t0=0.0, tf=1e30, scale_factor=0.5):
        """Admit one solve; returns its ticket or None when the pool is full."""
        X = np.ascontiguousarray(X, dtype=np.float64)
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        mesh = Mesh_(X.shape[1], conn.shape[0], _p(X), _p(conn), None)
        law, E, nu, rho = material
        mat = Material_(int(law), 0, float(E), float(nu), float(rho))
        barr = bc_array(bcs)
        opts = Opts_(t0, tf, scale_factor, max_steps, 0, 0)
        t = C.c_int64()
        st = load().msx_pool_submit(self.h, C.byref(mesh), C.byref(mat), _p(barr), len(barr),
                                    C.byref(opts), C.byref(t))
        if st == 9:
            return None
        _check(st)
        self.sizes[t.value] = X.shape[1]
        return t.value

    def step(self, steps=0):
        _check(load().msx_pool_step(self.h, steps))

    def serve(self, enabled=True):
        """Serving mode: a library thread steps the pool while solves are resident
        (submit, poll, wait and fetch keep working; step is refused)."""
        _check(load().msx_pool_serve(self.h, 1 if enabled else 0))

    def poll(self, max_results=4096):
        arr = (PoolResult_ * max_results)()
        n = C.c_int32()
        _check(load().msx_pool_poll(self.h, C.cast(arr, C.c_void_p), max_results, C.byref(n)))
        return [dict(ticket=arr[i].ticket, status=arr[i].status, steps=arr[i].steps, t=arr[i].t,
                     latency_ms=arr[i].submit_to_done_ms) for i in range(n.value)]

    def wait(self, ticket):
        """Step the pool until `ticket` has finished; its result (fetch it next)."""
        r = PoolResult_()
        _check(load().msx_pool_wait(self.h, ticket, C.byref(r)))
        return dict(ticket=r.ticket, status=r.status, steps=r.steps, t=r.t, latency_ms=r.submit_to_done_ms)

    def fetch(self, ticket, out=None):
        """u, v, a of a finished solve (into `out`, three contiguous float64 arrays
        of 3*nn, when given); releases its device memory."""
        nn = self.sizes[ticket]
        if out is None:
            out = tuple(np.zeros(3 * nn) for _ in range(3))
        for x in out:
            if x.dtype != np.float64 or x.size != 3 * nn or not x.flags.c_contiguous:
                raise ValueError("result buffers must be contiguous float64 arrays of 3*nn")
        u, v, a = out
        _check(load().msx_pool_fetch(self.h, ticket, _p(u), _p(v), _p(a)))
        del self.sizes[ticket]
        return u, v, a

    def inject_alloc_failures(self, count):
        """Make the next `count` submits fail their device allocation (MSX_ERR_OOM)."""
        _check(load().msx_pool_inject_alloc_failures(self.h, int(count)))

    def stats(self):
        st = PoolStats_()
        _check(load().msx_pool_stats_get(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in PoolStats_._fields_}

    def close(self):
        if getattr(self, "h", None):
            load().msx_pool_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
