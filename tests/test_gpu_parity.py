"""CUDA path against the reference's own outputs (golden fixtures) and the
oracle.  Tolerances: FP64_EXACT relative L2 <= 1e-12 (bit-identical where no
transcendental is involved), FP64 relative L2 <= 1e-10 (the bar of the plain FP64 path),
MIXED relative L2 <= 1e-5."""
import numpy as np
import pytest

import msx
import oracle as O
from golden_cases import load, load_loads, names

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="session", autouse=True)
def built():
    import build
    build.build()
    msx.load()


def rel(x, y):
    return np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300)


def run_case(name, precision, spg=0):
    mesh, mats, solvers, ref, steps = load(name)
    m = [(x.law, x.young, x.nu, x.rho) for x in mats]
    s0 = solvers[0]
    S = msx.Solver(mesh.X, mesh.conn, m, s0.bcs, s0.t0, s0.tf, s0.scale_factor, precision=precision,
                   elem_material=mesh.elem_mat, steps_per_graph=spg)
    L = load_loads(name)
    if L is not None:
        S.set_load_blocks(L.items)
    if mesh.act_time is not None:
        S.set_activation(mesh.act_time, s0.activation)
    if s0.viscosity:
        S.set_viscosity(*s0.viscosity)
    total = S.run().steps
    for s in solvers[1:]:
        S.next_solver(s.bcs, s.t0, s.tf, s.scale_factor, precision=precision, steps_per_graph=spg)
        if mesh.act_time is not None:
            S.set_activation(None, s.activation)
        S.set_viscosity(*(s.viscosity or (msx.VISC_NONE,)))
        total += S.run().steps
    out = S.state()
    S.close()
    return out, ref, total, steps


@pytest.mark.parametrize("name", names())
def test_exact_mode_matches_reference(name):
    (u, v, a), (ur, vr, ar), steps, ref_steps = run_case(name, msx.FP64_EXACT)
    assert steps == ref_steps
    assert rel(u, ur) <= 1e-12 and rel(v, vr) <= 1e-12 and rel(a, ar) <= 1e-11
    if all(m.law in (O.STVK, O.LINEAR_ELASTIC) for m in load(name)[1]):
        # no log/pow on these laws' path: bit-identical to the reference
        assert np.array_equal(u, ur) and np.array_equal(v, vr) and np.array_equal(a, ar)


@pytest.mark.parametrize("name", names())
def test_fp64_mode_matches_reference(name):
    (u, v, a), (ur, vr, ar), steps, ref_steps = run_case(name, msx.FP64)
    assert steps == ref_steps
    assert rel(u, ur) <= 1e-10, rel(u, ur)
    assert rel(v, vr) <= 1e-10


@pytest.mark.parametrize("name", names())
def test_double_word_mode_matches_reference(name):
    """FP64's algebra in double-word arithmetic: within the FP64 bar of the reference."""
    (u, v, a), (ur, vr, ar), steps, ref_steps = run_case(name, msx.DOUBLE_WORD)
    assert steps == ref_steps
    print("%s: double-word rel L2 u %.2e v %.2e" % (name, rel(u, ur), rel(v, vr)))
    assert rel(u, ur) <= 1e-10, rel(u, ur)
    assert rel(v, vr) <= 1e-10


@pytest.mark.parametrize("name", [n for n in names() if n.startswith("cube10")] +
                         ["cube4_le_ramp", "cube3_stvk_activation", "cube3_le_activation_chain"])
def test_mixed_mode_error_bound(name):
    (u, v, a), (ur, vr, ar), steps, ref_steps = run_case(name, msx.MIXED)
    # the stable dt is the FP64 minimum (FP32 screen + FP64 recheck), so the
    # mixed run takes the reference's steps
    assert steps == ref_steps
    assert rel(u, ur) <= 1e-5, rel(u, ur)


def cfl_dt_host(X, conn, u, Lref, c, sf):
    """sf * min_e min(Lref_e, 2 r(X + u)_e) / c in FP64 on the host: the
    inscribed-sphere diameter 2 |e1.(e2 x e3)| / (sum of face areas)
    (geometry.cpp:264-301, solvers.cpp:296-320)."""
    nn = X.shape[1]
    x = X + u.reshape(3, nn)
    p = [x[:, conn[:, k]].T for k in range(4)]
    e1, e2, e3 = p[1] - p[0], p[2] - p[0], p[3] - p[0]
    A, B, Cc = np.cross(e1, e2), np.cross(e1, e3), np.cross(e2, e3)
    D = Cc + A - B
    s = sum(np.sqrt((q * q).sum(1)) for q in (A, B, Cc, D))
    dist = 2 * np.abs((e1 * Cc).sum(1)) / s
    return sf * (np.minimum(dist, Lref) / c).min()


@pytest.mark.parametrize("law", [msx.COMPRESSIBLE_NH, msx.STVK])
def test_mixed_dt_is_the_fp64_cfl_of_its_state(law):
    """Each mixed step's dt is sf times the FP64 CFL minimum over the mesh at
    the mixed state (the FP32 screen only picks which elements to evaluate in
    FP64): after 150 steps of a deforming 10^3 cube, the next dt equals the
    host's FP64 evaluation to rounding (an FP32 CFL minimum would be ~1e-8 off)."""
    X, conn = msx.mesh_cube(10, seed=3)
    bcs = msx.cube_bcs(10, 0.5, msx.BC_VEL_RAMP, 20)
    E, nu, rho = 1e6, 0.3, 1000.0
    S = msx.Solver(X, conn, [(law, E, nu, rho)], bcs, 0.0, 1e30, 0.5, precision=msx.MIXED)
    S.run(150)
    u = S.state()[0]
    _, _, Lref, _ = S.element_data()
    dt = S.run(1).dt
    S.close()
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), 0.5 * E / (1 + nu)
    c = np.sqrt(E / rho) if law == msx.STVK else np.sqrt((lam + 2 * mu) / rho)
    ref = cfl_dt_host(X, conn, u, Lref, c, 0.5)
    assert np.abs(u).max() > 1e-3
    assert abs(dt - ref) <= 1e-13 * ref, (dt, ref, dt / ref - 1)


def test_graph_chunk_size_does_not_change_results():
    r1 = run_case("cube4_nh_ramp", msx.FP64, spg=2)[0]
    r2 = run_case("cube4_nh_ramp", msx.FP64, spg=128)[0]
    assert all(np.array_equal(x, y) for x, y in zip(r1, r2))


@pytest.mark.parametrize("precision", [msx.FP64, msx.MIXED])
def test_split_calls_replay_at_most_one_idle_step(precision):
    """Calls of any length run full chunks plus power-of-two remainders: the
    state after calls of 1, 2, 5, 20, 64 and 13 steps is bitwise that of one
    105-step call, and each call launches at most K + 2 step pairs."""
    X, conn = msx.mesh_cube(4, seed=3)
    bcs = msx.cube_bcs(4, 0.5, msx.BC_VEL_RAMP, 50)
    mat = [(msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0)]

    def solver():
        return msx.Solver(X, conn, mat, bcs, 0.0, 1e30, 0.5, max_steps=0, precision=precision,
                          steps_per_graph=16)

    A = solver()
    for k in (1, 2, 5, 20, 64, 13):
        rep = A.run(k)
        assert rep.steps == k
        assert k + 1 <= rep.kernel_launches // 2 <= k + 2, (k, rep.kernel_launches)
    B = solver()
    assert B.run(105).steps == 105
    assert all(np.array_equal(x, y) for x, y in zip(A.state(), B.state()))
    A.close()
    B.close()


def test_setup_data_bitwise_equal_to_oracle():
    mesh, mats, solvers, _, _ = load("cube4_stvk_ramp")
    S = msx.Solver(mesh.X, mesh.conn, [(m.law, m.young, m.nu, m.rho) for m in mats], solvers[0].bcs,
                   0.0, 0.02, 0.5)
    G, wJ, L, mass = S.element_data()
    dphi, wJo, Lo = O.precompute(mesh)
    assert np.array_equal(G.T.reshape(-1, 3, 3), dphi.reshape(-1, 4, 3)[:, 1:, :])
    assert np.array_equal(wJ, wJo) and np.array_equal(L, Lo)
    assert np.array_equal(mass, O.lumped_mass(mesh, mats, wJo))


def test_setup_data_bitwise_equal_to_oracle_large_two_materials():
    """A mesh of 2^20 elements or more takes the chunked connectivity upload,
    with the element set-up following each piece and the material ids and node
    lists on the second stream: its set-up data stay bit for bit the oracle's,
    with signed zeros among the coordinates (the Jacobian's (0 - x0) + x1 form)
    and two materials (the lumped mass's (3z) + z sum)."""
    n = 60
    X, conn = msx.mesh_cube(n, seed=5, jitter=0.1)
    assert conn.shape[0] >= 1 << 20
    X = X.copy()
    flat = X.reshape(-1)
    zeros = np.nonzero(flat == 0.0)[0]
    assert zeros.size > 100
    flat[zeros[::2]] = -0.0
    em = (np.arange(conn.shape[0]) % 3 == 0).astype(np.int32)
    mats = [O.Material(O.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0), O.Material(O.STVK, 3e6, 0.25, 2500.0)]
    mesh = O.Mesh(X, conn, elem_mat=em)
    S = msx.Solver(X, conn, [(m.law, m.young, m.nu, m.rho) for m in mats],
                   msx.cube_bcs(n, 0.1, msx.BC_VEL_RAMP, 200), 0.0, 0.02, 0.5, elem_material=em)
    G, wJ, L, mass = S.element_data()
    S.close()
    dphi, wJo, Lo = O.precompute(mesh)
    assert np.array_equal(G.T.reshape(-1, 3, 3), dphi.reshape(-1, 4, 3)[:, 1:, :])
    assert np.array_equal(wJ, wJo) and np.array_equal(L, Lo)
    assert np.array_equal(mass, O.lumped_mass(mesh, mats, wJo))


@pytest.mark.parametrize("law", [msx.NEO_HOOKEAN, msx.COMPRESSIBLE_NH, msx.STVK, msx.LINEAR_ELASTIC])
@pytest.mark.parametrize("precision,tol", [(msx.FP64_EXACT, 0.0), (msx.FP64, 1e-12), (msx.MIXED, 2e-5),
                                           (msx.DOUBLE_WORD, 1e-11)])
def test_internal_force_matches_oracle(law, precision, tol):
    X, conn = msx.mesh_cube(5, seed=7)
    mesh = O.Mesh(X, conn)
    rng = np.random.default_rng(law)
    u = 2e-3 * rng.standard_normal(3 * mesh.nn)
    mat = O.Material(law, 1e6, 0.3, 1000.0)
    S = msx.Solver(X, conn, [(law, 1e6, 0.3, 1000.0)], [], 0.0, 1.0, 0.5, precision=precision)
    f = S.internal_force(u)
    fo, _, _ = O.internal_force(mesh, [mat], u)
    if tol == 0.0 and law in (msx.STVK, msx.LINEAR_ELASTIC):
        assert np.array_equal(f, fo)
    else:
        assert rel(f, fo) <= max(tol, 1e-14), rel(f, fo)


def test_runs_are_deterministic():
    X, conn = msx.mesh_cube(12, seed=5)
    bcs = msx.cube_bcs(12, 0.1, msx.BC_VEL_RAMP, 50)
    outs = []
    for _ in range(2):
        S = msx.Solver(X, conn, [(1, 1e6, 0.3, 1000.0)], bcs, 0.0, 1e9, 0.5, max_steps=300)
        S.run()
        outs.append(S.state())
    assert all(np.array_equal(x, y) for x, y in zip(*outs))


@pytest.mark.parametrize("precision,tol", [(msx.FP64, 1e-10), (msx.MIXED, 1e-5), (msx.DOUBLE_WORD, 1e-10)])
def test_velocity_ramp_extension_matches_oracle(precision, tol):
    n = 8
    X, conn = msx.mesh_cube(n)
    bcs = msx.cube_bcs(n, 0.1, msx.BC_VEL_RAMP, 200)
    S = msx.Solver(X, conn, [(1, 1e6, 0.3, 1000.0)], bcs, 0.0, 1e9, 0.5, max_steps=400, precision=precision)
    rep = S.run()
    u, v, a = S.state()
    r = O.run(O.Mesh(X, conn), [O.Material(1)], [O.Solver(0.0, 1e9, 0.5, bcs, max_steps=400)], nthreads=4)
    assert rep.steps == r.steps == 400
    assert rel(u, r.u) <= tol, rel(u, r.u)


def test_max_steps_per_call_and_resume():
    n = 6
    X, conn = msx.mesh_cube(n)
    bcs = msx.cube_bcs(n, 0.02)
    S = msx.Solver(X, conn, [(2, 1e6, 0.3, 1000.0)], bcs, 0.0, 0.05, 0.5)
    r1 = S.run(7)
    assert r1.steps == 7
    r2 = S.run()
    u = S.state()[0]
    ro = O.run(O.Mesh(X, conn), [O.Material(2)], [O.Solver(0.0, 0.05, 0.5, bcs)])
    assert r1.steps + r2.steps == ro.steps
    assert rel(u, ro.u) <= 1e-10


def test_nan_in_displacement_is_reported():
    n = 3
    X, conn = msx.mesh_cube(n)
    S = msx.Solver(X, conn, [(1, 1e6, 0.3, 1000.0)], msx.cube_bcs(n, 0.001), 0.0, 0.05, 0.5)
    u0 = np.zeros(3 * S.nn)
    u0[1] = np.nan          # node 1, x: the one DOF the reference checks
    S.set_state(u=u0)
    with pytest.raises(msx.MsxError) as ei:
        S.run()
    assert ei.value.status == 4 and S.last_report.steps == 1


def test_degenerate_element_gives_negative_jacobian_error():
    X, conn = msx.mesh_cube(2)
    X = X.copy()
    X[2, conn[0]] = 0.0     # flatten element 0 into the z=0 plane... then its length is 0
    X[:, conn[0][3]] = X[:, conn[0][0]]
    S = msx.Solver(X, conn, [(2, 1e6, 0.3, 1000.0)], [], 0.0, 0.05, 0.5)
    with pytest.raises(msx.MsxError) as ei:
        S.run()
    assert ei.value.status == 3


@pytest.mark.parametrize("name", ["cube4_nh_ramp", "cube4_stvk_ramp", "cube10_cnh_S", "cube2_two_materials",
                                  "cube4_le_ramp", "cube2_le_cnh"])
def test_element_fields_match_oracle(name):
    mesh, mats, solvers, (u, v, a), _ = load(name)
    m = [(x.law, x.young, x.nu, x.rho) for x in mats]
    S = msx.Solver(mesh.X, mesh.conn, m, solvers[0].bcs, 0.0, 1.0, 0.5, elem_material=mesh.elem_mat)
    S.set_state(u=u)
    cau, E, vms = S.element_fields()
    S.close()
    oc, oE, ov = O.element_fields(mesh, mats, u)
    for x, y in ((cau, oc), (E, oE), (vms, ov)):
        assert rel(x, y) <= 1e-12, rel(x, y)


@pytest.mark.parametrize("name", ["cube3_cnh_force_gravity", "cube3_nh_gravity_force"])
def test_force_gravity_wrapper_equals_blocks(name):
    """msx_set_loads (forces + gravity) is the two-block case of msx_set_load_blocks."""
    mesh, mats, solvers, ref, steps = load(name)
    L = load_loads(name)
    m = [(x.law, x.young, x.nu, x.rho) for x in mats]
    s0 = solvers[0]
    out = []
    for use_blocks in (False, True):
        S = msx.Solver(mesh.X, mesh.conn, m, s0.bcs, s0.t0, s0.tf, s0.scale_factor, precision=msx.FP64_EXACT)
        if use_blocks:
            S.set_load_blocks(L.items)
        else:
            S.set_loads(L.force_entries(mesh.nn), L.gravity(), L.gravity_first())
        S.run()
        out.append(S.state())
        S.close()
    assert all(np.array_equal(x, y) for x, y in zip(*out))


def test_surface_load_errors():
    X, conn = msx.mesh_cube(2)
    S = msx.Solver(X, conn, [(msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0)], msx.cube_bcs(2, 0.0), 0.0, 0.01, 0.5)
    with pytest.raises(msx.MsxError):
        S.set_load_blocks([("pressure_inst", 0.0, 1.0, 1e3, 5, [0])])        # face 1..4 only
    with pytest.raises(msx.MsxError):
        S.set_load_blocks([("traction_inst", 0.0, 1.0, (1, 2, 3), 1, [len(conn)])])   # element range
    with pytest.raises(msx.MsxError):
        S.set_load_blocks([("pressure_ramp", 0.5, 0.5, 1e3, 1, [0])])        # ramp needs tf != t0
    S.close()


@pytest.mark.parametrize("precision,tol", [(msx.FP64_EXACT, 1e-12), (msx.FP64, 1e-10), (msx.MIXED, 2e-5),
                                           (msx.DOUBLE_WORD, 1e-10)])
def test_node_values_match_oracle(precision, tol):
    """msx_node_values: displacement, internal force (element-order sum) and
    external force of the last step, against the oracle at that state."""
    mesh, mats, solvers, _, _ = load("cube3_cnh_extraction")
    L = load_loads("cube3_cnh_extraction")
    s0 = solvers[0]
    m = [(x.law, x.young, x.nu, x.rho) for x in mats]
    S = msx.Solver(mesh.X, mesh.conn, m, s0.bcs, s0.t0, s0.tf, s0.scale_factor, precision=precision)
    S.set_load_blocks(L.items)
    rep = S.run(7)
    u = S.state()[0]
    nodes = np.arange(mesh.nn, dtype=np.int32)
    fint = O.internal_force(mesh, mats, u)[0]
    fext = O.external_force(mesh, mats, L, u, rep.t)
    for c in range(3):
        got_u = S.node_values(msx.FIELD_DISPLACEMENT, c, nodes)
        got_i = S.node_values(msx.FIELD_INTERNAL_FORCE, c, nodes)
        got_e = S.node_values(msx.FIELD_EXTERNAL_FORCE, c, nodes)
        assert np.array_equal(got_u, u[c * mesh.nn:(c + 1) * mesh.nn])
        ref_i, ref_e = fint[c * mesh.nn:(c + 1) * mesh.nn], fext[c * mesh.nn:(c + 1) * mesh.nn]
        assert np.abs(got_i - ref_i).max() <= tol * max(np.abs(fint).max(), 1e-300)
        assert np.abs(got_e - ref_e).max() <= 1e-12 * max(np.abs(fext).max(), 1e-300)
    S.close()


ELEMENT_QS = [q for q in msx.ELEMENT_QUANTITIES if q != "EXTERNAL_ENERGY"]


@pytest.mark.parametrize("name", ["cube3_cnh_element_extraction", "cube2_two_materials_element_extraction",
                                  "cube4_le_ramp"])
def test_element_values_match_oracle(name):
    """msx_element_values against the oracle at the same state (the reference's
    final u, v put in with msx_set_state): both follow the reference's operation
    order in FP64, so they agree to rounding (log and sqrt are the library's)."""
    mesh, mats, solvers, (u, v, a), _ = load(name)
    s0 = solvers[0]
    m = [(x.law, x.young, x.nu, x.rho) for x in mats]
    S = msx.Solver(mesh.X, mesh.conn, m, s0.bcs, s0.t0, s0.tf, s0.scale_factor, precision=msx.FP64_EXACT,
                   elem_material=mesh.elem_mat)
    S.set_state(u, v, a)
    some = np.array([7, 3, 3, 0, mesh.ne - 1], np.int32)
    for q in ELEMENT_QS:
        ref = O.element_values(mesh, mats, q, u, v)
        got = S.element_values(q)
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(got - ref).max() <= 1e-13 * scale, q
        assert np.array_equal(S.element_values(q, some), got[some]), q
    S.close()


@pytest.mark.parametrize("precision", [msx.FP64_EXACT, msx.FP64, msx.MIXED, msx.DOUBLE_WORD])
def test_element_reduce_matches_oracle(precision):
    """msx_element_reduce for every quantity and operation, over all elements
    and over a list with repeats in no order, against the oracle's reference-
    order reduction of the GPU's own state after 9 steps with loads (so the
    comparison isolates the extraction: tree sums against element-order sums)."""
    name = "cube3_cnh_element_extraction"
    mesh, mats, solvers, _, _ = load(name)
    L = load_loads(name)
    s0 = solvers[0]
    m = [(x.law, x.young, x.nu, x.rho) for x in mats]
    S = msx.Solver(mesh.X, mesh.conn, m, s0.bcs, s0.t0, s0.tf, s0.scale_factor, precision=precision)
    S.set_load_blocks(L.items)
    rep = S.run(9)
    u, v, _ = S.state()
    fext = O.external_force(mesh, mats, L, u, rep.t)
    lst = [90, 5, 17, 5, 60, 61, 62, 90, 1]
    _, wJ, _ = O.precompute(mesh)
    for q in msx.ELEMENT_QUANTITIES:
        vals = None if q == "EXTERNAL_ENERGY" else np.abs(O.element_values(mesh, mats, q, u, v))
        for op in ("Mean", "Min", "Max", "Sum"):
            if q == "VOLUME" and op == "Mean":
                with pytest.raises(msx.MsxError):
                    S.element_reduce(q, op)
                continue
            for el in (None, lst):
                ref = O.element_reduce(mesh, mats, q, op, u, v, el, fext)
                got = S.element_reduce(q, op, el)
                if q == "EXTERNAL_ENERGY":
                    scale = np.abs(u * fext).sum()
                elif op in ("Min", "Max"):
                    scale = abs(ref)
                else:   # the sum of the magnitudes a sum's rounding scales with
                    idx = np.arange(mesh.ne) if el is None else np.unique(el)
                    scale = (vals[idx] * (1.0 if q == "VOLUME" else wJ[idx])).sum()
                    scale /= wJ[idx].sum() if op == "Mean" else 1.0
                assert abs(got - ref) <= 1e-13 * max(scale, 1e-300), (q, op, el is None, got, ref)
    with pytest.raises(msx.MsxError):
        S.element_reduce("SVM", "Max", [])
    with pytest.raises(msx.MsxError):
        S.element_reduce("SVM", "Max", [mesh.ne])
    with pytest.raises(msx.MsxError):
        S.element_values("EXTERNAL_ENERGY")
    S.close()


def test_activation_api_errors_and_dead_elements():
    """msx_set_activation refuses to switch on without times; with every element
    dead the internal force is zero, so without loads the free DOFs stay at rest."""
    mesh, mats, solvers, _, _ = load("cube3_stvk_activation")
    s0 = solvers[0]
    m = [(x.law, x.young, x.nu, x.rho) for x in mats]
    S = msx.Solver(mesh.X, mesh.conn, m, s0.bcs, s0.t0, s0.tf, s0.scale_factor)
    with pytest.raises(msx.MsxError):
        S.set_activation(None, True)
    with pytest.raises(ValueError):
        S.set_activation(np.zeros(3), True)
    S.set_activation(np.full(mesh.ne, 1e9), True)   # nobody is born in this block
    S.run(5)
    nodes = np.arange(mesh.nn, dtype=np.int32)
    for c in range(3):
        assert not S.node_values(msx.FIELD_INTERNAL_FORCE, c, nodes).any()
    u = S.state()[0]
    fixed = np.zeros(3 * mesh.nn, bool)
    fixed[[b[0] for b in s0.bcs]] = True
    assert not u[~fixed].any() and u[fixed].any()
    S.set_activation(None, False)                   # everyone alive again
    S.run(1)
    assert any(S.node_values(msx.FIELD_INTERNAL_FORCE, c, nodes).any() for c in range(3))
    S.close()


VISC = (msx.VISC_BULK, 1.5, 0.8, 0.05, 40.0)   # kind, c1, cl, element size, c0


@pytest.mark.parametrize("law", [msx.COMPRESSIBLE_NH, msx.STVK])
@pytest.mark.parametrize("precision,tol", [(msx.FP64_EXACT, 1e-12), (msx.FP64, 1e-10), (msx.DOUBLE_WORD, 1e-10),
                                           (msx.MIXED, 1e-5)])
def test_bulk_viscosity_matches_oracle(law, precision, tol):
    """Bulk viscosity with an element size and c0 given (the reference leaves
    both unset): a cube compressed over a two-block chain, the viscosity kept
    on in the second block as the reference keeps it, against the oracle's
    restatement of the reference's formula; the result differs from the
    inviscid one by far more than the tolerance."""
    mesh = O.cube_mesh(4)
    solvers = [O.Solver(0.0, 0.01, 0.5, O.cube_bcs(4, -0.004), viscosity=VISC),
               O.Solver(0.01, 0.02, 0.45, O.cube_bcs(4, -0.006), viscosity=VISC)]
    ref = O.run(mesh, [O.Material(law)], solvers)
    plain = O.run(mesh, [O.Material(law)], [O.Solver(s.t0, s.tf, s.scale_factor, s.bcs) for s in solvers])
    assert rel(ref.u, plain.u) > 1e-3
    S = msx.Solver(mesh.X, mesh.conn, [(law, 1e6, 0.3, 1000.0)], solvers[0].bcs, 0.0, 0.01, 0.5,
                   precision=precision)
    S.set_viscosity(*VISC)
    steps = S.run().steps
    S.next_solver(solvers[1].bcs, 0.01, 0.02, 0.45, precision=precision)
    steps += S.run().steps
    u, v, a = S.state()
    S.close()
    assert steps == ref.steps
    assert rel(u, ref.u) <= tol, rel(u, ref.u)
    assert rel(v, ref.v) <= 10 * tol


def test_bulk_viscosity_across_a_precision_change():
    """FP64, mixed, FP64 blocks with bulk viscosity: each block starts from the
    handed-over state's F as the previous one, whatever the precision before."""
    mesh = O.cube_mesh(4)
    solvers = [O.Solver(0.0, 0.01, 0.5, O.cube_bcs(4, -0.004), viscosity=VISC),
               O.Solver(0.01, 0.02, 0.5, O.cube_bcs(4, -0.006), viscosity=VISC),
               O.Solver(0.02, 0.03, 0.5, O.cube_bcs(4, -0.007), viscosity=VISC)]
    ref = O.run(mesh, [O.Material(O.COMPRESSIBLE_NH)], solvers)
    S = msx.Solver(mesh.X, mesh.conn, [(msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0)], solvers[0].bcs, 0.0, 0.01, 0.5,
                   precision=msx.FP64)
    S.set_viscosity(*VISC)
    steps = S.run().steps
    for s, prec in zip(solvers[1:], (msx.MIXED, msx.FP64)):
        S.next_solver(s.bcs, s.t0, s.tf, s.scale_factor, precision=prec)
        steps += S.run().steps
    u = S.state()[0]
    S.close()
    assert steps == ref.steps
    assert rel(u, ref.u) <= 1e-5


def test_zero_element_size_viscosity_is_bitwise_inviscid():
    """The reference's own setting (element size and c0 never assigned, 0):
    bulk and deviatoric viscosity leave the FP64 run bit for bit unchanged."""
    X, conn = msx.mesh_cube(4, seed=3)
    bcs = msx.cube_bcs(4, 0.002)
    out = []
    for visc in (None, (msx.VISC_BULK, 0.06, 1.2, 0.0, 0.0), (msx.VISC_DEV, 1.0, 0.5, 0.0, 0.0)):
        S = msx.Solver(X, conn, [(msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0)], bcs, 0.0, 0.02, 0.5)
        if visc:
            S.set_viscosity(*visc)
        S.run()
        out.append(S.state())
        S.close()
    for o in out[1:]:
        assert all(np.array_equal(x, y) for x, y in zip(o, out[0]))


def test_bulk_viscosity_and_element_birth_are_refused_together():
    X, conn = msx.mesh_cube(2)
    S = msx.Solver(X, conn, [(msx.STVK, 1e6, 0.3, 1000.0)], [], 0.0, 0.01, 0.5)
    S.set_activation(np.zeros(S.ne), True)
    with pytest.raises(msx.MsxError) as ei:
        S.set_viscosity(*VISC)
    assert ei.value.status == 6
    S.set_activation(None, False)
    S.set_viscosity(*VISC)
    with pytest.raises(msx.MsxError) as ei:
        S.set_activation(None, True)
    assert ei.value.status == 6
    S.close()
