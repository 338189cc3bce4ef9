"""The oracle against the reference's own outputs (golden fixtures) and
against invariants of the element formulation.  CPU only."""
import numpy as np
import pytest

import oracle as O
from golden_cases import load, load_loads, names


@pytest.mark.parametrize("name", names())
def test_oracle_matches_reference_bitwise(name):
    mesh, mats, solvers, (u, v, a), steps = load(name)
    r = O.run(mesh, mats, solvers, nthreads=2, loads=load_loads(name))
    assert r.status == 0 and r.steps == steps
    # the oracle keeps the reference's operation order: identical bits
    assert np.array_equal(r.u, u)
    assert np.array_equal(r.v, v)
    assert np.array_equal(r.a, a)


def test_cube_generator_counts_and_volume():
    n = 5
    m = O.cube_mesh(n)
    assert m.nn == (n + 1) ** 3 and m.ne == 6 * n ** 3
    dphi, wJ, L = O.precompute(m)
    # wJ = 0.166666666667*|detJ| = (1+3e-13)*V: the tets tile the unit cube
    assert abs(wJ.sum() - 1.0) < 1e-9
    assert (L > 0).all()


@pytest.mark.parametrize("law", [O.NEO_HOOKEAN, O.COMPRESSIBLE_NH, O.STVK])
def test_stress_zero_at_identity_and_rotation(law):
    mat = O.Material(law)
    assert np.abs(O.stress(mat, np.eye(3))).max() < 1e-9
    th = 0.3
    R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    assert np.abs(O.stress(mat, R)).max() < 1e-6 * mat.young


@pytest.mark.parametrize("law", [O.COMPRESSIBLE_NH, O.STVK])
def test_stress_is_energy_gradient(law):
    """P = dW/dF for the laws whose energy the reference defines
    (hyperElasticNeoHookean.cpp:291-304, hyperElasticStVenantKirchhoff.cpp:251-274)."""
    mat = O.Material(law, 1e6, 0.3, 1000.0)
    lam = mat.young * mat.nu / ((1 + mat.nu) * (1 - 2 * mat.nu))
    mu = 0.5 * mat.young / (1 + mat.nu)

    def W(F):
        if law == O.COMPRESSIBLE_NH:
            J = np.linalg.det(F)
            return 0.5 * lam * np.log(J) ** 2 - mu * np.log(J) + 0.5 * mu * np.trace(F.T @ F)
        E = 0.5 * (F.T @ F - np.eye(3))
        return 0.5 * np.sum((2 * mu * E + lam * np.trace(E) * np.eye(3)) * E)

    rng = np.random.default_rng(3)
    F = np.eye(3) + 0.05 * rng.standard_normal((3, 3))
    P = O.stress(mat, F)
    h = 1e-6
    G = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            Fp, Fm = F.copy(), F.copy()
            Fp[i, j] += h
            Fm[i, j] -= h
            G[i, j] = (W(Fp) - W(Fm)) / (2 * h)
    assert np.abs(G - P).max() < 1e-5 * np.abs(P).max()


def test_rigid_translation_gives_zero_force():
    m = O.cube_mesh(3)
    u = np.zeros(3 * m.nn)
    u[: m.nn] = 0.3
    u[2 * m.nn:] = -0.1
    f, F, P = O.internal_force(m, [O.Material(O.COMPRESSIBLE_NH)], u)
    assert np.abs(f).max() < 1e-9


@pytest.mark.parametrize("name", names())
def test_oracle_output_fields_match_reference_vtk(name):
    """Cauchy, Green-Lagrange and von Mises of the final state against the
    reference's own VTK output (written with 6 significant digits)."""
    import numpy as np
    from golden_cases import GOLDEN
    mesh, mats, solvers, (u, v, a), steps = load(name)
    d = np.load(GOLDEN + "/" + name + ".npz")
    cau, E, vms = O.element_fields(mesh, mats, u)
    for mine, ref in ((cau.reshape(-1, 9), d["vtk_cauchy"]), (E.reshape(-1, 9), d["vtk_E"]), (vms, d["vtk_vms"])):
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.all(np.abs(mine - ref) <= 6e-6 * np.abs(ref) + 1e-6 * scale)


def _plane_faces(mesh, coord, value):
    import golden.make_golden as G   # noqa: E402  (face numbering helper of the fixture generator)
    return G.plane_faces(mesh, coord, value)


def test_surface_traction_totals_traction_times_area():
    m = O.cube_mesh(4)
    T = (1.5e3, -2e3, 3e3)
    loads = O.Loads([("traction_inst", 0.0, 1.0, T, S, el) for S, el in _plane_faces(m, 2, 1.0)])
    f = O.external_force(m, [O.Material()], loads, np.zeros(3 * m.nn), 0.5).reshape(3, -1)
    # one-point rule: each face node gets area/3 of the traction; the top face has area 1
    assert np.allclose(f.sum(axis=1), T, rtol=1e-12)
    # outside the window nothing is applied
    f2 = O.external_force(m, [O.Material()], loads, np.zeros(3 * m.nn), 1.5)
    assert not f2.any()


def test_surface_pressure_at_rest_is_p_area_normal():
    m = O.cube_mesh(3)
    P = 4e3
    faces = _plane_faces(m, 0, 1.0)
    inst = O.Loads([("pressure_inst", 0.0, 1.0, P, S, el) for S, el in faces])
    f = O.external_force(m, [O.Material()], inst, np.zeros(3 * m.nn), 0.25).reshape(3, -1)
    # F = I: the force is P A n0 with n0 the face's unit normal (+-x on the x = 1 face)
    total = f.sum(axis=1)
    assert abs(abs(total[0]) - P) < 1e-9 * P and np.abs(total[1:]).max() < 1e-9 * P
    # a follower load: a rigid rotation of the body rotates the force with it
    th = 0.2
    R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    u = (R @ m.X - m.X).reshape(-1)
    fr = O.external_force(m, [O.Material()], inst, u, 0.25).reshape(3, -1)
    assert np.allclose(fr.sum(axis=1), R @ total, rtol=1e-10, atol=1e-9 * P)


def test_surface_pressure_ramp_loads_first_tet_node():
    # the reference's ramp variant evaluates the bulk tet's shape functions at natural
    # coordinates 0: phi = (1, 0, 0, 0), the face force goes to the tet's first node
    m = O.cube_mesh(3)
    faces = _plane_faces(m, 0, 1.0)
    ramp = O.Loads([("pressure_ramp", 0.0, 1.0, 4e3, S, el) for S, el in faces])
    f = O.external_force(m, [O.Material()], ramp, np.zeros(3 * m.nn), 1.0).reshape(3, -1)
    loaded = set(np.nonzero(np.abs(f).sum(axis=0))[0])
    firsts = {int(m.conn[e][0]) for _, el in faces for e in el}
    assert loaded and loaded <= firsts
    # at t = tf the ramp has reached P: same total as the instantaneous load
    inst = O.Loads([("pressure_inst", 0.0, 1.0, 4e3, S, el) for S, el in faces])
    fi = O.external_force(m, [O.Material()], inst, np.zeros(3 * m.nn), 1.0).reshape(3, -1)
    assert np.allclose(f.sum(axis=1), fi.sum(axis=1), rtol=1e-12, atol=1e-9)


def element_extraction_rows(name):
    """[(file name, quantity, op, elems or None, [(t, value), ...])] of a case's
    *EXTRACTION, ELEMENT blocks, as the reference wrote them; a block whose file
    name repeats an earlier one is dropped, as the reference keeps the first."""
    from golden_cases import load_extractions
    ex, files = load_extractions(name)
    out, seen = [], set()
    for e in ex:
        if e[0] != "element":
            continue
        _, label, q, op, elems = e
        fname = ("All" if elems is None else label) + "_%s_%s.csv" % (q, op)
        if fname in seen:
            continue
        seen.add(fname)
        rows = [tuple(float(x) for x in r.split(",")) for r in files[fname].strip().split("\n")[1:]]
        out.append((fname, q, op, elems, rows))
    return out


ELEMENT_CASES = ["cube3_cnh_element_extraction", "cube2_two_materials_element_extraction", "cube4_le_ramp",
                 "cube3_stvk_activation"]


@pytest.mark.parametrize("name", ELEMENT_CASES)
def test_element_extraction_pinned_to_reference(name):
    """Every row of every element-extraction file the reference wrote, from the
    oracle's state after that many steps, to the digit (%.16g)."""
    mesh, mats, solvers, _, steps = load(name)
    loads = load_loads(name)
    blocks = element_extraction_rows(name)
    assert blocks and all(len(b[4]) == steps for b in blocks)
    s0 = solvers[0]
    for k in range(1, steps + 1):
        r = O.run(mesh, mats, [O.Solver(s0.t0, s0.tf, s0.scale_factor, s0.bcs, max_steps=k,
                                        activation=s0.activation)], loads=loads)
        fext = O.external_force(mesh, mats, loads, r.u, r.t) if loads else np.zeros(3 * mesh.nn)
        for fname, q, op, elems, rows in blocks:
            t, val = rows[k - 1]
            assert t == float("%.16g" % r.t), fname
            got = O.element_reduce(mesh, mats, q, op, r.u, r.v, elems, fext, s0.activation, r.t)
            assert float("%.16g" % got) == val, (fname, k, got, val)


def test_element_extraction_files_dedupe_names():
    blocks = element_extraction_rows("cube3_cnh_element_extraction")
    assert [b[0] for b in blocks].count("mid_SVM_Max.csv") == 1
    # the kept block is the first one, over the 40 'mid' elements
    assert len([b for b in blocks if b[0] == "mid_SVM_Max.csv"][0][3]) == 40


def test_element_values_agree_with_reductions():
    """Per-element values against the reductions built from them, and the
    identities the quantities obey (KVM = SVM det F, VOLUME = wJ det F)."""
    mesh, mats, solvers, (u, v, _), _ = load("cube3_cnh_element_extraction")
    _, wJ, _ = O.precompute(mesh)
    val = {q: O.element_values(mesh, mats, q, u, v) for q in ("FXX", "FYY", "FZZ", "FXY", "FYZ", "FZX", "FYX", "FZY",
                                                             "FXZ", "SVM", "KVM", "VOLUME", "DEFO_ENERGY", "KIN_ENERGY")}
    F = np.stack([val[k] for k in ("FXX", "FXY", "FXZ", "FYX", "FYY", "FYZ", "FZX", "FZY", "FZZ")], 1).reshape(-1, 3, 3)
    detF = np.linalg.det(F)
    assert np.allclose(val["KVM"], val["SVM"] * detF, rtol=1e-12)
    assert np.allclose(val["VOLUME"], wJ * detF, rtol=1e-12)
    assert abs(O.element_reduce(mesh, mats, "DEFO_ENERGY", "Sum", u, v) - (val["DEFO_ENERGY"] * wJ).sum()) <= \
        1e-12 * abs(val["DEFO_ENERGY"] * wJ).sum()
    assert O.element_reduce(mesh, mats, "SVM", "Max", u, v) == val["SVM"].max()
    mean = O.element_reduce(mesh, mats, "KIN_ENERGY", "Mean", u, v)
    assert abs(mean - (val["KIN_ENERGY"] * wJ).sum() / wJ.sum()) <= 1e-12 * abs(mean)


def test_print_forces_pinned_to_reference():
    """*Forces: every row the reference wrote (which steps, the internal force of
    each listed node DOF, the time), from the oracle's state after that step,
    formatted as the reference formats it (std::to_string, i.e. %f)."""
    from golden_cases import load_force_files
    mesh, mats, solvers, _, _ = load("cube3_cnh_print_forces")
    files = load_force_files("cube3_cnh_print_forces")
    nn = mesh.nn
    for b, s in enumerate(solvers):
        freq, pairs = s.forces_out
        name = "externalForces%f-%f.csv" % (s.t0, s.tf)
        rows = files[name].strip().split("\n")
        assert rows[0] == "Node,Direction,Force,Time,"
        expect, done, k = [], 0, 0
        while k < 10000:
            k += 1
            r = O.run(mesh, mats, solvers[:b] + [O.Solver(s.t0, s.tf, s.scale_factor, s.bcs, max_steps=k)])
            period = max(1.0 / freq, r.dt_last)
            if r.t >= done * period + s.t0:
                fint = O.internal_force(mesh, mats, r.u)[0]
                expect += ["%d,%d,%f,%f," % (nd + 1, c, fint[nd + c * nn], r.t) for nd, c in pairs]
                done += 1
            if r.t >= s.tf - 1e-12:
                break
        assert rows[1:] == expect, name


def test_viscosity_keywords_leave_the_reference_unchanged():
    """*Bulk viscosity and *Dev viscosity: the reference multiplies by its
    element size and c0, which it never assigns (0 in its builds), and its
    deviatoric branch maps a zero tensor, so its results with the keywords are
    bit for bit those without them (golden fixtures from the reference)."""
    for name in ("cube3_cnh_bulk_viscosity", "cube3_stvk_dev_viscosity"):
        mesh, mats, solvers, (u, v, a), steps = load(name)
        assert all(s.viscosity for s in solvers)
        plain = [O.Solver(s.t0, s.tf, s.scale_factor, s.bcs) for s in solvers]
        r = O.run(mesh, mats, plain)
        assert r.steps == steps
        assert np.array_equal(r.u, u) and np.array_equal(r.v, v) and np.array_equal(r.a, a)


@pytest.mark.parametrize("law", [O.COMPRESSIBLE_NH, O.STVK])
def test_bulk_viscosity_force_matches_its_formula(law):
    """One step from rest with bulk viscosity (element size and c0 given): the
    acceleration changes by -f_vis/m on the free DOFs against the same step
    without it, with f_vis = wJ B^T P_vis, P_vis = J qBV F^-T,
    qBV = rho/J h (c1^2 h |trD| min(0, trD) + cl c0 trD) and trD = tr(F - I)/dt
    (solverExplicit.cpp:381-421, 514-541), evaluated here in numpy."""
    mesh = O.cube_mesh(3)
    bcs = O.cube_bcs(3, -0.004)             # the top moves down: trD < 0 near it
    mat = O.Material(law)
    h, c1, cl, c0 = 0.05, 1.5, 0.8, 40.0
    base = O.run(mesh, [mat], [O.Solver(0.0, 1.0, 0.5, bcs, max_steps=1)])
    vis = O.run(mesh, [mat], [O.Solver(0.0, 1.0, 0.5, bcs, max_steps=1, viscosity=(O.VISC_BULK, c1, cl, h, c0))])
    assert np.array_equal(base.u, vis.u) and base.dt_last == vis.dt_last
    dt, nn = vis.dt_last, mesh.nn
    dphi, wJ, _ = O.precompute(mesh)
    f = np.zeros(3 * nn)
    for e in range(mesh.ne):
        nd = mesh.conn[e]
        g = dphi[e].reshape(4, 3)
        F = np.eye(3) + sum(np.outer(vis.u[nd[a] + nn * np.arange(3)], g[a]) for a in range(4))
        trD = np.trace(F - np.eye(3)) / dt
        J = np.linalg.det(F)
        q = mat.rho / J * h * (c1 * c1 * h * abs(trD) * min(0.0, trD) + cl * c0 * trD)
        P = J * q * np.linalg.inv(F).T
        for a in range(4):
            f[nd[a] + nn * np.arange(3)] += wJ[e] * P @ g[a]
    m = O.lumped_mass(mesh, [mat], wJ)
    free = np.ones(3 * nn, bool)
    free[[b[0] for b in bcs]] = False
    want = -f[free] / np.tile(m, 3)[free]
    got = (vis.a - base.a)[free]
    assert np.abs(want).max() > 0
    assert np.abs(got - want).max() <= 1e-9 * np.abs(want).max()
