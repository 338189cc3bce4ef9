"""Edge cases of the explicit step on the GPU, against the oracle: a single
tet, a mesh whose every DOF is prescribed, a solver chain that changes
precision between blocks, a block of zero length, malformed meshes, ramps
given by their rate, nodes shared by 100 and 1100 elements."""
import numpy as np
import pytest

import msx
import oracle as O

MODES = [(msx.FP64_EXACT, 1e-12), (msx.FP64, 1e-10), (msx.MIXED, 1e-5), (msx.DOUBLE_WORD, 1e-10)]


def rel(x, y):
    return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))


def run_gpu(mesh, law, solvers, precision):
    s0 = solvers[0]
    S = msx.Solver(mesh.X, mesh.conn, [(law, 1e6, 0.3, 1000.0)], s0.bcs, s0.t0, s0.tf, s0.scale_factor,
                   precision=precision[0] if isinstance(precision, tuple) else precision)
    steps = S.run().steps
    for k, s in enumerate(solvers[1:], 1):
        S.next_solver(s.bcs, s.t0, s.tf, s.scale_factor,
                      precision=precision[k] if isinstance(precision, tuple) else precision)
        steps += S.run().steps
    out = S.state()
    S.close()
    return out, steps


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", MODES)
def test_single_tet(precision, tol):
    X = np.array([[0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0]])
    mesh = O.Mesh(X, np.array([[0, 1, 2, 3]], np.int32))
    bcs = [(0 + c * 4, O.BC_RAMP, 0.0, 0) for c in range(3)] + [(3 + 2 * 4, O.BC_RAMP, 0.01, 0)]
    solvers = [O.Solver(0.0, 0.01, 0.5, bcs)]
    ref = O.run(mesh, [O.Material(O.COMPRESSIBLE_NH)], solvers)
    (u, v, a), steps = run_gpu(mesh, msx.COMPRESSIBLE_NH, solvers, precision)
    assert steps == ref.steps > 0
    assert rel(u, ref.u) <= tol and rel(v, ref.v) <= 10 * tol


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", MODES)
def test_every_dof_prescribed(precision, tol):
    mesh = O.cube_mesh(3)
    rng = np.random.default_rng(5)
    bcs = [(d, O.BC_RAMP, float(x), 0) for d, x in enumerate(rng.uniform(-1e-3, 1e-3, 3 * mesh.nn))]
    solvers = [O.Solver(0.0, 0.02, 0.5, bcs)]
    ref = O.run(mesh, [O.Material(O.STVK)], solvers)
    (u, v, a), steps = run_gpu(mesh, msx.STVK, solvers, precision)
    assert steps == ref.steps > 0
    # no DOF is free: u is the sum of the ramp increments, a stays zero
    assert rel(u, ref.u) <= tol and not a.any()


@pytest.mark.gpu
def test_chain_changes_precision():
    mesh = O.cube_mesh(4)
    solvers = [O.Solver(0.0, 0.01, 0.5, O.cube_bcs(4, 0.001)), O.Solver(0.01, 0.02, 0.5, O.cube_bcs(4, 0.002)),
               O.Solver(0.02, 0.03, 0.5, O.cube_bcs(4, 0.003))]
    ref = O.run(mesh, [O.Material(O.COMPRESSIBLE_NH)], solvers)
    (u, v, a), steps = run_gpu(mesh, msx.COMPRESSIBLE_NH, solvers, (msx.FP64, msx.MIXED, msx.FP64))
    assert steps == ref.steps
    assert rel(u, ref.u) <= 1e-5
    (u, v, a), steps = run_gpu(mesh, msx.COMPRESSIBLE_NH, solvers, (msx.DOUBLE_WORD, msx.FP64, msx.DOUBLE_WORD))
    assert steps == ref.steps
    assert rel(u, ref.u) <= 1e-10


@pytest.mark.gpu
def test_zero_length_block_takes_no_step():
    mesh = O.cube_mesh(2)
    bcs = [(d, O.BC_INST, 1e-4, 0) for d in range(3)]
    S = msx.Solver(mesh.X, mesh.conn, [(msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0)], bcs, 0.01, 0.01, 0.5)
    rep = S.run()
    u, v, a = S.state()
    S.close()
    assert rep.steps == 0 and not u.any() and not v.any()


@pytest.mark.gpu
def test_malformed_meshes_are_refused():
    X, conn = msx.mesh_cube(2)
    mat = [(msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0)]
    bad = conn.copy()
    bad[3, 2] = X.shape[1]                      # node index past the end
    with pytest.raises(msx.MsxError):
        msx.Solver(X, bad, mat, [], 0.0, 0.01, 0.5)
    bad = conn.copy()
    bad[0, 0] = -1
    with pytest.raises(msx.MsxError):
        msx.Solver(X, bad, mat, [], 0.0, 0.01, 0.5)
    with pytest.raises(msx.MsxError):
        msx.Solver(X, conn, mat, [(3 * X.shape[1], msx.BC_RAMP, 0.0, 0)], 0.0, 0.01, 0.5)   # DOF out of range
    with pytest.raises(msx.MsxError):
        msx.Solver(X, conn, [(msx.COMPRESSIBLE_NH, 1e6, 0.3, -1.0)], [], 0.0, 0.01, 0.5)  # negative density


@pytest.mark.gpu
@pytest.mark.parametrize("law", [O.COMPRESSIBLE_NH, O.NEO_HOOKEAN, O.STVK])
@pytest.mark.parametrize("precision", [msx.FP64, msx.DOUBLE_WORD])
def test_large_compression(law, precision):
    """A 4^3 cube squeezed by 30 % in z: J far from 1, so the log series gives way
    to the library log, 1/J is far from 1, and the strains are finite."""
    mesh = O.cube_mesh(4)
    solvers = [O.Solver(0.0, 0.05, 0.5, O.cube_bcs(4, -0.3))]
    ref = O.run(mesh, [O.Material(law)], solvers)
    (u, v, a), steps = run_gpu(mesh, law, solvers, precision)
    assert steps == ref.steps
    assert np.abs(u).max() > 0.2          # the top really moved
    assert rel(u, ref.u) <= 1e-10, rel(u, ref.u)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [msx.FP64_EXACT, msx.FP64, msx.MIXED, msx.DOUBLE_WORD])
def test_ramp_given_by_its_rate(precision):
    """MSX_BC_RAMP_RATE takes the rate a ramped classDirichlet stores
    (U / (tf - t0)); given the same division it is bit for bit MSX_BC_RAMP,
    in a two-block chain (rates of each block's own duration) and in the pool."""
    n, t0, t1, t2 = 4, 0.0, 0.013, 0.029
    X, conn = msx.mesh_cube(n, seed=5)
    ramp1, ramp2 = msx.cube_bcs(n, 0.002), msx.cube_bcs(n, 0.005)
    rate = lambda bcs, d: [(dof, msx.BC_RAMP_RATE, value / d, 0) for dof, _, value, _ in bcs]
    out = []
    for b1, b2 in ((ramp1, ramp2), (rate(ramp1, t1 - t0), rate(ramp2, t2 - t1))):
        S = msx.Solver(X, conn, [(msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0)], b1, t0, t1, 0.5, precision=precision)
        S.run()
        S.next_solver(b2, t1, t2, 0.5, precision=precision)
        S.run()
        out.append(S.state())
        S.close()
    for x, y in zip(*out):
        assert np.array_equal(x, y)
    if precision in (msx.FP64, msx.MIXED, msx.DOUBLE_WORD):
        P = msx.Pool(max_slots=2, precision=precision, steps_per_launch=4)
        ta = P.submit(X, conn, (msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0), ramp1, 0, t0, t1)
        tb = P.submit(X, conn, (msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0), rate(ramp1, t1 - t0), 0, t0, t1)
        P.wait(ta)
        P.wait(tb)
        ua, ub = P.fetch(ta), P.fetch(tb)
        P.close()
        for x, y in zip(ua, ub):
            assert np.array_equal(x, y)


def fan_mesh(m):
    """m tets sharing an apex (node 0) and a base centre (node 1) over a ring of
    m nodes: two nodes of degree m, the ring nodes of degree 2."""
    ang = 2 * np.pi * np.arange(m) / m
    X = np.zeros((3, m + 2))
    X[2, 0] = 1.0
    X[0, 2:], X[1, 2:] = np.cos(ang), np.sin(ang)
    conn = np.array([[0, 1, 2 + i, 2 + (i + 1) % m] for i in range(m)], np.int32)
    return O.Mesh(X, conn)


@pytest.mark.gpu
@pytest.mark.parametrize("m", [100, 1100])
def test_high_degree_nodes(m):
    """Node lists far longer than a tet mesh's ~24: 100 (sorted on the device)
    and 1100 (above the device builder's limit: built on the host).  Element
    order of every node's sum is kept: the reference-order mode equals the
    oracle bit for bit (St-Venant-Kirchhoff), the FP64 mode within 1e-10."""
    mesh = fan_mesh(m)
    bcs = [(i + c * mesh.nn, O.BC_RAMP, 0.0, 0) for i in range(2, mesh.nn) for c in range(3)]
    bcs += [(0 + 2 * mesh.nn, O.BC_RAMP, -0.01, 0)]
    solvers = [O.Solver(0.0, 1.0, 0.5, bcs, max_steps=6)]
    ref = O.run(mesh, [O.Material(O.STVK)], solvers)
    for precision, tol in ((msx.FP64_EXACT, 0.0), (msx.FP64, 1e-10)):
        S = msx.Solver(mesh.X, mesh.conn, [(msx.STVK, 1e6, 0.3, 1000.0)], bcs, 0.0, 1.0, 0.5, max_steps=6,
                       precision=precision)
        assert S.run().steps == ref.steps == 6
        u, v, a = S.state()
        S.close()
        if tol == 0.0:
            assert np.array_equal(u, ref.u) and np.array_equal(v, ref.v) and np.array_equal(a, ref.a)
        else:
            assert rel(u, ref.u) <= tol and rel(a, ref.a) <= tol


@pytest.mark.gpu
def test_double_word_refuses_values_outside_its_range():
    """The double-word mode's low words need FP32's normal range: material
    constants or nonzero coordinates outside [2^-100, 2^100] are refused
    (MSX_ERR_ARG) by msx_create, msx_next_solver and msx_pool_submit; the
    other modes take them."""
    X, conn = msx.mesh_cube(2)
    tiny = X * 2.0 ** -110                       # a mesh in absurd units
    bcs = msx.cube_bcs(2, 0.0)
    mat = (msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0)
    for Xc, m in ((tiny, mat), (X, (msx.COMPRESSIBLE_NH, 1e35, 0.3, 1000.0))):
        with pytest.raises(msx.MsxError) as ei:
            msx.Solver(Xc, conn, [m], bcs, 0.0, 1.0, 0.5, precision=msx.DOUBLE_WORD)
        assert ei.value.status == 1 and b"double-word" in msx.load().msx_last_error()
        S = msx.Solver(Xc, conn, [m], bcs, 0.0, 1.0, 0.5, precision=msx.FP64)
        with pytest.raises(msx.MsxError) as ei:
            S.next_solver(bcs, 1.0, 2.0, 0.5, precision=msx.DOUBLE_WORD)
        assert ei.value.status == 1
        S.close()
        P = msx.Pool(max_slots=2, precision=msx.DOUBLE_WORD)
        with pytest.raises(msx.MsxError) as ei:
            P.submit(Xc, conn, m, bcs, 5)
        assert ei.value.status == 1
        P.close()
    S = msx.Solver(X, conn, [mat], bcs, 0.0, 1.0, 0.5, precision=msx.DOUBLE_WORD)   # ordinary units
    S.close()
