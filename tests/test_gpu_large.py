"""The large configuration (100^3-hex cube, 6,000,000 tets, 1,030,301 nodes)
against the oracle, the CPU restatement pinned bit for bit to the reference on
the golden decks (the reference itself needs hours per run at this size).

Runs the configuration's full 2000 steps (MSX_LARGE_STEPS overrides it for a
shorter check) of the bench workload: compressible neo-Hookean, bottom fixed,
top z velocity ramped to 0.1 m/s over 200 steps, dt = 0.5 CFL.  The oracle
uses every host core (about 3 minutes on 16 cores) and runs once for all four
precision modes.
"""
import os

import numpy as np
import pytest

import msx
import oracle as O

N, SEED, V_TOP, RAMP = 100, 1234, 0.1, 200
STEPS = int(os.environ.get("MSX_LARGE_STEPS", "2000"))


def rel(x, y):
    return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))


@pytest.fixture(scope="module")
def large_reference():
    mesh = O.cube_mesh(N, SEED, 0.1)
    bcs = O.cube_bcs(N, V_TOP, O.BC_VEL_RAMP, RAMP)
    r = O.run(mesh, [O.Material(O.COMPRESSIBLE_NH)], [O.Solver(0.0, 1e30, 0.5, bcs, max_steps=STEPS)],
              nthreads=os.cpu_count() or 1)
    assert r.status == 0 and r.steps == STEPS
    return mesh, bcs, r


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(msx.FP64, 1e-10), (msx.FP64_EXACT, 1e-12), (msx.MIXED, 1e-5),
                                           (msx.DOUBLE_WORD, 1e-10)])
def test_large_cube_against_oracle(large_reference, precision, tol):
    mesh, bcs, ref = large_reference
    S = msx.Solver(mesh.X, mesh.conn, [(msx.COMPRESSIBLE_NH, 1e6, 0.3, 1000.0)], bcs, 0.0, 1e30, 0.5,
                   max_steps=STEPS, precision=precision)
    rep = S.run()
    u, v, a = S.state()
    S.close()
    assert rep.steps == STEPS and rep.status == 0
    print("large cube, %d steps, precision %d: rel L2 u %.3e v %.3e" % (STEPS, precision, rel(u, ref.u), rel(v, ref.v)))
    assert rel(u, ref.u) <= tol
    assert rel(v, ref.v) <= 10 * tol
