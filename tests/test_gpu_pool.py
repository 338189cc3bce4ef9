"""Batched / serving pool: every solve gives the same result in the mix as
alone (bit for bit: the pooled kernels run the same per-element and per-node
arithmetic, only the CTA schedule differs), admission respects the HBM budget,
and solves admitted while others run complete correctly."""
import numpy as np
import pytest

import msx

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="session", autouse=True)
def built():
    import build
    build.build()
    msx.load()


def case(n, E, nu, v_top, seed):
    X, conn = msx.mesh_cube(n, seed=seed)
    return X, conn, (msx.COMPRESSIBLE_NH, E, nu, 1000.0), msx.cube_bcs(n, v_top, msx.BC_VEL_RAMP, 20)


def alone(X, conn, mat, bcs, steps, precision):
    S = msx.Solver(X, conn, [mat], bcs, 0.0, 1e30, 0.5, max_steps=steps, precision=precision)
    S.run()
    out = S.state()
    S.close()
    return out


@pytest.mark.parametrize("precision", [msx.MIXED, msx.FP64, msx.DOUBLE_WORD])
def test_pool_results_equal_single_solves(precision):
    rng = np.random.default_rng(11)
    cases = [case(int(n), float(E), float(nu), float(v), s)
             for s, (n, E, nu, v) in enumerate(zip(rng.integers(3, 9, 6), 10 ** rng.uniform(5, 7, 6),
                                                   rng.uniform(0.25, 0.45, 6), rng.uniform(0.01, 0.2, 6)))]
    steps = [50 + 13 * k for k in range(len(cases))]
    P = msx.Pool(max_slots=8, precision=precision, steps_per_launch=8)
    tickets = [P.submit(X, c, m, b, st) for (X, c, m, b), st in zip(cases, steps)]
    assert all(t is not None for t in tickets)
    for _ in range(100):
        P.step()
    res = {r["ticket"]: r for r in P.poll()}
    assert set(res) == set(tickets)
    for t, (X, c, m, b), st in zip(tickets, cases, steps):
        assert res[t]["status"] == 0 and res[t]["steps"] == st
        u, v, a = P.fetch(t)
        ua, va, aa = alone(X, c, m, b, st, precision)
        assert np.array_equal(u, ua) and np.array_equal(v, va) and np.array_equal(a, aa)
    P.close()


def test_continuous_admission_and_budget():
    X, c, m, b = case(6, 1e6, 0.3, 0.1, 3)
    probe = msx.Pool(max_slots=4, precision=msx.MIXED)
    probe.submit(X, c, m, b, 2)
    one = probe.stats()["used_bytes"]
    probe.close()
    # a budget that fits two solves of this size but not three
    P = msx.Pool(max_slots=64, precision=msx.MIXED, hbm_budget_bytes=int(2.5 * one), steps_per_launch=4)
    admitted, waiting, done, got = [], list(range(6)), {}, {}
    while waiting or admitted:
        while waiting:
            t = P.submit(X, c, m, b, 30 + 4 * waiting[0])
            if t is None:
                break
            admitted.append((t, 30 + 4 * waiting.pop(0)))
        assert len(admitted) <= 2
        P.step()
        for r in P.poll():
            done[r["ticket"]] = r
            if waiting and len(admitted) == 2:
                # a finished solve holds its HBM until it is fetched
                assert P.submit(X, c, m, b, 1) is None
            got[r["ticket"]] = P.fetch(r["ticket"])[0]
            admitted = [(tt, s) for tt, s in admitted if tt != r["ticket"]]
    assert len(done) == 6 and all(r["status"] == 0 for r in done.values())
    ref = {s: alone(X, c, m, b, s, msx.MIXED)[0] for s in {r["steps"] for r in done.values()}}
    for t, r in done.items():
        assert np.array_equal(got[t], ref[r["steps"]])
    P.close()


def test_wait_for_one_ticket():
    """msx_pool_wait steps the pool until one solve is done; the others keep
    their results for poll/fetch, and every result equals the solve alone."""
    cases = [case(n, 1e6, 0.3, 0.05, s) for s, n in enumerate((4, 6, 5))]
    steps = [40, 90, 60]
    P = msx.Pool(max_slots=4, precision=msx.MIXED, steps_per_launch=8)
    tickets = [P.submit(X, c, m, b, st) for (X, c, m, b), st in zip(cases, steps)]
    r = P.wait(tickets[1])
    assert r["ticket"] == tickets[1] and r["status"] == 0 and r["steps"] == 90
    u1 = P.fetch(tickets[1])[0]
    done = {}
    for _ in range(50):
        for q in P.poll():
            done[q["ticket"]] = q
        if tickets[0] in done and tickets[2] in done:
            break
        P.step()
    assert tickets[0] in done and tickets[2] in done
    for t, (X, c, m, b), st in zip(tickets, cases, steps):
        u = u1 if t == tickets[1] else P.fetch(t)[0]
        assert np.array_equal(u, alone(X, c, m, b, st, msx.MIXED)[0])
    with pytest.raises(msx.MsxError):
        P.wait(tickets[1])   # already fetched
    P.close()


@pytest.mark.parametrize("precision", [msx.MIXED, msx.DOUBLE_WORD])
def test_serving_mode_concurrent_admission(precision):
    """Serving mode: the library's thread steps the pool while two host threads
    admit solves, one of them staggered so its admissions land while replays
    run.  Every result equals the solve alone; msx_pool_step is refused while
    serving; msx_pool_wait blocks on the serving thread; after serving is
    turned off the pool is stepped by hand again."""
    import threading
    import time
    rng = np.random.default_rng(23)
    cases = [case(int(n), float(E), float(nu), float(v), 40 + s)
             for s, (n, E, nu, v) in enumerate(zip(rng.integers(3, 10, 10), 10 ** rng.uniform(5, 7, 10),
                                                   rng.uniform(0.25, 0.45, 10), rng.uniform(0.01, 0.2, 10)))]
    steps = [int(x) for x in rng.integers(30, 160, len(cases))]
    P = msx.Pool(max_slots=6, precision=precision, steps_per_launch=4)
    P.serve(True)
    P.serve(True)   # already serving: no second thread
    with pytest.raises(msx.MsxError):
        P.step(4)
    tickets = {}
    lock = threading.Lock()

    def client(ks, pause):
        for k in ks:
            X, c, m, b = cases[k]
            while True:
                t = P.submit(X, c, m, b, steps[k])
                if t is not None:
                    break
                time.sleep(0.002)   # slots full: the serving thread frees them
            with lock:
                tickets[t] = k
            time.sleep(pause)

    th = [threading.Thread(target=client, args=(list(range(0, 10, 2)), 0.01)),
          threading.Thread(target=client, args=(list(range(1, 10, 2)), 0.0))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    done = {}
    first = next(iter(tickets))
    r = P.wait(first)
    assert r["ticket"] == first and r["status"] == 0
    done[first] = r
    deadline = time.time() + 120
    while len(done) < len(cases) and time.time() < deadline:
        for q in P.poll():
            done[q["ticket"]] = q
        time.sleep(0.001)
    assert len(done) == len(cases)
    for t, q in done.items():
        k = tickets[t]
        assert q["status"] == 0 and q["steps"] == steps[k]
        ua, va, aa = alone(*cases[k], steps[k], precision)
        u, v, a = P.fetch(t)
        assert np.array_equal(u, ua) and np.array_equal(v, va) and np.array_equal(a, aa)
    P.serve(False)
    X, c, m, b = cases[0]
    t = P.submit(X, c, m, b, 17)
    for _ in range(10):
        P.step()
    got = {q["ticket"]: q for q in P.poll()}
    assert got[t]["steps"] == 17
    assert np.array_equal(P.fetch(t)[0], alone(X, c, m, b, 17, precision)[0])
    P.close()


def collapsed_case(seed):
    """A cube with one element flattened to zero volume: its CFL length is 0,
    so the solve's first step stops with dt < 1e-20 ("Negative jacobian",
    solverExplicit.cpp:270-273), status 3."""
    X, c, m, b = case(3, 1e6, 0.3, 0.1, seed)
    X = X.copy()
    X[:, c[5][3]] = X[:, c[5][0]]
    return X, c, m, b


def nan_case(seed):
    """A cube whose input puts a NaN into u[1] (an instantaneous Dirichlet
    entry of value NaN on DOF 1): the NaN check of solverExplicit.cpp:306-308
    stops it with status 4."""
    X, c, m, b = case(4, 1e6, 0.3, 0.1, seed)
    return X, c, m, b + [(1, msx.BC_INST, float("nan"), 0)]


@pytest.mark.parametrize("precision", [msx.MIXED, msx.FP64, msx.DOUBLE_WORD])
def test_failed_solves_leave_the_others_unchanged(precision):
    """Solves that fail inside the pool report their own status and leave it;
    the healthy solves stepped in the same replays equal their runs alone bit
    for bit (failure isolation: no state is shared between solves)."""
    healthy = [case(4, 1e6, 0.3, 0.1, 1), case(5, 3e6, 0.4, 0.05, 2), case(3, 2e5, 0.25, 0.2, 3)]
    steps = [60, 45, 70]
    P = msx.Pool(max_slots=8, precision=precision, steps_per_launch=4)
    tb = P.submit(*collapsed_case(4), 50)
    tickets = [P.submit(X, c, m, b, st) for (X, c, m, b), st in zip(healthy, steps)]
    tn = P.submit(*nan_case(5), 50)
    assert None not in tickets + [tb, tn]
    for _ in range(40):
        P.step()
    res = {r["ticket"]: r for r in P.poll()}
    assert set(res) == set(tickets + [tb, tn])
    assert res[tb]["status"] == 3 and res[tb]["steps"] == 0
    assert res[tn]["status"] == 4 and 1 <= res[tn]["steps"] <= 2
    for t in (tb, tn):
        P.fetch(t)          # a failed solve's memory is released like any other
    for t, (X, c, m, b), st in zip(tickets, healthy, steps):
        assert res[t]["status"] == 0 and res[t]["steps"] == st
        got = P.fetch(t)
        ref = alone(X, c, m, b, st, precision)
        assert all(np.array_equal(x, y) for x, y in zip(got, ref))
    assert P.stats()["used_bytes"] == 0
    P.close()


def test_admission_allocation_failure_leaves_the_pool_intact():
    """An admission whose device allocation fails (injected on the host, as
    cudaMallocAsync running out of memory) returns MSX_ERR_OOM and releases
    its reservation; the resident solves run on unchanged, and the next
    admission succeeds."""
    A, B, Cc = case(5, 1e6, 0.3, 0.1, 7), case(4, 2e6, 0.35, 0.08, 8), case(3, 5e5, 0.3, 0.15, 9)
    P = msx.Pool(max_slots=4, precision=msx.MIXED, steps_per_launch=4)
    ta, tb = P.submit(*A, 120), P.submit(*B, 90)
    P.step(8)
    before = P.stats()
    P.inject_alloc_failures(1)
    with pytest.raises(msx.MsxError) as ei:
        P.submit(*Cc, 50)
    assert ei.value.status == 5 and b"injected" in msx.load().msx_last_error()
    after = P.stats()
    assert after["used_bytes"] == before["used_bytes"] and after["active"] == 2
    tc = P.submit(*Cc, 50)
    assert tc is not None
    out = {}
    for t in (ta, tb, tc):
        r = P.wait(t)
        assert r["status"] == 0
        out[t] = P.fetch(t)
    P.close()
    for t, (X, c, m, b), st in ((ta, A, 120), (tb, B, 90), (tc, Cc, 50)):
        ref = alone(X, c, m, b, st, msx.MIXED)
        assert all(np.array_equal(x, y) for x, y in zip(out[t], ref))


def test_concurrent_serving_stop_joins_once():
    """Two threads turning serving off at the same time: one joins the
    library's serving thread, the other waits for it; both return OK and the
    pool is stepped by msx_pool_step afterwards."""
    import threading
    X, c, m, b = case(4, 1e6, 0.3, 0.1, 12)
    P = msx.Pool(max_slots=2, precision=msx.MIXED, steps_per_launch=4)
    P.serve(True)
    t = P.submit(X, c, m, b, 400)
    errs = []

    def stop():
        try:
            P.serve(False)
        except Exception as e:   # noqa: BLE001
            errs.append(e)

    th = [threading.Thread(target=stop) for _ in range(2)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errs
    r = P.wait(t)
    assert r["status"] == 0 and r["steps"] == 400
    u = P.fetch(t)[0]
    P.close()
    assert np.array_equal(u, alone(X, c, m, b, 400, msx.MIXED)[0])
