"""The two rewrites of the element set-up and lumped-mass kernels that keep the
reference's bits with fewer FP64 operations, checked in IEEE double arithmetic
(numpy: one rounding per operation, no contraction) on random inputs that
include signed zeros, cancellations, subnormals and huge values.

- Jacobian entry of the linear tet (classLinearTetrahedra.cpp:171-268): the
  corner-order sum 0 + sum_k x_k natDev_kj with natDev's -1/0/1 entries equals
  (0 - x_0) + x_(j+1) for finite x.
- Lumped mass term (constitutiveAlgorithms.cpp:191-205): 0 + z + z + z + z
  equals (3 z) + z.
"""
import numpy as np

NAT_DEV = np.array([[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


def sample(rng, n):
    x = rng.standard_normal(n) * np.exp2(rng.integers(-60, 60, n).astype(float))
    kind = rng.integers(0, 6, n)
    x[kind == 0] = 0.0
    x[kind == 1] = -0.0
    x[kind == 2] = rng.integers(-2, 3, int((kind == 2).sum())).astype(float)
    x[kind == 3] = rng.standard_normal(int((kind == 3).sum())) * 5e-324 * 1e3
    return x


def bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def test_jacobian_entry_rewrite_keeps_bits():
    rng = np.random.default_rng(11)
    n = 1 << 20
    x = np.stack([sample(rng, n) for _ in range(4)])
    # equal and opposite corners, so that the sum cancels to zero
    pick = rng.integers(1, 4, n)
    same, opp = rng.random(n) < 0.2, rng.random(n) < 0.2
    x[pick[same], np.nonzero(same)[0]] = x[0, same]
    x[pick[opp], np.nonzero(opp)[0]] = -x[0, opp]
    with np.errstate(all="ignore"):
        for j in range(3):
            c = np.zeros(n)
            for k in range(4):
                c = c + x[k] * NAT_DEV[k, j]
            d = (0.0 - x[0]) + x[j + 1]
            assert np.array_equal(bits(c), bits(d)), j


def test_lumped_mass_sum_rewrite_keeps_bits():
    rng = np.random.default_rng(12)
    n = 1 << 20
    w = np.abs(sample(rng, n))
    rho = np.abs(sample(rng, n)) + 1e-300
    phi = -1.0 * 0.25 - 1.0 * 0.25 - 1.0 * 0.25 + 1.0
    with np.errstate(all="ignore"):
        z = w * rho * phi * phi
        me = np.zeros(n)
        for _ in range(4):
            me = me + z
        m0 = np.abs(sample(rng, n))
        ref = m0 + me
        new = m0 + ((3.0 * z) + z)
    ok = np.isfinite(ref)
    assert np.array_equal(bits(ref[ok]), bits(new[ok]))
    assert np.array_equal(np.isfinite(new), ok)
