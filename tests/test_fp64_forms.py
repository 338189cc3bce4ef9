"""The plain FP64 element kernel's two forms of the compressible neo-Hookean
corner forces agree (numpy restatement, FP64, random tets of both
orientations under small and moderate strain):

- cofactor form: F = I + sum_b du_b g_b^T, P = mu F + (lambda ln J - mu) F^-T,
  f_a = wJ P g_a (hyperElasticNeoHookean.cpp:235-259 for the law);
- F-free form: e_b = E_b + du_b, F g_a = sum_b M_ab e_b with M = G G^T,
  F^-T g_a = (e_c x e_d) / det e, J = det e / det E,
  f_a = wJ mu F g_a + wJ (lambda ln J - mu) (e_c x e_d) / det e.

Both cancel mu F against mu F^-T at small strain, so they agree to the rounding
of that cancellation: about 2.5e-16 / strain relative to the corner forces
(the reference's own cofactor-free order carries the same), far below the FP64
mode's bar on the displacements.
"""
import numpy as np


def forms(n, strain, seed):
    rng = np.random.default_rng(seed)
    E = np.eye(3)[None] * 0.01 + rng.standard_normal((n, 3, 3)) * 0.002      # E[:, b, i]: edge b
    flip = rng.random(n) < 0.5
    E[flip] = E[flip][:, [1, 0, 2], :]
    du = rng.standard_normal((n, 3, 3)) * 0.01 * strain
    mu, lam = 3.8e5, 5.7e5
    Jac = np.transpose(E, (0, 2, 1))             # columns are the edges
    G = np.linalg.inv(Jac)                        # rows g_1..g_3
    wJ = np.abs(np.linalg.det(Jac)) / 6
    F = np.eye(3)[None] + np.einsum("nbi,nbj->nij", du, G)
    J = np.linalg.det(F)
    P = mu * F + (lam * np.log(J) - mu)[:, None, None] * np.transpose(np.linalg.inv(F), (0, 2, 1))
    f_cof = wJ[:, None, None] * np.einsum("nij,naj->nai", P, G)
    e = E + du
    M = np.einsum("naj,nbj->nab", G, G)
    cr = np.stack([np.cross(e[:, 1], e[:, 2]), np.cross(e[:, 2], e[:, 0]), np.cross(e[:, 0], e[:, 1])], axis=1)
    det_e = np.einsum("ni,ni->n", e[:, 0], cr[:, 0])
    Jn = det_e / np.linalg.det(Jac)
    f_free = (mu * wJ)[:, None, None] * np.einsum("nab,nbi->nai", M, e) + \
        ((lam * np.log(Jn) - mu) * wJ / det_e)[:, None, None] * cr
    return J, Jn, f_cof, f_free


def test_f_free_corner_forces_match_the_cofactor_form():
    for strain, seed in ((1e-4, 1), (1e-2, 2), (1e-1, 3)):
        J, Jn, f_cof, f_free = forms(20000, strain, seed)
        ok = (J > 0.5) & (Jn > 0.5)
        assert ok.mean() > 0.99
        assert np.max(np.abs(Jn[ok] - J[ok]) / J[ok]) < 1e-12
        rel = np.abs(f_free - f_cof).max(axis=(1, 2))[ok] / np.abs(f_cof).max(axis=(1, 2))[ok]
        assert np.median(rel) < 2e-15 / strain, (strain, np.median(rel))
        assert rel.max() < 1e-13 / strain, (strain, rel.max())
