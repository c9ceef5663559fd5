"""The identities the hand-written adjoint kernel (csrc/adjoint.cu) relies on, checked in FP64
numpy on the D3Q19 set of the package (no GPU): the reverse of the collision contracts the ten
weighted moments of lam* (sum w lam times 1, e_a, e_a e_b) instead of running 19-term loops, and
the forward recomputation works on the stored deviations h = f - w rho0 without forming f or
f - f_eq.  Random inputs, each form against the per-direction loop it replaced."""
import numpy as np

from pour_over_coffee_lbm_gb300.solver import CX, CY, CZ, OPPOSITE, WEIGHTS

E = np.stack([CX, CY, CZ], axis=1).astype(np.float64)
W = WEIGHTS


def _moments(a):
    m = W * a
    return m.sum(), E.T @ m, np.einsum("q,qa,qb->ab", m, E, E)


def test_lattice_moments():
    # the isotropy the contractions use: sum w e e = I / 3, sum w e_a^4 = 1/3, sum w e_a^2 e_b^2 = 1/9
    assert np.allclose(np.einsum("q,qa,qb->ab", W, E, E), np.eye(3) / 3)
    assert np.allclose((W[:, None] * E ** 4).sum(0), 1 / 3)
    assert np.isclose((W * E[:, 0] ** 2 * E[:, 1] ** 2).sum(), 1 / 9)
    assert np.array_equal(E[OPPOSITE], -E)


def test_reverse_collision_through_moments():
    rng = np.random.default_rng(1)
    for _ in range(20):
        lam = rng.normal(size=19)
        u = rng.normal(size=3) * 0.05
        F = rng.normal(size=3) * 1e-4
        rho = 1 + rng.normal() * 1e-3
        omega = 1 / rng.uniform(0.55, 1.5)
        A = 1 - 0.5 * omega
        uF = u @ F
        P = rng.normal(size=6)  # bar P_xx, yy, zz (diagonal) and xy, xz, yz (coefficients of e_a e_b)
        # the 19-term loops
        bneq = (1 - omega) * lam
        bA, bF, bu = 0.0, np.zeros(3), np.zeros(3)
        for q in range(19):
            e = E[q]
            eu, eF = e @ u, e @ F
            bA += lam[q] * W[q] * (3 * (eF - uF) + 9 * eu * eF)
            bB = lam[q] * A * W[q]
            bF += bB * (3 * (e - u) + 9 * eu * e)
            bu += bB * (-3 * F + 9 * eF * e)
            bneq[q] += e[0] ** 2 * P[0] + e[1] ** 2 * P[1] + e[2] ** 2 * P[2] + e[0] * e[1] * P[3] + \
                e[0] * e[2] * P[4] + e[1] * e[2] * P[5]
        usq = u @ u
        br, bx = 0.0, np.zeros(3)
        for q in range(19):
            e = E[q]
            eu = e @ u
            wl = W[q] * (lam[q] - bneq[q])
            br += wl * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * usq)
            bx += wl * rho * (3 + 9 * eu) * e - wl * rho * 3 * u
        # the moment forms
        L0, L1, L2 = _moments(lam)
        assert np.isclose(bA, 3 * (F @ L1 - uF * L0) + 9 * u @ L2 @ F, rtol=1e-10, atol=1e-14)
        assert np.allclose(bF, A * (3 * (L1 - u * L0) + 9 * L2 @ u), rtol=1e-10, atol=1e-14)
        assert np.allclose(bu, A * (-3 * F * L0 + 9 * L2 @ F), rtol=1e-10, atol=1e-14)
        third, ninth = 1 / 3, 1 / 9
        D0 = omega * L0 - third * (P[0] + P[1] + P[2])
        D1 = omega * L1
        D2 = omega * L2 - np.array([[third * P[0] + ninth * (P[1] + P[2]), ninth * P[3], ninth * P[4]],
                                    [ninth * P[3], third * P[1] + ninth * (P[0] + P[2]), ninth * P[5]],
                                    [ninth * P[4], ninth * P[5], third * P[2] + ninth * (P[0] + P[1])]])
        assert np.isclose(br, D0 * (1 - 1.5 * usq) + 3 * u @ D1 + 4.5 * u @ D2 @ u, rtol=1e-10, atol=1e-14)
        assert np.allclose(bx, rho * (3 * D1 + 9 * D2 @ u - 3 * u * D0), rtol=1e-10, atol=1e-14)


def test_forward_recomputation_on_deviations():
    rng = np.random.default_rng(2)
    rho0 = 1.0
    for _ in range(20):
        h = rng.normal(size=19) * 1e-3
        f = h + W * rho0
        lam = rng.normal(size=19)
        rho, drho = f.sum(), h.sum()
        assert np.isclose(rho - rho0, drho, rtol=0, atol=1e-15)
        assert np.allclose(E.T @ f, E.T @ h, rtol=0, atol=1e-15)
        u = rng.normal(size=3) * 0.05
        usq = u @ u
        feq = W * rho * (1 + 3 * (E @ u) + 4.5 * (E @ u) ** 2 - 1.5 * usq)
        neq = f - feq
        Pi = np.einsum("q,qa,qb->ab", neq, E, E)
        S = np.einsum("q,qa,qb->ab", h, E, E)
        assert np.allclose(Pi, S - drho / 3 * np.eye(3) - rho * np.outer(u, u), rtol=1e-9, atol=1e-14)
        L0, L1, L2 = _moments(lam)
        bomega = -(lam * neq).sum()
        assert np.isclose(bomega, -(lam * h).sum() + L0 * (drho - 1.5 * rho * usq) +
                          rho * (3 * u @ L1 + 4.5 * u @ L2 @ u), rtol=1e-9, atol=1e-14)
