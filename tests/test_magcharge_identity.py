"""The identity behind the device's magnetic charge (no GPU): the argument of
the trace of the product of four projected links Pi(x) U Pi(x+mu) around a
plaquette, Pi = (1 + n.sigma)/2 (magfield.c:120-216, as the reference forms
it), equals the argument of z1 z2 conj(z3) conj(z4) with z = <n_a| U |n_b>,
for either chart of each site's spinor (the device takes the chart away from
the pole opposite to Sigma), and the cube's charge from 12 edge overlaps
equals the sum of its six face angles computed separately."""
import numpy as np


def su2(q):
    a, b, c, d = q
    return np.array([[a + 1j * d, c + 1j * b], [-c + 1j * b, a - 1j * d]])


def projector(s):
    n = s / np.linalg.norm(s)
    return np.array([[(1 + n[2]) / 2, (n[0] - 1j * n[1]) / 2], [(n[0] + 1j * n[1]) / 2, (1 - n[2]) / 2]])


def spinor(s, chart=None):
    m = np.linalg.norm(s)
    north = s[2] >= 0 if chart is None else chart
    if north:
        return np.array([m + s[2], s[0] + 1j * s[1]]) / np.sqrt(2 * m * (m + s[2]))
    return np.array([s[0] - 1j * s[1], m - s[2]]) / np.sqrt(2 * m * (m - s[2]))


def overlap(sa, q, sb):
    return np.conj(sa) @ (su2(q) @ sb)


def test_plaquette_angle_from_overlaps():
    rng = np.random.default_rng(7)
    worst = 0.0
    for t in range(500):
        qs = [q / np.linalg.norm(q) for q in rng.normal(size=(4, 4))]
        ss = list(rng.normal(size=(4, 3)))  # x, x+1, x+2, x+12
        px = [projector(s) for s in ss]
        u1 = px[0] @ su2(qs[0]) @ px[1]
        u2 = px[1] @ su2(qs[1]) @ px[3]
        u3 = px[2] @ su2(qs[2]) @ px[3]
        u4 = px[0] @ su2(qs[3]) @ px[2]
        ref = np.angle(np.trace(u1 @ u2 @ u3.conj().T @ u4.conj().T))
        for charts in (None, (True, False, True, False), (False, False, False, False)):
            sp = [spinor(s, None if charts is None else charts[k]) for k, s in enumerate(ss)]
            z = (overlap(sp[0], qs[0], sp[1]) * overlap(sp[1], qs[1], sp[3]) *
                 np.conj(overlap(sp[2], qs[2], sp[3])) * np.conj(overlap(sp[0], qs[3], sp[2])))
            d = abs((np.angle(z) - ref + np.pi) % (2 * np.pi) - np.pi)
            worst = max(worst, d)
    assert worst < 1e-12


def test_spinor_is_the_plus_one_eigenvector():
    rng = np.random.default_rng(8)
    sig = [np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.array([[1, 0], [0, -1]])]
    for s in rng.normal(size=(200, 3)):
        n = s / np.linalg.norm(s)
        ns = sum(n[k] * sig[k] for k in range(3))
        for chart in (True, False):
            v = spinor(s, chart)
            assert np.allclose(ns @ v, v) and abs(np.vdot(v, v) - 1) < 1e-12
            assert np.allclose(np.outer(v, np.conj(v)), projector(s))


def test_cube_charge_from_edges_equals_face_sum():
    rng = np.random.default_rng(9)
    L = 4
    trip = rng.normal(size=(L, L, L, 3))
    links = rng.normal(size=(L, L, L, 3, 4))
    links /= np.linalg.norm(links, axis=-1, keepdims=True)

    def sh(x, d):
        y = list(x)
        y[d] = (y[d] + 1) % L
        return tuple(y)

    def z(y, mu):
        return overlap(spinor(trip[y]), links[y][mu], spinor(trip[sh(y, mu)]))

    def alpha(y, d1, d2):
        return np.angle(z(y, d1) * z(sh(y, d1), d2) * np.conj(z(sh(y, d2), d1)) * np.conj(z(y, d2)))

    def fa(a, b, c, d):
        return np.angle(a * b * np.conj(c) * np.conj(d))

    charges = 0
    for x in np.ndindex(L, L, L):
        q = (alpha(sh(x, 0), 1, 2) - alpha(x, 1, 2) - alpha(sh(x, 1), 0, 2) + alpha(x, 0, 2)
             + alpha(sh(x, 2), 0, 1) - alpha(x, 0, 1))
        x0, x1, x2 = sh(x, 0), sh(x, 1), sh(x, 2)
        X0, X1, X2 = z(x, 0), z(x, 1), z(x, 2)
        A1, A2, B0, B2, E0, E1 = z(x0, 1), z(x0, 2), z(x1, 0), z(x1, 2), z(x2, 0), z(x2, 1)
        F2, G1, H0 = z(sh(x0, 1), 2), z(sh(x0, 2), 1), z(sh(x1, 2), 0)
        qc = (fa(A1, F2, G1, A2) - fa(X1, B2, E1, X2) - fa(B0, F2, H0, B2) + fa(X0, A2, E0, X2)
              + fa(E0, G1, H0, E1) - fa(X0, A1, B0, X1))
        assert abs(q - qc) < 1e-12
        # a charge is a multiple of 2 pi
        assert abs(q / (2 * np.pi) - round(q / (2 * np.pi))) < 1e-9
        charges += abs(round(q / (2 * np.pi)))
    assert charges > 0  # random fields carry monopoles: the test is not vacuous
