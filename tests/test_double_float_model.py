"""CPU model of the double-float arithmetic the FP32 element kernel uses for the strain's Gram
differences p_a . p_c - q_a . q_c (gbfem_element.cuh: the node pass's float pairs, the edges by
TwoSum, gram_diff). The steps are restated here in numpy float32, each rounding as the device
rounds it (an FMA's exact product error is the float64 product minus the rounded float32 one: a
product of two float32 values is exact in float64). Checked against exact rational arithmetic on
elements rotated by large angles and moved far from the origin with small strains, where a plain
FP32 evaluation loses the strain to cancellation."""

from fractions import Fraction

import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    e = f32(f32(a - f32(s - bb)) + f32(b - bb))
    return s, e


def pair(x):
    """An FP64 value as the node pass stores it: hi = x rounded, lo = the rest rounded."""
    hi = f32(x)
    return hi, f32(x - np.float64(hi))


def edge(xa, x0):
    """x_a - x_0 from float pairs: TwoSum of the hi parts, plus the lo difference, renormalised."""
    s, es = two_sum(xa[0], f32(-x0[0]))
    return two_sum(s, f32(es + f32(xa[1] - x0[1])))


def gram_diff(pa, pc, qg):
    """sum_k pa_k pc_k - qg with pa, pc float pairs per component and qg a float pair."""
    sh, sl = f32(0), f32(0)
    for k in range(3):
        ah, al = pa[k]
        ch, cl = pc[k]
        P = f32(ah * ch)
        e = f32(np.float64(ah) * np.float64(ch) - np.float64(P))  # FMA(ah, ch, -P), exact
        cross = f32(np.float64(ah) * np.float64(cl) + np.float64(f32(al * ch)))  # FMA(ah, cl, al*ch)
        t, et = two_sum(sh, P)
        sh = t
        sl = f32(sl + f32(et + f32(e + cross)))
    d, ed = two_sum(sh, f32(-qg[0]))
    return f32(d + f32(ed + f32(sl - qg[1])))


def rotation(axis, deg):
    k = np.asarray(axis, float) / np.linalg.norm(axis)
    t = np.radians(deg)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * (K @ K)


def test_double_float_gram_difference_keeps_the_strain_under_large_rigid_motion():
    rng = np.random.default_rng(3)
    worst_df, worst_f32 = 0.0, 0.0
    for trial in range(200):
        h = 0.01
        X = rng.uniform(0, h, (4, 3))                       # rest nodes of one element
        R = rotation(rng.normal(size=3), rng.uniform(30, 170))
        offset = rng.uniform(-10, 10, 3)                    # up to 1,000 element sizes away
        strain = 10.0 ** rng.uniform(-6, -2)
        x = (X @ R.T) + offset + rng.normal(0, strain * h, (4, 3))
        results = []
        for a, c in ((1, 1), (1, 2), (2, 3), (3, 3)):
            # exact value from the FP64 positions (the state the node pass reads)
            ex = [Fraction(float(x[a][k])) - Fraction(float(x[0][k])) for k in range(3)]
            ec = [Fraction(float(x[c][k])) - Fraction(float(x[0][k])) for k in range(3)]
            qa = [Fraction(float(X[a][k])) - Fraction(float(X[0][k])) for k in range(3)]
            qc = [Fraction(float(X[c][k])) - Fraction(float(X[0][k])) for k in range(3)]
            exact = sum(ex[k] * ec[k] for k in range(3)) - sum(qa[k] * qc[k] for k in range(3))
            # rest Gram as the host stores it: the FP64 Gram split into a float pair
            qg = pair(float(np.dot(X[a] - X[0], X[c] - X[0])))
            pa = [edge(pair(x[a][k]), pair(x[0][k])) for k in range(3)]
            pc = [edge(pair(x[c][k]), pair(x[0][k])) for k in range(3)]
            got = gram_diff(pa, pc, qg)
            naive = f32(np.dot(f32(x[a] - x[0]), f32(x[c] - x[0])) - f32(np.dot(X[a] - X[0], X[c] - X[0])))
            results.append((float(exact), float(got), float(naive)))
        # Errors relative to the element's strain scale (its largest Gram difference): a single
        # entry can be near zero by chance.
        scale = max(abs(r[0]) for r in results)
        for ex, got, naive in results:
            worst_df = max(worst_df, abs(got - ex) / scale)
            worst_f32 = max(worst_f32, abs(naive - ex) / scale)
    # The float-pair positions carry ~2^-48 relative error (2.8e-14 m at 10 m), against edges of
    # 1 cm strained by as little as 1e-6: up to ~4e-6 of the strain scale at worst (8.4e-7 on these
    # samples). The FP32 rounding of the result itself is 6e-8.
    assert worst_df < 4e-6, worst_df
    # the same quantity in plain FP32 is lost to cancellation at small strains
    assert worst_f32 > 1e-2, worst_f32


def hex_acc(sh, sl, a, b):
    """(sh, sl) += a * b for float pairs, as k_hex_rhs_df accumulates a row (gbfem_hex.cu)."""
    P = f32(a[0] * b[0])
    e = f32(np.float64(a[0]) * np.float64(b[0]) - np.float64(P))                 # FMA(a.hi, b.hi, -P)
    cross = f32(np.float64(a[0]) * np.float64(b[1]) + np.float64(f32(a[1] * b[0])))  # FMA(a.hi, b.lo, a.lo*b.hi)
    t, et = two_sum(sh, P)
    return t, f32(sl + f32(et + f32(e + cross)))


def test_double_float_row_sums_of_the_hexahedron_right_hand_side():
    """A row of K u + m w (81 blocks of 3 terms plus a mass term, values of both signs spanning six
    decades) from float-pair operands, renormalised once a block: within ~2^-44 of the terms'
    absolute sum, as the FP64 pass is within ~2^-52 * sqrt(terms)."""
    rng = np.random.default_rng(11)
    worst = 0.0
    for trial in range(50):
        nblk = 81
        K = rng.normal(size=(nblk, 3)) * 10.0 ** rng.uniform(-3, 3, (nblk, 1))
        u = rng.normal(size=(nblk, 3)) * 1e-3
        m = rng.uniform(0, 1e-2, nblk)
        w = rng.normal(size=nblk) * 1e-2
        sh, sl = f32(0), f32(0)
        exact = Fraction(0)
        absum = 0.0
        for b in range(nblk):
            for j in range(3):
                sh, sl = hex_acc(sh, sl, pair(K[b, j]), pair(u[b, j]))
                exact += Fraction(float(K[b, j])) * Fraction(float(u[b, j]))
                absum += abs(K[b, j] * u[b, j])
            sh, sl = hex_acc(sh, sl, pair(m[b]), pair(w[b]))
            exact += Fraction(float(m[b])) * Fraction(float(w[b]))
            absum += abs(m[b] * w[b])
            sh, sl = two_sum(sh, sl)
        got = np.float64(sh) + np.float64(sl)
        worst = max(worst, abs(got - float(exact)) / absum)
    assert worst < 2.0 ** -44, worst
