"""FP64 oracle of libmat's dist2mat (test infrastructure only).

Restates ClosestDistanceToLocalMat (src/dist2mat/dist2mat.cu:195-270) and its
distance formulas (:5-193) in float64: the signed distance |p - c| - r to a
sphere, to a cone (two spheres linearly interpolated, stationary point of
the distance along the axis, clamped to [0, 1]) and to a slab (three spheres
interpolated barycentrically: the interior stationary point by the
reference's case analysis on the radius differences, else the nearest of the
three edge cones); the closest-primitive index as the reference's 32-thread
block chooses it (lane j scans primitives j, j + 32, ... keeping the first
smallest; the last lane whose smallest distance is within 1e-10 of the
minimum wins).

With dtype=np.float32 the same expressions are evaluated in float32, one
rounding per operation, widening to float64 exactly where the reference's
source does (its double literals), so that the device's float results can be
compared closely where the closed forms are ill-conditioned.

`numeric_*` are an independent check of the closed forms: the distance to a
cone or a slab is a convex function of the interpolation parameters (the norm
of an affine map minus an affine map), minimised here by nested golden-section
search.
"""
import math

import numpy as np

BIG = 1e16


def sphere_d(p, s):
    q = p - s[:3]
    return np.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]) - s[3]


def _sq(x):
    """The reference's powf(x, 2.f): the square rounded once (glibc's powf
    and the device's restatement agree on it; numpy's float32 ** 2 does not
    always)."""
    return x * x


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _bary(m1, m2, m3, t1, t2):
    return m1 * t1 + m2 * t2 + m3 * (1.0 - t1 - t2)


def _roots(A, B, C):
    if A == 0.0:
        return (-C / B, -C / B) if B != 0.0 else (-1.0, -1.0)
    delta = B * B - 4.0 * A * C
    if delta < 0.0:
        return (-1.0, -1.0)
    sq = np.sqrt(delta)
    return ((-B - sq) / (2.0 * A), (-B + sq) / (2.0 * A))


def cone_d(p, m1, m2):
    if m1[3] > m2[3]:
        m1, m2 = m2, m1
    c21 = m1[:3] - m2[:3]
    cq2 = m2[:3] - p
    A = _dot(c21, c21)
    D = 2.0 * _dot(c21, cq2)
    F = _dot(cq2, cq2)
    R1 = m1[3] - m2[3]
    f = type(A)
    # in double as the reference's source (4.0 is a double literal)
    arg = (np.float64(D * D) - 4.0 * np.float64(A) * np.float64(F)) * np.float64(R1 * R1 - A) \
        * np.float64(R1) * np.float64(R1)
    with np.errstate(invalid="ignore", divide="ignore"):
        root = np.sqrt(f(arg))  # NaN for a (rounded) negative argument, as sqrtf
        t = (-(A * D - R1 * R1 * D) - root) / (2.0 * (A * A - A * R1 * R1))
    t = np.fmax(f(0.0), np.fmin(t, f(1.0)))  # clamp: fminf / fmaxf ignore a NaN
    # the reference's lerp(a, b, t) is b + t (a - b) (include/cuda_helper_math.h:911-925):
    # t runs from m2 (t = 0) to m1
    s = m2 + t * (m1 - m2)
    return sphere_d(p, s)


def _pick(p, m1, m2, m3, a, b):
    da = sphere_d(p, _bary(m1, m2, m3, *a))
    db = sphere_d(p, _bary(m1, m2, m3, *b))
    return b if db < da else a


def slab_d(p, m1, m2, m3):
    c31, c32, cm3 = m1[:3] - m3[:3], m2[:3] - m3[:3], m3[:3] - p
    R1, R2 = m1[3] - m3[3], m2[3] - m3[3]
    A, B, C = _dot(c31, c31), 2.0 * _dot(c31, c32), _dot(c32, c32)
    D, E, F = 2.0 * _dot(c31, cm3), 2.0 * _dot(c32, cm3), _dot(cm3, cm3)
    t1 = t2 = -1.0
    if R1 == 0.0 and R2 == 0.0:
        den = 4.0 * A * C - B * B
        f = type(A)
        t1 = f((np.float64(B * E) - 2.0 * np.float64(C) * np.float64(D)) / np.float64(den))
        t2 = f((np.float64(B * D) - 2.0 * np.float64(A) * np.float64(E)) / np.float64(den))
    elif R1 != 0.0 and R2 == 0.0:
        H2, K2 = -B / (2.0 * C), -E / (2.0 * C)
        W1 = _sq(2.0 * A + B * H2) - 4.0 * R1 * R1 * (A + B * H2 + C * H2 * H2)
        W2 = 2.0 * (2.0 * A + B * H2) * (B * K2 + D) - 4.0 * R1 * R1 * (B * K2 + 2.0 * C * H2 * K2 + D + E * H2)
        W3 = _sq(B * K2 + D) - 4.0 * R1 * R1 * (C * K2 * K2 + E * K2 + F)
        r = _roots(W1, W2, W3)
        t1, t2 = _pick(p, m1, m2, m3, (r[0], H2 * r[0] + K2), (r[1], H2 * r[1] + K2))
    elif R1 == 0.0 and R2 != 0.0:
        H1, K1 = -B / (2.0 * A), -D / (2.0 * A)
        W1 = _sq(2.0 * C + B * H1) - 4.0 * R2 * R2 * (C + B * H1 + A * H1 * H1)
        W2 = 2.0 * (2.0 * C + B * H1) * (B * K1 + E) - 4.0 * R2 * R2 * (B * K1 + 2.0 * A * H1 * K1 + E + D * H1)
        W3 = _sq(B * K1 + E) - 4.0 * R2 * R2 * (A * K1 * K1 + D * K1 + F)
        r = _roots(W1, W2, W3)
        t1, t2 = _pick(p, m1, m2, m3, (H1 * r[0] + K1, r[0]), (H1 * r[1] + K1, r[1]))
    else:
        L1, L2, L3 = 2.0 * A * R2 - B * R1, 2.0 * C * R1 - B * R2, E * R1 - D * R2
        if L1 == 0.0 and L2 != 0.0:
            t2 = -L3 / L2
            W1 = 4.0 * A * A - 4.0 * R1 * R1 * A
            W2 = 4.0 * A * (B * t2 + D) - 4.0 * R1 * R1 * (B * t2 + D)
            W3 = _sq(B * t2 + D) - (C * t2 * t2 + E * t2 + F)
            r = _roots(W1, W2, W3)
            t1, _ = _pick(p, m1, m2, m3, (r[0], t2), (r[1], t2))
        elif L1 != 0.0 and L2 == 0.0:
            t1 = L3 / L1
            W1 = 4.0 * C * C - 4.0 * R2 * R2 * C
            W2 = 4.0 * C * (B * t1 + E) - 4.0 * R2 * R2 * (B * t1 + E)
            W3 = _sq(B * t1 + E) - (A * t1 * t1 + D * t1 + F)
            r = _roots(W1, W2, W3)
            _, t2 = _pick(p, m1, m2, m3, (t1, r[0]), (t1, r[1]))
        else:
            H3, K3 = L2 / L1, L3 / L1
            W1 = _sq(2.0 * C + B * H3) - 4.0 * R2 * R2 * (A * H3 * H3 + B * H3 + C)
            W2 = 2.0 * (2.0 * C + B * H3) * (B * K3 + E) - 4.0 * R2 * R2 * (2.0 * A * H3 * K3 + B * K3 + D * H3 + E)
            W3 = _sq(B * K3 + E) - 4.0 * R2 * R2 * (A * K3 * K3 + D * K3 + F)
            r = _roots(W1, W2, W3)
            t1, t2 = _pick(p, m1, m2, m3, (H3 * r[0] + K3, r[0]), (H3 * r[1] + K3, r[1]))
    if t1 + t2 < 1.0 and 0.0 <= t1 <= 1.0 and 0.0 <= t2 <= 1.0:
        return sphere_d(p, _bary(m1, m2, m3, t1, t2))
    return min(cone_d(p, m1, m3), cone_d(p, m2, m3), cone_d(p, m1, m2))


def prim_d(p, spheres, pr):
    x, y, z = (int(v) for v in pr)
    if x == -1 and y == -1:
        return sphere_d(p, spheres[z])
    if x == -1:
        return cone_d(p, spheres[y], spheres[z])
    return slab_d(p, spheres[x], spheres[y], spheres[z])


def dist2mat(spheres, samples, offsets, counts, prims, dtype=np.float64):
    """(dist, closest, per-sample distance lists); closest chosen as the
    reference's block does on these values."""
    sph = np.asarray(spheres, dtype)
    out_d = np.zeros(len(samples))
    out_i = np.full(len(samples), -1, np.int64)
    all_d = []
    for s, p in enumerate(np.asarray(samples, dtype)):
        o, n = int(offsets[s]), int(counts[s])
        d = np.array([prim_d(p, sph, prims[o + i]) for i in range(n)])
        all_d.append(d)
        best = np.full(32, BIG)
        bid = np.full(32, -1)
        for i in range(n):
            j = i % 32
            if d[i] < best[j]:
                best[j], bid[j] = d[i], i
        m = best.min()
        out_d[s] = m
        for j in range(32):
            if abs(best[j] - m) < 1e-10:
                out_i[s] = bid[j]
    return out_d, out_i, all_d


def _golden(f, a, b, it=80):
    g = (math.sqrt(5.0) - 1.0) / 2.0
    x1, x2 = b - g * (b - a), a + g * (b - a)
    f1, f2 = f(x1), f(x2)
    for _ in range(it):
        if f1 < f2:
            b, x2, f2 = x2, x1, f1
            x1 = b - g * (b - a)
            f1 = f(x1)
        else:
            a, x1, f1 = x1, x2, f2
            x2 = a + g * (b - a)
            f2 = f(x2)
    return min(f1, f2, f(a), f(b))


def numeric_cone_d(p, m1, m2):
    return _golden(lambda t: sphere_d(p, m1 + (m2 - m1) * t), 0.0, 1.0)


def numeric_slab_d(p, m1, m2, m3):
    def inner(t1):
        return _golden(lambda t2: sphere_d(p, _bary(m1, m2, m3, t1, t2)), 0.0, 1.0 - t1, it=60)
    return _golden(inner, 0.0, 1.0, it=60)
