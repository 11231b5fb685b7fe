"""The exact-predicate extension (RPD_PRED_EXACT) in the oracle: the FP64
determinant's error bound and the exact sign by floating-point expansions,
both against exact rational arithmetic (fractions) on the same float
planes."""
from fractions import Fraction

import numpy as np

from oracle import oracle as O


def exact_det(p1, p2, p3, e):
    m = [[Fraction(float(c)) for c in (p1[r], p2[r], p3[r], e[r])] for r in range(4)]

    def det(a):
        if len(a) == 1:
            return a[0][0]
        return sum((-1) ** j * a[0][j] * det([row[:j] + row[j + 1:] for row in a[1:]])
                   for j in range(len(a)))

    return det(m)


def sgn(x):
    return (x > 0) - (x < 0)


def cases(rng, n):
    out = []
    for i in range(n):
        p = (rng.normal(0, 1, (3, 4)) * 10.0 ** rng.integers(-2, 4, (3, 1))).astype(np.float32)
        kind = i % 4
        if kind == 0:      # generic
            e = (rng.normal(0, 1, 4) * 100.0).astype(np.float32)
        elif kind == 1:    # exactly dependent: e = p1 (duplicate) scaled by 2
            e = (p[0] * np.float32(2.0)).astype(np.float32)
        elif kind == 2:    # nearly dependent: sum of two planes, rounded
            e = (p[0] + p[1]).astype(np.float32)
        else:              # dependent with tiny perturbation of one coefficient
            e = (p[0] - p[2]).astype(np.float32)
            e[rng.integers(0, 4)] = np.nextafter(e[rng.integers(0, 4)], np.float32(np.inf))
        out.append((p[0], p[1], p[2], e))
    return out


def test_exact_sign_matches_rationals():
    rng = np.random.default_rng(5)
    for p1, p2, p3, e in cases(rng, 400):
        assert O.det4x4_exact_sign(p1, p2, p3, e) == sgn(exact_det(p1, p2, p3, e))


def test_fp64_error_bound_holds_and_flags_wrong_signs():
    rng = np.random.default_rng(6)
    wrong = flagged = 0
    for p1, p2, p3, e in cases(rng, 400):
        d, bound = O.det4x4_bound(p1, p2, p3, e)
        x = exact_det(p1, p2, p3, e)
        assert abs(Fraction(d) - x) <= Fraction(bound)
        if sgn(d) != sgn(x):
            wrong += 1
            assert abs(d) <= bound  # a wrong FP64 sign is never certified
        flagged += abs(d) <= bound
    assert flagged >= wrong


def test_exact_mode_equals_fp64_on_generic_input(golden_cases):
    from tests.helpers import compare_cells, mesh_of

    for name, c in golden_cases.items():
        h0, p0, s0 = O.clip_cells(mesh_of(c), c["sites"], c["nbr"], c["tet_offsets"],
                                  c["pair_sites"], pred_mode=0)
        h2, p2, s2 = O.clip_cells(mesh_of(c), c["sites"], c["nbr"], c["tet_offsets"],
                                  c["pair_sites"], pred_mode=2)
        if s2[3] == 0:  # no FP64 sign was wrong: identical cells
            assert compare_cells(h0, p0, h2, p2) == 0, name
