"""The MRG32k3a jump-ahead of the path-start cursor (mrg_jump): matrix
powers of the two component recurrences (L'Ecuyer 1999) against stepping the
recurrences one by one in Python integers."""
import numpy as np

from oracle import oracle

M1, M2 = 4294967087, 4294944443


def step(s1, s2):
    """One step of both components, states oldest value first."""
    p1 = (1403580 * s1[1] - 810728 * s1[0]) % M1
    p2 = (527612 * s2[2] - 1370589 * s2[0]) % M2
    return [s1[1], s1[2], p1], [s2[1], s2[2], p2]


def test_jump_matches_stepping():
    rng = np.random.default_rng(3)
    for steps in (0, 1, 2, 3, 5, 24, 27, 192, 3 * 1024):
        s1 = [int(x) for x in rng.integers(1, M1, 3)]
        s2 = [int(x) for x in rng.integers(1, M2, 3)]
        a, b = list(s1), list(s2)
        for _ in range(steps):
            a, b = step(a, b)
        j1, j2 = oracle.mrg_jump(steps, s1, s2)
        assert [int(x) for x in j1] == a, steps
        assert [int(x) for x in j2] == b, steps


def test_jump_extreme_states():
    """States at the top of each modulus exercise every reduction branch."""
    for s1, s2 in (([M1 - 1] * 3, [M2 - 1] * 3), ([0, 0, 1], [1, 0, 0]), ([M1 - 1, 0, M1 - 1], [0, M2 - 1, 0])):
        a, b = list(s1), list(s2)
        for _ in range(24):
            a, b = step(a, b)
        j1, j2 = oracle.mrg_jump(24, s1, s2)
        assert [int(x) for x in j1] == a
        assert [int(x) for x in j2] == b
