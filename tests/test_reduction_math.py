"""CPU restatement of the DOT path's final reduction (k_dot_final in
einsums_gb300/csrc/kernels_fp64.cu with block_sum_compensated from
csrc/common.cuh): Neumaier summation of the partials per thread, then a fixed
shuffle-down tree of TwoSum merges over each warp and over the warp sums.  The
same order of IEEE double operations is replayed here and checked against an
exactly rounded sum (math.fsum) on partials with heavy cancellation."""
import math

import numpy as np
import pytest

NT = 256  # threads of the final block


def neumaier(values):
    s = c = 0.0
    for x in values:
        t = s + x
        c += (s - t) + x if abs(s) >= abs(x) else (x - t) + s
        s = t
    return s, c


def merge(a, ca, b, cb):
    t = a + b
    bb = t - a
    e = (a - (t - bb)) + (b - bb)
    return t, (ca + cb) + e


def warp_tree(s, c):
    """__shfl_down_sync tree: lane i merges lane i + o (its own value when i + o >= 32)."""
    s, c = list(s), list(c)
    o = 16
    while o > 0:
        s2 = [s[i + o] if i + o < 32 else s[i] for i in range(32)]
        c2 = [c[i + o] if i + o < 32 else c[i] for i in range(32)]
        for i in range(32):
            s[i], c[i] = merge(s[i], c[i], s2[i], c2[i])
        o //= 2
    return s[0], c[0]


def dot_final(partials):
    pairs = [neumaier(partials[t::NT]) for t in range(NT)]
    warp_sums = [warp_tree([p[0] for p in pairs[w * 32:(w + 1) * 32]], [p[1] for p in pairs[w * 32:(w + 1) * 32]])
                 for w in range(NT // 32)]
    s = [ws[0] for ws in warp_sums] + [0.0] * (32 - NT // 32)
    c = [ws[1] for ws in warp_sums] + [0.0] * (32 - NT // 32)
    S, C = warp_tree(s, c)
    return S + C


@pytest.mark.parametrize("seed", range(4))
def test_final_reduction_is_accurate_under_cancellation(seed):
    rng = np.random.default_rng(seed)
    n = 1216  # one partial per block of the DOT launch on 152 SMs
    big = rng.standard_normal(n // 2) * 1e12
    parts = np.concatenate([big, -big + rng.standard_normal(n // 2)])  # the large halves cancel
    rng.shuffle(parts)
    parts = [float(x) for x in parts]
    exact = math.fsum(parts)
    got = dot_final(parts)
    # compensated: the error is a few ulps of the large terms' rounding, far below plain summation's
    assert abs(got - exact) <= 1e-15 * sum(abs(x) for x in parts)
    naive = 0.0
    for x in parts:
        naive += x
    assert abs(got - exact) <= abs(naive - exact) + 1e-300


def test_final_reduction_is_deterministic_and_exact_on_integers():
    rng = np.random.default_rng(9)
    parts = [float(v) for v in rng.integers(-2 ** 40, 2 ** 40, size=1216)]
    assert dot_final(parts) == dot_final(list(parts)) == math.fsum(parts)
