"""The full minimisation of the semantic global variant (L <= 32) runs the
reference's sequential scan (m = fminf(m, t_s); if (m == t_s) arg = s,
from m = 1e15; ops/lbp_semantic_pw/src/lbp_min_sum_kernel.cu:96-108) as four
chains over the contiguous sender ranges [8c, 8c+8), the first starting at
1e15 and the others at +inf, combined in sender order:

    m = fminf(fminf(fminf(m0, m1), m2), m3)
    arg = the last chain c with m_c == m (its arg_c), else arg_0,

over all 32 senders, the ones beyond L contributing +inf (or NaN for an
infinite edge weight).  This checks on the host, in float32, that the
combination gives the single chain's value bit for bit and its index, under
each rule a min instruction may follow for operands that compare equal
(-0 and +0): return the second operand, return the first, or order -0 below
+0; NaN operands are ignored as fminf does.  No GPU: the kernel itself is
compared with the oracle in tests/test_lbp_forward_gpu.py."""
import numpy as np
import pytest

F = np.float32
INF = F(np.inf)
BIG = F(1e15)


def _min_second(a, b):
    if np.isnan(a):
        return b
    if np.isnan(b):
        return a
    return a if a < b else b


def _min_first(a, b):
    if np.isnan(a):
        return b
    if np.isnan(b):
        return a
    return b if b < a else a


def _min_ordered(a, b):
    if np.isnan(a):
        return b
    if np.isnan(b):
        return a
    if a == b:  # only -0 / +0 can differ: -0 below +0
        return a if np.signbit(a) else b
    return a if a < b else b


RULES = {"second": _min_second, "first": _min_first, "ordered": _min_ordered}


def _scan(fmin, terms, start):
    m, arg = F(start), 0
    for s, t in terms:
        m = fmin(m, t)
        if m == t:
            arg = s
    return m, arg


def _split(fmin, terms32):
    chains = [_scan(fmin, terms32[8 * c:8 * c + 8], BIG if c == 0 else INF) for c in range(4)]
    m, arg = chains[0]
    for c in range(1, 4):
        m = fmin(m, chains[c][0])
        if chains[c][0] == m:
            arg = chains[c][1]
    return m, arg


def _bits(x):
    return np.array([x], np.float32).view(np.uint32)[0]


@pytest.mark.parametrize("rule", sorted(RULES))
def test_four_chain_fold_equals_the_single_scan(rule):
    fmin = RULES[rule]
    g = np.random.default_rng(7)
    values = np.array([-1.0, -0.5, -0.0, 0.0, 0.5, 1.0, 2.0], np.float32)
    for trial in range(3000):
        L = int(g.integers(1, 33))
        t = g.choice(values, size=L).astype(np.float32)
        if trial % 7 == 0:
            t[g.integers(0, L)] = np.nan        # a NaN term (an infinite weight times zero)
        if trial % 11 == 0:
            t[:] = F(2e15)                      # every term above the reference's start value
        if trial % 13 == 0:
            t[g.integers(0, L)] = BIG           # a term equal to the start value
        pad = INF if trial % 2 else F(np.nan)   # senders beyond L: +inf, or NaN for an infinite w
        terms32 = [(s, t[s] if s < L else pad) for s in range(32)]
        m1, a1 = _scan(fmin, terms32[:L], BIG)
        m2, a2 = _split(fmin, terms32)
        assert _bits(m1) == _bits(m2), (rule, trial, m1, m2)
        assert a1 == a2, (rule, trial, a1, a2)
