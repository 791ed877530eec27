"""The coefficient tables (simplediffeq.jl_gb300/csrc/tableaus.h, extracted
from the reference) satisfy the Runge-Kutta order conditions of their
methods: Tsitouras 5(4), Verner 7(6), Verner 9(8).  Every rooted tree up to
the order is checked (b . Phi(t) = 1/gamma(t)), plus row sums (A 1 = c) and
the dense-output polynomials' consistency (b(theta=1) = b, sum b(theta) = theta).
"""
import itertools
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "simplediffeq.jl_gb300", "csrc", "tableaus.h")


def load_groups():
    groups, cur = {}, None
    for line in open(HEADER):
        m = re.match(r"namespace gbtab \{ namespace (\w+) \{", line)
        if m:
            cur = groups.setdefault(m.group(1), {})
            continue
        m = re.match(r"constexpr double (\w+) = (\S+);", line)
        if m and cur is not None:
            cur[m.group(1)] = float(m.group(2))
    return groups


G = load_groups()


# ---------------------------------------------------------------- rooted trees
def trees(order, _cache={}):
    """All rooted trees with `order` vertices, as sorted tuples of subtrees."""
    if order in _cache:
        return _cache[order]
    if order == 1:
        res = [()]
    else:
        res = set()
        # children multiset: partitions of order-1 into subtree orders
        for parts in _partitions(order - 1):
            choices = [trees(k) for k in parts]
            for combo in itertools.product(*choices):
                res.add(tuple(sorted(combo)))
        res = sorted(res)
    _cache[order] = res
    return res


def _partitions(n, maxpart=None):
    maxpart = maxpart or n
    if n == 0:
        yield []
        return
    for k in range(min(n, maxpart), 0, -1):
        for rest in _partitions(n - k, k):
            yield [k] + rest


def tree_order(t):
    return 1 + sum(tree_order(c) for c in t)


def gamma(t):
    g = tree_order(t)
    for c in t:
        g *= gamma(c)
    return g


def phi(t, A):
    v = np.ones(A.shape[0])
    for c in t:
        v = v * (A @ phi(c, A))
    return v


def check_order(A, b, p, tol):
    worst = 0.0
    for q in range(1, p + 1):
        for t in trees(q):
            r = b @ phi(t, A) - 1.0 / gamma(t)
            worst = max(worst, abs(r) * gamma(t))
    assert worst < tol, worst
    return worst


def test_tree_counts():
    assert [len(trees(k)) for k in range(1, 10)] == [1, 1, 2, 4, 9, 20, 48, 115, 286]


# ---------------------------------------------------------------- Tsit5
def tsit5_tableau():
    g = G["tsit5"]
    A = np.zeros((7, 7))
    rows = {1: ["a21"], 2: ["a31", "a32"], 3: ["a41", "a42", "a43"], 4: ["a51", "a52", "a53", "a54"],
            5: ["a61", "a62", "a63", "a64", "a65"], 6: ["a71", "a72", "a73", "a74", "a75", "a76"]}
    for i, names in rows.items():
        for j, nm in enumerate(names):
            A[i, j] = g[nm]
    c = np.array([0, g["c1"], g["c2"], g["c3"], g["c4"], g["c5"], g["c6"]])
    b = A[6].copy()  # FSAL: the solution weights are the last row
    bt = np.array([g["btilde%d" % k] for k in range(1, 8)])
    return A, b, c, bt


def test_tsit5_order_conditions():
    A, b, c, bt = tsit5_tableau()
    assert np.allclose(A.sum(1), c, atol=1e-14)
    check_order(A, b, 5, 1e-13)
    bhat = b - bt  # embedded 4th-order weights (btilde = b - bhat)
    check_order(A, bhat, 4, 1e-12)
    with pytest.raises(AssertionError):
        check_order(A, bhat, 5, 1e-12)


def test_tsit5_dense_output():
    g = G["tsit5"]
    A, b, c, bt = tsit5_tableau()

    def bth(th):
        b1 = th * (g["r11"] + th * (g["r12"] + th * (g["r13"] + th * g["r14"])))
        out = [b1]
        for i in range(2, 8):
            out.append(th * th * (g["r%d2" % i] + th * (g["r%d3" % i] + th * g["r%d4" % i])))
        return np.array(out)

    assert np.allclose(bth(1.0), np.append(b[:6], 0.0), atol=1e-12)
    for th in (0.1, 0.37, 0.8):
        v = bth(th)
        assert abs(v.sum() - th) < 1e-12
        assert abs(v @ c - th ** 2 / 2) < 1e-12
        assert abs(v @ c ** 2 - th ** 3 / 3) < 1e-12
        assert abs(v @ (A @ c) - th ** 3 / 6) < 1e-12


# ---------------------------------------------------------------- Vern7
V7_ROWS = {  # stage (0-based) -> (coefficient name, k slot) in the reference's order
    1: [("a021", 0)], 2: [("a031", 0), ("a032", 1)], 3: [("a041", 0), ("a043", 2)],
    4: [("a051", 0), ("a053", 2), ("a054", 3)], 5: [("a061", 0), ("a063", 2), ("a064", 3), ("a065", 4)],
    6: [("a071", 0), ("a073", 2), ("a074", 3), ("a075", 4), ("a076", 5)],
    7: [("a081", 0), ("a083", 2), ("a084", 3), ("a085", 4), ("a086", 5), ("a087", 6)],
    8: [("a091", 0), ("a093", 2), ("a094", 3), ("a095", 4), ("a096", 5), ("a097", 6), ("a098", 7)],
    9: [("a101", 0), ("a103", 2), ("a104", 3), ("a105", 4), ("a106", 5), ("a107", 6)],
}


def vern7_tableau(extra=False):
    g, x = G["vern7"], G["vern7x"]
    n = 16 if extra else 10
    A = np.zeros((n, n))
    for i, terms in V7_ROWS.items():
        for nm, j in terms:
            A[i, j] = g[nm]
    c = np.zeros(n)
    c[1:8] = [g["c%d" % k] for k in range(2, 9)]
    c[8] = c[9] = 1.0
    b = np.zeros(n)
    for k, slot in zip((1, 4, 5, 6, 7, 8, 9), (0, 3, 4, 5, 6, 7, 8)):
        b[slot] = g["b%d" % k]
    bt = np.zeros(n)
    for k, slot in zip((1, 4, 5, 6, 7, 8, 9, 10), (0, 3, 4, 5, 6, 7, 8, 9)):
        bt[slot] = g["btilde%d" % k]
    if extra:
        for s in range(11, 17):
            row = s - 1
            c[row] = x["c%d" % s]
            for nm, val in x.items():
                m = re.match(r"a%d(\d\d)$" % s, nm)
                if m:
                    A[row, int(m.group(1)) - 1] = val
    return A, b, c, bt


def test_vern7_order_conditions():
    A, b, c, bt = vern7_tableau()
    assert np.allclose(A.sum(1), c, atol=1e-13)
    check_order(A, b, 7, 1e-11)
    check_order(A, b - bt, 6, 1e-10)


def test_vern7_extra_stages_and_interpolant():
    A, b, c, bt = vern7_tableau(extra=True)
    assert np.allclose(A.sum(1), c, atol=1e-12)
    r = G["vern7r"]
    slots = {1: 0, 4: 3, 5: 4, 6: 5, 7: 6, 8: 7, 9: 8, 11: 10, 12: 11, 13: 12, 14: 13, 15: 14, 16: 15}

    def bth(th):
        v = np.zeros(16)
        for s, slot in slots.items():
            lo = 1 if s == 1 else 2
            v[slot] = sum(r["r%02d%d" % (s, k)] * th ** k for k in range(lo, 8))
        return v

    assert np.allclose(bth(1.0), b, atol=1e-10)
    for th in (0.2, 0.5, 0.9):
        v = bth(th)
        # the interpolant is of order 6 for every theta (its order-7 defect
        # vanishes only at theta = 1): sum_i b_i(theta) Phi_i(t) = theta^|t| / gamma(t)
        for q in range(1, 7):
            for t in trees(q):
                assert abs(v @ phi(t, A) - th ** q / gamma(t)) * gamma(t) / th ** q < 1e-9


# ---------------------------------------------------------------- Vern9
V9_SPARSE = {2: [1], 3: [1, 2], 4: [1, 3], 5: [1, 3, 4], 6: [1, 4, 5], 7: [1, 4, 5, 6], 8: [1, 6, 7],
             9: [1, 6, 7, 8], 10: [1, 6, 7, 8, 9], 11: [1, 6, 7, 8, 9, 10], 12: [1, 6, 7, 8, 9, 10, 11],
             13: [1, 6, 7, 8, 9, 10, 11, 12], 14: [1, 6, 7, 8, 9, 10, 11, 12, 13],
             15: [1, 6, 7, 8, 9, 10, 11, 12, 13, 14], 16: [1, 6, 7, 8, 9, 10, 11, 12, 13]}


def vern9_tableau():
    g = G["vern9"]
    A = np.zeros((16, 16))
    for s, js in V9_SPARSE.items():
        for j in js:
            A[s - 1, j - 1] = g["a%02d%02d" % (s, j)]
    c = np.zeros(16)
    c[1:14] = [g["c%d" % k] for k in range(1, 14)]
    c[14] = c[15] = 1.0
    b = np.zeros(16)
    for k in (1, 8, 9, 10, 11, 12, 13, 14, 15):
        b[k - 1] = g["b%d" % k]
    bt = np.zeros(16)
    for k in (1, 8, 9, 10, 11, 12, 13, 14, 15, 16):
        bt[k - 1] = g["btilde%d" % k]
    return A, b, c, bt


def test_vern9_order_conditions():
    A, b, c, bt = vern9_tableau()
    assert np.allclose(A.sum(1), c, atol=1e-12)
    check_order(A, b, 9, 1e-9)
    check_order(A, b - bt, 8, 1e-8)


def test_vern9_extra_stages_row_sums_and_interpolant_end():
    A, b, c, bt = vern9_tableau()
    x, r = G["vern9x"], G["vern9r"]
    # extra stages 17..26 couple to stages 1, 8..15 and to each other
    n = 26
    AA = np.zeros((n, n))
    AA[:16, :16] = A
    cc = np.zeros(n)
    cc[:16] = c
    for s in range(17, 27):
        cc[s - 1] = x["c%d" % s]
        for nm, val in x.items():
            m = re.match(r"a%d(\d\d)$" % s, nm)
            if m:
                AA[s - 1, int(m.group(1)) - 1] = val
    assert np.allclose(AA.sum(1), cc, atol=1e-11)
    slots = [1, 8, 9, 10, 11, 12, 13, 14, 15, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26]

    def bth(th):
        v = np.zeros(n)
        for s in slots:
            lo = 1 if s == 1 else 2
            v[s - 1] = sum(r["r%02d%d" % (s, k)] * th ** k for k in range(lo, 10))
        return v

    bb = np.zeros(n)
    bb[:16] = b
    assert np.allclose(bth(1.0), bb, atol=1e-9)
    for th in (0.25, 0.6):
        v = bth(th)
        # a 9th-order interpolant for every theta
        for q in range(1, 10):
            for t in trees(q):
                assert abs(v @ phi(t, AA) - th ** q / gamma(t)) * gamma(t) / th ** q < 1e-7


# root of a SimpleDiffEq.jl checkout, from the environment (the test is skipped without one)
REFERENCE_ROOT = os.environ.get("SIMPLEDIFFEQ_ROOT", "")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE_ROOT, "src")),
                    reason="SIMPLEDIFFEQ_ROOT does not name a SimpleDiffEq.jl checkout")
def test_header_regenerates_from_reference(tmp_path):
    """The committed header is exactly what the extractor produces from the
    reference's coefficient files."""
    out = tmp_path / "t.h"
    gen = os.path.join(ROOT, "simplediffeq.jl_gb300", "csrc", "gen_tableaus.py")
    subprocess.run([sys.executable, gen, REFERENCE_ROOT, str(out)], check=True)
    assert out.read_text() == open(HEADER).read()
