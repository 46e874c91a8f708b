"""Shared parity rules for the test suite.

Top-N comparison rule: two top-N lists are equivalent when they have the same
length and every combination present in only one of them has an exact (FP64
oracle) MI within ``tol`` (absolute) of the exact MI of the cutoff, i.e. they
differ only by ties that the tolerance cannot order.  Values of combinations
in both lists must agree within the stated per-value tolerance.
"""
from __future__ import annotations

import numpy as np


def as_set(combos):
    return {tuple(int(x) for x in c) for c in np.asarray(combos)}


def exact_mi(oracle, data, cw, tw, n_cases, n_ctrls, order, combos):
    """FP64 MI of arbitrary combinations from the oracle's tables."""
    combos = np.asarray(combos, np.int32).reshape(-1, order)
    if len(combos) == 0:
        return np.zeros(0)
    cc, tt = oracle.tables(data, cw, tw, order, combos)
    _, v64 = oracle.mi_batch(cc, tt, n_cases, n_ctrls)
    return v64


def assert_topn_equivalent(a_combos, b_combos, exact_of, tol):
    """exact_of(list of combos) -> FP64 MI array."""
    a, b = as_set(a_combos), as_set(b_combos)
    assert len(a_combos) == len(b_combos), (len(a_combos), len(b_combos))
    assert len(a) == len(a_combos) and len(b) == len(b_combos), "duplicate combinations"
    diff = sorted(a ^ b)
    if not diff:
        return
    union = sorted(a | b)
    ex = dict(zip(union, exact_of(union)))
    cut_a = min(ex[c] for c in a)
    cut_b = min(ex[c] for c in b)
    cutoff = max(cut_a, cut_b)
    for c in diff:
        assert abs(ex[c] - cutoff) <= tol, "combination %s (MI %.9g) differs beyond tie tolerance of cutoff %.9g" % (
            c, ex[c], cutoff)


def assert_sorted_desc(vals):
    v = np.asarray(vals)
    assert np.all(v[:-1] >= v[1:]), "results not sorted in descending order"


def assert_ascending_unique(combos):
    """tests/utils.h:16-45 of the reference: no repeated combination, indices strictly ascending."""
    c = np.asarray(combos)
    assert len(as_set(c)) == len(c), "repeated combination"
    if c.size:
        assert np.all(c[:, 1:] > c[:, :-1]), "combination indices not strictly ascending"
