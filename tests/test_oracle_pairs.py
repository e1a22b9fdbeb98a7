"""Pins of the oracle's neighbour search (CPU only).

* The pair set equals an O(N^2) brute force with the reference's exact test
  r < scale_k*(h_i+h_j)/2 (2_SPH_main_2018.f90:1345-1353).
* The walk order equals a literal simulation of grid_find_NEW's pointer linked list
  (2_SPH_main_2018.f90:1309-1401): nodes are refilled from `last` in list order, new nodes
  are prepended, a shorter step detaches the tail (keepit0/keepit1) and the next step
  re-attaches it.  Creation order comes from an independent Python restatement of the
  cell loop (:1242-1396).
"""
import numpy as np
import pytest

import cases
import orc


def grid_creation_order(x, h, itype, out, skf=1):
    """Pairs (i, j) in grid_find_NEW creation order (0-based), before Pint_Update."""
    n2 = len(h)
    X = x.reshape(-1, 2)
    scale_k = 2 if skf == 1 else 3
    act = out == 0
    xmin = np.zeros(2)
    delt = 2.0 * h[act].max()
    ndiv = [0, 0]
    for d in range(2):
        lo, hi = X[act, d].min(), X[act, d].max()
        length = hi - lo
        nd = int(length / delt + 1.0)
        length_new = nd * delt
        xmin[d] = (lo - (length_new - length) / 2.0) - float(np.float32(0.001)) * length
        ndiv[d] = nd
    cells = {}
    for i in range(n2):
        if not act[i]:
            continue
        idv = []
        for d in range(2):
            q = int((X[i, d] - xmin[d]) / delt + 1.0)
            idv.append(min(q, ndiv[d]))
        c = ndiv[0] * (idv[1] - 1) + idv[0]
        cells.setdefault(c, []).append(i)
    pairs = []
    for idy in range(1, ndiv[1] + 1):
        for idx in range(1, ndiv[0] + 1):
            c = ndiv[0] * (idy - 1) + idx
            lst = cells.get(c, [])
            for ii, it in enumerate(lst):
                for jdy in range(idy, min(ndiv[1], idy + 1) + 1):
                    for jdx in range(max(1, idx - 1), min(ndiv[0], idx + 1) + 1):
                        cj = ndiv[0] * (jdy - 1) + jdx
                        if cj < c:
                            continue
                        lj = cells.get(cj, [])
                        start = ii + 1 if cj == c else 0
                        for jt in lj[start:]:
                            dx = X[it, 0] - X[jt, 0]
                            dy = X[it, 1] - X[jt, 1]
                            r = np.sqrt(dx * dx + dy * dy)
                            if r < scale_k * ((h[it] + h[jt]) / 2.0):
                                pairs.append((it, jt))
    return pairs


class LinkedPairs:
    """Literal model of the reference's pair list: node objects chained by `next`."""

    class Node:
        __slots__ = ("pair", "next")

        def __init__(self):
            self.pair = None
            self.next = None

    def __init__(self):
        self.last = None
        self.m = 0
        self.n = 0
        self.keep0 = self.keep1 = None
        self.current = None

    def step(self, created, first):
        if first:
            self.m = 0
            self.n = 0
            self.last = None
        elif self.n < self.m:
            self.keep0.next = self.keep1
            self.current = self.last
        n = 0
        for pr in created:
            n += 1
            if n > self.m:
                node = self.Node()
                node.next = self.last
                self.last = node
                self.current = node
                self.m += 1
            self.current.pair = pr
            if n < self.m:
                self.keep0 = self.current
                self.current = self.current.next
        self.n = n
        if n < self.m:
            self.keep1 = self.current
            self.keep0.next = None
        self.current = self.last

    def walk(self):
        out = []
        node = self.last
        while node is not None:
            out.append(node.pair)
            node = node.next
        return out


def pint_oriented(pair, itype):
    i, j = pair
    ti, tj = itype[i], itype[j]
    if (ti, tj) in ((2, 1), (2, 25), (1, 25)):
        i, j = j, i
    return i, j


@pytest.fixture(scope="module")
def prob(built):
    return cases.bui_like(width=1.0, height=0.5, dx=0.05)


def test_pair_set_matches_bruteforce(prob):
    o = orc.context(prob.params_copy())
    o.upload_problem(prob)
    rng = np.random.default_rng(7)
    x = prob.x.copy()
    nt = prob.ntotal
    x[:2 * nt] += rng.normal(0, 0.01, 2 * nt)  # random snapshot around the lattice
    st = prob.state()
    st["x"] = x
    o.upload(**st)
    o.step(1, 0.0)
    pr = o.dump_pairs()
    got = set(zip(np.minimum(pr["pair_i"], pr["pair_j"]) - 1, np.maximum(pr["pair_i"], pr["pair_j"]) - 1))
    X = x.reshape(-1, 2)
    h = prob.hsml
    d = np.sqrt(((X[:, None, :] - X[None, :, :]) ** 2).sum(-1))
    thr = 2.0 * ((h[:, None] + h[None, :]) / 2.0)
    ii, jj = np.nonzero(np.triu(d < thr, 1))
    want = set(zip(ii, jj))
    assert got == want
    assert len(pr["pair_i"]) == len(got)


def test_walk_order_matches_linked_list(prob):
    o = orc.context(prob.params_copy())
    rng = np.random.default_rng(11)
    model = LinkedPairs()
    st = prob.state()
    nt = prob.ntotal
    counts = []
    # positions are uploaded step by step so that the pair count rises and falls
    for k, amp in enumerate([0.0, 0.004, 0.0, 0.012, 0.002, 0.02, 0.0]):
        x = prob.x.copy()
        x[:2 * nt] += rng.normal(0, amp, 2 * nt)
        st["x"] = x
        o.upload(**st)
        created = grid_creation_order(x, prob.hsml, prob.itype, np.zeros(prob.ntotal2, np.int32))
        model.step(created, first=(k == 0))
        o.step(1, 0.0)
        pr = o.dump_pairs()
        want = [pint_oriented(p, prob.itype) for p in model.walk()]
        got = list(zip(pr["pair_i"] - 1, pr["pair_j"] - 1))
        assert got == want, "step %d" % k
        counts.append(len(created))
    # the sequence must have exercised growth beyond and shrinkage below the list length
    assert max(counts) > counts[0] and min(counts[1:]) < max(counts)


def test_pint_types(prob):
    o = orc.context(prob.params_copy())
    o.upload_problem(prob)
    o.step(1, 0.0)
    pr = o.dump_pairs()
    it = prob.itype
    ti, tj = it[pr["pair_i"] - 1], it[pr["pair_j"] - 1]
    t = pr["pint_type"]
    assert np.all(ti[t == 1] == 1) and np.all(tj[t == 1] == 2)
    assert np.all((ti[t == 6] == 25) & (tj[t == 6] == 2))
    assert np.all((ti[t == 9] == 25) & (tj[t == 9] == 1))
    assert np.all((ti[t == 2] == 1) & (tj[t == 2] == 1))
    assert np.all((ti[t == 3] == 2) & (tj[t == 3] == 2))
    assert np.all((ti[t == 0] == 25) & (tj[t == 0] == 25))
    # the stored gradient points along x_pair_i - x_pair_j with a negative factor
    X = prob.x.reshape(-1, 2)
    dxx = X[pr["pair_i"] - 1, 0] - X[pr["pair_j"] - 1, 0]
    sel = np.abs(dxx) > 1e-9
    assert np.all(np.sign(pr["dwdx"][sel]) == -np.sign(dxx[sel]))
