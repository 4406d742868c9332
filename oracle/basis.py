"""Leg bases, fusion trees and their recoupling (test infrastructure only).

References:
  FusionTree:  include/Xped/Core/FusionTree.hpp:22-115, src/Core/FusionTree.cpp:26-412
  Qbasis:      include/Xped/Core/Qbasis.hpp, src/Core/Qbasis.cpp:34-495
  build trees: src/Core/TensorHelper.cpp:14-44
  treepair:    src/Core/treepair.cpp:35-217
  Permutation: include/Xped/Util/Permutations.hpp:88-241
"""
from __future__ import annotations

import numpy as np

from functools import lru_cache
from math import prod

EPS_TREE = 1.0e-12  # ScalarTraits<double>::epsilon(), include/Xped/Core/ScalarTraits.hpp:17


class FusionTree:
    """Immutable fusion tree.  Equality/hash use (q_uncoupled, q_intermediates,
    q_coupled, dims) like FusionTree::operator== without pedantic asserts
    (FusionTree.cpp:66-85); IS_DUAL is carried but not part of the key."""

    __slots__ = ("qu", "qi", "qc", "dims", "dual", "dim", "_key")

    def __init__(self, qu, qi, qc, dims, dual):
        self.qu = tuple(qu)
        self.qi = tuple(qi)
        self.qc = qc
        self.dims = tuple(dims)
        self.dual = tuple(bool(d) for d in dual)
        self.dim = prod(self.dims) if self.dims else 1  # computeDim (FusionTree.hpp:75)
        self._key = (self.qu, self.qi, self.qc, self.dims)

    @property
    def rank(self):
        return len(self.qu)

    def __eq__(self, other):
        return self._key == other._key

    def __hash__(self):
        return hash(self._key)

    def sort_key(self):
        # FusionTree::operator< (FusionTree.cpp:32-64): uncoupled, intermediates, coupled
        return (self.qu, self.qi, self.qc)

    def __repr__(self):
        return f"FT(qu={self.qu}, qi={self.qi}, qc={self.qc}, dims={self.dims}, dual={self.dual})"

    def replace(self, **kw):
        d = dict(qu=self.qu, qi=self.qi, qc=self.qc, dims=self.dims, dual=self.dual)
        d.update(kw)
        return FusionTree(**d)

    def enlarge(self, other: "FusionTree") -> "FusionTree":
        """FusionTree::enlarge (FusionTree.cpp:309-324)."""
        qi = list(self.qi)
        if self.rank + 1 >= 3:
            qi.append(self.qc)
        return FusionTree(self.qu + other.qu[:1], qi, self.qc, self.dims + other.dims[:1], self.dual + other.dual[:1])

    def as_tensor(self, sym):
        """FusionTree::asTensor (src/Core/FusionTree.cpp:155-285): the tree's
        Clebsch-Gordan tensor, indices (uncoupled legs..., coupled), built by
        chaining the vertices left to right through the intermediate irreps;
        every dual leg is then bent with the symmetry's 1j tensor."""
        deg = sym.degeneracy
        r = self.rank
        if r == 0:
            return np.ones(1)
        if r == 1:
            out = np.eye(deg(self.qu[0]), deg(self.qc))
        else:
            chain = [self.qu[0]] + list(self.qi) + [self.qc]
            out = sym.cgc(self.qu[0], self.qu[1], chain[1])
            for v in range(1, r - 1):
                vert = sym.cgc(chain[v], self.qu[v + 1], chain[v + 1])
                out = np.tensordot(out, vert, axes=([out.ndim - 1], [0]))
        for k in range(r):
            if self.dual[k]:
                oj = sym.one_j(self.qu[k])
                out = np.moveaxis(np.tensordot(oj, out, axes=([1], [k])), 0, k)
        return out

    def compute_intermediates(self, sym):
        """FusionTree::computeIntermediates (FusionTree.cpp:136-152), abelian only."""
        r = self.rank
        qi = []
        for i in range(max(r - 2, 0)):
            if i == 0:
                qi.append(sym.combine(self.qu[0], self.qu[1])[0])
            else:
                qi.append(sym.combine(qi[i - 1], self.qu[i + 1])[0])
        if r == 0:
            qc = self.qc
        elif r < 2:
            qc = self.qu[0]
        elif r == 2:
            qc = sym.combine(self.qu[0], self.qu[1])[0]
        else:
            qc = sym.combine(qi[-1], self.qu[-1])[0]
        return FusionTree(self.qu, qi, qc, self.dims, self.dual)

    # ---- recoupling -------------------------------------------------------
    def swap(self, sym, pos):
        """FusionTree::swap (FusionTree.cpp:353-412): exchange legs pos, pos+1."""
        r = self.rank
        assert pos < r - 1
        out = {}
        qu = list(self.qu)
        qu[pos], qu[pos + 1] = qu[pos + 1], qu[pos]
        dual = list(self.dual)
        dual[pos], dual[pos + 1] = dual[pos + 1], dual[pos]
        dims = list(self.dims)
        dims[pos], dims[pos + 1] = dims[pos + 1], dims[pos]
        if pos == 0:
            ql, qr = self.qu[0], self.qu[1]
            qf = self.qc if r == 2 else self.qi[0]
            coeff = sym.coeff_swap(ql, qr, qf)
            if abs(coeff) < EPS_TREE:
                return out
            out[FusionTree(qu, self.qi, self.qc, dims, dual)] = coeff
            return out
        q1 = self.qu[0] if pos == 1 else self.qi[pos - 2]
        q2 = self.qu[pos]
        q3 = self.qu[pos + 1]
        Q = self.qc if pos == r - 2 else self.qi[pos]
        Q12 = self.qi[pos - 1]
        for Q31 in sym.combine(q3, q1):
            qi = list(self.qi)
            qi[pos - 1] = Q31
            cgc = sym.coeff_swap(Q12, q3, Q) * sym.coeff_recouple(q3, q1, q2, Q, Q31, Q12) * sym.coeff_swap(q3, q1, Q31)
            if abs(cgc) < EPS_TREE:
                continue
            t = FusionTree(qu, qi, self.qc, dims, dual)
            out[t] = cgc  # std::unordered_map::insert keeps the first; trees here are distinct
        return out

    def permute(self, sym, p):
        """FusionTree::permute (FusionTree.cpp:326-351) via adjacent swaps."""
        out = {self: 1.0}
        for pos in decompose_permutation(p):
            tmp = {}
            for tree, coeff in out.items():
                for tree2, coeff2 in tree.swap(sym, pos).items():
                    if tree2 not in tmp:
                        tmp[tree2] = coeff * coeff2
                    else:
                        s = tmp[tree2] + coeff * coeff2
                        if abs(s) < EPS_TREE:
                            del tmp[tree2]
                        else:
                            tmp[tree2] = s
            out = tmp
        return out


def decompose_permutation(pi):
    """Permutation::decompose (Permutations.hpp:195-225): adjacent swaps that
    bring identity to ``pi``."""
    N = len(pi)
    a = list(range(N))
    out = []
    if a == list(pi):
        return out
    for i in range(N):
        index = a.index(pi[i])
        if index == 0:
            continue
        lo = 0 if i == 0 else i
        j = index - 1
        while j >= lo:
            a[j], a[j + 1] = a[j + 1], a[j]
            out.append(j)
            j -= 1
    assert a == list(pi)
    return out


def inverse_permutation(p):
    inv = [0] * len(p)
    for i, v in enumerate(p):
        inv[v] = i
    return inv


# ---- tree pairs --------------------------------------------------------------

def turn_right(sym, t1: FusionTree, t2: FusionTree):
    """treepair::turn_right (treepair.cpp:35-88): move the last codomain leg
    into the domain."""
    R, C = t1.rank, t2.rank
    assert C > 0
    qu1 = t1.qu + (sym.conj(t2.qu[-1]),)
    qi1 = list(t1.qi)
    if R + 1 > 2:
        qi1.append(t1.qc)
    dual1 = t1.dual + (not t2.dual[-1],)
    if C == 1:
        qc = sym.vacuum
    elif C == 2:
        qc = t2.qu[0]
    else:
        qc = t2.qi[-1]
    dims1 = t1.dims + (t2.dims[-1],)
    t1p = FusionTree(qu1, qi1, qc, dims1, dual1)
    qi2 = t2.qi[:-1] if C > 2 else ()
    t2p = FusionTree(t2.qu[:-1], qi2, qc, t2.dims[:-1], t2.dual[:-1])
    a = qc
    b = t2.qu[-1]
    c = t2.qc
    coeff = sym.coeff_turn(a, b, c)
    if t2.dual[-1]:
        coeff *= sym.coeff_FS(sym.conj(b))
    if abs(coeff) < EPS_TREE:
        return {}
    return {(t1p, t2p): coeff}


def turn_left(sym, t1, t2):
    """treepair::turn_left (treepair.cpp:90-101)."""
    return {(b, a): c for (a, b), c in turn_right(sym, t2, t1).items()}


def turn(sym, shift, t1, t2):
    """treepair::turn<shift> (treepair.cpp:103-141)."""
    if shift == 0:
        return {(t1, t2): 1.0}
    out = {}
    if shift > 0:
        for (a, b), c1 in turn_left(sym, t1, t2).items():
            for key, c2 in turn(sym, shift - 1, a, b).items():
                out[key] = c1 * c2  # insert-or-keep: keys are unique along a single turn chain
        return out
    for (a, b), c1 in turn_right(sym, t1, t2).items():
        for key, c2 in turn(sym, shift + 1, a, b).items():
            out[key] = c1 * c2
    return out


def treepair_permute(sym, shift, t1: FusionTree, t2: FusionTree, p):
    """treepair::permute<shift> (treepair.cpp:143-217)."""
    R, C = t1.rank, t2.rank
    newR, newC = R - shift, C + shift
    if sym.ABELIAN and not sym.FERMIONIC:
        qu_d, dims_d, dual_d = [], [], []
        for r in range(newR):
            src = p[r]
            if src < R:
                qu_d.append(t1.qu[src]); dims_d.append(t1.dims[src]); dual_d.append(t1.dual[src])
            else:
                qu_d.append(sym.conj(t2.qu[src - R])); dims_d.append(t2.dims[src - R]); dual_d.append(not t2.dual[src - R])
        qu_c, dims_c, dual_c = [], [], []
        for c in range(newC):
            src = p[c + newR]
            if src < R:
                qu_c.append(sym.conj(t1.qu[src])); dims_c.append(t1.dims[src]); dual_c.append(not t1.dual[src])
            else:
                qu_c.append(t2.qu[src - R]); dims_c.append(t2.dims[src - R]); dual_c.append(t2.dual[src - R])
        d = FusionTree(qu_d, (), sym.vacuum, dims_d, dual_d).compute_intermediates(sym)
        c = FusionTree(qu_c, (), sym.vacuum, dims_c, dual_c).compute_intermediates(sym)
        return {(d, c): 1.0}

    assert t1.qc == t2.qc
    pi_id = list(range(R + C))
    for i in range(C):
        pi_id[i + R] = (C - 1) - i + R
    pi_tmp = [pi_id[p[i]] for i in range(R + C)]
    pi_corr = pi_tmp[:newR] + [pi_tmp[(newC - 1) - i + newR] for i in range(newC)]
    reshift = C + shift
    out = {}
    for (t1p, triv), c1 in turn(sym, -C, t1, t2).items():
        for t1pp, c2 in t1p.permute(sym, pi_corr).items():
            for key, c3 in turn(sym, reshift, t1pp, triv).items():
                out[key] = out.get(key, 0.0) + c1 * c2 * c3
    return out


# ---- Qbasis --------------------------------------------------------------------

class Qbasis:
    """Irrep-sorted basis (Qbasis.hpp:37-271).  ``entries`` holds [q, dim] in
    storage order; ``trees`` maps q -> list of FusionTree (sorted)."""

    def __init__(self, sym, depth: int = 1):
        self.sym = sym
        self.depth = depth
        self.qs = []
        self.dims = []
        self.trees = {}
        self.CONJ = False
        self.IS_SORTED = False

    # -- construction ---------------------------------------------------
    @classmethod
    def from_pairs(cls, sym, pairs, sort=True):
        b = cls(sym, 1)
        for q, d in pairs:
            b.push_back(q, d)
        if sort:
            b.sort()
        return b

    @classmethod
    def trivial(cls, sym):
        b = cls(sym, 1)
        b.push_back(sym.vacuum, 1)
        return b

    def copy(self):
        b = Qbasis(self.sym, self.depth)
        b.qs = list(self.qs)
        b.dims = list(self.dims)
        b.trees = {q: list(v) for q, v in self.trees.items()}
        b.CONJ = self.CONJ
        b.IS_SORTED = self.IS_SORTED
        return b

    def push_back(self, q, inner_dim):
        """Qbasis::push_back(q, dim) (Qbasis.cpp:34-73)."""
        assert self.depth in (0, 1)
        if inner_dim == 0:
            return
        if q not in self.qs:
            if self.depth == 1:
                t = FusionTree((q,), (), q, (inner_dim,), (self.CONJ,))
            else:
                t = FusionTree((), (), q, (), ())
            self.trees[q] = [t]
            self.qs.append(q)
            self.dims.append(inner_dim)
            self.IS_SORTED = False
        else:
            i = self.qs.index(q)
            self.dims[i] += inner_dim
            t = self.trees[q][0]
            self.trees[q][0] = FusionTree(t.qu, t.qi, t.qc, (t.dims[0] + inner_dim,), t.dual)

    def push_back_trees(self, q, inner_dim, trees):
        """Qbasis::push_back(q, dim, trees) (Qbasis.cpp:75-91)."""
        assert q not in self.qs
        self.trees[q] = list(trees)
        self.qs.append(q)
        self.dims.append(inner_dim)
        self.IS_SORTED = False

    def sort(self):
        """Qbasis::sort (Qbasis.cpp:306-331)."""
        if len(self.qs) < 2:
            return [0]
        if self.CONJ:
            key = lambda i: self.sym.conj(self.qs[i])
        else:
            key = lambda i: self.qs[i]
        idx = sorted(range(len(self.qs)), key=key)
        self.qs = [self.qs[i] for i in idx]
        self.dims = [self.dims[i] for i in idx]
        self.IS_SORTED = True
        return idx

    def conj(self):
        """Qbasis::conj (Qbasis.cpp:418-439)."""
        assert self.depth == 1
        out = Qbasis(self.sym, 1)
        out.CONJ = not self.CONJ
        for q, d in zip(self.qs, self.dims):
            old = self.trees[q]
            assert len(old) == 1
            cq = self.sym.conj(q)
            t = FusionTree((cq,), (), cq, old[0].dims, (not old[0].dual[0],))
            out.push_back_trees(cq, d, [t])
        out.sort()
        return out

    def forget_history(self):
        """Qbasis::forgetHistory (Qbasis.cpp:410-416)."""
        out = Qbasis(self.sym, 1)
        for q, d in zip(self.qs, self.dims):
            out.push_back(q, d)
        return out

    def combine(self, other: "Qbasis", CONJ: bool = False) -> "Qbasis":
        """Qbasis::combine (Qbasis.cpp:441-495)."""
        sym = self.sym
        out = Qbasis(sym, self.depth + 1)
        trees = {}
        for q1 in self.qs:
            for q2o in other.qs:
                q2 = sym.conj(q2o) if CONJ else q2o
                for q in sym.combine(q1, q2):
                    for t1 in self.trees[q1]:
                        for t2 in other.trees[q2o if not CONJ else q2o]:
                            tt = t1.enlarge(t2)
                            tt = FusionTree(tt.qu, tt.qi, q, tt.dims, tt.dual)
                            lst = trees.setdefault(q, [])
                            if tt not in lst:
                                lst.append(tt)
        for q in trees:
            trees[q].sort(key=FusionTree.sort_key)
            out.push_back_trees(q, sum(t.dim for t in trees[q]), trees[q])
        out.sort()
        return out

    # -- queries ----------------------------------------------------------
    def dim(self):
        return sum(self.dims)

    def fullDim(self):
        return sum(d * self.sym.degeneracy(q) for q, d in zip(self.qs, self.dims))

    def Nq(self):
        return len(self.qs)

    def IS_PRESENT(self, q):
        return q in self.trees

    def inner_dim(self, q):
        try:
            return self.dims[self.qs.index(q)]
        except ValueError:
            return 0

    def index(self, q):
        return self.qs.index(q)

    def outer_num(self, q):
        i = self.qs.index(q)
        return sum(self.dims[:i])

    def full_outer_num(self, q):
        out = 0
        for p, d in zip(self.qs, self.dims):
            if p == q:
                return out
            out += d * self.sym.degeneracy(p)
        return out

    def left_offset(self, tree: FusionTree) -> int:
        """Qbasis::leftOffset (Qbasis.cpp:208-225)."""
        out = 0
        for t in self.trees[tree.qc]:
            if t == tree:
                break
            out += t.dim
        return out

    def key(self):
        return (self.depth, self.CONJ, tuple(self.qs), tuple(self.dims),
                tuple((q, tuple(t._key + (t.dual,) for t in self.trees[q])) for q in self.qs))

    def __eq__(self, other):
        # Qbasis::operator== compares data_ and trees (Qbasis.cpp:333-351)
        return (self.qs == other.qs and self.dims == other.dims
                and all(self.trees[q] == other.trees.get(q) for q in self.qs))

    def __repr__(self):
        c = "'" if self.CONJ else ""
        return "Qbasis" + c + "(" + ", ".join(f"{q}:{d}" for q, d in zip(self.qs, self.dims)) + ")"


_TREE_CACHE = {}


def build_fusion_tree(sym, uncoupled):
    """internal::build_FusionTree (TensorHelper.cpp:31-44): fold ``combine``
    left to right.  Rank 0 gives the vacuum basis of depth 0."""
    key = (sym.name, tuple(b.key() for b in uncoupled))
    hit = _TREE_CACHE.get(key)
    if hit is not None:
        return hit
    if len(uncoupled) == 0:
        out = Qbasis(sym, 0)
        out.push_back(sym.vacuum, 1)
    else:
        out = uncoupled[0]
        for b in uncoupled[1:]:
            out = out.combine(b)
    _TREE_CACHE[key] = out
    return out
