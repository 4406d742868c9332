"""Block-sparse symmetric tensor restated in numpy (test infrastructure only).

References:
  storage layout:   include/Xped/Core/storage/StorageType_contiguous.hpp:79-171
  permute:          src/Core/Tensor.cpp:83-214, 335-355
  permute_adj:      src/Core/Tensor.cpp:258-333
  twist:            src/Core/Tensor.cpp:357-377
  subBlock:         src/Core/Tensor.cpp:951-981
  operator*:        src/Core/TensorBase.cpp:237-288
  contract:         include/Xped/Core/Tensor.hpp:328-351, include/Xped/Util/Constfct.hpp:55-109
  tSVD / cutoff:    src/Core/Tensor.cpp:478-633
  tQR:              src/Core/Tensor.cpp:757-780
  maxNorm / diag:   src/Core/TensorBase.cpp:48-56, 191-201
  adjoint:          include/Xped/Core/AdjointOp.hpp:24-68 (+ Tensor.hpp:446-453 for eval order)
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla

from .basis import (FusionTree, Qbasis, build_fusion_tree, inverse_permutation,
                    treepair_permute)

COEFF_CUT = 1.0e-10  # Tensor.cpp:127,193


def get_permutations(a1, rank1, a2, rank2, rankres):
    """util::constFct::get_permutations (Constfct.hpp:55-109)."""
    a1 = list(a1)
    a2 = list(a2)
    r1, r2 = len(a1), len(a2)
    max1 = max(0, max(a1))
    max2 = max(0, max(a2))
    assert max1 == max2
    p2 = [0] * r2
    found2 = [-1] * r2
    for ind in range(max2):
        val = a2.index(ind + 1)
        found2[ind] = val
        p2[ind] = val
    for ind in range(max2, r2):
        val = next(i for i in range(r2) if i not in found2)
        found2[ind] = val
        p2[ind] = val
    p1 = [0] * r1
    found1 = [-1] * r1
    for ind in range(max1):
        val = a1.index(ind + 1)
        found1[ind] = val
        p1[r1 - max1 + ind] = val
    for k, ind in enumerate(range(max1, r1)):
        val = next(i for i in range(r1) if i not in found1)
        found1[ind] = val
        p1[k] = val
    tmp = [x for x in a1 if x < 0] + [x for x in a2 if x < 0]
    pres = sorted(range(len(tmp)), key=lambda i: -tmp[i])
    shift1 = rank1 - r1 + max1
    shift2 = rank2 - max2
    shiftres = r1 - max1 - rankres
    return p1, shift1, p2, shift2, pres, shiftres


class Tensor:
    """Tensor<double, Rank, CoRank, Symmetry> with contiguous column-major
    storage of one block per coupled sector."""

    def __init__(self, sym, dom, cod, fill=True):
        self.sym = sym
        self.dom = list(dom)
        self.cod = list(cod)
        self.cdom = build_fusion_tree(sym, self.dom)
        self.ccod = build_fusion_tree(sym, self.cod)
        self.sectors = []
        self.blocks = []
        self._dict = {}
        if fill:
            self.resize()

    # -- storage -----------------------------------------------------------
    @property
    def rank(self):
        return len(self.dom)

    @property
    def corank(self):
        return len(self.cod)

    def resize(self):
        """StorageType::resize (StorageType_contiguous.hpp:79-97): sectors in
        coupled-domain order that are present in the coupled codomain."""
        self.sectors, self.blocks, self._dict = [], [], {}
        for q, d in zip(self.cdom.qs, self.cdom.dims):
            if self.ccod.IS_PRESENT(q):
                self._dict[q] = len(self.sectors)
                self.sectors.append(q)
                self.blocks.append(np.zeros((d, self.ccod.inner_dim(q))))

    def push_back(self, q, M):
        """StorageType::push_back (StorageType_contiguous.hpp:161-171)."""
        self._dict[q] = len(self.sectors)
        self.sectors.append(q)
        self.blocks.append(np.array(M, dtype=float))

    def block(self, q):
        return self.blocks[self._dict[q]]

    def has(self, q):
        return q in self._dict

    def copy(self):
        t = Tensor(self.sym, self.dom, self.cod, fill=False)
        t.sectors = list(self.sectors)
        t.blocks = [b.copy() for b in self.blocks]
        t._dict = dict(self._dict)
        return t

    def plain_size(self):
        return sum(b.size for b in self.blocks)

    def data(self):
        """Flat column-major data in sector order (Tensor::data())."""
        if not self.blocks:
            return np.zeros(0)
        return np.concatenate([b.ravel(order="F") for b in self.blocks])

    def set_random(self, rng):
        """Seeded N(0,1) per block in sector order, column-major fill.
        (The reference draws uniform[-1,1] from std::mt19937,
        MatrixInterface_Eigen_impl.cpp:52-64; the generator here is the
        project's own and is applied identically to oracle and GPU.)"""
        for i, b in enumerate(self.blocks):
            self.blocks[i] = rng.standard_normal(b.size).reshape(b.shape, order="F")
        return self

    def set_identity(self):
        for i, b in enumerate(self.blocks):
            self.blocks[i] = np.eye(b.shape[0], b.shape[1])
        return self

    @classmethod
    def identity(cls, sym, dom, cod):
        return cls(sym, dom, cod).set_identity()

    # -- sub blocks ----------------------------------------------------------
    def sub_block(self, f1: FusionTree, f2: FusionTree):
        """Tensor::subBlock (Tensor.cpp:962-981) as an (f1.dims + f2.dims)
        column-major array."""
        b = self.block(f1.qc)
        r0 = self.cdom.left_offset(f1)
        c0 = self.ccod.left_offset(f2)
        M = b[r0:r0 + f1.dim, c0:c0 + f2.dim]
        return M.reshape(f1.dims + f2.dims, order="F")

    # -- permute ---------------------------------------------------------------
    def permute(self, shift, p):
        """Tensor::permute<shift, p...> dispatcher (Tensor.cpp:335-355)."""
        p = list(p)
        R, C = self.rank, self.corank
        if shift == 0 and p == list(range(R + C)):
            return self
        newR = R - shift
        pd, pc = p[:newR], p[newR:]
        if shift == 0 and all(x < R for x in pd) and all(x >= R for x in pc):
            return self._permute_within(pd, [x - R for x in pc])
        return self._permute_general(shift, p)

    def _permute_within(self, pd, pc):
        """permute_impl(pd, pc) (Tensor.cpp:83-146)."""
        sym = self.sym
        R = self.rank
        new_dom = [self.dom[i] for i in pd] if len(pd) > 1 else list(self.dom)
        new_cod = [self.cod[i] for i in pc] if len(pc) > 1 else list(self.cod)
        out = Tensor(sym, new_dom, new_cod)
        ptot = list(pd) + [x + R for x in pc]
        for q in self.sectors:
            for f1 in self.cdom.trees[q]:
                for f2 in self.ccod.trees[q]:
                    pf1 = f1.permute(sym, pd)
                    pf2 = f2.permute(sym, pc)
                    T = np.transpose(self.sub_block(f1, f2), ptot) if ptot else self.sub_block(f1, f2)
                    for g1, c1 in pf1.items():
                        for g2, c2 in pf2.items():
                            if abs(c1 * c2) < COEFF_CUT:
                                continue
                            ob = out.block(q)
                            r0 = out.cdom.left_offset(g1)
                            c0 = out.ccod.left_offset(g2)
                            ob[r0:r0 + g1.dim, c0:c0 + g2.dim] += (c1 * c2) * T.reshape((g1.dim, g2.dim), order="F")
        return out

    def _permute_general(self, shift, p):
        """permute_impl<shift>(p) (Tensor.cpp:148-214)."""
        sym = self.sym
        R, C = self.rank, self.corank
        newR, newC = R - shift, C + shift
        new_dom, new_cod = [], []
        for i in range(newR):
            if p[i] > R - 1 or R == 0:
                new_dom.append(self.cod[p[i] - R].conj())
            else:
                new_dom.append(self.dom[p[i]])
        for i in range(newC):
            if p[i + newR] > R - 1 or R == 0:
                new_cod.append(self.cod[p[i + newR] - R])
            else:
                new_cod.append(self.dom[p[i + newR]].conj())
        out = Tensor(sym, new_dom, new_cod)
        for q in self.sectors:
            for f1 in self.cdom.trees[q]:
                for f2 in self.ccod.trees[q]:
                    T = np.transpose(self.sub_block(f1, f2), p)
                    for (g1, g2), coeff in treepair_permute(sym, shift, f1, f2, p).items():
                        if abs(coeff) < COEFF_CUT:
                            continue
                        assert g1.qc == g2.qc
                        ob = out.block(g1.qc)
                        r0 = out.cdom.left_offset(g1)
                        c0 = out.ccod.left_offset(g2)
                        ob[r0:r0 + g1.dim, c0:c0 + g2.dim] += coeff * T.reshape((g1.dim, g2.dim), order="F")
        return out

    def permute_adj(self, shift, p):
        """Tensor::permute_adj<shift, p...> (Tensor.cpp:258-333): the transpose
        (with respect to the stored entries) of the linear map permute<shift, p>,
        applied to a tensor shaped like that map's output.  Returns a tensor shaped
        like the map's input."""
        p = list(p)
        sym = self.sym
        R, C = self.rank, self.corank
        if shift == 0 and p == list(range(R + C)):
            return self
        pinv = inverse_permutation(p)
        newR, newC = R + shift, C - shift
        new_dom, new_cod = [], []
        for i in range(newR):
            if pinv[i] > R - 1 or R == 0:
                new_dom.append(self.cod[pinv[i] - R].conj())
            else:
                new_dom.append(self.dom[pinv[i]])
        for i in range(newC):
            if pinv[i + newR] > R - 1 or R == 0:
                new_cod.append(self.cod[pinv[i + newR] - R])
            else:
                new_cod.append(self.dom[pinv[i + newR]].conj())
        out = Tensor(sym, new_dom, new_cod)
        for q in out.sectors:
            ob = out.block(q)
            for f1 in out.cdom.trees[q]:
                for f2 in out.ccod.trees[q]:
                    r0 = out.cdom.left_offset(f1)
                    c0 = out.ccod.left_offset(f2)
                    for (g1, g2), coeff in treepair_permute(sym, shift, f1, f2, p).items():
                        if abs(coeff) < COEFF_CUT:
                            continue
                        T = np.transpose(self.sub_block(g1, g2), pinv)
                        ob[r0:r0 + f1.dim, c0:c0 + f2.dim] += coeff * T.reshape((f1.dim, f2.dim), order="F")
        return out

    # -- elementwise --------------------------------------------------------------
    def twist(self, leg):
        """Tensor::twist (Tensor.cpp:357-377)."""
        sym = self.sym
        if not sym.FERMIONIC:
            return self
        out = self.copy()
        R = self.rank
        for i, q in enumerate(out.sectors):
            b = out.blocks[i]
            for f1 in out.cdom.trees[q]:
                for f2 in out.ccod.trees[q]:
                    c = sym.coeff_twist(f1.qu[leg]) if leg < R else sym.coeff_twist(f2.qu[leg - R])
                    r0 = out.cdom.left_offset(f1)
                    c0 = out.ccod.left_offset(f2)
                    b[r0:r0 + f1.dim, c0:c0 + f2.dim] *= c
        return out

    def adjoint(self):
        """AdjointOp evaluated into a Tensor: blocks transposed, domain and
        codomain exchanged, sectors pushed in the original sector order."""
        out = Tensor(self.sym, self.cod, self.dom, fill=False)
        for q, b in zip(self.sectors, self.blocks):
            out.push_back(q, b.T.copy())
        return out

    def scale(self, s):
        """CoeffUnaryOp s*x evaluated with push_back in sector order."""
        out = Tensor(self.sym, self.dom, self.cod, fill=False)
        for q, b in zip(self.sectors, self.blocks):
            out.push_back(q, b * s)
        return out

    def max_norm(self):
        """TensorBase::maxNorm (TensorBase.cpp:48-56)."""
        out = 0.0
        for b in self.blocks:
            if b.size:
                m = float(np.max(np.abs(b)))
                if out < m:
                    out = m
        return out

    def normalize_max(self):
        """``T * (1. / T.maxNorm())`` as used by the CTM renormalisation
        (src/PEPS/CTM.cpp:1372,1383,1405)."""
        return self.scale(1.0 / self.max_norm())

    def diag_apply(self, fn):
        """DiagCoeffUnaryOp: apply ``fn`` to the diagonal of every block."""
        out = Tensor(self.sym, self.dom, self.cod, fill=False)
        for q, b in zip(self.sectors, self.blocks):
            m = np.zeros_like(b)
            k = min(b.shape)
            idx = np.arange(k)
            m[idx, idx] = fn(b[idx, idx])
            out.push_back(q, m)
        return out

    def diag_sqrt(self):
        return self.diag_apply(np.sqrt)

    def diag_inv(self):
        return self.diag_apply(lambda x: 1.0 / x)

    def trace(self):
        return sum(float(np.trace(b)) * self.sym.degeneracy(q) for q, b in zip(self.sectors, self.blocks))

    def squared_norm(self):
        """TensorBase::squaredNorm = trace(T T^dagger) (TensorBase.cpp:58-64)."""
        return sum(float(np.sum(b * b)) * self.sym.degeneracy(q) for q, b in zip(self.sectors, self.blocks))

    def add(self, other, alpha=1.0):
        out = self.copy()
        for i, q in enumerate(out.sectors):
            if other.has(q):
                out.blocks[i] = out.blocks[i] + alpha * other.block(q)
        return out

    # -- products -------------------------------------------------------------------
    def __mul__(self, other):
        if isinstance(other, (int, float)):
            return self.scale(float(other))
        return matmul(self, other)

    def contract(self, other, a1, a2, rankres):
        """Tensor::contract<a1, a2, ResRank> (Tensor.hpp:328-351)."""
        p1, s1, p2, s2, pres, sres = get_permutations(a1, self.rank, a2, other.rank, rankres)
        left = self.permute(s1, p1)
        right = other.permute(s2, p2)
        return matmul(left, right).permute(sres, pres)

    # -- decompositions ------------------------------------------------------------------
    def tsvd(self, max_keep, eps_svd, preserve_multiplets=False, return_spec=False, sign_fix=True):
        """Tensor::tSVD (Tensor.cpp:478-633).  Returns (U, S, Vdag, truncWeight,
        entropy[, spec]).  The per-sector SVD is LAPACK dgesvd (Eigen's
        JacobiSVD under EIGEN_USE_LAPACKE).  Ties in the global descending sort
        are broken by (sector order, index within sector).  With ``sign_fix``
        every singular pair is normalised so that the largest-magnitude entry
        of u_j is positive (the gauge convention the GPU kernel uses; all
        gauge-invariant results are unchanged)."""
        sym = self.sym
        middle = Qbasis(sym, 1)
        for q, b in zip(self.sectors, self.blocks):
            middle.push_back(q, min(b.shape))
        U = Tensor(sym, self.dom, [middle], fill=False)
        S = Tensor(sym, [middle], [middle], fill=False)
        Vd = Tensor(sym, [middle], self.cod, fill=False)
        allsv = []
        for q, b in zip(self.sectors, self.blocks):
            if min(b.shape) == 0:
                u, s, vt = np.zeros((b.shape[0], 0)), np.zeros(0), np.zeros((0, b.shape[1]))
            else:
                u, s, vt = sla.svd(b, full_matrices=False, lapack_driver="gesvd")
                if sign_fix:
                    u, vt = fix_svd_signs(u, vt)
            for sv in s:
                allsv.append((q, float(sv)))
            U.push_back(q, u)
            S.push_back(q, np.diag(s))
            Vd.push_back(q, vt)
        return cutoff_matrices(self, U, S, Vd, allsv, max_keep, eps_svd, preserve_multiplets, return_spec)

    def tqr(self, return_lq=False):
        """Tensor::tQR (Tensor.cpp:757-780) with LAPACK dgeqrf/dorgqr
        (Eigen HouseholderQR)."""
        sym = self.sym
        middle = self.ccod.forget_history() if self.cdom.dim() > self.ccod.dim() else self.cdom.forget_history()
        Q = Tensor(sym, self.dom, [middle], fill=False)
        Rt = Tensor(sym, [middle], self.cod, fill=False)
        for q, b in zip(self.sectors, self.blocks):
            rows, cols = b.shape
            qf, rf = sla.qr(b, mode="full")  # qf rows x rows, rf rows x cols
            # Qmat * Identity(rows, cols): first cols columns (zero padded)
            Qm = np.zeros((rows, cols))
            k = min(rows, cols)
            Qm[:, :k] = qf[:, :k]
            Rm = np.zeros((cols, cols))
            Rm[:k, :] = rf[:k, :]
            if return_lq:
                Qm, Rm = Qm.T.copy(), Rm.T.copy()
            Q.push_back(q, Qm)
            Rt.push_back(q, Rm)
        return Q, Rt

    # -- dense expansion ------------------------------------------------------------------
    def _unitary(self, coupled, legs):
        """Tensor::unitaryDomain / unitaryCodomain (src/Core/Tensor.cpp:1000-1132): the
        dense map from the coupled basis (sorted, fused index = inner * deg(q) + m) to the
        uncoupled legs (sorted bases, index per leg = inner * deg(q_i) + m_i), one identity
        on the multiplicities times the tree's Clebsch-Gordan tensor per fusion tree."""
        sym = self.sym
        deg = sym.degeneracy
        out = np.zeros(tuple(b.fullDim() for b in legs) + (coupled.fullDim(),))
        for q in coupled.qs:
            col0 = coupled.full_outer_num(q)
            for tree in coupled.trees[q]:
                dims = [legs[i].inner_dim(tree.qu[i]) for i in range(len(legs))]
                ud = int(np.prod(dims)) if dims else 1
                tid = np.eye(ud).reshape(tuple(dims) + (ud,), order="F")
                cg = tree.as_tensor(sym)
                # tensorProd (src/Interfaces/TensorInterface_Eigen_impl.cpp:156-183): per index
                # the CGC index runs fastest, the multiplicity index slowest
                full = np.einsum(tid, list(range(0, 2 * tid.ndim, 2)), cg, list(range(1, 2 * tid.ndim, 2)))
                full = full.reshape(tuple(a * b for a, b in zip(tid.shape, cg.shape)))
                offs = [legs[i].full_outer_num(tree.qu[i]) for i in range(len(legs))]
                offs.append(col0 + coupled.left_offset(tree) * deg(q))
                out[tuple(slice(o, o + n) for o, n in zip(offs, full.shape))] = full
        return out

    def plain_tensor(self):
        """Tensor::plainTensor (src/Core/Tensor.cpp:1133-1310): the dense tensor over the
        sorted uncoupled legs (domain legs, then codomain legs).  Every block is expanded
        as block (x) identity(deg(q)) into the coupled domain x coupled codomain matrix,
        which is then contracted with the domain and codomain unitaries (fusion-tree
        Clebsch-Gordan tensors; for abelian symmetries every coefficient is 1)."""
        sym = self.sym
        deg = sym.degeneracy
        sdom = [b.copy() for b in self.dom]
        scod = [b.copy() for b in self.cod]
        for b in sdom + scod:
            b.sort()
        cdom = self.cdom.copy()
        ccod = self.ccod.copy()
        cdom.sort()
        ccod.sort()
        inner = np.zeros((cdom.fullDim(), ccod.fullDim()))
        for q, b in zip(self.sectors, self.blocks):
            d = deg(q)
            r0, c0 = cdom.full_outer_num(q), ccod.full_outer_num(q)
            inner[r0:r0 + d * b.shape[0], c0:c0 + d * b.shape[1]] += np.kron(b, np.eye(d))
        ud = self._unitary(cdom, sdom)
        uc = self._unitary(ccod, scod)
        mid = np.tensordot(ud, inner, axes=([ud.ndim - 1], [0]))
        return np.tensordot(mid, uc, axes=([mid.ndim - 1], [uc.ndim - 1]))


def fix_svd_signs(u, vt):
    """Gauge convention shared with the GPU kernel: flip (u_j, v_j) so that
    r.u_j > 0 for the fixed generic vector r_i = frac((i+1)*0.7548776662466927)
    + 0.25; when r.u_j is negligible (|r.u| <= 1e-8 sum r_i|u_i|) the first
    largest-magnitude entry of u_j is made positive instead.  Structured
    inputs (e.g. ket-bra fused environments) have singular vectors with
    entries of exactly equal magnitude, for which a largest-entry rule alone
    is decided by rounding."""
    u = u.copy()
    vt = vt.copy()
    y = np.arange(1, u.shape[0] + 1, dtype=np.float64) * 0.7548776662466927
    r = (y - np.floor(y)) + 0.25
    for j in range(u.shape[1]):
        dot = float(r @ u[:, j])
        mag = float(r @ np.abs(u[:, j]))
        if abs(dot) > 1.0e-8 * mag:
            neg = dot < 0
        else:
            neg = u[int(np.argmax(np.abs(u[:, j]))), j] < 0
        if neg:
            u[:, j] *= -1.0
            vt[j, :] *= -1.0
    return u, vt


def matmul(left: Tensor, right: Tensor) -> Tensor:
    """TensorBase::operator* (TensorBase.cpp:237-288): C_q += A_q B_q for the
    sectors of ``left`` that ``right`` also holds."""
    assert left.corank == right.rank
    out = Tensor(left.sym, left.dom, right.cod)
    for q, a in zip(left.sectors, left.blocks):
        if not right.has(q):
            continue
        idx = out._dict[q]
        out.blocks[idx] = out.blocks[idx] + a @ right.block(q)
    return out


TIE_RTOL = 1.0e-12


def tie_tolerant_order(values):
    """Global descending order of singular values used for truncation.

    The reference sorts with std::sort (unstable, Tensor.cpp:543-547), so the
    order of equal values - and hence which of two degenerate values survives
    the chi cut - is unspecified.  Here the order is made deterministic and
    insensitive to last-bit differences between LAPACK and the GPU kernel:
    values are sorted descending, consecutive values within TIE_RTOL
    (relative) form a tie group, and inside a group entries keep their
    (sector, index) position order."""
    n = len(values)
    exact = sorted(range(n), key=lambda i: (-values[i], i))
    groups = []
    for pos, i in enumerate(exact):
        if pos == 0 or values[exact[pos - 1]] - values[i] > TIE_RTOL * values[exact[pos - 1]]:
            groups.append([])
        groups[-1].append(i)
    out = []
    for g in groups:
        out.extend(sorted(g))
    return out


def cutoff_matrices(T, U, S, Vd, allsv, max_keep, eps_svd, preserve_multiplets, return_spec):
    """Tensor::cutoff_matrices (Tensor.cpp:523-633)."""
    sym = T.sym
    n = len(allsv)
    assert n > 0
    first_entry = allsv[0]
    allsv = [allsv[i] for i in tie_tolerant_order([v for _, v in allsv])]
    trunc_weight = 0.0
    for i in range(max_keep, len(allsv)):
        trunc_weight += sym.degeneracy(allsv[i][0]) * abs(allsv[i][1]) ** 2
    allsv = allsv[:min(max_keep, n)]
    if eps_svd > 0.0:
        allsv = [e for e in allsv if not (e[1] < eps_svd)]
    if preserve_multiplets:
        end = -1
        for i in range(len(allsv) - 1, 0, -1):
            rel = 2 * (allsv[i - 1][1] - allsv[i][1]) / (allsv[i - 1][1] + allsv[i][1])
            if rel > 0.1:
                end = i
                break
        if end != -1:
            allsv = allsv[:end]
    if len(allsv) == 0:
        allsv.append(first_entry)
    per_q = {}
    entropy = 0.0
    for q, s in allsv:
        per_q.setdefault(q, []).append(s)
        entropy += -sym.degeneracy(q) * s * s * math.log(s * s)
    trunc = Qbasis(sym, 1)
    for q in sorted(per_q):
        trunc.push_back(q, len(per_q[q]))
    tU = Tensor(sym, T.dom, [trunc], fill=False)
    tS = Tensor(sym, [trunc], [trunc], fill=False)
    tV = Tensor(sym, [trunc], T.cod, fill=False)
    spec = {}
    for q in sorted(per_q):
        k = len(per_q[q])
        tS.push_back(q, S.block(q)[:k, :k])
        if return_spec:
            spec[q] = np.diag(S.block(q))[:k].copy()
        tU.push_back(q, U.block(q)[:, :k])
        tV.push_back(q, Vd.block(q)[:k, :])
    if return_spec:
        return tU, tS, tV, trunc_weight, entropy, spec
    return tU, tS, tV, trunc_weight, entropy


def decompose(T1: Tensor, T2: Tensor, max_nsv: int):
    """decompose (src/PEPS/PEPSContractions.cpp:16-43): projector pair
    P1 = S^-1/2 U^dag T1, P2 = T2 V S^-1/2 from the tSVD of T1*T2."""
    prod = T1 * T2
    U, S, Vd, _tw, _ent = prod.tsvd(max_nsv, 1.0e-10, False)
    isqrtS = S.diag_sqrt().diag_inv()
    P1 = (isqrtS * U.adjoint()) * T1
    P2 = (T2 * Vd.adjoint()) * isqrtS
    return P1, P2


def svd_backward_block(U, s, Vd, dU, dS, dVd):
    """Reverse rule of the per-sector SVD A = U diag(s) Vd, real case
    (ADTensor.hpp:257-301): the cotangent of A from those of U, S (a k x k
    matrix) and Vd.  F_ij = 1 / (s_j^2 - s_i^2), with d -> d / (d^2 + 1e-12)
    for |d| < 1e-12 (vec_diff, PlainInterface_Eigen_impl.cpp:82-85)."""
    s = np.asarray(s, dtype=float)
    s2 = s * s
    Finv = s2[None, :] - s2[:, None]
    small = np.abs(Finv) < 1e-12
    F = np.where(small, Finv / (Finv * Finv + 1e-12), 1.0 / np.where(small, 1.0, Finv))
    S = np.diag(s)
    sinv = np.diag(1.0 / s)
    J = F * (U.T @ dU)
    K = F * (Vd @ dVd.T)
    dA = U @ (dS + (J + J.T) @ S + S @ (K + K.T)) @ Vd
    dA += (np.eye(U.shape[0]) - U @ U.T) @ dU @ sinv @ Vd
    dA += U @ sinv @ dVd @ (np.eye(Vd.shape[1]) - Vd.T @ Vd)
    return dA
