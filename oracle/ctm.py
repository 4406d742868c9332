"""CTMRG on a 1x1 unit cell, restated from the reference (test infrastructure only).

Covers CTM<double, Sym, TRank=2, ALL_OUT_LEGS=false> with CTM_INIT::FROM_A and
PROJECTION::CORNER.  References:
  iPEPS A / Adag:        src/PEPS/iPEPS.cpp:96-141, 201-212, 516-560
  init FROM_A:           src/PEPS/CTM.cpp:161-212
  grow_all:              src/PEPS/CTM.cpp:385-398
  moves:                 src/PEPS/CTM.cpp:924-1183
  get_projectors:        src/PEPS/CTM.cpp:1185-1337
  renormalize_*:         src/PEPS/CTM.cpp:1339-1641
  contractCorner:        src/PEPS/CTM.cpp:1643-1760
  decompose:             src/PEPS/PEPSContractions.cpp:16-43
  computeRDM_h / _v:     src/PEPS/CTM.cpp:530-698, 700-876 (TRank == 2 branch)
  avg (two-site op):     src/PEPS/LinearAlgebra.cpp:36-80
On a 1x1 cell every (x +- 1, y +- 1) index refers to the same site tensors.
"""
from __future__ import annotations

import numpy as np

from .basis import Qbasis
from .tensor import Tensor, decompose


class IPEPS:
    """Site tensor A: Tensor<2,3>({left, top}, {right, bottom, phys})."""

    def __init__(self, sym, aux: Qbasis, phys: Qbasis):
        self.sym = sym
        self.A = Tensor(sym, [aux, aux], [aux, aux, phys])
        self.update_adag()

    def set_random(self, rng):
        self.A.set_random(rng)
        self.update_adag()
        return self

    def update_adag(self):
        # Adags = As.adjoint().eval().permute<0, 3, 4, 2, 0, 1>()   (iPEPS.cpp:210)
        self.Adag = self.A.adjoint().permute(0, [3, 4, 2, 0, 1])

    def ket(self, leg):
        A = self.A
        return {"L": A.dom[0], "T": A.dom[1], "R": A.cod[0], "B": A.cod[1], "P": A.cod[2]}[leg]

    def bra(self, leg):
        D = self.Adag
        return {"L": D.dom[0], "T": D.dom[1], "R": D.cod[0], "B": D.cod[1], "P": D.dom[2]}[leg]


class CTM:
    def __init__(self, peps: IPEPS, chi: int):
        self.peps = peps
        self.chi = chi
        self.sym = peps.sym
        self.C1 = self.C2 = self.C3 = self.C4 = None
        self.T1 = self.T2 = self.T3 = self.T4 = None

    # -- init -----------------------------------------------------------------------
    def init(self):
        """FROM_A initialisation (CTM.cpp:161-212)."""
        s = self.sym
        P = self.peps
        A, Ad = P.A, P.Adag
        fused = lambda l: P.ket(l).combine(P.bra(l)).forget_history()
        fuse_ll = Tensor.identity(s, [fused("L")], [P.ket("L"), P.bra("L")])
        fuse_uu = Tensor.identity(s, [fused("T")], [P.ket("T"), P.bra("T")])
        fuse_rr = Tensor.identity(s, [P.ket("R"), P.bra("R")], [fused("R")])
        fuse_dd = Tensor.identity(s, [P.ket("B"), P.bra("B")], [fused("B")])
        tw = lambda T, *legs: _twists(T, legs)
        self.C1 = (A.contract(tw(Ad, 3, 4), [1, 2, -1, -2, 3], [1, 2, 3, -3, -4], 2)
                   .contract(fuse_rr, [1, -1, 2, -2], [1, 2, -3], 2)
                   .contract(fuse_dd, [1, 2, -2], [1, 2, -1], 0))
        self.C2 = (A.contract(tw(Ad, 4), [-1, 1, 2, -2, 3], [-3, 1, 3, 2, -4], 2)
                   .contract(tw(fuse_ll, 1, 2), [1, -1, 2, -2], [-3, 1, 2], 2)
                   .contract(fuse_dd, [1, 2, -1], [1, 2, -2], 1))
        self.C3 = (A.contract(Ad, [-1, -2, 1, 2, 3], [-3, -4, 3, 1, 2], 2)
                   .contract(tw(fuse_ll, 1, 2), [1, -1, 2, -2], [-3, 1, 2], 2)
                   .contract(tw(fuse_uu, 1, 2), [1, 2, -2], [-1, 1, 2], 2))
        self.C4 = (A.contract(tw(Ad, 3), [1, -1, -2, 2, 3], [1, -3, 3, -4, 2], 2)
                   .contract(tw(fuse_uu, 1, 2), [1, -1, 2, -2], [-3, 1, 2], 2)
                   .contract(fuse_rr, [1, 2, -1], [1, 2, -2], 1))
        self.T1 = (A.contract(tw(Ad, 3, 4), [-1, 1, -2, -3, 2], [-4, 1, 2, -5, -6], 3)
                   .contract(tw(fuse_ll, 1, 2), [1, -1, -2, 2, -3, -4], [-5, 1, 2], 4)
                   .contract(fuse_rr, [1, -3, 2, -4, -1], [1, 2, -2], 1))
        self.T2 = (A.contract(tw(Ad, 4), [-1, -2, 1, -3, 2], [-4, -5, 2, 1, -6], 3)
                   .contract(tw(fuse_uu, 1, 2), [-1, 1, -2, -3, 2, -4], [-5, 1, 2], 4)
                   .contract(fuse_dd, [-1, 1, -2, 2, -3], [1, 2, -4], 3))
        self.T3 = (A.contract(tw(Ad, 3), [-1, -2, -3, 1, 2], [-4, -5, 2, -6, 1], 3)
                   .contract(tw(fuse_ll, 1, 2), [1, -1, -2, 2, -3, -4], [-5, 1, 2], 4)
                   .contract(fuse_rr, [-1, 1, -2, 2, -3], [1, 2, -4], 3))
        self.T4 = (A.contract(tw(Ad, 3, 4), [1, -1, -2, -3, 2], [1, -4, 2, -5, -6], 3)
                   .contract(tw(fuse_uu, 1, 2), [1, -1, -2, 2, -3, -4], [-5, 1, 2], 4)
                   .contract(fuse_dd, [-3, 1, -4, 2, -1], [1, 2, -2], 1))
        return self

    # -- corners -----------------------------------------------------------------------
    def contract_corner(self, corner):
        """contractCorner, TRank == 2 branch (CTM.cpp:1667-1738)."""
        A, Ad = self.peps.A, self.peps.Adag
        tw = lambda T, *legs: _twists(T, legs)
        if corner == "UL":
            C1T1 = self.C1.contract(self.T1, [-1, 1], [1, -2, -3, -4], 1)
            T4C1T1 = self.T4.contract(tw(C1T1, 0), [1, -1, -2, -3], [1, -4, -5, -6], 3)
            T4C1T1A = T4C1T1.contract(A, [-1, 1, -2, -3, 2, -4], [1, 2, -5, -6, -7], 4)
            return T4C1T1A.contract(tw(Ad, 3, 4), [-1, 1, -4, 2, -5, -2, 3], [1, 2, 3, -6, -3], 3)
        if corner == "LL":
            C4T3 = self.C4.contract(self.T3, [-1, 1], [-2, -3, 1, -4], 1)
            T4C4T3 = self.T4.contract(C4T3, [-1, 1, -2, -3], [1, -4, -5, -6], 3)
            T4C4T3A = T4C4T3.contract(tw(A, 3), [-1, 1, -2, 2, -3, -4], [1, -5, -6, 2, -7], 4)
            return T4C4T3A.contract(tw(Ad, 3), [-4, 1, 2, -1, -5, -2, 3], [1, -6, 3, -3, 2], 3)
        if corner == "UR":
            T1C2 = self.T1.contract(self.C2, [-1, 1, -2, -3], [1, -4], 3)
            T1C2T2 = T1C2.contract(self.T2, [-1, -2, -3, 1], [-4, -5, 1, -6], 3)
            T1C2T2A = T1C2T2.contract(tw(A, 2), [-1, 1, -2, 2, -3, -4], [-5, 1, 2, -6, -7], 4)
            return T1C2T2A.contract(tw(Ad, 4), [-1, 1, 2, -4, -2, -5, 3], [-3, 1, 3, 2, -6], 3)
        if corner == "LR":
            C3T3 = tw(self.C3, 1).contract(self.T3, [-1, 1], [-2, -3, -4, 1], 1)
            T2C3T3 = self.T2.contract(C3T3, [-1, -2, -3, 1], [1, -4, -5, -6], 3)
            T2C3T3A = T2C3T3.contract(tw(A, 2, 3), [1, -1, -2, 2, -3, -4], [-5, -6, 1, 2, -7], 4)
            return T2C3T3A.contract(Ad, [1, -1, 2, -4, -5, -2, 3], [-6, -3, 3, 1, 2], 3)
        raise ValueError(corner)

    def get_projectors(self, direction):
        """get_projectors, CORNER projection (CTM.cpp:1195-1326)."""
        if direction == "L":
            Q1 = self.contract_corner("UL")
            Q4 = _twists(self.contract_corner("LL"), (3, 4, 5))
            return decompose(Q4, Q1, self.chi)
        if direction == "R":
            Q2 = self.contract_corner("UR")
            Q3 = self.contract_corner("LR")
            return decompose(Q2, Q3, self.chi)
        if direction == "T":
            Q1 = self.contract_corner("UL")
            Q2 = self.contract_corner("UR")
            return decompose(Q1, Q2, self.chi)
        if direction == "B":
            Q4 = _twists(self.contract_corner("LL"), (0, 1, 2))
            Q3 = self.contract_corner("LR")
            return decompose(Q3, Q4, self.chi)
        raise ValueError(direction)

    # -- renormalisation ------------------------------------------------------------------
    def renormalize(self, direction, P1, P2):
        """renormalize_left/right/top/bottom, TRank == 2 (CTM.cpp:1358-1627)."""
        A, Ad = self.peps.A, self.peps.Adag
        tw = lambda T, *legs: _twists(T, legs)
        if direction == "L":
            C1T1 = self.C1.contract(self.T1, [-1, 1], [1, -4, -2, -3], 3)
            C1n = tw(P1, 1, 2, 3).contract(C1T1, [-1, 1, 2, 3], [1, 2, 3, -2], 0)
            C4T3 = self.C4.contract(self.T3, [-2, 1], [-3, -4, 1, -1], 1)
            C4n = C4T3.contract(tw(P2, 0, 1, 2), [-2, 1, 2, 3], [1, 2, 3, -1], 1)
            P1T4 = tw(P1, 1, 2, 3).contract(self.T4, [-1, 1, -2, -3], [-4, 1, -5, -6], 3)
            P1T4A = P1T4.contract(A, [-1, 2, -2, -3, 1, -4], [1, -5, -6, 2, -7], 4)
            P1T4AAd = P1T4A.contract(tw(Ad, 3, 4), [-1, 2, -4, 1, -5, -2, 3], [1, -6, 3, -3, 2], 3)
            T4n = P1T4AAd.contract(tw(P2, 0, 1, 2), [-2, -3, -4, 1, 2, 3], [1, 2, 3, -1], 1)
            return C1n.normalize_max(), T4n.normalize_max(), C4n.normalize_max()
        if direction == "R":
            T1C2 = self.T1.contract(self.C2, [-1, 1, -3, -4], [1, -2], 1)
            C2n = T1C2.contract(P2, [-1, 1, 2, 3], [1, 2, 3, -2], 1)
            C3T3 = tw(self.C3, 1).contract(self.T3, [-1, 1], [-2, -3, -4, 1], 3)
            C3n = P1.contract(C3T3, [-1, 1, 2, 3], [1, 2, 3, -2], 2)
            P1T2 = P1.contract(self.T2, [-1, 1, -2, -3], [-4, -5, 1, -6], 3)
            P1T2A = P1T2.contract(tw(A, 2), [-1, 1, -2, 2, -3, -4], [-5, 1, 2, -6, -7], 4)
            P1T2AAd = P1T2A.contract(tw(Ad, 4), [-1, 1, 2, -4, -2, -5, 3], [-3, 1, 3, 2, -6], 3)
            T2n = P1T2AAd.contract(P2, [-3, -1, -2, 1, 2, 3], [1, 2, 3, -4], 3)
            return C2n.normalize_max(), T2n.normalize_max(), C3n.normalize_max()
        if direction == "T":
            T4C1 = self.T4.contract(tw(self.C1, 0), [1, -1, -3, -4], [1, -2], 1)
            C1n = T4C1.contract(P2, [-1, 1, 2, 3], [1, 2, 3, -2], 0)
            C2T2 = self.C2.contract(self.T2, [-1, 1], [-2, -3, 1, -4], 3)
            C2n = P1.contract(C2T2, [-1, 1, 2, 3], [1, 2, 3, -2], 1)
            P1T1 = P1.contract(self.T1, [-1, 1, -2, -3], [1, -4, -5, -6], 3)
            P1T1A = P1T1.contract(A, [-1, 1, -2, -3, 2, -4], [1, 2, -5, -6, -7], 4)
            P1T1AAd = P1T1A.contract(tw(Ad, 3, 4), [-1, 1, -4, 2, -5, -2, 3], [1, 2, 3, -6, -3], 3)
            T1n = P1T1AAd.contract(P2, [-1, -3, -4, 1, 2, 3], [1, 2, 3, -2], 1)
            return C1n.normalize_max(), T1n.normalize_max(), C2n.normalize_max()
        if direction == "B":
            T4C4 = self.T4.contract(self.C4, [-4, 1, -2, -3], [1, -1], 3)
            C4n = tw(P1, 1, 2, 3).contract(T4C4, [-2, 1, 2, 3], [1, 2, 3, -1], 1)
            T2C3 = self.T2.contract(self.C3, [-3, -4, -1, 1], [1, -2], 1)
            C3n = T2C3.contract(tw(P2, 0, 1, 2), [-1, 1, 2, 3], [1, 2, 3, -2], 2)
            P1T3 = tw(P1, 1, 2, 3).contract(tw(self.T3, 0), [-1, 1, -2, -3], [-4, -5, -6, 1], 3)
            P1T3A = P1T3.contract(A, [-1, 1, -2, 2, -3, -4], [-5, -6, 1, 2, -7], 4)
            P1T3AAd = P1T3A.contract(tw(Ad, 3), [-1, 1, 2, -4, -5, -2, 3], [-6, -3, 3, 1, 2], 3)
            T3n = P1T3AAd.contract(tw(P2, 0, 1, 2), [-4, -1, -2, 1, 2, 3], [1, 2, 3, -3], 3)
            return C4n.normalize_max(), T3n.normalize_max(), C3n.normalize_max()
        raise ValueError(direction)

    # -- moves -------------------------------------------------------------------------------
    def move(self, direction):
        P1, P2 = self.get_projectors(direction)
        a, b, c = self.renormalize(direction, P1, P2)
        if direction == "L":
            self.C1, self.T4, self.C4 = a, b, c
        elif direction == "R":
            self.C2, self.T2, self.C3 = a, b, c
        elif direction == "T":
            self.C1, self.T1, self.C2 = a, b, c
        else:
            self.C4, self.T3, self.C3 = a, b, c

    def grow_all(self):
        """CTM::grow_all (CTM.cpp:385-398): left, right, top, bottom."""
        for d in ("L", "R", "T", "B"):
            self.move(d)
        return self

    def solve(self, H, tol_E=1e-10, max_steps=100):
        """CTMSolver::solve without AD (src/PEPS/CTMSolver.cpp:50-80), 1x1 cell: grow_all, then
        E = <H>_h + <H>_v; stop when |E - E_prev| < tol_E or |E - E_prevprev| < tol_E."""
        prev = prevprev = 1000.0
        out = {"E": float("nan"), "steps": 0, "converged": False, "oscillation": False, "energies": []}
        for step in range(max_steps):
            self.grow_all()
            E = bond_expectation(self.rdm_h(), H) + bond_expectation(self.rdm_v(), H)
            out["energies"].append(E)
            out["E"], out["steps"] = E, step + 1
            if abs(E - prev) < tol_E:
                out["converged"] = True
                break
            if abs(E - prevprev) < tol_E:
                out["converged"] = out["oscillation"] = True
                break
            prevprev, prev = prev, E
        return out

    # -- reduced density matrices and bond energies ---------------------------------
    def rdm_h(self):
        """computeRDM_h, TRank == 2 (CTM.cpp:583-619): rho_h Tensor<2,2>
        (left phys, right phys | left phys', right phys'), normalised."""
        A, Ad = self.peps.A, self.peps.Adag
        C1T1 = self.C1.contract(self.T1, [-1, 1], [1, -2, -3, -4], 1)
        T4C1T1 = self.T4.contract(C1T1.twist(0), [1, -1, -2, -3], [1, -4, -5, -6], 3)
        T4C1T1A = T4C1T1.contract(A, [-1, 1, -2, -3, 2, -4], [1, 2, -5, -6, -7], 4)
        C4T3 = self.C4.contract(self.T3, [-1, 1], [-2, -3, 1, -4], 1)
        C4T3Ad = C4T3.contract(Ad.twist(3), [-1, -2, 1, -3], [-4, -5, -6, -7, 1], 3)
        left = T4C1T1A.contract(C4T3Ad, [1, 2, -1, 3, -2, 4, -3], [1, 4, -4, 2, 3, -5, -6], 3)
        T1C2 = self.T1.contract(self.C2, [-1, 1, -2, -3], [1, -4], 3)
        T1C2T2 = T1C2.contract(self.T2, [-1, -2, -3, 1], [-4, -5, 1, -6], 3)
        AT1C2T2 = A.twist(1).contract(T1C2T2, [-1, 1, 2, -2, -3], [-4, 1, -5, 2, -6, -7], 3)
        T3C3 = self.T3.contract(self.C3, [-1, -2, -3, 1], [-4, 1], 3)
        T3C3Ad = T3C3.contract(Ad, [-1, 1, -2, -3], [-4, -5, -6, -7, 1], 3)
        right = AT1C2T2.contract(T3C3Ad, [-1, 1, -2, -3, 2, 3, 4], [1, -4, 4, -5, 2, -6, 3], 3)
        rho = left.contract(right, [1, 2, -3, 3, -1, 4], [2, -4, 1, 3, 4, -2], 2)
        return _normalise_rdm(rho)

    def rdm_v(self):
        """computeRDM_v, TRank == 2 (CTM.cpp:756-781): rho_v Tensor<2,2>
        (upper phys, lower phys | upper phys', lower phys'), normalised."""
        A, Ad = self.peps.A, self.peps.Adag
        C1T1 = self.C1.contract(self.T1, [-1, 1], [1, -2, -3, -4], 1)
        T4C1T1 = self.T4.contract(C1T1.twist(0), [1, -1, -2, -3], [1, -4, -5, -6], 3)
        T4C1T1A = T4C1T1.contract(A, [-1, 1, -2, -3, 2, -4], [1, 2, -5, -6, -7], 4)
        C2T2 = self.C2.contract(self.T2, [-1, 1], [-2, -3, 1, -4], 1)
        AdC2T2 = Ad.twist(3).twist(4).contract(C2T2, [-1, -2, -3, 1, -4], [-5, -6, 1, -7], 4)
        upper = T4C1T1A.contract(AdC2T2, [-1, 1, 2, 3, 4, -2, -3], [1, 3, -4, -5, 2, 4, -6], 3)
        C4T3 = self.C4.contract(self.T3, [-1, 1], [-2, -3, 1, -4], 1)
        T4C4T3 = self.T4.contract(C4T3, [-1, 1, -2, -3], [1, -4, -5, -6], 3)
        AT4C4T3 = A.twist(0).contract(T4C4T3, [1, -1, -2, 2, -3], [-4, 1, -5, 2, -6, -7], 3)
        T2C3 = self.T2.contract(self.C3, [-1, -2, -3, 1], [1, -4], 3)
        T2C3Ad = T2C3.contract(Ad, [-1, 1, -2, -3], [-4, -5, -6, 1, -7], 3)
        lower = AT4C4T3.contract(T2C3Ad, [-1, 1, -2, -3, 2, 3, 4], [1, -4, 4, 2, -5, -6, 3], 3)
        rho = upper.contract(lower, [1, 2, -3, -1, 3, 4], [2, -4, 1, 4, 3, -2], 2)
        return _normalise_rdm(rho)

    def env(self):
        return dict(C1=self.C1, C2=self.C2, C3=self.C3, C4=self.C4,
                    T1=self.T1, T2=self.T2, T3=self.T3, T4=self.T4)


def _normalise_rdm(rho):
    """rho / tr(rho Id2.twist(0).twist(1)) (CTM.cpp:620-627)."""
    Id2 = Tensor.identity(rho.sym, rho.cod, rho.dom)
    norm = rho.contract(Id2.twist(0).twist(1), [1, 2, 3, 4], [3, 4, 1, 2], 0).trace()
    return rho.scale(1.0 / norm)


def bond_expectation(rho, op):
    """avg for a two-site operator (LinearAlgebra.cpp:58-64):
    tr(rho.twist(0).twist(1) contracted with op)."""
    return rho.twist(0).twist(1).contract(op, [1, 2, 3, 4], [3, 4, 1, 2], 0).trace()


def heisenberg_u1(sym, phys: Qbasis, J=1.0):
    """Spin-1/2 Heisenberg bond J (Sz Sz + (S+ S- + S- S+)/2) as a U(1)
    Tensor<2,2>({phys, phys}, {phys, phys}); phys charges are 2 Sz = -1, +1
    with degeneracy 1.  Built from its dense 4x4 matrix in the product basis
    |s1 s2> (s1 fastest) by projecting onto each coupled sector."""
    sz = {-1: -0.5, 1: 0.5}
    H = Tensor(sym, [phys, phys], [phys, phys])
    for i, q in enumerate(H.sectors):
        rows = _product_states(H.cdom, q)
        cols = _product_states(H.ccod, q)
        blk = np.zeros((len(rows), len(cols)))
        for r, (a1, a2) in enumerate(rows):
            for c, (b1, b2) in enumerate(cols):
                v = 0.0
                if (a1, a2) == (b1, b2):
                    v += sz[a1] * sz[a2]
                if a1 == b2 and a2 == b1 and a1 != a2:
                    v += 0.5
                blk[r, c] = J * v
        H.blocks[i] = blk
    return H


def _product_states(cbasis, q):
    """(q1, q2) of each row of coupled sector q, in the sector's fusion-tree
    order (every degeneracy is 1 for the spin-1/2 leg)."""
    out = []
    for t in cbasis.trees[q]:
        assert all(d == 1 for d in t.dims)
        out.append(tuple(t.qu))
    return out


def _twists(T, legs):
    for l in legs:
        T = T.twist(l)
    return T


def corner_spectrum(C: Tensor):
    """Gauge-invariant fingerprint of a corner: all singular values of its
    blocks, sorted descending (for comparing environments up to gauge)."""
    out = []
    for b in C.blocks:
        if b.size:
            out.extend(np.linalg.svd(b, compute_uv=False).tolist())
    return np.array(sorted(out, reverse=True))
