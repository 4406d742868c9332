"""CPU restatement of Xped's simple-update imaginary-time step (test
infrastructure: only the tests, the smoke check and the bench's CPU legs use
it).

An iPEPS unit cell given by a pattern of site labels (Pattern, with
periodic wrapping), one site tensor G per label (Tensor<2,3>: left, top |
right, bottom, phys) and one horizontal / vertical bond weight per label
(Tensor<1,1>, diagonal; whs(x, y) sits on the right leg of site (x, y),
wvs(x, y) on its top leg); nearest-neighbour gates, the same on every bond.
The reference requires neighbouring sites to carry different labels
(TimePropagator.cpp:86-87, 93-94), e.g. the checkerboard [[0, 1], [1, 0]].

Follows
  Pattern::index / coords / uniqueIndex src/PEPS/Pattern.cpp:8-80
  TimePropagator::t_step            src/PEPS/TimePropagator.cpp:7-110 (no diagonal terms, 83-109)
  TimePropagator::t_step_h          src/PEPS/TimePropagator.cpp:112-186
  TimePropagator::t_step_v          src/PEPS/TimePropagator.cpp:188-215
  SimpleUpdate::renormalize         src/PEPS/SimpleUpdate.cpp:5-14  (bond.tSVD(D, 1e-14))
  applyWeights                      src/PEPS/PEPSContractions.cpp:93-104
  iPEPS::initWeightTensors          src/PEPS/iPEPS.cpp:575-592     (identity weights)
  iPEPS::updateAtensors             src/PEPS/iPEPS.cpp:594-603
  iPEPS::Id_weight_h / Id_weight_v  src/PEPS/iPEPS.cpp:605-615
The gates U_h / U_v are inputs (the reference forms them as mexp(-dt H) of
the bond Hamiltonian, TimePropagator.cpp:453-487; ``gate`` below)."""
from __future__ import annotations

from typing import List, Sequence

from .tensor import Tensor

# tSVD(std::numeric_limits<std::size_t>::max(), 0.) keeps every singular value
KEEP_ALL = 1 << 62


def apply_weights(A: Tensor, wL: Tensor, wT: Tensor, wR: Tensor, wB: Tensor) -> Tensor:
    """applyWeights (PEPSContractions.cpp:93-104): weights on the left, top,
    right and bottom legs of a Tensor<2,3>; the left and top weights twisted
    on their second leg."""
    return (A.contract(wL.twist(1), [1, -2, -3, -4, -5], [-1, 1], 2)
             .contract(wT.twist(1), [-1, 1, -3, -4, -5], [-2, 1], 2)
             .contract(wR, [-1, -2, 1, -4, -5], [1, -3], 2)
             .contract(wB, [-1, -2, -3, 1, -5], [1, -4], 2))


class Pattern:
    """Pattern (Pattern.cpp): data[x][y] labels, Lx = len(data), Ly = len(data[0]);
    index(x, y) = x + y Lx after periodic wrapping; coords(i) = (i % Lx, i // Lx)."""

    def __init__(self, data: Sequence[Sequence[int]]):
        self.data = [list(r) for r in data]
        self.Lx, self.Ly = len(self.data), len(self.data[0])
        self.n = len({v for r in self.data for v in r})

    def label(self, x: int, y: int) -> int:
        return self.data[x % self.Lx][y % self.Ly]

    def coords(self, i: int):
        return i % self.Lx, i // self.Lx


def _identity_like(w: Tensor) -> Tensor:
    return Tensor.identity(w.sym, w.dom, w.cod)


class SimpleUpdate:
    """Simple-update state: per label a site tensor G and the weights wh, wv."""

    def __init__(self, pattern: Sequence[Sequence[int]], Gs: List[Tensor], D: int):
        self.pat = Pattern(pattern)
        assert len(Gs) == self.pat.n
        self.D = int(D)
        self.G = list(Gs)
        s = Gs[0].sym
        self.wh = [Tensor.identity(s, [g.cod[0]], [g.cod[0]]) for g in Gs]  # right leg
        self.wv = [Tensor.identity(s, [g.dom[1]], [g.dom[1]]) for g in Gs]  # top leg

    def _u(self, x, y):
        return self.pat.label(x, y)

    def step_h(self, x: int, y: int, Uh: Tensor):
        """t_step_h (TimePropagator.cpp:112-186) for the bond (x, y) - (x+1, y)."""
        u = self._u
        G, wh, wv = self.G, self.wh, self.wv
        left_full = apply_weights(G[u(x, y)], wh[u(x - 1, y)], wv[u(x, y)], wh[u(x, y)].diag_sqrt(), wv[u(x, y + 1)])
        right_full = apply_weights(G[u(x + 1, y)], wh[u(x, y)].diag_sqrt(), wv[u(x + 1, y)], wh[u(x + 1, y)],
                                   wv[u(x + 1, y + 1)])
        left, tmp_l, bond_l, _, _ = left_full.permute(-1, [0, 1, 3, 2, 4]).tsvd(KEEP_ALL, 0.0)
        bond_l = tmp_l * bond_l
        bond_r, tmp_r, right, _, _ = right_full.permute(0, [0, 4, 1, 2, 3]).tsvd(KEEP_ALL, 0.0)
        bond_r = bond_r * tmp_r
        bond = bond_l.contract(bond_r, [-1, 1, -2], [1, -3, -4], 2)
        enlarged = Uh.twist(0).twist(1).contract(bond, [1, 2, -1, -3], [-2, 1, 2, -4], 2)
        bond_lp, weight, bond_rp, _, _ = enlarged.tsvd(self.D, 1.0e-14)
        wh[u(x, y)] = weight.scale(1.0 / weight.max_norm())
        idh = _identity_like(wh[u(x, y)])
        g1 = left.contract(bond_lp, [-1, -2, -4, 1], [-5, 1, -3], 2)
        G[u(x, y)] = apply_weights(g1, wh[u(x - 1, y)].diag_inv(), wv[u(x, y)].diag_inv(), idh,
                                   wv[u(x, y + 1)].diag_inv())
        g1 = bond_rp.contract(right, [-1, -5, 1], [1, -2, -3, -4], 2)
        G[u(x + 1, y)] = apply_weights(g1, idh, wv[u(x + 1, y)].diag_inv(), wh[u(x + 1, y)].diag_inv(),
                                       wv[u(x + 1, y + 1)].diag_inv())

    def step_v(self, x: int, y: int, Uv: Tensor):
        """t_step_v (TimePropagator.cpp:188-215) for the bond (x, y-1) - (x, y)."""
        u = self._u
        G, wh, wv = self.G, self.wh, self.wv
        top_full = apply_weights(G[u(x, y - 1)], wh[u(x - 1, y - 1)], wv[u(x, y - 1)], wh[u(x, y - 1)],
                                 wv[u(x, y)].diag_sqrt())
        bottom_full = apply_weights(G[u(x, y)], wh[u(x - 1, y)], wv[u(x, y)].diag_sqrt(), wh[u(x, y)], wv[u(x, y + 1)])
        top, tmp_t, bond_t, _, _ = top_full.permute(-1, [0, 1, 2, 3, 4]).tsvd(KEEP_ALL, 0.0)
        bond_t = tmp_t * bond_t
        bond_b, tmp_b, bottom, _, _ = bottom_full.permute(0, [1, 4, 0, 2, 3]).tsvd(KEEP_ALL, 0.0)
        bond_b = bond_b * tmp_b
        bond = bond_t.contract(bond_b, [-1, 1, -2], [1, -3, -4], 2)
        enlarged = Uv.twist(0).twist(1).contract(bond, [1, 2, -1, -3], [-2, 1, 2, -4], 2)
        bond_tp, weight, bond_bp, _, _ = enlarged.tsvd(self.D, 1.0e-14)
        wv[u(x, y)] = weight.scale(1.0 / weight.max_norm())
        idv = _identity_like(wv[u(x, y)])
        g1 = top.contract(bond_tp, [-1, -2, -3, 1], [-5, 1, -4], 2)
        G[u(x, y - 1)] = apply_weights(g1, wh[u(x - 1, y - 1)].diag_inv(), wv[u(x, y - 1)].diag_inv(),
                                       wh[u(x, y - 1)].diag_inv(), idv)
        g1 = bond_bp.contract(bottom, [-2, -5, 1], [1, -1, -3, -4], 2)
        G[u(x, y)] = apply_weights(g1, wh[u(x - 1, y)].diag_inv(), idv, wh[u(x, y)].diag_inv(),
                                   wv[u(x, y + 1)].diag_inv())

    def step(self, Uh: Tensor, Uv: Tensor):
        """t_step with nearest-neighbour terms only (TimePropagator.cpp:83-109): horizontal
        bonds of every unique site, vertical ones, vertical in reverse, horizontal in reverse."""
        n = self.pat.n
        for i in range(n):
            self.step_h(*self.pat.coords(i), Uh)
        for i in range(n):
            self.step_v(*self.pat.coords(i), Uv)
        for i in reversed(range(n)):
            self.step_v(*self.pat.coords(i), Uv)
        for i in reversed(range(n)):
            self.step_h(*self.pat.coords(i), Uh)
        return self

    def site_tensor(self, i: int) -> Tensor:
        """iPEPS::updateAtensors (iPEPS.cpp:594-603) for the site at coords(i)."""
        x, y = self.pat.coords(i)
        u = self._u
        return apply_weights(self.G[u(x, y)], self.wh[u(x - 1, y)].diag_sqrt(), self.wv[u(x, y)].diag_sqrt(),
                             self.wh[u(x, y)].diag_sqrt(), self.wv[u(x, y + 1)].diag_sqrt())


def gate(H: Tensor, tau: float) -> Tensor:
    """exp(-tau H) of a bond operator Tensor<2,2>, block by block (TimePropagator::initU,
    TimePropagator.cpp:453-487, with PlainInterface mexp): the operator maps each coupled
    sector to itself, so its exponential is the exponential of every block."""
    import scipy.linalg as sla
    out = Tensor(H.sym, H.dom, H.cod, fill=False)
    for q, b in zip(H.sectors, H.blocks):
        out.push_back(q, sla.expm(-tau * b))
    return out
