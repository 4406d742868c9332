"""Python mirror of Xped's Tensor interface over the native GB300 backend.

Every operation is one call through the C-ABI (include/xgb_tensor.h); the
data stays in HBM.  Names and argument meaning follow the reference
(include/Xped/Core/Tensor.hpp): ``permute(shift, p)``, ``twist(leg)``,
``contract(other, a1, a2, rankres)``, ``tSVD(maxKeep, eps)``, ``tQR()``,
``maxNorm()``.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Sequence, Tuple

import numpy as np

from ._lib import (PermContrib, PermTask, GemmDesc, check, check_handle, ensure_device, lib)

SYM_IDS = {"U1": 0, "fU1": 1, "Z2": 2, "fZ2": 3, "SU2": 4}
GEMM_FORMS = {"fp64": 0, "3xtf32": 1, "bf16x9": 2, "fp32": 3, "f64tc": 4}  # XGB_PREC_* of xgb.h


def _i32(seq):
    arr = (C.c_int32 * max(len(seq), 1))(*seq)
    return arr


def _i64(seq):
    return (C.c_int64 * max(len(seq), 1))(*seq)


class Basis:
    """Qbasis<Symmetry, depth> (include/Xped/Core/Qbasis.hpp)."""

    def __init__(self, handle):
        self._h = check_handle(handle, "basis")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xgb_basis_release(h)
            self._h = None

    @classmethod
    def from_pairs(cls, sym: str, pairs: Sequence[Tuple[int, int]], sort: bool = True) -> "Basis":
        qs = [int(q) for q, _ in pairs]
        ds = [int(d) for _, d in pairs]
        return cls(lib().xgb_basis_create(SYM_IDS[sym], len(qs), _i32(qs), _i64(ds), 1 if sort else 0))

    def conj(self) -> "Basis":
        return Basis(lib().xgb_basis_conj(self._h))

    def combine(self, other: "Basis") -> "Basis":
        return Basis(lib().xgb_basis_combine(self._h, other._h))

    def forget_history(self) -> "Basis":
        return Basis(lib().xgb_basis_forget_history(self._h))

    def info(self):
        n = lib().xgb_basis_info(self._h, None, None, None, None)
        qs = (C.c_int32 * max(n, 1))()
        ds = (C.c_int64 * max(n, 1))()
        cj = C.c_int()
        dp = C.c_int()
        lib().xgb_basis_info(self._h, qs, ds, C.byref(cj), C.byref(dp))
        return list(qs[:n]), list(ds[:n]), bool(cj.value), dp.value

    @property
    def qs(self):
        return self.info()[0]

    @property
    def dims(self):
        return self.info()[1]

    def trees(self, i: int):
        """Fusion trees of irrep index i as tuples (qu, qi, qc, dims, dual_mask)."""
        need = check(lib().xgb_basis_trees(self._h, i, None, 0), "basis_trees")
        buf = (C.c_int64 * max(need, 1))()
        n = check(lib().xgb_basis_trees(self._h, i, buf, need), "basis_trees")
        out, k = [], 0
        for _ in range(n):
            r, qc, dual = buf[k], buf[k + 1], buf[k + 2]
            k += 3
            qu = tuple(buf[k:k + r]); k += r
            dims = tuple(buf[k:k + r]); k += r
            nqi = max(r - 2, 0)
            qi = tuple(buf[k:k + nqi]); k += nqi
            out.append((qu, qi, qc, dims, dual))
        return out


def _handles(bases):
    arr = (C.c_void_p * max(len(bases), 1))(*[b._h for b in bases])
    return arr


class Tensor:
    """Tensor<double, Rank, CoRank, Symmetry> with device-resident blocks."""

    def __init__(self, handle):
        self._h = check_handle(handle, "tensor")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xgb_tensor_release(h)
            self._h = None

    # -- construction ---------------------------------------------------------
    @classmethod
    def zeros(cls, dom: List[Basis], cod: List[Basis]) -> "Tensor":
        ensure_device()
        return cls(lib().xgb_tensor_zeros(len(dom), _handles(dom), len(cod), _handles(cod)))

    @classmethod
    def identity(cls, dom: List[Basis], cod: List[Basis]) -> "Tensor":
        ensure_device()
        return cls(lib().xgb_tensor_identity(len(dom), _handles(dom), len(cod), _handles(cod)))

    @classmethod
    def meta(cls, dom: List[Basis], cod: List[Basis]) -> "Tensor":
        """Metadata only, no device memory (usable without a GPU)."""
        return cls(lib().xgb_tensor_meta(len(dom), _handles(dom), len(cod), _handles(cod)))

    @classmethod
    def from_blocks(cls, dom, cod, blocks: Dict[int, np.ndarray]) -> "Tensor":
        t = cls.zeros(dom, cod)
        t.set_blocks(blocks)
        return t

    # -- metadata ----------------------------------------------------------------
    def sectors(self):
        n = lib().xgb_tensor_sectors(self._h, None, None, None)
        qs = (C.c_int32 * max(n, 1))()
        rs = (C.c_int64 * max(n, 1))()
        cs = (C.c_int64 * max(n, 1))()
        lib().xgb_tensor_sectors(self._h, qs, rs, cs)
        return list(qs[:n]), list(rs[:n]), list(cs[:n])

    @property
    def size(self) -> int:
        return int(lib().xgb_tensor_size(self._h))

    @property
    def rank(self):
        r, c = C.c_int(), C.c_int()
        lib().xgb_tensor_rank(self._h, C.byref(r), C.byref(c))
        return r.value, c.value

    def leg(self, i) -> Basis:
        return Basis(lib().xgb_tensor_leg(self._h, i))

    def coupled(self, codomain: bool) -> Basis:
        return Basis(lib().xgb_tensor_coupled(self._h, 1 if codomain else 0))

    # -- data ------------------------------------------------------------------------
    def data(self) -> np.ndarray:
        n = self.size
        out = np.empty(n, dtype=np.float64)
        check(lib().xgb_tensor_download(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), n), "download")
        return out

    def set_data(self, flat: np.ndarray):
        flat = np.ascontiguousarray(flat, dtype=np.float64)
        check(lib().xgb_tensor_upload(self._h, flat.ctypes.data_as(C.POINTER(C.c_double)), flat.size), "upload")

    def blocks(self) -> Dict[int, np.ndarray]:
        qs, rs, cs = self.sectors()
        flat = self.data()
        out, off = {}, 0
        for q, r, c in zip(qs, rs, cs):
            out[q] = flat[off:off + r * c].reshape((r, c), order="F").copy()
            off += r * c
        return out

    def to_bytes(self) -> bytes:
        """Checkpoint of this tensor (bases, sectors, data; the fields of the reference's
        StorageType_contiguous::serialize) in the library's byte layout."""
        n = C.c_int64()
        check(lib().xgb_tensor_serialize(self._h, None, 0, C.byref(n)), "tensor_serialize")
        buf = (C.c_uint8 * n.value)()
        check(lib().xgb_tensor_serialize(self._h, buf, n.value, C.byref(n)), "tensor_serialize")
        return bytes(buf)

    @staticmethod
    def from_bytes(data: bytes) -> "Tensor":
        buf = (C.c_uint8 * len(data)).from_buffer_copy(data)
        return Tensor(lib().xgb_tensor_deserialize(buf, len(data)))

    def set_blocks(self, blocks: Dict[int, np.ndarray]):
        qs, rs, cs = self.sectors()
        parts = []
        for q, r, c in zip(qs, rs, cs):
            b = np.asarray(blocks[q], dtype=np.float64)
            if b.shape != (r, c):
                raise ValueError(f"block {q}: shape {b.shape} != {(r, c)}")
            parts.append(b.ravel(order="F"))
        self.set_data(np.concatenate(parts) if parts else np.zeros(0))

    # -- operations ---------------------------------------------------------------------
    def permute(self, shift: int, p: Sequence[int]) -> "Tensor":
        return Tensor(lib().xgb_tensor_permute(self._h, int(shift), _i32(list(p)), len(p)))

    def permute_adj(self, shift: int, p: Sequence[int]) -> "Tensor":
        """Tensor::permute_adj<shift, p...>: transpose of permute on its output shape."""
        return Tensor(lib().xgb_tensor_permute_adj(self._h, int(shift), _i32(list(p)), len(p)))

    def matmul_backward(self, right: "Tensor", res_adj: "Tensor"):
        """Reverse rule of self * right: (self_adj, right_adj)."""
        la, ra = C.c_void_p(), C.c_void_p()
        check(lib().xgb_tensor_matmul_backward(self._h, right._h, res_adj._h, C.byref(la), C.byref(ra)),
              "matmul_backward")
        return Tensor(la.value), Tensor(ra.value)

    def svd_backward(self, U: "Tensor", S: "Tensor", Vdag: "Tensor", dU: "Tensor", dS: "Tensor",
                     dVdag: "Tensor") -> "Tensor":
        """Reverse rule of the per-sector SVD of self (untruncated factors)."""
        return Tensor(lib().xgb_tensor_svd_backward(self._h, U._h, S._h, Vdag._h, dU._h, dS._h, dVdag._h))

    def twist(self, leg: int) -> "Tensor":
        return Tensor(lib().xgb_tensor_twist(self._h, int(leg)))

    def adjoint(self) -> "Tensor":
        return Tensor(lib().xgb_tensor_adjoint(self._h))

    def matmul(self, other: "Tensor", adj_a=False, adj_b=False) -> "Tensor":
        return Tensor(lib().xgb_tensor_matmul(self._h, other._h, int(adj_a), int(adj_b)))

    def __mul__(self, other):
        if isinstance(other, Tensor):
            return self.matmul(other)
        return Tensor(lib().xgb_tensor_scale(self._h, float(other)))

    def contract(self, other: "Tensor", a1: Sequence[int], a2: Sequence[int], rankres: int) -> "Tensor":
        return Tensor(lib().xgb_tensor_contract(self._h, other._h, _i32(list(a1)), len(a1), _i32(list(a2)), len(a2),
                                                int(rankres)))

    def maxNorm(self) -> float:
        v = lib().xgb_tensor_max_norm(self._h)
        if v < 0:
            check(-3, "maxNorm")
        return v

    def normalize_max(self) -> "Tensor":
        return Tensor(lib().xgb_tensor_normalize_max(self._h))

    def tSVD(self, max_keep: int, eps_svd: float, preserve_multiplets: bool = False):
        U, S, V = C.c_void_p(), C.c_void_p(), C.c_void_p()
        tw, ent = C.c_double(), C.c_double()
        n = len(self.sectors()[0])
        keep = (C.c_int32 * max(n, 1))()
        check(lib().xgb_tensor_tsvd(self._h, int(max_keep), float(eps_svd), int(preserve_multiplets), C.byref(U),
                                    C.byref(S), C.byref(V), C.byref(tw), C.byref(ent), keep), "tSVD")
        return Tensor(U.value), Tensor(S.value), Tensor(V.value), tw.value, ent.value, list(keep[:n])

    def svspec(self):
        """SVspec of Tensor::tSVD with RETURN_SPEC (src/Core/Tensor.cpp:618-624) for a singular-value tensor
        returned by tSVD: {charge: kept values, descending}."""
        n = check(lib().xgb_tensor_svspec(self._h, None, None, None, 0), "svspec")
        qs = (C.c_int32 * max(n, 1))()
        begin = (C.c_int64 * (n + 1))()
        lib().xgb_tensor_svspec(self._h, qs, begin, None, 0)
        vals = np.zeros(max(begin[n], 1))
        check(lib().xgb_tensor_svspec(self._h, qs, begin, vals.ctypes.data_as(C.POINTER(C.c_double)), begin[n]),
              "svspec")
        return {int(qs[i]): vals[begin[i]:begin[i + 1]].copy() for i in range(n)}

    def tSVD_randomized(self, max_keep: int, eps_svd: float, sketch: Sequence[int], power_iters: int = 1,
                        seed: int = 0, warm: "Tensor" = None, res_tol: float = 0.0):
        """Randomized blockwise tSVD: ``sketch[i]`` Gaussian columns for sector i
        (<= 0: exact).  Returns (U, S, V, truncWeight, entropy, keep, width,
        n_saturated)."""
        U, S, V = C.c_void_p(), C.c_void_p(), C.c_void_p()
        tw, ent = C.c_double(), C.c_double()
        n = len(self.sectors()[0])
        if len(sketch) != n:
            raise ValueError("one sketch width per sector required")
        keep = (C.c_int32 * max(n, 1))()
        width = (C.c_int64 * max(n, 1))()
        nsat = C.c_int32()
        sk = (C.c_int64 * max(n, 1))(*[int(x) for x in sketch])
        check(lib().xgb_tensor_tsvd_randomized(self._h, int(max_keep), float(eps_svd), n, sk, int(power_iters),
                                               int(seed), warm._h if warm is not None else None, float(res_tol),
                                               C.byref(U),
                                               C.byref(S), C.byref(V), C.byref(tw),
                                               C.byref(ent), keep, width, C.byref(nsat)), "tSVD_randomized")
        return (Tensor(U.value), Tensor(S.value), Tensor(V.value), tw.value, ent.value, list(keep[:n]),
                list(width[:n]), nsat.value)

    def tQR(self):
        Q, R = C.c_void_p(), C.c_void_p()
        check(lib().xgb_tensor_tqr(self._h, C.byref(Q), C.byref(R)), "tQR")
        return Tensor(Q.value), Tensor(R.value)

    # -- host-only planning -----------------------------------------------------------------
    def permute_plan(self, shift: int, p: Sequence[int], twist_mask: int = 0):
        nt, nc = C.c_int(), C.c_int()
        pp = _i32(list(p))
        check(lib().xgb_permute_plan_host(self._h, int(shift), pp, len(p), twist_mask, C.byref(nt), C.byref(nc), None,
                                          0, None, 0, None), "permute_plan")
        tasks = (PermTask * max(nt.value, 1))()
        contribs = (PermContrib * max(nc.value, 1))()
        out = C.c_void_p()
        check(lib().xgb_permute_plan_host(self._h, int(shift), pp, len(p), twist_mask, C.byref(nt), C.byref(nc), tasks,
                                          nt.value, contribs, nc.value, C.byref(out)), "permute_plan")
        return list(tasks[:nt.value]), list(contribs[:nc.value]), Tensor(out.value)

    def gemm_plan(self, other: "Tensor", adj_a=False, adj_b=False):
        n = C.c_int()
        check(lib().xgb_gemm_plan_host(self._h, int(adj_a), other._h, int(adj_b), C.byref(n), None, 0, None), "gemm_plan")
        descs = (GemmDesc * max(n.value, 1))()
        out = C.c_void_p()
        check(lib().xgb_gemm_plan_host(self._h, int(adj_a), other._h, int(adj_b), C.byref(n), descs, n.value,
                                       C.byref(out)), "gemm_plan")
        return list(descs[:n.value]), Tensor(out.value)


def decompose(T1: Tensor, T2: Tensor, max_nsv: int):
    """decompose (src/PEPS/PEPSContractions.cpp:16-43)."""
    P1, P2 = C.c_void_p(), C.c_void_p()
    check(lib().xgb_decompose(T1._h, T2._h, int(max_nsv), C.byref(P1), C.byref(P2)), "decompose")
    return Tensor(P1.value), Tensor(P2.value)


def contract_perms(a1, rank1, a2, rank2, rankres):
    out = (C.c_int32 * (len(a1) + len(a2) + 16))()
    nres = check(lib().xgb_contract_perms(_i32(list(a1)), len(a1), rank1, _i32(list(a2)), len(a2), rank2, rankres, out),
                 "contract_perms")
    v = list(out)
    k = 0
    p1 = v[k:k + len(a1)]; k += len(a1)
    s1 = v[k]; k += 1
    p2 = v[k:k + len(a2)]; k += len(a2)
    s2 = v[k]; k += 1
    pres = v[k:k + nres]; k += nres
    sres = v[k]
    return p1, s1, p2, s2, pres, sres


class SimpleUpdate:
    """Simple-update imaginary-time evolution of an iPEPS with nearest-neighbour
    gates (TimePropagator::t_step, src/PEPS/TimePropagator.cpp:7-215;
    SimpleUpdate::renormalize, src/PEPS/SimpleUpdate.cpp:5-14), all tensor work on
    the GPU.  ``pattern``: data[x][y] site labels of the unit cell (the reference's
    Pattern; neighbours must differ, e.g. [[0, 1], [1, 0]]); ``Gs[label]``:
    Tensor<2,3> (left, top | right, bottom, phys); D: kept bond dimension; gates:
    Tensor<2,2> on (phys, phys)."""

    SLOTS = {"G": 0, "wh": 1, "wv": 2, "A": 3}

    def __init__(self, pattern: Sequence[Sequence[int]], Gs: Sequence[Tensor], D: int):
        Lx, Ly = len(pattern), len(pattern[0])
        labels = (C.c_int * (Lx * Ly))(*[int(pattern[x][y]) for x in range(Lx) for y in range(Ly)])
        hs = (C.c_void_p * len(Gs))(*[g._h for g in Gs])
        self._h = check_handle(lib().xgb_su_create(Lx, Ly, labels, len(Gs), hs, int(D)), "su_create")
        self.Lx, self.n = Lx, len(Gs)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xgb_su_release(h)
            self._h = None

    def step(self, Uh: Tensor, Uv: Tensor):
        """t_step: horizontal bonds of every site, vertical, vertical reversed, horizontal reversed."""
        check(lib().xgb_su_step(self._h, Uh._h, Uv._h), "su_step")
        return self

    def step_h(self, x: int, y: int, Uh: Tensor):
        check(lib().xgb_su_step_h(self._h, int(x), int(y), Uh._h), "su_step_h")
        return self

    def step_v(self, x: int, y: int, Uv: Tensor):
        check(lib().xgb_su_step_v(self._h, int(x), int(y), Uv._h), "su_step_v")
        return self

    def get(self, name: str, site: int = 0) -> Tensor:
        """"G", "wh", "wv" of label ``site``, or "A": the site tensor at coords(site) with
        sqrt weights on its four legs."""
        return Tensor(check_handle(lib().xgb_su_get(self._h, self.SLOTS[name], int(site)), "su_get"))


class CTM:
    """CTM<double, Sym, TRank=2, ALL_OUT_LEGS=false> on a 1x1 unit cell
    (src/PEPS/CTM.cpp), all tensor work on the GPU."""

    SLOTS = {"C1": 0, "C2": 1, "C3": 2, "C4": 3, "T1": 4, "T2": 5, "T3": 6, "T4": 7, "A": 8, "Adag": 9}

    def __init__(self, A: Tensor, chi: int):
        self._h = check_handle(lib().xgb_ctm_create(A._h, int(chi)), "ctm_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xgb_ctm_release(h)
            self._h = None

    def init(self):
        check(lib().xgb_ctm_init(self._h), "ctm_init")
        return self

    def grow_all(self):
        check(lib().xgb_ctm_grow_all(self._h), "grow_all")
        return self

    def move(self, d: str):
        check(lib().xgb_ctm_move(self._h, d.encode()), "ctm_move")

    def get(self, name: str) -> Tensor:
        return Tensor(lib().xgb_ctm_get(self._h, self.SLOTS[name]))

    def to_bytes(self) -> bytes:
        """Checkpoint of chi and the environment C1..C4, T1..T4 (the reference's CTM::serialize fields)."""
        n = C.c_int64()
        check(lib().xgb_ctm_serialize(self._h, None, 0, C.byref(n)), "ctm_serialize")
        buf = (C.c_uint8 * n.value)()
        check(lib().xgb_ctm_serialize(self._h, buf, n.value, C.byref(n)), "ctm_serialize")
        return bytes(buf)

    @classmethod
    def from_bytes(cls, A: Tensor, data: bytes) -> "CTM":
        """A CTM for site tensor A resumed from a checkpoint (projector-SVD settings are not part of it)."""
        buf = (C.c_uint8 * len(data)).from_buffer_copy(data)
        obj = cls.__new__(cls)
        obj._h = check_handle(lib().xgb_ctm_deserialize(A._h, buf, len(data)), "ctm_deserialize")
        return obj

    def set(self, name: str, t: Tensor):
        check(lib().xgb_ctm_set(self._h, self.SLOTS[name], t._h), "ctm_set")

    def env(self):
        return {k: self.get(k) for k in ("C1", "C2", "C3", "C4", "T1", "T2", "T3", "T4")}

    # -- projector SVD form, statistics, decomposition log --------------------------------
    def set_svd(self, mode: str = "exact", power_iters: int = 3, seed: int = 1, oversample: int = 16,
                growth: float = 0.5):
        """``mode`` "exact" (full FP64 tSVD) or "randomized" (sketch widths from the
        direction's last kept counts + max(oversample, growth * kept))."""
        m = {"exact": 0, "randomized": 1}[mode]
        check(lib().xgb_ctm_set_svd(self._h, m, int(power_iters), int(seed), int(oversample), float(growth)),
              "ctm_set_svd")
        return self

    def set_sketch_unseen(self, on: bool = True):
        """Sketch (instead of decomposing exactly) the sectors a direction has not seen yet."""
        check(lib().xgb_ctm_set_sketch_unseen(self._h, int(on)), "ctm_set_sketch_unseen")
        return self

    def set_sketch_precision(self, fp64_tail: int = 2):
        """Run the first sketch product and all but the last fp64_tail subspace
        iterations of the randomized projector SVD as 3xTF32 tensor-core GEMMs
        (negative: every product FP64, the default)."""
        check(lib().xgb_ctm_set_sketch_precision(self._h, int(fp64_tail)), "ctm_set_sketch_precision")
        return self

    def set_warm_start(self, warm_iters: int = 2):
        """Seed each randomized projector SVD with the direction's previous V^dag and
        run warm_iters subspace iterations (negative: off)."""
        check(lib().xgb_ctm_set_warm_start(self._h, int(warm_iters)), "ctm_set_warm_start")
        return self

    def set_residual_tol(self, tol: float):
        """Kept randomized triplets must satisfy ||A v - s u|| <= tol * s_max (0: off)."""
        check(lib().xgb_ctm_set_residual_tol(self._h, float(tol)), "ctm_set_residual_tol")
        return self

    def residual_stats(self):
        n, r = C.c_int64(), C.c_double()
        check(lib().xgb_ctm_residual_stats(self._h, C.byref(n), C.byref(r)), "ctm_residual_stats")
        return {"refinements": n.value, "max_residual": r.value}

    def set_gemm(self, precision: str = "fp64"):
        """Block GEMMs of the corner contractions / renormalisation: "fp64", "3xtf32" (tensor cores)
        or "fp32"; "f64tc" (FP64-accurate tensor-core form from exact BF16 slices) also takes the
        projector products and the randomized SVD's sketch products to the tensor cores."""
        check(lib().xgb_ctm_set_gemm_precision(self._h, GEMM_FORMS[precision]), "ctm_set_gemm")
        return self

    def set_rank_model(self, model, margin: float = 0.0, min_oversample: int = 2, power_iters: int = 3,
                       seed: int = 1):
        """Randomized projector SVD with widths predicted by a trained RankModel."""
        self._model = model  # keep the model alive as long as the CTM uses it
        check(lib().xgb_ctm_set_rank_model(self._h, model._h, float(margin), int(min_oversample), int(power_iters),
                                           int(seed)), "ctm_set_rank_model")
        return self

    def stats(self):
        out = (C.c_int64 * 5)()
        check(lib().xgb_ctm_stats(self._h, out), "ctm_stats")
        return dict(zip(("decompositions", "sketched_sectors", "exact_sectors", "redo", "sketch_cols"), out))

    def set_concurrent(self, on: bool = True):
        """Run the left/right and the top/bottom moves of grow_all two at a time on two streams (the
        default; randomized projector SVD only).  The result equals the sequential order's."""
        check(lib().xgb_ctm_set_concurrent(self._h, int(on)), "ctm_set_concurrent")
        return self

    def record(self, on: bool = True):
        check(lib().xgb_ctm_record(self._h, int(on)), "ctm_record")
        return self

    def records(self):
        """Logged projector decompositions: dicts with dir, sectors, features
        (n x F float32), keep, width, kmin, spectrum (list of per-sector arrays)."""
        out = []
        L = lib()
        for i in range(L.xgb_ctm_record_count(self._h)):
            d, n, ns = C.c_int(), C.c_int(), C.c_int64()
            check(L.xgb_ctm_record_get(self._h, i, C.byref(d), C.byref(n), C.byref(ns), None, None, None, None, None,
                                       None, None), "ctm_record_get")
            k = n.value
            sec = np.zeros(k, np.int32)
            feats = np.zeros(k * FEATURES, np.float32)
            keep = np.zeros(k, np.int64)
            width = np.zeros(k, np.int64)
            kmin = np.zeros(k, np.int64)
            spec = np.zeros(max(ns.value, 1))
            sb = np.zeros(k + 1, np.int64)
            f = lambda a, t: a.ctypes.data_as(C.POINTER(t))
            check(L.xgb_ctm_record_get(self._h, i, None, None, None, f(sec, C.c_int32), f(feats, C.c_float),
                                       f(keep, C.c_int64), f(width, C.c_int64), f(kmin, C.c_int64),
                                       f(spec, C.c_double), f(sb, C.c_int64)), "ctm_record_get")
            out.append(dict(dir=d.value, sectors=sec.tolist(), features=feats.reshape(k, FEATURES), keep=keep,
                            width=width, kmin=kmin, spectrum=[spec[sb[a]:sb[a + 1]].copy() for a in range(k)]))
        return out

    # -- observables ------------------------------------------------------------------------
    def rdm_h(self) -> Tensor:
        return Tensor(lib().xgb_ctm_rdm(self._h, 0))

    def rdm_v(self) -> Tensor:
        return Tensor(lib().xgb_ctm_rdm(self._h, 1))

    def solve(self, H: Tensor, tol_E: float = 1e-10, max_steps: int = 100):
        """CTMSolver::solve (src/PEPS/CTMSolver.cpp:50-80): grow_all until the bond energy per site
        changes by less than tol_E (or oscillates within it).  Returns a dict with the final
        energy, the steps run, whether it converged / stopped on oscillation and every step's energy."""
        E, steps, flags = C.c_double(), C.c_int(), C.c_int()
        buf = (C.c_double * max(max_steps, 1))()
        check(lib().xgb_ctm_solve(self._h, H._h, float(tol_E), int(max_steps), C.byref(E), C.byref(steps),
                                  C.byref(flags), buf, max_steps), "ctm_solve")
        return {"E": E.value, "steps": steps.value, "converged": bool(flags.value & 1),
                "oscillation": bool(flags.value & 2), "energies": list(buf[:steps.value])}


FEATURES = 8  # per-sector inputs of the rank predictor


def set_gemm_precision(precision: str = "fp64"):
    """Precision form of matmul / contract block GEMMs on this thread: "fp64", "3xtf32", "bf16x9", "fp32"
    or "f64tc" (FP64-accurate, exact BF16 slices on the tensor cores)."""
    check(lib().xgb_set_gemm_precision(GEMM_FORMS[precision]), "set_gemm_precision")


def bond_expectation(rho: Tensor, op: Tensor) -> float:
    out = C.c_double()
    check(lib().xgb_tensor_bond_expectation(rho._h, op._h, C.byref(out)), "bond_expectation")
    return out.value
