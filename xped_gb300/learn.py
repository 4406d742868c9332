"""Learned sketch widths for the randomized projector SVD.

The rank predictor is trained on the spectra the CTM itself produces: a CTM
run with the exact tSVD logs, per projector decomposition and sector, the
features the width policy sees (shape and the direction's previous
spectrum) and the outcome (kept count, full spectrum).  Labels:

  y0 = log2(1 + kept)
  y1 = log2(1 + p*),  p* = the smallest p >= 1 such that the first value a
       sketch of kept + p columns does not see, s[kept + p], is at most
       RHO * s[kept - 1] (or kept + p reaches min(rows, cols)); p* = 1 for a
       sector that keeps nothing.

A policy's outcome on a logged decomposition: a sector sketched with w
columns saturates (is redone) if it keeps >= w values, and is under-resolved
if w < kept + p*.  ``compare_policies`` reports columns, saturations and
under-resolved sectors of the learned widths and of the history rule
(previous kept + max(16, 50 %))."""
from __future__ import annotations

import ctypes as C
from typing import Dict, List

import numpy as np

from ._lib import check, check_handle, lib

RHO = 0.1


class RankModel:
    """Device MLP (FP32) with Adam; forward/backward are the library's kernels."""

    def __init__(self, seed: int = 0):
        self._h = check_handle(lib().xgb_rank_model_create(int(seed)), "rank_model_create")
        self.n_params = lib().xgb_rank_model_num_params()
        self.n_features = lib().xgb_rank_model_num_features()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().xgb_rank_model_release(h)
            self._h = None

    @staticmethod
    def _f(a):
        return a.ctypes.data_as(C.POINTER(C.c_float))

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        check(lib().xgb_rank_model_get_params(self._h, self._f(out), self.n_params), "rank_model_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().xgb_rank_model_set_params(self._h, self._f(p), p.size), "rank_model_set_params")

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], 2), np.float32)
        check(lib().xgb_rank_model_predict(self._h, self._f(X), X.shape[0], self._f(Y)), "rank_model_predict")
        return Y

    def gradient(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_double()
        check(lib().xgb_rank_model_gradient(self._h, self._f(X), self._f(T), X.shape[0], self._f(g), C.byref(loss)),
              "rank_model_gradient")
        return loss.value, g

    def train(self, X, T, steps: int, lr: float = 1e-3) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = C.c_double()
        check(lib().xgb_rank_model_train(self._h, self._f(X), self._f(T), X.shape[0], int(steps), float(lr),
                                         C.byref(loss)), "rank_model_train")
        return loss.value


def oversampling_label(spectrum: np.ndarray, keep: int, kmin: int, rho: float = RHO) -> int:
    if keep <= 0:
        return 1
    last = spectrum[keep - 1]
    p = 1
    while keep + p < kmin and keep + p < len(spectrum) and spectrum[keep + p] > rho * last:
        p += 1
    return p


def dataset(records: List[Dict], rho: float = RHO):
    """(X, T) over every sector that has history (feature 2 set)."""
    X, T = [], []
    for r in records:
        for a in range(len(r["sectors"])):
            f = r["features"][a]
            if f[2] < 0.5:
                continue
            k = int(r["keep"][a])
            p = oversampling_label(r["spectrum"][a], k, int(r["kmin"][a]), rho)
            X.append(f)
            T.append([np.log2(1.0 + k), np.log2(1.0 + p)])
    return np.asarray(X, np.float32), np.asarray(T, np.float32)


def _prev_keep(records: List[Dict]):
    """Per record: {sector: kept} of the previous record of the same direction."""
    last, out = {}, []
    for r in records:
        out.append(last.get(r["dir"]))
        last[r["dir"]] = dict(zip(r["sectors"], (int(k) for k in r["keep"])))
    return out


def history_widths(records: List[Dict], oversample: int = 16, growth: float = 0.5):
    out = []
    for r, prev in zip(records, _prev_keep(records)):
        w = []
        for q in r["sectors"]:
            if prev is None or q not in prev:
                w.append(0)
            else:
                k = prev[q]
                w.append(k + max(oversample, int(np.ceil(growth * k))))
        out.append(w)
    return out


def model_widths(model: RankModel, records: List[Dict], margin: float = 0.0, min_oversample: int = 2):
    out = []
    for r in records:
        Y = model.predict(r["features"])
        w = []
        for a in range(len(r["sectors"])):
            if r["features"][a][2] < 0.5:
                w.append(0)
                continue
            k = max(0.0, 2.0 ** float(Y[a, 0]) - 1.0)
            p = max(0.0, 2.0 ** float(Y[a, 1]) - 1.0)
            w.append(int(np.ceil(k * (1.0 + margin))) + max(min_oversample, int(np.ceil(p))))
        out.append(w)
    return out


def policy_outcome(records: List[Dict], widths, rho: float = RHO):
    """Sketch columns, columns of exactly decomposed sectors (min(rows, cols)),
    saturated and under-resolved sector counts of a width assignment."""
    cols = exact_cols = sat = under = sketched = 0
    for r, w in zip(records, widths):
        for a in range(len(r["sectors"])):
            kmin = int(r["kmin"][a])
            wa = int(w[a])
            if wa <= 0 or 2 * wa >= kmin:
                exact_cols += kmin
                continue
            sketched += 1
            k = int(r["keep"][a])
            cols += wa
            if k >= wa:
                sat += 1
            elif wa < k + oversampling_label(r["spectrum"][a], k, kmin, rho):
                under += 1
    return dict(columns=cols, saturated=sat, under_resolved=under, sketched=sketched, exact_columns=exact_cols)
