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


def sector_features(rows, cols, chi: int, hist=None) -> np.ndarray:
    """The predictor's 8 features per sector, as the native ``sector_features``
    (tensor.cpp) computes them in the CTM, for matrices decomposed outside it.
    ``hist[i]`` is None (no history) or a dict with the sector's previous
    ``keep``, ``s_first`` (largest value), ``s_last`` (last kept, 0 if none),
    ``s_next`` (first dropped, 0 if none) and the matrix's ``s_max``."""
    n = len(rows)
    X = np.zeros((n, 8), np.float32)

    def lg10(x, floor_):
        return max(np.log10(x), floor_) if x > 0 else floor_

    for i in range(n):
        X[i, 0] = np.log2(1.0 + rows[i]) / 12.0
        X[i, 1] = np.log2(1.0 + cols[i]) / 12.0
        X[i, 7] = np.log2(1.0 + chi) / 8.0
        h = None if hist is None else hist[i]
        if h is None:
            continue
        smax = h["s_max"] if h["s_max"] > 0 else 1.0
        X[i, 2] = 1.0
        X[i, 3] = np.log2(1.0 + h["keep"]) / 8.0
        X[i, 4] = lg10(h["s_first"] / smax, -16.0) / 16.0
        X[i, 5] = lg10(h["s_last"] / smax, -16.0) / 16.0
        X[i, 6] = (lg10(h["s_next"] / max(h["s_last"], 1e-300), -8.0) if h["keep"] > 0 and h["s_next"] > 0
                   else -8.0) / 8.0
    return X


def history_from_spectra(spectra, keep):
    """Per-sector history dicts (see ``sector_features``) from full descending
    spectra and kept counts."""
    smax = max((float(s[0]) for s in spectra if len(s)), default=0.0)
    out = []
    for s, k in zip(spectra, keep):
        k = int(k)
        out.append(dict(keep=k, s_first=float(s[0]) if len(s) else 0.0, s_last=float(s[k - 1]) if k > 0 else 0.0,
                        s_next=float(s[k]) if k < len(s) else 0.0, s_max=smax))
    return out


def widths_from_prediction(Y: np.ndarray, margin: float = 0.0, min_oversample: int = 2):
    """Sketch widths from predicted (log2(1+keep), log2(1+p)) rows, the rule
    ``MlpPolicy`` applies in the CTM."""
    w = []
    for y0, y1 in np.asarray(Y, np.float64):
        k = max(0.0, 2.0 ** y0 - 1.0)
        p = max(0.0, 2.0 ** y1 - 1.0)
        w.append(int(np.ceil(k * (1.0 + margin))) + max(min_oversample, int(np.ceil(p))))
    return w
