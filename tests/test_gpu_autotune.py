"""The FP64 grouped-GEMM tile-shape autotuner (tile edge 16/32/64 x split-K
target 0/1/2/4 waves) on two contrasting block lists: a long list of small
sector blocks and a short list of large ones.  The tuner must pick the fastest
of its own measurements, and an independent re-timing of every candidate must
agree that its pick is (within timing noise) the best; every candidate computes
the same product as numpy FP64; with autotuning on, the grouped GEMM entry
point tunes a bucket once, reuses it, and the cache survives a save / load."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lists():
    rng = np.random.default_rng(11)
    small = [tuple(int(x) for x in rng.integers(8, 49, size=3)) for _ in range(300)]
    large = [(768, 704, 832), (640, 768, 768), (512, 512, 1024)]
    return {"small_blocks": small, "large_blocks": large}


def _setup(L, blocks, seed=0):
    from xped_gb300._lib import GemmDesc
    rng = np.random.default_rng(seed)
    As, Bs, descs = [], [], []
    ao = bo = co = 0
    for (m, n, k) in blocks:
        A, B = rng.standard_normal((m, k)), rng.standard_normal((k, n))
        descs.append(GemmDesc(m, n, k, ao, m, bo, k, co, m, 0, 0))
        As.append(A); Bs.append(B)
        ao += A.size; bo += B.size; co += m * n
    bufs = []
    for h in (np.concatenate([a.ravel(order="F") for a in As]), np.concatenate([b.ravel(order="F") for b in Bs]),
              np.zeros(co)):
        p = C.c_void_p()
        assert L.xgb_malloc(C.byref(p), h.nbytes) == 0
        assert L.xgb_memcpy_h2d(p, h.ctypes.data, h.nbytes) == 0
        bufs.append(p)
    return (GemmDesc * len(descs))(*descs), bufs, As, Bs, co


def _check(L, blocks, bufs, As, Bs, co):
    out = np.empty(co)
    assert L.xgb_memcpy_d2h(out.ctypes.data, bufs[2], out.nbytes) == 0
    o = 0
    for (m, n, k), A, B in zip(blocks, As, Bs):
        ref = A @ B
        got = out[o:o + m * n].reshape((m, n), order="F")
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
        o += m * n


@pytest.mark.parametrize("which", ["small_blocks", "large_blocks"])
def test_tuner_picks_the_measured_best(which):
    from xped_gb300 import ensure_device, lib
    from xped_gb300._lib import last_error
    ensure_device(0)
    L = lib()
    blocks = _lists()[which]
    arr, bufs, As, Bs, co = _setup(L, blocks)
    ncand = L.xgb_autotune_candidates(None, None, 0)
    tiles, waves = (C.c_int32 * ncand)(), (C.c_int32 * ncand)()
    L.xgb_autotune_candidates(tiles, waves, ncand)
    times = (C.c_double * ncand)()
    best = C.c_int32()
    assert L.xgb_autotune_gemm(len(blocks), arr, bufs[0], bufs[1], times, C.byref(best)) == 0, last_error()
    t = np.array(times[:])
    # the measured fastest, or - within 3 % of it - the candidate with the largest tile, then the fewest
    # split waves (FP64-bound lists time alike on every tile edge; larger tiles mean shorter tables)
    near = [c for c in range(ncand) if t[c] <= 1.03 * t.min()]
    expect = max(near, key=lambda c: (tiles[c], -waves[c]))
    assert best.value == expect, (best.value, expect, t)
    # independent re-timing of every candidate through the public entry point (min of 3 runs, CUDA events
    # on the library stream; these times include the per-call table upload the tuner leaves out)
    re = []
    for c in range(ncand):
        run = lambda: L.xgb_grouped_gemm_f64_config(tiles[c], waves[c], len(blocks), arr, bufs[0], bufs[1], bufs[2],
                                                    1.0, 0.0, None)
        assert run() == 0, last_error()
        _check(L, blocks, bufs, As, Bs, co)
        ms = []
        for _ in range(3):
            L.xgb_synchronize()
            L.xgb_event_record(14)
            run()
            L.xgb_event_record(15)
            ms.append(L.xgb_event_elapsed_ms(14, 15))
        re.append(min(ms))
    re = np.array(re)
    print(which, "tuner pick", (tiles[best.value], waves[best.value]), "tuner ms", np.round(t, 4),
          "re-timed ms", np.round(re, 4))
    assert re[best.value] <= 1.25 * re.min() + 0.02, (re[best.value], re.min())
    for p in bufs:
        L.xgb_free(p)


def test_autotuned_entry_point_caches_and_persists(tmp_path):
    from xped_gb300 import ensure_device, lib
    from xped_gb300._lib import last_error
    ensure_device(0)
    L = lib()
    blocks = _lists()["small_blocks"]
    arr, bufs, As, Bs, co = _setup(L, blocks, seed=3)
    L.xgb_autotune_reset()
    assert L.xgb_autotune_set(1) == 0
    try:
        for _ in range(2):
            assert L.xgb_grouped_gemm(0, len(blocks), arr, bufs[0], bufs[1], bufs[2], 1.0, 0.0, None) == 0, \
                last_error()
        _check(L, blocks, bufs, As, Bs, co)
        measured, hits, ms = C.c_int64(), C.c_int64(), C.c_double()
        assert L.xgb_autotune_stats(C.byref(measured), C.byref(hits), C.byref(ms)) == 1
        assert measured.value == 1 and hits.value >= 1 and ms.value > 0
        tile, waves = (C.c_int32 * 1)(), (C.c_int32 * 1)()
        assert L.xgb_autotune_choices(tile, waves, 1) == 1
        path = str(tmp_path / "tune.txt").encode()
        assert L.xgb_autotune_save(path) == 0
        L.xgb_autotune_reset()
        assert L.xgb_autotune_load(path) == 1
        t2, w2 = (C.c_int32 * 1)(), (C.c_int32 * 1)()
        assert L.xgb_autotune_choices(t2, w2, 1) == 1
        assert (t2[0], w2[0]) == (tile[0], waves[0])
    finally:
        L.xgb_autotune_set(0)
        L.xgb_autotune_reset()
        for p in bufs:
            L.xgb_free(p)
