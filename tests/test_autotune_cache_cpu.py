"""The autotuner's cache file: entries are keyed by the GPU's name, entries of
another GPU model and malformed lines are skipped on load, and save writes back
exactly what was loaded.  Host code only (no measurement); without a CUDA
device the library names the GPU "unknown", so the test runs where no device
is present."""
import ctypes as C

import pytest


def test_cache_is_keyed_by_gpu_name(tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present (the GPU name would not be 'unknown')")
    from xped_gb300 import lib
    L = lib()
    src = tmp_path / "cache.txt"
    # name  groups flops area k tc-allowed | tile split tc-chosen
    src.write_text("\n".join([
        "unknown 3 20 9 10 0 16 2 0",
        "unknown 4 21 9 10 1 32 0 1",
        "unknown 5 22 9 10 0 24 0 0",       # not a tile edge of the kernel: skipped
        "OTHER_GPU 3 20 9 10 0 64 1 0",     # measured on another GPU model: skipped
        "not a cache line",
    ]) + "\n")
    L.xgb_autotune_reset()
    try:
        assert L.xgb_autotune_load(str(src).encode()) == 2
        tiles, splits = (C.c_int32 * 8)(), (C.c_int32 * 8)()
        assert L.xgb_autotune_choices(tiles, splits, 8) == 2
        assert list(tiles[:2]) == [16, 0]  # 0: the FP64-accurate tensor-core form
        assert list(splits[:2]) == [2, 0]
        out = tmp_path / "saved.txt"
        assert L.xgb_autotune_save(str(out).encode()) == 0
        assert out.read_text().splitlines() == ["unknown 3 20 9 10 0 16 2 0", "unknown 4 21 9 10 1 32 0 1"]
        L.xgb_autotune_reset()
        assert L.xgb_autotune_load(str(out).encode()) == 2
        assert L.xgb_autotune_load(str(tmp_path / "missing.txt").encode()) < 0
    finally:
        L.xgb_autotune_reset()
