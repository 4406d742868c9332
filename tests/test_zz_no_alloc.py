"""The allocation-free batched SVD (xgb_batched_svd_noalloc) against the
regular entry point (xgb_batched_svd with caller-provided workspace).

The no-alloc variant serves embedders that cannot call cudaMalloc (their
host framework owns every device allocation, or their device-memory budget
is fixed up front); it takes its workspace from a fixed device array held
by the library.  Both entry points run the same kernels (a 520 x 540 block
takes the grid-wide Jacobi kernel, the others the cluster kernel), so their
outputs must agree to round-off; the variant is called twice in a row
because the shared array keeps the previous call's contents, once on the
library stream and once on a stream the caller created.  This file is named
to be collected last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cudart():
    """The CUDA runtime the native library itself loaded (for a caller-owned stream)."""
    with open("/proc/self/maps") as f:
        for line in f:
            if "libcudart.so" in line:
                return C.CDLL(line.split()[-1])
    raise RuntimeError("libcudart is not loaded")


def _alloc(L, nbytes):
    p = C.c_void_p()
    assert L.xgb_malloc(C.byref(p), max(nbytes, 8)) == 0, "xgb_malloc failed"
    return p


def test_noalloc_svd_matches_allocating_entry_point():
    from xped_gb300 import ensure_device, lib
    from xped_gb300._lib import SvdDesc, last_error

    ensure_device(0)
    L = lib()
    rng = np.random.default_rng(17)
    shapes = [(40, 40), (57, 23), (18, 61), (96, 96), (5, 5), (1, 7), (130, 130), (520, 540)]
    descs, mats = [], []
    a_off = u_off = s_off = v_off = 0
    for m, n in shapes:
        k = min(m, n)
        descs.append(SvdDesc(m, n, a_off, u_off, s_off, v_off))
        mats.append(rng.standard_normal((m, n)))
        a_off += m * n
        u_off += m * k
        s_off += k
        v_off += k * n
    arr = (SvdDesc * len(descs))(*descs)
    flat = np.concatenate([a.ravel(order="F") for a in mats])
    dA = _alloc(L, flat.nbytes)
    assert L.xgb_memcpy_h2d(dA, flat.ctypes.data, flat.nbytes) == 0
    outs = {}
    for tag in ("ref", "call1", "call2"):
        outs[tag] = (_alloc(L, 8 * u_off), _alloc(L, 8 * s_off), _alloc(L, 8 * v_off))
    wbytes = L.xgb_svd_workspace_bytes(len(descs), arr)
    dW = _alloc(L, wbytes)
    U, S, V = outs["ref"]
    assert L.xgb_batched_svd(len(descs), arr, dA, U, S, V, dW, None) == 0, last_error()
    assert L.xgb_synchronize() == 0
    rt = _cudart()
    own = C.c_void_p()
    assert rt.cudaStreamCreate(C.byref(own)) == 0
    for tag, st in (("call1", None), ("call2", own)):
        U, S, V = outs[tag]
        rc = L.xgb_batched_svd_noalloc(len(descs), arr, dA, U, S, V, st)
        assert rc == 0, last_error()
    assert rt.cudaStreamSynchronize(own) == 0
    assert rt.cudaStreamDestroy(own) == 0
    assert L.xgb_synchronize() == 0

    def host(p, n):
        h = np.empty(n)
        assert L.xgb_memcpy_d2h(h.ctypes.data, p, 8 * n) == 0
        return h

    ref = [host(outs["ref"][0], u_off), host(outs["ref"][1], s_off), host(outs["ref"][2], v_off)]
    for tag in ("call1", "call2"):
        got = [host(outs[tag][0], u_off), host(outs[tag][1], s_off), host(outs[tag][2], v_off)]
        for r, g in zip(ref, got):
            assert np.allclose(g, r, rtol=1e-12, atol=1e-12), f"{tag}: max diff {np.abs(g - r).max():.3e}"
    # and the result is a correct SVD
    S = ref[1]
    o = 0
    for A in mats:
        k = min(A.shape)
        assert np.allclose(S[o:o + k], np.linalg.svd(A, compute_uv=False), rtol=1e-10, atol=1e-12)
        o += k
    for p in [dA, dW] + [x for t in outs.values() for x in t]:
        L.xgb_free(p)


def test_noalloc_svd_rejects_batches_beyond_capacity():
    from xped_gb300 import ensure_device, lib
    from xped_gb300._lib import SvdDesc, last_error

    ensure_device(0)
    L = lib()
    cap = L.xgb_batched_svd_noalloc_capacity_bytes()
    n = 1
    while L.xgb_svd_workspace_bytes(1, (SvdDesc * 1)(SvdDesc(n, n, 0, 0, 0, 0))) <= cap:
        n *= 2
    arr = (SvdDesc * 1)(SvdDesc(n, n, 0, 0, 0, 0))
    rc = L.xgb_batched_svd_noalloc(1, arr, None, None, None, None, None)
    assert rc < 0
    assert "capacity" in last_error()
