"""Split-precision (3xTF32) tensor-core grouped GEMM against FP64.

Error measure (per block): ||C - C_ref||_F / ||C_ref||_F with C_ref the
FP64 product; 3xTF32 with FP32 accumulation is expected near 1e-6, the
bound asserted is 2e-5 (K up to 512).  The tensor-memory accumulator is
restarted every 32-wide K slice and the slices are summed in FP32 registers,
so the error does not grow with k: 2e-6 is asserted at k = 3072."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PREC_3XTF32 = 1


def _run(blocks, alpha=1.0, beta=0.0, seed=0, prec=PREC_3XTF32):
    from xped_gb300 import ensure_device, lib
    from xped_gb300._lib import GemmDesc, last_error
    ensure_device(0)
    L = lib()
    rng = np.random.default_rng(seed)
    As, Bs, Cs, descs = [], [], [], []
    ao = bo = co = 0
    for (m, n, k, ta, tb) in blocks:
        A = rng.standard_normal((k, m) if ta else (m, k))
        B = rng.standard_normal((n, k) if tb else (k, n))
        Cm = rng.standard_normal((m, n))
        descs.append(GemmDesc(m, n, k, ao, A.shape[0], bo, B.shape[0], co, m, ta, tb))
        As.append(A); Bs.append(B); Cs.append(Cm)
        ao += A.size; bo += B.size; co += Cm.size
    fa = np.concatenate([a.ravel(order="F") for a in As])
    fb = np.concatenate([b.ravel(order="F") for b in Bs])
    fc = np.concatenate([c.ravel(order="F") for c in Cs])
    ptrs = []
    for h in (fa, fb, fc):
        p = C.c_void_p()
        assert L.xgb_malloc(C.byref(p), max(h.nbytes, 8)) == 0
        assert L.xgb_memcpy_h2d(p, h.ctypes.data, h.nbytes) == 0
        ptrs.append(p)
    arr = (GemmDesc * len(descs))(*descs)
    rc = L.xgb_grouped_gemm(prec, len(descs), arr, ptrs[0], ptrs[1], ptrs[2], alpha, beta, None)
    assert rc == 0, last_error()
    assert L.xgb_gemm_tc_status() == 0, last_error()
    out = np.empty_like(fc)
    assert L.xgb_memcpy_d2h(out.ctypes.data, ptrs[2], out.nbytes) == 0
    for p in ptrs:
        L.xgb_free(p)
    errs, o = [], 0
    for (m, n, k, ta, tb), A, B, Cm in zip(blocks, As, Bs, Cs):
        ref = alpha * ((A.T if ta else A) @ (B.T if tb else B)) + beta * Cm
        got = out[o:o + m * n].reshape((m, n), order="F")
        o += m * n
        errs.append(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300))
    return max(errs)


def test_single_tile():
    assert _run([(128, 128, 32, 0, 0)]) < 2e-5


def test_ragged_blocks_and_transposes():
    rng = np.random.default_rng(3)
    blocks = []
    for _ in range(40):
        m, n, k = (int(np.exp(rng.uniform(np.log(8), np.log(512)))) for _ in range(3))
        blocks.append((m, n, k, int(rng.integers(0, 2)), int(rng.integers(0, 2))))
    assert _run(blocks, seed=4) < 2e-5


@pytest.mark.parametrize("prec", [PREC_3XTF32, 2])
def test_long_k_error_does_not_grow(prec):
    """k = 3072 (96 slices), the reduction length of the SU(2) Tensor<2,2> product blocks:
    a single FP32 tensor-memory accumulator over the whole range drifted to 3e-5."""
    err = _run([(256, 192, 3072, 0, 0), (130, 70, 2000, 1, 0)], seed=9, prec=prec)
    print("long-k relative error", prec, err)
    assert err < 2e-6


def test_alpha_beta_and_empty_k():
    assert _run([(70, 130, 45, 0, 1), (33, 17, 0, 0, 0), (256, 64, 300, 1, 0)], alpha=-0.5, beta=2.0, seed=5) < 2e-5


def test_fp64_entry_unchanged():
    assert _run([(100, 90, 80, 1, 1), (8, 8, 8, 0, 0)], prec=0, seed=6) < 1e-13


PREC_FP32 = 3


@pytest.mark.parametrize("seed", [7, 8])
def test_fp32_form_ragged_blocks(seed):
    """FP32 form (operands rounded to FP32, FP32 accumulation on the CUDA
    cores): relative error ~1e-7 sqrt(k); bound 2e-5 for k up to 512."""
    rng = np.random.default_rng(seed)
    blocks = []
    for _ in range(30):
        m, n, k = (int(np.exp(rng.uniform(np.log(8), np.log(512)))) for _ in range(3))
        blocks.append((m, n, k, int(rng.integers(0, 2)), int(rng.integers(0, 2))))
    blocks.append((33, 17, 0, 0, 0))
    err = _run(blocks, alpha=1.5, beta=-0.5, seed=seed, prec=PREC_FP32)
    assert 0.0 < err < 2e-5  # rounded (not FP64) and within the FP32 budget


def test_unknown_form_is_rejected():
    from xped_gb300 import ensure_device, lib
    from xped_gb300._lib import GemmDesc
    ensure_device(0)
    arr = (GemmDesc * 1)(GemmDesc(8, 8, 8, 0, 8, 0, 8, 0, 8, 0, 0))
    assert lib().xgb_grouped_gemm(7, 1, arr, None, None, None, 1.0, 0.0, None) == -7  # XGB_E_UNSUPPORTED


PREC_BF16X9 = 2


@pytest.mark.parametrize("seed", [11, 12])
def test_bf16x9_form_ragged_blocks(seed):
    """BF16x9 (three BF16 pieces per operand, nine tensor-core products, FP32 accumulation):
    relative error ~1e-6 like 3xTF32; bound 2e-5 for k up to 512, and not FP64-exact."""
    rng = np.random.default_rng(seed)
    blocks = []
    for _ in range(30):
        m, n, k = (int(np.exp(rng.uniform(np.log(8), np.log(512)))) for _ in range(3))
        blocks.append((m, n, k, int(rng.integers(0, 2)), int(rng.integers(0, 2))))
    blocks += [(128, 128, 32, 0, 0), (33, 17, 0, 0, 0)]
    err = _run(blocks, alpha=-0.75, beta=1.5, seed=seed, prec=PREC_BF16X9)
    assert 0.0 < err < 2e-5


def test_bf16x9_form_through_the_tensor_api():
    from xped_gb300 import Basis, Tensor, ensure_device
    from xped_gb300.tensor import set_gemm_precision
    ensure_device(0)
    rng = np.random.default_rng(13)
    B = Basis.from_pairs("U1", [(-1, 20), (0, 30), (1, 20)])
    T1, T2 = Tensor.zeros([B, B], [B, B]), Tensor.zeros([B, B], [B, B])
    T1.set_data(rng.standard_normal(T1.size))
    T2.set_data(rng.standard_normal(T2.size))
    ref = T1.matmul(T2).blocks()
    set_gemm_precision("bf16x9")
    try:
        got = T1.matmul(T2).blocks()
    finally:
        set_gemm_precision("fp64")
    err = max(np.linalg.norm(got[q] - ref[q]) / np.linalg.norm(ref[q]) for q in ref)
    assert 0.0 < err < 2e-5


def test_fp32_form_through_the_tensor_api():
    from xped_gb300 import Basis, Tensor, ensure_device
    from xped_gb300.tensor import set_gemm_precision
    ensure_device(0)
    rng = np.random.default_rng(9)
    B = Basis.from_pairs("U1", [(-1, 20), (0, 30), (1, 20)])
    T1, T2 = Tensor.zeros([B, B], [B, B]), Tensor.zeros([B, B], [B, B])
    T1.set_data(rng.standard_normal(T1.size))
    T2.set_data(rng.standard_normal(T2.size))
    ref = T1.matmul(T2).blocks()
    set_gemm_precision("fp32")
    try:
        got = T1.matmul(T2).blocks()
    finally:
        set_gemm_precision("fp64")
    err = max(np.linalg.norm(got[q] - ref[q]) / np.linalg.norm(ref[q]) for q in ref)
    assert 0.0 < err < 2e-5


PREC_F64TC = 4


def test_f64tc_ragged_blocks_and_transposes():
    """FP64-accurate form from exact BF16 slices on ragged blocks of every transpose: relative error within
    3e-13 (measured ~5e-14; FP64 GEMM ~1e-15, 3xTF32 ~3e-7)."""
    rng = np.random.default_rng(21)
    blocks = [(int(m), int(n), int(k), int(ta), int(tb)) for (m, n, k), ta, tb in
              zip(rng.integers(1, 300, size=(10, 3)), rng.integers(0, 2, 10), rng.integers(0, 2, 10))]
    err = _run(blocks, seed=21, prec=PREC_F64TC)
    print("f64tc ragged relative error", err)
    assert err < 3e-13


def test_f64tc_long_k_and_alpha_beta():
    err = _run([(256, 192, 3072, 0, 0), (130, 70, 2000, 1, 0), (33, 17, 0, 0, 0)], alpha=-0.5, beta=2.0, seed=22,
               prec=PREC_F64TC)
    print("f64tc long-k relative error", err)
    assert err < 3e-13


def test_f64tc_short_k_many_tiles_without_split():
    """Outer-product-like list (k = 12, ~1000 output tiles): every tile takes its whole K range, so the plan
    has no split-K partials and no reduce table."""
    blocks = [(600, 600, 12, 0, 0), (1000, 1000, 12, 1, 0), (1400, 1400, 12, 0, 1), (1000, 1000, 12, 0, 0)]
    err = _run(blocks, alpha=1.5, beta=-0.5, seed=25, prec=PREC_F64TC)
    print("f64tc short-k relative error", err)
    assert err < 3e-13


@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (2.0, 0.0), (1.5, -0.5)])
def test_f64tc_wide_outputs_computed_transposed(alpha, beta):
    """Few rows and many columns: the plan computes C^T = op(B)^T op(A)^T (half the 128 x 64 tiles) and
    stores it transposed; every store form (C = acc, alpha acc, alpha acc + beta C), a split-K group
    (k = 2000) whose reduce writes transposed, a k = 0 group and both transposes."""
    blocks = [(20, 900, 12, 0, 0), (36, 1500, 40, 1, 1), (50, 700, 2000, 0, 1), (10, 300, 0, 0, 0),
              (130, 70, 64, 1, 0)]
    err = _run(blocks, alpha=alpha, beta=beta, seed=26, prec=PREC_F64TC)
    print("f64tc transposed relative error", alpha, beta, err)
    assert err < 3e-13


def test_f64tc_graded_rows_against_the_slice_error_bound():
    """Entries spanning twelve decades within each row and column: every element within the scheme's
    bound 4 k 2^-49 max_k|a_ik| max_k|b_kj| (the slices are taken relative to each row's and column's
    largest entry, so small entries of a graded row carry the row's absolute precision)."""
    from xped_gb300 import ensure_device, lib
    from xped_gb300._lib import GemmDesc, last_error
    ensure_device(0)
    L = lib()
    rng = np.random.default_rng(23)
    m, n, k = 150, 90, 700
    A = rng.standard_normal((m, k)) * 10.0 ** rng.uniform(-12, 0, size=(m, k))
    B = rng.standard_normal((k, n)) * 10.0 ** rng.uniform(-12, 0, size=(k, n))
    ptrs = []
    for h in (A.ravel(order="F"), B.ravel(order="F"), np.zeros(m * n)):
        p = C.c_void_p()
        assert L.xgb_malloc(C.byref(p), h.nbytes) == 0
        assert L.xgb_memcpy_h2d(p, h.ctypes.data, h.nbytes) == 0
        ptrs.append(p)
    arr = (GemmDesc * 1)(GemmDesc(m, n, k, 0, m, 0, k, 0, m, 0, 0))
    assert L.xgb_grouped_gemm(PREC_F64TC, 1, arr, ptrs[0], ptrs[1], ptrs[2], 1.0, 0.0, None) == 0, last_error()
    assert L.xgb_gemm_tc_status() == 0, last_error()
    got = np.empty(m * n)
    assert L.xgb_memcpy_d2h(got.ctypes.data, ptrs[2], got.nbytes) == 0
    for p in ptrs:
        L.xgb_free(p)
    got = got.reshape((m, n), order="F")
    bound = 4.0 * k * 2.0 ** -49 * np.outer(np.abs(A).max(axis=1), np.abs(B).max(axis=0))
    ratio = float((np.abs(got - A @ B) / bound).max())
    print("f64tc graded: largest error / (4 k 2^-49 max|a_i| max|b_j|)", ratio)
    assert ratio < 1.0


def test_f64tc_extreme_digits_over_several_exact_chunks():
    """Every entry carries balanced digits at their largest magnitude of one sign (127, 63, ..., 63), so each
    level adds close to its bound per k value; k spans three full 448-deep exact TMEM chunks and a ragged
    one.  A level sum that lost a bit in the FP32 accumulator would show as a ~6e-8 relative error."""
    from xped_gb300 import ensure_device, lib
    from xped_gb300._lib import GemmDesc, last_error
    ensure_device(0)
    L = lib()
    x = sum(d * 2.0 ** (-7 * (s + 1)) for s, d in enumerate([127, 63, 63, 63, 63, 63, 63]))
    m, n, k = 130, 70, 3 * 448 + 100
    A = np.full((m, k), x)
    B = np.full((k, n), x)
    A[::3] *= -1.0
    ptrs = []
    for h in (A.ravel(order="F"), B.ravel(order="F"), np.zeros(m * n)):
        p = C.c_void_p()
        assert L.xgb_malloc(C.byref(p), h.nbytes) == 0
        assert L.xgb_memcpy_h2d(p, h.ctypes.data, h.nbytes) == 0
        ptrs.append(p)
    arr = (GemmDesc * 1)(GemmDesc(m, n, k, 0, m, 0, k, 0, m, 0, 0))
    assert L.xgb_grouped_gemm(PREC_F64TC, 1, arr, ptrs[0], ptrs[1], ptrs[2], 1.0, 0.0, None) == 0, last_error()
    assert L.xgb_gemm_tc_status() == 0, last_error()
    got = np.empty(m * n)
    assert L.xgb_memcpy_d2h(got.ctypes.data, ptrs[2], got.nbytes) == 0
    for p in ptrs:
        L.xgb_free(p)
    got = got.reshape((m, n), order="F")
    ref = A @ B
    err = float(np.abs(got - ref).max() / np.abs(ref).max())
    print("f64tc extreme digits relative error", err)
    assert err < 4.0 * k * 2.0 ** -49


def test_f64tc_through_the_tensor_api():
    from xped_gb300 import Basis, Tensor, ensure_device
    from xped_gb300.tensor import set_gemm_precision
    ensure_device(0)
    rng = np.random.default_rng(24)
    B = Basis.from_pairs("U1", [(-2, 3), (-1, 9), (0, 14), (1, 9), (2, 3)])
    T1, T2 = Tensor.zeros([B, B], [B, B]), Tensor.zeros([B, B], [B, B])
    T1.set_data(rng.standard_normal(T1.size))
    T2.set_data(rng.standard_normal(T2.size))
    ref = T1.matmul(T2).data()
    set_gemm_precision("f64tc")
    try:
        got = T1.matmul(T2).data()
    finally:
        set_gemm_precision("fp64")
    err = float(np.abs(got - ref).max() / np.abs(ref).max())
    print("f64tc tensor api max relative error", err)
    assert err < 3e-13
