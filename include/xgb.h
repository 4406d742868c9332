/*
 * xgb.h -- C-ABI of the GB300 block-sparse tensor backend (kernel level).
 *
 * This is the plugin boundary an Xped storage/matrix backend binds: every
 * entry point takes plain device pointers, element offsets and sizes, and
 * processes ALL sector blocks of one tensor operation in one grouped launch.
 * Each replaces a per-block loop of the reference (paths relative to the
 * Xped source tree):
 *
 *   xgb_grouped_gemm   TensorBase::operator*  (src/Core/TensorBase.cpp:237-288),
 *                      PlainInterface::prod  (src/Interfaces/MatrixInterface_Eigen_impl.cpp:156-160),
 *                      AdjointOp operands    (include/Xped/Core/AdjointOp.hpp:49-59)
 *   xgb_permute        Tensor::permute_impl  (src/Core/Tensor.cpp:83-214):
 *                      subBlock + shuffle + add_to_block_from_tensor
 *                      (src/Interfaces/PlainInterface_Eigen_impl.cpp:32-42,68-79)
 *   xgb_batched_svd    full_svd_impl / PlainInterface::svd (src/Core/Tensor.cpp:494-521,
 *                      src/Interfaces/PlainInterface_Eigen_impl.cpp:114-127)
 *   xgb_truncate       cutoff_matrices       (src/Core/Tensor.cpp:523-633)
 *   xgb_batched_qr     Tensor::tQR / MatrixInterface::qr (src/Core/Tensor.cpp:757-780,
 *                      src/Interfaces/MatrixInterface_Eigen_impl.cpp:250-256)
 *   xgb_absmax,
 *   xgb_scale_by_inv_absmax  TensorBase::maxNorm + T*(1/maxNorm) (src/Core/TensorBase.cpp:48-56,
 *                      src/PEPS/CTM.cpp:1372,1383,1405)
 *   xgb_diag_apply     TensorBase::diag_sqrt / diag_inv (src/Core/TensorBase.cpp:191-201)
 *   xgb_copy2d_batched block slicing in cutoff_matrices (src/Core/Tensor.cpp:609-630)
 *
 * Conventions: all matrices are column-major FP64 inside one flat buffer per
 * tensor; offsets and leading dimensions are in elements.  Descriptor arrays
 * live in HOST memory and are copied by the call.  Every call is
 * stream-ordered on the library's stream (or `stream` when non-NULL) and
 * returns 0 on success or a negative XGB_E_* code; xgb_last_error() gives
 * the message.  No call allocates caller-visible memory except xgb_malloc.
 */
#ifndef XGB_H_
#define XGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  XGB_OK = 0,
  XGB_E_CUDA = -1,      /* a CUDA runtime call failed */
  XGB_E_OOM = -2,       /* device allocation failed */
  XGB_E_BADPLAN = -3,   /* inconsistent descriptors or sizes */
  XGB_E_TIMEOUT = -4,   /* a bounded device wait gave up */
  XGB_E_NONFINITE = -5, /* NaN/Inf met where a finite value is required */
  XGB_E_NOINIT = -6,    /* xgb_init was not called */
  XGB_E_UNSUPPORTED = -7
};

/* precision forms of the block GEMM */
enum { XGB_PREC_FP64 = 0, XGB_PREC_3XTF32 = 1, XGB_PREC_BF16X9 = 2, XGB_PREC_FP32 = 3, XGB_PREC_F64TC = 4 };

/* ---------------------------------------------------------------- runtime */
int xgb_init(int device);
int xgb_shutdown(void);
const char* xgb_last_error(void);
int xgb_synchronize(void);
int xgb_malloc(void** ptr, size_t bytes);
int xgb_free(void* ptr);
int xgb_memcpy_h2d(void* dst, const void* src, size_t bytes);
int xgb_memcpy_d2h(void* dst, const void* src, size_t bytes);
int xgb_memset_zero(void* dst, size_t bytes);
/* number of kernels this library launched since xgb_init */
int64_t xgb_launch_count(void);
/* the library's CUDA stream (cudaStream_t) for callers that order work with it */
void* xgb_stream_handle(void);
/* Instrumentation: with profiling enabled every launch is bracketed by CUDA
   events on the library stream.  kind: 0 gemm, 1 permute, 2 svd, 3 truncate,
   4 qr, 5 absmax, 6 scale, 7 copy2d, 8 diag, 9 tensor-core gemm, 10 sketch
   (Gaussian test matrices, sign fixing), 11 rank-predictor MLP, 12 FP32 gemm,
   13 FP64-accurate tensor-core gemm (slicing and product launches).  work is the
   algorithmic flop count (GEMMs) or bytes moved (everything else). */
int xgb_profile_enable(int on);
int xgb_profile_reset(void);
int xgb_profile_read(int kind, int64_t* launches, double* ms, double* work);
/* 16 user event slots recorded on the library stream */
int xgb_event_record(int slot);
double xgb_event_elapsed_ms(int a, int b);

/* ------------------------------------------------------- grouped block GEMM */
typedef struct xgb_gemm_desc {
  int64_t m, n, k;        /* C_g is m x n, inner dimension k (k == 0 writes beta*C) */
  int64_t a_off, lda;     /* op(A_g) = trans_a ? A^T : A, A stored lda-strided */
  int64_t b_off, ldb;
  int64_t c_off, ldc;
  int32_t trans_a, trans_b;
} xgb_gemm_desc;

/* C_g = alpha * op(A_g) op(B_g) + beta * C_g for every group g, one launch.
   precision XGB_PREC_FP64: FP64 FMA; XGB_PREC_3XTF32: FP64 in and out, products
   as three TF32 tensor-core products (hi*hi + hi*lo + lo*hi) accumulated in FP32
   (about 1e-6 relative); XGB_PREC_FP32: FP64 in and out, operands rounded to
   FP32 and FP32 accumulation on the CUDA cores (about 1e-7 relative per product,
   growing with k); XGB_PREC_BF16X9: FP64 in and out, every operand split into three BF16 pieces
   (24 significant bits) and all nine piece products accumulated in FP32 on the tensor cores
   (tcgen05.mma kind::f16; about 1e-6 relative, like 3xTF32); XGB_PREC_F64TC: FP64 in and out,
   every op(A) row / op(B) column scaled by a power of two above its largest entry and cut into
   seven exact 7-bit BF16 slices; the 28 slice products of significance s + t <= 8 are summed
   exactly in FP32 tensor memory over 128-deep k chunks (Ozaki, Ogita, Oishi, Rump 2012) and the
   chunks in double-FP32 registers: the error is of the order of FP64 rounding (about 1e-15 of
   max|a| max|b| k per element). */
int xgb_grouped_gemm(int precision, int n_groups, const xgb_gemm_desc* descs, const double* A, const double* B,
                     double* C, double alpha, double beta, void* stream);
/* Tile-shape autotuner of the FP64 grouped GEMM (no counterpart in the reference, whose
   per-sector loop hands every block to BLAS separately, src/Core/TensorBase.cpp:262-279).
   Candidates: output tile edge 16 / 32 / 64 x split-K target of 0 / 1 / 2 / 4 waves of CTAs
   (xgb_autotune_candidates lists them).  mode 1: the first GEMM list of a size bucket (group
   count, total flops, largest block area, longest k on a log2 scale) times every candidate on its
   own operands (CUDA events on the launching stream, output into scratch memory) and the fastest
   is cached for the bucket; mode 2 (frozen): cached choices, the built-in rule for unseen buckets and
   no measurement (for timed regions after a tuning warm-up); mode 0 (default): the built-in rule of
   each call site.
   xgb_autotune_save / _load write / read the cache as text lines keyed by the GPU's name (entries
   of other GPU models are skipped; load returns the number of entries taken).  xgb_autotune_stats
   returns the number of cached buckets (and, if non-NULL, buckets measured, cache hits and the
   milliseconds spent measuring); xgb_autotune_choices the cached (tile, split) pairs.
   xgb_autotune_gemm measures every candidate on one list now (times_ms: one entry per candidate,
   best: the index of the fastest), leaving the cache alone; xgb_grouped_gemm_f64_config runs one
   FP64 grouped GEMM with a given shape. */
int xgb_autotune_set(int mode);
int xgb_autotune_reset(void);
int xgb_autotune_stats(int64_t* buckets_measured, int64_t* hits, double* tune_ms);
int xgb_autotune_candidates(int32_t* tile, int32_t* split_waves, int cap);
int xgb_autotune_choices(int32_t* tile, int32_t* split_waves, int cap);
int xgb_autotune_gemm(int n_groups, const xgb_gemm_desc* descs, const double* A, const double* B, double* times_ms,
                      int32_t* best);
int xgb_grouped_gemm_f64_config(int tile, int split_waves, int n_groups, const xgb_gemm_desc* descs, const double* A,
                                const double* B, double* C, double alpha, double beta, void* stream);
int xgb_autotune_save(const char* path);
int xgb_autotune_load(const char* path);

/* Synchronises and reports whether a tensor-core GEMM CTA gave up on a bounded
   wait since the last call (XGB_E_TIMEOUT) - no counterpart in the reference. */
int xgb_gemm_tc_status(void);

/* ------------------------------------------------------------------ permute */
#define XGB_MAX_LEGS 8
typedef struct xgb_perm_task {
  int64_t dst_base;                   /* element offset of the output sub-block origin */
  int64_t nelem;                      /* prod(dims) */
  int32_t rank;                       /* legs of the sub-tensor (<= XGB_MAX_LEGS) */
  int32_t n_contrib;                  /* number of source sub-blocks that add into it */
  int32_t contrib0;                   /* first entry in the contribution array */
  int32_t pad;
  int32_t dims[XGB_MAX_LEGS];         /* output sub-tensor extents, leg 0 fastest */
  int64_t dst_stride[XGB_MAX_LEGS];   /* element stride in dst per output leg */
} xgb_perm_task;

typedef struct xgb_perm_contrib {
  int64_t src_base;                   /* element offset of the source sub-block origin */
  double coeff;                       /* recoupling coefficient (1, +-1, or SU(2) value) */
  int64_t src_stride[XGB_MAX_LEGS];   /* element stride in src per OUTPUT leg */
} xgb_perm_contrib;

/* dst[task elements] = sum_c coeff_c * src[...]; tasks must tile disjoint
   regions of dst.  Elements of dst not covered by a task are left untouched. */
int xgb_permute(int n_tasks, const xgb_perm_task* tasks, int n_contrib, const xgb_perm_contrib* contribs,
                const double* src, double* dst, void* stream);

/* -------------------------------------------------------------- batched SVD */
typedef struct xgb_svd_desc {
  int64_t m, n;           /* block is m x n, k = min(m, n) singular triplets */
  int64_t a_off;          /* A block, ld = m */
  int64_t u_off;          /* U block m x k, ld = m */
  int64_t s_off;          /* k singular values, descending */
  int64_t vt_off;         /* V^T block k x n, ld = k */
} xgb_svd_desc;

/* Thin SVD of every block (FP64, one-sided Jacobi).  Singular vectors are
   sign-normalised: the entry of largest magnitude of each u_j is positive.
   `work` must hold xgb_svd_workspace_bytes(...) bytes. */
size_t xgb_svd_workspace_bytes(int n, const xgb_svd_desc* descs);
int xgb_batched_svd(int n, const xgb_svd_desc* descs, const double* A, double* U, double* S, double* Vt, void* work,
                    void* stream);

/* xgb_batched_svd for callers that cannot allocate device memory (a plugin
   whose host framework owns all device allocations, or a service with a
   fixed device-memory budget).  No counterpart in the reference: it exists
   only for embedders of this library.  Same descriptors, outputs and kernels
   as xgb_batched_svd (blocks at least 512 wide on the grid-wide Jacobi
   kernel, the others on the cluster kernel), but the workspace comes from
   one fixed 16 MiB device array per GPU
   (xgb_batched_svd_noalloc_capacity_bytes()) that the library holds until
   exit; batches needing more return XGB_E_UNSUPPORTED (one square block of
   up to 647 columns fits: an n x n block needs about 5 n^2 doubles).  The array's address is looked up on the
   first call on each device, so make that first call before any stream
   capture.  All calls share the array: calls that overlap on the GPU
   (different streams or host threads) race and must be serialised by the
   caller.  Calls no cudaMalloc/cudaFree, records no sweep statistics
   (xgb_svd_last_sweeps reports none afterwards) and returns after the
   stream has finished.  Needs xgb_init (XGB_E_NOINIT otherwise). */
int xgb_batched_svd_noalloc(int n, const xgb_svd_desc* descs, const double* A, double* U, double* S, double* Vt,
                            void* stream);
size_t xgb_batched_svd_noalloc_capacity_bytes(void);

/* Diagnostics of the last batched SVD, 6 ints per block: FP32 sweeps, FP64
   sweeps, then the cycles/1024 spent in the FP32 sweeps, the FP64
   re-orthonormalisation, the FP64 sweeps and the output stage; returns the
   number of blocks written */
int xgb_svd_last_sweeps(int32_t* out, int cap);

/* ---------------------------------------------------------------- truncation */
/* Global truncation over all sectors' singular values (cutoff_matrices):
   s holds every sector's values back to back (descending within a sector),
   sector g owning [s_begin[g], s_begin[g+1]).  Writes keep[g] and
   out2[0] = truncated weight, out2[1] = entropy (device pointers). */
int xgb_truncate(int n_sectors, const int64_t* s_begin_host, const int32_t* degeneracy_host, const double* s,
                 int64_t max_keep, double eps_svd, int preserve_multiplets, int32_t* keep_dev, double* out2_dev,
                 void* stream);

/* ------------------------------------------------------------ batched QR */
typedef struct xgb_qr_desc {
  int64_t m, n;           /* block m x n */
  int64_t a_off;          /* ld = m */
  int64_t q_off, q_cols;  /* Q block m x q_cols (ld = m), zero padded past min(m,n) */
  int64_t r_off, r_rows;  /* R block r_rows x n (ld = r_rows), zero padded past min(m,n) */
} xgb_qr_desc;
size_t xgb_qr_workspace_bytes(int n, const xgb_qr_desc* descs);
int xgb_batched_qr(int n, const xgb_qr_desc* descs, const double* A, double* Q, double* R, void* work, void* stream);

/* ------------------------------------------------------------ elementwise */
/* out_dev[0] = max |x_i| over n elements (0 for n == 0) */
int xgb_absmax(const double* x, int64_t n, double* out_dev, void* stream);
/* x *= 1 / max|x| computed on the device (x unchanged if max == 0) */
int xgb_scale_by_inv_absmax(double* x, int64_t n, double* scratch_dev, void* stream);
int xgb_scale(double* x, int64_t n, double alpha, void* stream);

enum { XGB_DIAG_SQRT = 0, XGB_DIAG_INV = 1, XGB_DIAG_INV_SQRT = 2 };
typedef struct xgb_copy2d_desc {
  int64_t src_off, src_ld, dst_off, dst_ld, rows, cols;
} xgb_copy2d_desc;
/* dst block = src block, column-major, for every descriptor */
int xgb_copy2d_batched(int n, const xgb_copy2d_desc* descs, const double* src, double* dst, void* stream);
/* dst = diag(f(src_vec)) as k x k blocks: descs use src_off (vector), dst_off, rows = cols = k */
int xgb_diag_from_vec(int n, const xgb_copy2d_desc* descs, int fn, const double* src, double* dst, void* stream);
/* in-place f() on the diagonal of k x k blocks (off-diagonal zeroed) */
int xgb_diag_apply(int n, const xgb_copy2d_desc* descs, int fn, double* x, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* XGB_H_ */
