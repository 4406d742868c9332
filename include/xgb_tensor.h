/*
 * xgb_tensor.h -- C-ABI of the GB300 backend at the Tensor-operation level.
 *
 * Opaque handles to leg bases, device-resident block-sparse tensors and a
 * 1x1-cell CTM environment.  These are the calls an Xped storage backend
 * (XPED_STORAGE=Device) makes from the Tensor core in place of its per-block
 * loops; each replaces the reference function named beside it (paths relative
 * to the Xped source tree).  All functions return 0 / a valid handle on
 * success, a negative XGB_E_* code / NULL on failure (xgb_last_error()).
 * Handles are owned by the caller and released with the matching *_release.
 */
#ifndef XGB_TENSOR_H_
#define XGB_TENSOR_H_

#include <stdint.h>

#include "xgb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xgb_basis_s* xgb_basis;
typedef struct xgb_tensor_s* xgb_tensor;
typedef struct xgb_ctm_s* xgb_ctm;
typedef struct xgb_rank_model_s* xgb_rank_model;
typedef struct xgb_su_s* xgb_su;

/* symmetry kinds */
enum { XGB_SYM_U1 = 0, XGB_SYM_U1_FERMIONIC = 1, XGB_SYM_Z2 = 2, XGB_SYM_Z2_FERMIONIC = 3, XGB_SYM_SU2 = 4 };

/* ------------------------------------------------------------------ bases */
/* Qbasis::push_back per (q, dim) pair, then Qbasis::sort when sort != 0
   (src/Core/Qbasis.cpp:34-73, 306-331). */
xgb_basis xgb_basis_create(int sym, int n, const int32_t* qs, const int64_t* dims, int sort);
xgb_basis xgb_basis_conj(xgb_basis b);                      /* Qbasis::conj (Qbasis.cpp:418-439) */
xgb_basis xgb_basis_combine(xgb_basis a, xgb_basis b);      /* Qbasis::combine (Qbasis.cpp:441-495) */
xgb_basis xgb_basis_forget_history(xgb_basis b);            /* Qbasis::forgetHistory (Qbasis.cpp:410-416) */
/* number of irreps; fills qs/dims (may be NULL) in storage order */
int xgb_basis_info(xgb_basis b, int32_t* qs, int64_t* dims, int* conj_flag, int* depth);
/* fusion trees of irrep index i: per tree rank, qc, dual mask, qu[rank], dims[rank], qi[rank-2] packed into
   `out` (int64 entries, 3 + 2*rank + max(rank-2,0) per tree); returns the number of trees, or the number of
   int64 entries needed when out == NULL. */
int xgb_basis_trees(xgb_basis b, int i, int64_t* out, int cap);
void xgb_basis_release(xgb_basis b);

/* ---------------------------------------------------------------- tensors */
/* Tensor(basis_domain, basis_codomain) + setZero (include/Xped/Core/Tensor.hpp:106-110) */
xgb_tensor xgb_tensor_zeros(int rank, const xgb_basis* dom, int corank, const xgb_basis* cod);
/* Tensor::Identity (Tensor.hpp:229-236) */
xgb_tensor xgb_tensor_identity(int rank, const xgb_basis* dom, int corank, const xgb_basis* cod);
/* sectors in storage order: returns count, fills qs/rows/cols (may be NULL) */
int xgb_tensor_sectors(xgb_tensor t, int32_t* qs, int64_t* rows, int64_t* cols);
int64_t xgb_tensor_size(xgb_tensor t);                      /* Tensor::plainSize */
int xgb_tensor_rank(xgb_tensor t, int* rank, int* corank);
xgb_basis xgb_tensor_leg(xgb_tensor t, int leg);            /* uncoupled basis of leg (domain legs first) */
xgb_basis xgb_tensor_coupled(xgb_tensor t, int codomain);   /* coupledDomain / coupledCodomain */
/* Tensor::set_data / data(): flat column-major blocks in sector order (host buffers) */
int xgb_tensor_upload(xgb_tensor t, const double* host, int64_t n);
int xgb_tensor_download(xgb_tensor t, double* host, int64_t n);
/* device pointer of the block data (after pending twists are applied) */
double* xgb_tensor_device_data(xgb_tensor t);

xgb_tensor xgb_tensor_permute(xgb_tensor t, int shift, const int32_t* p, int n);   /* Tensor::permute (Tensor.cpp:335-355) */
/* Tensor::permute_adj<shift, p...> (Tensor.cpp:258-333): the transpose of permute<shift, p> on
   a tensor shaped like its output - the reverse rule of permute (ADTensor.hpp:172-184) */
xgb_tensor xgb_tensor_permute_adj(xgb_tensor t, int shift, const int32_t* p, int n);
/* reverse rule of the per-sector SVD (full_svd_impl, ADTensor.hpp:257-301), real scalars:
   dA from the untruncated factors U, S, Vdag of tSVD(A) and their cotangents dU, dS, dVdag
   (same structures as the factors); sectors of A without singular values get zero */
xgb_tensor xgb_tensor_svd_backward(xgb_tensor A, xgb_tensor U, xgb_tensor S, xgb_tensor Vdag, xgb_tensor dU,
                                   xgb_tensor dS, xgb_tensor dVdag);
/* reverse rule of operator* (ADTensor.hpp:741-752): left_adj = res_adj * right^dag,
   right_adj = left^dag * res_adj, each with exactly its operand's structure */
int xgb_tensor_matmul_backward(xgb_tensor left, xgb_tensor right, xgb_tensor res_adj, xgb_tensor* left_adj,
                               xgb_tensor* right_adj);
xgb_tensor xgb_tensor_twist(xgb_tensor t, int leg);                                /* Tensor::twist (Tensor.cpp:357-377) */
xgb_tensor xgb_tensor_adjoint(xgb_tensor t);                                       /* adjoint().eval() */
xgb_tensor xgb_tensor_matmul(xgb_tensor a, xgb_tensor b, int adj_a, int adj_b);    /* operator* (TensorBase.cpp:237-288) */
/* Tensor::contract<a1, a2, rankres> (Tensor.hpp:328-351) */
xgb_tensor xgb_tensor_contract(xgb_tensor a, xgb_tensor b, const int32_t* a1, int n1, const int32_t* a2, int n2,
                               int rankres);
xgb_tensor xgb_tensor_scale(xgb_tensor t, double s);
double xgb_tensor_max_norm(xgb_tensor t);                                          /* TensorBase::maxNorm */
xgb_tensor xgb_tensor_normalize_max(xgb_tensor t);                                 /* t * (1/maxNorm) */
/* Tensor::tSVD (Tensor.cpp:478-633); keep[] (may be NULL, one per input sector) gets kept counts */
int xgb_tensor_tsvd(xgb_tensor t, int64_t max_keep, double eps_svd, int preserve_multiplets, xgb_tensor* U,
                    xgb_tensor* S, xgb_tensor* Vdag, double* trunc_weight, double* entropy, int32_t* keep);
/* The SVspec map of Tensor::tSVD with RETURN_SPEC (src/Core/Tensor.cpp:486-491,618-624) from the truncated
   singular-value tensor S of xgb_tensor_tsvd: per sector its charge (qs[i]), and its kept values
   (descending) at values[begin[i] .. begin[i+1]); begin has n + 1 entries, values up to cap.  Returns the
   number of sectors n (any output pointer may be NULL to query the sizes). */
int xgb_tensor_svspec(xgb_tensor S, int32_t* qs, int64_t* begin, double* values, int64_t cap);
/* Randomized blockwise tSVD with per-sector sketch widths (no counterpart in the
   reference; its results follow Tensor::tSVD's cutoff_matrices semantics).
   sketch[i] <= 0 or 2*sketch[i] >= min(rows, cols) decomposes sector i exactly;
   power_iters subspace iterations; Gaussian test matrices from `seed`; `warm` (may
   be NULL): a V^dag of an earlier decomposition with the same column bases whose
   rows of charge q replace the first Gaussian columns of sector q; res_tol > 0: a
   sector whose kept triplets have ||A v - s u|| > res_tol * s_max gets power_iters
   more subspace iterations from its current basis (at most three times).  A sketched
   sector that keeps all of its sketch is redone with twice the columns, exactly
   after the third doubling (n_saturated counts the redos).
   keep[] and width[] (may be NULL) get, per input sector, the kept count and the
   sketch width used (min(rows, cols) for exact sectors). */
int xgb_tensor_tsvd_randomized(xgb_tensor t, int64_t max_keep, double eps_svd, int n_sectors, const int64_t* sketch,
                               int power_iters, uint64_t seed, xgb_tensor warm, double res_tol, xgb_tensor* U,
                               xgb_tensor* S, xgb_tensor* Vdag, double* trunc_weight, double* entropy, int32_t* keep,
                               int64_t* width, int32_t* n_saturated);
int xgb_tensor_tqr(xgb_tensor t, xgb_tensor* Q, xgb_tensor* R);                    /* Tensor::tQR (Tensor.cpp:757-780) */
/* decompose (src/PEPS/PEPSContractions.cpp:16-43) */
int xgb_decompose(xgb_tensor t1, xgb_tensor t2, int64_t max_nsv, xgb_tensor* P1, xgb_tensor* P2);
void xgb_tensor_release(xgb_tensor t);

/* -------------------------------------------------------------------- CTM */
/* CTM<double, Sym, 2, false> on a 1x1 unit cell with site tensor A: Tensor<2,3>
   (src/PEPS/CTM.cpp). which: 0..3 = C1..C4, 4..7 = T1..T4, 8 = A, 9 = Adag. */
xgb_ctm xgb_ctm_create(xgb_tensor A, int64_t chi);
int xgb_ctm_init(xgb_ctm c);                                /* CTM::init, FROM_A (CTM.cpp:161-212) */
int xgb_ctm_grow_all(xgb_ctm c);                            /* CTM::grow_all (CTM.cpp:385-398) */
int xgb_ctm_move(xgb_ctm c, char dir);                      /* 'L','R','T','B' moves (CTM.cpp:924-1183) */
xgb_tensor xgb_ctm_get(xgb_ctm c, int which);
int xgb_ctm_set(xgb_ctm c, int which, xgb_tensor t);
void xgb_ctm_release(xgb_ctm c);

/* ------------------------------------------------------------- checkpoints */
/* The fields the reference serialises for a tensor (StorageType_contiguous::serialize,
   include/Xped/Core/storage/StorageType_contiguous.hpp:191-204) and for a CTM environment
   (CTM::serialize, include/Xped/PEPS/CTM.hpp:184-204: chi, C1..C4, T1..T4) in this library's own
   byte layout (the reference's yas archive format is not claimed).  Plain leg bases only.
   With buf == NULL the call stores the needed byte count in *size; otherwise cap must hold it. */
int xgb_tensor_serialize(xgb_tensor t, uint8_t* buf, int64_t cap, int64_t* size);
xgb_tensor xgb_tensor_deserialize(const uint8_t* buf, int64_t size);
int xgb_ctm_serialize(xgb_ctm c, uint8_t* buf, int64_t cap, int64_t* size);
/* a CTM for site tensor A with chi and the environment of the checkpoint (the projector-SVD
   configuration and the sketch-width history are not part of it) */
xgb_ctm xgb_ctm_deserialize(xgb_tensor A, const uint8_t* buf, int64_t size);

/* ----------------------------------------------------------- simple update */
/* Simple-update imaginary-time evolution of an iPEPS with nearest-neighbour gates
   (TimePropagator::t_step / t_step_h / t_step_v, src/PEPS/TimePropagator.cpp:7-215;
   SimpleUpdate::renormalize, src/PEPS/SimpleUpdate.cpp:5-14).  Unit cell: Lx x Ly
   labels, labels[x * Ly + y] = data[x][y] of the reference's Pattern (periodic;
   site i sits at (i % Lx, i / Lx)); neighbouring sites must differ (the reference
   asserts it, TimePropagator.cpp:86-87, 93-94).  G[label]: Tensor<2,3> (left, top |
   right, bottom, phys); bond weights start as identities (iPEPS::initWeightTensors,
   src/PEPS/iPEPS.cpp:575-592); D: bond dimension kept by the bond tSVD (eps 1e-14).
   Gates Uh, Uv: Tensor<2,2> on (phys, phys), e.g. exp(-dt H) (TimePropagator::initU,
   TimePropagator.cpp:453-487), the same on every bond of their direction. */
xgb_su xgb_su_create(int Lx, int Ly, const int* labels, int n_sites, const xgb_tensor* G, int64_t D);
int xgb_su_step(xgb_su s, xgb_tensor Uh, xgb_tensor Uv);    /* t_step (TimePropagator.cpp:83-109) */
int xgb_su_step_h(xgb_su s, int x, int y, xgb_tensor Uh);   /* t_step_h: bond (x, y) - (x+1, y) */
int xgb_su_step_v(xgb_su s, int x, int y, xgb_tensor Uv);   /* t_step_v: bond (x, y-1) - (x, y) */
/* which: 0 = G, 1 = horizontal weight (right leg), 2 = vertical weight (top leg) of
   label `site`; 3 = site tensor at coords(site) with sqrt weights on its four legs
   (iPEPS::updateAtensors, iPEPS.cpp:594-603) */
xgb_tensor xgb_su_get(xgb_su s, int which, int site);
void xgb_su_release(xgb_su s);
/* Projector SVD form of the moves (no counterpart in the reference, which always
   runs the full tSVD): mode 0 exact FP64 tSVD, mode 1 randomized tSVD whose sketch
   widths are the direction's last kept counts + max(oversample, growth * kept)
   (exact for sectors not seen before); power_iters subspace iterations. */
int xgb_ctm_set_svd(xgb_ctm c, int mode, int power_iters, uint64_t seed, int64_t oversample, double growth);
/* Precision form of the block GEMMs behind xgb_tensor_matmul / xgb_tensor_contract
   issued from the calling host thread: XGB_PREC_FP64 (default), XGB_PREC_3XTF32 or
   XGB_PREC_FP32 (xgb.h).  Selects what XPED_MATRIX_LIB selects for operator* in the reference. */
int xgb_set_gemm_precision(int precision);
/* Precision form of the block GEMMs in the corner contractions and the
   renormalisation of the moves (XGB_PREC_FP64, XGB_PREC_3XTF32 or XGB_PREC_FP32);
   the projector SVD, the projector construction and the normalisation stay FP64. */
int xgb_ctm_set_gemm_precision(xgb_ctm c, int precision);
/* Sectors without history (the first decomposition of each direction) in the
   randomized form: exact FP64 tSVD (on = 0, the default) or a sketch of
   min(chi, min(rows, cols)) + 16 columns (on = 1), for either width rule. */
int xgb_ctm_set_sketch_unseen(xgb_ctm c, int on);
/* on != 0 (the default): grow_all runs the left and right moves, then the top and bottom moves, two at
 * a time on two CUDA streams driven by two host threads (the pairs touch disjoint environment tensors;
 * results equal the sequential order's).  Only with the randomized projector SVD, and not while
 * per-launch profiling or autotune measurement is on.  No counterpart in the reference, whose
 * CTM::grow_all (src/PEPS/CTM.cpp:385-398) runs the four moves one after the other. */
int xgb_ctm_set_concurrent(xgb_ctm c, int on);
/* Products of the randomized projector SVD's subspace iterations: fp64_tail >= 0
   runs the first product A Omega and all but the last fp64_tail iterations as
   3xTF32 tensor-core GEMMs (FP32 accumulation), the last fp64_tail iterations, the
   projection and the small SVDs in FP64; fp64_tail < 0 (the default) keeps every
   product FP64. */
int xgb_ctm_set_sketch_precision(xgb_ctm c, int fp64_tail);
/* Warm start of the randomized projector SVD: the direction's previous V^dag seeds
   the sketch and warm_iters subspace iterations are run instead of power_iters
   (warm_iters < 0: off, the default). */
int xgb_ctm_set_warm_start(xgb_ctm c, int warm_iters);
/* Residual control of the randomized projector SVD: kept triplets must satisfy
   ||A v - s u|| <= tol * s_max, else more subspace iterations (0: off) */
int xgb_ctm_set_residual_tol(xgb_ctm c, double tol);
/* refinement passes so far and the largest relative residual of the last decomposition */
int xgb_ctm_residual_stats(xgb_ctm c, int64_t* refinements, double* max_residual);
/* out5: decompositions, sketched sectors, exact sectors, sketch redos, sketch columns */
int xgb_ctm_stats(xgb_ctm c, int64_t* out5);
/* Decomposition log for learning sketch widths (features of the rank predictor,
   kept counts, widths, min(rows, cols), full computed spectra). on = 0 clears it. */
int xgb_ctm_record(xgb_ctm c, int on);
int xgb_ctm_record_count(xgb_ctm c);
int xgb_ctm_record_get(xgb_ctm c, int i, int* dir, int* n_sectors, int64_t* n_spectrum, int32_t* sectors,
                       float* features, int64_t* keep, int64_t* width, int64_t* kmin, double* spectrum,
                       int64_t* spec_begin);
/* computeRDM_h (vertical = 0) / computeRDM_v (vertical = 1), normalised
   (src/PEPS/CTM.cpp:583-627, 756-790) */
xgb_tensor xgb_ctm_rdm(xgb_ctm c, int vertical);
/* CTMSolver::solve without AD (src/PEPS/CTMSolver.cpp:50-80) on the 1x1 cell: grow_all steps until
   the bond energy per site E = <H>_h + <H>_v changes by less than tol_E, or comes back to within
   tol_E of the value two steps earlier (oscillation), at most max_steps steps.  Writes the last E,
   the steps run, flags (1 converged, 2 stopped on oscillation) and, if energies is non-NULL, the
   energy after each step (up to cap values). */
int xgb_ctm_solve(xgb_ctm c, xgb_tensor H, double tol_E, int max_steps, double* E, int* steps, int* flags,
                  double* energies, int cap);
/* Learned sketch widths (no counterpart in the reference).  A small MLP
   (xgb_rank_model_num_features() inputs per sector -> 3 x 64 ReLU -> 2 outputs,
   FP32) predicts log2(1 + kept count) and log2(1 + oversampling) of each sector of
   a projector decomposition from its shape and the direction's last spectrum;
   forward, backward and Adam run on the device.  Parameters are packed W1, b1,
   W2, b2, W3, b3, W4, b4 with row-major W[out][in]; loss = mean over samples of
   half the squared error summed over both outputs.  X is n x features, T and Y
   n x 2, row-major host arrays. */
int xgb_rank_model_num_params(void);
int xgb_rank_model_num_features(void);
xgb_rank_model xgb_rank_model_create(uint64_t seed);
void xgb_rank_model_release(xgb_rank_model m);
int xgb_rank_model_get_params(xgb_rank_model m, float* out, int cap);
int xgb_rank_model_set_params(xgb_rank_model m, const float* in, int n);  /* also resets the Adam state */
int xgb_rank_model_predict(xgb_rank_model m, const float* X, int64_t n, float* Y);
int xgb_rank_model_gradient(xgb_rank_model m, const float* X, const float* T, int64_t n, float* grad, double* loss);
/* steps full-batch Adam steps (beta 0.9 / 0.999, eps 1e-8); loss before the last step */
int xgb_rank_model_train(xgb_rank_model m, const float* X, const float* T, int64_t n, int steps, float lr,
                         double* loss);
/* Switch the CTM to the randomized projector SVD with model-predicted widths:
   ceil(k * (1 + margin)) + max(min_oversample, ceil(p)) columns per sector. */
int xgb_ctm_set_rank_model(xgb_ctm c, xgb_rank_model m, double margin, int64_t min_oversample, int power_iters,
                           uint64_t seed);
/* avg of a two-site operator on a bond RDM (src/PEPS/LinearAlgebra.cpp:58-64) */
int xgb_tensor_bond_expectation(xgb_tensor rho, xgb_tensor op, double* out);

/* ------------------------------------------------- host-only planning */
/* Metadata-only tensor (no device memory): sectors, blocks and the plans below
   can be inspected without a GPU. */
xgb_tensor xgb_tensor_meta(int rank, const xgb_basis* dom, int corank, const xgb_basis* cod);
/* The permute plan the device kernel would run for permute<shift>(p) with
   pending twists `twist_mask`; counts always written, arrays when non-NULL. */
int xgb_permute_plan_host(xgb_tensor t, int shift, const int32_t* p, int n, uint32_t twist_mask, int* n_tasks,
                          int* n_contrib, xgb_perm_task* tasks, int task_cap, xgb_perm_contrib* contribs,
                          int contrib_cap, xgb_tensor* out_meta);
/* The grouped-GEMM descriptors of operator*(a, b) (with adjoint operands). */
int xgb_gemm_plan_host(xgb_tensor a, int adj_a, xgb_tensor b, int adj_b, int* n, xgb_gemm_desc* descs, int cap,
                       xgb_tensor* out_meta);
/* get_permutations (include/Xped/Util/Constfct.hpp:55-109): writes
   p1[n1], shift1, p2[n2], shift2, pres[nres], shiftres into out; returns nres. */
int xgb_contract_perms(const int32_t* a1, int n1, int rank1, const int32_t* a2, int n2, int rank2, int rankres,
                       int32_t* out);

/* plan-cache counters: perm hits, perm misses, gemm hits, gemm misses */
int xgb_plan_cache_stats(int64_t* out4);

#ifdef __cplusplus
}
#endif
#endif /* XGB_TENSOR_H_ */
