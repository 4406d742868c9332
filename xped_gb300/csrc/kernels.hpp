// Internal launch interface shared by the host layer and the CUDA kernels.
// The host layer keeps its descriptor tables resident on the device (plans
// are cached), so these launchers take DEVICE descriptor pointers; the public
// xgb_* entry points in include/xgb.h upload host descriptors and call them.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "../../include/xgb.h"

namespace xgb {

// One output tile of a grouped GEMM: tile = edge length (16/32/64).  A split-K
// tile covers k in [k0, k1) (k1 < 0: all of k) and stores its raw partial sum
// into slot `slot` of a workspace (slot < 0: alpha/beta applied, stored in C).
struct GemmTile {
  int32_t g, tm, tn, tile;
  int32_t k0 = 0, k1 = -1, slot = -1, pad = 0;
};
// Fixed-order sum of the partial slots [first, first + count) of one output tile.
struct SplitReduce { int32_t g, tm, tn, first, count, pad; };
// Tiles in descending k extent: the block scheduler hands out CTAs in index
// order, so the longest tiles start first and the short ones fill the gaps
// (longest-processing-time-first) instead of a long tile starting last.
void order_tiles_by_work(std::vector<GemmTile>& tiles, const xgb_gemm_desc* descs);

// runtime ------------------------------------------------------------------------
// The stream of this host thread's lane: lane 0 is the runtime's stream; lanes 1 and 2 are the side
// streams of a fork-join section (run_pair), each driven by its own host thread.
cudaStream_t stream();
constexpr int kLanes = 3;
int lane();
struct LaneScope {  // this host thread enqueues on lane `l` until the scope ends
  int saved;
  explicit LaneScope(int l);
  ~LaneScope();
  LaneScope(const LaneScope&) = delete;
  LaneScope& operator=(const LaneScope&) = delete;
};
// Runs a() on lane 1 (a worker host thread) and b() on lane 2 (the calling thread) at the same time:
// both lanes first wait for the work enqueued so far on lane 0, and lane 0 then waits for both
// lanes, so the section is ordered like a() followed by b() on lane 0.  a() and b() must not touch
// device memory that the other writes or frees.  An exception of either is rethrown (a()'s first)
// once both have returned.  One section runs at a time; the caller must be on lane 0.
void run_pair(const std::function<void()>& a, const std::function<void()>& b);
bool lanes_used();  // a fork-join section has run since xgb_init
// makes `s` wait for the work enqueued so far on every other lane (device memory that several lanes
// may have used is freed on `s` after this)
void order_after_lanes(cudaStream_t s);
bool runtime_ready();  // xgb_init has run
int set_error(int code, const std::string& msg);
int check_cuda(cudaError_t e, const char* what);
void* dev_alloc(size_t bytes);          // stream-ordered; throws std::bad_alloc on failure
void dev_free(void* p);
void count_launch(int n = 1);
int num_sms();

// device scratch for small results (absmax, truncation outputs)
double* scalar_scratch();

// launchers (descriptor arrays are device pointers) -----------------------------------
void launch_gemm_f64(const xgb_gemm_desc* d_descs, const GemmTile* d_tiles, int n_tiles, int tile, const double* A,
                     const double* B, double* C, double alpha, double beta, cudaStream_t s);
// split-K form: `tiles` may hold partial tiles (slot >= 0) writing TILE*TILE raw sums
// into `ws`; `reduce` then adds the slots of each split output tile in slot order
void launch_gemm_f64_splitk(const xgb_gemm_desc* d_descs, const GemmTile* d_tiles, int n_tiles, int tile,
                            const SplitReduce* d_reduce, int n_reduce, const double* A, const double* B, double* C,
                            double* ws, double alpha, double beta, cudaStream_t s);
// FP32 form: same tiles, operands rounded to FP32, FP32 accumulation, FP64 store
void launch_gemm_f32(const xgb_gemm_desc* d_descs, const GemmTile* d_tiles, int n_tiles, int tile, const double* A,
                     const double* B, double* C, double alpha, double beta, cudaStream_t s);
// precision forms of the block GEMM this build implements (XGB_PREC_*)
inline bool gemm_precision_available(int p) {
  return p == XGB_PREC_FP64 || p == XGB_PREC_3XTF32 || p == XGB_PREC_FP32 || p == XGB_PREC_BF16X9 ||
         p == XGB_PREC_F64TC;
}
// permute launch shape: rows (runs along output leg 0) per task as prefix sums, and the number of
// threads that share one row (a power of two up to 32, from the element-weighted row length)
struct PermRows {
  std::vector<int64_t> row_start;
  int64_t total_rows = 0;
  int group = 1;
  bool narrow = true;  // every stride fits 32 bits (the kernel keeps them in 32-bit registers)
  bool single = true;  // every task has exactly one contribution (no SU(2) sums)
};
PermRows perm_rows(const xgb_perm_task* tasks, int n_tasks, const xgb_perm_contrib* contribs, int n_contrib);
void launch_permute(const xgb_perm_task* d_tasks, const int64_t* d_row_start, int n_tasks, int64_t total_rows,
                    int group, bool narrow, bool single, const xgb_perm_contrib* d_contribs, const double* src,
                    double* dst, cudaStream_t s);
// h_descs: host copy of the descriptors (blocks at least kSvdGridMin wide run one at a time on a
// grid-wide Jacobi kernel over all SMs; nullptr keeps every block on the cluster kernel)
void launch_svd(const xgb_svd_desc* d_descs, const xgb_svd_desc* h_descs, const int64_t* d_work_off, int n,
                int64_t max_k, const double* A, double* U, double* S, double* Vt, double* work, cudaStream_t s);
void launch_truncate(int n_sectors, const int64_t* d_s_begin, const int32_t* d_deg, const double* sv, int64_t total,
                     int64_t max_keep, double eps, int preserve, int32_t* keep, double* out2, cudaStream_t s);
void launch_qr(const xgb_qr_desc* d_descs, const int64_t* d_work_off, int n, const double* A, double* Q, double* R,
               double* work, cudaStream_t s);
void launch_absmax(const double* x, int64_t n, double* out, cudaStream_t s);
void launch_scale_by_inv(double* x, int64_t n, const double* m, cudaStream_t s);
void launch_scale(double* x, int64_t n, double alpha, cudaStream_t s);
void launch_copy2d(const xgb_copy2d_desc* d_descs, int n, int64_t max_elems, const double* src, double* dst, cudaStream_t s);
void launch_diag_from_vec(const xgb_copy2d_desc* d_descs, int n, int64_t max_k, int fn, const double* src, double* dst,
                          cudaStream_t s);
void launch_diag_apply(const xgb_copy2d_desc* d_descs, int n, int64_t max_k, int fn, double* x, cudaStream_t s);

// split-precision (3xTF32) tensor-core grouped GEMM (gemm_tc.cu): operands packed into
// 16 KB hi/lo chunks (128 rows x 32 K, canonical MMA layout), 128 x 128 output tiles
struct TcGroup {
  int64_t a_pack, b_pack;           // float offsets of the group's packed op(A) / op(B)^T chunks
  int32_t a_tiles, b_tiles, slices, pad;
};
struct TcPackTask { int32_t g, tile, slice, which; };  // which: 0 = A, 1 = B
struct TcPlanHost {
  std::vector<TcGroup> groups;
  std::vector<TcPackTask> tasks;
  std::vector<GemmTile> tiles;
  int64_t a_floats = 0, b_floats = 0;
};
// form 0 = 3xTF32, 1 = BF16x9 (pack sizes differ)
TcPlanHost build_tc_plan(const xgb_gemm_desc* descs, int n, int form = 0);
int gemm_tc_tile();
void launch_gemm_tc(const xgb_gemm_desc* d_descs, const TcGroup* d_groups, const TcPackTask* d_tasks, int n_tasks,
                    const GemmTile* d_tiles, int n_tiles, const double* A, const double* B, float* apack,
                    float* bpack, double* C, double alpha, double beta, cudaStream_t s, int form = 0);
// the pack step of launch_gemm_tc alone (operands packed once and reused by later launches
// whose task lists leave them out)
void launch_tc_pack(const xgb_gemm_desc* d_descs, const TcGroup* d_groups, const TcPackTask* d_tasks, int n_tasks,
                    const double* A, const double* B, float* apack, float* bpack, cudaStream_t s, int form = 0);
int gemm_tc_error(bool reset);  // 1 if a tensor-core GEMM CTA gave up waiting (synchronous read)
int* gemm_tc_error_flag();      // the device flag itself (allocated on first use)

// FP64-accurate tensor-core grouped GEMM from exact BF16 slices (gemm_oz.cu): 128 x 64 output tiles,
// 32-K slices, seven BF16 pieces per operand entry; per group the packed A / B slice blocks (bytes)
// and the offsets of its op(A) rows' / op(B) columns' largest magnitudes in the rowmax array
// swap != 0: the group is computed as C^T = op(B)^T op(A)^T (the product's "A" role is op(B)^T, read
// from the B buffer, and the tile is stored transposed), which wastes less of the 128 x 64 output tile
// when C has few rows and many columns
struct OzGroup {
  int64_t a_pack, b_pack, a_rowmax, b_rowmax;
  int32_t a_tiles, b_tiles, slices, swap;
};
struct OzPlanHost {
  std::vector<OzGroup> groups;
  std::vector<TcPackTask> tasks;            // tasks_a then tasks_b
  std::vector<TcPackTask> tasks_a, tasks_b;  // the op(A) and op(B) chunks alone
  std::vector<GemmTile> tiles;               // k0 / k1 in K slices; slot >= 0: split-K partial
  std::vector<SplitReduce> red;              // fixed-order sums of the split tiles
  int32_t slots = 0;                         // partial tiles (workspace slots x 128 x 64 doubles)
  int64_t a_bytes = 0, b_bytes = 0;
  int64_t rowmax = 0, rowmax_a = 0;  // entries in all; the op(A) rows come first
};
// allow_swap: groups with few rows and many columns may be computed transposed (not for callers that
// keep one operand's slices across products, whose roles must stay fixed)
OzPlanHost build_oz_plan(const xgb_gemm_desc* descs, int n, bool allow_swap = true);
// the row scales and slices of the given chunks (rowmax[clear_from .. + clear_count) zeroed first)
void launch_oz_pack(const xgb_gemm_desc* d_descs, const OzGroup* d_groups, const TcPackTask* d_tasks, int n_tasks,
                    const double* A, const double* B, unsigned long long* rowmax, int64_t clear_from,
                    int64_t clear_count, unsigned char* apack, unsigned char* bpack, cudaStream_t s);
// the product kernel (and, for split tiles, the fixed-order reduce; workspace allocated stream-ordered)
void launch_oz_gemm(const xgb_gemm_desc* d_descs, const OzGroup* d_groups, const GemmTile* d_tiles, int n_tiles,
                    const SplitReduce* d_red, int n_red, int slots, const unsigned char* apack,
                    const unsigned char* bpack, const unsigned long long* rowmax, double* C, double alpha, double beta,
                    cudaStream_t s);
void launch_gemm_oz(const xgb_gemm_desc* d_descs, const OzGroup* d_groups, const TcPackTask* d_tasks, int n_tasks,
                    const GemmTile* d_tiles, int n_tiles, const SplitReduce* d_red, int n_red, int slots,
                    const double* A, const double* B, unsigned long long* rowmax, int64_t n_rowmax,
                    unsigned char* apack, unsigned char* bpack, double* C, double alpha, double beta, cudaStream_t s);

// randomized tSVD helpers (rsvd.cu)
struct GaussBlock { int64_t offset, count, stream; };       // fill out[offset .. offset+count) from stream
struct SignFixDesc { int64_t m, n, k, u_off, v_off; };      // U m x k (ld m), V^T k x n (ld k)
void launch_gauss_fill(const GaussBlock* d_blocks, int n_blocks, int64_t max_count, uint64_t seed, double* out,
                       cudaStream_t s);
void launch_sign_fix(const SignFixDesc* d_descs, int n, int64_t max_k, double* U, double* Vt, cudaStream_t s);
// CholeskyQR helper (rsvd.cu): per sketch block m x l, Gram matrix l x l at g_off, of which only
// the upper triangle (i <= j) is read
struct CholDesc { int64_t m, l, g_off; };
void launch_chol_inv(const CholDesc* d_descs, int n, int64_t max_l, double* G, double* Rinv, double rel_shift, int* bad,
                     cudaStream_t s);
// SVD reverse rule helpers (rsvd.cu): per sector m x n block with k singular values;
// offsets of U / dU (m x k), the k x k diagonal S block, dS (k x k, ld ds_ld), V^dag / dV^dag (k x n),
// k x k work, W (k x n), P (m x k)
struct SvdBwdDesc { int64_t m, n, k, u_off, s_off, ds_off, ds_ld, v_off, kk_off, w_off, p_off; };
void launch_svd_bwd_mid(const SvdBwdDesc* d_descs, int n, int64_t max_kk, const double* S, const double* X,
                        const double* Y, const double* dS, double* N, double* XS, cudaStream_t s);
void launch_svd_bwd_scale(const SvdBwdDesc* d_descs, int n, int64_t max_elems, const double* S, const double* dVd,
                          const double* dU, double* W, double* P, cudaStream_t s);
// per-column residuals ||R[:, j] - S[j] U[:, j]|| (desc: m, n = output offset, k columns, u_off of R and U,
// v_off = offset of S)
void launch_residual_norms(const SignFixDesc* d_descs, int n, int64_t max_k, const double* R, const double* U,
                           const double* S, double* res, cudaStream_t s);
// transposed block copies: src block rows x cols (ld src_ld) -> dst cols x rows (ld dst_ld)
void launch_transpose_copy(const xgb_copy2d_desc* d_descs, int n, int64_t max_elems, const double* src, double* dst,
                           cudaStream_t s);

// rank-predictor MLP (mlp.cu): kMlpIn -> kMlpHidden x 3 (ReLU) -> kMlpOut, FP32,
// parameters packed as W1, b1, W2, b2, W3, b3, W4, b4 with row-major W[out][in]
constexpr int kMlpIn = 8, kMlpHidden = 64, kMlpOut = 2;
constexpr int kMlpParams = kMlpHidden * kMlpIn + kMlpHidden + 2 * (kMlpHidden * kMlpHidden + kMlpHidden) +
                           kMlpOut * kMlpHidden + kMlpOut;
int mlp_grad_slots(int64_t n);  // per-CTA gradient slots used by launch_mlp_grad for n samples
void launch_mlp_forward(const float* params, const float* X, int64_t n, float* Y, cudaStream_t s);
void launch_mlp_grad(const float* params, const float* X, const float* T, int64_t n, float* gpart, float* lpart,
                     cudaStream_t s);
void launch_mlp_reduce_adam(float* params, float* mom, float* vel, const float* gpart, int slots, float* grad_out,
                            int adam, float lr, float b1, float b2, float eps, int step, cudaStream_t s);

// per-kernel-kind instrumentation (CUDA events around each launch when enabled;
// algorithmic work - flops for GEMMs, bytes for data movement - always counted)
enum KernelKind { K_GEMM = 0, K_PERMUTE, K_SVD, K_TRUNC, K_QR, K_ABSMAX, K_SCALE, K_COPY2D, K_DIAG, K_GEMM_TC, K_SKETCH, K_MLP, K_GEMM_F32, K_GEMM_OZ, K_COUNT };
bool profiling();  // per-launch CUDA-event timing is on (it needs the launches of one lane only)
void prof_begin(int kind, cudaStream_t s);
void prof_end(int kind, cudaStream_t s, double work);

// FP64 grouped-GEMM launch shapes and their autotuner (autotune.cpp): tile edge 16/32/64 and a
// split-K target of split_waves x SMs CTAs (0: no split)
struct F64Config {
  int tile = 16;
  int split_waves = 0;
  bool tc = false;  // the FP64-accurate tensor-core form (XGB_PREC_F64TC) instead of the CUDA-core kernel
};
struct F64Plan {
  int tile = 16;
  std::vector<GemmTile> tiles;
  std::vector<SplitReduce> red;
  int32_t slots = 0;  // split-K partial tiles (workspace of slots x tile x tile doubles)
};
// Output structure the plan may exploit (every group of the list alike):
//  kGemmDense:    all tiles, full k;
//  kGemmSymUpper: C is symmetric (a Gram matrix op(A) = B^T): only tiles on or above the diagonal
//                 (tm <= tn) are computed; the strictly lower part of C is left unwritten;
//  kGemmTriB:     op(B) is upper triangular (rows below the diagonal are zero): output column tile tn
//                 sums k < min(k, (tn + 1) tile) only (the skipped terms are exact zeros).
// Split-K ranges follow the reduced work, so results are deterministic but not the bits of the dense plan.
enum GemmShape { kGemmDense = 0, kGemmSymUpper = 1, kGemmTriB = 2 };
F64Plan plan_gemm_f64(const xgb_gemm_desc* d, int n, F64Config c, int shape = kGemmDense);
// executes a plan whose tables are on the device (workspace allocated stream-ordered for split-K)
void run_f64_plan(const F64Plan& p, const xgb_gemm_desc* d_descs, const GemmTile* d_tiles, const SplitReduce* d_red,
                  const double* A, const double* B, double* C, double alpha, double beta, cudaStream_t s);
// plans, stages the tables and runs one configuration (host descriptors)
void run_gemm_f64_config(const xgb_gemm_desc* h_descs, int n, F64Config c, const double* A, const double* B, double* C,
                         double alpha, double beta, cudaStream_t s);
// the configuration to use for this list: tuned (measured on A, B the first time its size bucket is
// met) when autotuning is on, `fallback` otherwise; allow_tc adds the FP64-accurate tensor-core form
// to the candidates (callers that asked for FP64-class results on the tensor cores)
F64Config gemm_f64_config(const xgb_gemm_desc* d, int n, const double* A, const double* B, F64Config fallback,
                          cudaStream_t s, bool allow_tc = false);
// the FP64-accurate tensor-core GEMM of a host descriptor list (tables staged, pack buffers allocated
// stream-ordered and freed)
void run_gemm_oz_host(const xgb_gemm_desc* h_descs, int n, const double* A, const double* B, double* C, double alpha,
                      double beta, cudaStream_t s);
// built-in choice between the tensor-core form and the CUDA cores for a list whose caller allows both:
// the tensor-core form pays a fixed cost per 128 x 64 tile that only k >= 64 amortises
bool f64tc_heuristic(const xgb_gemm_desc* d, int n);
int autotune_mode();

// helpers
size_t svd_work_elems(int64_t m, int64_t n);
size_t qr_work_elems(int64_t m, int64_t n);
int choose_gemm_tile(const xgb_gemm_desc* descs, int n);  // host-side tile heuristic

}  // namespace xgb
