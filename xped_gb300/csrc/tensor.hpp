// Device-resident block-sparse symmetric tensor (host C++ side).
//
// Mirrors Xped::Tensor<double, Rank, CoRank, Symmetry> (include/Xped/Core/Tensor.hpp)
// with runtime rank: the metadata (leg bases, fusion trees, sector order,
// block offsets) lives on the host and is interned; the block data is one
// flat column-major FP64 buffer in HBM.  Each tensor operation turns into a
// cached plan (descriptor tables already on the device) plus ONE grouped
// kernel launch over all sectors.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <map>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "kernels.hpp"
#include "meta.hpp"

namespace xgb {

struct TensorMeta {
  Sym sym;
  std::vector<BasisPtr> dom, cod;     // uncoupled leg bases
  BasisPtr cdom, ccod;                // coupled (fused) bases with trees
  std::vector<int> sectors;           // storage order
  std::vector<int64_t> rows, cols, offset;
  int64_t size = 0;
  std::unordered_map<int, int> dict;  // q -> sector index
  uint64_t id = 0;
  int rank() const { return int(dom.size()); }
  int corank() const { return int(cod.size()); }
  int index(int q) const {
    auto it = dict.find(q);
    return it == dict.end() ? -1 : it->second;
  }
};
using MetaPtr = std::shared_ptr<const TensorMeta>;

// StorageType::resize order: coupled-domain order, present in the codomain.
MetaPtr make_meta(const Sym& s, const std::vector<BasisPtr>& dom, const std::vector<BasisPtr>& cod);
// push_back order (tSVD outputs, adjoint eval, scalar ops).
MetaPtr make_meta_ordered(const Sym& s, const std::vector<BasisPtr>& dom, const std::vector<BasisPtr>& cod,
                          const std::vector<int>& sectors);

struct DevBuf {
  double* p = nullptr;
  int64_t n = 0;
  explicit DevBuf(int64_t n_);
  ~DevBuf();
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

struct Tensor {
  MetaPtr meta;
  std::shared_ptr<DevBuf> buf;
  uint32_t twist_mask = 0;  // fermionic twists not yet applied to the data

  bool valid() const { return meta != nullptr; }
  double* data() const { return buf ? buf->p : nullptr; }
  int64_t size() const { return meta ? meta->size : 0; }
};

Tensor zeros(const MetaPtr& m);
Tensor empty_like_meta(const MetaPtr& m);

// Operations (names follow the reference).
Tensor materialize(const Tensor& t);  // apply pending twists
Tensor permute(const Tensor& t, int shift, const std::vector<int>& p);
// reverse rule of operator* (ADTensor.hpp:741-752): the cotangents of left and
// right (with exactly their structures) from the cotangent of left * right
std::pair<Tensor, Tensor> matmul_backward(const Tensor& left, const Tensor& right, const Tensor& res_adj);
// reverse rule of the per-sector SVD (full_svd_impl, ADTensor.hpp:257-301), real
// scalars: the cotangent of A from the factors U, S, V^dag of its (untruncated) tSVD
// and their cotangents (same structures as the factors)
Tensor tsvd_backward(const Tensor& A, const Tensor& U, const Tensor& S, const Tensor& Vdag, const Tensor& dU,
                     const Tensor& dS, const Tensor& dVdag);
// blocks of src placed in a zero tensor of the target structure (matching charges)
Tensor embed(const Tensor& src, const MetaPtr& target);
// Tensor::permute_adj<shift, p...>: transpose of permute<shift, p> applied to a
// tensor shaped like its output (the reverse rule of permute, ADTensor.hpp:172-184)
Tensor permute_adj(const Tensor& t, int shift, const std::vector<int>& p);
Tensor twist(const Tensor& t, int leg);
Tensor adjoint(const Tensor& t);
Tensor matmul(const Tensor& a, const Tensor& b, bool adj_a = false, bool adj_b = false);
Tensor contract(const Tensor& a, const Tensor& b, const std::vector<int>& a1, const std::vector<int>& a2, int rankres);
Tensor scale(const Tensor& t, double s);
double max_norm(const Tensor& t);
Tensor normalize_max(const Tensor& t);  // t * (1/maxNorm(t)), computed on the device
Tensor identity(const Sym& s, const std::vector<BasisPtr>& dom, const std::vector<BasisPtr>& cod);

struct SVDResult {
  Tensor U, S, Vdag;
  double trunc_weight = 0.0, entropy = 0.0;
  std::vector<int> keep;  // kept singular values per input sector
  // every computed singular value of the input (host copy, descending per
  // sector): sector i owns spectrum[spec_begin[i] .. spec_begin[i+1])
  std::vector<double> spectrum;
  std::vector<int64_t> spec_begin;
};
SVDResult tsvd(const Tensor& t, int64_t max_keep, double eps_svd, bool preserve_multiplets);

// Per-sector singular triplets of one tensor in flat device buffers: sector i
// owns k[i] values S[s_begin[i] .. s_begin[i+1]), U block rows(i) x k[i] at
// u_off[i] (ld rows(i)) and V^T block k[i] x cols(i) at v_off[i] (ld k[i]),
// values descending within a sector.
struct Spectra {
  double *U = nullptr, *S = nullptr, *V = nullptr;
  std::vector<int64_t> k, u_off, v_off, s_begin;
  int64_t* d_s_begin = nullptr;  // optional cached device copies
  int32_t* d_deg = nullptr;
};
// cutoff_matrices on given spectra (shared by the exact and randomized tSVD)
SVDResult truncate_spectra(const TensorMeta& m, const Spectra& sp, int64_t max_keep, double eps_svd,
                           bool preserve_multiplets);

// Randomized blockwise tSVD (the chosen form).  Sector i is sketched with
// sketch[i] seeded Gaussian columns (stream i of `seed`), refined by
// `power_iters` subspace iterations, and decomposed exactly in the sketch
// space: Q = orth(A Omega), B = Q^T A = U_B S V^T, U = Q U_B.  Sectors with
// sketch[i] <= 0 or 2 sketch[i] >= min(rows, cols) are decomposed exactly.
// A sketched sector that keeps all of its sketch columns (its next value was
// never seen) is redone with twice the columns, exactly after the third
// doubling, so the kept set is the one of the exact tSVD whenever the sketch
// resolves the kept values.
struct RsvdInfo {
  std::vector<int64_t> width;  // columns used per sector (min(rows, cols) for exact sectors)
  std::vector<int> saturated;  // sector indices, once per redo
  int64_t sketch_cols = 0;     // sum of widths over sketched sectors
  int exact_sectors = 0;
  int refinements = 0;         // refinement passes (more subspace iterations) taken
  double max_residual = 0;     // max over kept sketched triplets of ||A v - s u|| / s_max
};
// `warm` (optional): a V^dag from an earlier decomposition of a matrix with the
// same column bases; its rows of charge q become the first sketch columns of
// sector q (the remaining columns stay Gaussian).
// `res_tol` > 0: sectors whose kept triplets have ||A v_j - s_j u_j|| > res_tol * s_max
// get power_iters more subspace iterations from their current basis (up to three times).
// `fp64_tail` >= 0: the first product A Omega and the products of all but the last
// fp64_tail subspace iterations run as 3xTF32 tensor-core GEMMs (FP32 accumulation);
// the trailing iterations, the projection and everything after it stay FP64.
// < 0 (the default): every product in FP64.  `exact_tc`: every product A X / A^T X of the sketch
// (first product, subspace iterations, projection) on the FP64-accurate tensor-core form
// (exact BF16 slices, XGB_PREC_F64TC) instead; fp64_tail is then ignored.
SVDResult tsvd_randomized(const Tensor& t, int64_t max_keep, double eps_svd, const std::vector<int64_t>& sketch,
                          int power_iters, uint64_t seed, RsvdInfo* info = nullptr, const Tensor* warm = nullptr,
                          double res_tol = 0.0, int fp64_tail = -1, bool exact_tc = false);
std::pair<Tensor, Tensor> tqr(const Tensor& t);
std::pair<Tensor, Tensor> decompose(const Tensor& t1, const Tensor& t2, int64_t max_nsv);

// get_permutations (include/Xped/Util/Constfct.hpp:55-109)
struct ContractPerms {
  std::vector<int> p1, p2, pres;
  int shift1 = 0, shift2 = 0, shiftres = 0;
};
ContractPerms get_permutations(const std::vector<int>& a1, int rank1, const std::vector<int>& a2, int rank2, int rankres);

// P1 = S^-1/2 U^dag T1, P2 = T2 V S^-1/2 from a tSVD of T1*T2 (PEPSContractions.cpp:30-40)
std::pair<Tensor, Tensor> projectors_from_svd(const SVDResult& r, const Tensor& t1, const Tensor& t2);

// Last projector decomposition of one CTM direction, per sector charge.
struct SectorHistory {
  int64_t rows = 0, cols = 0, keep = 0, width = 0;
  double s_first = 0, s_last = 0, s_next = 0;  // first / last kept value, first dropped value (0 if none)
  double s_max = 0;                            // largest value of the whole matrix
};
using History = std::map<int, SectorHistory>;

// Sketch widths of the randomized projector SVD.
struct WidthPolicy {
  virtual ~WidthPolicy() = default;
  // one width per sector of `m` (sector order); <= 0 asks for an exact sector
  virtual std::vector<int64_t> widths(const TensorMeta& m, const History& last, int64_t chi) = 0;
};
// Without a model: last kept count + max(oversample, growth * kept); sectors
// with no history get 0 (exact, or the CTM's unseen-sector sketch).
struct HistoryPolicy : WidthPolicy {
  int64_t oversample = 16;
  double growth = 0.5;
  std::vector<int64_t> widths(const TensorMeta& m, const History& last, int64_t chi) override;
};

// Per-sector input features of the rank predictor (kFeatures floats per
// sector, sector order), from the matrix shape and the direction's history.
constexpr int kFeatures = 8;
void sector_features(const TensorMeta& m, const History& last, int64_t chi, std::vector<float>& out);

// One projector decomposition as seen by the learner: the features it was
// predicted from and what the decomposition then kept.
struct DecompRecord {
  int dir = 0;
  std::vector<int> sectors;
  std::vector<float> features;            // sectors x kFeatures
  std::vector<int64_t> keep, width, kmin;
  std::vector<double> spectrum;           // all computed values, per sector
  std::vector<int64_t> spec_begin;
};

struct CTMStats {
  int64_t decompositions = 0, sketched_sectors = 0, exact_sectors = 0, redo = 0, sketch_cols = 0;
  int64_t refinements = 0;  // residual-driven refinement passes
  double max_residual = 0;  // largest ||A v - s u|| / s_max of a kept sketched triplet (last decomposition)
};

// CTMRG environment on a 1x1 unit cell (src/PEPS/CTM.cpp).
class CTM {
 public:
  CTM(const Tensor& A, int64_t chi);
  void init();
  void grow_all();
  void move(char dir);
  Tensor contract_corner(const char* corner);
  std::pair<Tensor, Tensor> get_projectors(char dir);
  std::tuple<Tensor, Tensor, Tensor> renormalize(char dir, const Tensor& P1, const Tensor& P2);
  // computeRDM_h / computeRDM_v (src/PEPS/CTM.cpp:583-627, 756-790), normalised
  Tensor rdm(bool vertical);
  // CTMSolver::solve without AD (src/PEPS/CTMSolver.cpp:50-80): grow_all until the bond energy per
  // site changes by less than tol_E (or returns to within tol_E of the value two steps back)
  struct SolveResult {
    double E = 0.0;
    int steps = 0;
    bool converged = false, oscillation = false;
    std::vector<double> energies;
  };
  SolveResult solve(const Tensor& H, double tol_E, int max_steps);
  Tensor& slot(int which);  // 0..3 = C1..C4, 4..7 = T1..T4, 8 = A, 9 = Adag
  int64_t chi = 0;

  // block GEMMs of the corner contractions and the renormalisation:
  // XGB_PREC_FP64 or XGB_PREC_3XTF32 (the projector SVD, the projector
  // construction and the normalisation stay FP64); XGB_PREC_F64TC, being
  // FP64-accurate, also takes the projector products T1 T2, the projectors
  // and the randomized SVD's sketch products to the tensor cores
  int gemm_prec = XGB_PREC_FP64;
  // projector SVD form: 0 exact FP64 tSVD, 1 randomized with `policy` widths
  int svd_mode = 0;
  int power_iters = 3;
  // subspace iterations when the direction's previous V^dag (same matrix
  // structure) seeds the sketch; < 0 disables the warm start
  int warm_iters = -1;
  // sectors a direction has not seen yet: exact FP64 tSVD (false) or a sketch
  // of min(chi, min(rows, cols)) + 16 columns (true; a sector keeps at most chi
  // values, so this sketch cannot saturate)
  bool sketch_unseen = false;
  // > 0: kept sketched triplets must satisfy ||A v - s u|| <= res_tol * s_max
  // (unconverged sectors get more subspace iterations)
  double res_tol = 0.0;
  // >= 0: all but the last sketch_fp64_tail subspace iterations of the randomized
  // projector SVD multiply in 3xTF32 on the tensor cores; < 0: all FP64
  int sketch_fp64_tail = -1;
  uint64_t seed = 1;
  std::shared_ptr<WidthPolicy> policy;
  bool record = false;
  std::vector<DecompRecord> records;
  CTMStats stats;
  History hist[4];
  Tensor warm_v[4];  // last V^dag per direction (warm start of the randomized SVD)
  // grow_all runs the left/right and the top/bottom moves two at a time on the runtime's side lanes
  // (randomized projector SVD only; same results as one after the other)
  bool concurrent = true;

 private:
  std::pair<Tensor, Tensor> decompose_dir(int d, const Tensor& t1, const Tensor& t2);
  bool pairs_concurrent() const;
  void move_pair(char a, char b);
  // a direction's decomposition inside a fork-join section: its seed index, and its statistics and
  // record, committed in the sequential order once both moves have returned
  struct Deferred {
    bool on = false, residual_set = false;
    int64_t index = 0;
    CTMStats delta;
    std::vector<DecompRecord> records;
  };
  Deferred defer_[4];
  Tensor A, Ad;
  Tensor C1, C2, C3, C4, T1, T2, T3, T4;
};

// Precision form of the block GEMMs behind matmul / contract on this host
// thread: XGB_PREC_FP64 (default) or XGB_PREC_3XTF32 (tensor cores).
int gemm_precision();
void set_gemm_precision(int prec);
struct GemmPrecisionScope {
  int saved;
  explicit GemmPrecisionScope(int prec) : saved(gemm_precision()) { set_gemm_precision(prec); }
  ~GemmPrecisionScope() { set_gemm_precision(saved); }
};

// avg of a two-site operator (src/PEPS/LinearAlgebra.cpp:58-64)
double bond_expectation(const Tensor& rho, const Tensor& op);

// Checkpoints (checkpoint.cpp): the reference's serialised fields of a tensor / CTM environment in
// this library's byte layout; plain (depth-1) leg bases only.
std::vector<uint8_t> serialize_tensor(const Tensor& t);
Tensor deserialize_tensor(const uint8_t* p, size_t n);
class CTM;
std::vector<uint8_t> serialize_ctm(CTM& c);
std::unique_ptr<CTM> deserialize_ctm(const Tensor& A, const uint8_t* p, size_t n);

// fn (XGB_DIAG_SQRT / XGB_DIAG_INV / XGB_DIAG_INV_SQRT) on the main diagonal of every block
// (diag_sqrt / diag_inv of the reference, TensorBase.cpp:191-201); the rest of each block is copied
Tensor diag_apply(const Tensor& t, int fn);

// applyWeights (src/PEPS/PEPSContractions.cpp:93-104): weights on the left, top, right and
// bottom legs of a Tensor<2,3> site tensor; left and top weights twisted on their second leg
Tensor apply_weights(const Tensor& A, const Tensor& wL, const Tensor& wT, const Tensor& wR, const Tensor& wB);

// Simple-update imaginary-time evolution of an iPEPS with nearest-neighbour gates
// (TimePropagator::t_step / t_step_h / t_step_v, src/PEPS/TimePropagator.cpp:7-215;
// SimpleUpdate::renormalize, src/PEPS/SimpleUpdate.cpp:5-14).  The unit cell is a pattern of
// site labels data[x][y] (Pattern, src/PEPS/Pattern.cpp: periodic wrapping, coords(i) =
// (i % Lx, i / Lx)); per label a site tensor G: Tensor<2,3> (left, top | right, bottom,
// phys) and diagonal Tensor<1,1> weights wh (its right leg) and wv (its top leg), initially
// identities (iPEPS::initWeightTensors, iPEPS.cpp:575-592).  Neighbouring sites must carry
// different labels (TimePropagator.cpp:86-87, 93-94); one gate for every horizontal and one
// for every vertical bond.
class SimpleUpdate {
 public:
  SimpleUpdate(int Lx, int Ly, const std::vector<int>& labels, const std::vector<Tensor>& G, int64_t D);
  void step_h(int x, int y, const Tensor& Uh);  // bond (x, y) - (x+1, y)
  void step_v(int x, int y, const Tensor& Uv);  // bond (x, y-1) - (x, y)
  void step(const Tensor& Uh, const Tensor& Uv);  // TimePropagator.cpp:83-109
  Tensor site_tensor(int i) const;                // iPEPS::updateAtensors (iPEPS.cpp:594-603)
  int label(int x, int y) const;
  std::pair<int, int> coords(int i) const { return {i % Lx, i / Lx}; }
  int Lx, Ly;
  std::vector<int> labels;  // data[x][y] at x * Ly + y
  std::vector<Tensor> G, wh, wv;
  int64_t D;
};
// the single entry of a rank-0 tensor (0 if it holds no sector)
double scalar_value(const Tensor& t);

// Host-side plan tables (what the permute / GEMM kernels consume), built
// without touching the device; used by the CPU tests and by the plan caches.
struct PermTables {
  MetaPtr out;
  std::vector<xgb_perm_task> tasks;
  std::vector<xgb_perm_contrib> contribs;
  std::vector<int64_t> start;
  bool needs_zero = false;
};
PermTables build_perm_tables(const TensorMeta& in, uint32_t mask, int shift, const std::vector<int>& p);
PermTables build_perm_adj_tables(const TensorMeta& in, int shift, const std::vector<int>& p);
struct GemmTables {
  MetaPtr out;
  std::vector<xgb_gemm_desc> descs;
};
GemmTables build_gemm_tables(const TensorMeta& a, bool adj_a, const TensorMeta& b, bool adj_b);

// plan-cache statistics (for tests)
struct CacheStats {
  int64_t perm_hits = 0, perm_misses = 0, gemm_hits = 0, gemm_misses = 0;
};
CacheStats cache_stats();
void clear_plan_caches();

}  // namespace xgb
