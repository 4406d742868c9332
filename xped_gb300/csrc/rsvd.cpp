// Randomized blockwise truncated SVD (host orchestration).
//
// Every stage is one grouped launch over all sketched sectors: the Gaussian
// test matrices, the sketch GEMMs (A Omega, A^T Q, Q^T A, Q U_B), the
// orthonormalisations (shifted CholeskyQR3: grouped Gram / triangular-solve
// GEMMs and one small Cholesky launch per pass), the small exact SVD of
// B = Q^T A together with the exactly decomposed sectors, and the sign
// convention.  Truncation is the shared cutoff_matrices step
// (src/Core/Tensor.cpp:523-633) on the resulting per-sector spectra.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "tensor.hpp"

namespace xgb {
namespace {

void ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// Host tables packed into one device allocation and uploaded with one copy;
// the allocation is released in stream order when the object goes away.
class Staging {
 public:
  template <class T>
  size_t add(const std::vector<T>& v) {
    const size_t off = (host_.size() + 255) & ~size_t(255);
    host_.resize(off + sizeof(T) * v.size());
    if (!v.empty()) std::memcpy(host_.data() + off, v.data(), sizeof(T) * v.size());
    return off;
  }
  void upload(cudaStream_t s) {
    dev_ = static_cast<char*>(dev_alloc(std::max<size_t>(host_.size(), 256)));
    if (!host_.empty()) ok(cudaMemcpyAsync(dev_, host_.data(), host_.size(), cudaMemcpyHostToDevice, s), "h2d tables");
  }
  template <class T>
  T* at(size_t off) const { return reinterpret_cast<T*>(dev_ + off); }
  ~Staging() { if (dev_) dev_free(dev_); }

 private:
  std::vector<char> host_;
  char* dev_ = nullptr;
};

double* alloc_d(int64_t n) { return static_cast<double*>(dev_alloc(sizeof(double) * size_t(std::max<int64_t>(n, 1)))); }

// Grouped FP64 GEMM of the sketch pipeline.  When the output tiles cannot fill the SMs
// (the l x l Gram matrices Y^T Y: few tiles, k = the block's row count) the k range of each
// tile is split so that about two CTAs per SM run; the partial tiles land in a workspace and
// one reduce launch adds them in a fixed order (deterministic result).  With autotuning on, the
// tile edge and the split target are the tuned ones of the list's size bucket.
// allow_tc (callers running the FP64-accurate tensor-core form): the autotuner may also route the list
// to that form when it measures it faster (built-in rule: average k >= 64), computing C in full.
void grouped_gemm(const std::vector<xgb_gemm_desc>& d, const double* A, const double* B, double* C, cudaStream_t s,
                  double alpha = 1.0, double beta = 0.0, int shape = kGemmDense, bool allow_tc = false) {
  if (d.empty()) return;
  if (allow_tc) {
    const F64Config tfb{choose_gemm_tile(d.data(), int(d.size())), 2, f64tc_heuristic(d.data(), int(d.size()))};
    if (gemm_f64_config(d.data(), int(d.size()), A, B, tfb, s, true).tc) {
      double flops = 0;
      for (const auto& g : d) flops += 2.0 * double(g.m) * double(g.n) * double(g.k);
      prof_begin(K_GEMM_OZ, s);
      run_gemm_oz_host(d.data(), int(d.size()), A, B, C, alpha, beta, s);
      prof_end(K_GEMM_OZ, s, flops);
      return;
    }
  }
  const F64Config fallback{choose_gemm_tile(d.data(), int(d.size())), 2};
  const F64Config cfg = gemm_f64_config(d.data(), int(d.size()), A, B, fallback, s);
  const F64Plan p = plan_gemm_f64(d.data(), int(d.size()), cfg, shape);
  double flops = 0;
  for (const auto& g : d) flops += 2.0 * double(g.m) * double(g.n) * double(g.k) * (shape == kGemmDense ? 1.0 : 0.5);
  Staging st;
  const size_t od = st.add(d), ot = st.add(p.tiles), orr = st.add(p.red);
  st.upload(s);
  prof_begin(K_GEMM, s);
  run_f64_plan(p, st.at<xgb_gemm_desc>(od), st.at<GemmTile>(ot), st.at<SplitReduce>(orr), A, B, C, alpha, beta, s);
  prof_end(K_GEMM, s, flops);
}

// 3xTF32 tensor-core products op(A_q) X_q (gemm_tc.cu) over a fixed list of sector GEMMs, for the
// early products of a subspace iteration: their bases only have to approach the dominant
// subspace, which the trailing FP64 iterations then resolve to FP64 accuracy.  op(A_q) is split
// into TF32 hi / lo chunks once, at construction; every apply() packs only X and runs the MMA
// kernel.  A CTA that gives up waiting sets the tensor-core error flag, read after the
// decomposition's residual synchronisation.
class TcProducts {
 public:
  TcProducts(const std::vector<xgb_gemm_desc>& d, const double* A, cudaStream_t s) {
    TcPlanHost tp = build_tc_plan(d.data(), int(d.size()), 0);
    std::vector<TcPackTask> ta, tb;
    for (const auto& t : tp.tasks) (t.which == 0 ? ta : tb).push_back(t);
    n_tiles_ = int(tp.tiles.size());
    n_b_ = int(tb.size());
    for (const auto& g : d) flops_ += 2.0 * double(g.m) * double(g.n) * double(g.k);
    od_ = st_.add(d);
    og_ = st_.add(tp.groups);
    oa_ = st_.add(ta);
    ob_ = st_.add(tb);
    ot_ = st_.add(tp.tiles);
    st_.upload(s);
    ap_ = static_cast<float*>(dev_alloc(sizeof(float) * size_t(std::max<int64_t>(tp.a_floats, 4))));
    bp_ = static_cast<float*>(dev_alloc(sizeof(float) * size_t(std::max<int64_t>(tp.b_floats, 4))));
    prof_begin(K_GEMM_TC, s);
    launch_tc_pack(st_.at<xgb_gemm_desc>(od_), st_.at<TcGroup>(og_), st_.at<TcPackTask>(oa_), int(ta.size()), A,
                   nullptr, ap_, bp_, s, 0);
    prof_end(K_GEMM_TC, s, 0.0);
  }
  TcProducts(const TcProducts&) = delete;
  TcProducts& operator=(const TcProducts&) = delete;
  ~TcProducts() {
    dev_free(ap_);
    dev_free(bp_);
  }
  // C = op(A) X with the A packed at construction
  void apply(const double* A, const double* X, double* C, cudaStream_t s) {
    if (n_tiles_ == 0) return;
    prof_begin(K_GEMM_TC, s);
    launch_gemm_tc(st_.at<xgb_gemm_desc>(od_), st_.at<TcGroup>(og_), st_.at<TcPackTask>(ob_), n_b_,
                   st_.at<GemmTile>(ot_), n_tiles_, A, X, ap_, bp_, C, 1.0, 0.0, s, 0);
    prof_end(K_GEMM_TC, s, flops_);
  }

 private:
  Staging st_;
  size_t od_ = 0, og_ = 0, oa_ = 0, ob_ = 0, ot_ = 0;
  int n_tiles_ = 0, n_b_ = 0;
  double flops_ = 0;
  float* ap_ = nullptr;
  float* bp_ = nullptr;
};

// FP64-accurate tensor-core products op(A_q) X_q (gemm_oz.cu, exact BF16 slices) over a fixed list of
// sector GEMMs: op(A) is scaled and sliced once at construction, each apply() slices only X.
class OzProducts {
 public:
  OzProducts(const std::vector<xgb_gemm_desc>& d, const double* A, cudaStream_t s) {
    const OzPlanHost op = build_oz_plan(d.data(), int(d.size()), false);  // op(A) keeps the A role
    n_tiles_ = int(op.tiles.size());
    n_red_ = int(op.red.size());
    slots_ = op.slots;
    n_b_ = int(op.tasks_b.size());
    rowmax_a_ = op.rowmax_a;
    rowmax_ = op.rowmax;
    for (const auto& g : d) flops_ += 2.0 * double(g.m) * double(g.n) * double(g.k);
    od_ = st_.add(d);
    og_ = st_.add(op.groups);
    oa_ = st_.add(op.tasks_a);
    ob_ = st_.add(op.tasks_b);
    ot_ = st_.add(op.tiles);
    or_ = st_.add(op.red);
    st_.upload(s);
    rm_ = static_cast<unsigned long long*>(dev_alloc(sizeof(unsigned long long) * size_t(std::max<int64_t>(rowmax_, 1))));
    ap_ = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(op.a_bytes, 16))));
    bp_ = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(op.b_bytes, 16))));
    prof_begin(K_GEMM_OZ, s);
    launch_oz_pack(st_.at<xgb_gemm_desc>(od_), st_.at<OzGroup>(og_), st_.at<TcPackTask>(oa_), int(op.tasks_a.size()), A,
                   nullptr, rm_, 0, rowmax_a_, ap_, bp_, s);
    prof_end(K_GEMM_OZ, s, 0.0);
  }
  OzProducts(const OzProducts&) = delete;
  OzProducts& operator=(const OzProducts&) = delete;
  ~OzProducts() {
    dev_free(rm_);
    dev_free(ap_);
    dev_free(bp_);
  }
  // C = op(A) X with the A sliced at construction
  void apply(const double* A, const double* X, double* C, cudaStream_t s) {
    if (n_tiles_ == 0) return;
    prof_begin(K_GEMM_OZ, s);
    launch_oz_pack(st_.at<xgb_gemm_desc>(od_), st_.at<OzGroup>(og_), st_.at<TcPackTask>(ob_), n_b_, A, X, rm_,
                   rowmax_a_, rowmax_ - rowmax_a_, ap_, bp_, s);
    launch_oz_gemm(st_.at<xgb_gemm_desc>(od_), st_.at<OzGroup>(og_), st_.at<GemmTile>(ot_), n_tiles_,
                   st_.at<SplitReduce>(or_), n_red_, slots_, ap_, bp_, rm_, C, 1.0, 0.0, s);
    prof_end(K_GEMM_OZ, s, flops_);
  }

 private:
  Staging st_;
  size_t od_ = 0, og_ = 0, oa_ = 0, ob_ = 0, ot_ = 0, or_ = 0;
  int n_tiles_ = 0, n_b_ = 0, n_red_ = 0, slots_ = 0;
  int64_t rowmax_a_ = 0, rowmax_ = 0;
  double flops_ = 0;
  unsigned long long* rm_ = nullptr;
  unsigned char* ap_ = nullptr;
  unsigned char* bp_ = nullptr;
};

// Batched thin SVD through the cluster Jacobi kernel (work counted as the thin R-SVD flop count
// 6 m n^2 + 20 n^3, m >= n, Golub & Van Loan, Matrix Computations, Table 5.5.1).
void batched_svd(const std::vector<xgb_svd_desc>& d, const double* A, double* U, double* S, double* Vt, cudaStream_t s) {
  if (d.empty()) return;
  std::vector<int64_t> woff(d.size());
  int64_t wt = 0, maxk = 0;
  double flops = 0;
  for (size_t i = 0; i < d.size(); ++i) {
    woff[i] = wt;
    wt += int64_t(svd_work_elems(d[i].m, d[i].n));
    const double mm = double(std::max(d[i].m, d[i].n)), nn = double(std::min(d[i].m, d[i].n));
    maxk = std::max(maxk, std::min(d[i].m, d[i].n));
    flops += 6 * mm * nn * nn + 20 * nn * nn * nn;  // thin R-SVD count (U m x n, S, V)
  }
  Staging st;
  const size_t od = st.add(d), ow = st.add(woff);
  st.upload(s);
  double* W = alloc_d(wt);
  prof_begin(K_SVD, s);
  launch_svd(st.at<xgb_svd_desc>(od), d.data(), st.at<int64_t>(ow), int(d.size()), maxk, A, U, S, Vt, W, s);
  prof_end(K_SVD, s, flops);
  dev_free(W);
}

// Orthonormal basis of each tall m x l block of Y by shifted CholeskyQR3 (Fukaya,
// Kannan, Nakatsukasa, Yamamoto, Yanagisawa, SIAM J. Sci. Comput. 2020): one
// shifted pass Q1 = Y chol(Y^T Y + s I)^-1, s = 11 (m l + l (l + 1)) u ||Y||_F^2,
// then two plain CholeskyQR passes (passes = 3), or one (passes = 2: the bases
// between the products of a subspace iteration only have to stay well
// conditioned; their span is what the iteration carries).  Every pass is two
// grouped FP64 GEMMs (Gram matrix, Q R^-1) spread over all SMs plus one small
// Cholesky / triangular-inverse launch (one CTA per block).  The passes alternate
// between Y and Q; returns the buffer holding the basis (Q for 3 passes, Y for
// 2); the other one holds garbage afterwards.
double* orthonormalise(const std::vector<int64_t>& rows, const std::vector<int64_t>& cols,
                       const std::vector<int64_t>& y_off, double* Y, double* Q, cudaStream_t s, int passes = 3,
                       bool exact_tc = false) {
  const size_t n = rows.size();
  if (n == 0) return passes == 2 ? Y : Q;
  std::vector<CholDesc> cd;
  std::vector<xgb_gemm_desc> gram_y, gram_q, mul_yq, mul_qy;
  int64_t gt = 0;
  int64_t max_l = 0;
  for (size_t i = 0; i < n; ++i) {
    const int64_t m = rows[i], l = cols[i];
    max_l = std::max(max_l, l);
    cd.push_back({m, l, gt});
    gram_y.push_back({l, l, m, y_off[i], m, y_off[i], m, gt, l, 1, 0});  // G = Y^T Y
    gram_q.push_back({l, l, m, y_off[i], m, y_off[i], m, gt, l, 1, 0});  // same layout for Q
    mul_yq.push_back({m, l, l, y_off[i], m, gt, l, y_off[i], m, 0, 0});  // dst = src R^-1
    mul_qy.push_back(mul_yq.back());
    gt += l * l;
  }
  double* G = alloc_d(gt);
  double* Ri = alloc_d(gt);
  int* bad = static_cast<int*>(dev_alloc(sizeof(int)));
  ok(cudaMemsetAsync(bad, 0, sizeof(int), s), "memset");
  Staging sc;
  const size_t o = sc.add(cd);
  sc.upload(s);
  constexpr double kShift = 11.0 * 1.1102230246251565e-16;
  // pass 1 (shifted): Y -> Q;  pass 2: Q -> Y;  pass 3: Y -> Q.  The Gram matrices are computed on and
  // above the diagonal only (the Cholesky reads that triangle), and Q R^-1 skips the zero rows of the
  // upper-triangular R^-1: about half the FP64 work of the full products.
  grouped_gemm(gram_y, Y, Y, G, s, 1.0, 0.0, kGemmSymUpper, exact_tc);
  prof_begin(K_QR, s);
  launch_chol_inv(sc.at<CholDesc>(o), int(n), max_l, G, Ri, kShift, bad, s);
  prof_end(K_QR, s, 0.0);
  grouped_gemm(mul_yq, Y, Ri, Q, s, 1.0, 0.0, kGemmTriB);
  if (passes >= 2) {
    grouped_gemm(gram_q, Q, Q, G, s, 1.0, 0.0, kGemmSymUpper, exact_tc);
    prof_begin(K_QR, s);
    launch_chol_inv(sc.at<CholDesc>(o), int(n), max_l, G, Ri, 0.0, bad, s);
    prof_end(K_QR, s, 0.0);
    grouped_gemm(mul_qy, Q, Ri, Y, s, 1.0, 0.0, kGemmTriB);
  }
  if (passes >= 3) {
    grouped_gemm(gram_y, Y, Y, G, s, 1.0, 0.0, kGemmSymUpper, exact_tc);
    prof_begin(K_QR, s);
    launch_chol_inv(sc.at<CholDesc>(o), int(n), max_l, G, Ri, 0.0, bad, s);
    prof_end(K_QR, s, 0.0);
    grouped_gemm(mul_yq, Y, Ri, Q, s, 1.0, 0.0, kGemmTriB);
  }
  dev_free(G);
  dev_free(Ri);
  dev_free(bad);
  return passes == 2 ? Y : Q;
}

constexpr int kMaxRetries = 3;
constexpr int kInterPasses = 1;  // CholeskyQR passes of the bases between subspace-iteration products
constexpr int kMaxRefine = 3;  // refinement passes of unconverged sectors per round

}  // namespace

SVDResult tsvd_randomized(const Tensor& t0, int64_t max_keep, double eps_svd, const std::vector<int64_t>& sketch,
                          int power_iters, uint64_t seed, RsvdInfo* info, const Tensor* warm, double res_tol,
                          int fp64_tail, bool exact_tc) {
  Tensor t = materialize(t0);
  const TensorMeta& m = *t.meta;
  const int n = int(m.sectors.size());
  if (n == 0) throw std::runtime_error("tSVD of a tensor without sectors");
  if (int(sketch.size()) != n) throw std::runtime_error("randomized tSVD: one sketch width per sector required");
  if (power_iters < 0) throw std::runtime_error("randomized tSVD: negative number of power iterations");
  // leading iterations (and the first product A Omega) on the tensor cores; the last fp64_tail in FP64
  // (exact_tc: every product A X / A^T X on the FP64-accurate tensor-core form instead)
  const int tc_iters = (!exact_tc && fp64_tail >= 0) ? std::max(0, power_iters - fp64_tail) : 0;
  cudaStream_t st = stream();
  // warm-start rows per sector (a V^dag block of the same charge and column dimension)
  Tensor warm_t;
  std::vector<int64_t> w_off(n, -1), w_rows(n, 0);
  if (warm && warm->valid()) {
    warm_t = materialize(*warm);
    const TensorMeta& wm = *warm_t.meta;
    for (int i = 0; i < n; ++i) {
      const int wi = wm.index(m.sectors[i]);
      if (wi >= 0 && wm.cols[wi] == m.cols[i]) {
        w_off[i] = wm.offset[wi];
        w_rows[i] = wm.rows[wi];
      }
    }
  }
  std::vector<char> exact(n, 0);
  std::vector<int64_t> want(sketch);
  std::vector<int> saturated;
  int refinements = 0;
  double max_res = 0;
  for (int round = 0;; ++round) {
    // ---- widths and layout
    std::vector<int64_t> width(n);
    std::vector<int> R, E;  // sketched / exact sector indices
    for (int i = 0; i < n; ++i) {
      const int64_t kmin = std::min(m.rows[i], m.cols[i]);
      int64_t l = want[i];
      if (exact[i] || l <= 0 || 2 * l >= kmin) { exact[i] = 1; l = kmin; }
      width[i] = l;
      (exact[i] ? E : R).push_back(i);
    }
    Spectra sp;
    sp.k = width;
    sp.u_off.assign(n, 0);
    sp.v_off.assign(n, 0);
    sp.s_begin.assign(n + 1, 0);
    int64_t ut = 0, vt = 0;
    for (int i = 0; i < n; ++i) {
      sp.u_off[i] = ut;
      ut += m.rows[i] * width[i];
      sp.v_off[i] = vt;
      vt += width[i] * m.cols[i];
      sp.s_begin[i + 1] = sp.s_begin[i] + width[i];
    }
    // per sketched sector: Omega (n x l), Y (m x l), Q (m x l), Z / Qz (n x l), U_B (l x l)
    const int nr = int(R.size());
    std::vector<int64_t> rr(nr), rc(nr), rl(nr), om(nr), yo(nr), zo(nr), ub(nr), bo(n, 0);
    int64_t omt = 0, yt = 0, zt = 0, ubt = 0, bt = 0;
    for (int a = 0; a < nr; ++a) {
      const int i = R[a];
      rr[a] = m.rows[i];
      rc[a] = m.cols[i];
      rl[a] = width[i];
      om[a] = omt;
      omt += rc[a] * rl[a];
      yo[a] = yt;
      yt += rr[a] * rl[a];
      zo[a] = zt;
      zt += rc[a] * rl[a];
      ub[a] = ut + ubt;  // U_B lives behind the spectra's U blocks in the same buffer
      ubt += rl[a] * rl[a];
    }
    for (int i = 0; i < n; ++i) {
      bo[i] = bt;
      bt += exact[i] ? m.rows[i] * m.cols[i] : width[i] * m.cols[i];
    }
    sp.U = alloc_d(ut + ubt);
    sp.S = alloc_d(sp.s_begin.back());
    sp.V = alloc_d(vt);
    double* Bb = alloc_d(bt);
    double* Q = nr ? alloc_d(yt) : nullptr;
    double* Om = nr ? alloc_d(std::max(omt, zt)) : nullptr;
    double* Y = nr ? alloc_d(yt) : nullptr;
    double* Z = nr ? alloc_d(zt) : nullptr;

    // subspace iterations Q <- orth(A orth(A^T Q)) for the sketched sectors `sub` (indices into R);
    // the basis enters in `cur` (Q or Y) and leaves in Q (last orthonormalisation with 3 passes);
    // the products of the first `lead` iterations run as 3xTF32 tensor-core GEMMs through
    // tc_t (A^T X) and tc_n (A X), which cover all sketched sectors (sub = all)
    // FP64-accurate tensor-core products over every sketched sector (exact_tc), built once per round
    std::unique_ptr<OzProducts> oz_n, oz_t;
    auto iterate = [&](const std::vector<int>& sub, int iters, double* cur, int lead, TcProducts* tc_t,
                       TcProducts* tc_n) {
      if (lead > 0 && (!tc_t || !tc_n || int(sub.size()) != nr))
        throw std::logic_error("randomized tSVD: tensor-core products need every sketched sector");
      const bool use_oz = oz_t && oz_n && int(sub.size()) == nr;
      std::vector<int64_t> srr, src, srl, syo, szo;
      for (int a : sub) {
        srr.push_back(rr[a]);
        src.push_back(rc[a]);
        srl.push_back(rl[a]);
        syo.push_back(yo[a]);
        szo.push_back(zo[a]);
      }
      std::vector<xgb_gemm_desc> g;
      for (int p = 0; p < iters; ++p) {
        if (use_oz) {
          oz_t->apply(t.data(), cur, Z, st);
        } else if (p < lead) {
          tc_t->apply(t.data(), cur, Z, st);
        } else {
          g.clear();
          for (int a : sub) g.push_back({rc[a], rl[a], rr[a], m.offset[R[a]], rr[a], yo[a], rr[a], zo[a], rc[a], 1, 0});
          grouped_gemm(g, t.data(), cur, Z, st);
        }
        // Omega's storage holds Qz (same layout as Z)
        double* qz = orthonormalise(src, srl, szo, Z, Om, st, kInterPasses, exact_tc);
        if (use_oz) {
          oz_n->apply(t.data(), qz, Y, st);
        } else if (p < lead) {
          tc_n->apply(t.data(), qz, Y, st);
        } else {
          g.clear();
          for (int a : sub) g.push_back({rr[a], rl[a], rc[a], m.offset[R[a]], rr[a], zo[a], rc[a], yo[a], rr[a], 0, 0});
          grouped_gemm(g, t.data(), qz, Y, st);
        }
        cur = orthonormalise(srr, srl, syo, Y, Q, st, p + 1 == iters ? 3 : kInterPasses, exact_tc);
      }
    };
    // Rayleigh-Ritz on span(Q) for `sub`: the SVD of B = Q^T A (l x n) through its transpose's QR,
    // Z = A^T Q = Q_z R (shifted CholeskyQR3, R = Q_z^T Z), so that the Jacobi SVD runs on the l x l
    // factor R = U_R S V_R^T instead of the n-long rows of B: U_B = V_R, V_B^T = U_R^T Q_z^T.  R joins
    // the exact sectors `ex` in one batched SVD; then U = Q V_R, V^T = U_R^T Q_z^T and the sign rule.
    auto project = [&](const std::vector<int>& sub, const std::vector<int>& ex) {
      std::vector<xgb_gemm_desc> g;
      std::vector<int64_t> src, srl, szo, r_off;
      std::vector<xgb_copy2d_desc> zc, rc2;
      int64_t rt = 0, mxz = 0, mxr = 0;
      for (int a : sub) {
        const int i = R[a];
        g.push_back({rc[a], rl[a], rr[a], m.offset[i], rr[a], yo[a], rr[a], zo[a], rc[a], 1, 0});  // Z = A^T Q
        src.push_back(rc[a]);
        srl.push_back(rl[a]);
        szo.push_back(zo[a]);
        zc.push_back({zo[a], rc[a], bo[i], rc[a], rc[a], rl[a]});  // keep Z (n x l) in B's slot
        r_off.push_back(rt);
        rc2.push_back({rt, rl[a], bo[i], rl[a], rl[a], rl[a]});    // R (l x l) into B's slot
        rt += rl[a] * rl[a];
        mxz = std::max(mxz, rc[a] * rl[a]);
        mxr = std::max(mxr, rl[a] * rl[a]);
      }
      if (!sub.empty()) {
        if (oz_t && int(sub.size()) == nr) oz_t->apply(t.data(), Q, Z, st);  // same descriptors as A^T X
        else grouped_gemm(g, t.data(), Q, Z, st);
        Staging sc;
        const size_t oz = sc.add(zc), orr = sc.add(rc2);
        sc.upload(st);
        prof_begin(K_COPY2D, st);
        launch_copy2d(sc.at<xgb_copy2d_desc>(oz), int(zc.size()), mxz, Z, Bb, st);
        prof_end(K_COPY2D, st, 16.0 * double(zt));
        orthonormalise(src, srl, szo, Z, Om, st, 3, exact_tc);  // Q_z in Om (Z's layout)
        g.clear();
        for (size_t s2 = 0; s2 < sub.size(); ++s2) {  // R = Q_z^T Z (l x l) into Y
          const int a = sub[s2];
          g.push_back({rl[a], rl[a], rc[a], zo[a], rc[a], bo[R[a]], rc[a], r_off[s2], rl[a], 1, 0});
        }
        grouped_gemm(g, Om, Bb, Y, st, 1.0, 0.0, kGemmDense, exact_tc);
        prof_begin(K_COPY2D, st);
        launch_copy2d(sc.at<xgb_copy2d_desc>(orr), int(rc2.size()), mxr, Y, Bb, st);
        prof_end(K_COPY2D, st, 16.0 * double(rt));
      }
      std::vector<xgb_svd_desc> d;
      for (int i : ex) d.push_back({m.rows[i], m.cols[i], bo[i], sp.u_off[i], sp.s_begin[i], sp.v_off[i]});
      // U_R (l x l) behind the U blocks, V_R^T (l x l, ld l) at the sector's V^dag offset for now
      for (int a : sub) d.push_back({rl[a], rl[a], bo[R[a]], ub[a], sp.s_begin[R[a]], sp.v_off[R[a]]});
      batched_svd(d, Bb, sp.U, sp.S, sp.V, st);
      if (sub.empty()) return;
      g.clear();
      std::vector<SignFixDesc> sf;
      int64_t mx = 0;
      for (int a : sub) {
        const int i = R[a];
        g.push_back({rr[a], rl[a], rl[a], yo[a], rr[a], sp.v_off[i], rl[a], sp.u_off[i], rr[a], 0, 1});  // U = Q V_R
        sf.push_back({rr[a], rc[a], rl[a], sp.u_off[i], sp.v_off[i]});
        mx = std::max(mx, rl[a]);
      }
      grouped_gemm(g, Q, sp.V, sp.U, st);
      g.clear();
      for (int a : sub)  // V^dag = U_R^T Q_z^T (l x n)
        g.push_back({rl[a], rc[a], rl[a], ub[a], rl[a], zo[a], rc[a], sp.v_off[R[a]], rl[a], 1, 1});
      grouped_gemm(g, sp.U, Om, sp.V, st);
      Staging ss;
      const size_t o = ss.add(sf);
      ss.upload(st);
      prof_begin(K_SKETCH, st);
      launch_sign_fix(ss.at<SignFixDesc>(o), int(sf.size()), mx, sp.U, sp.V, st);
      prof_end(K_SKETCH, st, 16.0 * double(yt + vt));
    };

    if (nr) {
      // ---- Omega: seeded Gaussian columns, the first ones replaced by warm-start rows
      {
        std::vector<GaussBlock> gb;
        int64_t mx = 0;
        for (int a = 0; a < nr; ++a) {
          gb.push_back({om[a], rc[a] * rl[a], int64_t(R[a])});
          mx = std::max(mx, rc[a] * rl[a]);
        }
        Staging sg;
        const size_t o = sg.add(gb);
        sg.upload(st);
        prof_begin(K_SKETCH, st);
        launch_gauss_fill(sg.at<GaussBlock>(o), nr, mx, seed, Om, st);
        prof_end(K_SKETCH, st, 8.0 * double(omt));
      }
      if (warm_t.valid()) {
        std::vector<xgb_copy2d_desc> td;  // src k x n (ld k) -> dst n x k (ld n), transposed
        int64_t mx = 0;
        for (int a = 0; a < nr; ++a) {
          const int i = R[a];
          const int64_t kw = std::min<int64_t>(w_rows[i], rl[a]);
          if (w_off[i] < 0 || kw <= 0) continue;
          td.push_back({w_off[i], w_rows[i], om[a], rc[a], kw, rc[a]});
          mx = std::max(mx, kw * rc[a]);
        }
        if (!td.empty()) {
          Staging sw;
          const size_t o = sw.add(td);
          sw.upload(st);
          prof_begin(K_SKETCH, st);
          launch_transpose_copy(sw.at<xgb_copy2d_desc>(o), int(td.size()), mx, warm_t.data(), Om, st);
          prof_end(K_SKETCH, st, 16.0 * double(mx) * double(td.size()));
        }
      }
      // ---- Y = A Omega, Q = orth(Y), subspace iterations
      std::vector<xgb_gemm_desc> g, gt;
      for (int a = 0; a < nr; ++a) {
        // Omega (n x l, ld n) has Z's layout: om[a] == zo[a], so A Omega and A Q_z share descriptors
        g.push_back({rr[a], rl[a], rc[a], m.offset[R[a]], rr[a], om[a], rc[a], yo[a], rr[a], 0, 0});
        gt.push_back({rc[a], rl[a], rr[a], m.offset[R[a]], rr[a], yo[a], rr[a], zo[a], rc[a], 1, 0});
      }
      std::unique_ptr<TcProducts> tc_n, tc_t;
      if (exact_tc) {
        oz_n = std::make_unique<OzProducts>(g, t.data(), st);
        oz_t = std::make_unique<OzProducts>(gt, t.data(), st);
        oz_n->apply(t.data(), Om, Y, st);
      } else if (tc_iters > 0) {
        tc_n = std::make_unique<TcProducts>(g, t.data(), st);
        tc_t = std::make_unique<TcProducts>(gt, t.data(), st);
        tc_n->apply(t.data(), Om, Y, st);
      } else {
        grouped_gemm(g, t.data(), Om, Y, st);
      }
      double* q0 = orthonormalise(rr, rl, yo, Y, Q, st, power_iters > 0 ? kInterPasses : 3, exact_tc);
      std::vector<int> all(nr);
      for (int a = 0; a < nr; ++a) all[a] = a;
      iterate(all, power_iters, q0, tc_iters, tc_t.get(), tc_n.get());
    }
    // ---- exact sectors: their blocks join the batched SVD of the projected blocks
    if (!E.empty()) {
      std::vector<xgb_copy2d_desc> cd;
      int64_t mx = 0;
      for (int i : E) {
        cd.push_back({m.offset[i], m.rows[i], bo[i], m.rows[i], m.rows[i], m.cols[i]});
        mx = std::max(mx, m.rows[i] * m.cols[i]);
      }
      Staging sc;
      const size_t o = sc.add(cd);
      sc.upload(st);
      prof_begin(K_COPY2D, st);
      launch_copy2d(sc.at<xgb_copy2d_desc>(o), int(cd.size()), mx, t.data(), Bb, st);
      prof_end(K_COPY2D, st, 16.0 * double(bt));
    }
    std::vector<int> order(E.begin(), E.end());  // largest exact blocks first
    std::sort(order.begin(), order.end(), [&](int x, int y) {
      return m.rows[x] * m.cols[x] * std::min(m.rows[x], m.cols[x]) > m.rows[y] * m.cols[y] * std::min(m.rows[y], m.cols[y]);
    });
    std::vector<int> all(nr);
    for (int a = 0; a < nr; ++a) all[a] = a;
    project(all, order);

    // ---- residuals ||A v_j - s_j u_j|| of the sketched triplets; refinement of the sectors whose
    // kept triplets miss the tolerance (more subspace iterations from the current basis)
    SVDResult res = truncate_spectra(m, sp, max_keep, eps_svd, false);
    double smax = 0;
    for (double v : res.spectrum) smax = std::max(smax, v);
    for (int pass = 0; nr > 0; ++pass) {
      std::vector<xgb_gemm_desc> g;
      std::vector<SignFixDesc> rd;
      int64_t rtot = 0, mx = 0;
      std::vector<int64_t> r_off(nr);
      for (int a = 0; a < nr; ++a) {
        const int i = R[a];
        // A V into the residual buffer at the U offsets (V = (V^dag)^T, ld of V^dag = l)
        g.push_back({rr[a], rl[a], rc[a], m.offset[i], rr[a], sp.v_off[i], rl[a], sp.u_off[i], rr[a], 0, 1});
        r_off[a] = rtot;
        rd.push_back({rr[a], rtot, rl[a], sp.u_off[i], sp.s_begin[i]});
        rtot += rl[a];
        mx = std::max(mx, rl[a]);
      }
      double* Rb = alloc_d(ut);
      grouped_gemm(g, t.data(), sp.V, Rb, st);
      double* rv = alloc_d(rtot);
      {
        Staging sr;
        const size_t o = sr.add(rd);
        sr.upload(st);
        prof_begin(K_SKETCH, st);
        launch_residual_norms(sr.at<SignFixDesc>(o), nr, mx, Rb, sp.U, sp.S, rv, st);
        prof_end(K_SKETCH, st, 16.0 * double(ut));
      }
      std::vector<double> rh(size_t(std::max<int64_t>(rtot, 1)));
      ok(cudaMemcpyAsync(rh.data(), rv, sizeof(double) * size_t(rtot), cudaMemcpyDeviceToHost, st), "d2h residuals");
      ok(cudaStreamSynchronize(st), "sync");
      if (tc_iters > 0 && pass == 0 && gemm_tc_error(true))
        throw std::runtime_error("randomized tSVD: a tensor-core GEMM CTA gave up waiting for its MMAs");
      dev_free(rv);
      dev_free(Rb);
      std::vector<int> bad;
      double worst = 0;
      for (int a = 0; a < nr; ++a) {
        double ra = 0;
        for (int64_t j = 0; j < std::min<int64_t>(res.keep[R[a]], rl[a]); ++j) ra = std::max(ra, rh[size_t(r_off[a] + j)]);
        worst = std::max(worst, smax > 0 ? ra / smax : 0.0);
        if (res_tol > 0 && smax > 0 && ra > res_tol * smax) bad.push_back(a);
      }
      max_res = worst;
      if (bad.empty() || pass >= kMaxRefine) break;
      ++refinements;
      iterate(bad, std::max(power_iters, 1), Q, 0, nullptr, nullptr);
      project(bad, {});
      res = truncate_spectra(m, sp, max_keep, eps_svd, false);
    }
    if (nr) {
      dev_free(Om);
      dev_free(Y);
      dev_free(Z);
      dev_free(Q);
    }
    dev_free(Bb);
    dev_free(sp.U);
    dev_free(sp.S);
    dev_free(sp.V);
    std::vector<int> sat;
    for (int i : R)
      if (res.keep[i] >= width[i]) sat.push_back(i);
    if (sat.empty()) {
      if (info) {
        info->width = width;
        info->saturated = saturated;
        info->sketch_cols = 0;
        for (int i : R) info->sketch_cols += width[i];
        info->exact_sectors = int(E.size());
        info->refinements = refinements;
        info->max_residual = max_res;
      }
      return res;
    }
    // saturated sectors: double the sketch (the new columns extend the same
    // Gaussian stream); after kMaxRetries doublings they are decomposed exactly
    for (int i : sat) {
      want[i] = 2 * width[i];
      if (round + 1 >= kMaxRetries) exact[i] = 1;
      saturated.push_back(i);
    }
  }
}

Tensor tsvd_backward(const Tensor& A0, const Tensor& U0, const Tensor& S0, const Tensor& Vd0, const Tensor& dU0,
                     const Tensor& dS0, const Tensor& dVd0) {
  // reverse rule of full_svd_impl (ADTensor.hpp:257-301), real scalars, per sector:
  //   dA = U [dS + (J + J^T) S + S (K + K^T)] V^dag + (1 - U U^T) dU S^-1 V^dag + U S^-1 dV^dag (1 - V V^dag)
  //   J = F.(U^T dU), K = F.(V^dag dV^dag^T), F_ij = 1 / (s_j^2 - s_i^2)
  // evaluated as dA = U [N V^dag + S^-1 dV^dag] + (dU S^-1 - U X S^-1) V^dag with X = U^T dU,
  // Y = V^dag dV^dag^T and N = dS + (J + J^T) S + S (K + K^T) - S^-1 Y^T
  // (S^-1 dV^dag V^dag^T V^dag = S^-1 Y^T V^dag).
  Tensor A = materialize(A0), U = materialize(U0), S = materialize(S0), Vd = materialize(Vd0);
  Tensor dU = materialize(dU0), dS = materialize(dS0), dVd = materialize(dVd0);
  const TensorMeta &ma = *A.meta, &mu = *U.meta, &ms = *S.meta, &mv = *Vd.meta;
  if (dU.meta->id != mu.id || dS.meta->id != ms.id || dVd.meta->id != mv.id)
    throw std::runtime_error("svd backward: cotangents must have the structures of U, S, V^dag");
  cudaStream_t st = stream();
  std::vector<SvdBwdDesc> bd;
  std::vector<xgb_gemm_desc> gX, gY, gW, gP, gA1, gA2;
  std::vector<int64_t> a_off;
  int64_t kkt = 0, wt = 0, pt = 0, mxkk = 0, mxsc = 0;
  for (size_t iu = 0; iu < mu.sectors.size(); ++iu) {
    const int q = mu.sectors[iu];
    const int ia = ma.index(q), is = ms.index(q), iv = mv.index(q);
    if (ia < 0 || is < 0 || iv < 0) throw std::runtime_error("svd backward: sector missing in A, S or V^dag");
    const int64_t m = ma.rows[ia], n = ma.cols[ia], k = mu.cols[iu];
    if (mu.rows[iu] != m || mv.cols[iv] != n || mv.rows[iv] != k || ms.rows[is] != k || ms.cols[is] != k)
      throw std::runtime_error("svd backward: block shapes of A, U, S, V^dag disagree");
    SvdBwdDesc d{m, n, k, mu.offset[iu], ms.offset[is], ms.offset[is], k, mv.offset[iv], kkt, wt, pt};
    bd.push_back(d);
    gX.push_back({k, k, m, d.u_off, m, d.u_off, m, kkt, k, 1, 0});            // X = U^T dU
    gY.push_back({k, k, n, d.v_off, k, d.v_off, k, kkt, k, 0, 1});            // Y = V^dag dV^dag^T
    gW.push_back({k, n, k, kkt, k, d.v_off, k, wt, k, 0, 0});                 // W = N V^dag
    gP.push_back({m, k, k, d.u_off, m, kkt, k, pt, m, 0, 0});                 // P -= U XS
    gA1.push_back({m, n, k, d.u_off, m, wt, k, ma.offset[ia], m, 0, 0});      // dA = U W
    gA2.push_back({m, n, k, pt, m, d.v_off, k, ma.offset[ia], m, 0, 0});      // dA += P V^dag
    kkt += k * k;
    wt += k * n;
    pt += m * k;
    mxkk = std::max(mxkk, k * k);
    mxsc = std::max(mxsc, k * n + m * k);
  }
  Tensor dA = zeros(A.meta);
  if (bd.empty()) return dA;
  double* X = alloc_d(kkt);
  double* Y = alloc_d(kkt);
  double* N = alloc_d(kkt);
  double* XS = alloc_d(kkt);
  double* W = alloc_d(wt);
  double* P = alloc_d(pt);
  grouped_gemm(gX, U.data(), dU.data(), X, st);
  grouped_gemm(gY, Vd.data(), dVd.data(), Y, st);
  Staging sb;
  const size_t o = sb.add(bd);
  sb.upload(st);
  prof_begin(K_DIAG, st);
  launch_svd_bwd_mid(sb.at<SvdBwdDesc>(o), int(bd.size()), mxkk, S.data(), X, Y, dS.data(), N, XS, st);
  prof_end(K_DIAG, st, 48.0 * double(kkt));
  grouped_gemm(gW, N, Vd.data(), W, st);
  prof_begin(K_DIAG, st);
  launch_svd_bwd_scale(sb.at<SvdBwdDesc>(o), int(bd.size()), mxsc, S.data(), dVd.data(), dU.data(), W, P, st);
  prof_end(K_DIAG, st, 24.0 * double(wt + pt));
  grouped_gemm(gP, U.data(), XS, P, st, -1.0, 1.0);
  grouped_gemm(gA1, U.data(), W, dA.data(), st);
  grouped_gemm(gA2, P, Vd.data(), dA.data(), st, 1.0, 1.0);
  for (double* p : {X, Y, N, XS, W, P}) dev_free(p);
  return dA;
}

}  // namespace xgb
