// Tensor-level C-ABI (include/xgb_tensor.h) over the C++ host layer.
// No exception crosses the boundary: failures map to XGB_E_* / NULL.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <stdexcept>

#include "../../include/xgb_tensor.h"
#include "rank_model.hpp"
#include "tensor.hpp"

struct xgb_basis_s { xgb::BasisPtr b; };
struct xgb_tensor_s { xgb::Tensor t; };
struct xgb_ctm_s { std::unique_ptr<xgb::CTM> c; };
struct xgb_su_s { std::unique_ptr<xgb::SimpleUpdate> s; };

using namespace xgb;

namespace {
Sym sym_of(int kind) {
  Sym s;
  s.kind = kind;
  s.N = 2;
  return s;
}
xgb_tensor wrap(Tensor t) { return new xgb_tensor_s{std::move(t)}; }
xgb_basis wrapb(BasisPtr b) { return new xgb_basis_s{std::move(b)}; }
}  // namespace

#define GUARD(fail, ...)                               \
  try {                                                \
    __VA_ARGS__                                        \
  } catch (const std::bad_alloc&) {                    \
    set_error(XGB_E_OOM, "device allocation failed");  \
    return fail;                                       \
  } catch (const std::exception& e) {                  \
    set_error(XGB_E_BADPLAN, e.what());                \
    return fail;                                       \
  }

extern "C" {

xgb_basis xgb_basis_create(int sym, int n, const int32_t* qs, const int64_t* dims, int sort) {
  GUARD(nullptr, {
    if (sym < 0 || sym > XGB_SYM_SU2) throw std::runtime_error("unknown symmetry kind");
    std::vector<std::pair<int, int64_t>> pairs;
    for (int i = 0; i < n; ++i) pairs.push_back({qs[i], dims[i]});
    return wrapb(basis_from_pairs(sym_of(sym), pairs, sort != 0));
  })
}
xgb_basis xgb_basis_conj(xgb_basis b) { GUARD(nullptr, { return wrapb(basis_conj(b->b)); }) }
xgb_basis xgb_basis_combine(xgb_basis a, xgb_basis b) { GUARD(nullptr, { return wrapb(basis_combine(a->b, b->b)); }) }
xgb_basis xgb_basis_forget_history(xgb_basis b) { GUARD(nullptr, { return wrapb(basis_forget_history(b->b)); }) }

int xgb_basis_info(xgb_basis b, int32_t* qs, int64_t* dims, int* conj_flag, int* depth) {
  const Qbasis& B = *b->b;
  for (size_t i = 0; i < B.qs.size(); ++i) {
    if (qs) qs[i] = B.qs[i];
    if (dims) dims[i] = B.dims[i];
  }
  if (conj_flag) *conj_flag = B.conj_flag;
  if (depth) *depth = B.depth;
  return int(B.qs.size());
}

int xgb_basis_trees(xgb_basis b, int i, int64_t* out, int cap) {
  const Qbasis& B = *b->b;
  if (i < 0 || i >= int(B.qs.size())) return set_error(XGB_E_BADPLAN, "irrep index out of range");
  int need = 0;
  for (const auto& t : B.trees[i]) need += 3 + 2 * t.rank + t.nqi();
  if (!out) return need;
  if (cap < need) return set_error(XGB_E_BADPLAN, "buffer too small");
  int64_t* o = out;
  for (const auto& t : B.trees[i]) {
    *o++ = t.rank;
    *o++ = t.qc;
    *o++ = t.dual;
    for (int k = 0; k < t.rank; ++k) *o++ = t.qu[k];
    for (int k = 0; k < t.rank; ++k) *o++ = t.dims[k];
    for (int k = 0; k < t.nqi(); ++k) *o++ = t.qi[k];
  }
  return int(B.trees[i].size());
}

void xgb_basis_release(xgb_basis b) { delete b; }

static std::vector<BasisPtr> legs(int n, const xgb_basis* b) {
  std::vector<BasisPtr> v;
  for (int i = 0; i < n; ++i) v.push_back(b[i]->b);
  return v;
}

static Sym sym_from_legs(int rank, const xgb_basis* dom, int corank, const xgb_basis* cod) {
  if (rank > 0) return dom[0]->b->sym;
  if (corank > 0) return cod[0]->b->sym;
  throw std::runtime_error("tensor needs at least one leg");
}

xgb_tensor xgb_tensor_zeros(int rank, const xgb_basis* dom, int corank, const xgb_basis* cod) {
  GUARD(nullptr, {
    Sym s = sym_from_legs(rank, dom, corank, cod);
    return wrap(zeros(make_meta(s, legs(rank, dom), legs(corank, cod))));
  })
}

xgb_tensor xgb_tensor_identity(int rank, const xgb_basis* dom, int corank, const xgb_basis* cod) {
  GUARD(nullptr, {
    Sym s = sym_from_legs(rank, dom, corank, cod);
    return wrap(identity(s, legs(rank, dom), legs(corank, cod)));
  })
}

int xgb_tensor_sectors(xgb_tensor t, int32_t* qs, int64_t* rows, int64_t* cols) {
  const TensorMeta& m = *t->t.meta;
  for (size_t i = 0; i < m.sectors.size(); ++i) {
    if (qs) qs[i] = m.sectors[i];
    if (rows) rows[i] = m.rows[i];
    if (cols) cols[i] = m.cols[i];
  }
  return int(m.sectors.size());
}

int64_t xgb_tensor_size(xgb_tensor t) { return t->t.size(); }

int xgb_tensor_rank(xgb_tensor t, int* rank, int* corank) {
  *rank = t->t.meta->rank();
  *corank = t->t.meta->corank();
  return XGB_OK;
}

xgb_basis xgb_tensor_leg(xgb_tensor t, int leg) {
  const TensorMeta& m = *t->t.meta;
  if (leg < 0 || leg >= m.rank() + m.corank()) { set_error(XGB_E_BADPLAN, "leg out of range"); return nullptr; }
  return wrapb(leg < m.rank() ? m.dom[leg] : m.cod[leg - m.rank()]);
}

xgb_basis xgb_tensor_coupled(xgb_tensor t, int codomain) { return wrapb(codomain ? t->t.meta->ccod : t->t.meta->cdom); }

int xgb_tensor_upload(xgb_tensor t, const double* host, int64_t n) {
  if (n != t->t.size()) return set_error(XGB_E_BADPLAN, "upload: size mismatch");
  GUARD(XGB_E_CUDA, {
    t->t.twist_mask = 0;
    if (t->t.buf.use_count() > 1) t->t.buf = std::make_shared<DevBuf>(n);
    if (n) {
      cudaError_t e = cudaMemcpyAsync(t->t.data(), host, sizeof(double) * n, cudaMemcpyHostToDevice, stream());
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
      if (e != cudaSuccess) return set_error(XGB_E_CUDA, cudaGetErrorString(e));
    }
    return XGB_OK;
  })
}

int xgb_tensor_download(xgb_tensor t, double* host, int64_t n) {
  if (n != t->t.size()) return set_error(XGB_E_BADPLAN, "download: size mismatch");
  GUARD(XGB_E_CUDA, {
    Tensor m = materialize(t->t);
    if (n) {
      cudaError_t e = cudaMemcpyAsync(host, m.data(), sizeof(double) * n, cudaMemcpyDeviceToHost, stream());
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
      if (e != cudaSuccess) return set_error(XGB_E_CUDA, cudaGetErrorString(e));
    }
    return XGB_OK;
  })
}

int xgb_tensor_svspec(xgb_tensor S, int32_t* qs, int64_t* begin, double* values, int64_t cap) {
  // the SVspec map of Tensor::tSVD with RETURN_SPEC (src/Core/Tensor.cpp:618-624): per sector of the
  // truncated singular-value tensor, the diagonal of its block (the kept values, descending)
  GUARD(XGB_E_CUDA, {
    const TensorMeta& m = *S->t.meta;
    const int n = int(m.sectors.size());
    std::vector<double> h(size_t(S->t.size()));
    Tensor mt = materialize(S->t);
    if (!h.empty()) {
      cudaError_t e = cudaMemcpyAsync(h.data(), mt.data(), sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream());
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
      if (e != cudaSuccess) return set_error(XGB_E_CUDA, cudaGetErrorString(e));
    }
    int64_t pos = 0;
    for (int i = 0; i < n; ++i) {
      const int64_t k = std::min(m.rows[i], m.cols[i]);
      if (qs) qs[i] = m.sectors[i];
      if (begin) begin[i] = pos;
      for (int64_t j = 0; j < k; ++j, ++pos)
        if (values && pos < cap) values[pos] = h[size_t(m.offset[i] + j + j * m.rows[i])];
    }
    if (begin) begin[n] = pos;
    return n;
  })
}

double* xgb_tensor_device_data(xgb_tensor t) {
  GUARD(nullptr, {
    t->t = materialize(t->t);
    return t->t.data();
  })
}

xgb_tensor xgb_tensor_permute(xgb_tensor t, int shift, const int32_t* p, int n) {
  GUARD(nullptr, { return wrap(permute(t->t, shift, std::vector<int>(p, p + n))); })
}
xgb_tensor xgb_tensor_permute_adj(xgb_tensor t, int shift, const int32_t* p, int n) {
  GUARD(nullptr, { return wrap(permute_adj(t->t, shift, std::vector<int>(p, p + n))); })
}
xgb_tensor xgb_tensor_svd_backward(xgb_tensor A, xgb_tensor U, xgb_tensor S, xgb_tensor Vdag, xgb_tensor dU,
                                   xgb_tensor dS, xgb_tensor dVdag) {
  GUARD(nullptr, { return wrap(tsvd_backward(A->t, U->t, S->t, Vdag->t, dU->t, dS->t, dVdag->t)); })
}
int xgb_tensor_matmul_backward(xgb_tensor left, xgb_tensor right, xgb_tensor res_adj, xgb_tensor* left_adj,
                               xgb_tensor* right_adj) {
  GUARD(XGB_E_BADPLAN, {
    auto [la, ra] = matmul_backward(left->t, right->t, res_adj->t);
    if (left_adj) *left_adj = wrap(la);
    if (right_adj) *right_adj = wrap(ra);
    return XGB_OK;
  })
}
xgb_tensor xgb_tensor_twist(xgb_tensor t, int leg) { GUARD(nullptr, { return wrap(twist(t->t, leg)); }) }
xgb_tensor xgb_tensor_adjoint(xgb_tensor t) { GUARD(nullptr, { return wrap(adjoint(t->t)); }) }
xgb_tensor xgb_tensor_matmul(xgb_tensor a, xgb_tensor b, int adj_a, int adj_b) {
  GUARD(nullptr, { return wrap(matmul(a->t, b->t, adj_a != 0, adj_b != 0)); })
}
xgb_tensor xgb_tensor_contract(xgb_tensor a, xgb_tensor b, const int32_t* a1, int n1, const int32_t* a2, int n2,
                               int rankres) {
  GUARD(nullptr, {
    return wrap(contract(a->t, b->t, std::vector<int>(a1, a1 + n1), std::vector<int>(a2, a2 + n2), rankres));
  })
}
xgb_tensor xgb_tensor_scale(xgb_tensor t, double s) { GUARD(nullptr, { return wrap(scale(t->t, s)); }) }
double xgb_tensor_max_norm(xgb_tensor t) { GUARD(-1.0, { return max_norm(t->t); }) }
xgb_tensor xgb_tensor_normalize_max(xgb_tensor t) { GUARD(nullptr, { return wrap(normalize_max(t->t)); }) }

int xgb_tensor_tsvd(xgb_tensor t, int64_t max_keep, double eps_svd, int preserve_multiplets, xgb_tensor* U,
                    xgb_tensor* S, xgb_tensor* Vdag, double* trunc_weight, double* entropy, int32_t* keep) {
  GUARD(XGB_E_BADPLAN, {
    SVDResult r = tsvd(t->t, max_keep, eps_svd, preserve_multiplets != 0);
    if (U) *U = wrap(r.U);
    if (S) *S = wrap(r.S);
    if (Vdag) *Vdag = wrap(r.Vdag);
    if (trunc_weight) *trunc_weight = r.trunc_weight;
    if (entropy) *entropy = r.entropy;
    if (keep) for (size_t i = 0; i < r.keep.size(); ++i) keep[i] = r.keep[i];
    return XGB_OK;
  })
}

int xgb_tensor_tsvd_randomized(xgb_tensor t, int64_t max_keep, double eps_svd, int n_sectors, const int64_t* sketch,
                               int power_iters, uint64_t seed, xgb_tensor warm, double res_tol, xgb_tensor* U,
                               xgb_tensor* S, xgb_tensor* Vdag, double* trunc_weight, double* entropy, int32_t* keep,
                               int64_t* width, int32_t* n_saturated) {
  GUARD(XGB_E_BADPLAN, {
    if (n_sectors != int(t->t.meta->sectors.size()) || (n_sectors > 0 && !sketch))
      return set_error(XGB_E_BADPLAN, "randomized tSVD: one sketch width per sector required");
    RsvdInfo info;
    SVDResult r = tsvd_randomized(t->t, max_keep, eps_svd, std::vector<int64_t>(sketch, sketch + n_sectors),
                                  power_iters, seed, &info, warm ? &warm->t : nullptr, res_tol);
    if (U) *U = wrap(r.U);
    if (S) *S = wrap(r.S);
    if (Vdag) *Vdag = wrap(r.Vdag);
    if (trunc_weight) *trunc_weight = r.trunc_weight;
    if (entropy) *entropy = r.entropy;
    if (keep) for (size_t i = 0; i < r.keep.size(); ++i) keep[i] = r.keep[i];
    if (width) for (size_t i = 0; i < info.width.size(); ++i) width[i] = info.width[i];
    if (n_saturated) *n_saturated = int32_t(info.saturated.size());
    return XGB_OK;
  })
}

int xgb_tensor_tqr(xgb_tensor t, xgb_tensor* Q, xgb_tensor* R) {
  GUARD(XGB_E_BADPLAN, {
    auto [q, r] = tqr(t->t);
    *Q = wrap(q);
    *R = wrap(r);
    return XGB_OK;
  })
}

int xgb_decompose(xgb_tensor t1, xgb_tensor t2, int64_t max_nsv, xgb_tensor* P1, xgb_tensor* P2) {
  GUARD(XGB_E_BADPLAN, {
    auto [a, b] = decompose(t1->t, t2->t, max_nsv);
    *P1 = wrap(a);
    *P2 = wrap(b);
    return XGB_OK;
  })
}

void xgb_tensor_release(xgb_tensor t) { delete t; }

xgb_ctm xgb_ctm_create(xgb_tensor A, int64_t chi) {
  GUARD(nullptr, { return new xgb_ctm_s{std::make_unique<CTM>(A->t, chi)}; })
}
int xgb_ctm_init(xgb_ctm c) { GUARD(XGB_E_BADPLAN, { c->c->init(); return XGB_OK; }) }
int xgb_ctm_grow_all(xgb_ctm c) { GUARD(XGB_E_BADPLAN, { c->c->grow_all(); return XGB_OK; }) }
int xgb_ctm_move(xgb_ctm c, char dir) { GUARD(XGB_E_BADPLAN, { c->c->move(dir); return XGB_OK; }) }
xgb_tensor xgb_ctm_get(xgb_ctm c, int which) {
  GUARD(nullptr, {
    if (which < 0 || which > 9) throw std::runtime_error("ctm slot out of range");
    Tensor& t = c->c->slot(which);
    if (!t.valid()) throw std::runtime_error("ctm slot is empty (call xgb_ctm_init)");
    return wrap(t);
  })
}
int xgb_ctm_set(xgb_ctm c, int which, xgb_tensor t) {
  GUARD(XGB_E_BADPLAN, {
    if (which < 0 || which > 7) throw std::runtime_error("ctm slot out of range");
    c->c->slot(which) = t->t;
    return XGB_OK;
  })
}
void xgb_ctm_release(xgb_ctm c) { delete c; }

static int copy_out(const std::vector<uint8_t>& bytes, uint8_t* buf, int64_t cap, int64_t* size) {
  if (size) *size = int64_t(bytes.size());
  if (!buf) return XGB_OK;
  if (cap < int64_t(bytes.size())) return set_error(XGB_E_BADPLAN, "checkpoint: buffer too small");
  std::memcpy(buf, bytes.data(), bytes.size());
  return XGB_OK;
}

int xgb_tensor_serialize(xgb_tensor t, uint8_t* buf, int64_t cap, int64_t* size) {
  GUARD(XGB_E_BADPLAN, {
    if (!t) throw std::runtime_error("checkpoint: null tensor");
    return copy_out(serialize_tensor(t->t), buf, cap, size);
  })
}
xgb_tensor xgb_tensor_deserialize(const uint8_t* buf, int64_t size) {
  GUARD(nullptr, {
    if (!buf || size < 0) throw std::runtime_error("checkpoint: null buffer");
    return wrap(deserialize_tensor(buf, size_t(size)));
  })
}
int xgb_ctm_serialize(xgb_ctm c, uint8_t* buf, int64_t cap, int64_t* size) {
  GUARD(XGB_E_BADPLAN, {
    if (!c) throw std::runtime_error("checkpoint: null CTM");
    return copy_out(serialize_ctm(*c->c), buf, cap, size);
  })
}
xgb_ctm xgb_ctm_deserialize(xgb_tensor A, const uint8_t* buf, int64_t size) {
  GUARD(nullptr, {
    if (!A || !buf || size < 0) throw std::runtime_error("checkpoint: null argument");
    return new xgb_ctm_s{deserialize_ctm(A->t, buf, size_t(size))};
  })
}

xgb_su xgb_su_create(int Lx, int Ly, const int* labels, int n_sites, const xgb_tensor* G, int64_t D) {
  GUARD(nullptr, {
    if (Lx <= 0 || Ly <= 0 || !labels || n_sites <= 0 || !G) throw std::runtime_error("simple update: bad arguments");
    std::vector<Tensor> gs;
    for (int i = 0; i < n_sites; ++i) {
      if (!G[i]) throw std::runtime_error("simple update: null site tensor");
      gs.push_back(G[i]->t);
    }
    std::vector<int> lab(labels, labels + size_t(Lx) * size_t(Ly));
    return new xgb_su_s{std::make_unique<SimpleUpdate>(Lx, Ly, lab, gs, D)};
  })
}
int xgb_su_step(xgb_su s, xgb_tensor Uh, xgb_tensor Uv) {
  GUARD(XGB_E_BADPLAN, {
    if (!s || !Uh || !Uv) throw std::runtime_error("simple update: null argument");
    s->s->step(Uh->t, Uv->t);
    return XGB_OK;
  })
}
int xgb_su_step_h(xgb_su s, int x, int y, xgb_tensor Uh) {
  GUARD(XGB_E_BADPLAN, {
    if (!s || !Uh) throw std::runtime_error("simple update: null argument");
    s->s->step_h(x, y, Uh->t);
    return XGB_OK;
  })
}
int xgb_su_step_v(xgb_su s, int x, int y, xgb_tensor Uv) {
  GUARD(XGB_E_BADPLAN, {
    if (!s || !Uv) throw std::runtime_error("simple update: null argument");
    s->s->step_v(x, y, Uv->t);
    return XGB_OK;
  })
}
xgb_tensor xgb_su_get(xgb_su s, int which, int site) {
  GUARD(nullptr, {
    if (!s) throw std::runtime_error("simple update: null handle");
    if (site < 0 || site >= int(s->s->G.size())) throw std::runtime_error("simple update: site out of range");
    switch (which) {
      case 0: return wrap(s->s->G[size_t(site)]);
      case 1: return wrap(s->s->wh[size_t(site)]);
      case 2: return wrap(s->s->wv[size_t(site)]);
      case 3: return wrap(s->s->site_tensor(site));
      default: throw std::runtime_error("simple update slot out of range");
    }
  })
}
void xgb_su_release(xgb_su s) { delete s; }

int xgb_ctm_set_svd(xgb_ctm c, int mode, int power_iters, uint64_t seed, int64_t oversample, double growth) {
  GUARD(XGB_E_BADPLAN, {
    if (mode != 0 && mode != 1) throw std::runtime_error("svd mode must be 0 (exact) or 1 (randomized)");
    if (power_iters < 0 || oversample < 0 || growth < 0) throw std::runtime_error("negative randomized tSVD parameter");
    CTM& m = *c->c;
    m.svd_mode = mode;
    m.power_iters = power_iters;
    m.seed = seed;
    auto hp = std::make_shared<HistoryPolicy>();
    hp->oversample = oversample;
    hp->growth = growth;
    m.policy = hp;
    return XGB_OK;
  })
}

int xgb_set_gemm_precision(int precision) {
  GUARD(XGB_E_BADPLAN, {
    if (!gemm_precision_available(precision))
      return set_error(XGB_E_UNSUPPORTED, "GEMM precision form not available");
    set_gemm_precision(precision);
    return XGB_OK;
  })
}

int xgb_ctm_set_gemm_precision(xgb_ctm c, int precision) {
  GUARD(XGB_E_BADPLAN, {
    if (!gemm_precision_available(precision))
      return set_error(XGB_E_UNSUPPORTED, "GEMM precision form not available");
    c->c->gemm_prec = precision;
    return XGB_OK;
  })
}

int xgb_ctm_set_concurrent(xgb_ctm c, int on) {
  GUARD(XGB_E_BADPLAN, {
    c->c->concurrent = on != 0;
    return XGB_OK;
  })
}

int xgb_ctm_set_sketch_unseen(xgb_ctm c, int on) {
  GUARD(XGB_E_BADPLAN, {
    c->c->sketch_unseen = on != 0;
    return XGB_OK;
  })
}

int xgb_ctm_set_sketch_precision(xgb_ctm c, int fp64_tail) {
  GUARD(XGB_E_BADPLAN, {
    c->c->sketch_fp64_tail = fp64_tail < 0 ? -1 : fp64_tail;
    return XGB_OK;
  })
}

int xgb_ctm_set_warm_start(xgb_ctm c, int warm_iters) {
  GUARD(XGB_E_BADPLAN, {
    c->c->warm_iters = warm_iters < 0 ? -1 : warm_iters;
    if (warm_iters < 0)
      for (auto& w : c->c->warm_v) w = Tensor();
    return XGB_OK;
  })
}

int xgb_ctm_set_residual_tol(xgb_ctm c, double tol) {
  GUARD(XGB_E_BADPLAN, {
    if (!(tol >= 0)) throw std::runtime_error("residual tolerance must be >= 0");
    c->c->res_tol = tol;
    return XGB_OK;
  })
}

int xgb_ctm_residual_stats(xgb_ctm c, int64_t* refinements, double* max_residual) {
  GUARD(XGB_E_BADPLAN, {
    if (refinements) *refinements = c->c->stats.refinements;
    if (max_residual) *max_residual = c->c->stats.max_residual;
    return XGB_OK;
  })
}

int xgb_ctm_stats(xgb_ctm c, int64_t* out5) {
  GUARD(XGB_E_BADPLAN, {
    const CTMStats& s = c->c->stats;
    out5[0] = s.decompositions;
    out5[1] = s.sketched_sectors;
    out5[2] = s.exact_sectors;
    out5[3] = s.redo;
    out5[4] = s.sketch_cols;
    return XGB_OK;
  })
}

int xgb_ctm_record(xgb_ctm c, int on) {
  GUARD(XGB_E_BADPLAN, {
    c->c->record = on != 0;
    if (!on) c->c->records.clear();
    return XGB_OK;
  })
}

int xgb_ctm_record_count(xgb_ctm c) { GUARD(XGB_E_BADPLAN, { return int(c->c->records.size()); }) }

int xgb_ctm_record_get(xgb_ctm c, int i, int* dir, int* n_sectors, int64_t* n_spectrum, int32_t* sectors,
                       float* features, int64_t* keep, int64_t* width, int64_t* kmin, double* spectrum,
                       int64_t* spec_begin) {
  GUARD(XGB_E_BADPLAN, {
    const auto& R = c->c->records;
    if (i < 0 || i >= int(R.size())) throw std::runtime_error("record index out of range");
    const DecompRecord& r = R[size_t(i)];
    const size_t n = r.sectors.size();
    if (dir) *dir = r.dir;
    if (n_sectors) *n_sectors = int(n);
    if (n_spectrum) *n_spectrum = int64_t(r.spectrum.size());
    for (size_t a = 0; a < n; ++a) {
      if (sectors) sectors[a] = r.sectors[a];
      if (keep) keep[a] = r.keep[a];
      if (width) width[a] = r.width[a];
      if (kmin) kmin[a] = r.kmin[a];
    }
    if (features) std::memcpy(features, r.features.data(), sizeof(float) * r.features.size());
    if (spectrum) std::memcpy(spectrum, r.spectrum.data(), sizeof(double) * r.spectrum.size());
    if (spec_begin) std::memcpy(spec_begin, r.spec_begin.data(), sizeof(int64_t) * r.spec_begin.size());
    return XGB_OK;
  })
}

struct xgb_rank_model_s {
  std::shared_ptr<RankModel> m;
};

int xgb_rank_model_num_params(void) { return kMlpParams; }
int xgb_rank_model_num_features(void) { return kMlpIn; }

xgb_rank_model xgb_rank_model_create(uint64_t seed) {
  GUARD(nullptr, { return new xgb_rank_model_s{std::make_shared<RankModel>(seed)}; })
}
void xgb_rank_model_release(xgb_rank_model m) { delete m; }

int xgb_rank_model_get_params(xgb_rank_model m, float* out, int cap) {
  GUARD(XGB_E_BADPLAN, {
    if (cap < kMlpParams) throw std::runtime_error("parameter buffer too small");
    m->m->get_params(out);
    return XGB_OK;
  })
}
int xgb_rank_model_set_params(xgb_rank_model m, const float* in, int n) {
  GUARD(XGB_E_BADPLAN, {
    if (n != kMlpParams) throw std::runtime_error("wrong parameter count");
    m->m->set_params(in);
    return XGB_OK;
  })
}
int xgb_rank_model_predict(xgb_rank_model m, const float* X, int64_t n, float* Y) {
  GUARD(XGB_E_BADPLAN, {
    m->m->predict(X, n, Y);
    return XGB_OK;
  })
}
int xgb_rank_model_gradient(xgb_rank_model m, const float* X, const float* T, int64_t n, float* grad, double* loss) {
  GUARD(XGB_E_BADPLAN, {
    const double l = m->m->gradient(X, T, n, grad);
    if (loss) *loss = l;
    return XGB_OK;
  })
}
int xgb_rank_model_train(xgb_rank_model m, const float* X, const float* T, int64_t n, int steps, float lr,
                         double* loss) {
  GUARD(XGB_E_BADPLAN, {
    const double l = m->m->train(X, T, n, steps, lr);
    if (loss) *loss = l;
    return XGB_OK;
  })
}
int xgb_ctm_set_rank_model(xgb_ctm c, xgb_rank_model m, double margin, int64_t min_oversample, int power_iters,
                           uint64_t seed) {
  GUARD(XGB_E_BADPLAN, {
    if (margin < 0 || min_oversample < 0 || power_iters < 0) throw std::runtime_error("negative width parameter");
    auto pol = std::make_shared<MlpPolicy>();
    pol->model = m->m;
    pol->margin = margin;
    pol->min_oversample = min_oversample;
    CTM& t = *c->c;
    t.policy = pol;
    t.svd_mode = 1;
    t.power_iters = power_iters;
    t.seed = seed;
    return XGB_OK;
  })
}

xgb_tensor xgb_ctm_rdm(xgb_ctm c, int vertical) { GUARD(nullptr, { return wrap(c->c->rdm(vertical != 0)); }) }

int xgb_ctm_solve(xgb_ctm c, xgb_tensor H, double tol_E, int max_steps, double* E, int* steps, int* flags,
                  double* energies, int cap) {
  GUARD(XGB_E_BADPLAN, {
    if (!c || !H) return set_error(XGB_E_BADPLAN, "xgb_ctm_solve: null handle");
    if (max_steps < 0) return set_error(XGB_E_BADPLAN, "xgb_ctm_solve: max_steps < 0");
    const CTM::SolveResult r = c->c->solve(H->t, tol_E, max_steps);
    if (E) *E = r.E;
    if (steps) *steps = r.steps;
    if (flags) *flags = (r.converged ? 1 : 0) | (r.oscillation ? 2 : 0);
    if (energies)
      for (int i = 0; i < cap && i < int(r.energies.size()); ++i) energies[i] = r.energies[i];
    return XGB_OK;
  })
}

int xgb_tensor_bond_expectation(xgb_tensor rho, xgb_tensor op, double* out) {
  GUARD(XGB_E_BADPLAN, {
    *out = bond_expectation(rho->t, op->t);
    return XGB_OK;
  })
}

xgb_tensor xgb_tensor_meta(int rank, const xgb_basis* dom, int corank, const xgb_basis* cod) {
  GUARD(nullptr, {
    Sym s = sym_from_legs(rank, dom, corank, cod);
    Tensor t;
    t.meta = make_meta(s, legs(rank, dom), legs(corank, cod));
    return wrap(t);
  })
}

static xgb_tensor meta_handle(const MetaPtr& m) {
  Tensor t;
  t.meta = m;
  return wrap(t);
}

int xgb_permute_plan_host(xgb_tensor t, int shift, const int32_t* p, int n, uint32_t twist_mask, int* n_tasks,
                          int* n_contrib, xgb_perm_task* tasks, int task_cap, xgb_perm_contrib* contribs,
                          int contrib_cap, xgb_tensor* out_meta) {
  GUARD(XGB_E_BADPLAN, {
    const TensorMeta& m = *t->t.meta;
    if (n != m.rank() + m.corank()) throw std::runtime_error("permutation length mismatch");
    PermTables pt = build_perm_tables(m, twist_mask, shift, std::vector<int>(p, p + n));
    *n_tasks = int(pt.tasks.size());
    *n_contrib = int(pt.contribs.size());
    if (tasks) {
      if (task_cap < *n_tasks) throw std::runtime_error("task buffer too small");
      std::memcpy(tasks, pt.tasks.data(), sizeof(xgb_perm_task) * pt.tasks.size());
    }
    if (contribs) {
      if (contrib_cap < *n_contrib) throw std::runtime_error("contribution buffer too small");
      std::memcpy(contribs, pt.contribs.data(), sizeof(xgb_perm_contrib) * pt.contribs.size());
    }
    if (out_meta) *out_meta = meta_handle(pt.out);
    return XGB_OK;
  })
}

int xgb_gemm_plan_host(xgb_tensor a, int adj_a, xgb_tensor b, int adj_b, int* n, xgb_gemm_desc* descs, int cap,
                       xgb_tensor* out_meta) {
  GUARD(XGB_E_BADPLAN, {
    GemmTables gt = build_gemm_tables(*a->t.meta, adj_a != 0, *b->t.meta, adj_b != 0);
    *n = int(gt.descs.size());
    if (descs) {
      if (cap < *n) throw std::runtime_error("descriptor buffer too small");
      std::memcpy(descs, gt.descs.data(), sizeof(xgb_gemm_desc) * gt.descs.size());
    }
    if (out_meta) *out_meta = meta_handle(gt.out);
    return XGB_OK;
  })
}

int xgb_contract_perms(const int32_t* a1, int n1, int rank1, const int32_t* a2, int n2, int rank2, int rankres,
                       int32_t* out) {
  GUARD(XGB_E_BADPLAN, {
    ContractPerms cp = get_permutations(std::vector<int>(a1, a1 + n1), rank1, std::vector<int>(a2, a2 + n2), rank2, rankres);
    int k = 0;
    for (int x : cp.p1) out[k++] = x;
    out[k++] = cp.shift1;
    for (int x : cp.p2) out[k++] = x;
    out[k++] = cp.shift2;
    for (int x : cp.pres) out[k++] = x;
    out[k++] = cp.shiftres;
    return int(cp.pres.size());
  })
}

int xgb_plan_cache_stats(int64_t* out4) {
  CacheStats s = cache_stats();
  out4[0] = s.perm_hits;
  out4[1] = s.perm_misses;
  out4[2] = s.gemm_hits;
  out4[3] = s.gemm_misses;
  return XGB_OK;
}

}  // extern "C"
