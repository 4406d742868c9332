// Device tensor operations: plan building (host) + grouped launches (device).
// Every function cites the reference routine whose semantics it follows.
#include "tensor.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <unordered_map>
#include <mutex>
#include <numeric>
#include <sstream>
#include <stdexcept>

namespace xgb {

static constexpr double kCoeffCut = 1.0e-10;  // src/Core/Tensor.cpp:127,193

static void cuda_ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    set_error(XGB_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
  }
}

// Device copies of a plan's host tables.  Each table is a stream-ordered pool allocation filled by an
// asynchronous copy, so building a plan neither allocates with cudaMalloc nor waits for the device
// (both stall a queue that a synchronisation has just drained).  The host tables live as long as the
// plan, so no copy can read freed host memory; the device memory is released in stream order when
// the last user drops the plan.  Plans are shared by the lanes of a fork-join section: a side lane
// waits for its uploads before the plan is published (the other lane may use it at once), and once
// sections have run the release also waits for the work enqueued on every lane.
struct PlanMem {
  std::vector<void*> dev;
  std::vector<std::shared_ptr<const void>> host;
  PlanMem() = default;
  PlanMem(const PlanMem&) = delete;
  PlanMem& operator=(const PlanMem&) = delete;
  ~PlanMem() {
    if (dev.empty()) return;
    if (lanes_used()) order_after_lanes(stream());
    for (void* d : dev) dev_free(d);
  }
  template <class T>
  T* table(std::vector<T> v) {
    auto h = std::make_shared<const std::vector<T>>(std::move(v));
    T* d = static_cast<T*>(dev_alloc(sizeof(T) * std::max<size_t>(h->size(), 1)));
    dev.push_back(d);
    if (!h->empty())
      cuda_ok(cudaMemcpyAsync(d, h->data(), sizeof(T) * h->size(), cudaMemcpyHostToDevice, stream()), "plan upload");
    if (lane() != 0) cuda_ok(cudaStreamSynchronize(stream()), "plan upload");
    host.push_back(h);
    return d;
  }
};

// plan caches hold at most this many plans each; a full cache is emptied (plans still in use stay
// alive through their shared pointers), which bounds the memory of runs whose shapes keep changing
constexpr size_t kPlanCacheCap = 4096;

// ======================================================================= meta
namespace {
std::mutex g_meta_mu;
std::unordered_map<std::string, std::shared_ptr<const TensorMeta>> g_metas;  // metas are small; keep them for plan reuse
uint64_t g_meta_next = 1;
}  // namespace

static MetaPtr finish_meta(TensorMeta&& m) {
  std::ostringstream os;
  os << m.sym.kind << ':' << m.sym.N << '|';
  for (auto& b : m.dom) os << b->id << ',';
  os << '|';
  for (auto& b : m.cod) os << b->id << ',';
  os << '|';
  for (int q : m.sectors) os << q << ',';
  std::string key = os.str();
  std::lock_guard<std::mutex> lk(g_meta_mu);
  auto it = g_metas.find(key);
  if (it != g_metas.end()) return it->second;
  m.id = g_meta_next++;
  auto sp = std::make_shared<const TensorMeta>(std::move(m));
  g_metas[key] = sp;
  return sp;
}

static void fill_blocks(TensorMeta& m) {
  m.rows.clear(); m.cols.clear(); m.offset.clear(); m.dict.clear();
  int64_t cur = 0;
  for (size_t i = 0; i < m.sectors.size(); ++i) {
    int q = m.sectors[i];
    m.dict[q] = int(i);
    m.rows.push_back(m.cdom->inner_dim(q));
    m.cols.push_back(m.ccod->inner_dim(q));
    m.offset.push_back(cur);
    cur += m.rows.back() * m.cols.back();
  }
  m.size = cur;
}

MetaPtr make_meta(const Sym& s, const std::vector<BasisPtr>& dom, const std::vector<BasisPtr>& cod) {
  if (dom.size() + cod.size() > kMaxRank) throw std::runtime_error("tensor rank exceeds 8 legs");
  TensorMeta m;
  m.sym = s;
  m.dom = dom;
  m.cod = cod;
  m.cdom = build_fusion_tree(s, dom);
  m.ccod = build_fusion_tree(s, cod);
  for (int q : m.cdom->qs)
    if (m.ccod->index(q) >= 0) m.sectors.push_back(q);  // StorageType_contiguous.hpp:79-97
  fill_blocks(m);
  return finish_meta(std::move(m));
}

MetaPtr make_meta_ordered(const Sym& s, const std::vector<BasisPtr>& dom, const std::vector<BasisPtr>& cod,
                          const std::vector<int>& sectors) {
  TensorMeta m;
  m.sym = s;
  m.dom = dom;
  m.cod = cod;
  m.cdom = build_fusion_tree(s, dom);
  m.ccod = build_fusion_tree(s, cod);
  m.sectors = sectors;
  fill_blocks(m);
  return finish_meta(std::move(m));
}

DevBuf::DevBuf(int64_t n_) : n(n_) { p = static_cast<double*>(dev_alloc(sizeof(double) * std::max<int64_t>(n_, 1))); }
DevBuf::~DevBuf() { dev_free(p); }

Tensor empty_like_meta(const MetaPtr& m) {
  Tensor t;
  t.meta = m;
  t.buf = std::make_shared<DevBuf>(m->size);
  return t;
}

Tensor zeros(const MetaPtr& m) {
  Tensor t = empty_like_meta(m);
  if (m->size) cuda_ok(cudaMemsetAsync(t.data(), 0, sizeof(double) * m->size, stream()), "memset");
  return t;
}

// ======================================================================= permute plans
namespace {
struct PermPlan {
  PlanMem mem;
  MetaPtr out;
  bool needs_zero = false;
  int n_tasks = 0;
  int64_t total_rows = 0;
  int group = 1;
  bool narrow = true;
  bool single = true;
  xgb_perm_task* d_tasks = nullptr;
  int64_t* d_row_start = nullptr;
  xgb_perm_contrib* d_contribs = nullptr;
  double bytes = 0;  // algorithmic: every output written once, every contribution read once
};
struct GemmPlan {
  PlanMem mem;
  MetaPtr out;
  double flops = 0;  // useful 2*m*n*k summed over groups
  int n_tiles = 0, tile = 16;
  xgb_gemm_desc* d_descs = nullptr;
  GemmTile* d_tiles = nullptr;
  // tensor-core form (built on first use): packing tasks, groups, 128 x 128 tiles
  bool tc_ready = false;
  int n_tc_tiles = 0, n_tc_tasks = 0;
  int64_t tc_a_floats = 0, tc_b_floats = 0;
  TcGroup* d_tc_groups = nullptr;
  TcPackTask* d_tc_tasks = nullptr;
  GemmTile* d_tc_tiles = nullptr;
  std::vector<xgb_gemm_desc> host_descs;
  // FP64-accurate tensor-core form from exact BF16 slices (built on first use); oz_route: whether
  // this product takes it (k too short to amortise the per-tile cost: the FP64 CUDA-core kernel)
  bool oz_ready = false, oz_route = true, oz_routed = false;
  int n_oz_tiles = 0, n_oz_tasks = 0, n_oz_red = 0, oz_slots = 0;
  SplitReduce* d_oz_red = nullptr;
  int64_t oz_a_bytes = 0, oz_b_bytes = 0, oz_rowmax = 0;
  OzGroup* d_oz_groups = nullptr;
  TcPackTask* d_oz_tasks = nullptr;
  GemmTile* d_oz_tiles = nullptr;
  // FP64 launch shape (tile edge, split-K): the built-in rule, or the autotuner's choice (built on
  // first use); the FP32 form's one-CTA-per-tile list likewise
  bool f64_ready = false, tiles_ready = false;
  F64Plan f64;
  GemmTile* d_f64_tiles = nullptr;
  SplitReduce* d_f64_red = nullptr;
};
std::shared_ptr<PermPlan> upload_tables(const PermTables& t) {
  auto plan = std::make_shared<PermPlan>();
  plan->out = t.out;
  plan->n_tasks = int(t.tasks.size());
  plan->needs_zero = t.needs_zero;
  plan->d_tasks = plan->mem.table(t.tasks);
  const PermRows rows = perm_rows(t.tasks.data(), int(t.tasks.size()), t.contribs.data(), int(t.contribs.size()));
  plan->total_rows = rows.total_rows;
  plan->group = rows.group;
  plan->narrow = rows.narrow;
  plan->single = rows.single;
  plan->d_row_start = plan->mem.table(rows.row_start);
  plan->d_contribs = plan->mem.table(t.contribs);
  for (const auto& task : t.tasks) plan->bytes += 8.0 * double(task.nelem) * (1 + task.n_contrib);
  return plan;
}
std::mutex g_plan_mu;
std::unordered_map<std::string, std::shared_ptr<PermPlan>> g_perm_plans;
std::unordered_map<std::string, std::shared_ptr<GemmPlan>> g_gemm_plans;
CacheStats g_stats;

struct TaskBuilder {
  // one entry per contribution, in insertion order; tables() merges the entries of one destination
  // sub-block (abelian symmetries have exactly one, so no lookup structure is kept while adding)
  std::vector<xgb_perm_task> tasks;
  std::vector<xgb_perm_contrib> cons;

  void add(int64_t dst_base, int rank, const int32_t* dims, const int64_t* dst_stride, int64_t src_base,
           const int64_t* src_stride, double coeff) {
    xgb_perm_task t{};
    t.dst_base = dst_base;
    t.rank = rank;
    t.nelem = 1;
    for (int k = 0; k < rank; ++k) {
      t.dims[k] = dims[k];
      t.dst_stride[k] = dst_stride[k];
      t.nelem *= dims[k];
    }
    tasks.push_back(t);
    xgb_perm_contrib c{};
    c.src_base = src_base;
    c.coeff = coeff;
    for (int k = 0; k < rank; ++k) c.src_stride[k] = src_stride[k];
    cons.push_back(c);
  }

  // tasks in ascending destination offset, each task's contributions contiguous in insertion order
  PermTables tables(const MetaPtr& out) const {
    PermTables t;
    t.out = out;
    std::vector<int> order(tasks.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return tasks[a].dst_base < tasks[b].dst_base; });
    t.tasks.reserve(tasks.size());
    t.contribs.reserve(cons.size());
    t.start.reserve(tasks.size() + 1);
    t.start.push_back(0);
    for (size_t r = 0; r < order.size();) {
      size_t e = r + 1;
      while (e < order.size() && tasks[order[e]].dst_base == tasks[order[r]].dst_base) ++e;
      xgb_perm_task task = tasks[order[r]];
      for (size_t x = r + 1; x < e; ++x)
        for (int k = 0; k < task.rank; ++k)
          if (tasks[order[x]].dims[k] != task.dims[k])
            throw std::runtime_error("permute plan: inconsistent sub-block shapes");
      task.contrib0 = int32_t(t.contribs.size());
      task.n_contrib = int32_t(e - r);
      for (size_t x = r; x < e; ++x) t.contribs.push_back(cons[order[x]]);
      t.tasks.push_back(task);
      t.start.push_back(t.start.back() + task.nelem);
      r = e;
    }
    t.needs_zero = t.start.back() < out->size;
    return t;
  }

  std::shared_ptr<PermPlan> finish(const MetaPtr& out) const { return upload_tables(tables(out)); }
};

// column-major strides of a sub-tensor with the given leg dims; codomain
// legs are additionally scaled by the block's leading dimension.
void sub_strides(const FusionTree& f1, const FusionTree& f2, int64_t ld, int64_t* st) {
  int64_t acc = 1;
  for (int m = 0; m < f1.rank; ++m) { st[m] = acc; acc *= f1.dims[m]; }
  acc = ld;
  for (int m = 0; m < f2.rank; ++m) { st[f1.rank + m] = acc; acc *= f2.dims[m]; }
}

double twist_coeff(const Sym& s, uint32_t mask, const FusionTree& f1, const FusionTree& f2) {
  double c = 1.0;
  if (!mask) return c;
  for (int l = 0; l < f1.rank + f2.rank; ++l)
    if ((mask >> l) & 1u) c *= (l < f1.rank) ? s.coeff_twist(f1.qu[l]) : s.coeff_twist(f2.qu[l - f1.rank]);
  return c;
}

}  // namespace

PermTables build_perm_tables(const TensorMeta& in, uint32_t mask, int shift, const std::vector<int>& p) {
  const Sym& s = in.sym;
  const int R = in.rank(), C = in.corank(), N = R + C;
  const int newR = R - shift, newC = C + shift;
  std::vector<int> pd(p.begin(), p.begin() + newR), pc(p.begin() + newR, p.end());
  const bool identity = (shift == 0) && [&] {
    for (int i = 0; i < N; ++i) if (p[i] != i) return false;
    return true;
  }();
  const bool within = !identity && shift == 0 && std::all_of(pd.begin(), pd.end(), [&](int x) { return x < R; }) &&
                      std::all_of(pc.begin(), pc.end(), [&](int x) { return x >= R; });
  // output bases (Tensor.cpp:100-106 for the within path, 157-176 otherwise)
  std::vector<BasisPtr> nd, nc;
  if (identity) {
    nd = in.dom;
    nc = in.cod;
  } else if (within) {
    for (int x : pd) nd.push_back(in.dom[x]);
    for (int x : pc) nc.push_back(in.cod[x - R]);
  } else {
    for (int i = 0; i < newR; ++i) nd.push_back((p[i] > R - 1 || R == 0) ? in.cod[p[i] - R] : in.dom[p[i]]);
    for (int i = 0; i < newR; ++i) if (p[i] > R - 1 || R == 0) nd[i] = basis_conj(nd[i]);
    for (int i = 0; i < newC; ++i) {
      int x = p[i + newR];
      nc.push_back((x > R - 1 || R == 0) ? in.cod[x - R] : basis_conj(in.dom[x]));
    }
  }
  MetaPtr out = identity ? make_meta_ordered(s, nd, nc, in.sectors) : make_meta(s, nd, nc);
  std::vector<int> pdd, pcc;
  for (int x : pd) pdd.push_back(x);
  for (int x : pc) pcc.push_back(x - R);

  TaskBuilder tb;
  int64_t ist[kMaxRank], ost[kMaxRank], sst[kMaxRank];
  int32_t odims[kMaxRank];
  for (size_t si = 0; si < in.sectors.size(); ++si) {
    const int q = in.sectors[si];
    const int dq = in.cdom->index(q), cq = in.ccod->index(q);
    for (const auto& f1 : in.cdom->trees[dq]) {
      for (const auto& f2 : in.ccod->trees[cq]) {
        const double tw = twist_coeff(s, mask, f1, f2);
        const int64_t src_base = in.offset[si] + in.cdom->left_offset(f1) + in.ccod->left_offset(f2) * in.rows[si];
        sub_strides(f1, f2, in.rows[si], ist);
        auto emit = [&](const FusionTree& g1, const FusionTree& g2, double coeff, const std::vector<int>& ptot) {
          const int oq = out->index(g1.qc);
          if (oq < 0) throw std::runtime_error("permute plan: output sector missing");
          const int64_t dst_base = out->offset[oq] + out->cdom->left_offset(g1) + out->ccod->left_offset(g2) * out->rows[oq];
          sub_strides(g1, g2, out->rows[oq], ost);
          for (int k = 0; k < N; ++k) {
            odims[k] = (k < g1.rank) ? g1.dims[k] : g2.dims[k - g1.rank];
            sst[k] = ist[ptot[k]];
          }
          tb.add(dst_base, N, odims, ost, src_base, sst, coeff * tw);
        };
        if (identity) {
          std::vector<int> ptot(N);
          std::iota(ptot.begin(), ptot.end(), 0);
          emit(f1, f2, 1.0, ptot);
        } else if (within) {
          // permute_impl(pd, pc) (Tensor.cpp:83-146)
          TreeMap a = tree_permute(s, f1, pdd), b = tree_permute(s, f2, pcc);
          std::vector<int> ptot = p;
          for (const auto& [g1, c1] : a)
            for (const auto& [g2, c2] : b) {
              if (std::abs(c1 * c2) < kCoeffCut) continue;
              emit(g1, g2, c1 * c2, ptot);
            }
        } else if (s.abelian() && !s.fermionic()) {
          FusionTree g1, g2;  // the one permuted pair, coefficient 1
          treepair_permute_abelian(s, shift, f1, f2, p, g1, g2);
          emit(g1, g2, 1.0, p);
        } else {
          // permute_impl<shift>(p) (Tensor.cpp:148-214)
          for (const auto& [pr, c] : treepair_permute(s, shift, f1, f2, p)) {
            if (std::abs(c) < kCoeffCut) continue;
            emit(pr.first, pr.second, c, p);
          }
        }
      }
    }
  }
  return tb.tables(out);
}

PermTables build_perm_adj_tables(const TensorMeta& in, int shift, const std::vector<int>& p) {
  // Tensor::permute_adj<shift, p...> (Tensor.cpp:258-333): `in` is shaped like
  // the output of permute<shift, p>; every sub-block (f1, f2) of the result
  // (shaped like that permute's input) gathers coeff * shuffle^-1 of the
  // sub-blocks that the forward treepair::permute maps (f1, f2) to.
  const Sym& s = in.sym;
  const int R = in.rank(), C = in.corank(), N = R + C;
  const int newR = R + shift, newC = C - shift;
  std::vector<int> pinv(N);
  for (int i = 0; i < N; ++i) pinv[p[i]] = i;
  std::vector<BasisPtr> nd, nc;
  for (int i = 0; i < newR; ++i)
    nd.push_back((pinv[i] > R - 1 || R == 0) ? basis_conj(in.cod[pinv[i] - R]) : in.dom[pinv[i]]);
  for (int i = 0; i < newC; ++i) {
    const int x = pinv[i + newR];
    nc.push_back((x > R - 1 || R == 0) ? in.cod[x - R] : basis_conj(in.dom[x]));
  }
  MetaPtr out = make_meta(s, nd, nc);
  TaskBuilder tb;
  int64_t ist[kMaxRank], ost[kMaxRank], sst[kMaxRank];
  int32_t odims[kMaxRank];
  for (size_t so = 0; so < out->sectors.size(); ++so) {
    const int q = out->sectors[so];
    const int dq = out->cdom->index(q), cq = out->ccod->index(q);
    for (const auto& f1 : out->cdom->trees[dq]) {
      for (const auto& f2 : out->ccod->trees[cq]) {
        const int64_t dst_base = out->offset[so] + out->cdom->left_offset(f1) + out->ccod->left_offset(f2) * out->rows[so];
        sub_strides(f1, f2, out->rows[so], ost);
        for (int k = 0; k < N; ++k) odims[k] = (k < f1.rank) ? f1.dims[k] : f2.dims[k - f1.rank];
        for (const auto& [pr, c] : treepair_permute(s, shift, f1, f2, p)) {
          if (std::abs(c) < kCoeffCut) continue;
          const FusionTree& g1 = pr.first;
          const FusionTree& g2 = pr.second;
          const int si = in.index(g1.qc);
          if (si < 0) throw std::runtime_error("permute_adj plan: input sector missing");
          const int64_t src_base = in.offset[si] + in.cdom->left_offset(g1) + in.ccod->left_offset(g2) * in.rows[si];
          sub_strides(g1, g2, in.rows[si], ist);
          for (int k = 0; k < N; ++k) sst[k] = ist[pinv[k]];
          tb.add(dst_base, N, odims, ost, src_base, sst, c);
        }
      }
    }
  }
  return tb.tables(out);
}

namespace {
std::string perm_key(const TensorMeta& m, uint32_t mask, int shift, const std::vector<int>& p) {
  std::ostringstream os;
  os << m.id << '|' << mask << '|' << shift << '|';
  for (int x : p) os << x << ',';
  return os.str();
}

std::shared_ptr<PermPlan> get_perm_plan(const TensorMeta& m, uint32_t mask, int shift, const std::vector<int>& p) {
  std::string key = perm_key(m, mask, shift, p);
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_perm_plans.find(key);
    if (it != g_perm_plans.end()) { ++g_stats.perm_hits; return it->second; }
  }
  auto plan = upload_tables(build_perm_tables(m, mask, shift, p));
  std::lock_guard<std::mutex> lk(g_plan_mu);
  ++g_stats.perm_misses;
  if (g_perm_plans.size() >= kPlanCacheCap) g_perm_plans.clear();
  g_perm_plans[key] = plan;
  return plan;
}

Tensor run_perm_plan(const PermPlan& plan, const Tensor& src) {
  Tensor out = plan.needs_zero ? zeros(plan.out) : empty_like_meta(plan.out);
  prof_begin(K_PERMUTE, stream());
  launch_permute(plan.d_tasks, plan.d_row_start, plan.n_tasks, plan.total_rows, plan.group, plan.narrow, plan.single,
                 plan.d_contribs, src.data(), out.data(), stream());
  prof_end(K_PERMUTE, stream(), plan.bytes);
  return out;
}
}  // namespace

CacheStats cache_stats() { return g_stats; }

void clear_plan_caches() {
  // the plans' device tables are released in stream order by their last owners
  std::lock_guard<std::mutex> lk(g_plan_mu);
  g_perm_plans.clear();
  g_gemm_plans.clear();
}

Tensor materialize(const Tensor& t) {
  if (!t.twist_mask) return t;
  const int N = t.meta->rank() + t.meta->corank();
  std::vector<int> id(N);
  std::iota(id.begin(), id.end(), 0);
  auto plan = get_perm_plan(*t.meta, t.twist_mask, 0, id);
  return run_perm_plan(*plan, t);
}

Tensor permute(const Tensor& t, int shift, const std::vector<int>& p) {
  // Tensor::permute dispatcher (Tensor.cpp:335-355)
  const int R = t.meta->rank(), C = t.meta->corank();
  if (int(p.size()) != R + C) throw std::runtime_error("permute: permutation length mismatch");
  if (shift > R || -shift > C) throw std::runtime_error("permute: invalid shift");
  bool id = shift == 0;
  for (int i = 0; i < R + C && id; ++i) id = (p[i] == i);
  if (id) return materialize(t);
  auto plan = get_perm_plan(*t.meta, t.twist_mask, shift, p);
  return run_perm_plan(*plan, t);
}

Tensor permute_adj(const Tensor& t0, int shift, const std::vector<int>& p) {
  Tensor t = materialize(t0);
  const int R = t.meta->rank(), C = t.meta->corank();
  if (int(p.size()) != R + C) throw std::runtime_error("permute_adj: permutation length mismatch");
  if (-shift > R || shift > C) throw std::runtime_error("permute_adj: invalid shift");
  bool id = shift == 0;
  for (int i = 0; i < R + C && id; ++i) id = (p[i] == i);
  if (id) return t;
  std::ostringstream os;
  os << "padj|" << t.meta->id << '|' << shift << '|';
  for (int x : p) os << x << ',';
  const std::string key = os.str();
  std::shared_ptr<PermPlan> plan;
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_perm_plans.find(key);
    if (it != g_perm_plans.end()) { plan = it->second; ++g_stats.perm_hits; }
  }
  if (!plan) {
    plan = upload_tables(build_perm_adj_tables(*t.meta, shift, p));
    std::lock_guard<std::mutex> lk(g_plan_mu);
    ++g_stats.perm_misses;
    if (g_perm_plans.size() >= kPlanCacheCap) g_perm_plans.clear();
  g_perm_plans[key] = plan;
  }
  return run_perm_plan(*plan, t);
}

Tensor twist(const Tensor& t, int leg) {
  // Tensor::twist (Tensor.cpp:357-377): a +-1 per sub-block for abelian
  // fermionic charges; kept pending and folded into the next permute.
  if (!t.meta->sym.fermionic()) return t;
  if (leg < 0 || leg >= t.meta->rank() + t.meta->corank()) throw std::runtime_error("twist: leg out of range");
  Tensor out = t;
  out.twist_mask ^= (1u << leg);
  return out;
}

Tensor adjoint(const Tensor& t0) {
  // AdjointOp evaluated (AdjointOp.hpp:49-59, Tensor.hpp:446-453): blocks
  // transposed, domain <-> codomain, sectors kept in the original order.
  Tensor t = materialize(t0);
  const TensorMeta& m = *t.meta;
  MetaPtr out = make_meta_ordered(m.sym, m.cod, m.dom, m.sectors);
  std::string key = "adj|" + std::to_string(m.id);
  std::shared_ptr<PermPlan> plan;
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_perm_plans.find(key);
    if (it != g_perm_plans.end()) plan = it->second;
  }
  if (!plan) {
    TaskBuilder tb;
    for (size_t i = 0; i < m.sectors.size(); ++i) {
      const int64_t r = m.rows[i], c = m.cols[i];
      if (r * c == 0) continue;
      int32_t dims[2] = {int32_t(c), int32_t(r)};
      int64_t dst[2] = {1, c};
      int64_t src[2] = {r, 1};
      tb.add(out->offset[i], 2, dims, dst, m.offset[i], src, 1.0);
    }
    plan = tb.finish(out);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    if (g_perm_plans.size() >= kPlanCacheCap) g_perm_plans.clear();
  g_perm_plans[key] = plan;
  }
  return run_perm_plan(*plan, t);
}

// ======================================================================= GEMM
GemmTables build_gemm_tables(const TensorMeta& A, bool adj_a, const TensorMeta& B, bool adj_b) {
  const auto& adom = adj_a ? A.cod : A.dom;
  const auto& acod = adj_a ? A.dom : A.cod;
  const auto& bdom = adj_b ? B.cod : B.dom;
  const auto& bcod = adj_b ? B.dom : B.cod;
  if (acod.size() != bdom.size()) throw std::runtime_error("operator*: CoRank of left != Rank of right");
  GemmTables gt;
  gt.out = make_meta(A.sym, adom, bcod);
  const TensorMeta& O = *gt.out;
  std::vector<char> covered(O.sectors.size(), 0);
  for (size_t i = 0; i < A.sectors.size(); ++i) {
    const int q = A.sectors[i];
    const int j = B.index(q);
    if (j < 0) continue;
    const int o = O.index(q);
    if (o < 0) throw std::runtime_error("operator*: output sector missing");
    xgb_gemm_desc d{};
    d.m = adj_a ? A.cols[i] : A.rows[i];
    d.k = adj_a ? A.rows[i] : A.cols[i];
    const int64_t kb = adj_b ? B.cols[j] : B.rows[j];
    d.n = adj_b ? B.rows[j] : B.cols[j];
    if (kb != d.k || d.m != O.rows[o] || d.n != O.cols[o])
      throw std::runtime_error("operator*: block shapes do not match (coupled codomain != coupled domain)");
    d.a_off = A.offset[i]; d.lda = A.rows[i];
    d.b_off = B.offset[j]; d.ldb = B.rows[j];
    d.c_off = O.offset[o]; d.ldc = O.rows[o];
    d.trans_a = adj_a; d.trans_b = adj_b;
    gt.descs.push_back(d);
    covered[o] = 1;
  }
  // sectors of the output with no partner stay zero (Tout.setZero(), TensorBase.cpp:256-258): k = 0 groups
  for (size_t o = 0; o < O.sectors.size(); ++o) {
    if (covered[o] || O.rows[o] * O.cols[o] == 0) continue;
    xgb_gemm_desc d{};
    d.m = O.rows[o]; d.n = O.cols[o]; d.k = 0;
    d.lda = 1; d.ldb = 1;
    d.c_off = O.offset[o]; d.ldc = O.rows[o];
    gt.descs.push_back(d);
  }
  return gt;
}

// precision form of the block GEMMs issued by matmul (per host thread)
thread_local int g_gemm_precision = XGB_PREC_FP64;

Tensor matmul(const Tensor& a0, const Tensor& b0, bool adj_a, bool adj_b) {
  // TensorBase::operator* (TensorBase.cpp:237-288), with AdjointOp operands
  // handled as transposed GEMM operands (no materialised transpose).
  Tensor a = materialize(a0), b = materialize(b0);
  const TensorMeta& A = *a.meta;
  const TensorMeta& B = *b.meta;
  std::ostringstream os;
  os << A.id << (adj_a ? 'T' : 'N') << '|' << B.id << (adj_b ? 'T' : 'N');
  const std::string key = os.str();
  std::shared_ptr<GemmPlan> plan;
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_gemm_plans.find(key);
    if (it != g_gemm_plans.end()) { plan = it->second; ++g_stats.gemm_hits; }
  }
  if (!plan) {
    GemmTables gt = build_gemm_tables(A, adj_a, B, adj_b);
    plan = std::make_shared<GemmPlan>();
    plan->out = gt.out;
    const std::vector<xgb_gemm_desc>& descs = gt.descs;
    plan->tile = choose_gemm_tile(descs.data(), int(descs.size()));
    plan->host_descs = descs;
    plan->d_descs = plan->mem.table(descs);
    for (const auto& d : descs) plan->flops += 2.0 * double(d.m) * double(d.n) * double(d.k);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    ++g_stats.gemm_misses;
    if (g_gemm_plans.size() >= kPlanCacheCap) g_gemm_plans.clear();
    g_gemm_plans[key] = plan;
  }
  Tensor out = empty_like_meta(plan->out);
  if (g_gemm_precision == XGB_PREC_3XTF32) {
    {
      std::lock_guard<std::mutex> lk(g_plan_mu);
      if (!plan->tc_ready) {
        TcPlanHost tp = build_tc_plan(plan->host_descs.data(), int(plan->host_descs.size()));
        plan->n_tc_tiles = int(tp.tiles.size());
        plan->n_tc_tasks = int(tp.tasks.size());
        plan->tc_a_floats = tp.a_floats;
        plan->tc_b_floats = tp.b_floats;
        plan->d_tc_groups = plan->mem.table(tp.groups);
        plan->d_tc_tasks = plan->mem.table(tp.tasks);
        plan->d_tc_tiles = plan->mem.table(tp.tiles);
        plan->tc_ready = true;
      }
    }
    auto* ap = static_cast<float*>(dev_alloc(sizeof(float) * size_t(std::max<int64_t>(plan->tc_a_floats, 4))));
    auto* bp = static_cast<float*>(dev_alloc(sizeof(float) * size_t(std::max<int64_t>(plan->tc_b_floats, 4))));
    prof_begin(K_GEMM_TC, stream());
    launch_gemm_tc(plan->d_descs, plan->d_tc_groups, plan->d_tc_tasks, plan->n_tc_tasks, plan->d_tc_tiles,
                   plan->n_tc_tiles, a.data(), b.data(), ap, bp, out.data(), 1.0, 0.0, stream());
    prof_end(K_GEMM_TC, stream(), plan->flops);
    dev_free(ap);
    dev_free(bp);
    return out;
  }
  if (g_gemm_precision == XGB_PREC_F64TC && !plan->oz_routed) {
    // both routes are FP64-class: the tensor-core form or the FP64 CUDA-core kernel, whichever the
    // autotuner measures faster for this size bucket (built-in rule: average k >= 64)
    const auto& hd = plan->host_descs;
    const F64Config rc = gemm_f64_config(hd.data(), int(hd.size()), a.data(), b.data(),
                                         F64Config{plan->tile, 0, f64tc_heuristic(hd.data(), int(hd.size()))},
                                         stream(), true);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    plan->oz_route = rc.tc;
    plan->oz_routed = true;
  }
  if (g_gemm_precision == XGB_PREC_F64TC && plan->oz_route) {
    {
      std::lock_guard<std::mutex> lk(g_plan_mu);
      if (!plan->oz_ready) {
        OzPlanHost op = build_oz_plan(plan->host_descs.data(), int(plan->host_descs.size()));
        plan->n_oz_tiles = int(op.tiles.size());
        plan->n_oz_tasks = int(op.tasks.size());
        plan->oz_a_bytes = op.a_bytes;
        plan->oz_b_bytes = op.b_bytes;
        plan->oz_rowmax = op.rowmax;
        plan->d_oz_groups = plan->mem.table(op.groups);
        plan->d_oz_tasks = plan->mem.table(op.tasks);
        plan->d_oz_tiles = plan->mem.table(op.tiles);
        plan->d_oz_red = plan->mem.table(op.red);
        plan->n_oz_red = int(op.red.size());
        plan->oz_slots = op.slots;
        plan->oz_ready = true;
      }
    }
    cudaStream_t st = stream();
    auto* rm = static_cast<unsigned long long*>(
        dev_alloc(sizeof(unsigned long long) * size_t(std::max<int64_t>(plan->oz_rowmax, 1))));
    auto* ap = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(plan->oz_a_bytes, 16))));
    auto* bp = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(plan->oz_b_bytes, 16))));
    prof_begin(K_GEMM_OZ, st);
    launch_gemm_oz(plan->d_descs, plan->d_oz_groups, plan->d_oz_tasks, plan->n_oz_tasks, plan->d_oz_tiles,
                   plan->n_oz_tiles, plan->d_oz_red, plan->n_oz_red, plan->oz_slots, a.data(), b.data(), rm,
                   plan->oz_rowmax, ap, bp, out.data(), 1.0, 0.0, st);
    prof_end(K_GEMM_OZ, st, plan->flops);
    dev_free(rm);
    dev_free(ap);
    dev_free(bp);
    return out;
  }
  if (g_gemm_precision == XGB_PREC_BF16X9) {  // tables built per call (the cached ones are the 3xTF32 layout)
    TcPlanHost tp = build_tc_plan(plan->host_descs.data(), int(plan->host_descs.size()), 1);
    cudaStream_t st = stream();
    auto* dg = static_cast<TcGroup*>(dev_alloc(sizeof(TcGroup) * std::max<size_t>(tp.groups.size(), 1)));
    auto* dk = static_cast<TcPackTask*>(dev_alloc(sizeof(TcPackTask) * std::max<size_t>(tp.tasks.size(), 1)));
    auto* dt = static_cast<GemmTile*>(dev_alloc(sizeof(GemmTile) * std::max<size_t>(tp.tiles.size(), 1)));
    cuda_ok(cudaMemcpyAsync(dg, tp.groups.data(), sizeof(TcGroup) * tp.groups.size(), cudaMemcpyHostToDevice, st), "h2d");
    if (!tp.tasks.empty())
      cuda_ok(cudaMemcpyAsync(dk, tp.tasks.data(), sizeof(TcPackTask) * tp.tasks.size(), cudaMemcpyHostToDevice, st),
              "h2d");
    cuda_ok(cudaMemcpyAsync(dt, tp.tiles.data(), sizeof(GemmTile) * tp.tiles.size(), cudaMemcpyHostToDevice, st), "h2d");
    auto* ap = static_cast<float*>(dev_alloc(sizeof(float) * size_t(std::max<int64_t>(tp.a_floats, 4))));
    auto* bp = static_cast<float*>(dev_alloc(sizeof(float) * size_t(std::max<int64_t>(tp.b_floats, 4))));
    prof_begin(K_GEMM_TC, st);
    launch_gemm_tc(plan->d_descs, dg, dk, int(tp.tasks.size()), dt, int(tp.tiles.size()), a.data(), b.data(), ap, bp,
                   out.data(), 1.0, 0.0, st, 1);
    prof_end(K_GEMM_TC, st, plan->flops);
    for (void* p : {static_cast<void*>(dg), static_cast<void*>(dk), static_cast<void*>(dt), static_cast<void*>(ap),
                    static_cast<void*>(bp)})
      dev_free(p);
    return out;
  }
  if (g_gemm_precision == XGB_PREC_FP32) {
    {
      std::lock_guard<std::mutex> lk(g_plan_mu);
      if (!plan->tiles_ready) {  // one tile x tile CTA per output tile, longest k first
        const auto& descs = plan->host_descs;
        std::vector<GemmTile> tiles;
        for (size_t g = 0; g < descs.size(); ++g) {
          int64_t tm = (descs[g].m + plan->tile - 1) / plan->tile, tn = (descs[g].n + plan->tile - 1) / plan->tile;
          for (int64_t y = 0; y < tn; ++y)
            for (int64_t x = 0; x < tm; ++x) tiles.push_back({int32_t(g), int32_t(x), int32_t(y), plan->tile});
        }
        order_tiles_by_work(tiles, descs.data());
        plan->n_tiles = int(tiles.size());
        plan->d_tiles = plan->mem.table(std::move(tiles));
        plan->tiles_ready = true;
      }
    }
    prof_begin(K_GEMM_F32, stream());
    launch_gemm_f32(plan->d_descs, plan->d_tiles, plan->n_tiles, plan->tile, a.data(), b.data(), out.data(), 1.0, 0.0,
                    stream());
    prof_end(K_GEMM_F32, stream(), plan->flops);
    return out;
  }
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    if (!plan->f64_ready) {  // FP64 CUDA-core launch shape: the autotuner's choice or the built-in rule
      const auto& descs = plan->host_descs;
      const F64Config cfg =
          gemm_f64_config(descs.data(), int(descs.size()), a.data(), b.data(), {plan->tile, 0}, stream());
      plan->f64 = plan_gemm_f64(descs.data(), int(descs.size()), cfg);
      plan->d_f64_tiles = plan->mem.table(plan->f64.tiles);
      plan->d_f64_red = plan->mem.table(plan->f64.red);
      plan->f64_ready = true;
    }
  }
  prof_begin(K_GEMM, stream());
  run_f64_plan(plan->f64, plan->d_descs, plan->d_f64_tiles, plan->d_f64_red, a.data(), b.data(), out.data(), 1.0, 0.0,
               stream());
  prof_end(K_GEMM, stream(), plan->flops);
  return out;
}

Tensor embed(const Tensor& src0, const MetaPtr& target) {
  // blocks of `src` copied into a zero tensor with `target`'s structure, sector
  // by sector (charges absent from src stay zero; shapes must agree)
  Tensor src = materialize(src0);
  Tensor out = zeros(target);
  std::vector<xgb_copy2d_desc> d;
  int64_t mx = 0;
  for (size_t i = 0; i < target->sectors.size(); ++i) {
    const int si = src.meta->index(target->sectors[i]);
    if (si < 0) continue;
    if (src.meta->rows[si] != target->rows[i] || src.meta->cols[si] != target->cols[i])
      throw std::runtime_error("embed: block shapes differ");
    d.push_back({src.meta->offset[si], src.meta->rows[si], target->offset[i], target->rows[i], target->rows[i],
                 target->cols[i]});
    mx = std::max(mx, target->rows[i] * target->cols[i]);
  }
  if (d.empty()) return out;
  auto* dd = static_cast<xgb_copy2d_desc*>(dev_alloc(sizeof(xgb_copy2d_desc) * d.size()));
  cuda_ok(cudaMemcpyAsync(dd, d.data(), sizeof(xgb_copy2d_desc) * d.size(), cudaMemcpyHostToDevice, stream()), "h2d");
  prof_begin(K_COPY2D, stream());
  launch_copy2d(dd, int(d.size()), mx, src.data(), out.data(), stream());
  prof_end(K_COPY2D, stream(), 16.0 * double(target->size));
  dev_free(dd);
  return out;
}

std::pair<Tensor, Tensor> matmul_backward(const Tensor& left, const Tensor& right, const Tensor& res_adj) {
  // reverse rule of operator* (ADTensor.hpp:741-752):
  //   left.adj += res.adj * right^dag,  right.adj += left^dag * res.adj
  Tensor la = matmul(res_adj, right, false, true);
  Tensor ra = matmul(left, res_adj, true, false);
  return {embed(la, left.meta), embed(ra, right.meta)};
}

int gemm_precision() { return g_gemm_precision; }
void set_gemm_precision(int prec) {
  if (!gemm_precision_available(prec)) throw std::runtime_error("unsupported GEMM precision form");
  g_gemm_precision = prec;
}

// ======================================================================= contract
ContractPerms get_permutations(const std::vector<int>& a1, int rank1, const std::vector<int>& a2, int rank2, int rankres) {
  ContractPerms r;
  const int r1 = int(a1.size()), r2 = int(a2.size());
  int max1 = 0, max2 = 0;
  for (int x : a1) max1 = std::max(max1, x);
  for (int x : a2) max2 = std::max(max2, x);
  if (max1 != max2) throw std::runtime_error("contract: label sets do not match");
  auto pos = [](const std::vector<int>& a, int v) {
    auto it = std::find(a.begin(), a.end(), v);
    if (it == a.end()) throw std::runtime_error("contract: missing label");
    return int(it - a.begin());
  };
  r.p2.assign(r2, 0);
  std::vector<int> found2(r2, -1);
  for (int ind = 0; ind < max2; ++ind) { int v = pos(a2, ind + 1); found2[ind] = v; r.p2[ind] = v; }
  for (int ind = max2; ind < r2; ++ind) {
    int v = 0;
    while (std::find(found2.begin(), found2.end(), v) != found2.end()) ++v;
    found2[ind] = v;
    r.p2[ind] = v;
  }
  r.p1.assign(r1, 0);
  std::vector<int> found1(r1, -1);
  for (int ind = 0; ind < max1; ++ind) { int v = pos(a1, ind + 1); found1[ind] = v; r.p1[r1 - max1 + ind] = v; }
  for (int ind = max1, k = 0; ind < r1; ++ind, ++k) {
    int v = 0;
    while (std::find(found1.begin(), found1.end(), v) != found1.end()) ++v;
    found1[ind] = v;
    r.p1[k] = v;
  }
  std::vector<int> tmp;
  for (int x : a1) if (x < 0) tmp.push_back(x);
  for (int x : a2) if (x < 0) tmp.push_back(x);
  r.pres.resize(tmp.size());
  std::iota(r.pres.begin(), r.pres.end(), 0);
  std::stable_sort(r.pres.begin(), r.pres.end(), [&](int i, int j) { return tmp[i] > tmp[j]; });
  r.shift1 = rank1 - r1 + max1;
  r.shift2 = rank2 - max2;
  r.shiftres = r1 - max1 - rankres;
  return r;
}

Tensor contract(const Tensor& a, const Tensor& b, const std::vector<int>& a1, const std::vector<int>& a2, int rankres) {
  // Tensor::contract (Tensor.hpp:328-351): permute, operator*, permute
  ContractPerms cp = get_permutations(a1, a.meta->rank(), a2, b.meta->rank(), rankres);
  Tensor l = permute(a, cp.shift1, cp.p1);
  Tensor r = permute(b, cp.shift2, cp.p2);
  return permute(matmul(l, r), cp.shiftres, cp.pres);
}

// ======================================================================= scalar ops
Tensor scale(const Tensor& t0, double s) {
  Tensor t = materialize(t0);
  Tensor out = empty_like_meta(t.meta);
  if (t.size()) {
    cuda_ok(cudaMemcpyAsync(out.data(), t.data(), sizeof(double) * t.size(), cudaMemcpyDeviceToDevice, stream()), "copy");
    launch_scale(out.data(), t.size(), s, stream());
  }
  return out;
}

double max_norm(const Tensor& t) {
  // TensorBase::maxNorm (TensorBase.cpp:48-56); twists do not change |x|
  double* sc = scalar_scratch();
  launch_absmax(t.data(), t.size(), sc, stream());
  double h = 0;
  cuda_ok(cudaMemcpyAsync(&h, sc, sizeof(double), cudaMemcpyDeviceToHost, stream()), "d2h");
  cuda_ok(cudaStreamSynchronize(stream()), "sync");
  return h;
}

Tensor normalize_max(const Tensor& t0) {
  // T * (1. / T.maxNorm()) entirely on the device (CTM.cpp:1372,1383,1405)
  Tensor t = materialize(t0);
  Tensor out;
  if (t.buf.use_count() == 1) {
    out = t;
  } else {
    out = empty_like_meta(t.meta);
    if (t.size())
      cuda_ok(cudaMemcpyAsync(out.data(), t.data(), sizeof(double) * t.size(), cudaMemcpyDeviceToDevice, stream()), "copy");
  }
  double* sc = scalar_scratch();
  prof_begin(K_ABSMAX, stream());
  launch_absmax(out.data(), out.size(), sc, stream());
  prof_end(K_ABSMAX, stream(), 8.0 * out.size());
  prof_begin(K_SCALE, stream());
  launch_scale_by_inv(out.data(), out.size(), sc, stream());
  prof_end(K_SCALE, stream(), 16.0 * out.size());
  return out;
}

Tensor identity(const Sym& s, const std::vector<BasisPtr>& dom, const std::vector<BasisPtr>& cod) {
  // Tensor::Identity / setIdentity: ones on each block's main diagonal
  MetaPtr m = make_meta(s, dom, cod);
  Tensor t = zeros(m);
  std::vector<double> ones;
  std::vector<xgb_copy2d_desc> descs;
  int64_t mx = 0;
  for (size_t i = 0; i < m->sectors.size(); ++i) {
    int64_t k = std::min(m->rows[i], m->cols[i]);
    if (!k) continue;
    xgb_copy2d_desc d{};
    d.src_off = int64_t(ones.size());
    d.src_ld = 1;
    d.dst_off = m->offset[i];
    d.dst_ld = m->rows[i] + 1;  // walk the diagonal
    d.rows = 1;
    d.cols = k;
    descs.push_back(d);
    ones.insert(ones.end(), size_t(k), 1.0);
    mx = std::max(mx, k);
  }
  if (!descs.empty()) {
    double* dones = static_cast<double*>(dev_alloc(sizeof(double) * ones.size()));
    auto* dd = static_cast<xgb_copy2d_desc*>(dev_alloc(sizeof(xgb_copy2d_desc) * descs.size()));
    cuda_ok(cudaMemcpyAsync(dones, ones.data(), sizeof(double) * ones.size(), cudaMemcpyHostToDevice, stream()), "h2d");
    cuda_ok(cudaMemcpyAsync(dd, descs.data(), sizeof(xgb_copy2d_desc) * descs.size(), cudaMemcpyHostToDevice, stream()), "h2d");
    launch_copy2d(dd, int(descs.size()), mx, dones, t.data(), stream());
    dev_free(dones);
    dev_free(dd);
  }
  return t;
}

// ======================================================================= SVD / truncation
namespace {
struct SvdPlan {
  PlanMem mem;
  int n = 0;
  int64_t u_total = 0, s_total = 0, v_total = 0, work_total = 0, maxk = 0;
  double lapack_flops = 0;  // thin R-SVD work 6 m n^2 + 20 n^3 (m >= n; Golub & Van Loan, Table 5.5.1)
  std::vector<int64_t> s_begin;  // per sector prefix (host), size n+1
  std::vector<int64_t> u_off, s_off, v_off, kfull;
  xgb_svd_desc* d_descs = nullptr;
  std::vector<xgb_svd_desc> h_descs;
  int64_t* d_work_off = nullptr;
  int64_t* d_s_begin = nullptr;
  int32_t* d_deg = nullptr;
};
std::unordered_map<uint64_t, std::shared_ptr<SvdPlan>> g_svd_plans;
int32_t* g_keep_host[kLanes] = {nullptr, nullptr, nullptr};  // pinned, one per lane
double* g_out2_host[kLanes] = {nullptr, nullptr, nullptr};
int g_keep_cap[kLanes] = {0, 0, 0};

std::shared_ptr<SvdPlan> get_svd_plan(const TensorMeta& m) {
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_svd_plans.find(m.id);
    if (it != g_svd_plans.end()) return it->second;
  }
  auto p = std::make_shared<SvdPlan>();
  p->n = int(m.sectors.size());
  std::vector<xgb_svd_desc> descs;
  std::vector<int64_t> woff;
  std::vector<int32_t> deg;
  p->s_begin.push_back(0);
  for (int i = 0; i < p->n; ++i) {
    int64_t r = m.rows[i], c = m.cols[i], k = std::min(r, c);
    xgb_svd_desc d{};
    d.m = r; d.n = c; d.a_off = m.offset[i];
    d.u_off = p->u_total; d.s_off = p->s_total; d.vt_off = p->v_total;
    p->u_off.push_back(p->u_total); p->s_off.push_back(p->s_total); p->v_off.push_back(p->v_total); p->kfull.push_back(k);
    p->u_total += r * k; p->s_total += k; p->v_total += k * c;
    woff.push_back(p->work_total);
    p->work_total += int64_t(svd_work_elems(r, c));
    p->maxk = std::max(p->maxk, k);
    {
      const double M = double(std::max(r, c)), N = double(std::min(r, c));
      p->lapack_flops += 6.0 * M * N * N + 20.0 * N * N * N;
    }
    descs.push_back(d);
    deg.push_back(m.sym.deg(m.sectors[i]));
    p->s_begin.push_back(p->s_total);
  }
  if (p->maxk > 8192) throw std::runtime_error("tSVD: sector block larger than 8192 columns");
  p->d_descs = p->mem.table(descs);
  p->h_descs = descs;
  p->d_work_off = p->mem.table(woff);
  p->d_s_begin = p->mem.table(p->s_begin);
  p->d_deg = p->mem.table(deg);
  std::lock_guard<std::mutex> lk(g_plan_mu);
  if (g_svd_plans.size() >= kPlanCacheCap) g_svd_plans.clear();
  g_svd_plans[m.id] = p;
  return p;
}
}  // namespace

SVDResult truncate_spectra(const TensorMeta& m, const Spectra& sp, int64_t max_keep, double eps_svd,
                           bool preserve_multiplets) {
  // cutoff_matrices (Tensor.cpp:523-633) on per-sector spectra: global
  // truncation on the device, then U[:, :k], S[:k, :k], V^T[:k, :] per kept sector.
  cudaStream_t st = stream();
  const int n = int(m.sectors.size());
  const int64_t s_total = sp.s_begin.back();
  if (s_total == 0) throw std::runtime_error("tSVD: no singular values");
  int64_t* d_sb = sp.d_s_begin;
  int32_t* d_deg = sp.d_deg;
  bool own_tables = false;
  if (!d_sb || !d_deg) {
    std::vector<int32_t> deg;
    for (int q : m.sectors) deg.push_back(m.sym.deg(q));
    d_sb = static_cast<int64_t*>(dev_alloc(sizeof(int64_t) * sp.s_begin.size()));
    d_deg = static_cast<int32_t*>(dev_alloc(sizeof(int32_t) * std::max<size_t>(deg.size(), 1)));
    cuda_ok(cudaMemcpyAsync(d_sb, sp.s_begin.data(), sizeof(int64_t) * sp.s_begin.size(), cudaMemcpyHostToDevice, st), "h2d");
    cuda_ok(cudaMemcpyAsync(d_deg, deg.data(), sizeof(int32_t) * deg.size(), cudaMemcpyHostToDevice, st), "h2d");
    own_tables = true;
  }
  int32_t* keep_d = static_cast<int32_t*>(dev_alloc(sizeof(int32_t) * n));
  double* out2_d = scalar_scratch() + 8;
  prof_begin(K_TRUNC, st);
  launch_truncate(n, d_sb, d_deg, sp.S, s_total, max_keep, eps_svd, preserve_multiplets ? 1 : 0, keep_d, out2_d, st);
  prof_end(K_TRUNC, st, 8.0 * double(s_total));
  const int ln = lane();
  int32_t*& keep_host = g_keep_host[ln];
  double*& out2_host = g_out2_host[ln];
  if (g_keep_cap[ln] < n) {
    if (keep_host) cudaFreeHost(keep_host);
    cuda_ok(cudaMallocHost(&keep_host, sizeof(int32_t) * n), "pinned");
    g_keep_cap[ln] = n;
    if (!out2_host) cuda_ok(cudaMallocHost(&out2_host, sizeof(double) * 2), "pinned");
  }
  cuda_ok(cudaMemcpyAsync(keep_host, keep_d, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st), "d2h");
  cuda_ok(cudaMemcpyAsync(out2_host, out2_d, sizeof(double) * 2, cudaMemcpyDeviceToHost, st), "d2h");
  SVDResult res;
  res.spectrum.resize(size_t(s_total));
  res.spec_begin = sp.s_begin;
  cuda_ok(cudaMemcpyAsync(res.spectrum.data(), sp.S, sizeof(double) * size_t(s_total), cudaMemcpyDeviceToHost, st), "d2h");
  cuda_ok(cudaStreamSynchronize(st), "sync");
  dev_free(keep_d);
  for (double v : res.spectrum)
    if (!std::isfinite(v)) throw std::runtime_error("tSVD: non-finite singular value (non-finite input block?)");
  if (own_tables) {
    dev_free(d_sb);
    dev_free(d_deg);
  }

  res.trunc_weight = out2_host[0];
  res.entropy = out2_host[1];
  res.keep.assign(keep_host, keep_host + n);
  for (int i = 0; i < n; ++i)
    if (res.keep[i] < 0 || res.keep[i] > sp.k[i]) throw std::runtime_error("tSVD: truncation returned an invalid count");
  // truncated basis: charges with kept values in ascending order (std::map, Tensor.cpp:592-598)
  std::vector<std::pair<int, int>> kept;  // (q, sector index)
  for (int i = 0; i < n; ++i)
    if (res.keep[i] > 0) kept.push_back({m.sectors[i], i});
  std::sort(kept.begin(), kept.end());
  std::vector<std::pair<int, int64_t>> pairs;
  std::vector<int> qs;
  for (auto& [q, i] : kept) { pairs.push_back({q, res.keep[i]}); qs.push_back(q); }
  BasisPtr trunc = basis_from_pairs(m.sym, pairs, false);
  MetaPtr mu = make_meta_ordered(m.sym, m.dom, {trunc}, qs);
  MetaPtr ms = make_meta_ordered(m.sym, {trunc}, {trunc}, qs);
  MetaPtr mv = make_meta_ordered(m.sym, {trunc}, m.cod, qs);
  res.U = empty_like_meta(mu);
  res.S = empty_like_meta(ms);
  res.Vdag = empty_like_meta(mv);
  std::vector<xgb_copy2d_desc> du, dv, ds;
  int64_t mxu = 0, mxv = 0, mxs = 0;
  for (size_t a = 0; a < kept.size(); ++a) {
    const int i = kept[a].second;
    const int64_t k = res.keep[i], r = m.rows[i], c = m.cols[i], kf = sp.k[i];
    du.push_back({sp.u_off[i], r, mu->offset[a], r, r, k});
    dv.push_back({sp.v_off[i], kf, mv->offset[a], k, k, c});
    ds.push_back({sp.s_begin[i], 1, ms->offset[a], k, k, k});
    mxu = std::max(mxu, r * k);
    mxv = std::max(mxv, k * c);
    mxs = std::max(mxs, k);
  }
  const size_t nb = du.size();
  auto* dd = static_cast<xgb_copy2d_desc*>(dev_alloc(sizeof(xgb_copy2d_desc) * 3 * std::max<size_t>(nb, 1)));
  std::vector<xgb_copy2d_desc> all;
  all.insert(all.end(), du.begin(), du.end());
  all.insert(all.end(), dv.begin(), dv.end());
  all.insert(all.end(), ds.begin(), ds.end());
  cuda_ok(cudaMemcpyAsync(dd, all.data(), sizeof(xgb_copy2d_desc) * all.size(), cudaMemcpyHostToDevice, st), "h2d");
  prof_begin(K_COPY2D, st);
  launch_copy2d(dd, int(nb), mxu, sp.U, res.U.data(), st);
  launch_copy2d(dd + nb, int(nb), mxv, sp.V, res.Vdag.data(), st);
  launch_diag_from_vec(dd + 2 * nb, int(nb), mxs, -1, sp.S, res.S.data(), st);
  prof_end(K_COPY2D, st, 16.0 * double(res.U.size() + res.Vdag.size() + res.S.size()));
  dev_free(dd);  // stream-ordered: released after the copies (the pageable descriptors were staged on return)
  return res;
}

SVDResult tsvd(const Tensor& t0, int64_t max_keep, double eps_svd, bool preserve_multiplets) {
  // Tensor::tSVD = full_svd_impl + cutoff_matrices (Tensor.cpp:478-633)
  Tensor t = materialize(t0);
  const TensorMeta& m = *t.meta;
  if (m.sectors.empty()) throw std::runtime_error("tSVD of a tensor without sectors");
  auto plan = get_svd_plan(m);
  cudaStream_t st = stream();
  Spectra sp;
  sp.U = static_cast<double*>(dev_alloc(sizeof(double) * std::max<int64_t>(plan->u_total, 1)));
  sp.S = static_cast<double*>(dev_alloc(sizeof(double) * std::max<int64_t>(plan->s_total, 1)));
  sp.V = static_cast<double*>(dev_alloc(sizeof(double) * std::max<int64_t>(plan->v_total, 1)));
  double* W = static_cast<double*>(dev_alloc(sizeof(double) * std::max<int64_t>(plan->work_total, 1)));
  prof_begin(K_SVD, st);
  launch_svd(plan->d_descs, plan->h_descs.data(), plan->d_work_off, plan->n, plan->maxk, t.data(), sp.U, sp.S, sp.V, W,
             st);
  prof_end(K_SVD, st, plan->lapack_flops);
  dev_free(W);
  sp.k = plan->kfull;
  sp.u_off = plan->u_off;
  sp.v_off = plan->v_off;
  sp.s_begin = plan->s_begin;
  sp.d_s_begin = plan->d_s_begin;
  sp.d_deg = plan->d_deg;
  SVDResult res = truncate_spectra(m, sp, max_keep, eps_svd, preserve_multiplets);
  dev_free(sp.U);
  dev_free(sp.S);
  dev_free(sp.V);
  return res;
}

std::pair<Tensor, Tensor> tqr(const Tensor& t0) {
  // Tensor::tQR (Tensor.cpp:757-780): middle basis = coupled codomain when
  // the domain is larger, else the coupled domain (forgetHistory).
  Tensor t = materialize(t0);
  const TensorMeta& m = *t.meta;
  BasisPtr middle = (m.cdom->dim() > m.ccod->dim()) ? basis_forget_history(m.ccod) : basis_forget_history(m.cdom);
  MetaPtr mq = make_meta_ordered(m.sym, m.dom, {middle}, m.sectors);
  MetaPtr mr = make_meta_ordered(m.sym, {middle}, m.cod, m.sectors);
  Tensor Q = empty_like_meta(mq), R = empty_like_meta(mr);
  std::vector<xgb_qr_desc> descs;
  std::vector<int64_t> woff;
  int64_t wt = 0;
  for (size_t i = 0; i < m.sectors.size(); ++i) {
    xgb_qr_desc d{};
    d.m = m.rows[i]; d.n = m.cols[i]; d.a_off = m.offset[i];
    d.q_off = mq->offset[i]; d.q_cols = mq->cols[i];
    d.r_off = mr->offset[i]; d.r_rows = mr->rows[i];
    descs.push_back(d);
    woff.push_back(wt);
    wt += int64_t(qr_work_elems(d.m, d.n));
  }
  if (!descs.empty()) {
    cudaStream_t st = stream();
    auto* dd = static_cast<xgb_qr_desc*>(dev_alloc(sizeof(xgb_qr_desc) * descs.size()));
    auto* dw = static_cast<int64_t*>(dev_alloc(sizeof(int64_t) * woff.size()));
    double* W = static_cast<double*>(dev_alloc(sizeof(double) * std::max<int64_t>(wt, 1)));
    cuda_ok(cudaMemcpyAsync(dd, descs.data(), sizeof(xgb_qr_desc) * descs.size(), cudaMemcpyHostToDevice, st), "h2d");
    cuda_ok(cudaMemcpyAsync(dw, woff.data(), sizeof(int64_t) * woff.size(), cudaMemcpyHostToDevice, st), "h2d");
    launch_qr(dd, dw, int(descs.size()), t.data(), Q.data(), R.data(), W, st);
    dev_free(dd);
    dev_free(dw);
    dev_free(W);
  }
  return {Q, R};
}

// fn applied in place, in order, to the main diagonal of every block of `t`
static void diag_apply_inplace(Tensor& t, std::initializer_list<int> fns) {
  const TensorMeta& ms = *t.meta;
  std::vector<xgb_copy2d_desc> descs;
  int64_t mx = 0;
  for (size_t i = 0; i < ms.sectors.size(); ++i) {
    descs.push_back({ms.offset[i], ms.rows[i], ms.offset[i], ms.rows[i], ms.rows[i], ms.cols[i]});
    mx = std::max(mx, std::max(ms.rows[i], ms.cols[i]));
  }
  if (descs.empty()) return;
  auto* dd = static_cast<xgb_copy2d_desc*>(dev_alloc(sizeof(xgb_copy2d_desc) * descs.size()));
  cuda_ok(cudaMemcpyAsync(dd, descs.data(), sizeof(xgb_copy2d_desc) * descs.size(), cudaMemcpyHostToDevice, stream()), "h2d");
  for (int fn : fns) {
    prof_begin(K_DIAG, stream());
    launch_diag_apply(dd, int(descs.size()), mx, fn, t.data(), stream());
    prof_end(K_DIAG, stream(), 16.0 * double(mx) * double(descs.size()));
  }
  dev_free(dd);
}

Tensor diag_apply(const Tensor& t0, int fn) {
  Tensor t = materialize(t0);
  Tensor out = empty_like_meta(t.meta);
  cuda_ok(cudaMemcpyAsync(out.data(), t.data(), sizeof(double) * t.meta->size, cudaMemcpyDeviceToDevice, stream()),
          "copy");
  diag_apply_inplace(out, {fn});
  return out;
}

std::pair<Tensor, Tensor> projectors_from_svd(const SVDResult& r, const Tensor& t1, const Tensor& t2) {
  // isqrtS = S.diag_sqrt().diag_inv(): 1/sqrt(s) on the diagonal
  Tensor isq = empty_like_meta(r.S.meta);
  cuda_ok(cudaMemcpyAsync(isq.data(), r.S.data(), sizeof(double) * r.S.meta->size, cudaMemcpyDeviceToDevice, stream()),
          "copy");
  diag_apply_inplace(isq, {XGB_DIAG_SQRT, XGB_DIAG_INV});
  Tensor P1 = matmul(matmul(isq, r.U, false, true), t1);      // isqrtS * U.adjoint() * T1
  Tensor P2 = matmul(matmul(t2, r.Vdag, false, true), isq);   // T2 * Vdag.adjoint() * isqrtS
  return {P1, P2};
}

std::pair<Tensor, Tensor> decompose(const Tensor& t1, const Tensor& t2, int64_t max_nsv) {
  // decompose (src/PEPS/PEPSContractions.cpp:16-43)
  Tensor prod = matmul(t1, t2);
  SVDResult r = tsvd(prod, max_nsv, 1.0e-10, false);
  return projectors_from_svd(r, t1, t2);
}

// ======================================================================= width policies
std::vector<int64_t> HistoryPolicy::widths(const TensorMeta& m, const History& last, int64_t chi) {
  std::vector<int64_t> w(m.sectors.size(), 0);
  for (size_t i = 0; i < m.sectors.size(); ++i) {
    auto it = last.find(m.sectors[i]);
    if (it == last.end()) continue;  // never seen
    const int64_t k = it->second.keep;
    w[i] = std::min<int64_t>(chi, k) + std::max<int64_t>(oversample, int64_t(std::ceil(growth * double(k))));
  }
  return w;
}

void sector_features(const TensorMeta& m, const History& last, int64_t chi, std::vector<float>& out) {
  const size_t n = m.sectors.size();
  out.assign(n * kFeatures, 0.0f);
  auto lg10 = [](double x, double floor_) { return x > 0 ? std::max(std::log10(x), floor_) : floor_; };
  for (size_t i = 0; i < n; ++i) {
    float* f = out.data() + i * kFeatures;
    f[0] = float(std::log2(1.0 + double(m.rows[i])) / 12.0);
    f[1] = float(std::log2(1.0 + double(m.cols[i])) / 12.0);
    f[7] = float(std::log2(1.0 + double(chi)) / 8.0);
    auto it = last.find(m.sectors[i]);
    if (it == last.end()) continue;
    const SectorHistory& h = it->second;
    const double smax = h.s_max > 0 ? h.s_max : 1.0;
    f[2] = 1.0f;
    f[3] = float(std::log2(1.0 + double(h.keep)) / 8.0);
    f[4] = float(lg10(h.s_first / smax, -16.0) / 16.0);
    f[5] = float(lg10(h.s_last / smax, -16.0) / 16.0);
    f[6] = float((h.keep > 0 && h.s_next > 0 ? lg10(h.s_next / std::max(h.s_last, 1e-300), -8.0) : -8.0) / 8.0);
  }
}

// ======================================================================= simple update
Tensor apply_weights(const Tensor& A, const Tensor& wL, const Tensor& wT, const Tensor& wR, const Tensor& wB) {
  Tensor t = contract(A, twist(wL, 1), {1, -2, -3, -4, -5}, {-1, 1}, 2);
  t = contract(t, twist(wT, 1), {-1, 1, -3, -4, -5}, {-2, 1}, 2);
  t = contract(t, wR, {-1, -2, 1, -4, -5}, {1, -3}, 2);
  return contract(t, wB, {-1, -2, -3, 1, -5}, {1, -4}, 2);
}

namespace {
// tSVD(std::numeric_limits<std::size_t>::max(), 0.): every singular value kept
constexpr int64_t kKeepAll = int64_t(1) << 62;
Tensor id_like(const Tensor& w) { return identity(w.meta->sym, w.meta->dom, w.meta->cod); }
}  // namespace

SimpleUpdate::SimpleUpdate(int Lx_, int Ly_, const std::vector<int>& labels_, const std::vector<Tensor>& G_,
                           int64_t D_)
    : Lx(Lx_), Ly(Ly_), labels(labels_), D(D_) {
  if (Lx <= 0 || Ly <= 0 || int64_t(labels.size()) != int64_t(Lx) * Ly)
    throw std::runtime_error("simple update: pattern must have Lx * Ly labels");
  if (D <= 0) throw std::runtime_error("simple update: bond dimension must be positive");
  const int n = int(G_.size());
  std::vector<int> seen(size_t(std::max(n, 1)), 0);
  for (int v : labels) {
    if (v < 0 || v >= n) throw std::runtime_error("simple update: labels must be 0 .. number of site tensors - 1");
    seen[size_t(v)] = 1;
  }
  for (int v = 0; v < n; ++v)
    if (!seen[size_t(v)]) throw std::runtime_error("simple update: a site tensor has no label in the pattern");
  for (int i = 0; i < n; ++i) {
    auto [x, y] = coords(i);
    if (label(x, y) == label(x + 1, y) || label(x, y) == label(x, y + 1))
      throw std::runtime_error("simple update: neighbouring sites must carry different labels");
  }
  for (const Tensor& g0 : G_) {
    Tensor g = materialize(g0);
    if (g.meta->rank() != 2 || g.meta->corank() != 3)
      throw std::runtime_error("simple update: site tensors must be Tensor<2,3>");
    const Sym& s = g.meta->sym;
    wh.push_back(identity(s, {g.meta->cod[0]}, {g.meta->cod[0]}));  // right leg
    wv.push_back(identity(s, {g.meta->dom[1]}, {g.meta->dom[1]}));  // top leg
    G.push_back(g);
  }
}

int SimpleUpdate::label(int x, int y) const {
  x %= Lx;
  if (x < 0) x += Lx;
  y %= Ly;
  if (y < 0) y += Ly;
  return labels[size_t(x) * size_t(Ly) + size_t(y)];
}

void SimpleUpdate::step_h(int x, int y, const Tensor& Uh) {
  // t_step_h (TimePropagator.cpp:112-186)
  auto u = [&](int a, int b) { return size_t(label(a, b)); };
  const Tensor sq = diag_apply(wh[u(x, y)], XGB_DIAG_SQRT);
  Tensor left_full = apply_weights(G[u(x, y)], wh[u(x - 1, y)], wv[u(x, y)], sq, wv[u(x, y + 1)]);
  Tensor right_full = apply_weights(G[u(x + 1, y)], sq, wv[u(x + 1, y)], wh[u(x + 1, y)], wv[u(x + 1, y + 1)]);
  SVDResult l = tsvd(permute(left_full, -1, {0, 1, 3, 2, 4}), kKeepAll, 0.0, false);
  Tensor bond_l = matmul(l.S, l.Vdag);
  SVDResult r = tsvd(permute(right_full, 0, {0, 4, 1, 2, 3}), kKeepAll, 0.0, false);
  Tensor bond_r = matmul(r.U, r.S);
  Tensor bond = contract(bond_l, bond_r, {-1, 1, -2}, {1, -3, -4}, 2);
  Tensor enlarged = contract(twist(twist(Uh, 0), 1), bond, {1, 2, -1, -3}, {-2, 1, 2, -4}, 2);
  SVDResult b = tsvd(enlarged, D, 1.0e-14, false);  // SimpleUpdate::renormalize
  wh[u(x, y)] = normalize_max(b.S);
  const Tensor idh = id_like(wh[u(x, y)]);
  Tensor g1 = contract(l.U, b.U, {-1, -2, -4, 1}, {-5, 1, -3}, 2);
  G[u(x, y)] = apply_weights(g1, diag_apply(wh[u(x - 1, y)], XGB_DIAG_INV), diag_apply(wv[u(x, y)], XGB_DIAG_INV), idh,
                             diag_apply(wv[u(x, y + 1)], XGB_DIAG_INV));
  g1 = contract(b.Vdag, r.Vdag, {-1, -5, 1}, {1, -2, -3, -4}, 2);
  G[u(x + 1, y)] = apply_weights(g1, idh, diag_apply(wv[u(x + 1, y)], XGB_DIAG_INV),
                                 diag_apply(wh[u(x + 1, y)], XGB_DIAG_INV), diag_apply(wv[u(x + 1, y + 1)], XGB_DIAG_INV));
}

void SimpleUpdate::step_v(int x, int y, const Tensor& Uv) {
  // t_step_v (TimePropagator.cpp:188-215)
  auto u = [&](int a, int b) { return size_t(label(a, b)); };
  const Tensor sq = diag_apply(wv[u(x, y)], XGB_DIAG_SQRT);
  Tensor top_full = apply_weights(G[u(x, y - 1)], wh[u(x - 1, y - 1)], wv[u(x, y - 1)], wh[u(x, y - 1)], sq);
  Tensor bottom_full = apply_weights(G[u(x, y)], wh[u(x - 1, y)], sq, wh[u(x, y)], wv[u(x, y + 1)]);
  SVDResult t = tsvd(permute(top_full, -1, {0, 1, 2, 3, 4}), kKeepAll, 0.0, false);
  Tensor bond_t = matmul(t.S, t.Vdag);
  SVDResult v = tsvd(permute(bottom_full, 0, {1, 4, 0, 2, 3}), kKeepAll, 0.0, false);
  Tensor bond_b = matmul(v.U, v.S);
  Tensor bond = contract(bond_t, bond_b, {-1, 1, -2}, {1, -3, -4}, 2);
  Tensor enlarged = contract(twist(twist(Uv, 0), 1), bond, {1, 2, -1, -3}, {-2, 1, 2, -4}, 2);
  SVDResult b = tsvd(enlarged, D, 1.0e-14, false);
  wv[u(x, y)] = normalize_max(b.S);
  const Tensor idv = id_like(wv[u(x, y)]);
  Tensor g1 = contract(t.U, b.U, {-1, -2, -3, 1}, {-5, 1, -4}, 2);
  G[u(x, y - 1)] = apply_weights(g1, diag_apply(wh[u(x - 1, y - 1)], XGB_DIAG_INV),
                                 diag_apply(wv[u(x, y - 1)], XGB_DIAG_INV), diag_apply(wh[u(x, y - 1)], XGB_DIAG_INV), idv);
  g1 = contract(b.Vdag, v.Vdag, {-2, -5, 1}, {1, -1, -3, -4}, 2);
  G[u(x, y)] = apply_weights(g1, diag_apply(wh[u(x - 1, y)], XGB_DIAG_INV), idv, diag_apply(wh[u(x, y)], XGB_DIAG_INV),
                             diag_apply(wv[u(x, y + 1)], XGB_DIAG_INV));
}

void SimpleUpdate::step(const Tensor& Uh, const Tensor& Uv) {
  const int n = int(G.size());
  for (int i = 0; i < n; ++i) { auto [x, y] = coords(i); step_h(x, y, Uh); }
  for (int i = 0; i < n; ++i) { auto [x, y] = coords(i); step_v(x, y, Uv); }
  for (int i = n - 1; i >= 0; --i) { auto [x, y] = coords(i); step_v(x, y, Uv); }
  for (int i = n - 1; i >= 0; --i) { auto [x, y] = coords(i); step_h(x, y, Uh); }
}

Tensor SimpleUpdate::site_tensor(int i) const {
  auto [x, y] = coords(i);
  auto u = [&](int a, int b) { return size_t(label(a, b)); };
  return apply_weights(G[u(x, y)], diag_apply(wh[u(x - 1, y)], XGB_DIAG_SQRT), diag_apply(wv[u(x, y)], XGB_DIAG_SQRT),
                       diag_apply(wh[u(x, y)], XGB_DIAG_SQRT), diag_apply(wv[u(x, y + 1)], XGB_DIAG_SQRT));
}

// ======================================================================= CTM
static Tensor tw(const Tensor& t, std::initializer_list<int> legs) {
  Tensor o = t;
  for (int l : legs) o = twist(o, l);
  return o;
}

CTM::CTM(const Tensor& A_, int64_t chi_) : chi(chi_), policy(std::make_shared<HistoryPolicy>()), A(materialize(A_)) {
  if (A.meta->rank() != 2 || A.meta->corank() != 3) throw std::runtime_error("CTM: site tensor must be Tensor<2,3>");
  // Adags = As.adjoint().eval().permute<0, 3, 4, 2, 0, 1>()  (src/PEPS/iPEPS.cpp:210)
  Ad = permute(adjoint(A), 0, {3, 4, 2, 0, 1});
}

Tensor& CTM::slot(int which) {
  switch (which) {
    case 0: return C1; case 1: return C2; case 2: return C3; case 3: return C4;
    case 4: return T1; case 5: return T2; case 6: return T3; case 7: return T4;
    case 8: return A; default: return Ad;
  }
}

void CTM::init() {
  // CTM::init, FROM_A, TRank == 2, not ALL_OUT_LEGS (src/PEPS/CTM.cpp:161-212)
  const Sym s = A.meta->sym;
  auto ket = [&](char l) -> BasisPtr {
    switch (l) { case 'L': return A.meta->dom[0]; case 'T': return A.meta->dom[1]; case 'R': return A.meta->cod[0];
      case 'B': return A.meta->cod[1]; default: return A.meta->cod[2]; }
  };
  auto bra = [&](char l) -> BasisPtr {
    switch (l) { case 'L': return Ad.meta->dom[0]; case 'T': return Ad.meta->dom[1]; case 'R': return Ad.meta->cod[0];
      case 'B': return Ad.meta->cod[1]; default: return Ad.meta->dom[2]; }
  };
  auto fused = [&](char l) { return basis_forget_history(basis_combine(ket(l), bra(l))); };
  Tensor fuse_ll = identity(s, {fused('L')}, {ket('L'), bra('L')});
  Tensor fuse_uu = identity(s, {fused('T')}, {ket('T'), bra('T')});
  Tensor fuse_rr = identity(s, {ket('R'), bra('R')}, {fused('R')});
  Tensor fuse_dd = identity(s, {ket('B'), bra('B')}, {fused('B')});
  C1 = contract(contract(contract(A, tw(Ad, {3, 4}), {1, 2, -1, -2, 3}, {1, 2, 3, -3, -4}, 2), fuse_rr, {1, -1, 2, -2}, {1, 2, -3}, 2),
                fuse_dd, {1, 2, -2}, {1, 2, -1}, 0);
  C2 = contract(contract(contract(A, tw(Ad, {4}), {-1, 1, 2, -2, 3}, {-3, 1, 3, 2, -4}, 2), tw(fuse_ll, {1, 2}), {1, -1, 2, -2},
                         {-3, 1, 2}, 2),
                fuse_dd, {1, 2, -1}, {1, 2, -2}, 1);
  C3 = contract(contract(contract(A, Ad, {-1, -2, 1, 2, 3}, {-3, -4, 3, 1, 2}, 2), tw(fuse_ll, {1, 2}), {1, -1, 2, -2}, {-3, 1, 2}, 2),
                tw(fuse_uu, {1, 2}), {1, 2, -2}, {-1, 1, 2}, 2);
  C4 = contract(contract(contract(A, tw(Ad, {3}), {1, -1, -2, 2, 3}, {1, -3, 3, -4, 2}, 2), tw(fuse_uu, {1, 2}), {1, -1, 2, -2},
                         {-3, 1, 2}, 2),
                fuse_rr, {1, 2, -1}, {1, 2, -2}, 1);
  T1 = contract(contract(contract(A, tw(Ad, {3, 4}), {-1, 1, -2, -3, 2}, {-4, 1, 2, -5, -6}, 3), tw(fuse_ll, {1, 2}),
                         {1, -1, -2, 2, -3, -4}, {-5, 1, 2}, 4),
                fuse_rr, {1, -3, 2, -4, -1}, {1, 2, -2}, 1);
  T2 = contract(contract(contract(A, tw(Ad, {4}), {-1, -2, 1, -3, 2}, {-4, -5, 2, 1, -6}, 3), tw(fuse_uu, {1, 2}),
                         {-1, 1, -2, -3, 2, -4}, {-5, 1, 2}, 4),
                fuse_dd, {-1, 1, -2, 2, -3}, {1, 2, -4}, 3);
  T3 = contract(contract(contract(A, tw(Ad, {3}), {-1, -2, -3, 1, 2}, {-4, -5, 2, -6, 1}, 3), tw(fuse_ll, {1, 2}),
                         {1, -1, -2, 2, -3, -4}, {-5, 1, 2}, 4),
                fuse_rr, {-1, 1, -2, 2, -3}, {1, 2, -4}, 3);
  T4 = contract(contract(contract(A, tw(Ad, {3, 4}), {1, -1, -2, -3, 2}, {1, -4, 2, -5, -6}, 3), tw(fuse_uu, {1, 2}),
                         {1, -1, -2, 2, -3, -4}, {-5, 1, 2}, 4),
                fuse_dd, {-3, 1, -4, 2, -1}, {1, 2, -2}, 1);
}

Tensor CTM::contract_corner(const char* corner) {
  // contractCorner, TRank == 2 (src/PEPS/CTM.cpp:1667-1738)
  const std::string c(corner);
  if (c == "UL") {
    Tensor C1T1 = contract(C1, T1, {-1, 1}, {1, -2, -3, -4}, 1);
    Tensor T4C1T1 = contract(T4, tw(C1T1, {0}), {1, -1, -2, -3}, {1, -4, -5, -6}, 3);
    Tensor T4C1T1A = contract(T4C1T1, A, {-1, 1, -2, -3, 2, -4}, {1, 2, -5, -6, -7}, 4);
    return contract(T4C1T1A, tw(Ad, {3, 4}), {-1, 1, -4, 2, -5, -2, 3}, {1, 2, 3, -6, -3}, 3);
  }
  if (c == "LL") {
    Tensor C4T3 = contract(C4, T3, {-1, 1}, {-2, -3, 1, -4}, 1);
    Tensor T4C4T3 = contract(T4, C4T3, {-1, 1, -2, -3}, {1, -4, -5, -6}, 3);
    Tensor T4C4T3A = contract(T4C4T3, tw(A, {3}), {-1, 1, -2, 2, -3, -4}, {1, -5, -6, 2, -7}, 4);
    return contract(T4C4T3A, tw(Ad, {3}), {-4, 1, 2, -1, -5, -2, 3}, {1, -6, 3, -3, 2}, 3);
  }
  if (c == "UR") {
    Tensor T1C2 = contract(T1, C2, {-1, 1, -2, -3}, {1, -4}, 3);
    Tensor T1C2T2 = contract(T1C2, T2, {-1, -2, -3, 1}, {-4, -5, 1, -6}, 3);
    Tensor T1C2T2A = contract(T1C2T2, tw(A, {2}), {-1, 1, -2, 2, -3, -4}, {-5, 1, 2, -6, -7}, 4);
    return contract(T1C2T2A, tw(Ad, {4}), {-1, 1, 2, -4, -2, -5, 3}, {-3, 1, 3, 2, -6}, 3);
  }
  if (c == "LR") {
    Tensor C3T3 = contract(tw(C3, {1}), T3, {-1, 1}, {-2, -3, -4, 1}, 1);
    Tensor T2C3T3 = contract(T2, C3T3, {-1, -2, -3, 1}, {1, -4, -5, -6}, 3);
    Tensor T2C3T3A = contract(T2C3T3, tw(A, {2, 3}), {1, -1, -2, 2, -3, -4}, {-5, -6, 1, 2, -7}, 4);
    return contract(T2C3T3A, Ad, {1, -1, 2, -4, -5, -2, 3}, {-6, -3, 3, 1, 2}, 3);
  }
  throw std::runtime_error("contract_corner: unknown corner");
}

std::pair<Tensor, Tensor> CTM::decompose_dir(int d, const Tensor& t1, const Tensor& t2) {
  // decompose (src/PEPS/PEPSContractions.cpp:16-43) with the configured SVD form; the product, the
  // SVD and the projectors are FP64 (or the FP64-accurate tensor-core form) whatever the GEMM form
  const bool exact_tc = gemm_prec == XGB_PREC_F64TC;
  GemmPrecisionScope fp64(exact_tc ? XGB_PREC_F64TC : XGB_PREC_FP64);
  Tensor prod = matmul(t1, t2);
  const TensorMeta& m = *prod.meta;
  const size_t n = m.sectors.size();
  // inside a fork-join section the statistics and the record go to this direction's slot and are
  // committed in the sequential order afterwards; the seed is the one the sequential order gives
  Deferred* df = defer_[d].on ? &defer_[d] : nullptr;
  CTMStats& st = df ? df->delta : stats;
  const int64_t dec_index = df ? df->index : stats.decompositions;
  DecompRecord rec;
  if (record) {
    rec.dir = d;
    rec.sectors = m.sectors;
    sector_features(m, hist[d], chi, rec.features);
  }
  SVDResult r;
  std::vector<int64_t> width(n);
  if (svd_mode == 0) {
    r = tsvd(prod, chi, 1.0e-10, false);
    for (size_t i = 0; i < n; ++i) width[i] = std::min(m.rows[i], m.cols[i]);
    st.exact_sectors += int64_t(n);
  } else {
    if (!policy) throw std::runtime_error("CTM: randomized projector SVD without a width policy");
    std::vector<int64_t> want = policy->widths(m, hist[d], chi);
    if (sketch_unseen)
      for (size_t i = 0; i < n; ++i)
        if (want[i] <= 0 && hist[d].find(m.sectors[i]) == hist[d].end())
          want[i] = std::min<int64_t>(chi, std::min(m.rows[i], m.cols[i])) + 16;
    RsvdInfo info;
    const bool warm = warm_iters >= 0 && warm_v[d].valid() && warm_v[d].meta->cod == m.cod;
    r = tsvd_randomized(prod, chi, 1.0e-10, want, warm ? warm_iters : power_iters, seed + uint64_t(dec_index), &info,
                        warm ? &warm_v[d] : nullptr, res_tol, sketch_fp64_tail, exact_tc);
    st.refinements += info.refinements;
    st.max_residual = info.max_residual;
    if (df) df->residual_set = true;
    width = info.width;
    st.exact_sectors += info.exact_sectors;
    st.sketched_sectors += int64_t(n) - info.exact_sectors;
    st.redo += int64_t(info.saturated.size());
    st.sketch_cols += info.sketch_cols;
  }
  ++st.decompositions;
  // history for the next decomposition of this direction
  History h;
  double smax = 0;
  for (double v : r.spectrum) smax = std::max(smax, v);
  for (size_t i = 0; i < n; ++i) {
    SectorHistory e;
    e.rows = m.rows[i];
    e.cols = m.cols[i];
    e.keep = r.keep[i];
    e.width = width[i];
    const int64_t b = r.spec_begin[i], len = r.spec_begin[i + 1] - b;
    e.s_first = len > 0 ? r.spectrum[size_t(b)] : 0.0;
    e.s_last = e.keep > 0 ? r.spectrum[size_t(b + e.keep - 1)] : 0.0;
    e.s_next = e.keep < len ? r.spectrum[size_t(b + e.keep)] : 0.0;
    e.s_max = smax;
    h[m.sectors[i]] = e;
  }
  hist[d] = std::move(h);
  if (warm_iters >= 0) warm_v[d] = r.Vdag;
  if (record) {
    rec.keep.assign(r.keep.begin(), r.keep.end());
    rec.width = width;
    for (size_t i = 0; i < n; ++i) rec.kmin.push_back(std::min(m.rows[i], m.cols[i]));
    rec.spectrum = r.spectrum;
    rec.spec_begin = r.spec_begin;
    (df ? df->records : records).push_back(std::move(rec));
  }
  return projectors_from_svd(r, t1, t2);
}

Tensor CTM::rdm(bool vertical) {
  if (!vertical) {
    // computeRDM_h, TRank == 2 (src/PEPS/CTM.cpp:583-619)
    Tensor C1T1 = contract(C1, T1, {-1, 1}, {1, -2, -3, -4}, 1);
    Tensor T4C1T1 = contract(T4, twist(C1T1, 0), {1, -1, -2, -3}, {1, -4, -5, -6}, 3);
    Tensor T4C1T1A = contract(T4C1T1, A, {-1, 1, -2, -3, 2, -4}, {1, 2, -5, -6, -7}, 4);
    Tensor C4T3 = contract(C4, T3, {-1, 1}, {-2, -3, 1, -4}, 1);
    Tensor C4T3Ad = contract(C4T3, twist(Ad, 3), {-1, -2, 1, -3}, {-4, -5, -6, -7, 1}, 3);
    Tensor left = contract(T4C1T1A, C4T3Ad, {1, 2, -1, 3, -2, 4, -3}, {1, 4, -4, 2, 3, -5, -6}, 3);
    Tensor T1C2 = contract(T1, C2, {-1, 1, -2, -3}, {1, -4}, 3);
    Tensor T1C2T2 = contract(T1C2, T2, {-1, -2, -3, 1}, {-4, -5, 1, -6}, 3);
    Tensor AT1C2T2 = contract(twist(A, 1), T1C2T2, {-1, 1, 2, -2, -3}, {-4, 1, -5, 2, -6, -7}, 3);
    Tensor T3C3 = contract(T3, C3, {-1, -2, -3, 1}, {-4, 1}, 3);
    Tensor T3C3Ad = contract(T3C3, Ad, {-1, 1, -2, -3}, {-4, -5, -6, -7, 1}, 3);
    Tensor right = contract(AT1C2T2, T3C3Ad, {-1, 1, -2, -3, 2, 3, 4}, {1, -4, 4, -5, 2, -6, 3}, 3);
    Tensor rho = contract(left, right, {1, 2, -3, 3, -1, 4}, {2, -4, 1, 3, 4, -2}, 2);
    Tensor id2 = identity(rho.meta->sym, rho.meta->cod, rho.meta->dom);
    const double norm = scalar_value(contract(rho, twist(twist(id2, 0), 1), {1, 2, 3, 4}, {3, 4, 1, 2}, 0));
    return scale(rho, 1.0 / norm);
  }
  // computeRDM_v, TRank == 2 (src/PEPS/CTM.cpp:756-781)
  Tensor C1T1 = contract(C1, T1, {-1, 1}, {1, -2, -3, -4}, 1);
  Tensor T4C1T1 = contract(T4, twist(C1T1, 0), {1, -1, -2, -3}, {1, -4, -5, -6}, 3);
  Tensor T4C1T1A = contract(T4C1T1, A, {-1, 1, -2, -3, 2, -4}, {1, 2, -5, -6, -7}, 4);
  Tensor C2T2 = contract(C2, T2, {-1, 1}, {-2, -3, 1, -4}, 1);
  Tensor AdC2T2 = contract(twist(twist(Ad, 3), 4), C2T2, {-1, -2, -3, 1, -4}, {-5, -6, 1, -7}, 4);
  Tensor upper = contract(T4C1T1A, AdC2T2, {-1, 1, 2, 3, 4, -2, -3}, {1, 3, -4, -5, 2, 4, -6}, 3);
  Tensor C4T3 = contract(C4, T3, {-1, 1}, {-2, -3, 1, -4}, 1);
  Tensor T4C4T3 = contract(T4, C4T3, {-1, 1, -2, -3}, {1, -4, -5, -6}, 3);
  Tensor AT4C4T3 = contract(twist(A, 0), T4C4T3, {1, -1, -2, 2, -3}, {-4, 1, -5, 2, -6, -7}, 3);
  Tensor T2C3 = contract(T2, C3, {-1, -2, -3, 1}, {1, -4}, 3);
  Tensor T2C3Ad = contract(T2C3, Ad, {-1, 1, -2, -3}, {-4, -5, -6, 1, -7}, 3);
  Tensor lower = contract(AT4C4T3, T2C3Ad, {-1, 1, -2, -3, 2, 3, 4}, {1, -4, 4, 2, -5, -6, 3}, 3);
  Tensor rho = contract(upper, lower, {1, 2, -3, -1, 3, 4}, {2, -4, 1, 4, 3, -2}, 2);
  Tensor id2 = identity(rho.meta->sym, rho.meta->cod, rho.meta->dom);
  const double norm = scalar_value(contract(rho, twist(twist(id2, 0), 1), {1, 2, 3, 4}, {3, 4, 1, 2}, 0));
  return scale(rho, 1.0 / norm);
}

double scalar_value(const Tensor& t0) {
  Tensor t = materialize(t0);
  if (t.meta->size == 0) return 0.0;
  if (t.meta->size != 1) throw std::runtime_error("scalar_value: tensor holds more than one entry");
  double v = 0;
  cuda_ok(cudaMemcpyAsync(&v, t.data(), sizeof(double), cudaMemcpyDeviceToHost, stream()), "d2h");
  cuda_ok(cudaStreamSynchronize(stream()), "sync");
  return v;
}

double bond_expectation(const Tensor& rho, const Tensor& op) {
  return scalar_value(contract(twist(twist(rho, 0), 1), op, {1, 2, 3, 4}, {3, 4, 1, 2}, 0));
}

std::pair<Tensor, Tensor> CTM::get_projectors(char dir) {
  // get_projectors, PROJECTION::CORNER (src/PEPS/CTM.cpp:1195-1326)
  switch (dir) {
    case 'L': {
      Tensor Q1 = contract_corner("UL");
      Tensor Q4 = tw(contract_corner("LL"), {3, 4, 5});
      return decompose_dir(0, Q4, Q1);
    }
    case 'R': {
      Tensor Q2 = contract_corner("UR");
      Tensor Q3 = contract_corner("LR");
      return decompose_dir(1, Q2, Q3);
    }
    case 'T': {
      Tensor Q1 = contract_corner("UL");
      Tensor Q2 = contract_corner("UR");
      return decompose_dir(2, Q1, Q2);
    }
    default: {
      Tensor Q4 = tw(contract_corner("LL"), {0, 1, 2});
      Tensor Q3 = contract_corner("LR");
      return decompose_dir(3, Q3, Q4);
    }
  }
}

std::tuple<Tensor, Tensor, Tensor> CTM::renormalize(char dir, const Tensor& P1, const Tensor& P2) {
  // renormalize_left/right/top/bottom, TRank == 2 (src/PEPS/CTM.cpp:1358-1627)
  if (dir == 'L') {
    Tensor C1T1 = contract(C1, T1, {-1, 1}, {1, -4, -2, -3}, 3);
    Tensor C1n = contract(tw(P1, {1, 2, 3}), C1T1, {-1, 1, 2, 3}, {1, 2, 3, -2}, 0);
    Tensor C4T3 = contract(C4, T3, {-2, 1}, {-3, -4, 1, -1}, 1);
    Tensor C4n = contract(C4T3, tw(P2, {0, 1, 2}), {-2, 1, 2, 3}, {1, 2, 3, -1}, 1);
    Tensor P1T4 = contract(tw(P1, {1, 2, 3}), T4, {-1, 1, -2, -3}, {-4, 1, -5, -6}, 3);
    Tensor P1T4A = contract(P1T4, A, {-1, 2, -2, -3, 1, -4}, {1, -5, -6, 2, -7}, 4);
    Tensor P1T4AAd = contract(P1T4A, tw(Ad, {3, 4}), {-1, 2, -4, 1, -5, -2, 3}, {1, -6, 3, -3, 2}, 3);
    Tensor T4n = contract(P1T4AAd, tw(P2, {0, 1, 2}), {-2, -3, -4, 1, 2, 3}, {1, 2, 3, -1}, 1);
    return {normalize_max(C1n), normalize_max(T4n), normalize_max(C4n)};
  }
  if (dir == 'R') {
    Tensor T1C2 = contract(T1, C2, {-1, 1, -3, -4}, {1, -2}, 1);
    Tensor C2n = contract(T1C2, P2, {-1, 1, 2, 3}, {1, 2, 3, -2}, 1);
    Tensor C3T3 = contract(tw(C3, {1}), T3, {-1, 1}, {-2, -3, -4, 1}, 3);
    Tensor C3n = contract(P1, C3T3, {-1, 1, 2, 3}, {1, 2, 3, -2}, 2);
    Tensor P1T2 = contract(P1, T2, {-1, 1, -2, -3}, {-4, -5, 1, -6}, 3);
    Tensor P1T2A = contract(P1T2, tw(A, {2}), {-1, 1, -2, 2, -3, -4}, {-5, 1, 2, -6, -7}, 4);
    Tensor P1T2AAd = contract(P1T2A, tw(Ad, {4}), {-1, 1, 2, -4, -2, -5, 3}, {-3, 1, 3, 2, -6}, 3);
    Tensor T2n = contract(P1T2AAd, P2, {-3, -1, -2, 1, 2, 3}, {1, 2, 3, -4}, 3);
    return {normalize_max(C2n), normalize_max(T2n), normalize_max(C3n)};
  }
  if (dir == 'T') {
    Tensor T4C1 = contract(T4, tw(C1, {0}), {1, -1, -3, -4}, {1, -2}, 1);
    Tensor C1n = contract(T4C1, P2, {-1, 1, 2, 3}, {1, 2, 3, -2}, 0);
    Tensor C2T2 = contract(C2, T2, {-1, 1}, {-2, -3, 1, -4}, 3);
    Tensor C2n = contract(P1, C2T2, {-1, 1, 2, 3}, {1, 2, 3, -2}, 1);
    Tensor P1T1 = contract(P1, T1, {-1, 1, -2, -3}, {1, -4, -5, -6}, 3);
    Tensor P1T1A = contract(P1T1, A, {-1, 1, -2, -3, 2, -4}, {1, 2, -5, -6, -7}, 4);
    Tensor P1T1AAd = contract(P1T1A, tw(Ad, {3, 4}), {-1, 1, -4, 2, -5, -2, 3}, {1, 2, 3, -6, -3}, 3);
    Tensor T1n = contract(P1T1AAd, P2, {-1, -3, -4, 1, 2, 3}, {1, 2, 3, -2}, 1);
    return {normalize_max(C1n), normalize_max(T1n), normalize_max(C2n)};
  }
  Tensor T4C4 = contract(T4, C4, {-4, 1, -2, -3}, {1, -1}, 3);
  Tensor C4n = contract(tw(P1, {1, 2, 3}), T4C4, {-2, 1, 2, 3}, {1, 2, 3, -1}, 1);
  Tensor T2C3 = contract(T2, C3, {-3, -4, -1, 1}, {1, -2}, 1);
  Tensor C3n = contract(T2C3, tw(P2, {0, 1, 2}), {-1, 1, 2, 3}, {1, 2, 3, -2}, 2);
  Tensor P1T3 = contract(tw(P1, {1, 2, 3}), tw(T3, {0}), {-1, 1, -2, -3}, {-4, -5, -6, 1}, 3);
  Tensor P1T3A = contract(P1T3, A, {-1, 1, -2, 2, -3, -4}, {-5, -6, 1, 2, -7}, 4);
  Tensor P1T3AAd = contract(P1T3A, tw(Ad, {3}), {-1, 1, 2, -4, -5, -2, 3}, {-6, -3, 3, 1, 2}, 3);
  Tensor T3n = contract(P1T3AAd, tw(P2, {0, 1, 2}), {-4, -1, -2, 1, 2, 3}, {1, 2, 3, -3}, 3);
  return {normalize_max(C4n), normalize_max(T3n), normalize_max(C3n)};
}

void CTM::move(char dir) {
  GemmPrecisionScope prec(gemm_prec);
  auto [P1, P2] = get_projectors(dir);
  auto [a, b, c] = renormalize(dir, P1, P2);
  switch (dir) {
    case 'L': C1 = a; T4 = b; C4 = c; break;
    case 'R': C2 = a; T2 = b; C3 = c; break;
    case 'T': C1 = a; T1 = b; C2 = c; break;
    default: C4 = a; T3 = b; C3 = c; break;
  }
}

bool CTM::pairs_concurrent() const {
  // exact projector SVDs keep their wide blocks on the grid-wide kernel of lane 0; per-launch
  // profiling and autotune measurements time one lane at a time
  return concurrent && svd_mode != 0 && !profiling() && autotune_mode() != 1;
}

void CTM::move_pair(char a, char b) {
  auto dir = [](char c) { return c == 'L' ? 0 : c == 'R' ? 1 : c == 'T' ? 2 : 3; };
  const int da = dir(a), db = dir(b);
  defer_[da] = Deferred{};
  defer_[db] = Deferred{};
  defer_[da].on = defer_[db].on = true;
  defer_[da].index = stats.decompositions;
  defer_[db].index = stats.decompositions + 1;
  try {
    run_pair([&] { move(a); }, [&] { move(b); });
  } catch (...) {
    defer_[da].on = defer_[db].on = false;
    throw;
  }
  for (int d : {da, db}) {
    Deferred& f = defer_[d];
    f.on = false;
    stats.decompositions += f.delta.decompositions;
    stats.sketched_sectors += f.delta.sketched_sectors;
    stats.exact_sectors += f.delta.exact_sectors;
    stats.redo += f.delta.redo;
    stats.sketch_cols += f.delta.sketch_cols;
    stats.refinements += f.delta.refinements;
    if (f.residual_set) stats.max_residual = f.delta.max_residual;
    for (auto& r : f.records) records.push_back(std::move(r));
    f.records.clear();
  }
}

void CTM::grow_all() {
  // CTM::grow_all (src/PEPS/CTM.cpp:385-398): left, right, top, bottom.  The left and right moves
  // read and replace disjoint environment tensors (C1 T4 C4 and C2 T2 C3; both read T1 and T3), and
  // so do the top and bottom moves (C1 T1 C2 and C4 T3 C3; both read T2 and T4): each pair runs at
  // once on two lanes, with the result of the sequential order.
  if (!pairs_concurrent()) {
    move('L');
    move('R');
    move('T');
    move('B');
    return;
  }
  move_pair('L', 'R');
  move_pair('T', 'B');
}

CTM::SolveResult CTM::solve(const Tensor& H, double tol_E, int max_steps) {
  // CTMSolver::solve without AD (src/PEPS/CTMSolver.cpp:50-80) on a 1x1 cell: grow_all, the bond
  // energy per site E = <H>_h + <H>_v from computeRDM, stop when |E - E_prev| < tol_E or, as an
  // oscillation, |E - E_prevprev| < tol_E; `steps` counts the grow_all steps run
  SolveResult r;
  double prev = 1000.0, prevprev = 1000.0;
  for (int step = 0; step < max_steps; ++step) {
    grow_all();
    const double E = bond_expectation(rdm(false), H) + bond_expectation(rdm(true), H);
    r.energies.push_back(E);
    r.E = E;
    r.steps = step + 1;
    if (std::abs(E - prev) < tol_E) {
      r.converged = true;
      break;
    }
    if (std::abs(E - prevprev) < tol_E) {
      r.converged = true;
      r.oscillation = true;
      break;
    }
    prevprev = prev;
    prev = E;
  }
  return r;
}

}  // namespace xgb
