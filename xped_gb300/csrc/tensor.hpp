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
  // full spectrum of the input (device), for the learned-rank path
};
SVDResult tsvd(const Tensor& t, int64_t max_keep, double eps_svd, bool preserve_multiplets);
std::pair<Tensor, Tensor> tqr(const Tensor& t);
std::pair<Tensor, Tensor> decompose(const Tensor& t1, const Tensor& t2, int64_t max_nsv);

// get_permutations (include/Xped/Util/Constfct.hpp:55-109)
struct ContractPerms {
  std::vector<int> p1, p2, pres;
  int shift1 = 0, shift2 = 0, shiftres = 0;
};
ContractPerms get_permutations(const std::vector<int>& a1, int rank1, const std::vector<int>& a2, int rank2, int rankres);

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
  Tensor& slot(int which);  // 0..3 = C1..C4, 4..7 = T1..T4, 8 = A, 9 = Adag
  int64_t chi = 0;

 private:
  Tensor A, Ad;
  Tensor C1, C2, C3, C4, T1, T2, T3, T4;
};

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
