// Symmetry algebra, fusion trees and leg bases (host side).  See meta.hpp for
// the reference files each part restates.
#include "meta.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <unordered_set>

namespace xgb {

static constexpr double kTreeEps = 1.0e-12;  // ScalarTraits<double>::epsilon() (ScalarTraits.hpp:17)

static inline int posmod(int x, int n) { return (x % n + n) % n; }
static inline double phase(int q) { return (q % 2) ? -1.0 : 1.0; }  // functions.hpp:79-84

// ================================================================ Sym
int Sym::conj(int q) const {
  switch (kind) {
    case SYM_U1:
    case SYM_U1_FERMIONIC: return -q;                 // U1.hpp:104
    case SYM_Z2:
    case SYM_Z2_FERMIONIC: return posmod(-q, N);      // ZN.hpp:115
    default: return q;                                // SU2.hpp:111
  }
}

int Sym::combine(int ql, int qr, int* out) const {
  switch (kind) {
    case SYM_U1:
    case SYM_U1_FERMIONIC: out[0] = ql + qr; return 1;
    case SYM_Z2:
    case SYM_Z2_FERMIONIC: out[0] = posmod(ql + qr, N); return 1;
    default: {
      int qmin = std::abs(ql - qr) + 1, qmax = std::abs(ql + qr) - 1, n = 0;
      for (int i = qmin; i <= qmax && n < 64; i += 2) out[n++] = i;
      return n;
    }
  }
}

bool Sym::triangle(int q1, int q2, int q3) const {
  switch (kind) {
    case SYM_U1:
    case SYM_U1_FERMIONIC: return q1 + q2 == q3;
    case SYM_Z2:
    case SYM_Z2_FERMIONIC: return posmod(q1 + q2, N) == q3;
    default: return (q3 - 1 >= std::abs(q1 - q2)) && (q3 - 1 <= q1 + q2 - 2);  // SU2.cpp:114-119
  }
}

double Sym::coeff_swap(int ql, int qr, int qf) const {
  if (!triangle(ql, qr, qf)) return 0.0;
  if (kind == SYM_SU2) return phase((ql + qr - qf - 1) / 2);  // SU2.hpp:169-177
  double sign = 1.0;
  if (fermionic() && (ql % 2 != 0) && (qr % 2 != 0)) sign = -1.0;  // U1.hpp:174-182, ZN.hpp:185-193
  return sign;
}

double Sym::coeff_6j(int q1, int q2, int q3, int q4, int q5, int q6) const {
  if (kind == SYM_SU2) return wigner6j_twice(q1 - 1, q2 - 1, q3 - 1, q4 - 1, q5 - 1, q6 - 1);
  if (triangle(q1, q2, q3) && triangle(q1, q6, q5) && triangle(q2, q4, q6) && triangle(q3, q4, q5)) return 1.0;
  return 0.0;
}

double Sym::coeff_recouple(int q1, int q2, int q3, int Q, int Q12, int Q23) const {
  if (kind == SYM_SU2) {
    // SU2.hpp:164-167; the phase argument is (sum)/2. truncated to int
    double ph = phase(static_cast<int>((q1 + q2 + q3 + Q) / 2.0));
    return std::sqrt(static_cast<double>(Q12 * Q23)) * ph * coeff_6j(q1, q2, Q12, q3, Q, Q23);
  }
  return coeff_6j(q1, q2, Q12, q3, Q, Q23);
}

double Sym::coeff_turn(int ql, int qr, int qf) const {
  if (!triangle(ql, qr, qf)) return 0.0;
  if (kind == SYM_SU2) return coeff_swap(ql, qr, qf) * std::sqrt(static_cast<double>(qf) / static_cast<double>(ql));
  return 1.0;
}

double Sym::coeff_FS(int q) const {
  if (kind == SYM_SU2) return (q % 2 == 0) ? -1.0 : 1.0;  // SU2.cpp:35-39
  return 1.0;
}

double Sym::coeff_twist(int q) const {
  if (!fermionic()) return 1.0;
  return (q % 2 != 0) ? -1.0 : 1.0;
}

// Racah's formula with long-double factorials; exact enough for the spins
// that occur here (2j <= 40).
double wigner6j_twice(int a2, int b2, int c2, int d2, int e2, int f2) {
  auto tri = [](int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0) return false;
    if ((x + y + z) % 2) return false;
    return std::abs(x - y) <= z && z <= x + y;
  };
  if (!(tri(a2, b2, c2) && tri(a2, e2, f2) && tri(d2, b2, f2) && tri(d2, e2, c2))) return 0.0;
  static long double fact[200];
  static std::once_flag once;
  std::call_once(once, [] {
    fact[0] = 1.0L;
    for (int i = 1; i < 200; ++i) fact[i] = fact[i - 1] * i;
  });
  auto dsq = [&](int x, int y, int z) {
    return fact[(x + y - z) / 2] * fact[(x - y + z) / 2] * fact[(-x + y + z) / 2] / fact[(x + y + z) / 2 + 1];
  };
  long double pref = std::sqrt(dsq(a2, b2, c2) * dsq(a2, e2, f2) * dsq(d2, b2, f2) * dsq(d2, e2, c2));
  int s1 = (a2 + b2 + c2) / 2, s2 = (a2 + e2 + f2) / 2, s3 = (d2 + b2 + f2) / 2, s4 = (d2 + e2 + c2) / 2;
  int p1 = (a2 + b2 + d2 + e2) / 2, p2 = (a2 + c2 + d2 + f2) / 2, p3 = (b2 + c2 + e2 + f2) / 2;
  int tmin = std::max(std::max(s1, s2), std::max(s3, s4));
  int tmax = std::min(p1, std::min(p2, p3));
  long double sum = 0.0L;
  for (int t = tmin; t <= tmax; ++t) {
    long double term = fact[t + 1] / (fact[t - s1] * fact[t - s2] * fact[t - s3] * fact[t - s4] * fact[p1 - t] *
                                      fact[p2 - t] * fact[p3 - t]);
    sum += (t % 2) ? -term : term;
  }
  return static_cast<double>(pref * sum);
}

// ================================================================ trees
void FusionTree::compute_dim() {
  dim = 1;
  for (int i = 0; i < rank; ++i) dim *= dims[i];
}

bool FusionTree::operator==(const FusionTree& o) const {
  return rank == o.rank && qc == o.qc && qu == o.qu && qi == o.qi && dims == o.dims;
}

bool FusionTree::less(const FusionTree& o) const {
  for (int m = 0; m < rank; ++m) {
    if (qu[m] > o.qu[m]) return false;
    if (qu[m] < o.qu[m]) return true;
  }
  for (int m = 0; m < nqi(); ++m) {
    if (qi[m] > o.qi[m]) return false;
    if (qi[m] < o.qi[m]) return true;
  }
  return qc < o.qc;
}

size_t FusionTree::hash() const {
  uint64_t h = 1469598103934665603ull ^ static_cast<uint64_t>(rank);
  auto mix = [&](int64_t v) { h ^= static_cast<uint64_t>(v) + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2); };
  mix(qc);
  for (int i = 0; i < rank; ++i) { mix(qu[i]); mix(dims[i]); }
  for (int i = 0; i < nqi(); ++i) mix(qi[i]);
  return static_cast<size_t>(h);
}

FusionTree tree_enlarge(const FusionTree& t, const FusionTree& other) {
  // FusionTree::enlarge (FusionTree.cpp:309-324)
  FusionTree out;
  out.rank = t.rank + 1;
  for (int i = 0; i < t.rank; ++i) { out.qu[i] = t.qu[i]; out.dims[i] = t.dims[i]; }
  out.qu[t.rank] = other.qu[0];
  out.dims[t.rank] = other.dims[0];
  for (int i = 0; i < t.nqi(); ++i) out.qi[i] = t.qi[i];
  if (out.nqi() > 0) out.qi[out.nqi() - 1] = t.qc;
  out.dual = t.dual;
  out.set_dual(t.rank, other.is_dual(0));
  out.qc = t.qc;
  out.compute_dim();
  return out;
}

FusionTree tree_compute_intermediates(const Sym& s, FusionTree t) {
  // FusionTree::computeIntermediates (FusionTree.cpp:136-152), abelian only
  for (int i = 0; i < t.nqi(); ++i) t.qi[i] = (i == 0) ? s.combine1(t.qu[0], t.qu[1]) : s.combine1(t.qi[i - 1], t.qu[i + 1]);
  if (t.rank == 1) t.qc = t.qu[0];
  else if (t.rank == 2) t.qc = s.combine1(t.qu[0], t.qu[1]);
  else if (t.rank > 2) t.qc = s.combine1(t.qi[t.nqi() - 1], t.qu[t.rank - 1]);
  return t;
}

TreeMap tree_swap(const Sym& s, const FusionTree& t, int pos) {
  // FusionTree::swap (FusionTree.cpp:353-412)
  TreeMap out;
  FusionTree tree = t;
  std::swap(tree.qu[pos], tree.qu[pos + 1]);
  std::swap(tree.dims[pos], tree.dims[pos + 1]);
  bool d0 = t.is_dual(pos), d1 = t.is_dual(pos + 1);
  tree.set_dual(pos, d1);
  tree.set_dual(pos + 1, d0);
  if (pos == 0) {
    int ql = t.qu[0], qr = t.qu[1];
    int qf = (t.rank == 2) ? t.qc : t.qi[0];
    double c = s.coeff_swap(ql, qr, qf);
    if (std::abs(c) < kTreeEps) return out;
    out.emplace(tree, c);
    return out;
  }
  int q1 = (pos == 1) ? t.qu[0] : t.qi[pos - 2];
  int q2 = t.qu[pos];
  int q3 = t.qu[pos + 1];
  int Q = (pos == t.rank - 2) ? t.qc : t.qi[pos];
  int Q12 = t.qi[pos - 1];
  int buf[64];
  int n = s.combine(q3, q1, buf);
  for (int k = 0; k < n; ++k) {
    int Q31 = buf[k];
    tree.qi[pos - 1] = Q31;
    double cgc = s.coeff_swap(Q12, q3, Q) * s.coeff_recouple(q3, q1, q2, Q, Q31, Q12) * s.coeff_swap(q3, q1, Q31);
    if (std::abs(cgc) < kTreeEps) continue;
    out.emplace(tree, cgc);
  }
  return out;
}

std::vector<int> decompose_permutation(const std::vector<int>& pi) {
  // Permutation::decompose (Permutations.hpp:195-225)
  const int N = static_cast<int>(pi.size());
  std::vector<int> a(N), out;
  std::iota(a.begin(), a.end(), 0);
  if (a == pi) return out;
  for (int i = 0; i < N; ++i) {
    int index = static_cast<int>(std::find(a.begin(), a.end(), pi[i]) - a.begin());
    if (index == 0) continue;
    for (int j = index - 1; j >= i; --j) {
      std::swap(a[j], a[j + 1]);
      out.push_back(j);
    }
  }
  return out;
}

TreeMap tree_permute(const Sym& s, const FusionTree& t, const std::vector<int>& p) {
  // FusionTree::permute (FusionTree.cpp:326-351)
  TreeMap out;
  out.emplace(t, 1.0);
  for (int pos : decompose_permutation(p)) {
    TreeMap tmp;
    for (const auto& [tree, coeff] : out) {
      for (const auto& [tree2, coeff2] : tree_swap(s, tree, pos)) {
        auto it = tmp.find(tree2);
        if (it == tmp.end()) {
          tmp.emplace(tree2, coeff * coeff2);
        } else if (std::abs(it->second + coeff * coeff2) < kTreeEps) {
          tmp.erase(it);
        } else {
          it->second += coeff * coeff2;
        }
      }
    }
    out.swap(tmp);
  }
  return out;
}

static TreePairMap turn_right(const Sym& s, const FusionTree& t1, const FusionTree& t2) {
  // treepair::turn_right (treepair.cpp:35-88)
  const int R = t1.rank, C = t2.rank;
  FusionTree t1p;
  t1p.rank = R + 1;
  for (int i = 0; i < R; ++i) { t1p.qu[i] = t1.qu[i]; t1p.dims[i] = t1.dims[i]; }
  t1p.qu[R] = s.conj(t2.qu[C - 1]);
  t1p.dims[R] = t2.dims[C - 1];
  for (int i = 0; i < t1.nqi(); ++i) t1p.qi[i] = t1.qi[i];
  if (R + 1 > 2) t1p.qi[t1p.nqi() - 1] = t1.qc;
  t1p.dual = t1.dual;
  t1p.set_dual(R, !t2.is_dual(C - 1));
  int qc = (C == 1) ? s.vacuum() : (C == 2 ? t2.qu[0] : t2.qi[t2.nqi() - 1]);
  t1p.qc = qc;
  t1p.compute_dim();
  FusionTree t2p;
  t2p.rank = C - 1;
  for (int i = 0; i < C - 1; ++i) { t2p.qu[i] = t2.qu[i]; t2p.dims[i] = t2.dims[i]; t2p.set_dual(i, t2.is_dual(i)); }
  for (int i = 0; i < t2p.nqi(); ++i) t2p.qi[i] = t2.qi[i];
  t2p.qc = qc;
  t2p.compute_dim();
  int a = qc, b = t2.qu[C - 1], c = t2.qc;
  double coeff = s.coeff_turn(a, b, c);
  if (t2.is_dual(C - 1)) coeff *= s.coeff_FS(s.conj(b));
  TreePairMap out;
  if (std::abs(coeff) < kTreeEps) return out;
  out.emplace(std::make_pair(t1p, t2p), coeff);
  return out;
}

static TreePairMap turn_left(const Sym& s, const FusionTree& t1, const FusionTree& t2) {
  TreePairMap out;
  for (const auto& [pr, c] : turn_right(s, t2, t1)) out.emplace(std::make_pair(pr.second, pr.first), c);
  return out;
}

TreePairMap treepair_turn(const Sym& s, int shift, const FusionTree& t1, const FusionTree& t2) {
  // treepair::turn<shift> (treepair.cpp:103-141)
  TreePairMap out;
  if (shift == 0) {
    out.emplace(std::make_pair(t1, t2), 1.0);
    return out;
  }
  if (shift > 0) {
    for (const auto& [pr, c1] : turn_left(s, t1, t2))
      for (const auto& [pr2, c2] : treepair_turn(s, shift - 1, pr.first, pr.second)) out.emplace(pr2, c1 * c2);
    return out;
  }
  for (const auto& [pr, c1] : turn_right(s, t1, t2))
    for (const auto& [pr2, c2] : treepair_turn(s, shift + 1, pr.first, pr.second)) out.emplace(pr2, c1 * c2);
  return out;
}

void treepair_permute_abelian(const Sym& s, int shift, const FusionTree& t1, const FusionTree& t2,
                              const std::vector<int>& p, FusionTree& d, FusionTree& c) {
  // abelian, non-fermionic symmetries: the permuted pair is unique, with coefficient 1
  const int R = t1.rank, C = t2.rank;
  const int newR = R - shift, newC = C + shift;
  d = FusionTree{};
  c = FusionTree{};
  d.rank = newR;
  c.rank = newC;
  for (int r = 0; r < newR; ++r) {
    int src = p[r];
    if (src < R) { d.qu[r] = t1.qu[src]; d.dims[r] = t1.dims[src]; d.set_dual(r, t1.is_dual(src)); }
    else { d.qu[r] = s.conj(t2.qu[src - R]); d.dims[r] = t2.dims[src - R]; d.set_dual(r, !t2.is_dual(src - R)); }
  }
  for (int k = 0; k < newC; ++k) {
    int src = p[k + newR];
    if (src < R) { c.qu[k] = s.conj(t1.qu[src]); c.dims[k] = t1.dims[src]; c.set_dual(k, !t1.is_dual(src)); }
    else { c.qu[k] = t2.qu[src - R]; c.dims[k] = t2.dims[src - R]; c.set_dual(k, t2.is_dual(src - R)); }
  }
  d.qc = s.vacuum();
  c.qc = s.vacuum();
  d.compute_dim();
  c.compute_dim();
  d = tree_compute_intermediates(s, d);
  c = tree_compute_intermediates(s, c);
}

TreePairMap treepair_permute(const Sym& s, int shift, const FusionTree& t1, const FusionTree& t2, const std::vector<int>& p) {
  // treepair::permute<shift> (treepair.cpp:143-217)
  const int R = t1.rank, C = t2.rank;
  const int newR = R - shift, newC = C + shift;
  TreePairMap out;
  if (s.abelian() && !s.fermionic()) {
    FusionTree d, c;
    treepair_permute_abelian(s, shift, t1, t2, p, d, c);
    out.emplace(std::make_pair(d, c), 1.0);
    return out;
  }
  std::vector<int> pi_id(R + C);
  std::iota(pi_id.begin(), pi_id.end(), 0);
  for (int i = 0; i < C; ++i) pi_id[i + R] = (C - 1) - i + R;
  std::vector<int> pi_tmp(R + C), pi_corr(R + C);
  for (int i = 0; i < R + C; ++i) pi_tmp[i] = pi_id[p[i]];
  for (int i = 0; i < newR; ++i) pi_corr[i] = pi_tmp[i];
  for (int i = 0; i < newC; ++i) pi_corr[i + newR] = pi_tmp[(newC - 1) - i + newR];
  const int reshift = C + shift;
  for (const auto& [pr, c1] : treepair_turn(s, -C, t1, t2))
    for (const auto& [t1pp, c2] : tree_permute(s, pr.first, pi_corr))
      for (const auto& [fin, c3] : treepair_turn(s, reshift, t1pp, pr.second)) out[fin] += c1 * c2 * c3;
  return out;
}

// ================================================================ Qbasis
int Qbasis::index(int q) const {
  if (qindex.size() != qs.size()) {
    qindex.clear();
    for (size_t i = 0; i < qs.size(); ++i) qindex[qs[i]] = static_cast<int>(i);
  }
  auto it = qindex.find(q);
  return it == qindex.end() ? -1 : it->second;
}

int64_t Qbasis::dim() const { return std::accumulate(dims.begin(), dims.end(), int64_t(0)); }

int64_t Qbasis::full_dim() const {
  int64_t out = 0;
  for (size_t i = 0; i < qs.size(); ++i) out += dims[i] * sym.deg(qs[i]);
  return out;
}

int64_t Qbasis::full_outer_num(int q) const {
  int64_t out = 0;
  for (size_t i = 0; i < qs.size(); ++i) {
    if (qs[i] == q) return out;
    out += dims[i] * sym.deg(qs[i]);
  }
  return out;
}

int64_t Qbasis::left_offset(const FusionTree& t) const {
  int i = index(t.qc);
  if (i < 0) throw std::runtime_error("left_offset: coupled charge not in basis");
  if (offset_cache.size() != qs.size()) offset_cache.assign(qs.size(), {});
  auto& m = offset_cache[i];
  if (m.empty()) {
    int64_t off = 0;
    for (const auto& tr : trees[i]) {
      m.emplace(tr, off);
      off += tr.dim;
    }
  }
  auto it = m.find(t);
  if (it == m.end()) {
    // the reference returns the total sector size when the tree is absent
    int64_t off = 0;
    for (const auto& tr : trees[i]) off += tr.dim;
    return off;
  }
  return it->second;
}

std::string Qbasis::key() const {
  // binary, not text: combined bases hold thousands of trees and are keyed every time one is built
  size_t n = 16;
  for (const auto& ts : trees) n += 16 + ts.size() * (12 + 12 * kMaxRank);
  std::string k;
  k.reserve(n);
  auto put = [&](int64_t v) { k.append(reinterpret_cast<const char*>(&v), sizeof(v)); };
  put(int64_t(sym.kind));
  put(int64_t(sym.N));
  put(int64_t(depth) * 2 + (conj_flag ? 1 : 0));
  for (size_t i = 0; i < qs.size(); ++i) {
    put(qs[i]);
    put(dims[i]);
    put(int64_t(trees[i].size()));
    for (const auto& t : trees[i]) {
      put((int64_t(t.rank) << 48) ^ (int64_t(t.dual) << 32) ^ int64_t(uint32_t(t.qc)));
      for (int m = 0; m < t.rank; ++m) put((int64_t(t.qu[m]) << 32) ^ int64_t(uint32_t(t.dims[m])));
      for (int m = 0; m < t.nqi(); ++m) put(t.qi[m]);
    }
  }
  return k;
}

namespace {
std::mutex g_mu;
std::unordered_map<std::string, std::shared_ptr<const Qbasis>> g_interned;  // bases are small; ids stay stable
std::map<std::pair<uint64_t, uint64_t>, BasisPtr> g_combine;
std::map<std::vector<uint64_t>, BasisPtr> g_build;
uint64_t g_next_id = 1;
}  // namespace

BasisPtr intern_basis(Qbasis&& b) {
  std::string k = b.key();
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_interned.find(k);
  if (it != g_interned.end()) return it->second;
  b.id = g_next_id++;
  // the lookup caches are complete before the basis is shared: later lookups (from any host thread)
  // only read them
  b.qindex.clear();
  for (size_t i = 0; i < b.qs.size(); ++i) b.qindex[b.qs[i]] = static_cast<int>(i);
  b.offset_cache.assign(b.qs.size(), {});
  for (size_t i = 0; i < b.qs.size(); ++i) {
    int64_t off = 0;
    for (const auto& tr : b.trees[i]) {
      b.offset_cache[i].emplace(tr, off);
      off += tr.dim;
    }
  }
  auto sp = std::make_shared<const Qbasis>(std::move(b));
  g_interned[k] = sp;
  return sp;
}

static void push_back_plain(Qbasis& b, int q, int64_t d) {
  // Qbasis::push_back(q, dim) (Qbasis.cpp:34-73)
  if (d == 0) return;
  for (size_t i = 0; i < b.qs.size(); ++i) {
    if (b.qs[i] == q) {
      b.dims[i] += d;
      b.trees[i][0].dims[0] += static_cast<int32_t>(d);
      b.trees[i][0].compute_dim();
      return;
    }
  }
  FusionTree t;
  if (b.depth == 1) {
    t.rank = 1;
    t.qu[0] = q;
    t.qc = q;
    t.dims[0] = static_cast<int32_t>(d);
    t.set_dual(0, b.conj_flag);
    t.compute_dim();
  } else {
    t.rank = 0;
    t.qc = q;
    t.dim = 1;
  }
  b.qs.push_back(q);
  b.dims.push_back(d);
  b.trees.push_back({t});
}

static void sort_basis(Qbasis& b) {
  // Qbasis::sort (Qbasis.cpp:306-331)
  if (b.qs.size() < 2) return;
  std::vector<int> idx(b.qs.size());
  std::iota(idx.begin(), idx.end(), 0);
  const Sym s = b.sym;
  const bool cj = b.conj_flag;
  std::sort(idx.begin(), idx.end(), [&](int a, int c) {
    return cj ? s.conj(b.qs[a]) < s.conj(b.qs[c]) : b.qs[a] < b.qs[c];
  });
  std::vector<int> qs(idx.size());
  std::vector<int64_t> dims(idx.size());
  std::vector<std::vector<FusionTree>> trees(idx.size());
  for (size_t i = 0; i < idx.size(); ++i) {
    qs[i] = b.qs[idx[i]];
    dims[i] = b.dims[idx[i]];
    trees[i] = std::move(b.trees[idx[i]]);
  }
  b.qs.swap(qs);
  b.dims.swap(dims);
  b.trees.swap(trees);
  b.qindex.clear();  // lookup caches follow the new order when next used
  b.offset_cache.clear();
}

BasisPtr basis_from_pairs(const Sym& s, const std::vector<std::pair<int, int64_t>>& pairs, bool sort) {
  Qbasis b;
  b.sym = s;
  b.depth = 1;
  for (const auto& [q, d] : pairs) push_back_plain(b, q, d);
  if (sort) sort_basis(b);
  return intern_basis(std::move(b));
}

BasisPtr basis_vacuum0(const Sym& s) {
  Qbasis b;
  b.sym = s;
  b.depth = 0;
  push_back_plain(b, s.vacuum(), 1);
  return intern_basis(std::move(b));
}

BasisPtr basis_trivial(const Sym& s) { return basis_from_pairs(s, {{s.vacuum(), 1}}, false); }

BasisPtr basis_conj(const BasisPtr& src) {
  // Qbasis::conj (Qbasis.cpp:418-439)
  Qbasis b;
  b.sym = src->sym;
  b.depth = 1;
  b.conj_flag = !src->conj_flag;
  for (size_t i = 0; i < src->qs.size(); ++i) {
    const FusionTree& old = src->trees[i][0];
    FusionTree t;
    t.rank = 1;
    t.qu[0] = src->sym.conj(src->qs[i]);
    t.qc = t.qu[0];
    t.set_dual(0, !old.is_dual(0));
    t.dims[0] = old.dims[0];
    t.compute_dim();
    b.qs.push_back(t.qc);
    b.dims.push_back(src->dims[i]);
    b.trees.push_back({t});
  }
  sort_basis(b);
  return intern_basis(std::move(b));
}

BasisPtr basis_forget_history(const BasisPtr& src) {
  Qbasis b;
  b.sym = src->sym;
  b.depth = 1;
  for (size_t i = 0; i < src->qs.size(); ++i) push_back_plain(b, src->qs[i], src->dims[i]);
  return intern_basis(std::move(b));
}

BasisPtr basis_combine(const BasisPtr& a, const BasisPtr& bb) {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_combine.find({a->id, bb->id});
    if (it != g_combine.end()) return it->second;
  }
  // Qbasis::combine (Qbasis.cpp:441-495)
  const Sym& s = a->sym;
  // coupled charges in order of first appearance, each with its trees; a tree is the concatenation of
  // its two parents, so distinct parent pairs give distinct trees: only non-abelian symmetries (several
  // channels per pair) keep the membership check of the reference's insertion
  std::vector<int> order;
  std::vector<std::vector<FusionTree>> trees;
  std::unordered_map<int, int> slot;
  std::vector<std::unordered_set<FusionTree, TreeHash>> seen;
  const bool check = !s.abelian();
  int buf[64];
  for (size_t i1 = 0; i1 < a->qs.size(); ++i1) {
    for (size_t i2 = 0; i2 < bb->qs.size(); ++i2) {
      int n = s.combine(a->qs[i1], bb->qs[i2], buf);
      for (int k = 0; k < n; ++k) {
        const int q = buf[k];
        auto [it, fresh] = slot.try_emplace(q, int(order.size()));
        if (fresh) {
          order.push_back(q);
          trees.emplace_back();
          if (check) seen.emplace_back();
        }
        auto& lst = trees[size_t(it->second)];
        lst.reserve(lst.size() + a->trees[i1].size() * bb->trees[i2].size());
        for (const auto& t1 : a->trees[i1])
          for (const auto& t2 : bb->trees[i2]) {
            FusionTree tt = tree_enlarge(t1, t2);
            tt.qc = q;
            if (!check || seen[size_t(it->second)].insert(tt).second) lst.push_back(tt);
          }
      }
    }
  }
  Qbasis out;
  out.sym = s;
  out.depth = a->depth + 1;
  for (size_t o = 0; o < order.size(); ++o) {
    auto& lst = trees[o];
    std::sort(lst.begin(), lst.end(), [](const FusionTree& x, const FusionTree& y) { return x.less(y); });
    int64_t d = 0;
    for (const auto& t : lst) d += t.dim;
    out.qs.push_back(order[o]);
    out.dims.push_back(d);
    out.trees.push_back(std::move(lst));
  }
  sort_basis(out);
  BasisPtr res = intern_basis(std::move(out));
  std::lock_guard<std::mutex> lk(g_mu);
  g_combine[{a->id, bb->id}] = res;
  return res;
}

BasisPtr build_fusion_tree(const Sym& s, const std::vector<BasisPtr>& legs) {
  // internal::build_FusionTree (TensorHelper.cpp:31-44)
  if (legs.empty()) return basis_vacuum0(s);
  std::vector<uint64_t> key;
  for (const auto& b : legs) key.push_back(b->id);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_build.find(key);
    if (it != g_build.end()) return it->second;
  }
  BasisPtr out = legs[0];
  for (size_t i = 1; i < legs.size(); ++i) out = basis_combine(out, legs[i]);
  std::lock_guard<std::mutex> lk(g_mu);
  g_build[key] = out;
  return out;
}

}  // namespace xgb
