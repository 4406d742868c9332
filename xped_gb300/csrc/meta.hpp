// Host-side symmetric-tensor metadata: symmetry algebra, fusion trees, leg
// bases and their tensor products.  Everything here is integer bookkeeping
// plus recoupling coefficients; it must reproduce the reference's sector,
// tree and offset order bit for bit because it decides where every block
// lives in device memory.
//
// Reference (paths relative to the Xped source tree):
//   symmetries   include/Xped/Symmetry/{U1,ZN,SU2,SymBase}.hpp, src/Symmetry/SU2.cpp
//   FusionTree   include/Xped/Core/FusionTree.hpp, src/Core/FusionTree.cpp
//   Qbasis       include/Xped/Core/Qbasis.hpp, src/Core/Qbasis.cpp
//   treepair     src/Core/treepair.cpp
//   Permutation  include/Xped/Util/Permutations.hpp:195-225
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

namespace xgb {

constexpr int kMaxRank = 8;  // legs per tensor side and in total

// ---------------------------------------------------------------- symmetry
enum SymKind : int { SYM_U1 = 0, SYM_U1_FERMIONIC = 1, SYM_Z2 = 2, SYM_Z2_FERMIONIC = 3, SYM_SU2 = 4 };

struct Sym {
  int kind = SYM_U1;
  int N = 2;  // modulus for Z(N)

  bool abelian() const { return kind != SYM_SU2; }
  bool fermionic() const { return kind == SYM_U1_FERMIONIC || kind == SYM_Z2_FERMIONIC; }
  bool modular() const { return kind == SYM_Z2 || kind == SYM_Z2_FERMIONIC; }
  int vacuum() const { return kind == SYM_SU2 ? 1 : 0; }
  int conj(int q) const;
  int deg(int q) const { return kind == SYM_SU2 ? q : 1; }
  // Irreps of ql (x) qr in the reference's order (U1.hpp:189-194, ZN.hpp:199-205, SU2.cpp:17-27).
  int combine(int ql, int qr, int* out) const;  // returns count (<= 64)
  int combine1(int ql, int qr) const { int o[64]; combine(ql, qr, o); return o[0]; }
  bool triangle(int q1, int q2, int q3) const;
  double coeff_swap(int ql, int qr, int qf) const;
  double coeff_recouple(int q1, int q2, int q3, int Q, int Q12, int Q23) const;
  double coeff_turn(int ql, int qr, int qf) const;
  double coeff_FS(int q) const;
  double coeff_twist(int q) const;
  double coeff_6j(int q1, int q2, int q3, int q4, int q5, int q6) const;
  bool operator==(const Sym& o) const { return kind == o.kind && N == o.N; }
};

// Wigner 6j from doubled spins (Racah's closed form); replaces GSL's
// gsl_sf_coupling_6j used by the reference (SU2Wrappers.hpp:73-76).
double wigner6j_twice(int a2, int b2, int c2, int d2, int e2, int f2);

// ------------------------------------------------------------- fusion tree
struct FusionTree {
  int8_t rank = 0;
  int32_t qc = 0;
  std::array<int32_t, kMaxRank> qu{};
  std::array<int32_t, kMaxRank> qi{};    // rank-2 entries used
  std::array<int32_t, kMaxRank> dims{};
  uint16_t dual = 0;                     // IS_DUAL bitmask (not part of equality)
  int64_t dim = 1;

  int nqi() const { return rank >= 2 ? rank - 2 : 0; }
  void compute_dim();
  // FusionTree::operator== without XPED_PEDANTIC_ASSERTS (FusionTree.cpp:66-85)
  bool operator==(const FusionTree& o) const;
  bool operator!=(const FusionTree& o) const { return !(*this == o); }
  // FusionTree::operator< (FusionTree.cpp:32-64)
  bool less(const FusionTree& o) const;
  size_t hash() const;
  bool is_dual(int i) const { return (dual >> i) & 1; }
  void set_dual(int i, bool v) { dual = v ? (dual | (1u << i)) : (dual & ~(1u << i)); }
};

struct TreeHash { size_t operator()(const FusionTree& t) const { return t.hash(); } };
using TreeMap = std::unordered_map<FusionTree, double, TreeHash>;

struct PairHash {
  size_t operator()(const std::pair<FusionTree, FusionTree>& p) const { return p.first.hash() * 1000003u ^ p.second.hash(); }
};
using TreePairMap = std::unordered_map<std::pair<FusionTree, FusionTree>, double, PairHash>;

FusionTree tree_enlarge(const FusionTree& t, const FusionTree& other);
FusionTree tree_compute_intermediates(const Sym& s, FusionTree t);
TreeMap tree_swap(const Sym& s, const FusionTree& t, int pos);
TreeMap tree_permute(const Sym& s, const FusionTree& t, const std::vector<int>& p);
std::vector<int> decompose_permutation(const std::vector<int>& pi);
TreePairMap treepair_turn(const Sym& s, int shift, const FusionTree& t1, const FusionTree& t2);
TreePairMap treepair_permute(const Sym& s, int shift, const FusionTree& t1, const FusionTree& t2, const std::vector<int>& p);
// the same for abelian, non-fermionic symmetries (one result pair, coefficient 1), without a map
void treepair_permute_abelian(const Sym& s, int shift, const FusionTree& t1, const FusionTree& t2,
                              const std::vector<int>& p, FusionTree& d, FusionTree& c);

// ------------------------------------------------------------------ Qbasis
struct Qbasis;
using BasisPtr = std::shared_ptr<const Qbasis>;

struct Qbasis {
  Sym sym;
  int depth = 1;
  bool conj_flag = false;
  std::vector<int> qs;                           // storage order
  std::vector<int64_t> dims;                     // inner dims
  std::vector<std::vector<FusionTree>> trees;    // parallel to qs (sorted)
  uint64_t id = 0;                               // interned identity

  int index(int q) const;                        // -1 if absent
  int64_t inner_dim(int q) const { int i = index(q); return i < 0 ? 0 : dims[i]; }
  int64_t dim() const;
  int64_t full_dim() const;
  int64_t full_outer_num(int q) const;
  // Qbasis::leftOffset (Qbasis.cpp:208-225): row offset of a tree in its sector.
  int64_t left_offset(const FusionTree& t) const;
  std::string key() const;

  // lazily built tree -> offset lookup
  mutable std::vector<std::unordered_map<FusionTree, int64_t, TreeHash>> offset_cache;
  mutable std::unordered_map<int, int> qindex;
};

// Builders that mirror the reference; every result is interned.
BasisPtr basis_from_pairs(const Sym& s, const std::vector<std::pair<int, int64_t>>& pairs, bool sort);
BasisPtr basis_conj(const BasisPtr& b);
BasisPtr basis_forget_history(const BasisPtr& b);
BasisPtr basis_combine(const BasisPtr& a, const BasisPtr& b);
BasisPtr basis_vacuum0(const Sym& s);
BasisPtr basis_trivial(const Sym& s);
BasisPtr build_fusion_tree(const Sym& s, const std::vector<BasisPtr>& legs);
BasisPtr intern_basis(Qbasis&& b);

}  // namespace xgb
