// Checkpoints of device tensors and CTM environments: the fields the reference
// serialises for a tensor (StorageType_contiguous::serialize,
// include/Xped/Core/storage/StorageType_contiguous.hpp:191-204: data, sectors,
// uncoupled domain / codomain bases, offsets) and for a CTM (CTM::serialize,
// include/Xped/PEPS/CTM.hpp:184-204: chi and the corner / edge tensors), written
// little-endian into one byte buffer of this library's own layout.  The
// reference writes them through the yas library, which is not part of its
// source tree, so byte compatibility with its archives is not claimed.
//
// Tensor layout: "XGBT" | u32 version | i32 symmetry kind | i32 N | i32 rank |
// i32 corank | per leg: i32 depth (1) | i32 conj | i32 n | n x (i32 q, i64 dim)
// in storage order | u64 sectors | per sector: i32 q, i64 rows, i64 cols |
// u64 size | size x f64 (column-major blocks at the storage offsets).
// CTM layout: "XGBC" | u32 version | i64 chi | 8 tensors (C1..C4, T1..T4),
// each as u64 byte count + tensor layout.
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "kernels.hpp"
#include "tensor.hpp"

namespace xgb {
namespace {

constexpr uint32_t kVersion = 1;

struct Writer {
  std::vector<uint8_t> out;
  template <class T>
  void put(T v) {
    const size_t o = out.size();
    out.resize(o + sizeof(T));
    std::memcpy(out.data() + o, &v, sizeof(T));
  }
  void bytes(const void* p, size_t n) {
    const size_t o = out.size();
    out.resize(o + n);
    if (n) std::memcpy(out.data() + o, p, n);
  }
};

struct Reader {
  const uint8_t* p;
  size_t n, at = 0;
  template <class T>
  T get() {
    if (at + sizeof(T) > n) throw std::runtime_error("checkpoint: truncated buffer");
    T v;
    std::memcpy(&v, p + at, sizeof(T));
    at += sizeof(T);
    return v;
  }
  const uint8_t* take(size_t k) {
    if (at + k > n) throw std::runtime_error("checkpoint: truncated buffer");
    const uint8_t* r = p + at;
    at += k;
    return r;
  }
};

void put_basis(Writer& w, const BasisPtr& b) {
  if (b->depth != 1) throw std::runtime_error("checkpoint: only plain (depth-1) leg bases are supported");
  w.put<int32_t>(b->depth);
  w.put<int32_t>(b->conj_flag ? 1 : 0);
  w.put<int32_t>(int32_t(b->qs.size()));
  for (size_t i = 0; i < b->qs.size(); ++i) {
    w.put<int32_t>(b->qs[i]);
    w.put<int64_t>(b->dims[i]);
  }
}

BasisPtr get_basis(Reader& r, const Sym& s) {
  const int32_t depth = r.get<int32_t>(), conj = r.get<int32_t>(), n = r.get<int32_t>();
  if (depth != 1 || n < 0) throw std::runtime_error("checkpoint: unsupported leg basis");
  std::vector<std::pair<int, int64_t>> pairs(static_cast<size_t>(n));
  for (auto& [q, d] : pairs) {
    q = r.get<int32_t>();
    d = r.get<int64_t>();
  }
  BasisPtr b;
  if (conj) {  // Qbasis::conj of the plain basis with the conjugate charges
    std::vector<std::pair<int, int64_t>> orig;
    for (const auto& [q, d] : pairs) orig.push_back({s.conj(q), d});
    b = basis_conj(basis_from_pairs(s, orig, false));
  } else {
    b = basis_from_pairs(s, pairs, false);
  }
  if (b->qs.size() != pairs.size()) throw std::runtime_error("checkpoint: leg basis does not rebuild");
  for (size_t i = 0; i < pairs.size(); ++i)
    if (b->qs[i] != pairs[i].first || b->dims[i] != pairs[i].second)
      throw std::runtime_error("checkpoint: leg basis does not rebuild");
  return b;
}

}  // namespace

std::vector<uint8_t> serialize_tensor(const Tensor& t0) {
  Tensor t = materialize(t0);
  const TensorMeta& m = *t.meta;
  Writer w;
  w.bytes("XGBT", 4);
  w.put<uint32_t>(kVersion);
  w.put<int32_t>(m.sym.kind);
  w.put<int32_t>(m.sym.N);
  w.put<int32_t>(m.rank());
  w.put<int32_t>(m.corank());
  for (const auto& b : m.dom) put_basis(w, b);
  for (const auto& b : m.cod) put_basis(w, b);
  w.put<uint64_t>(m.sectors.size());
  for (size_t i = 0; i < m.sectors.size(); ++i) {
    w.put<int32_t>(m.sectors[i]);
    w.put<int64_t>(m.rows[i]);
    w.put<int64_t>(m.cols[i]);
  }
  w.put<uint64_t>(uint64_t(m.size));
  std::vector<double> host(size_t(m.size));
  if (m.size) {
    cudaError_t e = cudaMemcpyAsync(host.data(), t.data(), sizeof(double) * size_t(m.size), cudaMemcpyDeviceToHost,
                                    stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
    if (e != cudaSuccess) throw std::runtime_error(std::string("checkpoint: download: ") + cudaGetErrorString(e));
  }
  w.bytes(host.data(), sizeof(double) * host.size());
  return std::move(w.out);
}

static Tensor read_tensor(Reader& r) {
  const uint8_t* magic = r.take(4);
  if (std::memcmp(magic, "XGBT", 4) != 0) throw std::runtime_error("checkpoint: not a tensor record");
  if (r.get<uint32_t>() != kVersion) throw std::runtime_error("checkpoint: unknown version");
  Sym s;
  s.kind = r.get<int32_t>();
  s.N = r.get<int32_t>();
  if (s.kind < SYM_U1 || s.kind > SYM_SU2) throw std::runtime_error("checkpoint: unknown symmetry");
  const int32_t rank = r.get<int32_t>(), corank = r.get<int32_t>();
  if (rank < 0 || corank < 0 || rank + corank > 8) throw std::runtime_error("checkpoint: bad rank");
  std::vector<BasisPtr> dom, cod;
  for (int i = 0; i < rank; ++i) dom.push_back(get_basis(r, s));
  for (int i = 0; i < corank; ++i) cod.push_back(get_basis(r, s));
  const uint64_t ns = r.get<uint64_t>();
  if (ns > (uint64_t(1) << 24)) throw std::runtime_error("checkpoint: bad sector count");
  std::vector<int> sectors(ns);
  std::vector<int64_t> rows(ns), cols(ns);
  for (uint64_t i = 0; i < ns; ++i) {
    sectors[i] = r.get<int32_t>();
    rows[i] = r.get<int64_t>();
    cols[i] = r.get<int64_t>();
  }
  MetaPtr meta = make_meta(s, dom, cod);
  if (meta->sectors != sectors) meta = make_meta_ordered(s, dom, cod, sectors);  // push_back order
  if (meta->sectors != sectors) throw std::runtime_error("checkpoint: sectors do not match the leg bases");
  for (uint64_t i = 0; i < ns; ++i)
    if (meta->rows[i] != rows[i] || meta->cols[i] != cols[i])
      throw std::runtime_error("checkpoint: block shapes do not match the leg bases");
  const uint64_t size = r.get<uint64_t>();
  if (int64_t(size) != meta->size) throw std::runtime_error("checkpoint: data size does not match");
  const uint8_t* data = r.take(sizeof(double) * size);
  Tensor t = empty_like_meta(meta);
  if (size) {
    cudaError_t e = cudaMemcpyAsync(t.data(), data, sizeof(double) * size, cudaMemcpyHostToDevice, stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
    if (e != cudaSuccess) throw std::runtime_error(std::string("checkpoint: upload: ") + cudaGetErrorString(e));
  }
  return t;
}

Tensor deserialize_tensor(const uint8_t* p, size_t n) {
  Reader r{p, n};
  Tensor t = read_tensor(r);
  if (r.at != n) throw std::runtime_error("checkpoint: trailing bytes");
  return t;
}

std::vector<uint8_t> serialize_ctm(CTM& c) {
  Writer w;
  w.bytes("XGBC", 4);
  w.put<uint32_t>(kVersion);
  w.put<int64_t>(c.chi);
  for (int k = 0; k < 8; ++k) {
    if (!c.slot(k).valid()) throw std::runtime_error("checkpoint: CTM environment not initialised");
    std::vector<uint8_t> t = serialize_tensor(c.slot(k));
    w.put<uint64_t>(t.size());
    w.bytes(t.data(), t.size());
  }
  return std::move(w.out);
}

std::unique_ptr<CTM> deserialize_ctm(const Tensor& A, const uint8_t* p, size_t n) {
  Reader r{p, n};
  const uint8_t* magic = r.take(4);
  if (std::memcmp(magic, "XGBC", 4) != 0) throw std::runtime_error("checkpoint: not a CTM record");
  if (r.get<uint32_t>() != kVersion) throw std::runtime_error("checkpoint: unknown version");
  const int64_t chi = r.get<int64_t>();
  if (chi <= 0) throw std::runtime_error("checkpoint: bad chi");
  auto c = std::make_unique<CTM>(A, chi);
  for (int k = 0; k < 8; ++k) {
    const uint64_t len = r.get<uint64_t>();
    Reader sub{r.take(size_t(len)), size_t(len)};
    c->slot(k) = read_tensor(sub);
    if (sub.at != sub.n) throw std::runtime_error("checkpoint: trailing bytes in a tensor record");
  }
  if (r.at != n) throw std::runtime_error("checkpoint: trailing bytes");
  return c;
}

}  // namespace xgb
