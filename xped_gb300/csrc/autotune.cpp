// Tile-shape autotuner of the grouped FP64 block GEMM (no counterpart in the reference, whose
// per-sector loop hands every block to Eigen/BLAS separately: src/Core/TensorBase.cpp:262-279).
//
// A grouped GEMM launch over the sector blocks of one contraction is shaped by two choices:
//  * the output tile edge of gemm_simt_kernel (16, 32 or 64): larger tiles re-use more operand
//    data per CTA, smaller ones spread a short list over more SMs;
//  * split-K: when the output tiles cannot fill the GPU, the k range of every tile is cut so that
//    about `split_waves` x SMs CTAs run, and a fixed-order reduce adds the partial tiles.
// FP64 runs on GB300's narrow DFMA pipe, so which choice wins depends on the block-size histogram
// of the list (how many tiles, how long k is) more than on any single block.  With autotuning on,
// the first list of a size bucket (group count, total flops, largest block area, longest k, all
// on a log2 scale) times every candidate on its own operands (CUDA events on the launching stream,
// output into a scratch buffer) and the fastest is cached for the bucket; later lists of the bucket
// use it without measuring.  The cache can be saved to and loaded from a text file keyed by the
// GPU's name.  With autotuning off the built-in rule of each call site is used (the default, so
// results are reproducible run to run).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "kernels.hpp"

namespace xgb {

namespace {
constexpr int kTiles[] = {16, 32, 64};
constexpr int kWaves[] = {0, 1, 2, 4};
constexpr int kNumCandidates = 12;
constexpr int64_t kMinChunk = 64;  // k per partial tile: a multiple of the kernel's 16-deep k step

struct Key {
  int groups, flops, area, k;
  int tc;  // 1: the FP64-accurate tensor-core form is among the candidates
  bool operator<(const Key& o) const {
    if (groups != o.groups) return groups < o.groups;
    if (flops != o.flops) return flops < o.flops;
    if (area != o.area) return area < o.area;
    if (k != o.k) return k < o.k;
    return tc < o.tc;
  }
};

std::mutex g_mu;
int g_mode = 0;  // 0 off, 1 on (measure unseen buckets), 2 frozen (cached choices only)
std::map<Key, F64Config> g_cache;
int64_t g_tuned = 0, g_hits = 0;
double g_tune_ms = 0.0;

int ilog2_ceil(double x) { return x <= 1.0 ? 0 : int(std::ceil(std::log2(x))); }

Key key_of(const xgb_gemm_desc* d, int n) {
  double flops = 0, area = 0, k = 0;
  for (int g = 0; g < n; ++g) {
    flops += 2.0 * double(d[g].m) * double(d[g].n) * double(d[g].k);
    area = std::max(area, double(d[g].m) * double(d[g].n));
    k = std::max(k, double(d[g].k));
  }
  return {ilog2_ceil(n), ilog2_ceil(flops), ilog2_ceil(area) / 2, ilog2_ceil(k), 0};
}

std::string gpu_name() {
  int dev = 0;
  cudaDeviceProp p{};
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "unknown";
  std::string s(p.name);
  for (char& c : s)
    if (c == ' ' || c == '|') c = '_';
  return s;
}

template <class T>
T* stage(const std::vector<T>& v, cudaStream_t s) {
  T* d = static_cast<T*>(dev_alloc(sizeof(T) * std::max<size_t>(v.size(), 1)));
  if (!v.empty()) cudaMemcpyAsync(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s);
  return d;
}
}  // namespace

F64Config f64_candidate(int idx) { return {kTiles[idx / 4], kWaves[idx % 4]}; }
int f64_candidate_count() { return kNumCandidates; }

F64Plan plan_gemm_f64(const xgb_gemm_desc* d, int n, F64Config c, int shape) {
  F64Plan p;
  p.tile = c.tile;
  const int tile = c.tile;
  auto keep = [&](int64_t x, int64_t y) { return shape != kGemmSymUpper || x <= y; };
  auto kmax = [&](int g, int64_t y) {
    return shape == kGemmTriB ? std::min<int64_t>(d[g].k, (y + 1) * tile) : d[g].k;
  };
  int64_t n_out = 0;
  for (int g = 0; g < n; ++g) {
    const int64_t tm = (d[g].m + tile - 1) / tile, tn = (d[g].n + tile - 1) / tile;
    for (int64_t y = 0; y < tn; ++y)
      for (int64_t x = 0; x < tm; ++x) n_out += keep(x, y);
  }
  const int64_t target = int64_t(c.split_waves) * int64_t(num_sms() > 0 ? num_sms() : 152);
  const int64_t want = (c.split_waves > 0 && n_out > 0) ? (target + n_out - 1) / n_out : 1;
  for (int g = 0; g < n; ++g) {
    const int64_t tm = (d[g].m + tile - 1) / tile, tn = (d[g].n + tile - 1) / tile;
    for (int64_t y = 0; y < tn; ++y) {
      const int64_t kk = kmax(g, y);
      const int64_t splits = std::max<int64_t>(1, std::min<int64_t>(want, kk / kMinChunk));
      const int64_t chunk = splits > 1 ? (((kk + splits - 1) / splits + 15) / 16) * 16 : kk;
      for (int64_t x = 0; x < tm; ++x) {
        if (!keep(x, y)) continue;
        if (splits == 1) {
          if (kk == d[g].k) p.tiles.push_back({int32_t(g), int32_t(x), int32_t(y), tile});
          else p.tiles.push_back({int32_t(g), int32_t(x), int32_t(y), tile, 0, int32_t(kk)});
          continue;
        }
        const int32_t first = p.slots;
        for (int64_t k0 = 0; k0 < kk; k0 += chunk)
          p.tiles.push_back({int32_t(g), int32_t(x), int32_t(y), tile, int32_t(k0),
                             int32_t(std::min<int64_t>(k0 + chunk, kk)), p.slots++});
        p.red.push_back({int32_t(g), int32_t(x), int32_t(y), first, p.slots - first, 0});
      }
    }
  }
  order_tiles_by_work(p.tiles, d);
  return p;
}

void run_f64_plan(const F64Plan& p, const xgb_gemm_desc* d_descs, const GemmTile* d_tiles, const SplitReduce* d_red,
                  const double* A, const double* B, double* C, double alpha, double beta, cudaStream_t s) {
  if (p.tiles.empty()) return;
  if (p.red.empty()) {
    launch_gemm_f64(d_descs, d_tiles, int(p.tiles.size()), p.tile, A, B, C, alpha, beta, s);
    return;
  }
  auto* ws = static_cast<double*>(dev_alloc(sizeof(double) * size_t(p.slots) * size_t(p.tile) * size_t(p.tile)));
  launch_gemm_f64_splitk(d_descs, d_tiles, int(p.tiles.size()), p.tile, d_red, int(p.red.size()), A, B, C, ws, alpha,
                         beta, s);
  dev_free(ws);
}

void run_gemm_f64_config(const xgb_gemm_desc* h_descs, int n, F64Config c, const double* A, const double* B, double* C,
                         double alpha, double beta, cudaStream_t s) {
  if (n <= 0) return;
  const F64Plan p = plan_gemm_f64(h_descs, n, c);
  std::vector<xgb_gemm_desc> dv(h_descs, h_descs + n);
  auto* dd = stage(dv, s);
  auto* dt = stage(p.tiles, s);
  auto* dr = stage(p.red, s);
  run_f64_plan(p, dd, dt, dr, A, B, C, alpha, beta, s);
  dev_free(dd);
  dev_free(dt);
  dev_free(dr);
}

// times every CUDA-core candidate (and, with allow_tc, the tensor-core form as index kNumCandidates);
// returns the index of the fastest
int tune_gemm_f64(const xgb_gemm_desc* d, int n, const double* A, const double* B, cudaStream_t s, double* times_ms,
                  bool allow_tc = false) {
  // scratch output covering every block's C range; the candidates write there with beta = 0
  int64_t extent = 1;
  for (int g = 0; g < n; ++g)
    if (d[g].m > 0 && d[g].n > 0) extent = std::max(extent, d[g].c_off + (d[g].n - 1) * d[g].ldc + d[g].m);
  auto* scratch = static_cast<double*>(dev_alloc(sizeof(double) * size_t(extent)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  std::vector<xgb_gemm_desc> dv(d, d + n);
  auto* dd = stage(dv, s);
  int best = 0;
  for (int c = 0; c < kNumCandidates; ++c) {
    // tables staged once per candidate; only the launches (and the stream-ordered split-K
    // workspace) are inside the timed region
    const F64Plan p = plan_gemm_f64(d, n, f64_candidate(c));
    auto* dt = stage(p.tiles, s);
    auto* dr = stage(p.red, s);
    run_f64_plan(p, dd, dt, dr, A, B, scratch, 1.0, 0.0, s);  // warm-up
    float best_ms = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, s);
      run_f64_plan(p, dd, dt, dr, A, B, scratch, 1.0, 0.0, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best_ms = std::min(best_ms, ms);
    }
    dev_free(dt);
    dev_free(dr);
    times_ms[c] = best_ms;
  }
  // the fastest, except that a candidate within 3 % of it with a larger tile (then fewer split waves)
  // wins: FP64-bound lists time alike on every tile edge, and larger tiles mean shorter launch tables
  // to build whenever a step brings new shapes
  for (int c = 1; c < kNumCandidates; ++c)
    if (times_ms[c] < times_ms[best]) best = c;
  const double near = 1.03 * times_ms[best];
  for (int c = kNumCandidates - 1; c >= 0; --c)
    if (times_ms[c] <= near) {
      const bool larger = kTiles[c / 4] > kTiles[best / 4];
      const bool fewer = kTiles[c / 4] == kTiles[best / 4] && kWaves[c % 4] < kWaves[best % 4];
      if (larger || fewer) best = c;
    }
  if (allow_tc) {
    // like the CUDA-core candidates, and like a matmul whose plan is cached: the slicing plan is built
    // and its tables staged before the timed region; the launches and their stream-ordered scratch
    // (row scales, slices, split-K partials) are inside it
    const OzPlanHost op = build_oz_plan(d, n);
    auto* dg = stage(op.groups, s);
    auto* dk = stage(op.tasks, s);
    auto* dt = stage(op.tiles, s);
    auto* dr = stage(op.red, s);
    auto run_oz = [&]() {
      if (op.tiles.empty()) return;
      auto* rm = static_cast<unsigned long long*>(
          dev_alloc(sizeof(unsigned long long) * size_t(std::max<int64_t>(op.rowmax, 1))));
      auto* ap = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(op.a_bytes, 16))));
      auto* bp = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(op.b_bytes, 16))));
      launch_gemm_oz(dd, dg, dk, int(op.tasks.size()), dt, int(op.tiles.size()), dr, int(op.red.size()), op.slots,
                     A, B, rm, op.rowmax, ap, bp, scratch, 1.0, 0.0, s);
      dev_free(rm);
      dev_free(ap);
      dev_free(bp);
    };
    run_oz();  // warm-up
    float best_ms = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, s);
      run_oz();
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best_ms = std::min(best_ms, ms);
    }
    dev_free(dg);
    dev_free(dk);
    dev_free(dt);
    dev_free(dr);
    times_ms[kNumCandidates] = best_ms;
    if (times_ms[kNumCandidates] < times_ms[best]) best = kNumCandidates;
  }
  dev_free(dd);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dev_free(scratch);
  return best;
}

F64Config gemm_f64_config(const xgb_gemm_desc* d, int n, const double* A, const double* B, F64Config fallback,
                          cudaStream_t s, bool allow_tc) {
  Key k;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_mode == 0 || n <= 0) return fallback;
    k = key_of(d, n);
    k.tc = allow_tc ? 1 : 0;
    auto it = g_cache.find(k);
    if (it != g_cache.end()) {
      ++g_hits;
      return it->second;
    }
    if (g_mode == 2) return fallback;  // frozen: no measurement, the built-in rule for unseen buckets
  }
  double times[kNumCandidates + 1];
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, s);
  const int best = tune_gemm_f64(d, n, A, B, s, times, allow_tc);
  cudaEventRecord(t1, s);
  cudaEventSynchronize(t1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  std::lock_guard<std::mutex> lk(g_mu);
  if (best == kNumCandidates) {
    F64Config c = fallback;
    c.tc = true;
    g_cache[k] = c;
  } else {
    g_cache[k] = f64_candidate(best);
  }
  ++g_tuned;
  g_tune_ms += ms;
  return g_cache[k];
}

void autotune_set_mode(int mode) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_mode = mode;
}

int autotune_mode() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_mode;
}

}  // namespace xgb

using namespace xgb;

extern "C" {

int xgb_autotune_set(int mode) {
  if (mode < 0 || mode > 2) return set_error(XGB_E_BADPLAN, "autotune mode must be 0 (off), 1 (on) or 2 (frozen)");
  autotune_set_mode(mode);
  return XGB_OK;
}

int xgb_autotune_reset(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_cache.clear();
  g_tuned = g_hits = 0;
  g_tune_ms = 0.0;
  return XGB_OK;
}

int xgb_autotune_stats(int64_t* buckets, int64_t* hits, double* tune_ms) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (buckets) *buckets = g_tuned;
  if (hits) *hits = g_hits;
  if (tune_ms) *tune_ms = g_tune_ms;
  return int(g_cache.size());
}

int xgb_autotune_candidates(int32_t* tile, int32_t* split_waves, int cap) {
  const int n = std::min(cap, kNumCandidates);
  for (int i = 0; i < n; ++i) {
    const F64Config c = f64_candidate(i);
    if (tile) tile[i] = c.tile;
    if (split_waves) split_waves[i] = c.split_waves;
  }
  return kNumCandidates;
}

int xgb_autotune_choices(int32_t* tile, int32_t* split_waves, int cap) {
  std::lock_guard<std::mutex> lk(g_mu);
  int i = 0;
  for (const auto& kv : g_cache) {
    if (i >= cap) break;
    if (tile) tile[i] = kv.second.tc ? 0 : kv.second.tile;  // 0: the FP64-accurate tensor-core form
    if (split_waves) split_waves[i] = kv.second.split_waves;
    ++i;
  }
  return int(g_cache.size());
}

int xgb_autotune_gemm(int n, const xgb_gemm_desc* descs, const double* A, const double* B, double* times_ms,
                      int32_t* best) {
  if (!runtime_ready()) return set_error(XGB_E_NOINIT, "xgb_init was not called");
  if (n <= 0 || !descs) return set_error(XGB_E_BADPLAN, "autotune needs a non-empty GEMM list");
  try {
    double t[kNumCandidates];
    const int b = tune_gemm_f64(descs, n, A, B, stream(), t);
    if (times_ms) std::copy(t, t + kNumCandidates, times_ms);
    if (best) *best = b;
    return check_cuda(cudaGetLastError(), "autotune launch");
  } catch (const std::bad_alloc&) {
    return XGB_E_OOM;
  } catch (const std::exception& ex) {
    return set_error(XGB_E_BADPLAN, ex.what());
  }
}

int xgb_grouped_gemm_f64_config(int tile, int split_waves, int n, const xgb_gemm_desc* descs, const double* A,
                                const double* B, double* C, double alpha, double beta, void* stream_) {
  if (!runtime_ready()) return set_error(XGB_E_NOINIT, "xgb_init was not called");
  if (tile != 16 && tile != 32 && tile != 64) return set_error(XGB_E_BADPLAN, "tile edge must be 16, 32 or 64");
  if (split_waves < 0 || split_waves > 16) return set_error(XGB_E_BADPLAN, "split_waves out of range");
  try {
    for (int g = 0; g < n; ++g)
      if (descs[g].m < 0 || descs[g].n < 0 || descs[g].k < 0) return set_error(XGB_E_BADPLAN, "negative GEMM extent");
    run_gemm_f64_config(descs, n, {tile, split_waves}, A, B, C, alpha, beta,
                        stream_ ? static_cast<cudaStream_t>(stream_) : stream());
    return check_cuda(cudaGetLastError(), "gemm launch");
  } catch (const std::bad_alloc&) {
    return XGB_E_OOM;
  } catch (const std::exception& ex) {
    return set_error(XGB_E_BADPLAN, ex.what());
  }
}

int xgb_autotune_save(const char* path) {
  if (!path) return set_error(XGB_E_BADPLAN, "no path");
  std::lock_guard<std::mutex> lk(g_mu);
  std::ofstream f(path, std::ios::trunc);
  if (!f) return set_error(XGB_E_BADPLAN, std::string("cannot write ") + path);
  const std::string gpu = gpu_name();
  for (const auto& kv : g_cache)
    f << gpu << ' ' << kv.first.groups << ' ' << kv.first.flops << ' ' << kv.first.area << ' ' << kv.first.k << ' '
      << kv.first.tc << ' ' << kv.second.tile << ' ' << kv.second.split_waves << ' ' << (kv.second.tc ? 1 : 0) << '\n';
  return f.good() ? XGB_OK : set_error(XGB_E_BADPLAN, std::string("write failed: ") + path);
}

int xgb_autotune_load(const char* path) {
  if (!path) return set_error(XGB_E_BADPLAN, "no path");
  std::ifstream f(path);
  if (!f) return set_error(XGB_E_BADPLAN, std::string("cannot read ") + path);
  const std::string gpu = gpu_name();
  std::lock_guard<std::mutex> lk(g_mu);
  std::string line;
  int loaded = 0;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    std::string name;
    Key k{};
    F64Config c{};
    int ctc = 0;
    if (!(is >> name >> k.groups >> k.flops >> k.area >> k.k >> k.tc >> c.tile >> c.split_waves >> ctc)) continue;
    c.tc = ctc != 0;
    if (name != gpu) continue;  // entries measured on another GPU model do not apply
    if (c.tile != 16 && c.tile != 32 && c.tile != 64) continue;
    g_cache[k] = c;
    ++loaded;
  }
  return loaded;
}

}  // extern "C"
