// CUDA kernels of the GB300 block-sparse tensor backend (sm_103a) and the
// kernel-level C-ABI declared in include/xgb.h.
//
// Data layout: one flat column-major FP64 buffer per tensor, one block per
// coupled sector at a known element offset (the reference's contiguous
// storage, include/Xped/Core/storage/StorageType_contiguous.hpp:79-122).
// Every kernel processes all sectors of one tensor operation in a single
// launch driven by a descriptor table.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <map>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <new>
#include <string>
#include <vector>

#include "kernels.hpp"

namespace xgb {

// ======================================================================= runtime
namespace {
struct Runtime {
  bool ready = false;
  int device = 0;
  int sms = 152;
  cudaStream_t stream = nullptr;  // lane 0
  double* scratch = nullptr;      // 64 doubles of device scratch per lane
  cudaStream_t side[kLanes - 1] = {nullptr, nullptr};
  double* side_scratch[kLanes - 1] = {nullptr, nullptr};
  cudaEvent_t fork_ev = nullptr, join_ev[kLanes - 1] = {nullptr, nullptr};
};
Runtime g_rt;
std::atomic<int64_t> g_launches{0};
std::atomic<bool> g_lanes_used{false};
thread_local std::string g_err;
thread_local int t_lane = 0;

// The worker host thread of lane 1: runs one task at a time, handed over under a mutex.
class LaneWorker {
 public:
  ~LaneWorker() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    if (th_.joinable()) th_.join();
  }
  void start(std::function<void()> f) {
    std::lock_guard<std::mutex> lk(mu_);
    if (!th_.joinable()) th_ = std::thread([this] { loop(); });
    task_ = std::move(f);
    err_ = nullptr;
    has_ = true;
    done_ = false;
    cv_.notify_all();
  }
  void wait() {
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [this] { return done_; });
    if (err_) {
      std::exception_ptr e = err_;
      err_ = nullptr;
      std::rethrow_exception(e);
    }
  }

 private:
  void loop() {
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      cv_.wait(lk, [this] { return stop_ || has_; });
      if (stop_) return;
      std::function<void()> f = std::move(task_);
      has_ = false;
      lk.unlock();
      std::exception_ptr e;
      try {
        cudaSetDevice(g_rt.device);  // the current device is per host thread
        f();
      } catch (...) {
        e = std::current_exception();
      }
      lk.lock();
      err_ = e;
      done_ = true;
      cv_.notify_all();
    }
  }
  std::mutex mu_;
  std::condition_variable cv_;
  std::thread th_;
  std::function<void()> task_;
  std::exception_ptr err_;
  bool has_ = false, done_ = true, stop_ = false;
};

LaneWorker& lane_worker() {
  static LaneWorker w;
  return w;
}
std::mutex g_pair_mu;  // one fork-join section at a time
}  // namespace

cudaStream_t stream() { return t_lane == 0 ? g_rt.stream : g_rt.side[t_lane - 1]; }
int lane() { return t_lane; }
LaneScope::LaneScope(int l) : saved(t_lane) { t_lane = l; }
LaneScope::~LaneScope() { t_lane = saved; }
bool lanes_used() { return g_lanes_used.load(); }
bool runtime_ready() { return g_rt.ready; }
int num_sms() { return g_rt.sms; }
double* scalar_scratch() { return t_lane == 0 ? g_rt.scratch : g_rt.side_scratch[t_lane - 1]; }
void count_launch(int n) { g_launches += n; }

void run_pair(const std::function<void()>& a, const std::function<void()>& b) {
  if (t_lane != 0) throw std::runtime_error("run_pair: called from a side lane");
  std::lock_guard<std::mutex> lk(g_pair_mu);
  g_lanes_used = true;
  if (cudaEventRecord(g_rt.fork_ev, g_rt.stream) != cudaSuccess ||
      cudaStreamWaitEvent(g_rt.side[0], g_rt.fork_ev, 0) != cudaSuccess ||
      cudaStreamWaitEvent(g_rt.side[1], g_rt.fork_ev, 0) != cudaSuccess)
    throw std::runtime_error("run_pair: fork failed");
  LaneWorker& w = lane_worker();
  w.start([&a] {
    LaneScope ls(1);
    a();
  });
  std::exception_ptr eb, ea;
  try {
    LaneScope ls(2);
    b();
  } catch (...) {
    eb = std::current_exception();
  }
  try {
    w.wait();
  } catch (...) {
    ea = std::current_exception();
  }
  for (int i = 0; i < kLanes - 1; ++i) {
    cudaEventRecord(g_rt.join_ev[i], g_rt.side[i]);
    cudaStreamWaitEvent(g_rt.stream, g_rt.join_ev[i], 0);
  }
  if (ea) std::rethrow_exception(ea);
  if (eb) std::rethrow_exception(eb);
}

void order_after_lanes(cudaStream_t s) {
  for (int l = 0; l < kLanes; ++l) {
    cudaStream_t o = l == 0 ? g_rt.stream : g_rt.side[l - 1];
    if (o == s || !o) continue;
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) continue;
    cudaEventRecord(e, o);
    cudaStreamWaitEvent(s, e, 0);
    cudaEventDestroy(e);  // released once the wait has been satisfied
  }
}

int set_error(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return XGB_OK;
  return set_error(e == cudaErrorMemoryAllocation ? XGB_E_OOM : XGB_E_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

void* dev_alloc(size_t bytes) {
  if (bytes == 0) bytes = 8;
  void* p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes, stream());
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error(XGB_E_OOM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    throw std::bad_alloc();
  }
  return p;
}

void dev_free(void* p) {
  if (p && g_rt.ready) cudaFreeAsync(p, stream());
}

// ======================================================================= instrumentation
namespace {
struct ProfEvent {
  int kind;
  cudaEvent_t a, b;
  double work;
};
bool g_prof_on = false;
std::mutex g_prof_mu;
std::vector<ProfEvent> g_prof_events;
std::vector<cudaEvent_t> g_event_pool;
int64_t g_prof_launches[K_COUNT] = {0};
double g_prof_work[K_COUNT] = {0};
double g_prof_ms[K_COUNT] = {0};
cudaEvent_t g_pending_a[K_COUNT] = {nullptr};
cudaEvent_t g_user_events[16] = {nullptr};

cudaEvent_t pool_event() {
  if (!g_event_pool.empty()) {
    cudaEvent_t e = g_event_pool.back();
    g_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

void prof_drain() {
  for (auto& ev : g_prof_events) {
    float ms = 0.f;
    cudaEventSynchronize(ev.b);
    cudaEventElapsedTime(&ms, ev.a, ev.b);
    g_prof_ms[ev.kind] += ms;
    g_event_pool.push_back(ev.a);
    g_event_pool.push_back(ev.b);
  }
  g_prof_events.clear();
}
}  // namespace

bool profiling() { return g_prof_on; }

void prof_begin(int kind, cudaStream_t s) {
  if (!g_prof_on) return;
  g_pending_a[kind] = pool_event();
  cudaEventRecord(g_pending_a[kind], s);
}

void prof_end(int kind, cudaStream_t s, double work) {
  {
    std::lock_guard<std::mutex> lk(g_prof_mu);  // lanes count concurrently (profiling itself runs on lane 0)
    g_prof_launches[kind] += 1;
    g_prof_work[kind] += work;
  }
  if (!g_prof_on || !g_pending_a[kind]) return;
  cudaEvent_t b = pool_event();
  cudaEventRecord(b, s);
  g_prof_events.push_back({kind, g_pending_a[kind], b, work});
  g_pending_a[kind] = nullptr;
  if (g_prof_events.size() > 4096) prof_drain();
}

// ======================================================================= GEMM
// Grouped GEMM on the CUDA cores: C_g = alpha*op(A_g)op(B_g) + beta*C_g.  One
// CTA per TILE x TILE output tile of one group; 256 threads, each owning a
// (TILE/16)^2 micro-tile.  T = double is the FP64 form (FP64 on GB300 runs on
// the narrow DFMA pipe, so the host picks the tile edge that spreads the work
// over the most SMs); T = float is the FP32 form (operands rounded to FP32 as
// they are staged, FP32 accumulation, alpha/beta and the store in FP64).
template <int TILE, typename T>
__global__ void __launch_bounds__(256) gemm_simt_kernel(const xgb_gemm_desc* __restrict__ descs,
                                                        const GemmTile* __restrict__ tiles, const double* __restrict__ A,
                                                        const double* __restrict__ B, double* __restrict__ C,
                                                        double alpha, double beta, double* __restrict__ ws) {
  constexpr int BK = 16;
  constexpr int R = TILE / 16;
  constexpr int PER = TILE * BK / 256;  // staged elements of A (and of B) per thread and k step
  // two stages: the global loads of k step s + 1 are in flight (in registers) while step s is
  // multiplied out of shared memory, and one barrier per step separates the stages
  __shared__ T As[2][BK][TILE + 1];
  __shared__ T Bs[2][BK][TILE + 1];
  const GemmTile t = tiles[blockIdx.x];
  const xgb_gemm_desc d = descs[t.g];
  const int64_t kbeg = t.k0, kend = t.k1 < 0 ? d.k : t.k1;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t row0 = int64_t(t.tm) * TILE, col0 = int64_t(t.tn) * TILE;
  // a warp whose outputs all lie outside the block (an edge tile of a block narrower than the tile)
  // skips the multiply-adds: GB300's narrow FP64 pipe takes as long for a warp instruction whatever
  // its active lanes; its share of the staging loads and the barriers stays
  bool live = false;
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int c = 0; c < R; ++c) live |= row0 + tx + 16 * r < d.m && col0 + ty + 16 * c < d.n;
  const bool warp_live = __any_sync(0xffffffffu, live);
  T acc[R][R];
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int j = 0; j < R; ++j) acc[i][j] = T(0);

  T ra[PER], rb[PER];
  auto fetch = [&](int64_t k0) {
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = tid + 256 * u;
      int i, kk;
      if (d.trans_a) { kk = e % BK; i = e / BK; } else { i = e % TILE; kk = e / TILE; }
      const int64_t gi = row0 + i, gk = k0 + kk;
      double v = 0.0;
      if (gi < d.m && gk < kend) v = d.trans_a ? A[d.a_off + gk + gi * d.lda] : A[d.a_off + gi + gk * d.lda];
      ra[u] = T(v);
      int j, kb;
      if (d.trans_b) { j = e % TILE; kb = e / TILE; } else { kb = e % BK; j = e / BK; }
      const int64_t gj = col0 + j, gkb = k0 + kb;
      double w = 0.0;
      if (gj < d.n && gkb < kend) w = d.trans_b ? B[d.b_off + gj + gkb * d.ldb] : B[d.b_off + gkb + gj * d.ldb];
      rb[u] = T(w);
    }
  };
  auto stash = [&](int st) {
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = tid + 256 * u;
      int i, kk;
      if (d.trans_a) { kk = e % BK; i = e / BK; } else { i = e % TILE; kk = e / TILE; }
      As[st][kk][i] = ra[u];
      int j, kb;
      if (d.trans_b) { j = e % TILE; kb = e / TILE; } else { kb = e % BK; j = e / BK; }
      Bs[st][kb][j] = rb[u];
    }
  };
  if (kbeg < kend) {
    fetch(kbeg);
    stash(0);
  }
  __syncthreads();
  int st = 0;
  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
    const bool more = k0 + BK < kend;
    if (more) fetch(k0 + BK);
    const int kmax = !warp_live ? 0 : (kend - k0) < BK ? int(kend - k0) : BK;
    for (int kk = 0; kk < kmax; ++kk) {
      T a[R], b[R];
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = As[st][kk][tx + 16 * r];
#pragma unroll
      for (int c = 0; c < R; ++c) b[c] = Bs[st][kk][ty + 16 * c];
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
    if (more) stash(st ^ 1);
    __syncthreads();
    st ^= 1;
  }
  if (t.slot >= 0) {  // split-K partial: the whole tile, raw sums, column-major TILE x TILE
    double* w = ws + int64_t(t.slot) * TILE * TILE;
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int c = 0; c < R; ++c) w[(tx + 16 * r) + (ty + 16 * c) * TILE] = double(acc[r][c]);
    return;
  }
  // FP64 operations go through GB300's narrow FP64 pipe: alpha = 1, beta = 0 stores the sums as they are
  const bool scaled = alpha != 1.0, accumulate = beta != 0.0;
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int c = 0; c < R; ++c) {
      int64_t i = row0 + tx + 16 * r, j = col0 + ty + 16 * c;
      if (i < d.m && j < d.n) {
        double* p = C + d.c_off + i + j * d.ldc;
        double v = scaled ? alpha * double(acc[r][c]) : double(acc[r][c]);
        if (accumulate) v += beta * (*p);
        *p = v;
      }
    }
}

void launch_gemm_f64(const xgb_gemm_desc* d_descs, const GemmTile* d_tiles, int n_tiles, int tile, const double* A,
                     const double* B, double* C, double alpha, double beta, cudaStream_t s) {
  if (n_tiles <= 0) return;
  if (tile == 64) gemm_simt_kernel<64, double><<<n_tiles, 256, 0, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, nullptr);
  else if (tile == 32) gemm_simt_kernel<32, double><<<n_tiles, 256, 0, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, nullptr);
  else gemm_simt_kernel<16, double><<<n_tiles, 256, 0, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, nullptr);
  count_launch();
}

// C tile = alpha * (sum of its partial slots in slot order) + beta * C: the result does not
// depend on which CTA finished first
__global__ void __launch_bounds__(256) splitk_reduce_kernel(const xgb_gemm_desc* __restrict__ descs,
                                                            const SplitReduce* __restrict__ red, int tile,
                                                            const double* __restrict__ ws, double* __restrict__ C,
                                                            double alpha, double beta) {
  const SplitReduce r = red[blockIdx.x];
  const xgb_gemm_desc d = descs[r.g];
  const int64_t tt = int64_t(tile) * tile;
  for (int64_t e = threadIdx.x; e < tt; e += blockDim.x) {
    const int64_t i = int64_t(r.tm) * tile + e % tile, j = int64_t(r.tn) * tile + e / tile;
    if (i >= d.m || j >= d.n) continue;
    double acc = ws[int64_t(r.first) * tt + e];
    for (int p = 1; p < r.count; ++p) acc += ws[(int64_t(r.first) + p) * tt + e];
    double* c = C + d.c_off + i + j * d.ldc;
    double v = alpha == 1.0 ? acc : alpha * acc;
    if (beta != 0.0) v += beta * (*c);
    *c = v;
  }
}

void launch_gemm_f64_splitk(const xgb_gemm_desc* d_descs, const GemmTile* d_tiles, int n_tiles, int tile,
                            const SplitReduce* d_reduce, int n_reduce, const double* A, const double* B, double* C,
                            double* ws, double alpha, double beta, cudaStream_t s) {
  if (n_tiles <= 0) return;
  if (tile == 64) gemm_simt_kernel<64, double><<<n_tiles, 256, 0, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, ws);
  else if (tile == 32) gemm_simt_kernel<32, double><<<n_tiles, 256, 0, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, ws);
  else gemm_simt_kernel<16, double><<<n_tiles, 256, 0, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, ws);
  count_launch();
  if (n_reduce <= 0) return;
  splitk_reduce_kernel<<<n_reduce, 256, 0, s>>>(d_descs, d_reduce, tile, ws, C, alpha, beta);
  count_launch();
}

void launch_gemm_f32(const xgb_gemm_desc* d_descs, const GemmTile* d_tiles, int n_tiles, int tile, const double* A,
                     const double* B, double* C, double alpha, double beta, cudaStream_t s) {
  if (n_tiles <= 0) return;
  if (tile == 64) gemm_simt_kernel<64, float><<<n_tiles, 256, 0, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, nullptr);
  else if (tile == 32) gemm_simt_kernel<32, float><<<n_tiles, 256, 0, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, nullptr);
  else gemm_simt_kernel<16, float><<<n_tiles, 256, 0, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, nullptr);
  count_launch();
}

void order_tiles_by_work(std::vector<GemmTile>& tiles, const xgb_gemm_desc* descs) {
  // stable counting sort on the k extent, longest first: a list holds few distinct extents but up to
  // ~10^5 tiles, and the plans of a step whose shapes changed are built while the GPU waits
  auto extent = [&](const GemmTile& t) { return int64_t(t.k1 < 0 ? descs[t.g].k : t.k1) - t.k0; };
  std::map<int64_t, size_t, std::greater<int64_t>> slot;  // extent -> first position, descending
  for (const auto& t : tiles) ++slot[extent(t)];
  if (slot.size() <= 1) return;
  size_t off = 0;
  for (auto& [e, c] : slot) {
    const size_t n = c;
    c = off;
    off += n;
  }
  std::vector<GemmTile> out(tiles.size());
  int64_t last_e = -1;
  size_t* last_slot = nullptr;
  for (const auto& t : tiles) {
    const int64_t e = extent(t);
    if (e != last_e) {  // runs of equal extents are common: one map lookup per run
      last_slot = &slot.find(e)->second;
      last_e = e;
    }
    out[(*last_slot)++] = t;
  }
  tiles.swap(out);
}

int choose_gemm_tile(const xgb_gemm_desc* descs, int n) {
  // Largest tile edge that still yields >= 2 CTAs per SM; FP64 throughput is
  // per SM, so spreading tiles over SMs beats bigger tiles' reuse here.
  const int target = 2 * (g_rt.sms > 0 ? g_rt.sms : 152);
  for (int tile : {64, 32}) {
    int64_t cnt = 0;
    for (int g = 0; g < n; ++g) cnt += ((descs[g].m + tile - 1) / tile) * ((descs[g].n + tile - 1) / tile);
    if (cnt >= target) return tile;
  }
  return 16;
}

// ======================================================================= permute
// Gather-permute with recoupling coefficients, one ROW at a time: a row is the run of a task's
// output sub-block along output leg 0 (all other leg indices fixed), which is contiguous in the
// output (leg 0 fastest) and, for the permutations that keep the block's leading leg in front,
// contiguous in the source too.  A group of G threads (G a power of two up to a warp, chosen on
// the host from the rows' typical length) takes a chunk of kRowsPerChunk consecutive rows: the
// first row's multi-index is decoded once (32-bit division), the following rows step it like an
// odometer (leg 1 fastest, adding the legs' strides), and the lanes walk each row with unit stride,
// so a warp's loads and stores cover whole 32-byte sectors.  Four rows' loads are issued before
// their stores.  Tasks with several contributions (SU(2) recoupling) accumulate them in a fixed
// order.
constexpr int kRowsPerChunk = 8;

// Row cursor with the current task's extents, strides and coefficient held in registers (loaded
// once per task, not per row): SI is int32_t when every stride of the plan fits (the host checks),
// int64_t otherwise.  All per-leg arrays are indexed only inside fully unrolled loops.
template <typename SI>
struct RowCursor {
  int ti = -1;          // task
  int64_t row_end = 0;  // first row past the task
  int rank = 0, d0 = 1, n_contrib = 1, contrib0 = 0;
  double coeff = 0.0;
  int dims[XGB_MAX_LEGS];
  SI dstr[XGB_MAX_LEGS], sstr[XGB_MAX_LEGS];  // sstr: strides of the single contribution
  int idx[XGB_MAX_LEGS];                      // multi-index of legs 1..rank-1
  int64_t dofs = 0, sofs = 0;
};

template <typename SI>
__device__ __forceinline__ void cursor_seek(RowCursor<SI>& c, const xgb_perm_task* __restrict__ tasks,
                                            const int64_t* __restrict__ row_start, int n_tasks,
                                            const xgb_perm_contrib* __restrict__ contribs, int64_t r) {
  int ti = c.ti >= 0 ? c.ti : 0;
  if (!(r >= row_start[ti] && r < row_start[ti + 1])) {
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (row_start[mid] <= r) lo = mid; else hi = mid - 1;
    }
    ti = lo;
  }
  const xgb_perm_task& t = tasks[ti];
  if (ti != c.ti) {  // task fields into registers
    c.ti = ti;
    c.row_end = row_start[ti + 1];
    c.rank = t.rank;
    c.d0 = t.rank > 0 ? t.dims[0] : 1;
    c.n_contrib = t.n_contrib;
    c.contrib0 = t.contrib0;
    const bool single = t.n_contrib == 1;
    c.coeff = single ? contribs[t.contrib0].coeff : 0.0;
#pragma unroll
    for (int k = 0; k < XGB_MAX_LEGS; ++k) {
      const bool on = k < t.rank;
      c.dims[k] = on ? t.dims[k] : 1;
      c.dstr[k] = on ? SI(t.dst_stride[k]) : SI(0);
      c.sstr[k] = (on && single) ? SI(contribs[t.contrib0].src_stride[k]) : SI(0);
    }
  }
  int64_t rem = r - row_start[ti];
  c.dofs = t.dst_base;
  c.sofs = c.n_contrib == 1 ? contribs[c.contrib0].src_base : 0;
#pragma unroll
  for (int k = 1; k < XGB_MAX_LEGS; ++k) {
    c.idx[k] = 0;
    if (k < c.rank) {
      const int dk = c.dims[k];
      int ik;
      if (rem < (int64_t(1) << 31)) {  // 32-bit division for the common case
        const uint32_t r32 = uint32_t(rem), q = r32 / uint32_t(dk);
        ik = int(r32 - q * uint32_t(dk));
        rem = q;
      } else {
        const int64_t q = rem / dk;
        ik = int(rem - q * dk);
        rem = q;
      }
      c.idx[k] = ik;
      c.dofs += int64_t(ik) * c.dstr[k];
      c.sofs += int64_t(ik) * c.sstr[k];
    }
  }
}

// next row of the same task: leg 1 fastest, carrying into the higher legs
template <typename SI>
__device__ __forceinline__ void cursor_step(RowCursor<SI>& c) {
#pragma unroll
  for (int k = 1; k < XGB_MAX_LEGS; ++k) {
    if (k >= c.rank) return;
    c.dofs += c.dstr[k];
    c.sofs += c.sstr[k];
    if (++c.idx[k] < c.dims[k]) return;
    c.idx[k] = 0;
    c.dofs -= int64_t(c.dims[k]) * c.dstr[k];
    c.sofs -= int64_t(c.dims[k]) * c.sstr[k];
  }
}

template <int G, typename SI>
__global__ void __launch_bounds__(256) permute_rows_kernel(const xgb_perm_task* __restrict__ tasks,
                                                           const int64_t* __restrict__ row_start, int n_tasks,
                                                           int64_t total_rows, const xgb_perm_contrib* __restrict__ contribs,
                                                           const double* __restrict__ src, double* __restrict__ dst) {
  constexpr int U = 4;
  const int lane = int(threadIdx.x) % G;
  const int64_t group = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) / G;
  const int64_t ngroups = int64_t(gridDim.x) * blockDim.x / G;
  const int64_t nchunks = (total_rows + kRowsPerChunk - 1) / kRowsPerChunk;
  RowCursor<SI> cur;
  for (int64_t chunk = group; chunk < nchunks; chunk += ngroups) {
    const int64_t r0 = chunk * kRowsPerChunk;
    const int64_t r1 = r0 + kRowsPerChunk < total_rows ? r0 + kRowsPerChunk : total_rows;
    cursor_seek(cur, tasks, row_start, n_tasks, contribs, r0);
    for (int64_t rb = r0; rb < r1; rb += U) {
      int64_t doff[U], soff[U];
      SI ds0[U], ss0[U];
      double coeff[U];
      int len[U];
      int maxlen = 0;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        len[u] = 0;
        doff[u] = soff[u] = 0;
        ds0[u] = ss0[u] = 0;
        coeff[u] = 0.0;
        const int64_t r = rb + u;
        if (r >= r1) continue;
        if (r >= cur.row_end) cursor_seek(cur, tasks, row_start, n_tasks, contribs, r);
        if (cur.n_contrib == 1) {
          doff[u] = cur.dofs;
          soff[u] = cur.sofs;
          ds0[u] = cur.dstr[0];
          ss0[u] = cur.sstr[0];
          coeff[u] = cur.coeff;
          len[u] = cur.d0;
          maxlen = max(maxlen, cur.d0);
          cursor_step(cur);
          continue;
        }
        // several source sub-blocks add into this row (SU(2)): fixed contribution order
        for (int i = lane; i < cur.d0; i += G) {
          double v = 0.0;
          for (int c = 0; c < cur.n_contrib; ++c) {
            const xgb_perm_contrib& cc = contribs[cur.contrib0 + c];
            int64_t so = cc.src_base + int64_t(i) * (cur.rank > 0 ? cc.src_stride[0] : 0);
#pragma unroll
            for (int k = 1; k < XGB_MAX_LEGS; ++k)
              if (k < cur.rank) so += cur.idx[k] * cc.src_stride[k];
            v = fma(cc.coeff, __ldg(src + so), v);
          }
          dst[cur.dofs + int64_t(i) * cur.dstr[0]] = v;
        }
        cursor_step(cur);
      }
      for (int i = lane; i < maxlen; i += G) {
        double v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (i < len[u]) v[u] = coeff[u] * __ldg(src + soff[u] + int64_t(i) * ss0[u]);
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (i < len[u]) dst[doff[u] + int64_t(i) * ds0[u]] = v[u];
      }
    }
  }
}

// Wide-row form (groups of G >= 8 lanes, rows of about G or more elements).  The row cursor above
// keeps every leg's extent and strides in registers (128 per thread for G = 32: two CTAs per SM),
// which leaves too few loads in flight to cover HBM latency on large tensors.  Here lane u < 8 of a
// group decodes row u of the group's 8-row chunk on its own (task by the cached range or a binary
// search, multi-index by 32-bit division, the per-leg fields read from the L1-resident task table
// in a loop rather than held in registers), and the row's offsets, strides, length and coefficient
// reach the other lanes by shuffles.  The loads go through shared memory instead of registers:
// every lane copies the first 2G elements of each of the chunk's 8 rows (16 elements) with 8-byte
// cp.async into its own column of the warp's staging buffer, so that in-flight data costs no
// registers.  Two stages per warp: the next chunk is decoded and its copies issued before the
// current chunk's copies are awaited, scaled by the coefficient and stored.  Elements past 2G of a
// long row are copied directly.  It serves plans in which every task has exactly one contribution
// (every abelian permute); plans with several contributions per task (SU(2) recoupling) take the
// cursor kernel above.  Loop bounds that contain shuffles are warp-uniform (chunks are taken per
// warp).
constexpr int kWideSlots = 2;      // staged elements per row and lane
constexpr int kWideThreads = 128;  // 4 warps per CTA: 32 KB of staging

__device__ __forceinline__ void find_task(const int64_t* __restrict__ row_start, int n_tasks, int64_t r, int& ti,
                                          int64_t& lo, int64_t& hi) {
  if (r >= lo && r < hi) return;
  int a = 0, b = n_tasks - 1;
  while (a < b) {
    const int mid = (a + b + 1) >> 1;
    if (row_start[mid] <= r) a = mid; else b = mid - 1;
  }
  ti = a;
  lo = row_start[a];
  hi = row_start[a + 1];
}

__device__ __forceinline__ int split_index(int64_t& rem, int dk) {
  if (rem < (int64_t(1) << 31)) {  // 32-bit division for the common case
    const uint32_t r32 = uint32_t(rem), q = r32 / uint32_t(dk);
    rem = q;
    return int(r32 - q * uint32_t(dk));
  }
  const int64_t q = rem / dk;
  const int ik = int(rem - q * dk);
  rem = q;
  return ik;
}

__device__ __forceinline__ void cp_async8(double* smem, const double* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <typename SI>
struct WideRow {  // one decoded row (len 0: no row)
  long long dofs = 0, sofs = 0;
  double coeff = 0.0;
  int len = 0;
  SI ds0 = 0, ss0 = 0;
};

template <typename SI>
__device__ __forceinline__ WideRow<SI> wide_decode(const xgb_perm_task* __restrict__ tasks,
                                                   const int64_t* __restrict__ row_start, int n_tasks,
                                                   int64_t total_rows, const xgb_perm_contrib* __restrict__ contribs,
                                                   int64_t r, bool valid, int& ti, int64_t& lo, int64_t& hi) {
  WideRow<SI> w;
  if (!valid || r >= total_rows) return w;
  find_task(row_start, n_tasks, r, ti, lo, hi);
  const xgb_perm_task& t = tasks[ti];
  const xgb_perm_contrib& c = contribs[t.contrib0];  // the only contribution
  const int rank = t.rank;
  int64_t rem = r - lo;
  int64_t dofs = t.dst_base, sofs = c.src_base;
  for (int k = 1; k < rank; ++k) {
    const int ik = split_index(rem, t.dims[k]);
    dofs += int64_t(ik) * t.dst_stride[k];
    sofs += int64_t(ik) * c.src_stride[k];
  }
  w.dofs = dofs;
  w.sofs = sofs;
  w.coeff = c.coeff;
  w.len = rank > 0 ? t.dims[0] : 1;
  w.ds0 = rank > 0 ? SI(t.dst_stride[0]) : SI(0);
  w.ss0 = rank > 0 ? SI(c.src_stride[0]) : SI(0);
  return w;
}

template <int G, typename SI>
__global__ void __launch_bounds__(kWideThreads, 6) permute_rows_wide_kernel(const xgb_perm_task* __restrict__ tasks,
                                                                            const int64_t* __restrict__ row_start,
                                                                            int n_tasks, int64_t total_rows,
                                                                            const xgb_perm_contrib* __restrict__ contribs,
                                                                            const double* __restrict__ src,
                                                                            double* __restrict__ dst) {
  static_assert(G >= kRowsPerChunk && G <= 32, "one decoding lane per row of the chunk");
  constexpr int kGroupsPerWarp = 32 / G;
  constexpr int kHead = kWideSlots * G;  // staged elements per row
  constexpr unsigned kFull = 0xffffffffu;
  __shared__ double stage[kWideThreads / 32][2][kRowsPerChunk * kWideSlots][32];
  const int lane = int(threadIdx.x) & 31;
  const int wib = int(threadIdx.x) >> 5;
  const int gl = lane % G;
  const bool decoder = gl < kRowsPerChunk;
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  const int64_t nchunks = (total_rows + kRowsPerChunk - 1) / kRowsPerChunk;
  const int64_t step = nwarps * kGroupsPerWarp;
  int ti = 0;
  int64_t lo = 0, hi = 0;  // rows of task ti (empty: the first row searches)

  // copies of the first kHead elements of the chunk's rows into stage st (one commit group)
  auto issue = [&](const WideRow<SI>& w, int st) {
#pragma unroll
    for (int u = 0; u < kRowsPerChunk; ++u) {
      const long long so = __shfl_sync(kFull, w.sofs, u, G);
      const SI ss = __shfl_sync(kFull, w.ss0, u, G);
      const int lu = __shfl_sync(kFull, w.len, u, G);
#pragma unroll
      for (int j = 0; j < kWideSlots; ++j) {
        const int i = j * G + gl;
        if (i < lu) cp_async8(&stage[wib][st][u * kWideSlots + j][lane], src + so + int64_t(i) * ss);
      }
    }
    cp_async_commit();
  };
  // scaled stores of the staged elements, then the elements past kHead of long rows
  auto drain = [&](const WideRow<SI>& w, int st) {
#pragma unroll
    for (int u = 0; u < kRowsPerChunk; ++u) {
      const long long dof = __shfl_sync(kFull, w.dofs, u, G);
      const SI ds = __shfl_sync(kFull, w.ds0, u, G);
      const int lu = __shfl_sync(kFull, w.len, u, G);
      const double cf = __shfl_sync(kFull, w.coeff, u, G);
#pragma unroll
      for (int j = 0; j < kWideSlots; ++j) {
        const int i = j * G + gl;
        if (i < lu) dst[dof + int64_t(i) * ds] = cf * stage[wib][st][u * kWideSlots + j][lane];
      }
    }
    if (__reduce_max_sync(kFull, w.len) > kHead) {
      for (int u = 0; u < kRowsPerChunk; ++u) {
        const long long so = __shfl_sync(kFull, w.sofs, u, G);
        const long long dof = __shfl_sync(kFull, w.dofs, u, G);
        const SI ss = __shfl_sync(kFull, w.ss0, u, G);
        const SI ds = __shfl_sync(kFull, w.ds0, u, G);
        const int lu = __shfl_sync(kFull, w.len, u, G);
        const double cf = __shfl_sync(kFull, w.coeff, u, G);
        for (int i = kHead + gl; i < lu; i += G) dst[dof + int64_t(i) * ds] = cf * __ldg(src + so + int64_t(i) * ss);
      }
    }
  };

  int64_t cb = warp * kGroupsPerWarp;
  if (cb >= nchunks) return;  // warp-uniform
  int64_t chunk = cb + lane / G;
  WideRow<SI> cur = wide_decode<SI>(tasks, row_start, n_tasks, total_rows, contribs, chunk * kRowsPerChunk + gl,
                                    decoder && chunk < nchunks, ti, lo, hi);
  issue(cur, 0);
  int st = 0;
  for (; cb < nchunks; cb += step) {
    const int64_t nb = cb + step;
    WideRow<SI> nxt;
    if (nb < nchunks) {  // warp-uniform
      chunk = nb + lane / G;
      nxt = wide_decode<SI>(tasks, row_start, n_tasks, total_rows, contribs, chunk * kRowsPerChunk + gl,
                            decoder && chunk < nchunks, ti, lo, hi);
      issue(nxt, st ^ 1);
      cp_async_wait<1>();  // the current chunk's group has landed
    } else {
      cp_async_wait<0>();
    }
    drain(cur, st);
    cur = nxt;
    st ^= 1;
  }
}

PermRows perm_rows(const xgb_perm_task* tasks, int n_tasks, const xgb_perm_contrib* contribs, int n_contrib) {
  PermRows r;
  r.row_start.assign(size_t(n_tasks) + 1, 0);
  double elems = 0, weighted = 0;
  for (int t = 0; t < n_tasks; ++t) {
    const int64_t d0 = tasks[t].rank > 0 ? std::max<int64_t>(tasks[t].dims[0], 1) : 1;
    const int64_t rows = d0 > 0 ? tasks[t].nelem / d0 : 0;
    r.row_start[t + 1] = r.row_start[t] + rows;
    elems += double(tasks[t].nelem);
    weighted += double(tasks[t].nelem) * double(d0);
  }
  r.total_rows = r.row_start.back();
  for (int t = 0; t < n_tasks && r.single; ++t) r.single = tasks[t].n_contrib == 1;
  auto wide = [](int64_t v) { return v > INT32_MAX || v < INT32_MIN; };
  for (int t = 0; t < n_tasks && r.narrow; ++t)
    for (int k = 0; k < tasks[t].rank; ++k)
      if (wide(tasks[t].dst_stride[k])) r.narrow = false;
  for (int c = 0; c < n_contrib && r.narrow; ++c)
    for (int k = 0; k < XGB_MAX_LEGS; ++k)
      if (wide(contribs[c].src_stride[k])) r.narrow = false;
  const double avg = elems > 0 ? weighted / elems : 1.0;  // element-weighted row length
  r.group = 1;
  while (r.group < 32 && 2.0 * r.group <= avg * 1.25) r.group *= 2;
  return r;
}

template <typename SI>
void launch_permute_t(const xgb_perm_task* d_tasks, const int64_t* d_row_start, int n_tasks, int64_t total_rows,
                      int group, bool single, const xgb_perm_contrib* d_contribs, const double* src, double* dst,
                      cudaStream_t s) {
  if (total_rows <= 0 || n_tasks <= 0) return;
  // one group per chunk of kRowsPerChunk rows; enough CTAs to fill the GPU a few times over
  const int64_t groups_needed = (total_rows + kRowsPerChunk - 1) / kRowsPerChunk;
  const int64_t per_block = 256 / group;
  const int64_t cap = int64_t(num_sms() > 0 ? num_sms() : 152) * 16;
  const unsigned blocks = unsigned(std::max<int64_t>(1, std::min<int64_t>(cap, (groups_needed + per_block - 1) / per_block)));
  // wide-row kernel: 128-thread CTAs, about one resident wave (six per SM) looping over the chunks
  const int64_t wide_per_block = kWideThreads / group;
  const unsigned wblocks = unsigned(std::max<int64_t>(
      1, std::min<int64_t>(int64_t(num_sms() > 0 ? num_sms() : 152) * 6, (groups_needed + wide_per_block - 1) / wide_per_block)));
  // the wide-row kernel for single-contribution plans whose rows fill a group of 8 or more lanes
  switch (single || group < kRowsPerChunk ? group : -group) {
    case 32: permute_rows_wide_kernel<32, SI><<<wblocks, kWideThreads, 0, s>>>(d_tasks, d_row_start, n_tasks, total_rows, d_contribs, src, dst); break;
    case 16: permute_rows_wide_kernel<16, SI><<<wblocks, kWideThreads, 0, s>>>(d_tasks, d_row_start, n_tasks, total_rows, d_contribs, src, dst); break;
    case 8: permute_rows_wide_kernel<8, SI><<<wblocks, kWideThreads, 0, s>>>(d_tasks, d_row_start, n_tasks, total_rows, d_contribs, src, dst); break;
    case 4: permute_rows_kernel<4, SI><<<blocks, 256, 0, s>>>(d_tasks, d_row_start, n_tasks, total_rows, d_contribs, src, dst); break;
    case 2: permute_rows_kernel<2, SI><<<blocks, 256, 0, s>>>(d_tasks, d_row_start, n_tasks, total_rows, d_contribs, src, dst); break;
    case -32: permute_rows_kernel<32, SI><<<blocks, 256, 0, s>>>(d_tasks, d_row_start, n_tasks, total_rows, d_contribs, src, dst); break;
    case -16: permute_rows_kernel<16, SI><<<blocks, 256, 0, s>>>(d_tasks, d_row_start, n_tasks, total_rows, d_contribs, src, dst); break;
    case -8: permute_rows_kernel<8, SI><<<blocks, 256, 0, s>>>(d_tasks, d_row_start, n_tasks, total_rows, d_contribs, src, dst); break;
    default: permute_rows_kernel<1, SI><<<blocks, 256, 0, s>>>(d_tasks, d_row_start, n_tasks, total_rows, d_contribs, src, dst); break;
  }
  count_launch();
}

void launch_permute(const xgb_perm_task* d_tasks, const int64_t* d_row_start, int n_tasks, int64_t total_rows,
                    int group, bool narrow, bool single, const xgb_perm_contrib* d_contribs, const double* src,
                    double* dst, cudaStream_t s) {
  if (narrow)
    launch_permute_t<int32_t>(d_tasks, d_row_start, n_tasks, total_rows, group, single, d_contribs, src, dst, s);
  else launch_permute_t<int64_t>(d_tasks, d_row_start, n_tasks, total_rows, group, single, d_contribs, src, dst, s);
}

// ======================================================================= shared helpers
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ======================================================================= truncation
// cutoff_matrices on the device (src/Core/Tensor.cpp:523-633).  The global
// descending order of all singular values is made deterministic and robust
// to last-bit differences: values are ranked exactly (ties by position),
// consecutive values within kTieRtol (relative) form a tie group, and inside
// a group entries keep their (sector, index) position order.  Then: keep the
// first max_keep, drop values < eps, optionally cut the last multiplet, fall
// back to the first value of the first sector when nothing survives, and
// count kept values per sector.  One CTA; n is the number of singular values
// of one tensor (thousands at most).
constexpr double kTieRtol = 1.0e-12;

__global__ void __launch_bounds__(1024) truncate_kernel(int n_sectors, const int64_t* __restrict__ s_begin,
                                                        const int32_t* __restrict__ deg, const double* __restrict__ s,
                                                        int64_t total, int64_t max_keep, double eps, int preserve,
                                                        int32_t* __restrict__ keep, double* __restrict__ out2,
                                                        int64_t* __restrict__ ws) {
  __shared__ double red_w[32], red_e[32];
  int64_t* exact = ws;                 // exact[r] = index with exact rank r
  int64_t* gstart = ws + total;        // group start position for each exact position
  int64_t* order = ws + 2 * total;     // order[f] = index at final position f
  int64_t* flag = ws + 3 * total;      // flag[i] = 1 kept, 0 dropped; fpos stored in gstart reuse below
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int g = tid; g < n_sectors; g += blockDim.x) keep[g] = 0;
  // exact ranks under a total order (NaN ranks below every number, ties by
  // index), so that `exact` is a permutation whatever the values are
  auto key = [](double v) { return v == v ? v : -INFINITY; };
  for (int64_t i = tid; i < total; i += blockDim.x) {
    const double si = key(s[i]);
    int64_t r = 0;
    for (int64_t j = 0; j < total; ++j) {
      const double sj = key(s[j]);
      r += (sj > si) || (sj == si && j < i);
    }
    exact[r] = i;
    flag[i] = 0;
  }
  __syncthreads();
  if (tid == 0) {
    int64_t start = 0;
    for (int64_t p = 0; p < total; ++p) {
      if (p > 0) {
        const double prev = s[exact[p - 1]], cur = s[exact[p]];
        if (prev - cur > kTieRtol * prev) start = p;
      }
      gstart[p] = start;
    }
  }
  __syncthreads();
  for (int64_t p = tid; p < total; p += blockDim.x) {
    const int64_t i = exact[p], g0 = gstart[p];
    int64_t f = g0;
    for (int64_t q = g0; q < total && gstart[q] == g0; ++q) f += (exact[q] < i);
    order[f] = i;
  }
  __syncthreads();
  if (tid == 0) {
    const int64_t lim = total < max_keep ? total : max_keep;
    // kept list in final order, stored compactly at the front of `exact`
    int64_t nk = 0;
    for (int64_t f = 0; f < lim; ++f) {
      const int64_t i = order[f];
      if (eps > 0.0 && s[i] < eps) continue;
      exact[nk++] = i;
    }
    if (preserve) {
      int64_t end = -1;
      for (int64_t k = nk - 1; k > 0; --k) {
        const double a = s[exact[k - 1]], b = s[exact[k]];
        if (2.0 * (a - b) / (a + b) > 0.1) { end = k; break; }
      }
      if (end != -1) nk = end;
    }
    if (nk == 0) { exact[0] = 0; nk = 1; }  // first entry: first value of the first sector
    for (int64_t k = 0; k < nk; ++k) flag[exact[k]] = 1;
    // positions >= max_keep contribute to the truncated weight
    for (int64_t f = lim; f < total; ++f) flag[order[f]] |= 2;
  }
  __syncthreads();
  double wsum = 0.0, esum = 0.0;
  for (int64_t i = tid; i < total; i += blockDim.x) {
    int lo = 0, hi = n_sectors - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_begin[mid] <= i) lo = mid; else hi = mid - 1;
    }
    const double v = s[i];
    if (flag[i] & 2) wsum += deg[lo] * v * v;
    if (flag[i] & 1) {
      atomicAdd(&keep[lo], 1);
      esum += -deg[lo] * v * v * log(v * v);
    }
  }
  wsum = warp_sum(wsum);
  esum = warp_sum(esum);
  if (lane == 0) { red_w[warp] = wsum; red_e[warp] = esum; }
  __syncthreads();
  if (tid == 0) {
    double a = 0, b = 0;
    for (int w = 0; w < int(blockDim.x + 31) / 32; ++w) { a += red_w[w]; b += red_e[w]; }
    out2[0] = a;
    out2[1] = b;
  }
}

void launch_truncate(int n_sectors, const int64_t* d_s_begin, const int32_t* d_deg, const double* s, int64_t total,
                     int64_t max_keep, double eps, int preserve, int32_t* keep, double* out2, cudaStream_t st) {
  int64_t* ws = static_cast<int64_t*>(dev_alloc(sizeof(int64_t) * 4 * std::max<int64_t>(total, 1)));
  truncate_kernel<<<1, 1024, 0, st>>>(n_sectors, d_s_begin, d_deg, s, total, max_keep, eps, preserve, keep, out2, ws);
  count_launch();
  dev_free(ws);
}

// ======================================================================= QR
// Batched Householder QR in FP64 with LAPACK's dlarfg sign convention
// (beta = -sign(alpha)*||x||), so Q and R agree with dgeqrf/dorgqr.
__global__ void __launch_bounds__(256) qr_kernel(const xgb_qr_desc* __restrict__ descs, const int64_t* __restrict__ work_off,
                                                 const double* __restrict__ A, double* __restrict__ Q,
                                                 double* __restrict__ R, double* __restrict__ work) {
  const xgb_qr_desc d = descs[blockIdx.x];
  const int64_t m = d.m, n = d.n, kk = m < n ? m : n;
  double* W = work + work_off[blockIdx.x];  // m x n working copy (Householder vectors below diagonal)
  double* tau = W + m * n;                  // kk
  double* Qw = tau + kk;                    // m x m accumulation
  __shared__ double red[8];
  __shared__ double bcast[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int64_t e = tid; e < m * n; e += 256) W[e] = A[d.a_off + e];
  __syncthreads();
  auto block_sum = [&](double v) {
    v = warp_sum(v);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = 0;
    if (tid == 0) { for (int w = 0; w < 8; ++w) r += red[w]; bcast[0] = r; }
    __syncthreads();
    r = bcast[0];
    __syncthreads();
    return r;
  };
  for (int64_t j = 0; j < kk; ++j) {
    double* col = W + j * m;
    double part = 0;
    for (int64_t i = j + 1 + tid; i < m; i += 256) part = fma(col[i], col[i], part);
    double xnorm2 = block_sum(part);
    double alpha = col[j];
    double t = 0.0, beta = alpha;
    if (xnorm2 > 0.0) {
      beta = -copysign(sqrt(alpha * alpha + xnorm2), alpha);
      t = (beta - alpha) / beta;
      double scal = 1.0 / (alpha - beta);
      for (int64_t i = j + 1 + tid; i < m; i += 256) col[i] *= scal;
    }
    __syncthreads();
    if (tid == 0) { tau[j] = t; col[j] = beta; }
    __syncthreads();
    if (t != 0.0) {
      for (int64_t c = j + 1 + warp; c < n; c += 8) {
        double* cc = W + c * m;
        double w = (lane == 0) ? cc[j] : 0.0;
        for (int64_t i = j + 1 + lane; i < m; i += 32) w = fma(col[i], cc[i], w);
        w = warp_sum(w) * t;
        if (lane == 0) cc[j] -= w;
        for (int64_t i = j + 1 + lane; i < m; i += 32) cc[i] -= w * col[i];
      }
    }
    __syncthreads();
  }
  // R (r_rows x n): upper triangle of W in the first kk rows
  for (int64_t e = tid; e < d.r_rows * n; e += 256) {
    int64_t i = e % d.r_rows, c = e / d.r_rows;
    R[d.r_off + e] = (i < kk && i <= c) ? W[i + c * m] : 0.0;
  }
  // Q = H_0 H_1 ... H_{kk-1} applied to the first q_cols columns of I (backward accumulation)
  const int64_t qc = d.q_cols < m ? d.q_cols : m;
  for (int64_t e = tid; e < m * qc; e += 256) Qw[e] = ((e % m) == (e / m)) ? 1.0 : 0.0;
  __syncthreads();
  for (int64_t j = kk - 1; j >= 0; --j) {
    const double t = tau[j];
    if (t == 0.0) continue;
    const double* v = W + j * m;
    for (int64_t c = warp; c < qc; c += 8) {
      double* cc = Qw + c * m;
      double w = (lane == 0) ? cc[j] : 0.0;
      for (int64_t i = j + 1 + lane; i < m; i += 32) w = fma(v[i], cc[i], w);
      w = warp_sum(w) * t;
      if (lane == 0) cc[j] -= w;
      for (int64_t i = j + 1 + lane; i < m; i += 32) cc[i] -= w * v[i];
    }
    __syncthreads();
  }
  for (int64_t e = tid; e < m * d.q_cols; e += 256) {
    int64_t c = e / m;
    Q[d.q_off + e] = (c < qc && c < kk) ? Qw[e] : 0.0;
  }
}

size_t qr_work_elems(int64_t m, int64_t n) { return size_t(m * n + std::min(m, n) + m * m); }

void launch_qr(const xgb_qr_desc* d_descs, const int64_t* d_work_off, int n, const double* A, double* Q, double* R,
               double* work, cudaStream_t s) {
  if (n <= 0) return;
  qr_kernel<<<n, 256, 0, s>>>(d_descs, d_work_off, A, Q, R, work);
  count_launch();
}

// ======================================================================= elementwise
__global__ void absmax_kernel(const double* __restrict__ x, int64_t n, unsigned long long* __restrict__ out) {
  double m = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    m = fmax(m, fabs(x[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  // non-negative doubles order like their bit patterns
  if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(out, __double_as_longlong(m));
}

void launch_absmax(const double* x, int64_t n, double* out, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(double), s);
  if (n <= 0) return;
  int blocks = int(std::min<int64_t>((n + 255) / 256, int64_t(num_sms()) * 8));
  absmax_kernel<<<blocks, 256, 0, s>>>(x, n, reinterpret_cast<unsigned long long*>(out));
  count_launch();
}

__global__ void scale_by_inv_kernel(double* __restrict__ x, int64_t n, const double* __restrict__ m) {
  const double mv = *m;
  if (mv == 0.0) return;
  const double inv = 1.0 / mv;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) x[i] *= inv;
}

void launch_scale_by_inv(double* x, int64_t n, const double* m, cudaStream_t s) {
  if (n <= 0) return;
  int blocks = int(std::min<int64_t>((n + 255) / 256, int64_t(num_sms()) * 8));
  scale_by_inv_kernel<<<blocks, 256, 0, s>>>(x, n, m);
  count_launch();
}

__global__ void scale_kernel(double* __restrict__ x, int64_t n, double a) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) x[i] *= a;
}

void launch_scale(double* x, int64_t n, double alpha, cudaStream_t s) {
  if (n <= 0) return;
  int blocks = int(std::min<int64_t>((n + 255) / 256, int64_t(num_sms()) * 8));
  scale_kernel<<<blocks, 256, 0, s>>>(x, n, alpha);
  count_launch();
}

__global__ void copy2d_kernel(const xgb_copy2d_desc* __restrict__ descs, const double* __restrict__ src,
                              double* __restrict__ dst) {
  const xgb_copy2d_desc d = descs[blockIdx.y];
  const int64_t ne = d.rows * d.cols;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < ne; e += int64_t(gridDim.x) * blockDim.x) {
    int64_t i = e % d.rows, j = e / d.rows;
    dst[d.dst_off + i + j * d.dst_ld] = src[d.src_off + i + j * d.src_ld];
  }
}

void launch_copy2d(const xgb_copy2d_desc* d_descs, int n, int64_t max_elems, const double* src, double* dst, cudaStream_t s) {
  if (n <= 0 || max_elems <= 0) return;
  dim3 grid(unsigned(std::min<int64_t>((max_elems + 255) / 256, 1024)), unsigned(n));
  copy2d_kernel<<<grid, 256, 0, s>>>(d_descs, src, dst);
  count_launch();
}

__device__ __forceinline__ double diag_fn(int fn, double x) {
  switch (fn) {
    case XGB_DIAG_SQRT: return sqrt(x);
    case XGB_DIAG_INV: return 1.0 / x;
    default: return 1.0 / sqrt(x);
  }
}

__global__ void diag_from_vec_kernel(const xgb_copy2d_desc* __restrict__ descs, int fn, const double* __restrict__ src,
                                     double* __restrict__ dst) {
  const xgb_copy2d_desc d = descs[blockIdx.y];
  const int64_t k = d.rows;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < k * k; e += int64_t(gridDim.x) * blockDim.x) {
    int64_t i = e % k, j = e / k;
    dst[d.dst_off + e] = (i == j) ? (fn < 0 ? src[d.src_off + i] : diag_fn(fn, src[d.src_off + i])) : 0.0;
  }
}

void launch_diag_from_vec(const xgb_copy2d_desc* d_descs, int n, int64_t max_k, int fn, const double* src, double* dst,
                          cudaStream_t s) {
  if (n <= 0 || max_k <= 0) return;
  dim3 grid(unsigned(std::min<int64_t>((max_k * max_k + 255) / 256, 1024)), unsigned(n));
  diag_from_vec_kernel<<<grid, 256, 0, s>>>(d_descs, fn, src, dst);
  count_launch();
}

__global__ void diag_apply_kernel(const xgb_copy2d_desc* __restrict__ descs, int fn, double* __restrict__ x) {
  const xgb_copy2d_desc d = descs[blockIdx.y];
  const int64_t r = d.rows, c = d.cols;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < r * c; e += int64_t(gridDim.x) * blockDim.x) {
    int64_t i = e % r, j = e / r;
    double* p = x + d.dst_off + i + j * d.dst_ld;
    *p = (i == j) ? diag_fn(fn, *p) : 0.0;
  }
}

void launch_diag_apply(const xgb_copy2d_desc* d_descs, int n, int64_t max_k, int fn, double* x, cudaStream_t s) {
  if (n <= 0 || max_k <= 0) return;
  dim3 grid(unsigned(std::min<int64_t>((max_k * max_k + 255) / 256, 1024)), unsigned(n));
  diag_apply_kernel<<<grid, 256, 0, s>>>(d_descs, fn, x);
  count_launch();
}

// ======================================================================= C-ABI helpers
namespace {
template <class T>
T* upload(const T* host, size_t n, cudaStream_t s) {
  T* d = static_cast<T*>(dev_alloc(sizeof(T) * std::max<size_t>(n, 1)));
  if (n) cudaMemcpyAsync(d, host, sizeof(T) * n, cudaMemcpyHostToDevice, s);
  return d;
}
cudaStream_t pick(void* s) { return s ? static_cast<cudaStream_t>(s) : g_rt.stream; }
#define XGB_REQUIRE_INIT() \
  if (!g_rt.ready) return set_error(XGB_E_NOINIT, "xgb_init was not called")
#define XGB_GUARD_BEGIN try {
#define XGB_GUARD_END                                                         \
  }                                                                           \
  catch (const std::bad_alloc&) {                                             \
    return XGB_E_OOM;                                                         \
  }                                                                           \
  catch (const std::exception& ex) {                                          \
    return set_error(XGB_E_BADPLAN, ex.what());                               \
  }
}  // namespace

}  // namespace xgb

using namespace xgb;

extern "C" {

int xgb_init(int device) {
  if (g_rt.ready) return XGB_OK;
  int rc = check_cuda(cudaSetDevice(device), "cudaSetDevice");
  if (rc) return rc;
  cudaDeviceProp prop{};
  if ((rc = check_cuda(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties"))) return rc;
  g_rt.sms = prop.multiProcessorCount;
  g_rt.device = device;
  if ((rc = check_cuda(cudaStreamCreateWithFlags(&g_rt.stream, cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
  for (int i = 0; i < kLanes - 1; ++i) {
    if ((rc = check_cuda(cudaStreamCreateWithFlags(&g_rt.side[i], cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
    if ((rc = check_cuda(cudaMalloc(&g_rt.side_scratch[i], 64 * sizeof(double)), "cudaMalloc scratch"))) return rc;
    if ((rc = check_cuda(cudaEventCreateWithFlags(&g_rt.join_ev[i], cudaEventDisableTiming), "cudaEventCreate")))
      return rc;
  }
  if ((rc = check_cuda(cudaEventCreateWithFlags(&g_rt.fork_ev, cudaEventDisableTiming), "cudaEventCreate"))) return rc;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    // memory freed on one lane is not handed to another lane's allocation behind an inserted wait
    // (that would serialise the lanes); it is reused there once its free has completed
    int no = 0;
    cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no);
  }
  if ((rc = check_cuda(cudaMalloc(&g_rt.scratch, 64 * sizeof(double)), "cudaMalloc scratch"))) return rc;
  g_rt.ready = true;
  return XGB_OK;
}

int xgb_shutdown(void) {
  if (!g_rt.ready) return XGB_OK;
  cudaStreamSynchronize(g_rt.stream);
  for (int i = 0; i < kLanes - 1; ++i) {
    cudaStreamSynchronize(g_rt.side[i]);
    cudaFree(g_rt.side_scratch[i]);
    cudaStreamDestroy(g_rt.side[i]);
    cudaEventDestroy(g_rt.join_ev[i]);
  }
  cudaEventDestroy(g_rt.fork_ev);
  cudaFree(g_rt.scratch);
  cudaStreamDestroy(g_rt.stream);
  g_rt = Runtime{};
  g_lanes_used = false;
  return XGB_OK;
}

const char* xgb_last_error(void) { return g_err.c_str(); }

int xgb_synchronize(void) {
  XGB_REQUIRE_INIT();
  return check_cuda(cudaStreamSynchronize(g_rt.stream), "cudaStreamSynchronize");
}

int64_t xgb_launch_count(void) { return g_launches.load(); }

int xgb_profile_enable(int on) {
  XGB_REQUIRE_INIT();
  if (!on) prof_drain();
  g_prof_on = on != 0;
  return XGB_OK;
}

int xgb_profile_reset(void) {
  XGB_REQUIRE_INIT();
  cudaStreamSynchronize(g_rt.stream);
  prof_drain();
  for (int k = 0; k < K_COUNT; ++k) { g_prof_launches[k] = 0; g_prof_work[k] = 0; g_prof_ms[k] = 0; }
  return XGB_OK;
}

int xgb_profile_read(int kind, int64_t* launches, double* ms, double* work) {
  XGB_REQUIRE_INIT();
  if (kind < 0 || kind >= K_COUNT) return set_error(XGB_E_BADPLAN, "kernel kind out of range");
  cudaStreamSynchronize(g_rt.stream);
  prof_drain();
  *launches = g_prof_launches[kind];
  *ms = g_prof_ms[kind];
  *work = g_prof_work[kind];
  return XGB_OK;
}

int xgb_event_record(int slot) {
  XGB_REQUIRE_INIT();
  if (slot < 0 || slot >= 16) return set_error(XGB_E_BADPLAN, "event slot out of range");
  if (!g_user_events[slot]) cudaEventCreate(&g_user_events[slot]);
  return check_cuda(cudaEventRecord(g_user_events[slot], g_rt.stream), "cudaEventRecord");
}

double xgb_event_elapsed_ms(int a, int b) {
  if (a < 0 || a >= 16 || b < 0 || b >= 16 || !g_user_events[a] || !g_user_events[b]) return -1.0;
  cudaEventSynchronize(g_user_events[b]);
  float ms = -1.f;
  if (cudaEventElapsedTime(&ms, g_user_events[a], g_user_events[b]) != cudaSuccess) return -1.0;
  return ms;
}

void* xgb_stream_handle(void) { return g_rt.stream; }

int xgb_malloc(void** ptr, size_t bytes) {
  XGB_REQUIRE_INIT();
  return check_cuda(cudaMalloc(ptr, bytes ? bytes : 8), "cudaMalloc");
}
int xgb_free(void* ptr) {
  XGB_REQUIRE_INIT();
  cudaStreamSynchronize(g_rt.stream);
  return check_cuda(cudaFree(ptr), "cudaFree");
}
int xgb_memcpy_h2d(void* dst, const void* src, size_t bytes) {
  XGB_REQUIRE_INIT();
  int rc = check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g_rt.stream), "h2d");
  if (rc) return rc;
  return check_cuda(cudaStreamSynchronize(g_rt.stream), "h2d sync");
}
int xgb_memcpy_d2h(void* dst, const void* src, size_t bytes) {
  XGB_REQUIRE_INIT();
  int rc = check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g_rt.stream), "d2h");
  if (rc) return rc;
  return check_cuda(cudaStreamSynchronize(g_rt.stream), "d2h sync");
}
int xgb_memset_zero(void* dst, size_t bytes) {
  XGB_REQUIRE_INIT();
  return check_cuda(cudaMemsetAsync(dst, 0, bytes, g_rt.stream), "memset");
}

int xgb_grouped_gemm(int precision, int n_groups, const xgb_gemm_desc* descs, const double* A, const double* B,
                     double* C, double alpha, double beta, void* stream_) {
  XGB_REQUIRE_INIT();
  if (!gemm_precision_available(precision))
    return set_error(XGB_E_UNSUPPORTED, "precision form not available through this entry");
  if (n_groups < 0) return set_error(XGB_E_BADPLAN, "n_groups < 0");
  XGB_GUARD_BEGIN
  cudaStream_t s = pick(stream_);
  for (int g = 0; g < n_groups; ++g)
    if (descs[g].m < 0 || descs[g].n < 0 || descs[g].k < 0) return set_error(XGB_E_BADPLAN, "negative GEMM extent");
  if (precision == XGB_PREC_F64TC) {
    OzPlanHost op = build_oz_plan(descs, n_groups);
    if (op.tiles.empty()) return XGB_OK;
    double flops = 0;
    for (int g = 0; g < n_groups; ++g) flops += 2.0 * double(descs[g].m) * double(descs[g].n) * double(descs[g].k);
    auto* dd = upload(descs, size_t(n_groups), s);
    auto* dg = upload(op.groups.data(), op.groups.size(), s);
    auto* dk = upload(op.tasks.data(), op.tasks.size(), s);
    auto* dt = upload(op.tiles.data(), op.tiles.size(), s);
    auto* dr = upload(op.red.data(), op.red.size(), s);
    auto* rm = static_cast<unsigned long long*>(dev_alloc(sizeof(unsigned long long) * size_t(std::max<int64_t>(op.rowmax, 1))));
    auto* ap = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(op.a_bytes, 16))));
    auto* bp = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(op.b_bytes, 16))));
    prof_begin(K_GEMM_OZ, s);
    launch_gemm_oz(dd, dg, dk, int(op.tasks.size()), dt, int(op.tiles.size()), dr, int(op.red.size()), op.slots, A, B,
                   rm, op.rowmax, ap, bp, C, alpha, beta, s);
    prof_end(K_GEMM_OZ, s, flops);
    for (void* p : {static_cast<void*>(dd), static_cast<void*>(dg), static_cast<void*>(dk), static_cast<void*>(dt),
                    static_cast<void*>(dr), static_cast<void*>(rm), static_cast<void*>(ap), static_cast<void*>(bp)})
      dev_free(p);
    return check_cuda(cudaGetLastError(), "f64tc gemm launch");
  }
  if (precision == XGB_PREC_3XTF32 || precision == XGB_PREC_BF16X9) {
    const int form = precision == XGB_PREC_BF16X9 ? 1 : 0;
    TcPlanHost tp = build_tc_plan(descs, n_groups, form);
    if (tp.tiles.empty()) return XGB_OK;
    double flops = 0;
    for (int g = 0; g < n_groups; ++g) flops += 2.0 * double(descs[g].m) * double(descs[g].n) * double(descs[g].k);
    auto* dd = upload(descs, size_t(n_groups), s);
    auto* dg = upload(tp.groups.data(), tp.groups.size(), s);
    auto* dk = upload(tp.tasks.data(), tp.tasks.size(), s);
    auto* dt = upload(tp.tiles.data(), tp.tiles.size(), s);
    auto* ap = static_cast<float*>(dev_alloc(sizeof(float) * size_t(std::max<int64_t>(tp.a_floats, 4))));
    auto* bp = static_cast<float*>(dev_alloc(sizeof(float) * size_t(std::max<int64_t>(tp.b_floats, 4))));
    prof_begin(K_GEMM_TC, s);
    launch_gemm_tc(dd, dg, dk, int(tp.tasks.size()), dt, int(tp.tiles.size()), A, B, ap, bp, C, alpha, beta, s, form);
    prof_end(K_GEMM_TC, s, flops);
    for (void* p : {static_cast<void*>(dd), static_cast<void*>(dg), static_cast<void*>(dk), static_cast<void*>(dt),
                    static_cast<void*>(ap), static_cast<void*>(bp)})
      dev_free(p);
    return check_cuda(cudaGetLastError(), "tensor-core gemm launch");
  }
  const int tile = choose_gemm_tile(descs, n_groups);
  if (precision == XGB_PREC_FP64) {
    // FP64: the built-in shape (no split-K) or, with autotuning on, the tuned one of the list's bucket
    const F64Config cfg = gemm_f64_config(descs, n_groups, A, B, {tile, 0}, s);
    run_gemm_f64_config(descs, n_groups, cfg, A, B, C, alpha, beta, s);
    return check_cuda(cudaGetLastError(), "gemm launch");
  }
  std::vector<GemmTile> tiles;
  for (int g = 0; g < n_groups; ++g) {
    int64_t tm = (descs[g].m + tile - 1) / tile, tn = (descs[g].n + tile - 1) / tile;
    for (int64_t j = 0; j < tn; ++j)
      for (int64_t i = 0; i < tm; ++i) tiles.push_back({g, int32_t(i), int32_t(j), tile});
  }
  if (tiles.empty()) return XGB_OK;
  order_tiles_by_work(tiles, descs);
  auto* dd = upload(descs, size_t(n_groups), s);
  auto* dt = upload(tiles.data(), tiles.size(), s);
  double flops = 0;  // XGB_PREC_FP32 (the other forms returned above)
  for (int g = 0; g < n_groups; ++g) flops += 2.0 * double(descs[g].m) * double(descs[g].n) * double(descs[g].k);
  prof_begin(K_GEMM_F32, s);
  launch_gemm_f32(dd, dt, int(tiles.size()), tile, A, B, C, alpha, beta, s);
  prof_end(K_GEMM_F32, s, flops);
  dev_free(dd);
  dev_free(dt);
  return check_cuda(cudaGetLastError(), "gemm launch");
  XGB_GUARD_END
}

int xgb_gemm_tc_status(void) {
  XGB_REQUIRE_INIT();
  XGB_GUARD_BEGIN
  cudaStreamSynchronize(stream());
  return gemm_tc_error(true) ? set_error(XGB_E_TIMEOUT, "tensor-core GEMM: a CTA gave up waiting for its MMAs") : XGB_OK;
  XGB_GUARD_END
}

int xgb_permute(int n_tasks, const xgb_perm_task* tasks, int n_contrib, const xgb_perm_contrib* contribs,
                const double* src, double* dst, void* stream_) {
  XGB_REQUIRE_INIT();
  XGB_GUARD_BEGIN
  cudaStream_t s = pick(stream_);
  for (int t = 0; t < n_tasks; ++t) {
    if (tasks[t].rank < 0 || tasks[t].rank > XGB_MAX_LEGS) return set_error(XGB_E_BADPLAN, "task rank out of range");
    if (tasks[t].contrib0 < 0 || tasks[t].contrib0 + tasks[t].n_contrib > n_contrib)
      return set_error(XGB_E_BADPLAN, "contribution index out of range");
    int64_t prod = 1;
    for (int k = 0; k < tasks[t].rank; ++k) {
      if (tasks[t].dims[k] <= 0) return set_error(XGB_E_BADPLAN, "task extent must be positive");
      prod *= tasks[t].dims[k];
    }
    if (prod != tasks[t].nelem) return set_error(XGB_E_BADPLAN, "task nelem differs from the product of its extents");
  }
  if (n_tasks == 0) return XGB_OK;
  const PermRows rows = perm_rows(tasks, n_tasks, contribs, n_contrib);
  if (rows.total_rows == 0) return XGB_OK;
  auto* dt = upload(tasks, size_t(n_tasks), s);
  auto* ds = upload(rows.row_start.data(), rows.row_start.size(), s);
  auto* dc = upload(contribs, size_t(n_contrib), s);
  launch_permute(dt, ds, n_tasks, rows.total_rows, rows.group, rows.narrow, rows.single, dc, src, dst, s);
  dev_free(dt);
  dev_free(ds);
  dev_free(dc);
  return check_cuda(cudaGetLastError(), "permute launch");
  XGB_GUARD_END
}

size_t xgb_svd_workspace_bytes(int n, const xgb_svd_desc* descs) {
  size_t e = 0;
  for (int i = 0; i < n; ++i) e += svd_work_elems(descs[i].m, descs[i].n);
  return e * sizeof(double);
}

int xgb_batched_svd(int n, const xgb_svd_desc* descs, const double* A, double* U, double* S, double* Vt, void* work,
                    void* stream_) {
  XGB_REQUIRE_INIT();
  XGB_GUARD_BEGIN
  cudaStream_t s = pick(stream_);
  std::vector<int64_t> off(size_t(std::max(n, 0)), 0);
  int64_t acc = 0, maxk = 0;
  for (int i = 0; i < n; ++i) {
    if (descs[i].m < 0 || descs[i].n < 0) return set_error(XGB_E_BADPLAN, "negative SVD extent");
    off[i] = acc;
    acc += int64_t(svd_work_elems(descs[i].m, descs[i].n));
    maxk = std::max(maxk, std::min(descs[i].m, descs[i].n));
  }
  if (maxk > 8192) return set_error(XGB_E_UNSUPPORTED, "SVD block larger than 8192 columns");
  if (n == 0) return XGB_OK;
  auto* dd = upload(descs, size_t(n), s);
  auto* dof = upload(off.data(), off.size(), s);
  launch_svd(dd, descs, dof, n, maxk, A, U, S, Vt, static_cast<double*>(work), s);
  dev_free(dd);
  dev_free(dof);
  return check_cuda(cudaGetLastError(), "svd launch");
  XGB_GUARD_END
}

int xgb_truncate(int n_sectors, const int64_t* s_begin_host, const int32_t* degeneracy_host, const double* s,
                 int64_t max_keep, double eps_svd, int preserve_multiplets, int32_t* keep_dev, double* out2_dev,
                 void* stream_) {
  XGB_REQUIRE_INIT();
  XGB_GUARD_BEGIN
  if (n_sectors <= 0) return set_error(XGB_E_BADPLAN, "truncation needs at least one sector");
  cudaStream_t st = pick(stream_);
  const int64_t total = s_begin_host[n_sectors];
  if (total <= 0) return set_error(XGB_E_BADPLAN, "no singular values");
  auto* db = upload(s_begin_host, size_t(n_sectors) + 1, st);
  auto* dg = upload(degeneracy_host, size_t(n_sectors), st);
  launch_truncate(n_sectors, db, dg, s, total, max_keep, eps_svd, preserve_multiplets, keep_dev, out2_dev, st);
  dev_free(db);
  dev_free(dg);
  return check_cuda(cudaGetLastError(), "truncate launch");
  XGB_GUARD_END
}

size_t xgb_qr_workspace_bytes(int n, const xgb_qr_desc* descs) {
  size_t e = 0;
  for (int i = 0; i < n; ++i) e += qr_work_elems(descs[i].m, descs[i].n);
  return e * sizeof(double);
}

int xgb_batched_qr(int n, const xgb_qr_desc* descs, const double* A, double* Q, double* R, void* work, void* stream_) {
  XGB_REQUIRE_INIT();
  XGB_GUARD_BEGIN
  cudaStream_t s = pick(stream_);
  std::vector<int64_t> off(size_t(std::max(n, 0)), 0);
  int64_t acc = 0;
  for (int i = 0; i < n; ++i) {
    off[i] = acc;
    acc += int64_t(qr_work_elems(descs[i].m, descs[i].n));
  }
  if (n == 0) return XGB_OK;
  auto* dd = upload(descs, size_t(n), s);
  auto* dof = upload(off.data(), off.size(), s);
  launch_qr(dd, dof, n, A, Q, R, static_cast<double*>(work), s);
  dev_free(dd);
  dev_free(dof);
  return check_cuda(cudaGetLastError(), "qr launch");
  XGB_GUARD_END
}

int xgb_absmax(const double* x, int64_t n, double* out_dev, void* stream_) {
  XGB_REQUIRE_INIT();
  launch_absmax(x, n, out_dev, pick(stream_));
  return check_cuda(cudaGetLastError(), "absmax launch");
}

int xgb_scale_by_inv_absmax(double* x, int64_t n, double* scratch_dev, void* stream_) {
  XGB_REQUIRE_INIT();
  cudaStream_t s = pick(stream_);
  launch_absmax(x, n, scratch_dev, s);
  launch_scale_by_inv(x, n, scratch_dev, s);
  return check_cuda(cudaGetLastError(), "scale launch");
}

int xgb_scale(double* x, int64_t n, double alpha, void* stream_) {
  XGB_REQUIRE_INIT();
  launch_scale(x, n, alpha, pick(stream_));
  return check_cuda(cudaGetLastError(), "scale launch");
}

int xgb_copy2d_batched(int n, const xgb_copy2d_desc* descs, const double* src, double* dst, void* stream_) {
  XGB_REQUIRE_INIT();
  XGB_GUARD_BEGIN
  if (n <= 0) return XGB_OK;
  cudaStream_t s = pick(stream_);
  int64_t mx = 0;
  for (int i = 0; i < n; ++i) mx = std::max(mx, descs[i].rows * descs[i].cols);
  auto* dd = upload(descs, size_t(n), s);
  launch_copy2d(dd, n, mx, src, dst, s);
  dev_free(dd);
  return check_cuda(cudaGetLastError(), "copy2d launch");
  XGB_GUARD_END
}

int xgb_diag_from_vec(int n, const xgb_copy2d_desc* descs, int fn, const double* src, double* dst, void* stream_) {
  XGB_REQUIRE_INIT();
  XGB_GUARD_BEGIN
  if (n <= 0) return XGB_OK;
  cudaStream_t s = pick(stream_);
  int64_t mx = 0;
  for (int i = 0; i < n; ++i) mx = std::max(mx, descs[i].rows);
  auto* dd = upload(descs, size_t(n), s);
  launch_diag_from_vec(dd, n, mx, fn, src, dst, s);
  dev_free(dd);
  return check_cuda(cudaGetLastError(), "diag launch");
  XGB_GUARD_END
}

int xgb_diag_apply(int n, const xgb_copy2d_desc* descs, int fn, double* x, void* stream_) {
  XGB_REQUIRE_INIT();
  XGB_GUARD_BEGIN
  if (n <= 0) return XGB_OK;
  cudaStream_t s = pick(stream_);
  int64_t mx = 0;
  for (int i = 0; i < n; ++i) mx = std::max(mx, std::max(descs[i].rows, descs[i].cols));
  auto* dd = upload(descs, size_t(n), s);
  launch_diag_apply(dd, n, mx, fn, x, s);
  dev_free(dd);
  return check_cuda(cudaGetLastError(), "diag launch");
  XGB_GUARD_END
}

}  // extern "C"
