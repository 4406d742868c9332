// Batched thin SVD for the truncated tSVD (sm_103a).
//
// Replaces the per-sector LAPACK/Eigen SVD of full_svd_impl
// (src/Core/Tensor.cpp:494-521, src/Interfaces/PlainInterface_Eigen_impl.cpp:114-127).
//
// Algorithm: one-sided (Hestenes) Jacobi, mixed precision, one thread-block
// CLUSTER per sector block.  GB300 executes FP64 on a narrow pipe (about two
// DFMA per clock per SM), so the FP64 work is (a) cut by first converging in
// FP32 and (b) spread over the SMs of a cluster:
//   1. W32 = op(A) in FP32, V32 = I; FP32 Jacobi sweeps until the columns of W32
//      are orthogonal to FP32 accuracy.
//   2. V64 = classical Gram-Schmidt of V32 in FP64 (V32 is orthogonal to ~1e-6,
//      so one pass gives FP64 orthogonality), W64 = op(A) V64 in FP64.
//   3. FP64 Jacobi sweeps on (W64, V64) until |w_p.w_q| <= tol |w_p||w_q|;
//      starting from nearly orthogonal columns this takes two or three sweeps.
//   4. sigma_j = |w_j|, sorted descending (ties by column), u_j = w_j/sigma_j,
//      v_j = V64[:, j]; each pair sign-normalised so the largest |u_ij| > 0.
// op(A) = A when m >= n, else A^T (then U and V swap roles).
// All CTAs of a cluster share W/V/norms in global memory (L2-resident, read
// and written with .cg so every SM sees the L2 copy); rounds of disjoint
// rotation pairs are separated by cluster barriers.  Every loop has a fixed
// bound (max sweeps), and all CTAs of a cluster take identical control flow,
// so every barrier is reached by all of them.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "kernels.hpp"

namespace cg = cooperative_groups;

namespace xgb {
namespace {

constexpr int kThreads = 256;
constexpr int kCluster = 8;
constexpr int kMaxSweeps32 = 30;
constexpr int kMaxSweeps64 = 20;

template <class T>
__device__ __forceinline__ T wsum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void rr_pair(int round, int k, int N, int& p, int& q) {
  // circle method over N (even) slots: slot 0 fixed, 1..N-1 rotate
  auto pos = [&](int i) { return (round + i) % (N - 1) + 1; };
  if (k == 0) { p = 0; q = pos(0); }
  else { p = pos(k); q = pos(N - 1 - k); }
}

__device__ __forceinline__ float ld(const float* p) { return __ldcg(p); }
__device__ __forceinline__ double ld(const double* p) { return __ldcg(p); }
__device__ __forceinline__ void st(float* p, float v) { __stcg(p, v); }
__device__ __forceinline__ void st(double* p, double v) { __stcg(p, v); }

__device__ __forceinline__ float tsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double tsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float thypot(float a, float b) { return hypotf(a, b); }
__device__ __forceinline__ double thypot(double a, double b) { return hypot(a, b); }

struct Ctx {
  int tid, lane, warp, gw, gnw, gtid, gnt;
};

// Jacobi sweeps over the columns of W (mm x nn) with V (nn x nn) accumulated.
// norms[nn] and flag live in global memory shared by the cluster.
template <class T>
__device__ int jacobi_sweeps(cg::cluster_group& cl, const Ctx& c, T* W, T* V, T* norms, int* flag, int64_t mm, int nn,
                             T tol, int max_sweeps) {
  const int N = nn + (nn & 1);
  int sweeps = 0;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    for (int j = c.gw; j < nn; j += c.gnw) {
      const T* w = W + int64_t(j) * mm;
      T a = 0;
      for (int64_t i = c.lane; i < mm; i += 32) { const T x = ld(w + i); a = fma(x, x, a); }
      a = wsum(a);
      if (c.lane == 0) st(norms + j, a);
    }
    if (cl.block_rank() == 0 && c.tid == 0) atomicExch(flag, 0);
    cl.sync();
    for (int round = 0; round < N - 1; ++round) {
      for (int k = c.gw; k < N / 2; k += c.gnw) {
        int p, q;
        rr_pair(round, k, N, p, q);
        if (p >= nn || q >= nn) continue;
        const T al = ld(norms + p), be = ld(norms + q);
        if (!(al > T(0)) || !(be > T(0))) continue;
        T* wp = W + int64_t(p) * mm;
        T* wq = W + int64_t(q) * mm;
        T ga = 0;
        for (int64_t i = c.lane; i < mm; i += 32) ga = fma(ld(wp + i), ld(wq + i), ga);
        ga = wsum(ga);
        if (fabs(ga) <= tol * tsqrt(al) * tsqrt(be)) continue;
        const T zeta = (be - al) / (T(2) * ga);
        const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + thypot(T(1), zeta));
        const T cs = T(1) / tsqrt(T(1) + t * t);
        const T sn = cs * t;
        for (int64_t i = c.lane; i < mm; i += 32) {
          const T x = ld(wp + i), y = ld(wq + i);
          st(wp + i, cs * x - sn * y);
          st(wq + i, sn * x + cs * y);
        }
        T* vp = V + int64_t(p) * nn;
        T* vq = V + int64_t(q) * nn;
        for (int i = c.lane; i < nn; i += 32) {
          const T x = ld(vp + i), y = ld(vq + i);
          st(vp + i, cs * x - sn * y);
          st(vq + i, sn * x + cs * y);
        }
        if (c.lane == 0) {
          st(norms + p, al - t * ga);
          st(norms + q, be + t * ga);
          atomicExch(flag, 1);
        }
      }
      cl.sync();
    }
    ++sweeps;
    const int any = atomicAdd(flag, 0);
    cl.sync();  // everybody has read the flag before the next sweep resets it
    if (!any) break;
  }
  return sweeps;
}

__global__ void __cluster_dims__(kCluster, 1, 1) __launch_bounds__(kThreads)
    svd_cluster_kernel(const xgb_svd_desc* __restrict__ descs, const int64_t* __restrict__ work_off,
                       const double* __restrict__ A, double* __restrict__ U, double* __restrict__ S,
                       double* __restrict__ Vt, double* __restrict__ work, int* __restrict__ sweep_stats) {
  cg::cluster_group cl = cg::this_cluster();
  const int sector = blockIdx.x / kCluster;
  const xgb_svd_desc d = descs[sector];
  const bool tr = d.m < d.n;
  const int64_t mm = tr ? d.n : d.m;
  const int nn = int(tr ? d.m : d.n);
  if (nn == 0) return;  // uniform across the cluster

  Ctx c;
  c.tid = threadIdx.x;
  c.lane = c.tid & 31;
  c.warp = c.tid >> 5;
  const int nw = kThreads / 32;
  c.gw = int(cl.block_rank()) * nw + c.warp;
  c.gnw = kCluster * nw;
  c.gtid = int(cl.block_rank()) * kThreads + c.tid;
  c.gnt = kCluster * kThreads;

  // workspace layout (doubles): W64 mm*nn | V64 nn*nn | norms64 nn | misc 8 | then floats W32 mm*nn | V32 nn*nn | norms32 nn
  double* W64 = work + work_off[sector];
  double* V64 = W64 + mm * nn;
  double* n64 = V64 + int64_t(nn) * nn;
  int* flag = reinterpret_cast<int*>(n64 + nn);
  float* W32 = reinterpret_cast<float*>(n64 + nn + 8);
  float* V32 = W32 + mm * nn;
  float* n32 = V32 + int64_t(nn) * nn;

  auto opA = [&](int64_t i, int64_t j) { return tr ? A[d.a_off + j + i * d.m] : A[d.a_off + i + j * d.m]; };

  // ---- phase 1: FP32 Jacobi
  for (int64_t e = c.gtid; e < mm * nn; e += c.gnt) st(W32 + e, float(opA(e % mm, e / mm)));
  for (int64_t e = c.gtid; e < int64_t(nn) * nn; e += c.gnt) st(V32 + e, (e % nn) == (e / nn) ? 1.f : 0.f);
  cl.sync();
  const float tol32 = 8.0f * sqrtf(float(mm)) * 6.0e-8f;
  int sw32 = nn > 1 ? jacobi_sweeps<float>(cl, c, W32, V32, n32, flag, mm, nn, tol32, kMaxSweeps32) : 0;

  // ---- phase 2: V64 = Gram-Schmidt(V32), W64 = op(A) V64
  for (int64_t e = c.gtid; e < int64_t(nn) * nn; e += c.gnt) st(V64 + e, double(ld(V32 + e)));
  cl.sync();
  for (int j = 0; j < nn; ++j) {
    double* vj = V64 + int64_t(j) * nn;
    for (int i = c.gw; i < j; i += c.gnw) {  // d_i = <v_i, v_j>
      const double* vi = V64 + int64_t(i) * nn;
      double a = 0;
      for (int r = c.lane; r < nn; r += 32) a = fma(ld(vi + r), ld(vj + r), a);
      a = wsum(a);
      if (c.lane == 0) st(n64 + i, a);
    }
    cl.sync();
    for (int r = c.gtid; r < nn; r += c.gnt) {
      double x = ld(vj + r);
      for (int i = 0; i < j; ++i) x = fma(-ld(n64 + i), ld(V64 + int64_t(i) * nn + r), x);
      st(vj + r, x);
    }
    cl.sync();
    // normalise v_j (every CTA computes the same norm redundantly: no extra barrier)
    double a = 0;
    for (int r = c.lane; r < nn; r += 32) { const double x = ld(vj + r); a = fma(x, x, a); }
    a = wsum(a);
    const double inv = a > 0 ? 1.0 / sqrt(a) : 0.0;
    cl.sync();
    for (int r = c.gtid; r < nn; r += c.gnt) st(vj + r, ld(vj + r) * inv);
    cl.sync();
  }
  for (int64_t e = c.gtid; e < mm * nn; e += c.gnt) {
    const int64_t i = e % mm, j = e / mm;
    const double* vj = V64 + j * nn;
    double acc = 0;
    for (int l = 0; l < nn; ++l) acc = fma(opA(i, l), ld(vj + l), acc);
    st(W64 + e, acc);
  }
  cl.sync();

  // ---- phase 3: FP64 Jacobi polish
  const double tol64 = 1.0e-13;
  int sw64 = nn > 1 ? jacobi_sweeps<double>(cl, c, W64, V64, n64, flag, mm, nn, tol64, kMaxSweeps64) : 0;

  // ---- phase 4: sort, sign, write
  double* sval = n64;  // reuse: exact column norms
  for (int j = c.gw; j < nn; j += c.gnw) {
    const double* w = W64 + int64_t(j) * mm;
    double a = 0;
    for (int64_t i = c.lane; i < mm; i += 32) { const double x = ld(w + i); a = fma(x, x, a); }
    a = wsum(a);
    if (c.lane == 0) st(sval + j, sqrt(a));
  }
  cl.sync();
  const int64_t k = nn;
  for (int j = c.gw; j < nn; j += c.gnw) {
    const double sj = ld(sval + j);
    int r = 0;
    for (int i = c.lane; i < nn; i += 32) {
      const double si = ld(sval + i);
      r += (si > sj) || (si == sj && i < j);
    }
    r = wsum(r);
    const double inv = sj > 0 ? 1.0 / sj : 0.0;
    const double* ucol = tr ? V64 + int64_t(j) * nn : W64 + int64_t(j) * mm;
    const double uscale = tr ? 1.0 : inv;
    const int64_t ulen = tr ? nn : mm;
    double best = -1.0, bval = 0.0;
    long long bidx = 0;
    for (int64_t i = c.lane; i < ulen; i += 32) {
      const double x = ld(ucol + i), a = fabs(x);
      if (a > best) { best = a; bval = x; bidx = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const double ov = __shfl_xor_sync(0xffffffffu, bval, o);
      const long long oi = __shfl_xor_sync(0xffffffffu, bidx, o);
      if (ob > best || (ob == best && oi < bidx)) { best = ob; bval = ov; bidx = oi; }
    }
    const double sg = (bval < 0) ? -1.0 : 1.0;
    for (int64_t i = c.lane; i < ulen; i += 32) U[d.u_off + i + int64_t(r) * d.m] = sg * uscale * ld(ucol + i);
    const double* vcol = tr ? W64 + int64_t(j) * mm : V64 + int64_t(j) * nn;
    const double vscale = tr ? inv : 1.0;
    const int64_t vlen = tr ? mm : nn;
    for (int64_t cc = c.lane; cc < vlen; cc += 32) Vt[d.vt_off + r + cc * k] = sg * vscale * ld(vcol + cc);
    if (c.lane == 0) S[d.s_off + r] = sj;
  }
  if (sweep_stats && cl.block_rank() == 0 && c.tid == 0) {
    sweep_stats[2 * sector] = sw32;
    sweep_stats[2 * sector + 1] = sw64;
  }
}

}  // namespace

size_t svd_work_elems(int64_t m, int64_t n) {
  const int64_t mm = std::max(m, n), nn = std::min(m, n);
  const int64_t doubles = mm * nn + nn * nn + nn + 8;
  const int64_t floats = mm * nn + nn * nn + nn;
  return size_t(doubles + (floats + 1) / 2 + 2);
}

void launch_svd(const xgb_svd_desc* d_descs, const int64_t* d_work_off, int n, int64_t /*max_k*/, const double* A,
                double* U, double* S, double* Vt, double* work, cudaStream_t s) {
  if (n <= 0) return;
  svd_cluster_kernel<<<n * kCluster, kThreads, 0, s>>>(d_descs, d_work_off, A, U, S, Vt, work, nullptr);
  count_launch();
}

}  // namespace xgb
