// Kernels of the randomized blockwise tSVD: the seeded Gaussian test
// matrices and the singular-vector sign convention applied after the
// sketch-space singular vectors are lifted back (U = Q U_B).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "kernels.hpp"

namespace xgb {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  // splitmix64 finaliser (Steele, Lea, Flood 2014)
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Standard normal number `e` of stream `stream` under `seed`: Box-Muller on
// two counter-hashed uniforms u1 in (0, 1], u2 in [0, 1).
__device__ double gauss_at(uint64_t seed, uint64_t stream, uint64_t e) {
  const uint64_t base = mix64(seed ^ mix64(stream));
  const uint64_t h1 = mix64(base ^ (2 * e)), h2 = mix64(base ^ (2 * e + 1));
  const double u1 = double((h1 >> 11) + 1) * 0x1.0p-53;
  const double u2 = double(h2 >> 11) * 0x1.0p-53;
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

__global__ void gauss_fill_kernel(const GaussBlock* __restrict__ blocks, int n_blocks, uint64_t seed,
                                  double* __restrict__ out) {
  const GaussBlock b = blocks[blockIdx.y];
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < b.count; e += int64_t(gridDim.x) * blockDim.x)
    out[b.offset + e] = gauss_at(seed, uint64_t(b.stream), uint64_t(e));
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Same rule as the batched SVD kernel: s = sign(r . u) with
// r_i = frac((i+1) * 0.7548776662466927) + 0.25, or the sign of the first
// largest-magnitude entry when |r . u| <= 1e-8 sum_i r_i |u_i|.
__global__ void sign_fix_kernel(const SignFixDesc* __restrict__ descs, double* __restrict__ U, double* __restrict__ Vt) {
  const SignFixDesc d = descs[blockIdx.y];
  const int lane = threadIdx.x & 31;
  const int64_t j = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= d.k) return;
  double* u = U + d.u_off + j * d.m;
  double dot = 0, mag = 0, best = -1, bval = 0;
  long long bidx = 0;
  for (int64_t i = lane; i < d.m; i += 32) {
    const double x = u[i];
    const double y = double(i + 1) * 0.7548776662466927;
    const double r = (y - floor(y)) + 0.25;
    dot = fma(r, x, dot);
    mag = fma(r, fabs(x), mag);
    if (fabs(x) > best) { best = fabs(x); bval = x; bidx = i; }
  }
  dot = warp_sum_d(dot);
  mag = warp_sum_d(mag);
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const double ov = __shfl_xor_sync(0xffffffffu, bval, o);
    const long long oi = __shfl_xor_sync(0xffffffffu, bidx, o);
    if (ob > best || (ob == best && oi < bidx)) { best = ob; bval = ov; bidx = oi; }
  }
  const bool neg = fabs(dot) > 1.0e-8 * mag ? dot < 0 : bval < 0;
  if (!neg) return;
  for (int64_t i = lane; i < d.m; i += 32) u[i] = -u[i];
  double* v = Vt + d.v_off + j;
  for (int64_t c = lane; c < d.n; c += 32) v[c * d.k] = -v[c * d.k];
}

// dst[d.dst_off + c + j * d.dst_ld] = src[d.src_off + j + c * d.src_ld] for j < rows, c < cols
// (descriptor: rows = k rows of the source block, cols = n its columns)
__global__ void transpose_copy_kernel(const xgb_copy2d_desc* __restrict__ descs, const double* __restrict__ src,
                                      double* __restrict__ dst) {
  const xgb_copy2d_desc d = descs[blockIdx.y];
  const int64_t ne = d.rows * d.cols;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < ne; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = e % d.cols, j = e / d.cols;  // consecutive threads write consecutive dst rows
    dst[d.dst_off + c + j * d.dst_ld] = src[d.src_off + j + c * d.src_ld];
  }
}

// res[out_off + j] = || R[:, j] - s_j U[:, j] ||_2 for the k columns of one
// sector (R = A V, one warp per column); descriptor fields reused from
// SignFixDesc: m rows, k columns, u_off (U and R share offsets), v_off = s_off,
// n = out_off.
__global__ void residual_norms_kernel(const SignFixDesc* __restrict__ descs, const double* __restrict__ R,
                                      const double* __restrict__ U, const double* __restrict__ S,
                                      double* __restrict__ res) {
  const SignFixDesc d = descs[blockIdx.y];
  const int lane = threadIdx.x & 31;
  const int64_t j = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= d.k) return;
  const double sj = S[d.v_off + j];
  const double* r = R + d.u_off + j * d.m;
  const double* u = U + d.u_off + j * d.m;
  double acc = 0;
  for (int64_t i = lane; i < d.m; i += 32) {
    const double x = r[i] - sj * u[i];
    acc = fma(x, x, acc);
  }
  acc = warp_sum_d(acc);
  if (lane == 0) res[d.n + j] = sqrt(acc);
}

// Middle factor of the SVD reverse rule for one k x k sector (column-major;
// S is the k x k diagonal block, s_i = S[i + i k]):
//   N  = dS + (F.X + (F.X)^T) S + S (F.Y + (F.Y)^T) - S^-1 Y^T
//   XS = X S^-1
// with F_ij = 1 / (s_j^2 - s_i^2) (d -> d / (d^2 + 1e-12) for |d| < 1e-12).
__global__ void svd_bwd_mid_kernel(const SvdBwdDesc* __restrict__ descs, const double* __restrict__ S,
                                   const double* __restrict__ X, const double* __restrict__ Y,
                                   const double* __restrict__ dS, double* __restrict__ N, double* __restrict__ XS) {
  const SvdBwdDesc d = descs[blockIdx.y];
  const int64_t k = d.k, kk = k * k;
  auto F = [&](int64_t i, int64_t j) {
    const double si = S[d.s_off + i * (k + 1)], sj = S[d.s_off + j * (k + 1)];
    const double dd = sj * sj - si * si;
    return fabs(dd) < 1e-12 ? dd / (dd * dd + 1e-12) : 1.0 / dd;
  };
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < kk; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = e % k, j = e / k;
    const double si = S[d.s_off + i * (k + 1)], sj = S[d.s_off + j * (k + 1)];
    const double xij = X[d.kk_off + i + j * k], xji = X[d.kk_off + j + i * k];
    const double yij = Y[d.kk_off + i + j * k], yji = Y[d.kk_off + j + i * k];
    const double fij = F(i, j), fji = F(j, i);
    const double jsym = fij * xij + fji * xji;  // (F.X + (F.X)^T)_ij
    const double ksym = fij * yij + fji * yji;
    N[d.kk_off + e] = dS[d.ds_off + i + j * d.ds_ld] + jsym * sj + si * ksym - yji / si;
    XS[d.kk_off + e] = xij / sj;
  }
}

// W (k x n) += S^-1 dVd  (rows scaled) and P (m x k) = dU S^-1 (columns scaled), one sector per grid row
__global__ void svd_bwd_scale_kernel(const SvdBwdDesc* __restrict__ descs, const double* __restrict__ S,
                                     const double* __restrict__ dVd, const double* __restrict__ dU,
                                     double* __restrict__ W, double* __restrict__ P) {
  const SvdBwdDesc d = descs[blockIdx.y];
  const int64_t kn = d.k * d.n, mk = d.m * d.k;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < kn + mk; e += int64_t(gridDim.x) * blockDim.x) {
    if (e < kn) {
      const int64_t i = e % d.k;
      W[d.w_off + e] += dVd[d.v_off + e] / S[d.s_off + i * (d.k + 1)];
    } else {
      const int64_t f = e - kn, j = f / d.m;
      P[d.p_off + f] = dU[d.u_off + f] / S[d.s_off + j * (d.k + 1)];
    }
  }
}

// Upper-triangular inverse factor of the Gram matrix of one sketch block, for
// CholeskyQR: G (l x l, column-major at d.g_off) = L L^T with L lower
// triangular after adding `shift` = rel_shift * (m l + l (l + 1)) * trace(G)
// to the diagonal (shifted CholeskyQR, Fukaya et al. 2020; rel_shift = 0 for
// the unshifted passes); Rinv (at the same offset) = L^-T, upper triangular,
// zeros below the diagonal.  A pivot at or below eps * trace / l (a direction
// the block does not span) becomes sqrt(eps * trace / l) with a zero column
// below it, so the factor stays finite and well scaled; such pivots are
// counted in *bad.
//
// Both factorisations are right-looking, so every step is a parallel update
// of a trailing block: Cholesky by columns (scale the column, rank-1 update of
// the trailing lower triangle), the inverse by forward elimination of the
// identity (X <- rows of L^-1 as they are finished).  Matrices live in shared
// memory, row-major with an odd leading dimension, when two of them fit;
// larger blocks use the same loops on global memory.
//
// kInverse = false: the Cholesky factor only; L (lower triangle and diagonal) is
// left column-major in G for trinv_kernel, which forms L^-1 with many CTAs.
template <bool kShared, bool kInverse>
__device__ void chol_inv_body(const CholDesc& d, double* __restrict__ Gg, double* __restrict__ Xg, double rel_shift,
                              int* __restrict__ bad, double* sm) {
  const int l = int(d.l), tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int ld = kShared ? (l | 1) : l;
  double* Ls = kShared ? sm : Gg;
  double* Xs = kShared ? sm + int64_t(ld) * l : Xg;
  // element accessors: shared row-major (ld odd) or global column-major (ld = l); symmetric G
  auto LA = [&](int i, int k) -> double& { return kShared ? Ls[i * ld + k] : Ls[i + int64_t(k) * l]; };
  auto XA = [&](int i, int k) -> double& { return kShared ? Xs[i * ld + k] : Xs[i + int64_t(k) * l]; };
  __shared__ double red[32];
  __shared__ double bcast;
  // G is read from its upper triangle (the Gram products compute only that one): LA(i, k) = G(min, max)
  if (kShared) {
    for (int e = tid; e < l * l; e += nt) {
      const int i = e % l, k = e / l;
      LA(i, k) = Gg[i <= k ? e : k + int64_t(i) * l];
    }
  } else {
    for (int e = tid; e < l * l; e += nt) {
      const int i = e % l, k = e / l;
      if (i > k) Gg[e] = Gg[k + int64_t(i) * l];
    }
  }
  if (kInverse)
    for (int e = tid; e < l * l; e += nt) XA(e % l, e / l) = (e % l == e / l) ? 1.0 : 0.0;
  __syncthreads();
  // the trace in the order of a 1024-thread block whatever blockDim is (one element per thread, butterfly
  // sums per 32 elements, added in order), so that blocks of any size give the same shift and the same bits
  __shared__ double trace_s;
  if (l <= 1024) {
    if (warp == 0) {
      double t = 0;
      for (int g0 = 0; g0 < l; g0 += 32) t += warp_sum_d(g0 + lane < l ? LA(g0 + lane, g0 + lane) : 0.0);
      if (lane == 0) trace_s = t;
    }
  } else {
    double tr = 0;
    for (int i = tid; i < l; i += nt) tr += LA(i, i);
    tr = warp_sum_d(tr);
    if (lane == 0) red[warp] = tr;
  }
  __syncthreads();
  __shared__ double floor_s;
  if (tid == 0) {
    double t = 0;
    if (l <= 1024) t = trace_s;
    else
      for (int w = 0; w < (nt >> 5); ++w) t += red[w];
    bcast = rel_shift * (double(d.m) * l + double(l) * (l + 1)) * t;
    const double avg = t > 0.0 ? t / l : 0.0;
    floor_s = fmax(2.220446049250313e-16 * avg, 1e-300);
  }
  __syncthreads();
  const double shift = bcast, dfloor = floor_s;
  for (int i = tid; i < l; i += nt) LA(i, i) += shift;
  __syncthreads();
  // Cholesky (right-looking, one column of look-ahead), lower triangle in place.  Iteration j, with
  // column j final (updated by every earlier column and scaled by its pivot's reciprocal):
  //   warp 0 finishes the diagonal element j + 1 and forms its pivot, warp 1 applies column j to the
  //   rest of column j + 1 and scales it with the pivot's reciprocal (two-warp barrier in between),
  //   warps 2.. apply column j to the trailing columns j + 2 .. l - 1,
  // and one barrier ends the iteration.  The pivot chain - on GB300 a dependent FP64 operation takes
  // ~64 cycles, sqrt ~675 and a division ~430, so the pivot is r = rsqrt(d) (~430) with L_jj = d r and
  // 1 / L_jj = r - runs beside the trailing update instead of between two barriers.  Every element sees
  // the same FMAs in the same order as in the unblocked column algorithm.
  const unsigned full_warp = 0xffffffffu;
  auto panel = [&](int c) {  // warp 0: pivot of column c and its scaling (first column); lane ln owns rows c + ln + 32 r
    double r = 0.0;
    int dd = 0;
    if (lane == 0) {
      const double dj = LA(c, c);
      dd = !(dj > dfloor);  // also true for NaN
      if (dd) atomicAdd(bad, 1);
      const double v = dd ? dfloor : dj;
      r = rsqrt(v);
      LA(c, c) = v * r;
    }
    r = __shfl_sync(full_warp, r, 0);
    dd = __shfl_sync(full_warp, dd, 0);
    for (int i = c + lane; i < l; i += 32)
      if (i > c) LA(i, c) = dd ? 0.0 : LA(i, c) * r;
    __syncwarp();
  };
  if (warp == 0 && l > 0) panel(0);
  __syncthreads();
  // warp 0 forms the next pivot (one lane: the diagonal's last FMA, then rsqrt) while warp 1 applies
  // column j to the rest of column j + 1; a two-warp barrier hands the reciprocal over for the scaling
  __shared__ double piv_r;
  __shared__ int piv_dead;
  for (int j = 0; j + 1 < l; ++j) {
    const int nc = j + 1;  // the next column
    if (warp == 0) {
      if (lane == 0) {
        const double ljj = LA(nc, j);
        const double dj = fma(-ljj, ljj, LA(nc, nc));  // row nc of the column update, as in the unblocked order
        const int dd = !(dj > dfloor);               // also true for NaN
        if (dd) atomicAdd(bad, 1);
        const double v = dd ? dfloor : dj;
        const double r = rsqrt(v);
        LA(nc, nc) = v * r;
        piv_r = r;
        piv_dead = dd;
      }
      asm volatile("bar.sync 1, 64;" ::: "memory");
    } else if (warp == 1) {
      const double ljj = LA(nc, j);
      for (int i = nc + 1 + lane; i < l; i += 32) LA(i, nc) = fma(-LA(i, j), ljj, LA(i, nc));
      asm volatile("bar.sync 1, 64;" ::: "memory");
      const double r = piv_r;
      const bool dd = piv_dead != 0;
      for (int i = nc + 1 + lane; i < l; i += 32) LA(i, nc) = dd ? 0.0 : LA(i, nc) * r;
    } else {
      // trailing lower triangle (rows i >= k >= j + 2) folded into whole columns: column c and column
      // t-1-c together hold t+1 elements; an odd t leaves the middle column alone
      const int t = l - j - 2, half = t >> 1;
      const int total = (t + 1) * half + ((t & 1) ? (t + 1) >> 1 : 0);
      for (int e = tid - 64; e < total; e += nt - 64) {
        int i, k;
        if (e < (t + 1) * half) {
          const int r = e % (t + 1), c = e / (t + 1);
          if (r < t - c) { i = c + r; k = c; } else { i = (t - 1 - c) + (r - (t - c)); k = t - 1 - c; }
        } else {
          k = (t - 1) >> 1;
          i = k + (e - (t + 1) * half);
        }
        i += j + 2;
        k += j + 2;
        LA(i, k) = fma(-LA(i, j), LA(k, j), LA(i, k));
      }
    }
    __syncthreads();
  }
  if constexpr (!kInverse) {
    if (kShared)  // L back to G, column-major, lower triangle and diagonal
      for (int e = tid; e < l * l; e += nt) {
        const int i = e % l, k = e / l;
        if (i >= k) Gg[e] = LA(i, k);
      }
    return;
  } else {
    // X = L^-1 by forward elimination of the identity: row j of X is final after
    // dividing by L[j][j]; then rows i > j subtract L[i][j] * row j (columns c <= j)
    __shared__ double inv_s[1];
    for (int j = 0; j < l; ++j) {
      if (tid == 0) inv_s[0] = 1.0 / LA(j, j);
      __syncthreads();
      const double inv = inv_s[0];
      for (int c = tid; c <= j; c += nt) XA(j, c) *= inv;
      __syncthreads();
      const int t = l - j - 1;
      for (int e = tid; e < t * (j + 1); e += nt) {
        const int i = j + 1 + e % t, c = e / t;
        XA(i, c) = fma(-LA(i, j), XA(j, c), XA(i, c));
      }
      __syncthreads();
    }
    // Rinv = X^T, column-major l x l: Rinv[c + i l] = X[i][c]
    if (kShared) {
      for (int e = tid; e < l * l; e += nt) {
        const int c = e % l, i = e / l;
        Xg[e] = XA(i, c);
      }
    } else {
      for (int e = tid; e < l * l; e += nt) {
        const int i = e % l, c = e / l;
        if (i > c) {
          const double a = Xg[i + int64_t(c) * l], b = Xg[c + int64_t(i) * l];
          Xg[i + int64_t(c) * l] = b;
          Xg[c + int64_t(i) * l] = a;
        }
      }
    }
  }
}

template <bool kInverse>
__global__ void __launch_bounds__(1024) chol_inv_kernel(const CholDesc* __restrict__ descs, double* __restrict__ G,
                                                      double* __restrict__ Rinv, double rel_shift,
                                                      int* __restrict__ bad, int smem_cap_l) {
  extern __shared__ double sm[];
  const CholDesc d = descs[blockIdx.x];
  if (d.l <= smem_cap_l)
    chol_inv_body<true, kInverse>(d, G + d.g_off, Rinv + d.g_off, rel_shift, bad, sm);
  else
    chol_inv_body<false, kInverse>(d, G + d.g_off, Rinv + d.g_off, rel_shift, bad, sm);
}

// The same shifted Cholesky as chol_inv_body<true, false> for blocks up to kCholWarpL wide, run by one
// warp per block with no block-wide barriers: the lanes own rows (i = lane + 32 j), every lane forms
// the pivot itself, and each element sees the same FMAs in the same order as in the 1024-thread
// kernel (the trace, which sets the shift, is summed in that kernel's order too), so both give the
// same bits.  For narrow blocks the 1024-thread kernel spends two block barriers per column on a few
// hundred FMAs; a lane's share grows like l^3 / 192 dependent shared-memory FMAs, so above 48 columns
// (measured: ~390 us per launch at widths up to 128, against ~110 us) the block kernel is used.
constexpr int kCholWarpL = 48;
__global__ void __launch_bounds__(32) chol_warp_kernel(const CholDesc* __restrict__ descs, double* __restrict__ G,
                                                       double rel_shift, int* __restrict__ bad) {
  extern __shared__ double wsm[];
  const CholDesc d = descs[blockIdx.x];
  const int l = int(d.l), lane = threadIdx.x, ld = l | 1;
  double* Gg = G + d.g_off;
  auto LA = [&](int i, int k) -> double& { return wsm[i * ld + k]; };
  for (int e = lane; e < l * l; e += 32) {  // upper triangle of G, as in chol_inv_body
    const int i = e % l, k = e / l;
    LA(i, k) = Gg[i <= k ? e : k + i * l];
  }
  __syncwarp();
  double t = 0;
  for (int g0 = 0; g0 < l; g0 += 32) t += warp_sum_d(g0 + lane < l ? LA(g0 + lane, g0 + lane) : 0.0);
  const double shift = rel_shift * (double(d.m) * l + double(l) * (l + 1)) * t;
  const double avg = t > 0.0 ? t / l : 0.0;
  const double dfloor = fmax(2.220446049250313e-16 * avg, 1e-300);
  for (int i = lane; i < l; i += 32) LA(i, i) += shift;
  __syncwarp();
  for (int j = 0; j < l; ++j) {
    const double dj = LA(j, j);
    const int dd = !(dj > dfloor);  // also true for NaN
    const double v = dd ? dfloor : dj;
    const double inv = rsqrt(v);
    const double p = v * inv;
    __syncwarp();
    if (lane == 0) {
      LA(j, j) = p;
      if (dd) atomicAdd(bad, 1);
    }
    for (int i = j + 1 + lane; i < l; i += 32) LA(i, j) = dd ? 0.0 : LA(i, j) * inv;
    __syncwarp();
    for (int i = j + 1 + lane; i < l; i += 32)
      for (int k = j + 1; k <= i; ++k) LA(i, k) = fma(-LA(i, j), LA(k, j), LA(i, k));
    __syncwarp();
  }
  for (int e = lane; e < l * l; e += 32) {
    const int i = e % l, k = e / l;
    if (i >= k) Gg[e] = LA(i, k);
  }
}

// Rinv = L^-T from the Cholesky factor L (column-major, lower triangle, in G): one warp per
// column c of X = L^-1, kTrinvCols columns per CTA, so the l^3/6 FMAs of a block spread over
// ceil(l / kTrinvCols) SMs.  Column c by forward substitution in the same operation order as
// the single-CTA elimination (x_k = r_k * (1 / L_kk), then r_i -= L_ik x_k for i > k), so
// both give the same bits; lane t keeps r_i for i = t + 32 j in registers (j < T).
constexpr int kTrinvCols = 8;
constexpr int kTrinvStageL = 150;  // trailing factor staged in shared memory up to this width (176 KB)
template <int T, bool kStaged>
__global__ void __launch_bounds__(32 * kTrinvCols) trinv_kernel(const CholDesc* __restrict__ descs, int chunks,
                                                                 const double* __restrict__ G,
                                                                 double* __restrict__ Rinv) {
  extern __shared__ double tsm[];
  const int sector = blockIdx.x / chunks, c0 = (blockIdx.x % chunks) * kTrinvCols;
  const CholDesc d = descs[sector];
  const int l = int(d.l);
  if (c0 >= l) return;  // uniform over the CTA
  const int lt = l - c0;  // trailing order: rows / columns c0 .. l-1 are all this CTA reads
  double* inv_diag = tsm;
  const double* L = G + d.g_off;
  double* R = Rinv + d.g_off;
  for (int k = c0 + int(threadIdx.x); k < l; k += blockDim.x) inv_diag[k - c0] = 1.0 / L[k + int64_t(k) * l];
  // staged: column k of the trailing factor at Ls + (k - c0) * lt, rows c0 .. l-1
  double* Ls = tsm + lt;
  if (kStaged)
    for (int e = threadIdx.x; e < lt * lt; e += blockDim.x) {
      const int i = e % lt, k = e / lt;
      Ls[e] = i >= k ? L[(c0 + i) + int64_t(c0 + k) * l] : 0.0;
    }
  __syncthreads();
  const int lane = threadIdx.x & 31, c = c0 + int(threadIdx.x >> 5);
  if (c >= l) return;
  double r[T];
#pragma unroll
  for (int j = 0; j < T; ++j) r[j] = (lane + 32 * j == c) ? 1.0 : 0.0;
  for (int k = c; k < l; ++k) {
    const int slot = k >> 5;
    double v = 0.0;
#pragma unroll
    for (int j = 0; j < T; ++j)
      if (j == slot) v = r[j];
    const double xk = __shfl_sync(0xffffffffu, v, k & 31) * inv_diag[k - c0];
    // column k of L: staged rows start at c0, global rows at 0
    const double* Lk = kStaged ? Ls + int64_t(k - c0) * lt : L + int64_t(k) * l;
    const int base = kStaged ? c0 : 0;
#pragma unroll
    for (int j = 0; j < T; ++j) {
      if (32 * j + 31 < k) continue;  // warp-uniform: rows of this slot are all finished
      const int i = lane + 32 * j;
      if (i == k) r[j] = xk;
      else if (i > k && i < l) r[j] = fma(-(kStaged ? Lk[i - base] : __ldg(Lk + i)), xk, r[j]);
    }
  }
  // row c of Rinv (= column c of X): Rinv[c + i l] = X[i][c], zero for i < c
#pragma unroll
  for (int j = 0; j < T; ++j) {
    const int i = lane + 32 * j;
    if (i < l) R[c + int64_t(i) * l] = i >= c ? r[j] : 0.0;
  }
}

}  // namespace

void launch_chol_inv(const CholDesc* d_descs, int n, int64_t max_l, double* G, double* Rinv, double rel_shift,
                     int* bad, cudaStream_t s) {
  if (n <= 0 || max_l <= 0) return;
  static std::once_flag attr;
  // Cholesky alone: one l x (l | 1) matrix in shared memory up to l = 167 (< 227 KB)
  constexpr int kCapChol = 167;
  // Cholesky and inverse in one CTA (blocks wider than the register-resident inverse allows):
  // two matrices up to l = 119
  constexpr int kCapBoth = 119;
  constexpr int kBytesChol = kCapChol * (kCapChol | 1) * int(sizeof(double));
  constexpr int kBytesBoth = 2 * kCapBoth * (kCapBoth | 1) * int(sizeof(double));
  std::call_once(attr, [] {
    cudaFuncSetAttribute(chol_inv_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBytesChol);
    cudaFuncSetAttribute(chol_inv_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBytesBoth);
  });
  if (max_l > 64 * 32) {
    chol_inv_kernel<true><<<n, 1024, kBytesBoth, s>>>(d_descs, G, Rinv, rel_shift, bad, kCapBoth);
    count_launch();
    return;
  }
  if (max_l <= kCholWarpL) {
    static std::once_flag wattr;
    std::call_once(wattr, [] {
      cudaFuncSetAttribute(chol_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kCholWarpL * (kCholWarpL | 1) * int(sizeof(double)));
    });
    const int lw = int(max_l);
    chol_warp_kernel<<<n, 32, lw * (lw | 1) * int(sizeof(double)), s>>>(d_descs, G, rel_shift, bad);
  } else {
    // 1024 threads: the rank-1 update of a column is spread thinnest (measured: 128 / 256 threads per block
    // made the CTM step's factorisations 55 % slower at widths 48-130)
    const int lc = int(std::min<int64_t>(max_l, kCapChol));
    chol_inv_kernel<false><<<n, 1024, lc * (lc | 1) * int(sizeof(double)), s>>>(d_descs, G, Rinv, rel_shift, bad,
                                                                                  kCapChol);
  }
  count_launch();
  const int chunks = int((max_l + kTrinvCols - 1) / kTrinvCols);
  if (max_l <= kTrinvStageL) {
    static std::once_flag tattr;
    std::call_once(tattr, [] {
      for (auto f : {trinv_kernel<4, true>, trinv_kernel<8, true>})
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(sizeof(double)) * kTrinvStageL * (kTrinvStageL + 1));
    });
    const size_t sm = sizeof(double) * size_t(max_l) * size_t(max_l + 1);
    if (max_l <= 128)
      trinv_kernel<4, true><<<n * chunks, 32 * kTrinvCols, sm, s>>>(d_descs, chunks, G, Rinv);
    else
      trinv_kernel<8, true><<<n * chunks, 32 * kTrinvCols, sm, s>>>(d_descs, chunks, G, Rinv);
  } else {
    const size_t sm = sizeof(double) * size_t(max_l);
    if (max_l <= 256)
      trinv_kernel<8, false><<<n * chunks, 32 * kTrinvCols, sm, s>>>(d_descs, chunks, G, Rinv);
    else if (max_l <= 512)
      trinv_kernel<16, false><<<n * chunks, 32 * kTrinvCols, sm, s>>>(d_descs, chunks, G, Rinv);
    else if (max_l <= 1024)
      trinv_kernel<32, false><<<n * chunks, 32 * kTrinvCols, sm, s>>>(d_descs, chunks, G, Rinv);
    else
      trinv_kernel<64, false><<<n * chunks, 32 * kTrinvCols, sm, s>>>(d_descs, chunks, G, Rinv);
  }
  count_launch();
}

void launch_svd_bwd_mid(const SvdBwdDesc* d_descs, int n, int64_t max_kk, const double* S, const double* X,
                        const double* Y, const double* dS, double* N, double* XS, cudaStream_t s) {
  if (n <= 0 || max_kk <= 0) return;
  const int64_t want = (max_kk + 255) / 256;
  dim3 grid(unsigned(want < 1024 ? want : 1024), unsigned(n));
  svd_bwd_mid_kernel<<<grid, 256, 0, s>>>(d_descs, S, X, Y, dS, N, XS);
  count_launch();
}

void launch_svd_bwd_scale(const SvdBwdDesc* d_descs, int n, int64_t max_elems, const double* S, const double* dVd,
                          const double* dU, double* W, double* P, cudaStream_t s) {
  if (n <= 0 || max_elems <= 0) return;
  const int64_t want = (max_elems + 255) / 256;
  dim3 grid(unsigned(want < 1024 ? want : 1024), unsigned(n));
  svd_bwd_scale_kernel<<<grid, 256, 0, s>>>(d_descs, S, dVd, dU, W, P);
  count_launch();
}

void launch_residual_norms(const SignFixDesc* d_descs, int n, int64_t max_k, const double* R, const double* U,
                           const double* S, double* res, cudaStream_t s) {
  if (n <= 0 || max_k <= 0) return;
  dim3 grid(unsigned((max_k + 7) / 8), unsigned(n));
  residual_norms_kernel<<<grid, 256, 0, s>>>(d_descs, R, U, S, res);
  count_launch();
}

void launch_transpose_copy(const xgb_copy2d_desc* d_descs, int n, int64_t max_elems, const double* src, double* dst,
                           cudaStream_t s) {
  if (n <= 0 || max_elems <= 0) return;
  const int64_t want = (max_elems + 255) / 256;
  dim3 grid(unsigned(want < 1024 ? want : 1024), unsigned(n));
  transpose_copy_kernel<<<grid, 256, 0, s>>>(d_descs, src, dst);
  count_launch();
}

void launch_gauss_fill(const GaussBlock* d_blocks, int n_blocks, int64_t max_count, uint64_t seed, double* out,
                       cudaStream_t s) {
  if (n_blocks <= 0 || max_count <= 0) return;
  const int64_t want = (max_count + 255) / 256;
  dim3 grid(unsigned(want < 1024 ? want : 1024), unsigned(n_blocks));
  gauss_fill_kernel<<<grid, 256, 0, s>>>(d_blocks, n_blocks, seed, out);
  count_launch();
}

void launch_sign_fix(const SignFixDesc* d_descs, int n, int64_t max_k, double* U, double* Vt, cudaStream_t s) {
  if (n <= 0 || max_k <= 0) return;
  dim3 grid(unsigned((max_k + 7) / 8), unsigned(n));
  sign_fix_kernel<<<grid, 256, 0, s>>>(d_descs, U, Vt);
  count_launch();
}

}  // namespace xgb
