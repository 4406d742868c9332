// Split-precision grouped GEMM on the 5th-generation tensor cores.
//
// C_g = alpha op(A_g) op(B_g) + beta C_g for FP64 column-major blocks, with
// the products taken as three TF32 tensor-core products per K slice
// (3xTF32): every FP64 operand x is split in the kernel into
// hi = tf32(x) and lo = tf32(x - hi), and C ~ Ahi Bhi + Ahi Blo + Alo Bhi
// is accumulated in FP32 in tensor memory (TMEM).  The dropped Alo Blo term
// and the TF32 rounding of lo bound the product error near 2^-21 of |A||B|.
//
// One CTA computes one 128 x 128 output tile: threads load FP64 K slices of
// 32, split them and store the four operand tiles (Ahi, Alo, Bhi, Blo) into
// shared memory in the K-major, unswizzled canonical layout (8-row x 16-byte
// core matrices); thread 0 issues the tcgen05.mma instructions and commits
// them to an mbarrier; two slice buffers alternate so that loading the next
// slice overlaps the tensor cores working on the current one.  The
// epilogue reads the accumulator with tcgen05.ld and writes FP64.
//
// Every mbarrier wait is bounded; on timeout the CTA records an error flag,
// skips the epilogue and still frees its TMEM.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.hpp"

namespace xgb {
namespace {

constexpr int BM = 128, BN = 128, BK = 32;
constexpr int kThreads = 256;
constexpr int kTileBytes = BM * BK * 4;                 // one operand tile (A or B, hi or lo): 16 KB
constexpr int kStageBytes = 4 * kTileBytes;             // Ahi, Alo, Bhi, Blo
constexpr int kStages = 2;
constexpr int kSmemBytes = kStages * kStageBytes + 1024;  // + alignment slack
constexpr uint32_t kTmemCols = 128;                     // FP32 accumulator, N = 128 columns
constexpr long long kSpinLimit = 1ll << 26;

// K-major canonical layout, no swizzle: element (r, k) of a 128-row tile at
// byte (k / 4) * LBO + (r / 8) * SBO + (r % 8) * 16 + (k % 4) * 4
constexpr uint32_t SBO = 128;           // next 8-row group
constexpr uint32_t LBO = (BM / 8) * 128;  // next 4-column (16-byte) K group: 2048 bytes

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFF);          // start address
  d |= uint64_t((LBO >> 4) & 0x3FFF) << 16;       // leading-dimension byte offset (K direction)
  d |= uint64_t((SBO >> 4) & 0x3FFF) << 32;       // stride-dimension byte offset (M/N direction)
  d |= uint64_t(1) << 46;                          // descriptor version for tcgen05
  // base offset 0, absolute LBO mode off, layout type 0 = no swizzle
  return d;
}

// kind::tf32 instruction descriptor: FP32 accumulate, TF32 A and B, both K-major, N = BN, M = BM
__host__ __device__ constexpr uint32_t make_idesc() {
  return (1u << 4)                       // D format F32
         | (2u << 7)                     // A format TF32
         | (2u << 10)                    // B format TF32
         | (uint32_t(BN >> 3) << 17)     // N >> 3
         | (uint32_t(BM >> 4) << 24);    // M >> 4
}

__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

// bounded wait for the completion of the phase with the given parity
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (long long it = 0; it < kSpinLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// op(X)[r][k] of a 128 x 32 slice into hi / lo tiles (rows >= rows_valid or k >= k_valid are zero)
__device__ __forceinline__ void load_split(const double* __restrict__ X, int64_t off, int64_t ld, int trans,
                                           int64_t r0, int64_t rows_valid, int64_t k0, int64_t k_valid,
                                           unsigned char* hi, unsigned char* lo) {
  for (int e = threadIdx.x; e < BM * BK; e += kThreads) {
    // consecutive threads walk the contiguous direction of the stored block
    int r, k;
    if (!trans) { r = e % BM; k = e / BM; } else { k = e % BK; r = e / BK; }
    const int64_t gr = r0 + r, gk = k0 + k;
    double x = 0.0;
    if (gr < rows_valid && gk < k_valid) x = trans ? X[off + gk + gr * ld] : X[off + gr + gk * ld];
    const float h = to_tf32(float(x));
    const float l = to_tf32(float(x - double(h)));
    const uint32_t b = uint32_t(k >> 2) * LBO + uint32_t(r >> 3) * SBO + uint32_t(r & 7) * 16 + uint32_t(k & 3) * 4;
    *reinterpret_cast<float*>(hi + b) = h;
    *reinterpret_cast<float*>(lo + b) = l;
  }
}

__global__ void __launch_bounds__(kThreads, 1)
    gemm_tc_kernel(const xgb_gemm_desc* __restrict__ descs, const GemmTile* __restrict__ tiles,
                   const double* __restrict__ A, const double* __restrict__ B, double* __restrict__ C, double alpha,
                   double beta, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t bars[kStages];
  __shared__ uint32_t tmem_slot;
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));

  const GemmTile t = tiles[blockIdx.x];
  const xgb_gemm_desc d = descs[t.g];
  const int64_t m0 = int64_t(t.tm) * BM, n0 = int64_t(t.tn) * BN;
  const int warp = threadIdx.x >> 5;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  const int64_t K = d.k;
  const int nk = int((K + BK - 1) / BK);
  uint32_t parity[kStages] = {0, 0};
  bool ok = true;
  const uint32_t idesc = make_idesc();

  for (int kc = 0; kc < nk && ok; ++kc) {
    const int s = kc % kStages;
    unsigned char* st = smem + s * kStageBytes;
    if (kc >= kStages) {  // the MMAs of slice kc - 2 read this buffer
      if (!mbar_wait(&bars[s], parity[s])) ok = false;
      parity[s] ^= 1u;
    }
    if (!__syncthreads_and(ok)) { ok = false; break; }
    const int64_t k0 = int64_t(kc) * BK;
    load_split(A, d.a_off, d.lda, d.trans_a, m0, d.m, k0, K, st, st + kTileBytes);
    load_split(B, d.b_off, d.ldb, !d.trans_b, n0, d.n, k0, K, st + 2 * kTileBytes, st + 3 * kTileBytes);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = smem_u32(st);
      const uint32_t ahi = base, alo = base + kTileBytes, bhi = base + 2 * kTileBytes, blo = base + 3 * kTileBytes;
#pragma unroll
      for (int kk = 0; kk < BK / 8; ++kk) {
        const uint32_t ko = uint32_t(kk) * 2 * LBO;  // 8 TF32 = two 16-byte K groups
        const uint32_t first = (kc == 0 && kk == 0) ? 0u : 1u;
        mma_tf32(tmem, make_desc(ahi + ko), make_desc(bhi + ko), idesc, first);
        mma_tf32(tmem, make_desc(ahi + ko), make_desc(blo + ko), idesc, 1u);
        mma_tf32(tmem, make_desc(alo + ko), make_desc(bhi + ko), idesc, 1u);
      }
      mma_commit(&bars[s]);
    }
  }
  // drain: wait for every outstanding commit
  for (int kc = (nk > kStages ? nk - kStages : 0); kc < nk; ++kc) {
    const int s = kc % kStages;
    if (ok && !mbar_wait(&bars[s], parity[s])) ok = false;
    parity[s] ^= 1u;
  }
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (ok && nk > 0) {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, columns (w / 4) * 64 .. +63
    const int lane_grp = warp & 3, half = warp >> 2;
    const int64_t row = m0 + lane_grp * 32 + (threadIdx.x & 31);
    for (int c = 0; c < BN / 2; c += 8) {
      const int col0 = half * (BN / 2) + c;
      uint32_t v[8];
      const uint32_t taddr = tmem + (uint32_t(lane_grp * 32) << 16) + uint32_t(col0);
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                   : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                   : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < d.m) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int64_t col = n0 + col0 + j;
          if (col < d.n) {
            double* cp = C + d.c_off + row + col * d.ldc;
            const double acc = double(__uint_as_float(v[j]));
            *cp = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * *cp);
          }
        }
      }
    }
  } else if (ok && nk == 0) {
    for (int e = threadIdx.x; e < BM * BN; e += kThreads) {
      const int64_t row = m0 + e % BM, col = n0 + e / BM;
      if (row < d.m && col < d.n) {
        double* cp = C + d.c_off + row + col * d.ldc;
        *cp = beta == 0.0 ? 0.0 : beta * *cp;
      }
    }
  }
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

bool g_tc_attr = false;
int* g_tc_err = nullptr;

}  // namespace

int gemm_tc_tile() { return BM; }

void launch_gemm_tc(const xgb_gemm_desc* d_descs, const GemmTile* d_tiles, int n_tiles, const double* A,
                    const double* B, double* C, double alpha, double beta, cudaStream_t s) {
  if (n_tiles <= 0) return;
  if (!g_tc_attr) {
    cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    cudaMalloc(&g_tc_err, sizeof(int));
    cudaMemset(g_tc_err, 0, sizeof(int));
    g_tc_attr = true;
  }
  gemm_tc_kernel<<<n_tiles, kThreads, kSmemBytes, s>>>(d_descs, d_tiles, A, B, C, alpha, beta, g_tc_err);
  count_launch();
}

int gemm_tc_error(bool reset) {
  if (!g_tc_err) return 0;
  int h = 0;
  cudaMemcpy(&h, g_tc_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (reset && h) cudaMemset(g_tc_err, 0, sizeof(int));
  return h;
}

}  // namespace xgb
