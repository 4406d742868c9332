// Split-precision grouped GEMM on the 5th-generation tensor cores.
//
// C_g = alpha op(A_g) op(B_g) + beta C_g for FP64 column-major blocks, with
// the products taken as three TF32 tensor-core products (3xTF32): every FP64
// operand x is split into hi = tf32(x) and lo = tf32(x - hi), and
// C ~ Ahi Bhi + Ahi Blo + Alo Bhi is accumulated in FP32 in tensor memory
// (TMEM).  The dropped Alo Blo term and the TF32 rounding of lo bound the
// product error near 2^-21 of |A||B|.
//
// Two kernels:
//  * pack: every operand is split once into 16 KB chunks - one 128-row x
//    32-K slice, hi or lo - already in the K-major, unswizzled canonical
//    layout the MMA reads (8-row x 16-byte core matrices), zero padded past
//    the block edges.  A chunk is read through shared memory so that the
//    FP64 loads are coalesced whatever the operand's transpose.
//  * gemm: one CTA per 128 x 128 output tile.  Thread 0 streams the chunks
//    of the tile's A rows and B columns into a 3-stage shared-memory ring
//    with bulk asynchronous copies (cp.async.bulk, completion counted in
//    bytes on an mbarrier); thread 32 issues the tcgen05.mma instructions of
//    each slice and commits them to the slice's "empty" mbarrier, which
//    frees the stage for the next copy; the four warps then read the
//    accumulator with tcgen05.ld and write FP64.
//
// BF16x9 form (same kernels, templated): every FP64 operand is split into three
// BF16 pieces hi + mid + lo (8-bit significands, 24 bits together) and all nine
// products of the pieces are accumulated in FP32 with tcgen05.mma kind::f16
// (BF16 A and B), K = 16 per instruction; chunks are 8 KB (128 x 32 BF16).
//
// Every mbarrier wait is bounded; on timeout the CTA records an error flag,
// skips the epilogue and still frees its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "kernels.hpp"

namespace xgb {
namespace {

constexpr int BM = 128, BN = 128, BK = 32;
constexpr int kChunkFloats = BM * BK;               // 4096 floats = 16 KB (3xTF32 chunk)
constexpr int kChunkBytes = kChunkFloats * 4;
constexpr int kStageBytes = 4 * kChunkBytes;        // Ahi, Alo, Bhi, Blo
constexpr int kStages = 3;
constexpr int kSmemBytes = kStages * kStageBytes + 1024;  // + alignment slack (the larger of the two forms)
constexpr int kThreads = 128;

// per split form (0 = 3xTF32, 1 = BF16x9): pieces per operand, bytes per element and per chunk,
// chunk size in float units (the pack buffers are float arrays), stage bytes
template <int F> struct Form;
template <> struct Form<0> {
  static constexpr int pieces = 2, elem = 4, chunk_bytes = BM * BK * elem, chunk_units = chunk_bytes / 4;
  static constexpr int stage_bytes = 2 * pieces * chunk_bytes, kstep = 8;
};
template <> struct Form<1> {
  static constexpr int pieces = 3, elem = 2, chunk_bytes = BM * BK * elem, chunk_units = chunk_bytes / 4;
  static constexpr int stage_bytes = 2 * pieces * chunk_bytes, kstep = 16;
};
static_assert(kStages * Form<1>::stage_bytes + 1024 <= kSmemBytes, "BF16x9 stages fit the TF32 budget");
constexpr uint32_t kTmemCols = 128;                 // FP32 accumulator, N = 128 columns
constexpr long long kSpinLimit = 1ll << 26;

// K-major canonical layout, no swizzle: element (r, k) of a 128-row chunk at
// byte (k / 4) * LBO + (r / 8) * SBO + (r % 8) * 16 + (k % 4) * 4
constexpr uint32_t SBO = 128;             // next 8-row group
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

// instruction descriptor: FP32 accumulate, both operands K-major, N = BN, M = BM; A and B formats
// TF32 (code 2, kind::tf32) or BF16 (code 1, kind::f16) - always the same type for A and B
template <int F>
__host__ __device__ constexpr uint32_t make_idesc() {
  constexpr uint32_t fmt = F == 0 ? 2u : 1u;
  return (1u << 4)                       // D format F32
         | (fmt << 7)                    // A format
         | (fmt << 10)                   // B format
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

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

template <int F>
__device__ __forceinline__ void mma_form(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  if constexpr (F == 0) mma_tf32(tmem_d, adesc, bdesc, idesc, acc);
  else mma_bf16(tmem_d, adesc, bdesc, idesc, acc);
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ----------------------------------------------------------------------------- pack
// One CTA per 128-row x 32-K slice of op(A) or op(B)^T: its pieces (hi, lo or hi, mid, lo) as chunks.
template <int F>
__global__ void __launch_bounds__(256) tc_pack_kernel(const xgb_gemm_desc* __restrict__ descs,
                                                       const TcGroup* __restrict__ groups,
                                                       const TcPackTask* __restrict__ tasks,
                                                       const double* __restrict__ A, const double* __restrict__ B,
                                                       float* __restrict__ apack, float* __restrict__ bpack) {
  __shared__ double X[BM][BK + 1];
  const TcPackTask t = tasks[blockIdx.x];
  const xgb_gemm_desc d = descs[t.g];
  const TcGroup gr = groups[t.g];
  const bool isB = t.which != 0;
  const double* src = isB ? B : A;
  const int64_t off = isB ? d.b_off : d.a_off, ld = isB ? d.ldb : d.lda;
  const int64_t rows = isB ? d.n : d.m;
  // element (r, k) of the chunk is op(X)[r0 + r][k0 + k]; "rowfast" when r is the contiguous direction
  const bool rowfast = isB ? d.trans_b != 0 : d.trans_a == 0;
  const int64_t r0 = int64_t(t.tile) * BM, k0 = int64_t(t.slice) * BK;
  for (int e = threadIdx.x; e < BM * BK; e += 256) {
    int r, k;
    if (rowfast) { r = e % BM; k = e / BM; } else { k = e % BK; r = e / BK; }
    const int64_t gr_ = r0 + r, gk = k0 + k;
    double x = 0.0;
    if (gr_ < rows && gk < d.k) x = rowfast ? src[off + gr_ + gk * ld] : src[off + gk + gr_ * ld];
    X[r][k] = x;
  }
  __syncthreads();
  const int64_t chunk = (int64_t(t.tile) * gr.slices + t.slice) * Form<F>::pieces;
  float* hi = (isB ? bpack + gr.b_pack : apack + gr.a_pack) + chunk * Form<F>::chunk_units;
  if constexpr (F == 1) {
    // element (r, k) at byte (k / 8) * LBO + (r / 8) * SBO + (r % 8) * 16 + (k % 8) * 2 of each piece
    unsigned char* base = reinterpret_cast<unsigned char*>(hi);
    for (int e = threadIdx.x; e < BM * (BK / 8); e += 256) {
      const int r = e % BM, kq = e / BM;  // one 16-byte core-matrix row: 8 consecutive K of row r
      __nv_bfloat16 ph[8], pm[8], pl[8];
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        const double x = X[r][kq * 8 + kk];
        ph[kk] = __float2bfloat16_rn(float(x));
        const double r1 = x - double(__bfloat162float(ph[kk]));
        pm[kk] = __float2bfloat16_rn(float(r1));
        const double r2 = r1 - double(__bfloat162float(pm[kk]));
        pl[kk] = __float2bfloat16_rn(float(r2));
      }
      const uint32_t bo = uint32_t(kq) * LBO + uint32_t(r >> 3) * SBO + uint32_t(r & 7) * 16;
      *reinterpret_cast<uint4*>(base + bo) = *reinterpret_cast<const uint4*>(ph);
      *reinterpret_cast<uint4*>(base + Form<1>::chunk_bytes + bo) = *reinterpret_cast<const uint4*>(pm);
      *reinterpret_cast<uint4*>(base + 2 * Form<1>::chunk_bytes + bo) = *reinterpret_cast<const uint4*>(pl);
    }
    return;
  }
  float* lo = hi + kChunkFloats;
  for (int e = threadIdx.x; e < BM * (BK / 4); e += 256) {
    const int r = e % BM, kq = e / BM;  // one 16-byte core-matrix row: 4 consecutive K of row r
    float4 h, l;
    float* hp = &h.x;
    float* lp = &l.x;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const double x = X[r][kq * 4 + kk];
      hp[kk] = to_tf32(float(x));
      lp[kk] = to_tf32(float(x - double(hp[kk])));
    }
    const uint32_t fo = (uint32_t(kq) * LBO + uint32_t(r >> 3) * SBO + uint32_t(r & 7) * 16) / 4;
    *reinterpret_cast<float4*>(hi + fo) = h;
    *reinterpret_cast<float4*>(lo + fo) = l;
  }
}

// ----------------------------------------------------------------------------- gemm
// One CTA (10 warps) per 128 x 128 output tile, warp-specialised:
//  * warp 8 (lane 0) streams the A and B piece chunks of every 32-K slice into the 3-stage
//    shared-memory ring with bulk copies;
//  * warp 9 (lane 0) issues the slice's tcgen05.mma instructions into one of two 128-column TMEM
//    accumulators (slice kc into buffer kc % 2), starting that buffer from zero, and commits the slice
//    to the stage's "empty" barrier (frees the smem stage) and to the buffer's "full" barrier;
//  * warps 0-7 drain every slice: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows) and columns
//    64 (w / 4) .. + 63, adds the slice's partial products into FP32 register sums (round to nearest),
//    then releases the buffer ("acc empty", one arrival per drain warp).
// A TMEM partial therefore holds one slice's products only (12 accumulator additions for 3xTF32, 18
// for BF16x9) instead of the whole K range.  The tensor core's own accumulation loses about 2^-26 of
// the running sum per addition with a consistent sign, so an accumulator kept over k ~ 3000 drifts by
// ~3e-5; restarted every slice and summed in round-to-nearest FP32 the error stays near 5e-7 of |C|
// (with the 2^-22 operand split of 3xTF32) whatever k is.  The MMAs of slice kc + 1 run while the
// drain warps read slice kc.
constexpr int kDrainWarps = 8, kDrainCols = BN / (kDrainWarps / 4);  // 64 columns per drain warp
constexpr int kTcWarps = kDrainWarps + 2, kTcThreads = kTcWarps * 32;
constexpr int kProducerWarp = kDrainWarps, kMmaWarp = kDrainWarps + 1;
constexpr uint32_t kTmemAlloc = 2 * kTmemCols;  // two accumulator buffers

template <int F>
__global__ void __launch_bounds__(kTcThreads, 1)
    gemm_tc_kernel(const xgb_gemm_desc* __restrict__ descs, const TcGroup* __restrict__ groups,
                   const GemmTile* __restrict__ tiles, const float* __restrict__ apack,
                   const float* __restrict__ bpack, double* __restrict__ C, double alpha, double beta,
                   int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[kStages], empty[kStages], accf[2], acce[2], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int fail, issued, consumed;
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));

  const GemmTile t = tiles[blockIdx.x];
  const xgb_gemm_desc d = descs[t.g];
  const TcGroup gr = groups[t.g];
  const int64_t m0 = int64_t(t.tm) * BM, n0 = int64_t(t.tn) * BN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = gr.slices;

  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemAlloc));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], kDrainWarps);
    }
    mbar_init(&done, 1);
    fail = 0;
    issued = 0;
    consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  // drain-warp state: TMEM lane quarter (rows), column group and the FP32 sums of its 64 columns
  const int quarter = warp & 3, colq = warp >> 2;
  float sum[kDrainCols];
#pragma unroll
  for (int j = 0; j < kDrainCols; ++j) sum[j] = 0.f;

  if (nk > 0 && warp == kProducerWarp) {
    if (lane == 0) {
      // producer: bulk copies of the A and B pieces of every slice into the stage ring
      constexpr int P = Form<F>::pieces, CU = Form<F>::chunk_units, CB = Form<F>::chunk_bytes;
      const float* a_base = apack + gr.a_pack + int64_t(t.tm) * gr.slices * P * CU;
      const float* b_base = bpack + gr.b_pack + int64_t(t.tn) * gr.slices * P * CU;
      uint32_t ph[kStages] = {0, 0, 0};
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % kStages;
        if (kc >= kStages) {
          if (!mbar_wait(&empty[s], ph[s])) { atomicExch(&fail, 1); break; }
          ph[s] ^= 1u;
        }
        unsigned char* st = smem + s * Form<F>::stage_bytes;
        mbar_expect_tx(&full[s], Form<F>::stage_bytes);
        bulk_copy(st, a_base + int64_t(kc) * P * CU, P * CB, &full[s]);
        bulk_copy(st + P * CB, b_base + int64_t(kc) * P * CU, P * CB, &full[s]);
        issued = kc + 1;
      }
    }
  } else if (nk > 0 && warp == kMmaWarp) {
    if (lane == 0) {
      // MMA issuer, per K step (8 TF32 or 16 BF16 = two 16-byte K groups): 3xTF32 takes hi*hi + hi*lo +
      // lo*hi, BF16x9 all nine products of (hi, mid, lo) x (hi, mid, lo)
      constexpr int P = Form<F>::pieces, CB = Form<F>::chunk_bytes;
      const uint32_t idesc = make_idesc<F>();
      uint32_t ph[kStages] = {0, 0, 0};
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % kStages, b = kc & 1;
        if (kc >= 2 && !mbar_wait(&acce[b], uint32_t(((kc >> 1) - 1) & 1))) { atomicExch(&fail, 1); break; }
        if (!mbar_wait(&full[s], ph[s])) { atomicExch(&fail, 1); break; }
        ph[s] ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t base = smem_u32(smem + s * Form<F>::stage_bytes);
        const uint32_t acc = tmem + uint32_t(b) * kTmemCols;
        bool first = true;
#pragma unroll
        for (int kk = 0; kk < BK / Form<F>::kstep; ++kk) {
          const uint32_t ko = uint32_t(kk) * 2 * LBO;
#pragma unroll
          for (int i = 0; i < P; ++i)
#pragma unroll
            for (int j = 0; j < P; ++j) {
              if (F == 0 && i + j > 1) continue;  // 3xTF32 drops lo*lo
              mma_form<F>(acc, make_desc(base + i * CB + ko), make_desc(base + (P + j) * CB + ko), idesc,
                          first ? 0u : 1u);
              first = false;
            }
        }
        mma_commit(&empty[s]);
        mma_commit(&accf[b]);
        consumed = kc + 1;
      }
      mma_commit(&done);  // arrives when every MMA issued above has completed
    }
  } else if (nk > 0 && warp < kDrainWarps) {
    for (int kc = 0; kc < nk; ++kc) {
      const int b = kc & 1;
      // warp-uniform decision: the TMEM loads below are warp-collective
      const bool got = __all_sync(0xffffffffu, mbar_wait(&accf[b], uint32_t((kc >> 1) & 1)));
      if (!got) {
        if (lane == 0) atomicExch(&fail, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c = 0; c < kDrainCols / 8; ++c) {
        uint32_t v[8];
        const uint32_t taddr = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(b) * kTmemCols +
                               uint32_t(colq * kDrainCols + c * 8);
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                       "=r"(v[7])
                     : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 8; ++j) sum[c * 8 + j] = __fadd_rn(sum[c * 8 + j], __uint_as_float(v[j]));
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acce[b])) : "memory");
    }
  }
  // the drain warps have read every slice; make sure every MMA has retired before TMEM is freed
  bool ok = true;
  if (nk > 0) ok = mbar_wait(&done, 0);
  __syncthreads();
  ok = ok && (fail == 0);
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (ok && nk > 0 && warp < kDrainWarps) {
    const int64_t row = m0 + quarter * 32 + lane;
    if (row < d.m) {
#pragma unroll
      for (int j = 0; j < kDrainCols; ++j) {
        const int64_t col = n0 + colq * kDrainCols + j;
        if (col < d.n) {
          double* cp = C + d.c_off + row + col * d.ldc;
          const double acc = double(sum[j]);
          *cp = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * *cp);
        }
      }
    }
  } else if (ok && nk == 0) {
    for (int e = threadIdx.x; e < BM * BN; e += kTcThreads) {
      const int64_t row = m0 + e % BM, col = n0 + e / BM;
      if (row < d.m && col < d.n) {
        double* cp = C + d.c_off + row + col * d.ldc;
        *cp = beta == 0.0 ? 0.0 : beta * *cp;
      }
    }
  }
  if (!ok && threadIdx.x == 0) {
    atomicExch(err, 1);
    // copies still in flight must land before the CTA leaves: wait (bounded) for
    // every slice that was issued but not consumed
    for (int kc = consumed; kc < issued; ++kc) mbar_wait(&full[kc % kStages], uint32_t((kc / kStages) & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kMmaWarp)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemAlloc));
}

std::once_flag g_tc_attr, g_tc_err_once;
int* g_tc_err = nullptr;

}  // namespace

int gemm_tc_tile() { return BM; }

TcPlanHost build_tc_plan(const xgb_gemm_desc* descs, int n, int form) {
  TcPlanHost p;
  const int64_t per_slice = form == 1 ? Form<1>::pieces * Form<1>::chunk_units : Form<0>::pieces * Form<0>::chunk_units;
  for (int g = 0; g < n; ++g) {
    const xgb_gemm_desc& d = descs[g];
    TcGroup gr{};
    gr.a_tiles = int32_t((d.m + BM - 1) / BM);
    gr.b_tiles = int32_t((d.n + BN - 1) / BN);
    gr.slices = int32_t((d.k + BK - 1) / BK);
    gr.a_pack = p.a_floats;
    gr.b_pack = p.b_floats;
    p.a_floats += int64_t(gr.a_tiles) * gr.slices * per_slice;
    p.b_floats += int64_t(gr.b_tiles) * gr.slices * per_slice;
    for (int32_t s = 0; s < gr.slices; ++s) {
      for (int32_t t = 0; t < gr.a_tiles; ++t) p.tasks.push_back({g, t, s, 0});
      for (int32_t t = 0; t < gr.b_tiles; ++t) p.tasks.push_back({g, t, s, 1});
    }
    for (int32_t y = 0; y < gr.b_tiles; ++y)
      for (int32_t x = 0; x < gr.a_tiles; ++x) p.tiles.push_back({g, x, y, BM});
    p.groups.push_back(gr);
  }
  return p;
}

void launch_gemm_tc(const xgb_gemm_desc* d_descs, const TcGroup* d_groups, const TcPackTask* d_tasks, int n_tasks,
                    const GemmTile* d_tiles, int n_tiles, const double* A, const double* B, float* apack,
                    float* bpack, double* C, double alpha, double beta, cudaStream_t s, int form) {
  if (n_tiles <= 0) return;
  std::call_once(g_tc_attr, [] {
    cudaFuncSetAttribute(gemm_tc_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    cudaFuncSetAttribute(gemm_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  });
  gemm_tc_error_flag();
  if (form == 1) {
    if (n_tasks > 0) {
      tc_pack_kernel<1><<<n_tasks, 256, 0, s>>>(d_descs, d_groups, d_tasks, A, B, apack, bpack);
      count_launch();
    }
    gemm_tc_kernel<1><<<n_tiles, kTcThreads, kSmemBytes, s>>>(d_descs, d_groups, d_tiles, apack, bpack, C, alpha, beta,
                                                            g_tc_err);
  } else {
    if (n_tasks > 0) {
      tc_pack_kernel<0><<<n_tasks, 256, 0, s>>>(d_descs, d_groups, d_tasks, A, B, apack, bpack);
      count_launch();
    }
    gemm_tc_kernel<0><<<n_tiles, kTcThreads, kSmemBytes, s>>>(d_descs, d_groups, d_tiles, apack, bpack, C, alpha, beta,
                                                            g_tc_err);
  }
  count_launch();
}

void launch_tc_pack(const xgb_gemm_desc* d_descs, const TcGroup* d_groups, const TcPackTask* d_tasks, int n_tasks,
                    const double* A, const double* B, float* apack, float* bpack, cudaStream_t s, int form) {
  if (n_tasks <= 0) return;
  if (form == 1)
    tc_pack_kernel<1><<<n_tasks, 256, 0, s>>>(d_descs, d_groups, d_tasks, A, B, apack, bpack);
  else
    tc_pack_kernel<0><<<n_tasks, 256, 0, s>>>(d_descs, d_groups, d_tasks, A, B, apack, bpack);
  count_launch();
}

int* gemm_tc_error_flag() {
  std::call_once(g_tc_err_once, [] {
    cudaMalloc(&g_tc_err, sizeof(int));
    cudaMemset(g_tc_err, 0, sizeof(int));
  });
  return g_tc_err;
}

int gemm_tc_error(bool reset) {
  if (!g_tc_err) return 0;
  int h = 0;
  cudaMemcpy(&h, g_tc_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (reset && h) cudaMemset(g_tc_err, 0, sizeof(int));
  return h;
}

}  // namespace xgb
