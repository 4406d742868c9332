// FP64-accurate grouped GEMM on the 5th-generation tensor cores from exact BF16 slices.
//
// C_g = alpha op(A_g) op(B_g) + beta C_g for FP64 column-major blocks.  Every row i of op(A) is
// written relative to a power of two 2^e_i above its largest entry (taken over the whole k range)
// and cut into seven balanced base-128 digits, a_ik = 2^e_i (sum_s m_s 2^(-7 s) + O(2^-50)) with
// integers |m_1| <= 128 and |m_s| <= 64 for s >= 2; every column of op(B) likewise (2^f_j).  A slice
// m_s 2^(-7 s) is exact in BF16, the product of two slices is exact in FP32, and all products of a
// "level" L = s + t share the unit 2^(-7 L).  Per k value a level adds at most 2 x 128 x 64 + 5 x 64 x 64
// = 36864 units, so a sum over 448 k values (14 K slices) stays below 2^24 and is exact in the FP32
// tensor-memory accumulator whatever order the tensor core adds in.  The row and column scales
// 2^(e_i + f_j) go into the exponent field when the tile is stored.  This is the slicing scheme of
// Ozaki, Ogita, Oishi and Rump ("Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer. Algorithms 59 (2012)), with BF16
// tcgen05.mma as the fast routine.
//
// GB300 runs FP64 arithmetic at a small fraction of its FP32 and tensor rates, so nothing here
// computes in FP64 but the one addition that joins the two FP32 halves of a result: the row
// maxima, scales and slices are integer operations on the IEEE bits.
//
// Kernels (one launch each, all groups of the list):
//  * oz_rowmax_kernel: per 128-row (A) / 64-row (B) x 32-K chunk, the largest |entry| of every row
//    into a max over the whole k range (atomicMax on the IEEE bits of a non-negative double);
//  * oz_pack_kernel: the seven slices of every chunk as BF16 in the K-major, unswizzled canonical
//    layout the MMA reads (8-row x 16-byte core matrices), zero padded past the block edges; the
//    slices come from integer arithmetic on the FP64 significand (|x| rounded to 49 bits below the
//    row's scale, balanced digits, every slice with the sign of its entry);
//  * oz_gemm_kernel: one CTA (10 warps) per 128 x 64 output tile and K range.  Warp 8 streams the
//    slices of each 32-wide K slice of the tile's rows and columns into a 2-stage shared-memory ring
//    (84 KB per stage, bulk copies counted on mbarriers); warp 9 issues, per 16-deep k step, the 28
//    BF16 MMAs of the slice pairs with s + t <= 8 into seven 64-column TMEM accumulators (one per
//    level, 448 of 512 columns); after every fourteen K slices (the exactness bound) and at the end
//    of the range warps 0-7 read the seven levels and add them into double-FP32 (hi + lo) register
//    sums, then the next chunk starts from zero.  The slice rounding (2^-50 of the row / column
//    scale), the dropped pairs (s + t > 8) and the double-FP32 sums bound the error of an element by
//    a small multiple of 2^-49 k max_k |a_ik| max_k |b_kj|: about 5e-14 of ||C|| for Gaussian blocks,
//    against ~1e-15 for an FP64 dot product and ~3e-7 for 3xTF32.
//
// Every mbarrier wait is bounded; on timeout the CTA records an error flag (shared with the 3xTF32
// kernel, xgb_gemm_tc_status), skips the epilogue and still frees its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "kernels.hpp"

namespace xgb {
namespace {

constexpr int OM = 128, ON = 64, OK = 32;          // output tile rows / columns, K per slice
constexpr int kPieces = 7, kBits = 7;               // seven 7-bit slices per entry
constexpr int kLevels = kPieces;                    // levels s + t = 2 .. 8 (1-based slices)
constexpr int kChunk = 14;                          // K slices per exact TMEM accumulation (448 x 36864 < 2^24)
constexpr int kMinSplit = 4;                        // smallest K range of a split-K CTA, in K slices
constexpr int kAPieceBytes = OM * OK * 2;           // 8 KB
constexpr int kBPieceBytes = ON * OK * 2;           // 4 KB
constexpr int kOzStageBytes = kPieces * (kAPieceBytes + kBPieceBytes);  // 84 KB
constexpr int kOzStages = 2;
constexpr int kOzSmem = kOzStages * kOzStageBytes + 1024;
constexpr uint32_t kOzTmemCols = 512;               // 7 levels x 64 columns used
constexpr int kOzWarps = 10, kOzThreads = kOzWarps * 32;
constexpr int kOzProducer = 8, kOzMma = 9, kOzDrainWarps = 8;
constexpr long long kOzSpin = 1ll << 26;
constexpr uint32_t kSboBytes = 128;                 // next 8-row group
// A: seven separate 128-row pieces.  B: the seven 64-row pieces stacked into one 448-row operand (row
// group g of piece s is row group 8 s + g), so that pieces t .. t + c - 1 form one N = 64 c operand
constexpr uint32_t kLboA = (OM / 8) * 128;          // next 16-byte K group, 128-row pieces
constexpr uint32_t kBPieceStride = (ON / 8) * 128;  // 1 KB: next B piece within a K group
constexpr uint32_t kLboB = kPieces * kBPieceStride; // 7 KB: next 16-byte K group of the stacked B
static_assert(kLevels * ON <= int(kOzTmemCols), "level accumulators fit TMEM");
static_assert(kOzSmem <= 227 * 1024, "stages fit shared memory");

__device__ __forceinline__ uint32_t s_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ uint64_t oz_desc(uint32_t saddr, uint32_t lbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFF);
  d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
  d |= uint64_t((kSboBytes >> 4) & 0x3FFF) << 32;
  d |= uint64_t(1) << 46;  // tcgen05 descriptor version; base offset 0, no swizzle
  return d;
}

// FP32 accumulate, BF16 A and B (kind::f16), both K-major, M = 128, N = 64 NC (NC stacked B pieces)
template <int NC>
__host__ __device__ constexpr uint32_t oz_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t((ON * NC) >> 3) << 17) | (uint32_t(OM >> 4) << 24);
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = s_u32(bar);
  for (long long it = 0; it < kOzSpin; ++it) {
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

__device__ __forceinline__ void bar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(s_u32(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(s_u32(bar))
      : "memory");
}

template <int NC>
__device__ __forceinline__ void mma_bf16_oz(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(oz_idesc<NC>()), "r"(acc));
}

__device__ __forceinline__ void commit_to(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(s_u32(bar))
               : "memory");
}

// ----------------------------------------------------------------------------- row scales
// task: (group, tile of OM rows of op(A) or ON rows of op(B)^T, K slice, which)
__global__ void __launch_bounds__(256) oz_rowmax_kernel(const xgb_gemm_desc* __restrict__ descs,
                                                         const OzGroup* __restrict__ groups,
                                                         const TcPackTask* __restrict__ tasks,
                                                         const double* __restrict__ A, const double* __restrict__ B,
                                                         unsigned long long* __restrict__ rowmax) {
  // |x| as IEEE bits: for non-negative doubles the integer order is the numeric order
  __shared__ unsigned long long X[OM][OK + 1];
  const TcPackTask t = tasks[blockIdx.x];
  const xgb_gemm_desc d = descs[t.g];
  const OzGroup gr = groups[t.g];
  const bool isB = t.which != 0;
  const bool sb = isB != (gr.swap != 0);  // the rows of this role are op(B)^T's (columns of op(B))
  const double* src = sb ? B : A;
  const int64_t off = sb ? d.b_off : d.a_off, ld = sb ? d.ldb : d.lda;
  const int64_t rows = sb ? d.n : d.m;
  const int tr = isB ? ON : OM;
  const bool rowfast = sb ? d.trans_b != 0 : d.trans_a == 0;
  const int64_t r0 = int64_t(t.tile) * tr, k0 = int64_t(t.slice) * OK;
  for (int e = threadIdx.x; e < tr * OK; e += 256) {
    int r, k;
    if (rowfast) { r = e % tr; k = e / tr; } else { k = e % OK; r = e / OK; }
    const int64_t gr_ = r0 + r, gk = k0 + k;
    double x = 0.0;
    if (gr_ < rows && gk < d.k) x = rowfast ? src[off + gr_ + gk * ld] : src[off + gk + gr_ * ld];
    X[r][k] = static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7FFFFFFFFFFFFFFFull;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < tr; r += 256) {
    if (r0 + r >= rows) continue;
    unsigned long long m = 0;
    for (int k = 0; k < OK; ++k) m = m > X[r][k] ? m : X[r][k];
    if (m) atomicMax(rowmax + (isB ? gr.b_rowmax : gr.a_rowmax) + r0 + r, m);
  }
}

// exponent e with |x| < 2^e for every entry of the row, from the bits of its largest |entry|
// m = f 2^e, f in [0.5, 1): the biased exponent less 1022.  A zero row, or one whose largest entry
// is subnormal (its slices are all zero), gets 0.
__device__ __forceinline__ int row_scale(unsigned long long bits) {
  const int be = int((bits >> 52) & 0x7FF);
  return be == 0 ? 0 : be - 1022;
}

// seven balanced base-128 digits of x relative to 2^e (|x| < 2^e):
// x = 2^e sum_s m_s 2^(-7 s) + O(2^(e - 50)), |m_1| <= 128, |m_s| <= 64 for s >= 2
__device__ __forceinline__ void slice7(double x, int e, float* out) {
  const long long bits = __double_as_longlong(x);
  const int ex = int((bits >> 52) & 0x7FF);
  const bool neg = bits < 0;
  long long q = 0;
  if (ex != 0) {  // normal numbers (subnormals are below every slice of any realistic row)
    const unsigned long long mant = (static_cast<unsigned long long>(bits) & ((1ull << 52) - 1)) | (1ull << 52);
    // x = mant 2^(ex - 1075); |x| rounded to the nearest multiple of 2^(e - 49) (ties up): shift right
    // by sh = e - 49 - (ex - 1075) >= 4 (|x| < 2^e) with one guard bit; q <= 2^49
    const int sh = e - 49 - (ex - 1075);
    q = sh >= 64 ? 0ll : static_cast<long long>(((mant >> (sh - 1)) + 1ull) >> 1);
  }
  // lowest digit first: m in [-64, 63] and the carry moves into q; what is left after six digits is
  // the leading digit, round(q / 2^42) <= 128
  int m[kPieces];
#pragma unroll
  for (int s = kPieces; s >= 2; --s) {
    int dg = int(q & ((1ll << kBits) - 1));
    if (dg >= 64) dg -= 128;
    m[s - 1] = dg;
    q = (q - dg) >> kBits;
  }
  m[0] = int(q);
#pragma unroll
  for (int s = 1; s <= kPieces; ++s) {
    const float v = __fmul_rn(float(neg ? -m[s - 1] : m[s - 1]), __int_as_float((127 - kBits * s) << 23));  // x 2^(-7 s)
    out[s - 1] = v;
  }
}

__global__ void __launch_bounds__(256) oz_pack_kernel(const xgb_gemm_desc* __restrict__ descs,
                                                       const OzGroup* __restrict__ groups,
                                                       const TcPackTask* __restrict__ tasks,
                                                       const double* __restrict__ A, const double* __restrict__ B,
                                                       const unsigned long long* __restrict__ rowmax,
                                                       unsigned char* __restrict__ apack,
                                                       unsigned char* __restrict__ bpack) {
  __shared__ double X[OM][OK + 1];
  __shared__ int E[OM];
  const TcPackTask t = tasks[blockIdx.x];
  const xgb_gemm_desc d = descs[t.g];
  const OzGroup gr = groups[t.g];
  const bool isB = t.which != 0;
  const bool sb = isB != (gr.swap != 0);  // the rows of this role are op(B)^T's (columns of op(B))
  const double* src = sb ? B : A;
  const int64_t off = sb ? d.b_off : d.a_off, ld = sb ? d.ldb : d.lda;
  const int64_t rows = sb ? d.n : d.m;
  const int tr = isB ? ON : OM;
  const bool rowfast = sb ? d.trans_b != 0 : d.trans_a == 0;
  const int64_t r0 = int64_t(t.tile) * tr, k0 = int64_t(t.slice) * OK;
  for (int e = threadIdx.x; e < tr * OK; e += 256) {
    int r, k;
    if (rowfast) { r = e % tr; k = e / tr; } else { k = e % OK; r = e / OK; }
    const int64_t gr_ = r0 + r, gk = k0 + k;
    double x = 0.0;
    if (gr_ < rows && gk < d.k) x = rowfast ? src[off + gr_ + gk * ld] : src[off + gk + gr_ * ld];
    X[r][k] = x;
  }
  for (int r = threadIdx.x; r < tr; r += 256)
    E[r] = (r0 + r < rows) ? row_scale(rowmax[(isB ? gr.b_rowmax : gr.a_rowmax) + r0 + r]) : 0;
  __syncthreads();
  // slice block of this (tile, K slice): kPieces pieces of tr x OK BF16, each in canonical layout
  const int piece_bytes = isB ? kBPieceBytes : kAPieceBytes;
  const int piece_stride = isB ? int(kBPieceStride) : kAPieceBytes;
  const uint32_t lbo = isB ? kLboB : kLboA;
  unsigned char* base = (isB ? bpack + gr.b_pack : apack + gr.a_pack) +
                        (int64_t(t.tile) * gr.slices + t.slice) * int64_t(kPieces) * piece_bytes;
  for (int e = threadIdx.x; e < tr * (OK / 8); e += 256) {
    const int r = e % tr, kq = e / tr;  // one 16-byte core-matrix row: 8 consecutive K of row r
    __nv_bfloat16 pc[kPieces][8];
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      float v[kPieces];
      slice7(X[r][kq * 8 + kk], E[r], v);
#pragma unroll
      for (int s = 0; s < kPieces; ++s) pc[s][kk] = __float2bfloat16_rn(v[s]);  // exact: <= 7 significant bits
    }
    const uint32_t bo = uint32_t(kq) * lbo + uint32_t(r >> 3) * kSboBytes + uint32_t(r & 7) * 16;
#pragma unroll
    for (int s = 0; s < kPieces; ++s)
      *reinterpret_cast<uint4*>(base + int64_t(s) * piece_stride + bo) = *reinterpret_cast<const uint4*>(pc[s]);
  }
}

// ----------------------------------------------------------------------------- gemm
// the rare cases of scaled_double (subnormal, infinite or out-of-range results), out of line so that
// the common path is never if-converted into the FP64 conversion and ldexp
__device__ __noinline__ double scaled_double_slow(float v, int sc) { return ldexp(double(v), sc); }

// v 2^sc as a double, assembled from the FP32 bits (exact; no FP64 arithmetic) while the result is a
// normal double, else through ldexp
__device__ __forceinline__ double scaled_double(float v, int sc) {
  const uint32_t b = __float_as_uint(v);
  const int e8 = int((b >> 23) & 0xFF);
  if ((b & 0x7FFFFFFFu) == 0u) return __longlong_as_double(static_cast<long long>(uint64_t(b >> 31) << 63));
  const int e = e8 - 127 + 1023 + sc;
  if (e8 == 0 || e8 == 255 || e <= 0 || e >= 2047) return scaled_double_slow(v, sc);
  return __longlong_as_double(static_cast<long long>((uint64_t(b >> 31) << 63) | (uint64_t(e) << 52) |
                                                     (uint64_t(b & 0x7FFFFFu) << 29)));
}

__global__ void __launch_bounds__(kOzThreads, 1)
    oz_gemm_kernel(const xgb_gemm_desc* __restrict__ descs, const OzGroup* __restrict__ groups,
                   const GemmTile* __restrict__ tiles, const unsigned char* __restrict__ apack,
                   const unsigned char* __restrict__ bpack, const unsigned long long* __restrict__ rowmax,
                   double* __restrict__ C, double alpha, double beta, double* __restrict__ ws,
                   int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[kOzStages], empty[kOzStages], accf, acce, done;
  __shared__ uint32_t tmem_slot;
  __shared__ int fail, issued, consumed;
  __shared__ int rsc[OM], csc[ON];  // row and column scale exponents of the tile
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));

  const GemmTile t = tiles[blockIdx.x];
  const xgb_gemm_desc d = descs[t.g];
  const OzGroup gr = groups[t.g];
  const int64_t m0 = int64_t(t.tm) * OM, n0 = int64_t(t.tn) * ON;
  // extents of the computed product: C, or C^T for a swapped group (element (r, c) of C^T is C[c + r ldc])
  const bool swp = gr.swap != 0;
  const int64_t pm = swp ? d.n : d.m, pn = swp ? d.m : d.n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // split-K: this CTA takes K slices [ks, ks + nk) and, with a slot, stores its raw partial tile
  const int ks = t.k0, nk = (t.k1 < 0 ? gr.slices : t.k1) - t.k0;
  const int nchunks = (nk + kChunk - 1) / kChunk;

  for (int i = threadIdx.x; i < OM + ON; i += kOzThreads) {
    if (i < OM) rsc[i] = m0 + i < pm ? row_scale(rowmax[gr.a_rowmax + m0 + i]) : 0;
    else csc[i - OM] = n0 + (i - OM) < pn ? row_scale(rowmax[gr.b_rowmax + n0 + (i - OM)]) : 0;
  }
  if (warp == kOzMma) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_u32(&tmem_slot)),
                 "r"(kOzTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kOzStages; ++s) {
      bar_init(&full[s], 1);
      bar_init(&empty[s], 1);
    }
    bar_init(&accf, 1);
    bar_init(&acce, kOzDrainWarps);
    bar_init(&done, 1);
    fail = 0;
    issued = 0;
    consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  // drain-warp state: TMEM lane quarter (rows) and 32-column group; double-FP32 sums of 32 columns
  const int quarter = warp & 3, colg = warp >> 2;
  float hi[32], lo[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) { hi[j] = 0.f; lo[j] = 0.f; }

  if (nk > 0 && warp == kOzProducer) {
    if (lane == 0) {
      const unsigned char* a_base =
          apack + gr.a_pack + (int64_t(t.tm) * gr.slices + ks) * kPieces * kAPieceBytes;
      const unsigned char* b_base =
          bpack + gr.b_pack + (int64_t(t.tn) * gr.slices + ks) * kPieces * kBPieceBytes;
      uint32_t ph[kOzStages] = {0, 0};
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % kOzStages;
        if (kc >= kOzStages) {
          if (!bar_wait(&empty[s], ph[s])) { atomicExch(&fail, 1); break; }
          ph[s] ^= 1u;
        }
        unsigned char* st = smem + s * kOzStageBytes;
        bar_expect_tx(&full[s], kOzStageBytes);
        bulk_g2s(st, a_base + int64_t(kc) * kPieces * kAPieceBytes, kPieces * kAPieceBytes, &full[s]);
        bulk_g2s(st + kPieces * kAPieceBytes, b_base + int64_t(kc) * kPieces * kBPieceBytes, kPieces * kBPieceBytes,
                 &full[s]);
        issued = kc + 1;
      }
    }
  } else if (nk > 0 && warp == kOzMma) {
    if (lane == 0) {
      uint32_t ph[kOzStages] = {0, 0};
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % kOzStages, cs = kc % kChunk, ch = kc / kChunk;
        // a new chunk overwrites the level accumulators: the previous chunk must be drained
        if (cs == 0 && ch > 0 && !bar_wait(&acce, uint32_t((ch - 1) & 1))) { atomicExch(&fail, 1); break; }
        if (!bar_wait(&full[s], ph[s])) { atomicExch(&fail, 1); break; }
        ph[s] ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t abase = s_u32(smem + s * kOzStageBytes);
        const uint32_t bbase = abase + kPieces * kAPieceBytes;
#pragma unroll
        for (int kk = 0; kk < OK / 16; ++kk) {
          // slice pairs (i, j), j <= 6 - i, in MMAs of up to four stacked B pieces: the product of A piece
          // i with B pieces j0 .. j0 + c - 1 lands in levels i + j0 .. i + j0 + c - 1, the adjacent
          // 64-column accumulators from column 64 (i + j0); ten MMAs cover the 28 pairs
          const uint64_t ad[kPieces] = {
              oz_desc(abase + 0 * kAPieceBytes + kk * 2 * kLboA, kLboA), oz_desc(abase + 1 * kAPieceBytes + kk * 2 * kLboA, kLboA),
              oz_desc(abase + 2 * kAPieceBytes + kk * 2 * kLboA, kLboA), oz_desc(abase + 3 * kAPieceBytes + kk * 2 * kLboA, kLboA),
              oz_desc(abase + 4 * kAPieceBytes + kk * 2 * kLboA, kLboA), oz_desc(abase + 5 * kAPieceBytes + kk * 2 * kLboA, kLboA),
              oz_desc(abase + 6 * kAPieceBytes + kk * 2 * kLboA, kLboA)};
          auto bd = [&](int j0) { return oz_desc(bbase + j0 * kBPieceStride + kk * 2 * kLboB, kLboB); };
          const uint32_t a0 = (cs == 0 && kk == 0) ? 0u : 1u;  // the i = 0 MMAs open every level of a chunk
          auto col = [&](int lvl) { return tmem + uint32_t(lvl * ON); };
          mma_bf16_oz<4>(col(0), ad[0], bd(0), a0);
          mma_bf16_oz<3>(col(4), ad[0], bd(4), a0);
          mma_bf16_oz<4>(col(1), ad[1], bd(0), 1u);
          mma_bf16_oz<2>(col(5), ad[1], bd(4), 1u);
          mma_bf16_oz<4>(col(2), ad[2], bd(0), 1u);
          mma_bf16_oz<1>(col(6), ad[2], bd(4), 1u);
          mma_bf16_oz<4>(col(3), ad[3], bd(0), 1u);
          mma_bf16_oz<3>(col(4), ad[4], bd(0), 1u);
          mma_bf16_oz<2>(col(5), ad[5], bd(0), 1u);
          mma_bf16_oz<1>(col(6), ad[6], bd(0), 1u);
        }
        commit_to(&empty[s]);
        if (cs == kChunk - 1 || kc == nk - 1) commit_to(&accf);
        consumed = kc + 1;
      }
      commit_to(&done);
    }
  } else if (nk > 0 && warp < kOzDrainWarps) {
    for (int ch = 0; ch < nchunks; ++ch) {
      const bool got = __all_sync(0xffffffffu, bar_wait(&accf, uint32_t(ch & 1)));
      if (!got) {
        if (lane == 0) atomicExch(&fail, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
      for (int level = kLevels - 1; level >= 0; --level) {  // smallest contributions first
        uint32_t v[32];
        const uint32_t taddr = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(level * ON + colg * 32);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
              "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
              "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          // two-sum of hi and the exact level partial; the rounding error goes to lo
          const float x = __uint_as_float(v[j]);
          const float s = __fadd_rn(hi[j], x);
          const float bb = __fsub_rn(s, hi[j]);
          const float e = __fadd_rn(__fsub_rn(hi[j], __fsub_rn(s, bb)), __fsub_rn(x, bb));
          hi[j] = s;
          lo[j] = __fadd_rn(lo[j], e);
        }
      }
#pragma unroll
      for (int j = 0; j < 32; ++j) {  // renormalise: |lo| stays below one unit of hi
        const float s = __fadd_rn(hi[j], lo[j]);
        lo[j] = __fsub_rn(lo[j], __fsub_rn(s, hi[j]));
        hi[j] = s;
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(s_u32(&acce)) : "memory");
    }
  }
  bool ok = true;
  if (nk > 0) ok = bar_wait(&done, 0);
  __syncthreads();
  ok = ok && (fail == 0);
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // 0: partial tile to the workspace, 1: C = acc, 2: C = alpha acc, 3: C = alpha acc + beta C
  const int mode = t.slot >= 0 ? 0 : beta != 0.0 ? 3 : alpha != 1.0 ? 2 : 1;
  if (ok && nk > 0 && warp < kOzDrainWarps) {
    const int64_t row = m0 + quarter * 32 + lane;
    const int ei = rsc[quarter * 32 + lane];
    if (mode != 0 && swp) {
      // transposed store through shared memory (the stages are idle now): thread (r, 32 columns) puts
      // its values at T[c][r] (row pitch 129 doubles), then each warp writes 32 consecutive rows of C
      double* T = reinterpret_cast<double*>(smem);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int c = colg * 32 + j;
        const int sc = ei + csc[c];
        T[c * (OM + 1) + quarter * 32 + lane] = scaled_double(hi[j], sc) + scaled_double(lo[j], sc);
      }
      asm volatile("bar.sync 1, %0;" ::"n"(kOzDrainWarps * 32) : "memory");
      for (int e = threadIdx.x; e < OM * ON; e += kOzDrainWarps * 32) {
        const int c = e % ON, r = e / ON;  // C row n0 + c, C column m0 + r
        if (m0 + r < pm && n0 + c < pn) {
          const double acc = T[c * (OM + 1) + r];
          double* cp = C + d.c_off + (n0 + c) + (m0 + r) * d.ldc;
          if (mode == 1) *cp = acc;
          else if (mode == 2) *cp = alpha * acc;
          else *cp = fma(alpha, acc, beta * *cp);
        }
      }
    } else if (row < pm) {
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int64_t col = n0 + colg * 32 + j;
        if (col < pn) {
          const int sc = ei + csc[colg * 32 + j];
          const double acc = scaled_double(hi[j], sc) + scaled_double(lo[j], sc);
          if (mode == 0) {  // split-K partial: raw sum, tile-local column-major OM x ON
            ws[int64_t(t.slot) * OM * ON + (quarter * 32 + lane) + int64_t(colg * 32 + j) * OM] = acc;
          } else {
            double* cp = C + d.c_off + row + col * d.ldc;
            if (mode == 1) *cp = acc;
            else if (mode == 2) *cp = alpha * acc;
            else *cp = fma(alpha, acc, beta * *cp);
          }
        }
      }
    }
  } else if (ok && nk == 0) {
    for (int e = threadIdx.x; e < OM * ON; e += kOzThreads) {
      const int64_t row = m0 + e % OM, col = n0 + e / OM;
      if (row < pm && col < pn) {
        double* cp = C + d.c_off + (swp ? col + row * d.ldc : row + col * d.ldc);
        *cp = beta == 0.0 ? 0.0 : beta * *cp;
      }
    }
  }
  if (!ok && threadIdx.x == 0) {
    atomicExch(err, 1);
    for (int kc = consumed; kc < issued; ++kc) bar_wait(&full[kc % kOzStages], uint32_t((kc / kOzStages) & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kOzMma)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kOzTmemCols));
}

// C tile = alpha * (the split-K partials of the tile, added in slot order) + beta * C
__global__ void __launch_bounds__(256) oz_splitk_reduce_kernel(const xgb_gemm_desc* __restrict__ descs,
                                                                const OzGroup* __restrict__ groups,
                                                                const SplitReduce* __restrict__ red,
                                                                const double* __restrict__ ws, double* __restrict__ C,
                                                                double alpha, double beta) {
  const SplitReduce r = red[blockIdx.x];
  const xgb_gemm_desc d = descs[r.g];
  const bool swp = groups[r.g].swap != 0;
  const int64_t pm = swp ? d.n : d.m, pn = swp ? d.m : d.n;
  // blockIdx.y: a 1024-element part of the tile (eight CTAs per tile keep the sums spread over the SMs);
  // consecutive threads take consecutive rows of C (tile rows, or tile columns of a swapped group)
  const int e0 = int(blockIdx.y) * 1024, e1 = e0 + 1024 < OM * ON ? e0 + 1024 : OM * ON;
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int li = swp ? e / ON : e % OM, lj = swp ? e % ON : e / OM;  // tile-local row / column
    const int64_t i = int64_t(r.tm) * OM + li, j = int64_t(r.tn) * ON + lj;
    if (i >= pm || j >= pn) continue;
    const int64_t w = li + int64_t(lj) * OM;
    double acc = ws[int64_t(r.first) * OM * ON + w];
    for (int p = 1; p < r.count; ++p) acc += ws[(int64_t(r.first) + p) * OM * ON + w];
    double* c = C + d.c_off + (swp ? j + i * d.ldc : i + j * d.ldc);
    *c = beta != 0.0 ? fma(alpha, acc, beta * *c) : alpha == 1.0 ? acc : alpha * acc;
  }
}

std::once_flag g_oz_attr;

}  // namespace

OzPlanHost build_oz_plan(const xgb_gemm_desc* descs, int n, bool allow_swap) {
  // A group is computed transposed (C^T = op(B)^T op(A)^T) when that needs at most 3/4 of the 128 x 64
  // output tiles (few rows, many columns: the 128-row tile would be mostly padding).
  auto tiles_of = [](int64_t r, int64_t c) { return ((r + OM - 1) / OM) * ((c + ON - 1) / ON); };
  std::vector<char> swap(size_t(n), 0);
  if (allow_swap)
    for (int g = 0; g < n; ++g) swap[g] = 4 * tiles_of(descs[g].n, descs[g].m) <= 3 * tiles_of(descs[g].m, descs[g].n);
  // rowmax layout: every group's rows of the "A" role first, then every group's rows of the "B" role
  // (columns of the product), so that the B part can be cleared and recomputed alone when only B
  // changes between products
  OzPlanHost p;
  for (int g = 0; g < n; ++g) p.rowmax_a += swap[g] ? descs[g].n : descs[g].m;
  int64_t ra = 0, rb = p.rowmax_a;
  for (int g = 0; g < n; ++g) {
    const xgb_gemm_desc& d = descs[g];
    const int64_t pm = swap[g] ? d.n : d.m, pn = swap[g] ? d.m : d.n;  // extents of the computed product
    OzGroup gr{};
    gr.swap = swap[g];
    gr.a_tiles = int32_t((pm + OM - 1) / OM);
    gr.b_tiles = int32_t((pn + ON - 1) / ON);
    gr.slices = int32_t((d.k + OK - 1) / OK);
    gr.a_pack = p.a_bytes;
    gr.b_pack = p.b_bytes;
    gr.a_rowmax = ra;
    gr.b_rowmax = rb;
    ra += pm;
    rb += pn;
    p.a_bytes += int64_t(gr.a_tiles) * gr.slices * kPieces * kAPieceBytes;
    p.b_bytes += int64_t(gr.b_tiles) * gr.slices * kPieces * kBPieceBytes;
    for (int32_t s = 0; s < gr.slices; ++s) {
      for (int32_t t = 0; t < gr.a_tiles; ++t) p.tasks_a.push_back({g, t, s, 0});
      for (int32_t t = 0; t < gr.b_tiles; ++t) p.tasks_b.push_back({g, t, s, 1});
    }
    p.groups.push_back(gr);
  }
  // output tiles and their K ranges.  One CTA runs per SM (its stages and TMEM fill one), so the K
  // slices of all tiles are cut into ranges of at most `cap` slices (at least kMinSplit), the largest
  // tiles split the most: cap starts at total / SMs and grows until the CTAs fit one wave (a second,
  // partial wave costs a whole CTA's fixed part - first load, drain, epilogue - on the SMs it uses).
  // The partial tiles of a split tile are added by a fixed-order reduce.
  int64_t work = 0, smax = 0;
  for (const auto& gr : p.groups) {
    work += int64_t(gr.a_tiles) * gr.b_tiles * gr.slices;
    smax = std::max<int64_t>(smax, gr.slices);
  }
  const int64_t sms = num_sms() > 0 ? num_sms() : 152;
  auto ctas = [&](int64_t cp) {
    int64_t c = 0;
    for (const auto& gr : p.groups) c += int64_t(gr.a_tiles) * gr.b_tiles * std::max<int64_t>(1, (gr.slices + cp - 1) / cp);
    return c;
  };
  int64_t cap = std::max<int64_t>(kMinSplit, (work + sms - 1) / sms);
  while (cap < smax && ctas(cap) > sms) ++cap;
  for (int g = 0; g < n; ++g) {
    const OzGroup& gr = p.groups[g];
    const int64_t splits = std::max<int64_t>(1, (gr.slices + cap - 1) / cap);
    const int64_t per = (gr.slices + splits - 1) / splits;
    for (int32_t y = 0; y < gr.b_tiles; ++y)
      for (int32_t x = 0; x < gr.a_tiles; ++x) {
        if (splits == 1) {
          p.tiles.push_back({g, x, y, OM});
          continue;
        }
        const int32_t first = p.slots;
        for (int64_t k0 = 0; k0 < gr.slices; k0 += per)
          p.tiles.push_back({g, x, y, OM, int32_t(k0), int32_t(std::min<int64_t>(k0 + per, gr.slices)), p.slots++});
        p.red.push_back({g, x, y, first, p.slots - first, 0});
      }
  }
  // longest K ranges first: CTAs start in index order, so the short ones fill the tail of the wave
  auto range = [&](const GemmTile& t) { return (t.k1 < 0 ? p.groups[t.g].slices : t.k1) - t.k0; };
  std::stable_sort(p.tiles.begin(), p.tiles.end(),
                   [&](const GemmTile& a, const GemmTile& b) { return range(a) > range(b); });
  p.rowmax = rb;
  p.tasks = p.tasks_a;
  p.tasks.insert(p.tasks.end(), p.tasks_b.begin(), p.tasks_b.end());
  return p;
}

void launch_oz_pack(const xgb_gemm_desc* d_descs, const OzGroup* d_groups, const TcPackTask* d_tasks, int n_tasks,
                    const double* A, const double* B, unsigned long long* rowmax, int64_t clear_from,
                    int64_t clear_count, unsigned char* apack, unsigned char* bpack, cudaStream_t s) {
  if (n_tasks <= 0) return;
  if (clear_count > 0) cudaMemsetAsync(rowmax + clear_from, 0, sizeof(unsigned long long) * size_t(clear_count), s);
  oz_rowmax_kernel<<<n_tasks, 256, 0, s>>>(d_descs, d_groups, d_tasks, A, B, rowmax);
  count_launch();
  oz_pack_kernel<<<n_tasks, 256, 0, s>>>(d_descs, d_groups, d_tasks, A, B, rowmax, apack, bpack);
  count_launch();
}

void launch_oz_gemm(const xgb_gemm_desc* d_descs, const OzGroup* d_groups, const GemmTile* d_tiles, int n_tiles,
                    const SplitReduce* d_red, int n_red, int slots, const unsigned char* apack,
                    const unsigned char* bpack, const unsigned long long* rowmax, double* C, double alpha, double beta,
                    cudaStream_t s) {
  if (n_tiles <= 0) return;
  std::call_once(g_oz_attr, [] {
    cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kOzSmem);
  });
  double* ws = slots > 0 ? static_cast<double*>(dev_alloc(sizeof(double) * size_t(slots) * OM * ON)) : nullptr;
  oz_gemm_kernel<<<n_tiles, kOzThreads, kOzSmem, s>>>(d_descs, d_groups, d_tiles, apack, bpack, rowmax, C, alpha,
                                                     beta, ws, gemm_tc_error_flag());
  count_launch();
  if (n_red > 0) {
    oz_splitk_reduce_kernel<<<dim3(unsigned(n_red), (OM * ON + 1023) / 1024), 256, 0, s>>>(d_descs, d_groups, d_red,
                                                                                            ws, C, alpha, beta);
    count_launch();
  }
  if (ws) dev_free(ws);
}

bool f64tc_heuristic(const xgb_gemm_desc* d, int n) {
  double flops = 0, out = 0;
  for (int g = 0; g < n; ++g) {
    flops += 2.0 * double(d[g].m) * double(d[g].n) * double(d[g].k);
    out += double(d[g].m) * double(d[g].n);
  }
  return out > 0 && flops / out >= 128.0;  // average k >= 64
}

void run_gemm_oz_host(const xgb_gemm_desc* h_descs, int n, const double* A, const double* B, double* C, double alpha,
                      double beta, cudaStream_t s) {
  if (n <= 0) return;
  OzPlanHost op = build_oz_plan(h_descs, n);
  if (op.tiles.empty()) return;
  auto up = [&](const void* h, size_t bytes) {
    void* d = dev_alloc(std::max<size_t>(bytes, 16));
    if (bytes) cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s);
    return d;
  };
  auto* dd = static_cast<xgb_gemm_desc*>(up(h_descs, sizeof(xgb_gemm_desc) * size_t(n)));
  auto* dg = static_cast<OzGroup*>(up(op.groups.data(), sizeof(OzGroup) * op.groups.size()));
  auto* dk = static_cast<TcPackTask*>(up(op.tasks.data(), sizeof(TcPackTask) * op.tasks.size()));
  auto* dt = static_cast<GemmTile*>(up(op.tiles.data(), sizeof(GemmTile) * op.tiles.size()));
  auto* dr = static_cast<SplitReduce*>(up(op.red.data(), sizeof(SplitReduce) * op.red.size()));
  auto* rm = static_cast<unsigned long long*>(dev_alloc(sizeof(unsigned long long) * size_t(std::max<int64_t>(op.rowmax, 1))));
  auto* ap = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(op.a_bytes, 16))));
  auto* bp = static_cast<unsigned char*>(dev_alloc(size_t(std::max<int64_t>(op.b_bytes, 16))));
  launch_gemm_oz(dd, dg, dk, int(op.tasks.size()), dt, int(op.tiles.size()), dr, int(op.red.size()), op.slots, A, B,
                 rm, op.rowmax, ap, bp, C, alpha, beta, s);
  for (void* p : {static_cast<void*>(dd), static_cast<void*>(dg), static_cast<void*>(dk), static_cast<void*>(dt),
                  static_cast<void*>(dr), static_cast<void*>(rm), static_cast<void*>(ap), static_cast<void*>(bp)})
    dev_free(p);
}

void launch_gemm_oz(const xgb_gemm_desc* d_descs, const OzGroup* d_groups, const TcPackTask* d_tasks, int n_tasks,
                    const GemmTile* d_tiles, int n_tiles, const SplitReduce* d_red, int n_red, int slots,
                    const double* A, const double* B, unsigned long long* rowmax, int64_t n_rowmax,
                    unsigned char* apack, unsigned char* bpack, double* C, double alpha, double beta, cudaStream_t s) {
  if (n_tiles <= 0) return;
  launch_oz_pack(d_descs, d_groups, d_tasks, n_tasks, A, B, rowmax, 0, n_rowmax, apack, bpack, s);
  launch_oz_gemm(d_descs, d_groups, d_tiles, n_tiles, d_red, n_red, slots, apack, bpack, rowmax, C, alpha, beta, s);
}

}  // namespace xgb
