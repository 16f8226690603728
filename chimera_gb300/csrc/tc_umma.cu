// tcgen05 (5th-generation tensor core) GEMM of the split-precision form.
//
//   C(M, N) = A(M, K) * B(K, N),  A, C FP32 column-major, B a prepared
//   operator mode; computed as sum_{i+j<=2} A_i B_j with A = A0+A1+A2 and
//   B = B0+B1+B2 the 3-term BF16 splits.
//
// Two kernels per batch:
//   split_a_kernel  each distinct A plane (plane pointer + reflection) -> its
//                   three BF16 terms in the tensor-core operand layout, one
//                   8 KB block per (128-row tile, 32-wide K step) and term,
//                   so the product kernel loads A like B, with bulk copies;
//   umma_kernel     persistent: one CTA per SM walks the batch's output tiles
//                   (128 rows x TNC columns, TNC <= 128 a multiple of 16).
//
// Accumulation.  The tensor core's FP32 accumulation is not round-to-nearest:
// with all six term pairs summed into one TMEM accumulator the error grows
// about linearly with the number of MMAs per accumulator (measured on GB300:
// 4e-7 relative at K = 64, 2.3e-6 at K = 256, against 2e-7 for an emulated
// round-to-nearest FP32 sum).  So:
//   - the leading pair A0 B0 goes into one of two TMEM accumulators H0 / H1
//     that take turns over chunks of kChunk K steps (32 K values each); the
//     row threads drain a finished chunk into FP32 registers (one
//     round-to-nearest add per chunk) while the tensor core fills the other;
//   - the five correction pairs (2^-8 and smaller relative to the result)
//     go into an accumulator L over the tile's whole K range (error scaled by
//     the same 2^-8); L0 / L1 take turns over tiles, so the next tile's MMAs
//     start while the row threads finish the previous tile.
// TMEM: H0, H1, L0, L1 of TNC columns each (512 columns at TNC = 128).
//
// Roles in umma_kernel (320 threads):
//   - warps 0..7, the row threads: warp w takes rows 32 (w % 4) .. +31 (the
//     TMEM lanes its quarter may access) and column half w / 4 of the tile;
//     they drain the H chunks and the L accumulator into registers and write
//     the tile (complex shift and factor epilogues; the factor block of a
//     tile is staged in shared memory after the stage ring);
//   - warp 8, lane 0: issues the 12 tcgen05.mma of every K step (6 term
//     pairs x 2 K halves) and the commits that release stages and
//     accumulators;
//   - warp 9, lane 0: streams the A and B terms of every K step into a
//     4-stage ring with bulk-copy TMA (cp.async.bulk, mbarrier completion).
// Every mbarrier wait has an iteration limit.  The pipeline waits use a limit
// set from the host (chm_sp_set_umma_spin_limit, so that a test can make
// them run out); on a timeout the CTA records an error, stops issuing work,
// waits with the full limit for its own bulk copies and MMAs, frees its TMEM
// and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "tc_gemm.cuh"

using namespace chm;

namespace {

constexpr int TH = 128;                 // rows per tile (UMMA M)
constexpr int KB = 32;                  // K step (elements)
// K steps per H accumulator chunk: 4 (128 K values).  Measured at 4096 x 512
// x 3 modes: chunks of 2 drained often enough to hold the tensor core back
// while the row threads wrote a tile (fb_eb_out 0.94 ms, product error
// 9.1e-8 at K = 512); 4: 0.84 ms, 1.28e-7; 8: 0.82 ms, 2.3e-7
constexpr int kChunk = 4;
constexpr int STAGES = 4;
constexpr int kRowThreads = 2 * TH;     // two threads per row (column halves)
constexpr int kMmaThread = kRowThreads;         // warp 8, lane 0
constexpr int kLoadThread = kRowThreads + 32;   // warp 9, lane 0
constexpr int kThreads = kRowThreads + 64;
constexpr int CH = TH / 2;              // tile columns per row thread
constexpr int kMaxBatch = 64;
constexpr long long kSpinLimit = 1LL << 20;  // try_wait polls; each may block briefly
constexpr uint32_t kATermBytes = TH * KB * 2;  // one BF16 term of an A block (8 KB)
constexpr uint32_t kABytes = 3 * kATermBytes;
constexpr int kSplitBlock = TH * KB;           // elements of one A block and term

__device__ int g_umma_error;  // first failing CTA records a code here
long long g_spin_limit = kSpinLimit;

// ----------------------------------------------------------------------
// PTX helpers
// ----------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// bounded wait for the phase with parity `parity` to complete
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit) {
  const uint32_t a = smem_u32(bar);
  for (long long it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// shared-memory matrix descriptor (SWIZZLE_NONE, K-major core matrices of 8
// rows x 16 bytes: LBO = 128 B between K groups, SBO = 512 B between row
// groups); the start address sits in bits 0..13 (address >> 4), so adding
// (offset >> 4) to a descriptor moves it by offset bytes
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(128u >> 4) << 16;
  d |= (uint64_t)(((KB / 8) * 128u) >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;
}

// instruction descriptor: kind::f16, BF16 x BF16 -> F32, K-major A and B
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                          // D format F32
         | (1u << 7)                        // A format BF16
         | (1u << 10)                       // B format BF16
         | ((uint32_t)(N >> 3) << 17)       // N / 8
         | ((uint32_t)(M >> 4) << 24);      // M / 16
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 16 consecutive FP32 accumulator columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tmem_ld16(uint32_t (&v)[16], uint32_t taddr) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// acc[0 .. nc) += the nc accumulator columns starting at column `col`
// (nc a multiple of 16, at most 64; loads issued in pairs before one wait)
__device__ __forceinline__ void tmem_add_row(float (&acc)[CH], uint32_t tmem_lane, uint32_t col, int nc) {
#pragma unroll
  for (int c0 = 0; c0 < CH; c0 += 32) {
    if (c0 < nc) {
      uint32_t va[16], vb[16];
      const bool two = c0 + 16 < nc;
      tmem_ld16(va, tmem_lane + col + (uint32_t)c0);
      if (two) tmem_ld16(vb, tmem_lane + col + (uint32_t)(c0 + 16));
      tmem_wait_ld();
#pragma unroll
      for (int j = 0; j < 16; ++j) acc[c0 + j] += __uint_as_float(va[j]);
      if (two) {
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[c0 + 16 + j] += __uint_as_float(vb[j]);
      }
    }
  }
}

// AND of v over the row threads (named barrier 1, warps 0..7): their loop
// exits stay uniform, so the named barriers of the factor epilogue never
// wait for a thread that has left
__device__ __forceinline__ bool row_threads_all(bool v) {
  uint32_t r;
  asm volatile(
      "{\n"
      ".reg .pred p, q;\n"
      "setp.ne.u32 q, %1, 0;\n"
      "bar.red.and.pred p, 1, %2, q;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(kRowThreads)
      : "memory");
  return r != 0;
}

// ----------------------------------------------------------------------
// A split: FP32 plane -> three BF16 terms in the operand layout
// ----------------------------------------------------------------------
struct SplitJobs {
  const float *A[kMaxBatch];
  __nv_bfloat16 *T[kMaxBatch];  // term 0; term t at + t * term_stride
  int reflect[kMaxBatch];
};

// x ~ t0 + t1 + t2 for two values at a time: each term the round-to-nearest
// BF16 of the remainder (the pair conversions pack two values per register)
__device__ __forceinline__ void split_pair(float x0, float x1, uint32_t &t0, uint32_t &t1, uint32_t &t2) {
  const __nv_bfloat162 b0 = __floats2bfloat162_rn(x0, x1);
  const float2 f0 = __bfloat1622float2(b0);
  const float r0 = x0 - f0.x, r1 = x1 - f0.y;
  const __nv_bfloat162 b1 = __floats2bfloat162_rn(r0, r1);
  const float2 f1 = __bfloat1622float2(b1);
  const __nv_bfloat162 b2 = __floats2bfloat162_rn(r0 - f1.x, r1 - f1.y);
  t0 = *reinterpret_cast<const uint32_t *>(&b0);
  t1 = *reinterpret_cast<const uint32_t *>(&b1);
  t2 = *reinterpret_cast<const uint32_t *>(&b2);
}

// blockIdx = (row tile, K step, job); thread = row of the tile.  Element
// (r, k) of a block sits at ((r / 8) * 4 + k / 8) * 64 + (r % 8) * 8 + k % 8;
// rows past M and K values past K are zero.  A reflected plane: row (x, c)
// is (c ? 1 : -1) * row ((M/2 - x) mod M/2, c) of the stored plane.
__global__ void __launch_bounds__(TH) split_a_kernel(const __grid_constant__ SplitJobs J, int M, int K,
                                                    int nkb, long long term_stride) {
  const int r = threadIdx.x, mt = blockIdx.x, kb = blockIdx.y, job = blockIdx.z;
  const long long gm = (long long)mt * TH + r;
  const bool row_ok = gm < M;
  long long src = gm;
  float sgn = 1.0f;
  if (J.reflect[job] && row_ok) {
    const long long x = gm >> 1, nxh = M >> 1;
    src = 2 * (x == 0 ? 0 : nxh - x) + (gm & 1);
    if ((gm & 1) == 0) sgn = -1.0f;
  }
  const float *Arow = J.A[job] + src;
  float v[KB];
#pragma unroll
  for (int k = 0; k < KB; ++k) {
    const int gk = kb * KB + k;
    v[k] = (row_ok && gk < K) ? sgn * __ldg(Arow + (long long)gk * M) : 0.0f;
  }
  __nv_bfloat16 *T = J.T[job] + ((long long)mt * nkb + kb) * kSplitBlock;
#pragma unroll
  for (int kg = 0; kg < KB / 8; ++kg) {
    uint32_t w0[4], w1[4], w2[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) split_pair(v[kg * 8 + 2 * q], v[kg * 8 + 2 * q + 1], w0[q], w1[q], w2[q]);
    const int off = ((r >> 3) * (KB / 8) + kg) * 64 + (r & 7) * 8;
    *reinterpret_cast<uint4 *>(T + off) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
    *reinterpret_cast<uint4 *>(T + term_stride + off) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
    *reinterpret_cast<uint4 *>(T + 2 * term_stride + off) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
  }
}

// ----------------------------------------------------------------------
// MMA kernel
// ----------------------------------------------------------------------
struct UmmaProb {
  const __nv_bfloat16 *A;  // split A, term 0 (terms at + a_term_stride)
  float *C;
  const float *fac;
  const __nv_bfloat16 *B[3];  // split B terms of this problem's mode
};

struct UmmaBatch {
  UmmaProb p[kMaxBatch];
};

struct UmmaArgs {
  int M, N, Np, nkb;
  int tnc, ntn, nmt, ntiles;  // tile columns, column tiles, row tiles, tiles of the batch
  long long a_term_stride;    // elements between the split terms of one A plane
  const float2 *shift;
  uint32_t tmem_cols;
  long long spin;             // iteration limit of the pipeline waits
};

template <int EPI>
__global__ void __launch_bounds__(kThreads, 1) umma_kernel(const __grid_constant__ UmmaBatch P, UmmaArgs A) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], hfull[2], hempty[2], lfull[2], lempty[2],
      done;
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  const int warp = threadIdx.x >> 5;
  const int tnc = A.tnc, nkb = A.nkb;
  const int nchunk = (nkb + kChunk - 1) / kChunk;
  const uint32_t b_term = (uint32_t)tnc * KB * 2;  // one B term of a stage
  const uint32_t stage_bytes = kABytes + 3 * b_term;
  const long long spin = A.spin;
  volatile int *vfail = &fail;
  // this CTA's tiles: blockIdx.x, blockIdx.x + gridDim.x, ...; the column
  // tile varies fastest, so the CTAs running at once share A rows in L2
  const int my_tiles = A.ntiles > (int)blockIdx.x ? (A.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&hfull[b], 1);
      mbar_init(&hempty[b], kRowThreads);
      mbar_init(&lfull[b], 1);
      mbar_init(&lempty[b], kRowThreads);
    }
    mbar_init(&done, 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaThread / 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(A.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t smem0 = smem_u32(smem);
  float *facs = reinterpret_cast<float *>(smem + (size_t)STAGES * stage_bytes);  // factor epilogue

  if (threadIdx.x == kLoadThread) {
    // ---- bulk copies of the A and B terms of every K step
    int last[STAGES];
    for (int s = 0; s < STAGES; ++s) last[s] = -1;
    long long g = 0;
    bool ok = true;
    for (int i = 0; i < my_tiles && ok && !*vfail; ++i) {
      const int t = (int)blockIdx.x + i * (int)gridDim.x;
      const int rest = t % (A.nmt * A.ntn), prob = t / (A.nmt * A.ntn);
      const int mt = rest / A.ntn, nt = rest % A.ntn;
      const UmmaProb &Q = P.p[prob];
      const __nv_bfloat16 *Ab = Q.A + (long long)mt * nkb * kSplitBlock;
      for (int kb = 0; kb < nkb; ++kb, ++g) {
        const int s = (int)(g % STAGES);
        if (g >= STAGES && !mbar_wait(&empty[s], (uint32_t)(g / STAGES - 1) & 1u, spin)) {
          *vfail = 1;
          atomicCAS(&g_umma_error, 0, 3);
          ok = false;
          break;
        }
        const uint32_t st = smem0 + (uint32_t)s * stage_bytes, bar = smem_u32(&full[s]);
        mbar_expect_tx(&full[s], kABytes + 3 * b_term);
        for (int tt = 0; tt < 3; ++tt) {
          bulk_g2s(st + tt * kATermBytes, Ab + tt * A.a_term_stride + (long long)kb * kSplitBlock,
                   kATermBytes, bar);
          bulk_g2s(st + kABytes + tt * b_term, Q.B[tt] + (long long)kb * A.Np * KB + (long long)nt * tnc * KB,
                   b_term, bar);
        }
        last[s] = (int)(g / STAGES);
      }
    }
    // the copies issued last on every stage land before the CTA goes on
    for (int s = 0; s < STAGES; ++s)
      if (last[s] >= 0 && !mbar_wait(&full[s], (uint32_t)last[s] & 1u, kSpinLimit))
        atomicCAS(&g_umma_error, 0, 5);
  } else if (threadIdx.x == kMmaThread) {
    // ---- MMA issue
    const uint32_t idesc = idesc_bf16(TH, tnc);
    long long g = 0;
    bool ok = true;
    for (int i = 0; i < my_tiles && ok; ++i) {
      const int lb = i & 1;
      for (int kb = 0; kb < nkb; ++kb, ++g) {
        const int s = (int)(g % STAGES);
        const long long c = (long long)i * nchunk + kb / kChunk;
        const bool first = (kb % kChunk) == 0;
        const bool last = (kb % kChunk) == kChunk - 1 || kb == nkb - 1;
        if (first && c >= 2 && !mbar_wait(&hempty[c & 1], (uint32_t)((c >> 1) - 1) & 1u, spin)) ok = false;
        if (ok && kb == 0 && i >= 2 && !mbar_wait(&lempty[lb], (uint32_t)((i >> 1) - 1) & 1u, spin))
          ok = false;
        if (ok && !mbar_wait(&full[s], (uint32_t)(g / STAGES) & 1u, spin)) ok = false;
        if (!ok || *vfail) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = smem0 + (uint32_t)s * stage_bytes;
        const uint64_t a0 = smem_desc(st), b0 = smem_desc(st + kABytes);
        const uint32_t dH = tmem + (uint32_t)((c & 1) * tnc), dL = tmem + (uint32_t)((2 + lb) * tnc);
        // term pairs (i, j): (0, 0) into H, the others into L
        const int pi[6] = {0, 2, 1, 0, 1, 0}, pj[6] = {0, 0, 1, 2, 0, 1};
#pragma unroll
        for (int q = 0; q < 6; ++q) {
#pragma unroll
          for (int ks = 0; ks < KB / 16; ++ks) {
            const uint64_t ad = a0 + ((pi[q] * kATermBytes + ks * 256) >> 4);
            const uint64_t bd = b0 + ((pj[q] * b_term + ks * 256) >> 4);
            if (q == 0)
              umma_bf16(dH, ad, bd, idesc, (first && ks == 0) ? 0u : 1u);
            else
              umma_bf16(dL, ad, bd, idesc, (kb == 0 && q == 1 && ks == 0) ? 0u : 1u);
          }
        }
        umma_commit(&empty[s]);
        if (last) umma_commit(&hfull[c & 1]);
        if (kb == nkb - 1) umma_commit(&lfull[lb]);
      }
    }
    umma_commit(&done);
    if (!ok) {
      *vfail = 1;
      atomicCAS(&g_umma_error, 0, 1);
    }
  } else if (threadIdx.x < kRowThreads) {
    // ---- row threads: drain the accumulators, write the tiles
    const int half = warp >> 2;
    const int col0 = half * CH;
    const int ncol = max(0, min(CH, tnc - col0));  // a multiple of 16
    const uint32_t tmem_lane = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const int row = (warp & 3) * 32 + (threadIdx.x & 31);
    float acc[CH];
    for (int i = 0; i < my_tiles; ++i) {
      const int t = (int)blockIdx.x + i * (int)gridDim.x;
      const int rest = t % (A.nmt * A.ntn), prob = t / (A.nmt * A.ntn);
      const int mt = rest / A.ntn, nt = rest % A.ntn;
      const int lb = i & 1;
      const UmmaProb &Q = P.p[prob];
      const long long gm = (long long)mt * TH + row;
      const bool rok = gm < A.M;
#pragma unroll
      for (int j = 0; j < CH; ++j) acc[j] = 0.0f;
      if (EPI == TC_EPI_SHIFT_FAC) {
        // the tile's factor block (64 x-rows x tnc columns) into shared
        // memory before the accumulator waits, so that its load latency is
        // hidden; the row threads meet before (the previous tile's epilogue
        // has read the block) and after writing it
        asm volatile("bar.sync 1, %0;" ::"n"(kRowThreads) : "memory");
        const long long xr0 = (long long)mt * (TH / 2);
        const long long rows = min((long long)(TH / 2), (long long)(A.M >> 1) - xr0);
        for (int e = threadIdx.x; e < (TH / 2) * tnc; e += kRowThreads) {
          const int col = e / (TH / 2), xx = e % (TH / 2), n = nt * tnc + col;
          facs[e] = (xx < rows && n < A.N) ? __ldg(Q.fac + xr0 + xx + (long long)(A.M >> 1) * n) : 1.0f;
        }
        asm volatile("bar.sync 1, %0;" ::"n"(kRowThreads) : "memory");
      }
      bool ok = true;
      for (int cc = 0; cc < nchunk; ++cc) {
        const long long c = (long long)i * nchunk + cc;
        const int b = (int)(c & 1);
        ok = ok && !*vfail && mbar_wait(&hfull[b], (uint32_t)(c >> 1) & 1u, spin);
        if (ok) {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          tmem_add_row(acc, tmem_lane, (uint32_t)(b * tnc + col0), ncol);
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        }
        mbar_arrive(&hempty[b]);
      }
      ok = ok && !*vfail && mbar_wait(&lfull[lb], (uint32_t)(i >> 1) & 1u, spin);
      if (ok) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        tmem_add_row(acc, tmem_lane, (uint32_t)((2 + lb) * tnc + col0), ncol);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      }
      mbar_arrive(&lempty[lb]);
      if (!ok) atomicCAS(&g_umma_error, 0, 4);
      if (!row_threads_all(ok && !*vfail)) {
        *vfail = 1;
        break;
      }
      // epilogue from registers, while the tensor core runs the next tile
      float2 sh = make_float2(1.f, 0.f);
      if (EPI != TC_EPI_STORE && rok) sh = A.shift[gm >> 1];
#pragma unroll
      for (int jj = 0; jj < CH; ++jj) {
        if (jj < ncol) {
          float x = acc[jj];
          const int n = nt * tnc + col0 + jj;
          if (EPI != TC_EPI_STORE) {
            // rows 2x (re) and 2x+1 (im) sit in adjacent lanes
            const float other = __shfl_xor_sync(0xffffffffu, x, 1);
            const float re = (row & 1) ? other : x, im = (row & 1) ? x : other;
            x = (row & 1) ? (re * sh.y + im * sh.x) : (re * sh.x - im * sh.y);
            if (EPI == TC_EPI_SHIFT_FAC) x *= facs[(col0 + jj) * (TH / 2) + (row >> 1)];
          }
          if (rok && n < A.N) Q.C[gm + (long long)n * A.M] = x;
        }
      }
    }
  }
  __syncthreads();
  // every MMA complete before the TMEM is freed (the full limit: this wait
  // must not leave MMAs in flight)
  if (!mbar_wait(&done, 0, kSpinLimit) && threadIdx.x == 0) atomicCAS(&g_umma_error, 0, 2);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kMmaThread / 32) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(A.tmem_cols)
                 : "memory");
  }
}

inline long long rup(long long a, long long b) { return (a + b - 1) / b * b; }

// Column-tile width of the products.  Every multiple of 16 that divides
// Np = tc_np(N) and is at most 128 gives the same output bitwise: each
// output element's K sum runs through the same MMAs and chunk drains in the
// same order whatever the width, which changes only the number of tiles,
// the B bytes per stage and the TMEM columns.  The width for a shape
// (M, N, K, batch count, epilogue) is picked by timing: the first launch of
// the shape outside stream capture runs every candidate width (one warm-up
// and three timed launches each, CUDA events on the launch stream) and
// keeps the fastest.  g_cols_mode: -1 tune (the default), 0 the default
// width tc_tile_cols(N), > 0 that width where it is a candidate.
int g_cols_mode = -1;
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int, int>, int> g_tuned;  // shape -> width

// the default width tc_tile_cols(N) first, then the narrower multiples of
// 16 (32 and up) that divide Np
std::vector<int> col_candidates(int N) {
  const int Np = tc_np(N), w0 = tc_tile_cols(N);
  std::vector<int> c{w0};
  for (int w = w0 - 16; w >= 32; w -= 16)
    if (Np % w == 0) c.push_back(w);
  return c;
}

size_t umma_smem(int tnc, int epi) {
  return (size_t)STAGES * (kABytes + 3 * (size_t)tnc * KB * 2) + 1024 +
         (epi == TC_EPI_SHIFT_FAC ? (size_t)(TH / 2) * tnc * 4 : 0);
}

}  // namespace

namespace chm {

long long tc_split_bytes(int M, int K, int count) {
  return (long long)count * 6 * rup(M, TH) * rup(K, KB) + 256;
}

int tc_umma_launch(const TcProblem *p, int count, int M, int N, int K, int epi, const float2 *shift,
                   void *ws, long long ws_bytes, cudaStream_t st) {
  const int Np = tc_np(N);
  const int nkb = (int)(rup(K, KB) / KB), nmt = (int)((M + TH - 1) / TH);
  const std::vector<int> cands = col_candidates(N);
  if (cands.empty() || cands[0] > TH) {
    set_error("umma: no column tile for N = %d", N);
    return CHM_ERR_RANGE;
  }
  if (M % 2) {
    set_error("umma: M must be even (complex rows)");
    return CHM_ERR_ARG;
  }
  for (int i = 0; i < count; ++i)
    if (!p[i].B.bf[0] || !p[i].B.bf[1] || !p[i].B.bf[2] || p[i].B.K != K || p[i].B.N != N) {
      set_error("umma: problem %d has no prepared %dx%d operator", i, K, N);
      return CHM_ERR_ARG;
    }
  const long long term_stride = (long long)nmt * nkb * kSplitBlock;  // elements
  const long long split_one = 3 * term_stride * 2;                     // bytes per A plane
  char *wsp = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(ws) + 255) & ~(uintptr_t)255);
  const long long avail = ws ? ws_bytes - (wsp - reinterpret_cast<char *>(ws)) : 0;
  void (*kern)(const UmmaBatch, UmmaArgs) =
      epi == TC_EPI_STORE ? umma_kernel<TC_EPI_STORE>
                          : (epi == TC_EPI_SHIFT ? umma_kernel<TC_EPI_SHIFT> : umma_kernel<TC_EPI_SHIFT_FAC>);
  // (the widest candidate needs the most shared memory)
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)umma_smem(cands[0], epi));
  // one product launch of the batch chunk ub (cnt problems) at width tnc
  auto launch = [&](const UmmaBatch &ub, const UmmaArgs &base, int cnt, int tnc) {
    UmmaArgs ua = base;
    ua.tnc = tnc;
    ua.ntn = Np / tnc;
    ua.ntiles = cnt * nmt * ua.ntn;
    uint32_t cols = 32;
    while (cols < (uint32_t)(4 * tnc)) cols <<= 1;  // H0, H1, L0, L1
    ua.tmem_cols = cols;
    const int grid = ua.ntiles < sm_count() ? ua.ntiles : sm_count();
    kern<<<grid, kThreads, umma_smem(tnc, epi), st>>>(ub, ua);
    count_launch();
  };
  for (int c0 = 0; c0 < count; c0 += kMaxBatch) {
    const int cnt = count - c0 < kMaxBatch ? count - c0 : kMaxBatch;
    // split every distinct A plane (pointer and reflection) once
    SplitJobs J;
    int njobs = 0;
    UmmaBatch ub;
    for (int i = 0; i < cnt; ++i) {
      const TcProblem &q = p[c0 + i];
      int j = 0;
      while (j < njobs && !(J.A[j] == q.A && J.reflect[j] == q.reflect)) ++j;
      if (j == njobs) {
        if ((long long)(njobs + 1) * split_one > avail) {
          set_error("umma: workspace of %lld bytes holds no room for %d split A planes", ws_bytes,
                    njobs + 1);
          return CHM_ERR_WS;
        }
        J.A[j] = q.A;
        J.reflect[j] = q.reflect;
        J.T[j] = reinterpret_cast<__nv_bfloat16 *>(wsp + (long long)j * split_one);
        ++njobs;
      }
      ub.p[i] = UmmaProb{J.T[j], q.C, q.fac,
                         {reinterpret_cast<const __nv_bfloat16 *>(q.B.bf[0]),
                          reinterpret_cast<const __nv_bfloat16 *>(q.B.bf[1]),
                          reinterpret_cast<const __nv_bfloat16 *>(q.B.bf[2])}};
    }
    split_a_kernel<<<dim3(nmt, nkb, njobs), TH, 0, st>>>(J, M, K, nkb, term_stride);
    count_launch();
    UmmaArgs ua{};
    ua.M = M;
    ua.N = N;
    ua.Np = Np;
    ua.nkb = nkb;
    ua.nmt = nmt;
    ua.a_term_stride = term_stride;
    ua.shift = shift;
    ua.spin = g_spin_limit;
    // the column-tile width: forced, the widest, or the tuned one (timed on
    // the first launch of this shape; the product reads only the split A
    // planes and B and overwrites C, so the timed launches can repeat)
    int tnc = cands[0];
    bool tune = false;
    const auto key = std::make_tuple(M, N, K, cnt, epi);
    if (g_cols_mode > 0) {
      for (int w : cands)
        if (w == g_cols_mode) tnc = w;
    } else if (g_cols_mode < 0 && cands.size() > 1) {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto it = g_tuned.find(key);
      if (it != g_tuned.end()) {
        tnc = it->second;
      } else {
        // (not inside a stream capture, and not under a test's wait limit)
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(st, &cs);
        tune = cs == cudaStreamCaptureStatusNone && g_spin_limit == kSpinLimit;
      }
    }
    if (tune) {
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      float best = 0.0f;
      for (int w : cands) {
        launch(ub, ua, cnt, w);  // warm-up
        cudaEventRecord(e0, st);
        for (int r = 0; r < 3; ++r) launch(ub, ua, cnt, w);
        cudaEventRecord(e1, st);
        float ms = 0.0f;
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
          break;
        if (w == cands[0] || ms < best) {
          best = ms;
          tnc = w;
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      std::lock_guard<std::mutex> lock(g_tune_mu);
      g_tuned[key] = tnc;
    }
    launch(ub, ua, cnt, tnc);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("umma: %s", cudaGetErrorString(e));
    return CHM_ERR_CUDA;
  }
  return CHM_OK;
}

}  // namespace chm

extern "C" int chm_sp_umma_status(void) {
  int v = 0, z = 0;
  cudaMemcpyFromSymbol(&v, g_umma_error, sizeof(int));
  if (v) cudaMemcpyToSymbol(g_umma_error, &z, sizeof(int));
  return v;
}

extern "C" int chm_sp_set_umma_cols(int mode) {
  const int prev = g_cols_mode;
  g_cols_mode = mode < 0 ? -1 : mode;
  return prev;
}

extern "C" int chm_sp_umma_tuned(int32_t *out, int max_shapes) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  int n = 0;
  for (const auto &kv : g_tuned) {
    if (out && n < max_shapes) {
      int32_t *o = out + 6 * n;
      o[0] = std::get<0>(kv.first);
      o[1] = std::get<1>(kv.first);
      o[2] = std::get<2>(kv.first);
      o[3] = std::get<3>(kv.first);
      o[4] = std::get<4>(kv.first);
      o[5] = kv.second;
    }
    ++n;
  }
  return n;
}

extern "C" int chm_sp_umma_tune_reset(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned.clear();
  return CHM_OK;
}

extern "C" int64_t chm_sp_set_umma_spin_limit(int64_t polls) {
  const long long prev = g_spin_limit;
  g_spin_limit = polls < 0 ? kSpinLimit : polls;
  return prev;
}
