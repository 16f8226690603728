// tcgen05 (5th-generation tensor core) GEMM of the split-precision form.
//
//   C(M, N) = A(M, K) * B(K, N),  A, C FP32 column-major, B a prepared
//   operator mode; computed as sum_{i+j<=2} A_i B_j with A = A0+A1+A2 and
//   B = B0+B1+B2 the 3-term BF16 splits.
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
//     go into a third accumulator L over the whole K range; its error is
//     scaled by the same 2^-8.
//
// One CTA computes a 128-row x TNC-column tile (TNC <= 128, a multiple of
// 16) of one problem of a batch; grid = (row tiles, column tiles, problems):
//   - warps 0..7 are the row threads: warp w takes rows 32 (w % 4) .. +31
//     (the TMEM lanes its quarter may access) and half w / 4 of every 32-wide
//     K step and of the tile's columns.  Each thread loads its 16 FP32 A
//     values of the step, splits them into the three BF16 terms, stores them
//     into the stage in the tensor-core operand layout (K-major core
//     matrices of 8 rows x 16 bytes), drains its 64 columns of the H chunks
//     into registers and writes them;
//   - warp 8's lane 0 streams the prepared B terms of the step with bulk-copy
//     TMA (cp.async.bulk, completion on an mbarrier) and issues the 12
//     tcgen05.mma of the step (6 term pairs x 2 K halves), releasing the
//     stage with tcgen05.commit.
// Every mbarrier wait has an iteration limit.  The pipeline waits use a limit
// set from the host (chm_sp_set_umma_spin_limit, so that a test can make
// them run out); on a timeout the CTA records an error, waits with the full
// limit for its own bulk copies and MMAs, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "tc_gemm.cuh"

using namespace chm;

namespace {

constexpr int TH = 128;                 // rows per tile (UMMA M)
constexpr int KB = 32;                  // K step (elements)
constexpr int kChunk = 2;               // K steps per H accumulator chunk
constexpr int STAGES = 4;
constexpr int kProducers = 2 * TH;      // two threads per row (K and column halves)
constexpr int kThreads = kProducers + 32;
constexpr int KH = KB / 2;              // K values of a step per row thread
constexpr int CH = TH / 2;              // tile columns per row thread
constexpr int kMaxBatch = 64;
constexpr long long kSpinLimit = 1LL << 20;  // try_wait polls; each may block briefly
constexpr uint32_t kATermBytes = TH * KB * 2;  // one BF16 term of the A block
constexpr uint32_t kABytes = 3 * kATermBytes;

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

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t smem_desc(const void *p, uint32_t lbo, uint32_t sbo) {
  const uint64_t a = (smem_u32(p) & 0x3FFFFu) >> 4;
  uint64_t d = a;
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  // base offset 0, lbo mode 0, layout SWIZZLE_NONE (0)
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

__device__ __forceinline__ uint32_t bf16_bits(__nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(b);
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

// ----------------------------------------------------------------------
// MMA kernel
// ----------------------------------------------------------------------
struct UmmaProb {
  const float *A;
  float *C;
  const float *fac;
  const __nv_bfloat16 *B[3];  // split B terms of this problem's mode
  int reflect;                // read A reflected (see TcProblem)
};

struct UmmaBatch {
  UmmaProb p[kMaxBatch];
};

struct UmmaArgs {
  int M, N, Np, K, Kp;
  int tnc;            // columns per tile (multiple of 16, <= 128)
  const float2 *shift;
  int fac_staged;     // factor block staged in shared memory for the epilogue
  uint32_t tmem_cols;
  long long spin;     // iteration limit of the pipeline waits
};

template <int EPI>
__global__ void __launch_bounds__(kThreads, 1) umma_kernel(const __grid_constant__ UmmaBatch P, UmmaArgs A) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t afull[STAGES], bfull[STAGES], empty[STAGES], hfull[2], hempty[2],
      done;
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  const int prob = blockIdx.z, nt = blockIdx.y, mt = blockIdx.x;
  const int warp = threadIdx.x >> 5;
  const int tnc = A.tnc, n0 = nt * tnc;
  const uint32_t b_term = (uint32_t)tnc * KB * 2;  // one B term of a stage
  const uint32_t stage_bytes = kABytes + 3 * b_term;
  const int nkb = A.Kp / KB;
  const int nchunk = (nkb + kChunk - 1) / kChunk;
  const UmmaProb &Q = P.p[prob];
  const long long spin = A.spin;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&afull[s], kProducers);
      mbar_init(&bfull[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&hfull[b], 1);
      mbar_init(&hempty[b], kProducers);
    }
    mbar_init(&done, 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kProducers / 32) {
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
  const uint32_t colL = 2u * (uint32_t)tnc;  // the correction-pair accumulator

  // row threads: rows 32 (warp % 4) + lane, K half and column half warp / 4
  const int half = (warp >> 2) & 1;
  const int col0 = half * CH;                                  // first tile column of this thread
  const int ncol = max(0, min(CH, tnc - col0));                // its columns (multiple of 16)
  float acc[CH];  // this thread's sum of the drained H chunks
#pragma unroll
  for (int j = 0; j < CH; ++j) acc[j] = 0.0f;
  const uint32_t tmem_lane = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  volatile int *vfail = &fail;

  if (threadIdx.x < kProducers) {
    // ---- row threads: FP32 A -> three BF16 terms in the stage; drain H
    const int r = (warp & 3) * 32 + (threadIdx.x & 31);
    const long long gm = (long long)mt * TH + r;
    const bool row_ok = gm < A.M;
    long long src = gm;
    uint32_t neg = 0;  // sign flip of the BF16 terms (reflected real part)
    if (Q.reflect && row_ok) {
      const long long x = gm >> 1, nxh = A.M >> 1;
      src = 2 * (x == 0 ? 0 : nxh - x) + (gm & 1);
      if ((gm & 1) == 0) neg = 0x80008000u;
    }
    const float *Arow = Q.A + src;
    float v[KH];
    auto load = [&](int kb) {
#pragma unroll
      for (int k = 0; k < KH; ++k) {
        const int gk = kb * KB + half * KH + k;
        v[k] = (row_ok && gk < A.K) ? Arow[(long long)gk * A.M] : 0.0f;
      }
    };
    // drain chunk c (H accumulator c & 1) into acc, then hand it back
    auto drain = [&](int c) {
      const int b = c & 1;
      bool ok = !*vfail && mbar_wait(&hfull[b], (uint32_t)(c >> 1) & 1u, spin);
      if (!ok) {
        *vfail = 1;
        atomicCAS(&g_umma_error, 0, 4);
      } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        tmem_add_row(acc, tmem_lane, (uint32_t)(b * tnc + col0), ncol);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      }
      mbar_arrive(&hempty[b]);
    };
    int drained = 0;
    load(0);
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % STAGES;
      bool ok = true;
      if (kb >= STAGES) ok = !*vfail && mbar_wait(&empty[s], (uint32_t)(kb / STAGES - 1) & 1u, spin);
      if (!ok) {
        *vfail = 1;
        atomicCAS(&g_umma_error, 0, 3);
      } else {
        unsigned char *st = smem + (size_t)s * stage_bytes;
        const int rr = r;
#pragma unroll
        for (int kh = 0; kh < KH / 8; ++kh) {
          const int kg = half * (KH / 8) + kh;  // 8-wide K group of the step
          uint32_t w0[4], w1[4], w2[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            uint32_t t0[2], t1[2], t2[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
              const float x = v[kh * 8 + 2 * q + e];
              const __nv_bfloat16 b0 = __float2bfloat16_rn(x);
              const float r1 = x - __bfloat162float(b0);
              const __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
              const float r2 = r1 - __bfloat162float(b1);
              t0[e] = bf16_bits(b0);
              t1[e] = bf16_bits(b1);
              t2[e] = bf16_bits(__float2bfloat16_rn(r2));
            }
            w0[q] = (t0[0] | (t0[1] << 16)) ^ neg;
            w1[q] = (t1[0] | (t1[1] << 16)) ^ neg;
            w2[q] = (t2[0] | (t2[1] << 16)) ^ neg;
          }
          // element (rr, k) of a 128 x 32 term block at ((rr/8)*4 + k/8)*64 + (rr%8)*8 + k%8
          const uint32_t off = (((rr >> 3) * (KB / 8) + kg) * 64 + (rr & 7) * 8) * 2;
          *reinterpret_cast<uint4 *>(st + off) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
          *reinterpret_cast<uint4 *>(st + kATermBytes + off) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
          *reinterpret_cast<uint4 *>(st + 2 * kATermBytes + off) =
              make_uint4(w2[0], w2[1], w2[2], w2[3]);
        }
      }
      // generic-proxy stores -> visible to the tensor core (async proxy)
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&afull[s]);
      if (kb + 1 < nkb) load(kb + 1);
      // chunk c is drained once the stages of chunk c + 1 are written, so the
      // tensor core has the next chunk's operands while the rows drain
      const int c_ready = (kb + 1) / kChunk - 2;
      while (drained <= c_ready) drain(drained++);
    }
    while (drained < nchunk) drain(drained++);
  } else if (EPI == TC_EPI_SHIFT_FAC && A.fac_staged && threadIdx.x > kProducers) {
    // idle lanes of the MMA warp: start the tile's factor block (read by the
    // epilogue) towards L2, one or two 128-byte lines per column
    const int xr0p = mt * (TH / 2);
    const int rows = min(TH / 2, (A.M >> 1) - xr0p);
    for (int t = threadIdx.x - kProducers - 1; t < 2 * tnc; t += 31) {
      const int n = n0 + (t >> 1), part = t & 1;
      if (part * 32 < rows && n < A.N)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(Q.fac + xr0p + part * 32 + (long long)(A.M >> 1) * n));
    }
  } else if (threadIdx.x == kProducers) {
    // ---- B streaming and MMA issue
    const uint32_t idesc = idesc_bf16(TH, tnc);
    int last_b[STAGES];
    for (int s = 0; s < STAGES; ++s) last_b[s] = -1;
    auto load_b = [&](int kb) {
      const int s = kb % STAGES;
      unsigned char *st = smem + (size_t)s * stage_bytes + kABytes;
      mbar_expect_tx(&bfull[s], 3 * b_term);
      for (int t = 0; t < 3; ++t)
        bulk_g2s(st + t * b_term, Q.B[t] + (long long)kb * A.Np * KB + (long long)n0 * KB, b_term,
                 &bfull[s]);
      last_b[s] = kb;
    };
    bool ok = true;
    for (int kb = 0; kb < STAGES && kb < nkb; ++kb) load_b(kb);
    for (int kb = 0; kb < nkb && ok; ++kb) {
      const int s = kb % STAGES;
      const uint32_t par = (uint32_t)(kb / STAGES) & 1u;
      const int c = kb / kChunk;
      const bool first = (kb % kChunk) == 0;
      const bool last = (kb % kChunk) == kChunk - 1 || kb == nkb - 1;
      if (first && c >= 2 && !mbar_wait(&hempty[c & 1], (uint32_t)((c >> 1) - 1) & 1u, spin)) {
        ok = false;
        break;
      }
      if (!mbar_wait(&bfull[s], par, spin) || !mbar_wait(&afull[s], par, spin)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      unsigned char *st = smem + (size_t)s * stage_bytes;
      const uint32_t dH = tmem + (uint32_t)((c & 1) * tnc), dL = tmem + colL;
      // term pairs (i, j): (0, 0) into H, the others into L
      const int pi[6] = {0, 2, 1, 0, 1, 0}, pj[6] = {0, 0, 1, 2, 0, 1};
#pragma unroll
      for (int q = 0; q < 6; ++q) {
#pragma unroll
        for (int ks = 0; ks < KB / 16; ++ks) {
          const uint64_t bd = smem_desc(st + kABytes + pj[q] * b_term + ks * 256, 128, (KB / 8) * 128);
          const uint64_t ad = smem_desc(st + pi[q] * kATermBytes + ks * 256, 128, (KB / 8) * 128);
          if (q == 0)
            umma_bf16(dH, ad, bd, idesc, (first && ks == 0) ? 0u : 1u);
          else
            umma_bf16(dL, ad, bd, idesc, (kb == 0 && q == 1 && ks == 0) ? 0u : 1u);
        }
      }
      umma_commit(&empty[s]);
      if (last) umma_commit(&hfull[c & 1]);
      // refill the stage of the previous step once its MMAs have drained
      if (kb >= 1 && kb - 1 + STAGES < nkb) {
        const int sp = (kb - 1) % STAGES;
        if (!mbar_wait(&empty[sp], (uint32_t)((kb - 1) / STAGES) & 1u, spin)) {
          ok = false;
          break;
        }
        load_b(kb - 1 + STAGES);
      }
    }
    umma_commit(&done);
    if (!ok) {
      *vfail = 1;
      atomicCAS(&g_umma_error, 0, 1);
      // let the bulk copies already issued land before the CTA exits
      for (int s = 0; s < STAGES; ++s)
        if (last_b[s] >= 0) mbar_wait(&bfull[s], (uint32_t)(last_b[s] / STAGES) & 1u, kSpinLimit);
    }
  }
  __syncthreads();
  // all MMAs complete before the L accumulator is read and the stages are
  // reused (the full limit: this wait must not leave MMAs in flight)
  const bool drained = mbar_wait(&done, 0, kSpinLimit);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool use = __syncthreads_and(drained && !fail);
  if (!drained && threadIdx.x == 0) atomicCAS(&g_umma_error, 0, 2);
  // factor epilogue: the tile's factor block (64 x-rows x tnc columns, one
  // contiguous run per column, started towards L2 during the K loop) is
  // copied into the drained stages with 16-byte loads, all threads at once
  constexpr int nxr = TH / 2;
  const int xr0 = mt * nxr;
  const float *facs = reinterpret_cast<const float *>(smem);
  bool fac_smem = false;
  if (EPI == TC_EPI_SHIFT_FAC && use && A.fac_staged) {
    const int rows = min(nxr, (A.M >> 1) - xr0);  // a multiple of 4 (host check)
    constexpr int nq = nxr / 4;
    const int total = nq * tnc;  // float4 per column, in the block
    float4 *dst = reinterpret_cast<float4 *>(smem);
    constexpr int kBatch = 13;
    for (int t0 = threadIdx.x; t0 < total; t0 += kBatch * (int)blockDim.x) {
      float4 vv[kBatch];
#pragma unroll
      for (int b = 0; b < kBatch; ++b) {
        const int t = t0 + b * (int)blockDim.x;
        const int n = t / nq, q = t - n * nq;
        vv[b] = (t < total && 4 * q < rows && n0 + n < A.N)
                    ? __ldg(reinterpret_cast<const float4 *>(Q.fac + xr0 + (long long)(A.M >> 1) * (n0 + n)) + q)
                    : make_float4(1.f, 1.f, 1.f, 1.f);
      }
#pragma unroll
      for (int b = 0; b < kBatch; ++b) {
        const int t = t0 + b * (int)blockDim.x;
        if (t < total) dst[t] = vv[b];
      }
    }
    __syncthreads();
    fac_smem = true;
  }
  if (use && threadIdx.x < kProducers) {
    tmem_add_row(acc, tmem_lane, colL + (uint32_t)col0, ncol);  // + the correction pairs
    const int row = (warp & 3) * 32 + (threadIdx.x & 31);
    const long long gm = (long long)mt * TH + row;
    float2 sh = make_float2(1.f, 0.f);
    if (EPI != TC_EPI_STORE && gm < A.M) sh = A.shift[gm >> 1];
    float *C = Q.C;
    const float *fac = Q.fac;
    const bool rok = gm < A.M;
#pragma unroll
    for (int jj = 0; jj < CH; ++jj) {
      if (jj < ncol) {
        float x = acc[jj];
        const int j = col0 + jj, n = n0 + j;
        if (EPI != TC_EPI_STORE) {
          // rows 2x (re) and 2x+1 (im) sit in adjacent lanes
          const float other = __shfl_xor_sync(0xffffffffu, x, 1);
          const float re = (row & 1) ? other : x, im = (row & 1) ? x : other;
          x = (row & 1) ? (re * sh.y + im * sh.x) : (re * sh.x - im * sh.y);
          if (EPI == TC_EPI_SHIFT_FAC) {
            const float f = fac_smem ? facs[j * nxr + (row >> 1)]
                                     : ((rok && n < A.N) ? __ldg(fac + (gm >> 1) + (long long)(A.M >> 1) * n)
                                                         : 1.0f);
            x *= f;
          }
        }
        if (rok && n < A.N) C[gm + (long long)n * A.M] = x;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kProducers / 32) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(A.tmem_cols)
                 : "memory");
  }
}

inline long long rup(long long a, long long b) { return (a + b - 1) / b * b; }

}  // namespace

namespace chm {

int tc_umma_launch(const TcProblem *p, int count, int M, int N, int K, int epi, const float2 *shift,
                   cudaStream_t st) {
  const int tnc = tc_tile_cols(N), ntn = tc_col_tiles(N), Np = tc_np(N), Kp = (int)rup(K, KB);
  if (tnc > TH || tnc % 16) {
    set_error("umma: bad column tile %d", tnc);
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
  const int mt = (int)((M + TH - 1) / TH);
  const uint32_t b_term = (uint32_t)tnc * KB * 2;
  const size_t stage_bytes = kABytes + 3 * (size_t)b_term;
  const size_t smem = (size_t)STAGES * stage_bytes + 1024;
  void (*kern)(const UmmaBatch, UmmaArgs) =
      epi == TC_EPI_STORE ? umma_kernel<TC_EPI_STORE>
                          : (epi == TC_EPI_SHIFT ? umma_kernel<TC_EPI_SHIFT> : umma_kernel<TC_EPI_SHIFT_FAC>);
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  uint32_t cols = 32;
  while (cols < (uint32_t)(3 * tnc)) cols <<= 1;  // H0, H1 and L
  UmmaArgs ua{};
  ua.M = M;
  ua.N = N;
  ua.Np = Np;
  ua.K = K;
  ua.Kp = Kp;
  ua.tnc = tnc;
  ua.shift = shift;
  ua.tmem_cols = cols;
  ua.spin = g_spin_limit;
  // the staged factor block is read with 16-byte loads: M/2 a multiple of 4
  // and 16-byte aligned factor planes; it (64 x tnc FP32) fits in the stages
  ua.fac_staged = (epi == TC_EPI_SHIFT_FAC && (M / 2) % 4 == 0 &&
                   (size_t)(TH / 2) * tnc * 4 <= (size_t)STAGES * stage_bytes) ? 1 : 0;
  for (int i = 0; i < count && ua.fac_staged; ++i)
    if (!p[i].fac || (reinterpret_cast<uintptr_t>(p[i].fac) & 15)) ua.fac_staged = 0;
  for (int c0 = 0; c0 < count; c0 += kMaxBatch) {
    const int cnt = count - c0 < kMaxBatch ? count - c0 : kMaxBatch;
    UmmaBatch ub;
    for (int i = 0; i < cnt; ++i) {
      const TcProblem &q = p[c0 + i];
      ub.p[i] = UmmaProb{q.A, q.C, q.fac,
                         {reinterpret_cast<const __nv_bfloat16 *>(q.B.bf[0]),
                          reinterpret_cast<const __nv_bfloat16 *>(q.B.bf[1]),
                          reinterpret_cast<const __nv_bfloat16 *>(q.B.bf[2])},
                         q.reflect};
    }
    kern<<<dim3(mt, ntn, cnt), kThreads, smem, st>>>(ub, ua);
    count_launch();
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

extern "C" int64_t chm_sp_set_umma_spin_limit(int64_t polls) {
  const long long prev = g_spin_limit;
  g_spin_limit = polls < 0 ? kSpinLimit : polls;
  return prev;
}
