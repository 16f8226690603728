// tcgen05 (5th-generation tensor core) GEMM of the split-precision form.
//
//   C(M, N) = A(M, K) * B(K, N),  A, C FP32 column-major, B a prepared
//   operator mode; computed as sum_{i+j<=2} A_i B_j with A = A0+A1+A2 and
//   B = B0+B1+B2 the 3-term BF16 splits, accumulated in FP32 in TMEM.
//
// Structure:
//   1. split kernel: A (FP32) -> three BF16 planes written in the tensor-core
//      operand layout (K-major, core matrices of 8 rows x 16 bytes), one
//      128 x 32 tile per (M tile, K block), contiguous;
//   2. MMA kernel: one CTA per 128-row M tile and problem.  Thread 0 streams
//      the A and B tiles of each 32-wide K block into a 3-stage shared-memory
//      ring with bulk-copy TMA (cp.async.bulk, completion on an mbarrier),
//      issues 12 tcgen05.mma (6 term pairs x 2 K steps of 16) per block into
//      a TMEM accumulator and releases stages with tcgen05.commit; the four
//      warps then read TMEM (tcgen05.ld 32x32b) and apply the epilogue.
// Every mbarrier wait has an iteration limit; on timeout the CTA records an
// error, waits (bounded) for its own transfers, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "tc_gemm.cuh"

using namespace chm;

namespace {

constexpr int TM = 128;        // rows per CTA (UMMA M)
constexpr int KB = 32;         // K block (elements)
constexpr int STAGES = 3;
constexpr int kSplitThreads = 256;
constexpr long long kSpinLimit = 1LL << 20;  // try_wait polls; each may block briefly

__device__ int g_umma_error;  // first failing CTA records a code here

// ----------------------------------------------------------------------
// A -> 3 BF16 planes in tile layout
// ----------------------------------------------------------------------
struct SplitProb {
  const float *A[64];
  __nv_bfloat16 *T[64];  // 3 planes of tiles, plane stride = tile_stride
  int count;
};

// tile (mt, kb) of a plane holds rows mt*128.., k kb*32..; element (r, k) at
// ((r/8)*(KB/8) + k/8)*64 + (r%8)*8 + k%8
__global__ void __launch_bounds__(kSplitThreads)
    split_a_kernel(SplitProb P, int M, int K, int Kp, long long plane_elems) {
  __shared__ float tile[KB][TM + 1];
  const int prob = blockIdx.z;
  const int mt = blockIdx.x, kb = blockIdx.y;
  const float *A = P.A[prob];
  // coalesced load along m
  for (int t = threadIdx.x; t < TM * KB; t += kSplitThreads) {
    const int r = t % TM, k = t / TM;
    const int gm = mt * TM + r, gk = kb * KB + k;
    tile[k][r] = (gm < M && gk < K) ? A[gm + (long long)gk * M] : 0.0f;
  }
  __syncthreads();
  const int nkb = Kp / KB;
  const long long tbase = ((long long)mt * nkb + kb) * (TM * KB);
  // each thread writes 8 consecutive k of one row (16 bytes) per term
  for (int t = threadIdx.x; t < TM * (KB / 8); t += kSplitThreads) {
    const int r = t % TM, kg = t / TM;
    __align__(16) __nv_bfloat16 o0[8], o1[8], o2[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float v = tile[kg * 8 + q][r];
      const __nv_bfloat16 b0 = __float2bfloat16_rn(v);
      const float r1 = v - __bfloat162float(b0);
      const __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
      const float r2 = r1 - __bfloat162float(b1);
      o0[q] = b0;
      o1[q] = b1;
      o2[q] = __float2bfloat16_rn(r2);
    }
    const long long off = tbase + ((long long)(r / 8) * (KB / 8) + kg) * 64 + (r % 8) * 8;
    __nv_bfloat16 *T = P.T[prob];
    *reinterpret_cast<uint4 *>(T + off) = *reinterpret_cast<uint4 *>(o0);
    *reinterpret_cast<uint4 *>(T + plane_elems + off) = *reinterpret_cast<uint4 *>(o1);
    *reinterpret_cast<uint4 *>(T + 2 * plane_elems + off) = *reinterpret_cast<uint4 *>(o2);
  }
}

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

// bounded wait for the phase with parity `parity` to complete
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (long long it = 0; it < kSpinLimit; ++it) {
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

// ----------------------------------------------------------------------
// MMA kernel
// ----------------------------------------------------------------------
struct UmmaProb {
  const __nv_bfloat16 *At[64];  // split A planes (3 consecutive, plane stride)
  float *C[64];
  const float *fac[64];
  int count;
};

struct UmmaArgs {
  int M, N, Np, K, Kp;
  long long a_plane;             // elements per A term plane
  const __nv_bfloat16 *B[3];     // B term tiles for this mode
  const float2 *shift;
  int epi;
  uint32_t tmem_cols;
};

__global__ void __launch_bounds__(128, 1) umma_kernel(UmmaProb P, UmmaArgs A) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], done;
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  const int prob = blockIdx.y, mt = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t a_bytes = TM * KB * 2;          // one A term tile
  const uint32_t b_bytes = (uint32_t)A.Np * KB * 2;  // one B term tile
  const uint32_t stage_bytes = 3 * a_bytes + 3 * b_bytes;
  const int nkb = A.Kp / KB;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
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

  if (threadIdx.x == 0) {
    const __nv_bfloat16 *Abase = P.At[prob];
    auto load_stage = [&](int kb) {
      unsigned char *st = smem + (size_t)(kb % STAGES) * stage_bytes;
      mbar_expect_tx(&full[kb % STAGES], stage_bytes);
      for (int t = 0; t < 3; ++t) {
        const __nv_bfloat16 *src = Abase + (long long)t * A.a_plane + ((long long)mt * nkb + kb) * (TM * KB);
        bulk_g2s(st + t * a_bytes, src, a_bytes, &full[kb % STAGES]);
      }
      for (int t = 0; t < 3; ++t) {
        const __nv_bfloat16 *src = A.B[t] + (long long)kb * A.Np * KB;
        bulk_g2s(st + 3 * a_bytes + t * b_bytes, src, b_bytes, &full[kb % STAGES]);
      }
    };
    const uint32_t idesc = idesc_bf16(TM, A.Np);
    bool ok = true;
    for (int kb = 0; kb < STAGES && kb < nkb; ++kb) load_stage(kb);
    for (int kb = 0; kb < nkb && ok; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait(&full[s], (uint32_t)(kb / STAGES) & 1u)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      unsigned char *st = smem + (size_t)s * stage_bytes;
      // term pairs (i, j) with i + j <= 2, smallest terms first
      const int pi[6] = {2, 1, 0, 1, 0, 0}, pj[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
      for (int q = 0; q < 6; ++q) {
#pragma unroll
        for (int ks = 0; ks < KB / 16; ++ks) {
          const uint64_t ad = smem_desc(st + pi[q] * a_bytes + ks * 256, 128, (KB / 8) * 128);
          const uint64_t bd = smem_desc(st + 3 * a_bytes + pj[q] * b_bytes + ks * 256, 128, (KB / 8) * 128);
          umma_bf16(tmem, ad, bd, idesc, (kb > 0 || q > 0 || ks > 0) ? 1u : 0u);
        }
      }
      umma_commit(&empty[s]);
      // refill the stage of the previous block once its MMAs have drained
      if (kb >= 1 && kb - 1 + STAGES < nkb) {
        const int sp = (kb - 1) % STAGES;
        if (!mbar_wait(&empty[sp], (uint32_t)((kb - 1) / STAGES) & 1u)) {
          ok = false;
          break;
        }
        load_stage(kb - 1 + STAGES);
      }
    }
    umma_commit(&done);
    if (!ok) {
      fail = 1;
      atomicCAS(&g_umma_error, 0, 1);
      // let the bulk copies already issued land before the CTA exits
      for (int s = 0; s < STAGES; ++s) mbar_wait(&full[s], 0), mbar_wait(&full[s], 1);
    }
  }
  __syncthreads();
  // all MMAs complete before the accumulator is read (bounded wait)
  const bool drained = mbar_wait(&done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool use = __syncthreads_and(drained && !fail);
  if (!drained && threadIdx.x == 0) atomicCAS(&g_umma_error, 0, 2);
  if (use) {
    const int row = warp * 32 + lane;  // TMEM lane = row of the tile
    const int gm = mt * TM + row;
    float2 sh = make_float2(1.f, 0.f);
    if (A.epi != TC_EPI_STORE && gm < A.M) sh = A.shift[gm >> 1];
    float *C = P.C[prob];
    const float *fac = P.fac[prob];
    for (int c0 = 0; c0 < A.Np; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
            "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float x = __uint_as_float(v[j]);
        if (A.epi != TC_EPI_STORE) {
          // rows 2x (re) and 2x+1 (im) sit in adjacent lanes
          const float other = __shfl_xor_sync(0xffffffffu, x, 1);
          const float re = (row & 1) ? other : x, im = (row & 1) ? x : other;
          x = (row & 1) ? (re * sh.y + im * sh.x) : (re * sh.x - im * sh.y);
          const int n = c0 + j;
          if (A.epi == TC_EPI_SHIFT_FAC && gm < A.M && n < A.N) x *= fac[(gm >> 1) + (long long)(A.M >> 1) * n];
        }
        const int n = c0 + j;
        if (gm < A.M && n < A.N) C[gm + (long long)n * A.M] = x;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(A.tmem_cols)
                 : "memory");
  }
}

inline long long rup(long long a, long long b) { return (a + b - 1) / b * b; }

}  // namespace

namespace chm {

int64_t tc_scratch_bytes(int64_t M, int64_t K, int64_t count) {
  const int64_t c = count < 64 ? count : 64;
  return (int64_t)3 * rup(M, TM) * rup(K, KB) * 2 * c + 256;
}

int tc_umma_launch(const TcProblem *p, int count, int M, int N, int K, const TcOperand &B, int epi,
                   const float2 *shift, void *scratch, int64_t scratch_bytes, cudaStream_t st) {
  const int Np = (int)rup(N, 16), Kp = (int)rup(K, KB);
  const int Kp_ops = Kp;
  if (Np > 256) {
    set_error("umma: N must be <= 256");
    return CHM_ERR_RANGE;
  }
  if (M % 2) {
    set_error("umma: M must be even (complex rows)");
    return CHM_ERR_ARG;
  }
  const int mt = (int)((M + TM - 1) / TM);
  const long long a_plane = (long long)mt * TM * Kp;  // elements per term plane
  (void)Kp_ops;
  if (!scratch || scratch_bytes < tc_scratch_bytes(M, K, count)) {
    set_error("umma: scratch of %lld bytes < %lld required", (long long)scratch_bytes,
              (long long)tc_scratch_bytes(M, K, count));
    return CHM_ERR_WS;
  }
  struct {
    void *p;
  } S{scratch};
  const uint32_t a_bytes = TM * KB * 2, b_bytes = (uint32_t)Np * KB * 2;
  const size_t smem = (size_t)STAGES * (3 * a_bytes + 3 * b_bytes) + 1024;
  cudaFuncSetAttribute(umma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  uint32_t cols = 32;
  while (cols < (uint32_t)Np) cols <<= 1;
  for (int c0 = 0; c0 < count; c0 += 64) {
    const int cnt = count - c0 < 64 ? count - c0 : 64;
    SplitProb sp{};
    UmmaProb up{};
    sp.count = up.count = cnt;
    for (int i = 0; i < cnt; ++i) {
      __nv_bfloat16 *T = reinterpret_cast<__nv_bfloat16 *>(S.p) + (size_t)3 * a_plane * i;
      sp.A[i] = p[c0 + i].A;
      sp.T[i] = T;
      up.At[i] = T;
      up.C[i] = p[c0 + i].C;
      up.fac[i] = p[c0 + i].fac;
    }
    split_a_kernel<<<dim3(mt, Kp / KB, cnt), kSplitThreads, 0, st>>>(sp, M, K, Kp, a_plane);
    count_launch();
    UmmaArgs ua{};
    ua.M = M;
    ua.N = N;
    ua.Np = Np;
    ua.K = K;
    ua.Kp = Kp;
    ua.a_plane = a_plane;
    for (int t = 0; t < 3; ++t) ua.B[t] = reinterpret_cast<const __nv_bfloat16 *>(B.bf[t]);
    ua.shift = shift;
    ua.epi = epi;
    ua.tmem_cols = cols;
    umma_kernel<<<dim3(mt, cnt), 128, smem, st>>>(up, ua);
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
  int v = 0;
  cudaMemcpyFromSymbol(&v, g_umma_error, sizeof(int));
  return v;
}
