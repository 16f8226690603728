// Dense products of the split-precision form and their operator sets.
//
// Engines:
//   0  FP32 SIMT (register-tiled), the accuracy reference of the split form
//   1  tcgen05 tensor cores, 3-term split-BF16 with FP32 accumulation in
//      TMEM (tc_umma.cu)
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_bf16.h>

#include "tc_gemm.cuh"

using namespace chm;

namespace {

constexpr int TB_M = 64, TB_N = 64, TB_K = 16, kThreads = 256;
constexpr int kMaxProb = 64;

struct Prob32 {
  TcProblem p[kMaxProb];
  int count;
};

template <int EPI>
__global__ void __launch_bounds__(kThreads)
    sgemm_kernel(const __grid_constant__ Prob32 batch, int M, int N, int K,
                 const float2 *__restrict__ shift) {
  __shared__ __align__(16) float As[TB_K][TB_M];
  __shared__ __align__(16) float Bs[TB_K][TB_N + 1];
  const TcProblem &P = batch.p[blockIdx.z];
  const float *__restrict__ B = P.B.f32;
  const int m0 = blockIdx.x * TB_M, n0 = blockIdx.y * TB_N;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += TB_K) {
    for (int t = threadIdx.x; t < TB_M * TB_K; t += kThreads) {
      int mm = t % TB_M, kk = t / TB_M;
      int gm = m0 + mm, gk = k0 + kk;
      float a = 0.0f;
      if (gm < M && gk < K) {
        int src = gm;
        float sgn = 1.0f;
        if (P.reflect) {
          const int x = gm >> 1;
          src = 2 * (x == 0 ? 0 : (M >> 1) - x) + (gm & 1);
          if ((gm & 1) == 0) sgn = -1.0f;
        }
        a = sgn * P.A[src + (i64)gk * M];
      }
      As[kk][mm] = a;
    }
    for (int t = threadIdx.x; t < TB_N * TB_K; t += kThreads) {
      int kk = t % TB_K, nn = t / TB_K;
      int gk = k0 + kk, gn = n0 + nn;
      Bs[kk][nn] = (gk < K && gn < N) ? B[gk + (i64)gn * K] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TB_K; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tx * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gn = n0 + ty * 4 + j;
    if (gn >= N) continue;
#pragma unroll
    for (int i = 0; i < 4; i += 2) {
      const int gm = m0 + tx * 4 + i;
      if (gm >= M) continue;
      float2 v = make_float2(acc[i][j], acc[i + 1][j]);
      if (EPI != TC_EPI_STORE) {
        const int x = gm >> 1;
        const float2 s = shift[x];
        v = make_float2(v.x * s.x - v.y * s.y, v.x * s.y + v.y * s.x);
        if (EPI == TC_EPI_SHIFT_FAC) {
          const float f = P.fac[x + (i64)(M >> 1) * gn];
          v.x *= f;
          v.y *= f;
        }
      }
      *reinterpret_cast<float2 *>(P.C + gm + (i64)gn * M) = v;
    }
  }
}

// FP64 matrices -> FP32 copy and 3-term BF16 split.  The split terms are
// stored per (mode, 32-wide K block) as the tensor-core operand tile of
// Np = tc_np(N) columns: core matrices of 8 rows (n) x 16 bytes (8 k
// values), ordered k-group fastest (LBO = 128 B), then row group (SBO =
// 512 B), so the columns of one column tile form a contiguous run.
__global__ void prepare_kernel(const double *__restrict__ mats, int K, int N, int nmodes, int Kp,
                               int Np, float *__restrict__ f32, __nv_bfloat16 *__restrict__ t0,
                               __nv_bfloat16 *__restrict__ t1, __nv_bfloat16 *__restrict__ t2) {
  const i64 total = (i64)Kp * Np * nmodes;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < total; t += (i64)gridDim.x * blockDim.x) {
    const int k = (int)(t % Kp);
    const i64 rest = t / Kp;
    const int n = (int)(rest % Np);
    const int m = (int)(rest / Np);
    const double v = (k < K && n < N) ? mats[k + (i64)K * (n + (i64)N * m)] : 0.0;
    if (k < K && n < N) f32[k + (i64)K * (n + (i64)N * m)] = (float)v;
    const __nv_bfloat16 b0 = __double2bfloat16(v);
    const double r1 = v - (double)__bfloat162float(b0);
    const __nv_bfloat16 b1 = __double2bfloat16(r1);
    const double r2 = r1 - (double)__bfloat162float(b1);
    const __nv_bfloat16 b2 = __double2bfloat16(r2);
    // tile position
    const int kb = k / 32, kk = k % 32;
    const i64 tile = ((i64)m * (Kp / 32) + kb) * ((i64)Np * 32);
    const i64 off = tile + ((i64)(n / 8) * 4 + kk / 8) * 64 + (n % 8) * 8 + (kk % 8);
    t0[off] = b0;
    t1[off] = b1;
    t2[off] = b2;
  }
}

inline i64 rup(i64 a, i64 b) { return (a + b - 1) / b * b; }

}  // namespace

namespace chm {

int tc_umma_launch(const TcProblem *p, int count, int M, int N, int K, int epi, const float2 *shift,
                   void *ws, long long ws_bytes, cudaStream_t st);

// engine 1: tensor cores (every product of the split form); 0: the FP32 SIMT
// kernel, reached only through chm_sp_gemm as the tests' accuracy reference
static int launch(const TcProblem *p, int count, int M, int N, int K, int epi, const float2 *shift,
                  void *ws, long long ws_bytes, cudaStream_t st, int engine) {
  if (count <= 0) return CHM_OK;
  count_gemm_flops((double)count * 2.0 * M * N * K);
  if (engine == 1) return tc_umma_launch(p, count, M, N, K, epi, shift, ws, ws_bytes, st);
  for (int c0 = 0; c0 < count; c0 += kMaxProb) {
    Prob32 b{};
    b.count = count - c0 < kMaxProb ? count - c0 : kMaxProb;
    for (int i = 0; i < b.count; ++i) b.p[i] = p[c0 + i];
    dim3 grid((M + TB_M - 1) / TB_M, (N + TB_N - 1) / TB_N, b.count);
    if (epi == TC_EPI_STORE) sgemm_kernel<TC_EPI_STORE><<<grid, kThreads, 0, st>>>(b, M, N, K, shift);
    else if (epi == TC_EPI_SHIFT) sgemm_kernel<TC_EPI_SHIFT><<<grid, kThreads, 0, st>>>(b, M, N, K, shift);
    else sgemm_kernel<TC_EPI_SHIFT_FAC><<<grid, kThreads, 0, st>>>(b, M, N, K, shift);
    count_launch();
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("sgemm: %s", cudaGetErrorString(e));
    return CHM_ERR_CUDA;
  }
  return CHM_OK;
}

int tc_gemm_launch(const TcProblem *p, int count, int M, int N, int K, int epi, const float2 *shift,
                   void *ws, long long ws_bytes, cudaStream_t st) {
  return launch(p, count, M, N, K, epi, shift, ws, ws_bytes, st, 1);
}

TcMatrices tc_matrices(const chm_sp_ops *ops) {
  TcMatrices T;
  memset(&T, 0, sizeof(T));
  const i64 Kp = rup(ops->K, 32), Np = tc_np(ops->N);
  for (int m = 0; m < ops->nmodes && m < 16; ++m) {
    TcOperand &o = T.mode[m];
    o.K = ops->K;
    o.N = ops->N;
    o.f32 = ops->f32 + (i64)ops->K * ops->N * m;
    for (int t = 0; t < 3; ++t)
      o.bf[t] = ops->bf16[t] ? reinterpret_cast<const uint16_t *>(ops->bf16[t]) + Kp * Np * m : nullptr;
  }
  return T;
}

}  // namespace chm

extern "C" {

int64_t chm_sp_ops_bytes(int64_t K, int64_t N, int64_t nmodes) {
  if (K <= 0 || N <= 0 || N > 65536 || nmodes <= 0) return 0;
  const i64 Kp = rup(K, 32), Np = tc_np((int)N);
  return rup(4 * K * N * nmodes, 256) + 3 * rup(2 * Kp * Np * nmodes, 256);
}

int chm_sp_prepare_ops(chm_sp_ops *ops, const double *mats, int64_t K, int64_t N, int64_t nmodes,
                       void *buf, int64_t buf_bytes, void *stream) {
  CHM_REQUIRE(ops && mats && buf && K > 0 && N > 0 && nmodes > 0 && nmodes <= 16,
              "sp_prepare_ops: bad args");
  CHM_REQUIRE(N <= 65536, "sp_prepare_ops: N must be <= 65536");
  CHM_REQUIRE(buf_bytes >= chm_sp_ops_bytes(K, N, nmodes), "sp_prepare_ops: buffer too small");
  const i64 Kp = rup(K, 32), Np = tc_np((int)N);
  char *p = reinterpret_cast<char *>(buf);
  float *f32 = reinterpret_cast<float *>(p);
  p += rup(4 * K * N * nmodes, 256);
  __nv_bfloat16 *t[3];
  for (int i = 0; i < 3; ++i) {
    t[i] = reinterpret_cast<__nv_bfloat16 *>(p);
    p += rup(2 * Kp * Np * nmodes, 256);
  }
  prepare_kernel<<<grid_for(Kp * Np * nmodes, 256), 256, 0, as_stream(stream)>>>(
      mats, (int)K, (int)N, (int)nmodes, (int)Kp, (int)Np, f32, t[0], t[1], t[2]);
  count_launch();
  CHM_CHECK_LAUNCH();
  ops->K = (int32_t)K;
  ops->N = (int32_t)N;
  ops->nmodes = (int32_t)nmodes;
  ops->pad = 0;
  ops->f32 = f32;
  for (int i = 0; i < 3; ++i) ops->bf16[i] = t[i];
  return CHM_OK;
}

int64_t chm_sp_gemm_ws_bytes(int64_t M, int64_t K, int64_t count) {
  // the BF16 split of the A planes of the tensor-core path
  return tc_split_bytes((int)M, (int)K, (int)(count > 0 ? count : 1));
}

int chm_sp_gemm(float *C, const float *A, const chm_sp_ops *ops, int64_t mode, int64_t M, int engine,
                void *ws, int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(C && A && ops && mode >= 0 && mode < ops->nmodes && M > 0 && M % 2 == 0,
              "sp_gemm: bad args");
  CHM_REQUIRE(engine == 0 || engine == 1, "sp_gemm: engine must be 0 (SIMT) or 1 (tensor cores)");
  TcMatrices T = tc_matrices(ops);
  TcProblem p{A, C, nullptr, T.mode[mode], 0};
  return launch(&p, 1, (int)M, p.B.N, p.B.K, TC_EPI_STORE, nullptr, ws, ws_bytes, as_stream(stream),
                engine);
}

}  // extern "C"
