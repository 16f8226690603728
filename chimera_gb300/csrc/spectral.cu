// Fourier-Bessel transforms (fb_io.f90), spectral operators (fb_math*.f90)
// and the PSATD / Poisson elementwise kernels (maxwell_solvers.f90), FP64.
//
// The discrete Hankel transform along r and every mode-coupling product of
// fb_math is a dense real-matrix x complex-matrix product.  Viewing a complex
// column-major (nx, k) plane as a real (2 nx, k) matrix, each becomes a real
// GEMM  C(2nx, N) = A(2nx, K) * B(K, N)  with B the per-mode DHT or DpS2S /
// DmS2S matrix.  The FFT along x commutes with the DHT along r, so the
// forward transform is "FFT lines, then GEMM with the e^{-i kx leftX} x
// DepFact epilogue" and the inverse is "GEMM with the e^{+i kx leftX}
// epilogue, then inverse FFT lines with the eb_correction epilogue".
#include <math.h>

#include "common.cuh"
#include "fft.cuh"

using namespace chm;

namespace {

// -------------------------------------------------------------------------
// FP64 batched GEMM, register-tiled (64 x 64 tile, 4 x 4 per thread).
// GB300's FP64 pipe retires ~2 FMA/clk/SM, so this tiling is FP64-bound.
// -------------------------------------------------------------------------
constexpr int BM = 64, BN = 64, BK = 16, kGemmThreads = 256;
constexpr int kMaxProblems = 48;

struct GemmProblem {
  const double *A;    // (M, K) column-major, lda
  const double *B;    // (K, N) column-major, ldb
  double *C;          // (M, N) column-major, ldc
  const double *fac;  // optional real (M/2, N) factor, ld = M/2
};

struct GemmBatch {
  GemmProblem p[kMaxProblems];
  int count;
};

enum Epi { EPI_STORE = 0, EPI_SHIFT = 1 };

template <int EPI>
__global__ void __launch_bounds__(kGemmThreads)
    dgemm_kernel(GemmBatch batch, int M, int N, int K, i64 lda, i64 ldb, i64 ldc,
                 const double2 *__restrict__ shift) {
  __shared__ __align__(16) double As[BK][BM];
  __shared__ __align__(16) double Bs[BK][BN + 1];
  const GemmProblem P = batch.p[blockIdx.z];
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int k0 = 0; k0 < K; k0 += BK) {
    // A tile: BK x BM, coalesced along m
    for (int t = threadIdx.x; t < BM * BK; t += kGemmThreads) {
      int mm = t % BM, kk = t / BM;
      int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? P.A[gm + (i64)gk * lda] : 0.0;
    }
    // B tile: BK x BN, coalesced along k
    for (int t = threadIdx.x; t < BN * BK; t += kGemmThreads) {
      int kk = t % BK, nn = t / BK;
      int gk = k0 + kk, gn = n0 + nn;
      Bs[kk][nn] = (gk < K && gn < N) ? P.B[gk + (i64)gn * ldb] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tx * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gn = n0 + ty * 4 + j;
    if (gn >= N) continue;
#pragma unroll
    for (int i = 0; i < 4; i += 2) {
      const int gm = m0 + tx * 4 + i;  // even: real part row
      if (gm >= M) continue;
      double2 v = make_double2(acc[i][j], acc[i + 1][j]);
      if (EPI == EPI_SHIFT) {
        const int x = gm >> 1;
        v = cmul(v, shift[x]);
        if (P.fac) v = cscale(v, P.fac[x + (i64)(M >> 1) * gn]);
      }
      *reinterpret_cast<double2 *>(P.C + gm + (i64)gn * ldc) = v;
    }
  }
}

int gemm_launch(int epi, const GemmBatch &b, int M, int N, int K, i64 lda, i64 ldb, i64 ldc,
                const double2 *shift, cudaStream_t st) {
  if (b.count == 0) return CHM_OK;
  dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN, b.count);
  if (epi == EPI_STORE)
    dgemm_kernel<EPI_STORE><<<grid, kGemmThreads, 0, st>>>(b, M, N, K, lda, ldb, ldc, shift);
  else
    dgemm_kernel<EPI_SHIFT><<<grid, kGemmThreads, 0, st>>>(b, M, N, K, lda, ldb, ldc, shift);
  chm::count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("gemm: %s", cudaGetErrorString(e));
    return CHM_ERR_CUDA;
  }
  return CHM_OK;
}

// Batches larger than kMaxProblems are split.
struct GemmList {
  int epi;
  int M, N, K;
  i64 lda, ldb, ldc;
  const double2 *shift;
  GemmBatch b;
  cudaStream_t st;
  int err = CHM_OK;
  void add(const double *A, const double *B, double *C, const double *fac = nullptr) {
    if (err) return;
    count_gemm_flops(2.0 * M * N * K);  // algorithmic: 4 nx N K per complex x real product
    b.p[b.count++] = GemmProblem{A, B, C, fac};
    if (b.count == kMaxProblems) flush();
  }
  void flush() {
    if (err) return;
    err = gemm_launch(epi, b, M, N, K, lda, ldb, ldc, shift, st);
    b.count = 0;
  }
};

// shift[x] = exp(sign * i * kx[x] * leftX) (fb_io.f90:40 / :120)
__global__ void shift_kernel(double2 *shift, const double *kx, double leftX, int sign, i64 nx) {
  for (i64 x = blockIdx.x * (i64)blockDim.x + threadIdx.x; x < nx; x += (i64)gridDim.x * blockDim.x) {
    double s, c;
    sincos(leftX * kx[x], &s, &c);
    shift[x] = make_double2(c, sign * s);
  }
}

__global__ void zero_kernel(double2 *p, i64 n) {
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < n; t += (i64)gridDim.x * blockDim.x)
    p[t] = make_double2(0.0, 0.0);
}

// ext(x, k) = -conj(src(-x, k)) (index 0 fixed): the reflected m = 1 plane
// standing in for the m = -1 neighbour of m = 0 (fb_math.f90:35-36).
__global__ void reflect_kernel(double2 *__restrict__ dst, const double2 *__restrict__ src, i64 nx,
                               i64 nk) {
  const i64 n = nx * nk;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < n; t += (i64)gridDim.x * blockDim.x) {
    i64 x = t % nx, k = t / nx;
    i64 xs = x == 0 ? 0 : nx - x;
    dst[t] = make_double2(-src[xs + k * nx].x, src[xs + k * nx].y);
  }
}

// Workspace layout helpers ------------------------------------------------
struct WsCursor {
  char *p;
  i64 left;
  template <typename T>
  T *take(i64 n) {
    i64 bytes = ((n * (i64)sizeof(T)) + 255) / 256 * 256;
    if (bytes > left) return nullptr;
    T *r = reinterpret_cast<T *>(p);
    p += bytes;
    left -= bytes;
    return r;
  }
};

inline i64 rnd256(i64 b) { return (b + 255) / 256 * 256; }

}  // namespace

// =========================================================================
// fb_io.f90
// =========================================================================
extern "C" {

int64_t chm_fb_ws_bytes(int64_t nx, int64_t nr, int64_t nkr, int64_t nm, int64_t ncomp) {
  i64 rows = nr - 1 > nkr ? nr - 1 : nkr;
  return rnd256(16 * nx) * 2 + rnd256(16 * nx * rows * nm * ncomp) + 256;
}

int chm_fb_in(chm_c128 *vec_fb, const chm_c128 *vec, double leftX, const double *kx,
              const double *In, const double *fact, int64_t nx, int64_t nr, int64_t nkr,
              int64_t nm, int64_t ncomp, void *ws, int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(vec_fb && vec && kx && In && nx > 0 && nr > 1 && nkr > 0 && nm > 0 && ncomp > 0,
              "fb_in: bad args");
  if (ws_bytes < chm_fb_ws_bytes(nx, nr, nkr, nm, ncomp) || !ws) {
    set_error("fb_in: workspace too small");
    return CHM_ERR_WS;
  }
  cudaStream_t st = as_stream(stream);
  WsCursor c{reinterpret_cast<char *>(ws), ws_bytes};
  double2 *tw = c.take<double2>(nx);
  double2 *shift = c.take<double2>(nx);
  const i64 nrr = nr - 1;
  double2 *tmp = c.take<double2>(nx * nrr * nm * ncomp);
  shift_kernel<<<grid_for(nx, 256), 256, 0, st>>>(shift, kx, leftX, -1, nx); chm::count_launch();
  // 1) forward FFT of rows 1..nr-1 of every (mode, component) plane
  FftLines L{};
  L.in = reinterpret_cast<const double2 *>(vec);
  L.out = tmp;
  L.in_rows = (int)nrr;
  L.in_rows_tot = (int)nr;
  L.in_row_off = 1;
  L.out_rows = (int)nrr;
  L.out_rows_tot = (int)nrr;
  L.out_row_off = 0;
  L.nm = (int)nm;
  L.sign = -1;
  L.filt_mode = -1;
  int rc = fft_launch(L, (int)nx, nrr * nm * ncomp, tw, st);
  if (rc) return rc;
  // 2) DHT: out(x, k) = shift(x) fact(x,k,m) sum_r tmp(x, r) In(r, k, m)
  GemmList g;
  g.epi = EPI_SHIFT;
  g.M = (int)(2 * nx);
  g.N = (int)nkr;
  g.K = (int)nrr;
  g.lda = 2 * nx;
  g.ldb = nrr;
  g.ldc = 2 * nx;
  g.shift = shift;
  g.b.count = 0;
  g.st = st;
  for (i64 l = 0; l < ncomp; ++l)
    for (i64 m = 0; m < nm; ++m)
      g.add(reinterpret_cast<const double *>(tmp + nx * nrr * (m + nm * l)), In + nrr * nkr * m,
            reinterpret_cast<double *>(vec_fb) + 2 * nx * nkr * (m + nm * l),
            fact ? fact + nx * nkr * m : nullptr);
  g.flush();
  return g.err;
}

int chm_fb_out(chm_c128 *vec, const chm_c128 *vec_fb, double leftX, const double *kx,
               const double *Out, int64_t nx, int64_t nr, int64_t nkr, int64_t nm, int64_t ncomp,
               int eb_mode, void *ws, int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(vec && vec_fb && kx && Out && nx > 0 && nr > 1 && nkr > 0 && nm > 0 && ncomp > 0,
              "fb_out: bad args");
  if (ws_bytes < chm_fb_ws_bytes(nx, nr, nkr, nm, ncomp) || !ws) {
    set_error("fb_out: workspace too small");
    return CHM_ERR_WS;
  }
  cudaStream_t st = as_stream(stream);
  WsCursor c{reinterpret_cast<char *>(ws), ws_bytes};
  double2 *tw = c.take<double2>(nx);
  double2 *shift = c.take<double2>(nx);
  const i64 nrr = nr - 1;
  double2 *tmp = c.take<double2>(nx * nrr * nm * ncomp);
  shift_kernel<<<grid_for(nx, 256), 256, 0, st>>>(shift, kx, leftX, +1, nx); chm::count_launch();
  // 1) inverse DHT with the shift epilogue: tmp(x, r) = shift(x) sum_k vfb(x,k) Out(k,r)
  GemmList g;
  g.epi = EPI_SHIFT;
  g.M = (int)(2 * nx);
  g.N = (int)nrr;
  g.K = (int)nkr;
  g.lda = 2 * nx;
  g.ldb = nkr;
  g.ldc = 2 * nx;
  g.shift = shift;
  g.b.count = 0;
  g.st = st;
  for (i64 l = 0; l < ncomp; ++l)
    for (i64 m = 0; m < nm; ++m)
      g.add(reinterpret_cast<const double *>(vec_fb) + 2 * nx * nkr * (m + nm * l),
            Out + nkr * nrr * m, reinterpret_cast<double *>(tmp + nx * nrr * (m + nm * l)));
  g.flush();
  if (g.err) return g.err;
  // 2) inverse FFT into rows 1..nr-1; row 0 = 0 or the eb_correction ghost
  if (!eb_mode) {
    // fb_io.f90:117: vec = 0 (row 0 stays zero)
    for (i64 ml = 0; ml < nm * ncomp; ++ml)
      cudaMemsetAsync(reinterpret_cast<double2 *>(vec) + nx * nr * ml, 0, sizeof(double2) * nx, st);
  }
  FftLines L{};
  L.in = tmp;
  L.out = reinterpret_cast<double2 *>(vec);
  L.in_rows = (int)nrr;
  L.in_rows_tot = (int)nrr;
  L.in_row_off = 0;
  L.out_rows = (int)nrr;
  L.out_rows_tot = (int)nr;
  L.out_row_off = 1;
  L.nm = (int)nm;
  L.eb_mode = eb_mode;
  L.sign = +1;
  L.filt_mode = -1;
  return fft_launch(L, (int)nx, nrr * nm * ncomp, tw, st);
}

int chm_fb_eb_out(chm_c128 *eb, const chm_c128 *e_fb, const chm_c128 *b_fb, double leftX,
                  const double *kx, const double *Out, int64_t nx, int64_t nr, int64_t nkr,
                  int64_t nm, int eb_mode, void *ws, int64_t ws_bytes, void *stream) {
  int rc = chm_fb_out(eb, e_fb, leftX, kx, Out, nx, nr, nkr, nm, 3, eb_mode, ws, ws_bytes, stream);
  if (rc) return rc;
  return chm_fb_out(eb + nx * nr * nm * 3, b_fb, leftX, kx, Out, nx, nr, nkr, nm, 3, eb_mode, ws,
                    ws_bytes, stream);
}

int chm_fb_filtr(chm_c128 *vec, double leftX, const double *kx, const double *filtr,
                 int64_t nxfilt, int modefilt, int64_t nx, int64_t nkr, int64_t nm, int64_t ncomp,
                 void *ws, int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(vec && kx && nx > 0 && nkr > 0 && nm > 0 && ncomp > 0, "fb_filtr: bad args");
  CHM_REQUIRE(modefilt >= 0 && modefilt <= 2, "fb_filtr: modefilt must be 0, 1 or 2");
  CHM_REQUIRE(nxfilt >= 0 && nxfilt <= nx && (nxfilt == 0 || filtr), "fb_filtr: bad filter");
  if (ws_bytes < rnd256(16 * nx) * 2 || !ws) {
    set_error("fb_filtr: workspace too small");
    return CHM_ERR_WS;
  }
  cudaStream_t st = as_stream(stream);
  WsCursor c{reinterpret_cast<char *>(ws), ws_bytes};
  double2 *tw = c.take<double2>(nx);
  double2 *shift = c.take<double2>(nx);
  shift_kernel<<<grid_for(nx, 256), 256, 0, st>>>(shift, kx, leftX, +1, nx); chm::count_launch();
  FftLines L{};
  L.in = reinterpret_cast<const double2 *>(vec);
  L.out = reinterpret_cast<double2 *>(vec);
  L.in_rows = L.in_rows_tot = L.out_rows = L.out_rows_tot = (int)nkr;
  L.nm = (int)nm;
  L.sign = +1;
  L.pre_shift = shift;
  L.filt_mode = modefilt;
  L.filtr = filtr;
  L.nxfilt = (int)nxfilt;
  return fft_launch(L, (int)nx, nkr * nm * ncomp, tw, st);
}

}  // extern "C"

// =========================================================================
// fb_math.f90 / fb_math_env.f90
// =========================================================================
namespace {

// Combination kernels.  Products are planes (nx, nkr) of the scratch array
// `P`, indexed P[slot][m] (slot per operator), nullptr = absent (zero).
struct Planes {
  const double2 *p[8];  // per slot base (mode 0); mode stride = nx * nkr
};

__device__ __forceinline__ double2 ld(const double2 *base, i64 off) {
  return base ? base[off] : make_double2(0.0, 0.0);
}

// op codes
enum Op { OP_GRAD = 0, OP_DIV = 1, OP_ROT = 2, OP_ROT_ENV = 3 };

// Generic per-element combine.  has_m/has_p(m) tell whether the lower/upper
// neighbour product exists for mode index m.
struct CombineArgs {
  int op;
  i64 nx, nk;
  int nm;       // output modes
  int env;
  const double2 *in;  // input field (scalar for grad, vector planes for div/rot)
  i64 in_comp_stride; // nx * nk * nm_in
  double2 *out;
  i64 out_comp_stride;
  const double *kx;
  // products: [slot] -> base pointer; element (x, k, m) at base + x + nx*(k + nk*m)
  const double2 *um[3];  // lower-neighbour (Dm) products, components 1..3
  const double2 *up[3];  // upper-neighbour (Dp) products
  const unsigned char *has_m, *has_p;  // per output mode (device) -- unused
  int lo_valid_from;  // modes m >= this have a lower product (0 plain incl. ext, 1 env)
  int hi_valid_to;    // modes m <  this have an upper product
};

__global__ void combine_kernel(CombineArgs A) {
  const i64 plane = A.nx * A.nk;
  const i64 n = plane * A.nm;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < n; t += (i64)gridDim.x * blockDim.x) {
    const i64 x = t % A.nx;
    const int m = (int)(t / plane);
    const double kxv = A.kx[x];
    const bool lo = m >= A.lo_valid_from, hi = m < A.hi_valid_to;
    double2 m1 = lo ? ld(A.um[0], t) : make_double2(0, 0), m2 = lo ? ld(A.um[1], t) : make_double2(0, 0),
            m3 = lo ? ld(A.um[2], t) : make_double2(0, 0);
    double2 p1 = hi ? ld(A.up[0], t) : make_double2(0, 0), p2 = hi ? ld(A.up[1], t) : make_double2(0, 0),
            p3 = hi ? ld(A.up[2], t) : make_double2(0, 0);
    if (A.op == OP_GRAD) {
      // out1 = i kx s; out2 = -Pm + Pp; out3 = i (Pm + Pp)
      double2 s = A.in[t];
      A.out[t] = cscale(cmuli(s), kxv);
      A.out[t + A.out_comp_stride] = csub(p1, m1);
      A.out[t + 2 * A.out_comp_stride] = cmuli(cadd(m1, p1));
    } else if (A.op == OP_DIV) {
      double2 v1 = A.in[t];
      double2 r = cscale(cmuli(v1), kxv);
      if (!A.env) {
        // fb_math.f90:176-194: Dm (i b3 - b2) + Dp (i v3 + v2)
        r = cadd(r, csub(cmuli(m3), m2));
        r = cadd(r, cadd(cmuli(p3), p2));
      } else {
        // fb_math_env.f90:86-99: -Dm (v2 - i v3) + Dp (v2 + i v3)
        r = csub(r, csub(m2, cmuli(m3)));
        r = cadd(r, cadd(p2, cmuli(p3)));
      }
      A.out[t] = r;
    } else {  // OP_ROT / OP_ROT_ENV
      double2 v2 = A.in[t + A.in_comp_stride], v3 = A.in[t + 2 * A.in_comp_stride];
      double2 o1 = make_double2(0, 0);
      double2 o2 = cscale(cmuli(v3), -kxv);
      double2 o3 = cscale(cmuli(v2), kxv);
      // upper: o1 -= (i p2 - p3); o2 += i p1; o3 -= p1
      o1 = csub(o1, csub(cmuli(p2), p3));
      o2 = cadd(o2, cmuli(p1));
      o3 = csub(o3, p1);
      // lower: o1 -= (i m2 + m3) [plain only]; o2 += i m1; o3 += m1
      if (A.op == OP_ROT) o1 = csub(o1, cadd(cmuli(m2), m3));
      o2 = cadd(o2, cmuli(m1));
      o3 = cadd(o3, m1);
      A.out[t] = o1;
      A.out[t + A.out_comp_stride] = o2;
      A.out[t + 2 * A.out_comp_stride] = o3;
    }
  }
}

// Divergence-to-scalar for graddiv: scl on ns modes.  Mode index ms of the
// scalar; the vector has nm modes at input index ms - off (off = 0 plain,
// 1 env).  kx term only where the vector mode exists.
struct DivExtArgs {
  i64 nx, nk;
  int ns, nm, off, env;
  const double2 *in;
  i64 in_comp_stride;
  double2 *out;
  const double *kx;
  const double2 *um[3];
  const double2 *up[3];
  const unsigned char *lo_ok, *hi_ok;  // per scalar mode flags (host-built, in param space)
};

struct ModeFlags {
  unsigned char lo[64], hi[64];
};

__global__ void div_ext_kernel(DivExtArgs A, ModeFlags F) {
  const i64 plane = A.nx * A.nk;
  const i64 n = plane * A.ns;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < n; t += (i64)gridDim.x * blockDim.x) {
    const i64 x = t % A.nx;
    const int ms = (int)(t / plane);
    const i64 e = t - (i64)ms * plane;  // (x, k) offset within a plane
    const int mv = ms - A.off;
    double2 r = make_double2(0.0, 0.0);
    if (mv >= 0 && mv < A.nm) r = cscale(cmuli(A.in[e + plane * mv]), A.kx[x]);
    if (F.lo[ms]) {
      double2 m2 = A.um[1][t], m3 = A.um[2][t];
      if (!A.env) r = cadd(r, csub(cmuli(m3), m2));
      else r = csub(r, csub(m2, cmuli(m3)));
    }
    if (F.hi[ms]) {
      double2 p2 = A.up[1][t], p3 = A.up[2][t];
      if (!A.env) r = cadd(r, cadd(cmuli(p3), p2));
      else r = cadd(r, cadd(p2, cmuli(p3)));
    }
    A.out[t] = r;
  }
}

// Gradient of an extended scalar (ns modes) into nm output modes; the
// output mode m uses scalar modes m+off-1 (Dm) and m+off+1 (Dp).
__global__ void grad_ext_kernel(i64 nx, i64 nk, int nm, int off, const double2 *__restrict__ scl,
                                const double2 *__restrict__ qm, const double2 *__restrict__ qp,
                                double2 *__restrict__ out, i64 out_comp_stride,
                                const double *__restrict__ kx) {
  const i64 plane = nx * nk;
  const i64 n = plane * nm;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < n; t += (i64)gridDim.x * blockDim.x) {
    const i64 x = t % nx;
    const int m = (int)(t / plane);
    const i64 e = t - (i64)m * plane;
    double2 s = scl[e + plane * (m + off)];
    double2 a = qm[t], b = qp[t];
    out[t] = cscale(cmuli(s), kx[x]);
    out[t + out_comp_stride] = csub(b, a);
    out[t + 2 * out_comp_stride] = cmuli(cadd(a, b));
  }
}

}  // namespace

extern "C" {

int64_t chm_fbmath_ws_bytes(int64_t nx, int64_t nkr, int64_t nm) {
  // scalar with nm+2 modes, 6 product planes per mode (nm+2), 3 reflected planes
  i64 plane = 16 * nx * nkr;
  return rnd256(plane * (nm + 2)) + 6 * rnd256(plane * (nm + 2)) + 3 * rnd256(plane) + 4096;
}

}  // extern "C"

namespace {

struct FbmCtx {
  i64 nx, nk, nm;
  const double *Dp, *Dm, *kx;
  int env;
  cudaStream_t st;
  WsCursor c;
  i64 plane() const { return nx * nk; }
};

GemmList make_gemm(const FbmCtx &F) {
  GemmList g;
  g.epi = EPI_STORE;
  g.M = (int)(2 * F.nx);
  g.N = (int)F.nk;
  g.K = (int)F.nk;
  g.lda = 2 * F.nx;
  g.ldb = F.nk;
  g.ldc = 2 * F.nx;
  g.shift = nullptr;
  g.b.count = 0;
  g.st = F.st;
  return g;
}

inline const double *dmat(const double *D, i64 nk, i64 md) { return D + nk * nk * md; }

// Products of `ncomp` vector components (component c at in + c*cs) with the
// lower (Dm) and upper (Dp) neighbours, for output modes 0..nout-1.  Output
// mode m takes input mode m - 1 + shift_in (lower) / m + 1 + shift_in
// (upper) and D mode md = m + dshift.  For the plain solver the lower
// neighbour of m = 0 is the reflected m = 1 plane (refl).
int neighbour_products(FbmCtx &F, const double2 *in, i64 cs, int ncomp, int nin, int nout,
                       int shift_in, int dshift, const double2 *const *refl, double2 *um[3],
                       double2 *up[3], unsigned char lo_ok[64], unsigned char hi_ok[64]) {
  const i64 plane = F.plane();
  GemmList g = make_gemm(F);
  for (int m = 0; m < nout; ++m) {
    const int mlo = m - 1 + shift_in, mhi = m + 1 + shift_in;
    const i64 md = m + dshift;
    lo_ok[m] = 0;
    hi_ok[m] = 0;
    for (int c = 0; c < ncomp; ++c) {
      const double2 *src = nullptr;
      if (mlo >= 0 && mlo < nin) src = in + c * cs + plane * mlo;
      else if (mlo == -1 && refl) src = refl[c];
      if (src) {
        g.add(reinterpret_cast<const double *>(src), dmat(F.Dm, F.nk, md),
              reinterpret_cast<double *>(um[c] + plane * m));
        lo_ok[m] = 1;
      }
      if (mhi >= 0 && mhi < nin) {
        g.add(reinterpret_cast<const double *>(in + c * cs + plane * mhi), dmat(F.Dp, F.nk, md),
              reinterpret_cast<double *>(up[c] + plane * m));
        hi_ok[m] = 1;
      }
    }
  }
  g.flush();
  return g.err;
}

int fbm_check(const char *name, const void *out, const void *in, const double *Dp, const double *Dm,
              const double *kx, i64 nx, i64 nk, i64 nm, int env, void *ws, i64 ws_bytes) {
  if (!(out && in && Dp && Dm && kx && nx > 0 && nk > 0 && nm > 0)) {
    set_error("%s: bad args", name);
    return CHM_ERR_ARG;
  }
  if (env && nm % 2 == 0) {
    set_error("%s: env needs an odd mode count", name);
    return CHM_ERR_ARG;
  }
  if (nm + 2 > 64) {
    set_error("%s: too many modes", name);
    return CHM_ERR_RANGE;
  }
  if (!ws || ws_bytes < chm_fbmath_ws_bytes(nx, nk, nm)) {
    set_error("%s: workspace too small", name);
    return CHM_ERR_WS;
  }
  return CHM_OK;
}

}  // namespace

extern "C" {

int chm_fb_grad(chm_c128 *out, const chm_c128 *scl, const double *Dp, const double *Dm,
                const double *kx, int64_t nx, int64_t nkr, int64_t nm, int env, void *ws,
                int64_t ws_bytes, void *stream) {
  int rc = fbm_check("fb_grad", out, scl, Dp, Dm, kx, nx, nkr, nm, env, ws, ws_bytes);
  if (rc) return rc;
  FbmCtx F{nx, nkr, nm, Dp, Dm, kx, env, as_stream(stream), WsCursor{(char *)ws, ws_bytes}};
  const i64 plane = F.plane();
  const double2 *s = reinterpret_cast<const double2 *>(scl);
  double2 *um[3] = {F.c.take<double2>(plane * nm), nullptr, nullptr};
  double2 *up[3] = {F.c.take<double2>(plane * nm), nullptr, nullptr};
  double2 *ext = F.c.take<double2>(plane);
  const double2 *refl[3] = {ext, nullptr, nullptr};
  if (!env) {
    if (nm > 1) { reflect_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext, s + plane, nx, nkr); chm::count_launch(); }
    else { zero_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext, plane); chm::count_launch(); }
  }
  unsigned char lo[64], hi[64];
  // plain: D mode md = m; env: md = m + 1 (D covers -K-1..K+1)
  rc = neighbour_products(F, s, 0, 1, (int)nm, (int)nm, 0, env ? 1 : 0, env ? nullptr : refl, um, up,
                          lo, hi);
  if (rc) return rc;
  CombineArgs A{};
  A.op = OP_GRAD;
  A.nx = nx;
  A.nk = nkr;
  A.nm = (int)nm;
  A.env = env;
  A.in = s;
  A.out = reinterpret_cast<double2 *>(out);
  A.out_comp_stride = plane * nm;
  A.kx = kx;
  A.um[0] = um[0];
  A.up[0] = up[0];
  A.lo_valid_from = env ? 1 : 0;
  A.hi_valid_to = (int)nm - 1;
  combine_kernel<<<grid_for(plane * nm, 256), 256, 0, F.st>>>(A); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_fb_div(chm_c128 *out, const chm_c128 *vec, const double *Dp, const double *Dm,
               const double *kx, int64_t nx, int64_t nkr, int64_t nm, int env, void *ws,
               int64_t ws_bytes, void *stream) {
  int rc = fbm_check("fb_div", out, vec, Dp, Dm, kx, nx, nkr, nm, env, ws, ws_bytes);
  if (rc) return rc;
  FbmCtx F{nx, nkr, nm, Dp, Dm, kx, env, as_stream(stream), WsCursor{(char *)ws, ws_bytes}};
  const i64 plane = F.plane();
  const double2 *v = reinterpret_cast<const double2 *>(vec);
  const i64 cs = plane * nm;
  double2 *um[3] = {nullptr, F.c.take<double2>(plane * nm), F.c.take<double2>(plane * nm)};
  double2 *up[3] = {nullptr, F.c.take<double2>(plane * nm), F.c.take<double2>(plane * nm)};
  double2 *ext2 = F.c.take<double2>(plane), *ext3 = F.c.take<double2>(plane);
  const double2 *refl[3] = {nullptr, ext2, ext3};
  if (!env) {
    if (nm > 1) {
      reflect_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext2, v + cs + plane, nx, nkr); chm::count_launch();
      reflect_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext3, v + 2 * cs + plane, nx, nkr); chm::count_launch();
    } else {
      zero_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext2, plane); chm::count_launch();
      zero_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext3, plane); chm::count_launch();
    }
  }
  // only components 2, 3 are coupled: shift the base by one component
  double2 *um23[3] = {um[1], um[2], nullptr}, *up23[3] = {up[1], up[2], nullptr};
  const double2 *refl23[3] = {refl[1], refl[2], nullptr};
  unsigned char lo[64], hi[64];
  rc = neighbour_products(F, v + cs, cs, 2, (int)nm, (int)nm, 0, env ? 1 : 0,
                          env ? nullptr : refl23, um23, up23, lo, hi);
  if (rc) return rc;
  CombineArgs A{};
  A.op = OP_DIV;
  A.nx = nx;
  A.nk = nkr;
  A.nm = (int)nm;
  A.env = env;
  A.in = v;
  A.out = reinterpret_cast<double2 *>(out);
  A.kx = kx;
  A.um[1] = um[1];
  A.um[2] = um[2];
  A.up[1] = up[1];
  A.up[2] = up[2];
  A.lo_valid_from = env ? 1 : 0;
  A.hi_valid_to = (int)nm - 1;
  combine_kernel<<<grid_for(plane * nm, 256), 256, 0, F.st>>>(A); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_fb_rot(chm_c128 *out, const chm_c128 *vec, const double *Dp, const double *Dm,
               const double *kx, int64_t nx, int64_t nkr, int64_t nm, int env, void *ws,
               int64_t ws_bytes, void *stream) {
  int rc = fbm_check("fb_rot", out, vec, Dp, Dm, kx, nx, nkr, nm, env, ws, ws_bytes);
  if (rc) return rc;
  FbmCtx F{nx, nkr, nm, Dp, Dm, kx, env, as_stream(stream), WsCursor{(char *)ws, ws_bytes}};
  const i64 plane = F.plane();
  const double2 *v = reinterpret_cast<const double2 *>(vec);
  const i64 cs = plane * nm;
  double2 *um[3], *up[3];
  for (int c = 0; c < 3; ++c) {
    um[c] = F.c.take<double2>(plane * nm);
    up[c] = F.c.take<double2>(plane * nm);
  }
  double2 *ext[3];
  for (int c = 0; c < 3; ++c) ext[c] = F.c.take<double2>(plane);
  const double2 *refl[3] = {ext[0], ext[1], ext[2]};
  if (!env) {
    for (int c = 0; c < 3; ++c) {
      if (nm > 1) { reflect_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext[c], v + c * cs + plane, nx, nkr); chm::count_launch(); }
      else { zero_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext[c], plane); chm::count_launch(); }
    }
  }
  unsigned char lo[64], hi[64];
  double2 *umc[3] = {um[0], um[1], um[2]}, *upc[3] = {up[0], up[1], up[2]};
  if (env) {
    // the env curl drops the lower-neighbour term of component 1
    rc = neighbour_products(F, v, cs, 3, (int)nm, (int)nm, 0, 1, nullptr, umc, upc, lo, hi);
  } else {
    rc = neighbour_products(F, v, cs, 3, (int)nm, (int)nm, 0, 0, refl, umc, upc, lo, hi);
  }
  if (rc) return rc;
  CombineArgs A{};
  A.op = env ? OP_ROT_ENV : OP_ROT;
  A.nx = nx;
  A.nk = nkr;
  A.nm = (int)nm;
  A.env = env;
  A.in = v;
  A.in_comp_stride = cs;
  A.out = reinterpret_cast<double2 *>(out);
  A.out_comp_stride = cs;
  A.kx = kx;
  for (int c = 0; c < 3; ++c) {
    A.um[c] = um[c];
    A.up[c] = up[c];
  }
  A.lo_valid_from = env ? 1 : 0;
  A.hi_valid_to = (int)nm - 1;
  combine_kernel<<<grid_for(plane * nm, 256), 256, 0, F.st>>>(A); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_fb_graddiv(chm_c128 *vec, const double *Dp, const double *Dm, const double *kx,
                   int64_t nx, int64_t nkr, int64_t nm, int env, void *ws, int64_t ws_bytes,
                   void *stream) {
  int rc = fbm_check("fb_graddiv", vec, vec, Dp, Dm, kx, nx, nkr, nm, env, ws, ws_bytes);
  if (rc) return rc;
  FbmCtx F{nx, nkr, nm, Dp, Dm, kx, env, as_stream(stream), WsCursor{(char *)ws, ws_bytes}};
  const i64 plane = F.plane();
  double2 *v = reinterpret_cast<double2 *>(vec);
  const i64 cs = plane * nm;
  const int ns = (int)(env ? nm + 2 : nm + 1);  // scalar modes
  const int off = env ? 1 : 0;                   // scalar index of vector mode 0
  double2 *scl = F.c.take<double2>(plane * (nm + 2));
  double2 *um[3], *up[3];
  for (int c = 0; c < 3; ++c) {
    um[c] = F.c.take<double2>(plane * (nm + 2));
    up[c] = F.c.take<double2>(plane * (nm + 2));
  }
  double2 *ext[3];
  for (int c = 0; c < 3; ++c) ext[c] = F.c.take<double2>(plane);
  // --- divergence on ns modes (fb_math.f90:222-252 / fb_math_env.f90:180-206)
  if (!env) {
    if (nm > 1) {
      reflect_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext[1], v + cs + plane, nx, nkr); chm::count_launch();
      reflect_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext[2], v + 2 * cs + plane, nx, nkr); chm::count_launch();
    } else {
      zero_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext[1], plane); chm::count_launch();
      zero_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext[2], plane); chm::count_launch();
    }
  }
  ModeFlags fl{};
  {
    const double2 *refl23[3] = {ext[1], ext[2], nullptr};
    double2 *um23[3] = {um[1], um[2], nullptr}, *up23[3] = {up[1], up[2], nullptr};
    // scalar mode ms has vector neighbours ms-1-off (Dm) and ms+1-off (Dp);
    // D mode = ms (plain: D has nm+1 modes; env: nm+2)
    rc = neighbour_products(F, v + cs, cs, 2, (int)nm, ns, -off, 0, env ? nullptr : refl23, um23,
                            up23, fl.lo, fl.hi);
    if (rc) return rc;
    if (env) {
      // fb_math_env.f90:190-201: lower term only for m > -K, upper for m < K
      for (int ms = 0; ms < ns; ++ms) {
        const int m = ms - 1 - (int)(nm - 1) / 2;
        const int K = (int)(nm - 1) / 2;
        if (!(m > -K)) fl.lo[ms] = 0;
        if (!(m < K)) fl.hi[ms] = 0;
      }
    } else {
      // fb_math.f90:231-247: upper term only for ms < nm-1 ("iO < nkO")
      for (int ms = 0; ms < ns; ++ms)
        if (!(ms < (int)nm - 1)) fl.hi[ms] = 0;
    }
    DivExtArgs D{};
    D.nx = nx;
    D.nk = nkr;
    D.ns = ns;
    D.nm = (int)nm;
    D.off = off;
    D.env = env;
    D.in = v;
    D.in_comp_stride = cs;
    D.out = scl;
    D.kx = kx;
    for (int c = 0; c < 3; ++c) {
      D.um[c] = um[c];
      D.up[c] = up[c];
    }
    div_ext_kernel<<<grid_for(plane * ns, 256), 256, 0, F.st>>>(D, fl); chm::count_launch();
    CHM_CHECK_LAUNCH();
  }
  // --- gradient of the extended scalar back onto nm modes (in place)
  {
    if (!env) {
      if (nm > 1) { reflect_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext[0], scl + plane, nx, nkr); chm::count_launch(); }
      else { zero_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(ext[0], plane); chm::count_launch(); }
    }
    GemmList g = make_gemm(F);
    for (int m = 0; m < nm; ++m) {
      const int ms = m + off;
      const i64 md = m + off;  // D mode
      const double2 *lo = (ms - 1 >= 0) ? scl + plane * (ms - 1) : ext[0];
      g.add(reinterpret_cast<const double *>(lo), dmat(Dm, nkr, md),
            reinterpret_cast<double *>(um[0] + plane * m));
      g.add(reinterpret_cast<const double *>(scl + plane * (ms + 1)), dmat(Dp, nkr, md),
            reinterpret_cast<double *>(up[0] + plane * m));
    }
    g.flush();
    if (g.err) return g.err;
    grad_ext_kernel<<<grid_for(plane * nm, 256), 256, 0, F.st>>>(nx, nkr, (int)nm, off, scl, um[0],
                                                                 up[0], v, cs, kx); chm::count_launch();
    CHM_CHECK_LAUNCH();
  }
  return CHM_OK;
}

}  // extern "C"

// =========================================================================
// maxwell_solvers.f90 elementwise kernels
// =========================================================================
namespace {

__global__ void psatd_spchrg_kernel(double2 *__restrict__ eg, const double2 *__restrict__ j,
                                    const double2 *__restrict__ gn, const double2 *__restrict__ gnp1,
                                    const double *__restrict__ c1, const double *__restrict__ c2,
                                    i64 P) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P; i += (i64)gridDim.x * blockDim.x) {
    const double a0 = c1[i], a1 = c1[i + P], a2 = c1[i + 2 * P], a3 = c1[i + 3 * P], a4 = c1[i + 4 * P];
    const double b0 = c2[i], b1 = c2[i + P], b2 = c2[i + 2 * P], b3 = c2[i + 3 * P], b4 = c2[i + 4 * P];
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      double2 e = eg[i + P * l], g = eg[i + P * (3 + l)], jj = j[i + P * l], ra = gn[i + P * l],
              rb = gnp1[i + P * l];
      double2 en, gw;
      en.x = a0 * e.x + a1 * g.x + a2 * jj.x + a3 * ra.x + a4 * rb.x;
      en.y = a0 * e.y + a1 * g.y + a2 * jj.y + a3 * ra.y + a4 * rb.y;
      gw.x = b0 * e.x + b1 * g.x + b2 * jj.x + b3 * ra.x + b4 * rb.x;
      gw.y = b0 * e.y + b1 * g.y + b2 * jj.y + b3 * ra.y + b4 * rb.y;
      eg[i + P * (3 + l)] = gw;
      eg[i + P * l] = en;
    }
  }
}

__global__ void psatd_wo_kernel(double2 *__restrict__ eg, const double2 *__restrict__ j,
                                const double2 *__restrict__ c1, const double2 *__restrict__ c2, i64 P) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P; i += (i64)gridDim.x * blockDim.x) {
    const double2 a0 = c1[i], a1 = c1[i + P], a2 = c1[i + 2 * P];
    const double2 b0 = c2[i], b1 = c2[i + P], b2 = c2[i + 2 * P];
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      double2 e = eg[i + P * l], g = eg[i + P * (3 + l)], jj = j[i + P * l];
      double2 en = cadd(cadd(cmul(a0, e), cmul(a1, g)), cmul(a2, jj));
      double2 gw = cadd(cadd(cmul(b0, e), cmul(b1, g)), cmul(b2, jj));
      eg[i + P * (3 + l)] = gw;
      eg[i + P * l] = en;
    }
  }
}

__global__ void init_push_kernel(double2 *__restrict__ eg, const double2 *__restrict__ j,
                                 const double2 *__restrict__ gn, const double2 *__restrict__ c1,
                                 const double2 *__restrict__ c2, i64 P) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P; i += (i64)gridDim.x * blockDim.x) {
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      double2 jj = j[i + P * l], g = gn[i + P * l];
      eg[i + P * l] = cadd(cadd(eg[i + P * l], cmul(c1[i], jj)), cmul(c1[i + P], g));
      eg[i + P * (3 + l)] = cadd(cadd(eg[i + P * (3 + l)], cmul(c2[i], jj)), cmul(c2[i + P], g));
    }
  }
}

__global__ void poiss_corr_kernel(double2 *__restrict__ j, const double2 *__restrict__ gdj,
                                  const double2 *__restrict__ gn, const double2 *__restrict__ gnp1,
                                  double dt_inv, const double *__restrict__ w2, i64 P) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P; i += (i64)gridDim.x * blockDim.x) {
    const double f = w2[i];
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      double2 a = gdj[i + P * l];
      double2 d = csub(gnp1[i + P * l], gn[i + P * l]);
      double2 t = make_double2(a.x + d.x * dt_inv, a.y + d.y * dt_inv);
      j[i + P * l] = cadd(j[i + P * l], cscale(t, f));
    }
  }
}

__global__ void poiss_corr_stat_kernel(double2 *__restrict__ j, const double2 *__restrict__ gdj,
                                       const double2 *__restrict__ gn, const double2 *__restrict__ DT,
                                       const double *__restrict__ w2, i64 P, i64 nx) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P; i += (i64)gridDim.x * blockDim.x) {
    const double f = w2[i];
    const double2 dt = DT[i % nx];
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      double2 t = cadd(gdj[i + P * l], cmul(dt, gn[i + P * l]));
      j[i + P * l] = cadd(j[i + P * l], cscale(t, f));
    }
  }
}

__global__ void field_drift_kernel(double2 *__restrict__ eg, const double *__restrict__ kx, double beta0,
                                   double dt, i64 P, i64 nx) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < 6 * P; i += (i64)gridDim.x * blockDim.x) {
    // exp(fact kx) with fact = -0.5 i dt beta0: purely imaginary argument
    double s, c;
    sincos(-0.5 * dt * beta0 * kx[i % nx], &s, &c);
    eg[i] = cmul(eg[i], make_double2(c, s));
  }
}

__global__ void mult_kernel(double2 *__restrict__ v, const double *__restrict__ A, i64 P, i64 ncomp) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P; i += (i64)gridDim.x * blockDim.x) {
    const double a = A[i];
    for (i64 l = 0; l < ncomp; ++l) v[i + P * l] = cscale(v[i + P * l], a);
  }
}

__global__ void add_kernel(double2 *__restrict__ v, const double2 *__restrict__ A, i64 n) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    v[i] = cadd(v[i], A[i]);
}

}  // namespace

extern "C" {

int chm_maxwell_push_with_spchrg(chm_c128 *eg, const chm_c128 *j, const chm_c128 *gn,
                                 const chm_c128 *gnp1, const double *c1, const double *c2,
                                 int64_t nx, int64_t nkr, int64_t nm, void *stream) {
  CHM_REQUIRE(eg && j && gn && gnp1 && c1 && c2, "maxwell_push_with_spchrg: null pointer");
  const i64 P = nx * nkr * nm;
  psatd_spchrg_kernel<<<grid_for(P, 256), 256, 0, as_stream(stream)>>>(
      (double2 *)eg, (const double2 *)j, (const double2 *)gn, (const double2 *)gnp1, c1, c2, P); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_maxwell_push_wo_spchrg(chm_c128 *eg, const chm_c128 *j, const chm_c128 *c1,
                               const chm_c128 *c2, int64_t nx, int64_t nkr, int64_t nm,
                               void *stream) {
  CHM_REQUIRE(eg && j && c1 && c2, "maxwell_push_wo_spchrg: null pointer");
  const i64 P = nx * nkr * nm;
  psatd_wo_kernel<<<grid_for(P, 256), 256, 0, as_stream(stream)>>>(
      (double2 *)eg, (const double2 *)j, (const double2 *)c1, (const double2 *)c2, P); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_maxwell_init_push(chm_c128 *eg, const chm_c128 *j, const chm_c128 *gn, const chm_c128 *c1,
                          const chm_c128 *c2, int64_t nx, int64_t nkr, int64_t nm, void *stream) {
  CHM_REQUIRE(eg && j && gn && c1 && c2, "maxwell_init_push: null pointer");
  const i64 P = nx * nkr * nm;
  init_push_kernel<<<grid_for(P, 256), 256, 0, as_stream(stream)>>>(
      (double2 *)eg, (const double2 *)j, (const double2 *)gn, (const double2 *)c1,
      (const double2 *)c2, P); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_poiss_corr(chm_c128 *j, const chm_c128 *gdj, const chm_c128 *gn, const chm_c128 *gnp1,
                   double dt_inv, const double *w2_inv, int64_t nx, int64_t nkr, int64_t nm,
                   void *stream) {
  CHM_REQUIRE(j && gdj && gn && gnp1 && w2_inv, "poiss_corr: null pointer");
  const i64 P = nx * nkr * nm;
  poiss_corr_kernel<<<grid_for(P, 256), 256, 0, as_stream(stream)>>>(
      (double2 *)j, (const double2 *)gdj, (const double2 *)gn, (const double2 *)gnp1, dt_inv,
      w2_inv, P); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_poiss_corr_stat(chm_c128 *j, const chm_c128 *gdj, const chm_c128 *gn, const chm_c128 *DT,
                        const double *w2_inv, int64_t nx, int64_t nkr, int64_t nm, void *stream) {
  CHM_REQUIRE(j && gdj && gn && DT && w2_inv, "poiss_corr_stat: null pointer");
  const i64 P = nx * nkr * nm;
  poiss_corr_stat_kernel<<<grid_for(P, 256), 256, 0, as_stream(stream)>>>(
      (double2 *)j, (const double2 *)gdj, (const double2 *)gn, (const double2 *)DT, w2_inv, P, nx); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_field_drift(chm_c128 *eg, const double *kx, double beta0, double dt, int64_t nx,
                    int64_t nkr, int64_t nm, void *stream) {
  CHM_REQUIRE(eg && kx, "field_drift: null pointer");
  const i64 P = nx * nkr * nm;
  field_drift_kernel<<<grid_for(6 * P, 256), 256, 0, as_stream(stream)>>>((double2 *)eg, kx, beta0,
                                                                           dt, P, nx); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_omp_mult(chm_c128 *v, const double *A, int64_t P, int64_t ncomp, void *stream) {
  CHM_REQUIRE(v && A && P >= 0 && ncomp > 0, "omp_mult: bad args");
  if (P == 0) return CHM_OK;
  mult_kernel<<<grid_for(P, 256), 256, 0, as_stream(stream)>>>((double2 *)v, A, P, ncomp); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_omp_add(chm_c128 *v, const chm_c128 *A, int64_t n, void *stream) {
  CHM_REQUIRE(v && A && n >= 0, "omp_add: bad args");
  if (n == 0) return CHM_OK;
  add_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>((double2 *)v, (const double2 *)A, n); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"
