// Spectral stage of the split-precision form: complex64 fields, FP32 FFT
// along x, dense DHT / mode-coupling products on the tensor cores (see
// tc_gemm.cu) and fused FP32 epilogues.
//
// Differences from the FP64 path that keep memory traffic down:
//  - the forward transforms read the 64-bit deposit accumulators directly
//    (scale, ghost-row fold and the background density are applied on load);
//  - the gradient of the Poisson correction updates J in place
//    (maxwell_solvers.f90:131-164 fused into fb_graddiv's epilogue);
//  - the curl that turns G into B applies PoissFact in its epilogue;
//  - eb_correction is applied by the inverse FFT (as in the FP64 path).
#include <math.h>

#include "common.cuh"
#include "tc_gemm.cuh"

using namespace chm;

namespace {

constexpr int kMaxN = 4096;
constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ float2 fadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 fsub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 fmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 fscl(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 fmi(float2 a) { return make_float2(-a.y, a.x); }  // i a

struct Plan {
  int n, ns;
  int radix[24];
  int log2n;  // >= 0 when n is a power of two (radix-4/2 passes, shift index math)
};

bool make_plan(int n, Plan *p) {
  if (n < 1 || n > kMaxN) return false;
  p->n = n;
  p->ns = 0;
  p->log2n = -1;
  if ((n & (n - 1)) == 0 && n >= 4) {
    int l = 0;
    while ((1 << l) < n) ++l;
    p->log2n = l;
  }
  int m = n;
  while (m % 4 == 0) {
    p->radix[p->ns++] = 4;
    m /= 4;
  }
  const int small[4] = {2, 3, 5, 7};
  for (int s = 0; s < 4; ++s)
    while (m % small[s] == 0 && p->ns < 24) {
      p->radix[p->ns++] = small[s];
      m /= small[s];
    }
  for (int f = 11; m > 1 && p->ns < 24;) {
    if ((i64)f * f > m) f = m;
    if (m % f == 0) {
      p->radix[p->ns++] = f;
      m /= f;
    } else {
      f += 2;
    }
  }
  return m == 1;
}

// exp(-2 pi i t / n) in FP32 from an FP64 evaluation
__global__ void twiddle32_kernel(float2 *tw, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)t / (double)n, &s, &c);
    tw[t] = make_float2((float)c, (float)-s);
  }
}

// exp(sign i kx leftX) evaluated in FP64 (the argument can be large), stored
// FP32; with tw, also the FFT twiddles exp(-2 pi i t / nx) (as twiddle32_kernel).
// Launched with warp-sized blocks: the FP64 trigonometry spreads over as
// many SMs as there are warps of work.
// (win: the device window origin, when given, instead of leftX)
__global__ void shift32_kernel(float2 *shift, const double *kx, double leftX, int sign, i64 nx,
                               float2 *tw, const chm_sp_window *win = nullptr) {
  if (win) leftX = win->leftX;
  for (i64 x = blockIdx.x * (i64)blockDim.x + threadIdx.x; x < nx; x += (i64)gridDim.x * blockDim.x) {
    double s, c;
    sincos(leftX * kx[x], &s, &c);
    shift[x] = make_float2((float)c, (float)(sign * s));
    if (tw) {
      sincospi(2.0 * (double)x / (double)nx, &s, &c);
      tw[x] = make_float2((float)c, (float)-s);
    }
  }
}

// the window record: k = floor((leftX - X0) / dx), f = the rest (FP64)
__global__ void window_kernel(chm_sp_window *w, int set, double leftX, double X0, double dx,
                              double shift) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (set) {
    w->leftX = leftX;
    w->X0 = X0;
    w->dx = dx;
    const double sv = (leftX - X0) / dx;
    const double k = floor(sv);
    w->k = (int32_t)k;
    w->fd = sv - k;
  } else {
    // the cell position advances by shift / dx from the previous one (a
    // whole-cell move leaves the fraction exactly as it was)
    w->leftX = w->leftX + shift;
    const double s = w->fd + shift / w->dx;
    const double fl = floor(s);
    w->k = w->k + (int32_t)fl;
    w->fd = s - fl;
  }
  w->f = (float)w->fd;
}

__device__ __forceinline__ float2 tw32(const float2 *tw, int t, int sign) {
  float2 w = tw[t];
  if (sign > 0) w.y = -w.y;
  return w;
}

__device__ void pass32(const float2 *__restrict__ src, float2 *__restrict__ dst, int n, int R, int Ns,
                       const float2 *__restrict__ tw, int sign) {
  const int nb = n / R;
  for (int j = threadIdx.x; j < nb; j += blockDim.x) {
    const int k = j % Ns;
    const int tstep = (n / (Ns * R)) * k;
    const int base = (j / Ns) * Ns * R + k;
    if (R == 4) {
      float2 v[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        float2 a = src[j + r * nb];
        if (r > 0 && k > 0) a = fmul(a, tw32(tw, (r * tstep) % n, sign));
        v[r] = a;
      }
      float2 a0 = fadd(v[0], v[2]), a1 = fsub(v[0], v[2]);
      float2 a2 = fadd(v[1], v[3]), a3 = fsub(v[1], v[3]);
      float2 a3r = sign < 0 ? make_float2(a3.y, -a3.x) : make_float2(-a3.y, a3.x);
      dst[base] = fadd(a0, a2);
      dst[base + Ns] = fadd(a1, a3r);
      dst[base + 2 * Ns] = fsub(a0, a2);
      dst[base + 3 * Ns] = fsub(a1, a3r);
    } else if (R == 2) {
      float2 a = src[j], b = src[j + nb];
      if (k > 0) b = fmul(b, tw32(tw, tstep % n, sign));
      dst[base] = fadd(a, b);
      dst[base + Ns] = fsub(a, b);
    } else {
      const int step = n / R;
      for (int q = 0; q < R; ++q) {
        float2 acc = make_float2(0.f, 0.f);
        for (int r = 0; r < R; ++r) {
          float2 a = src[j + r * nb];
          if (r > 0 && k > 0) a = fmul(a, tw32(tw, (r * tstep) % n, sign));
          acc = fadd(acc, fmul(a, tw32(tw, ((r * q) % R) * step, sign)));
        }
        dst[base + q * Ns] = acc;
      }
    }
  }
}

__device__ float2 *run32(const Plan &P, float2 *a, float2 *b, const float2 *tw, int sign) {
  int Ns = 1;
  for (int s = 0; s < P.ns; ++s) {
    __syncthreads();
    pass32(a, b, P.n, P.radix[s], Ns, tw, sign);
    Ns *= P.radix[s];
    float2 *t = a;
    a = b;
    b = t;
  }
  __syncthreads();
  return a;
}

// Power-of-two Stockham passes: the index arithmetic of pass32 with shifts
// and the twiddles read from a shared-memory table.
__device__ void pass4p(const float2 *__restrict__ src, float2 *__restrict__ dst, int n, int l2n,
                       int lNs, const float2 *__restrict__ tw, int sign) {
  const int nb = n >> 2, Ns = 1 << lNs;
  for (int j = threadIdx.x; j < nb; j += blockDim.x) {
    const int k = j & (Ns - 1);
    const int tstep = k << (l2n - lNs - 2);
    const int base = ((j >> lNs) << (lNs + 2)) + k;
    float2 v[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      float2 a = src[j + r * nb];
      if (r > 0) a = fmul(a, tw32(tw, r * tstep, sign));
      v[r] = a;
    }
    float2 a0 = fadd(v[0], v[2]), a1 = fsub(v[0], v[2]);
    float2 a2 = fadd(v[1], v[3]), a3 = fsub(v[1], v[3]);
    float2 a3r = sign < 0 ? make_float2(a3.y, -a3.x) : make_float2(-a3.y, a3.x);
    dst[base] = fadd(a0, a2);
    dst[base + Ns] = fadd(a1, a3r);
    dst[base + 2 * Ns] = fsub(a0, a2);
    dst[base + 3 * Ns] = fsub(a1, a3r);
  }
}

__device__ void pass2p(const float2 *__restrict__ src, float2 *__restrict__ dst, int n, int l2n,
                       int lNs, const float2 *__restrict__ tw, int sign) {
  const int nb = n >> 1, Ns = 1 << lNs;
  for (int j = threadIdx.x; j < nb; j += blockDim.x) {
    const int k = j & (Ns - 1);
    const int tstep = k << (l2n - lNs - 1);
    const int base = ((j >> lNs) << (lNs + 1)) + k;
    const float2 a = src[j], b = fmul(src[j + nb], tw32(tw, tstep, sign));
    dst[base] = fadd(a, b);
    dst[base + Ns] = fsub(a, b);
  }
}

__device__ float2 *run32p(const Plan &P, float2 *a, float2 *b, const float2 *tw, int sign) {
  int lNs = 0;
  for (; lNs + 2 <= P.log2n; lNs += 2) {
    __syncthreads();
    pass4p(a, b, P.n, P.log2n, lNs, tw, sign);
    float2 *t = a;
    a = b;
    b = t;
  }
  if (lNs < P.log2n) {
    __syncthreads();
    pass2p(a, b, P.n, P.log2n, lNs, tw, sign);
    float2 *t = a;
    a = b;
    b = t;
  }
  __syncthreads();
  return a;
}

// ---------------------------------------------------------------------------
// Register passes for power-of-two n >= 512: each thread keeps 16 points in
// registers and does a 16-point DFT (4 x 4) per pass, so a 2048-point line
// takes three passes (16, 16, 8) through one shared-memory buffer instead of
// six radix-4 passes through two.  Stockham indexing as pass32; the twiddles
// come from a global table (L1/L2) of n entries exp(-2 pi i t / n).
// ---------------------------------------------------------------------------
// x * (sign i): -i x for sign < 0, +i x for sign > 0
__device__ __forceinline__ float2 mul_si(float2 x, int sign) {
  return sign < 0 ? make_float2(x.y, -x.x) : make_float2(-x.y, x.x);
}

__device__ __forceinline__ void dft2r(float2 &x0, float2 &x1) {
  const float2 a = x0;
  x0 = fadd(a, x1);
  x1 = fsub(a, x1);
}

// 4-point DFT in place, natural order (exponent sign `sign`)
__device__ __forceinline__ void dft4r(float2 &x0, float2 &x1, float2 &x2, float2 &x3, int sign) {
  const float2 a0 = fadd(x0, x2), a1 = fsub(x0, x2), a2 = fadd(x1, x3);
  const float2 a3 = mul_si(fsub(x1, x3), sign);
  x0 = fadd(a0, a2);
  x2 = fsub(a0, a2);
  x1 = fadd(a1, a3);
  x3 = fsub(a1, a3);
}

// e^{sign 2 pi i m / 16} for m = 0..9 (the exact values of the angles)
__device__ __forceinline__ float2 w16(int m, int sign) {
  const float c1 = 0.92387953251128674f, s1 = 0.38268343236508977f, h = 0.70710678118654752f;
  float2 w;
  switch (m) {
    case 1: w = make_float2(c1, s1); break;
    case 2: w = make_float2(h, h); break;
    case 3: w = make_float2(s1, c1); break;
    case 4: w = make_float2(0.f, 1.f); break;
    case 6: w = make_float2(-h, h); break;
    case 9: w = make_float2(-c1, -s1); break;
    default: w = make_float2(1.f, 0.f); break;
  }
  if (sign < 0) w.y = -w.y;
  return w;
}

// 16-point DFT: v in natural order; result X[k1 + 4 k2] left in v[4 k1 + k2]
__device__ __forceinline__ void dft16r(float2 (&v)[16], int sign) {
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4r(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12], sign);
#pragma unroll
  for (int k1 = 1; k1 < 4; ++k1)
#pragma unroll
    for (int n2 = 1; n2 < 4; ++n2) v[n2 + 4 * k1] = fmul(v[n2 + 4 * k1], w16(n2 * k1, sign));
  // A(k1, n2) sits at v[4 k1 + n2]: second stage over n2 for each k1
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4r(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3], sign);
}

// 8-point DFT: result X[k1 + 4 k2] left in v[2 k1 + k2]
__device__ __forceinline__ void dft8r(float2 (&v)[8], int sign) {
#pragma unroll
  for (int n2 = 0; n2 < 2; ++n2) dft4r(v[n2], v[n2 + 2], v[n2 + 4], v[n2 + 6], sign);
  // A(k1, 1) at v[1 + 2 k1] times e^{sign 2 pi i k1 / 8}
  v[3] = fmul(v[3], w16(2, sign));
  v[5] = mul_si(v[5], sign);
  v[7] = fmul(v[7], w16(6, sign));
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft2r(v[2 * k1], v[2 * k1 + 1]);
}

__device__ __forceinline__ float2 tw_at(const float2 *__restrict__ tw, int t, int sign) {
  float2 w = __ldg(tw + t);
  if (sign > 0) w.y = -w.y;
  return w;
}

// One in-place Stockham pass of radix R over the line in a[0..n), T threads
// (t = this thread), butterflies j = t, t + T, ... < n / R.
template <int R, typename Src, typename Sink>
__device__ void pass_reg(float2 *a, int n, int l2n, int lNs, const float2 *__restrict__ tw, int sign,
                         int t, int T, Src src, Sink sink) {
  constexpr int lR = R == 16 ? 4 : R == 8 ? 3 : R == 4 ? 2 : 1;
  constexpr int B = 16 / R;  // butterflies per thread (T = n / 16)
  const int nb = n >> lR, Ns = 1 << lNs;
  const int tsh = l2n - lNs - lR;  // twiddle index stride log2
  float2 v[B][R];
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int j = t + b * T;
    const int k = j & (Ns - 1);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      float2 x = src(j + r * nb);
      if (r > 0 && k > 0) x = fmul(x, tw_at(tw, (r * k) << tsh, sign));
      v[b][r] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int j = t + b * T;
    const int k = j & (Ns - 1);
    const int base = ((j >> lNs) << (lNs + lR)) + k;
    if constexpr (R == 16) {
      dft16r(v[b], sign);
#pragma unroll
      for (int q = 0; q < 16; ++q) sink(base + q * Ns, v[b][4 * (q & 3) + (q >> 2)]);
    } else if constexpr (R == 8) {
      dft8r(v[b], sign);
#pragma unroll
      for (int q = 0; q < 8; ++q) sink(base + q * Ns, v[b][2 * (q & 3) + (q >> 2)]);
    } else if constexpr (R == 4) {
      dft4r(v[b][0], v[b][1], v[b][2], v[b][3], sign);
#pragma unroll
      for (int q = 0; q < 4; ++q) sink(base + q * Ns, v[b][q]);
    } else {
      dft2r(v[b][0], v[b][1]);
      sink(base, v[b][0]);
      sink(base + Ns, v[b][1]);
    }
  }
  __syncthreads();
}

// The whole transform (n = 2^l2n >= 512, blockDim = n / 16) through the
// buffer a.  The first pass reads its 16 points per thread from `first`
// (the line's source, or the buffer), the last one writes through `last`;
// the passes between use the buffer.  A thread's points in the first pass
// are x = t + m T, m = 0..15, the ones its load loop would take.  (Writing
// the last pass straight to the line's sink measured slower than through
// the buffer and a coalesced store loop.)
template <typename First, typename Last>
__device__ void run16(float2 *a, int n, int l2n, const float2 *__restrict__ tw, int sign,
                      First first, Last last) {
  const int t = threadIdx.x, T = blockDim.x;
  auto src = [a](int i) { return a[i]; };
  auto dst = [a](int i, float2 v) { a[i] = v; };
  const int n16 = l2n >> 2, rem = l2n & 3;  // radix-16 passes, remainder
  __syncthreads();
  if (n16 == 1 && rem == 0) pass_reg<16>(a, n, l2n, 0, tw, sign, t, T, first, last);
  else pass_reg<16>(a, n, l2n, 0, tw, sign, t, T, first, dst);
  for (int p = 1; p < n16; ++p) {
    if (p == n16 - 1 && rem == 0) pass_reg<16>(a, n, l2n, 4 * p, tw, sign, t, T, src, last);
    else pass_reg<16>(a, n, l2n, 4 * p, tw, sign, t, T, src, dst);
  }
  const int lNs = 4 * n16;
  if (rem == 3) pass_reg<8>(a, n, l2n, lNs, tw, sign, t, T, src, last);
  else if (rem == 2) pass_reg<4>(a, n, l2n, lNs, tw, sign, t, T, src, last);
  else if (rem == 1) pass_reg<2>(a, n, l2n, lNs, tw, sign, t, T, src, last);
}

// 64-bit fixed-point value -> FP32 (two 32-bit conversions, no 64-bit unit)
__device__ __forceinline__ float fix2f(long long v) {
  const int hi = (int)(v >> 32);
  const unsigned lo = (unsigned)(v & 0xffffffffULL);
  return fmaf((float)hi, 4294967296.0f, (float)lo);
}

// Line sources/sinks of the FP32 FFT.
struct Lines32 {
  // input: either complex64 rows or a 64-bit deposit accumulator
  const float2 *in;
  const long long *acc;   // (n, rows_tot, planes) x {re, im}, or null
  const double *acc_scale;
  const long long *acc2;  // optional second accumulator (background density)
  const double *acc2_scale;
  int in_rows, in_rows_tot, in_row_off;
  float2 *out;
  int out_rows, out_rows_tot, out_row_off;
  int nm, eb_mode, sign;
  const float2 *pre_shift;  // multiply inputs (filter path)
  int filt_mode, nxfilt;
  const float *filtr;
};

// MODE 0: any n (run32, mixed radix); 1: power of two, radix-4 passes with a
// per-block twiddle table; 2: power of two >= 512, register radix-16 passes
// in place (one buffer, blockDim = n / 16, twiddles from the global table)
template <int MODE>
__global__ void __launch_bounds__(MODE == 2 ? 256 : 512, MODE == 2 ? 4 : 1)
    lines32_kernel(Plan P, const float2 *__restrict__ tw, Lines32 L) {
  extern __shared__ __align__(16) float2 sm32[];
  constexpr bool POW2 = MODE == 1;
  const int n = P.n;
  float2 *a = sm32, *b = sm32 + n;
  if (POW2) {
    // exp(-2 pi i t / n) for the power-of-two passes
    float2 *tws = sm32 + 2 * n;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      float sv, cv;
      sincospif(2.0f * (float)t / (float)n, &sv, &cv);
      tws[t] = make_float2(cv, -sv);
    }
    tw = tws;  // the first pass synchronises before reading it
  }
  const i64 line = blockIdx.x;
  const i64 ib = line / L.in_rows, ir = line % L.in_rows;
  const i64 row = ib * L.in_rows_tot + ir + L.in_row_off;
  // the line's input value at x
  float inv = 0.0f, inv2 = 0.0f;
  bool fold = false;
  i64 row0 = 0;
  if (L.acc) {
    // deposit accumulator: value / scale with the ghost fold row1 -= row0
    // (the scales are powers of two, so the FP32 inverses are exact)
    inv = 1.0f / (float)L.acc_scale[0];
    inv2 = L.acc2 ? 1.0f / (float)L.acc2_scale[0] : 0.0f;
    fold = (ir + L.in_row_off) == 1;
    row0 = ib * L.in_rows_tot;
  }
  auto load_elem = [&](int x) -> float2 {
    if (L.acc) {
      const longlong2 *A1 = reinterpret_cast<const longlong2 *>(L.acc);
      const longlong2 *A2 = reinterpret_cast<const longlong2 *>(L.acc2);
      const i64 e = row * n + x;
      const longlong2 q = A1[e];
      float re = fix2f(q.x) * inv, im = fix2f(q.y) * inv;
      if (A2) {
        const longlong2 q2 = A2[e];
        re += fix2f(q2.x) * inv2;
        im += fix2f(q2.y) * inv2;
      }
      if (fold) {
        const i64 e0 = row0 * n + x;
        const longlong2 q0 = A1[e0];
        re -= fix2f(q0.x) * inv;
        im -= fix2f(q0.y) * inv;
        if (A2) {
          const longlong2 q2 = A2[e0];
          re -= fix2f(q2.x) * inv2;
          im -= fix2f(q2.y) * inv2;
        }
      }
      return make_float2(re, im);
    }
    float2 v = L.in[row * (i64)n + x];
    if (L.pre_shift) v = fmul(v, L.pre_shift[x]);
    return v;
  };
  if constexpr (MODE != 2)
    for (int x = threadIdx.x; x < n; x += blockDim.x) a[x] = load_elem(x);
  // the line's output at x (the inverse shift of the filter path, the
  // eb_correction scale and ghost row)
  const i64 ob = line / L.out_rows, orow = line % L.out_rows;
  float2 *dstl = L.out + (ob * L.out_rows_tot + orow + L.out_row_off) * (i64)n;
  float fac = 1.0f, sg = 1.0f;
  if (L.eb_mode == 1) {
    const int m = (int)(ob % L.nm);
    fac = (float)((m == 0) ? 0.5 / kPi : 1.0 / kPi);
    sg = (m == 0) ? 1.0f : -1.0f;
  } else if (L.eb_mode == 2) {
    // envelope modes (grid_deps_env.f90:240-283): 1 / pi for every mode,
    // the ghost row mirrored with sign -1 unless a single mode is stored
    fac = (float)(1.0 / kPi);
    sg = L.nm == 1 ? 1.0f : -1.0f;
  }
  const bool ghost = L.eb_mode && orow == 0;
  float2 *gdst = L.out + (ob * L.out_rows_tot) * (i64)n;
  auto store_elem = [&](int x, float2 v) {
    if (L.filt_mode >= 0) {
      float2 s = L.pre_shift[x];
      float inv = 1.0f / ((float)n * (s.x * s.x + s.y * s.y));
      v = fmul(v, make_float2(s.x * inv, -s.y * inv));
    }
    if (L.eb_mode) v = fscl(v, fac);
    dstl[x] = v;
    if (ghost) gdst[x] = fscl(v, sg);
  };
  auto edge_filter = [&](float2 *res) {
    for (int x = threadIdx.x; x < L.nxfilt; x += blockDim.x)
      if (L.filt_mode == 0 || L.filt_mode == 2) res[x] = fscl(res[x], L.filtr[x]);
    __syncthreads();
    for (int x = threadIdx.x; x < L.nxfilt; x += blockDim.x)
      if (L.filt_mode == 1 || L.filt_mode == 2) res[n - 1 - x] = fscl(res[n - 1 - x], L.filtr[x]);
  };
  if constexpr (MODE == 2) {
    auto buf_src = [a](int i) { return a[i]; };
    auto buf_dst = [a](int i, float2 v) { a[i] = v; };
    run16(a, n, P.log2n, tw, L.sign, load_elem, buf_dst);
    if (L.filt_mode >= 0) {
      edge_filter(a);
      run16(a, n, P.log2n, tw, -1, buf_src, buf_dst);
    }
    for (int x = threadIdx.x; x < n; x += blockDim.x) store_elem(x, a[x]);
    return;
  }
  float2 *res = POW2 ? run32p(P, a, b, tw, L.sign) : run32(P, a, b, tw, L.sign);
  if (L.filt_mode >= 0) {
    edge_filter(res);
    float2 *other = (res == a) ? b : a;
    res = POW2 ? run32p(P, res, other, tw, -1) : run32(P, res, other, tw, -1);
  }
  for (int x = threadIdx.x; x < n; x += blockDim.x) store_elem(x, res[x]);
}

// tw: room for n twiddles exp(-2 pi i t / n); already filled (shift32_kernel)
// when tw_ready
int lines32_launch(const Lines32 &L, int n, i64 nlines, float2 *tw, cudaStream_t st,
                   bool tw_ready = false) {
  Plan P;
  if (!make_plan(n, &P)) {
    set_error("split fft: unsupported length %d", n);
    return CHM_ERR_RANGE;
  }
  if (nlines <= 0) return CHM_OK;
  if (P.log2n >= 9) {
    if (!tw_ready) {
      twiddle32_kernel<<<(n + 255) / 256, 256, 0, st>>>(tw, n);
      chm::count_launch();
    }
    const size_t smem = (size_t)n * sizeof(float2);
    cudaFuncSetAttribute(lines32_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    lines32_kernel<2><<<(unsigned)nlines, n / 16, smem, st>>>(P, tw, L);
  } else if (P.log2n >= 0) {
    // the twiddle table is built per block in shared memory
    const int threads = n >= 256 ? 256 : 128;
    const size_t smem = 3 * (size_t)n * sizeof(float2);
    cudaFuncSetAttribute(lines32_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    lines32_kernel<1><<<(unsigned)nlines, threads, smem, st>>>(P, nullptr, L);
  } else {
    const int threads = n >= 1024 ? 512 : (n >= 256 ? 256 : 128);
    twiddle32_kernel<<<(n + 255) / 256, 256, 0, st>>>(tw, n);
    chm::count_launch();
    const size_t smem = 2 * (size_t)n * sizeof(float2);
    cudaFuncSetAttribute(lines32_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    lines32_kernel<0><<<(unsigned)nlines, threads, smem, st>>>(P, tw, L);
  }
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

// -------------------------------------------------------------------------
// Workspace
// -------------------------------------------------------------------------
struct Ws {
  char *p;
  i64 left;
  template <typename T>
  T *take(i64 n) {
    i64 bytes = (n * (i64)sizeof(T) + 255) / 256 * 256;
    if (bytes > left) return nullptr;
    T *r = reinterpret_cast<T *>(p);
    p += bytes;
    left -= bytes;
    return r;
  }
};

inline i64 r256(i64 b) { return (b + 255) / 256 * 256; }

// -------------------------------------------------------------------------
// Elementwise / combine kernels
// -------------------------------------------------------------------------
__global__ void zero32_kernel(float2 *p, i64 n) {
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < n; t += (i64)gridDim.x * blockDim.x)
    p[t] = make_float2(0.f, 0.f);
}

// grad of a scalar: out1 = i kx s, out2 = up - lo, out3 = i (lo + up)
// (fb_math.f90:96-149); with `poiss` the result updates J in place:
// J += (grad + (gnxt - gprv) dt_inv) * PF (maxwell_solvers.f90:131-164), or
// J += grad * PF without space charge (solvers.py:328-331).
struct GradArgs {
  i64 nx, nk;
  int nm, off;  // scalar index of output mode 0
  const float2 *scl;
  const float2 *lo, *up;  // products per output mode
  const float *kx;
  float2 *out;            // vector (nx, nk, nm, 3)
  i64 cs;                 // component stride of out
  int poiss;              // 0: store; 1: J update with charge; 2: J update, no charge
  const float2 *gprv, *gnxt;
  const float *pf;
  float dt_inv;
  int up_from;            // modes m < up_to have an upper product
  int up_to;
  // PSATD fused into the J update (maxwell_solvers.f90:18-96): with eg set,
  // the element's E and G advance with the new J (real FP32 coefficients
  // c1, c2 of nterm terms, planes of pstride elements)
  float2 *eg;
  const float *c1, *c2;
  int nterm;
  i64 pstride;
};

// the PSATD update of one spectral element from its new current jn
__device__ __forceinline__ void psatd_elem(float2 *__restrict__ eg, const float *__restrict__ c1,
                                           const float *__restrict__ c2, int nterm, i64 P, i64 i,
                                           const float2 *jn, const float2 *ga, const float2 *gb) {
  float a[5], b[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    a[k] = k < nterm ? c1[i + k * P] : 0.f;
    b[k] = k < nterm ? c2[i + k * P] : 0.f;
  }
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    const float2 e = eg[i + P * l], g = eg[i + P * (3 + l)], jj = jn[l];
    float2 en = fadd(fadd(fscl(e, a[0]), fscl(g, a[1])), fscl(jj, a[2]));
    float2 gn = fadd(fadd(fscl(e, b[0]), fscl(g, b[1])), fscl(jj, b[2]));
    if (nterm == 5) {
      const float2 x = ga[l], y = gb[l];
      en = fadd(en, fadd(fscl(x, a[3]), fscl(y, a[4])));
      gn = fadd(gn, fadd(fscl(x, b[3]), fscl(y, b[4])));
    }
    eg[i + P * (3 + l)] = gn;
    eg[i + P * l] = en;
  }
}

// The elementwise kernels below take one x line per block: blockIdx.x = kr,
// blockIdx.y = mode, threads along x (no index division per element).
__global__ void grad32_kernel(GradArgs A) {
  const i64 plane = A.nx * A.nk;
  const int m = blockIdx.y;
  const i64 line = A.nx * (i64)blockIdx.x;
  for (int x = threadIdx.x; x < A.nx; x += blockDim.x) {
    const i64 e = line + x;
    const i64 t = e + (i64)m * plane;
    const float2 s = A.scl[e + plane * (m + A.off)];
    const float2 lo = A.lo[t];
    const float2 up = (m < A.up_to) ? A.up[t] : make_float2(0.f, 0.f);
    float2 g[3];
    g[0] = fscl(fmi(s), A.kx[x]);
    g[1] = fsub(up, lo);
    g[2] = fmi(fadd(lo, up));
    if (A.poiss == 0) {
#pragma unroll
      for (int c = 0; c < 3; ++c) A.out[t + c * A.cs] = g[c];
    } else {
      const float f = A.pf[t];
      float2 jn[3], ga[3], gb[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float2 v = g[c];
        if (A.poiss == 1) {
          ga[c] = A.gprv[t + c * A.cs];
          gb[c] = A.gnxt[t + c * A.cs];
          v = fadd(v, fscl(fsub(gb[c], ga[c]), A.dt_inv));
        }
        jn[c] = fadd(A.out[t + c * A.cs], fscl(v, f));
        A.out[t + c * A.cs] = jn[c];
      }
      if (A.eg) psatd_elem(A.eg, A.c1, A.c2, A.nterm, A.pstride, t, jn, ga, gb);
    }
  }
}

// divergence on ns scalar modes (fb_math.f90:222-252)
struct DivArgs {
  i64 nx, nk;
  int ns, nm;
  const float2 *v;  // (nx, nk, nm, 3)
  i64 cs;
  const float2 *lo2, *lo3, *up2, *up3;  // per scalar mode
  const float *kx;
  float2 *scl;
  unsigned char lo_ok[16], up_ok[16];
};

__global__ void div32_kernel(DivArgs A) {
  const i64 plane = A.nx * A.nk;
  const int ms = blockIdx.y;
  const i64 line = A.nx * (i64)blockIdx.x;
  for (int x = threadIdx.x; x < A.nx; x += blockDim.x) {
    const i64 e = line + x;
    const i64 t = e + (i64)ms * plane;
    float2 r = make_float2(0.f, 0.f);
    if (ms < A.nm) r = fscl(fmi(A.v[e + plane * ms]), A.kx[x]);
    if (A.lo_ok[ms]) r = fadd(r, fsub(fmi(A.lo3[t]), A.lo2[t]));
    if (A.up_ok[ms]) r = fadd(r, fadd(fmi(A.up3[t]), A.up2[t]));
    A.scl[t] = r;
  }
}

// curl of G with PoissFact: B = rot(G) * PF (fb_math.f90:18-94, solvers.py:536-553)
struct RotArgs {
  i64 nx, nk;
  int nm;
  int env;  // envelope curl (fb_math_env.f90): no lower-neighbour term in component 1
  const float2 *v;
  i64 cs;
  const float2 *lo[3], *up[3];
  const float *kx, *pf;
  float2 *out;
};

__global__ void rot32_kernel(RotArgs A) {
  const i64 plane = A.nx * A.nk;
  const int m = blockIdx.y;
  const i64 line = A.nx * (i64)blockIdx.x;
  for (int x = threadIdx.x; x < A.nx; x += blockDim.x) {
    const i64 t = line + x + (i64)m * plane;
    const float kxv = A.kx[x];
    const float2 v2 = A.v[t + A.cs], v3 = A.v[t + 2 * A.cs];
    const bool hi = m < A.nm - 1;
    const float2 z = make_float2(0.f, 0.f);
    const float2 p1 = hi ? A.up[0][t] : z, p2 = hi ? A.up[1][t] : z, p3 = hi ? A.up[2][t] : z;
    const float2 m1 = A.lo[0][t], m2 = A.lo[1][t], m3 = A.lo[2][t];
    float2 o1 = fsub(make_float2(0.f, 0.f), fsub(fmi(p2), p3));
    if (!A.env) o1 = fsub(o1, fadd(fmi(m2), m3));
    float2 o2 = fadd(fscl(fmi(v3), -kxv), fadd(fmi(p1), fmi(m1)));
    float2 o3 = fadd(fscl(fmi(v2), kxv), fsub(m1, p1));
    const float f = A.pf[t];
    A.out[t] = fscl(o1, f);
    A.out[t + A.cs] = fscl(o2, f);
    A.out[t + 2 * A.cs] = fscl(o3, f);
  }
}

// PSATD (maxwell_solvers.f90:18-96), FP32 real coefficients, 3 or 5 terms
__global__ void psatd32_kernel(float2 *__restrict__ eg, const float2 *__restrict__ j,
                               const float2 *__restrict__ ga, const float2 *__restrict__ gb,
                               const float *__restrict__ c1, const float *__restrict__ c2, int nterm,
                               i64 P) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P; i += (i64)gridDim.x * blockDim.x) {
    float a[5], b[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      a[k] = k < nterm ? c1[i + k * P] : 0.f;
      b[k] = k < nterm ? c2[i + k * P] : 0.f;
    }
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      const float2 e = eg[i + P * l], g = eg[i + P * (3 + l)], jj = j[i + P * l];
      float2 en = fadd(fadd(fscl(e, a[0]), fscl(g, a[1])), fscl(jj, a[2]));
      float2 gn = fadd(fadd(fscl(e, b[0]), fscl(g, b[1])), fscl(jj, b[2]));
      if (nterm == 5) {
        const float2 x = ga[i + P * l], y = gb[i + P * l];
        en = fadd(en, fadd(fscl(x, a[3]), fscl(y, a[4])));
        gn = fadd(gn, fadd(fscl(x, b[3]), fscl(y, b[4])));
      }
      eg[i + P * (3 + l)] = gn;
      eg[i + P * l] = en;
    }
  }
}

// PSATD without space charge, complex FP32 coefficients (the envelope
// solver's, maxwell_solvers.f90:62-96)
__global__ void psatd32c_kernel(float2 *__restrict__ eg, const float2 *__restrict__ j,
                                const float2 *__restrict__ c1, const float2 *__restrict__ c2, i64 P) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P; i += (i64)gridDim.x * blockDim.x) {
    const float2 a0 = c1[i], a1 = c1[i + P], a2 = c1[i + 2 * P];
    const float2 b0 = c2[i], b1 = c2[i + P], b2 = c2[i + 2 * P];
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      const float2 e = eg[i + P * l], g = eg[i + P * (3 + l)], jj = j[i + P * l];
      const float2 en = fadd(fadd(fmul(a0, e), fmul(a1, g)), fmul(a2, jj));
      const float2 gn = fadd(fadd(fmul(b0, e), fmul(b1, g)), fmul(b2, jj));
      eg[i + P * (3 + l)] = gn;
      eg[i + P * l] = en;
    }
  }
}

// -------------------------------------------------------------------------
// dense products C(2nx, N) = A(2nx, K) * B(K, N) for a batch of planes
// -------------------------------------------------------------------------
struct Batch32 {
  TcProblem p[64];
  int count;
  void add(const float2 *A, float2 *C, const float *fac, const TcOperand &B, int reflect = 0) {
    p[count++] = TcProblem{reinterpret_cast<const float *>(A), reinterpret_cast<float *>(C), fac, B,
                           reflect};
  }
};

// W: the caller's remaining workspace (by value: the split A planes live
// there only while the product runs, stream-ordered before later kernels)
int gemm32(const Batch32 &b, int M, int N, int K, int epi, const float2 *shift, Ws W, cudaStream_t st) {
  if (b.count == 0) return CHM_OK;
  return tc_gemm_launch(b.p, b.count, M, N, K, epi, shift, W.p, W.left, st);
}

struct Fb32 {
  i64 nx, nk, nm;
  TcMatrices Dp, Dm;  // per-mode operands (split for the tensor cores)
  const float *kx;
  cudaStream_t st;
  Ws ws;
};

}  // namespace

// =========================================================================
// C ABI of the split-form spectral stage
// =========================================================================
extern "C" {

int64_t chm_sp_fb_ws_bytes(int64_t nx, int64_t nr, int64_t nkr, int64_t nm) {
  const i64 rows = nr - 1 > nkr ? nr - 1 : nkr;
  const i64 plane = 8 * nx * (rows > nkr ? rows : nkr);
  // + the BF16 split of the A planes of the largest product batch (6 nm
  // planes in fb_eb_out and the curl, 4 (nm + 1) in the Poisson correction)
  const i64 most = 6 * nm > 4 * (nm + 1) ? 6 * nm : 4 * (nm + 1);
  return 4 * r256(8 * nx) + r256(plane * nm * 6) + 8 * r256(plane * (nm + 2)) + 8192 +
         tc_split_bytes((int)(2 * nx), (int)rows, (int)most);
}

// fb_vec_in / fb_scl_in of a deposit accumulator (ncomp 3 or 1), with
// DepFact: out = shift * fact * DHT(FFT(acc / scale [+ acc2 / scale2]))
int chm_sp_fb_in_acc(void *out_c64, const int64_t *acc, const double *scale, const int64_t *acc2,
                     const double *scale2, double leftX, const double *kx, const void *In_ops,
                     const float *fact, int64_t nx, int64_t nr, int64_t nkr, int64_t nm,
                     int64_t ncomp, void *ws, int64_t ws_bytes, void *stream,
                     const chm_sp_window *win) {
  CHM_REQUIRE(out_c64 && acc && scale && kx && In_ops && fact, "sp_fb_in_acc: null pointer");
  CHM_REQUIRE(ws && ws_bytes >= chm_sp_fb_ws_bytes(nx, nr, nkr, nm), "sp_fb_in_acc: workspace");
  cudaStream_t st = as_stream(stream);
  Ws W{(char *)ws, ws_bytes};
  float2 *tw = W.take<float2>(nx);
  float2 *shift = W.take<float2>(nx);
  const i64 nrr = nr - 1;
  float2 *tmp = W.take<float2>(nx * nrr * nm * ncomp);
  if (!tmp) {
    set_error("sp_fb_in_acc: workspace exhausted");
    return CHM_ERR_WS;
  }
  shift32_kernel<<<grid_for(nx, 32), 32, 0, st>>>(shift, kx, leftX, -1, nx, tw, win); chm::count_launch();
  Lines32 L{};
  L.acc = reinterpret_cast<const long long *>(acc);
  L.acc_scale = scale;
  L.acc2 = reinterpret_cast<const long long *>(acc2);
  L.acc2_scale = scale2;
  L.in_rows = (int)nrr;
  L.in_rows_tot = (int)nr;
  L.in_row_off = 1;
  L.out = tmp;
  L.out_rows = L.out_rows_tot = (int)nrr;
  L.nm = (int)nm;
  L.sign = -1;
  L.filt_mode = -1;
  int rc = lines32_launch(L, (int)nx, nrr * nm * ncomp, tw, st, true);
  if (rc) return rc;
  const TcMatrices In = tc_matrices(reinterpret_cast<const chm_sp_ops *>(In_ops));
  Batch32 b{};  // every mode and component in one launch
  for (i64 m = 0; m < nm; ++m)
    for (i64 l = 0; l < ncomp; ++l)
      b.add(tmp + nx * nrr * (m + nm * l), reinterpret_cast<float2 *>(out_c64) + nx * nkr * (m + nm * l),
            fact + nx * nkr * m, In.mode[m]);
  return gemm32(b, (int)(2 * nx), (int)nkr, (int)nrr, TC_EPI_SHIFT_FAC, shift, W, st);
}

}  // extern "C"

namespace {

// fb_eb_out + eb_correction (fb_io.f90:182-228, grid_deps.f90:219-266;
// eb_mode 2: grid_deps_env.f90:240-283)
int eb_out_impl(void *eb_c64, const void *e_c64, const void *b_c64, double leftX, const double *kx,
                const void *Out_ops, int64_t nx, int64_t nr, int64_t nkr, int64_t nm, void *ws,
                int64_t ws_bytes, void *stream, const chm_sp_window *win, int eb_mode) {
  CHM_REQUIRE(eb_c64 && e_c64 && b_c64 && kx && Out_ops, "sp_fb_eb_out: null pointer");
  CHM_REQUIRE(ws && ws_bytes >= chm_sp_fb_ws_bytes(nx, nr, nkr, nm), "sp_fb_eb_out: workspace");
  cudaStream_t st = as_stream(stream);
  Ws W{(char *)ws, ws_bytes};
  float2 *tw = W.take<float2>(nx);
  float2 *shift = W.take<float2>(nx);
  const i64 nrr = nr - 1;
  float2 *tmp = W.take<float2>(nx * nrr * nm * 6);
  if (!tmp) {
    set_error("sp_fb_eb_out: workspace exhausted");
    return CHM_ERR_WS;
  }
  shift32_kernel<<<grid_for(nx, 32), 32, 0, st>>>(shift, kx, leftX, +1, nx, tw, win); chm::count_launch();
  const TcMatrices Out = tc_matrices(reinterpret_cast<const chm_sp_ops *>(Out_ops));
  Batch32 b{};  // every mode and component in one launch
  for (i64 m = 0; m < nm; ++m)
    for (int l = 0; l < 6; ++l) {
      const float2 *src = (l < 3 ? reinterpret_cast<const float2 *>(e_c64) + nx * nkr * (m + nm * l)
                                 : reinterpret_cast<const float2 *>(b_c64) + nx * nkr * (m + nm * (l - 3)));
      b.add(src, tmp + nx * nrr * (m + nm * l), nullptr, Out.mode[m]);
    }
  int rc = gemm32(b, (int)(2 * nx), (int)nrr, (int)nkr, TC_EPI_SHIFT, shift, W, st);
  if (rc) return rc;
  Lines32 L{};
  L.in = tmp;
  L.in_rows = L.in_rows_tot = (int)nrr;
  L.out = reinterpret_cast<float2 *>(eb_c64);
  L.out_rows = (int)nrr;
  L.out_rows_tot = (int)nr;
  L.out_row_off = 1;
  L.nm = (int)nm;
  L.eb_mode = eb_mode;
  L.sign = +1;
  L.filt_mode = -1;
  return lines32_launch(L, (int)nx, nrr * nm * 6, tw, st, true);
}

}  // namespace

extern "C" {

int chm_sp_fb_eb_out(void *eb_c64, const void *e_c64, const void *b_c64, double leftX,
                     const double *kx, const void *Out_ops, int64_t nx, int64_t nr, int64_t nkr,
                     int64_t nm, void *ws, int64_t ws_bytes, void *stream, const chm_sp_window *win) {
  return eb_out_impl(eb_c64, e_c64, b_c64, leftX, kx, Out_ops, nx, nr, nkr, nm, ws, ws_bytes, stream,
                     win, 1);
}

int chm_sp_fb_eb_out_env(void *eb_c64, const void *e_c64, const void *b_c64, double leftX,
                         const double *kx, const void *Out_ops, int64_t nx, int64_t nr,
                         int64_t nkr, int64_t nm, void *ws, int64_t ws_bytes, void *stream,
                         const chm_sp_window *win) {
  return eb_out_impl(eb_c64, e_c64, b_c64, leftX, kx, Out_ops, nx, nr, nkr, nm, ws, ws_bytes, stream,
                     win, 2);
}

// fb_filtr on complex64 planes (fb_io.f90:230-308)
int chm_sp_fb_filtr(void *vec_c64, double leftX, const double *kx, const float *filtr,
                    int64_t nxfilt, int modefilt, int64_t nx, int64_t nkr, int64_t nm,
                    int64_t ncomp, void *ws, int64_t ws_bytes, void *stream,
                    const chm_sp_window *win) {
  CHM_REQUIRE(vec_c64 && kx && (nxfilt == 0 || filtr) && modefilt >= 0 && modefilt <= 2,
              "sp_fb_filtr: bad args");
  CHM_REQUIRE(ws && ws_bytes >= 2 * r256(8 * nx), "sp_fb_filtr: workspace");
  cudaStream_t st = as_stream(stream);
  Ws W{(char *)ws, ws_bytes};
  float2 *tw = W.take<float2>(nx);
  float2 *shift = W.take<float2>(nx);
  shift32_kernel<<<grid_for(nx, 32), 32, 0, st>>>(shift, kx, leftX, +1, nx, tw, win); chm::count_launch();
  Lines32 L{};
  L.in = reinterpret_cast<const float2 *>(vec_c64);
  L.out = reinterpret_cast<float2 *>(vec_c64);
  L.in_rows = L.in_rows_tot = L.out_rows = L.out_rows_tot = (int)nkr;
  L.nm = (int)nm;
  L.sign = +1;
  L.pre_shift = shift;
  L.filt_mode = modefilt;
  L.filtr = filtr;
  L.nxfilt = (int)nxfilt;
  return lines32_launch(L, (int)nx, nkr * nm * ncomp, tw, st, true);
}

}  // extern "C"

namespace {

// lower / upper neighbour products of `ncomp` components for output modes
// 0..nout-1 (input mode m-1+shift / m+1+shift, D mode m + dshift: 1 for
// the envelope solver, whose D operators start one mode below -K).  The lower
// neighbour of input mode -1 is the m = 1 plane `refl[c]` read reflected by
// the product; without one (a single mode) that product is zero.
int neighbours32(Fb32 &F, const float2 *in, i64 cs, int ncomp, int nin, int nout, int shift,
                 const float2 *const *refl, float2 *lo[3], float2 *up[3], unsigned char *lo_ok,
                 unsigned char *up_ok, int dshift = 0) {
  const i64 plane = F.nx * F.nk;
  Batch32 b{};  // every output mode, neighbour and component in one launch
  for (int m = 0; m < nout; ++m) {
    const int mlo = m - 1 + shift, mhi = m + 1 + shift;
    lo_ok[m] = up_ok[m] = 0;
    for (int c = 0; c < ncomp; ++c) {
      if (mlo >= 0 && mlo < nin) {
        b.add(in + c * cs + plane * mlo, lo[c] + plane * m, nullptr, F.Dm.mode[m + dshift]);
        lo_ok[m] = 1;
      } else if (mlo == -1 && refl) {
        b.add(refl[c], lo[c] + plane * m, nullptr, F.Dm.mode[m + dshift], 1);
        lo_ok[m] = 1;
      } else if (mlo == -1) {
        zero32_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(lo[c] + plane * m, plane);
        chm::count_launch();
      }
      if (mhi >= 0 && mhi < nin) {
        b.add(in + c * cs + plane * mhi, up[c] + plane * m, nullptr, F.Dp.mode[m + dshift]);
        up_ok[m] = 1;
      }
    }
  }
  return gemm32(b, (int)(2 * F.nx), (int)F.nk, (int)F.nk, TC_EPI_STORE, nullptr, F.ws, F.st);
}

}  // namespace

extern "C" {

// fb_grad (fb_math.f90:96-149) on complex64
int chm_sp_fb_grad(void *out_c64, const void *scl_c64, const void *Dp_ops, const void *Dm_ops,
                   const float *kx, int64_t nx, int64_t nkr, int64_t nm, void *ws,
                   int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(out_c64 && scl_c64 && Dp_ops && Dm_ops && kx && nm <= 14, "sp_fb_grad: bad args");
  CHM_REQUIRE(ws && ws_bytes >= chm_sp_fb_ws_bytes(nx, nkr + 1, nkr, nm), "sp_fb_grad: workspace");
  Fb32 F{nx, nkr, nm, tc_matrices(reinterpret_cast<const chm_sp_ops *>(Dp_ops)),
         tc_matrices(reinterpret_cast<const chm_sp_ops *>(Dm_ops)), kx, as_stream(stream), Ws{(char *)ws, ws_bytes}};
  const i64 plane = nx * nkr;
  const float2 *s = reinterpret_cast<const float2 *>(scl_c64);
  float2 *lo[3] = {F.ws.take<float2>(plane * nm), nullptr, nullptr};
  float2 *up[3] = {F.ws.take<float2>(plane * nm), nullptr, nullptr};
  if (!up[0]) {
    set_error("sp_fb_grad: workspace exhausted");
    return CHM_ERR_WS;
  }
  const float2 *refl[3] = {s + plane, nullptr, nullptr};
  unsigned char lok[16], uok[16];
  int rc = neighbours32(F, s, 0, 1, (int)nm, (int)nm, 0, nm > 1 ? refl : nullptr, lo, up, lok, uok);
  if (rc) return rc;
  GradArgs A{};
  A.nx = nx;
  A.nk = nkr;
  A.nm = (int)nm;
  A.off = 0;
  A.scl = s;
  A.lo = lo[0];
  A.up = up[0];
  A.kx = kx;
  A.out = reinterpret_cast<float2 *>(out_c64);
  A.cs = plane * nm;
  A.up_to = (int)nm - 1;
  grad32_kernel<<<dim3((unsigned)nkr, (unsigned)nm), 256, 0, F.st>>>(A); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

// The Poisson correction of solvers.py:301-331 on complex64: `iters` times
//   v = grad(div(J)) (fb_graddiv, fb_math.f90:201-293)
//   J += (v + (gnxt - gprv) dt_inv) PF      (space charge)
//   J += v PF                               (otherwise)
}  // extern "C"

namespace {

int poisson_impl(void *J_c64, const void *gprv_c64, const void *gnxt_c64, const float *pf,
                 float dt_inv, const void *Dp_ops, const void *Dm_ops, const float *kx, int64_t nx,
                 int64_t nkr, int64_t nm, int iters, int space_charge, void *eg_c64,
                 const float *c1, const float *c2, int nterm, void *ws, int64_t ws_bytes,
                 void *stream) {
  CHM_REQUIRE(J_c64 && pf && Dp_ops && Dm_ops && kx && nm <= 14, "sp_poisson: bad args");
  CHM_REQUIRE(!space_charge || (gprv_c64 && gnxt_c64), "sp_poisson: missing charge gradients");
  CHM_REQUIRE(ws && ws_bytes >= chm_sp_fb_ws_bytes(nx, nkr + 1, nkr, nm), "sp_poisson: workspace");
  Fb32 F{nx, nkr, nm, tc_matrices(reinterpret_cast<const chm_sp_ops *>(Dp_ops)),
         tc_matrices(reinterpret_cast<const chm_sp_ops *>(Dm_ops)), kx, as_stream(stream), Ws{(char *)ws, ws_bytes}};
  const i64 plane = nx * nkr;
  const i64 cs = plane * nm;
  const int ns = (int)nm + 1;
  float2 *J = reinterpret_cast<float2 *>(J_c64);
  float2 *scl = F.ws.take<float2>(plane * ns);
  float2 *lo[3], *up[3];
  for (int c = 0; c < 3; ++c) {
    lo[c] = F.ws.take<float2>(plane * ns);
    up[c] = F.ws.take<float2>(plane * ns);
  }
  if (!up[2]) {
    set_error("sp_poisson: workspace exhausted");
    return CHM_ERR_WS;
  }
  for (int it = 0; it < iters; ++it) {
    // divergence on nm + 1 modes
    const float2 *refl23[3] = {J + cs + plane, J + 2 * cs + plane, nullptr};
    float2 *lo23[3] = {lo[1], lo[2], nullptr}, *up23[3] = {up[1], up[2], nullptr};
    DivArgs D{};
    int rc = neighbours32(F, J + cs, cs, 2, (int)nm, ns, 0, nm > 1 ? refl23 : nullptr, lo23, up23,
                          D.lo_ok, D.up_ok);
    if (rc) return rc;
    for (int ms = 0; ms < ns; ++ms)
      if (!(ms < (int)nm - 1)) D.up_ok[ms] = 0;
    D.nx = nx;
    D.nk = nkr;
    D.ns = ns;
    D.nm = (int)nm;
    D.v = J;
    D.cs = cs;
    D.lo2 = lo[1];
    D.lo3 = lo[2];
    D.up2 = up[1];
    D.up3 = up[2];
    D.kx = kx;
    D.scl = scl;
    div32_kernel<<<dim3((unsigned)nkr, (unsigned)ns), 256, 0, F.st>>>(D); chm::count_launch();
    // gradient of the nm + 1 scalar modes back onto nm modes, fused with the
    // J update; the m = -1 neighbour of mode 0 is scalar mode 1 reflected
    // (zero with a single mode)
    Batch32 bg{};  // both neighbours of every mode in one launch
    for (int m = 0; m < (int)nm; ++m) {
      if (m >= 1) {
        bg.add(scl + plane * (m - 1), lo[0] + plane * m, nullptr, F.Dm.mode[m]);
      } else if (nm > 1) {
        bg.add(scl + plane, lo[0], nullptr, F.Dm.mode[0], 1);
      } else {
        zero32_kernel<<<grid_for(plane, 256), 256, 0, F.st>>>(lo[0], plane);
        chm::count_launch();
      }
      bg.add(scl + plane * (m + 1), up[0] + plane * m, nullptr, F.Dp.mode[m]);
    }
    rc = gemm32(bg, (int)(2 * nx), (int)nkr, (int)nkr, TC_EPI_STORE, nullptr, F.ws, F.st);
    if (rc) return rc;
    GradArgs A{};
    A.nx = nx;
    A.nk = nkr;
    A.nm = (int)nm;
    A.off = 0;
    A.scl = scl;
    A.lo = lo[0];
    A.up = up[0];
    A.kx = kx;
    A.out = J;
    A.cs = cs;
    A.poiss = space_charge ? 1 : 2;
    A.gprv = reinterpret_cast<const float2 *>(gprv_c64);
    A.gnxt = reinterpret_cast<const float2 *>(gnxt_c64);
    A.pf = pf;
    A.dt_inv = dt_inv;
    A.up_to = (int)nm;
    if (eg_c64 && it == iters - 1) {
      A.eg = reinterpret_cast<float2 *>(eg_c64);
      A.c1 = c1;
      A.c2 = c2;
      A.nterm = nterm;
      A.pstride = cs;
    }
    grad32_kernel<<<dim3((unsigned)nkr, (unsigned)nm), 256, 0, F.st>>>(A); chm::count_launch();
  }
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // namespace

extern "C" {

int chm_sp_poisson(void *J_c64, const void *gprv_c64, const void *gnxt_c64, const float *pf,
                   float dt_inv, const void *Dp_ops, const void *Dm_ops, const float *kx,
                   int64_t nx, int64_t nkr, int64_t nm, int iters, int space_charge, void *ws,
                   int64_t ws_bytes, void *stream) {
  return poisson_impl(J_c64, gprv_c64, gnxt_c64, pf, dt_inv, Dp_ops, Dm_ops, kx, nx, nkr, nm, iters,
                      space_charge, nullptr, nullptr, nullptr, 0, ws, ws_bytes, stream);
}

// the Poisson correction with the PSATD update fused into its last J update
int chm_sp_poisson_psatd(void *J_c64, const void *gprv_c64, const void *gnxt_c64, const float *pf,
                         float dt_inv, const void *Dp_ops, const void *Dm_ops, const float *kx,
                         int64_t nx, int64_t nkr, int64_t nm, int iters, int space_charge,
                         void *eg_c64, const float *c1, const float *c2, int nterm, void *ws,
                         int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(eg_c64 && c1 && c2 && iters >= 1, "sp_poisson_psatd: bad args");
  CHM_REQUIRE((space_charge && nterm == 5) || (!space_charge && nterm == 3),
              "sp_poisson_psatd: 5 PSATD terms with space charge, 3 without");
  return poisson_impl(J_c64, gprv_c64, gnxt_c64, pf, dt_inv, Dp_ops, Dm_ops, kx, nx, nkr, nm, iters,
                      space_charge, eg_c64, c1, c2, nterm, ws, ws_bytes, stream);
}

}  // extern "C"

namespace {

// B = rot(G) * PoissFact (solvers.py:536-553); env: the envelope curl
// (fb_math_env.f90) on the stored modes -K..K, no reflected neighbour
int rot_b_impl(void *B_c64, const void *G_c64, const float *pf, const void *Dp_ops,
               const void *Dm_ops, const float *kx, int64_t nx, int64_t nkr, int64_t nm, void *ws,
               int64_t ws_bytes, void *stream, int env) {
  CHM_REQUIRE(B_c64 && G_c64 && pf && Dp_ops && Dm_ops && kx && nm <= 14, "sp_rot_b: bad args");
  CHM_REQUIRE(!env || nm % 2 == 1, "sp_rot_b_env: the envelope solver stores an odd mode count");
  CHM_REQUIRE(ws && ws_bytes >= chm_sp_fb_ws_bytes(nx, nkr + 1, nkr, nm), "sp_rot_b: workspace");
  Fb32 F{nx, nkr, nm, tc_matrices(reinterpret_cast<const chm_sp_ops *>(Dp_ops)),
         tc_matrices(reinterpret_cast<const chm_sp_ops *>(Dm_ops)), kx, as_stream(stream), Ws{(char *)ws, ws_bytes}};
  const i64 plane = nx * nkr;
  const i64 cs = plane * nm;
  const float2 *G = reinterpret_cast<const float2 *>(G_c64);
  float2 *lo[3], *up[3];
  for (int c = 0; c < 3; ++c) {
    lo[c] = F.ws.take<float2>(plane * nm);
    up[c] = F.ws.take<float2>(plane * nm);
  }
  if (!up[2]) {
    set_error("sp_rot_b: workspace exhausted");
    return CHM_ERR_WS;
  }
  const float2 *refl[3] = {G + plane, G + cs + plane, G + 2 * cs + plane};
  unsigned char lok[16], uok[16];
  int rc = neighbours32(F, G, cs, 3, (int)nm, (int)nm, 0, (nm > 1 && !env) ? refl : nullptr, lo, up,
                        lok, uok, env ? 1 : 0);
  if (rc) return rc;
  RotArgs A{};
  A.nx = nx;
  A.nk = nkr;
  A.nm = (int)nm;
  A.env = env;
  A.v = G;
  A.cs = cs;
  for (int c = 0; c < 3; ++c) {
    A.lo[c] = lo[c];
    A.up[c] = up[c];
  }
  A.kx = kx;
  A.pf = pf;
  A.out = reinterpret_cast<float2 *>(B_c64);
  rot32_kernel<<<dim3((unsigned)nkr, (unsigned)nm), 256, 0, F.st>>>(A); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // namespace

extern "C" {

int chm_sp_rot_b(void *B_c64, const void *G_c64, const float *pf, const void *Dp_ops,
                 const void *Dm_ops, const float *kx, int64_t nx, int64_t nkr, int64_t nm, void *ws,
                 int64_t ws_bytes, void *stream) {
  return rot_b_impl(B_c64, G_c64, pf, Dp_ops, Dm_ops, kx, nx, nkr, nm, ws, ws_bytes, stream, 0);
}

int chm_sp_rot_b_env(void *B_c64, const void *G_c64, const float *pf, const void *Dp_ops,
                     const void *Dm_ops, const float *kx, int64_t nx, int64_t nkr, int64_t nm,
                     void *ws, int64_t ws_bytes, void *stream) {
  return rot_b_impl(B_c64, G_c64, pf, Dp_ops, Dm_ops, kx, nx, nkr, nm, ws, ws_bytes, stream, 1);
}

int chm_sp_psatd_c(void *eg_c64, const void *j_c64, const void *c1_c64, const void *c2_c64,
                   int64_t P, void *stream) {
  CHM_REQUIRE(eg_c64 && j_c64 && c1_c64 && c2_c64 && P >= 0, "sp_psatd_c: bad args");
  if (P == 0) return CHM_OK;
  psatd32c_kernel<<<grid_for(P, 256), 256, 0, as_stream(stream)>>>(
      (float2 *)eg_c64, (const float2 *)j_c64, (const float2 *)c1_c64, (const float2 *)c2_c64, P);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_psatd(void *eg_c64, const void *j_c64, const void *gprv_c64, const void *gnxt_c64,
                 const float *c1, const float *c2, int nterm, int64_t P, void *stream) {
  CHM_REQUIRE(eg_c64 && j_c64 && c1 && c2 && (nterm == 3 || nterm == 5), "sp_psatd: bad args");
  CHM_REQUIRE(nterm == 3 || (gprv_c64 && gnxt_c64), "sp_psatd: missing charge gradients");
  psatd32_kernel<<<grid_for(P, 256), 256, 0, as_stream(stream)>>>(
      (float2 *)eg_c64, (const float2 *)j_c64, (const float2 *)gprv_c64, (const float2 *)gnxt_c64,
      c1, c2, nterm, P); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"

extern "C" {

int chm_sp_window_set(chm_sp_window *win, double leftX, double X0, double dx, void *stream) {
  CHM_REQUIRE(win && dx > 0, "sp_window_set: bad args");
  window_kernel<<<1, 32, 0, as_stream(stream)>>>(win, 1, leftX, X0, dx, 0.0);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_window_advance(chm_sp_window *win, double shift, void *stream) {
  CHM_REQUIRE(win, "sp_window_advance: bad args");
  window_kernel<<<1, 32, 0, as_stream(stream)>>>(win, 0, 0.0, 0.0, 0.0, shift);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"
