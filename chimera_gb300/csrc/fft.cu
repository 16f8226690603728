// Batched shared-memory FFT along x (FP64).  See fft.cuh.
#include <math.h>

#include "fft.cuh"

namespace chm {

static constexpr double kPi = 3.14159265358979323846;

bool fft_make_plan(int n, FftPlan *p) {
  if (n < 1 || n > kFftMaxN) return false;
  p->n = n;
  p->nstages = 0;
  int m = n;
  while (m % 4 == 0 && p->nstages < kFftMaxStages) {
    p->radix[p->nstages++] = 4;
    m /= 4;
  }
  const int small[4] = {2, 3, 5, 7};
  for (int s = 0; s < 4; ++s)
    while (m % small[s] == 0 && p->nstages < kFftMaxStages) {
      p->radix[p->nstages++] = small[s];
      m /= small[s];
    }
  for (int f = 11; m > 1 && p->nstages < kFftMaxStages;) {
    if ((i64)f * f > m) f = m;
    if (m % f == 0) {
      p->radix[p->nstages++] = f;
      m /= f;
    } else {
      f += 2;
    }
  }
  return m == 1;
}

__global__ void fft_twiddle_kernel(double2 *tw, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s, c;
    // exp(-2 pi i t / n); sincospi keeps the argument exact
    sincospi(2.0 * (double)t / (double)n, &s, &c);
    tw[t] = make_double2(c, -s);
  }
}

// W^t for the table of the forward transform; sign=+1 conjugates.
__device__ __forceinline__ double2 twid(const double2 *__restrict__ tw, int t, int sign) {
  double2 w = tw[t];
  if (sign > 0) w.y = -w.y;
  return w;
}

// One Stockham pass with radix R over a line in shared memory.
__device__ void stockham_pass(const double2 *__restrict__ src, double2 *__restrict__ dst, int n,
                              int R, int Ns, const double2 *__restrict__ tw, int sign) {
  const int nb = n / R;
  for (int j = threadIdx.x; j < nb; j += blockDim.x) {
    const int k = j % Ns;
    double2 v[16];
    const int tstep = (n / (Ns * R)) * k;  // twiddle index step per r
    if (R <= 16) {
      for (int r = 0; r < R; ++r) {
        double2 a = src[j + r * nb];
        if (r > 0 && k > 0) a = cmul(a, twid(tw, (r * tstep) % n, sign));
        v[r] = a;
      }
      const int base = (j / Ns) * Ns * R + k;
      if (R == 2) {
        dst[base] = cadd(v[0], v[1]);
        dst[base + Ns] = csub(v[0], v[1]);
      } else if (R == 4) {
        double2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        double2 a2 = cadd(v[1], v[3]), a3 = csub(v[1], v[3]);
        // multiply a3 by -i (forward) or +i (backward)
        double2 a3r = sign < 0 ? make_double2(a3.y, -a3.x) : make_double2(-a3.y, a3.x);
        dst[base] = cadd(a0, a2);
        dst[base + Ns] = cadd(a1, a3r);
        dst[base + 2 * Ns] = csub(a0, a2);
        dst[base + 3 * Ns] = csub(a1, a3r);
      } else {
        const int step = n / R;
        for (int q = 0; q < R; ++q) {
          double2 acc = v[0];
          for (int r = 1; r < R; ++r) acc = cadd(acc, cmul(v[r], twid(tw, ((r * q) % R) * step, sign)));
          dst[base + q * Ns] = acc;
        }
      }
    } else {
      // large prime radix: direct DFT reading straight from src
      const int base = (j / Ns) * Ns * R + k;
      const int step = n / R;
      for (int q = 0; q < R; ++q) {
        double2 acc = make_double2(0.0, 0.0);
        for (int r = 0; r < R; ++r) {
          double2 a = src[j + r * nb];
          if (r > 0 && k > 0) a = cmul(a, twid(tw, (r * tstep) % n, sign));
          acc = cadd(acc, cmul(a, twid(tw, ((r * q) % R) * step, sign)));
        }
        dst[base + q * Ns] = acc;
      }
    }
  }
}

// Runs all passes; returns the buffer holding the result.
__device__ double2 *run_fft(FftPlan plan, double2 *a, double2 *b, const double2 *__restrict__ tw,
                            int sign) {
  int Ns = 1;
  for (int s = 0; s < plan.nstages; ++s) {
    const int R = plan.radix[s];
    __syncthreads();
    stockham_pass(a, b, plan.n, R, Ns, tw, sign);
    Ns *= R;
    double2 *t = a;
    a = b;
    b = t;
  }
  __syncthreads();
  return a;
}

__global__ void fft_lines_kernel(FftPlan plan, const double2 *__restrict__ tw, FftLines L) {
  extern __shared__ __align__(16) double2 sm[];
  const int n = plan.n;
  double2 *a = sm, *b = sm + n;
  const i64 line = blockIdx.x;
  const i64 ib = line / L.in_rows, ir = line % L.in_rows;
  const double2 *src = L.in + (ib * L.in_rows_tot + ir + L.in_row_off) * (i64)n;
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    double2 v = src[x];
    if (L.pre_shift) v = cmul(v, L.pre_shift[x]);
    a[x] = v;
  }
  double2 *res = run_fft(plan, a, b, tw, L.sign);
  if (L.filt_mode >= 0) {
    // fb_io.f90:255-304: profile on the first / last nxfilt cells, then the
    // forward FFT and 1/(N shift)
    for (int x = threadIdx.x; x < L.nxfilt; x += blockDim.x) {
      if (L.filt_mode == 0 || L.filt_mode == 2) res[x] = cscale(res[x], L.filtr[x]);
    }
    __syncthreads();
    for (int x = threadIdx.x; x < L.nxfilt; x += blockDim.x) {
      if (L.filt_mode == 1 || L.filt_mode == 2) res[n - 1 - x] = cscale(res[n - 1 - x], L.filtr[x]);
    }
    double2 *other = (res == a) ? b : a;
    res = run_fft(plan, res, other, tw, -1);
  }
  const i64 ob = line / L.out_rows, orow = line % L.out_rows;
  double2 *dst = L.out + (ob * L.out_rows_tot + orow + L.out_row_off) * (i64)n;
  double fac = 1.0, sg = 1.0;
  if (L.eb_mode) {
    const int m = (int)(ob % L.nm);
    const double pi_inv = 1.0 / kPi;
    if (L.eb_mode == 1) {
      fac = (m == 0) ? 0.5 * pi_inv : pi_inv;
      sg = (m == 0) ? 1.0 : -1.0;
    } else {
      fac = pi_inv;
      sg = (L.nm == 1) ? 1.0 : -1.0;
    }
  }
  const bool ghost = L.eb_mode && orow == 0;
  double2 *gdst = L.out + (ob * L.out_rows_tot) * (i64)n;
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    double2 v = res[x];
    if (L.filt_mode >= 0) {
      // times 1/(N e^{+i kx leftX}) = conj(shift)/N with |shift| = 1 is not
      // bit-identical; divide as the Fortran does
      double2 s = L.pre_shift[x];
      double d = (double)n * (s.x * s.x + s.y * s.y);
      v = cmul(v, make_double2(s.x / d, -s.y / d));
    }
    if (L.eb_mode) v = cscale(v, fac);
    dst[x] = v;
    if (ghost) gdst[x] = cscale(v, sg);
  }
}

int fft_launch(const FftLines &L, int n, i64 nlines, double2 *tw, cudaStream_t st) {
  FftPlan plan;
  if (!fft_make_plan(n, &plan)) {
    set_error("fft: unsupported length %d (max %d)", n, kFftMaxN);
    return CHM_ERR_RANGE;
  }
  if (nlines <= 0) return CHM_OK;
  fft_twiddle_kernel<<<(n + 255) / 256, 256, 0, st>>>(tw, n); chm::count_launch();
  const size_t smem = 2 * (size_t)n * sizeof(double2);
  cudaFuncSetAttribute(fft_lines_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int threads = n >= 1024 ? 512 : (n >= 256 ? 256 : 128);
  fft_lines_kernel<<<(unsigned)nlines, threads, smem, st>>>(plan, tw, L); chm::count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("fft: %s", cudaGetErrorString(e));
    return CHM_ERR_CUDA;
  }
  return CHM_OK;
}

}  // namespace chm
