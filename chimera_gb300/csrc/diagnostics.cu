// Field diagnostics of the reference's Diagnostics class, as device
// reductions over the FP64 grids (no host round trip of the fields):
//   chm_em_energy      -- nrg_out (diagnostics.py:109-122): electromagnetic
//                         energy per kx from the spectral E field
//   chm_power_profile  -- pwr_out (diagnostics.py:124-149): laser power per
//                         x from the spatial E field
//   chm_intens_profo   -- intens_profO (utils.f90:18-57): intensity over
//                         NO azimuthal angles and r
// Every sum runs in a fixed order (a fixed thread-to-element assignment, then
// a fixed tree), so the results are bitwise reproducible run to run.
#include "common.cuh"

using namespace chm;

namespace {

constexpr int kRedThreads = 256;

// Block sum of one double per thread, fixed tree order; the result is valid
// in thread 0.
__device__ double block_sum(double v, double *sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
  __syncthreads();
  return t;
}

__device__ __forceinline__ double abs2(double2 a) { return a.x * a.x + a.y * a.y; }

// out[x] = sum_{kr, m} efact(x, kr, m) sum_{l < 3} |eg(x, kr, m, l)|^2
// (eg: (nx, nkr, nm, ncomp) with the E field in components 0-2)
__global__ void __launch_bounds__(kRedThreads) em_energy_kernel(double *out, const double2 *eg,
                                                               const double *efact, i64 nx,
                                                               i64 nkr, i64 nm) {
  __shared__ double sm[kRedThreads / 32];
  const i64 x = blockIdx.x;
  const i64 plane = nx * nkr * nm;
  double acc = 0.0;
  for (i64 t = threadIdx.x; t < nkr * nm; t += blockDim.x) {
    const i64 e = x + nx * t;  // (x, kr, m) with t = kr + nkr m
    double s = 0.0;
    for (int l = 0; l < 3; ++l) s += abs2(eg[e + plane * l]);
    acc += s * efact[e];
  }
  const double tot = block_sum(acc, sm);
  if (threadIdx.x == 0) out[x] = tot;
}

// out[x] = fac sum_r rgrid[r] sum_{m, l} |v(x, r, m, l)|^2, v: (nx, nr, nm, 3)
__global__ void __launch_bounds__(kRedThreads) power_profile_kernel(double *out, const double2 *v,
                                                                   const double *rgrid, double fac,
                                                                   i64 nx, i64 nr, i64 nm) {
  __shared__ double sm[kRedThreads / 32];
  const i64 x = blockIdx.x;
  const i64 plane = nx * nr * nm;
  double acc = 0.0;
  for (i64 r = threadIdx.x; r < nr; r += blockDim.x) {
    double s = 0.0;
    for (i64 m = 0; m < nm; ++m)
      for (int l = 0; l < 3; ++l) s += abs2(v[x + nx * (r + nr * m) + plane * l]);
    acc += s * rgrid[r];
  }
  const double tot = block_sum(acc, sm);
  if (threadIdx.x == 0) out[x] = fac * tot;
}

// pwr(iO, ir - 1) = sum_l sum_ix |sum_k e^{i k phi_iO} fld(ix, ir, k, l)|^2,
// phi_iO = 2 pi (iO - 1) / (NO - 1), k = -K..K, for ir = 1 .. NR - 1 (the
// ghost row 0 is skipped as in the Fortran); fld: (NX, NR, 2K + 1, 3).
// One block per (iO, ir), iO fastest so the blocks of one row share L2.
__global__ void __launch_bounds__(kRedThreads) intens_profo_kernel(double *pwr, const double2 *fld,
                                                                  i64 NO, i64 NX, i64 NR, i64 K) {
  __shared__ double sm[kRedThreads / 32];
  __shared__ double2 ph[64];
  const i64 io = blockIdx.x % NO, ir = 1 + blockIdx.x / NO;
  const i64 NM = 2 * K + 1;
  if (threadIdx.x < NM) {
    // e^{i k phi} with k = threadIdx.x - K
    double s, c;
    sincospi(2.0 * (double)io * (double)(threadIdx.x - K) / (double)(NO - 1), &s, &c);
    ph[threadIdx.x] = make_double2(c, s);
  }
  __syncthreads();
  const i64 plane = NX * NR * NM;
  double acc = 0.0;
  for (i64 ix = threadIdx.x; ix < NX; ix += blockDim.x) {
    for (int l = 0; l < 3; ++l) {
      double2 s = make_double2(0.0, 0.0);
      for (i64 k = 0; k < NM; ++k) s = cadd(s, cmul(ph[k], fld[ix + NX * (ir + NR * k) + plane * l]));
      acc += abs2(s);
    }
  }
  const double tot = block_sum(acc, sm);
  if (threadIdx.x == 0) pwr[io + NO * (ir - 1)] = tot;
}

}  // namespace

extern "C" {

int chm_em_energy(double *out, const chm_c128 *eg, const double *efact, int64_t nx, int64_t nkr,
                  int64_t nm, int64_t ncomp, void *stream) {
  CHM_REQUIRE(out && eg && efact, "em_energy: null pointer");
  CHM_REQUIRE(nx > 0 && nkr > 0 && nm > 0 && ncomp >= 3, "em_energy: bad dims");
  em_energy_kernel<<<(unsigned)nx, kRedThreads, 0, as_stream(stream)>>>(
      out, reinterpret_cast<const double2 *>(eg), efact, nx, nkr, nm);
  count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_power_profile(double *out, const chm_c128 *vec, const double *rgrid, double fac, int64_t nx,
                      int64_t nr, int64_t nm, void *stream) {
  CHM_REQUIRE(out && vec && rgrid, "power_profile: null pointer");
  CHM_REQUIRE(nx > 0 && nr > 0 && nm > 0, "power_profile: bad dims");
  power_profile_kernel<<<(unsigned)nx, kRedThreads, 0, as_stream(stream)>>>(
      out, reinterpret_cast<const double2 *>(vec), rgrid, fac, nx, nr, nm);
  count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_intens_profo(double *pwr, const chm_c128 *fld, int64_t NO, int64_t NX, int64_t NR,
                     int64_t NM, void *stream) {
  CHM_REQUIRE(pwr && fld, "intens_profo: null pointer");
  CHM_REQUIRE(NO >= 2 && NX > 0 && NR > 1 && NM >= 1 && NM % 2 == 1 && NM <= 63,
              "intens_profo: bad dims (NO >= 2, an odd mode count -K..K up to 63)");
  const i64 blocks = NO * (NR - 1);
  CHM_REQUIRE(blocks < (1LL << 31), "intens_profo: too many (angle, row) pairs");
  intens_profo_kernel<<<(unsigned)blocks, kRedThreads, 0, as_stream(stream)>>>(
      pwr, reinterpret_cast<const double2 *>(fld), NO, NX, NR, (NM - 1) / 2);
  count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"
