// Particle push, field gather and external-field ("device") kernels, FP64.
//
// Every particle kernel is a grid-stride stream over the structure-of-arrays
// particle buffers: one thread per particle, strided loads that coalesce when
// part_stride == 1.  The gather reads the 2x2-node stencil of every stored
// mode straight from the column-major spectral-space grid (L1/L2 resident
// for cell-ordered particles).
#include <math.h>

#include "common.cuh"

using namespace chm;

namespace {

constexpr int kThreads = 256;
constexpr double kPi = 3.14159265358979323846;

// particle_tools.f90:18-56
__global__ void push_velocs_kernel(double *__restrict__ p, i64 p_cs, i64 p_ps,
                                   const double *__restrict__ f, i64 f_cs, i64 f_ps,
                                   double dt, i64 np) {
  const double dt_2 = 0.5 * dt;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < np;
       i += (i64)gridDim.x * blockDim.x) {
    double um[3], t[3], s[3], u0[3], up[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) um[c] = p[c * p_cs + i * p_ps] + dt_2 * f[c * f_cs + i * f_ps];
    double gamma = sqrt(1.0 + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]));
#pragma unroll
    for (int c = 0; c < 3; ++c) t[c] = dt_2 * f[(3 + c) * f_cs + i * f_ps] / gamma;
    double t2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
#pragma unroll
    for (int c = 0; c < 3; ++c) s[c] = 2 * t[c] / (1 + t2);
    u0[0] = um[0] + um[1] * t[2] - um[2] * t[1];
    u0[1] = um[1] - um[0] * t[2] + um[2] * t[0];
    u0[2] = um[2] + um[0] * t[1] - um[1] * t[0];
    up[0] = um[0] + u0[1] * s[2] - u0[2] * s[1];
    up[1] = um[1] - u0[0] * s[2] + u0[2] * s[0];
    up[2] = um[2] + u0[0] * s[1] - u0[1] * s[0];
#pragma unroll
    for (int c = 0; c < 3; ++c) p[c * p_cs + i * p_ps] = up[c] + dt_2 * f[c * f_cs + i * f_ps];
  }
}

// particle_tools.f90:58-82
__global__ void push_coords_kernel(double *__restrict__ x, i64 x_cs, i64 x_ps,
                                   const double *__restrict__ p, i64 p_cs, i64 p_ps,
                                   double *__restrict__ h, i64 h_cs, i64 h_ps, double dt,
                                   i64 np) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < np;
       i += (i64)gridDim.x * blockDim.x) {
    double pp[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) pp[c] = p[c * p_cs + i * p_ps];
    double dt_gp = dt / sqrt(1.0 + (pp[0] * pp[0] + pp[1] * pp[1] + pp[2] * pp[2]));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double xo = x[c * x_cs + i * x_ps];
      double xn = xo + pp[c] * dt_gp;
      x[c * x_cs + i * x_ps] = xn;
      h[c * h_cs + i * h_ps] = 0.5 * (xo + xn);
    }
  }
}

// Gather of one particle (grid_deps.f90:169-213 / grid_deps_env.f90:184-234).
// ENV: modes -K..K at index m+K, carrier e^{+i kx0 x}, on-axis phase 1.
template <bool ENV, int NMAX>
__device__ __forceinline__ void gather_one(double xp, double yp, double zp, double leftX,
                                           const double *__restrict__ rgrid, double rmax,
                                           double dx_inv, double dr_inv, double kx0,
                                           const double2 *__restrict__ fld, i64 nx, i64 nr,
                                           int nm, double acc[6]) {
  double rp = sqrt(yp * yp + zp * zp);
#pragma unroll
  for (int l = 0; l < 6; ++l) acc[l] = 0.0;
  if (!(rp < rmax)) return;  // also rejects NaN radii
  double fx = (xp - leftX) * dx_inv;
  if (!(fx > -1.0e15 && fx < 1.0e15)) return;  // non-finite or absurd x
  i64 ix = (i64)floor(fx);
  i64 ir = (i64)floor((rp - rgrid[0]) * dr_inv);
  if (ir < 0 || ir > nr - 2) return;  // rounding at r = Rgrid(nr)
  double sx1 = fx - (double)ix, sx0 = 1.0 - sx1;
  double sr1 = (rp - rgrid[ir]) * dr_inv, sr0 = 1.0 - sr1;
  double2 ph;
  if (rp > 0.0) ph = make_double2(yp / rp, zp / rp);
  else ph = ENV ? make_double2(1.0, 0.0) : make_double2(0.0, 0.0);
  double2 carrier = make_double2(1.0, 0.0);
  if (ENV) {
    double s, c;
    sincos(xp * kx0, &s, &c);
    carrier = make_double2(c, s);
  }
  const bool okx0 = (ix >= 0 && ix < nx);
  const bool okx1 = (ix + 1 >= 0 && ix + 1 < nx);
  const i64 plane = nx * nr;
  const int K = ENV ? (nm - 1) / 2 : 0;
  const int nph = ENV ? K + 1 : nm;
  double2 phm = make_double2(1.0, 0.0);
  for (int mi = 0; mi < nph; ++mi) {
    if (mi > 0) phm = cmul(phm, ph);
    for (int side = 0; side < ((ENV && mi > 0) ? 2 : 1); ++side) {
      double2 pm = side ? cconj(phm) : phm;
      if (ENV) pm = cmul(carrier, pm);
      int slot = ENV ? (side ? K - mi : K + mi) : mi;
      // projcomp(k, j) = S0r(j) * S0x(k) * phase
      double2 w00 = cscale(pm, sr0 * sx0), w01 = cscale(pm, sr0 * sx1);
      double2 w10 = cscale(pm, sr1 * sx0), w11 = cscale(pm, sr1 * sx1);
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        const double2 *b = fld + (i64)(slot + (i64)nm * l) * plane + ir * nx + ix;
        double a = 0.0;
        if (okx0) {
          double2 f0 = b[0], f1 = b[nx];
          a += w00.x * f0.x - w00.y * f0.y;
          a += w10.x * f1.x - w10.y * f1.y;
        }
        if (okx1) {
          double2 f0 = b[1], f1 = b[nx + 1];
          a += w01.x * f0.x - w01.y * f0.y;
          a += w11.x * f1.x - w11.y * f1.y;
        }
        acc[l] += a;
      }
    }
  }
}

template <bool ENV>
__global__ void proj_fld_kernel(const double *__restrict__ x, i64 x_cs, i64 x_ps,
                                const double *__restrict__ w, i64 w_ps,
                                const double2 *__restrict__ fld, double *__restrict__ ft,
                                i64 f_cs, i64 f_ps, double leftX,
                                const double *__restrict__ rgrid, double dx_inv,
                                double dr_inv, double kx0, i64 np, i64 nx, i64 nr, int nm) {
  const double rmax = rgrid[nr - 1];
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < np;
       i += (i64)gridDim.x * blockDim.x) {
    if (w[i * w_ps] == 0.0) continue;
    double acc[6];
    gather_one<ENV, 8>(x[i * x_ps], x[x_cs + i * x_ps], x[2 * x_cs + i * x_ps], leftX, rgrid,
                       rmax, dx_inv, dr_inv, kx0, fld, nx, nr, nm, acc);
#pragma unroll
    for (int l = 0; l < 6; ++l) ft[l * f_cs + i * f_ps] += acc[l];
  }
}

// grid_deps.f90:219-266 / grid_deps_env.f90:240-283.  One thread per
// (ix, ir, m, l); the ghost row is written from row 1 by the row-1 thread.
template <bool ENV>
__global__ void eb_correction_kernel(double2 *__restrict__ eb, i64 nx, i64 nr, int nm) {
  const double pi_inv = 1.0 / kPi, pi2_inv = 0.5 * pi_inv;
  i64 n = nx * (nr - 1) * nm * 6;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < n;
       t += (i64)gridDim.x * blockDim.x) {
    i64 ix = t % nx;
    i64 rest = t / nx;
    i64 r = rest % (nr - 1) + 1;
    i64 ml = rest / (nr - 1);
    int m = (int)(ml % nm);
    double f = (!ENV && m == 0) ? pi2_inv : pi_inv;
    double2 *p = eb + ml * nx * nr;
    double2 v = cscale(p[r * nx + ix], f);
    p[r * nx + ix] = v;
    if (r == 1) {
      double sg;
      if (ENV) sg = (nm == 1) ? 1.0 : -1.0;
      else sg = (m == 0) ? 1.0 : -1.0;
      p[ix] = cscale(v, sg);
    }
  }
}

__device__ __forceinline__ double ramp_ampl(double x, double X0, double Lx, double lam) {
  if (x <= X0 || x >= X0 + Lx) return 0.0;
  if (x > X0 && x < X0 + lam) return (x - X0) / lam;
  if (x > X0 + Lx - lam && x < X0 + Lx) return (X0 + Lx - x) / lam;
  return 1.0;
}

struct DevParams {
  double v[8];
};

// devices.f90:117-203 (undul_analytic[_taper])
template <bool TAPER>
__global__ void undul_analytic_kernel(const double *__restrict__ x, i64 x_cs, i64 x_ps,
                                      double *__restrict__ f, i64 f_cs, i64 f_ps,
                                      DevParams prm, i64 np) {
  const double a0 = prm.v[0], lam = prm.v[1], X0 = prm.v[2], Lx = prm.v[3];
  const double taper = TAPER ? prm.v[4] : 0.0;
  const double ku = 2. * kPi / lam;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < np;
       i += (i64)gridDim.x * blockDim.x) {
    double xp = x[i * x_ps], yp = x[x_cs + i * x_ps];
    double ampl = ramp_ampl(xp, X0, Lx, lam);
    if constexpr (TAPER) ampl = ampl * (1 + taper * (xp - X0 - 0.5 * Lx) / (0.5 * Lx));
    ampl = ampl * a0;
    double s, c;
    sincos(ku * (xp - X0), &s, &c);
    f[4 * f_cs + i * f_ps] += ampl * s * cosh(ku * yp);
    f[3 * f_cs + i * f_ps] += ampl * c * sinh(ku * yp);
  }
}

// devices.f90:18-115 (undul_mapped[_tap])
template <bool TAPER>
__global__ void undul_mapped_kernel(const double *__restrict__ x, i64 x_cs, i64 x_ps,
                                    double *__restrict__ f, i64 f_cs, i64 f_ps,
                                    const double *__restrict__ a0, i64 nmap, DevParams prm,
                                    i64 np) {
  const double lam = prm.v[0], Xleft = prm.v[1], dx = prm.v[2];
  const double Lx = TAPER ? prm.v[3] : 0.0, taper = TAPER ? prm.v[4] : 0.0;
  const double ku = 2. * kPi / lam, dx_inv = 1.0 / dx;
  const double Xright = Xleft + nmap * dx;
  const double x_shift = 0.5 * (nmap * dx - Lx);
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < np;
       i += (i64)gridDim.x * blockDim.x) {
    double xp = x[i * x_ps];
    if (xp < Xleft + dx || xp > Xright - dx) continue;
    double yp = x[x_cs + i * x_ps];
    i64 ix = (i64)floor((xp - Xleft) * dx_inv + 0.5);
    double ddx = (xp - Xleft) * dx_inv - ix;
    double S[3] = {0.5 * (0.5 - ddx) * (0.5 - ddx), 0.75 - ddx * ddx,
                   0.5 * (0.5 + ddx) * (0.5 + ddx)};
    double s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      i64 col = ix - 2 + q;
      if (col < 0 || col >= nmap) continue;
      s1 += S[q] * a0[2 * col];
      s2 += S[q] * a0[2 * col + 1];
    }
    double amp = 1.0;
    if constexpr (TAPER) amp = 1 + taper * (xp - x_shift - Xleft - 0.5 * Lx) / (0.5 * Lx);
    f[4 * f_cs + i * f_ps] += amp * s1 * cosh(ku * yp);
    f[3 * f_cs + i * f_ps] += amp * s2 * sinh(ku * yp);
  }
}

// devices.f90:205-252
__global__ void planewave_kernel(const double *__restrict__ x, i64 x_cs, i64 x_ps,
                                 double *__restrict__ f, i64 f_cs, i64 f_ps, double t,
                                 DevParams prm, i64 np) {
  const double a0 = prm.v[0], lam = prm.v[1], X0 = prm.v[2], Lx = prm.v[3], ramp = prm.v[4],
               theta = prm.v[5], phi0 = prm.v[6];
  double sinth, costh;
  sincos(theta, &sinth, &costh);
  const double k0 = 2. * kPi / lam;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < np;
       i += (i64)gridDim.x * blockDim.x) {
    double xp = x[i * x_ps], yp = x[x_cs + i * x_ps];
    double ampl = ramp_ampl(xp, X0, Lx, ramp);
    ampl = a0 * ampl * sin(k0 * (xp * costh + yp * sinth - t) + phi0);
    f[2 * f_cs + i * f_ps] += ampl;
    f[3 * f_cs + i * f_ps] += ampl * sinth;
    f[4 * f_cs + i * f_ps] -= ampl * costh;
  }
}

// devices.f90:254-297
__global__ void gaussbeam_kernel(const double *__restrict__ x, i64 x_cs, i64 x_ps,
                                 double *__restrict__ f, i64 f_cs, i64 f_ps, double time,
                                 double a0, DevParams prm, i64 np) {
  const double lam = prm.v[0], axis = prm.v[1], x0 = prm.v[2], y0 = prm.v[3], z0 = prm.v[4];
  const double lx2 = 1.0 / (prm.v[5] * prm.v[5]), ly2 = 1.0 / (prm.v[6] * prm.v[6]),
               lz2 = 1.0 / (prm.v[7] * prm.v[7]);
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < np;
       i += (i64)gridDim.x * blockDim.x) {
    double xp = x[i * x_ps] - x0 - axis * time;
    double yp = x[x_cs + i * x_ps] - y0, zp = x[2 * x_cs + i * x_ps] - z0;
    double E = a0 * exp(-xp * xp * lx2 - yp * yp * ly2 - zp * zp * lz2) * sin(2. * kPi / lam * xp);
    f[2 * f_cs + i * f_ps] += E;
    f[4 * f_cs + i * f_ps] -= axis * E;
  }
}

DevParams load_params(const double *host, int n) {
  DevParams p;
  for (int i = 0; i < 8; ++i) p.v[i] = (i < n && host) ? host[i] : 0.0;
  return p;
}

}  // namespace

extern "C" {

int chm_push_velocs(double *momenta, int64_t p_cs, int64_t p_ps, const double *fld, int64_t f_cs,
                    int64_t f_ps, double dt, int64_t np, void *stream) {
  CHM_REQUIRE(np >= 0, "push_velocs: np < 0");
  if (np == 0) return CHM_OK;
  CHM_REQUIRE(momenta && fld, "push_velocs: null pointer");
  push_velocs_kernel<<<grid_for(np, kThreads), kThreads, 0, as_stream(stream)>>>(
      momenta, p_cs, p_ps, fld, f_cs, f_ps, dt, np); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_push_coords(double *coord, int64_t x_cs, int64_t x_ps, const double *momenta,
                    int64_t p_cs, int64_t p_ps, double *coord_cntr, int64_t h_cs, int64_t h_ps,
                    double dt, int64_t np, void *stream) {
  CHM_REQUIRE(np >= 0, "push_coords: np < 0");
  if (np == 0) return CHM_OK;
  CHM_REQUIRE(coord && momenta && coord_cntr, "push_coords: null pointer");
  push_coords_kernel<<<grid_for(np, kThreads), kThreads, 0, as_stream(stream)>>>(
      coord, x_cs, x_ps, momenta, p_cs, p_ps, coord_cntr, h_cs, h_ps, dt, np); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

static int proj_common(bool env, const double *coord, int64_t x_cs, int64_t x_ps,
                       const double *wghts, int64_t w_ps, const chm_c128 *fld, double *fld_tot,
                       int64_t f_cs, int64_t f_ps, double leftX, const double *rgrid,
                       double dx_inv, double dr_inv, double kx0, int64_t np, int64_t nx,
                       int64_t nr, int64_t nm, void *stream) {
  CHM_REQUIRE(np >= 0 && nx > 1 && nr > 1 && nm >= 1, "proj_fld: bad dims");
  CHM_REQUIRE(!env || (nm % 2 == 1), "proj_fld_env: nm must be odd");
  if (np == 0) return CHM_OK;
  CHM_REQUIRE(coord && wghts && fld && fld_tot && rgrid, "proj_fld: null pointer");
  auto k = env ? proj_fld_kernel<true> : proj_fld_kernel<false>;
  k<<<grid_for(np, kThreads), kThreads, 0, as_stream(stream)>>>(
      coord, x_cs, x_ps, wghts, w_ps, reinterpret_cast<const double2 *>(fld), fld_tot, f_cs,
      f_ps, leftX, rgrid, dx_inv, dr_inv, kx0, np, nx, nr, (int)nm); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_proj_fld(const double *coord, int64_t x_cs, int64_t x_ps, const double *wghts,
                 int64_t w_ps, const chm_c128 *fld, double *fld_tot, int64_t f_cs, int64_t f_ps,
                 double leftX, const double *rgrid, double dx_inv, double dr_inv, int64_t np,
                 int64_t nx, int64_t nr, int64_t nm, void *stream) {
  return proj_common(false, coord, x_cs, x_ps, wghts, w_ps, fld, fld_tot, f_cs, f_ps, leftX,
                     rgrid, dx_inv, dr_inv, 0.0, np, nx, nr, nm, stream);
}

int chm_proj_fld_env(const double *coord, int64_t x_cs, int64_t x_ps, const double *wghts,
                     int64_t w_ps, const chm_c128 *fld, double *fld_tot, int64_t f_cs,
                     int64_t f_ps, double leftX, const double *rgrid, double dx_inv,
                     double dr_inv, double kx0, int64_t np, int64_t nx, int64_t nr, int64_t nm,
                     void *stream) {
  return proj_common(true, coord, x_cs, x_ps, wghts, w_ps, fld, fld_tot, f_cs, f_ps, leftX,
                     rgrid, dx_inv, dr_inv, kx0, np, nx, nr, nm, stream);
}

int chm_eb_correction(chm_c128 *eb, int64_t nx, int64_t nr, int64_t nm, void *stream) {
  CHM_REQUIRE(eb && nx > 0 && nr > 1 && nm >= 1, "eb_correction: bad args");
  i64 n = nx * (nr - 1) * nm * 6;
  eb_correction_kernel<false><<<grid_for(n, kThreads), kThreads, 0, as_stream(stream)>>>(
      reinterpret_cast<double2 *>(eb), nx, nr, (int)nm); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_eb_correction_env(chm_c128 *eb, int64_t nx, int64_t nr, int64_t nm, void *stream) {
  CHM_REQUIRE(eb && nx > 0 && nr > 1 && nm >= 1, "eb_correction_env: bad args");
  i64 n = nx * (nr - 1) * nm * 6;
  eb_correction_kernel<true><<<grid_for(n, kThreads), kThreads, 0, as_stream(stream)>>>(
      reinterpret_cast<double2 *>(eb), nx, nr, (int)nm); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_undul_analytic(const double *coord, int64_t x_cs, int64_t x_ps, double *fld,
                       int64_t f_cs, int64_t f_ps, double t, const double *params, int64_t np,
                       void *stream) {
  CHM_REQUIRE(params, "undul_analytic: params (host) is null");
  if (np == 0) return CHM_OK;
  CHM_REQUIRE(params[1] != 0.0, "undul_analytic: lambda_u is zero");
  undul_analytic_kernel<false><<<grid_for(np, kThreads), kThreads, 0, as_stream(stream)>>>(
      coord, x_cs, x_ps, fld, f_cs, f_ps, load_params(params, 4), np); chm::count_launch();
  (void)t;
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_undul_analytic_taper(const double *coord, int64_t x_cs, int64_t x_ps, double *fld,
                             int64_t f_cs, int64_t f_ps, double t, const double *params,
                             int64_t np, void *stream) {
  CHM_REQUIRE(params, "undul_analytic_taper: params (host) is null");
  if (np == 0) return CHM_OK;
  undul_analytic_kernel<true><<<grid_for(np, kThreads), kThreads, 0, as_stream(stream)>>>(
      coord, x_cs, x_ps, fld, f_cs, f_ps, load_params(params, 5), np); chm::count_launch();
  (void)t;
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_undul_mapped(const double *coord, int64_t x_cs, int64_t x_ps, double *fld, int64_t f_cs,
                     int64_t f_ps, double t, const double *a0, int64_t nmap,
                     const double *params, int64_t np, void *stream) {
  CHM_REQUIRE(params && a0 && nmap > 0, "undul_mapped: bad args");
  if (np == 0) return CHM_OK;
  undul_mapped_kernel<false><<<grid_for(np, kThreads), kThreads, 0, as_stream(stream)>>>(
      coord, x_cs, x_ps, fld, f_cs, f_ps, a0, nmap, load_params(params, 3), np); chm::count_launch();
  (void)t;
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_undul_mapped_tap(const double *coord, int64_t x_cs, int64_t x_ps, double *fld,
                         int64_t f_cs, int64_t f_ps, double t, const double *a0, int64_t nmap,
                         const double *params, int64_t np, void *stream) {
  CHM_REQUIRE(params && a0 && nmap > 0, "undul_mapped_tap: bad args");
  if (np == 0) return CHM_OK;
  undul_mapped_kernel<true><<<grid_for(np, kThreads), kThreads, 0, as_stream(stream)>>>(
      coord, x_cs, x_ps, fld, f_cs, f_ps, a0, nmap, load_params(params, 5), np); chm::count_launch();
  (void)t;
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_planewave(const double *coord, int64_t x_cs, int64_t x_ps, double *fld, int64_t f_cs,
                  int64_t f_ps, double t, const double *params, int64_t np, void *stream) {
  CHM_REQUIRE(params, "planewave: params (host) is null");
  if (np == 0) return CHM_OK;
  planewave_kernel<<<grid_for(np, kThreads), kThreads, 0, as_stream(stream)>>>(
      coord, x_cs, x_ps, fld, f_cs, f_ps, t, load_params(params, 7), np); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_gaussbeam(const double *coord, int64_t x_cs, int64_t x_ps, double *fld, int64_t f_cs,
                  int64_t f_ps, double time, double a0, const double *params, int64_t np,
                  void *stream) {
  CHM_REQUIRE(params, "gaussbeam: params (host) is null");
  if (np == 0) return CHM_OK;
  gaussbeam_kernel<<<grid_for(np, kThreads), kThreads, 0, as_stream(stream)>>>(
      coord, x_cs, x_ps, fld, f_cs, f_ps, time, a0, load_params(params, 8), np); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"
