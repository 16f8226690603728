/*
 * chimera_oracle.c -- CPU FP64 restatement of CHIMERA's per-step PIC kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA library is
 * checked against.  It is never linked into, loaded by or called from the
 * product (chimera_gb300/); only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py load it, and only as the checker / the timed
 * CPU baseline.
 *
 * Every routine restates one Fortran subroutine of the reference (cited by
 * file:line) in plain C99 + OpenMP, with the same argument meaning, the same
 * column-major (Fortran) array layout and the same loop / summation order, so
 * that FP64 results agree to round-off.  Complex arrays are interleaved
 * {re, im} doubles (numpy complex128).  Dimensions that f2py hides are passed
 * explicitly as array extents:
 *   NX  = number of x nodes          (Fortran 0:nx  -> NX = nx+1)
 *   NR  = number of r rows incl. the ghost row at r=-dr/2 (Fortran 0:nr)
 *   NM  = number of stored azimuthal modes (0:nkO -> NM = nkO+1, or
 *         -nkO:nkO -> NM = 2 nkO + 1 for the envelope solver)
 *   NKR = number of spectral radial modes.
 *
 * Deliberate, documented differences from the Fortran (only where the Fortran
 * is undefined behaviour):
 *   - grid deposits/gathers drop stencil nodes with an x index outside
 *     [0, NX-1] (the Fortran writes/reads neighbouring memory there);
 *   - the chunked deposits add the right guard buffers after all chunks have
 *     finished (the Fortran adds them before its barrier, racing with the
 *     neighbouring chunk's direct deposits);
 *   - fb_rot/fb_grad/fb_div with a single stored mode treat the absent m=1
 *     mode as zero (the Fortran reads past the array);
 *   - fb_filtr modes 1/2 filter the last nxfilt cells (the Fortran's array
 *     sections there are non-conformable).
 * The x-FFT is our own mixed-radix DFT (the reference calls FFTW3); both are
 * the unnormalised DFT with sign -1 (forward) / +1 (backward).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;
typedef long long i64;

#define II (_Complex_I)

static const double PI = 3.14159265358979323846264338327950288;

/* ------------------------------------------------------------------------ */
/* Mixed-radix FFT (decimation in time, recursive, one twiddle table).       */
/* ------------------------------------------------------------------------ */
typedef struct {
  int n;
  int nf;
  int fac[64];
  cplx *tw; /* tw[j] = exp(sign*2*pi*i*j/n) */
  int sign;
} fft_plan;

static void fft_plan_init(fft_plan *p, int n, int sign) {
  p->n = n;
  p->sign = sign;
  p->nf = 0;
  int m = n, f = 4;
  while (m > 1) {
    while (m % f) {
      if (f == 4) f = 2;
      else if (f == 2) f = 3;
      else f += 2;
      if (f * f > m) f = m;
    }
    p->fac[p->nf++] = f;
    m /= f;
  }
  p->tw = (cplx *)malloc(sizeof(cplx) * (size_t)(n > 0 ? n : 1));
  for (int j = 0; j < n; ++j) {
    double a = sign * 2.0 * PI * (double)j / (double)n;
    p->tw[j] = cos(a) + II * sin(a);
  }
}

static void fft_plan_free(fft_plan *p) { free(p->tw); }

static void fft_rec(const fft_plan *p, cplx *out, const cplx *in, int n,
                    i64 istride, int fi, int twstride, cplx *scratch) {
  if (n == 1) {
    out[0] = in[0];
    return;
  }
  int r = p->fac[fi];
  int m = n / r;
  for (int q = 0; q < r; ++q)
    fft_rec(p, out + q * m, in + q * istride, m, istride * r, fi + 1,
            twstride * r, scratch);
  /* butterflies: out[k + s m] = sum_q out[k + q m] w_n^{q k} w_r^{q s} */
  for (int k = 0; k < m; ++k) {
    for (int q = 0; q < r; ++q)
      scratch[q] = out[k + q * m] * p->tw[((i64)q * k * twstride) % p->n];
    for (int s = 0; s < r; ++s) {
      cplx acc = 0.0;
      for (int q = 0; q < r; ++q)
        acc += scratch[q] * p->tw[(((i64)q * s) % r) * (p->n / r)];
      out[k + s * m] = acc;
    }
  }
}

/* out = DFT(in), length p->n, contiguous; in and out must not alias */
static void fft_exec(const fft_plan *p, const cplx *in, cplx *out,
                     cplx *scratch) {
  fft_rec(p, out, in, p->n, 1, 0, 1, scratch);
}

/* exported for the oracle's own FFT test against numpy */
void orc_fft(const cplx *in, cplx *out, i64 n, int sign) {
  fft_plan p;
  fft_plan_init(&p, (int)n, sign);
  cplx *scr = (cplx *)malloc(sizeof(cplx) * (size_t)n);
  fft_exec(&p, in, out, scr);
  free(scr);
  fft_plan_free(&p);
}

/* ------------------------------------------------------------------------ */
/* particle_tools.f90                                                        */
/* ------------------------------------------------------------------------ */

/* particle_tools.f90:18-56 (push_velocs): Boris rotation with two half
 * E-kicks.  momenta(3,np), Fld(6,np) = (Ex,Ey,Ez,Bx,By,Bz). */
void orc_push_velocs(double *momenta, const double *fld, double dt, i64 np) {
  const double dt_2 = 0.5 * dt;
#pragma omp parallel for schedule(static)
  for (i64 ip = 0; ip < np; ++ip) {
    const double *F = fld + 6 * ip;
    double *P = momenta + 3 * ip;
    double um[3], t[3], s[3], u0[3], up[3];
    for (int c = 0; c < 3; ++c) um[c] = P[c] + dt_2 * F[c];
    double gamma = sqrt(1.0 + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]));
    for (int c = 0; c < 3; ++c) t[c] = dt_2 * F[3 + c] / gamma;
    double t2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
    for (int c = 0; c < 3; ++c) s[c] = 2 * t[c] / (1 + t2);
    u0[0] = um[0] + um[1] * t[2] - um[2] * t[1];
    u0[1] = um[1] - um[0] * t[2] + um[2] * t[0];
    u0[2] = um[2] + um[0] * t[1] - um[1] * t[0];
    up[0] = um[0] + u0[1] * s[2] - u0[2] * s[1];
    up[1] = um[1] - u0[0] * s[2] + u0[2] * s[0];
    up[2] = um[2] + u0[0] * s[1] - u0[1] * s[0];
    for (int c = 0; c < 3; ++c) P[c] = up[c] + dt_2 * F[c];
  }
}

/* particle_tools.f90:58-82 (push_coords): leap-frog coordinate push; the
 * half-step coordinates are the mean of the old and new positions. */
void orc_push_coords(double *coord, const double *momenta, double *coord_cntr,
                     double dt, i64 np) {
#pragma omp parallel for schedule(static)
  for (i64 ip = 0; ip < np; ++ip) {
    double *X = coord + 3 * ip;
    const double *P = momenta + 3 * ip;
    double *XC = coord_cntr + 3 * ip;
    double dt_gp = dt / sqrt(1.0 + (P[0] * P[0] + P[1] * P[1] + P[2] * P[2]));
    for (int c = 0; c < 3; ++c) {
      double xo = X[c];
      double xn = xo + P[c] * dt_gp;
      X[c] = xn;
      XC[c] = 0.5 * (xo + xn);
    }
  }
}

/* particle_tools.f90:84-128 (genparts): fill cells with the fixed per-cell
 * pattern (PackX, PackR, PackO) rotated by a random angle per cell.
 * coord(4,np) out; returns the number of particles written. */
i64 orc_genparts(double *coord, i64 np, const double *xgrid, i64 nx,
                 const double *rgrid, i64 nr, const double *randpacko,
                 const double *packx, const double *packr, const cplx *packo,
                 i64 ppc) {
  memset(coord, 0, sizeof(double) * 4 * (size_t)np);
  double dr_2 = 0.5 * (rgrid[1] - rgrid[0]);
  i64 ind = 0;
  for (i64 ir = 0; ir < nr - 1; ++ir) {
    for (i64 ix = 0; ix < nx - 1; ++ix) {
      double r0 = rgrid[ir] + dr_2, r1 = rgrid[ir + 1] + dr_2;
      double x0 = xgrid[ix], x1 = xgrid[ix + 1];
      double osh = 2.0 * PI * randpacko[ix + nx * ir];
      cplx oshft = cos(osh) + II * sin(osh);
      for (i64 ip = 0; ip < ppc; ++ip) {
        double cx = x0 + (x1 - x0) * packx[ip];
        double cr = r0 + (r1 - r0) * packr[ip];
        cplx oc = packo[ip] * oshft;
        if (cr <= 0) continue;
        if (ind >= np) return -1;
        coord[4 * ind + 0] = cx;
        coord[4 * ind + 1] = cr * cimag(oc);
        coord[4 * ind + 2] = cr * creal(oc);
        coord[4 * ind + 3] = cr;
        ++ind;
      }
    }
  }
  return ind;
}

/* particle_tools.f90:130-153 (sortpartsout): indices (0-based) of particles
 * inside lims = (xmin, xmax, r2min, r2max); returns their number. */
i64 orc_sortpartsout(i64 *indx2stay, const double *coord, const double *lims,
                     i64 np) {
  i64 n = 0;
  for (i64 ip = 0; ip < np; ++ip) indx2stay[ip] = 0;
  for (i64 ip = 0; ip < np; ++ip) {
    double x = coord[3 * ip];
    double r2 = coord[3 * ip + 1] * coord[3 * ip + 1] +
                coord[3 * ip + 2] * coord[3 * ip + 2];
    if (x >= lims[0] && x <= lims[1] && r2 >= lims[2] && r2 <= lims[3])
      indx2stay[n++] = ip;
  }
  return n;
}

/* particle_tools.f90:155-208 (chunk_coords_boundaries): x-chunk id per
 * particle (int8, -2 for particles leaving lims), chunk offsets
 * IndInChnk(0:nchnk) and the number of leaving particles. */
i64 orc_chunk_coords_boundaries(signed char *chunked_indx, int *indinchnk,
                                const double *coord, const double *lims,
                                const double *xgrid, i64 nxg, i64 nchnk,
                                i64 np) {
  /* xgrid has nxg entries: Fortran Xgrid(0:nx) with nx = nxg-1 */
  i64 nx = nxg - 1;
  double cl_inv;
  if (nchnk > 1)
    cl_inv = 1. / (xgrid[(nx + 1) / nchnk] - xgrid[0]);
  else
    cl_inv = 1. / (xgrid[nx] - xgrid[0]);
  i64 *num = (i64 *)calloc((size_t)nchnk, sizeof(i64));
  i64 goout = 0;
  for (i64 ip = 0; ip < np; ++ip) {
    chunked_indx[ip] = -2;
    i64 ich = (i64)floor((coord[3 * ip] - xgrid[0]) * cl_inv);
    double x = coord[3 * ip];
    double r2 = coord[3 * ip + 1] * coord[3 * ip + 1] +
                coord[3 * ip + 2] * coord[3 * ip + 2];
    if (x >= lims[0] && x <= lims[1] && r2 >= lims[2] && r2 <= lims[3]) {
      if (ich >= 0 && ich < nchnk) num[ich] += 1;
      chunked_indx[ip] = (signed char)ich;
    } else {
      goout += 1;
    }
  }
  indinchnk[0] = 0;
  for (i64 c = 0; c < nchnk; ++c) indinchnk[c + 1] = indinchnk[c] + (int)num[c];
  free(num);
  return goout;
}

/* particle_tools.f90:270-324 (align_data_vec / align_data_scl): gather
 * dat(:, idx(ip)) into the first np slots, in place. */
void orc_align_data(double *dat, i64 ncomp, const i64 *idx, i64 np) {
  double *tmp = (double *)malloc(sizeof(double) * (size_t)(ncomp * np + 1));
#pragma omp parallel for schedule(static)
  for (i64 ip = 0; ip < np; ++ip)
    for (i64 c = 0; c < ncomp; ++c) tmp[ncomp * ip + c] = dat[ncomp * idx[ip] + c];
  memcpy(dat, tmp, sizeof(double) * (size_t)(ncomp * np));
  free(tmp);
}

/* ------------------------------------------------------------------------ */
/* grid_deps.f90 / grid_deps_chnk.f90 / grid_deps_env*.f90                   */
/* ------------------------------------------------------------------------ */

/* Common per-particle stencil: cell (ix, ir), linear weights S0(k,1) in x and
 * S0(k,2) in r (r nodes at Rgrid), grid_deps.f90:46-53. */
typedef struct {
  i64 ix, ir;
  double sx[2], sr[2];
} stencil_t;

static inline stencil_t make_stencil(double xp, double rp, double leftX,
                                     const double *rgrid, double dx_inv,
                                     double dr_inv) {
  stencil_t s;
  s.ix = (i64)floor((xp - leftX) * dx_inv);
  s.ir = (i64)floor((rp - rgrid[0]) * dr_inv);
  s.sx[1] = (xp - leftX) * dx_inv - (double)s.ix;
  s.sx[0] = 1.0 - s.sx[1];
  s.sr[1] = (rp - rgrid[s.ir]) * dr_inv;
  s.sr[0] = 1.0 - s.sr[1];
  return s;
}

/* ghost-row fold grid_deps.f90:80-84 / :144-145 for ncomp planes */
static void ghost_fold(cplx *a, i64 NX, i64 NR, i64 NM, i64 ncomp) {
  for (i64 l = 0; l < ncomp; ++l)
    for (i64 m = 0; m < NM; ++m) {
      cplx *p = a + NX * NR * (m + NM * l);
      for (i64 ix = 0; ix < NX; ++ix) {
        p[ix + NX] = p[ix + NX] - p[ix];
        p[ix] = 0.0;
      }
    }
}

/* Deposit of one particle's complex contribution val * S0x(k) * S0r(j) into
 * plane `pl` (one mode, one component), dropping x-nodes outside the grid. */
static inline void dep_node2x2(cplx *pl, i64 NX, const stencil_t *s, cplx val) {
  for (int j = 0; j < 2; ++j)
    for (int k = 0; k < 2; ++k) {
      i64 gx = s->ix + k;
      if (gx < 0 || gx >= NX) continue;
      pl[gx + NX * (s->ir + j)] += val * (s->sx[k] * s->sr[j]);
    }
}

/* grid_deps.f90:18-87 (dep_curr): serial current deposit,
 * curr(NX,NR,NM,3) += w v/gamma S e^{-i m theta}, then the ghost fold. */
void orc_dep_curr(const double *coord, const double *momenta,
                  const double *wghts, cplx *curr, double leftX,
                  const double *rgrid, double dx_inv, double dr_inv, i64 np,
                  i64 NX, i64 NR, i64 NM) {
  double rmax = rgrid[NR - 1];
  cplx *phaseO = (cplx *)malloc(sizeof(cplx) * (size_t)NM);
  for (i64 ip = 0; ip < np; ++ip) {
    double wp = wghts[ip];
    if (wp == 0.0) continue;
    double xp = coord[3 * ip], yp = coord[3 * ip + 1], zp = coord[3 * ip + 2];
    double v[3] = {momenta[3 * ip], momenta[3 * ip + 1], momenta[3 * ip + 2]};
    double rp = sqrt(yp * yp + zp * zp);
    if (rp >= rmax || (fabs(v[0]) + fabs(v[1]) + fabs(v[2])) == 0.0) continue;
    double gp = sqrt(1 + v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int c = 0; c < 3; ++c) v[c] = v[c] * wp / gp;
    stencil_t s = make_stencil(xp, rp, leftX, rgrid, dx_inv, dr_inv);
    cplx phase_m = (rp > 0.0) ? (yp - II * zp) / rp : 0.0;
    phaseO[0] = 1.0;
    for (i64 m = 1; m < NM; ++m) phaseO[m] = phaseO[m - 1] * phase_m;
    for (int l = 0; l < 3; ++l)
      for (i64 m = 0; m < NM; ++m)
        dep_node2x2(curr + NX * NR * (m + NM * l), NX, &s, phaseO[m] * v[l]);
  }
  free(phaseO);
  ghost_fold(curr, NX, NR, NM, 3);
}

/* grid_deps.f90:89-147 (dep_dens): serial density deposit + ghost fold. */
void orc_dep_dens(const double *coord, const double *wghts, cplx *dens,
                  double leftX, const double *rgrid, double dx_inv,
                  double dr_inv, i64 np, i64 NX, i64 NR, i64 NM) {
  double rmax = rgrid[NR - 1];
  cplx *phaseO = (cplx *)malloc(sizeof(cplx) * (size_t)NM);
  for (i64 ip = 0; ip < np; ++ip) {
    double wp = wghts[ip];
    if (wp == 0.0) continue;
    double xp = coord[3 * ip], yp = coord[3 * ip + 1], zp = coord[3 * ip + 2];
    double rp = sqrt(yp * yp + zp * zp);
    if (rp >= rmax) continue;
    stencil_t s = make_stencil(xp, rp, leftX, rgrid, dx_inv, dr_inv);
    cplx phase_m = (rp > 0.0) ? (yp - II * zp) / rp : 0.0;
    phaseO[0] = 1.0;
    for (i64 m = 1; m < NM; ++m) phaseO[m] = phaseO[m - 1] * phase_m;
    for (i64 m = 0; m < NM; ++m)
      dep_node2x2(dens + NX * NR * m, NX, &s, phaseO[m] * wp);
  }
  free(phaseO);
  ghost_fold(dens, NX, NR, NM, 1);
}

/* Envelope deposits (grid_deps_env.f90:18-95, :97-162).  Modes -K..K stored
 * at index m + K.  The carrier phase e^{-i kx0 x} multiplies the weight.  Only
 * the third current component is deposited (grid_deps_env.f90:76), and the
 * density weight is applied twice (grid_deps_env.f90:145-147). */
void orc_dep_curr_env(const double *coord, const double *momenta,
                      const double *wghts, cplx *curr, double leftX,
                      const double *rgrid, double dx_inv, double dr_inv,
                      double kx0, i64 np, i64 NX, i64 NR, i64 NM) {
  i64 K = (NM - 1) / 2;
  double rmax = rgrid[NR - 1];
  cplx *phaseO = (cplx *)malloc(sizeof(cplx) * (size_t)(K + 1));
  for (i64 ip = 0; ip < np; ++ip) {
    if (wghts[ip] == 0.0) continue;
    double xp = coord[3 * ip], yp = coord[3 * ip + 1], zp = coord[3 * ip + 2];
    double v[3] = {momenta[3 * ip], momenta[3 * ip + 1], momenta[3 * ip + 2]};
    double rp = sqrt(yp * yp + zp * zp);
    if (rp >= rmax || (fabs(v[0]) + fabs(v[1]) + fabs(v[2])) == 0.0) continue;
    double gp = sqrt(1.0 + v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int c = 0; c < 3; ++c) v[c] = v[c] / gp;
    cplx wp = wghts[ip] * (cos(xp * kx0) - II * sin(xp * kx0));
    stencil_t s = make_stencil(xp, rp, leftX, rgrid, dx_inv, dr_inv);
    cplx phase_m = (rp > 0.0) ? (yp - II * zp) / rp : 0.0;
    phaseO[0] = 1.0;
    for (i64 m = 1; m <= K; ++m) phaseO[m] = phaseO[m - 1] * phase_m;
    int l = 2;
    for (i64 m = 0; m <= K; ++m) {
      dep_node2x2(curr + NX * NR * ((m + K) + NM * l), NX, &s,
                  phaseO[m] * v[l] * wp);
      if (m > 0)
        dep_node2x2(curr + NX * NR * ((K - m) + NM * l), NX, &s,
                    conj(phaseO[m]) * v[l] * wp);
    }
  }
  free(phaseO);
  ghost_fold(curr, NX, NR, NM, 3);
}

void orc_dep_dens_env(const double *coord, const double *wghts, cplx *dens,
                      double leftX, const double *rgrid, double dx_inv,
                      double dr_inv, double kx0, i64 np, i64 NX, i64 NR,
                      i64 NM) {
  i64 K = (NM - 1) / 2;
  double rmax = rgrid[NR - 1];
  cplx *phaseO = (cplx *)malloc(sizeof(cplx) * (size_t)(K + 1));
  for (i64 ip = 0; ip < np; ++ip) {
    if (wghts[ip] == 0.0) continue;
    double xp = coord[3 * ip], yp = coord[3 * ip + 1], zp = coord[3 * ip + 2];
    double rp = sqrt(yp * yp + zp * zp);
    if (rp >= rmax) continue;
    cplx wp = wghts[ip] * (cos(xp * kx0) - II * sin(xp * kx0));
    stencil_t s = make_stencil(xp, rp, leftX, rgrid, dx_inv, dr_inv);
    cplx phase_m = (rp > 0.0) ? (yp - II * zp) / rp : 0.0;
    phaseO[0] = 1.0;
    for (i64 m = 1; m <= K; ++m) phaseO[m] = phaseO[m - 1] * phase_m;
    cplx ww = wp * wp;
    for (i64 m = 0; m <= K; ++m) {
      dep_node2x2(dens + NX * NR * (m + K), NX, &s, phaseO[m] * ww);
      if (m > 0)
        dep_node2x2(dens + NX * NR * (K - m), NX, &s, conj(phaseO[m]) * ww);
    }
  }
  free(phaseO);
  ghost_fold(dens, NX, NR, NM, 1);
}

/* Chunked deposits (grid_deps_chnk.f90:18-234, grid_deps_env_chnk.f90:18-261):
 * chunk c = [IndInChunk[c], IndInChunk[c+1]) is deposited by one thread into
 * the grid directly, except for x-nodes at local index <= 0 (left guard
 * buffer) or >= chunk_size (right guard buffer).  Right buffers are added for
 * every chunk whose buffer lies inside the grid, left buffers for every chunk
 * but the first: contributions of chunk 0 to x-node 0 are dropped, as in the
 * Fortran.  kind: 0 = curr, 1 = dens, 2 = curr_env, 3 = dens_env. */
static void dep_chnk_generic(int kind, const double *coord,
                             const double *momenta, const double *wghts,
                             cplx *grid, const int *indinchunk, i64 nchnk,
                             i64 guards, double leftX, const double *rgrid,
                             double dx_inv, double dr_inv, double kx0, i64 NX,
                             i64 NR, i64 NM) {
  int env = (kind >= 2);
  int is_curr = (kind == 0 || kind == 2);
  i64 ncomp = is_curr ? 3 : 1;
  i64 K = env ? (NM - 1) / 2 : 0;
  i64 nphase = env ? K + 1 : NM;
  i64 cs = NX / nchnk;
  i64 gw = guards + 1; /* guard buffer width */
  double rmax = rgrid[NR - 1];
  size_t bufsz = (size_t)(gw * NR * NM * ncomp);
  cplx *left = (cplx *)calloc(bufsz * (size_t)nchnk, sizeof(cplx));
  cplx *right = (cplx *)calloc(bufsz * (size_t)nchnk, sizeof(cplx));
#pragma omp parallel for schedule(static, 1) num_threads((int)nchnk)
  for (i64 ich = 0; ich < nchnk; ++ich) {
    cplx *phaseO = (cplx *)malloc(sizeof(cplx) * (size_t)nphase);
    cplx *lb = left + bufsz * (size_t)ich, *rb = right + bufsz * (size_t)ich;
    i64 nxleft = ich * cs;
    for (i64 ip = indinchunk[ich]; ip < indinchunk[ich + 1]; ++ip) {
      if (wghts[ip] == 0.0) continue;
      double xp = coord[3 * ip], yp = coord[3 * ip + 1], zp = coord[3 * ip + 2];
      double rp = sqrt(yp * yp + zp * zp);
      double v[3] = {0, 0, 0};
      if (is_curr) {
        v[0] = momenta[3 * ip];
        v[1] = momenta[3 * ip + 1];
        v[2] = momenta[3 * ip + 2];
        if (rp >= rmax || (fabs(v[0]) + fabs(v[1]) + fabs(v[2])) == 0.0)
          continue;
      } else if (rp >= rmax) {
        continue;
      }
      cplx wp;
      if (env)
        wp = wghts[ip] * (cos(xp * kx0) - II * sin(xp * kx0));
      else
        wp = wghts[ip];
      if (is_curr) {
        double gp = sqrt(1.0 + v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int c = 0; c < 3; ++c) v[c] = env ? v[c] / gp : v[c] * creal(wp) / gp;
      }
      stencil_t s = make_stencil(xp, rp, leftX, rgrid, dx_inv, dr_inv);
      i64 ixl = s.ix - nxleft;
      cplx phase_m = (rp > 0.0) ? (yp - II * zp) / rp : 0.0;
      phaseO[0] = 1.0;
      for (i64 m = 1; m < nphase; ++m) phaseO[m] = phaseO[m - 1] * phase_m;
      for (i64 l = 0; l < ncomp; ++l) {
        if (kind == 2 && l != 2) continue; /* grid_deps_env_chnk.f90:92 */
        for (i64 mi = 0; mi < nphase; ++mi) {
          for (int side = 0; side < (env && mi > 0 ? 2 : 1); ++side) {
            cplx ph = side ? conj(phaseO[mi]) : phaseO[mi];
            i64 mslot = env ? (side ? K - mi : K + mi) : mi;
            cplx val;
            if (kind == 0) val = ph * v[l];
            else if (kind == 1) val = ph * wp;
            else if (kind == 2) val = ph * v[l] * wp;
            else val = ph * wp * wp;
            for (int k = 0; k < 2; ++k) {
              i64 lx = ixl + k;
              for (int j = 0; j < 2; ++j) {
                cplx add = val * (s.sx[k] * s.sr[j]);
                i64 rr = s.ir + j;
                if (lx <= 0) {
                  i64 b = lx + guards; /* -guards..0 -> 0..guards */
                  if (b < 0) continue;
                  lb[b + gw * (rr + NR * (mslot + NM * l))] += add;
                } else if (lx >= cs) {
                  i64 b = lx - cs;
                  if (b > guards) continue;
                  rb[b + gw * (rr + NR * (mslot + NM * l))] += add;
                } else {
                  grid[(nxleft + lx) + NX * (rr + NR * (mslot + NM * l))] += add;
                }
              }
            }
          }
        }
      }
    }
    free(phaseO);
  }
  /* right guards (grid_deps_chnk.f90:110-113), then left guards (:115-118) */
  for (int pass = 0; pass < 2; ++pass)
    for (i64 ich = 0; ich < nchnk; ++ich) {
      i64 nxleft = ich * cs;
      i64 x0 = pass == 0 ? nxleft + cs : nxleft - guards;
      int ok = pass == 0 ? (nxleft + cs + guards <= NX - 1) : (nxleft - guards >= 0);
      if (!ok) continue;
      cplx *b = (pass == 0 ? right : left) + bufsz * (size_t)ich;
      for (i64 l = 0; l < ncomp; ++l)
        for (i64 m = 0; m < NM; ++m)
          for (i64 r = 0; r < NR; ++r)
            for (i64 g = 0; g < gw; ++g)
              grid[(x0 + g) + NX * (r + NR * (m + NM * l))] +=
                  b[g + gw * (r + NR * (m + NM * l))];
    }
  free(left);
  free(right);
  ghost_fold(grid, NX, NR, NM, ncomp);
}

void orc_dep_curr_chnk(const double *coord, const double *momenta,
                       const double *wghts, cplx *curr, const int *indinchunk,
                       i64 nchnk, i64 guards, double leftX, const double *rgrid,
                       double dx_inv, double dr_inv, i64 NX, i64 NR, i64 NM) {
  dep_chnk_generic(0, coord, momenta, wghts, curr, indinchunk, nchnk, guards,
                   leftX, rgrid, dx_inv, dr_inv, 0.0, NX, NR, NM);
}
void orc_dep_dens_chnk(const double *coord, const double *wghts, cplx *dens,
                       const int *indinchunk, i64 nchnk, i64 guards,
                       double leftX, const double *rgrid, double dx_inv,
                       double dr_inv, i64 NX, i64 NR, i64 NM) {
  dep_chnk_generic(1, coord, NULL, wghts, dens, indinchunk, nchnk, guards,
                   leftX, rgrid, dx_inv, dr_inv, 0.0, NX, NR, NM);
}
void orc_dep_curr_env_chnk(const double *coord, const double *momenta,
                           const double *wghts, cplx *curr,
                           const int *indinchunk, i64 nchnk, i64 guards,
                           double leftX, const double *rgrid, double dx_inv,
                           double dr_inv, double kx0, i64 NX, i64 NR, i64 NM) {
  dep_chnk_generic(2, coord, momenta, wghts, curr, indinchunk, nchnk, guards,
                   leftX, rgrid, dx_inv, dr_inv, kx0, NX, NR, NM);
}
void orc_dep_dens_env_chnk(const double *coord, const double *wghts,
                           cplx *dens, const int *indinchunk, i64 nchnk,
                           i64 guards, double leftX, const double *rgrid,
                           double dx_inv, double dr_inv, double kx0, i64 NX,
                           i64 NR, i64 NM) {
  dep_chnk_generic(3, coord, NULL, wghts, dens, indinchunk, nchnk, guards,
                   leftX, rgrid, dx_inv, dr_inv, kx0, NX, NR, NM);
}

/* grid_deps.f90:149-217 (proj_fld) and grid_deps_env.f90:164-238
 * (proj_fld_env): gather Re(sum_m S e^{+i m theta} F_m) for 6 components and
 * add it to Fld_tot(6,np).  On axis the phase is 0 (plain) / 1 (env). */
void orc_proj_fld(const double *coord, const double *wghts, const cplx *fld,
                  double *fld_tot, double leftX, const double *rgrid,
                  double dx_inv, double dr_inv, i64 np, i64 NX, i64 NR,
                  i64 NM) {
  double rmax = rgrid[NR - 1];
#pragma omp parallel
  {
    cplx *phaseO = (cplx *)malloc(sizeof(cplx) * (size_t)NM);
#pragma omp for schedule(static)
    for (i64 ip = 0; ip < np; ++ip) {
      if (wghts[ip] == 0.0) continue;
      double xp = coord[3 * ip], yp = coord[3 * ip + 1], zp = coord[3 * ip + 2];
      double rp = sqrt(yp * yp + zp * zp);
      if (rp >= rmax) continue;
      stencil_t s = make_stencil(xp, rp, leftX, rgrid, dx_inv, dr_inv);
      cplx phase_p = (rp > 0.0) ? (yp + II * zp) / rp : 0.0;
      phaseO[0] = 1.0;
      for (i64 m = 1; m < NM; ++m) phaseO[m] = phaseO[m - 1] * phase_p;
      for (int l = 0; l < 6; ++l) {
        double acc = 0.0;
        for (i64 m = 0; m < NM; ++m)
          for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 2; ++k) {
              i64 gx = s.ix + k;
              if (gx < 0 || gx >= NX) continue;
              cplx pc = (s.sr[j] * s.sx[k]) * phaseO[m];
              acc += creal(pc * fld[gx + NX * ((s.ir + j) + NR * (m + NM * l))]);
            }
        fld_tot[6 * ip + l] += acc;
      }
    }
    free(phaseO);
  }
}

void orc_proj_fld_env(const double *coord, const double *wghts,
                      const cplx *fld, double *fld_tot, double leftX,
                      const double *rgrid, double dx_inv, double dr_inv,
                      double kx0, i64 np, i64 NX, i64 NR, i64 NM) {
  i64 K = (NM - 1) / 2;
  double rmax = rgrid[NR - 1];
#pragma omp parallel
  {
    cplx *phaseO = (cplx *)malloc(sizeof(cplx) * (size_t)(K + 1));
#pragma omp for schedule(static)
    for (i64 ip = 0; ip < np; ++ip) {
      if (wghts[ip] == 0.0) continue;
      double xp = coord[3 * ip], yp = coord[3 * ip + 1], zp = coord[3 * ip + 2];
      double rp = sqrt(yp * yp + zp * zp);
      if (rp >= rmax) continue;
      stencil_t s = make_stencil(xp, rp, leftX, rgrid, dx_inv, dr_inv);
      cplx phase_p = (rp > 0.0) ? (yp + II * zp) / rp : 1.0;
      phaseO[0] = 1.0;
      for (i64 m = 1; m <= K; ++m) phaseO[m] = phaseO[m - 1] * phase_p;
      cplx carrier = cos(xp * kx0) + II * sin(xp * kx0);
      double acc[6] = {0, 0, 0, 0, 0, 0};
      for (i64 m = 0; m <= K; ++m)
        for (int side = 0; side < (m > 0 ? 2 : 1); ++side) {
          cplx ph = side ? conj(phaseO[m]) : phaseO[m];
          i64 ms = side ? K - m : K + m;
          for (int l = 0; l < 6; ++l)
            for (int j = 0; j < 2; ++j)
              for (int k = 0; k < 2; ++k) {
                i64 gx = s.ix + k;
                if (gx < 0 || gx >= NX) continue;
                cplx pc = (s.sr[j] * s.sx[k]) * carrier * ph;
                acc[l] += creal(pc * fld[gx + NX * ((s.ir + j) + NR * (ms + NM * l))]);
              }
        }
      for (int l = 0; l < 6; ++l) fld_tot[6 * ip + l] += acc[l];
    }
    free(phaseO);
  }
}

/* grid_deps.f90:219-266 (eb_correction): m=0 scaled by 1/(2 pi), m>0 by
 * 1/pi; ghost row 0 = +row 1 (m=0) or -row 1 (m>0).
 * grid_deps_env.f90:240-283 (eb_correction_env): all modes by 1/pi; ghost
 * row = +row 1 if a single mode is stored, else -row 1 for every mode. */
void orc_eb_correction(cplx *eb, i64 NX, i64 NR, i64 NM, int env) {
  double pi_inv = 1. / PI, pi2_inv = 0.5 * pi_inv;
  for (i64 l = 0; l < 6; ++l)
    for (i64 m = 0; m < NM; ++m) {
      cplx *p = eb + NX * NR * (m + NM * l);
      double f = (!env && m == 0) ? pi2_inv : pi_inv;
      for (i64 i = 0; i < NX * NR; ++i) p[i] = f * p[i];
      double sg;
      if (env) sg = (NM == 1) ? 1.0 : -1.0;
      else sg = (m == 0) ? 1.0 : -1.0;
      for (i64 ix = 0; ix < NX; ++ix) p[ix] = sg * p[ix + NX];
    }
}

/* ------------------------------------------------------------------------ */
/* fb_io.f90                                                                 */
/* ------------------------------------------------------------------------ */

/* fb_io.f90:18-98 (fb_vec_in / fb_scl_in): for every component, mode and
 * spectral radial index k: A(x) = sum_{r=1..NR-1} In(r,k,m) v(x,r,m); then the
 * forward FFT along x, times e^{-i kx leftX}.  v(NX,NR,NM,ncomp),
 * In(NR-1,NKR,NM), out(NX,NKR,NM,ncomp). */
void orc_fb_in(cplx *out, const cplx *v, double leftX, const double *kx,
               const double *In, i64 NX, i64 NR, i64 NM, i64 NKR, i64 ncomp) {
  i64 nr = NR - 1;
  cplx *shiftX = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
  for (i64 i = 0; i < NX; ++i) shiftX[i] = cos(leftX * kx[i]) - II * sin(leftX * kx[i]);
  memset(out, 0, sizeof(cplx) * (size_t)(NX * NKR * NM * ncomp));
  fft_plan plan;
  fft_plan_init(&plan, (int)NX, -1);
#pragma omp parallel
  {
    cplx *a = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    cplx *f = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    cplx *scr = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 l = 0; l < ncomp; ++l)
      for (i64 m = 0; m < NM; ++m) {
#pragma omp for schedule(static)
        for (i64 k = 0; k < NKR; ++k) {
          for (i64 x = 0; x < NX; ++x) a[x] = 0.0;
          for (i64 r = 0; r < nr; ++r) {
            double c = In[r + nr * (k + NKR * m)];
            const cplx *vv = v + NX * ((r + 1) + NR * (m + NM * l));
            for (i64 x = 0; x < NX; ++x) a[x] += c * vv[x];
          }
          fft_exec(&plan, a, f, scr);
          cplx *o = out + NX * (k + NKR * (m + NM * l));
          for (i64 x = 0; x < NX; ++x) o[x] += f[x] * shiftX[x];
        }
      }
    free(a);
    free(f);
    free(scr);
  }
  fft_plan_free(&plan);
  free(shiftX);
}

/* fb_io.f90:100-180 (fb_vec_out / fb_scl_out) and :182-228 (fb_eb_out):
 * for every r >= 1: A(x) = e^{+i kx leftX} sum_k Out(k,r,m) v_fb(x,k,m), then
 * the unnormalised backward FFT along x, ADDED to out(x, r, m) (callers zero
 * `out` first, as the Fortran does).  Out(NKR,NR-1,NM). */
void orc_fb_out(cplx *out, const cplx *vfb, double leftX, const double *kx,
                const double *Out, i64 NX, i64 NR, i64 NM, i64 NKR,
                i64 ncomp) {
  i64 nr = NR - 1;
  cplx *shiftX = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
  for (i64 i = 0; i < NX; ++i) shiftX[i] = cos(leftX * kx[i]) + II * sin(leftX * kx[i]);
  fft_plan plan;
  fft_plan_init(&plan, (int)NX, +1);
#pragma omp parallel
  {
    cplx *a = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    cplx *f = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    cplx *scr = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 l = 0; l < ncomp; ++l)
      for (i64 m = 0; m < NM; ++m) {
#pragma omp for schedule(static)
        for (i64 r = 0; r < nr; ++r) {
          for (i64 x = 0; x < NX; ++x) a[x] = 0.0;
          for (i64 k = 0; k < NKR; ++k) {
            double c = Out[k + NKR * (r + nr * m)];
            const cplx *vv = vfb + NX * (k + NKR * (m + NM * l));
            for (i64 x = 0; x < NX; ++x) a[x] += c * vv[x];
          }
          for (i64 x = 0; x < NX; ++x) a[x] *= shiftX[x];
          fft_exec(&plan, a, f, scr);
          cplx *o = out + NX * ((r + 1) + NR * (m + NM * l));
          for (i64 x = 0; x < NX; ++x) o[x] += f[x];
        }
      }
    free(a);
    free(f);
    free(scr);
  }
  fft_plan_free(&plan);
  free(shiftX);
}

/* fb_io.f90:230-308 (fb_filtr): per (k, m, l) line: v*e^{+i kx leftX} ->
 * backward FFT -> multiply the filtered cells by the profile -> forward FFT
 * -> times 1/(NX e^{+i kx leftX}).  mode 0: first nxfilt cells, 1: last nxfilt
 * cells with the reversed profile, 2: both. */
void orc_fb_filtr(cplx *vec, double leftX, const double *kx,
                  const double *filtr, i64 nxfilt, int modefilt, i64 NX,
                  i64 NKR, i64 NM, i64 ncomp) {
  cplx *shiftX = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
  cplx *shinv = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
  for (i64 i = 0; i < NX; ++i) {
    shiftX[i] = cos(leftX * kx[i]) + II * sin(leftX * kx[i]);
    shinv[i] = 1.0 / ((double)NX * shiftX[i]);
  }
  fft_plan pin, pout;
  fft_plan_init(&pin, (int)NX, -1);
  fft_plan_init(&pout, (int)NX, +1);
#pragma omp parallel
  {
    cplx *a = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    cplx *f = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    cplx *scr = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 l = 0; l < ncomp; ++l)
      for (i64 m = 0; m < NM; ++m) {
#pragma omp for schedule(static)
        for (i64 k = 0; k < NKR; ++k) {
          cplx *v = vec + NX * (k + NKR * (m + NM * l));
          for (i64 x = 0; x < NX; ++x) a[x] = v[x] * shiftX[x];
          fft_exec(&pout, a, f, scr);
          if (modefilt == 0 || modefilt == 2)
            for (i64 i = 0; i < nxfilt; ++i) f[i] *= filtr[i];
          if (modefilt == 1 || modefilt == 2)
            for (i64 i = 0; i < nxfilt; ++i) f[NX - 1 - i] *= filtr[i];
          fft_exec(&pin, f, a, scr);
          for (i64 x = 0; x < NX; ++x) v[x] = a[x] * shinv[x];
        }
      }
    free(a);
    free(f);
    free(scr);
  }
  fft_plan_free(&pin);
  fft_plan_free(&pout);
  free(shiftX);
  free(shinv);
}

/* ------------------------------------------------------------------------ */
/* fb_math.f90 (plain modes 0..NM-1)                                         */
/* D(nkr, nkr_loc, NM+1) are DpS2S / DmS2S (after the solver's swapaxes).     */
/* ------------------------------------------------------------------------ */

/* acc(x) += sign * sum_k D(k, kl, m) * src(x, k) for one x-line output */
static inline void dht_line(cplx *acc, const double *D, i64 nkr, i64 nkl,
                            i64 kl, i64 m, const cplx *src, i64 NX, i64 srcstride,
                            cplx coef) {
  (void)nkl;
  for (i64 k = 0; k < nkr; ++k) {
    double d = D[k + nkr * (kl + nkl * m)];
    const cplx *s = src + srcstride * k;
    cplx dc = d * coef;
    for (i64 x = 0; x < NX; ++x) acc[x] += dc * s[x];
  }
}

/* Helper: reflected m=1 copy for the m=0 lower neighbour,
 * ext(x) = -conj(v(-x)) with index 0 fixed (fb_math.f90:35-36). */
static void reflect_conj(cplx *dst, const cplx *src, i64 NX) {
  dst[0] = -conj(src[0]);
  for (i64 x = 1; x < NX; ++x) dst[x] = -conj(src[NX - x]);
}

/* fb_math.f90:18-94 (fb_rot) */
void orc_fb_rot(cplx *out, const cplx *v, const double *Dp, const double *Dm,
                const double *kx, i64 NX, i64 NKR, i64 NM, i64 NKL) {
  i64 NMD = NM + 1; /* modes in Dp/Dm */
  (void)NMD;
  memset(out, 0, sizeof(cplx) * (size_t)(NX * NKL * NM * 3));
  cplx *ext = (cplx *)calloc((size_t)(NX * NKR * 3), sizeof(cplx));
  if (NM > 1)
    for (int c = 0; c < 3; ++c)
      for (i64 k = 0; k < NKR; ++k)
        reflect_conj(ext + NX * (k + NKR * c), v + NX * (k + NKR * (1 + NM * c)), NX);
#define V(c, m) (v + NX * NKR * ((m) + NM * (c)))
#define O(c, m, kl) (out + NX * ((kl) + NKL * ((m) + NM * (c))))
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = 0; m < NM; ++m) {
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o1 = O(0, m, kl), *o2 = O(1, m, kl), *o3 = O(2, m, kl);
        const cplx *v2 = V(1, m) + NX * kl, *v3 = V(2, m) + NX * kl;
        for (i64 x = 0; x < NX; ++x) {
          o2[x] = o2[x] - II * kx[x] * v3[x];
          o3[x] = o3[x] + II * kx[x] * v2[x];
        }
        if (m < NM - 1) {
          for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
          /* sl -= Dp (i v2 - v3) */
          for (i64 k = 0; k < NKR; ++k) {
            double d = Dp[k + NKR * (kl + NKL * m)];
            const cplx *a2 = V(1, m + 1) + NX * k, *a3 = V(2, m + 1) + NX * k;
            for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] - d * (II * a2[x] - a3[x]);
          }
          for (i64 x = 0; x < NX; ++x) o1[x] += sl[x];
          for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
          for (i64 k = 0; k < NKR; ++k) {
            double d = Dp[k + NKR * (kl + NKL * m)];
            const cplx *a1 = V(0, m + 1) + NX * k;
            for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] + d * a1[x];
          }
          for (i64 x = 0; x < NX; ++x) {
            o2[x] += II * sl[x];
            o3[x] -= sl[x];
          }
        }
        const cplx *b1, *b2, *b3;
        i64 bstride = NX;
        if (m > 0) {
          b1 = V(0, m - 1);
          b2 = V(1, m - 1);
          b3 = V(2, m - 1);
        } else {
          b1 = ext;
          b2 = ext + NX * NKR;
          b3 = ext + 2 * NX * NKR;
        }
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        for (i64 k = 0; k < NKR; ++k) {
          double d = Dm[k + NKR * (kl + NKL * m)];
          const cplx *a2 = b2 + bstride * k, *a3 = b3 + bstride * k;
          for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] - d * (II * a2[x] + a3[x]);
        }
        for (i64 x = 0; x < NX; ++x) o1[x] += sl[x];
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        for (i64 k = 0; k < NKR; ++k) {
          double d = Dm[k + NKR * (kl + NKL * m)];
          const cplx *a1 = b1 + bstride * k;
          for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] + d * a1[x];
        }
        for (i64 x = 0; x < NX; ++x) {
          o2[x] += II * sl[x];
          o3[x] += sl[x];
        }
      }
    }
    free(sl);
  }
#undef V
#undef O
  free(ext);
}

/* fb_math.f90:96-149 (fb_grad) */
void orc_fb_grad(cplx *out, const cplx *s, const double *Dp, const double *Dm,
                 const double *kx, i64 NX, i64 NKR, i64 NM, i64 NKL) {
  memset(out, 0, sizeof(cplx) * (size_t)(NX * NKL * NM * 3));
  cplx *ext = (cplx *)calloc((size_t)(NX * NKR), sizeof(cplx));
  if (NM > 1)
    for (i64 k = 0; k < NKR; ++k) reflect_conj(ext + NX * k, s + NX * (k + NKR * 1), NX);
#define S(m) (s + NX * NKR * (m))
#define O(c, m, kl) (out + NX * ((kl) + NKL * ((m) + NM * (c))))
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = 0; m < NM; ++m) {
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o1 = O(0, m, kl), *o2 = O(1, m, kl), *o3 = O(2, m, kl);
        const cplx *sm = S(m) + NX * kl;
        for (i64 x = 0; x < NX; ++x) o1[x] = o1[x] + II * kx[x] * sm[x];
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        dht_line(sl, Dm, NKR, NKL, kl, m, m > 0 ? S(m - 1) : ext, NX, NX, 1.0);
        for (i64 x = 0; x < NX; ++x) {
          o2[x] -= sl[x];
          o3[x] += II * sl[x];
        }
        if (m < NM - 1) {
          for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
          dht_line(sl, Dp, NKR, NKL, kl, m, S(m + 1), NX, NX, 1.0);
          for (i64 x = 0; x < NX; ++x) {
            o2[x] += sl[x];
            o3[x] += II * sl[x];
          }
        }
      }
    }
    free(sl);
  }
#undef S
#undef O
  free(ext);
}

/* fb_math.f90:151-199 (fb_div) */
void orc_fb_div(cplx *out, const cplx *v, const double *Dp, const double *Dm,
                const double *kx, i64 NX, i64 NKR, i64 NM, i64 NKL) {
  memset(out, 0, sizeof(cplx) * (size_t)(NX * NKL * NM));
  cplx *ext = (cplx *)calloc((size_t)(NX * NKR * 2), sizeof(cplx));
  if (NM > 1)
    for (int c = 0; c < 2; ++c)
      for (i64 k = 0; k < NKR; ++k)
        reflect_conj(ext + NX * (k + NKR * c), v + NX * (k + NKR * (1 + NM * (c + 1))), NX);
#define V(c, m) (v + NX * NKR * ((m) + NM * (c)))
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = 0; m < NM; ++m) {
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o = out + NX * (kl + NKL * m);
        const cplx *v1 = V(0, m) + NX * kl;
        for (i64 x = 0; x < NX; ++x) o[x] = o[x] + II * kx[x] * v1[x];
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        const cplx *b2 = m > 0 ? V(1, m - 1) : ext;
        const cplx *b3 = m > 0 ? V(2, m - 1) : ext + NX * NKR;
        for (i64 k = 0; k < NKR; ++k) {
          double d = Dm[k + NKR * (kl + NKL * m)];
          const cplx *a2 = b2 + NX * k, *a3 = b3 + NX * k;
          for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] + d * (II * a3[x] - a2[x]);
        }
        if (m < NM - 1) {
          for (i64 k = 0; k < NKR; ++k) {
            double d = Dp[k + NKR * (kl + NKL * m)];
            const cplx *a2 = V(1, m + 1) + NX * k, *a3 = V(2, m + 1) + NX * k;
            for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] + d * (II * a3[x] + a2[x]);
          }
        }
        for (i64 x = 0; x < NX; ++x) o[x] += sl[x];
      }
    }
    free(sl);
  }
#undef V
  free(ext);
}

/* fb_math.f90:201-293 (fb_graddiv): in place grad(div(v)); the divergence
 * is formed on NM+1 modes (the extra mode feeds the m+1 coupling of the top
 * mode). */
void orc_fb_graddiv(cplx *v, const double *Dp, const double *Dm,
                    const double *kx, i64 NX, i64 NKR, i64 NM, i64 NKL) {
  i64 NS = NM + 1;
  cplx *scl = (cplx *)calloc((size_t)(NX * NKL * NS), sizeof(cplx));
  cplx *aux = (cplx *)calloc((size_t)(NX * NKR * 2), sizeof(cplx));
  if (NM > 1)
    for (int c = 0; c < 2; ++c)
      for (i64 k = 0; k < NKR; ++k)
        reflect_conj(aux + NX * (k + NKR * c), v + NX * (k + NKR * (1 + NM * (c + 1))), NX);
#define V(c, m) (v + NX * NKR * ((m) + NM * (c)))
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = 0; m < NS; ++m) {
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o = scl + NX * (kl + NKL * m);
        if (m < NM) {
          const cplx *v1 = V(0, m) + NX * kl;
          for (i64 x = 0; x < NX; ++x) o[x] = o[x] + II * kx[x] * v1[x];
        }
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        const cplx *b2 = m > 0 ? V(1, m - 1) : aux;
        const cplx *b3 = m > 0 ? V(2, m - 1) : aux + NX * NKR;
        for (i64 k = 0; k < NKR; ++k) {
          double d = Dm[k + NKR * (kl + NKL * m)];
          const cplx *a2 = b2 + NX * k, *a3 = b3 + NX * k;
          for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] + d * (II * a3[x] - a2[x]);
        }
        if (m < NM - 1) {
          for (i64 k = 0; k < NKR; ++k) {
            double d = Dp[k + NKR * (kl + NKL * m)];
            const cplx *a2 = V(1, m + 1) + NX * k, *a3 = V(2, m + 1) + NX * k;
            for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] + d * (II * a3[x] + a2[x]);
          }
        }
        for (i64 x = 0; x < NX; ++x) o[x] += sl[x];
      }
    }
    free(sl);
  }
  memset(v, 0, sizeof(cplx) * (size_t)(NX * NKR * NM * 3));
  memset(aux, 0, sizeof(cplx) * (size_t)(NX * NKR * 2));
  if (NM > 1)
    for (i64 k = 0; k < NKR; ++k) reflect_conj(aux + NX * k, scl + NX * (k + NKL * 1), NX);
#define O(c, m, kl) (v + NX * ((kl) + NKL * ((m) + NM * (c))))
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = 0; m < NM; ++m) {
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o1 = O(0, m, kl), *o2 = O(1, m, kl), *o3 = O(2, m, kl);
        const cplx *sm = scl + NX * (kl + NKL * m);
        for (i64 x = 0; x < NX; ++x) o1[x] = o1[x] + II * kx[x] * sm[x];
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        dht_line(sl, Dm, NKR, NKL, kl, m, m > 0 ? scl + NX * NKL * (m - 1) : aux, NX, NX, 1.0);
        for (i64 x = 0; x < NX; ++x) {
          o2[x] -= sl[x];
          o3[x] += II * sl[x];
        }
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        dht_line(sl, Dp, NKR, NKL, kl, m, scl + NX * NKL * (m + 1), NX, NX, 1.0);
        for (i64 x = 0; x < NX; ++x) {
          o2[x] += sl[x];
          o3[x] += II * sl[x];
        }
      }
    }
    free(sl);
  }
#undef O
#undef V
  free(scl);
  free(aux);
}

/* ------------------------------------------------------------------------ */
/* fb_math_env.f90 (modes -K..K at index m+K; Dp/Dm hold modes -K-1..K+1 at  */
/* index m+K+1).                                                             */
/* ------------------------------------------------------------------------ */

/* fb_math_env.f90:18-61 (fb_grad_env) */
void orc_fb_grad_env(cplx *out, const cplx *s, const double *Dp,
                     const double *Dm, const double *kx, i64 NX, i64 NKR,
                     i64 NM, i64 NKL) {
  i64 K = (NM - 1) / 2;
  memset(out, 0, sizeof(cplx) * (size_t)(NX * NKL * NM * 3));
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = -K; m <= K; ++m) {
      i64 mi = m + K, md = m + K + 1;
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o1 = out + NX * (kl + NKL * (mi + NM * 0));
        cplx *o2 = out + NX * (kl + NKL * (mi + NM * 1));
        cplx *o3 = out + NX * (kl + NKL * (mi + NM * 2));
        const cplx *sm = s + NX * (kl + NKR * mi);
        for (i64 x = 0; x < NX; ++x) o1[x] = o1[x] + II * kx[x] * sm[x];
        if (m > -K) {
          for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
          dht_line(sl, Dm, NKR, NKL, kl, md, s + NX * NKR * (mi - 1), NX, NX, 1.0);
          for (i64 x = 0; x < NX; ++x) {
            o2[x] -= sl[x];
            o3[x] += II * sl[x];
          }
        }
        if (m < K) {
          for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
          dht_line(sl, Dp, NKR, NKL, kl, md, s + NX * NKR * (mi + 1), NX, NX, 1.0);
          for (i64 x = 0; x < NX; ++x) {
            o2[x] += sl[x];
            o3[x] += II * sl[x];
          }
        }
      }
    }
    free(sl);
  }
}

/* fb_math_env.f90:63-104 (fb_div_env) */
void orc_fb_div_env(cplx *out, const cplx *v, const double *Dp,
                    const double *Dm, const double *kx, i64 NX, i64 NKR,
                    i64 NM, i64 NKL) {
  i64 K = (NM - 1) / 2;
  memset(out, 0, sizeof(cplx) * (size_t)(NX * NKL * NM));
#define V(c, mi) (v + NX * NKR * ((mi) + NM * (c)))
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = -K; m <= K; ++m) {
      i64 mi = m + K, md = m + K + 1;
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o = out + NX * (kl + NKL * mi);
        const cplx *v1 = V(0, mi) + NX * kl;
        for (i64 x = 0; x < NX; ++x) o[x] = o[x] + II * kx[x] * v1[x];
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        if (m > -K)
          for (i64 k = 0; k < NKR; ++k) {
            double d = Dm[k + NKR * (kl + NKL * md)];
            const cplx *a2 = V(1, mi - 1) + NX * k, *a3 = V(2, mi - 1) + NX * k;
            for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] - d * (a2[x] - II * a3[x]);
          }
        if (m < K)
          for (i64 k = 0; k < NKR; ++k) {
            double d = Dp[k + NKR * (kl + NKL * md)];
            const cplx *a2 = V(1, mi + 1) + NX * k, *a3 = V(2, mi + 1) + NX * k;
            for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] + d * (a2[x] + II * a3[x]);
          }
        for (i64 x = 0; x < NX; ++x) o[x] += sl[x];
      }
    }
    free(sl);
  }
#undef V
}

/* fb_math_env.f90:106-162 (fb_rot_env).  The m-1 term of the first
 * component is computed and then discarded by the Fortran (its sliceKR is
 * reset before use, :146-151), so it does not appear here. */
void orc_fb_rot_env(cplx *out, const cplx *v, const double *Dp,
                    const double *Dm, const double *kx, i64 NX, i64 NKR,
                    i64 NM, i64 NKL) {
  i64 K = (NM - 1) / 2;
  memset(out, 0, sizeof(cplx) * (size_t)(NX * NKL * NM * 3));
#define V(c, mi) (v + NX * NKR * ((mi) + NM * (c)))
#define O(c, mi, kl) (out + NX * ((kl) + NKL * ((mi) + NM * (c))))
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = -K; m <= K; ++m) {
      i64 mi = m + K, md = m + K + 1;
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o1 = O(0, mi, kl), *o2 = O(1, mi, kl), *o3 = O(2, mi, kl);
        const cplx *v2 = V(1, mi) + NX * kl, *v3 = V(2, mi) + NX * kl;
        for (i64 x = 0; x < NX; ++x) {
          o2[x] = o2[x] - II * kx[x] * v3[x];
          o3[x] = o3[x] + II * kx[x] * v2[x];
        }
        if (m < K) {
          for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
          for (i64 k = 0; k < NKR; ++k) {
            double d = Dp[k + NKR * (kl + NKL * md)];
            const cplx *a2 = V(1, mi + 1) + NX * k, *a3 = V(2, mi + 1) + NX * k;
            for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] - d * (II * a2[x] - a3[x]);
          }
          for (i64 x = 0; x < NX; ++x) o1[x] += sl[x];
          for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
          dht_line(sl, Dp, NKR, NKL, kl, md, V(0, mi + 1), NX, NX, 1.0);
          for (i64 x = 0; x < NX; ++x) {
            o2[x] += II * sl[x];
            o3[x] -= sl[x];
          }
        }
        if (m > -K) {
          for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
          dht_line(sl, Dm, NKR, NKL, kl, md, V(0, mi - 1), NX, NX, 1.0);
          for (i64 x = 0; x < NX; ++x) {
            o2[x] += II * sl[x];
            o3[x] += sl[x];
          }
        }
      }
    }
    free(sl);
  }
#undef V
#undef O
}

/* fb_math_env.f90:164-233 (fb_graddiv_env): the divergence lives on modes
 * -K-1..K+1 (index m+K+1 of an NM+2 array). */
void orc_fb_graddiv_env(cplx *v, const double *Dp, const double *Dm,
                        const double *kx, i64 NX, i64 NKR, i64 NM, i64 NKL) {
  i64 K = (NM - 1) / 2;
  i64 NS = NM + 2;
  cplx *scl = (cplx *)calloc((size_t)(NX * NKL * NS), sizeof(cplx));
#define V(c, mi) (v + NX * NKR * ((mi) + NM * (c)))
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = -K - 1; m <= K + 1; ++m) {
      i64 mi = m + K, md = m + K + 1;
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o = scl + NX * (kl + NKL * md);
        if (m >= -K && m <= K) {
          const cplx *v1 = V(0, mi) + NX * kl;
          for (i64 x = 0; x < NX; ++x) o[x] = o[x] + II * kx[x] * v1[x];
        }
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        if (m > -K)
          for (i64 k = 0; k < NKR; ++k) {
            double d = Dm[k + NKR * (kl + NKL * md)];
            const cplx *a2 = V(1, mi - 1) + NX * k, *a3 = V(2, mi - 1) + NX * k;
            for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] - d * (a2[x] - II * a3[x]);
          }
        if (m < K)
          for (i64 k = 0; k < NKR; ++k) {
            double d = Dp[k + NKR * (kl + NKL * md)];
            const cplx *a2 = V(1, mi + 1) + NX * k, *a3 = V(2, mi + 1) + NX * k;
            for (i64 x = 0; x < NX; ++x) sl[x] = sl[x] + d * (a2[x] + II * a3[x]);
          }
        for (i64 x = 0; x < NX; ++x) o[x] += sl[x];
      }
    }
    free(sl);
  }
#undef V
  memset(v, 0, sizeof(cplx) * (size_t)(NX * NKR * NM * 3));
#define O(c, mi, kl) (v + NX * ((kl) + NKL * ((mi) + NM * (c))))
#pragma omp parallel
  {
    cplx *sl = (cplx *)malloc(sizeof(cplx) * (size_t)NX);
    for (i64 m = -K; m <= K; ++m) {
      i64 mi = m + K, md = m + K + 1;
#pragma omp for schedule(static)
      for (i64 kl = 0; kl < NKL; ++kl) {
        cplx *o1 = O(0, mi, kl), *o2 = O(1, mi, kl), *o3 = O(2, mi, kl);
        const cplx *sm = scl + NX * (kl + NKL * md);
        for (i64 x = 0; x < NX; ++x) o1[x] = o1[x] + II * kx[x] * sm[x];
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        dht_line(sl, Dm, NKR, NKL, kl, md, scl + NX * NKL * (md - 1), NX, NX, 1.0);
        for (i64 x = 0; x < NX; ++x) {
          o2[x] -= sl[x];
          o3[x] += II * sl[x];
        }
        for (i64 x = 0; x < NX; ++x) sl[x] = 0.0;
        dht_line(sl, Dp, NKR, NKL, kl, md, scl + NX * NKL * (md + 1), NX, NX, 1.0);
        for (i64 x = 0; x < NX; ++x) {
          o2[x] += sl[x];
          o3[x] += II * sl[x];
        }
      }
    }
    free(sl);
  }
#undef O
  free(scl);
}

/* ------------------------------------------------------------------------ */
/* maxwell_solvers.f90                                                       */
/* ------------------------------------------------------------------------ */

/* maxwell_solvers.f90:18-60 (maxwell_push_with_spchrg): real C1, C2 with 5
 * terms [E, G, J, grad rho_n, grad rho_n+1]; EG(NX,NKR,NM,6). */
void orc_maxwell_push_with_spchrg(cplx *eg, const cplx *j, const cplx *gn,
                                  const cplx *gnp1, const double *c1,
                                  const double *c2, i64 NX, i64 NKR, i64 NM) {
  i64 P = NX * NKR * NM;
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < P; ++i)
    for (int l = 0; l < 3; ++l) {
      cplx e = eg[i + P * l], g = eg[i + P * (3 + l)];
      cplx jj = j[i + P * l], a = gn[i + P * l], b = gnp1[i + P * l];
      cplx en = c1[i] * e + c1[i + P] * g + c1[i + 2 * P] * jj +
                c1[i + 3 * P] * a + c1[i + 4 * P] * b;
      cplx gnw = c2[i] * e + c2[i + P] * g + c2[i + 2 * P] * jj +
                 c2[i + 3 * P] * a + c2[i + 4 * P] * b;
      eg[i + P * (3 + l)] = gnw;
      eg[i + P * l] = en;
    }
}

/* maxwell_solvers.f90:62-96 (maxwell_push_wo_spchrg): complex C1, C2 with 3
 * terms [E, G, J]. */
void orc_maxwell_push_wo_spchrg(cplx *eg, const cplx *j, const cplx *c1,
                                const cplx *c2, i64 NX, i64 NKR, i64 NM) {
  i64 P = NX * NKR * NM;
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < P; ++i)
    for (int l = 0; l < 3; ++l) {
      cplx e = eg[i + P * l], g = eg[i + P * (3 + l)], jj = j[i + P * l];
      cplx en = c1[i] * e + c1[i + P] * g + c1[i + 2 * P] * jj;
      cplx gnw = c2[i] * e + c2[i + P] * g + c2[i + 2 * P] * jj;
      eg[i + P * (3 + l)] = gnw;
      eg[i + P * l] = en;
    }
}

/* maxwell_solvers.f90:98-129 (maxwell_init_push): complex C1, C2 (2 terms). */
void orc_maxwell_init_push(cplx *eg, const cplx *j, const cplx *gn,
                           const cplx *c1, const cplx *c2, i64 NX, i64 NKR,
                           i64 NM) {
  i64 P = NX * NKR * NM;
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < P; ++i)
    for (int l = 0; l < 3; ++l) {
      eg[i + P * l] = eg[i + P * l] + c1[i] * j[i + P * l] + c1[i + P] * gn[i + P * l];
      eg[i + P * (3 + l)] =
          eg[i + P * (3 + l)] + c2[i] * j[i + P * l] + c2[i + P] * gn[i + P * l];
    }
}

/* maxwell_solvers.f90:131-164 (poiss_corr) */
void orc_poiss_corr(cplx *j, const cplx *gdj, const cplx *gn, const cplx *gnp1,
                    double dt_inv, const double *w2_inv, i64 NX, i64 NKR,
                    i64 NM) {
  i64 P = NX * NKR * NM;
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < P; ++i)
    for (int l = 0; l < 3; ++l)
      j[i + P * l] = j[i + P * l] +
                     (gdj[i + P * l] + (gnp1[i + P * l] - gn[i + P * l]) * dt_inv) * w2_inv[i];
}

/* maxwell_solvers.f90:166-197 (poiss_corr_stat): DT(NX) complex */
void orc_poiss_corr_stat(cplx *j, const cplx *gdj, const cplx *gn,
                         const cplx *DT, const double *w2_inv, i64 NX, i64 NKR,
                         i64 NM) {
  i64 P = NX * NKR * NM;
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < P; ++i)
    for (int l = 0; l < 3; ++l)
      j[i + P * l] = j[i + P * l] + (gdj[i + P * l] + DT[i % NX] * gn[i + P * l]) * w2_inv[i];
}

/* maxwell_solvers.f90:199-226 (field_drift): EG *= exp(-i dt beta0 kx / 2) */
void orc_field_drift(cplx *eg, const double *kx, double beta0, double dt,
                     i64 NX, i64 NKR, i64 NM) {
  cplx fact = -0.5 * II * dt * beta0;
  i64 P = NX * NKR * NM;
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < 6 * P; ++i) eg[i] = eg[i] * cexp(fact * kx[i % NX]);
}

/* maxwell_solvers.f90:228-318 (omp_mult_vec/scl, omp_add_vec/scl) */
void orc_mult(cplx *v, const double *A, i64 P, i64 ncomp) {
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < P; ++i)
    for (i64 l = 0; l < ncomp; ++l) v[i + P * l] = v[i + P * l] * A[i];
}
void orc_add(cplx *v, const cplx *A, i64 n) {
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < n; ++i) v[i] = v[i] + A[i];
}

/* ------------------------------------------------------------------------ */
/* devices.f90                                                               */
/* ------------------------------------------------------------------------ */

static inline double ramp_ampl(double x, double X0, double Lx, double lam) {
  if (x <= X0 || x >= X0 + Lx) return 0.0;
  if (x > X0 && x < X0 + lam) return (x - X0) / lam;
  if (x > X0 + Lx - lam && x < X0 + Lx) return (X0 + Lx - x) / lam;
  return 1.0;
}

/* devices.f90:162-203 (undul_analytic): planar undulator with one-period
 * linear ramps; params = (a0, lambda_u, X0, Lx). */
void orc_undul_analytic(const double *coord, double *fld, double t,
                        const double *params, i64 np) {
  (void)t;
  double a0 = params[0], lam = params[1], X0 = params[2], Lx = params[3];
  double ku = 2. * PI / lam;
#pragma omp parallel for schedule(static)
  for (i64 ip = 0; ip < np; ++ip) {
    double x = coord[3 * ip], y = coord[3 * ip + 1];
    double ampl = ramp_ampl(x, X0, Lx, lam) * a0;
    fld[6 * ip + 4] += ampl * sin(ku * (x - X0)) * cosh(ku * y);
    fld[6 * ip + 3] += ampl * cos(ku * (x - X0)) * sinh(ku * y);
  }
}

/* devices.f90:117-160 (undul_analytic_taper); params = (a0, lambda_u, X0,
 * Lx, taper). */
void orc_undul_analytic_taper(const double *coord, double *fld, double t,
                              const double *params, i64 np) {
  (void)t;
  double a0 = params[0], lam = params[1], X0 = params[2], Lx = params[3],
         taper = params[4];
  double ku = 2. * PI / lam;
#pragma omp parallel for schedule(static)
  for (i64 ip = 0; ip < np; ++ip) {
    double x = coord[3 * ip], y = coord[3 * ip + 1];
    double ampl = ramp_ampl(x, X0, Lx, lam);
    ampl = ampl * (1 + taper * (x - X0 - 0.5 * Lx) / (0.5 * Lx));
    ampl = ampl * a0;
    fld[6 * ip + 4] += ampl * sin(ku * (x - X0)) * cosh(ku * y);
    fld[6 * ip + 3] += ampl * cos(ku * (x - X0)) * sinh(ku * y);
  }
}

/* devices.f90:18-62 (undul_mapped) and :64-115 (undul_mapped_tap): field map
 * a0(2, nx) interpolated with quadratic splines; params = (lambda_u, Xleft,
 * dx[, Lx, taper]). */
void orc_undul_mapped(const double *coord, double *fld, double t,
                      const double *a0, i64 nx, const double *params,
                      int tapered, i64 np) {
  (void)t;
  double lam = params[0], Xleft = params[1], dx = params[2];
  double ku = 2. * PI / lam, dx_inv = 1.0 / dx;
  double Xright = Xleft + nx * dx;
  double Lx = tapered ? params[3] : 0.0, taper = tapered ? params[4] : 0.0;
  double x_shift = 0.5 * (nx * dx - Lx);
#pragma omp parallel for schedule(static)
  for (i64 ip = 0; ip < np; ++ip) {
    double xp = coord[3 * ip];
    if (xp < Xleft + dx || xp > Xright - dx) continue;
    double yp = coord[3 * ip + 1];
    i64 ix = (i64)floor((xp - Xleft) * dx_inv + 0.5);
    double ddx = (xp - Xleft) * dx_inv - ix;
    double S[3] = {0.5 * (0.5 - ddx) * (0.5 - ddx), 0.75 - ddx * ddx,
                   0.5 * (0.5 + ddx) * (0.5 + ddx)};
    /* Fortran a0(1:2, 1:nx) indexed at ix-1..ix+1 (1-based) */
    double s1 = 0.0, s2 = 0.0;
    for (int q = 0; q < 3; ++q) {
      i64 col = ix - 1 + q - 1; /* 0-based column */
      if (col < 0 || col >= nx) continue;
      s1 += S[q] * a0[2 * col];
      s2 += S[q] * a0[2 * col + 1];
    }
    double amp = 1.0;
    if (tapered) amp = 1 + taper * (xp - x_shift - Xleft - 0.5 * Lx) / (0.5 * Lx);
    fld[6 * ip + 4] += amp * s1 * cosh(ku * yp);
    fld[6 * ip + 3] += amp * s2 * sinh(ku * yp);
  }
}

/* devices.f90:205-252 (planewave); params = (a0, lambda, X0, Lx, ramp,
 * theta, phi0). */
void orc_planewave(const double *coord, double *fld, double t,
                   const double *params, i64 np) {
  double a0 = params[0], lam = params[1], X0 = params[2], Lx = params[3],
         ramp = params[4], theta = params[5], phi0 = params[6];
  double sinth = sin(theta), costh = cos(theta), k0 = 2. * PI / lam;
#pragma omp parallel for schedule(static)
  for (i64 ip = 0; ip < np; ++ip) {
    double x = coord[3 * ip], y = coord[3 * ip + 1];
    double ampl = ramp_ampl(x, X0, Lx, ramp);
    ampl = a0 * ampl * sin(k0 * (x * costh + y * sinth - t) + phi0);
    fld[6 * ip + 2] += ampl;
    fld[6 * ip + 3] += ampl * sinth;
    fld[6 * ip + 4] -= ampl * costh;
  }
}

/* devices.f90:254-297 (gaussbeam); params = (lambda, axis, x0, y0, z0, Lx,
 * Ly, Lz). */
void orc_gaussbeam(const double *coord, double *fld, double time, double a0,
                   const double *params, i64 np) {
  double lam = params[0], axis = params[1], x0 = params[2], y0 = params[3],
         z0 = params[4];
  double lx2 = 1.0 / (params[5] * params[5]), ly2 = 1.0 / (params[6] * params[6]),
         lz2 = 1.0 / (params[7] * params[7]);
#pragma omp parallel for schedule(static)
  for (i64 ip = 0; ip < np; ++ip) {
    double xp = coord[3 * ip] - x0 - axis * time;
    double yp = coord[3 * ip + 1] - y0, zp = coord[3 * ip + 2] - z0;
    double E = a0 * exp(-xp * xp * lx2 - yp * yp * ly2 - zp * zp * lz2) *
               sin(2. * PI / lam * xp);
    fld[6 * ip + 2] += E;
    fld[6 * ip + 4] -= axis * E;
  }
}

/* ------------------------------------------------------------------------ */
/* utils.f90:18-57 intens_profO.  pwr (NO, NR-1); fld (NX, NR, NM, 3) with    */
/* NM = 2 nkO + 1 (modes -nkO..nkO).  The angle phases are built by repeated */
/* products as the Fortran does (Os(iO) = Os(iO-1) * phase_p).               */
/* ------------------------------------------------------------------------ */
void orc_intens_profo(double *pwr, const cplx *fld, i64 NO, i64 NX, i64 NR, i64 NM) {
  const i64 nkO = (NM - 1) / 2;
  const i64 nr = NR - 1;
  cplx *Os = (cplx *)malloc(sizeof(cplx) * (size_t)NO);
  cplx *phaseO = (cplx *)malloc(sizeof(cplx) * (size_t)NM);
  memset(pwr, 0, sizeof(double) * (size_t)(NO * nr));
  Os[0] = 1.0;
  const cplx step = cos(2.0 * PI / (double)(NO - 1)) + II * sin(2.0 * PI / (double)(NO - 1));
  for (i64 io = 1; io < NO; ++io) Os[io] = Os[io - 1] * step;
  for (i64 io = 0; io < NO; ++io) {
    const cplx pp = Os[io], pm = 1.0 / Os[io];
    for (i64 k = 0; k < NM; ++k) phaseO[k] = 1.0;
    for (i64 k = 1; k <= nkO; ++k) {
      phaseO[nkO + k] = phaseO[nkO + k - 1] * pp;
      phaseO[nkO - k] = phaseO[nkO - k + 1] * pm;
    }
    for (int l = 0; l < 3; ++l)
      for (i64 ir = 1; ir <= nr; ++ir)
        for (i64 ix = 0; ix < NX; ++ix) {
          cplx s = 0.0;
          for (i64 k = 0; k < NM; ++k) s += phaseO[k] * fld[ix + NX * (ir + NR * (k + NM * l))];
          const double a = cabs(s);
          pwr[io + NO * (ir - 1)] += a * a;
        }
  }
  free(Os);
  free(phaseO);
}
