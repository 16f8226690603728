/*
 * chimera_gb300.h -- C ABI of libchimera_gb300.so, the GB300 (sm_103a)
 * implementation of CHIMERA's per-step particle-in-cell hot path.
 *
 * Every entry point replaces one subroutine of the reference's f2py module
 * `chimera.moduls.fimera` (built from the f90 sources, Makefile:6-11,32-34); the
 * comment above each declaration cites the Fortran routine it replaces.  The
 * argument meaning follows the Fortran; the dimensions that f2py hides are
 * explicit.
 *
 * Conventions
 *   - All array arguments are DEVICE pointers (cudaMalloc'd or owned by any
 *     allocator, e.g. torch), except where a comment says "host".
 *   - Grid and spectral arrays are column-major (Fortran order) and dense:
 *       spatial  grid  (nx, nr, nm[, ncomp]) complex128
 *       spectral grid  (nx, nkr, nm[, ncomp]) complex128
 *     with nr counting the ghost row at r = -dr/2 (index 0), nm the stored
 *     azimuthal modes (0..M-1, or -K..K for the envelope "env" solver).
 *   - complex128 = interleaved {re, im} doubles (chm_c128).
 *   - Particle arrays (3,np) / (6,np) / (np) are strided: element (c, i) is
 *     at ptr[c * comp_stride + i * part_stride].  The reference's F-ordered
 *     (3,np) arrays have comp_stride = 1, part_stride = 3; the structure-of-
 *     arrays buffers used by chimera_gb300 have part_stride = 1.
 *   - `stream` is a cudaStream_t; every call is asynchronous on it.
 *   - Return value: CHM_OK or an error code; chm_last_error() gives the text.
 *   - No entry point allocates device memory.  Scratch space is passed in by
 *     the caller (`ws`, `ws_bytes`), sized with the matching *_ws_bytes query.
 */
#ifndef CHIMERA_GB300_H
#define CHIMERA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double re, im;
} chm_c128;

enum {
  CHM_OK = 0,
  CHM_ERR_ARG = 1,      /* bad shape / stride / pointer */
  CHM_ERR_CUDA = 2,     /* a CUDA launch or runtime call failed */
  CHM_ERR_WS = 3,       /* workspace too small */
  CHM_ERR_CAPACITY = 4, /* particle capacity exceeded */
  CHM_ERR_RANGE = 5     /* a value is out of the supported range */
};

/* Text of the last error reported by this thread's last failing call. */
const char *chm_last_error(void);
/* Library version string. */
const char *chm_version(void);
/* Diagnostics (no reference counterpart): number of kernels this library has
 * launched since it was loaded, and the algorithmic FLOPs of the dense
 * DHT / mode-coupling products it has issued (4 nx N K per complex plane
 * times real matrix product). */
int64_t chm_launch_count(void);
double chm_gemm_flops(void);

/* ======================================================================== */
/* Particle push                                                             */
/* ======================================================================== */

/* particle_tools.f90:18-56 push_velocs(momenta, Fld, dt): Boris rotation. */
int chm_push_velocs(double *momenta, int64_t p_cs, int64_t p_ps,
                    const double *fld, int64_t f_cs, int64_t f_ps, double dt,
                    int64_t np, void *stream);

/* particle_tools.f90:58-82 push_coords(coord, momenta, coord_cntr, dt). */
int chm_push_coords(double *coord, int64_t x_cs, int64_t x_ps,
                    const double *momenta, int64_t p_cs, int64_t p_ps,
                    double *coord_cntr, int64_t h_cs, int64_t h_ps, double dt,
                    int64_t np, void *stream);

/* ======================================================================== */
/* Field gather                                                              */
/* ======================================================================== */

/* grid_deps.f90:149-217 proj_fld(coord, wghts, Fld, Fld_tot, leftX, Rgrid,
 * dx_inv, dr_inv): Fld_tot(6,np) += Re(sum_m S e^{i m theta} Fld_m).
 * rgrid: device array of nr doubles. */
int chm_proj_fld(const double *coord, int64_t x_cs, int64_t x_ps,
                 const double *wghts, int64_t w_ps, const chm_c128 *fld,
                 double *fld_tot, int64_t f_cs, int64_t f_ps, double leftX,
                 const double *rgrid, double dx_inv, double dr_inv, int64_t np,
                 int64_t nx, int64_t nr, int64_t nm, void *stream);

/* grid_deps_env.f90:164-238 proj_fld_env(..., kx0): modes -K..K, carrier
 * e^{+i kx0 x}, on-axis phase 1. */
int chm_proj_fld_env(const double *coord, int64_t x_cs, int64_t x_ps,
                     const double *wghts, int64_t w_ps, const chm_c128 *fld,
                     double *fld_tot, int64_t f_cs, int64_t f_ps, double leftX,
                     const double *rgrid, double dx_inv, double dr_inv,
                     double kx0, int64_t np, int64_t nx, int64_t nr,
                     int64_t nm, void *stream);

/* grid_deps.f90:219-266 eb_correction(eb_spc) and grid_deps_env.f90:240-283
 * eb_correction_env(eb_spc): mode normalisation + ghost row. */
int chm_eb_correction(chm_c128 *eb, int64_t nx, int64_t nr, int64_t nm,
                      void *stream);
int chm_eb_correction_env(chm_c128 *eb, int64_t nx, int64_t nr, int64_t nm,
                          void *stream);

/* ======================================================================== */
/* External fields ("devices"), devices.f90                                  */
/* ======================================================================== */

/* devices.f90:162-203 undul_analytic(coord, Fld, t, params[4]); params is a
 * HOST array (a0, lambda_u, X0, Lx). */
int chm_undul_analytic(const double *coord, int64_t x_cs, int64_t x_ps,
                       double *fld, int64_t f_cs, int64_t f_ps, double t,
                       const double *params, int64_t np, void *stream);
/* devices.f90:117-160 undul_analytic_taper(coord, Fld, t, params[5]) */
int chm_undul_analytic_taper(const double *coord, int64_t x_cs, int64_t x_ps,
                             double *fld, int64_t f_cs, int64_t f_ps, double t,
                             const double *params, int64_t np, void *stream);
/* devices.f90:18-62 undul_mapped(coord, Fld, t, a0(2,nmap), params[3]) and
 * devices.f90:64-115 undul_mapped_tap(..., params[5]); a0 is a device array,
 * params a host array. */
int chm_undul_mapped(const double *coord, int64_t x_cs, int64_t x_ps,
                     double *fld, int64_t f_cs, int64_t f_ps, double t,
                     const double *a0, int64_t nmap, const double *params,
                     int64_t np, void *stream);
int chm_undul_mapped_tap(const double *coord, int64_t x_cs, int64_t x_ps,
                         double *fld, int64_t f_cs, int64_t f_ps, double t,
                         const double *a0, int64_t nmap, const double *params,
                         int64_t np, void *stream);
/* devices.f90:205-252 planewave(coord, Fld, t, params[7]) */
int chm_planewave(const double *coord, int64_t x_cs, int64_t x_ps, double *fld,
                  int64_t f_cs, int64_t f_ps, double t, const double *params,
                  int64_t np, void *stream);
/* devices.f90:254-297 gaussbeam(coord, Fld, time, a0, params[8]) */
int chm_gaussbeam(const double *coord, int64_t x_cs, int64_t x_ps, double *fld,
                  int64_t f_cs, int64_t f_ps, double time, double a0,
                  const double *params, int64_t np, void *stream);

/* ======================================================================== */
/* Grid deposition (deterministic: 64-bit fixed-point accumulation, no float */
/* atomics; results are bitwise reproducible run to run)                     */
/* ======================================================================== */

/* Workspace for any deposit onto a grid of nx*nr*nm*ncomp complex values. */
int64_t chm_dep_ws_bytes(int64_t nx, int64_t nr, int64_t nm, int64_t ncomp,
                         int64_t np);

/* grid_deps.f90:18-87 dep_curr(coord, momenta, wghts, curr, leftX, Rgrid,
 * dx_inv, dr_inv): curr(nx,nr,nm,3) += w v/gamma S e^{-i m theta}; ghost
 * fold.  coord are the half-step coordinates. */
int chm_dep_curr(const double *coord, int64_t x_cs, int64_t x_ps,
                 const double *momenta, int64_t p_cs, int64_t p_ps,
                 const double *wghts, int64_t w_ps, chm_c128 *curr,
                 double leftX, const double *rgrid, double dx_inv,
                 double dr_inv, int64_t np, int64_t nx, int64_t nr, int64_t nm,
                 void *ws, int64_t ws_bytes, void *stream);
/* No counterpart in the reference.  The current deposit of chm_dep_curr for
 * callers that cannot allocate device memory (an FFI host with no CUDA
 * allocator of its own, or a loop with a device memory budget fixed at
 * start-up that may not call cudaMalloc mid-run).  Same arguments minus the
 * workspace: the scratch lives in a 16 MiB static device array that every
 * GPU loading the library keeps until exit (chm_dep_noalloc_max_bytes()).
 * Grids needing more scratch than that are rejected with CHM_ERR_RANGE.  The
 * first call on a device resolves the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * All calls share the one array, which keeps the last call's contents (the
 * accumulator is cleared at the start of each call): calls that overlap on
 * the GPU (concurrent streams or host threads) race on it. */
int64_t chm_dep_noalloc_max_bytes(void);
int chm_dep_curr_noalloc(const double *coord, int64_t x_cs, int64_t x_ps,
                         const double *momenta, int64_t p_cs, int64_t p_ps,
                         const double *wghts, int64_t w_ps, chm_c128 *curr,
                         double leftX, const double *rgrid, double dx_inv,
                         double dr_inv, int64_t np, int64_t nx, int64_t nr,
                         int64_t nm, void *stream);

/* grid_deps.f90:89-147 dep_dens(coord, wghts, dens, leftX, Rgrid, dx_inv,
 * dr_inv) */
int chm_dep_dens(const double *coord, int64_t x_cs, int64_t x_ps,
                 const double *wghts, int64_t w_ps, chm_c128 *dens,
                 double leftX, const double *rgrid, double dx_inv,
                 double dr_inv, int64_t np, int64_t nx, int64_t nr, int64_t nm,
                 void *ws, int64_t ws_bytes, void *stream);
/* grid_deps_env.f90:18-95 dep_curr_env(..., kx0) (third component only) */
int chm_dep_curr_env(const double *coord, int64_t x_cs, int64_t x_ps,
                     const double *momenta, int64_t p_cs, int64_t p_ps,
                     const double *wghts, int64_t w_ps, chm_c128 *curr,
                     double leftX, const double *rgrid, double dx_inv,
                     double dr_inv, double kx0, int64_t np, int64_t nx,
                     int64_t nr, int64_t nm, void *ws, int64_t ws_bytes,
                     void *stream);
/* grid_deps_env.f90:97-162 dep_dens_env(..., kx0) (weight applied twice) */
int chm_dep_dens_env(const double *coord, int64_t x_cs, int64_t x_ps,
                     const double *wghts, int64_t w_ps, chm_c128 *dens,
                     double leftX, const double *rgrid, double dx_inv,
                     double dr_inv, double kx0, int64_t np, int64_t nx,
                     int64_t nr, int64_t nm, void *ws, int64_t ws_bytes,
                     void *stream);
/* grid_deps_chnk.f90:18-130 dep_curr_chnk(coord, momenta, wghts, curr,
 * IndInChunk, guards, leftX, Rgrid, dx_inv, dr_inv); ind_in_chunk is a
 * device int32 array of nchnk+1 offsets.  Same guard-buffer semantics as
 * the Fortran: chunk 0 drops its contributions to x-node 0. */
int chm_dep_curr_chnk(const double *coord, int64_t x_cs, int64_t x_ps,
                      const double *momenta, int64_t p_cs, int64_t p_ps,
                      const double *wghts, int64_t w_ps, chm_c128 *curr,
                      const int32_t *ind_in_chunk, int64_t nchnk,
                      int64_t guards, double leftX, const double *rgrid,
                      double dx_inv, double dr_inv, int64_t np, int64_t nx,
                      int64_t nr, int64_t nm, void *ws, int64_t ws_bytes,
                      void *stream);
/* grid_deps_chnk.f90:132-234 dep_dens_chnk(...) */
int chm_dep_dens_chnk(const double *coord, int64_t x_cs, int64_t x_ps,
                      const double *wghts, int64_t w_ps, chm_c128 *dens,
                      const int32_t *ind_in_chunk, int64_t nchnk,
                      int64_t guards, double leftX, const double *rgrid,
                      double dx_inv, double dr_inv, int64_t np, int64_t nx,
                      int64_t nr, int64_t nm, void *ws, int64_t ws_bytes,
                      void *stream);
/* grid_deps_env_chnk.f90:18-145 dep_curr_env_chnk(..., kx0) */
int chm_dep_curr_env_chnk(const double *coord, int64_t x_cs, int64_t x_ps,
                          const double *momenta, int64_t p_cs, int64_t p_ps,
                          const double *wghts, int64_t w_ps, chm_c128 *curr,
                          const int32_t *ind_in_chunk, int64_t nchnk,
                          int64_t guards, double leftX, const double *rgrid,
                          double dx_inv, double dr_inv, double kx0, int64_t np,
                          int64_t nx, int64_t nr, int64_t nm, void *ws,
                          int64_t ws_bytes, void *stream);
/* grid_deps_env_chnk.f90:147-261 dep_dens_env_chnk(..., kx0) */
int chm_dep_dens_env_chnk(const double *coord, int64_t x_cs, int64_t x_ps,
                          const double *wghts, int64_t w_ps, chm_c128 *dens,
                          const int32_t *ind_in_chunk, int64_t nchnk,
                          int64_t guards, double leftX, const double *rgrid,
                          double dx_inv, double dr_inv, double kx0, int64_t np,
                          int64_t nx, int64_t nr, int64_t nm, void *ws,
                          int64_t ws_bytes, void *stream);

/* ======================================================================== */
/* Fourier-Bessel transforms, fb_io.f90                                      */
/* ======================================================================== */

/* Workspace for the FB transforms of ncomp components. */
int64_t chm_fb_ws_bytes(int64_t nx, int64_t nr, int64_t nkr, int64_t nm,
                        int64_t ncomp);

/* fb_io.f90:18-59 fb_vec_in(vec_fb, vec, leftX, kx, In) and fb_io.f90:61-98
 * fb_scl_in (ncomp = 1).  vec (nx,nr,nm,ncomp), In (nr-1,nkr,nm) real,
 * kx (nx) real, out vec_fb (nx,nkr,nm,ncomp).  If `fact` is not NULL the
 * result is also multiplied by the real (nx,nkr,nm) array fact (this fuses
 * the omp_mult_vec(J_fb, DepFact) that follows every call in
 * solvers.py:417-420). */
int chm_fb_in(chm_c128 *vec_fb, const chm_c128 *vec, double leftX,
              const double *kx, const double *In, const double *fact,
              int64_t nx, int64_t nr, int64_t nkr, int64_t nm, int64_t ncomp,
              void *ws, int64_t ws_bytes, void *stream);

/* fb_io.f90:100-180 fb_vec_out / fb_scl_out: vec(nx,nr,nm,ncomp) = IFFT_x(
 * e^{+i kx leftX} sum_k Out(k,r,m) vec_fb); Out (nkr,nr-1,nm); row 0 = 0.
 * eb_mode: 0 = plain output, 1 = apply eb_correction, 2 = eb_correction_env
 * (fuses grid_deps.f90:219-266 into the transform). */
int chm_fb_out(chm_c128 *vec, const chm_c128 *vec_fb, double leftX,
               const double *kx, const double *Out, int64_t nx, int64_t nr,
               int64_t nkr, int64_t nm, int64_t ncomp, int eb_mode, void *ws,
               int64_t ws_bytes, void *stream);

/* fb_io.f90:182-228 fb_eb_out(eb_spc, e_fb, b_fb, leftX, kx, Out): the 6
 * components of eb_spc from e_fb(:,:,:,1:3) and b_fb(:,:,:,1:3).  e_fb and
 * b_fb point to the first component of 3 contiguous component planes. */
int chm_fb_eb_out(chm_c128 *eb, const chm_c128 *e_fb, const chm_c128 *b_fb,
                  double leftX, const double *kx, const double *Out,
                  int64_t nx, int64_t nr, int64_t nkr, int64_t nm, int eb_mode,
                  void *ws, int64_t ws_bytes, void *stream);

/* fb_io.f90:230-308 fb_filtr(vec, leftX, kx, filtr, modefilt): absorbing
 * layer applied in x-space to vec (nx,nkr,nm,ncomp). filtr: device array. */
int chm_fb_filtr(chm_c128 *vec, double leftX, const double *kx,
                 const double *filtr, int64_t nxfilt, int modefilt, int64_t nx,
                 int64_t nkr, int64_t nm, int64_t ncomp, void *ws,
                 int64_t ws_bytes, void *stream);

/* ======================================================================== */
/* Spectral differential operators, fb_math.f90 / fb_math_env.f90            */
/* Dp, Dm: (nkr, nkr, nm+1) plain / (nkr, nkr, nm+2) env, real.              */
/* ======================================================================== */

int64_t chm_fbmath_ws_bytes(int64_t nx, int64_t nkr, int64_t nm);

/* fb_math.f90:18-94 fb_rot(vec_fb_loc, vec_fb, DpS2S, DmS2S, kx) */
int chm_fb_rot(chm_c128 *out, const chm_c128 *vec, const double *Dp,
               const double *Dm, const double *kx, int64_t nx, int64_t nkr,
               int64_t nm, int env, void *ws, int64_t ws_bytes, void *stream);
/* fb_math.f90:96-149 fb_grad(vec_fb_loc, scl_fb, DpS2S, DmS2S, kx) */
int chm_fb_grad(chm_c128 *out, const chm_c128 *scl, const double *Dp,
                const double *Dm, const double *kx, int64_t nx, int64_t nkr,
                int64_t nm, int env, void *ws, int64_t ws_bytes, void *stream);
/* fb_math.f90:151-199 fb_div(scl_fb_loc, vec_fb, DpS2S, DmS2S, kx) */
int chm_fb_div(chm_c128 *out, const chm_c128 *vec, const double *Dp,
               const double *Dm, const double *kx, int64_t nx, int64_t nkr,
               int64_t nm, int env, void *ws, int64_t ws_bytes, void *stream);
/* fb_math.f90:201-293 fb_graddiv(vec_fb, DpS2S, DmS2S, kx), in place */
int chm_fb_graddiv(chm_c128 *vec, const double *Dp, const double *Dm,
                   const double *kx, int64_t nx, int64_t nkr, int64_t nm,
                   int env, void *ws, int64_t ws_bytes, void *stream);

/* ======================================================================== */
/* PSATD update and spectral elementwise ops, maxwell_solvers.f90            */
/* ======================================================================== */

/* maxwell_solvers.f90:18-60 maxwell_push_with_spchrg(EG_fb, j_fb,
 * grad_rho_n_fb, grad_rho_np1_fb, C1, C2); C1, C2 real (nx,nkr,nm,5). */
int chm_maxwell_push_with_spchrg(chm_c128 *eg, const chm_c128 *j,
                                 const chm_c128 *gn, const chm_c128 *gnp1,
                                 const double *c1, const double *c2,
                                 int64_t nx, int64_t nkr, int64_t nm,
                                 void *stream);
/* maxwell_solvers.f90:62-96 maxwell_push_wo_spchrg(EG_fb, j_fb, C1, C2);
 * C1, C2 complex (nx,nkr,nm,3). */
int chm_maxwell_push_wo_spchrg(chm_c128 *eg, const chm_c128 *j,
                               const chm_c128 *c1, const chm_c128 *c2,
                               int64_t nx, int64_t nkr, int64_t nm,
                               void *stream);
/* maxwell_solvers.f90:98-129 maxwell_init_push(EG_fb, j_fb, grad_rho_n_fb,
 * C1, C2); C1, C2 complex (nx,nkr,nm,2). */
int chm_maxwell_init_push(chm_c128 *eg, const chm_c128 *j, const chm_c128 *gn,
                          const chm_c128 *c1, const chm_c128 *c2, int64_t nx,
                          int64_t nkr, int64_t nm, void *stream);
/* maxwell_solvers.f90:131-164 poiss_corr(j_fb, grad_div_j_fb,
 * grad_rho_n_fb, grad_rho_np1_fb, dt_inv, w2_inv) */
int chm_poiss_corr(chm_c128 *j, const chm_c128 *gdj, const chm_c128 *gn,
                   const chm_c128 *gnp1, double dt_inv, const double *w2_inv,
                   int64_t nx, int64_t nkr, int64_t nm, void *stream);
/* maxwell_solvers.f90:166-197 poiss_corr_stat(j_fb, grad_div_j_fb,
 * grad_rho_n_fb, DT, w2_inv); DT complex (nx). */
int chm_poiss_corr_stat(chm_c128 *j, const chm_c128 *gdj, const chm_c128 *gn,
                        const chm_c128 *DT, const double *w2_inv, int64_t nx,
                        int64_t nkr, int64_t nm, void *stream);
/* maxwell_solvers.f90:199-226 field_drift(EG_fb, kx, beta0, dt) */
int chm_field_drift(chm_c128 *eg, const double *kx, double beta0, double dt,
                    int64_t nx, int64_t nkr, int64_t nm, void *stream);
/* maxwell_solvers.f90:228-272 omp_mult_vec / omp_mult_scl: v(P,ncomp) *= A(P)
 * with P = nx*nkr*nm. */
int chm_omp_mult(chm_c128 *v, const double *A, int64_t P, int64_t ncomp,
                 void *stream);
/* maxwell_solvers.f90:274-318 omp_add_vec / omp_add_scl: v(n) += A(n) */
int chm_omp_add(chm_c128 *v, const chm_c128 *A, int64_t n, void *stream);

/* ======================================================================== */
/* Particle bookkeeping, particle_tools.f90                                  */
/* ======================================================================== */

/* particle_tools.f90:130-153 sortpartsout(coord, lims): indx2stay (device,
 * int64, np) gets the 0-based indices of particles inside
 * lims = (xmin, xmax, r2min, r2max) (host array) in increasing order;
 * *num2stay (host) their number.  Synchronises the stream. */
int64_t chm_sortpartsout_ws_bytes(int64_t np);
int chm_sortpartsout(int64_t *indx2stay, int64_t *num2stay,
                     const double *coord, int64_t x_cs, int64_t x_ps,
                     const double *lims, int64_t np, void *ws,
                     int64_t ws_bytes, void *stream);

/* particle_tools.f90:155-208 chunk_coords_boundaries(coord, lims, Xgrid,
 * nchnk): chunked_indx (device int8, np), ind_in_chnk (device int32,
 * nchnk+1) and *go_out (host).  xgrid0, xgridc are Xgrid(0) and
 * Xgrid((nx+1)/nchnk) (or Xgrid(nx) for one chunk).  Synchronises. */
int chm_chunk_coords_boundaries(int8_t *chunked_indx, int32_t *ind_in_chnk,
                                int64_t *go_out, const double *coord,
                                int64_t x_cs, int64_t x_ps, const double *lims,
                                double xgrid0, double xgridc, int64_t nchnk,
                                int64_t np, void *ws, int64_t ws_bytes,
                                void *stream);

/* Stable order of the particles by chunk id, dropping ids outside
 * [0, nchnk): the permutation index2stay.argsort()[go_out:] of
 * species.py:379-383 (the reference's argsort is numpy's default, unstable
 * quicksort; this one keeps the particles' relative order inside a chunk).
 * idx_out (device int64) receives *n_kept (host) indices.  Synchronises. */
int64_t chm_chunk_order_ws_bytes(int64_t np, int64_t nchnk);
int chm_chunk_order(int64_t *idx_out, int64_t *n_kept, const int8_t *chunked_indx,
                    int64_t nchnk, int64_t np, void *ws, int64_t ws_bytes,
                    void *stream);

/* particle_tools.f90:270-324 align_data_vec / align_data_scl(dat, idx):
 * dst(:, i) = src(:, idx(i)) for i < n (idx device int64).  src and dst must
 * not overlap (the Fortran's temporary copy). */
int chm_align_data(double *dst, int64_t d_cs, int64_t d_ps, const double *src,
                   int64_t s_cs, int64_t s_ps, int64_t ncomp,
                   const int64_t *idx, int64_t n, void *stream);

/* ======================================================================== */
/* Split-precision form (a precision form of the same step; no counterpart  */
/* entry point in the reference): FP32 particles stored as int32 cell index +*/
/* FP32 offset, complex64 fields, DHT / coupling products on the tensor      */
/* cores as 3-term split-BF16 with FP32 accumulation.  FP64 stays in the     */
/* operator build and the window origin.                                     */
/* ======================================================================== */

/* A prepared per-mode operator set (DHT In/Out or DpS2S/DmS2S): FP32 copy
 * and split-BF16 terms in device memory owned by the caller. */
typedef struct {
  int32_t K, N, nmodes, pad;
  const float *f32;       /* (K, N, nmodes) column-major */
  const void *bf16[3];    /* split terms, tensor-core operand layout */
} chm_sp_ops;

/* Bytes of device memory chm_sp_prepare_ops needs for (K, N, nmodes). */
int64_t chm_sp_ops_bytes(int64_t K, int64_t N, int64_t nmodes);
/* Convert FP64 matrices mats(K, N, nmodes) (device) into `buf`, filling
 * *ops (host struct).  Used once per run (solvers.py:717-759 operators). */
int chm_sp_prepare_ops(chm_sp_ops *ops, const double *mats, int64_t K, int64_t N,
                       int64_t nmodes, void *buf, int64_t buf_bytes, void *stream);

/* Split-form particle storage: eight SoA arrays ix (int32), fx, y, z, px,
 * py, pz, w (float) in tiles of 512: particle i (its index in the species)
 * sits at slot chm_sp_slot(i) = (i / 512) * 512 + 32 (i % 16) + (i / 16) % 32,
 * so the 16 consecutive particles of a run belong to one GPU thread and a
 * warp's loads are contiguous.  Arrays (and the uint8 dead flags) hold
 * chm_sp_capacity(n) slots; slots of the last tile past n are not read.
 * Arrays start on 16-byte boundaries. */
int64_t chm_sp_capacity(int64_t n);
int64_t chm_sp_slot(int64_t i);

/* The moving window's origin in device memory, for the split-form entry
 * points below that take `win`: the grid's left edge leftX (FP64, for the
 * transforms' shift phases) and its position in cells from the particles'
 * origin X0, k + fd (k whole cells, fd in [0, 1) in FP64, f = fd in FP32).
 * chm_sp_window_set writes it from leftX (k = floor((leftX - X0) / dx));
 * chm_sp_window_advance adds a shift (leftX + shift, as the window moves:
 * chimera_main.py:286-290, and fd + shift / dx carried into k), so a move by
 * a whole number of cells keeps f exact and a step captured in a CUDA graph
 * replays with the current origin.  With win == NULL the entry points use
 * their scalar arguments (win_k, win_f, leftX). */
typedef struct {
  double leftX, X0, dx, fd;
  int32_t k;
  float f;
} chm_sp_window;
int chm_sp_window_set(chm_sp_window *win, double leftX, double X0, double dx,
                      void *stream);
int chm_sp_window_advance(chm_sp_window *win, double shift, void *stream);

/* Deterministic global deposit scale: scale2[0] = 2^min(61 - ceil(log2 B),
 * 120), scale2[1] = B = sum |w| (device doubles). */
int64_t chm_sp_scale_ws_bytes(void);
int chm_sp_weight_scale(double *scale2, const float *w, int64_t n, void *ws,
                        int64_t ws_bytes, void *stream);

/* push_coords + current deposit at the half step + charge deposit at the
 * new position, fused (particle_tools.f90:58-82, grid_deps.f90:18-147).
 * Particles: ix, fx, y, z, px, py, pz, w (n).  accJ (nx,nr,nm,3) and accR
 * (nx,nr,nm) are int64 {re, im} accumulators (either may be NULL) at the
 * scales scaleJ / scaleR.  win_k, win_f: window origin in cells.  push=0
 * deposits charge without moving (Still species). */
int chm_sp_push_deposit(int32_t *ix, float *fx, float *y, float *z, float *px,
                        float *py, float *pz, float *w, int64_t n, int win_k,
                        float win_f, float dx_inv, float dr_inv, float dt,
                        int nx, int nr, int nm, int push, uint64_t *accJ,
                        const double *scaleJ, uint64_t *accR,
                        const double *scaleR, void *stream,
                        const chm_sp_window *win);

/* proj_fld + push_velocs fused (grid_deps.f90:149-217,
 * particle_tools.f90:18-56): gather from the complex64 EB grid and Boris. */
int chm_sp_gather_push(int32_t *ix, float *fx, float *y, float *z, float *px,
                       float *py, float *pz, float *w, int64_t n, int win_k,
                       float win_f, float dr_inv, const void *eb_c64, int nx,
                       int nr, int nm, float dtq, void *stream,
                        const chm_sp_window *win);

/* The same two operations with the per-particle kernels for every nm (each
 * value rounded separately): the reference the cell-run kernels (nm <= 3)
 * are tested against.  The entry points above use the cell-run kernels for
 * nm <= 3 and these kernels beyond. */
int chm_sp_push_deposit_generic(int32_t *ix, float *fx, float *y, float *z,
                                float *px, float *py, float *pz, float *w,
                                int64_t n, int win_k, float win_f, float dx_inv,
                                float dr_inv, float dt, int nx, int nr, int nm,
                                int push, uint64_t *accJ, const double *scaleJ,
                                uint64_t *accR, const double *scaleR, void *stream,
                        const chm_sp_window *win);
int chm_sp_gather_push_generic(int32_t *ix, float *fx, float *y, float *z,
                               float *px, float *py, float *pz, float *w,
                               int64_t n, int win_k, float win_f, float dr_inv,
                               const void *eb_c64, int nx, int nr, int nm,
                               float dtq, void *stream,
                        const chm_sp_window *win);

/* Background density of a still species (the deposit of dep_bg,
 * chimera_main.py:220-248, with the run kernels, nm <= 3, n < 2^31) into
 * accR (nx,nr,nm) int64 {re, im} at the scale scaleR.  shift_cells = 0:
 * the full deposit (accR zeroed by the caller), recording each block's
 * cell range into ext (int2, at least ceil(n / 2048) entries).
 * shift_cells = ns > 0, after a window move by exactly ns cells with the
 * particles unchanged since the full deposit: the grid moves ns columns
 * left and only the blocks whose cells reach the ns entering columns
 * deposit there; bitwise the full deposit at the new window. */
int chm_sp_deposit_background(int32_t *ix, float *fx, float *y, float *z,
                              float *px, float *py, float *pz, float *w,
                              int64_t n, int win_k, float win_f, float dr_inv,
                              int nx, int nr, int nm, uint64_t *accR,
                              const double *scaleR, void *ext_int2,
                              int64_t ext_len, int shift_cells, void *stream,
                              const chm_sp_window *win);

/* Envelope (KxShift) solver, nm = 2K + 1 stored modes -K..K (K <= 2).
 * chm_sp_carrier fills tab (ntab >= nx + 4 complex64) with the carrier
 * e^{-i kx0 (X0 + (k + c - 2) dx)} of the window's cells c (k = the window
 * cell win->k, or win_k without a record), in FP64; the kernels below take
 * a particle's carrier as tab[ix - k + 2] e^{-i kdx fx}, kdx = kx0 dx, and
 * reject a table (ntab entries) shorter than nx + 4. */
int chm_sp_carrier(void *tab_c64, int64_t ntab, double kx0, double X0, double dx,
                   int win_k, void *stream, const chm_sp_window *win);
/* push_coords + dep_curr_env (particle_tools.f90:58-82,
 * grid_deps_env.f90:18-95): the coordinate push, then J_z only (the
 * reference's envelope deposit writes the third component alone) with
 * value (p_z / gamma) w e^{-i kx0 x} e^{-+i m theta} at mode slot K +- m,
 * into accJ (nx,nr,nm,3) int64 {re, im} at the scale scaleJ.  When a step
 * spans c dt / dx >= 2 cells (dt, dx in FP64), the x push takes the
 * light-speed step exactly and the slip (1 - v_x) separately. */
int chm_sp_push_deposit_env(int32_t *ix, float *fx, float *y, float *z,
                            float *px, float *py, float *pz, float *w, int64_t n,
                            int win_k, float win_f, float dx_inv, float dr_inv,
                            double dt, double dx, int nx, int nr, int nm,
                            uint64_t *accJ, const double *scaleJ,
                            const void *carrier_c64, int64_t ntab, float kdx,
                            void *stream, const chm_sp_window *win);
/* proj_fld_env + an undulator + push_velocs (grid_deps_env.f90:164-238,
 * devices.f90:18-203, particle_tools.f90:18-56): gather with the carrier
 * e^{+i kx0 x} and e^{+-i m theta} (1 on the axis), the undulator field at
 * the particle's x = X0 + (ix + fx) dx of und_kind 1 (undul_analytic: und =
 * a0, period, start, length), 2 (undul_analytic_taper: und = a0, period,
 * start, length, taper), 3 (undul_mapped: und = period, Xleft, map step;
 * und_map the map's nmap columns as FP32 pairs (a(0, c), a(1, c)), 8-byte
 * aligned device memory) or 4
 * (undul_mapped_tap: und = period, Xleft, map step, length, taper), 0 for
 * none, then the Boris push. */
int chm_sp_gather_push_env(int32_t *ix, float *fx, float *y, float *z,
                           float *px, float *py, float *pz, float *w, int64_t n,
                           int win_k, float win_f, float dr_inv,
                           const void *eb_c64, int nx, int nr, int nm, float dtq,
                           const void *carrier_c64, int64_t ntab, float kdx,
                           int und_kind, const double *und, const void *und_map,
                           int64_t nmap, double X0, double dx, void *stream,
                           const chm_sp_window *win);

/* FP64 (3,n)/(n) particle arrays (particle order) <-> split layout; from_f64
 * writes particles offset .. offset+n-1 and clears their dead flags (dead
 * may be NULL). */
int chm_sp_from_f64(int32_t *ix, float *fx, float *y, float *z, float *px,
                    float *py, float *pz, float *w, uint8_t *dead, int64_t offset,
                    const double *coord, int64_t x_cs, int64_t x_ps,
                    const double *momenta, int64_t p_cs, int64_t p_ps,
                    const double *wghts, int64_t w_ps, double X0, double dx,
                    int64_t n, void *stream);
int chm_sp_to_f64(const int32_t *ix, const float *fx, const float *y,
                  const float *z, const float *px, const float *py,
                  const float *pz, const float *w, int64_t n, double *coord,
                  int64_t x_cs, int64_t x_ps, double *momenta, int64_t p_cs,
                  int64_t p_ps, double *wghts, int64_t w_ps, double X0,
                  double dx, void *stream);
/* Absorbing boundary of the moving window (species.py:351-398, the SimDom
 * test of chunk_and_damp).  A live particle outside xmin <= x <= xmax,
 * y^2 + z^2 <= r2max (x in window cells) gets dead[i] = 1 and w = 0, so it
 * deposits nothing; counters[0] (device uint64) counts dead particles.
 * chm_sp_compact later drops them.  The same pass refreshes the deposit
 * scale of the surviving weights into scale2 (as chm_sp_weight_scale);
 * ws: chm_sp_scale_ws_bytes().  Arrays start on 16-byte boundaries. */
int chm_sp_absorb(const int32_t *ix, const float *fx, const float *y,
                  const float *z, float *w, uint8_t *dead, int64_t n, int win_k,
                  float win_f, float xmin_cells, float xmax_cells, float r2max,
                  uint64_t *counters, double *scale2, void *ws, int64_t ws_bytes,
                  void *stream);
/* counters[1] += n - counters[0] (live particles of the step, for rates). */
int chm_sp_count_live(uint64_t *counters, int64_t n, void *stream);
/* Stable compaction of the particles with dead[i] == 0 into the *_out
 * arrays; *n_out (device int64) receives their number.  n < 2^31. */
int64_t chm_sp_compact_ws_bytes(int64_t n);
int chm_sp_compact(const int32_t *ix, const float *fx, const float *y,
                   const float *z, const float *px, const float *py,
                   const float *pz, const float *w, const uint8_t *dead, int64_t n,
                   int32_t *ix_out, float *fx_out, float *y_out, float *z_out,
                   float *px_out, float *py_out, float *pz_out, float *w_out,
                   int64_t *n_out, void *ws, int64_t ws_bytes, void *stream);

/* Re-sort of the particles by deposit cell (the reference re-buckets its
 * particles by x chunk at a cadence: chimera_main.py:306-318,
 * species.py:351-398, particle_tools.f90:155-208): a stable sort of the
 * live particles by the key of their deposit cell -- 4 x 4-cell patches of
 * generation cells (x cells from the window origin win_k, r cells of width
 * 1 / dr_inv) in serpentine order, the cells of a patch in serpentine order,
 * then the lower or upper deposit cell of the generation cell -- written in
 * tile layout to the *_out arrays (the capacity of the input); dead
 * particles are dropped and *n_out (device int64) receives the live count.
 * The key of a particle is (((((pr P + px') 4 + lr) 4 + lx') 2 + half) 16
 * + 4 qx + qr with gx = min(max(ix - win_k + 8, 0), nx + 24), gr =
 * min(floor(s), nr + 4), s = sqrt(y y + z z) dr_inv, fr = s - floor(s),
 * half = (fr >= 0.5), px = gx / 4, lx = gx % 4, pr = gr / 4, lr = gr % 4,
 * P = (nx + 24) / 4 + 1, px' = pr odd ? P - 1 - px : px, lx' = lr odd ?
 * 3 - lx : lx, and the quarter of the deposit cell qx = min(3, floor(4 sx)),
 * qr = min(3, floor(4 sr)) with d = fx - win_f, sx = d - floor(d), sr =
 * half ? fr - 1/2 : fr + 1/2 (each operation rounded in FP32); ties keep the
 * slot order.  n < 2^31. */
int64_t chm_sp_sort_ws_bytes(int64_t n);
int chm_sp_sort_cells(const int32_t *ix, const float *fx, const float *y,
                      const float *z, const float *px, const float *py,
                      const float *pz, const float *w, const uint8_t *dead,
                      int64_t n, int win_k, float win_f, int nx, int nr,
                      float dr_inv, int32_t *ix_out, float *fx_out, float *y_out, float *z_out,
                      float *px_out, float *py_out, float *pz_out, float *w_out,
                      int64_t *n_out, void *ws, int64_t ws_bytes, void *stream);

/* Spectral stage on complex64 (nx, nkr, nm, comps) planes. */
int64_t chm_sp_fb_ws_bytes(int64_t nx, int64_t nr, int64_t nkr, int64_t nm);
int chm_sp_fb_in_acc(void *out_c64, const int64_t *acc, const double *scale,
                     const int64_t *acc2, const double *scale2, double leftX,
                     const double *kx, const void *In_ops, const float *fact,
                     int64_t nx, int64_t nr, int64_t nkr, int64_t nm,
                     int64_t ncomp, void *ws, int64_t ws_bytes, void *stream,
                        const chm_sp_window *win);
int chm_sp_fb_eb_out(void *eb_c64, const void *e_c64, const void *b_c64,
                     double leftX, const double *kx, const void *Out_ops,
                     int64_t nx, int64_t nr, int64_t nkr, int64_t nm, void *ws,
                     int64_t ws_bytes, void *stream,
                        const chm_sp_window *win);
/* fb_eb_out with the envelope solver's eb_correction
 * (grid_deps_env.f90:240-283): 1/pi for every mode, the ghost row -1 times
 * row 1 unless nm = 1.  kx: the envelope's kx_env. */
int chm_sp_fb_eb_out_env(void *eb_c64, const void *e_c64, const void *b_c64,
                         double leftX, const double *kx, const void *Out_ops,
                         int64_t nx, int64_t nr, int64_t nkr, int64_t nm,
                         void *ws, int64_t ws_bytes, void *stream,
                         const chm_sp_window *win);
int chm_sp_fb_filtr(void *vec_c64, double leftX, const double *kx,
                    const float *filtr, int64_t nxfilt, int modefilt,
                    int64_t nx, int64_t nkr, int64_t nm, int64_t ncomp,
                    void *ws, int64_t ws_bytes, void *stream,
                        const chm_sp_window *win);
int chm_sp_fb_grad(void *out_c64, const void *scl_c64, const void *Dp_ops,
                   const void *Dm_ops, const float *kx, int64_t nx,
                   int64_t nkr, int64_t nm, void *ws, int64_t ws_bytes,
                   void *stream);
int chm_sp_poisson(void *J_c64, const void *gprv_c64, const void *gnxt_c64,
                   const float *pf, float dt_inv, const void *Dp_ops,
                   const void *Dm_ops, const float *kx, int64_t nx,
                   int64_t nkr, int64_t nm, int iters, int space_charge,
                   void *ws, int64_t ws_bytes, void *stream);
/* chm_sp_poisson followed by chm_sp_psatd (maxwell_push_with_spchrg /
 * maxwell_push_wo_spchrg, maxwell_solvers.f90:18-96) in one pass: the last
 * J update of the correction also advances E and G of eg_c64 (nx, nkr, nm,
 * 6) with the FP32 coefficients c1, c2 (nx, nkr, nm, nterm); nterm 5 with
 * space charge, 3 without.  Bitwise the two calls' result. */
int chm_sp_poisson_psatd(void *J_c64, const void *gprv_c64, const void *gnxt_c64,
                         const float *pf, float dt_inv, const void *Dp_ops,
                         const void *Dm_ops, const float *kx, int64_t nx,
                         int64_t nkr, int64_t nm, int iters, int space_charge,
                         void *eg_c64, const float *c1, const float *c2, int nterm,
                         void *ws, int64_t ws_bytes, void *stream);
int chm_sp_rot_b(void *B_c64, const void *G_c64, const float *pf,
                 const void *Dp_ops, const void *Dm_ops, const float *kx,
                 int64_t nx, int64_t nkr, int64_t nm, void *ws,
                 int64_t ws_bytes, void *stream);
int chm_sp_psatd(void *eg_c64, const void *j_c64, const void *gprv_c64,
                 const void *gnxt_c64, const float *c1, const float *c2,
                 int nterm, int64_t P, void *stream);
/* The envelope curl B = rot_env(G) * PoissFact (fb_math_env.f90 curl on
 * the stored modes -K..K, Dp/Dm holding the modes -K-1..K+1; no
 * lower-neighbour term in the first component) and the PSATD update without
 * space charge with complex64 coefficients c1, c2 (nx, nkr, nm, 3)
 * (maxwell_push_wo_spchrg, maxwell_solvers.f90:62-96). */
int chm_sp_rot_b_env(void *B_c64, const void *G_c64, const float *pf,
                     const void *Dp_ops, const void *Dm_ops, const float *kx,
                     int64_t nx, int64_t nkr, int64_t nm, void *ws,
                     int64_t ws_bytes, void *stream);
int chm_sp_psatd_c(void *eg_c64, const void *j_c64, const void *c1_c64,
                   const void *c2_c64, int64_t P, void *stream);
/* Dense product C(M,N) = A(M,K) B(K,N) with B a prepared operator mode, on
 * the tensor cores (tcgen05, split-BF16) or, with engine = 0, on the FP32
 * SIMT path; for tests and tuning. */
int64_t chm_sp_gemm_ws_bytes(int64_t M, int64_t K, int64_t count);
int chm_sp_gemm(float *C, const float *A, const chm_sp_ops *ops, int64_t mode,
                int64_t M, int engine, void *ws, int64_t ws_bytes, void *stream);
/* Nonzero if a tensor-core GEMM CTA hit a wait limit since the last call
 * (then reset): 1 or 3 the operand pipeline, 4 an accumulator hand-over,
 * 2 the final drain.  The CTA that gave up wrote no output. */
int chm_sp_umma_status(void);
/* Column-tile width of the tensor-core products for launches after this
 * call: -1 picks it per shape (M, N, K, batch count, epilogue) by timing
 * every candidate on the first launch of the shape outside stream capture
 * (the default), 0 the default width (N rounded up to 16 and cut into the
 * fewest tiles of at most 128 columns), > 0 that width where it is a
 * candidate (a multiple of 16, at least 32, dividing the padded N), else
 * the default.  The width changes no output bit.  Returns the previous
 * mode. */
int chm_sp_set_umma_cols(int mode);
/* The widths picked so far: up to max_shapes records of six int32 (M, N,
 * K, batch count, epilogue, width) into out (may be null); returns the
 * number of shapes tuned. */
int chm_sp_umma_tuned(int32_t *out, int max_shapes);
/* Forgets the tuned widths (the next launch of each shape tunes again). */
int chm_sp_umma_tune_reset(void);
/* Iteration limit of the tensor-core GEMM's pipeline waits for launches
 * after this call (polls of mbarrier.try_wait; < 0 restores the default
 * 2^20); returns the previous limit.  A test hook: with 0 every pipeline
 * wait gives up at once, and the kernel must report it and free its tensor
 * memory (its clean-up waits keep the default limit). */
int64_t chm_sp_set_umma_spin_limit(int64_t polls);
/* Deposit cells of the split-form run kernels that fell outside their
 * block's box while inside the grid since the last call (then reset).  The
 * block plan bounds every finite particle's deposit cells, so this is 0
 * unless positions are corrupt (NaN or moved faster than c). */
int64_t chm_sp_deposit_dropped(void);

/* Plasma generation (particle_tools.f90:84-128 genparts, fixed per-cell
 * pattern; species.py:132-215): particle (ir, ix, ip) of the nrc x nxc cells
 * and npc pattern points is written at row_base[ir] + ix row_count[ir] +
 * row_rank[ir + nrc ip] (row_rank < 0: dropped) with x = cx[ix + nxc ip],
 * (y, z) = cr[ir + nrc ip] (Im, Re) of packo[ip] e^{2 pi i rand_o[ix + ldr ir]},
 * weight = cr[ir + nrc ip] wfac[ix + nxc ip].  coords: (3, n) with component
 * stride cstride, part stride 1; packo complex128 (npc). */
int chm_gen_fixed_cell(double *coords, int64_t cstride, double *weights, const double *cx,
                       const double *cr, const double *wfac, const double *packo,
                       const double *rand_o, int64_t ldr, const int64_t *row_base,
                       const int32_t *row_rank, const int32_t *row_count, int64_t nxc, int64_t nrc,
                       int64_t npc, void *stream);

/* ------------------------------------------------------------------------
 * Diagnostics (moduls/diagnostics.py, f90/utils.f90): device reductions of
 * the FP64 grids, each in a fixed summation order (bitwise reproducible).
 * ------------------------------------------------------------------------ */
/* nrg_out (diagnostics.py:109-122), before its fftshift-style reordering:
 * out[x] = sum_{kr, m} efact(x, kr, m) * sum_{l < 3} |eg(x, kr, m, l)|^2.
 * eg: (nx, nkr, nm, ncomp) complex128 with the E field in components 0-2
 * (the solver's EG_fb, ncomp = 6); efact: (nx, nkr, nm) EnergyFact
 * (solvers.py:143-149); out: nx doubles. */
int chm_em_energy(double *out, const chm_c128 *eg, const double *efact, int64_t nx, int64_t nkr,
                  int64_t nm, int64_t ncomp, void *stream);
/* pwr_out (diagnostics.py:124-149), power per x of a spatial field:
 * out[x] = fac * sum_r rgrid[r] * sum_{m, l} |vec(x, r, m, l)|^2 with vec
 * (nx, nr, nm, 3) complex128 (fb_vec_out of EG_fb[..., :3]), rgrid (nr)
 * (RgridFull) and fac = PwrFctr * 2 dr. */
int chm_power_profile(double *out, const chm_c128 *vec, const double *rgrid, double fac, int64_t nx,
                      int64_t nr, int64_t nm, void *stream);
/* intens_profO (utils.f90:18-57): pwr (NO, NR - 1) with
 * pwr(iO, ir) = sum_l sum_ix |sum_k e^{i k 2 pi iO / (NO - 1)} fld(ix, ir, k, l)|^2
 * for iO = 0 .. NO - 1, ir = 1 .. NR - 1 and k = -K .. K; fld is
 * (NX, NR, NM = 2K + 1, 3) complex128 (the Fortran's Fld(0:nx, 0:nr,
 * -nkO:nkO, 3); f2py infers nkO, so NM is odd). */
int chm_intens_profo(double *pwr, const chm_c128 *fld, int64_t NO, int64_t NX, int64_t NR,
                     int64_t NM, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CHIMERA_GB300_H */
