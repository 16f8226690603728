// Deterministic charge / current deposition (grid_deps*.f90), FP64.
//
// Each particle's 2x2-node x (modes) x (components) complex contribution is
// converted to 64-bit fixed point and summed with integer atomics.  Integer
// addition is associative, so the accumulated grid is bitwise identical
// whatever order the particles are processed in: no float atomics reach
// memory and two runs give the same bits.
//
// The fixed-point scale is a power of two chosen from a deterministic bound
// B >= sum_p |w_p| (|w_p|^2 for the envelope density, which applies the
// weight twice): scale = 2^(61 - ceil(log2 B)), so no partial sum can
// overflow and the quantum is B * 2^-61 (~1e-18 relative to B).
//
// Work is privatised per thread block: each block takes a contiguous range
// of particles, and when the cells they touch fit a shared-memory box the
// block accumulates there and flushes the box once with global integer
// atomics; otherwise it adds straight to the global accumulator.  Particles
// kept in cell order (genparts order or after a sort) almost always fit.
#include <climits>
#include <math.h>

#include "common.cuh"

using namespace chm;

namespace {

constexpr int kDepThreads = 256;
constexpr int kPartPerBlock = 1024;  // particles per block
constexpr int kBoxBytes = 96 * 1024;  // shared accumulator budget
constexpr int kRedBlocks = 1024;

enum Kind { CURR = 0, DENS = 1, CURR_ENV = 2, DENS_ENV = 3 };

__host__ __device__ constexpr int ncomp_of(int kind) { return (kind == CURR || kind == CURR_ENV) ? 3 : 1; }

// Deterministic partial sums of |w| (or w^2), fixed tree order.
__global__ void wsum_partial_kernel(const double *__restrict__ w, i64 w_ps, i64 np, int squared,
                                    double *__restrict__ partial) {
  __shared__ double sh[kDepThreads];
  i64 per = (np + gridDim.x - 1) / gridDim.x;
  i64 b0 = blockIdx.x * per, b1 = min(np, b0 + per);
  double s = 0.0;
  for (i64 i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
    double v = fabs(w[i * w_ps]);
    s += squared ? v * v : v;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void wsum_final_kernel(const double *__restrict__ partial, int n, double *scale_out) {
  __shared__ double sh[kRedBlocks];
  for (int i = threadIdx.x; i < kRedBlocks; i += blockDim.x) sh[i] = i < n ? partial[i] : 0.0;
  __syncthreads();
  for (int st = kRedBlocks / 2; st > 0; st >>= 1) {
    for (int i = threadIdx.x; i < st; i += blockDim.x) sh[i] += sh[i + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double B = sh[0];
    if (!(B > 0.0) || !isfinite(B)) B = 1.0;
    int e;
    frexp(B, &e);  // B < 2^e
    scale_out[0] = ldexp(1.0, 61 - e);
  }
}

__global__ void set_one_kernel(double *p) { p[0] = 1.0; }

struct DepArgs {
  const double *x;
  i64 x_cs, x_ps;
  const double *p;
  i64 p_cs, p_ps;
  const double *w;
  i64 w_ps;
  double leftX, dx_inv, dr_inv, kx0;
  const double *rgrid;
  i64 np, nx, nr;
  int nm;
  const int32_t *ind;  // chunk offsets or null
  int nchnk;
  i64 cs, guards;
  unsigned long long *acc;  // (nx, nr, nm, ncomp) x {re, im} int64
  const double *scale;
};

__device__ __forceinline__ void put(unsigned long long *a, double v, double scale) {
  long long q = __double2ll_rn(v * scale);
  if (q != 0) atomicAdd(a, (unsigned long long)q);
}

// Contribution of one particle; `emit(ml, r, x, value)` receives the
// (mode + nm*component, r node, x node) of every accepted stencil node.
template <int KIND, typename Emit>
__device__ __forceinline__ void particle_contrib(const DepArgs &A, i64 i, int chunk, Emit emit) {
  const double wp = A.w[i * A.w_ps];
  if (wp == 0.0) return;
  const double xp = A.x[i * A.x_ps], yp = A.x[A.x_cs + i * A.x_ps], zp = A.x[2 * A.x_cs + i * A.x_ps];
  const double rp = sqrt(yp * yp + zp * zp);
  const double rmax = A.rgrid[A.nr - 1];
  double v[3] = {0.0, 0.0, 0.0};
  if (KIND == CURR || KIND == CURR_ENV) {
    v[0] = A.p[i * A.p_ps];
    v[1] = A.p[A.p_cs + i * A.p_ps];
    v[2] = A.p[2 * A.p_cs + i * A.p_ps];
    if (!(rp < rmax) || (fabs(v[0]) + fabs(v[1]) + fabs(v[2])) == 0.0) return;
    double gp = sqrt(1.0 + v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = (KIND == CURR) ? v[c] * wp / gp : v[c] / gp;
  } else {
    if (!(rp < rmax)) return;
  }
  double2 wc = make_double2(wp, 0.0);
  if (KIND == CURR_ENV || KIND == DENS_ENV) {
    double s, c;
    sincos(xp * A.kx0, &s, &c);
    wc = make_double2(wp * c, -wp * s);
  }
  const double fx = (xp - A.leftX) * A.dx_inv;
  if (!(fx > -1.0e15 && fx < 1.0e15)) return;
  const i64 ix = (i64)floor(fx);
  const i64 ir = (i64)floor((rp - A.rgrid[0]) * A.dr_inv);
  if (ir < 0 || ir > A.nr - 2) return;
  const double sx[2] = {1.0 - (fx - (double)ix), fx - (double)ix};
  const double sr1 = (rp - A.rgrid[ir]) * A.dr_inv;
  const double sr[2] = {1.0 - sr1, sr1};
  const double2 ph = (rp > 0.0) ? make_double2(yp / rp, -zp / rp) : make_double2(0.0, 0.0);

  // x-node acceptance (grid bounds + chunk guard semantics)
  bool okx[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    i64 gx = ix + k;
    bool ok = (gx >= 0 && gx < A.nx);
    if (ok && A.ind) {
      i64 nxleft = (i64)chunk * A.cs;
      i64 lx = gx - nxleft;
      if (lx <= 0) ok = (nxleft - A.guards >= 0) && (lx >= -A.guards);
      else if (lx >= A.cs) ok = (nxleft + A.cs + A.guards <= A.nx - 1) && (lx <= A.cs + A.guards);
    }
    okx[k] = ok;
  }
  const int ncomp = ncomp_of(KIND);
  const bool env = (KIND == CURR_ENV || KIND == DENS_ENV);
  const int K = env ? (A.nm - 1) / 2 : 0;
  const int nph = env ? K + 1 : A.nm;
  double2 phm = make_double2(1.0, 0.0);
  for (int mi = 0; mi < nph; ++mi) {
    if (mi > 0) phm = cmul(phm, ph);
    for (int side = 0; side < ((env && mi > 0) ? 2 : 1); ++side) {
      const double2 pm = side ? cconj(phm) : phm;
      const int slot = env ? (side ? K - mi : K + mi) : mi;
      for (int l = 0; l < ncomp; ++l) {
        if (KIND == CURR_ENV && l != 2) continue;  // grid_deps_env.f90:76
        double2 val;
        if (KIND == CURR) val = cscale(pm, v[l]);
        else if (KIND == DENS) val = cscale(pm, wp);
        else if (KIND == CURR_ENV) val = cmul(cscale(pm, v[l]), wc);
        else val = cmul(pm, cmul(wc, wc));
        const i64 ml = slot + (i64)A.nm * l;
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
          for (int k = 0; k < 2; ++k)
            if (okx[k]) emit(ml, ir + j, ix + k, cscale(val, sx[k] * sr[j]));
      }
    }
  }
}

__device__ __forceinline__ int chunk_of(const int32_t *ind_sh, int nchnk, i64 i) {
  // ind_sh sorted; returns c with ind[c] <= i < ind[c+1], or -1
  if (i < ind_sh[0] || i >= ind_sh[nchnk]) return -1;
  int lo = 0, hi = nchnk;  // invariant ind[lo] <= i < ind[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (ind_sh[mid] <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <int KIND>
__global__ void __launch_bounds__(kDepThreads) deposit_kernel(DepArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int32_t ind_sh[257];
  __shared__ long long box_sh[4];  // ixmin, ixmax, irmin, irmax
  const double scale = A.scale[0];
  const i64 p0 = (i64)blockIdx.x * kPartPerBlock;
  const i64 p1 = min(A.np, p0 + kPartPerBlock);
  if (A.ind) {
    for (int t = threadIdx.x; t <= A.nchnk; t += blockDim.x) ind_sh[t] = A.ind[t];
  }
  if (threadIdx.x == 0) {
    box_sh[0] = LLONG_MAX;
    box_sh[1] = LLONG_MIN;
    box_sh[2] = LLONG_MAX;
    box_sh[3] = LLONG_MIN;
  }
  __syncthreads();
  // 1) bounding box of the cells touched by this block
  {
    long long bx0 = LLONG_MAX, bx1 = LLONG_MIN, br0 = LLONG_MAX, br1 = LLONG_MIN;
    for (i64 i = p0 + threadIdx.x; i < p1; i += blockDim.x) {
      const double xp = A.x[i * A.x_ps], yp = A.x[A.x_cs + i * A.x_ps],
                   zp = A.x[2 * A.x_cs + i * A.x_ps];
      const double rp = sqrt(yp * yp + zp * zp);
      const double fx = (xp - A.leftX) * A.dx_inv;
      if (!(fx > -1.0e15 && fx < 1.0e15) || !(rp < 1.0e300)) continue;
      long long ix = (long long)floor(fx), ir = (long long)floor((rp - A.rgrid[0]) * A.dr_inv);
      bx0 = min(bx0, ix);
      bx1 = max(bx1, ix + 1);
      br0 = min(br0, ir);
      br1 = max(br1, ir + 1);
    }
    // warp reduce then one atomic per warp (integer min/max: order-free)
    for (int o = 16; o > 0; o >>= 1) {
      bx0 = min(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
      bx1 = max(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
      br0 = min(br0, __shfl_xor_sync(0xffffffffu, br0, o));
      br1 = max(br1, __shfl_xor_sync(0xffffffffu, br1, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&box_sh[0], bx0);
      atomicMax(&box_sh[1], bx1);
      atomicMin(&box_sh[2], br0);
      atomicMax(&box_sh[3], br1);
    }
  }
  __syncthreads();
  const long long bx0 = max(box_sh[0], 0LL), bx1 = min(box_sh[1], (long long)A.nx - 1);
  const long long br0 = max(box_sh[2], 0LL), br1 = min(box_sh[3], (long long)A.nr - 1);
  const int ncomp = ncomp_of(KIND);
  const long long bnx = bx1 - bx0 + 1, bnr = br1 - br0 + 1;
  const long long nvals = (bnx > 0 && bnr > 0) ? bnx * bnr * A.nm * ncomp * 2 : 0;
  const bool use_box = nvals > 0 && nvals * 8 <= kBoxBytes;
  unsigned long long *box = reinterpret_cast<unsigned long long *>(smem_raw);
  if (use_box) {
    for (long long t = threadIdx.x; t < nvals; t += blockDim.x) box[t] = 0ull;
  }
  __syncthreads();
  for (i64 i = p0 + threadIdx.x; i < p1; i += blockDim.x) {
    int chunk = 0;
    if (A.ind) {
      chunk = chunk_of(ind_sh, A.nchnk, i);
      if (chunk < 0) continue;
    }
    if (use_box) {
      particle_contrib<KIND>(A, i, chunk, [&](i64 ml, i64 gr, i64 gx, double2 v) {
        i64 b = ((ml * bnr + (gr - br0)) * bnx + (gx - bx0)) * 2;
        long long qx = __double2ll_rn(v.x * scale), qy = __double2ll_rn(v.y * scale);
        if (qx) atomicAdd(&box[b], (unsigned long long)qx);
        if (qy) atomicAdd(&box[b + 1], (unsigned long long)qy);
      });
    } else {
      particle_contrib<KIND>(A, i, chunk, [&](i64 ml, i64 gr, i64 gx, double2 v) {
        const i64 e = (ml * A.nr + gr) * A.nx + gx;
        put(&A.acc[2 * e], v.x, scale);
        put(&A.acc[2 * e + 1], v.y, scale);
      });
    }
  }
  if (use_box) {
    __syncthreads();
    for (long long t = threadIdx.x; t < nvals; t += blockDim.x) {
      unsigned long long q = box[t];
      if (q == 0ull) continue;
      long long c2 = t & 1;
      long long b = t >> 1;
      long long bx = b % bnx;
      long long rest = b / bnx;
      long long br = rest % bnr;
      long long ml = rest / bnr;
      i64 e = (ml * A.nr + (br + br0)) * A.nx + (bx + bx0);
      atomicAdd(&A.acc[2 * e + c2], q);
    }
  }
}

// out = existing + acc / scale, then the ghost-row fold
// (grid_deps.f90:80-84): row1 -= row0; row0 = 0.
__global__ void finalize_kernel(double2 *__restrict__ out, const long long *__restrict__ acc,
                                const double *__restrict__ scale_p, i64 nx, i64 nr, i64 nml) {
  const double inv = 1.0 / scale_p[0];
  const i64 n = nx * nr * nml;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < n;
       t += (i64)gridDim.x * blockDim.x) {
    const i64 x = t % nx;
    const i64 rest = t / nx;
    const i64 r = rest % nr;
    if (r == 0) continue;
    double2 v = out[t];
    v.x += (double)acc[2 * t] * inv;
    v.y += (double)acc[2 * t + 1] * inv;
    if (r == 1) {
      const i64 t0 = t - nx;
      double2 g = out[t0];
      g.x += (double)acc[2 * t0] * inv;
      g.y += (double)acc[2 * t0 + 1] * inv;
      v = csub(v, g);
      out[t0] = make_double2(0.0, 0.0);
    }
    out[t] = v;
    (void)x;
  }
}

int deposit_common(int kind, const double *coord, i64 x_cs, i64 x_ps, const double *momenta,
                   i64 p_cs, i64 p_ps, const double *wghts, i64 w_ps, chm_c128 *grid,
                   const int32_t *ind, i64 nchnk, i64 guards, double leftX,
                   const double *rgrid, double dx_inv, double dr_inv, double kx0, i64 np, i64 nx,
                   i64 nr, i64 nm, void *ws, i64 ws_bytes, void *stream) {
  const int ncomp = ncomp_of(kind);
  CHM_REQUIRE(np >= 0 && nx > 1 && nr > 1 && nm >= 1, "deposit: bad dims");
  CHM_REQUIRE(kind < 2 || (nm % 2 == 1), "deposit env: nm must be odd");
  CHM_REQUIRE(grid && rgrid, "deposit: null grid/rgrid");
  CHM_REQUIRE(!ind || (nchnk >= 1 && nchnk <= 256), "deposit: nchnk must be in [1, 256]");
  const i64 need = chm_dep_ws_bytes(nx, nr, nm, ncomp, np);
  if (!ws || ws_bytes < need) {
    set_error("deposit: workspace %lld bytes < %lld required", (long long)ws_bytes,
              (long long)need);
    return CHM_ERR_WS;
  }
  cudaStream_t st = as_stream(stream);
  const i64 nacc = nx * nr * nm * ncomp * 2;
  unsigned long long *acc = reinterpret_cast<unsigned long long *>(ws);
  double *partial = reinterpret_cast<double *>(acc + nacc);
  double *scale = partial + kRedBlocks;
  if (cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * nacc, st) != cudaSuccess) {
    set_error("deposit: memset failed");
    return CHM_ERR_CUDA;
  }
  if (np > 0) {
    CHM_REQUIRE(coord && wghts && (ncomp == 1 || momenta), "deposit: null particle array");
    wsum_partial_kernel<<<kRedBlocks, kDepThreads, 0, st>>>(wghts, w_ps, np, kind == DENS_ENV,
                                                            partial); chm::count_launch();
    wsum_final_kernel<<<1, 256, 0, st>>>(partial, kRedBlocks, scale); chm::count_launch();
    DepArgs A{};
    A.x = coord;
    A.x_cs = x_cs;
    A.x_ps = x_ps;
    A.p = momenta;
    A.p_cs = p_cs;
    A.p_ps = p_ps;
    A.w = wghts;
    A.w_ps = w_ps;
    A.leftX = leftX;
    A.dx_inv = dx_inv;
    A.dr_inv = dr_inv;
    A.kx0 = kx0;
    A.rgrid = rgrid;
    A.np = np;
    A.nx = nx;
    A.nr = nr;
    A.nm = (int)nm;
    A.ind = ind;
    A.nchnk = (int)nchnk;
    A.cs = ind ? nx / nchnk : nx;
    A.guards = guards;
    A.acc = acc;
    A.scale = scale;
    const unsigned blocks = (unsigned)((np + kPartPerBlock - 1) / kPartPerBlock);
    switch (kind) {
#define LAUNCH(K)                                                                         \
  case K:                                                                                 \
    cudaFuncSetAttribute(deposit_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                         kBoxBytes);                                                      \
    deposit_kernel<K><<<blocks, kDepThreads, kBoxBytes, st>>>(A); chm::count_launch();                         \
    break;
      LAUNCH(CURR)
      LAUNCH(DENS)
      LAUNCH(CURR_ENV)
      LAUNCH(DENS_ENV)
#undef LAUNCH
    }
    CHM_CHECK_LAUNCH();
  } else {
    // nothing deposited: only the fold of the existing content
    set_one_kernel<<<1, 1, 0, st>>>(scale); chm::count_launch();
  }
  const i64 nml = nm * ncomp;
  finalize_kernel<<<grid_for(nx * nr * nml, 256), 256, 0, st>>>(
      reinterpret_cast<double2 *>(grid), reinterpret_cast<const long long *>(acc), scale, nx,
      nr, nml); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // namespace

extern "C" {

int64_t chm_dep_ws_bytes(int64_t nx, int64_t nr, int64_t nm, int64_t ncomp, int64_t np) {
  (void)np;
  return 8 * (nx * nr * nm * ncomp * 2) + 8 * kRedBlocks + 256;
}

int chm_dep_curr(const double *coord, int64_t x_cs, int64_t x_ps, const double *momenta,
                 int64_t p_cs, int64_t p_ps, const double *wghts, int64_t w_ps, chm_c128 *curr,
                 double leftX, const double *rgrid, double dx_inv, double dr_inv, int64_t np,
                 int64_t nx, int64_t nr, int64_t nm, void *ws, int64_t ws_bytes, void *stream) {
  return deposit_common(CURR, coord, x_cs, x_ps, momenta, p_cs, p_ps, wghts, w_ps, curr, nullptr,
                        0, 0, leftX, rgrid, dx_inv, dr_inv, 0.0, np, nx, nr, nm, ws, ws_bytes,
                        stream);
}

int chm_dep_dens(const double *coord, int64_t x_cs, int64_t x_ps, const double *wghts,
                 int64_t w_ps, chm_c128 *dens, double leftX, const double *rgrid, double dx_inv,
                 double dr_inv, int64_t np, int64_t nx, int64_t nr, int64_t nm, void *ws,
                 int64_t ws_bytes, void *stream) {
  return deposit_common(DENS, coord, x_cs, x_ps, nullptr, 0, 0, wghts, w_ps, dens, nullptr, 0, 0,
                        leftX, rgrid, dx_inv, dr_inv, 0.0, np, nx, nr, nm, ws, ws_bytes, stream);
}

int chm_dep_curr_env(const double *coord, int64_t x_cs, int64_t x_ps, const double *momenta,
                     int64_t p_cs, int64_t p_ps, const double *wghts, int64_t w_ps,
                     chm_c128 *curr, double leftX, const double *rgrid, double dx_inv,
                     double dr_inv, double kx0, int64_t np, int64_t nx, int64_t nr, int64_t nm,
                     void *ws, int64_t ws_bytes, void *stream) {
  return deposit_common(CURR_ENV, coord, x_cs, x_ps, momenta, p_cs, p_ps, wghts, w_ps, curr,
                        nullptr, 0, 0, leftX, rgrid, dx_inv, dr_inv, kx0, np, nx, nr, nm, ws,
                        ws_bytes, stream);
}

int chm_dep_dens_env(const double *coord, int64_t x_cs, int64_t x_ps, const double *wghts,
                     int64_t w_ps, chm_c128 *dens, double leftX, const double *rgrid,
                     double dx_inv, double dr_inv, double kx0, int64_t np, int64_t nx, int64_t nr,
                     int64_t nm, void *ws, int64_t ws_bytes, void *stream) {
  return deposit_common(DENS_ENV, coord, x_cs, x_ps, nullptr, 0, 0, wghts, w_ps, dens, nullptr, 0,
                        0, leftX, rgrid, dx_inv, dr_inv, kx0, np, nx, nr, nm, ws, ws_bytes,
                        stream);
}

int chm_dep_curr_chnk(const double *coord, int64_t x_cs, int64_t x_ps, const double *momenta,
                      int64_t p_cs, int64_t p_ps, const double *wghts, int64_t w_ps,
                      chm_c128 *curr, const int32_t *ind_in_chunk, int64_t nchnk, int64_t guards,
                      double leftX, const double *rgrid, double dx_inv, double dr_inv,
                      int64_t np, int64_t nx, int64_t nr, int64_t nm, void *ws, int64_t ws_bytes,
                      void *stream) {
  CHM_REQUIRE(ind_in_chunk, "dep_curr_chnk: null IndInChunk");
  return deposit_common(CURR, coord, x_cs, x_ps, momenta, p_cs, p_ps, wghts, w_ps, curr,
                        ind_in_chunk, nchnk, guards, leftX, rgrid, dx_inv, dr_inv, 0.0, np, nx,
                        nr, nm, ws, ws_bytes, stream);
}

int chm_dep_dens_chnk(const double *coord, int64_t x_cs, int64_t x_ps, const double *wghts,
                      int64_t w_ps, chm_c128 *dens, const int32_t *ind_in_chunk, int64_t nchnk,
                      int64_t guards, double leftX, const double *rgrid, double dx_inv,
                      double dr_inv, int64_t np, int64_t nx, int64_t nr, int64_t nm, void *ws,
                      int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(ind_in_chunk, "dep_dens_chnk: null IndInChunk");
  return deposit_common(DENS, coord, x_cs, x_ps, nullptr, 0, 0, wghts, w_ps, dens, ind_in_chunk,
                        nchnk, guards, leftX, rgrid, dx_inv, dr_inv, 0.0, np, nx, nr, nm, ws,
                        ws_bytes, stream);
}

int chm_dep_curr_env_chnk(const double *coord, int64_t x_cs, int64_t x_ps, const double *momenta,
                          int64_t p_cs, int64_t p_ps, const double *wghts, int64_t w_ps,
                          chm_c128 *curr, const int32_t *ind_in_chunk, int64_t nchnk,
                          int64_t guards, double leftX, const double *rgrid, double dx_inv,
                          double dr_inv, double kx0, int64_t np, int64_t nx, int64_t nr,
                          int64_t nm, void *ws, int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(ind_in_chunk, "dep_curr_env_chnk: null IndInChunk");
  return deposit_common(CURR_ENV, coord, x_cs, x_ps, momenta, p_cs, p_ps, wghts, w_ps, curr,
                        ind_in_chunk, nchnk, guards, leftX, rgrid, dx_inv, dr_inv, kx0, np, nx,
                        nr, nm, ws, ws_bytes, stream);
}

int chm_dep_dens_env_chnk(const double *coord, int64_t x_cs, int64_t x_ps, const double *wghts,
                          int64_t w_ps, chm_c128 *dens, const int32_t *ind_in_chunk,
                          int64_t nchnk, int64_t guards, double leftX, const double *rgrid,
                          double dx_inv, double dr_inv, double kx0, int64_t np, int64_t nx,
                          int64_t nr, int64_t nm, void *ws, int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(ind_in_chunk, "dep_dens_env_chnk: null IndInChunk");
  return deposit_common(DENS_ENV, coord, x_cs, x_ps, nullptr, 0, 0, wghts, w_ps, dens,
                        ind_in_chunk, nchnk, guards, leftX, rgrid, dx_inv, dr_inv, kx0, np, nx,
                        nr, nm, ws, ws_bytes, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free current deposit
//
// Some callers of this library cannot allocate device memory: a host code
// that reaches the GPU only through this C ABI (an FFI binding with no CUDA
// allocator of its own), or a loop whose device memory budget is fixed at
// start-up and that may not call cudaMalloc mid-run (cudaMalloc can
// synchronise the device and stall other streams).  For them,
// chm_dep_curr_noalloc runs the same deposit as chm_dep_curr with its scratch
// (the 64-bit accumulator, the weight partial sums and the scale) in the
// static device array below instead of a caller-provided workspace.
// ---------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr int64_t kNoAllocScratchBytes = 16LL << 20;  // 16 MiB, held per GPU until exit
static __device__ __align__(256) unsigned char g_dep_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[128] = {};  // device address of g_dep_scratch, per device

// Resolves (once per device, with that device current) the device address of
// the static scratch; host code cannot pass g_dep_scratch itself, whose name
// on the host is only a stand-in for the symbol.
int noalloc_scratch(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128) {
    set_error("dep_curr_noalloc: cudaGetDevice failed (%s)", cudaGetErrorString(e));
    return CHM_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_dep_scratch);
    if (e != cudaSuccess || !p) {
      set_error("dep_curr_noalloc: cudaGetSymbolAddress failed (%s)", cudaGetErrorString(e));
      return CHM_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return CHM_OK;
}

}  // namespace

extern "C" int64_t chm_dep_noalloc_max_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int chm_dep_curr_noalloc(const double *coord, int64_t x_cs, int64_t x_ps,
                                    const double *momenta, int64_t p_cs, int64_t p_ps,
                                    const double *wghts, int64_t w_ps, chm_c128 *curr,
                                    double leftX, const double *rgrid, double dx_inv,
                                    double dr_inv, int64_t np, int64_t nx, int64_t nr, int64_t nm,
                                    void *stream) {
  // the grid's own rules first (as chm_dep_curr checks them), then its size
  // against the static array, without an overflowing product
  if (nx <= 1 || nr <= 1 || nm < 1) {
    set_error("dep_curr_noalloc: bad grid (%lld, %lld, %lld): nx > 1, nr > 1 and nm >= 1 are "
              "required", (long long)nx, (long long)nr, (long long)nm);
    return CHM_ERR_ARG;
  }
  int64_t nodes = 0, need = 0;
  const bool big = __builtin_mul_overflow(nx, nr, &nodes) || __builtin_mul_overflow(nodes, nm, &nodes) ||
                   nodes > (kNoAllocScratchBytes - 8 * kRedBlocks - 256) / 48;
  if (!big) need = chm_dep_ws_bytes(nx, nr, nm, 3, np);
  if (big || need > kNoAllocScratchBytes) {
    set_error("dep_curr_noalloc: a (%lld, %lld, %lld, 3) grid needs more scratch than the "
              "%lld-byte static array; use chm_dep_curr with a workspace",
              (long long)nx, (long long)nr, (long long)nm, (long long)kNoAllocScratchBytes);
    return CHM_ERR_RANGE;
  }
  void *scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  // deposit_common zeroes the accumulator at the start of every call
  return deposit_common(CURR, coord, x_cs, x_ps, momenta, p_cs, p_ps, wghts, w_ps, curr, nullptr, 0,
                        0, leftX, rgrid, dx_inv, dr_inv, 0.0, np, nx, nr, nm, scratch,
                        kNoAllocScratchBytes, stream);
}
