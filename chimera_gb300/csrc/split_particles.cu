// Particle kernels of the split-precision form (FP32 particles).
//
// Particle layout (structure of arrays, 32 B per particle):
//   ix  int32   x cell index relative to the fixed origin X0
//   fx  float   offset inside that cell, [0, 1)
//   y, z float  transverse position
//   px, py, pz  float momenta (units of m c)
//   w   float   weight
// so x = X0 + (ix + fx) dx.  The running window origin leftX stays FP64 on
// the host and enters as (k, f): leftX = X0 + (k + f) dx, k integer, f in
// [0, 1); the grid-relative position is (ix - k) + (fx - f).
//
// Order in memory: tiles of 512 particles.  Particle i (its place in the
// species) is run r = (i / 16) mod 32, slot j = i mod 16 of tile i / 512, and
// sits at tile * 512 + 32 j + r.  A warp takes a tile, lane r the run r: the
// 16 consecutive particles of a run (one deposit cell when the particles are
// stored cell by cell) belong to one thread, and every load of a warp reads
// 32 consecutive words.  Arrays hold whole tiles; slots past the last
// particle are not read.
//
// Deposition stays deterministic without float atomics: each block adds its
// values as 32-bit integers at its own power-of-two scales (from the block's
// sum |w| and sum |w| max|v|) into a shared-memory box of its nodes, then adds the box into the
// global 64-bit accumulator (scale 2^(61 - ceil(log2 sum |w|))) with an exact
// power-of-two shift.  Integer sums are order-independent; the run kernel
// sums the particles of a run in FP32 before rounding, which depends only on
// the (fixed) particle order.
#include <climits>
#include <cstdlib>
#include <cstring>
#include <math.h>
#include <type_traits>

#include "common.cuh"

using namespace chm;

namespace {

constexpr int kRunLen = 16;                        // particles per run
constexpr int kTileRuns = 32;                      // runs per tile (lanes of a warp)
constexpr int kTile = kRunLen * kTileRuns;         // 512 particles per tile
constexpr int kDepWarps = 4;                       // tiles per block
constexpr int kDepThreads = 32 * kDepWarps;        // 128
constexpr int kDepBlock = kTile * kDepWarps;       // 2048 particles per block
constexpr int kSpBoxBytes = 40 * 1024;             // 10240 int32 values
// rho-only run kernel (still species): a smaller box (a block's box holds
// 2 nm - 1 values per node) and fewer registers, for more resident blocks
constexpr int kRhoBoxBytes = 16 * 1024;

// deposit cells dropped outside a block box while inside the grid (corrupt
// positions); read and reset by chm_sp_deposit_dropped
__device__ unsigned int g_dep_dropped;

// physical slot of particle i and the particle of a slot
__host__ __device__ __forceinline__ i64 phys_of(i64 i) {
  return (i & ~(i64)(kTile - 1)) | ((i & (kRunLen - 1)) << 5) | ((i >> 4) & (kTileRuns - 1));
}
__host__ __device__ __forceinline__ i64 logical_of(i64 p) {
  return (p & ~(i64)(kTile - 1)) | ((p & (kTileRuns - 1)) << 4) | ((p >> 5) & (kRunLen - 1));
}
__host__ __device__ inline i64 tiles_of(i64 n) { return (n + kTile - 1) / kTile; }

struct SpParts {
  int32_t *ix;
  float *fx, *y, *z, *px, *py, *pz, *w;
  i64 n;
};

// Starts the particle data of one tile (512 slots; 16 rows of 32
// consecutive slots per array) towards L2: one prefetch per 128-byte row,
// the warp's lanes taking rows in turn (the unstaged run kernels).
__device__ __forceinline__ void prefetch_tile(const SpParts &P, i64 tile, int lane, bool momenta) {
  if (tile >= P.n) return;
  const int narr = momenta ? 8 : 5;
  for (int k = lane; k < kRunLen * narr; k += 32) {
    const int row = k & (kRunLen - 1), arr = k >> 4;
    const float *b = arr == 0 ? P.w : arr == 1 ? (const float *)P.ix : arr == 2 ? P.fx
                   : arr == 3 ? P.y : arr == 4 ? P.z : arr == 5 ? P.px : arr == 6 ? P.py : P.pz;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(b + tile + (i64)row * kTileRuns));
  }
}

struct SpGrid {
  int win_k;      // window origin, whole cells from X0
  float win_f;    // window origin, fraction of a cell
  float dr_inv;   // 1/dr; r node j sits at (j - 1/2) dr
  int nx, nr, nm;  // spatial grid
};

// the window origin from the device record when there is one
__device__ __forceinline__ SpGrid window_grid(SpGrid G, const chm_sp_window *w) {
  if (w) {
    G.win_k = w->k;
    G.win_f = w->f;
  }
  return G;
}

// ceil(log2 v) of a positive finite float, and the exponent of a power of
// two held in a double (from its bits): the per-block plan stays off the
// FP64 pipe
__device__ __forceinline__ int ceil_log2f(float v) {
  int e;
  const float m = frexpf(v, &e);  // v = m 2^e, m in [0.5, 1)
  return (m == 0.5f) ? e - 1 : e;
}
__device__ __forceinline__ int pow2_exponent(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1023;
}

__device__ __forceinline__ int ceil_log2(double v) {
  int e;
  double m = frexp(v, &e);  // v = m 2^e, m in [0.5, 1)
  return (m == 0.5) ? e - 1 : e;
}

// Cell and fraction of a grid-relative x position and of r.
struct Loc {
  int cx, cr;
  float sx1, sr1;
  float phr, phi;  // e^{i theta} = (y + i z) / r (0 on axis)
  bool ok;
};

__device__ __forceinline__ Loc locate(int ix, float fx, float y, float z, const SpGrid &G) {
  Loc L;
  float d = fx - G.win_f;
  float fl = floorf(d);
  L.cx = ix - G.win_k + (int)fl;
  L.sx1 = d - fl;
  // r and 1/r from one reciprocal square root (a few ulp, FP32)
  const float r2 = y * y + z * z;
  const float ri = r2 > 0.0f ? rsqrtf(r2) : 0.0f;
  const float r = r2 * ri;
  float s = r * G.dr_inv + 0.5f;
  float sf = floorf(s);
  L.cr = (int)sf;
  L.sr1 = s - sf;
  L.ok = (L.cr >= 0 && L.cr <= G.nr - 2);
  L.phr = y * ri;  // 0 on the axis
  L.phi = z * ri;
  return L;
}

// Deposit of one particle: J (3 components, value vJ[l] = w v_l / gamma) at
// location a, and/or rho (value w) at location b; complex mode phases
// e^{-i m theta}.  emit(plane, r, x, re, im) with plane = mode + nm*comp
// (J) or nm*3 + mode (rho).
template <typename Emit>
__device__ __forceinline__ void deposit_at(const Loc &L, const float *val, int ncomp, int plane0,
                                           const SpGrid &G, Emit emit) {
  if (!L.ok) return;
  const float sx[2] = {1.0f - L.sx1, L.sx1};
  const float sr[2] = {1.0f - L.sr1, L.sr1};
  float pr = 1.0f, pi = 0.0f;  // e^{-i m theta}
  for (int m = 0; m < G.nm; ++m) {
    if (m > 0) {
      float nr_ = pr * L.phr + pi * L.phi;  // (pr + i pi)(phr - i phi)
      float ni_ = pi * L.phr - pr * L.phi;
      pr = nr_;
      pi = ni_;
    }
    for (int l = 0; l < ncomp; ++l) {
      const float vr = pr * val[l], vi = pi * val[l];
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const int gx = L.cx + k;
          if (gx < 0 || gx >= G.nx) continue;
          const float s = sx[k] * sr[j];
          emit(plane0 + m + G.nm * l, L.cr + j, gx, vr * s, vi * s);
        }
    }
  }
}

// round-to-nearest float -> int64 without the 64-bit conversion unit: below
// 2^31 the 32-bit conversion, above it the float is an integer and its bits
// give the value (|v| < 2^62 for accumulator values)
__device__ __forceinline__ long long f2ll(float v) {
  if (fabsf(v) < 2147483520.0f) return (long long)__float2int_rn(v);
  const unsigned u = __float_as_uint(v);
  const int sh = (int)((u >> 23) & 0xffu) - 127 - 23;
  const long long r = (long long)((u & 0x7fffffu) | 0x800000u) << min(sh, 39);
  return (u >> 31) ? -r : r;
}

struct PushDepArgs {
  SpParts P;
  SpGrid G;
  float dt;        // time step
  float dx_inv;    // 1 / dx
  int push;        // advance the coordinates (moving species)
  int dep_j;       // deposit J at the half step
  int dep_rho;     // deposit rho at the new position
  unsigned long long *accJ;  // (nx, nr, nm, 3) x {re, im}
  unsigned long long *accR;  // (nx, nr, nm) x {re, im}
  const double *scaleJ, *scaleR;  // global scales 2^e
  const chm_sp_window *win;       // device window origin (or null: G's)
  // (envelope kernel) a light-speed step of D = c dt / dx cells, split
  // exactly into whole cells and an FP32 fraction, for the full and the
  // half step; far: D >= 2
  int far, d_int, dh_int;
  float d_frac, dh_frac, d_cells;
  // (still species' background pass) nodes x < gx_min are not written; a
  // block records the x range of its live particles' cells (absolute cell
  // indices) into ext_out, or skips itself when ext_in shows that its
  // nodes cannot reach x >= gx_min
  int gx_min;
  int2 *ext_out;
  const int2 *ext_in;
};

// Block box: 32-bit fixed-point values at the block's own scales 2^elJ,
// 2^elR (from bounds of the block's sum of |J| and |rho| values, so the box
// cannot overflow), added into the global 64-bit grid (scales 2^eJ, 2^eR) by
// an exact power-of-two shift when the block is done.  A node holds
// ncomp (2 nm - 1) values: for each deposited component (J_x, J_y, J_z and/or
// rho; c0 the first) the parts (mode 0 re; mode 1 re, im; ...) -- mode 0 has
// no imaginary part.  Value (c, part) of node (r, x) sits at
// (((c - c0) P + part) bnr + r - br0) bnx + x - bx0, P = 2 nm - 1.
struct BoxGeo {
  int *box;
  int bx0, br0, bnx, bnr;
  int c0;                        // first component held (0: J and rho, 3: rho only)
  int elJ, elR, eJ, eR;          // local (J, rho) and global quantum exponents
  unsigned long long *gJ, *gR;   // global accumulators
  int nx, nr, nm;                // grid
  int gx_min;                    // first grid column written (0: all)
};

// value at the local quantum 2^-el -> global quantum 2^-eg: an exact left
// shift when eg >= el (the usual case: a block holds a small share of the
// total weight), otherwise a right shift rounded half away from zero
__device__ __forceinline__ long long rescale(long long q, int el, int eg) {
  const int s = el - eg;
  if (s <= 0) return q << min(-s, 62);
  if (s >= 62) return 0;
  const long long h = 1LL << (s - 1);
  return (q >= 0) ? ((q + h) >> s) : -((-q + h) >> s);
}

// part index of (mode m, imaginary flag)
__device__ __forceinline__ int part_of(int m, int im) { return m == 0 ? 0 : 2 * m - 1 + im; }

// Adds v (local quantum) at node (r, x) of plane (m + nm l for J, 3 nm + m
// for rho), part im, to the box; a node outside the box (the plan bounds
// every deposit location, so this is a guard only) goes to the global
// accumulator directly.
__device__ __forceinline__ void box_put(const BoxGeo &B, long long plane, int r, int x, int im,
                                        int v) {
  const int c = (int)(plane / B.nm), m = (int)(plane - (long long)c * B.nm);
  if (m == 0 && im) return;  // mode 0 deposits no imaginary part
  const int rr = r - B.br0, xx = x - B.bx0;
  if (rr >= 0 && rr < B.bnr && xx >= 0 && xx < B.bnx) {
    const int cp = (c - B.c0) * (2 * B.nm - 1) + part_of(m, im);
    atomicAdd(&B.box[(cp * B.bnr + rr) * B.bnx + xx], v);
    return;
  }
  const bool isj = c < 3;
  const long long q = isj ? rescale(v, B.elJ, B.eJ) : rescale(v, B.elR, B.eR);
  if (q == 0) return;
  const long long pl = isj ? plane : m;
  unsigned long long *acc = isj ? B.gJ : B.gR;
  atomicAdd(&acc[2 * ((pl * B.nr + r) * B.nx + x) + im], (unsigned long long)q);
}

// q = t / d for t < 2^16, 2 <= d < 2^16 by a multiply-high with
// m = floor((2^32 - 1) / d) + 1: m d = 2^32 + e with 0 <= e < d, and
// t e < 2^32 keeps floor(t m / 2^32) = floor(t / d); d = 1 is passed through
__device__ __forceinline__ unsigned div_magic(unsigned d) { return d > 1 ? 0xffffffffu / d + 1u : 0u; }
__device__ __forceinline__ unsigned div_small(unsigned t, unsigned m) { return m ? __umulhi(t, m) : t; }

// Adds the block box into the global accumulators: the threads walk the box
// values in storage order (a warp reads 32 consecutive values, whatever the
// box width), each nonzero value rescaled to the global quantum.
__device__ void flush_box(const BoxGeo &B, long long nvals) {
  const unsigned bnx = (unsigned)B.bnx, plane_n = (unsigned)(B.bnx * B.bnr);
  const unsigned P = 2 * B.nm - 1;
  const unsigned mx = div_magic(bnx), mp = div_magic(plane_n), mP = div_magic(P);
  for (unsigned t = threadIdx.x; t < (unsigned)nvals; t += blockDim.x) {
    const int v = B.box[t];
    if (v == 0) continue;
    const unsigned cp = div_small(t, mp), rem = t - cp * plane_n;
    const unsigned rr = div_small(rem, mx), xx = rem - rr * bnx;
    const int gx = B.bx0 + (int)xx;
    if (gx < B.gx_min || gx >= B.nx) continue;  // the nodes beyond the grid's ends
    const unsigned cb = div_small(cp, mP);
    const int part = (int)(cp - cb * P), c = (int)cb + B.c0;
    const int m = (part + 1) >> 1, im = (part > 0 && (part & 1) == 0) ? 1 : 0;
    const bool isj = c < 3;
    const long long q = rescale(v, isj ? B.elJ : B.elR, isj ? B.eJ : B.eR);
    if (q == 0) continue;
    const int pl = isj ? m + B.nm * c : m;
    unsigned long long *acc = isj ? B.gJ : B.gR;
    atomicAdd(acc + 2 * (((i64)pl * B.nr + (rr + B.br0)) * B.nx + gx) + im,
              (unsigned long long)q);
  }
}

// Particle update of push_coords (particle_tools.f90:58-82) in cell units:
// half-step and new positions.
struct Pushed {
  int ixh, ixn;
  float fxh, fxn, yh, zh, yn, zn;
  float vj[3];
  bool moving;  // nonzero momentum (particles at rest carry no current)
};

__device__ __forceinline__ Pushed push_vals(const PushDepArgs &A, int ix, float fx, float y, float z,
                                            float px, float py, float pz, float w) {
  Pushed o;
  const float ig = rsqrtf(1.0f + (px * px + py * py + pz * pz));  // 1 / gamma
  const float dtg = A.push ? A.dt * ig : 0.0f;
  const float dxc = px * dtg * A.dx_inv;  // displacement in cells
  float xh = fx + 0.5f * dxc, xn = fx + dxc;
  float flh = floorf(xh), fln = floorf(xn);
  o.ixh = ix + (int)flh;
  o.fxh = xh - flh;
  o.ixn = ix + (int)fln;
  o.fxn = xn - fln;
  o.yh = y + 0.5f * py * dtg;
  o.zh = z + 0.5f * pz * dtg;
  o.yn = y + py * dtg;
  o.zn = z + pz * dtg;
  // grid_deps.f90:42: particles at rest deposit no current
  const bool moving = (fabsf(px) + fabsf(py) + fabsf(pz)) != 0.0f;
  o.moving = moving;
  const float wg = moving ? w * ig : 0.0f;
  o.vj[0] = px * wg;
  o.vj[1] = py * wg;
  o.vj[2] = pz * wg;
  return o;
}

__device__ __forceinline__ Pushed push_one(const PushDepArgs &A, i64 i) {
  const SpParts &P = A.P;
  return push_vals(A, P.ix[i], P.fx[i], P.y[i], P.z[i], P.px[i], P.py[i], P.pz[i], P.w[i]);
}

// The same push for a species that moves many cells per step (a
// relativistic beam, D = c dt / dx >> 1): the x displacement D v_x is
// taken as D - D (1 - v_x), the light-speed part D added exactly in whole
// cells plus its FP32 fraction, the slip D (1 - v_x) computed without
// cancellation, (1 - v_x) = (1 + p_y^2 + p_z^2) / (gamma (gamma + p_x)) for
// p_x >= 0 (1 - p_x / gamma otherwise).  An FP32 product p_x dt / gamma
// would carry an error of the order of D 2^-24 cells per step instead.
__device__ __forceinline__ Pushed push_vals_far(const PushDepArgs &A, int ix, float fx, float y,
                                                float z, float px, float py, float pz, float w) {
  Pushed o;
  const float pt2 = py * py + pz * pz;
  const float ig = rsqrtf(1.0f + (px * px + pt2));  // 1 / gamma
  const float g = 1.0f / ig;
  const float slip = px >= 0.0f ? (1.0f + pt2) / (g * (g + px)) : 1.0f - px * ig;
  const float dtg = A.dt * ig;
  float xh = fx + (A.dh_frac - 0.5f * A.d_cells * slip);
  float xn = fx + (A.d_frac - A.d_cells * slip);
  const float flh = floorf(xh), fln = floorf(xn);
  o.ixh = ix + A.dh_int + (int)flh;
  o.fxh = xh - flh;
  o.ixn = ix + A.d_int + (int)fln;
  o.fxn = xn - fln;
  o.yh = y + 0.5f * py * dtg;
  o.zh = z + 0.5f * pz * dtg;
  o.yn = y + py * dtg;
  o.zn = z + pz * dtg;
  const bool moving = (fabsf(px) + fabsf(py) + fabsf(pz)) != 0.0f;
  o.moving = moving;
  const float wg = moving ? w * ig : 0.0f;
  o.vj[0] = px * wg;
  o.vj[1] = py * wg;
  o.vj[2] = pz * wg;
  return o;
}

// ----------------------------------------------------------------------
// Shared-memory staging of a block's particles: the run kernels first copy
// the block's 2048 slots of every array they read into shared memory with
// 16-byte asynchronous copies (cp.async, only the tiles that exist), then
// plan and walk the runs from there, so no particle load of the main loops
// waits on L2 or DRAM.  Arrays in the stage: w, ix, fx, y, z, px, py, pz.
// ----------------------------------------------------------------------
constexpr int kStageArrays = 8;

struct StageView {  // particle values by slot (global arrays or the stage)
  const int32_t *ix;
  const float *fx, *y, *z, *px, *py, *pz, *w;
};

__device__ __forceinline__ StageView global_view(const SpParts &P, i64 base) {
  return StageView{P.ix + base, P.fx + base, P.y + base, P.z + base,
                   P.px + base, P.py + base, P.pz + base, P.w + base};
}

__device__ __forceinline__ StageView stage_view(const unsigned char *sm) {
  const float *f = reinterpret_cast<const float *>(sm);
  return StageView{reinterpret_cast<const int32_t *>(f + kDepBlock), f + 2 * kDepBlock,
                   f + 3 * kDepBlock, f + 4 * kDepBlock, f + 5 * kDepBlock, f + 6 * kDepBlock,
                   f + 7 * kDepBlock, f};
}

// copies the block's slots [base, base + 2048) of the first narr arrays
// (5: w, ix, fx, y, z; 8: and the momenta) into sm; slots of tiles past the
// last particle are not copied (and are never read)
__device__ __forceinline__ void stage_block(const SpParts &P, i64 base, int narr, unsigned char *sm) {
  const i64 ntiles = tiles_of(P.n);
  const int tiles = (int)max((i64)0, min((i64)(kDepBlock / kTile), ntiles - base / kTile));
  const int nchunk = tiles * kTile / 4;  // 16-byte chunks per array
  const uint32_t s0 = static_cast<uint32_t>(__cvta_generic_to_shared(sm));
  for (int c = threadIdx.x; c < narr * nchunk; c += blockDim.x) {
    const int a = c / nchunk, k = c - a * nchunk;
    const float *src = a == 0 ? P.w : a == 1 ? reinterpret_cast<const float *>(P.ix) : a == 2 ? P.fx
                     : a == 3 ? P.y : a == 4 ? P.z : a == 5 ? P.px : a == 6 ? P.py : P.pz;
    const uint32_t dst = s0 + (uint32_t)((a * kDepBlock + 4 * k) * 4);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src + base + 4 * k)
                 : "memory");
  }
  asm volatile("cp.async.commit_group;\ncp.async.wait_all;" ::: "memory");
  __syncthreads();
}

// Block plan shared by the deposit kernels: the box of nodes the block's
// deposits can touch, from every particle of its 2048 slots.  The box is
// bounded without pushing: a particle moves less than c dt, so its deposit
// cells lie within ceil(dt/dx) cells of its x cell and within dt of its
// radius.  (Nodes outside the box go straight to the global accumulator.)
struct BlockPlan {
  int bx0, br0, bnx, bnr;
  long long nvals;
  int c0;          // first component held by the box
  bool use_box;
  float lJ, lR;    // local scales 2^elJ, 2^elR
  int elJ, elR;    // local quantum exponents
  int eJ, eR;      // global quantum exponents
  float sJ, sR;    // global scales 2^eJ, 2^eR (path without a box)
};

template <bool STAGED>
__device__ BlockPlan plan_block(const PushDepArgs &A, const SpGrid &G, i64 base, int *bb,
                                int box_bytes, const StageView &V) {
  __shared__ float wsm[2][8];  // per-warp partial sums (blocks of up to 8 warps)
  if (threadIdx.x == 0) {
    bb[0] = INT_MAX;
    bb[1] = INT_MIN;
    bb[2] = INT_MAX;
    bb[3] = INT_MIN;
  }
  __syncthreads();
  int xlo = INT_MAX, xhi = INT_MIN;
  float r2lo = INFINITY, r2hi = -INFINITY, wsum = 0.0f, jsum = 0.0f;
  // independent loads (no load depends on another), 4 slots per step
#pragma unroll 4
  for (int s = threadIdx.x; s < kDepBlock; s += blockDim.x) {
    const i64 p = base + s;
    const bool valid = logical_of(p) < A.P.n;
    // (V: the block's stage when STAGED, else the arguments' arrays)
    const int qs = valid ? s : 0;  // slot 0 of the block always holds a particle
    const i64 q = base + qs;
    const float w = STAGED ? V.w[qs] : A.P.w[q];
    // (the rho-only pass reads global memory: its fx starts towards L2 here)
    if (!STAGED && !A.push && !A.dep_j) asm volatile("prefetch.global.L2 [%0];" ::"l"(A.P.fx + q));
    const int ix = STAGED ? V.ix[qs] : A.P.ix[q];
    const float y = STAGED ? V.y[qs] : A.P.y[q], z = STAGED ? V.z[qs] : A.P.z[q];
    float pp = 0.0f;
    if (A.dep_j) {
      const float px = STAGED ? V.px[qs] : A.P.px[q], py = STAGED ? V.py[qs] : A.P.py[q],
                  pz = STAGED ? V.pz[qs] : A.P.pz[q];
      // max_l |v_l| = max_l |p_l| / gamma
      pp = fmaxf(fabsf(px), fmaxf(fabsf(py), fabsf(pz))) *
           rsqrtf(1.0f + (px * px + py * py + pz * pz));
    }
    if (!valid || w == 0.0f) continue;
    xlo = min(xlo, ix);
    xhi = max(xhi, ix);
    const float r2 = y * y + z * z;
    r2lo = fminf(r2lo, r2);
    r2hi = fmaxf(r2hi, r2);
    wsum += fabsf(w);
    // |w v_l| <= |w| max_l |v_l|: a bound of the current values (with a
    // little room for the reciprocal square root)
    jsum += fabsf(w) * fminf(1.0f, pp * 1.0001f);
  }
  int x0 = INT_MAX, x1 = INT_MIN, r0 = INT_MAX, r1 = INT_MIN;
  if (xlo <= xhi) {
    const int D = A.push ? (int)ceilf(A.dt * A.dx_inv) : 0;
    const float drc = A.push ? A.dt : 0.0f;
    x0 = xlo - G.win_k - 1 - D;
    x1 = xhi - G.win_k + 1 + D;
    r0 = max(0, (int)floorf((sqrtf(r2lo) - drc) * G.dr_inv + 0.5f) - 1);
    r1 = (int)floorf((sqrtf(r2hi) + drc) * G.dr_inv + 0.5f) + 2;
  }
  x0 = __reduce_min_sync(0xffffffffu, x0);
  x1 = __reduce_max_sync(0xffffffffu, x1);
  r0 = __reduce_min_sync(0xffffffffu, r0);
  r1 = __reduce_max_sync(0xffffffffu, r1);
  for (int o = 16; o > 0; o >>= 1) {
    wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
    jsum += __shfl_xor_sync(0xffffffffu, jsum, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&bb[0], x0);
    atomicMax(&bb[1], x1);
    atomicMin(&bb[2], r0);
    atomicMax(&bb[3], r1);
    wsm[0][threadIdx.x >> 5] = wsum;
    wsm[1][threadIdx.x >> 5] = jsum;
  }
  __syncthreads();
  if (A.ext_out && threadIdx.x == 0) {
    // the block's live cells, absolute (x0 = xlo - win_k - 1 - D, x1 = xhi - win_k + 1 + D)
    const int D = A.push ? (int)ceilf(A.dt * A.dx_inv) : 0;
    A.ext_out[blockIdx.x] = bb[0] <= bb[1] ? make_int2(bb[0] + G.win_k + 1 + D, bb[1] + G.win_k - 1 - D)
                                           : make_int2(INT_MAX, INT_MIN);
  }
  BlockPlan P;
  float Bl = 0.0f, Bj = 0.0f;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {  // fixed order
    Bl += wsm[0][k];
    Bj += wsm[1][k];
  }
  // in x the box reaches one node beyond the grid on each side, so that the
  // cells at the grid's ends stay inside it (those nodes are dropped at the
  // flush, as the reference drops them)
  P.bx0 = max(bb[0], -1);
  P.br0 = max(bb[2], 0);
  const int bx1 = min(bb[1], G.nx), br1 = min(bb[3], G.nr - 1);
  P.bnx = bx1 - P.bx0 + 1;
  P.bnr = br1 - P.br0 + 1;
  // deposited components (J_x, J_y, J_z and/or rho) x mode parts
  const int per_node = (3 * (A.dep_j ? 1 : 0) + (A.dep_rho ? 1 : 0)) * (2 * G.nm - 1);
  P.c0 = A.dep_j ? 0 : 3;
  P.nvals = (bb[0] <= bb[1] && P.bnx > 0 && P.bnr > 0) ? (long long)P.bnx * P.bnr * per_node : 0;
  P.use_box = P.nvals > 0 && P.nvals * 4 <= box_bytes && Bl > 0.0f && isfinite(Bl);
  // a node value of a particle is at most |w| (rho) or |w| max_l |v_l| (J),
  // so each part of the box stays below 2^30 (one bit of margin for the
  // FP32 sums and the per-run rounding)
  P.elR = P.use_box ? min(30 - ceil_log2f(Bl), 120) : 0;
  P.elJ = (P.use_box && Bj > 0.0f) ? min(30 - ceil_log2f(Bj), 120) : P.elR;
  P.lR = ldexpf(1.0f, P.elR);
  P.lJ = ldexpf(1.0f, P.elJ);
  // the global scales are powers of two 2^e, e <= 120
  P.eJ = A.scaleJ ? pow2_exponent(A.scaleJ[0]) : 0;
  P.eR = A.scaleR ? pow2_exponent(A.scaleR[0]) : 0;
  P.sJ = ldexpf(1.0f, P.eJ);
  P.sR = ldexpf(1.0f, P.eR);
  return P;
}

__device__ __forceinline__ BoxGeo make_geo(int *box, const BlockPlan &P, const PushDepArgs &A) {
  return BoxGeo{box, P.bx0, P.br0, P.bnx, P.bnr, P.c0, P.elJ, P.elR, P.eJ, P.eR, A.accJ, A.accR,
                A.G.nx, A.G.nr, A.G.nm, A.gx_min};
}

// Generic push + deposit (any nm): one particle per thread and slot, each
// value rounded to the block quantum and added to the box (or, without a
// box, to the global quantum and added to the global accumulator).
__global__ void __launch_bounds__(kDepThreads) push_deposit_kernel(PushDepArgs A) {
  const SpGrid G = window_grid(A.G, A.win);
  extern __shared__ __align__(16) int box[];
  __shared__ int bb[4];
  const i64 base = (i64)blockIdx.x * kDepBlock;
  const BlockPlan Pl = plan_block<false>(A, G, base, bb, kSpBoxBytes, StageView{});
  if (Pl.use_box)
    for (long long t = threadIdx.x; t < Pl.nvals; t += kDepThreads) box[t] = 0;
  __syncthreads();
  const BoxGeo geo = make_geo(box, Pl, A);
  for (int s = threadIdx.x; s < kDepBlock; s += kDepThreads) {
    const i64 p = base + s;
    if (logical_of(p) >= A.P.n) continue;
    const float w = A.P.w[p];
    const Pushed q = push_one(A, p);
    if (w != 0.0f) {
      if (A.dep_j) {
        const Loc L = locate(q.ixh, q.fxh, q.yh, q.zh, G);
        deposit_at(L, q.vj, 3, 0, G, [&](int plane, int r, int x, float re, float im) {
          if (Pl.use_box) {
            const int qr = __float2int_rn(re * Pl.lJ), qi = __float2int_rn(im * Pl.lJ);
            if (qr) box_put(geo, plane, r, x, 0, qr);
            if (qi) box_put(geo, plane, r, x, 1, qi);
          } else {
            const long long qr = f2ll(re * Pl.sJ), qi = f2ll(im * Pl.sJ);
            const i64 e = ((i64)plane * G.nr + r) * G.nx + x;
            if (qr) atomicAdd(&A.accJ[2 * e], (unsigned long long)qr);
            if (qi) atomicAdd(&A.accJ[2 * e + 1], (unsigned long long)qi);
          }
        });
      }
      if (A.dep_rho) {
        const Loc L = locate(q.ixn, q.fxn, q.yn, q.zn, G);
        const float wv[1] = {w};
        deposit_at(L, wv, 1, 3 * G.nm, G, [&](int plane, int r, int x, float re, float im) {
          if (Pl.use_box) {
            const int qr = __float2int_rn(re * Pl.lR), qi = __float2int_rn(im * Pl.lR);
            if (qr) box_put(geo, plane, r, x, 0, qr);
            if (qi) box_put(geo, plane, r, x, 1, qi);
          } else {
            const long long qr = f2ll(re * Pl.sR), qi = f2ll(im * Pl.sR);
            const i64 e = ((i64)(plane - 3 * G.nm) * G.nr + r) * G.nx + x;
            if (qr) atomicAdd(&A.accR[2 * e], (unsigned long long)qr);
            if (qi) atomicAdd(&A.accR[2 * e + 1], (unsigned long long)qi);
          }
        });
      }
    }
    if (A.push) {
      A.P.ix[p] = q.ixn;
      A.P.fx[p] = q.fxn;
      A.P.y[p] = q.yn;
      A.P.z[p] = q.zn;
    }
  }
  if (!Pl.use_box) return;
  __syncthreads();
  flush_box(geo, Pl.nvals);
}

// ----------------------------------------------------------------------
// Run form of push + deposit for nm = 1..3: lane r of a warp walks the 16
// particles of run r of its tile, sums their node values (already at the
// block's fixed-point scale) in FP32 registers while the deposit cell stays
// the same, and adds the sums, rounded to the block quantum, to the block
// box when the cell changes and at the end.
// ----------------------------------------------------------------------

// node sums of one deposit cell at the block scale: v[comp][part][node],
// part 0 = mode 0 re, then (re, im) of modes 1 .. NM-1; node = 2 j + k
// (r + j, x + k)
template <int NM, int NC>
struct CellAcc {
  int cx, cr;
  bool live;
  float v[NC][2 * NM - 1][4];
};

template <int NM, int NC>
__device__ __forceinline__ void acc_flush(CellAcc<NM, NC> &c, int plane0, const SpGrid &G,
                                          const BoxGeo &B) {
  if (!c.live) return;
  c.live = false;
  const int rr = c.cr - B.br0, xx = c.cx - B.bx0;
  if (rr >= 0 && rr + 1 < B.bnr && xx >= 0 && xx + 1 < B.bnx) {
    // all four nodes inside the box
    const int rs = B.bnx, ps = rs * B.bnr;  // row and (component, part) strides
    int *b0 = B.box + (rr * rs + xx);
    const int c0 = plane0 / NM;  // first component: 0 (J) or 3 (rho)
#pragma unroll
    for (int l = 0; l < NC; ++l)
#pragma unroll
      for (int p = 0; p < 2 * NM - 1; ++p) {
        int *bp = b0 + ((c0 + l - B.c0) * (2 * NM - 1) + p) * ps;
#pragma unroll
        for (int nd = 0; nd < 4; ++nd) {
          const int v = __float2int_rn(c.v[l][p][nd]);
          if (v) atomicAdd(bp + (nd >> 1) * rs + (nd & 1), v);
        }
      }
    return;
  }
  // a cell with nodes outside the block box: the plan bounds the deposit
  // cells of every finite particle with |v| < c inside the box (and the box
  // reaches one node past each x end of the grid), so such a cell has all its
  // nodes past the grid's x ends (dropped, as the reference drops them), or
  // comes from a corrupt position.  Its values are dropped; the second case
  // is counted (chm_sp_deposit_dropped).
  if (c.cx >= -1 && c.cx < G.nx && c.cr >= 0 && c.cr + 1 < G.nr) atomicAdd(&g_dep_dropped, 1u);
}

// val: the particle's values already multiplied by the block scale
template <int NM, int NC>
__device__ __forceinline__ void acc_add(CellAcc<NM, NC> &c, const Loc &L, const float *val,
                                        int plane0, const SpGrid &G, const BoxGeo &B) {
  if (!L.ok) return;
  if (!c.live || c.cx != L.cx || c.cr != L.cr) {
    acc_flush(c, plane0, G, B);
    c.cx = L.cx;
    c.cr = L.cr;
    c.live = true;
#pragma unroll
    for (int l = 0; l < NC; ++l)
#pragma unroll
      for (int p = 0; p < 2 * NM - 1; ++p)
#pragma unroll
        for (int nd = 0; nd < 4; ++nd) c.v[l][p][nd] = 0.0f;
  }
  const float sx[2] = {1.0f - L.sx1, L.sx1};
  const float sr[2] = {1.0f - L.sr1, L.sr1};
  float pr = 1.0f, pi = 0.0f;  // e^{-i m theta}
#pragma unroll
  for (int m = 0; m < NM; ++m) {
    if (m > 0) {
      float nr_ = pr * L.phr + pi * L.phi;
      float ni_ = pi * L.phr - pr * L.phi;
      pr = nr_;
      pi = ni_;
    }
#pragma unroll
    for (int l = 0; l < NC; ++l) {
      const float vr = pr * val[l], vi = pi * val[l];
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const float s = sx[k] * sr[j];
          const int nd = 2 * j + k;
          if (m == 0) {
            c.v[l][0][nd] += vr * s;
          } else {
            c.v[l][2 * m - 1][nd] += vr * s;
            c.v[l][2 * m][nd] += vi * s;
          }
        }
    }
  }
}

// A particle's values in a run kernel's registers.
struct RunPart {
  int ix;
  float fx, y, z, px, py, pz, w;
};

// A particle of a block without a box: its values straight to the global
// accumulators at the global scales.
template <bool DJ, bool DR>
__device__ __forceinline__ void deposit_global(const PushDepArgs &A, const SpGrid &G,
                                               const BlockPlan &Pl, const Pushed &u, float w) {
  if (DJ && u.moving) {
    const Loc L = locate(u.ixh, u.fxh, u.yh, u.zh, G);
    const float vs[3] = {u.vj[0] * Pl.sJ, u.vj[1] * Pl.sJ, u.vj[2] * Pl.sJ};
    deposit_at(L, vs, 3, 0, G, [&](int plane, int r, int x, float re, float im) {
      const i64 e = ((i64)plane * G.nr + r) * G.nx + x;
      const long long qr = f2ll(re), qi = f2ll(im);
      if (qr) atomicAdd(&A.accJ[2 * e], (unsigned long long)qr);
      if (qi) atomicAdd(&A.accJ[2 * e + 1], (unsigned long long)qi);
    });
  }
  if (DR) {
    const Loc L = locate(u.ixn, u.fxn, u.yn, u.zn, G);
    const float ws[1] = {w * Pl.sR};
    deposit_at(L, ws, 1, 0, G, [&](int plane, int r, int x, float re, float im) {
      const i64 e = ((i64)plane * G.nr + r) * G.nx + x;
      const long long qr = f2ll(re), qi = f2ll(im);
      if (qr) atomicAdd(&A.accR[2 * e], (unsigned long long)qr);
      if (qi) atomicAdd(&A.accR[2 * e + 1], (unsigned long long)qi);
    });
  }
}

// Run kernels of the moving species with one or two modes and of the still
// species' rho-only pass: unstaged, the warp's tile started towards L2 first
// (measured faster than staged at 2048 x 256 x 2 modes), 4 blocks per SM at
// 128 registers (moving) or 8 at 64 (rho-only: 20 B per particle read once;
// 6 with three modes, whose sums spill at 64).
constexpr int kRhoMinBlocks = 8;
constexpr int kRhoGroup = 1;  // particles loaded ahead per lane (rho-only pass)

template <int NM, bool PUSH, bool DJ, bool DR>
__global__ void __launch_bounds__(kDepThreads, DJ ? 4 : kRhoMinBlocks)
    push_deposit_run_kernel(PushDepArgs A) {
  if (A.win) {  // the window origin from the device record
    A.G.win_k = A.win->k;
    A.G.win_f = A.win->f;
  }
  if (A.ext_in) {
    // a block whose cells' nodes (at most one cell right of its live
    // particles' cells) stay left of gx_min has nothing to write
    const int2 e = A.ext_in[blockIdx.x];
    if (e.x > e.y || e.y - A.G.win_k + 1 < A.gx_min) return;
  }
  extern __shared__ __align__(16) int box[];
  __shared__ int bb[4];
  // slot indices: 32-bit in the rho-only kernel (measured faster there; the
  // host launches it for n < 2^31 only), 64-bit otherwise
  using Idx = typename std::conditional<DJ, i64, unsigned>::type;
  const Idx base = (Idx)blockIdx.x * kDepBlock;
  // (the rho-only pass starts only fx towards L2, in the plan: measured
  // faster there than the whole tile)
  if (PUSH || DJ) prefetch_tile(A.P, (i64)base + (threadIdx.x >> 5) * kTile, threadIdx.x & 31, true);
  const BlockPlan Pl = plan_block<false>(A, A.G, (i64)base, bb, DJ ? kSpBoxBytes : kRhoBoxBytes,
                                         StageView{});
  if (Pl.use_box)
    for (int t = threadIdx.x; t < (int)Pl.nvals; t += kDepThreads) box[t] = 0;
  __syncthreads();
  const BoxGeo geo = make_geo(box, Pl, A);
  const int lane = threadIdx.x & 31;
  const Idx tile = base + (Idx)(threadIdx.x >> 5) * kTile;
  const Idx first = tile + (Idx)lane * kRunLen;  // this lane's run, in particle order
  CellAcc<NM, 3> cj;
  CellAcc<NM, 1> cr;
  cj.live = false;
  cr.live = false;
  const int cnt = (int)max((i64)0, min((i64)kRunLen, A.P.n - (i64)first));
  if (!Pl.use_box) {
    // a block whose nodes do not fit a box (a wide footprint): each particle
    // straight to the global accumulators at the global scales, apart from
    // the main loop so that the loop does not carry this path's registers
    for (int j = 0; j < cnt; ++j) {
      const Idx p = tile + (Idx)j * kTileRuns + lane;
      const float w = A.P.w[p];
      Pushed u;
      if (PUSH || DJ) {
        u = push_one(A, p);
      } else {
        u.ixh = u.ixn = A.P.ix[p];
        u.fxh = u.fxn = A.P.fx[p];
        u.yh = u.yn = A.P.y[p];
        u.zh = u.zn = A.P.z[p];
      }
      if (PUSH) {
        A.P.ix[p] = u.ixn;
        A.P.fx[p] = u.fxn;
        A.P.y[p] = u.yn;
        A.P.z[p] = u.zn;
      }
      if (w == 0.0f) continue;
      if (DJ && u.moving) {
        const Loc L = locate(u.ixh, u.fxh, u.yh, u.zh, A.G);
        const float vs[3] = {u.vj[0] * Pl.sJ, u.vj[1] * Pl.sJ, u.vj[2] * Pl.sJ};
        deposit_at(L, vs, 3, 0, A.G, [&](int plane, int r, int x, float re, float im) {
          const i64 e = ((i64)plane * A.G.nr + r) * A.G.nx + x;
          const long long qr = f2ll(re), qi = f2ll(im);
          if (qr) atomicAdd(&A.accJ[2 * e], (unsigned long long)qr);
          if (qi) atomicAdd(&A.accJ[2 * e + 1], (unsigned long long)qi);
        });
      }
      if (DR) {
        const Loc L = locate(u.ixn, u.fxn, u.yn, u.zn, A.G);
        const float ws[1] = {w * Pl.sR};
        deposit_at(L, ws, 1, 0, A.G, [&](int plane, int r, int x, float re, float im) {
          if (x < A.gx_min) return;
          const i64 e = ((i64)plane * A.G.nr + r) * A.G.nx + x;
          const long long qr = f2ll(re), qi = f2ll(im);
          if (qr) atomicAdd(&A.accR[2 * e], (unsigned long long)qr);
          if (qi) atomicAdd(&A.accR[2 * e + 1], (unsigned long long)qi);
        });
      }
    }
    return;
  }
  // software pipeline: the next group of particles is loaded before this
  // group's results are stored (the stores could alias the loads
  // otherwise); G particles per group (kRhoGroup for the rho-only pass:
  // one measured best at its 64-register budget)
  constexpr int G = DJ ? 1 : kRhoGroup;
  struct Part {
    int ix;
    float fx, y, z, px, py, pz, w;
  };
  auto load = [&](int j) {
    Part q;
    const Idx p = tile + (Idx)j * kTileRuns + lane;
    q.w = A.P.w[p];
    q.ix = A.P.ix[p];
    q.fx = A.P.fx[p];
    q.y = A.P.y[p];
    q.z = A.P.z[p];
    if (PUSH || DJ) {
      q.px = A.P.px[p];
      q.py = A.P.py[p];
      q.pz = A.P.pz[p];
    }
    return q;
  };
  Part cur[G], nxt[G];
#pragma unroll
  for (int g = 0; g < G; ++g)
    if (g < cnt) cur[g] = load(g);
  for (int j0 = 0; j0 < cnt; j0 += G) {
#pragma unroll
    for (int g = 0; g < G; ++g)
      if (j0 + G + g < cnt) nxt[g] = load(j0 + G + g);
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int j = j0 + g;
      if (j >= cnt) break;
      const Part &c = cur[g];
      const Idx p = tile + (Idx)j * kTileRuns + lane;
      const float w = c.w;
      Pushed u;
      if (PUSH || DJ) {
        u = push_vals(A, c.ix, c.fx, c.y, c.z, c.px, c.py, c.pz, w);
      } else {
        u.ixh = u.ixn = c.ix;
        u.fxh = u.fxn = c.fx;
        u.yh = u.yn = c.y;
        u.zh = u.zn = c.z;
      }
      if (PUSH) {
        A.P.ix[p] = u.ixn;
        A.P.fx[p] = u.fxn;
        A.P.y[p] = u.yn;
        A.P.z[p] = u.zn;
      }
      if (w == 0.0f) continue;
      if (DJ && u.moving) {  // grid_deps.f90:42: no current from particles at rest
        const Loc L = locate(u.ixh, u.fxh, u.yh, u.zh, A.G);
        const float vs[3] = {u.vj[0] * Pl.lJ, u.vj[1] * Pl.lJ, u.vj[2] * Pl.lJ};
        acc_add(cj, L, vs, 0, A.G, geo);
      }
      if (DR) {
        const Loc L = locate(u.ixn, u.fxn, u.yn, u.zn, A.G);
        const float ws[1] = {w * Pl.lR};
        acc_add(cr, L, ws, 3 * NM, A.G, geo);
      }
    }
#pragma unroll
    for (int g = 0; g < G; ++g) cur[g] = nxt[g];
  }
  if (DJ) acc_flush(cj, 0, A.G, geo);
  if (DR) acc_flush(cr, 3 * NM, A.G, geo);
  __syncthreads();
  flush_box(geo, Pl.nvals);
}

// Run kernel of the moving species with three modes: the block's 2048
// slots of the eight particle arrays are first copied into shared memory
// (cp.async, 64 KB) ahead of its box, and two warps take each tile of the
// block (256 threads), both pushing the tile's particles: the even warp sums
// J_x and J_y, the odd warp J_z and rho, 40 node values per lane instead of
// 80, so the sums fit 128 registers and an SM holds 16 warps of the pass
// (2 blocks; one warp per tile with all 80 sums took 213 registers, 8 warps
// per SM, and ran 2.12 against 1.73 ms for 50.3M electrons of the 4096 x
// 512 x 3-mode case, bitwise the same sums).  Only the even warp stores the
// new positions.
template <int NM, bool PUSH, bool DR>
__global__ void __launch_bounds__(2 * kDepThreads, 2) push_deposit_pair_kernel(PushDepArgs A) {
  constexpr bool DJ = true;
  const SpGrid G = window_grid(A.G, A.win);
  extern __shared__ __align__(16) unsigned char dsm[];
  int *box = reinterpret_cast<int *>(dsm + (size_t)kStageArrays * kDepBlock * 4);
  __shared__ int bb[4];
  const i64 base = (i64)blockIdx.x * kDepBlock;
  stage_block(A.P, base, kStageArrays, dsm);
  const StageView V = stage_view(dsm);
  const BlockPlan Pl = plan_block<true>(A, G, base, bb, kSpBoxBytes, V);
  if (Pl.use_box)
    for (int t = threadIdx.x; t < (int)Pl.nvals; t += blockDim.x) box[t] = 0;
  __syncthreads();
  const BoxGeo geo = make_geo(box, Pl, A);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool second = warp & 1;  // J_z and rho (else J_x, J_y)
  const int ltile = (warp >> 1) * kTile;  // this warp pair's tile, local slots
  const i64 first = base + ltile + (i64)lane * kRunLen;
  const int cnt = (int)max((i64)0, min((i64)kRunLen, A.P.n - first));
  auto load = [&](int j) {
    RunPart q;
    const int ls = ltile + j * kTileRuns + lane;
    q.w = V.w[ls];
    q.ix = V.ix[ls];
    q.fx = V.fx[ls];
    q.y = V.y[ls];
    q.z = V.z[ls];
    q.px = V.px[ls];
    q.py = V.py[ls];
    q.pz = V.pz[ls];
    return q;
  };
  auto store = [&](int j, const Pushed &u) {
    if (PUSH && !second) {
      const i64 p = base + ltile + j * kTileRuns + lane;
      A.P.ix[p] = u.ixn;
      A.P.fx[p] = u.fxn;
      A.P.y[p] = u.yn;
      A.P.z[p] = u.zn;
    }
  };
  if (!Pl.use_box) {
    // a block whose nodes do not fit a box: the even warps push and deposit
    // every component straight to the global accumulators
    if (!second)
      for (int j = 0; j < cnt; ++j) {
        const RunPart q = load(j);
        const Pushed u = push_vals(A, q.ix, q.fx, q.y, q.z, q.px, q.py, q.pz, q.w);
        store(j, u);
        if (q.w == 0.0f) continue;
        deposit_global<DJ, DR>(A, G, Pl, u, q.w);
      }
    return;
  }
  if (!second) {
    CellAcc<NM, 2> cxy;
    cxy.live = false;
    for (int j = 0; j < cnt; ++j) {
      const RunPart q = load(j);
      const Pushed u = push_vals(A, q.ix, q.fx, q.y, q.z, q.px, q.py, q.pz, q.w);
      store(j, u);
      if (q.w == 0.0f || !u.moving) continue;  // grid_deps.f90:42
      const Loc L = locate(u.ixh, u.fxh, u.yh, u.zh, G);
      const float vs[2] = {u.vj[0] * Pl.lJ, u.vj[1] * Pl.lJ};
      acc_add(cxy, L, vs, 0, G, geo);
    }
    acc_flush(cxy, 0, G, geo);
  } else {
    CellAcc<NM, 1> cz, cr;
    cz.live = false;
    cr.live = false;
    for (int j = 0; j < cnt; ++j) {
      const RunPart q = load(j);
      const Pushed u = push_vals(A, q.ix, q.fx, q.y, q.z, q.px, q.py, q.pz, q.w);
      if (q.w == 0.0f) continue;
      if (u.moving) {
        const Loc L = locate(u.ixh, u.fxh, u.yh, u.zh, G);
        const float vs[1] = {u.vj[2] * Pl.lJ};
        acc_add(cz, L, vs, 2 * NM, G, geo);
      }
      if (DR) {
        const Loc L = locate(u.ixn, u.fxn, u.yn, u.zn, G);
        const float ws[1] = {q.w * Pl.lR};
        acc_add(cr, L, ws, 3 * NM, G, geo);
      }
    }
    acc_flush(cz, 2 * NM, G, geo);
    if (DR) acc_flush(cr, 3 * NM, G, geo);
  }
  __syncthreads();
  flush_box(geo, Pl.nvals);
}

// Weight sums for the global scale 2^(61 - ceil(log2 B)), B = sum |w|, in a
// fixed order: block b sums the slots [b R, (b+1) R) (R a multiple of 16),
// thread t the 16-slot chunks b R + 16 t + 4096 k in FP32, the block adds its
// threads' sums in FP64 in a fixed tree, the final kernel adds the block
// sums.  With ABSORB the same pass applies the absorbing boundary first
// (species.py:351-398, SimDom test): a live particle outside xmin <= x <=
// xmax, r^2 <= r2max (window cells, (k, f) convention) is marked dead and its
// weight zeroed, so it deposits nothing until a compaction drops it;
// counters[0] counts the dead particles.
constexpr int kWsThreads = 256;
constexpr int kWsChunk = 16;
constexpr int kWsMaxBlocks = 4096;

struct AbsorbBox {
  int win_k;
  float win_f, xmin, xmax, r2max;
};

__device__ __forceinline__ bool outside(const AbsorbBox &Bx, int ix, float fx, float y, float z) {
  const float xc = (float)(ix - Bx.win_k) + (fx - Bx.win_f);
  const float r2 = y * y + z * z;
  return !(xc >= Bx.xmin && xc <= Bx.xmax && r2 <= Bx.r2max);
}

template <bool ABSORB>
__global__ void __launch_bounds__(kWsThreads) weights_kernel(SpParts P, uint8_t *__restrict__ dead,
                                                             AbsorbBox Bx, i64 nphys, i64 R,
                                                             double *__restrict__ partial,
                                                             unsigned long long *counters) {
  const i64 b0 = (i64)blockIdx.x * R, b1 = min(nphys, b0 + R);
  float s = 0.0f;
  unsigned cnt = 0;
  for (i64 c = b0 + (i64)threadIdx.x * kWsChunk; c < b1; c += (i64)kWsThreads * kWsChunk) {
    // a chunk of 16 slots (16-aligned, inside one tile)
    float wv[16];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 t = *reinterpret_cast<const float4 *>(P.w + c + 4 * q);
      wv[4 * q] = t.x, wv[4 * q + 1] = t.y, wv[4 * q + 2] = t.z, wv[4 * q + 3] = t.w;
    }
#pragma unroll
    for (int j = 0; j < kWsChunk; ++j)
      if (logical_of(c + j) >= P.n) wv[j] = 0.0f;  // slots past the last particle
    if (ABSORB) {
      uint4 dv = *reinterpret_cast<const uint4 *>(dead + c);
      uint8_t *db = reinterpret_cast<uint8_t *>(&dv);
      bool changed = false;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int4 ixq = *reinterpret_cast<const int4 *>(P.ix + c + 4 * q);
        const float4 fq = *reinterpret_cast<const float4 *>(P.fx + c + 4 * q);
        const float4 yq = *reinterpret_cast<const float4 *>(P.y + c + 4 * q);
        const float4 zq = *reinterpret_cast<const float4 *>(P.z + c + 4 * q);
        const int xi[4] = {ixq.x, ixq.y, ixq.z, ixq.w};
        const float xf[4] = {fq.x, fq.y, fq.z, fq.w}, yy[4] = {yq.x, yq.y, yq.z, yq.w},
                    zz[4] = {zq.x, zq.y, zq.z, zq.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int j = 4 * q + e;
          if (logical_of(c + j) < P.n && !db[j] && outside(Bx, xi[e], xf[e], yy[e], zz[e])) {
            db[j] = 1;
            wv[j] = 0.0f;
            ++cnt;
            changed = true;
          }
        }
      }
      if (changed) {  // (slots past the last particle get a zero weight)
        *reinterpret_cast<uint4 *>(dead + c) = dv;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          *reinterpret_cast<float4 *>(P.w + c + 4 * q) =
              make_float4(wv[4 * q], wv[4 * q + 1], wv[4 * q + 2], wv[4 * q + 3]);
      }
    }
#pragma unroll
    for (int j = 0; j < kWsChunk; ++j) s += fabsf(wv[j]);
  }
  double d = (double)s;
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
  __shared__ double wsm[kWsThreads / 32];
  if ((threadIdx.x & 31) == 0) wsm[threadIdx.x >> 5] = d;
  if (ABSORB) {
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&counters[0], (unsigned long long)cnt);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kWsThreads / 32; ++k) t += wsm[k];
    partial[blockIdx.x] = t;
  }
}

// sum of the block sums (fixed order: 4 consecutive per thread, then a fixed
// tree) -> out[0] = 2^min(61 - ceil(log2 B), 120), out[1] = B
__global__ void __launch_bounds__(1024) sp_scale_kernel(const double *__restrict__ partial, int np,
                                                        double *out) {
  __shared__ double wsm[32];
  double d = 0.0;
  for (int i = threadIdx.x * 4; i < min(np, (int)threadIdx.x * 4 + 4); ++i) d += partial[i];
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
  if ((threadIdx.x & 31) == 0) wsm[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double B = 0.0;
    for (int k = 0; k < 32; ++k) B += wsm[k];
    if (!(B > 0.0) || !isfinite(B)) B = 1.0;
    // the exponent stays inside the FP32 range the deposit kernels use
    out[0] = ldexp(1.0, min(61 - ceil_log2(B), 120));
    out[1] = B;
  }
}

// blocks and per-block range of the fixed partition of nphys slots
inline void ws_partition(i64 nphys, int *nblocks, i64 *R) {
  i64 nb = (nphys + 4095) / 4096;
  if (nb > kWsMaxBlocks) nb = kWsMaxBlocks;
  if (nb < 1) nb = 1;
  i64 r = (nphys + nb - 1) / nb;
  r = (r + kWsChunk - 1) / kWsChunk * kWsChunk;
  *nblocks = (int)nb;
  *R = r;
}

// Boris rotation (particle_tools.f90:18-56) of one momentum in FP32: 1/gamma
// from a reciprocal square root, one division for 2/(1 + t^2)
__device__ __forceinline__ void boris(float &px, float &py, float &pz, const float *F, float hh) {
  const float um0 = px + hh * F[0], um1 = py + hh * F[1], um2 = pz + hh * F[2];
  const float ig = rsqrtf(1.0f + (um0 * um0 + um1 * um1 + um2 * um2));
  const float t0 = hh * F[3] * ig, t1 = hh * F[4] * ig, t2 = hh * F[5] * ig;
  const float f = 2.0f / (1.0f + (t0 * t0 + t1 * t1 + t2 * t2));
  const float s0 = t0 * f, s1 = t1 * f, s2 = t2 * f;
  const float u0 = um0 + um1 * t2 - um2 * t1, u1 = um1 - um0 * t2 + um2 * t0,
              u2 = um2 + um0 * t1 - um1 * t0;
  px = um0 + u1 * s2 - u2 * s1 + hh * F[0];
  py = um1 - u0 * s2 + u2 * s0 + hh * F[1];
  pz = um2 + u0 * s1 - u1 * s0 + hh * F[2];
}

// gather (proj_fld) + Boris (push_velocs), FP32
struct GatherArgs {
  SpParts P;
  SpGrid G;
  const float2 *eb;  // (nx, nr, nm, 6) complex64, Fortran order
  float dtq;          // push_fact * dt
  const chm_sp_window *win;  // device window origin (or null: G's)
};

// generic gather (any nm), one particle per thread and slot
__global__ void __launch_bounds__(256) gather_push_kernel(GatherArgs A, i64 nphys) {
  const SpGrid G = window_grid(A.G, A.win);
  const i64 plane = (i64)G.nx * G.nr;
  for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < nphys;
       p += (i64)gridDim.x * blockDim.x) {
    if (logical_of(p) >= A.P.n) continue;
    float F[6] = {0, 0, 0, 0, 0, 0};
    const float w = A.P.w[p];
    if (w != 0.0f) {
      Loc L = locate(A.P.ix[p], A.P.fx[p], A.P.y[p], A.P.z[p], G);
      if (L.ok) {
        const float sx[2] = {1.0f - L.sx1, L.sx1};
        const float sr[2] = {1.0f - L.sr1, L.sr1};
        const bool okx0 = L.cx >= 0 && L.cx < G.nx, okx1 = L.cx + 1 >= 0 && L.cx + 1 < G.nx;
        float pr = 1.0f, pi = 0.0f;  // e^{+i m theta}
        for (int m = 0; m < G.nm; ++m) {
          if (m > 0) {
            float a = pr * L.phr - pi * L.phi, b = pr * L.phi + pi * L.phr;
            pr = a;
            pi = b;
          }
#pragma unroll
          for (int l = 0; l < 6; ++l) {
            const float2 *b = A.eb + (i64)(m + G.nm * l) * plane + (i64)L.cr * G.nx + L.cx;
            float acc = 0.0f;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              if (okx0) {
                float2 f = b[j * G.nx];
                acc += sr[j] * sx[0] * (pr * f.x - pi * f.y);
              }
              if (okx1) {
                float2 f = b[j * G.nx + 1];
                acc += sr[j] * sx[1] * (pr * f.x - pi * f.y);
              }
            }
            F[l] += acc;
          }
        }
      }
    }
    float px = A.P.px[p], py = A.P.py[p], pz = A.P.pz[p];
    boris(px, py, pz, F, 0.5f * A.dtq);
    A.P.px[p] = px;
    A.P.py[p] = py;
    A.P.pz[p] = pz;
  }
}

// Run form of gather + Boris for nm = 1..3: lane r walks run r of its tile
// and keeps the fields of the current cell in registers (mode 0: real parts;
// modes >= 1: complex) as their bilinear form over the cell, rebuilt only
// when the cell changes (3 FMAs per value and particle instead of 4 node
// products).  The same interpolation and rotation as gather_push_kernel, up
// to FP32 rounding.
// (staged in shared memory with three modes, as the deposit; unstaged with
// its tile started towards L2 and 4 blocks per SM otherwise)
template <int NM>
__global__ void __launch_bounds__(kDepThreads, NM >= 3 ? 3 : 4) gather_push_run_kernel(GatherArgs A) {
  extern __shared__ __align__(16) unsigned char gsm[];
  const SpGrid G = window_grid(A.G, A.win);
  const i64 plane = (i64)G.nx * G.nr;
  const int lane = threadIdx.x & 31;
  const i64 base = (i64)blockIdx.x * kDepBlock;
  if (NM >= 3) stage_block(A.P, base, kStageArrays, gsm);
  else prefetch_tile(A.P, base + (threadIdx.x >> 5) * kTile, lane, true);
  const StageView V = NM >= 3 ? stage_view(gsm) : global_view(A.P, base);
  const int ltile = (threadIdx.x >> 5) * kTile;  // this warp's tile, local slots
  const i64 tile = base + ltile;
  const i64 first = tile + (i64)lane * kRunLen;
  int ccx = INT_MIN, ccr = INT_MIN;
  float f0[6][4];
  float2 f1[NM > 1 ? NM - 1 : 1][6][4];
  const int cnt = (int)max((i64)0, min((i64)kRunLen, A.P.n - first));
  struct Part {
    int ix;
    float fx, y, z, px, py, pz, w;
  };
  auto load = [&](int j) {
    Part q;
    const int ls = ltile + j * kTileRuns + lane;
    if (NM >= 3) {
      q.w = V.w[ls];
      q.ix = V.ix[ls];
      q.fx = V.fx[ls];
      q.y = V.y[ls];
      q.z = V.z[ls];
      q.px = V.px[ls];
      q.py = V.py[ls];
      q.pz = V.pz[ls];
    } else {  // straight from the arguments' arrays
      const i64 p = base + ls;
      q.w = A.P.w[p];
      q.ix = A.P.ix[p];
      q.fx = A.P.fx[p];
      q.y = A.P.y[p];
      q.z = A.P.z[p];
      q.px = A.P.px[p];
      q.py = A.P.py[p];
      q.pz = A.P.pz[p];
    }
    return q;
  };
  Part cur;
  if (cnt > 0) cur = load(0);
  for (int j = 0; j < cnt; ++j) {
    Part nxt;
    if (j + 1 < cnt) nxt = load(j + 1);  // loaded before this particle's store
    const i64 p = tile + (i64)j * kTileRuns + lane;
    float F[6] = {0, 0, 0, 0, 0, 0};
    if (cur.w != 0.0f) {
      const Loc L = locate(cur.ix, cur.fx, cur.y, cur.z, G);
      if (L.ok) {
        if (L.cx != ccx || L.cr != ccr) {
          ccx = L.cx;
          ccr = L.cr;
#pragma unroll
          for (int nd = 0; nd < 4; ++nd) {
            const int gx = L.cx + (nd & 1), gr = L.cr + (nd >> 1);
            const bool okx = gx >= 0 && gx < G.nx;
#pragma unroll
            for (int l = 0; l < 6; ++l) {
              const float2 *b = A.eb + (i64)(G.nm * l) * plane + (i64)gr * G.nx + gx;
              f0[l][nd] = okx ? b[0].x : 0.0f;
#pragma unroll
              for (int m = 1; m < NM; ++m)
                f1[m - 1][l][nd] = okx ? b[(i64)m * plane] : make_float2(0.0f, 0.0f);
            }
          }
          // the cell's bilinear form v00 + sx1 (v01 - v00 + sr1 d) + sr1
          // (v10 - v00), d = v11 - v10 - v01 + v00, kept in place of the
          // node values (nd: 0 the constant, 1 the x slope, 2 the r slope, 3 d)
#pragma unroll
          for (int l = 0; l < 6; ++l) {
            const float v00 = f0[l][0], v01 = f0[l][1], v10 = f0[l][2], v11 = f0[l][3];
            f0[l][1] = v01 - v00;
            f0[l][2] = v10 - v00;
            f0[l][3] = (v11 - v10) - (v01 - v00);
#pragma unroll
            for (int m = 1; m < NM; ++m) {
              const float2 u00 = f1[m - 1][l][0], u01 = f1[m - 1][l][1], u10 = f1[m - 1][l][2],
                           u11 = f1[m - 1][l][3];
              f1[m - 1][l][1] = make_float2(u01.x - u00.x, u01.y - u00.y);
              f1[m - 1][l][2] = make_float2(u10.x - u00.x, u10.y - u00.y);
              f1[m - 1][l][3] = make_float2((u11.x - u10.x) - (u01.x - u00.x),
                                            (u11.y - u10.y) - (u01.y - u00.y));
            }
          }
        }
        const float s1 = L.sx1, t1 = L.sr1;
#pragma unroll
        for (int l = 0; l < 6; ++l)
          F[l] += fmaf(s1, fmaf(f0[l][3], t1, f0[l][1]), fmaf(f0[l][2], t1, f0[l][0]));
        float pr = 1.0f, pi = 0.0f;  // e^{+i m theta}
#pragma unroll
        for (int m = 1; m < NM; ++m) {
          const float a = pr * L.phr - pi * L.phi, b2 = pr * L.phi + pi * L.phr;
          pr = a;
          pi = b2;
#pragma unroll
          for (int l = 0; l < 6; ++l) {
            const float2 *c = f1[m - 1][l];
            const float ur = fmaf(s1, fmaf(c[3].x, t1, c[1].x), fmaf(c[2].x, t1, c[0].x));
            const float ui = fmaf(s1, fmaf(c[3].y, t1, c[1].y), fmaf(c[2].y, t1, c[0].y));
            F[l] += pr * ur - pi * ui;
          }
        }
      }
    }
    float px = cur.px, py = cur.py, pz = cur.pz;
    boris(px, py, pz, F, 0.5f * A.dtq);
    A.P.px[p] = px;
    A.P.py[p] = py;
    A.P.pz[p] = pz;
    cur = nxt;
  }
}


// ----------------------------------------------------------------------
// Envelope (KxShift) solver: the beam's current deposit and its gather +
// external undulator field + Boris push (grid_deps_env.f90:18-95, 164-238;
// devices.f90:117-203).  The solver stores the modes -K..K at slots
// 0..2K.  The carrier e^{-i kx0 x} of a position (ix, fx) is a per-cell
// table value (built in FP64 for the window's cells, chm_sp_carrier) times
// e^{-i kx0 dx fx} in FP32, so its phase error stays at the FP32 rounding
// of kx0 dx fx instead of growing with kx0 x.
// ----------------------------------------------------------------------
struct EnvArgs {
  const float2 *tab;  // e^{-i kx0 (X0 + (k + c - 2) dx)}, c = 0 .. nx + 3, k the window cell
  float kdx;          // kx0 dx
};

// Background density of a still species after a window move by a whole
// number of cells ns: every node value moves ns columns left (the
// particles' positions relative to the grid shift by exactly ns cells, so
// their cells, weights, block plans and run sums are those of the previous
// deposit), the ns columns entering at the right are left zero for the
// masked deposit.  One block per row of the (nx, rows) {re, im} int64 grid.
constexpr int kShiftThreads = 1024;
constexpr int kShiftMaxNx = 14000;  // a row of 16-byte values in shared memory

__global__ void __launch_bounds__(kShiftThreads) shift_acc_kernel(longlong2 *acc, int nx, int ns) {
  extern __shared__ __align__(16) longlong2 srow[];
  longlong2 *row = acc + (i64)blockIdx.x * nx;
  for (int x = threadIdx.x; x < nx; x += kShiftThreads) srow[x] = row[x];
  __syncthreads();  // the whole row read before any write
  for (int x = threadIdx.x; x < nx; x += kShiftThreads)
    row[x] = x + ns < nx ? srow[x + ns] : make_longlong2(0, 0);
}


__global__ void carrier_kernel(float2 *tab, int ntab, double kx0, double X0, double dx, int win_k,
                               const chm_sp_window *win) {
  const int k = win ? win->k : win_k;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ntab; c += gridDim.x * blockDim.x) {
    double sv, cv;
    sincos(kx0 * (X0 + (double)(k + c - 2) * dx), &sv, &cv);
    tab[c] = make_float2((float)cv, (float)-sv);
  }
}

// e^{-i kx0 x} at (ix, fx); zero outside the table (no node of such a
// position lies in the grid: window-relative cells -1 .. nx keep c in
// 1 .. nx + 2)
__device__ __forceinline__ float2 env_carrier(const EnvArgs &E, const SpGrid &G, int ix, float fx) {
  const int c = ix - G.win_k + 2;
  if (c < 0 || c >= G.nx + 4) return make_float2(0.f, 0.f);
  float sv, cv;
  sincosf(E.kdx * fx, &sv, &cv);
  const float2 t = E.tab[c];
  return make_float2(t.x * cv + t.y * sv, t.y * cv - t.x * sv);  // t (cv - i sv)
}

__device__ __forceinline__ float2 cmf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Push + J deposit of the envelope solver's moving species (NM = 2K + 1
// stored modes): the coordinate push of push_coords, then at the half step
// J_z only (grid_deps_env.f90:76 deposits the third component alone) with
// value (p_z / gamma) w e^{-i kx0 x} e^{-+i m theta} at slot K +- m.  Lane r
// walks run r of its tile (the tile layout) and sums its particles' node
// values in FP32 registers while the deposit cell stays the same; the sums,
// already at the global quantum, are rounded and added to the 64-bit
// accumulator when the cell changes.
template <int NM>
__global__ void __launch_bounds__(kDepThreads) push_deposit_env_kernel(PushDepArgs A, EnvArgs E) {
  constexpr int K = (NM - 1) / 2;
  const SpGrid G = window_grid(A.G, A.win);
  const float sJ = (float)A.scaleJ[0];
  const int lane = threadIdx.x & 31;
  const i64 tile = (i64)blockIdx.x * kDepBlock + (i64)(threadIdx.x >> 5) * kTile;
  const i64 first = tile + (i64)lane * kRunLen;
  const int cnt = (int)max((i64)0, min((i64)kRunLen, A.P.n - first));
  prefetch_tile(A.P, tile, lane, true);
  int ccx = 0, ccr = 0;
  bool live = false;
  float v[NM][4][2];
  auto flush = [&]() {
    if (!live) return;
#pragma unroll
    for (int sl = 0; sl < NM; ++sl)
#pragma unroll
      for (int nd = 0; nd < 4; ++nd) {
        const int gx = ccx + (nd & 1), r = ccr + (nd >> 1);
        if (gx < 0 || gx >= G.nx) continue;
        const i64 e = ((i64)(sl + NM * 2) * G.nr + r) * G.nx + gx;
        const long long qr = f2ll(v[sl][nd][0]), qi = f2ll(v[sl][nd][1]);
        if (qr) atomicAdd(&A.accJ[2 * e], (unsigned long long)qr);
        if (qi) atomicAdd(&A.accJ[2 * e + 1], (unsigned long long)qi);
      }
    live = false;
  };
  // the next particle is loaded before this one is processed (its stores
  // could alias the loads otherwise)
  auto load = [&](int j) {
    RunPart q;
    const i64 p = tile + (i64)j * kTileRuns + lane;
    q.w = A.P.w[p];
    q.ix = A.P.ix[p];
    q.fx = A.P.fx[p];
    q.y = A.P.y[p];
    q.z = A.P.z[p];
    q.px = A.P.px[p];
    q.py = A.P.py[p];
    q.pz = A.P.pz[p];
    return q;
  };
  RunPart cur, nxt;
  if (cnt > 0) cur = load(0);
  for (int j = 0; j < cnt; ++j) {
    if (j + 1 < cnt) nxt = load(j + 1);
    const RunPart q = cur;
    cur = nxt;
    const i64 p = tile + (i64)j * kTileRuns + lane;
    const float w = q.w;
    const Pushed u = A.far ? push_vals_far(A, q.ix, q.fx, q.y, q.z, q.px, q.py, q.pz, w)
                           : push_vals(A, q.ix, q.fx, q.y, q.z, q.px, q.py, q.pz, w);
    A.P.ix[p] = u.ixn;
    A.P.fx[p] = u.fxn;
    A.P.y[p] = u.yn;
    A.P.z[p] = u.zn;
    if (w == 0.0f || !u.moving) continue;
    const Loc L = locate(u.ixh, u.fxh, u.yh, u.zh, G);
    if (!L.ok) continue;
    if (!live || L.cx != ccx || L.cr != ccr) {
      flush();
      ccx = L.cx;
      ccr = L.cr;
      live = true;
#pragma unroll
      for (int sl = 0; sl < NM; ++sl)
#pragma unroll
        for (int nd = 0; nd < 4; ++nd) v[sl][nd][0] = v[sl][nd][1] = 0.0f;
    }
    const float2 car = env_carrier(E, G, u.ixh, u.fxh);
    const float a = u.vj[2] * sJ;  // p_z w / gamma at the global quantum
    const float2 base = make_float2(car.x * a, car.y * a);
    const float sx[2] = {1.0f - L.sx1, L.sx1};
    const float sr[2] = {1.0f - L.sr1, L.sr1};
    const float2 ph = make_float2(L.phr, -L.phi);  // e^{-i theta} (0 on the axis)
    float2 phm = make_float2(1.0f, 0.0f);
#pragma unroll
    for (int mi = 0; mi <= K; ++mi) {
      if (mi > 0) phm = cmf(phm, ph);
#pragma unroll
      for (int side = 0; side < (mi > 0 ? 2 : 1); ++side) {
        const float2 pm = side ? make_float2(phm.x, -phm.y) : phm;
        const int sl = side ? K - mi : K + mi;
        const float2 val = cmf(pm, base);
#pragma unroll
        for (int nd = 0; nd < 4; ++nd) {
          const float sh = sx[nd & 1] * sr[nd >> 1];
          v[sl][nd][0] += val.x * sh;
          v[sl][nd][1] += val.y * sh;
        }
      }
    }
  }
  flush();
}

// The undulators of devices.f90 on a particle at x (its cell ix, offset fx):
//   undul_analytic[_taper] (devices.f90:117-203): with xr = x - X0u,
//     B_y += a s cosh(ku y), B_x += a c sinh(ku y), (s, c) = sincos(ku xr),
//     a = a0 ramp(xr) [taper], ramps of one period at both ends;
//   undul_mapped[_tap] (devices.f90:18-115): the amplitudes a(2, nmap) of a
//     field map of step mdx from Xleft, interpolated with quadratic weights
//     at xm = x - Xleft (the reference's columns ix - 2 .. ix), B_y += amp
//     s1 cosh(ku y), B_x += amp s2 sinh(ku y), amp the taper or 1.
// Positions relative to the undulator are formed from FP64 cell offsets.
struct UndArgs {
  int kind;          // 0 none, 1 undul_analytic, 2 _taper, 3 undul_mapped, 4 _tap
  float a0, lam, ku, len, taper;
  double xo, dx;     // X0 (particles' origin) - undulator start (X0u or Xleft); cell size
  const float2 *map; // mapped: (a(0, col), a(1, col)) per column
  int nmap;
  float mdx, mdx_inv, x_shift;
};

__device__ __forceinline__ void undulator(float *F, int ix, float fx, float y, const UndArgs &U) {
  const float xr = (float)(U.xo + (double)ix * U.dx) + fx * (float)U.dx;
  if (U.kind >= 3) {
    if (xr < U.mdx || xr > U.nmap * U.mdx - U.mdx) return;
    const float u = xr * U.mdx_inv;
    const int im = (int)floorf(u + 0.5f);
    const float d = u - (float)im;
    const float S[3] = {0.5f * (0.5f - d) * (0.5f - d), 0.75f - d * d, 0.5f * (0.5f + d) * (0.5f + d)};
    float s1 = 0.0f, s2 = 0.0f;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int col = im - 2 + q;
      if (col < 0 || col >= U.nmap) continue;
      const float2 a = U.map[col];
      s1 += S[q] * a.x;
      s2 += S[q] * a.y;
    }
    const float amp =
        U.kind == 4 ? 1.0f + U.taper * (xr - U.x_shift - 0.5f * U.len) / (0.5f * U.len) : 1.0f;
    F[4] += amp * s1 * coshf(U.ku * y);
    F[3] += amp * s2 * sinhf(U.ku * y);
    return;
  }
  float ampl;
  if (xr <= 0.0f || xr >= U.len) ampl = 0.0f;
  else if (xr < U.lam) ampl = xr / U.lam;
  else if (xr > U.len - U.lam) ampl = (U.len - xr) / U.lam;
  else ampl = 1.0f;
  if (U.kind == 2) ampl *= 1.0f + U.taper * (xr - 0.5f * U.len) / (0.5f * U.len);
  ampl *= U.a0;
  float sv, cv;
  sincosf(U.ku * xr, &sv, &cv);
  F[4] += ampl * sv * coshf(U.ku * y);
  F[3] += ampl * cv * sinhf(U.ku * y);
}

// Gather of the envelope fields (carrier e^{+i kx0 x}, phase e^{+-i m theta}
// at slot K +- m, 1 on the axis), the undulator field, Boris push
template <int NM>
__global__ void __launch_bounds__(kDepThreads) gather_push_env_kernel(GatherArgs A, EnvArgs E,
                                                                     UndArgs U) {
  constexpr int K = (NM - 1) / 2;
  const SpGrid G = window_grid(A.G, A.win);
  const i64 plane = (i64)G.nx * G.nr;
  // lane r walks run r of its tile (the tile layout), the next particle
  // loaded before this one is processed
  const int lane = threadIdx.x & 31;
  const i64 tile = (i64)blockIdx.x * kDepBlock + (i64)(threadIdx.x >> 5) * kTile;
  const i64 first = tile + (i64)lane * kRunLen;
  const int cnt = (int)max((i64)0, min((i64)kRunLen, A.P.n - first));
  prefetch_tile(A.P, tile, lane, true);
  auto load = [&](int j) {
    RunPart q;
    const i64 p = tile + (i64)j * kTileRuns + lane;
    q.w = A.P.w[p];
    q.ix = A.P.ix[p];
    q.fx = A.P.fx[p];
    q.y = A.P.y[p];
    q.z = A.P.z[p];
    q.px = A.P.px[p];
    q.py = A.P.py[p];
    q.pz = A.P.pz[p];
    return q;
  };
  RunPart cur, nxt;
  if (cnt > 0) cur = load(0);
  for (int j = 0; j < cnt; ++j) {
    if (j + 1 < cnt) nxt = load(j + 1);
    const RunPart q = cur;
    cur = nxt;
    const i64 p = tile + (i64)j * kTileRuns + lane;
    float F[6] = {0, 0, 0, 0, 0, 0};
    if (q.w != 0.0f) {
      const Loc L = locate(q.ix, q.fx, q.y, q.z, G);
      if (L.ok) {
        const float sx[2] = {1.0f - L.sx1, L.sx1};
        const float sr[2] = {1.0f - L.sr1, L.sr1};
        const bool okx0 = L.cx >= 0 && L.cx < G.nx, okx1 = L.cx + 1 >= 0 && L.cx + 1 < G.nx;
        const float2 c0 = env_carrier(E, G, q.ix, q.fx);
        const float2 car = make_float2(c0.x, -c0.y);  // e^{+i kx0 x}
        const bool axis = !(q.y * q.y + q.z * q.z > 0.0f);
        const float2 ph = axis ? make_float2(1.0f, 0.0f) : make_float2(L.phr, L.phi);
        float2 phm = make_float2(1.0f, 0.0f);
#pragma unroll
        for (int mi = 0; mi <= K; ++mi) {
          if (mi > 0) phm = cmf(phm, ph);
#pragma unroll
          for (int side = 0; side < (mi > 0 ? 2 : 1); ++side) {
            const float2 pm = cmf(car, side ? make_float2(phm.x, -phm.y) : phm);
            const int sl = side ? K - mi : K + mi;
#pragma unroll
            for (int l = 0; l < 6; ++l) {
              const float2 *b = A.eb + (i64)(sl + NM * l) * plane + (i64)L.cr * G.nx + L.cx;
              float acc = 0.0f;
#pragma unroll
              for (int jr = 0; jr < 2; ++jr) {
                if (okx0) {
                  const float2 f = b[jr * G.nx];
                  acc += sr[jr] * sx[0] * (pm.x * f.x - pm.y * f.y);
                }
                if (okx1) {
                  const float2 f = b[jr * G.nx + 1];
                  acc += sr[jr] * sx[1] * (pm.x * f.x - pm.y * f.y);
                }
              }
              F[l] += acc;
            }
          }
        }
      }
    }
    if (U.kind) undulator(F, q.ix, q.fx, q.y, U);
    float px = q.px, py = q.py, pz = q.pz;
    boris(px, py, pz, F, 0.5f * A.dtq);
    A.P.px[p] = px;
    A.P.py[p] = py;
    A.P.pz[p] = pz;
  }
}


// FP64 (3, n) strided particle arrays -> split layout, as particles off ..
// off + n - 1 (their dead flags cleared)
__global__ void from_f64_kernel(SpParts P, uint8_t *dead, i64 off, const double *__restrict__ x,
                                i64 x_cs, i64 x_ps, const double *__restrict__ p, i64 p_cs,
                                i64 p_ps, const double *__restrict__ w, i64 w_ps, double X0,
                                double dx_inv, i64 n) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const double s = (x[i * x_ps] - X0) * dx_inv;
    const double fl = floor(s);
    float fr = (float)(s - fl);
    int ix = (int)fl;
    if (fr >= 1.0f) {  // rounding up to the next cell
      fr = 0.0f;
      ix += 1;
    }
    const i64 q = phys_of(off + i);
    P.ix[q] = ix;
    P.fx[q] = fr;
    P.y[q] = (float)x[x_cs + i * x_ps];
    P.z[q] = (float)x[2 * x_cs + i * x_ps];
    P.px[q] = (float)p[i * p_ps];
    P.py[q] = (float)p[p_cs + i * p_ps];
    P.pz[q] = (float)p[2 * p_cs + i * p_ps];
    P.w[q] = (float)w[i * w_ps];
    if (dead) dead[q] = 0;
  }
}

__global__ void to_f64_kernel(SpParts P, double *__restrict__ x, i64 x_cs, i64 x_ps,
                              double *__restrict__ p, i64 p_cs, i64 p_ps, double *__restrict__ w,
                              i64 w_ps, double X0, double dx) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P.n; i += (i64)gridDim.x * blockDim.x) {
    const i64 q = phys_of(i);
    x[i * x_ps] = X0 + ((double)P.ix[q] + (double)P.fx[q]) * dx;
    x[x_cs + i * x_ps] = P.y[q];
    x[2 * x_cs + i * x_ps] = P.z[q];
    p[i * p_ps] = P.px[q];
    p[p_cs + i * p_ps] = P.py[q];
    p[2 * p_cs + i * p_ps] = P.pz[q];
    if (w) w[i * w_ps] = P.w[q];
  }
}

// counters[1] += n - counters[0]: live particles of this step
__global__ void live_steps_kernel(unsigned long long *counters, i64 n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) counters[1] += (unsigned long long)n - counters[0];
}

// Stable compaction of the live particles (in particle order): counts per
// 4096 particles, one scan, scatter.
constexpr int kCmpThreads = 256;
constexpr int kCmpTile = 4096;  // particles per count

__global__ void __launch_bounds__(kCmpThreads) compact_count_kernel(const uint8_t *__restrict__ dead,
                                                                    i64 n, int *__restrict__ cnt) {
  const i64 t0 = (i64)blockIdx.x * kCmpTile, t1 = min(n, t0 + kCmpTile);
  int c = 0;
  for (i64 i = t0 + threadIdx.x; i < t1; i += kCmpThreads) c += dead[phys_of(i)] ? 0 : 1;
  c = __reduce_add_sync(0xffffffffu, c);
  __shared__ int ws[kCmpThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < kCmpThreads / 32; ++k) s += ws[k];
    cnt[blockIdx.x] = s;
  }
}

// exclusive scan of the counts in place (one block), total -> n_out
__global__ void __launch_bounds__(1024) compact_scan_kernel(int *__restrict__ cnt, int ntiles,
                                                            int64_t *__restrict__ n_out) {
  __shared__ long long part[1024];
  const int per = (ntiles + 1023) / 1024;
  const int a = threadIdx.x * per, b = min(ntiles, a + per);
  long long s = 0;
  for (int i = a; i < b; ++i) s += cnt[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan
    const long long v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  long long run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int i = a; i < b; ++i) {
    const int c = cnt[i];
    cnt[i] = (int)run;  // offsets stay below 2^31: checked on the host
    run += c;
  }
  if (threadIdx.x == 1023) *n_out = part[1023];
}

__global__ void __launch_bounds__(kCmpThreads) compact_scatter_kernel(SpParts S, SpParts D,
                                                                      const uint8_t *__restrict__ dead,
                                                                      const int *__restrict__ off) {
  const i64 t0 = (i64)blockIdx.x * kCmpTile, t1 = min(S.n, t0 + kCmpTile);
  __shared__ int wsum[kCmpThreads / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = off[blockIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (i64 c0 = t0; c0 < t1; c0 += kCmpThreads) {
    const i64 i = c0 + threadIdx.x;
    const i64 q = phys_of(i);
    const bool live = i < t1 && !dead[q];
    const unsigned m = __ballot_sync(0xffffffffu, live);
    if (lane == 0) wsum[warp] = __popc(m);
    __syncthreads();
    int before = carry;
    for (int k = 0; k < warp; ++k) before += wsum[k];
    if (live) {
      const i64 j = phys_of((i64)before + __popc(m & ((1u << lane) - 1u)));
      D.ix[j] = S.ix[q];
      D.fx[j] = S.fx[q];
      D.y[j] = S.y[q];
      D.z[j] = S.z[q];
      D.px[j] = S.px[q];
      D.py[j] = S.py[q];
      D.pz[j] = S.pz[q];
      D.w[j] = S.w[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int k = 0; k < kCmpThreads / 32; ++k) t += wsum[k];
      carry += t;
    }
    __syncthreads();
  }
}

}  // namespace

extern "C" {

// The split-form particle entry points take the eight SoA arrays in the
// order ix, fx, y, z, px, py, pz, w (n particles in the tile order above,
// arrays of chm_sp_capacity(n) slots).

int64_t chm_sp_capacity(int64_t n) { return n <= 0 ? 0 : tiles_of(n) * kTile; }

int64_t chm_sp_slot(int64_t i) { return phys_of(i); }

int64_t chm_sp_scale_ws_bytes(void) { return 8 * (int64_t)kWsMaxBlocks + 256; }

int chm_sp_weight_scale(double *scale2, const float *w, int64_t n, void *ws, int64_t ws_bytes,
                        void *stream) {
  CHM_REQUIRE(scale2 && n >= 0 && ws && ws_bytes >= chm_sp_scale_ws_bytes(),
              "sp_weight_scale: bad args");
  cudaStream_t st = as_stream(stream);
  double *partial = reinterpret_cast<double *>(ws);
  int nb = 1;
  if (n > 0) {
    CHM_REQUIRE(w && (reinterpret_cast<uintptr_t>(w) & 15u) == 0,
                "sp_weight_scale: weights must start on a 16-byte boundary");
    i64 R;
    const i64 nphys = tiles_of(n) * kTile;
    ws_partition(nphys, &nb, &R);
    SpParts P{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, const_cast<float *>(w), n};
    weights_kernel<false><<<nb, kWsThreads, 0, st>>>(P, nullptr, AbsorbBox{}, nphys, R, partial,
                                                     nullptr);
    chm::count_launch();
  } else {
    cudaMemsetAsync(partial, 0, 8, st);
  }
  sp_scale_kernel<<<1, 1024, 0, st>>>(partial, nb, scale2); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"

namespace {

// push + deposit with the cell-run kernels for nm <= 3 (the per-particle
// kernel for more modes), or the per-particle kernel for every nm (generic)
int push_deposit(int32_t *ix, float *fx, float *y, float *z, float *px, float *py, float *pz,
                 float *w, int64_t n, int win_k, float win_f, float dx_inv, float dr_inv, float dt,
                 int nx, int nr, int nm, int push, uint64_t *accJ, const double *scaleJ,
                 uint64_t *accR, const double *scaleR, void *stream, bool generic,
                 const chm_sp_window *win) {
  CHM_REQUIRE(n >= 0 && nx > 1 && nr > 1 && nm >= 1 && nm <= 8, "sp_push_deposit: bad dims");
  if (n == 0) return CHM_OK;
  CHM_REQUIRE(ix && fx && y && z && px && py && pz && w, "sp_push_deposit: null particle array");
  CHM_REQUIRE(!accJ || scaleJ, "sp_push_deposit: J accumulator without scale");
  CHM_REQUIRE(!accR || scaleR, "sp_push_deposit: rho accumulator without scale");
  PushDepArgs A{};
  A.P = SpParts{ix, fx, y, z, px, py, pz, w, n};
  A.G = SpGrid{win_k, win_f, dr_inv, nx, nr, nm};
  A.dt = dt;
  A.dx_inv = dx_inv;
  A.push = push;
  A.dep_j = accJ != nullptr;
  A.dep_rho = accR != nullptr;
  A.accJ = reinterpret_cast<unsigned long long *>(accJ);
  A.accR = reinterpret_cast<unsigned long long *>(accR);
  A.scaleJ = scaleJ;
  A.scaleR = scaleR;
  A.win = win;
  const unsigned blocks = (unsigned)((n + kDepBlock - 1) / kDepBlock);
  cudaStream_t st = as_stream(stream);
  // run kernels for nm 1..3 and the three uses: moving species (push, J,
  // rho), moving species without the fused rho, still species (rho)
  void (*kern)(PushDepArgs) = nullptr;
  if (!generic && nm >= 1 && nm <= 3) {
    const int mode = (push ? 4 : 0) | (A.dep_j ? 2 : 0) | (A.dep_rho ? 1 : 0);
    if (mode == 7) kern = nm == 1 ? push_deposit_run_kernel<1, true, true, true>
                        : nm == 2 ? push_deposit_run_kernel<2, true, true, true>
                                  : push_deposit_pair_kernel<3, true, true>;
    if (mode == 6) kern = nm == 1 ? push_deposit_run_kernel<1, true, true, false>
                        : nm == 2 ? push_deposit_run_kernel<2, true, true, false>
                                  : push_deposit_pair_kernel<3, true, false>;
    if (mode == 1 && n < (i64)INT32_MAX - kDepBlock)
      kern = nm == 1 ? push_deposit_run_kernel<1, false, false, true>
           : nm == 2 ? push_deposit_run_kernel<2, false, false, true>
                     : push_deposit_run_kernel<3, false, false, true>;
  }
  int box_bytes = kSpBoxBytes;
  if (!kern) {
    kern = push_deposit_kernel;
  } else {
    // the three-mode moving species' kernels stage the block's particles
    // ahead of the box
    box_bytes = !A.dep_j ? kRhoBoxBytes
              : (nm >= 3 ? kStageArrays * kDepBlock * 4 + kSpBoxBytes : kSpBoxBytes);
  }
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, box_bytes);
  // (the three-mode moving species' kernel runs two warps per tile, 2 blocks
  // of 104 KB per SM)
  const bool pair = kern != push_deposit_kernel && A.dep_j && nm >= 3;
  if (pair) cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  const int threads = pair ? 2 * kDepThreads : kDepThreads;
  kern<<<blocks, threads, box_bytes, st>>>(A);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int gather_push(int32_t *ix, float *fx, float *y, float *z, float *px, float *py, float *pz,
                float *w, int64_t n, int win_k, float win_f, float dr_inv, const void *eb_c64, int nx,
                int nr, int nm, float dtq, void *stream, bool generic, const chm_sp_window *win) {
  CHM_REQUIRE(n >= 0 && nx > 1 && nr > 1 && nm >= 1, "sp_gather_push: bad dims");
  if (n == 0) return CHM_OK;
  CHM_REQUIRE(ix && fx && y && z && px && py && pz && w && eb_c64, "sp_gather_push: null pointer");
  GatherArgs A{};
  A.P = SpParts{ix, fx, y, z, px, py, pz, w, n};
  A.G = SpGrid{win_k, win_f, dr_inv, nx, nr, nm};
  A.eb = reinterpret_cast<const float2 *>(eb_c64);
  A.dtq = dtq;
  A.win = win;
  cudaStream_t st = as_stream(stream);
  if (!generic && nm >= 1 && nm <= 3) {
    const unsigned blocks = (unsigned)((n + kDepBlock - 1) / kDepBlock);
    // with three modes each block stages its 2048 slots of the eight particle
    // arrays (a two-warps-per-tile form with the E and B halves in separate
    // warps measured 1.14 against 1.01 ms at 4096 x 512 x 3 modes)
    const int sm = nm >= 3 ? kStageArrays * kDepBlock * 4 : 0;
    void (*kern)(GatherArgs) =
        nm == 1 ? gather_push_run_kernel<1> : nm == 2 ? gather_push_run_kernel<2> : gather_push_run_kernel<3>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    kern<<<blocks, kDepThreads, sm, st>>>(A);
  } else {
    const i64 nphys = tiles_of(n) * kTile;
    gather_push_kernel<<<grid_for(nphys, 256, 16), 256, 0, st>>>(A, nphys);
  }
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // namespace

extern "C" {

int chm_sp_push_deposit(int32_t *ix, float *fx, float *y, float *z, float *px, float *py,
                        float *pz, float *w, int64_t n, int win_k, float win_f, float dx_inv,
                        float dr_inv, float dt, int nx, int nr, int nm, int push,
                        uint64_t *accJ, const double *scaleJ, uint64_t *accR,
                        const double *scaleR, void *stream, const chm_sp_window *win) {
  return push_deposit(ix, fx, y, z, px, py, pz, w, n, win_k, win_f, dx_inv, dr_inv, dt, nx, nr, nm,
                      push, accJ, scaleJ, accR, scaleR, stream, false, win);
}

int chm_sp_push_deposit_generic(int32_t *ix, float *fx, float *y, float *z, float *px, float *py,
                                float *pz, float *w, int64_t n, int win_k, float win_f,
                                float dx_inv, float dr_inv, float dt, int nx, int nr, int nm,
                                int push, uint64_t *accJ, const double *scaleJ, uint64_t *accR,
                                const double *scaleR, void *stream, const chm_sp_window *win) {
  return push_deposit(ix, fx, y, z, px, py, pz, w, n, win_k, win_f, dx_inv, dr_inv, dt, nx, nr, nm,
                      push, accJ, scaleJ, accR, scaleR, stream, true, win);
}

int64_t chm_sp_deposit_dropped(void) {
  unsigned int v = 0, z = 0;
  cudaMemcpyFromSymbol(&v, g_dep_dropped, sizeof(v));
  cudaMemcpyToSymbol(g_dep_dropped, &z, sizeof(z));
  return (int64_t)v;
}

int chm_sp_gather_push(int32_t *ix, float *fx, float *y, float *z, float *px, float *py, float *pz,
                       float *w, int64_t n, int win_k, float win_f, float dr_inv,
                       const void *eb_c64, int nx, int nr, int nm, float dtq, void *stream,
                       const chm_sp_window *win) {
  return gather_push(ix, fx, y, z, px, py, pz, w, n, win_k, win_f, dr_inv, eb_c64, nx, nr, nm, dtq,
                     stream, false, win);
}

int chm_sp_gather_push_generic(int32_t *ix, float *fx, float *y, float *z, float *px, float *py,
                               float *pz, float *w, int64_t n, int win_k, float win_f,
                               float dr_inv, const void *eb_c64, int nx, int nr, int nm, float dtq,
                               void *stream, const chm_sp_window *win) {
  return gather_push(ix, fx, y, z, px, py, pz, w, n, win_k, win_f, dr_inv, eb_c64, nx, nr, nm, dtq,
                     stream, true, win);
}

int chm_sp_carrier(void *tab_c64, int64_t ntab, double kx0, double X0, double dx, int win_k,
                   void *stream, const chm_sp_window *win) {
  CHM_REQUIRE(tab_c64 && ntab > 0 && ntab < (1 << 30), "sp_carrier: bad args");
  carrier_kernel<<<grid_for(ntab, 128), 128, 0, as_stream(stream)>>>(
      reinterpret_cast<float2 *>(tab_c64), (int)ntab, kx0, X0, dx, win_k, win);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_deposit_background(int32_t *ix, float *fx, float *y, float *z, float *px, float *py,
                              float *pz, float *w, int64_t n, int win_k, float win_f, float dr_inv,
                              int nx, int nr, int nm, uint64_t *accR, const double *scaleR,
                              void *ext_int2, int64_t ext_len, int shift_cells, void *stream,
                              const chm_sp_window *win) {
  CHM_REQUIRE(n >= 0 && nx > 1 && nr > 1 && nm >= 1 && nm <= 3 && n < (i64)INT32_MAX - kDepBlock,
              "sp_deposit_background: bad dims (nm 1..3, n < 2^31)");
  CHM_REQUIRE(shift_cells >= 0 && shift_cells < nx && nx <= kShiftMaxNx,
              "sp_deposit_background: bad shift");
  CHM_REQUIRE(accR && scaleR && ext_int2, "sp_deposit_background: null pointer");
  const unsigned blocks = (unsigned)((n + kDepBlock - 1) / kDepBlock);
  CHM_REQUIRE(ext_len >= (i64)blocks, "sp_deposit_background: block extent table too short");
  cudaStream_t st = as_stream(stream);
  if (shift_cells > 0) {
    const int sm = nx * (int)sizeof(longlong2);
    cudaFuncSetAttribute(shift_acc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    shift_acc_kernel<<<(unsigned)((i64)nr * nm), kShiftThreads, sm, st>>>(
        reinterpret_cast<longlong2 *>(accR), nx, shift_cells);
    chm::count_launch();
  }
  if (n == 0) return CHM_OK;
  CHM_REQUIRE(ix && fx && y && z && px && py && pz && w, "sp_deposit_background: null particle array");
  PushDepArgs A{};
  A.P = SpParts{ix, fx, y, z, px, py, pz, w, n};
  A.G = SpGrid{win_k, win_f, dr_inv, nx, nr, nm};
  A.dep_rho = 1;
  A.accR = reinterpret_cast<unsigned long long *>(accR);
  A.scaleR = scaleR;
  A.win = win;
  int2 *ext = reinterpret_cast<int2 *>(ext_int2);
  if (shift_cells > 0) {
    A.gx_min = nx - shift_cells;
    A.ext_in = ext;
  } else {
    A.ext_out = ext;
  }
  void (*kern)(PushDepArgs) = nm == 1 ? push_deposit_run_kernel<1, false, false, true>
                            : nm == 2 ? push_deposit_run_kernel<2, false, false, true>
                                      : push_deposit_run_kernel<3, false, false, true>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kRhoBoxBytes);
  kern<<<blocks, kDepThreads, kRhoBoxBytes, st>>>(A);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_push_deposit_env(int32_t *ix, float *fx, float *y, float *z, float *px, float *py,
                            float *pz, float *w, int64_t n, int win_k, float win_f, float dx_inv,
                            float dr_inv, double dt, double dx, int nx, int nr, int nm,
                            uint64_t *accJ, const double *scaleJ, const void *carrier_c64,
                            int64_t ntab, float kdx, void *stream, const chm_sp_window *win) {
  CHM_REQUIRE(n >= 0 && nx > 1 && nr > 1 && (nm == 1 || nm == 3 || nm == 5) && dt > 0.0 && dx > 0.0,
              "sp_push_deposit_env: bad dims (the envelope modes -K..K, K <= 2)");
  if (n == 0) return CHM_OK;
  CHM_REQUIRE(ix && fx && y && z && px && py && pz && w && accJ && scaleJ && carrier_c64,
              "sp_push_deposit_env: null pointer");
  CHM_REQUIRE(ntab >= (int64_t)nx + 4, "sp_push_deposit_env: carrier table shorter than nx + 4");
  PushDepArgs A{};
  A.P = SpParts{ix, fx, y, z, px, py, pz, w, n};
  A.G = SpGrid{win_k, win_f, dr_inv, nx, nr, nm};
  A.dt = (float)dt;
  A.dx_inv = dx_inv;
  A.push = 1;
  A.dep_j = 1;
  A.accJ = reinterpret_cast<unsigned long long *>(accJ);
  A.scaleJ = scaleJ;
  A.win = win;
  // the light-speed step in cells, from FP64 dt and dx
  const double D = dt / dx;
  A.far = D >= 2.0;
  A.d_cells = (float)D;
  A.d_int = (int)floor(D);
  A.d_frac = (float)(D - floor(D));
  A.dh_int = (int)floor(0.5 * D);
  A.dh_frac = (float)(0.5 * D - floor(0.5 * D));
  const EnvArgs E{reinterpret_cast<const float2 *>(carrier_c64), kdx};
  const unsigned blocks = (unsigned)((n + kDepBlock - 1) / kDepBlock);
  cudaStream_t st = as_stream(stream);
  if (nm == 1) push_deposit_env_kernel<1><<<blocks, kDepThreads, 0, st>>>(A, E);
  else if (nm == 3) push_deposit_env_kernel<3><<<blocks, kDepThreads, 0, st>>>(A, E);
  else push_deposit_env_kernel<5><<<blocks, kDepThreads, 0, st>>>(A, E);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_gather_push_env(int32_t *ix, float *fx, float *y, float *z, float *px, float *py,
                           float *pz, float *w, int64_t n, int win_k, float win_f, float dr_inv,
                           const void *eb_c64, int nx, int nr, int nm, float dtq,
                           const void *carrier_c64, int64_t ntab, float kdx, int und_kind,
                           const double *und, const void *und_map, int64_t nmap,
                           double X0, double dx, void *stream, const chm_sp_window *win) {
  CHM_REQUIRE(n >= 0 && nx > 1 && nr > 1 && (nm == 1 || nm == 3 || nm == 5),
              "sp_gather_push_env: bad dims (the envelope modes -K..K, K <= 2)");
  CHM_REQUIRE(und_kind >= 0 && und_kind <= 4 && (und_kind == 0 || und) &&
                  (und_kind < 3 || (und_map && nmap > 0 && nmap < (1 << 30) && und[2] > 0.0 &&
                                    (reinterpret_cast<uintptr_t>(und_map) & 7u) == 0)),
              "sp_gather_push_env: bad undulator (a map needs nmap in [1, 2^30), a positive "
              "step and 8-byte alignment)");
  if (n == 0) return CHM_OK;
  CHM_REQUIRE(ix && fx && y && z && px && py && pz && w && eb_c64 && carrier_c64,
              "sp_gather_push_env: null pointer");
  CHM_REQUIRE(ntab >= (int64_t)nx + 4, "sp_gather_push_env: carrier table shorter than nx + 4");
  GatherArgs A{};
  A.P = SpParts{ix, fx, y, z, px, py, pz, w, n};
  A.G = SpGrid{win_k, win_f, dr_inv, nx, nr, nm};
  A.eb = reinterpret_cast<const float2 *>(eb_c64);
  A.dtq = dtq;
  A.win = win;
  const EnvArgs E{reinterpret_cast<const float2 *>(carrier_c64), kdx};
  UndArgs U{};
  U.kind = und_kind;
  if (und_kind == 1 || und_kind == 2) {
    // (a0, period, start, length[, taper]) as devices.f90 takes them
    U.a0 = (float)und[0];
    U.lam = (float)und[1];
    U.ku = (float)(2.0 * 3.14159265358979323846 / und[1]);
    U.len = (float)und[3];
    U.taper = und_kind == 2 ? (float)und[4] : 0.0f;
    U.xo = X0 - und[2];
    U.dx = dx;
  } else if (und_kind >= 3) {
    // (period, Xleft, map step[, length, taper]) and the map a(2, nmap)
    U.lam = (float)und[0];
    U.ku = (float)(2.0 * 3.14159265358979323846 / und[0]);
    U.xo = X0 - und[1];
    U.dx = dx;
    U.mdx = (float)und[2];
    U.mdx_inv = (float)(1.0 / und[2]);
    U.map = reinterpret_cast<const float2 *>(und_map);
    U.nmap = (int)nmap;
    if (und_kind == 4) {
      U.len = (float)und[3];
      U.taper = (float)und[4];
      U.x_shift = (float)(0.5 * ((double)nmap * und[2] - und[3]));
    }
  }
  const unsigned blocks = (unsigned)((n + kDepBlock - 1) / kDepBlock);
  cudaStream_t st = as_stream(stream);
  if (nm == 1) gather_push_env_kernel<1><<<blocks, kDepThreads, 0, st>>>(A, E, U);
  else if (nm == 3) gather_push_env_kernel<3><<<blocks, kDepThreads, 0, st>>>(A, E, U);
  else gather_push_env_kernel<5><<<blocks, kDepThreads, 0, st>>>(A, E, U);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_from_f64(int32_t *ix, float *fx, float *y, float *z, float *px, float *py, float *pz,
                    float *w, uint8_t *dead, int64_t offset, const double *coord, int64_t x_cs,
                    int64_t x_ps, const double *momenta, int64_t p_cs, int64_t p_ps,
                    const double *wghts, int64_t w_ps, double X0, double dx, int64_t n,
                    void *stream) {
  CHM_REQUIRE(n >= 0 && offset >= 0 && dx > 0, "sp_from_f64: bad args");
  if (n == 0) return CHM_OK;
  SpParts P{ix, fx, y, z, px, py, pz, w, offset + n};
  from_f64_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      P, dead, offset, coord, x_cs, x_ps, momenta, p_cs, p_ps, wghts, w_ps, X0, 1.0 / dx, n);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_to_f64(const int32_t *ix, const float *fx, const float *y, const float *z,
                  const float *px, const float *py, const float *pz, const float *w, int64_t n,
                  double *coord, int64_t x_cs, int64_t x_ps, double *momenta, int64_t p_cs,
                  int64_t p_ps, double *wghts, int64_t w_ps, double X0, double dx, void *stream) {
  CHM_REQUIRE(n >= 0, "sp_to_f64: bad args");
  if (n == 0) return CHM_OK;
  SpParts P{const_cast<int32_t *>(ix), const_cast<float *>(fx), const_cast<float *>(y),
            const_cast<float *>(z), const_cast<float *>(px), const_cast<float *>(py),
            const_cast<float *>(pz), const_cast<float *>(w), n};
  to_f64_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(P, coord, x_cs, x_ps, momenta,
                                                                 p_cs, p_ps, wghts, w_ps, X0, dx);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_absorb(const int32_t *ix, const float *fx, const float *y, const float *z, float *w,
                  uint8_t *dead, int64_t n, int win_k, float win_f, float xmin_cells,
                  float xmax_cells, float r2max, uint64_t *counters, double *scale2, void *ws,
                  int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(n >= 0 && counters && scale2, "sp_absorb: bad args");
  CHM_REQUIRE(ws && ws_bytes >= chm_sp_scale_ws_bytes(), "sp_absorb: workspace too small");
  cudaStream_t st = as_stream(stream);
  double *partial = reinterpret_cast<double *>(ws);
  int nb = 1;
  if (n > 0) {
    CHM_REQUIRE(ix && fx && y && z && w && dead, "sp_absorb: null pointer");
    CHM_REQUIRE(((reinterpret_cast<uintptr_t>(ix) | reinterpret_cast<uintptr_t>(fx) |
                  reinterpret_cast<uintptr_t>(y) | reinterpret_cast<uintptr_t>(z) |
                  reinterpret_cast<uintptr_t>(w) | reinterpret_cast<uintptr_t>(dead)) & 15u) == 0,
                "sp_absorb: arrays must start on 16-byte boundaries");
    i64 R;
    const i64 nphys = tiles_of(n) * kTile;
    ws_partition(nphys, &nb, &R);
    SpParts P{const_cast<int32_t *>(ix), const_cast<float *>(fx), const_cast<float *>(y),
              const_cast<float *>(z), nullptr, nullptr, nullptr, w, n};
    weights_kernel<true><<<nb, kWsThreads, 0, st>>>(
        P, dead, AbsorbBox{win_k, win_f, xmin_cells, xmax_cells, r2max}, nphys, R, partial,
        reinterpret_cast<unsigned long long *>(counters));
    chm::count_launch();
  } else {
    cudaMemsetAsync(partial, 0, 8, st);
  }
  sp_scale_kernel<<<1, 1024, 0, st>>>(partial, nb, scale2); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_count_live(uint64_t *counters, int64_t n, void *stream) {
  CHM_REQUIRE(counters && n >= 0, "sp_count_live: bad args");
  live_steps_kernel<<<1, 32, 0, as_stream(stream)>>>(reinterpret_cast<unsigned long long *>(counters), n);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int64_t chm_sp_compact_ws_bytes(int64_t n) {
  return ((n + kCmpTile - 1) / kCmpTile) * 4 + 256;
}

int chm_sp_compact(const int32_t *ix, const float *fx, const float *y, const float *z,
                   const float *px, const float *py, const float *pz, const float *w,
                   const uint8_t *dead, int64_t n, int32_t *ix_out, float *fx_out, float *y_out,
                   float *z_out, float *px_out, float *py_out, float *pz_out, float *w_out,
                   int64_t *n_out, void *ws, int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(n >= 0 && n_out, "sp_compact: bad args");
  CHM_REQUIRE(n < ((int64_t)1 << 31), "sp_compact: more than 2^31 - 1 particles");
  CHM_REQUIRE(ws && ws_bytes >= chm_sp_compact_ws_bytes(n), "sp_compact: workspace too small");
  cudaStream_t st = as_stream(stream);
  if (n == 0) {
    cudaMemsetAsync(n_out, 0, sizeof(int64_t), st);
    return CHM_OK;
  }
  CHM_REQUIRE(ix && fx && y && z && px && py && pz && w && dead && ix_out && fx_out && y_out &&
                  z_out && px_out && py_out && pz_out && w_out,
              "sp_compact: null pointer");
  const int ntiles = (int)((n + kCmpTile - 1) / kCmpTile);
  int *cnt = reinterpret_cast<int *>(ws);
  SpParts S{const_cast<int32_t *>(ix), const_cast<float *>(fx), const_cast<float *>(y),
            const_cast<float *>(z), const_cast<float *>(px), const_cast<float *>(py),
            const_cast<float *>(pz), const_cast<float *>(w), n};
  SpParts D{ix_out, fx_out, y_out, z_out, px_out, py_out, pz_out, w_out, n};
  compact_count_kernel<<<ntiles, kCmpThreads, 0, st>>>(dead, n, cnt);
  chm::count_launch();
  compact_scan_kernel<<<1, 1024, 0, st>>>(cnt, ntiles, n_out);
  chm::count_launch();
  compact_scatter_kernel<<<ntiles, kCmpThreads, 0, st>>>(S, D, dead, cnt);
  chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Plasma generation on the device (particle_tools.f90:84-128 genparts with
// the fixed per-cell pattern, species.py:132-215 gen_parts): the host draws
// the random numbers (the reference's RNG stream) and evaluates the pattern
// positions and profile weights on the few distinct values; the kernel
// builds every particle.
// ---------------------------------------------------------------------------
namespace {

// candidate (ir, ix, ip) -> output particle row_base[ir] + ix row_count[ir]
// + row_rank[ir, ip] (row_rank < 0: the pattern point is dropped, r <= 0)
__global__ void gen_fixed_cell_kernel(double *__restrict__ coords, i64 cstride,
                                      double *__restrict__ weights, const double *__restrict__ cx,
                                      const double *__restrict__ cr, const double *__restrict__ wfac,
                                      const double2 *__restrict__ packo,
                                      const double *__restrict__ rand_o, i64 ldr,
                                      const i64 *__restrict__ row_base,
                                      const int *__restrict__ row_rank,
                                      const int *__restrict__ row_count, i64 nxc, i64 nrc, i64 npc) {
  const i64 ncand = nrc * nxc * npc;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < ncand;
       t += (i64)gridDim.x * blockDim.x) {
    const i64 ip = t % npc, ix = (t / npc) % nxc, ir = t / (npc * nxc);
    const int rank = row_rank[ir + nrc * ip];
    if (rank < 0) continue;
    const i64 o = row_base[ir] + ix * row_count[ir] + rank;
    // angle 2 pi u of the cell; the pattern point packo rotated by it
    // (complex product in the order (a c - b d, a d + b c), no contraction)
    const double ang = __dmul_rn(6.283185307179586, rand_o[ix + ldr * ir]);
    double s, c;
    sincos(ang, &s, &c);
    const double2 po = packo[ip];
    const double ore = __dsub_rn(__dmul_rn(po.x, c), __dmul_rn(po.y, s));
    const double oim = __dadd_rn(__dmul_rn(po.x, s), __dmul_rn(po.y, c));
    const double r = cr[ir + nrc * ip];
    coords[o] = cx[ix + nxc * ip];
    coords[o + cstride] = __dmul_rn(r, oim);
    coords[o + 2 * cstride] = __dmul_rn(r, ore);
    weights[o] = __dmul_rn(r, wfac[ix + nxc * ip]);
  }
}

}  // namespace

extern "C" int chm_gen_fixed_cell(double *coords, int64_t cstride, double *weights,
                                  const double *cx, const double *cr, const double *wfac,
                                  const double *packo, const double *rand_o, int64_t ldr,
                                  const int64_t *row_base, const int32_t *row_rank,
                                  const int32_t *row_count, int64_t nxc, int64_t nrc, int64_t npc,
                                  void *stream) {
  CHM_REQUIRE(nxc >= 0 && nrc >= 0 && npc > 0 && ldr >= nxc, "gen_fixed_cell: bad dims");
  if (nxc == 0 || nrc == 0) return CHM_OK;
  CHM_REQUIRE(coords && weights && cx && cr && wfac && packo && rand_o && row_base && row_rank &&
                  row_count,
              "gen_fixed_cell: null pointer");
  const i64 ncand = nrc * nxc * npc;
  gen_fixed_cell_kernel<<<grid_for(ncand, 256), 256, 0, as_stream(stream)>>>(
      coords, cstride, weights, cx, cr, wfac, reinterpret_cast<const double2 *>(packo), rand_o, ldr,
      row_base, row_rank, row_count, nxc, nrc, npc);
  count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}
