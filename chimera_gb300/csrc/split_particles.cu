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
// Deposition stays deterministic without float atomics: each block
// accumulates its particles' contributions in 32-bit fixed point in shared
// memory (scale 2^e_l from the block's own sum |w|), then adds the block box
// into the global 64-bit accumulator after an exact power-of-two rescale to
// the global scale 2^e_g.  Integer sums are order-independent, so the result
// depends only on which particles share a block, which is fixed.
#include <climits>
#include <math.h>

#include "common.cuh"

using namespace chm;

namespace {

constexpr int kSpThreads = 256;
constexpr int kSpPerThread = 8;
constexpr int kSpPerBlock = kSpThreads * kSpPerThread;
constexpr int kSpBoxBytes = 64 * 1024;

struct SpParts {
  int32_t *ix;
  float *fx, *y, *z, *px, *py, *pz, *w;
  i64 n;
};

struct SpGrid {
  int win_k;      // window origin, whole cells from X0
  float win_f;    // window origin, fraction of a cell
  float dr_inv;   // 1/dr; r node j sits at (j - 1/2) dr
  int nx, nr, nm;  // spatial grid
};

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
  float r = sqrtf(y * y + z * z);
  float s = r * G.dr_inv + 0.5f;
  float sf = floorf(s);
  L.cr = (int)sf;
  L.sr1 = s - sf;
  L.ok = (L.cr >= 0 && L.cr <= G.nr - 2);
  if (r > 0.0f) {
    float ri = 1.0f / r;
    L.phr = y * ri;
    L.phi = z * ri;
  } else {
    L.phr = 0.0f;
    L.phi = 0.0f;
  }
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
  const double *scaleJ, *scaleR;  // global scales 2^e_g
};

// Particle update of push_coords (particle_tools.f90:58-82) in cell units:
// half-step and new positions.
struct Pushed {
  int ixh, ixn;
  float fxh, fxn, yh, zh, yn, zn;
  float vj[3];
};

__device__ __forceinline__ Pushed push_one(const PushDepArgs &A, i64 i) {
  const SpParts &P = A.P;
  Pushed o;
  const int ix = P.ix[i];
  const float fx = P.fx[i], y = P.y[i], z = P.z[i];
  const float px = P.px[i], py = P.py[i], pz = P.pz[i], w = P.w[i];
  const float g = sqrtf(1.0f + (px * px + py * py + pz * pz));
  const float dtg = A.push ? A.dt / g : 0.0f;
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
  const float wg = moving ? w / g : 0.0f;
  o.vj[0] = px * wg;
  o.vj[1] = py * wg;
  o.vj[2] = pz * wg;
  return o;
}

__global__ void __launch_bounds__(kSpThreads) push_deposit_kernel(PushDepArgs A) {
  extern __shared__ __align__(16) int box[];
  __shared__ long long bb[4];
  __shared__ double wred[kSpThreads / 32];
  const i64 p0 = (i64)blockIdx.x * kSpPerBlock, p1 = min(A.P.n, p0 + (i64)kSpPerBlock);
  if (threadIdx.x == 0) {
    bb[0] = LLONG_MAX;
    bb[1] = LLONG_MIN;
    bb[2] = LLONG_MAX;
    bb[3] = LLONG_MIN;
  }
  __syncthreads();
  // pass 1: box of every deposit location and the block's sum |w|
  long long x0 = LLONG_MAX, x1 = LLONG_MIN, r0 = LLONG_MAX, r1 = LLONG_MIN;
  double wsum = 0.0;
  for (i64 i = p0 + threadIdx.x; i < p1; i += kSpThreads) {
    const float w = A.P.w[i];
    if (w == 0.0f) continue;
    Pushed q = push_one(A, i);
    wsum += fabs((double)w);
    if (A.dep_j) {
      Loc L = locate(q.ixh, q.fxh, q.yh, q.zh, A.G);
      if (L.ok) {
        x0 = min(x0, (long long)L.cx);
        x1 = max(x1, (long long)L.cx + 1);
        r0 = min(r0, (long long)L.cr);
        r1 = max(r1, (long long)L.cr + 1);
      }
    }
    if (A.dep_rho) {
      Loc L = locate(q.ixn, q.fxn, q.yn, q.zn, A.G);
      if (L.ok) {
        x0 = min(x0, (long long)L.cx);
        x1 = max(x1, (long long)L.cx + 1);
        r0 = min(r0, (long long)L.cr);
        r1 = max(r1, (long long)L.cr + 1);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    x0 = min(x0, __shfl_xor_sync(0xffffffffu, x0, o));
    x1 = max(x1, __shfl_xor_sync(0xffffffffu, x1, o));
    r0 = min(r0, __shfl_xor_sync(0xffffffffu, r0, o));
    r1 = max(r1, __shfl_xor_sync(0xffffffffu, r1, o));
    wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&bb[0], x0);
    atomicMax(&bb[1], x1);
    atomicMin(&bb[2], r0);
    atomicMax(&bb[3], r1);
    wred[threadIdx.x >> 5] = wsum;
  }
  __syncthreads();
  double Bl = 0.0;
  for (int k = 0; k < kSpThreads / 32; ++k) Bl += wred[k];  // fixed order
  const long long bx0 = max(bb[0], 0LL), bx1 = min(bb[1], (long long)A.G.nx - 1);
  const long long br0 = max(bb[2], 0LL), br1 = min(bb[3], (long long)A.G.nr - 1);
  const long long bnx = bx1 - bx0 + 1, bnr = br1 - br0 + 1;
  const int nplanes = A.G.nm * 4;  // J: 3 nm planes, rho: nm planes
  const long long nvals = (bnx > 0 && bnr > 0) ? bnx * bnr * nplanes * 2 : 0;
  const bool use_box = nvals > 0 && nvals * 4 <= kSpBoxBytes && Bl > 0.0;
  const int el = use_box ? 29 - ceil_log2(Bl) : 0;
  const float lscale = ldexpf(1.0f, el);
  const int eJ = ilogb(A.scaleJ ? A.scaleJ[0] : 1.0);
  const int eR = ilogb(A.scaleR ? A.scaleR[0] : 1.0);
  if (use_box)
    for (long long t = threadIdx.x; t < nvals; t += kSpThreads) box[t] = 0;
  __syncthreads();
  // pass 2: push, deposit, store
  for (i64 i = p0 + threadIdx.x; i < p1; i += kSpThreads) {
    const float w = A.P.w[i];
    Pushed q = push_one(A, i);
    if (w != 0.0f) {
      auto to_box = [&](int plane, int r, int x, float re, float im) {
        const long long b = (((long long)plane * bnr + (r - br0)) * bnx + (x - bx0)) * 2;
        const int qr = __float2int_rn(re * lscale), qi = __float2int_rn(im * lscale);
        if (qr) atomicAdd(&box[b], qr);
        if (qi) atomicAdd(&box[b + 1], qi);
      };
      if (A.dep_j) {
        Loc L = locate(q.ixh, q.fxh, q.yh, q.zh, A.G);
        if (use_box) {
          deposit_at(L, q.vj, 3, 0, A.G, to_box);
        } else {
          const float sc = ldexpf(1.0f, eJ);
          deposit_at(L, q.vj, 3, 0, A.G, [&](int plane, int r, int x, float re, float im) {
            const i64 e = ((i64)plane * A.G.nr + r) * A.G.nx + x;
            long long qr = __double2ll_rn((double)re * sc), qi = __double2ll_rn((double)im * sc);
            if (qr) atomicAdd(&A.accJ[2 * e], (unsigned long long)qr);
            if (qi) atomicAdd(&A.accJ[2 * e + 1], (unsigned long long)qi);
          });
        }
      }
      if (A.dep_rho) {
        Loc L = locate(q.ixn, q.fxn, q.yn, q.zn, A.G);
        const float wv[1] = {w};
        if (use_box) {
          deposit_at(L, wv, 1, 3 * A.G.nm, A.G, to_box);
        } else {
          const float sc = ldexpf(1.0f, eR);
          deposit_at(L, wv, 1, 0, A.G, [&](int plane, int r, int x, float re, float im) {
            const i64 e = ((i64)plane * A.G.nr + r) * A.G.nx + x;
            long long qr = __double2ll_rn((double)re * sc), qi = __double2ll_rn((double)im * sc);
            if (qr) atomicAdd(&A.accR[2 * e], (unsigned long long)qr);
            if (qi) atomicAdd(&A.accR[2 * e + 1], (unsigned long long)qi);
          });
        }
      }
    }
    if (A.push) {
      A.P.ix[i] = q.ixn;
      A.P.fx[i] = q.fxn;
      A.P.y[i] = q.yn;
      A.P.z[i] = q.zn;
    }
  }
  if (!use_box) return;
  __syncthreads();
  // flush: local 2^el -> global 2^eg is an exact shift (el >= eg)
  for (long long t = threadIdx.x; t < nvals; t += kSpThreads) {
    const int v = box[t];
    if (v == 0) continue;
    const long long c2 = t & 1;
    const long long b = t >> 1;
    const long long bx = b % bnx;
    const long long rest = b / bnx;
    const long long br = rest % bnr;
    const long long plane = rest / bnr;
    const bool isj = plane < 3 * A.G.nm;
    const int eg = isj ? eJ : eR;
    const long long pl = isj ? plane : plane - 3 * A.G.nm;
    // local quantum 2^-el -> global quantum 2^-eg: an exact left shift when
    // eg >= el (the usual case: the block holds a small share of the total
    // weight), otherwise a right shift rounded half away from zero
    const int s = el - eg;
    const long long q = (long long)v;
    long long qq;
    if (s <= 0) {
      qq = q << (-s);
    } else if (s >= 62) {
      qq = 0;
    } else {
      const long long h = 1LL << (s - 1);
      qq = (q >= 0) ? ((q + h) >> s) : -((-q + h) >> s);
    }
    if (qq == 0) continue;
    const i64 e = (pl * A.G.nr + (br + br0)) * A.G.nx + (bx + bx0);
    unsigned long long *acc = isj ? A.accJ : A.accR;
    atomicAdd(&acc[2 * e + c2], (unsigned long long)qq);
  }
}

// Global scale 2^(61 - ceil(log2 B)), B = sum |w| (deterministic order).
__global__ void sp_wsum_kernel(const float *__restrict__ w, i64 n, double *__restrict__ partial) {
  __shared__ double sh[256];
  const i64 per = (n + gridDim.x - 1) / gridDim.x;
  const i64 b0 = blockIdx.x * per, b1 = min(n, b0 + per);
  double s = 0.0;
  for (i64 i = b0 + threadIdx.x; i < b1; i += blockDim.x) s += fabs((double)w[i]);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void sp_scale_kernel(const double *__restrict__ partial, int np, double *out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double B = 0.0;
    for (int i = 0; i < np; ++i) B += partial[i];
    if (!(B > 0.0) || !isfinite(B)) B = 1.0;
    out[0] = ldexp(1.0, 61 - ceil_log2(B));
    out[1] = B;
  }
}

// gather (proj_fld) + Boris (push_velocs), FP32
struct GatherArgs {
  SpParts P;
  SpGrid G;
  const float2 *eb;  // (nx, nr, nm, 6) complex64, Fortran order
  float dtq;          // push_fact * dt
};

__global__ void __launch_bounds__(256) gather_push_kernel(GatherArgs A) {
  const SpGrid &G = A.G;
  const i64 plane = (i64)G.nx * G.nr;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < A.P.n;
       i += (i64)gridDim.x * blockDim.x) {
    float F[6] = {0, 0, 0, 0, 0, 0};
    const float w = A.P.w[i];
    if (w != 0.0f) {
      Loc L = locate(A.P.ix[i], A.P.fx[i], A.P.y[i], A.P.z[i], G);
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
    // Boris rotation (particle_tools.f90:18-56)
    const float h = 0.5f * A.dtq;
    float um[3] = {A.P.px[i] + h * F[0], A.P.py[i] + h * F[1], A.P.pz[i] + h * F[2]};
    const float g = sqrtf(1.0f + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]));
    float t[3] = {h * F[3] / g, h * F[4] / g, h * F[5] / g};
    const float t2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
    float s[3] = {2 * t[0] / (1 + t2), 2 * t[1] / (1 + t2), 2 * t[2] / (1 + t2)};
    float u0[3] = {um[0] + um[1] * t[2] - um[2] * t[1], um[1] - um[0] * t[2] + um[2] * t[0],
                   um[2] + um[0] * t[1] - um[1] * t[0]};
    A.P.px[i] = um[0] + u0[1] * s[2] - u0[2] * s[1] + h * F[0];
    A.P.py[i] = um[1] - u0[0] * s[2] + u0[2] * s[0] + h * F[1];
    A.P.pz[i] = um[2] + u0[0] * s[1] - u0[1] * s[0] + h * F[2];
  }
}

// FP64 (3, n) strided particle arrays -> split layout
__global__ void from_f64_kernel(SpParts P, i64 off, const double *__restrict__ x, i64 x_cs, i64 x_ps,
                                const double *__restrict__ p, i64 p_cs, i64 p_ps,
                                const double *__restrict__ w, i64 w_ps, double X0, double dx_inv,
                                i64 n) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const double s = (x[i * x_ps] - X0) * dx_inv;
    const double fl = floor(s);
    float fr = (float)(s - fl);
    int ix = (int)fl;
    if (fr >= 1.0f) {  // rounding up to the next cell
      fr = 0.0f;
      ix += 1;
    }
    P.ix[off + i] = ix;
    P.fx[off + i] = fr;
    P.y[off + i] = (float)x[x_cs + i * x_ps];
    P.z[off + i] = (float)x[2 * x_cs + i * x_ps];
    P.px[off + i] = (float)p[i * p_ps];
    P.py[off + i] = (float)p[p_cs + i * p_ps];
    P.pz[off + i] = (float)p[2 * p_cs + i * p_ps];
    P.w[off + i] = (float)w[i * w_ps];
  }
}

__global__ void to_f64_kernel(SpParts P, double *__restrict__ x, i64 x_cs, i64 x_ps,
                              double *__restrict__ p, i64 p_cs, i64 p_ps, double *__restrict__ w,
                              i64 w_ps, double X0, double dx) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P.n; i += (i64)gridDim.x * blockDim.x) {
    x[i * x_ps] = X0 + ((double)P.ix[i] + (double)P.fx[i]) * dx;
    x[x_cs + i * x_ps] = P.y[i];
    x[2 * x_cs + i * x_ps] = P.z[i];
    p[i * p_ps] = P.px[i];
    p[p_cs + i * p_ps] = P.py[i];
    p[2 * p_cs + i * p_ps] = P.pz[i];
    if (w) w[i * w_ps] = P.w[i];
  }
}

// absorption flags: inside the box xmin <= x and r^2 <= r2max (x in the
// window-relative cell units of the same (k, f) convention)
__global__ void keep_flags_kernel(SpParts P, int win_k, float win_f, float xmin_cells,
                                  float xmax_cells, float r2max, int *__restrict__ flag) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < P.n; i += (i64)gridDim.x * blockDim.x) {
    const float xc = (float)(P.ix[i] - win_k) + (P.fx[i] - win_f);
    const float r2 = P.y[i] * P.y[i] + P.z[i] * P.z[i];
    flag[i] = (xc >= xmin_cells && xc <= xmax_cells && r2 <= r2max) ? 1 : 0;
  }
}

}  // namespace

extern "C" {

// The split-form particle entry points take the eight SoA arrays in the
// order ix, fx, y, z, px, py, pz, w (n particles).

int64_t chm_sp_scale_ws_bytes(void) { return 8 * 512 + 256; }

int chm_sp_weight_scale(double *scale2, const float *w, int64_t n, void *ws, int64_t ws_bytes,
                        void *stream) {
  CHM_REQUIRE(scale2 && n >= 0 && ws && ws_bytes >= chm_sp_scale_ws_bytes(),
              "sp_weight_scale: bad args");
  cudaStream_t st = as_stream(stream);
  double *partial = reinterpret_cast<double *>(ws);
  if (n > 0) {
    CHM_REQUIRE(w, "sp_weight_scale: null weights");
    sp_wsum_kernel<<<512, 256, 0, st>>>(w, n, partial); chm::count_launch();
  } else {
    cudaMemsetAsync(partial, 0, 8 * 512, st);
  }
  sp_scale_kernel<<<1, 32, 0, st>>>(partial, 512, scale2); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_push_deposit(int32_t *ix, float *fx, float *y, float *z, float *px, float *py,
                        float *pz, float *w, int64_t n, int win_k, float win_f, float dx_inv,
                        float dr_inv, float dt, int nx, int nr, int nm, int push,
                        uint64_t *accJ, const double *scaleJ, uint64_t *accR,
                        const double *scaleR, void *stream) {
  CHM_REQUIRE(n >= 0 && nx > 1 && nr > 1 && nm >= 1 && nm <= 8, "sp_push_deposit: bad dims");
  if (n == 0) return CHM_OK;
  CHM_REQUIRE(ix && fx && y && z && px && py && pz && w, "sp_push_deposit: null particle array");
  CHM_REQUIRE(!accJ || scaleJ, "sp_push_deposit: J accumulator without scale");
  CHM_REQUIRE(!accR || scaleR, "sp_push_deposit: rho accumulator without scale");
  PushDepArgs A;
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
  cudaFuncSetAttribute(push_deposit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       kSpBoxBytes);
  const unsigned blocks = (unsigned)((n + kSpPerBlock - 1) / kSpPerBlock);
  push_deposit_kernel<<<blocks, kSpThreads, kSpBoxBytes, as_stream(stream)>>>(A); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_gather_push(int32_t *ix, float *fx, float *y, float *z, float *px, float *py, float *pz,
                       float *w, int64_t n, int win_k, float win_f, float dr_inv,
                       const void *eb_c64, int nx, int nr, int nm, float dtq, void *stream) {
  CHM_REQUIRE(n >= 0 && nx > 1 && nr > 1 && nm >= 1, "sp_gather_push: bad dims");
  if (n == 0) return CHM_OK;
  CHM_REQUIRE(ix && fx && y && z && px && py && pz && w && eb_c64, "sp_gather_push: null pointer");
  GatherArgs A;
  A.P = SpParts{ix, fx, y, z, px, py, pz, w, n};
  A.G = SpGrid{win_k, win_f, dr_inv, nx, nr, nm};
  A.eb = reinterpret_cast<const float2 *>(eb_c64);
  A.dtq = dtq;
  gather_push_kernel<<<grid_for(n, 256, 16), 256, 0, as_stream(stream)>>>(A); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_from_f64(int32_t *ix, float *fx, float *y, float *z, float *px, float *py, float *pz,
                    float *w, int64_t offset, const double *coord, int64_t x_cs, int64_t x_ps,
                    const double *momenta, int64_t p_cs, int64_t p_ps, const double *wghts,
                    int64_t w_ps, double X0, double dx, int64_t n, void *stream) {
  CHM_REQUIRE(n >= 0 && offset >= 0 && dx > 0, "sp_from_f64: bad args");
  if (n == 0) return CHM_OK;
  SpParts P{ix, fx, y, z, px, py, pz, w, offset + n};
  from_f64_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
      P, offset, coord, x_cs, x_ps, momenta, p_cs, p_ps, wghts, w_ps, X0, 1.0 / dx, n); chm::count_launch();
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
                                                                 p_cs, p_ps, wghts, w_ps, X0, dx); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

int chm_sp_keep_flags(const int32_t *ix, const float *fx, const float *y, const float *z,
                      int64_t n, int win_k, float win_f, float xmin_cells, float xmax_cells,
                      float r2max, int32_t *flag, void *stream) {
  CHM_REQUIRE(n >= 0, "sp_keep_flags: bad args");
  if (n == 0) return CHM_OK;
  SpParts P{const_cast<int32_t *>(ix), const_cast<float *>(fx), const_cast<float *>(y),
            const_cast<float *>(z), nullptr, nullptr, nullptr, nullptr, n};
  keep_flags_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(P, win_k, win_f, xmin_cells,
                                                                     xmax_cells, r2max, flag); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"
