// Re-sorting the split-form particles by deposit cell on the device.
//
// The reference re-buckets its particles every Xchunked[1] + 1 steps
// (moduls/chimera_main.py:306-318 chunk_particles, moduls/species.py:351-398
// chunk_and_damp: chunk_coords_boundaries, particle_tools.f90:155-208, then
// an argsort and align_data); its buckets are x chunks for the OpenMP
// deposit.  Here the buckets are the deposit cells themselves, in the order
// the cell-run deposit and gather kernels want: 4 x 4-cell patches of
// generation cells in a serpentine order, the cells of a patch in a
// serpentine order, and within a cell its two deposit cells (r nodes at
// (j - 1/2) dr), so that the 16 particles of a run share a deposit cell and a
// block of 2048 covers a compact patch of the grid.  Dead (absorbed)
// particles sort to the end and are dropped, so a sort also compacts.
//
// Stable LSD radix sort of 32-bit keys with 8-bit digits: per pass a
// histogram kernel (per 4096-key block), an exclusive scan of the
// digit-major block counts and a scatter that ranks keys stably (warp
// match + per-warp digit prefixes); then a gather of the eight particle
// arrays into the tile layout of the output buffers.
#include <stdint.h>

#include "common.cuh"

using namespace chm;

namespace {

constexpr int kRunLen = 16, kTileRuns = 32, kTile = kRunLen * kTileRuns;
constexpr int kSortThreads = 256;
constexpr int kKeysPerThread = 16;
constexpr int kSortTile = kSortThreads * kKeysPerThread;  // keys per block
constexpr int kRadix = 256;
constexpr int kScanBlock = 1024;
constexpr int kScanTile = kScanBlock * 4;

// particle (position in the species) of a slot of the tile layout
__host__ __device__ __forceinline__ i64 logical_of(i64 p) {
  return (p & ~(i64)(kTile - 1)) | ((p & (kTileRuns - 1)) << 4) | ((p >> 5) & (kRunLen - 1));
}

// deposit-order key of a live particle; dead particles get 0xffffffff
struct KeyGeo {
  int win_k;       // window origin in whole cells from X0
  float win_f;     // window origin, fraction of a cell
  int npx;         // patch columns (bound)
  float dr_inv;
  unsigned rmax;   // generation rows clamp
  unsigned xmax;   // generation columns clamp (relative to win_k - 8)
};

// The last 4 bits order the particles of a deposit cell by quarter of the
// cell in x, then in r: particles that cross into the same neighbour cell
// at the half step stay together in a run (measured: with the tie order of
// the slots instead, a cfg2-sized step slowed by 11% right after a sort).
// (the products and sums are rounded one by one, without contraction, so the
// key is reproducible on the host)
__device__ __forceinline__ uint32_t cell_key(int ix, float fx, float y, float z, const KeyGeo &G) {
  const float s = __fmul_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(y, y), __fmul_rn(z, z))), G.dr_inv);
  const float gr_f = floorf(s);
  unsigned gr = (unsigned)max(0, (int)gr_f);
  const float fr = __fsub_rn(s, gr_f);
  const unsigned half = fr >= 0.5f ? 1u : 0u;
  // quarter of the deposit cell: x offset from the window's node, r offset
  // from the deposit cell's lower node (fr + 1/2 modulo 1)
  const float dxf = __fsub_rn(fx, G.win_f);
  const float sx = __fsub_rn(dxf, floorf(dxf));
  const float sr = half ? __fsub_rn(fr, 0.5f) : __fadd_rn(fr, 0.5f);
  const unsigned qx = min(3u, (unsigned)(sx * 4.0f)), qr = min(3u, (unsigned)(sr * 4.0f));
  int gxi = ix - G.win_k + 8;
  unsigned gx = (unsigned)max(0, gxi);
  gx = min(gx, G.xmax);
  gr = min(gr, G.rmax);
  const unsigned px = gx >> 2, lx = gx & 3u, pr = gr >> 2, lr = gr & 3u;
  const unsigned pxs = (pr & 1u) ? (unsigned)G.npx - 1u - px : px;  // serpentine patch rows
  const unsigned lxs = (lr & 1u) ? 3u - lx : lx;                     // serpentine rows of a patch
  return (((((pr * (unsigned)G.npx + pxs) * 4u + lr) * 4u + lxs) * 2u + half) << 4) | (qx << 2) | qr;
}

// keys and values of the slots (slot order, coalesced): a slot past the
// last particle or holding a dead one gets the dead key
__global__ void keys_kernel(const int32_t *__restrict__ ix, const float *__restrict__ fx,
                            const float *__restrict__ y, const float *__restrict__ z,
                            const uint8_t *__restrict__ dead, i64 n,
                            i64 nphys, KeyGeo G, uint32_t *__restrict__ keys,
                            uint32_t *__restrict__ vals) {
  for (i64 q = blockIdx.x * (i64)blockDim.x + threadIdx.x; q < nphys; q += (i64)gridDim.x * blockDim.x) {
    const bool live = logical_of(q) < n && !(dead && dead[q]);
    keys[q] = live ? cell_key(ix[q], fx[q], y[q], z[q], G) : 0xffffffffu;
    vals[q] = (uint32_t)q;
  }
}

// counts[d * nblocks + b] = keys of block b with digit d
__global__ void __launch_bounds__(kSortThreads) hist_kernel(const uint32_t *__restrict__ keys, i64 n,
                                                            int shift, int nblocks,
                                                            uint32_t *__restrict__ counts) {
  __shared__ uint32_t h[kRadix];
  h[threadIdx.x] = 0;
  __syncthreads();
  const i64 base = (i64)blockIdx.x * kSortTile;
  for (int k = threadIdx.x; k < kSortTile; k += kSortThreads) {
    const i64 i = base + k;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  counts[(i64)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan of counts (length m) in three kernels: tile sums, a scan of
// the tile sums (one block), and the tiles' scans with their offsets
__global__ void __launch_bounds__(kScanBlock) scan_sums_kernel(const uint32_t *__restrict__ a, i64 m,
                                                               uint32_t *__restrict__ sums) {
  __shared__ uint32_t ws[kScanBlock / 32];
  const i64 base = (i64)blockIdx.x * kScanTile;
  uint32_t s = 0;
  for (int k = 0; k < 4; ++k) {
    const i64 i = base + (i64)threadIdx.x * 4 + k;
    if (i < m) s += a[i];
  }
  s = __reduce_add_sync(0xffffffffu, s);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int k = 0; k < kScanBlock / 32; ++k) t += ws[k];
    sums[blockIdx.x] = t;
  }
}

// in-place exclusive scan of up to kScanBlock * 4 values in one block
__device__ void block_exclusive_scan4(uint32_t *v, int m) {
  __shared__ uint32_t ws[kScanBlock / 32];
  uint32_t x[4], loc = 0;
  for (int k = 0; k < 4; ++k) {
    const int i = threadIdx.x * 4 + k;
    x[k] = i < m ? v[i] : 0;
    loc += x[k];
  }
  // inclusive warp scan of the thread totals
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t inc = loc;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t t = ws[lane];
    uint32_t it = t;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, it, o);
      if (lane >= o) it += u;
    }
    ws[lane] = it - t;  // exclusive warp offsets
  }
  __syncthreads();
  uint32_t run = ws[w] + inc - loc;
  for (int k = 0; k < 4; ++k) {
    const int i = threadIdx.x * 4 + k;
    if (i < m) v[i] = run;
    run += x[k];
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kScanBlock) scan_top_kernel(uint32_t *__restrict__ sums, int nt) {
  // nt <= kScanTile (checked on the host)
  block_exclusive_scan4(sums, nt);
}

__global__ void __launch_bounds__(kScanBlock) scan_apply_kernel(uint32_t *__restrict__ a, i64 m,
                                                                const uint32_t *__restrict__ sums) {
  __shared__ uint32_t buf[kScanTile];
  const i64 base = (i64)blockIdx.x * kScanTile;
  const int cnt = (int)min((i64)kScanTile, m - base);
  for (int k = threadIdx.x; k < kScanTile; k += kScanBlock) buf[k] = k < cnt ? a[base + k] : 0;
  __syncthreads();
  block_exclusive_scan4(buf, cnt);
  const uint32_t off = sums[blockIdx.x];
  for (int k = threadIdx.x; k < cnt; k += kScanBlock) a[base + k] = buf[k] + off;
}

// stable scatter of one pass: warp w of a block takes keys [w 512, w 512 +
// 512) of the block in 16 chunks of 32; a key's position is the block's
// digit offset + the counts of the digit in the warps before + its rank in
// its warp (earlier chunks, then earlier lanes of its chunk)
__global__ void __launch_bounds__(kSortThreads) scatter_kernel(const uint32_t *__restrict__ kin,
                                                               const uint32_t *__restrict__ vin, i64 n,
                                                               int shift, int nblocks,
                                                               const uint32_t *__restrict__ offs,
                                                               uint32_t *__restrict__ kout,
                                                               uint32_t *__restrict__ vout) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ uint32_t wc[kWarps][kRadix];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < kWarps * kRadix; k += kSortThreads) (&wc[0][0])[k] = 0;
  __syncthreads();
  const i64 base = (i64)blockIdx.x * kSortTile + (i64)w * (kKeysPerThread * 32);
  uint32_t key[kKeysPerThread], rank[kKeysPerThread];
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int c = 0; c < kKeysPerThread; ++c) {
    const i64 i = base + c * 32 + lane;
    const bool ok = i < n;
    key[c] = ok ? kin[i] : 0xffffffffu;
    const uint32_t d = (key[c] >> shift) & (kRadix - 1);
    const uint32_t act = __ballot_sync(0xffffffffu, ok);
    const uint32_t peers = __match_any_sync(0xffffffffu, ok ? d : 0xffffffffu) & act;
    const uint32_t before = ok ? wc[w][d] : 0;
    rank[c] = before + __popc(peers & lt);
    __syncwarp();
    if (ok && (peers & lt) == 0) wc[w][d] = before + __popc(peers);  // the group's first lane
    __syncwarp();
  }
  __syncthreads();
  // per digit: counts of the warps before (exclusive), in place
  {
    const int d = threadIdx.x;  // kSortThreads == kRadix
    uint32_t run = 0;
    for (int ww = 0; ww < kWarps; ++ww) {
      const uint32_t t = wc[ww][d];
      wc[ww][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < kKeysPerThread; ++c) {
    const i64 i = base + c * 32 + lane;
    if (i >= n) continue;
    const uint32_t d = (key[c] >> shift) & (kRadix - 1);
    const uint32_t pos = offs[(i64)d * nblocks + blockIdx.x] + wc[w][d] + rank[c];
    kout[pos] = key[c];
    vout[pos] = vin[i];
  }
}

// output slot q holds sorted position j = logical_of(q), the particle of
// slot vals[j]; positions past the live particles are cleared
__global__ void gather_kernel(const int32_t *__restrict__ ix, const float *__restrict__ fx,
                              const float *__restrict__ y, const float *__restrict__ z,
                              const float *__restrict__ px, const float *__restrict__ py,
                              const float *__restrict__ pz, const float *__restrict__ w,
                              const uint32_t *__restrict__ vals, const int64_t *__restrict__ nlive_p,
                              int32_t *__restrict__ ox, float *__restrict__ ofx, float *__restrict__ oy,
                              float *__restrict__ oz, float *__restrict__ opx, float *__restrict__ opy,
                              float *__restrict__ opz, float *__restrict__ ow, i64 n) {
  const i64 nlive = *nlive_p;
  for (i64 q = blockIdx.x * (i64)blockDim.x + threadIdx.x; q < n; q += (i64)gridDim.x * blockDim.x) {
    const i64 j = logical_of(q);
    if (j >= nlive) {  // slots past the live particles
      ox[q] = 0;
      ofx[q] = oy[q] = oz[q] = opx[q] = opy[q] = opz[q] = ow[q] = 0.0f;
      continue;
    }
    const i64 p = (i64)vals[j];
    ox[q] = ix[p];
    ofx[q] = fx[p];
    oy[q] = y[p];
    oz[q] = z[p];
    opx[q] = px[p];
    opy[q] = py[p];
    opz[q] = pz[p];
    ow[q] = w[p];
  }
}

// live particles = position of the first dead key (keys sorted ascending)
__global__ void count_live_kernel(const uint32_t *__restrict__ keys, i64 n, int64_t *nlive) {
  // binary search for the first 0xffffffff
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  i64 lo = 0, hi = n;
  while (lo < hi) {
    const i64 mid = (lo + hi) >> 1;
    if (keys[mid] == 0xffffffffu) hi = mid;
    else lo = mid + 1;
  }
  *nlive = lo;
}

inline i64 rup(i64 a, i64 b) { return (a + b - 1) / b * b; }

struct SortWs {
  uint32_t *k0, *v0, *k1, *v1, *counts, *sums;
  i64 nblocks, ncounts, nsums;
};

SortWs carve(void *ws, i64 n) {
  SortWs S;
  S.nblocks = (n + kSortTile - 1) / kSortTile;
  S.ncounts = S.nblocks * kRadix;
  S.nsums = (S.ncounts + kScanTile - 1) / kScanTile;
  char *p = reinterpret_cast<char *>(ws);
  auto take = [&](i64 cnt) {
    uint32_t *r = reinterpret_cast<uint32_t *>(p);
    p += rup(cnt * 4, 256);
    return r;
  };
  S.k0 = take(n);
  S.v0 = take(n);
  S.k1 = take(n);
  S.v1 = take(n);
  S.counts = take(S.ncounts);
  S.sums = take(S.nsums);
  return S;
}

}  // namespace

extern "C" {

int64_t chm_sp_sort_ws_bytes(int64_t n) {
  if (n <= 0) return 256;
  n = rup(n, kTile);
  const i64 nb = (n + kSortTile - 1) / kSortTile, nc = nb * kRadix;
  return 4 * rup(n * 4, 256) + rup(nc * 4, 256) + rup(((nc + kScanTile - 1) / kScanTile) * 4, 256) + 256;
}

int chm_sp_sort_cells(const int32_t *ix, const float *fx, const float *y, const float *z,
                      const float *px, const float *py, const float *pz, const float *w,
                      const uint8_t *dead, int64_t n, int win_k, float win_f, int nx, int nr,
                      float dr_inv,
                      int32_t *ix_out, float *fx_out, float *y_out, float *z_out, float *px_out,
                      float *py_out, float *pz_out, float *w_out, int64_t *n_out, void *ws,
                      int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(n >= 0 && n < ((int64_t)1 << 31) && nx > 1 && nr > 1 && n_out,
              "sp_sort_cells: bad args");
  CHM_REQUIRE(ws && ws_bytes >= chm_sp_sort_ws_bytes(n), "sp_sort_cells: workspace too small");
  cudaStream_t st = as_stream(stream);
  if (n == 0) {
    cudaMemsetAsync(n_out, 0, sizeof(int64_t), st);
    return CHM_OK;
  }
  CHM_REQUIRE(ix && fx && y && z && px && py && pz && w && ix_out && fx_out && y_out && z_out &&
                  px_out && py_out && pz_out && w_out,
              "sp_sort_cells: null pointer");
  const i64 nphys = rup(n, kTile);  // the sort runs over slots (padding slots are dead)
  SortWs S = carve(ws, nphys);
  CHM_REQUIRE(S.nsums <= kScanTile, "sp_sort_cells: too many particles for the scan");
  KeyGeo G;
  G.win_k = win_k;
  G.win_f = win_f;
  G.xmax = (unsigned)(nx + 24);
  G.npx = (int)(G.xmax / 4 + 1);
  G.rmax = (unsigned)(nr + 4);
  G.dr_inv = dr_inv;
  // key bits: (((((pr npx + px) 4 + lr) 4 + lx) 2 + half) 16 + quarter
  const uint64_t kmax = (((((uint64_t)(G.rmax / 4) * G.npx + G.npx) * 4 + 3) * 4 + 3) * 2 + 1) * 16 + 15;
  CHM_REQUIRE(kmax < 0xffffffffull, "sp_sort_cells: grid too large for 32-bit keys");
  // enough key bits that the dead key's low bits (all ones) stay above
  // every live key: kmax + 1 < 2^bits
  int bits = 0;
  while (bits < 32 && ((kmax + 1) >> bits)) ++bits;
  const int passes = (bits + 7) / 8;
  keys_kernel<<<grid_for(nphys, 256), 256, 0, st>>>(ix, fx, y, z, dead, n, nphys, G, S.k0, S.v0);
  count_launch();
  uint32_t *kin = S.k0, *vin = S.v0, *kout = S.k1, *vout = S.v1;
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    hist_kernel<<<(unsigned)S.nblocks, kSortThreads, 0, st>>>(kin, nphys, shift, (int)S.nblocks,
                                                              S.counts);
    scan_sums_kernel<<<(unsigned)S.nsums, kScanBlock, 0, st>>>(S.counts, S.ncounts, S.sums);
    scan_top_kernel<<<1, kScanBlock, 0, st>>>(S.sums, (int)S.nsums);
    scan_apply_kernel<<<(unsigned)S.nsums, kScanBlock, 0, st>>>(S.counts, S.ncounts, S.sums);
    scatter_kernel<<<(unsigned)S.nblocks, kSortThreads, 0, st>>>(kin, vin, nphys, shift,
                                                                 (int)S.nblocks, S.counts, kout, vout);
    for (int k = 0; k < 5; ++k) count_launch();
    uint32_t *tk = kin, *tv = vin;
    kin = kout;
    vin = vout;
    kout = tk;
    vout = tv;
  }
  // the dead keys (all ones) sort last; the live count is the first of them
  // (pass count keeps every key bit, so a dead key is the largest)
  count_live_kernel<<<1, 32, 0, st>>>(kin, nphys, n_out);
  count_launch();
  gather_kernel<<<grid_for(nphys, 256), 256, 0, st>>>(ix, fx, y, z, px, py, pz, w, vin, n_out, ix_out,
                                                      fx_out, y_out, z_out, px_out, py_out, pz_out,
                                                      w_out, nphys);
  count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"
