// Particle bookkeeping (particle_tools.f90:130-324): stable compaction,
// chunk binning and the stable counting sort that orders particles by
// x-chunk, plus the gather used to apply a permutation.
//
// All passes are deterministic: counts use integer atomics, ranks within a
// tile come from warp ballots in index order, so the produced permutation is
// the stable one (particles keep their relative order inside a chunk).
#include "common.cuh"

using namespace chm;

namespace {

constexpr int kTile = 2048;       // elements per block in the scan passes
constexpr int kSortThreads = 256;  // 8 warps, each owning kTile/8 elements
constexpr int kMaxBuckets = 258;

__device__ __forceinline__ bool inside(const double *x, i64 cs, i64 ps, i64 i, const double lims[4]) {
  const double xp = x[i * ps], y = x[cs + i * ps], z = x[2 * cs + i * ps];
  const double r2 = y * y + z * z;
  return xp >= lims[0] && xp <= lims[1] && r2 >= lims[2] && r2 <= lims[3];
}

struct Lims {
  double v[4];
};

// Bucket of element i for the generic stable counting sort.
// mode 0: sortpartsout (bucket 0 = stays, 1 = leaves)
// mode 1: chunk order (bucket = chunk id, nchnk = leaves)
struct BucketSrc {
  int mode;
  const double *x;
  i64 cs, ps;
  Lims lims;
  const int8_t *ids;
  int nchnk;
  __device__ int operator()(i64 i) const {
    if (mode == 0) return inside(x, cs, ps, i, lims.v) ? 0 : 1;
    int c = ids[i];
    return (c >= 0 && c < nchnk) ? c : nchnk;
  }
};

// pass 1: per-tile bucket histogram hist[bucket * ntiles + tile]
__global__ void hist_kernel(BucketSrc B, i64 n, int nb, i64 ntiles, int *__restrict__ hist) {
  __shared__ int h[kMaxBuckets];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const i64 t0 = (i64)blockIdx.x * kTile, t1 = min(n, t0 + kTile);
  for (i64 i = t0 + threadIdx.x; i < t1; i += blockDim.x) atomicAdd(&h[B(i)], 1);
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) hist[(i64)b * ntiles + blockIdx.x] = h[b];
}

// pass 2: exclusive scan of hist in (bucket, tile) order -- one block
__global__ void scan_kernel(int *__restrict__ hist, i64 len, int *__restrict__ total) {
  __shared__ long long carry;
  __shared__ int warp_sums[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (i64 base = 0; base < len; base += blockDim.x) {
    i64 i = base + threadIdx.x;
    int v = i < len ? hist[i] : 0;
    // inclusive warp scan
    int s = v;
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, s, o);
      if ((threadIdx.x & 31) >= o) s += t;
    }
    if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      int w = threadIdx.x < (blockDim.x >> 5) ? warp_sums[threadIdx.x] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, w, o);
        if (threadIdx.x >= o) w += t;
      }
      warp_sums[threadIdx.x] = w;
    }
    __syncthreads();
    int warp_off = (threadIdx.x >> 5) ? warp_sums[(threadIdx.x >> 5) - 1] : 0;
    if (i < len) hist[i] = (int)(carry + warp_off + s - v);
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += warp_off + s;
    __syncthreads();
  }
  if (threadIdx.x == 0) total[0] = (int)carry;
}

// pass 3: stable scatter.  Each warp owns a contiguous kTile/8 slice of the
// tile; ranks inside a 32-element step come from __match_any_sync, across
// steps from a per-warp running count, across warps from a prefix over the
// warps' bucket counts.
__global__ void scatter_kernel(BucketSrc B, i64 n, int nb, i64 ntiles, const int *__restrict__ off,
                               i64 *__restrict__ idx_out, int keep_buckets) {
  __shared__ int wcount[kSortThreads / 32][kMaxBuckets];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const i64 t0 = (i64)blockIdx.x * kTile, t1 = min(n, t0 + kTile);
  const int per = kTile / nw;
  const i64 w0 = t0 + (i64)warp * per, w1 = min(t1, w0 + per);
  for (int b = lane; b < nb; b += 32) wcount[warp][b] = 0;
  __syncwarp();
  // count per warp
  for (i64 i = w0 + lane; i < w1; i += 32) atomicAdd(&wcount[warp][B(i)], 1);
  __syncthreads();
  // exclusive prefix over warps for each bucket
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    int s = 0;
    for (int w = 0; w < nw; ++w) {
      int c = wcount[w][b];
      wcount[w][b] = s;
      s += c;
    }
  }
  __syncthreads();
  for (i64 base = w0; base < w1; base += 32) {
    const i64 i = base + lane;
    const bool valid = i < w1;
    const int b = valid ? B(i) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && b < keep_buckets) {
      const i64 pos = (i64)off[(i64)b * ntiles + blockIdx.x] + wcount[warp][b] + rank;
      idx_out[pos] = i;
    }
    __syncwarp();
    // leader of each bucket group advances the running count
    if (valid && rank == 0) wcount[warp][b] += __popc(peers);
    __syncwarp();
  }
}

__global__ void chunk_ids_kernel(const double *__restrict__ x, i64 cs, i64 ps, Lims lims,
                                 double x0, double cl_inv, int nchnk, i64 n, int8_t *__restrict__ ids,
                                 int *__restrict__ counts) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const double xp = x[i * ps];
    const double f = floor((xp - x0) * cl_inv);
    int8_t id = -2;
    if (inside(x, cs, ps, i, lims.v)) {
      const long long c = (f > -1.0e9 && f < 1.0e9) ? (long long)f : -1;
      if (c >= 0 && c < nchnk) atomicAdd(&counts[c], 1);
      id = (int8_t)c;
    } else {
      atomicAdd(&counts[nchnk], 1);
    }
    ids[i] = id;
  }
}

__global__ void offsets_kernel(const int *__restrict__ counts, int nchnk, int32_t *__restrict__ ind) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int s = 0;
    ind[0] = 0;
    for (int c = 0; c < nchnk; ++c) {
      s += counts[c];
      ind[c + 1] = s;
    }
  }
}

__global__ void gather_kernel(double *__restrict__ dst, i64 d_cs, i64 d_ps, const double *__restrict__ src,
                              i64 s_cs, i64 s_ps, int ncomp, const i64 *__restrict__ idx, i64 n) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const i64 j = idx[i];
    for (int c = 0; c < ncomp; ++c) dst[c * d_cs + i * d_ps] = src[c * s_cs + j * s_ps];
  }
}

i64 sort_ws(i64 n, int nb) {
  const i64 ntiles = (n + kTile - 1) / kTile;
  return 4 * (ntiles * nb + 64) + 256;
}

int stable_bucket_order(const BucketSrc &B, i64 n, int nb, int keep, i64 *idx_out, int *kept,
                        void *ws, i64 ws_bytes, cudaStream_t st) {
  const i64 ntiles = (n + kTile - 1) / kTile;
  if (ws_bytes < sort_ws(n, nb) || !ws) {
    set_error("sort: workspace too small");
    return CHM_ERR_WS;
  }
  int *hist = reinterpret_cast<int *>(ws);
  int *total = hist + ntiles * nb;
  hist_kernel<<<(unsigned)ntiles, kSortThreads, 0, st>>>(B, n, nb, ntiles, hist); chm::count_launch();
  scan_kernel<<<1, 1024, 0, st>>>(hist, ntiles * nb, total); chm::count_launch();
  scatter_kernel<<<(unsigned)ntiles, kSortThreads, 0, st>>>(B, n, nb, ntiles, hist, idx_out, keep); chm::count_launch();
  CHM_CHECK_LAUNCH();
  // kept = offset of bucket `keep` (first dropped bucket) = sum of kept buckets
  if (kept) {
    if (keep < nb) {
      if (cudaMemcpyAsync(kept, hist + (i64)keep * ntiles, sizeof(int), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess) {
        set_error("sort: copy of the kept count failed");
        return CHM_ERR_CUDA;
      }
    } else if (cudaMemcpyAsync(kept, total, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) {
      set_error("sort: copy of the total failed");
      return CHM_ERR_CUDA;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) {
      set_error("sort: stream synchronisation failed");
      return CHM_ERR_CUDA;
    }
  }
  return CHM_OK;
}

}  // namespace

extern "C" {

int64_t chm_sortpartsout_ws_bytes(int64_t np) { return sort_ws(np, kMaxBuckets); }

int chm_sortpartsout(int64_t *indx2stay, int64_t *num2stay, const double *coord, int64_t x_cs,
                     int64_t x_ps, const double *lims, int64_t np, void *ws, int64_t ws_bytes,
                     void *stream) {
  CHM_REQUIRE(num2stay && lims && np >= 0, "sortpartsout: bad args");
  *num2stay = 0;
  if (np == 0) return CHM_OK;
  CHM_REQUIRE(np < (1LL << 31), "sortpartsout: np must be < 2^31");
  CHM_REQUIRE(indx2stay && coord, "sortpartsout: null pointer");
  BucketSrc B{};
  B.mode = 0;
  B.x = coord;
  B.cs = x_cs;
  B.ps = x_ps;
  for (int i = 0; i < 4; ++i) B.lims.v[i] = lims[i];
  int kept = 0;
  int rc = stable_bucket_order(B, np, 2, 1, indx2stay, &kept, ws, ws_bytes, as_stream(stream));
  *num2stay = kept;
  return rc;
}

int chm_chunk_coords_boundaries(int8_t *chunked_indx, int32_t *ind_in_chnk, int64_t *go_out,
                                const double *coord, int64_t x_cs, int64_t x_ps, const double *lims,
                                double xgrid0, double xgridc, int64_t nchnk, int64_t np, void *ws,
                                int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(lims && go_out && nchnk >= 1 && nchnk <= 127, "chunk_coords_boundaries: bad args");
  CHM_REQUIRE(ws && ws_bytes >= 4 * (nchnk + 2), "chunk_coords_boundaries: workspace too small");
  cudaStream_t st = as_stream(stream);
  int *counts = reinterpret_cast<int *>(ws);
  cudaMemsetAsync(counts, 0, sizeof(int) * (nchnk + 1), st);
  if (np > 0) {
    CHM_REQUIRE(chunked_indx && coord, "chunk_coords_boundaries: null pointer");
    Lims L;
    for (int i = 0; i < 4; ++i) L.v[i] = lims[i];
    chunk_ids_kernel<<<grid_for(np, 256), 256, 0, st>>>(coord, x_cs, x_ps, L, xgrid0,
                                                        1.0 / (xgridc - xgrid0), (int)nchnk, np,
                                                        chunked_indx, counts); chm::count_launch();
  }
  offsets_kernel<<<1, 32, 0, st>>>(counts, (int)nchnk, ind_in_chnk); chm::count_launch();
  CHM_CHECK_LAUNCH();
  int go = 0;
  cudaMemcpyAsync(&go, counts + nchnk, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    set_error("chunk_coords_boundaries: synchronisation failed");
    return CHM_ERR_CUDA;
  }
  *go_out = go;
  return CHM_OK;
}

// Stable order of the particles by chunk id (ids outside [0, nchnk) are
// dropped): the permutation `index2stay.argsort()[go_out:]` of
// species.py:379-383 with a stable sort.  idx_out receives *n_kept indices.
int64_t chm_chunk_order_ws_bytes(int64_t np, int64_t nchnk) { return sort_ws(np, (int)nchnk + 1); }

int chm_chunk_order(int64_t *idx_out, int64_t *n_kept, const int8_t *chunked_indx, int64_t nchnk,
                    int64_t np, void *ws, int64_t ws_bytes, void *stream) {
  CHM_REQUIRE(n_kept && nchnk >= 1 && nchnk <= 127, "chunk_order: bad args");
  *n_kept = 0;
  if (np == 0) return CHM_OK;
  CHM_REQUIRE(np < (1LL << 31), "chunk_order: np must be < 2^31");
  CHM_REQUIRE(idx_out && chunked_indx, "chunk_order: null pointer");
  BucketSrc B{};
  B.mode = 1;
  B.ids = chunked_indx;
  B.nchnk = (int)nchnk;
  int kept = 0;
  int rc = stable_bucket_order(B, np, (int)nchnk + 1, (int)nchnk, idx_out, &kept, ws, ws_bytes,
                               as_stream(stream));
  *n_kept = kept;
  return rc;
}

int chm_align_data(double *dst, int64_t d_cs, int64_t d_ps, const double *src, int64_t s_cs,
                   int64_t s_ps, int64_t ncomp, const int64_t *idx, int64_t n, void *stream) {
  CHM_REQUIRE(n >= 0 && ncomp >= 1, "align_data: bad args");
  if (n == 0) return CHM_OK;
  CHM_REQUIRE(dst && src && idx && dst != src, "align_data: null or aliased pointers");
  gather_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(dst, d_cs, d_ps, src, s_cs, s_ps,
                                                                 (int)ncomp, idx, n); chm::count_launch();
  CHM_CHECK_LAUNCH();
  return CHM_OK;
}

}  // extern "C"
