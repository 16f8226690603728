// Dense products of the split-precision form:
//   C(M, N) = A(M, K) * B(K, N), A = a complex64 plane viewed as real
//   (M = 2 nx rows), B = a per-mode real DHT / coupling matrix.
#pragma once
#include "common.cuh"

namespace chm {

// Column tiling of the tensor-core products: N is cut into tc_col_tiles(N)
// tiles of tc_tile_cols(N) columns (a multiple of 16, at most 128), and the
// prepared split terms hold tc_np(N) = tiles x columns per K block (the
// columns past N are zero), so every tile reads a whole block.
inline int tc_col_tiles(int N) { return ((N + 15) / 16 * 16 + 127) / 128; }
inline int tc_tile_cols(int N) {
  const int nt = tc_col_tiles(N), np = (N + 15) / 16 * 16;
  return ((np + nt - 1) / nt + 15) / 16 * 16;
}
inline int tc_np(int N) { return tc_col_tiles(N) * tc_tile_cols(N); }

// One mode's B operand: FP32 copy and the 3-term BF16 split
// (b = b0 + b1 + b2 exactly to ~2^-24) in the tensor-core operand layout.
struct TcOperand {
  const float *f32;        // (K, N) column-major
  const uint16_t *bf[3];   // split terms, see tc_gemm.cu
  int K, N;
};

struct TcMatrices {
  TcOperand mode[16];
};

// One product of a batch; every problem of a batch has the same M, N, K and
// epilogue but its own operator (mode).
struct TcProblem {
  const float *A;    // (M, K) column-major, ld = M
  float *C;          // (M, N) column-major, ld = M
  const float *fac;  // optional (M/2, N) real factor
  TcOperand B;
  // read A as the reflected complex plane: row (x, c) of A is
  // (c ? 1 : -1) * row ((M/2 - x) mod M/2, c) of the stored plane, the
  // m = -1 neighbour of a mode-1 field (fb_math.f90 reflection)
  int reflect;
};

enum { TC_EPI_STORE = 0, TC_EPI_SHIFT = 1, TC_EPI_SHIFT_FAC = 2 };

// Batched product.  ws holds the BF16 split of every distinct A plane of
// the batch (at most tc_split_bytes(M, K, count) bytes), in use until the
// product completes on the stream.
int tc_gemm_launch(const TcProblem *p, int count, int M, int N, int K, int epi,
                   const float2 *shift, void *ws, long long ws_bytes, cudaStream_t st);
long long tc_split_bytes(int M, int K, int count);

// Host view of a prepared operator set (chm_sp_ops) as per-mode operands.
TcMatrices tc_matrices(const chm_sp_ops *ops);

}  // namespace chm
