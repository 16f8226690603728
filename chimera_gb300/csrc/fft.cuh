// Batched shared-memory FFT along x (FP64), one thread block per line.
//
// Mixed-radix Stockham (radices 4, 2, 3, 5, 7, and any other prime as a
// direct DFT), ping-ponging between two shared-memory line buffers.  The
// twiddle table tw[t] = exp(-2 pi i t / N) lives in global memory (L1/L2
// resident) and is written once per call by fft_twiddle_kernel.
#pragma once
#include "common.cuh"

namespace chm {

constexpr int kFftMaxN = 4096;  // 2 x 4096 x 16 B = 128 KB of shared memory
constexpr int kFftMaxStages = 24;

struct FftPlan {
  int n;
  int nstages;
  int radix[kFftMaxStages];
};

// Host: factorise n; returns false if a stage would exceed the limits.
bool fft_make_plan(int n, FftPlan *p);

__global__ void fft_twiddle_kernel(double2 *tw, int n);

// Line addressing: line b of the batch reads input row
//   in + ((b / in_rows) * in_rows_tot + (b % in_rows) + in_row_off) * n
// and writes output row likewise.  Pre/post operations:
//   pre_shift  : multiply the input by shift[x] (complex) before the FFT
//   post_scale : multiply the output by a per-mode real factor (eb modes)
//   ghost      : the first row of every mode also writes row 0 (= sign * row)
//   filter     : fb_filtr (backward FFT, profile, forward FFT, 1/(N shift))
struct FftLines {
  const double2 *in;
  double2 *out;
  int in_rows, in_rows_tot, in_row_off;
  int out_rows, out_rows_tot, out_row_off;
  int nm;               // modes (for per-mode post factors)
  int eb_mode;          // 0 none, 1 eb_correction, 2 eb_correction_env
  int sign;             // -1 forward, +1 backward
  const double2 *pre_shift;  // or null
  // fb_filtr
  int filt_mode;        // -1 none, else 0/1/2
  const double *filtr;
  int nxfilt;
};

__global__ void fft_lines_kernel(FftPlan plan, const double2 *__restrict__ tw, FftLines L);

int fft_launch(const FftLines &L, int n, i64 nlines, double2 *tw, cudaStream_t st);

}  // namespace chm
