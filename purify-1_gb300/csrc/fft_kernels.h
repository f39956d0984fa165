// Row passes of the FP32 padded-grid FFT with Z S and S^H Z^H fused in, for
// power-of-two grid widths Nu = 64 ... 4096.
//
// The 2-D transform of the padded grid is a transform of its rows then of its
// columns (either order).  Only the Ny rows y0 ... y0+Ny-1 of the padded grid
// are nonzero on the way in, and only they are needed on the way out, so:
//   forward  x -> grid: the row pass reads each image row with the correction
//            S applied, places it at columns x0 ... x0+Nx-1 of a length-Nu row
//            and writes its transform to grid row y0 + j (the other rows of
//            the grid stay zero); a batched column transform (cuFFT) follows;
//   adjoint  grid -> x: the column transform (cuFFT) first, then the inverse
//            row pass reads grid rows y0 ... y0+Ny-1 and writes only the
//            columns x0 ... x0+Nx-1, times S.
// Both are unnormalised; the 1/sqrt(Nu Nv) of the unitary FFT is folded into
// S, as for the 2-D cuFFT path they replace.
#pragma once
#include <cuda_runtime_api.h>

#include <vector>

namespace pg {

struct FftArgs {
  int Nx = 0, Ny = 0, Nu = 0, Nv = 0, x0 = 0, y0 = 0;
  int ld = 0;                                // row stride of the grid in cells (0: Nu)
  const float *su = nullptr, *sv = nullptr;  // correction per column / row of the image
  const void *tw_u = nullptr;                // float2 exp(-2 pi i m / Nu), m < Nu
};

// True when the fused row passes handle grids Nu wide.
bool fft_rows_supported(int Nu);
// exp(-2 pi i m / N) for m < N, FP64-generated, as interleaved float pairs.
std::vector<float> fft_twiddles(int N);
// x (Ny x Nx) -> rows y0 ... of grid (Nv x Nu), row-transformed.
cudaError_t launch_fft_rows_forward(const FftArgs &a, const void *x, void *grid, cudaStream_t s);
// rows y0 ... of grid (column-transformed) -> x (Ny x Nx).
cudaError_t launch_fft_rows_inverse(const FftArgs &a, const void *grid, void *x, cudaStream_t s);

// Column transforms of a grid Nv high (power of two, 64 ... 2048) over its
// first W columns (row stride ld >= W): forward reads only rows y0 ...
// y0+Ny-1 of `in` (the others are taken as zero) and writes every row of
// `out`; inverse reads every row and writes only rows y0 ... y0+Ny-1.  in and
// out may be the same buffer.  With members set (a batch size group in the
// interleaved layout), column c belongs to channel members[c / Nu] of the
// ChannelIO<float> table chans, whose y0 and Ny apply.  Unnormalised.
struct FftColArgs {
  const void *in = nullptr;
  void *out = nullptr;
  int Nv = 0, W = 0, ld = 0, y0 = 0, Ny = 0;
  const void *tw_v = nullptr;  // float2 exp(-2 pi i m / Nv), m < Nv
  const void *chans = nullptr;
  const int *members = nullptr;
  int Nu = 0;
};
// True when the column pass handles W columns of height Nv.
bool fft_cols_supported(int Nv, int W);
cudaError_t launch_fft_cols(bool inverse, const FftColArgs &c, cudaStream_t s);

// The same passes over the channels of a batch that share one grid width Nu,
// in one launch (blockIdx.y = member): channel members[k] of the ChannelIO<float>
// table `chans` reads x_in and writes pad (forward), or reads work and writes
// x_out (inverse), with its own image size, offsets and corrections; every
// member's grids have row stride ld.  max_ny is the largest member Ny.
cudaError_t launch_fft_rows_group(bool inverse, const void *chans, const int *members, int nmembers,
                                  int Nu, int max_ny, int ld, const void *tw_u, cudaStream_t s);

}  // namespace pg
