// mcrg_rgnn.cu -- forward pass of the reference's RG neural network on the
// device-resident configuration (RenormalizationGroupNeuralNetwork::
// scalar_output, src/rgnn.cpp:281-307): the 2x2 filter
//   out(i, j) = || W * block(2i, 2j, 2, 2) ||_1
// is applied until one value remains.  The value of level k at (i, j) depends
// only on the 2^k x 2^k tile under it, so each CTA reduces a tile of up to
// 32 x 32 inputs through five levels in shared memory and writes one value;
// log2(L) / 5 passes finish the pyramid (L = 16384: three passes, the first
// reading the int8 split layout directly).  FP64 in the reference's order of
// operations, without fused multiply-adds, so results equal the reference's
// bit for bit.
#include <cstdint>

#include "mcrg_internal.cuh"

namespace mcrg {
namespace {

struct Filter {
  double w00, w01, w10, w11;
};

// conv(r, c) = W(r, 0) B(0, c) + W(r, 1) B(1, c); L1 = (|c00| + |c01|) + (|c10| + |c11|)
__device__ __forceinline__ double filter(const Filter& f, double b00, double b01, double b10, double b11) {
  const double c00 = __dadd_rn(__dmul_rn(f.w00, b00), __dmul_rn(f.w01, b10));
  const double c01 = __dadd_rn(__dmul_rn(f.w00, b01), __dmul_rn(f.w01, b11));
  const double c10 = __dadd_rn(__dmul_rn(f.w10, b00), __dmul_rn(f.w11, b10));
  const double c11 = __dadd_rn(__dmul_rn(f.w10, b01), __dmul_rn(f.w11, b11));
  return __dadd_rn(__dadd_rn(fabs(c00), fabs(c01)), __dadd_rn(fabs(c10), fabs(c11)));
}

constexpr int kTile = 32;

// One CTA per T x T tile of the level of side n (T = min(n, 32)).  Input: the
// split-layout spins (level 0) or the FP64 values of a level, row-major.
__global__ void __launch_bounds__(256) rgnn_tile_kernel(const uint8_t* __restrict__ split,
                                                        const double* __restrict__ vin, int n, int T, Filter f,
                                                        double* __restrict__ vout) {
  __shared__ double v[kTile * kTile];
  const int tiles_x = n / T;
  const int ti = blockIdx.x / tiles_x, tj = blockIdx.x % tiles_x;
  const size_t half = (size_t)(n / 2);
  for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
    const int i = ti * T + e / T, j = tj * T + e % T;
    double x;
    if (split) {
      const int c = (i + j) & 1;
      x = split[(size_t)c * n * half + (size_t)i * half + (j >> 1)] ? 1.0 : -1.0;
    } else {
      x = vin[(size_t)i * n + j];
    }
    v[e] = x;  // tile row-major, stride T
  }
  __syncthreads();
  for (int m = T; m > 1; m >>= 1) {
    const int h = m / 2;
    double r = 0.0;
    const int a = threadIdx.x / h, b = threadIdx.x % h;
    const bool mine = threadIdx.x < h * h;  // h <= 16: at most 256 outputs
    if (mine)
      r = filter(f, v[(2 * a) * T + 2 * b], v[(2 * a) * T + 2 * b + 1], v[(2 * a + 1) * T + 2 * b],
                 v[(2 * a + 1) * T + 2 * b + 1]);
    __syncthreads();
    if (mine) v[a * T + b] = r;
    __syncthreads();
  }
  if (threadIdx.x == 0) vout[blockIdx.x] = v[0];
}

}  // namespace

// Scalar output of the network for a lattice of side n in split layout on the
// device; `work` holds (n/32)^2 + (n/1024)^2 doubles.  Result left in *d_out.
cudaError_t launch_rgnn_scalar(const uint8_t* d_split, int n, const double W[4], double* work, double* d_out,
                               cudaStream_t s) {
  const Filter f{W[0], W[1], W[2], W[3]};
  const double* cur = nullptr;
  double* bufs[2] = {work, work + (size_t)(n / kTile) * (n / kTile) + 1};
  int side = n, pass = 0;
  while (side > 1) {
    const int T = side < kTile ? side : kTile;
    const int tiles = (side / T) * (side / T);
    double* dst = (side / T == 1) ? d_out : bufs[pass & 1];
    rgnn_tile_kernel<<<tiles, 256, 0, s>>>(pass == 0 ? d_split : nullptr, cur, side, T, f, dst);
    cur = dst;
    side /= T;
    ++pass;
  }
  return cudaGetLastError();
}

}  // namespace mcrg
