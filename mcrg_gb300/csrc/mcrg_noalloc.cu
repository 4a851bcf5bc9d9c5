// mcrg_noalloc.cu -- coupling sums of a host lattice without any device
// allocation.
//
// mcrg_lattice_couplings() stages the lattice in device buffers it obtains
// with cudaMalloc and releases with cudaFree on every call.  Some callers
// cannot allow that: a program that has already handed the rest of the GPU's
// memory to its own pool, or that runs under a fixed memory budget, gets a
// failed or refused cudaMalloc in the middle of a run; and cudaMalloc /
// cudaFree may synchronise the whole device, which stalls every other stream
// of a caller that keeps the GPU busy between calls.  This entry point gives
// such callers the same result from a scratch area that is part of the
// library image itself: a file-scope __device__ array, reserved on every GPU
// that loads libmcrg.so for as long as the process lives.
//
// Limits and rules of use:
//   - lattices up to MCRG_NOALLOC_MAX_L x MCRG_NOALLOC_MAX_L (larger ones are
//     rejected with MCRG_ENOSPC); the array holds 2 * MAX_L^2 + 256 bytes;
//   - the first call on a device looks up the array's device address (once
//     per device, with that device current), so make that first call before
//     any stream capture;
//   - every call reuses the same array and leaves the last call's data in it;
//     the sums are cleared at the start of each call;
//   - calls are serialised per device by a host lock; calls that overlap on
//     the GPU in any other way (for example from code that writes the array
//     through its own copy of the address) race on the array.
#include <cstdint>
#include <mutex>

#include "mcrg_internal.cuh"

namespace {

constexpr size_t kSumsBytes = 256;  // int32 sums[5] + int32 bad flag, padded
constexpr size_t kLatticeBytes = (size_t)MCRG_NOALLOC_MAX_L * MCRG_NOALLOC_MAX_L;

// layout: [sums | natural staging copy | split-layout copy]
static __device__ __align__(256) uint8_t g_noalloc_scratch[kSumsBytes + 2 * kLatticeBytes];

std::mutex g_noalloc_mu[64];
uint8_t* g_noalloc_addr[64] = {};

__global__ void noalloc_split_kernel(const int8_t* __restrict__ nat, int N, uint8_t* __restrict__ split,
                                     int* __restrict__ bad) {
  const int half = N / 2;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N * N; s += gridDim.x * blockDim.x) {
    const int i = s / N, j = s % N;
    const int8_t v = nat[s];
    if (v != 1 && v != -1) atomicOr(bad, 1);
    split[(size_t)((i + j) & 1) * N * half + (size_t)i * half + (j >> 1)] = v > 0 ? 1 : 0;
  }
}

}  // namespace

extern "C" int mcrg_lattice_couplings_noalloc(int32_t N, const int8_t* host_in, int32_t n_couplings, int64_t* out,
                                              int32_t device) {
  if (!host_in || !out || N < 2 || (N & (N - 1)) || n_couplings < 1 || n_couplings > MCRG_MAX_COUPLINGS ||
      device < 0 || device >= 64)
    return MCRG_EINVAL;
  if (N > MCRG_NOALLOC_MAX_L) return MCRG_ENOSPC;
  if (cudaSetDevice(device) != cudaSuccess) return MCRG_EIO;
  std::lock_guard<std::mutex> lk(g_noalloc_mu[device]);
  if (!g_noalloc_addr[device]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MCRG_EIO;
    g_noalloc_addr[device] = static_cast<uint8_t*>(p);
  }
  uint8_t* base = g_noalloc_addr[device];
  int* sums = reinterpret_cast<int*>(base);
  int8_t* nat = reinterpret_cast<int8_t*>(base + kSumsBytes);
  uint8_t* split = base + kSumsBytes + kLatticeBytes;
  const size_t NN = (size_t)N * N;
  cudaStream_t s = 0;
  int h[8] = {0};
  if (cudaMemsetAsync(sums, 0, kSumsBytes, s) != cudaSuccess) return MCRG_EIO;
  if (cudaMemcpyAsync(nat, host_in, NN, cudaMemcpyHostToDevice, s) != cudaSuccess) return MCRG_EIO;
  int blocks = (int)((NN + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  noalloc_split_kernel<<<blocks, 256, 0, s>>>(nat, N, split, sums + 7);
  if (mcrg::launch_couplings_once(split, N, n_couplings, sums, s) != cudaSuccess) return MCRG_EIO;
  if (cudaMemcpyAsync(h, sums, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess) return MCRG_EIO;
  if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) return MCRG_EIO;
  if (h[7]) return MCRG_EINVAL;
  for (int c = 0; c < n_couplings; ++c) out[c] = h[c];
  return MCRG_OK;
}
