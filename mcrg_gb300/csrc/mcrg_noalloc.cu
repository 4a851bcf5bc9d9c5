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
//   - the first call on a device sets that device up, with it current: it
//     looks up the array's device address and creates one non-blocking
//     stream that every later call on the device uses, so no call touches
//     the legacy default stream and none waits for the caller's other
//     streams; make that first call before any stream capture;
//   - every call reuses the same array and leaves the last call's data in it;
//     the sums are cleared at the start of each call;
//   - calls are serialised per device by a host lock held until the call's
//     device work has finished (on error paths too); calls that overlap on
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

// Per-device set-up, done once by the first call on the device.
struct NoallocDevice {
  std::mutex mu;
  uint8_t* addr = nullptr;        // device address of g_noalloc_scratch on this device
  cudaStream_t stream = nullptr;  // non-blocking: no implicit sync with the legacy default stream
};
NoallocDevice g_noalloc[64];

// Runs the call's device work on `s`; any failure after the first enqueue
// waits for the stream before it returns, so the caller's lock covers all of
// this call's writes to the array.
int couplings_from_scratch(uint8_t* base, cudaStream_t s, int32_t N, const int8_t* host_in, int32_t n_couplings,
                           int64_t* out) {
  int* sums = reinterpret_cast<int*>(base);
  int8_t* nat = reinterpret_cast<int8_t*>(base + kSumsBytes);
  uint8_t* split = base + kSumsBytes + kLatticeBytes;
  const size_t NN = (size_t)N * N;
  int h[8] = {0};
  if (cudaMemsetAsync(sums, 0, kSumsBytes, s) != cudaSuccess) return MCRG_EIO;
  if (cudaMemcpyAsync(nat, host_in, NN, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      mcrg::launch_nat_to_split(nat, N, split, sums + 7, s) != cudaSuccess ||
      mcrg::launch_couplings_once(split, N, n_couplings, sums, s) != cudaSuccess ||
      cudaMemcpyAsync(h, sums, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess) {
    cudaStreamSynchronize(s);
    return MCRG_EIO;
  }
  // the stream's own status is the authority: a stale error of the caller's is neither reported nor consumed
  if (cudaStreamSynchronize(s) != cudaSuccess) return MCRG_EIO;
  if (h[7]) return MCRG_EINVAL;
  for (int c = 0; c < n_couplings; ++c) out[c] = h[c];
  return MCRG_OK;
}

}  // namespace

extern "C" int mcrg_lattice_couplings_noalloc(int32_t N, const int8_t* host_in, int32_t n_couplings, int64_t* out,
                                              int32_t device) {
  if (!host_in || !out || N < 2 || (N & (N - 1)) || n_couplings < 1 || n_couplings > MCRG_MAX_COUPLINGS ||
      device < 0 || device >= 64)
    return MCRG_EINVAL;
  if (N > MCRG_NOALLOC_MAX_L) return MCRG_ENOSPC;
  if (cudaSetDevice(device) != cudaSuccess) return MCRG_EIO;
  NoallocDevice& d = g_noalloc[device];
  std::lock_guard<std::mutex> lk(d.mu);
  if (!d.addr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MCRG_EIO;
    if (!d.stream && cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking) != cudaSuccess) {
      d.stream = nullptr;
      return MCRG_EIO;
    }
    d.addr = static_cast<uint8_t*>(p);
  }
  return couplings_from_scratch(d.addr, d.stream, N, host_in, n_couplings, out);
}
