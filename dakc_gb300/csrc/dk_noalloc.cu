// dk_count_small_noalloc: count a small read set without allocating memory.
//
// Why it exists: some callers cannot call cudaMalloc (or any allocating
// routine) at the point where they want a count -- code running inside an
// allocator's own callback, a real-time or serving loop whose latency budget
// rules out the allocator's locks and device-wide synchronisation, or a
// host program that owns every byte of device memory through its own pool
// and forbids other libraries from reserving more.  dk_count and
// dk_count_device allocate their work buffers (key partitions, staging) in
// the engine context, so such callers cannot use them.  This entry point
// needs no context: the caller passes device input and output buffers, and
// the kernel's scratch (the unsorted k-mers, before they are sorted into
// shared memory) is one fixed array in this file, g_noalloc_keys, that the
// library holds on every device that loads it, until the process exits.
//
// Limits and sharing rules:
//   * at most kNoAllocMaxKmers (12,288) k-mer occurrences per call, judged by
//     the upper bound lines * (line_width - k + 1); larger inputs are
//     rejected with DK_ERR_ADMISSION before anything is launched;
//   * every call on a device uses the same scratch array, which keeps the
//     last call's contents; each call writes every entry it reads, so nothing
//     needs clearing, but calls that overlap on the GPU (different streams or
//     host threads with no ordering between them) race on it: order them;
//   * the first call on a device (with that device current) does a one-time
//     set-up: it looks up the scratch array's device address with
//     cudaGetSymbolAddress and raises the kernel's shared-memory limit.  Make
//     that first call before any stream capture on that device.  A device
//     reset (cudaDeviceReset) invalidates that set-up: use a new process.
//
// The kernel is a single-CTA variant of the engine's bin count: it extracts
// the k-mers of every line (the same warp-per-line extraction), counting-sorts
// them into shared memory by their top bits, finishes each digit range by
// insertion or bitonic sort and run-length reduces into the caller's table.
#include "dk_device.cuh"
#include "../../include/dakc_gb300.h"

#include <cuda_runtime.h>
#include <mutex>

namespace dk {

namespace {

using namespace dev;

constexpr int kNoAllocMaxKmers = 12288;
constexpr int kNoAllocThreads = 512;
// dynamic shared memory: the sorted k-mers, then the run heads (uint32)
constexpr size_t kNoAllocSmem = (size_t)kNoAllocMaxKmers * 12;

// The scratch: the unsorted k-mers of one call (98,304 bytes per device).
// Host code reaches it only through the address cudaGetSymbolAddress gives.
static __device__ __align__(256) unsigned long long g_noalloc_keys[kNoAllocMaxKmers];

template <int C>
__global__ void __launch_bounds__(kNoAllocThreads)
    k_count_small_static(const uint8_t* __restrict__ text, uint64_t n_lines, int W, int k,
                         unsigned long long* __restrict__ keys, uint64_t* __restrict__ out_k,
                         uint32_t* __restrict__ out_c, uint64_t* __restrict__ summary) {
  extern __shared__ unsigned long long skeys[];  // kNoAllocMaxKmers, then the heads
  __shared__ uint32_t hist[1u << 12];
  __shared__ unsigned long long tmp[32];
  __shared__ uint8_t lut[256];
  __shared__ uint16_t long_list[512];
  __shared__ uint32_t s_n, n_long;
  __shared__ unsigned long long s_first_nul;
  // the raw k-mers wait in the scratch array (keys) until they are sorted
  // into shared memory
  uint32_t* heads = reinterpret_cast<uint32_t*>(skeys + kNoAllocMaxKmers);
  if (threadIdx.x == 0) {
    s_n = 0;
    n_long = 0;
    s_first_nul = n_lines;
  }
  init_lut(lut);
  __syncthreads();
  const uint64_t stride = (uint64_t)W + 1;
  // parsing stops before the first line (after line 0) whose first byte is NUL
  for (uint64_t l = 1 + threadIdx.x; l < n_lines; l += blockDim.x)
    if (text[l * stride] == 0) atomicMin(&s_first_nul, (unsigned long long)l);
  __syncthreads();
  const uint64_t L = s_first_nul;
  const uint64_t kmask = (~0ull) >> (64 - 2 * k);
  const uint32_t warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (uint64_t l = warp; l < L; l += nwarps) {
    warp_line_kmers<C>(text + l * stride, W, k, kmask, lut, [&](int, uint64_t key, bool valid) {
      if (valid) {
        const uint32_t slot = atomicAdd(&s_n, 1u);
        if (slot < kNoAllocMaxKmers) __stcg(keys + slot, (unsigned long long)key);
      }
    });
  }
  __syncthreads();
  const uint32_t n = s_n;
  if (n > kNoAllocMaxKmers) {  // unreachable after the host's bound check
    if (threadIdx.x == 0) { summary[0] = 0; summary[1] = n; summary[2] = 1; }
    return;
  }
  // counting sort on the top D bits into shared memory
  const int bits = 2 * k;
  int D = n <= 1 ? 0 : 32 - __clz(n - 1);
  D = max(4, min(D, 12));
  D = min(D, bits);
  const int sh = bits - D;
  const uint32_t R = 1u << D;
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) hist[j] = 0;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
    atomicAdd(&hist[(uint32_t)(__ldcg(keys + i) >> sh) & (R - 1)], 1u);
  __syncthreads();
  block_scan_array<uint32_t>(hist, (int)R, reinterpret_cast<uint32_t*>(tmp));
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    const unsigned long long key = __ldcg(keys + i);
    skeys[atomicAdd(&hist[(uint32_t)(key >> sh) & (R - 1)], 1u)] = key;
  }
  __syncthreads();
  // finish each digit range (hist[j] is now the end of range j)
  if (sh > 0) {
    for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) {
      const uint32_t lo = j ? hist[j - 1] : 0, hi = hist[j];
      const uint32_t len = hi - lo;
      if (len <= 1) continue;
      if (len <= 32) {
        for (uint32_t x = lo + 1; x < hi; ++x) {
          const unsigned long long v = skeys[x];
          uint32_t y = x;
          while (y > lo && skeys[y - 1] > v) { skeys[y] = skeys[y - 1]; --y; }
          skeys[y] = v;
        }
      } else {
        long_list[atomicAdd(&n_long, 1u)] = (uint16_t)j;
      }
    }
    __syncthreads();
    const uint32_t nl = n_long;
    for (uint32_t q = 0; q < nl; ++q) {
      const uint32_t j = long_list[q];
      const uint32_t lo = j ? hist[j - 1] : 0, hi = hist[j];
      block_bitonic(skeys + lo, hi - lo);
    }
    __syncthreads();
  }
  // run-length reduce straight into the caller's table
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = min(n, threadIdx.x * per), hi = min(n, lo + per);
  uint32_t nh = 0;
  for (uint32_t i = lo; i < hi; ++i) nh += (i == 0 || skeys[i] != skeys[i - 1]);
  uint32_t total;
  const uint32_t r0 = block_excl_scan<uint32_t>(nh, reinterpret_cast<uint32_t*>(tmp), &total);
  uint32_t r = r0;
  for (uint32_t i = lo; i < hi; ++i)
    if (i == 0 || skeys[i] != skeys[i - 1]) {
      out_k[r] = skeys[i];
      heads[r] = i;
      ++r;
    }
  __syncthreads();
  for (uint32_t q = threadIdx.x; q < total; q += blockDim.x) {
    const uint32_t end = (q + 1 < total) ? heads[q + 1] : n;
    out_c[q] = end - heads[q];
  }
  if (threadIdx.x == 0) {
    summary[0] = total;
    summary[1] = n;
    summary[2] = 0;
  }
}

struct DeviceSetup {
  bool ready = false;
  unsigned long long* scratch = nullptr;  // device address of g_noalloc_keys
};
constexpr int kMaxDevices = 128;
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

template <int C>
cudaError_t prepare_kernel() {
  return cudaFuncSetAttribute(k_count_small_static<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kNoAllocSmem);
}

// one-time, per-device set-up (the device must be current): the scratch
// array's device address and the kernel's shared-memory limit
int setup_device(int dev, unsigned long long** scratch) {
  std::lock_guard<std::mutex> g(g_setup_mu);
  DeviceSetup& s = g_setup[dev];
  if (!s.ready) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_keys) != cudaSuccess || !p) {
      cudaGetLastError();
      return DK_ERR_CUDA;
    }
    s.scratch = static_cast<unsigned long long*>(p);
    cudaError_t e = cudaSuccess;
    for (cudaError_t x : {prepare_kernel<1>(), prepare_kernel<2>(), prepare_kernel<4>(),
                          prepare_kernel<5>(), prepare_kernel<8>(), prepare_kernel<16>(),
                          prepare_kernel<32>()})
      if (x != cudaSuccess) e = x;
    if (e != cudaSuccess) {
      cudaGetLastError();
      return DK_ERR_CUDA;
    }
    s.ready = true;
  }
  *scratch = s.scratch;
  return DK_OK;
}

}  // namespace
}  // namespace dk

extern "C" int dk_count_small_noalloc(const char* d_text, uint64_t nbytes, int line_width, int k,
                                      uint64_t* d_kmers, uint32_t* d_counts, uint64_t capacity,
                                      uint64_t* d_summary, void* stream) {
  using namespace dk;
  if (k < 1 || k > 32 || line_width < 1 || line_width > 1024 || !d_kmers || !d_counts ||
      !d_summary || (!d_text && nbytes))
    return DK_ERR_INVALID_ARG;
  const uint64_t stride = (uint64_t)line_width + 1;
  uint64_t lines = 0;
  if (nbytes) {
    const uint64_t rem = nbytes % stride;
    if (rem != 0 && rem != (uint64_t)line_width) return DK_ERR_INVALID_ARG;
    lines = (nbytes + 1) / stride;
  }
  const uint64_t per_line = line_width >= k ? (uint64_t)(line_width - k + 1) : 0;
  const uint64_t bound = lines * per_line;
  if (bound > (uint64_t)kNoAllocMaxKmers) return DK_ERR_ADMISSION;
  if (capacity < bound) return DK_ERR_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return DK_ERR_NO_DEVICE;
  }
  unsigned long long* scratch = nullptr;
  const int rc = setup_device(dev, &scratch);
  if (rc != DK_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint8_t* t = reinterpret_cast<const uint8_t*>(d_text);
  const size_t smem = kNoAllocSmem;
  const int c = (line_width + 31) / 32;
  if (c <= 1) k_count_small_static<1><<<1, kNoAllocThreads, smem, s>>>(t, lines, line_width, k, scratch, d_kmers, d_counts, d_summary);
  else if (c <= 2) k_count_small_static<2><<<1, kNoAllocThreads, smem, s>>>(t, lines, line_width, k, scratch, d_kmers, d_counts, d_summary);
  else if (c <= 4) k_count_small_static<4><<<1, kNoAllocThreads, smem, s>>>(t, lines, line_width, k, scratch, d_kmers, d_counts, d_summary);
  else if (c <= 5) k_count_small_static<5><<<1, kNoAllocThreads, smem, s>>>(t, lines, line_width, k, scratch, d_kmers, d_counts, d_summary);
  else if (c <= 8) k_count_small_static<8><<<1, kNoAllocThreads, smem, s>>>(t, lines, line_width, k, scratch, d_kmers, d_counts, d_summary);
  else if (c <= 16) k_count_small_static<16><<<1, kNoAllocThreads, smem, s>>>(t, lines, line_width, k, scratch, d_kmers, d_counts, d_summary);
  else k_count_small_static<32><<<1, kNoAllocThreads, smem, s>>>(t, lines, line_width, k, scratch, d_kmers, d_counts, d_summary);
  if (cudaGetLastError() != cudaSuccess) return DK_ERR_CUDA;
  return DK_OK;
}
