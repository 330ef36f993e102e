// Operations on a finished (k-mer, count) table: the count histogram and
// PakMan*'s min-bucket cut-off (pakman_star/src/kmer_histogram.cpp:72-123),
// filtering by a minimum count, lookups of query k-mers, and the packed
// 12-byte (k-mer, count) records PakMan* keeps (KmerPairs,
// pakman_star/includes/distribute_kmers.h:690-696).
//
// The tables are the engine's own: device memory or its page-locked host
// pool, both addressable by the GPU, so every operation runs as kernels over
// the table where it lies.
#include "dk_engine.hpp"
#include "dk_device.cuh"
#include "../../include/dakc_gb300.h"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

namespace dk {
namespace {

using dev::block_excl_scan;

constexpr int kOpsThreads = 256;
constexpr uint32_t kHistSmemBuckets = 8192;  // larger histograms count in global memory

// hist[c] += number of entries with count c < nb
__global__ void __launch_bounds__(kOpsThreads) k_count_hist(const uint32_t* __restrict__ counts,
                                                            uint64_t n, uint32_t nb,
                                                            unsigned long long* __restrict__ hist) {
  __shared__ uint32_t sh[kHistSmemBuckets];
  const bool local = nb <= kHistSmemBuckets;
  if (local)
    for (uint32_t j = threadIdx.x; j < nb; j += blockDim.x) sh[j] = 0;
  __syncthreads();
  // most k-mers share a few small counts: lanes with the same count add once
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t span = (n + stride - 1) / stride * stride;  // whole warps stay in the loop
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < span; i += stride) {
    const uint32_t c = i < n ? counts[i] : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, c);
    if (c < nb && (int)(threadIdx.x & 31) == __ffs(peers) - 1) {
      if (local) atomicAdd(&sh[c], (uint32_t)__popc(peers));
      else atomicAdd(&hist[c], (unsigned long long)__popc(peers));
    }
  }
  __syncthreads();
  if (local)
    for (uint32_t j = threadIdx.x; j < nb; j += blockDim.x)
      if (sh[j]) atomicAdd(&hist[j], (unsigned long long)sh[j]);
}

// Histogram of at most kLaneHistBuckets buckets: every lane owns a column of
// the shared histogram (bucket * 32 + lane), so its adds never conflict with
// another lane of its warp; the 32 columns are summed at the end.
constexpr uint32_t kLaneHistBuckets = 256;
__global__ void __launch_bounds__(kOpsThreads) k_count_hist_lanes(const uint32_t* __restrict__ counts,
                                                                  uint64_t n, uint32_t nb,
                                                                  unsigned long long* __restrict__ hist) {
  __shared__ uint32_t sh[kLaneHistBuckets * 32];
  for (uint32_t j = threadIdx.x; j < nb * 32; j += blockDim.x) sh[j] = 0;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {  // four loads in flight
    const uint32_t c0 = counts[i], c1 = counts[i + stride], c2 = counts[i + 2 * stride],
                   c3 = counts[i + 3 * stride];
    if (c0 < nb) atomicAdd(&sh[c0 * 32 + lane], 1u);
    if (c1 < nb) atomicAdd(&sh[c1 * 32 + lane], 1u);
    if (c2 < nb) atomicAdd(&sh[c2 * 32 + lane], 1u);
    if (c3 < nb) atomicAdd(&sh[c3 * 32 + lane], 1u);
  }
  for (; i < n; i += stride) {
    const uint32_t c = counts[i];
    if (c < nb) atomicAdd(&sh[c * 32 + lane], 1u);
  }
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < nb; j += blockDim.x) {
    unsigned long long s = 0;
    for (uint32_t l = 0; l < 32; ++l) s += sh[j * 32 + ((l + j) & 31)];  // rotated: no bank conflict
    if (s) atomicAdd(&hist[j], s);
  }
}

// Stable compaction of the entries with count >= min_count, in chunks of
// kOpsThreads * kPer consecutive entries per block.  Pass 1 counts the kept
// entries per chunk; pass 2 writes them at the chunk's offset.
constexpr int kPer = 16;
constexpr uint64_t kChunk = (uint64_t)kOpsThreads * kPer;

__global__ void __launch_bounds__(kOpsThreads) k_filter_count(const uint32_t* __restrict__ counts,
                                                              uint64_t n, uint32_t min_count,
                                                              uint64_t* __restrict__ kept) {
  __shared__ uint64_t tmp[32];
  const uint64_t c0 = blockIdx.x * kChunk;
  uint64_t mine = 0;
  for (int u = 0; u < kPer; ++u) {
    const uint64_t i = c0 + (uint64_t)u * kOpsThreads + threadIdx.x;  // coalesced
    if (i < n && counts[i] >= min_count) ++mine;
  }
  uint64_t total;
  block_excl_scan<uint64_t>(mine, tmp, &total);
  if (threadIdx.x == 0) kept[blockIdx.x] = total;
}

// exclusive scan of the chunk counts in place, by one block; *total = their sum
__global__ void __launch_bounds__(1024) k_exclusive_scan_block(uint64_t* v, uint64_t n, uint64_t* total) {
  __shared__ uint64_t tmp[32];
  const uint64_t t = dev::block_scan_array<uint64_t>(v, (int)n, tmp);
  if (threadIdx.x == 0) *total = t;
}

// Rounds of 256 consecutive entries: a warp ballot orders the kept entries
// of each 32, a scan over the eight warps orders the round.
__global__ void __launch_bounds__(kOpsThreads) k_filter_write(const uint64_t* __restrict__ kmers,
                                                              const uint32_t* __restrict__ counts,
                                                              uint64_t n, uint32_t min_count,
                                                              const uint64_t* __restrict__ base,
                                                              uint64_t* __restrict__ out_k,
                                                              uint32_t* __restrict__ out_c) {
  __shared__ uint32_t wsum[kOpsThreads / 32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t c0 = blockIdx.x * kChunk;
  uint64_t pos = base[blockIdx.x];
  for (int u = 0; u < kPer; ++u) {
    const uint64_t i = c0 + (uint64_t)u * kOpsThreads + threadIdx.x;
    const bool keep = i < n && counts[i] >= min_count;
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, keep);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, round = 0;
#pragma unroll
    for (int w = 0; w < kOpsThreads / 32; ++w) {
      before += (w < (int)warp) ? wsum[w] : 0u;
      round += wsum[w];
    }
    if (keep) {
      const uint64_t o = pos + before + __popc(bal & ((1u << lane) - 1u));
      out_k[o] = kmers[i];
      out_c[o] = counts[i];
    }
    pos += round;
    __syncthreads();
  }
}

// counts of query k-mers in an ascending table (binary search; 0 if absent)
__global__ void __launch_bounds__(kOpsThreads) k_lookup(const uint64_t* __restrict__ kmers,
                                                        const uint32_t* __restrict__ counts,
                                                        uint64_t n, const uint64_t* __restrict__ q,
                                                        uint64_t nq, uint32_t* __restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t key = q[i];
    uint64_t lo = 0, hi = n;  // first entry >= key
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (kmers[mid] < key) lo = mid + 1; else hi = mid;
    }
    out[i] = (lo < n && kmers[lo] == key) ? counts[lo] : 0u;
  }
}

// *sum += sum of counts
__global__ void __launch_bounds__(kOpsThreads) k_sum_counts(const uint32_t* __restrict__ counts,
                                                            uint64_t n,
                                                            unsigned long long* __restrict__ sum) {
  __shared__ unsigned long long tmp[32];
  unsigned long long mine = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    mine += counts[i];
  unsigned long long total;
  block_excl_scan<unsigned long long>(mine, tmp, &total);
  if (threadIdx.x == 0 && total) atomicAdd(sum, total);
}

// packed 12-byte (u64 k-mer, u32 count) records
__global__ void __launch_bounds__(kOpsThreads) k_pack_pairs(const uint64_t* __restrict__ kmers,
                                                            const uint32_t* __restrict__ counts,
                                                            uint64_t n, uint8_t* __restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t* w = reinterpret_cast<uint32_t*>(out + 12 * i);  // 4-byte aligned
    const uint64_t k = kmers[i];
    w[0] = (uint32_t)k;
    w[1] = (uint32_t)(k >> 32);
    w[2] = counts[i];
  }
}

uint32_t grid_for(uint64_t n, int sm_count) {
  const uint64_t want = (n + kOpsThreads - 1) / kOpsThreads;
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)sm_count * 8));
}

}  // namespace

// A table the engine handed out: its pointers are device memory or the
// engine's page-locked host pool, both addressable by kernels.
static bool table_ok(const dk_table* t) {
  return t && (t->n == 0 || (t->kmers && t->counts && t->handle));
}

int Engine::table_histogram(const dk_table* t, uint32_t nb, uint64_t* hist, uint32_t* min_bucket) {
  Engine* e = this;
  std::lock_guard<std::mutex> g(mu);
  if (!table_ok(t) || !hist || nb == 0 || nb > (1u << 24)) {
    set_error("invalid histogram arguments");
    return DK_ERR_INVALID_ARG;
  }
  DK_CUDA(cudaSetDevice(device));
  DK_TRY(Arena::ensure(this, aux, (size_t)nb * 8));
  DK_CUDA(cudaMemsetAsync(aux.p, 0, (size_t)nb * 8, stream));
  if (t->n && nb <= kLaneHistBuckets)
    k_count_hist_lanes<<<grid_for(t->n, sm_count), kOpsThreads, 0, stream>>>(
        t->counts, t->n, nb, (unsigned long long*)aux.p);
  else if (t->n)
    k_count_hist<<<grid_for(t->n, sm_count), kOpsThreads, 0, stream>>>(
        t->counts, t->n, nb, (unsigned long long*)aux.p);
  DK_CUDA(cudaGetLastError());
  DK_TRY(sync_read(aux.p, (size_t)nb * 8, hist));
  // the cut-off bucket: the first minimum of hist[1 .. nb-1] (0 when nb == 1),
  // as std::min_element over those buckets picks it
  if (min_bucket) {
    uint32_t best = nb > 1 ? 1 : 0;
    for (uint32_t c = 2; c < nb; ++c)
      if (hist[c] < hist[best]) best = c;
    *min_bucket = best;
  }
  return DK_OK;
}

int Engine::table_filter(const dk_table* t, uint32_t min_count, dk_table* out) {
  Engine* e = this;
  std::lock_guard<std::mutex> g(mu);
  if (!table_ok(t) || !out) {
    set_error("invalid filter arguments");
    return DK_ERR_INVALID_ARG;
  }
  std::memset(out, 0, sizeof(*out));
  DK_CUDA(cudaSetDevice(device));
  const uint64_t n = t->n;
  const uint64_t chunks = (n + kChunk - 1) / kChunk;
  DK_TRY(Arena::ensure(this, aux, (chunks + 2) * 8));
  uint64_t* kept = (uint64_t*)aux.p;
  uint64_t total = 0;
  if (n) {
    k_filter_count<<<(uint32_t)chunks, kOpsThreads, 0, stream>>>(t->counts, n, min_count, kept);
    k_exclusive_scan_block<<<1, 1024, 0, stream>>>(kept, chunks, kept + chunks);
    DK_CUDA(cudaGetLastError());
    DK_TRY(sync_read(kept + chunks, 8, &total));
  }
  TableBuf* tb = nullptr;
  DK_TRY(acquire_table(std::max<uint64_t>(total, 1), t->on_device != 0, &tb));
  // the kept entries and their occurrences; on failure the new table goes
  // back to its pool and *out stays empty
  auto fill = [&]() -> int {
    if (total) {
      k_filter_write<<<(uint32_t)chunks, kOpsThreads, 0, stream>>>(
          t->kmers, t->counts, n, min_count, kept, (uint64_t*)tb->k, (uint32_t*)tb->c);
      DK_CUDA(cudaGetLastError());
    }
    DK_CUDA(cudaStreamSynchronize(stream));
    if (total) {
      // occurrences of the kept k-mers = the sum of their counts
      DK_TRY(Arena::ensure(this, aux, (chunks + 2) * 8 + 8));
      uint64_t* sum = (uint64_t*)aux.p + chunks + 1;
      DK_CUDA(cudaMemsetAsync(sum, 0, 8, stream));
      k_sum_counts<<<grid_for(total, sm_count), kOpsThreads, 0, stream>>>(
          (const uint32_t*)tb->c, total, (unsigned long long*)sum);
      DK_CUDA(cudaGetLastError());
      DK_TRY(sync_read(sum, 8, &out->n_kmers));
    }
    return DK_OK;
  };
  const int rc = fill();
  if (rc != DK_OK) {
    release_table(tb->id);
    std::memset(out, 0, sizeof(*out));
    return rc;
  }
  out->kmers = (uint64_t*)tb->k;
  out->counts = (uint32_t*)tb->c;
  out->n = total;
  out->on_device = t->on_device;
  out->variant_used = t->variant_used;
  out->handle = tb->id;
  return DK_OK;
}

int Engine::table_lookup(const dk_table* t, const uint64_t* q, uint64_t nq, uint32_t* counts) {
  Engine* e = this;
  std::lock_guard<std::mutex> g(mu);
  if (!table_ok(t) || (nq && (!q || !counts))) {
    set_error("invalid lookup arguments");
    return DK_ERR_INVALID_ARG;
  }
  if (!nq) return DK_OK;
  DK_CUDA(cudaSetDevice(device));
  DK_TRY(Arena::ensure(this, aux, (size_t)nq * 12 + 16));
  uint64_t* dq = (uint64_t*)aux.p;
  uint32_t* dout = (uint32_t*)(dq + nq);
  DK_CUDA(cudaMemcpyAsync(dq, q, nq * 8, cudaMemcpyHostToDevice, stream));
  k_lookup<<<grid_for(nq, sm_count), kOpsThreads, 0, stream>>>(t->kmers, t->counts, t->n, dq, nq,
                                                                 dout);
  DK_CUDA(cudaGetLastError());
  DK_CUDA(cudaMemcpyAsync(counts, dout, nq * 4, cudaMemcpyDeviceToHost, stream));
  DK_CUDA(cudaStreamSynchronize(stream));
  return DK_OK;
}

int Engine::table_pairs(const dk_table* t, void* out) {
  Engine* e = this;
  std::lock_guard<std::mutex> g(mu);
  if (!table_ok(t) || (t->n && !out)) {
    set_error("invalid pair-export arguments");
    return DK_ERR_INVALID_ARG;
  }
  if (!t->n) return DK_OK;
  if (reinterpret_cast<uintptr_t>(out) & 3) {
    set_error("the record buffer must be 4-byte aligned");
    return DK_ERR_INVALID_ARG;
  }
  DK_CUDA(cudaSetDevice(device));
  cudaPointerAttributes at;
  const bool addressable = cudaPointerGetAttributes(&at, out) == cudaSuccess &&
                           (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeHost ||
                            at.type == cudaMemoryTypeManaged);
  cudaGetLastError();
  const uint64_t bytes = t->n * 12;
  uint8_t* dst = (uint8_t*)out;
  if (!addressable) {  // pageable host buffer: pack in device memory, then copy
    DK_TRY(Arena::ensure(this, aux, bytes));
    dst = (uint8_t*)aux.p;
  }
  k_pack_pairs<<<grid_for(t->n, sm_count), kOpsThreads, 0, stream>>>(t->kmers, t->counts, t->n, dst);
  DK_CUDA(cudaGetLastError());
  if (!addressable) DK_CUDA(cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, stream));
  DK_CUDA(cudaStreamSynchronize(stream));
  return DK_OK;
}

Engine* engine_of(dk_ctx* ctx);

}  // namespace dk

extern "C" {

int dk_table_histogram(dk_ctx* ctx, const dk_table* t, uint32_t num_buckets, uint64_t* hist,
                       uint32_t* min_bucket) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  return dk::engine_of(ctx)->table_histogram(t, num_buckets, hist, min_bucket);
}

int dk_table_filter(dk_ctx* ctx, const dk_table* t, uint32_t min_count, dk_table* out) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  return dk::engine_of(ctx)->table_filter(t, min_count, out);
}

int dk_table_lookup(dk_ctx* ctx, const dk_table* t, const uint64_t* queries, uint64_t n,
                    uint32_t* counts) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  return dk::engine_of(ctx)->table_lookup(t, queries, n, counts);
}

int dk_table_pairs(dk_ctx* ctx, const dk_table* t, void* out) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  return dk::engine_of(ctx)->table_pairs(t, out);
}

}  // extern "C"
