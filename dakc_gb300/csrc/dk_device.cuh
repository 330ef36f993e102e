// Device helpers shared by the engine kernels (warp-per-line k-mer
// extraction, block scans, shared-memory bitonic sort).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dk {
namespace dev {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }

// Code of one text byte.
// DAKC (conv 0): C=0 A=1 T=2 G=3 (either case), M/m=0xF0 (ends the line),
//   anything else 0xFF (splits the run) -- char2base, dakc/src/common/common.hpp:72-92.
// PakMan* (conv 1): (byte >> 1) & 7 for every byte (A=0 C=1 T=2 G=3; other
//   bytes give 4..7 and are OR'ed into the window as PakMan* does,
//   char_to_el / kmer_shift, pakman_star/includes/distribute_kmers.h), and
//   '\n' (the end of a read) = 0xF0.
__device__ __forceinline__ void init_lut(uint8_t* lut, int conv = 0) {
  for (int c = threadIdx.x; c < 256; c += blockDim.x) {
    uint8_t v = 0xFF;
    if (conv == 1) {
      v = c == '\n' ? 0xF0 : (uint8_t)((c >> 1) & 7);
    } else {
      const int u = c | 0x20;  // exact case fold for the five letters below
      if (u == 'c') v = 0;
      else if (u == 'a') v = 1;
      else if (u == 't') v = 2;
      else if (u == 'g') v = 3;
      else if (u == 'm') v = 0xF0;
    }
    lut[c] = v;
  }
}

// Walk one line with one warp.  Lane i owns positions seg + i*C .. seg + i*C + C-1.
// f(t, key, valid) is called for t = 0..C-1 (once per segment of 32*C positions).
// CONV 0: DAKC's rules (codes 0-3, 0xFF splits the run, 0xF0 ends the line).
// CONV 1: PakMan*'s (kmer = ((kmer << 2) | code) & mask with 3-bit codes,
// Sliding_window, pakman_star/src/kmer_counting.cpp:313-341): nothing splits
// a run, '\n' (0xF0) ends the read, and a k-mer ends at every position from
// the k-th.  A code's bit 2 lands on bit 0 of the slot before it, so the key
// is the 2-bit window of the codes' low bits OR'ed with a second window of
// their bit 2, one slot up; both windows are carried across lanes alike.
template <int C, int CONV = 0, typename F>
__device__ __forceinline__ void warp_line_kmers(const uint8_t* __restrict__ line, int W, int k,
                                                uint64_t kmask, const uint8_t* __restrict__ lut,
                                                F&& f) {
  const uint32_t lane = lane_id();
  constexpr int B = 2 * C;  // bits per lane chunk
  uint64_t carry_win = 0, carry_sp = 0;
  int carry_lb = -1;
  int carry_stop = W;
  // k = 1 keeps a final run only if it starts before W-1 (kcounter_funcs.cpp:97)
  const bool k1_drop_last = CONV == 0 && (k == 1) && (W == 1 || lut[line[W - 2]] == 0xFF);
  for (int seg = 0; seg < W; seg += 32 * C) {
    const int p0 = seg + (int)lane * C;
    uint64_t chunk = 0, spill = 0;
    int lb_lane = -1, firstM = 0x7FFFFFFF;
    uint32_t bad_mask = 0;  // bit t: position p0+t is not a base
#pragma unroll
    for (int t = 0; t < C; ++t) {
      const int p = p0 + t;
      if (CONV == 0) {
        uint8_t c = 0xFF;
        if (p < W) c = lut[line[p]];  // shared-memory tile or global line
        chunk = (chunk << 2) | (c & 3u);
        if (c >= 4) { lb_lane = p; bad_mask |= (1u << t); }
        if (c == 0xF0 && firstM == 0x7FFFFFFF) firstM = p;
      } else {
        const uint32_t c = p < W ? lut[line[p]] : 0u;  // past the line: never a key's
        const bool end = c == 0xF0u;
        chunk = (chunk << 2) | (end ? 0u : (c & 3u));
        spill = (spill << 2) | (end ? 0u : (c >> 2));
        if (end && firstM == 0x7FFFFFFF) firstM = p;
      }
    }
    // first 'M' over the warp
    int m = firstM;
#pragma unroll
    for (int o = 16; o; o >>= 1) m = min(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    const int stop = min(carry_stop, m);
    // last non-base position before this lane's chunk (exclusive max scan)
    int lb_inc = lb_lane;
    if (CONV == 0) {
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xFFFFFFFFu, lb_inc, o);
        if ((int)lane >= o) lb_inc = max(lb_inc, v);
      }
    }
    int lb_exc = -1;
    if (CONV == 0) {
      lb_exc = __shfl_up_sync(0xFFFFFFFFu, lb_inc, 1);
      if (lane == 0) lb_exc = -1;
      lb_exc = max(lb_exc, carry_lb);
    }
    // 2-bit window of all bases before this lane's chunk (exclusive shift-or scan)
    uint64_t w_inc = chunk, s_inc = spill;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t v = __shfl_up_sync(0xFFFFFFFFu, w_inc, o);
      if ((int)lane >= o && B * o < 64) w_inc |= v << (B * o);
      if (CONV != 0) {
        const uint64_t sv = __shfl_up_sync(0xFFFFFFFFu, s_inc, o);
        if ((int)lane >= o && B * o < 64) s_inc |= sv << (B * o);
      }
    }
    uint64_t w_exc = __shfl_up_sync(0xFFFFFFFFu, w_inc, 1);
    if (lane == 0) w_exc = 0;
    if (B * (int)lane < 64) w_exc |= carry_win << (B * lane);
    uint64_t s_exc = 0;
    if (CONV != 0) {
      s_exc = __shfl_up_sync(0xFFFFFFFFu, s_inc, 1);
      if (lane == 0) s_exc = 0;
      if (B * (int)lane < 64) s_exc |= carry_sp << (B * lane);
    }
    // k-mers ending at each of this lane's positions
    int lb = lb_exc;
#pragma unroll
    for (int t = 0; t < C; ++t) {
      const int p = p0 + t;
      if (CONV == 0 && (bad_mask & (1u << t))) lb = p;
      const int up = 2 * (t + 1);
      uint64_t win = (up < 64 ? (w_exc << up) : 0ull) | (chunk >> (2 * (C - 1 - t)));
      if (CONV != 0)
        win |= ((up < 64 ? (s_exc << up) : 0ull) | (spill >> (2 * (C - 1 - t)))) << 2;
      const uint64_t key = win & kmask;
      bool valid = (p < stop) && (p - lb >= k);
      if (k1_drop_last && p == W - 1) valid = false;
      f(t, key, valid);
    }
    // carry to the next segment
    const uint64_t win_all = __shfl_sync(0xFFFFFFFFu, w_inc, 31);
    carry_win = (B * 32 < 64) ? ((carry_win << (B * 32)) | win_all) : win_all;
    if (CONV != 0) {
      const uint64_t sp_all = __shfl_sync(0xFFFFFFFFu, s_inc, 31);
      carry_sp = (B * 32 < 64) ? ((carry_sp << (B * 32)) | sp_all) : sp_all;
    }
    if (CONV == 0) carry_lb = max(carry_lb, __shfl_sync(0xFFFFFFFFu, lb_inc, 31));
    carry_stop = stop;
  }
}

// block-wide exclusive scan of one value per thread; returns exclusive prefix,
// *total receives the block sum.  `tmp` needs 32 slots.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* tmp, T* total) {
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if ((int)lane >= o) x += y;
  }
  if (lane == 31) tmp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = (lane < nw) ? tmp[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if ((int)lane >= o) w += y;
    }
    if (lane < nw) tmp[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  const T warp_base = warp ? tmp[warp - 1] : T(0);
  if (total) *total = tmp[nw - 1];
  __syncthreads();
  return warp_base + x - v;
}

// exclusive scan of arr[0..len) in shared memory by the whole block; returns the total
template <typename T>
__device__ T block_scan_array(T* arr, int len, T* tmp) {
  const int per = (len + blockDim.x - 1) / blockDim.x;
  const int lo = min(len, (int)threadIdx.x * per), hi = min(len, lo + per);
  T s = 0;
  for (int i = lo; i < hi; ++i) s += arr[i];
  T total;
  T base = block_excl_scan<T>(s, tmp, &total);
  for (int i = lo; i < hi; ++i) { const T c = arr[i]; arr[i] = base; base += c; }
  __syncthreads();
  return total;
}

__device__ __forceinline__ void lines_of_block(uint64_t n_lines, uint64_t* lo, uint64_t* hi) {
  *lo = n_lines * blockIdx.x / gridDim.x;
  *hi = n_lines * (blockIdx.x + 1) / gridDim.x;
}

__device__ __forceinline__ int ceil_log2_u64(uint64_t x) { return x <= 1 ? 0 : 64 - __clzll(x - 1); }

// sort skeys[lo, lo+m) ascending with the whole block (always-ascending
// bitonic network; out-of-range partners act as +inf and never move)
__device__ inline void block_bitonic(unsigned long long* s, uint32_t m) {
  int lg = 0;
  while ((1u << lg) < m) ++lg;
  const uint32_t P = 1u << lg;
  for (int sz = 1; sz <= lg; ++sz) {  // merge blocks of 2^sz
    const uint32_t hmask = (1u << (sz - 1)) - 1;
    for (uint32_t i = threadIdx.x; i < P / 2; i += blockDim.x) {
      const uint32_t a = ((i >> (sz - 1)) << sz) | (i & hmask);
      const uint32_t b = a ^ ((1u << sz) - 1);
      if (b < m) {
        const unsigned long long x = s[a], y = s[b];
        if (y < x) { s[a] = y; s[b] = x; }
      }
    }
    __syncthreads();
    for (int st = sz - 2; st >= 0; --st) {
      const uint32_t smask = (1u << st) - 1;
      for (uint32_t i = threadIdx.x; i < P / 2; i += blockDim.x) {
        const uint32_t a = ((i >> st) << (st + 1)) | (i & smask);
        const uint32_t b = a + (1u << st);
        if (b < m) {
          const unsigned long long x = s[a], y = s[b];
          if (y < x) { s[a] = y; s[b] = x; }
        }
      }
      __syncthreads();
    }
  }
}

// ------------------------------------------------ TMA bulk copy + mbarrier
// Asynchronous L2 prefetch of the 16-byte-aligned interior of [p, p + bytes):
// no shared memory, no completion to wait for.
__device__ __forceinline__ void prefetch_l2_range(const void* p, uint64_t bytes) {
  const uint64_t a = (reinterpret_cast<uint64_t>(p) + 15) & ~15ull;
  const uint64_t e = (reinterpret_cast<uint64_t>(p) + bytes) & ~15ull;
  for (uint64_t x = a; x < e; x += (1u << 20)) {  // pieces of at most 1 MB
    const uint32_t n = (uint32_t)min(e - x, (uint64_t)(1u << 20));
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(x), "r"(n) : "memory");
  }
}

// 1-D bulk copies (cp.async.bulk) global -> shared, completed on an mbarrier.
// Addresses must be 16-byte aligned and sizes multiples of 16.

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

// make initialised barriers visible to the async (TMA) proxy
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for phase `parity` of `bar` for at most `limit_ns`; false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint64_t limit_ns = 2000000000ull) {
  if (mbar_test(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_test(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}

// Stage bytes [src, src+len) of global memory into shared memory at dst16
// (16-byte aligned, at least len + 32 bytes).  The bulk copy covers the
// 16-byte-aligned middle; bytes that a whole-16-byte copy would take beyond
// `limit` (end of the readable global buffer) are loaded by plain loads after
// the wait.  Returns the offset in dst16 where src's first byte lands.  Call
// with the whole block; one thread issues the copy.
struct StagedCopy {
  uint32_t lead;     // dst16 + lead == copy of src
  uint32_t bulk;     // bytes moved by the bulk copy
  const uint8_t* tail_src;
  uint32_t tail_dst;  // offset in dst16
  uint32_t tail_len;
};

__device__ __forceinline__ StagedCopy plan_stage(const uint8_t* src, uint64_t len,
                                                 const uint8_t* limit) {
  StagedCopy c;
  const uintptr_t s = reinterpret_cast<uintptr_t>(src);
  const uintptr_t a = s & ~uintptr_t(15);
  c.lead = static_cast<uint32_t>(s - a);
  const uintptr_t want_end = (s + len + 15) & ~uintptr_t(15);
  const uintptr_t lim = reinterpret_cast<uintptr_t>(limit) & ~uintptr_t(15);
  const uintptr_t bulk_end = want_end <= reinterpret_cast<uintptr_t>(limit) ? want_end
                                                                            : (lim > a ? lim : a);
  c.bulk = static_cast<uint32_t>(bulk_end - a);
  const uintptr_t need_end = s + len;
  c.tail_src = reinterpret_cast<const uint8_t*>(bulk_end);
  c.tail_dst = c.bulk;
  c.tail_len = need_end > bulk_end ? static_cast<uint32_t>(need_end - bulk_end) : 0u;
  return c;
}

}  // namespace dev
}  // namespace dk
