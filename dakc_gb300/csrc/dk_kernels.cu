// sm_103a kernels of the k-mer counting engine (integer-only, HBM-bound).
//
// Pipeline (one read set):
//   l1_count    text -> k-mers -> per-CTA histogram of level-1 buckets
//               (bucket = top B1 bits of the k-mer; B1 <= 12)
//   l1_scan     per-(bucket, CTA) write offsets; level-1 nodes
//   l1_scatter  text -> k-mers again -> keys written bucket-contiguously
//               (replaces DAKC's owner hash + actor send: the scatter IS the
//               all-to-all, kcounter.cpp:146-245,287-299)
//   classify / tile_hist / node_scan / tile_scatter
//               MSD partition of nodes still larger than a bin by the next
//               8 bits (deterministic: per-tile histograms, no global atomics
//               on key positions)
//   bin_count   per final node: shared-memory counting sort on 12 more bits,
//               then insertion / bitonic sort of each digit range and a
//               run-length reduce (replaces ska_sort + the run-length loop of
//               kcounter.cpp:385-414); nodes with <= 12 free bits are counted
//               densely (a histogram IS the sorted run-length table)
//   aggregate / offsets / compact
//               distinct counts up the tree, output offsets down the tree,
//               staged pairs copied to the final table
//
// k-mer extraction (read_till_buf_max + get_kmers, kcounter_funcs.cpp:25-111)
// runs one warp per line: each lane decodes C consecutive bytes, and warp
// scans carry the 2-bit window (shift-or), the last break position (max) and
// the first 'M' (min) across lanes, so every k-mer is formed in registers.
#include "dk_internal.cuh"
#include "dk_device.cuh"
#include <algorithm>
#include <cstdio>
#include <vector>

namespace dk {

namespace {

using namespace dev;

// Optional bounds self-checks (build with -DDK_BOUNDS_CHECK): a failed check
// records (code, detail) in g_check and skips the access.
#ifdef DK_BOUNDS_CHECK
__device__ unsigned long long g_check[4];
#define DK_OK_IDX(cond, code, detail)                                                  \
  ((cond) ? true                                                                       \
          : (atomicCAS(&g_check[0], 0ull, (unsigned long long)(code)) == 0ull          \
                 ? (g_check[1] = (unsigned long long)(detail), false)                  \
                 : false))
#else
#define DK_OK_IDX(cond, code, detail) true
#endif

// Optional per-phase cycle counters for the bin kernel (build with
// -DDK_PHASE_TIMING; read them with dk_debug_phases).  Compiled out otherwise.
#ifdef DK_PHASE_TIMING
__device__ unsigned long long g_phase[32];
#define DK_PHASE_BEGIN() unsigned long long _ph_t = clock64()
#define DK_PHASE(k)                                                    \
  do {                                                                 \
    __syncthreads();                                                   \
    if (threadIdx.x == 0) {                                            \
      const unsigned long long _u = clock64();                         \
      atomicAdd(&g_phase[k], _u - _ph_t);                              \
      _ph_t = _u;                                                      \
    }                                                                  \
  } while (0)
#define DK_PHASE_ADD(k, v) do { if (threadIdx.x == 0) atomicAdd(&g_phase[k], (unsigned long long)(v)); } while (0)
#define DK_WARP_ADD(k, v) do { if ((threadIdx.x & 31) == 0) atomicAdd(&g_phase[k], (unsigned long long)(v)); } while (0)
#else
#define DK_WARP_ADD(k, v) do {} while (0)
#define DK_PHASE_BEGIN() do {} while (0)
#define DK_PHASE(k) do {} while (0)
#define DK_PHASE_ADD(k, v) do {} while (0)
#endif


// ------------------------------------------------------------- level 1
// Text tiles of a CTA's line range, staged into shared memory by 1-D TMA bulk
// copies (double-buffered: tile t+1 streams in while tile t is parsed).
struct TextTiles {
  const uint8_t* text;
  uint64_t nbytes, stride, lo, hi;
  uint32_t lt;  // lines per tile
  uint8_t* buf0;  // tile buffers (even / odd tiles); two members, not an array,
  uint8_t* buf1;  // so that the struct stays in registers
  __device__ __forceinline__ uint8_t* bufof(uint32_t t) const { return (t & 1) ? buf1 : buf0; }
  uint64_t* bar;  // 2 mbarriers

  __device__ __forceinline__ uint32_t ntiles() const { return (uint32_t)((hi - lo + lt - 1) / lt); }
  __device__ __forceinline__ void range(uint32_t t, uint64_t* l0, uint64_t* l1) const {
    *l0 = lo + (uint64_t)t * lt;
    *l1 = min(hi, *l0 + lt);
  }
  __device__ __forceinline__ StagedCopy plan(uint32_t t) const {
    uint64_t l0, l1;
    range(t, &l0, &l1);
    const uint64_t b0 = l0 * stride, b1 = min(l1 * stride, nbytes);
    return plan_stage(text + b0, b1 - b0, text + nbytes);
  }
  // one thread: start the copy of tile t into buffer t&1
  __device__ __forceinline__ void issue(uint32_t t) const {
    uint64_t l0, l1;
    range(t, &l0, &l1);
    const StagedCopy c = plan(t);
    uint64_t* b = &bar[t & 1];
    fence_barrier_init();  // order earlier generic writes of the buffer before the async copy
    mbar_arrive_expect_tx(b, c.bulk);
    if (c.bulk) tma_load_1d(bufof(t), text + l0 * stride - c.lead, c.bulk, b);
  }
  // whole block: wait for tile t, fetch its unaligned tail, return its first
  // line in shared memory (nullptr, with *err set, when the copy timed out)
  __device__ __forceinline__ const uint8_t* acquire(uint32_t t, unsigned long long* err) const {
    const StagedCopy c = plan(t);
    const bool ok = mbar_wait_bounded(&bar[t & 1], (t >> 1) & 1);
    for (uint32_t i = threadIdx.x; i < c.tail_len; i += blockDim.x)
      bufof(t)[c.tail_dst + i] = c.tail_src[i];
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicMax(err, 1ull);
      return nullptr;
    }
    return bufof(t) + c.lead;
  }
  // after a timeout: bounded wait for a copy still in flight into our smem
  __device__ __forceinline__ void drain(uint32_t t_next) const {
    if (threadIdx.x == 0 && t_next < ntiles()) mbar_wait_bounded(&bar[t_next & 1], (t_next >> 1) & 1);
    __syncthreads();
  }
};

__host__ __device__ inline uint32_t tile_buf_bytes(uint32_t lt, uint64_t stride) {
  return (uint32_t)(((uint64_t)lt * stride + 32 + 127) & ~127ull);
}

// level-1 bucket rule of one job in batch mode: bucket = base + (key >> shift),
// shift = 64 (no split) when the job has a single bucket
struct JobBucket {
  uint32_t base = 0;
  uint32_t shift = 64;
  JobBucket() = default;
  __device__ __forceinline__ JobBucket(const ExtractArgs& a, uint32_t job) {
    const uint32_t bits = __ldg(a.job_bits + job);
    base = __ldg(a.job_base + job);
    shift = bits ? 2u * (uint32_t)a.k - bits : 64u;
  }
  __device__ __forceinline__ uint32_t operator()(uint64_t key) const {
    return base + (shift < 64 ? (uint32_t)(key >> shift) : 0u);
  }
};

// job that owns line l in batch mode: binary search over job_start within
// jobs [lo, hi) (the whole set by default)
__device__ __forceinline__ uint32_t job_of_line(const ExtractArgs& a, uint64_t l, uint32_t lo = 0,
                                                uint32_t hi = 0xFFFFFFFFu) {
  hi = min(hi, (uint32_t)a.njobs);
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(a.job_start + mid) <= l) lo = mid; else hi = mid;
  }
  return lo;
}

// jobs owning the first and last line of a tile [l0, l1) (batch mode): the
// tile's lines search only between them.  Call with the whole block.
__device__ __forceinline__ void tile_jobs(const ExtractArgs& a, uint64_t l0, uint64_t l1,
                                          uint32_t* s_jobs) {
  if (a.njobs) {
    if (threadIdx.x == 0) s_jobs[0] = job_of_line(a, l0);
    if (threadIdx.x == 32) s_jobs[1] = job_of_line(a, l1 - 1) + 1;
  }
  __syncthreads();
}

// counters[0] = k-mers, [1] = n_lines - (first NUL-led line), [3] = device error.
// CONV: the k-mer convention (0 DAKC, 1 PakMan*), a kernel of its own each.
template <int C, int CONV>
__global__ void __launch_bounds__(512) k_l1_count(ExtractArgs a, uint32_t* __restrict__ H,
                                                  unsigned long long* __restrict__ counters,
                                                  uint32_t lt) {
  extern __shared__ __align__(128) uint8_t smraw[];
  const uint64_t stride = (uint64_t)a.W + 1;
  const uint32_t bb = tile_buf_bytes(lt, stride);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  uint8_t* tb = smraw + 128;
  uint32_t* hist = reinterpret_cast<uint32_t*>(tb + 2 * bb);
  uint8_t* lut = reinterpret_cast<uint8_t*>(hist + a.F1);
  TextTiles T;
  T.text = a.text;
  T.nbytes = a.nbytes;
  T.stride = stride;
  lines_of_block(a.n_lines, &T.lo, &T.hi);
  T.lt = lt;
  T.buf0 = tb;
  T.buf1 = tb + bb;
  T.bar = bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
  }
  for (int b = threadIdx.x; b < a.F1; b += blockDim.x) hist[b] = 0;
  init_lut(lut, a.conv);
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint32_t nt = T.ntiles();
  uint32_t mine = 0;
  if (threadIdx.x == 0 && nt) T.issue(0);
  for (uint32_t t = 0; t < nt; ++t) {
    if (threadIdx.x == 0 && t + 1 < nt) T.issue(t + 1);
    const uint8_t* base = T.acquire(t, &counters[3]);
    if (!base) {
      T.drain(t + 1);
      return;
    }
    uint64_t l0, l1;
    T.range(t, &l0, &l1);
    for (uint64_t l = l0 + warp; l < l1; l += nwarps) {
      const uint8_t* line = base + (l - l0) * stride;
      if (a.njobs) {
        const uint32_t job = job_of_line(a, l);
        if (l >= __ldg(a.job_end + job)) continue;  // past the job's first NUL-led line
        if (lane_id() == 0 && l > __ldg(a.job_start + job) && line[0] == 0) {
          atomicMin(&a.job_nul[job], (unsigned long long)l);
          atomicMax(&counters[1], 1ull);
        }
        const JobBucket jb(a, job);
        auto on_kmer = [&](int, uint64_t key, bool valid) {
          if (valid) { atomicAdd(&hist[jb(key)], 1u); ++mine; }
        };
        warp_line_kmers<C, CONV>(line, a.W, a.k, a.kmask, lut, on_kmer);
        continue;
      }
      if (lane_id() == 0 && a.line_base + l > 0 && line[0] == 0)
        atomicMax(&counters[1], a.lines_total - (a.line_base + l));
      auto on_kmer = [&](int, uint64_t key, bool valid) {
        if (valid) { atomicAdd(&hist[key >> a.shift1], 1u); ++mine; }
      };
      warp_line_kmers<C, CONV>(line, a.W, a.k, a.kmask, lut, on_kmer);
    }
    __syncthreads();
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) mine += __shfl_xor_sync(0xFFFFFFFFu, mine, o);
  if (lane_id() == 0 && mine) atomicAdd(&counters[0], (unsigned long long)mine);
  __syncthreads();
  uint32_t* row = H + (size_t)blockIdx.x * a.F1;
  for (int b = threadIdx.x; b < a.F1; b += blockDim.x) row[b] = hist[b];
}

// bucket totals: nodes[b].n = sum_g H[g][b]
__global__ void k_l1_totals(const uint32_t* __restrict__ H, int G, int F1, Node* nodes) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= F1) return;
  uint64_t s = 0;
  for (int g = 0; g < G; ++g) s += H[(size_t)g * F1 + b];
  nodes[b].n = s;
}

// bucket starts (single block): exclusive scan of totals, node init
__global__ void k_l1_starts(Node* nodes, int F1, int shift1, const int16_t* bucket_shift) {
  __shared__ unsigned long long tmp[32];
  const int per = (F1 + blockDim.x - 1) / blockDim.x;
  const int lo = min(F1, (int)threadIdx.x * per), hi = min(F1, lo + per);
  unsigned long long s = 0;
  for (int i = lo; i < hi; ++i) s += nodes[i].n;
  unsigned long long total = 0;
  unsigned long long base = block_excl_scan<unsigned long long>(s, tmp, &total);
  for (int i = lo; i < hi; ++i) {
    Node& nd = nodes[i];
    nd.start = base;
    base += nd.n;
    nd.d = 0;
    nd.out_off = 0;
    nd.first_child = 0;
    nd.shift = bucket_shift ? bucket_shift[i] : (int16_t)shift1;
    nd.buf = 0;
    nd.state = 0;
    nd.tile_base = 0;
    nd.ntiles = 0;
    nd.th_base = 0;
    nd.width = 0;
    // most of all keys and too many for the partition's 32-bit offsets once
    // split: a hot k-mer, counted whole by a big hash bin
    nd.skewed = nd.n * 2 > total && nd.n >= (1ull << 31);
  }
}

// per-(CTA, bucket) absolute write offsets O[g][b]
__global__ void k_l1_offsets_rows(const uint32_t* __restrict__ H, int G, int F1,
                                  const Node* nodes, uint64_t* __restrict__ O) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= F1) return;
  uint64_t run = nodes[b].start;
  for (int g = 0; g < G; ++g) {
    O[(size_t)g * F1 + b] = run;
    run += H[(size_t)g * F1 + b];
  }
}

// one upload chunk's bucket totals T_c[b] = sum_g H_c[g][b]
__global__ void k_chunk_totals(const uint32_t* __restrict__ H, int G, int F1, uint32_t* T) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= F1) return;
  uint32_t s = 0;
  for (int g = 0; g < G; ++g) s += H[(size_t)g * F1 + b];
  T[b] = s;
}

// its bucket starts (single block): its region follows the *running keys of
// the earlier chunks, and *running grows by its own
__global__ void k_chunk_starts(const uint32_t* __restrict__ T, int F1, uint64_t* __restrict__ S,
                               unsigned long long* running) {
  __shared__ unsigned long long tmp[32];
  const unsigned long long before = *running;
  const int per = (F1 + blockDim.x - 1) / blockDim.x;
  const int lo = min(F1, (int)threadIdx.x * per), hi = min(F1, lo + per);
  unsigned long long s = 0;
  for (int i = lo; i < hi; ++i) s += T[i];
  unsigned long long tot;
  // the block scan synchronises: every thread has read *running before it changes
  unsigned long long base = before + block_excl_scan<unsigned long long>(s, tmp, &tot);
  for (int i = lo; i < hi; ++i) {
    S[i] = base;
    base += T[i];
  }
  if (threadIdx.x == 0) *running = before + tot;
}

// its per-(CTA, bucket) write offsets
__global__ void k_chunk_offsets_rows(const uint32_t* __restrict__ H, int G, int F1,
                                     const uint64_t* __restrict__ S, uint64_t* __restrict__ O) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= F1) return;
  uint64_t run = S[b];
  for (int g = 0; g < G; ++g) {
    O[(size_t)g * F1 + b] = run;
    run += H[(size_t)g * F1 + b];
  }
}

// Thread-per-line level-1 passes (lines of at most kLineMaxW bytes).  A tile
// of blockDim.x lines is staged in shared memory (TMA, double-buffered) and
// each thread walks one line, rolling its 2-bit key one base at a time.
// Both passes see the same lines per CTA (lines_of_block) and the same
// buckets, so the scatter fills exactly the ranges the count reserved.

// One line's rolling state.  step() consumes the byte code of position p and
// says whether a k-mer ends there (DAKC's rules: 'M' ends the line, any other
// non-base splits it, and k = 1 keeps a final run only if it starts before
// W-1, kcounter_funcs.cpp:69-111).
// With the PakMan* convention (pak) no byte splits a run: every code is
// OR'ed into the shifted window ((key << 2) | code) and a k-mer ends at every
// position from the k-th on (Sliding_window, pakman_star/src/
// kmer_counting.cpp:313-341).
// Roll modes: DAKC's convention for k >= 2, PakMan*'s convention, and DAKC's
// for k = 1, whose last position follows the reference's last-run rule
// (kcounter_funcs.cpp:102-110) and needs the previous code.  The k >= 2 form
// carries neither that rule nor the previous code through its steps.
enum : int { kRollDakc = 0, kRollPak = 1, kRollDakcK1 = 2 };

__host__ __device__ constexpr int roll_mode(int conv, int k) {
  return conv == 1 ? kRollPak : (k == 1 ? kRollDakcK1 : kRollDakc);
}

struct LineRoll {
  uint64_t key;
  int run;
  uint32_t prev;
  bool stopped;
  __device__ __forceinline__ void reset() { key = 0; run = 0; prev = 0; stopped = false; }
  template <int MODE>
  __device__ __forceinline__ bool step(uint32_t c, int p, int W, int k, uint64_t kmask) {
    if (stopped || c == 0xF0u) { stopped = true; return false; }
    if (MODE == kRollPak) {
      key = ((key << 2) | c) & kmask;
      ++run;
      return run >= k;
    }
    bool emit = false;
    if (c >= 4u) {
      run = 0;
    } else {
      key = ((key << 2) | c) & kmask;
      ++run;
      emit = run >= k;
      if (MODE == kRollDakcK1) emit = emit && !(p == W - 1 && (W == 1 || prev == 0xFFu));
    }
    if (MODE == kRollDakcK1) prev = c;
    return emit;
  }
};

// k-mer windows of a line a chunk of positions at a time (DAKC's convention,
// k >= 2), with no step depending on the one before: the 2-bit codes of the
// 32 positions before the chunk (P) and their break bits (B) carry from chunk
// to chunk; the k-mer ending at chunk position q is a fixed bit field of
// P:C (C: the chunk's codes), and it is counted when no break lies in its
// window (B:Bc smeared over k positions) and no stop came before it.
// Codes: 0-3 bases, 0xFF break, 0xF0 stop (bit 7 marks both; bit 0 tells
// them apart).  Emits exactly what LineRoll::step<kRollDakc> emits.
__device__ __forceinline__ uint32_t pack4_codes(uint32_t w) {  // first code in bits 7..6
  const uint32_t x = w & 0x03030303u;
  return ((x & 3u) << 6) | ((x >> 4) & 0x30u) | ((x >> 14) & 0x0Cu) | (x >> 24);
}
__device__ __forceinline__ uint32_t byte_flags4(uint32_t m) {  // bit 7 of byte u -> bit u
  return ((((m >> 7) & 0x01010101u) * 0x00204081u) >> 21) & 0xFu;
}
struct LineWin {
  uint64_t P;    // codes of positions p0-32 .. p0-1, position p0-1 in bits 1..0
  uint32_t B;    // their break bits, bit i: position p0-32+i (before the line: set)
  bool stopped;  // a stop came before p0
  // pack a chunk of CH codes (cw: byte u of word g is position 4g+u)
  template <int CH>
  __device__ __forceinline__ static void pack(const uint32_t* cw, uint64_t* C, uint32_t* brk,
                                              uint32_t* stp) {
    uint64_t c = 0;
    uint32_t b = 0, t = 0;
#pragma unroll
    for (int g = 0; g < CH / 4; ++g) {
      const uint32_t w = cw[g];
      c |= (uint64_t)pack4_codes(w) << (2 * CH - 8 - 8 * g);
      b |= byte_flags4(w & 0x80808080u) << (4 * g);
      t |= byte_flags4(w & ~(w << 7) & 0x80808080u) << (4 * g);
    }
    *C = c;
    *brk = b;
    *stp = t;
  }
  // the 32 positions before the first chunk (iw: codes of positions
  // p0-32 .. p0-1, breaks before the line)
  __device__ __forceinline__ void init(const uint32_t* iw) {
    uint32_t t;
    pack<32>(iw, &P, &B, &t);
    stopped = t != 0;
  }
  // emit mask of a chunk (bit q: the k-mer ending at p0+q); *M keeps the
  // combined break bits for advance()
  template <int CH>
  __device__ __forceinline__ uint32_t valid(uint32_t brk, uint32_t stp, int k,
                                            uint64_t* M) const {
    const uint64_t m = ((uint64_t)brk << 32) | B;
    uint64_t sm = m;  // bit i: a break among positions i-k+1 .. i
    int w = 1;
    while (2 * w <= k) {
      sm |= sm << w;
      w <<= 1;
    }
    if (w < k) sm |= sm << (k - w);
    uint32_t v = ~(uint32_t)(sm >> 32);
    if (CH < 32) v &= (1u << (CH & 31)) - 1u;  // (CH & 31: no shift by 32 in the dead branch)
    if (stopped) v = 0;
    if (stp) v &= (1u << (__ffs(stp) - 1)) - 1u;
    *M = m;
    return v;
  }
  template <int CH>
  __device__ __forceinline__ uint64_t key(uint64_t C, int q, uint64_t kmask) const {
    const int s = 2 * (CH - 1 - q);  // a constant once q's loop is unrolled
    const uint64_t lo = CH == 32 ? C : ((P << (2 * CH)) | C);
    const uint64_t hi = CH == 32 ? P : (P >> (64 - 2 * CH));
    const uint64_t x = s == 0 ? lo : ((lo >> s) | (hi << (64 - s)));
    return x & kmask;
  }
  template <int CH>
  __device__ __forceinline__ void advance(uint64_t C, uint64_t M, uint32_t stp) {
    P = CH == 32 ? C : ((P << (2 * CH)) | C);
    B = (uint32_t)(M >> CH);
    stopped = stopped || stp != 0;
  }
};

// Per-line prologue of a tile: is line l parsed, and its bucket rule (batch
// mode); records NUL-led lines.
__device__ __forceinline__ bool line_prologue(const ExtractArgs& a, uint64_t l, uint64_t l1,
                                              const uint8_t* line, JobBucket* jb,
                                              unsigned long long* counters,
                                              const uint32_t* s_jobs) {
  if (l >= l1) return false;
  if (a.njobs) {
    const uint32_t job = job_of_line(a, l, s_jobs[0], s_jobs[1]);
    if (l >= __ldg(a.job_end + job)) return false;  // past the job's first NUL-led line
    if (l > __ldg(a.job_start + job) && line[0] == 0) {
      atomicMin(&a.job_nul[job], (unsigned long long)l);
      atomicMax(&counters[1], 1ull);
    }
    *jb = JobBucket(a, job);
  } else if (a.line_base + l > 0 && line[0] == 0) {
    atomicMax(&counters[1], a.lines_total - (a.line_base + l));
  }
  return true;
}

__device__ __forceinline__ void setup_tiles(TextTiles* T, const ExtractArgs& a, uint8_t* smraw,
                                            uint32_t bb) {
  T->text = a.text;
  T->nbytes = a.nbytes;
  T->stride = (uint64_t)a.W + 1;
  lines_of_block(a.n_lines, &T->lo, &T->hi);
  T->lt = blockDim.x;
  T->bar = reinterpret_cast<uint64_t*>(smraw);
  T->buf0 = smraw + 128;
  T->buf1 = smraw + 128 + bb;
  if (threadIdx.x == 0) {
    mbar_init(&T->bar[0], 1);
    mbar_init(&T->bar[1], 1);
    fence_barrier_init();
  }
}

// COUNT: per-CTA bucket histogram H[cta][bucket] and the k-mer total.
template <int MODE>
__global__ void __launch_bounds__(kCountThreads) k_l1_lines_count(ExtractArgs a,
                                                                 uint32_t* __restrict__ H,
                                                                 unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(128) uint8_t smraw[];
  const int W = a.W, k = a.k;
  const uint64_t stride = (uint64_t)W + 1;
  const uint32_t bb = tile_buf_bytes(blockDim.x, stride);
  uint32_t* cnt = reinterpret_cast<uint32_t*>(smraw + 128 + bb);  // F1
  uint8_t* lut = reinterpret_cast<uint8_t*>(cnt + a.F1);              // 256
  __shared__ uint32_t s_jobs[2];
  TextTiles T;
  setup_tiles(&T, a, smraw, bb);
  T.buf1 = T.buf0;  // one buffer: tile t+1 is fetched once tile t is done
  for (int b = threadIdx.x; b < a.F1; b += blockDim.x) cnt[b] = 0;
  init_lut(lut, a.conv);
  __syncthreads();
  uint32_t mine = 0;
  const uint32_t nt = T.ntiles();
  if (threadIdx.x == 0 && nt) T.issue(0);
  for (uint32_t ti = 0; ti < nt; ++ti) {
    const uint8_t* tile = T.acquire(ti, &counters[3]);
    if (!tile) return;  // nothing else is in flight into this CTA's shared memory
    uint64_t l0, l1;
    T.range(ti, &l0, &l1);
    tile_jobs(a, l0, l1, s_jobs);
    const uint64_t l = l0 + threadIdx.x;
    const uint8_t* line = tile + (l - l0) * stride;
    JobBucket jb;
    if (line_prologue(a, l, l1, line, &jb, counters, s_jobs)) {
      LineRoll r;
      r.reset();
      for (int p0 = 0; p0 < W && !r.stopped; p0 += 8) {  // 8 independent loads per group
        uint32_t c8[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) c8[u] = p0 + u < W ? lut[line[p0 + u]] : 0xF0u;
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (r.template step<MODE>(c8[u], p0 + u, W, k, a.kmask)) {
            atomicAdd(&cnt[a.njobs ? jb(r.key) : (uint32_t)(r.key >> a.shift1)], 1u);
            ++mine;
          }
      }
    }
    // every thread's generic accesses of the buffer are ordered before the
    // bulk copy that refills it (one buffer: more CTAs per SM hide the wait)
    fence_barrier_init();
    __syncthreads();
    if (threadIdx.x == 0 && ti + 1 < nt) T.issue(ti + 1);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) mine += __shfl_xor_sync(0xFFFFFFFFu, mine, o);
  if (lane_id() == 0 && mine) atomicAdd(&counters[0], (unsigned long long)mine);
  __syncthreads();
  uint32_t* row = H + (size_t)blockIdx.x * a.F1;
  for (int b = threadIdx.x; b < a.F1; b += blockDim.x) row[b] = cnt[b];
}

// Level-1 bucket of a key, key >> shift1.  With kHi (shift1 >= 32, e.g.
// k = 31 at up to 12 bucket bits) only the key's high word is needed, so the
// key's low word and a 64-bit shift by a run-time amount drop out (level-1
// scatter on large_100m: 5% fewer instructions, 9.35 -> 9.31 ms; the level-1
// count's compiled code already did without them).
template <bool kHi>
__device__ __forceinline__ uint32_t l1_bucket(uint64_t key, int shift1) {
  return kHi ? (uint32_t)(key >> 32) >> (shift1 - 32) : (uint32_t)(key >> shift1);
}

// Plain-count scatter, thread per line: a tile's k-mers leave in chunks of
// kLineChunk positions per line.  For each chunk every thread rolls its
// line's positions once to count the chunk's keys per bucket, the block scans
// those counts, and the thread rolls the same positions again (from the saved
// state) to place each key in shared memory grouped by bucket; each bucket's
// keys then leave as one contiguous run at this CTA's cursor of the bucket.
// One text buffer (the next tile is fetched after the current one is done)
// keeps shared memory at two CTAs per SM.  A chunk's codes are read from the
// tile once, with independent loads, into registers (4 per word); both rolls
// step through them unrolled.  On the window path (DAKC's convention, k >= 2)
// the count pass's atomics already give each k-mer its rank in its bucket;
// the ranks stay in registers, two 16-bit ranks a word, and place the keys
// with no second atomic (large_100m: 9.31 -> 9.20 ms; 109 registers, under
// the 128 that two 256-thread CTAs per SM allow).
template <int MODE, int CH, bool kHi>
__global__ void __launch_bounds__(kLineThreads, 2) k_l1_lines_chunked(ExtractArgs a,
                                                                     const uint64_t* __restrict__ O,
                                                                     uint64_t* __restrict__ keys_out,
                                                                     unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(128) uint8_t smraw[];
  constexpr int chunk = CH;
  const int W = a.W, k = a.k, F1 = a.F1;
  const uint64_t stride = (uint64_t)W + 1;
  const uint32_t bb = tile_buf_bytes(blockDim.x, stride);
  unsigned long long* stage = reinterpret_cast<unsigned long long*>(smraw + 128 + bb);  // chunk keys
  unsigned long long* cursor = stage + (size_t)blockDim.x * chunk;                       // F1
  uint32_t* cnt2 = reinterpret_cast<uint32_t*>(cursor + F1);                              // 2 x F1
  uint32_t* coff = cnt2 + 2 * F1;                                                         // F1
  uint32_t* tmp = coff + F1;                                                              // 32
  uint8_t* lut = reinterpret_cast<uint8_t*>(tmp + 32);                                    // 256
  TextTiles T;
  setup_tiles(&T, a, smraw, bb);
  T.buf1 = T.buf0;  // one buffer: tile t+1 is fetched once tile t is done
  for (int b = threadIdx.x; b < F1; b += blockDim.x) {
    cursor[b] = O[(size_t)blockIdx.x * F1 + b];
    cnt2[b] = 0;
    cnt2[F1 + b] = 0;
    coff[b] = 0;
  }
  // Bucket counts alternate between two arrays by chunk: chunk c counts in
  // cnt2[c & 1], and the next chunk advances the cursors by them (after its
  // first barrier, when every thread has finished chunk c's flush) and clears
  // them for the chunk after.  While a chunk flushes, cursor[b] holds its
  // bucket's output position minus the bucket's offset in the stage (modulo
  // 2^64), so a staged key at stage index i goes to cursor[b] + i; the next
  // chunk adds the offset back with the counts.
  int cur = 0;
  init_lut(lut, a.conv);
  __syncthreads();
  const uint32_t nt = T.ntiles();
  if (threadIdx.x == 0 && nt) T.issue(0);
  for (uint32_t ti = 0; ti < nt; ++ti) {
    const uint8_t* tile = T.acquire(ti, &counters[3]);
    if (!tile) return;  // nothing else is in flight into this CTA's shared memory
    uint64_t l0, l1;
    T.range(ti, &l0, &l1);
    const uint64_t l = l0 + threadIdx.x;
    const uint8_t* line = tile + (l - l0) * stride;
    JobBucket jb;
    const uint32_t no_jobs[2] = {0, 0};
    const bool live = line_prologue(a, l, l1, line, &jb, counters, no_jobs);
    LineRoll r;
    r.reset();
    if (!live) r.stopped = true;
    // warm-up: positions before the first possible k-mer end emit nothing
    const int warm = min(k - 1, W);
    LineWin win;
    if (MODE == kRollDakc) {
      // the window of the 32 positions before the first chunk
      uint32_t iw[8];
#pragma unroll
      for (int g = 0; g < 8; ++g) {
        uint32_t w = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int p = warm - 32 + g * 4 + u;
          w |= (p < 0 ? 0xFFu : (live ? (uint32_t)lut[line[p]] : 0xF0u)) << (8 * u);
        }
        iw[g] = w;
      }
      win.init(iw);
    } else {
      for (int p0 = 0; p0 < warm; p0 += 4) {
        uint32_t c4[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) c4[u] = live && p0 + u < warm ? lut[line[p0 + u]] : 0xF0u;
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (p0 + u < warm) r.template step<MODE>(c4[u], p0 + u, W, k, a.kmask);
      }
    }
    for (int p0 = warm; p0 < W; p0 += chunk) {  // uniform over the block
      const int np = min(W - p0, chunk);        // positions of this chunk (uniform)
      uint32_t* ccount = cnt2 + (cur ? F1 : 0);  // this chunk's counts
      uint32_t* cprev = cnt2 + (cur ? 0 : F1);   // the previous chunk's
      uint32_t cw[CH / 4];  // the chunk's codes, byte q & 3 of word q >> 2
      {
        // the chunk's bytes through aligned 32-bit loads, 9 instead of 32 byte
        // loads (large_100m: 9.56 -> 9.41 ms).  A few bytes past the line are
        // read from the tile buffer's slack or the stage after it, and never
        // used: positions past np are stops
        const uintptr_t ad = reinterpret_cast<uintptr_t>(line + p0);
        const uint32_t* wp = reinterpret_cast<const uint32_t*>(ad & ~(uintptr_t)3);
        const uint32_t fs = (uint32_t)(ad & 3) * 8;
        uint32_t tw[CH / 4 + 1];
#pragma unroll
        for (int g = 0; g <= CH / 4; ++g) tw[g] = wp[g];
#pragma unroll
        for (int g = 0; g < CH / 4; ++g) {
          const uint32_t b4 = __funnelshift_r(tw[g], tw[g + 1], fs);
          uint32_t w = 0;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int q = g * 4 + u;
            w |= (live && q < np ? (uint32_t)lut[(b4 >> (8 * u)) & 0xFFu] : 0xF0u) << (8 * u);
          }
          cw[g] = w;
        }
      }
      const LineRoll r0 = r;
      uint64_t wc = 0, wm = 0;  // window path: the chunk's codes and break bits
      uint32_t wv = 0, wstp = 0;
      uint32_t rk2[CH / 2];  // window path: each k-mer's rank in its bucket, two per word
      if (MODE == kRollDakc) {
        uint32_t brk;
        LineWin::pack<CH>(cw, &wc, &brk, &wstp);
        wv = win.valid<CH>(brk, wstp, k, &wm);
#pragma unroll
        for (int q = 0; q < CH; ++q) {
          uint32_t rq = 0;
          if ((wv >> q) & 1u)
            rq = atomicAdd(&ccount[l1_bucket<kHi>(win.key<CH>(wc, q, a.kmask), a.shift1)], 1u);
          if (q & 1) rk2[q >> 1] |= rq << 16;
          else rk2[q >> 1] = rq;
        }
      } else {
#pragma unroll
        for (int q = 0; q < CH; ++q)
          if (q < np && r.template step<MODE>((cw[q >> 2] >> (8 * (q & 3))) & 0xFFu, p0 + q, W, k,
                                             a.kmask))
            atomicAdd(&ccount[l1_bucket<kHi>(r.key, a.shift1)], 1u);
      }
      __syncthreads();
      for (int b = threadIdx.x; b < F1; b += blockDim.x) {
        cursor[b] += coff[b] + cprev[b];  // the previous chunk's offset and count
        coff[b] = ccount[b];
        if (MODE != kRollDakc) ccount[b] = 0;  // the rolling paths rank again below
        cprev[b] = 0;
      }
      __syncthreads();
      const uint32_t Tn = block_scan_array<uint32_t>(coff, F1, tmp);
      for (int b = threadIdx.x; b < F1; b += blockDim.x) cursor[b] -= coff[b];
      if (MODE == kRollDakc) {
#pragma unroll
        for (int q = 0; q < CH; ++q)
          if ((wv >> q) & 1u) {
            const uint64_t key = win.key<CH>(wc, q, a.kmask);
            const uint32_t b = l1_bucket<kHi>(key, a.shift1);
            const uint32_t pos = coff[b] + ((rk2[q >> 1] >> (16 * (q & 1))) & 0xFFFFu);
            if (DK_OK_IDX(pos < (uint32_t)blockDim.x * chunk, 41, pos)) stage[pos] = key;
          }
        win.advance<CH>(wc, wm, wstp);
      } else {
        r = r0;
#pragma unroll
        for (int q = 0; q < CH; ++q)
          if (q < np && r.template step<MODE>((cw[q >> 2] >> (8 * (q & 3))) & 0xFFu, p0 + q, W, k,
                                             a.kmask)) {
            const uint32_t b = l1_bucket<kHi>(r.key, a.shift1);
            const uint32_t pos = coff[b] + atomicAdd(&ccount[b], 1u);
            if (DK_OK_IDX(pos < (uint32_t)blockDim.x * chunk, 41, pos)) stage[pos] = r.key;
          }
      }
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < Tn; i += blockDim.x) {
        const uint64_t key = stage[i];
        keys_out[cursor[l1_bucket<kHi>(key, a.shift1)] + i] = key;
      }
      cur ^= 1;
    }
    // every thread's generic accesses of the buffer are ordered before the
    // bulk copy that refills it
    fence_barrier_init();
    __syncthreads();
    if (threadIdx.x == 0 && ti + 1 < nt) T.issue(ti + 1);
  }
}

// Batch-mode scatter: each k-mer goes straight to its bucket at this CTA's
// cursor, O[cta][bucket] + (its rank among this CTA's keys of the bucket).
// A wave's jobs own up to 4,096 level-1 buckets, so a tile holds about one
// key per bucket and staging would not lengthen the runs; writing directly
// keeps shared memory small (text tiles and cursors only).  Consecutive keys
// of a bucket land next to each other, so L2 merges the 8-byte stores.
template <int MODE>
__global__ void __launch_bounds__(kLineThreads) k_l1_lines_direct(ExtractArgs a,
                                                                  const uint64_t* __restrict__ O,
                                                                  uint64_t* __restrict__ keys_out,
                                                                  unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(128) uint8_t smraw[];
  const int W = a.W, k = a.k;
  const uint64_t stride = (uint64_t)W + 1;
  const uint32_t bb = tile_buf_bytes(blockDim.x, stride);
  unsigned long long* cursor = reinterpret_cast<unsigned long long*>(smraw + 128 + 2 * bb);  // F1
  uint32_t* cnt = reinterpret_cast<uint32_t*>(cursor + a.F1);                                 // F1
  uint8_t* lut = reinterpret_cast<uint8_t*>(cnt + a.F1);                                      // 256
  __shared__ uint32_t s_jobs[2];
  TextTiles T;
  setup_tiles(&T, a, smraw, bb);
  for (int b = threadIdx.x; b < a.F1; b += blockDim.x) {
    cursor[b] = O[(size_t)blockIdx.x * a.F1 + b];
    cnt[b] = 0;
  }
  init_lut(lut, a.conv);
  __syncthreads();
  const uint32_t nt = T.ntiles();
  if (threadIdx.x == 0 && nt) T.issue(0);
  for (uint32_t ti = 0; ti < nt; ++ti) {
    if (threadIdx.x == 0 && ti + 1 < nt) T.issue(ti + 1);
    const uint8_t* tile = T.acquire(ti, &counters[3]);
    if (!tile) {
      T.drain(ti + 1);
      return;
    }
    uint64_t l0, l1;
    T.range(ti, &l0, &l1);
    tile_jobs(a, l0, l1, s_jobs);
    const uint64_t l = l0 + threadIdx.x;
    const uint8_t* line = tile + (l - l0) * stride;
    JobBucket jb;
    if (line_prologue(a, l, l1, line, &jb, counters, s_jobs)) {
      LineRoll r;
      r.reset();
      for (int p0 = 0; p0 < W && !r.stopped; p0 += 4) {
        uint32_t c4[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) c4[u] = p0 + u < W ? lut[line[p0 + u]] : 0xF0u;
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (r.template step<MODE>(c4[u], p0 + u, W, k, a.kmask)) {
            const uint32_t b = a.njobs ? jb(r.key) : (uint32_t)(r.key >> a.shift1);
            keys_out[cursor[b] + atomicAdd(&cnt[b], 1u)] = r.key;
          }
      }
    }
    __syncthreads();  // the buffer is refilled two tiles on
  }
}

template <int C, int LPW, int CONV>
__global__ void __launch_bounds__(512, 2) k_l1_scatter(ExtractArgs a, const uint64_t* __restrict__ O,
                                                    uint64_t* __restrict__ keys_out,
                                                    int stage_cap,
                                                    unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(128) uint8_t smraw[];
  const int F1 = a.F1;
  const uint32_t nwarps = blockDim.x >> 5;
  const uint32_t lt = nwarps * LPW;
  const uint64_t stride = (uint64_t)a.W + 1;
  const uint32_t bb = tile_buf_bytes(lt, stride);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  uint8_t* tb = smraw + 128;
  unsigned long long* cursor = reinterpret_cast<unsigned long long*>(tb + 2 * bb);  // F1
  unsigned long long* staging = cursor + F1;                              // stage_cap
  uint32_t* tile_hist = reinterpret_cast<uint32_t*>(staging + stage_cap);  // F1
  uint32_t* tile_off = tile_hist + F1;                                    // F1
  uint32_t* tmp = tile_off + F1;                                          // 32
  uint8_t* lut = reinterpret_cast<uint8_t*>(tmp + 32);                    // 256
  uint16_t* staged_b = reinterpret_cast<uint16_t*>(lut + 256);            // stage_cap (batch mode)
  TextTiles T;
  T.text = a.text;
  T.nbytes = a.nbytes;
  T.stride = stride;
  lines_of_block(a.n_lines, &T.lo, &T.hi);
  T.lt = lt;
  T.buf0 = tb;
  T.buf1 = tb + bb;
  T.bar = bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
  }
  for (int b = threadIdx.x; b < F1; b += blockDim.x) {
    cursor[b] = O[(size_t)blockIdx.x * F1 + b];
    tile_hist[b] = 0;
  }
  init_lut(lut, a.conv);
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5;
  const uint32_t nt = T.ntiles();
  if (threadIdx.x == 0 && nt) T.issue(0);
  for (uint32_t ti = 0; ti < nt; ++ti) {
    if (threadIdx.x == 0 && ti + 1 < nt) T.issue(ti + 1);
    const uint8_t* base = T.acquire(ti, &counters[3]);
    if (!base) {
      T.drain(ti + 1);
      return;
    }
    uint64_t t0, t1;
    T.range(ti, &t0, &t1);
    uint64_t kr[LPW][C];
    uint32_t sr[LPW][C];
    JobBucket jbr[LPW];  // batch mode: bucket rule of each line's job
#pragma unroll
    for (int j = 0; j < LPW; ++j) {
      const uint64_t l = t0 + (uint64_t)j * nwarps + warp;
      uint32_t job = 0;
      bool live = l < t1;
      if (live && a.njobs) {
        job = job_of_line(a, l);
        live = l < __ldg(a.job_end + job);
      }
      if (live) {
        if (a.njobs) jbr[j] = JobBucket(a, job);
        const JobBucket jb = jbr[j];
        auto on_kmer = [&](int t, uint64_t key, bool valid) {
          kr[j][t] = key;
          const uint32_t bkt = a.njobs ? jb(key) : (uint32_t)(key >> a.shift1);
          sr[j][t] = valid ? atomicAdd(&tile_hist[bkt], 1u) : 0xFFFFFFFFu;
        };
        warp_line_kmers<C, CONV>(base + (l - t0) * stride, a.W, a.k, a.kmask, lut, on_kmer);
      } else {
#pragma unroll
        for (int t = 0; t < C; ++t) { kr[j][t] = 0; sr[j][t] = 0xFFFFFFFFu; }
      }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < F1; b += blockDim.x) tile_off[b] = tile_hist[b];
    __syncthreads();
    const uint32_t Tn = block_scan_array<uint32_t>(tile_off, F1, tmp);
#pragma unroll
    for (int j = 0; j < LPW; ++j)
#pragma unroll
      for (int t = 0; t < C; ++t)
        if (sr[j][t] != 0xFFFFFFFFu) {
          const uint32_t bkt = a.njobs ? jbr[j](kr[j][t]) : (uint32_t)(kr[j][t] >> a.shift1);
          staging[tile_off[bkt] + sr[j][t]] = kr[j][t];
          if (a.njobs) staged_b[tile_off[bkt] + sr[j][t]] = (uint16_t)bkt;
        }
    __syncthreads();
    if (a.njobs) {
      // batch mode: the bucket was staged with the key
      for (uint32_t i = threadIdx.x; i < Tn; i += blockDim.x) {
        const uint32_t b = staged_b[i];
        keys_out[cursor[b] + (i - tile_off[b])] = staging[i];
      }
    } else {
      for (uint32_t i = threadIdx.x; i < Tn; i += blockDim.x) {
        const uint64_t key = staging[i];
        const uint32_t b = (uint32_t)(key >> a.shift1);
        keys_out[cursor[b] + (i - tile_off[b])] = key;
      }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < F1; b += blockDim.x) {
      cursor[b] += tile_hist[b];
      tile_hist[b] = 0;
    }
    __syncthreads();
  }
}

// Warp-aggregated shared-memory atomics: lanes holding the same value add
// once (by the lowest such lane).  Hot k-mers (many copies of one key in a
// bin) otherwise serialise on one shared-memory word.
__device__ __forceinline__ void agg_add_u32(uint32_t* ctr, uint32_t v, bool hot) {
  if (!hot) { atomicAdd(&ctr[v], 1u); return; }
  const uint32_t mask = __activemask();
  const uint32_t peers = __match_any_sync(mask, v);
  if ((int)lane_id() == __ffs(peers) - 1) atomicAdd(&ctr[v], (uint32_t)__popc(peers));
}

// returns this lane's slot: leader reserves popc(peers) slots, peers take ranks
__device__ __forceinline__ uint32_t agg_reserve_u32(uint32_t* ctr, uint32_t v, bool hot) {
  if (!hot) return atomicAdd(&ctr[v], 1u);
  const uint32_t mask = __activemask();
  const uint32_t peers = __match_any_sync(mask, v);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(&ctr[v], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + (uint32_t)__popc(peers & ((1u << lane_id()) - 1u));
}

__device__ __forceinline__ void agg_add_u64(unsigned long long* ctr, uint32_t v) {
  const uint32_t mask = __activemask();
  const uint32_t peers = __match_any_sync(mask, v);
  if ((int)lane_id() == __ffs(peers) - 1) atomicAdd(&ctr[v], (unsigned long long)__popc(peers));
}

// Rank of this lane's key within its digit v (an atomic on ctr[v]); in a hot
// tile, lanes of the warp with the same digit reserve together.  Every lane
// of the warp calls it; `valid` lanes get a rank.
__device__ __forceinline__ uint32_t rank_in_digit(uint32_t* ctr, uint32_t v, bool valid, bool hot) {
  if (!hot) return valid ? atomicAdd(&ctr[v], 1u) : 0u;
  const uint32_t peers = __match_any_sync(0xFFFFFFFFu, valid ? v : 0xFFFFFFFFu);
  if (!valid) return 0u;
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(&ctr[v], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + (uint32_t)__popc(peers & ((1u << lane_id()) - 1u));
}

// ---------------------------------------------------- partition levels
// A split node is split on its next `width` bits, width chosen so that the
// children average about half a bin: wide for big nodes, narrow for small.

// node i's keys lie in several ranges (a level-1 bucket of a chunked upload)
__device__ __forceinline__ bool multi_range(const Ranges& rg, uint32_t i) {
  return rg.C > 0 && i < (uint32_t)rg.F1;
}

// partition tiles of node i: kTileKeys-key slices of each of its ranges
__device__ __forceinline__ uint32_t node_tiles(const Node& nd, uint32_t i, const Ranges& rg) {
  if (!multi_range(rg, i)) return (uint32_t)((nd.n + kTileKeys - 1) / kTileKeys);
  uint32_t nt = 0;
  for (int c = 0; c < rg.C; ++c) nt += (rg.T[(size_t)c * rg.F1 + i] + kTileKeys - 1) / kTileKeys;
  return nt;
}

// Mark each node of the level final / split / empty; count what the split
// nodes need (children, tiles, histogram entries).
__device__ __forceinline__ void classify_node(Node* nodes, uint32_t i, uint32_t* final_list,
                                              uint32_t* big_list, LevelCounters* ctr,
                                              int bin_cap, int split_target, int big_ok,
                                              const Ranges& rg, int max_bits) {
  const Node nd = nodes[i];
  if (nd.n == 0) {
    nodes[i].state = NODE_EMPTY;
    nodes[i].d = 0;
    return;
  }
  // a skewed node holds a hot k-mer: splitting peels off few keys per level,
  // while one hash bin streams any number of copies (it is re-partitioned if
  // it holds too many distinct keys).  A node of several ranges splits (into
  // one range per child) whatever its size.
  // big_ok 1: any such node; big_ok 2: only one of 2^31 keys or more (its
  // split would need as many partition levels, each over all its keys, and
  // near 2^32 the partition's 32-bit per-child offsets)
  if (!multi_range(rg, i) &&
      (nd.n <= (uint64_t)bin_cap || nd.shift <= kDenseBits ||
       (big_ok && nd.skewed && (big_ok == 1 || nd.n >= (1ull << 31))))) {
    nodes[i].state = NODE_FINAL;
    if (nd.n > (uint64_t)bin_cap && nd.shift > kDenseBits)
      big_list[atomicAdd(&ctr->n_big_final, 1u)] = i;
    else
      final_list[atomicAdd(&ctr->n_final, 1u)] = i;
    return;
  }
  const uint64_t target = (uint64_t)max(1, split_target / 2);  // children ~ target keys
  int w = ceil_log2_u64((nd.n + target - 1) / target);
  w = max(1, min(w, max_bits));
  const uint32_t nt = node_tiles(nd, i, rg);
  nodes[i].state = NODE_SPLIT;
  nodes[i].width = (uint8_t)w;
  atomicAdd(&ctr->n_split, 1u);
  atomicAdd(&ctr->split_keys, (unsigned long long)nd.n);
  atomicAdd(&ctr->n_tiles, nt);
  atomicAdd(&ctr->n_children, 1u << w);
  atomicAdd(&ctr->th_entries, (unsigned long long)nt << w);
  atomicMax(&ctr->max_width, (uint32_t)w);
  if (nd.n >= (1ull << 32)) atomicOr(&ctr->too_big, 1u);
}

__global__ void k_classify(Node* nodes, uint32_t lo, uint32_t hi, uint32_t* final_list,
                           uint32_t* big_list, LevelCounters* ctr, int bin_cap, int split_target,
                           int big_ok, Ranges rg) {
  const uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi) return;
  classify_node(nodes, i, final_list, big_list, ctr, bin_cap, split_target, big_ok, rg,
                kMaxSplitBits);
}

// Give each split node its children block, its partition tiles and their
// histogram rows (buffers sized by the host from k_classify's counts); one
// warp per node, its lanes write the tiles.
__device__ __forceinline__ void assign_node(Node* nodes, uint32_t i, uint32_t child_base,
                                            Tile* tiles, LevelCounters* ctr, const Ranges& rg) {
  const Node nd = nodes[i];
  if (nd.state != NODE_SPLIT) return;
  const uint32_t R = 1u << nd.width;
  const uint32_t nt = node_tiles(nd, i, rg);
  uint32_t tb = 0, fc = 0;
  unsigned long long thb = 0;
  if (lane_id() == 0) {
    tb = atomicAdd(&ctr->n_tiles_assigned, nt);
    fc = child_base + atomicAdd(&ctr->n_children_assigned, R);
    thb = atomicAdd(&ctr->th_assigned, (unsigned long long)nt * R);
    nodes[i].first_child = fc;
    nodes[i].tile_base = tb;
    nodes[i].ntiles = nt;
    nodes[i].th_base = thb;
  }
  tb = __shfl_sync(0xFFFFFFFFu, tb, 0);
  thb = __shfl_sync(0xFFFFFFFFu, thb, 0);
  if (multi_range(rg, i)) {  // the tiles of each range in turn
    uint32_t t0 = 0;
    for (int c = 0; c < rg.C; ++c) {
      const uint32_t cn = rg.T[(size_t)c * rg.F1 + i];
      const uint64_t cs = rg.S[(size_t)c * rg.F1 + i];
      const uint32_t ntc = (cn + kTileKeys - 1) / kTileKeys;
      for (uint32_t u = lane_id(); u < ntc; u += 32) {
        Tile tl;
        tl.start = cs + (uint64_t)u * kTileKeys;
        tl.n = min((uint32_t)kTileKeys, cn - u * (uint32_t)kTileKeys);
        tl.node = i;
        tl.th = thb + (uint64_t)(t0 + u) * R;
        tl.hot = 0;
        tl.pad = 0;
        tiles[tb + t0 + u] = tl;
      }
      t0 += ntc;
    }
    return;
  }
  for (uint32_t t = lane_id(); t < nt; t += 32) {
    Tile tl;
    tl.start = nd.start + (uint64_t)t * kTileKeys;
    tl.n = (uint32_t)min((uint64_t)kTileKeys, nd.n - (uint64_t)t * kTileKeys);
    tl.node = i;
    tl.th = thb + (uint64_t)t * R;
    tl.hot = 0;
    tl.pad = 0;
    tiles[tb + t] = tl;
  }
}

__global__ void k_assign(Node* nodes, uint32_t lo, uint32_t hi, uint32_t child_base, Tile* tiles,
                         LevelCounters* ctr, Ranges rg) {
  const uint32_t i = lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (i >= hi) return;  // warp-uniform
  assign_node(nodes, i, child_base, tiles, ctr, rg);
}

__device__ __forceinline__ uint32_t digit_of(uint64_t key, int shift, int width) {
  return (uint32_t)(key >> (shift - width)) & ((1u << width) - 1u);
}

// Pull tile t's keys into L2 (thread 0; nothing waits for it): with one
// block per tile, blocks start in index order, so the block that takes tile
// blockIdx + (resident blocks) starts about one tile's time later.
__device__ __forceinline__ void prefetch_tile(const Node* nodes, const Tile* tiles, uint32_t t,
                                              uint32_t n_tiles, const uint64_t* A,
                                              const uint64_t* B) {
  if (threadIdx.x != 0 || t >= n_tiles) return;
  const Tile tl = tiles[t];
  const Node& nd = nodes[tl.node];
  prefetch_l2_range((nd.buf ? B : A) + tl.start, (uint64_t)tl.n * 8);
}

// one tile's digit histogram (the whole block; hist: 2^kMaxSplitBits entries)
__device__ __forceinline__ void tile_hist_one(const Node* nodes, const Tile* tiles, uint32_t t,
                                              const uint64_t* A, const uint64_t* B, uint32_t* TH,
                                              uint32_t* hist) {
  const Tile tl = tiles[t];
  const Node nd = nodes[tl.node];
  const uint32_t R = 1u << nd.width;
  const uint64_t* src = (nd.buf ? B : A) + tl.start;
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) hist[j] = 0;
  __syncthreads();
  const bool hot = nd.skewed;  // the node kept most of its parent's keys: a hot k-mer
  uint32_t i = threadIdx.x;
  const uint32_t T = blockDim.x;
  for (; i + 3 * T < tl.n; i += 4 * T) {
    const uint64_t k0 = __ldg(src + i), k1 = __ldg(src + i + T), k2 = __ldg(src + i + 2 * T),
                   k3 = __ldg(src + i + 3 * T);
    agg_add_u32(hist, digit_of(k0, nd.shift, nd.width), hot);
    agg_add_u32(hist, digit_of(k1, nd.shift, nd.width), hot);
    agg_add_u32(hist, digit_of(k2, nd.shift, nd.width), hot);
    agg_add_u32(hist, digit_of(k3, nd.shift, nd.width), hot);
  }
  for (; i < tl.n; i += T) agg_add_u32(hist, digit_of(__ldg(src + i), nd.shift, nd.width), hot);
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) TH[tl.th + j] = hist[j];
}

__global__ void __launch_bounds__(256) k_tile_hist(const Node* nodes, const Tile* tiles,
                                                   const uint64_t* A, const uint64_t* B,
                                                   uint32_t* TH) {
  __shared__ uint32_t hist[1u << kMaxSplitBits];
  tile_hist_one(nodes, tiles, blockIdx.x, A, B, TH, hist);
}

// one CTA per node of the level; split nodes turn their tiles' counts into
// offsets within each child and create the 2^width children
// one node's scan (the whole block; csize: 2^kMaxSplitBits entries)
__device__ __forceinline__ void node_scan_one(Node* nodes, uint32_t i, Tile* tiles, uint32_t* TH,
                                              unsigned long long* csize,
                                              unsigned long long* tmp) {
  const Node nd = nodes[i];
  if (nd.state != NODE_SPLIT) return;
  const uint32_t R = 1u << nd.width;
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) {
    uint32_t run = 0;
    uint32_t* col = TH + nd.th_base + j;
    // sixteen tiles at a time: their loads are independent, only the running
    // sum is serial
    uint32_t t = 0;
    // a digit with more than a quarter of a full tile marks that tile hot
    constexpr uint32_t kHotCount = kTileKeys / 4;
    for (; t + 16 <= nd.ntiles; t += 16) {
      uint32_t c[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) c[u] = col[(t + u) * R];  // < 2^32: a node's ntiles * R
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        col[(t + u) * R] = run;
        run += c[u];
        if (c[u] > kHotCount) tiles[nd.tile_base + t + u].hot = 1;
      }
    }
    for (; t < nd.ntiles; ++t) {
      const uint32_t c = col[t * R];
      col[t * R] = run;
      run += c;
      if (c > kHotCount) tiles[nd.tile_base + t].hot = 1;
    }
    csize[j] = run;
  }
  __syncthreads();
  // child starts: exclusive scan of the child sizes (kept separately: csize
  // becomes the starts, sizes are re-derived from neighbouring starts)
  const unsigned long long total = block_scan_array<unsigned long long>(csize, (int)R, tmp);
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) {
    Node ch;
    ch.start = nd.start + csize[j];
    ch.n = (j + 1 < R ? csize[j + 1] : total) - csize[j];
    ch.d = 0;
    ch.out_off = 0;
    ch.first_child = 0;
    ch.shift = (int16_t)(nd.shift - nd.width);
    ch.buf = (uint8_t)(1 - nd.buf);
    ch.state = 0;
    ch.tile_base = 0;
    ch.ntiles = 0;
    ch.th_base = 0;
    ch.width = 0;
    ch.skewed = ch.n * 2 > nd.n;
    nodes[nd.first_child + j] = ch;
  }
}

__global__ void __launch_bounds__(1024) k_node_scan(Node* nodes, uint32_t lo, Tile* tiles,
                                                    uint32_t* TH) {
  __shared__ unsigned long long csize[1u << kMaxSplitBits];
  __shared__ unsigned long long tmp[32];
  node_scan_one(nodes, lo + blockIdx.x, tiles, TH, csize, tmp);
}

// Partition one tile by the node's next `width` bits.  Pass 1 ranks every key
// within its digit (shared atomics); the tile is then laid out digit by digit
// in shared memory (keys re-read from L2) so each digit's keys leave as one
// contiguous, coalesced run at the tile's offset inside the child.
constexpr int kTileThreads = 512;
constexpr int kTileKeysPerThread = kTileKeys / kTileThreads;
static_assert(kTileKeys <= 65536 && kTileKeysPerThread % 2 == 0, "ranks are packed as 16-bit pairs");

#ifndef DK_TILE_CTAS
#define DK_TILE_CTAS 2
#endif
// one tile (the whole block): dsm holds kTileKeys keys and 2^max_width
// (base, count, location) entries
__device__ __forceinline__ void tile_scatter_one(const Node* nodes, const Tile* tiles, uint32_t t,
                                                 uint64_t* A, uint64_t* B, const uint32_t* TH,
                                                 int max_width, unsigned long long* dsm,
                                                 uint32_t* tmp) {
  unsigned long long* stage = dsm;                                  // kTileKeys
  unsigned long long* gbase = stage + kTileKeys;                    // 2^max_width
  uint32_t* cnt = reinterpret_cast<uint32_t*>(gbase + (1u << max_width));
  uint32_t* loc = cnt + (1u << max_width);
  const Tile tl = tiles[t];
  const Node nd = nodes[tl.node];
  const uint32_t R = 1u << nd.width;
  const int sh = nd.shift, w = nd.width;
  const uint64_t* src = (nd.buf ? B : A) + tl.start;
  uint64_t* dst = nd.buf ? A : B;
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) {
    gbase[j] = nodes[nd.first_child + j].start + TH[tl.th + j];
    cnt[j] = 0;
  }
  __syncthreads();
  const bool hot = tl.hot != 0;  // a skewed tile: ranks are reserved per warp
  // all of this thread's keys are loaded first (their loads overlap) and kept
  // in registers for the staging pass
  uint64_t kr[kTileKeysPerThread];
#pragma unroll
  for (int u = 0; u < kTileKeysPerThread; ++u) {
    const uint32_t i = threadIdx.x + u * kTileThreads;
    kr[u] = i < tl.n ? __ldg(src + i) : 0ull;
  }
  uint32_t rank[kTileKeysPerThread / 2];  // two 16-bit ranks per word
#pragma unroll
  for (int u = 0; u < kTileKeysPerThread; ++u) {
    const uint32_t i = threadIdx.x + u * kTileThreads;
    // every lane reaches the reserve (in a hot tile its match is warp-wide)
    const uint32_t r = rank_in_digit(cnt, digit_of(kr[u], sh, w), i < tl.n, hot);
    if (u & 1) rank[u >> 1] |= r << 16;
    else rank[u >> 1] = r;
  }
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) loc[j] = cnt[j];
  __syncthreads();
  block_scan_array<uint32_t>(loc, (int)R, tmp);
#pragma unroll
  for (int u = 0; u < kTileKeysPerThread; ++u) {
    const uint32_t i = threadIdx.x + u * kTileThreads;
    if (i < tl.n) {
      const uint32_t r = (rank[u >> 1] >> ((u & 1) * 16)) & 0xFFFFu;
      stage[loc[digit_of(kr[u], sh, w)] + r] = kr[u];
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < tl.n; i += blockDim.x) {
    const uint64_t key = stage[i];
    const uint32_t d = digit_of(key, sh, w);
    dst[gbase[d] + (i - loc[d])] = key;
  }
}

__global__ void __launch_bounds__(kTileThreads, DK_TILE_CTAS) k_tile_scatter(const Node* nodes,
                                                                  const Tile* tiles, uint64_t* A,
                                                                  uint64_t* B,
                                                                  const uint32_t* TH,
                                                                  int max_width, uint32_t ahead) {
  extern __shared__ __align__(16) unsigned long long dsm[];
  __shared__ uint32_t tmp[32];
  prefetch_tile(nodes, tiles, blockIdx.x + ahead, gridDim.x, A, B);
  tile_scatter_one(nodes, tiles, blockIdx.x, A, B, TH, max_width, dsm, tmp);
}

// ------------------------------------------------------------ bin count
constexpr uint32_t kThreadSortMax = 16;  // larger digit ranges are sorted by a warp

// Block-wide exclusive scan of (sum, max) pairs; returns both exclusive
// values and the block totals.  `tmp` needs 64 u32 slots.
__device__ __forceinline__ void block_scan_sum_max(uint32_t v, int m, uint32_t* tmp,
                                                   uint32_t* ex_sum, int* ex_max,
                                                   uint32_t* tot_sum) {
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t xs = v;
  int xm = m;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t ys = __shfl_up_sync(0xFFFFFFFFu, xs, o);
    const int ym = __shfl_up_sync(0xFFFFFFFFu, xm, o);
    if ((int)lane >= o) { xs += ys; xm = max(xm, ym); }
  }
  if (lane == 31) { tmp[warp] = xs; tmp[32 + warp] = (uint32_t)xm; }
  __syncthreads();
  if (warp == 0) {
    uint32_t ws = lane < nw ? tmp[lane] : 0u;
    int wm = lane < nw ? (int)tmp[32 + lane] : -1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t ys = __shfl_up_sync(0xFFFFFFFFu, ws, o);
      const int ym = __shfl_up_sync(0xFFFFFFFFu, wm, o);
      if ((int)lane >= o) { ws += ys; wm = max(wm, ym); }
    }
    if (lane < nw) { tmp[lane] = ws; tmp[32 + lane] = (uint32_t)wm; }
  }
  __syncthreads();
  const uint32_t bs = warp ? tmp[warp - 1] : 0u;
  const int bm = warp ? (int)tmp[32 + warp - 1] : -1;
  *ex_sum = bs + xs - v;
  // exclusive max within the warp: inclusive max of the previous lane
  int pm = __shfl_up_sync(0xFFFFFFFFu, xm, 1);
  if (lane == 0) pm = -1;
  *ex_max = max(bm, pm);
  *tot_sum = tmp[nw - 1];
  __syncthreads();
}

// Dense count of a node with shift <= 12 free bits: the histogram over the
// free bits is already the sorted run-length table.  hist64 holds 4096 u64.
__device__ void bin_dense(Node* nodes, uint32_t ni, const Node& nd, uint64_t* keys, uint32_t* cnt,
                          unsigned long long* hist, unsigned long long* tmp,
                          unsigned long long* overflow) {
  const int s = nd.shift;
  const uint32_t R = 1u << s;
  const uint64_t mask = (uint64_t)R - 1;
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) hist[j] = 0;
  __syncthreads();
  const uint64_t prefix = (keys[0] >> s) << s;
  const uint64_t T = blockDim.x;
  uint64_t i = threadIdx.x;
  for (; i + 3 * T < nd.n; i += 4 * T) {
    const uint64_t k0 = __ldg(keys + i), k1 = __ldg(keys + i + T), k2 = __ldg(keys + i + 2 * T),
                   k3 = __ldg(keys + i + 3 * T);
    agg_add_u64(hist, (uint32_t)(k0 & mask));
    agg_add_u64(hist, (uint32_t)(k1 & mask));
    agg_add_u64(hist, (uint32_t)(k2 & mask));
    agg_add_u64(hist, (uint32_t)(k3 & mask));
  }
  for (; i < nd.n; i += T) agg_add_u64(hist, (uint32_t)(__ldg(keys + i) & mask));
  __syncthreads();
  const uint32_t per = (R + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = min(R, threadIdx.x * per), hi = min(R, lo + per);
  unsigned long long c = 0;
  for (uint32_t j = lo; j < hi; ++j) c += (hist[j] != 0);
  unsigned long long total;
  unsigned long long r = block_excl_scan<unsigned long long>(c, tmp, &total);
  for (uint32_t j = lo; j < hi; ++j) {
    const unsigned long long h = hist[j];
    if (h) {
      keys[r] = prefix | j;
      if (h > 0xFFFFFFFFull) atomicMax(overflow, 1ull);
      cnt[r] = (uint32_t)h;
      ++r;
    }
  }
  if (threadIdx.x == 0) nodes[ni].d = total;
}

// Sort s[0, m) in place with one warp when it holds at most 32*K distinct
// keys: gather (key, count) pairs with __match_any_sync (entry e lives in
// lane e%32, slot e/32), sort them with a bitonic network across lanes
// (shuffles) and slots (registers), and rewrite the range.  Returns false,
// leaving the range untouched, when there are more distinct keys.
template <int K>
__device__ bool warp_sort_few_distinct(unsigned long long* s, uint32_t m) {
  const uint32_t lane = lane_id();
  unsigned long long dk[K];
  uint32_t dc[K];
#pragma unroll
  for (int u = 0; u < K; ++u) { dk[u] = 0; dc[u] = 0; }
  uint32_t nd = 0;
  for (uint32_t base = 0; base < m; base += 32) {
    const uint32_t i = base + lane;
    const bool valid = i < m;
    const unsigned long long key = valid ? s[i] : 0ull;
    const uint32_t active = __ballot_sync(0xFFFFFFFFu, valid);
    uint32_t peers = 0;
    if (valid) peers = __match_any_sync(active, key);
    const bool leader = valid && (__ffs(peers) - 1 == (int)lane);
    uint32_t leaders = __ballot_sync(0xFFFFFFFFu, leader);
    while (leaders) {
      const int l = __ffs(leaders) - 1;
      leaders &= leaders - 1;
      const unsigned long long kl = __shfl_sync(0xFFFFFFFFu, key, l);
      const uint32_t cl = __shfl_sync(0xFFFFFFFFu, (uint32_t)__popc(peers), l);
      bool found = false;
#pragma unroll
      for (int u = 0; u < K; ++u) {
        const uint32_t hit = __ballot_sync(0xFFFFFFFFu, (u * 32 + lane) < nd && dk[u] == kl);
        if (hit) {
          if (!found && (int)lane == __ffs(hit) - 1) dc[u] += cl;
          found = true;
        }
      }
      if (!found) {
        if (nd == 32u * K) return false;
#pragma unroll
        for (int u = 0; u < K; ++u)
          if (nd == u * 32 + lane) { dk[u] = kl; dc[u] = cl; }
        ++nd;
      }
    }
  }
  // bitonic sort of the 32*K entries (index e = u*32 + lane; e >= nd is +inf)
  bool inf[K];
#pragma unroll
  for (int u = 0; u < K; ++u) inf[u] = (u * 32 + lane) >= nd;
#pragma unroll
  for (int size = 2; size <= 32 * K; size <<= 1) {
#pragma unroll
    for (int st = size >> 1; st > 0; st >>= 1) {
      if (st >= 32) {  // partner in another slot of the same lane
        const int su = st >> 5;
#pragma unroll
        for (int u = 0; u < K; ++u) {
          if (u & su) continue;
          const int v = u | su;
          const uint32_t e = u * 32 + lane;
          const bool up = (e & size) == 0;
          const bool v_less = !inf[v] && (inf[u] || dk[v] < dk[u]);
          const bool u_less = !inf[u] && (inf[v] || dk[u] < dk[v]);
          if (up ? v_less : u_less) {
            const unsigned long long tk = dk[u]; dk[u] = dk[v]; dk[v] = tk;
            const uint32_t tc = dc[u]; dc[u] = dc[v]; dc[v] = tc;
            const bool ti = inf[u]; inf[u] = inf[v]; inf[v] = ti;
          }
        }
      } else {  // partner in another lane, same slot
#pragma unroll
        for (int u = 0; u < K; ++u) {
          const unsigned long long ok = __shfl_xor_sync(0xFFFFFFFFu, dk[u], st);
          const uint32_t oc = __shfl_xor_sync(0xFFFFFFFFu, dc[u], st);
          const bool oinf = __shfl_xor_sync(0xFFFFFFFFu, (int)inf[u], st) != 0;
          const uint32_t e = u * 32 + lane;
          const bool up = (e & size) == 0;
          const bool lower = (lane & st) == 0;
          const bool other_less = !oinf && (inf[u] || ok < dk[u]);
          const bool other_greater = !inf[u] && (oinf || dk[u] < ok);
          const bool take = (lower == up) ? other_less : other_greater;
          if (take) { dk[u] = ok; dc[u] = oc; inf[u] = oinf; }
        }
      }
    }
  }
  // offsets in entry order, then all lanes write each key's run
  uint32_t off[K];
  uint32_t run = 0;
#pragma unroll
  for (int u = 0; u < K; ++u) {
    uint32_t x = inf[u] ? 0u : dc[u];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if ((int)lane >= o) x += y;
    }
    off[u] = run + x - (inf[u] ? 0u : dc[u]);
    run += __shfl_sync(0xFFFFFFFFu, x, 31);
  }
  __syncwarp();
#pragma unroll
  for (int u = 0; u < K; ++u) {
    const uint32_t lim = nd > (uint32_t)(u * 32) ? min(32u, nd - u * 32) : 0u;
    for (uint32_t q = 0; q < lim; ++q) {
      const unsigned long long kq = __shfl_sync(0xFFFFFFFFu, dk[u], q);
      const uint32_t oq = __shfl_sync(0xFFFFFFFFu, off[u], q), cq = __shfl_sync(0xFFFFFFFFu, dc[u], q);
      for (uint32_t t = lane; t < cq; t += 32)
        if (DK_OK_IDX(oq + t < m, 21, ((uint64_t)(oq + t) << 32) | m)) s[oq + t] = kq;
    }
  }
  __syncwarp();
  return true;
}

// one-warp sort of m <= 32 keys in place: each lane ranks its key against all
// others (stable for equal keys) and writes it to its final slot
__device__ void warp_rank_sort(unsigned long long* s, uint32_t m) {
  const uint32_t lane = lane_id();
  const unsigned long long v = lane < m ? s[lane] : 0ull;
  uint32_t rank = 0;
  for (uint32_t j = 0; j < m; ++j) {
    const unsigned long long o = __shfl_sync(0xFFFFFFFFu, v, j);
    rank += (o < v) || (o == v && j < lane);
  }
  __syncwarp();
  if (lane < m && DK_OK_IDX(rank < m, 22, ((uint64_t)rank << 32) | m)) s[rank] = v;
  __syncwarp();
}

// one-warp bitonic sort of s[0, m) in shared memory (out-of-range partners
// act as +inf and never move)
__device__ void warp_bitonic(unsigned long long* s, uint32_t m) {
  int lg = 0;
  while ((1u << lg) < m) ++lg;
  const uint32_t P = 1u << lg;
  for (int sz = 1; sz <= lg; ++sz) {  // merge blocks of 2^sz
    const uint32_t hmask = (1u << (sz - 1)) - 1;
    for (uint32_t i = lane_id(); i < P / 2; i += 32) {
      const uint32_t a = ((i >> (sz - 1)) << sz) | (i & hmask);
      const uint32_t b = a ^ ((1u << sz) - 1);
      if (b < m) {
        const unsigned long long x = s[a], y = s[b];
        if (y < x) { s[a] = y; s[b] = x; }
      }
    }
    __syncwarp();
    for (int st = sz - 2; st >= 0; --st) {
      const uint32_t smask = (1u << st) - 1;
      for (uint32_t i = lane_id(); i < P / 2; i += 32) {
        const uint32_t a = ((i >> st) << (st + 1)) | (i & smask);
        const uint32_t b = a + (1u << st);
        if (b < m) {
          const unsigned long long x = s[a], y = s[b];
          if (y < x) { s[a] = y; s[b] = x; }
        }
      }
      __syncwarp();
    }
  }
}

constexpr uint32_t kDeferMax = 64;  // ranges per bin left to the block-wide sort

// Shared-memory sort + run-length reduce of one bin (n <= kBinCap keys,
// more than kDenseBits free bits).  Counting sort on the top D free bits,
// then each digit range is finished by insertion sort (<= 32 keys) or a
// block bitonic sort; the run-length pass finds head/tail positions with one
// block scan and writes (key, count) over the bin's own key range.
__device__ void bin_sorted(Node* nodes, uint32_t ni, const Node& nd, uint64_t* keys, uint32_t* cnt,
                           unsigned long long* skeys, uint32_t* hist, uint32_t* tmp,
                           uint32_t* mark, uint16_t* defer, uint32_t* n_defer, bool hot) {
  const uint32_t n = (uint32_t)nd.n;
  DK_PHASE_BEGIN();
  int D = ceil_log2_u64(n);
  D = max(4, min(D, kBinDigitBits));
  D = min(D, (int)nd.shift);
  const int sh = nd.shift - D;
  const uint32_t R = 1u << D, M = R - 1;
  const uint32_t T = blockDim.x;
  for (uint32_t j = threadIdx.x; j < R; j += T) hist[j] = 0;
  __syncthreads();
  DK_PHASE(0);
  uint32_t i = threadIdx.x;
  for (; i + 3 * T < n; i += 4 * T) {
    const uint64_t k0 = __ldg(keys + i), k1 = __ldg(keys + i + T), k2 = __ldg(keys + i + 2 * T),
                   k3 = __ldg(keys + i + 3 * T);
    agg_add_u32(hist, (uint32_t)(k0 >> sh) & M, hot);
    agg_add_u32(hist, (uint32_t)(k1 >> sh) & M, hot);
    agg_add_u32(hist, (uint32_t)(k2 >> sh) & M, hot);
    agg_add_u32(hist, (uint32_t)(k3 >> sh) & M, hot);
  }
  for (; i < n; i += T) agg_add_u32(hist, (uint32_t)(__ldg(keys + i) >> sh) & M, hot);
  __syncthreads();
  DK_PHASE(1);
  block_scan_array<uint32_t>(hist, (int)R, tmp);
  DK_PHASE(2);
  i = threadIdx.x;
  for (; i + 3 * T < n; i += 4 * T) {
    const uint64_t k0 = __ldg(keys + i), k1 = __ldg(keys + i + T), k2 = __ldg(keys + i + 2 * T),
                   k3 = __ldg(keys + i + 3 * T);
    uint32_t p0 = agg_reserve_u32(hist, (uint32_t)(k0 >> sh) & M, hot);
    uint32_t p1 = agg_reserve_u32(hist, (uint32_t)(k1 >> sh) & M, hot);
    uint32_t p2 = agg_reserve_u32(hist, (uint32_t)(k2 >> sh) & M, hot);
    uint32_t p3 = agg_reserve_u32(hist, (uint32_t)(k3 >> sh) & M, hot);
    if (DK_OK_IDX(p0 < n && p1 < n && p2 < n && p3 < n, 11, n)) {
      skeys[p0] = k0; skeys[p1] = k1; skeys[p2] = k2; skeys[p3] = k3;
    }
  }
  for (; i < n; i += T) {
    const uint64_t k0 = __ldg(keys + i);
    const uint32_t p0 = agg_reserve_u32(hist, (uint32_t)(k0 >> sh) & M, hot);
    if (DK_OK_IDX(p0 < n, 12, n)) skeys[p0] = k0;
  }
  __syncthreads();
  DK_PHASE(3);
  // hist[j] is now the end of digit range j.  Within a range the keys are in
  // arbitrary order; mark the ranges that hold a descent (a key smaller than
  // its predecessor in the same range) and sort only those, one warp each.
  // A range made of one repeated k-mer has no descent and costs nothing.
  if (sh > 0) {
    for (uint32_t w = threadIdx.x; w < (R + 31) / 32; w += T) mark[w] = 0;
    if (threadIdx.x == 0) *n_defer = 0;
    __syncthreads();
    const uint32_t per_e = (n + T - 1) / T;
    const uint32_t e0 = min(n, threadIdx.x * per_e), e1 = min(n, e0 + per_e);
    unsigned long long prev = e0 ? skeys[e0 - 1] : 0ull;
    for (uint32_t x = e0; x < e1; ++x) {
      const unsigned long long v = skeys[x];
      if (x > 0 && (v >> sh) == (prev >> sh) && v < prev) {
        const uint32_t d = (uint32_t)(v >> sh) & M;
        atomicOr(&mark[d >> 5], 1u << (d & 31));
      }
      prev = v;
    }
    __syncthreads();
    DK_PHASE(4);
    // small marked ranges: sorted by the thread that owns the digit
    {
      const uint32_t per = (R + T - 1) / T;
      const uint32_t j0 = min(R, threadIdx.x * per), j1 = min(R, j0 + per);
      for (uint32_t j = j0; j < j1; ++j) {
        if (!(mark[j >> 5] & (1u << (j & 31)))) continue;
        const uint32_t lo = j ? hist[j - 1] : 0, hi = hist[j];
        if (!DK_OK_IDX(lo <= hi && hi <= n, 16, ((uint64_t)lo << 32) | hi)) continue;
        if (hi - lo > kThreadSortMax) continue;
        for (uint32_t x = lo + 1; x < hi; ++x) {
          const unsigned long long v = skeys[x];
          uint32_t y = x;
          while (y > lo && skeys[y - 1] > v) {
            skeys[y] = skeys[y - 1];
            --y;
          }
          skeys[y] = v;
        }
      }
    }
    __syncthreads();
    const uint32_t warp = threadIdx.x >> 5, nwarps = T >> 5;
    for (uint32_t w = warp; w < (R + 31) / 32; w += nwarps) {
      uint32_t bits = mark[w];
      while (bits) {
        const uint32_t j = w * 32 + (__ffs(bits) - 1);
        bits &= bits - 1;
        const uint32_t lo = j ? hist[j - 1] : 0, hi = hist[j];
        const uint32_t m = hi - lo;
        if (!DK_OK_IDX(lo <= hi && hi <= n && j < R, 13, ((uint64_t)lo << 32) | hi)) continue;
        if (m <= kThreadSortMax) continue;  // done above
        if (m <= 32) {
          warp_rank_sort(skeys + lo, m);
          DK_WARP_ADD(11, 1);
        } else if (!warp_sort_few_distinct<1>(skeys + lo, m)) {
          // many distinct keys: sorted below by the whole block
          uint32_t q = 0;
          if (lane_id() == 0) q = atomicAdd(n_defer, 1u);
          q = __shfl_sync(0xFFFFFFFFu, q, 0);
          if (q < kDeferMax) {
            if (lane_id() == 0) defer[q] = (uint16_t)j;
          } else {
            warp_bitonic(skeys + lo, m);
          }
          DK_WARP_ADD(13, 1);
          DK_WARP_ADD(14, m);
        } else {
          DK_WARP_ADD(12, 1);
          DK_WARP_ADD(15, m);
        }
      }
    }
    __syncthreads();
    const uint32_t nd_ = min(*n_defer, (uint32_t)kDeferMax);
    for (uint32_t q = 0; q < nd_; ++q) {
      const uint32_t j = defer[q];
      const uint32_t lo = j ? hist[j - 1] : 0, hi = hist[j];
      block_bitonic(skeys + lo, hi - lo);
    }
    __syncthreads();
    DK_PHASE(5);
  }
  // run-length reduce
  const uint32_t per = (n + T - 1) / T;
  const uint32_t lo = min(n, threadIdx.x * per), hi = min(n, lo + per);
  uint32_t heads = 0;
  int last_head = -1;
  for (uint32_t x = lo; x < hi; ++x)
    if (x == 0 || skeys[x] != skeys[x - 1]) { ++heads; last_head = (int)x; }
  uint32_t r0, total;
  int cur;
  DK_PHASE(6);
  block_scan_sum_max(heads, last_head, tmp, &r0, &cur, &total);
  DK_PHASE(7);
  int r = (int)r0 - 1;  // rank of the run that contains lo (when lo is not a head)
  for (uint32_t x = lo; x < hi; ++x) {
    const unsigned long long v = skeys[x];
    if (x == 0 || v != skeys[x - 1]) {
      ++r;
      cur = (int)x;
      if (DK_OK_IDX(r >= 0 && (uint32_t)r < n, 14, r)) keys[r] = v;
    }
    if (x == n - 1 || skeys[x + 1] != v)
      if (DK_OK_IDX(r >= 0 && (uint32_t)r < n && cur >= 0 && (uint32_t)cur <= x, 15, ((uint64_t)(uint32_t)r << 32) | (uint32_t)cur))
        cnt[r] = x - (uint32_t)cur + 1;
  }
  DK_PHASE(8);
  DK_PHASE_ADD(9, 1);
  DK_PHASE_ADD(10, n);
  if (threadIdx.x == 0) nodes[ni].d = total;
}

// ---- hash variant: aggregate the bin in a shared-memory hash table first
constexpr int kHashSlotBits = kBinCap >= 8192 ? 12 : 11;
constexpr uint32_t kHashSlots = 1u << kHashSlotBits;  // table slots per bin
constexpr uint32_t kHashMaxProbe = 64;                // a longer probe sends the bin to sorting
// sorted pairs that fit beside the table (a multiple of 64)
constexpr uint32_t kHashMaxDistinct = ((kBinCap * 8 - kHashSlots * 12) / 12) & ~63u;
constexpr unsigned long long kEmptyKey = ~0ull;       // never a k-mer when k <= 31
static_assert(kHashSlots * 12 + kHashMaxDistinct * 12 <= kBinCap * 8,
              "table and sorted pairs share the bin's shared-memory region");
static_assert(kBinCap >= (1 << kDenseBits) * 8 / 8, "a dense bin's 2^kDenseBits u64 counters fit the region");

// (key, count) pair version of the warp bitonic sort
__device__ void warp_bitonic_pairs(unsigned long long* s, uint32_t* c, uint32_t m) {
  int lg = 0;
  while ((1u << lg) < m) ++lg;
  const uint32_t P = 1u << lg;
  for (int sz = 1; sz <= lg; ++sz) {
    const uint32_t hmask = (1u << (sz - 1)) - 1;
    for (uint32_t i = lane_id(); i < P / 2; i += 32) {
      const uint32_t a = ((i >> (sz - 1)) << sz) | (i & hmask);
      const uint32_t b = a ^ ((1u << sz) - 1);
      if (b < m && s[b] < s[a]) {
        const unsigned long long x = s[a]; s[a] = s[b]; s[b] = x;
        const uint32_t y = c[a]; c[a] = c[b]; c[b] = y;
      }
    }
    __syncwarp();
    for (int st = sz - 2; st >= 0; --st) {
      const uint32_t smask = (1u << st) - 1;
      for (uint32_t i = lane_id(); i < P / 2; i += 32) {
        const uint32_t a = ((i >> st) << (st + 1)) | (i & smask);
        const uint32_t b = a + (1u << st);
        if (b < m && s[b] < s[a]) {
          const unsigned long long x = s[a]; s[a] = s[b]; s[b] = x;
          const uint32_t y = c[a]; c[a] = c[b]; c[b] = y;
        }
      }
      __syncwarp();
    }
  }
}

constexpr uint32_t kRankMax = 256;  // longer digit ranges are sorted by a warp

// Aggregate the bin's keys in a shared-memory open-addressing table (linear
// probing on a multiplicative hash, 64-bit atomicCAS on the key, atomicAdd on
// its count; a new key also counts its digit, the top D free bits), place the
// distinct (key, count) pairs by digit (counting sort), and write each pair
// at its rank inside its digit range, found by comparing it with the range's
// other keys (ranges of more than kRankMax keys are sorted by a warp instead).
// Returns false, having written nothing, when a probe runs past
// kHashMaxProbe slots or the bin holds more than kHashMaxDistinct keys.
__device__ bool bin_hashed(Node* nodes, uint32_t ni, const Node& nd, uint64_t* keys, uint32_t* cnt,
                           unsigned long long* region, uint32_t* hist, uint32_t* tmp,
                           uint32_t* mark, uint32_t* flags, bool hot,
                           unsigned long long* overflow) {
  unsigned long long* tk = region;                                  // kHashSlots keys
  uint32_t* tc = reinterpret_cast<uint32_t*>(tk + kHashSlots);       // kHashSlots counts
  unsigned long long* sk = reinterpret_cast<unsigned long long*>(tc + kHashSlots);  // by digit
  uint32_t* sc = reinterpret_cast<uint32_t*>(sk + kHashMaxDistinct);
  const uint64_t n = nd.n;  // a big bin may hold 2^32 keys or more
  const uint32_t T = blockDim.x;
  DK_PHASE_BEGIN();
  // digits: the top D free bits, about n / 8 of them (ranks within a digit
  // range compare its few keys; the digit scan and marks shrink with R)
  int D = ceil_log2_u64(n) - 3;
  D = max(4, min(D, kBinDigitBits));
  D = min(D, (int)nd.shift);
  const int sh = nd.shift - D;
  const uint32_t R = 1u << D, M = R - 1;
  static_assert(kHashSlots % kBinThreads == 0, "slot loops");
  // slot loops step by kBinThreads (the launch's block size), so they unroll
  // into independent iterations (clear and place: bin count 23.23 -> 22.82 ms
  // on 2.4 G k-mers)
#pragma unroll
  for (uint32_t u = 0; u < kHashSlots / kBinThreads; ++u) {
    const uint32_t j = threadIdx.x + u * kBinThreads;
    tk[j] = kEmptyKey;
    tc[j] = 0;
  }
  for (uint32_t j = threadIdx.x; j < R; j += T) hist[j] = 0;
  for (uint32_t w = threadIdx.x; w < (R + 31) / 32; w += T) mark[w] = 0;
  if (threadIdx.x == 0) flags[1] = 0;
  __syncthreads();
  // keys in flight per thread: 12 x 512 covers a typical 4-6 K-key bin in one
  // trip (bin count 23.2 ms on 2.4 G k-mers, against 23.6 ms with 8, 23.3
  // with 10 and 23.4 with 16)
  constexpr int kBatch = 12;
  for (uint64_t i0 = 0; i0 < n; i0 += (uint64_t)kBatch * T) {
    // a failed table stops the pass early (a large bin would otherwise probe
    // the full table for every remaining key); warp-uniform exit
    if (__any_sync(0xFFFFFFFFu, *reinterpret_cast<volatile uint32_t*>(&flags[1]) != 0)) break;
    unsigned long long kk[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const uint64_t i = i0 + (uint64_t)u * T + threadIdx.x;
      kk[u] = i < n ? __ldg(keys + i) : kEmptyKey;
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (i0 + (uint64_t)u * T >= n) break;  // uniform: no lane has a key from here on
      const unsigned long long key = kk[u];
      bool live = key != kEmptyKey;
      uint32_t mult = 1;
      if (hot) {  // copies of one key in this warp insert once with their multiplicity
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        live = live && (int)lane_id() == __ffs(peers) - 1;
        mult = (uint32_t)__popc(peers);
      }
      if (!live) continue;
      uint32_t slot = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - kHashSlotBits));
      for (uint32_t probe = 0;; ++probe) {
        if (probe == kHashMaxProbe) {  // table too full (or adversarial keys): sort instead
          flags[1] = 1;
          break;
        }
        const unsigned long long prev = atomicCAS(&tk[slot], kEmptyKey, key);
        if (prev == kEmptyKey || prev == key) {
          if (atomicAdd(&tc[slot], mult) > 0xFFFFFFFFu - mult) atomicMax(overflow, 1ull);
          if (prev == kEmptyKey) atomicAdd(&hist[(uint32_t)(key >> sh) & M], 1u);
          break;
        }
        slot = (slot + 1) & (kHashSlots - 1);
      }
    }
  }
  __syncthreads();
  DK_PHASE(17);
  if (flags[1]) return false;
  const uint32_t d = block_scan_array<uint32_t>(hist, (int)R, tmp);  // distinct keys
  if (d > kHashMaxDistinct) return false;  // uniform: d is the block total
  DK_PHASE(18);
#pragma unroll
  for (uint32_t u = 0; u < kHashSlots / kBinThreads; ++u) {
    const uint32_t j = threadIdx.x + u * kBinThreads;
    const unsigned long long key = tk[j];
    if (key != kEmptyKey) {
      const uint32_t pos = atomicAdd(&hist[(uint32_t)(key >> sh) & M], 1u);
      if (DK_OK_IDX(pos < d, 31, pos)) { sk[pos] = key; sc[pos] = tc[j]; }
    }
  }
  __syncthreads();
  DK_PHASE(20);
  // hist[j] is now the end of digit range j; keys within a range are in
  // arbitrary order.  Each pair finds its rank among the range's keys (all
  // distinct) and goes straight to the output.  A range's pairs sit on
  // consecutive threads, so the comparisons read shared memory as
  // broadcasts; ranges of more than kRankMax keys are marked instead.
  for (uint32_t x = threadIdx.x; x < d; x += T) {
    const unsigned long long v = sk[x];
    const uint32_t j = (uint32_t)(v >> sh) & M;
    const uint32_t lo = j ? hist[j - 1] : 0, hi = hist[j];
    if (hi - lo > kRankMax) {
      atomicOr(&mark[j >> 5], 1u << (j & 31));
      continue;
    }
    uint32_t r = lo;
    for (uint32_t y = lo; y < hi; ++y) r += sk[y] < v;
    if (DK_OK_IDX(r < d, 32, r)) {
      keys[r] = v;
      cnt[r] = sc[x];
    }
  }
  __syncthreads();
  DK_PHASE(21);
  const uint32_t warp = threadIdx.x >> 5, nwarps = T >> 5;
  for (uint32_t w = warp; w < (R + 31) / 32; w += nwarps) {
    uint32_t bits = mark[w];
    while (bits) {
      const uint32_t j = w * 32 + (__ffs(bits) - 1);
      bits &= bits - 1;
      const uint32_t lo = j ? hist[j - 1] : 0, hi = hist[j];
      if (!DK_OK_IDX(lo <= hi && hi <= d, 33, ((uint64_t)lo << 32) | hi)) continue;
      warp_bitonic_pairs(sk + lo, sc + lo, hi - lo);
      for (uint32_t x = lo + lane_id(); x < hi; x += 32) {
        keys[x] = sk[x];
        cnt[x] = sc[x];
      }
    }
  }
  DK_PHASE(22);
  DK_PHASE_ADD(24, 1);
  DK_PHASE_ADD(25, n);
  DK_PHASE_ADD(26, d);
  if (threadIdx.x == 0) nodes[ni].d = d;
  return true;
}

// ---- packed hash bins: one 64-bit word per distinct key
// A bin's keys share their bits [s, 2k) (s = nd.shift free bits), so a key is
// its low s bits.  Entry = (free bits << (64 - s)) | count: the free bits sit
// at the top, the count at the bottom.  Entries compare as the keys they
// hold, 0 is an empty slot, a new key enters with one 64-bit CAS and a repeat
// adds to the low 32-bit word.  With s <= 50 the count field (>= 14 bits)
// holds any count of a bin of at most kBinCap keys; with more free bits (bins
// of small read sets, which few levels split) the field is narrower, every
// add checks it, and a bin whose count would not fit is left to k_bin_count.
// Normal bins are counted this way by their own kernel (k_bin_packed), whose
// small shared-memory footprint (53 KB) and 30 registers fit four 512-thread
// CTAs per SM: a bin's work is a chain of dependent shared-memory steps, so
// bins in flight are what pays (2.4 G keys of large_100m: 20.1 ms with 4
// CTAs, 21.9 ms with 3 CTAs of a 5,120-slot table, 21.5 ms with 2 keys per
// thread per batch; the general kernel at 2 CTAs: 22.8 ms).  Bins it cannot
// take go to a list that k_bin_count handles after it.
#ifndef DK_PACK_SLOTS
#define DK_PACK_SLOTS 4096
#define DK_PACK_SLOT_BITS 12
#define DK_PACK_MAXD 2048
#define DK_PACK_CTAS 4
#endif
constexpr uint32_t kPackSlots = DK_PACK_SLOTS;        // table slots (32 KB)
constexpr int kPackSlotBits = DK_PACK_SLOT_BITS;
constexpr uint32_t kPackMaxDistinct = DK_PACK_MAXD;   // sorted entries (16 KB): load <= 0.5
constexpr int kPackDigitBits = 10;                    // counting-sort digits (4 KB)
constexpr uint32_t kPackMaxProbe = 64;
constexpr int kPackWideShift = 50;  // up to here the count field holds >= 14 bits
constexpr int kPackMaxShift = 62;   // beyond: at most 1 count bit, not worth a try
constexpr int kPackThreads = 512;
constexpr int kPackBlocksPerSM = DK_PACK_CTAS;
#ifndef DK_PACK_BATCH
#define DK_PACK_BATCH 4
#endif
constexpr int kPackBatch = DK_PACK_BATCH;  // keys a thread loads before inserting them
constexpr size_t kPackSmem = kPackSlots * 8 + kPackMaxDistinct * 8 + (4u << kPackDigitBits);
static_assert(kBinCap < (1 << (64 - kPackWideShift)), "a bin's largest count fits a wide field");
static_assert(kPackMaxDistinct * 12 <= kPackSlots * 8, "the output stage fits the table");
static_assert(kPackSlots % (2 * kPackThreads) == 0, "slot loops");
static_assert(kPackSlots == (1u << kPackSlotBits), "the probe cursor masks its slot");
static_assert(kPackDigitBits <= 32, "digits come from the entry's high word");

// Insert one occurrence of a key (rk = key << (64 - s)); false when the probe
// runs past kPackMaxProbe slots or (kNarrow: a count field of at most cmax)
// its count would not fit.  A new key enters with count 1 and counts its
// digit, the top D bits of rk (hist[(rk >> 32) >> dsh32], dsh32 = 32 - D).
// The probe walks a cursor whose low bits are the slot.  kNarrow: the count
// field may carry (s > kPackWideShift; cmax >= 3, since s <= kPackMaxShift);
// the wide form skips those checks (C2: bin count 21.30 -> 21.14 ms).
template <bool kNarrow>
__device__ __forceinline__ bool pack_insert(unsigned long long* tab, unsigned long long rk,
                                           unsigned long long himask, uint32_t* hist, int dsh32,
                                           uint32_t cmax) {
  const uint32_t hi = (uint32_t)(rk >> 32);
  const uint32_t h = (hi ^ (uint32_t)rk) * 0x9E3779B1u;
  uint32_t slot = h >> (32 - kPackSlotBits);  // h scaled to [0, kPackSlots)
  for (const uint32_t end = slot + kPackMaxProbe; slot != end; ++slot) {
#ifdef DK_PHASE_TIMING
    {  // probe steps: lanes (g_phase[0]) and warp iterations (g_phase[3])
      const unsigned am = __activemask();
      if (lane_id() == __ffs(am) - 1) {
        atomicAdd(&g_phase[0], (unsigned long long)__popc(am));
        atomicAdd(&g_phase[3], 1ull);
      }
    }
#endif
    unsigned long long* const p = &tab[slot & (kPackSlots - 1)];
    unsigned long long e = *reinterpret_cast<volatile unsigned long long*>(p);
    if (e == 0ull) {
      e = atomicCAS(p, 0ull, rk | 1ull);
      if (e == 0ull) {
        atomicAdd(&hist[hi >> dsh32], 1u);
        return true;
      }
    }
    if ((e & himask) == rk) {
      unsigned int* lo = reinterpret_cast<unsigned int*>(p);  // the low word
      if (!kNarrow) {
        atomicAdd(lo, 1u);
        return true;
      }
      // a carry out of a narrow field corrupts the entry: the bin is dropped
      return (atomicAdd(lo, 1u) & cmax) + 1u <= cmax;
    }
  }
  return false;
}

// Insert a bin's keys[0, n) into the packed table, kPackBatch keys per thread
// at a time.  flags[1] is set when the bin fails (a long probe, a full count
// field), and every thread then stops inserting at its next batch: the bin's
// keys are counted again elsewhere.  A bin with more distinct keys than the
// sorted stage holds is caught after the digit scan, and a full table ends
// every probe at kPackMaxProbe slots, so nothing is tallied per batch (a
// per-warp tally of new keys cost 17.34 against 16.73 ms on large_100m).  The
// count field's width is chosen once per bin, outside the key loop.  There is
// no warp-wide call per key either: copies of a hot k-mer in one warp add to
// their entry one by one.  A hot-k-mer path (__match_any_sync per key, copies
// inserted once with their multiplicity, in warps whose first 32 keys repeat
// one key four times) made the whole kernel slower even where no warp took
// it: large_100m bin count 17.35 ms without it against 20.90-20.98 ms with it
// (inline, or as a second loop chosen per warp); Zipf-skewed reads (k = 31,
// 17) 8.36 / 9.66 ms against 10.45 / 12.06.  Nodes made of one hot k-mer are
// counted by k_bin_count.
template <bool kNarrow>
__device__ __forceinline__ void pack_insert_keys(unsigned long long* tab, const uint64_t* keys,
                                                 uint32_t n, int cbits,
                                                 unsigned long long himask, uint32_t* hist,
                                                 int dsh32, uint32_t cmax, uint32_t* flags) {
  constexpr uint32_t T = kPackThreads;
  constexpr int kBatch = kPackBatch;
  bool ok = true;
  for (uint32_t i0 = 0; i0 < n; i0 += kBatch * T) {
    if (*reinterpret_cast<volatile uint32_t*>(&flags[1])) ok = false;
    unsigned long long rk[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const uint32_t i = i0 + (uint32_t)u * T + threadIdx.x;
      rk[u] = i < n ? __ldg(keys + i) << cbits : 0ull;
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (i0 + (uint32_t)u * T >= n) break;  // uniform
      if (i0 + (uint32_t)u * T + threadIdx.x < n && ok)
        ok = pack_insert<kNarrow>(tab, rk[u], himask, hist, dsh32, cmax);
    }
    if (!ok) flags[1] = 1;
  }
}

// One bin with at most kBinCap keys and kDenseBits < s <= kPackMaxShift free
// bits: insert every key into the packed table, place the distinct entries by
// their top D bits (counting sort), rank each inside its digit range, stage
// the sorted (key, count) pairs in the freed table and write them to the
// bin's region with coalesced stores.  Returns false, having written nothing,
// when a probe runs too long, a count outgrows a narrow field or the bin
// holds more than kPackMaxDistinct keys.
__device__ bool bin_packed(Node* nodes, uint32_t ni, const Node& nd, uint64_t* keys, uint32_t* cnt,
                           unsigned long long* region, uint32_t* tmp, uint32_t* mark,
                           uint32_t* flags) {
  constexpr uint32_t T = kPackThreads;
  unsigned long long* tab = region;                                          // kPackSlots
  unsigned long long* sorted = region + kPackSlots;                          // by digit
  uint32_t* hist = reinterpret_cast<uint32_t*>(sorted + kPackMaxDistinct);   // 2^D
  const uint32_t n = (uint32_t)nd.n;
  const int s = nd.shift;
  const int cbits = 64 - s;
  const unsigned long long himask = ~((1ull << cbits) - 1ull);
  const uint32_t cmask = cbits >= 32 ? 0xFFFFFFFFu : ((1u << cbits) - 1u);
  const uint32_t cmax = s > kPackWideShift ? cmask : 0u;  // a narrow count field
  int D = ceil_log2_u64(n) - 3;
  D = max(4, min(D, kPackDigitBits));
  D = min(D, s);
  const int dsh32 = 32 - D;  // an entry's digit: its high word >> dsh32
  const uint32_t R = 1u << D;
  const uint64_t prefix = n ? (__ldg(keys) >> s) << s : 0ull;
  DK_PHASE_BEGIN();
  {
    uint4* t4 = reinterpret_cast<uint4*>(tab);
#pragma unroll
    for (uint32_t u = 0; u < kPackSlots / 2 / T; ++u)
      t4[threadIdx.x + u * T] = make_uint4(0u, 0u, 0u, 0u);
  }
  for (uint32_t j = threadIdx.x; j < R; j += T) hist[j] = 0;
  for (uint32_t w = threadIdx.x; w < (R + 31) / 32; w += T) mark[w] = 0;
  if (threadIdx.x == 0) flags[1] = 0;  // the bin has failed
  __syncthreads();
  DK_PHASE(11);
  if (cmax)
    pack_insert_keys<true>(tab, keys, n, cbits, himask, hist, dsh32, cmax, flags);
  else
    pack_insert_keys<false>(tab, keys, n, cbits, himask, hist, dsh32, cmax, flags);
  __syncthreads();
  DK_PHASE(12);
  if (flags[1]) return false;
  const uint32_t d = block_scan_array<uint32_t>(hist, (int)R, tmp);  // distinct keys
  if (d > kPackMaxDistinct) return false;  // uniform
  DK_PHASE(13);
  // place: hist[j] becomes the end of digit range j
  {
    const ulonglong2* t2 = reinterpret_cast<const ulonglong2*>(tab);
#pragma unroll
    for (uint32_t u = 0; u < kPackSlots / 2 / T; ++u) {
      const ulonglong2 e = t2[threadIdx.x + u * T];
      if (e.x) sorted[atomicAdd(&hist[(uint32_t)(e.x >> 32) >> dsh32], 1u)] = e.x;
      if (e.y) sorted[atomicAdd(&hist[(uint32_t)(e.y >> 32) >> dsh32], 1u)] = e.y;
    }
  }
  __syncthreads();
  DK_PHASE(14);
  // rank inside the digit range and stage the pair (the table is free now);
  // ranges of more than kRankMax entries are marked for a warp sort
  unsigned long long* ok_ = tab;                          // d keys
  uint32_t* oc = reinterpret_cast<uint32_t*>(tab + d);    // d counts
  for (uint32_t x = threadIdx.x; x < d; x += T) {
    const unsigned long long v = sorted[x];
    const uint32_t j = (uint32_t)(v >> 32) >> dsh32;
    const uint32_t lo = j ? hist[j - 1] : 0, hi = hist[j];
    if (hi - lo > kRankMax) {
      atomicOr(&mark[j >> 5], 1u << (j & 31));
      continue;
    }
    uint32_t r = lo;
    for (uint32_t y = lo; y < hi; ++y) r += sorted[y] < v;
    DK_WARP_ADD(2, hi - lo);  // rank comparisons, lane 0's (instrumented builds)
    ok_[r] = prefix | (v >> cbits);
    oc[r] = (uint32_t)v & cmask;
  }
  __syncthreads();
  DK_PHASE(15);
  const uint32_t warp = threadIdx.x >> 5;
  for (uint32_t w = warp; w < (R + 31) / 32; w += T / 32) {
    uint32_t bits = mark[w];
    while (bits) {
      const uint32_t j = w * 32 + (__ffs(bits) - 1);
      bits &= bits - 1;
      const uint32_t lo = j ? hist[j - 1] : 0, hi = hist[j];
      warp_bitonic(sorted + lo, hi - lo);
      for (uint32_t x = lo + lane_id(); x < hi; x += 32) {
        const unsigned long long v = sorted[x];
        ok_[x] = prefix | (v >> cbits);
        oc[x] = (uint32_t)v & cmask;
      }
    }
  }
  __syncthreads();
  DK_PHASE(16);
  for (uint32_t x = threadIdx.x; x < d; x += T) {
    keys[x] = ok_[x];
    cnt[x] = oc[x];
  }
  DK_PHASE(19);
  DK_PHASE_ADD(23, 1);
  DK_PHASE_ADD(27, n);
  DK_PHASE_ADD(28, d);
  if (threadIdx.x == 0) nodes[ni].d = d;
  return true;
}

// Persistent packed-bin counter over the final list: CTAs take bins by
// ticket (ctr[19]); while the CTA counts one bin, one thread takes the next
// ticket, stages that bin's node in shared memory and pulls its keys into L2.
// Bins it does not count -- dense ones (at most kDenseBits free bits), ones
// with more than kPackMaxShift free bits, and ones the packed table cannot
// hold -- are appended to fb_list (ctr[20] entries) for k_bin_count; ctr[21]
// counts the bins it finished and ctr[22] the ones it left, over all passes.
__global__ void __launch_bounds__(kPackThreads, kPackBlocksPerSM)
    k_bin_packed(Node* nodes, const uint32_t* __restrict__ finals, uint32_t n_bins, uint64_t* A,
                 uint64_t* B, uint32_t* C, unsigned long long* ctr, uint32_t* fb_list,
                 const uint32_t* n_bins_dev) {
  extern __shared__ __align__(16) unsigned long long region[];
  __shared__ uint32_t tmp[64];
  __shared__ uint32_t mark[(1u << kPackDigitBits) / 32];
  __shared__ uint32_t flags[2];
  // the current and the next bin: ticket, node index and node, so that one
  // thread fetches the next bin's node while the CTA counts the current one
  __shared__ uint32_t s_b[2], s_ni[2];
  __shared__ Node s_node[2];
  // with n_bins_dev the final list's length is only known on the device
  if (n_bins_dev) n_bins = *n_bins_dev;
  unsigned int* ticket = reinterpret_cast<unsigned int*>(&ctr[19]);
  auto take = [&](int slot) {
    const uint32_t nb = atomicAdd(ticket, 1u);
    s_b[slot] = nb;
    if (nb < n_bins) {
      const uint32_t nn = finals[nb];
      const Node nx = nodes[nn];
      s_ni[slot] = nn;
      s_node[slot] = nx;
      prefetch_l2_range((nx.buf ? B : A) + nx.start, nx.n * 8);
    }
  };
  if (threadIdx.x == 32) take(0);
  __syncthreads();
  for (int cur = 0;; cur ^= 1) {
    const uint32_t b = s_b[cur];
    if (b >= n_bins) break;
    const uint32_t ni = s_ni[cur];
    const Node nd = s_node[cur];
    uint64_t* keys = (nd.buf ? B : A) + nd.start;
    uint32_t* cnt = C + nd.start;
    if (threadIdx.x == 32) take(cur ^ 1);
    const bool eligible = nd.shift > kDenseBits && nd.shift <= kPackMaxShift &&
                          nd.n <= (uint64_t)kBinCap;
    bool done = false;
    if (eligible) done = bin_packed(nodes, ni, nd, keys, cnt, region, tmp, mark, flags);
    if (threadIdx.x == 0) {
      if (done) {
        atomicAdd(&ctr[21], 1ull);
      } else {
        fb_list[atomicAdd(reinterpret_cast<unsigned int*>(&ctr[20]), 1u)] = ni;
        atomicAdd(&ctr[22], 1ull);
      }
    }
    __syncthreads();
  }
}

// Persistent bin counter: CTAs take final nodes from a ticket until none are
// left.  Two CTAs fit per SM (96 KB keys + 16 KB histogram each).
__device__ __forceinline__ uint32_t bin_at(const uint32_t* big, uint32_t n_big,
                                           const uint32_t* finals, uint32_t b) {
  return b < n_big ? big[b] : finals[b - n_big];
}

__global__ void __launch_bounds__(kBinThreads, kBinBlocksPerSM) k_bin_count(Node* nodes,
                                                              const uint32_t* __restrict__ bigs,
                                                              uint32_t n_big,
                                                              const uint32_t* __restrict__ finals,
                                                              uint32_t n_bins, uint64_t* A,
                                                              uint64_t* B, uint32_t* C,
                                                              unsigned long long* ctr,
                                                              int use_hash,
                                                              const unsigned int* n_finals_dev,
                                                              const uint32_t* n_big_dev) {
  extern __shared__ __align__(16) unsigned long long skeys[];  // kBinCap keys / 4096 u64 counts
  __shared__ uint32_t hist[1u << kBinDigitBits];
  __shared__ uint32_t tmp[64];
  __shared__ uint32_t mark[(1u << kBinDigitBits) / 32];
  __shared__ uint16_t defer[kDeferMax];
  __shared__ uint32_t s_bin, n_defer;
  __shared__ uint32_t hflags[2];
  __shared__ bool s_hot;
  // with n_finals_dev the final list's length is only known on the device
  // (the packed bins' fallback list)
  if (n_big_dev) n_big = *n_big_dev;
  if (n_finals_dev) n_bins = n_big + *n_finals_dev;
  if (threadIdx.x == 0) s_bin = atomicAdd(reinterpret_cast<unsigned int*>(&ctr[4]), 1u);
  __syncthreads();
  for (;;) {
    const uint32_t b = s_bin;
    if (b >= n_bins) break;
    const uint32_t ni = bin_at(bigs, n_big, finals, b);
    const Node nd = nodes[ni];
    uint64_t* keys = (nd.buf ? B : A) + nd.start;
    uint32_t* cnt = C + nd.start;
    __syncthreads();  // every thread has read s_bin
    if (threadIdx.x == 32) {
      // take the next bin now and start pulling its keys into L2 while this one runs
      const uint32_t nb = atomicAdd(reinterpret_cast<unsigned int*>(&ctr[4]), 1u);
      s_bin = nb;
      if (nb < n_bins) {
        const Node& nx = nodes[bin_at(bigs, n_big, finals, nb)];
        prefetch_l2_range((nx.buf ? B : A) + nx.start, nx.n * 8);
      }
    }
    // hot bin: a sample of 32 keys spread over the bin repeats one key >= 4
    // times; its atomics are then aggregated per warp
    if (threadIdx.x < 32) {
      const uint64_t smp = nd.n ? __ldg(keys + (nd.n * threadIdx.x) / 32) : 0ull;
      const uint32_t peers = __match_any_sync(0xFFFFFFFFu, smp);
      const uint32_t dup = __reduce_max_sync(0xFFFFFFFFu, (uint32_t)__popc(peers));
      if (threadIdx.x == 0) s_hot = dup >= 4;
    }
    __syncthreads();
    const bool hot = s_hot;
    if (nd.shift <= kDenseBits) {
      bin_dense(nodes, ni, nd, keys, cnt, skeys, reinterpret_cast<unsigned long long*>(tmp),
                &ctr[5]);
    } else if (nd.n > (uint64_t)kBinCap) {
      // a large skewed bin: the hash bin streams its keys; with too many
      // distinct keys it is left, unwritten, for the host to re-partition
      const bool done = bin_hashed(nodes, ni, nd, keys, cnt, skeys, hist, tmp, mark, hflags, hot,
                                   &ctr[5]);
      if (threadIdx.x == 0) {
        atomicAdd(&ctr[17], 1ull);
        if (!done) {
          nodes[ni].state = NODE_RETRY;
          atomicAdd(&ctr[7], 1ull);
        }
      }
    } else {
      bool done = false;
      if (use_hash) {
        done = bin_hashed(nodes, ni, nd, keys, cnt, skeys, hist, tmp, mark, hflags, hot, &ctr[5]);
        if (!done && threadIdx.x == 0) atomicAdd(&ctr[6], 1ull);  // bins that fell back
        __syncthreads();
      }
      // the sort path counts its digits without per-warp aggregation: a bin
      // here holds at most kBinCap keys, so a hot k-mer's adds stay few, and
      // the aggregated form made every bin slower (large_100m, sort variant:
      // 92.7 -> 89.8 ms; Zipf k = 31: 20.1 -> 18.7 ms)
      if (!done) bin_sorted(nodes, ni, nd, keys, cnt, skeys, hist, tmp, mark, defer, &n_defer, false);
    }
    __syncthreads();
  }
}

// ----------------------------------------------------- tree reductions
// one warp per node: a split node's distinct keys are its children's
__device__ __forceinline__ void aggregate_node(Node* nodes, uint32_t i) {
  const uint32_t state = nodes[i].state;
  if (state != NODE_SPLIT) return;
  const uint32_t R = 1u << nodes[i].width, fc = nodes[i].first_child;
  unsigned long long d = 0;
  for (uint32_t j = lane_id(); j < R; j += 32) d += nodes[fc + j].d;
#pragma unroll
  for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xFFFFFFFFu, d, o);
  if (lane_id() == 0) nodes[i].d = d;
}

__global__ void k_aggregate(Node* nodes, uint32_t lo, uint32_t hi) {
  const uint32_t i = lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (i >= hi) return;  // warp-uniform
  aggregate_node(nodes, i);
}

// output offsets of level-1 nodes [b0, b1): they follow the *total_d distinct
// keys placed before them, and *total_d grows by theirs
__device__ __forceinline__ void l1_out_offsets_body(Node* nodes, uint32_t b0, uint32_t b1,
                                                    unsigned long long* total_d,
                                                    unsigned long long* tmp) {
  const uint32_t n1 = b1 - b0;
  const unsigned long long before = *total_d;
  const uint32_t per = (n1 + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = b0 + min(n1, threadIdx.x * per), hi = min(b1, lo + per);
  unsigned long long s = 0;
  for (uint32_t i = lo; i < hi; ++i) s += nodes[i].d;
  unsigned long long tot;
  // the block scan synchronises: every thread has read *total_d before it changes
  unsigned long long base = before + block_excl_scan<unsigned long long>(s, tmp, &tot);
  for (uint32_t i = lo; i < hi; ++i) {
    nodes[i].out_off = base;
    base += nodes[i].d;
  }
  if (threadIdx.x == 0) *total_d = before + tot;
}

__global__ void k_l1_out_offsets(Node* nodes, uint32_t b0, uint32_t b1,
                                 unsigned long long* total_d) {
  __shared__ unsigned long long tmp[32];
  l1_out_offsets_body(nodes, b0, b1, total_d, tmp);
}

__device__ __forceinline__ void child_offsets_one(Node* nodes, uint32_t i,
                                                  unsigned long long* tmp) {
  const Node nd = nodes[i];
  if (nd.state != NODE_SPLIT) return;
  const uint32_t R = 1u << nd.width;
  const uint32_t per = (R + blockDim.x - 1) / blockDim.x;
  const uint32_t j0 = min(R, threadIdx.x * per), j1 = min(R, j0 + per);
  unsigned long long s = 0;
  for (uint32_t j = j0; j < j1; ++j) s += nodes[nd.first_child + j].d;
  unsigned long long base = nd.out_off + block_excl_scan<unsigned long long>(s, tmp, nullptr);
  for (uint32_t j = j0; j < j1; ++j) {
    Node& ch = nodes[nd.first_child + j];
    ch.out_off = base;
    base += ch.d;
  }
}

__global__ void __launch_bounds__(256) k_child_offsets(Node* nodes, uint32_t lo) {
  __shared__ unsigned long long tmp[32];
  child_offsets_one(nodes, lo + blockIdx.x, tmp);
}

// Re-partition NODE_RETRY nodes: each gets a proxy copy appended after the
// existing nodes (which then splits like any other node) and becomes a split
// node of width 0 whose one child is that proxy, so the tree passes sum and
// place its keys through the proxy.
__global__ void k_make_proxies(Node* nodes, const uint32_t* __restrict__ finals, uint32_t n_final,
                               uint32_t n_nodes, unsigned int* count) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n_final) return;
  const uint32_t i = finals[f];
  if (nodes[i].state != NODE_RETRY) return;
  const uint32_t j = n_nodes + atomicAdd(count, 1u);
  Node px = nodes[i];
  px.d = 0;
  px.out_off = 0;
  px.first_child = 0;
  px.state = 0;
  px.tile_base = 0;
  px.ntiles = 0;
  px.th_base = 0;
  px.width = 0;
  px.skewed = 0;  // split normally from here
  nodes[j] = px;
  nodes[i].state = NODE_SPLIT;
  nodes[i].width = 0;
  nodes[i].first_child = j;
}

// one warp per final node: staged pairs -> output table
__device__ __forceinline__ void compact_one(const Node* nodes, uint32_t ni, const uint64_t* A,
                                            const uint64_t* B, const uint32_t* C,
                                            uint64_t* __restrict__ out_k,
                                            uint32_t* __restrict__ out_c) {
  const Node nd = nodes[ni];
  if (nd.state != NODE_FINAL) return;  // re-partitioned after its bin count failed
  const uint64_t* __restrict__ sk = (nd.buf ? B : A) + nd.start;
  const uint32_t* __restrict__ sc = C + nd.start;
  // both loads of a pair are issued before its stores (read-only path: the
  // staged pairs were written by an earlier kernel)
  for (uint64_t i = lane_id(); i < nd.d; i += 32) {
    const uint64_t kv = __ldg(sk + i);
    const uint32_t cv = __ldg(sc + i);
    out_k[nd.out_off + i] = kv;
    out_c[nd.out_off + i] = cv;
  }
}

__global__ void k_compact(const Node* nodes, const uint32_t* __restrict__ finals, uint32_t n_final,
                          const uint64_t* A, const uint64_t* B, const uint32_t* C,
                          uint64_t* __restrict__ out_k, uint32_t* __restrict__ out_c) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= n_final) return;
  compact_one(nodes, finals[w], A, B, C, out_k, out_c);
}

// ------------------------------------------------ graph-driven wave tail
// The kernels of a wave graph: each reads the extents it works on from the
// WaveCtl and loops over them with a grid fixed when the graph was built.

// A level begins: its node range (the range the previous level's plan set)
// and its counters cleared (n_final and n_big_final run over all levels).
__global__ void k_g_level_begin(LevelCounters* lc, WaveCtl* wc) {
  if (threadIdx.x || blockIdx.x || wc->stop) return;
  if (wc->n_levels) {
    wc->lo = wc->next_lo;
    wc->hi = wc->next_hi;
  }
  lc->n_split = 0;
  lc->n_tiles = 0;
  lc->too_big = 0;
  lc->n_children = 0;
  lc->max_width = 0;
  lc->split_keys = 0;
  lc->th_entries = 0;
  lc->n_tiles_assigned = 0;
  lc->n_children_assigned = 0;
  lc->th_assigned = 0;
}

__global__ void k_g_classify(Node* nodes, uint32_t* finals, uint32_t* bigs, LevelCounters* lc,
                             int bin_cap, int split_target, int big_ok, const WaveCtl* wc) {
  if (wc->stop) return;
  const uint32_t lo = wc->lo, hi = wc->hi;
  const Ranges rg{nullptr, nullptr, 0, 0};
  for (uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi;
       i += gridDim.x * blockDim.x)
    classify_node(nodes, i, finals, bigs, lc, bin_cap, split_target, big_ok, rg,
                  kGraphSplitBits);
}

// What the host does between classify and assign: record the level, end the
// loop when nothing splits (or a buffer would overflow), else lay out the
// children and tiles of the split nodes.  One thread.
__global__ void k_g_plan(LevelCounters* lc, WaveCtl* wc, cudaGraphConditionalHandle h) {
  if (threadIdx.x || blockIdx.x) return;
  if (wc->stop) {
    cudaGraphSetConditional(h, 0);
    return;
  }
  const uint32_t L = wc->n_levels;
  bool end = false;
  if (L >= (uint32_t)kGraphMaxLevels) {
    wc->overflow = 1;
    end = true;
  } else {
    wc->lv_lo[L] = wc->lo;
    wc->lv_hi[L] = wc->hi;
    wc->n_levels = L + 1;
    if (lc->too_big) {
      wc->too_big = 1;
      end = true;
    } else if (lc->n_split == 0) {
      end = true;
    } else if ((unsigned long long)wc->node_end + lc->n_children > wc->nodes_cap ||
               lc->n_tiles > wc->tiles_cap || lc->th_entries > wc->th_cap) {
      wc->overflow = 1;
      end = true;
    }
  }
  if (end) {
    wc->stop = 1;
    if (wc->overflow || wc->too_big) {  // nothing after the levels runs
      lc->n_final = 0;
      lc->n_big_final = 0;
    }
    cudaGraphSetConditional(h, 0);
    return;
  }
  wc->split_keys += lc->split_keys;
  wc->n_tiles = lc->n_tiles;
  wc->tk_hist = 0;
  wc->tk_scatter = 0;
  wc->child_base = wc->node_end;
  wc->next_lo = wc->node_end;
  wc->next_hi = wc->node_end + lc->n_children;
  wc->node_end = wc->next_hi;
}

__global__ void k_g_assign(Node* nodes, Tile* tiles, LevelCounters* lc, const WaveCtl* wc) {
  if (wc->stop) return;
  const uint32_t lo = wc->lo, hi = wc->hi, cb = wc->child_base;
  const Ranges rg{nullptr, nullptr, 0, 0};
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < hi; i += nw)
    assign_node(nodes, i, cb, tiles, lc, rg);  // warp-uniform
}

// the next work ticket of the block (thread 0 takes it, all threads get it)
__device__ __forceinline__ uint32_t block_ticket(uint32_t* tk, uint32_t* s_t) {
  if (threadIdx.x == 0) *s_t = atomicAdd(tk, 1u);
  __syncthreads();
  const uint32_t t = *s_t;
  __syncthreads();  // every thread has read it before it is replaced
  return t;
}

__global__ void __launch_bounds__(256) k_g_tile_hist(const Node* nodes, const Tile* tiles,
                                                     const uint64_t* A, const uint64_t* B,
                                                     uint32_t* TH, WaveCtl* wc) {
  __shared__ uint32_t hist[1u << kMaxSplitBits];
  __shared__ uint32_t s_t;
  if (wc->stop) return;
  const uint32_t nt = wc->n_tiles;
  for (uint32_t t = block_ticket(&wc->tk_hist, &s_t); t < nt; t = block_ticket(&wc->tk_hist, &s_t)) {
    tile_hist_one(nodes, tiles, t, A, B, TH, hist);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_g_node_scan(Node* nodes, Tile* tiles, uint32_t* TH,
                                                     const WaveCtl* wc) {
  __shared__ unsigned long long csize[1u << kMaxSplitBits];
  __shared__ unsigned long long tmp[32];
  if (wc->stop) return;
  const uint32_t lo = wc->lo, hi = wc->hi;
  for (uint32_t i = lo + blockIdx.x; i < hi; i += gridDim.x) {
    node_scan_one(nodes, i, tiles, TH, csize, tmp);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kTileThreads, DK_TILE_CTAS) k_g_tile_scatter(
    const Node* nodes, const Tile* tiles, uint64_t* A, uint64_t* B, const uint32_t* TH,
    WaveCtl* wc) {
  extern __shared__ __align__(16) unsigned long long dsm[];
  __shared__ uint32_t tmp[32];
  __shared__ uint32_t s_t;
  if (wc->stop) return;
  const uint32_t nt = wc->n_tiles;
  for (uint32_t t = block_ticket(&wc->tk_scatter, &s_t); t < nt;
       t = block_ticket(&wc->tk_scatter, &s_t)) {
    tile_scatter_one(nodes, tiles, t, A, B, TH, kGraphSplitBits, dsm, tmp);
    __syncthreads();
  }
}

// Tree passes over the recorded levels: bottom-up (up = 1, distinct counts)
// from the last splitting level, top-down (up = 0, offsets) from level 0.
__global__ void k_g_pass_begin(WaveCtl* wc, int up) {
  if (threadIdx.x || blockIdx.x) return;
  wc->pass = up ? (int)wc->n_levels - 2 : 0;
  wc->tk_compact[0] = 0;
  wc->tk_compact[1] = 0;
}

__global__ void k_g_pass_step(WaveCtl* wc, cudaGraphConditionalHandle h, int up) {
  if (threadIdx.x || blockIdx.x) return;
  const int p = wc->pass, last = (int)wc->n_levels - 2;  // the levels that split
  if (wc->overflow || wc->too_big || p < 0 || p > last) {
    wc->pass_skip = 1;
    cudaGraphSetConditional(h, 0);
    return;
  }
  wc->pass_skip = 0;
  wc->cur_lo = wc->lv_lo[p];
  wc->cur_hi = wc->lv_hi[p];
  const int np = up ? p - 1 : p + 1;
  wc->pass = np;
  cudaGraphSetConditional(h, (np >= 0 && np <= last) ? 1u : 0u);
}

__global__ void k_g_aggregate(Node* nodes, const WaveCtl* wc) {
  if (wc->pass_skip) return;
  const uint32_t lo = wc->cur_lo, hi = wc->cur_hi;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < hi; i += nw)
    aggregate_node(nodes, i);  // warp-uniform
}

__global__ void __launch_bounds__(256) k_g_child_offsets(Node* nodes, const WaveCtl* wc) {
  __shared__ unsigned long long tmp[32];
  if (wc->pass_skip) return;
  const uint32_t lo = wc->cur_lo, hi = wc->cur_hi;
  for (uint32_t i = lo + blockIdx.x; i < hi; i += gridDim.x) {
    child_offsets_one(nodes, i, tmp);
    __syncthreads();
  }
}

__global__ void k_g_l1_offsets(Node* nodes, unsigned long long* total_d, const WaveCtl* wc) {
  __shared__ unsigned long long tmp[32];
  if (wc->overflow || wc->too_big) return;
  l1_out_offsets_body(nodes, 0, wc->F1, total_d, tmp);
}

// one warp per node, nodes taken by ticket (*tk)
__global__ void k_g_compact(const Node* nodes, const uint32_t* __restrict__ finals,
                            const uint32_t* n_dev, uint32_t* tk, const uint64_t* A,
                            const uint64_t* B, const uint32_t* C, const WaveCtl* wc) {
  const uint32_t n = *n_dev;
  uint64_t* __restrict__ out_k = wc->out_k;
  uint32_t* __restrict__ out_c = wc->out_c;
  for (;;) {
    uint32_t w = 0;
    if (lane_id() == 0) w = atomicAdd(tk, 1u);
    w = __shfl_sync(0xFFFFFFFFu, w, 0);
    if (w >= n) break;  // warp-uniform
    compact_one(nodes, finals[w], A, B, C, out_k, out_c);
  }
}

// Small copies between device and page-locked host memory done by a kernel
// (the GPU reads or writes the host side over the chip-to-chip link), so that
// an engine's control traffic never queues behind a bulk copy that occupies a
// copy engine.
__global__ void k_copy_small(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                             uint64_t bytes) {
  const uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst) | bytes) & 7) == 0) {
    const uint64_t* s = reinterpret_cast<const uint64_t*>(src);
    uint64_t* d = reinterpret_cast<uint64_t*>(dst);
    for (uint64_t i = i0; i < bytes / 8; i += step) d[i] = s[i];
  } else {
    for (uint64_t i = i0; i < bytes; i += step) dst[i] = src[i];
  }
}

// Host reads into device memory by the SMs, for host memory the GPU reads in
// place: pageable memory where the device uses the host's page tables
// (coherent chip-to-chip access), or page-locked memory.  Any alignment of
// either side.  Each lane writes one 16-byte word of the destination; its
// bytes come from the two 16-byte-aligned source words that straddle them,
// the second being the next lane's first (the last lane loads it), so each
// source word crosses the link once.  A source word is read only if it holds
// a byte of the source range: an aligned 16-byte word never crosses a page,
// so no read leaves the pages the range occupies.  The words at either end
// of the destination range are written byte by byte.
__global__ void k_copy_in(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                          uint64_t bytes) {
  const uintptr_t d_lo = reinterpret_cast<uintptr_t>(dst), d_hi = d_lo + bytes;
  const uintptr_t d0 = d_lo & ~(uintptr_t)15;
  const uint64_t nw = (d_hi - d0 + 15) >> 4;  // destination words touched
  const uintptr_t s_lo = reinterpret_cast<uintptr_t>(src), s_hi = s_lo + bytes;
  const uintptr_t delta = s_lo - d_lo;        // source address = destination + delta (mod 2^64)
  const uint32_t m = (uint32_t)((d0 + delta) & 15);  // a word's first byte inside its source word
  const uint32_t q = m >> 2, r = (m & 3) * 8;
  const uint32_t lane = lane_id();
  const uint64_t wstep = (uint64_t)gridDim.x * (blockDim.x >> 5) * 32;
  auto load = [&](uintptr_t a) -> uint4 {
    if (a < s_hi && a + 16 > s_lo) return *reinterpret_cast<const uint4*>(a);
    return make_uint4(0u, 0u, 0u, 0u);
  };
  for (uint64_t wb = ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; wb < nw;
       wb += wstep) {  // uniform over the warp
    const uint64_t j = wb + lane;
    const uintptr_t D = d0 + 16 * j;
    const uintptr_t A = D + delta - m;  // 16-byte aligned
    const uint4 w = load(A);
    uint4 o = w;
    if (m) {
      uint4 v;
      v.x = __shfl_down_sync(0xFFFFFFFFu, w.x, 1);
      v.y = __shfl_down_sync(0xFFFFFFFFu, w.y, 1);
      v.z = __shfl_down_sync(0xFFFFFFFFu, w.z, 1);
      v.w = __shfl_down_sync(0xFFFFFFFFu, w.w, 1);
      if (lane == 31) v = load(A + 16);
      uint32_t a0 = w.x, a1 = w.y, a2 = w.z, a3 = w.w, a4 = v.x, a5 = v.y, a6 = v.z, a7 = v.w;
      if (q & 2) { a0 = a2; a1 = a3; a2 = a4; a3 = a5; a4 = a6; a5 = a7; }
      if (q & 1) { a0 = a1; a1 = a2; a2 = a3; a3 = a4; a4 = a5; }
      o.x = __funnelshift_r(a0, a1, r);
      o.y = __funnelshift_r(a1, a2, r);
      o.z = __funnelshift_r(a2, a3, r);
      o.w = __funnelshift_r(a3, a4, r);
    }
    if (j >= nw) continue;
    if (D >= d_lo && D + 16 <= d_hi) {
      *reinterpret_cast<uint4*>(D) = o;
    } else {
      const uint8_t* ob = reinterpret_cast<const uint8_t*>(&o);
      for (uint32_t b = 0; b < 16; ++b)
        if (D + b >= d_lo && D + b < d_hi) reinterpret_cast<uint8_t*>(D)[b] = ob[b];
    }
  }
}

}  // namespace

int launch_copy_small(const void* src, void* dst, uint64_t bytes, cudaStream_t s) {
  if (!bytes) return 0;
  const uint64_t units = (bytes + 7) / 8;
  const uint32_t blocks = (uint32_t)std::min<uint64_t>(64, (units + 255) / 256);
  k_copy_small<<<blocks, 256, 0, s>>>((const uint8_t*)src, (uint8_t*)dst, bytes);
  return 1;
}

int launch_copy_in(const void* src, void* dst, uint64_t bytes, int sm_count, cudaStream_t s) {
  if (!bytes) return 0;
  const uint64_t words = bytes / 16 + 2;
  // a CTA on every other SM: the chunked upload overlaps the level-1 kernels,
  // which it slows least at this size (large_100m end to end, pageable reads:
  // 71.0 ms with 76 CTAs, 76.3 with 152, 74.6 with 38; page-locked 69.0)
#ifndef DK_COPY_IN_CTAS_PCT
#define DK_COPY_IN_CTAS_PCT 50
#endif
  const uint64_t ctas = std::max<uint64_t>(1, (uint64_t)sm_count * DK_COPY_IN_CTAS_PCT / 100);
  const uint32_t blocks = (uint32_t)std::min<uint64_t>(ctas, (words + 255) / 256);
  k_copy_in<<<blocks, 256, 0, s>>>((const uint8_t*)src, (uint8_t*)dst, bytes);
  return 1;
}

// ------------------------------------------------------------ launchers
// Every launcher raises a kernel's dynamic shared-memory limit to the same
// value, everything the block may use beside its static shared memory:
// engines on other host threads launch the same kernels with other sizes, and
// a per-launch value set by one thread could undercut another thread's launch
// between its set and its launch.
template <typename K>
static void allow_max_smem(K* kernel) {
  int dev = 0, optin = 0;
  cudaFuncAttributes fa;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, kernel) != cudaSuccess)
    return;  // the launch itself reports the failure
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       optin - (int)fa.sharedSizeBytes);
}

static int choose_c(int W) {
  const int c = (W + 31) / 32;
  if (c <= 1) return 1;
  if (c <= 2) return 2;
  if (c <= 4) return 4;
  if (c <= 5) return 5;
  if (c <= 8) return 8;
  if (c <= 16) return 16;
  return 32;
}

template <int C>
static void count_launch(const ExtractArgs& a, int grid, uint32_t* H, unsigned long long* counters,
                         cudaStream_t s) {
  const uint64_t stride = (uint64_t)a.W + 1;
  const uint32_t lt = (uint32_t)std::max<uint64_t>(16, std::min<uint64_t>(128, 16384 / stride));
  const size_t smem = 128 + 2 * (size_t)tile_buf_bytes(lt, stride) + (size_t)a.F1 * 4 + 256;
  auto* kern = a.conv == 1 ? k_l1_count<C, 1> : k_l1_count<C, 0>;
  allow_max_smem(kern);
  kern<<<grid, 512, smem, s>>>(a, H, counters, lt);
}

static size_t lines_smem(const ExtractArgs& a, bool scatter) {
  return 128 + 2 * (size_t)tile_buf_bytes(kLineThreads, (uint64_t)a.W + 1) +
         (size_t)a.F1 * (scatter ? 12 : 4) + 256;
}

// the count kernel keeps one tile buffer of kCountThreads lines
static size_t count_lines_smem(const ExtractArgs& a) {
  return 128 + (size_t)tile_buf_bytes(kCountThreads, (uint64_t)a.W + 1) + (size_t)a.F1 * 4 + 256;
}

// batch waves (jobs) with lines the thread-per-line kernels take scatter
// directly; plain counts stage their tiles (k_l1_scatter)
static bool direct_scatter(int W, bool jobs) { return jobs && W <= kLineMaxW; }

static size_t chunked_smem(const ExtractArgs& a, int chunk) {
  return 128 + (size_t)tile_buf_bytes(kLineThreads, (uint64_t)a.W + 1) +
         (size_t)kLineThreads * chunk * 8 + (size_t)a.F1 * 20 + 32 * 4 + 256;
}
// plain counts whose chunked thread-per-line scatter fits two CTAs per SM
static bool chunked_scatter(const ExtractArgs& a) {
  return !a.njobs && a.W <= kLineMaxW &&
         chunked_smem(a, kLineChunk) <= kMaxSmemPerBlock / 2 - 1024;
}
// positions per chunk: twice kLineChunk where that still fits two CTAs per SM
// (half the chunk barriers and bucket scans, bucket runs twice as long)
static int chunk_positions(const ExtractArgs& a) {
  return chunked_smem(a, 2 * kLineChunk) <= kMaxSmemPerBlock / 2 - 1024 ? 2 * kLineChunk
                                                                        : kLineChunk;
}

int launch_l1_count(const ExtractArgs& a, int grid, uint32_t* H, unsigned long long* counters,
                    cudaStream_t s) {
  if (a.W <= kLineMaxW) {
    const int m = roll_mode(a.conv, a.k);
    auto* kern = m == kRollPak ? k_l1_lines_count<kRollPak>
                               : (m == kRollDakcK1 ? k_l1_lines_count<kRollDakcK1>
                                                   : k_l1_lines_count<kRollDakc>);
    allow_max_smem(kern);
    kern<<<grid, kCountThreads, count_lines_smem(a), s>>>(a, H, counters);
    return 1;
  }
  switch (choose_c(a.W)) {
    case 1: count_launch<1>(a, grid, H, counters, s); break;
    case 2: count_launch<2>(a, grid, H, counters, s); break;
    case 4: count_launch<4>(a, grid, H, counters, s); break;
    case 5: count_launch<5>(a, grid, H, counters, s); break;
    case 8: count_launch<8>(a, grid, H, counters, s); break;
    case 16: count_launch<16>(a, grid, H, counters, s); break;
    default: count_launch<32>(a, grid, H, counters, s); break;
  }
  return 1;
}

int launch_chunk_scan(const uint32_t* H_c, int G, int F1, uint32_t* T_c, uint64_t* S_c,
                      unsigned long long* running, uint64_t* O_c, cudaStream_t s) {
  const int tb = 256, nb = (F1 + tb - 1) / tb;
  k_chunk_totals<<<nb, tb, 0, s>>>(H_c, G, F1, T_c);
  k_chunk_starts<<<1, 1024, 0, s>>>(T_c, F1, S_c, running);
  k_chunk_offsets_rows<<<nb, tb, 0, s>>>(H_c, G, F1, S_c, O_c);
  return 3;
}

int launch_l1_nodes(const uint32_t* H, int rows, int F1, Node* nodes, int shift1, cudaStream_t s) {
  const int tb = 256, nb = (F1 + tb - 1) / tb;
  k_l1_totals<<<nb, tb, 0, s>>>(H, rows, F1, nodes);
  k_l1_starts<<<1, 1024, 0, s>>>(nodes, F1, shift1, nullptr);
  return 2;
}

int launch_l1_scan(const uint32_t* H, int grid, int F1, uint64_t* O, Node* nodes, int shift1,
                   const int16_t* bucket_shift, cudaStream_t s) {
  const int tb = 256, nb = (F1 + tb - 1) / tb;
  k_l1_totals<<<nb, tb, 0, s>>>(H, grid, F1, nodes);
  k_l1_starts<<<1, 1024, 0, s>>>(nodes, F1, shift1, bucket_shift);
  k_l1_offsets_rows<<<nb, tb, 0, s>>>(H, grid, F1, nodes, O);
  return 3;
}

static int lpw_of(int c) { return c <= 2 ? 4 : (c <= 8 ? 2 : 1); }

static size_t scatter_smem(int W, int F1, bool jobs) {
  const int C = choose_c(W);
  const uint32_t lt = 16u * (uint32_t)lpw_of(C);
  const size_t stage_cap = (size_t)lt * 32 * C;
  return 128 + 2 * (size_t)tile_buf_bytes(lt, (uint64_t)W + 1) + (size_t)F1 * 16 +
         stage_cap * 8 + 32 * 4 + 256 + (jobs ? stage_cap * 2 : 0);
}

int l1_max_buckets(int W, bool jobs) {
  int f = 1 << kMaxL1Bits;
  ExtractArgs a{};
  a.W = W;
  a.F1 = f;
  if (direct_scatter(W, jobs)) {
    while (f > 1 && lines_smem(a, true) > kMaxSmemPerBlock) a.F1 = (f >>= 1);
    return f;
  }
  if (!jobs && W <= kLineMaxW) {  // the chunked thread-per-line scatter, two CTAs per SM
    while (f > 1 && !chunked_scatter(a)) a.F1 = (f >>= 1);
    return f;
  }
  while (f > 1 && scatter_smem(W, f, jobs) > kMaxSmemPerBlock) f >>= 1;
  return f;
}

template <int C, int LPW>
static void scatter_launch(const ExtractArgs& a, int grid, const uint64_t* O, uint64_t* keys,
                           unsigned long long* counters, cudaStream_t s) {
  const int threads = 512;
  const uint32_t lt = (threads / 32) * LPW;
  const int stage_cap = (int)lt * 32 * C;  // >= k-mers of one tile
  static_assert(LPW == (C <= 2 ? 4 : (C <= 8 ? 2 : 1)), "scatter_smem mirrors this tiling");
  const size_t smem = scatter_smem(a.W, a.F1, a.njobs != 0);
  auto* kern = a.conv == 1 ? k_l1_scatter<C, LPW, 1> : k_l1_scatter<C, LPW, 0>;
  allow_max_smem(kern);
  kern<<<grid, threads, smem, s>>>(a, O, keys, stage_cap, counters);
}

// the chunked scatter for roll mode m
template <int CH, bool kHi>
static auto chunked_kernel(int m) -> decltype(&k_l1_lines_chunked<kRollDakc, CH, kHi>) {
  return m == kRollPak ? k_l1_lines_chunked<kRollPak, CH, kHi>
                       : (m == kRollDakcK1 ? k_l1_lines_chunked<kRollDakcK1, CH, kHi>
                                           : k_l1_lines_chunked<kRollDakc, CH, kHi>);
}

int launch_l1_scatter(const ExtractArgs& a, int grid, const uint64_t* O, uint64_t* keys,
                      unsigned long long* counters, cudaStream_t s) {
  if (chunked_scatter(a)) {
    const int chunk = chunk_positions(a);
    const int m = roll_mode(a.conv, a.k);
    const bool hi = a.shift1 >= 32;
    auto* kern = chunk == 2 * kLineChunk
                     ? (hi ? chunked_kernel<2 * kLineChunk, true>(m)
                           : chunked_kernel<2 * kLineChunk, false>(m))
                     : (hi ? chunked_kernel<kLineChunk, true>(m) : chunked_kernel<kLineChunk, false>(m));
    allow_max_smem(kern);
    kern<<<grid, kLineThreads, chunked_smem(a, chunk), s>>>(a, O, keys, counters);
    return 1;
  }
  if (direct_scatter(a.W, a.njobs != 0)) {
    const int m = roll_mode(a.conv, a.k);
    auto* kern = m == kRollPak ? k_l1_lines_direct<kRollPak>
                               : (m == kRollDakcK1 ? k_l1_lines_direct<kRollDakcK1>
                                                   : k_l1_lines_direct<kRollDakc>);
    allow_max_smem(kern);
    kern<<<grid, kLineThreads, lines_smem(a, true), s>>>(a, O, keys, counters);
    return 1;
  }
  switch (choose_c(a.W)) {
    case 1: scatter_launch<1, 4>(a, grid, O, keys, counters, s); break;
    case 2: scatter_launch<2, 4>(a, grid, O, keys, counters, s); break;
    case 4: scatter_launch<4, 2>(a, grid, O, keys, counters, s); break;
    case 5: scatter_launch<5, 2>(a, grid, O, keys, counters, s); break;
    case 8: scatter_launch<8, 2>(a, grid, O, keys, counters, s); break;
    case 16: scatter_launch<16, 1>(a, grid, O, keys, counters, s); break;
    default: scatter_launch<32, 1>(a, grid, O, keys, counters, s); break;
  }
  return 1;
}

int launch_classify(Node* nodes, uint32_t lo, uint32_t hi, uint32_t* final_list,
                    uint32_t* big_list, LevelCounters* ctr, int bin_cap, int split_target,
                    int big_ok, const Ranges& rg, cudaStream_t s) {
  const uint32_t n = hi - lo;
  if (!n) return 0;
  k_classify<<<(n + 255) / 256, 256, 0, s>>>(nodes, lo, hi, final_list, big_list, ctr, bin_cap,
                                            split_target, big_ok, rg);
  return 1;
}

int launch_make_proxies(Node* nodes, const uint32_t* final_list, uint32_t n_final,
                        uint32_t n_nodes, unsigned int* count, cudaStream_t s) {
  if (!n_final) return 0;
  k_make_proxies<<<(n_final + 255) / 256, 256, 0, s>>>(nodes, final_list, n_final, n_nodes, count);
  return 1;
}

int launch_assign(Node* nodes, uint32_t lo, uint32_t hi, uint32_t child_base, Tile* tiles,
                  LevelCounters* ctr, const Ranges& rg, cudaStream_t s) {
  const uint32_t n = hi - lo;
  if (!n) return 0;
  k_assign<<<(uint32_t)(((uint64_t)n * 32 + 255) / 256), 256, 0, s>>>(nodes, lo, hi, child_base,
                                                                      tiles, ctr, rg);
  return 1;
}

int launch_tile_hist(const Node* nodes, const Tile* tiles, uint32_t n_tiles, const uint64_t* A,
                     const uint64_t* B, uint32_t* TH, cudaStream_t s) {
  if (!n_tiles) return 0;
  k_tile_hist<<<n_tiles, 256, 0, s>>>(nodes, tiles, A, B, TH);
  return 1;
}

int launch_node_scan(Node* nodes, uint32_t lo, uint32_t hi, Tile* tiles, uint32_t* TH,
                     cudaStream_t s) {
  if (hi <= lo) return 0;
  // few nodes (large ones) get wide CTAs: each thread then scans fewer digits
  k_node_scan<<<hi - lo, (hi - lo) <= 4096 ? 1024 : 256, 0, s>>>(nodes, lo, tiles, TH);
  return 1;
}

int launch_tile_scatter(const Node* nodes, const Tile* tiles, uint32_t n_tiles, uint64_t* A,
                        uint64_t* B, const uint32_t* TH, int max_width, cudaStream_t s) {
  if (!n_tiles) return 0;
  const size_t smem = (size_t)kTileKeys * 8 + ((size_t)1 << max_width) * 16;
  allow_max_smem(k_tile_scatter);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // prefetch one resident wave ahead (large_100m: partition scatter 9.90 ->
  // 9.33 ms; two waves ahead 10.07 ms).  The same prefetch slowed the
  // bandwidth-bound kernels: text tiles of the level-1 count, tiles of the
  // partition histogram (2.94 -> 3.24 ms), bins of the compact (2.90 -> 3.68)
  k_tile_scatter<<<n_tiles, kTileThreads, smem, s>>>(nodes, tiles, A, B, TH, max_width,
                                                     (uint32_t)(DK_TILE_CTAS * sms));
  return 1;
}

int bin_count_smem_bytes(int) { return kBinCap * 8; }

int launch_bin_count(Node* nodes, const uint32_t* big_list, uint32_t n_big,
                     const uint32_t* final_list, uint32_t n_final, uint64_t* A, uint64_t* B,
                     uint32_t* C, int use_hash, unsigned long long* ctr, int sm_count,
                     cudaStream_t s, uint32_t* fb_list) {
  const uint32_t n_bins = n_big + n_final;
  if (!n_bins) return 0;
  allow_max_smem(k_bin_count);
  if (!use_hash || !fb_list) {
    const uint32_t grid = std::min<uint32_t>(n_bins, (uint32_t)(kBinBlocksPerSM * sm_count));
    k_bin_count<<<grid, kBinThreads, kBinCap * 8, s>>>(nodes, big_list, n_big, final_list, n_bins,
                                                       A, B, C, ctr, use_hash, nullptr, nullptr);
    return 1;
  }
  // hash variant: the packed kernel takes the final list; what it leaves
  // (fb_list) follows the big bins through k_bin_count
  int launches = 0;
  if (n_final) {
    allow_max_smem(k_bin_packed);
    const uint32_t grid = std::min<uint32_t>(n_final, (uint32_t)(kPackBlocksPerSM * sm_count));
    k_bin_packed<<<grid, kPackThreads, kPackSmem, s>>>(nodes, final_list, n_final, A, B, C, ctr,
                                                       fb_list, nullptr);
    ++launches;
  }
  const uint32_t grid = std::min<uint32_t>(n_bins, (uint32_t)(kBinBlocksPerSM * sm_count));
  k_bin_count<<<grid, kBinThreads, kBinCap * 8, s>>>(nodes, big_list, n_big, fb_list, 0, A, B, C,
                                                     ctr, use_hash,
                                                     reinterpret_cast<const unsigned int*>(&ctr[20]),
                                                     nullptr);
  return launches + 1;
}

int launch_aggregate(Node* nodes, uint32_t lo, uint32_t hi, cudaStream_t s) {
  if (hi <= lo) return 0;
  k_aggregate<<<(uint32_t)(((uint64_t)(hi - lo) * 32 + 255) / 256), 256, 0, s>>>(nodes, lo, hi);
  return 1;
}

int launch_l1_offsets(Node* nodes, uint32_t b0, uint32_t b1, unsigned long long* total_d,
                      cudaStream_t s) {
  k_l1_out_offsets<<<1, 1024, 0, s>>>(nodes, b0, b1, total_d);
  return 1;
}

int launch_child_offsets(Node* nodes, uint32_t lo, uint32_t hi, cudaStream_t s) {
  if (hi <= lo) return 0;
  k_child_offsets<<<hi - lo, 256, 0, s>>>(nodes, lo);
  return 1;
}

int launch_compact(const Node* nodes, const uint32_t* final_list, uint32_t n_final,
                   const uint64_t* A, const uint64_t* B, const uint32_t* C, uint64_t* out_k,
                   uint32_t* out_c, cudaStream_t s) {
  if (!n_final) return 0;
  const uint32_t warps_per_block = 8;
  k_compact<<<(n_final + warps_per_block - 1) / warps_per_block, 256, 0, s>>>(
      nodes, final_list, n_final, A, B, C, out_k, out_c);
  return 1;
}


// The wave graph (see dk_internal.cuh):
//   WHILE level: [begin, classify, plan, assign, tile hist, node scan, tile scatter]
//   packed bins -> general bins -> up-pass start
//   WHILE up:    [pass step, aggregate]
//   level-1 offsets -> down-pass start
//   WHILE down:  [pass step, child offsets]
//   compact finals -> compact big bins
// Segments between conditional nodes are captured from `cs` into the graph.
// Grids are fixed: the memory-bound kernels fill every SM (8 CTAs of 256
// threads), as the host path's one-block-per-item launches do.
namespace {

#define DK_GTRY(x)                          \
  do {                                      \
    const cudaError_t _e = (x);             \
    if (_e != cudaSuccess) return _e;       \
  } while (0)

// add a WHILE node after deps; *body receives its body graph
cudaError_t add_while(cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps,
                      cudaGraphConditionalHandle* h, cudaGraphNode_t* node, cudaGraph_t* body) {
  DK_GTRY(cudaGraphConditionalHandleCreate(h, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = *h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  DK_GTRY(cudaGraphAddNode(node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                           &p));
  *body = p.conditional.phGraph_out[0];
  return cudaSuccess;
}

// end a capture into g, returning the nodes the next segment depends on
cudaError_t end_segment(cudaStream_t cs, cudaGraph_t g, std::vector<cudaGraphNode_t>* leaves) {
  cudaStreamCaptureStatus st;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  DK_GTRY(cudaStreamGetCaptureInfo(cs, &st, nullptr, nullptr, &deps, nullptr, &nd));
  std::vector<cudaGraphNode_t> v(deps, deps + nd);
  cudaGraph_t out = g;
  DK_GTRY(cudaStreamEndCapture(cs, &out));
  *leaves = v;
  return cudaSuccess;
}

cudaError_t begin_segment(cudaStream_t cs, cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps) {
  return cudaStreamBeginCaptureToGraph(cs, g, deps.empty() ? nullptr : deps.data(), nullptr,
                                       deps.size(), cudaStreamCaptureModeRelaxed);
}

}  // namespace

cudaError_t build_wave_graph(const WaveGraphArgs& a, cudaStream_t cs, cudaGraph_t* out) {
  const int S = a.sm_count;
  const size_t scatter_smem = (size_t)kTileKeys * 8 + ((size_t)1 << kGraphSplitBits) * 16;
  allow_max_smem(k_g_tile_scatter);
  allow_max_smem(k_bin_packed);
  allow_max_smem(k_bin_count);
  cudaGraph_t g = nullptr;
  DK_GTRY(cudaGraphCreate(&g, 0));
  cudaError_t err = [&]() -> cudaError_t {
    // the level loop
    cudaGraphConditionalHandle h_lvl, h_up, h_down;
    cudaGraphNode_t n_lvl, n_up, n_down;
    cudaGraph_t body;
    DK_GTRY(add_while(g, {}, &h_lvl, &n_lvl, &body));
    DK_GTRY(begin_segment(cs, body, {}));
    k_g_level_begin<<<1, 32, 0, cs>>>(a.lc, a.wc);
    k_g_classify<<<4 * S, 256, 0, cs>>>(a.nodes, a.finals, a.bigs, a.lc, a.bin_cap,
                                        a.split_target, a.big_ok, a.wc);
    k_g_plan<<<1, 32, 0, cs>>>(a.lc, a.wc, h_lvl);
    k_g_assign<<<4 * S, 256, 0, cs>>>(a.nodes, a.tiles, a.lc, a.wc);
    k_g_tile_hist<<<8 * S, 256, 0, cs>>>(a.nodes, a.tiles, a.A, a.B, a.TH, a.wc);
    k_g_node_scan<<<4 * S, 256, 0, cs>>>(a.nodes, a.tiles, a.TH, a.wc);
    k_g_tile_scatter<<<DK_TILE_CTAS * S, kTileThreads, scatter_smem, cs>>>(a.nodes, a.tiles, a.A,
                                                                          a.B, a.TH, a.wc);
    std::vector<cudaGraphNode_t> leaves;
    DK_GTRY(end_segment(cs, body, &leaves));
    // the bins of the final nodes, big bins first
    DK_GTRY(begin_segment(cs, g, {n_lvl}));
    const uint32_t* n_final = &a.lc->n_final;
    const uint32_t* n_big = &a.lc->n_big_final;
    if (a.use_hash) {
      k_bin_packed<<<kPackBlocksPerSM * S, kPackThreads, kPackSmem, cs>>>(
          a.nodes, a.finals, 0, a.A, a.B, a.C, a.ctr, a.fb_list, n_final);
      k_bin_count<<<kBinBlocksPerSM * S, kBinThreads, kBinCap * 8, cs>>>(
          a.nodes, a.bigs, 0, a.fb_list, 0, a.A, a.B, a.C, a.ctr, 1,
          reinterpret_cast<const unsigned int*>(&a.ctr[20]), n_big);
    } else {
      k_bin_count<<<kBinBlocksPerSM * S, kBinThreads, kBinCap * 8, cs>>>(
          a.nodes, a.bigs, 0, a.finals, 0, a.A, a.B, a.C, a.ctr, 0, n_final, n_big);
    }
    k_g_pass_begin<<<1, 32, 0, cs>>>(a.wc, 1);
    DK_GTRY(end_segment(cs, g, &leaves));
    // distinct counts up the tree
    DK_GTRY(add_while(g, leaves, &h_up, &n_up, &body));
    DK_GTRY(begin_segment(cs, body, {}));
    k_g_pass_step<<<1, 32, 0, cs>>>(a.wc, h_up, 1);
    k_g_aggregate<<<8 * S, 256, 0, cs>>>(a.nodes, a.wc);
    DK_GTRY(end_segment(cs, body, &leaves));
    // level-1 offsets, then offsets down the tree
    DK_GTRY(begin_segment(cs, g, {n_up}));
    k_g_l1_offsets<<<1, 1024, 0, cs>>>(a.nodes, &a.ctr[2], a.wc);
    k_g_pass_begin<<<1, 32, 0, cs>>>(a.wc, 0);
    DK_GTRY(end_segment(cs, g, &leaves));
    DK_GTRY(add_while(g, leaves, &h_down, &n_down, &body));
    DK_GTRY(begin_segment(cs, body, {}));
    k_g_pass_step<<<1, 32, 0, cs>>>(a.wc, h_down, 0);
    k_g_child_offsets<<<8 * S, 256, 0, cs>>>(a.nodes, a.wc);
    DK_GTRY(end_segment(cs, body, &leaves));
    // the bins' pairs into the table
    DK_GTRY(begin_segment(cs, g, {n_down}));
    k_g_compact<<<8 * S, 256, 0, cs>>>(a.nodes, a.finals, n_final, &a.wc->tk_compact[0], a.A,
                                       a.B, a.C, a.wc);
    k_g_compact<<<8 * S, 256, 0, cs>>>(a.nodes, a.bigs, n_big, &a.wc->tk_compact[1], a.A, a.B,
                                       a.C, a.wc);
    DK_GTRY(end_segment(cs, g, &leaves));
    return cudaGetLastError();
  }();
  if (err != cudaSuccess) {
    cudaStreamCaptureStatus st;
    if (cudaStreamIsCapturing(cs, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(cs, &junk);
    }
    cudaGraphDestroy(g);
    cudaGetLastError();
    return err;
  }
  *out = g;
  return cudaSuccess;
}

}  // namespace dk

#ifdef DK_PHASE_TIMING
extern "C" int dk_debug_phases(unsigned long long* out) {
  return (int)cudaMemcpyFromSymbol(out, dk::g_phase, sizeof(unsigned long long) * 32);
}
extern "C" int dk_debug_reset() {
  unsigned long long z[32] = {0};
  return (int)cudaMemcpyToSymbol(dk::g_phase, z, sizeof(z));
}
#endif

#ifdef DK_BOUNDS_CHECK
extern "C" int dk_debug_check(unsigned long long* out) {
  return (int)cudaMemcpyFromSymbol(out, dk::g_check, sizeof(unsigned long long) * 4);
}
#endif
