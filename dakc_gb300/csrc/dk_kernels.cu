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
#include <cstdio>

namespace dk {

namespace {

using namespace dev;


// ------------------------------------------------------------- level 1
template <int C>
__global__ void __launch_bounds__(512) k_l1_count(ExtractArgs a, uint32_t* __restrict__ H,
                                                  unsigned long long* __restrict__ counters) {
  extern __shared__ uint32_t sh[];
  uint32_t* hist = sh;
  uint8_t* lut = reinterpret_cast<uint8_t*>(sh + a.F1);
  for (int b = threadIdx.x; b < a.F1; b += blockDim.x) hist[b] = 0;
  init_lut(lut);
  __syncthreads();
  uint64_t lo, hi;
  lines_of_block(a.n_lines, &lo, &hi);
  const uint32_t warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint64_t stride = (uint64_t)a.W + 1;
  uint32_t mine = 0;
  for (uint64_t l = lo + warp; l < hi; l += nwarps) {
    const uint8_t* line = a.text + l * stride;
    if (lane_id() == 0 && l > 0 && line[0] == 0) atomicMax(&counters[1], a.n_lines - l);
    warp_line_kmers<C>(line, a.W, a.k, a.kmask, lut, [&](int, uint64_t key, bool valid) {
      if (valid) { atomicAdd(&hist[key >> a.shift1], 1u); ++mine; }
    });
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
__global__ void k_l1_starts(Node* nodes, int F1, int shift1) {
  __shared__ unsigned long long tmp[32];
  const int per = (F1 + blockDim.x - 1) / blockDim.x;
  const int lo = min(F1, (int)threadIdx.x * per), hi = min(F1, lo + per);
  unsigned long long s = 0;
  for (int i = lo; i < hi; ++i) s += nodes[i].n;
  unsigned long long base = block_excl_scan<unsigned long long>(s, tmp, nullptr);
  for (int i = lo; i < hi; ++i) {
    Node& nd = nodes[i];
    nd.start = base;
    base += nd.n;
    nd.d = 0;
    nd.out_off = 0;
    nd.first_child = 0;
    nd.shift = (int16_t)shift1;
    nd.buf = 0;
    nd.state = 0;
    nd.tile_base = 0;
    nd.ntiles = 0;
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

template <int C, int LPW>
__global__ void __launch_bounds__(512) k_l1_scatter(ExtractArgs a, const uint64_t* __restrict__ O,
                                                    uint64_t* __restrict__ keys_out,
                                                    int stage_cap) {
  extern __shared__ unsigned long long shs[];
  const int F1 = a.F1;
  unsigned long long* cursor = shs;                                  // F1
  unsigned long long* staging = cursor + F1;                         // stage_cap
  uint32_t* tile_hist = reinterpret_cast<uint32_t*>(staging + stage_cap);  // F1
  uint32_t* tile_off = tile_hist + F1;                                // F1
  uint32_t* tmp = tile_off + F1;                                      // 32
  uint8_t* lut = reinterpret_cast<uint8_t*>(tmp + 32);                // 256
  for (int b = threadIdx.x; b < F1; b += blockDim.x) {
    cursor[b] = O[(size_t)blockIdx.x * F1 + b];
    tile_hist[b] = 0;
  }
  init_lut(lut);
  __syncthreads();
  uint64_t lo, hi;
  lines_of_block(a.n_lines, &lo, &hi);
  const uint32_t warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint64_t stride = (uint64_t)a.W + 1;
  const uint64_t lines_per_tile = (uint64_t)nwarps * LPW;
  for (uint64_t t0 = lo; t0 < hi; t0 += lines_per_tile) {
    uint64_t kr[LPW][C];
    uint32_t sr[LPW][C];
#pragma unroll
    for (int j = 0; j < LPW; ++j) {
      const uint64_t l = t0 + (uint64_t)j * nwarps + warp;
      if (l < hi) {
        warp_line_kmers<C>(a.text + l * stride, a.W, a.k, a.kmask, lut,
                           [&](int t, uint64_t key, bool valid) {
                             kr[j][t] = key;
                             sr[j][t] = valid ? atomicAdd(&tile_hist[key >> a.shift1], 1u)
                                              : 0xFFFFFFFFu;
                           });
      } else {
#pragma unroll
        for (int t = 0; t < C; ++t) { kr[j][t] = 0; sr[j][t] = 0xFFFFFFFFu; }
      }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < F1; b += blockDim.x) tile_off[b] = tile_hist[b];
    __syncthreads();
    const uint32_t T = block_scan_array<uint32_t>(tile_off, F1, tmp);
#pragma unroll
    for (int j = 0; j < LPW; ++j)
#pragma unroll
      for (int t = 0; t < C; ++t)
        if (sr[j][t] != 0xFFFFFFFFu) staging[tile_off[kr[j][t] >> a.shift1] + sr[j][t]] = kr[j][t];
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < T; i += blockDim.x) {
      const uint64_t key = staging[i];
      const uint32_t b = (uint32_t)(key >> a.shift1);
      keys_out[cursor[b] + (i - tile_off[b])] = key;
    }
    __syncthreads();
    for (int b = threadIdx.x; b < F1; b += blockDim.x) {
      cursor[b] += tile_hist[b];
      tile_hist[b] = 0;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------- partition levels
// Mark each node of the level final / split / empty; count splits and tiles.
__global__ void k_classify(Node* nodes, uint32_t lo, uint32_t hi, uint32_t* final_list,
                           LevelCounters* ctr, int bin_cap) {
  const uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi) return;
  const Node nd = nodes[i];
  if (nd.n == 0) {
    nodes[i].state = NODE_EMPTY;
    nodes[i].d = 0;
    return;
  }
  if (nd.n <= (uint64_t)bin_cap || nd.shift <= kDenseBits) {
    nodes[i].state = NODE_FINAL;
    final_list[atomicAdd(&ctr->n_final, 1u)] = i;
    return;
  }
  nodes[i].state = NODE_SPLIT;
  atomicAdd(&ctr->n_split, 1u);
  atomicAdd(&ctr->split_keys, (unsigned long long)nd.n);
  atomicAdd(&ctr->n_tiles, (uint32_t)((nd.n + kTileKeys - 1) / kTileKeys));
  if (nd.n >= (1ull << 32)) atomicOr(&ctr->too_big, 1u);
}

// Give each split node its children block and its partition tiles (buffers
// sized by the host from k_classify's counts).
__global__ void k_assign(Node* nodes, uint32_t lo, uint32_t hi, uint32_t child_base, Tile* tiles,
                         LevelCounters* ctr) {
  const uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi) return;
  const Node nd = nodes[i];
  if (nd.state != NODE_SPLIT) return;
  const uint32_t nt = (uint32_t)((nd.n + kTileKeys - 1) / kTileKeys);
  const uint32_t tb = atomicAdd(&ctr->n_tiles_assigned, nt);
  const uint32_t fc = child_base + atomicAdd(&ctr->n_children, (uint32_t)kFanout);
  nodes[i].first_child = fc;
  nodes[i].tile_base = tb;
  nodes[i].ntiles = nt;
  for (uint32_t t = 0; t < nt; ++t) {
    Tile tl;
    tl.start = nd.start + (uint64_t)t * kTileKeys;
    tl.n = (uint32_t)min((uint64_t)kTileKeys, nd.n - (uint64_t)t * kTileKeys);
    tl.node = i;
    tiles[tb + t] = tl;
  }
}

__device__ __forceinline__ uint32_t digit_of(uint64_t key, int shift) {
  return (uint32_t)(key >> (shift - kDigitBits)) & (kFanout - 1);
}

__global__ void __launch_bounds__(256) k_tile_hist(const Node* nodes, const Tile* tiles,
                                                   const uint64_t* A, const uint64_t* B,
                                                   uint32_t* TH) {
  __shared__ uint32_t hist[kFanout];
  const Tile tl = tiles[blockIdx.x];
  const Node nd = nodes[tl.node];
  const uint64_t* src = (nd.buf ? B : A) + tl.start;
  hist[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < tl.n; i += blockDim.x)
    atomicAdd(&hist[digit_of(__ldg(src + i), nd.shift)], 1u);
  __syncthreads();
  TH[(size_t)blockIdx.x * kFanout + threadIdx.x] = hist[threadIdx.x];
}

// one CTA per node of the level; split nodes turn their tiles' counts into
// offsets within each child and create the children
__global__ void __launch_bounds__(256) k_node_scan(Node* nodes, uint32_t lo, const Tile* tiles,
                                                   uint32_t* TH) {
  __shared__ unsigned long long tmp[32];
  const uint32_t i = lo + blockIdx.x;
  const Node nd = nodes[i];
  if (nd.state != NODE_SPLIT) return;
  const int j = threadIdx.x;
  uint32_t run = 0;
  for (uint32_t t = 0; t < nd.ntiles; ++t) {
    uint32_t* p = TH + (size_t)(nd.tile_base + t) * kFanout + j;
    const uint32_t c = *p;
    *p = run;
    run += c;
  }
  unsigned long long excl = block_excl_scan<unsigned long long>(run, tmp, nullptr);
  Node ch;
  ch.start = nd.start + excl;
  ch.n = run;
  ch.d = 0;
  ch.out_off = 0;
  ch.first_child = 0;
  ch.shift = (int16_t)(nd.shift - kDigitBits);
  ch.buf = (uint8_t)(1 - nd.buf);
  ch.state = 0;
  ch.tile_base = 0;
  ch.ntiles = 0;
  nodes[nd.first_child + j] = ch;
}

__global__ void __launch_bounds__(256) k_tile_scatter(const Node* nodes, const Tile* tiles,
                                                      uint64_t* A, uint64_t* B,
                                                      const uint32_t* TH) {
  __shared__ unsigned long long cursor[kFanout];
  const Tile tl = tiles[blockIdx.x];
  const Node nd = nodes[tl.node];
  const uint64_t* src = (nd.buf ? B : A) + tl.start;
  uint64_t* dst = nd.buf ? A : B;
  cursor[threadIdx.x] = nodes[nd.first_child + threadIdx.x].start +
                        TH[(size_t)blockIdx.x * kFanout + threadIdx.x];
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < tl.n; i += blockDim.x) {
    const uint64_t key = src[i];
    const unsigned long long pos = atomicAdd(&cursor[digit_of(key, nd.shift)], 1ull);
    dst[pos] = key;
  }
}

// ------------------------------------------------------------ bin count

// Dense count of a node with shift <= 12 free bits: the histogram over the
// free bits is already the sorted run-length table.
__device__ void bin_dense(Node* nodes, uint32_t ni, const Node& nd, uint64_t* keys, uint32_t* cnt,
                          unsigned long long* hist, unsigned long long* tmp, int* overflow) {
  const int s = nd.shift;
  const uint32_t R = 1u << s;
  const uint64_t mask = (uint64_t)R - 1;
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) hist[j] = 0;
  __syncthreads();
  const uint64_t prefix = (keys[0] >> s) << s;
  for (uint64_t i = threadIdx.x; i < nd.n; i += blockDim.x)
    atomicAdd(&hist[__ldg(keys + i) & mask], 1ull);
  __syncthreads();
  // rank nonzero digits
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
      if (h > 0xFFFFFFFFull) *overflow = 1;
      cnt[r] = (uint32_t)h;
      ++r;
    }
  }
  if (threadIdx.x == 0) nodes[ni].d = total;
}

__global__ void __launch_bounds__(kBinThreads) k_bin_sort(Node* nodes,
                                                          const uint32_t* __restrict__ finals,
                                                          uint64_t* A, uint64_t* B, uint32_t* C,
                                                          int* overflow) {
  extern __shared__ unsigned long long skeys[];               // kBinCap
  __shared__ unsigned long long hist64[1u << kDenseBits];     // 32 KB (u32 view for the sort path)
  __shared__ unsigned long long tmp[32];
  __shared__ uint16_t long_list[512];
  __shared__ uint32_t n_long;
  const uint32_t ni = finals[blockIdx.x];
  const Node nd = nodes[ni];
  uint64_t* keys = (nd.buf ? B : A) + nd.start;
  uint32_t* cnt = C + nd.start;
  if (nd.shift <= kDenseBits) {
    bin_dense(nodes, ni, nd, keys, cnt, hist64, tmp, overflow);
    return;
  }
  // ---- shared-memory sort path (nd.n <= kBinCap)
  const uint32_t n = (uint32_t)nd.n;
  int D = ceil_log2_u64(n);
  D = max(4, min(D, kDenseBits));
  D = min(D, (int)nd.shift);
  const int sh = nd.shift - D;
  const uint32_t R = 1u << D;
  uint32_t* hist = reinterpret_cast<uint32_t*>(hist64);
  for (uint32_t j = threadIdx.x; j < R; j += blockDim.x) hist[j] = 0;
  if (threadIdx.x == 0) n_long = 0;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
    atomicAdd(&hist[(uint32_t)(__ldg(keys + i) >> sh) & (R - 1)], 1u);
  __syncthreads();
  block_scan_array<uint32_t>(hist, (int)R, reinterpret_cast<uint32_t*>(tmp));
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    const uint64_t key = keys[i];
    const uint32_t pos = atomicAdd(&hist[(uint32_t)(key >> sh) & (R - 1)], 1u);
    skeys[pos] = key;
  }
  __syncthreads();
  // hist[j] is now the end of digit range j
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
  // run-length reduce: heads write key + head position, tails turn it into a count
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = min(n, threadIdx.x * per), hi = min(n, lo + per);
  uint32_t heads = 0;
  for (uint32_t i = lo; i < hi; ++i) heads += (i == 0 || skeys[i] != skeys[i - 1]);
  uint32_t total;
  const uint32_t r0 = block_excl_scan<uint32_t>(heads, reinterpret_cast<uint32_t*>(tmp), &total);
  uint32_t r = r0;
  for (uint32_t i = lo; i < hi; ++i) {
    if (i == 0 || skeys[i] != skeys[i - 1]) {
      keys[r] = skeys[i];
      __stcg(cnt + r, i);
      ++r;
    }
  }
  __syncthreads();
  r = r0;
  for (uint32_t i = lo; i < hi; ++i) {
    if (i == 0 || skeys[i] != skeys[i - 1]) ++r;
    if (i == n - 1 || skeys[i] != skeys[i + 1]) {
      const uint32_t head = __ldcg(cnt + (r - 1));
      __stcg(cnt + (r - 1), i - head + 1);
    }
  }
  if (threadIdx.x == 0) nodes[ni].d = total;
}

// ----------------------------------------------------- tree reductions
__global__ void k_aggregate(Node* nodes, uint32_t lo, uint32_t hi) {
  const uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi) return;
  const Node nd = nodes[i];
  if (nd.state != NODE_SPLIT) return;
  uint64_t d = 0;
  for (int j = 0; j < kFanout; ++j) d += nodes[nd.first_child + j].d;
  nodes[i].d = d;
}

__global__ void k_l1_out_offsets(Node* nodes, uint32_t n1, unsigned long long* total_d) {
  __shared__ unsigned long long tmp[32];
  const uint32_t per = (n1 + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = min(n1, threadIdx.x * per), hi = min(n1, lo + per);
  unsigned long long s = 0;
  for (uint32_t i = lo; i < hi; ++i) s += nodes[i].d;
  unsigned long long tot;
  unsigned long long base = block_excl_scan<unsigned long long>(s, tmp, &tot);
  for (uint32_t i = lo; i < hi; ++i) {
    nodes[i].out_off = base;
    base += nodes[i].d;
  }
  if (threadIdx.x == 0) *total_d = tot;
}

__global__ void __launch_bounds__(256) k_child_offsets(Node* nodes, uint32_t lo) {
  __shared__ unsigned long long tmp[32];
  const Node nd = nodes[lo + blockIdx.x];
  if (nd.state != NODE_SPLIT) return;
  Node& ch = nodes[nd.first_child + threadIdx.x];
  const unsigned long long e = block_excl_scan<unsigned long long>(ch.d, tmp, nullptr);
  ch.out_off = nd.out_off + e;
}

// one warp per final node: staged pairs -> output table
__global__ void k_compact(const Node* nodes, const uint32_t* __restrict__ finals, uint32_t n_final,
                          const uint64_t* A, const uint64_t* B, const uint32_t* C,
                          uint64_t* __restrict__ out_k, uint32_t* __restrict__ out_c) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= n_final) return;
  const Node nd = nodes[finals[w]];
  const uint64_t* sk = (nd.buf ? B : A) + nd.start;
  const uint32_t* sc = C + nd.start;
  for (uint64_t i = lane_id(); i < nd.d; i += 32) {
    out_k[nd.out_off + i] = sk[i];
    out_c[nd.out_off + i] = sc[i];
  }
}

}  // namespace

// ------------------------------------------------------------ launchers
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

int launch_l1_count(const ExtractArgs& a, int grid, uint32_t* H, unsigned long long* counters,
                    cudaStream_t s) {
  const size_t smem = (size_t)a.F1 * 4 + 256;
  switch (choose_c(a.W)) {
    case 1: k_l1_count<1><<<grid, 512, smem, s>>>(a, H, counters); break;
    case 2: k_l1_count<2><<<grid, 512, smem, s>>>(a, H, counters); break;
    case 4: k_l1_count<4><<<grid, 512, smem, s>>>(a, H, counters); break;
    case 5: k_l1_count<5><<<grid, 512, smem, s>>>(a, H, counters); break;
    case 8: k_l1_count<8><<<grid, 512, smem, s>>>(a, H, counters); break;
    case 16: k_l1_count<16><<<grid, 512, smem, s>>>(a, H, counters); break;
    default: k_l1_count<32><<<grid, 512, smem, s>>>(a, H, counters); break;
  }
  return 1;
}

int launch_l1_scan(const uint32_t* H, int grid, int F1, uint64_t* O, Node* nodes, int shift1,
                   cudaStream_t s) {
  const int tb = 256, nb = (F1 + tb - 1) / tb;
  k_l1_totals<<<nb, tb, 0, s>>>(H, grid, F1, nodes);
  k_l1_starts<<<1, 1024, 0, s>>>(nodes, F1, shift1);
  k_l1_offsets_rows<<<nb, tb, 0, s>>>(H, grid, F1, nodes, O);
  return 3;
}

template <int C, int LPW>
static void scatter_launch(const ExtractArgs& a, int grid, const uint64_t* O, uint64_t* keys,
                           cudaStream_t s) {
  const int threads = 512;
  const int stage_cap = (threads / 32) * LPW * 32 * C;  // >= k-mers of one tile
  const size_t smem = (size_t)a.F1 * 8 + (size_t)stage_cap * 8 + (size_t)a.F1 * 8 + 32 * 4 + 256;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_l1_scatter<C, LPW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         232448);
    attr_set = true;
  }
  k_l1_scatter<C, LPW><<<grid, threads, smem, s>>>(a, O, keys, stage_cap);
}

int launch_l1_scatter(const ExtractArgs& a, int grid, const uint64_t* O, uint64_t* keys,
                      cudaStream_t s) {
  switch (choose_c(a.W)) {
    case 1: scatter_launch<1, 4>(a, grid, O, keys, s); break;
    case 2: scatter_launch<2, 4>(a, grid, O, keys, s); break;
    case 4: scatter_launch<4, 2>(a, grid, O, keys, s); break;
    case 5: scatter_launch<5, 2>(a, grid, O, keys, s); break;
    case 8: scatter_launch<8, 2>(a, grid, O, keys, s); break;
    case 16: scatter_launch<16, 1>(a, grid, O, keys, s); break;
    default: scatter_launch<32, 1>(a, grid, O, keys, s); break;
  }
  return 1;
}

int launch_classify(Node* nodes, uint32_t lo, uint32_t hi, uint32_t* final_list,
                    LevelCounters* ctr, int bin_cap, cudaStream_t s) {
  const uint32_t n = hi - lo;
  if (!n) return 0;
  k_classify<<<(n + 255) / 256, 256, 0, s>>>(nodes, lo, hi, final_list, ctr, bin_cap);
  return 1;
}

int launch_assign(Node* nodes, uint32_t lo, uint32_t hi, uint32_t child_base, Tile* tiles,
                  LevelCounters* ctr, cudaStream_t s) {
  const uint32_t n = hi - lo;
  if (!n) return 0;
  k_assign<<<(n + 255) / 256, 256, 0, s>>>(nodes, lo, hi, child_base, tiles, ctr);
  return 1;
}

int launch_tile_hist(const Node* nodes, const Tile* tiles, uint32_t n_tiles, const uint64_t* A,
                     const uint64_t* B, uint32_t* TH, cudaStream_t s) {
  if (!n_tiles) return 0;
  k_tile_hist<<<n_tiles, 256, 0, s>>>(nodes, tiles, A, B, TH);
  return 1;
}

int launch_node_scan(Node* nodes, uint32_t lo, uint32_t hi, const Tile* tiles, uint32_t* TH,
                     cudaStream_t s) {
  if (hi <= lo) return 0;
  k_node_scan<<<hi - lo, 256, 0, s>>>(nodes, lo, tiles, TH);
  return 1;
}

int launch_tile_scatter(const Node* nodes, const Tile* tiles, uint32_t n_tiles, uint64_t* A,
                        uint64_t* B, const uint32_t* TH, cudaStream_t s) {
  if (!n_tiles) return 0;
  k_tile_scatter<<<n_tiles, 256, 0, s>>>(nodes, tiles, A, B, TH);
  return 1;
}

int bin_count_smem_bytes(int) { return kBinCap * 8; }

int launch_bin_count(Node* nodes, const uint32_t* final_list, uint32_t n_final, uint64_t* A,
                     uint64_t* B, uint32_t* C, int, int* overflow, cudaStream_t s) {
  if (!n_final) return 0;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_bin_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, kBinCap * 8);
    attr_set = true;
  }
  k_bin_sort<<<n_final, kBinThreads, kBinCap * 8, s>>>(nodes, final_list, A, B, C, overflow);
  return 1;
}

int launch_aggregate(Node* nodes, uint32_t lo, uint32_t hi, cudaStream_t s) {
  if (hi <= lo) return 0;
  k_aggregate<<<(hi - lo + 255) / 256, 256, 0, s>>>(nodes, lo, hi);
  return 1;
}

int launch_l1_offsets(Node* nodes, uint32_t n1, unsigned long long* total_d, cudaStream_t s) {
  k_l1_out_offsets<<<1, 1024, 0, s>>>(nodes, n1, total_d);
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

}  // namespace dk
