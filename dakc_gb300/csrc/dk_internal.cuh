// Internal declarations shared by the engine's host pipeline and its kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dk {

// A node of the MSD partition tree.  All keys of a node share their bits
// [shift, 2k); the node's keys occupy index range [start, start+n) of buffer
// `buf` (0 = A, 1 = B).  Children of a split node are 2^width consecutive
// nodes starting at `first_child`, in digit (= key) order, and occupy
// consecutive sub-ranges of the parent's index range in the other buffer, so
// index order is key order at every level.
struct Node {
  uint64_t start;
  uint64_t n;
  uint64_t d;        // distinct keys in the subtree (filled bottom-up)
  uint64_t out_off;  // output offset of the subtree's first distinct key
  uint32_t first_child;  // valid when split: 2^width children from here
  int16_t shift;     // remaining low bits not fixed by the path to this node
  uint8_t buf;
  uint8_t state;     // NODE_FINAL / NODE_SPLIT / NODE_EMPTY
  uint32_t tile_base;  // first partition tile (split nodes)
  uint32_t ntiles;
  uint64_t th_base;  // first tile-histogram entry (rows of 2^width per tile)
  uint8_t width;     // digit bits this node is split on (split nodes)
  uint8_t skewed;    // kept more than half of its parent's keys (a hot k-mer)
  uint8_t pad[6];
};
static_assert(sizeof(Node) == 64, "Node layout");
// NODE_RETRY: a large skewed node counted as one hash bin (k_bin_count) that
// held too many distinct keys; the host re-partitions it through a proxy child
enum : uint8_t { NODE_FINAL = 1, NODE_SPLIT = 2, NODE_EMPTY = 3, NODE_RETRY = 4 };

struct Tile {  // a slice of a split node's keys, partitioned by one CTA
  uint64_t start;
  uint32_t n;
  uint32_t node;  // global node index
  uint64_t th;    // first entry of this tile's histogram row
  uint32_t hot;   // one digit holds more than a quarter of the tile (set by the node scan)
  uint32_t pad;
};
static_assert(sizeof(Tile) == 32, "Tile layout");

// counters written by the classify / assign kernels.  n_final and n_big_final
// accumulate over all levels; the others are per level (zeroed from byte 8 on).
struct LevelCounters {
  uint32_t n_final;      // entries of the final list
  uint32_t n_big_final;  // entries of the big-bin list (final nodes larger than a bin)
  uint32_t n_split;
  uint32_t n_tiles;
  uint32_t too_big;      // a split node holds >= 2^32 keys
  uint32_t n_children;   // sum of 2^width over split nodes
  uint32_t max_width;
  uint32_t pad;
  unsigned long long split_keys;  // keys held by this level's split nodes
  unsigned long long th_entries;  // sum of ntiles * 2^width
  uint32_t n_tiles_assigned;
  uint32_t n_children_assigned;
  unsigned long long th_assigned;
};
static_assert(sizeof(LevelCounters) == 64, "LevelCounters is read back as 64 bytes");

constexpr int kDigitBits = 8;           // typical partition fan-out (level-1 sizing)
constexpr int kFanout = 1 << kDigitBits;
constexpr int kMaxSplitBits = 12;       // widest per-node split (4096 children)
#ifndef DK_TILE_KEYS
#define DK_TILE_KEYS 8192
#endif
constexpr int kTileKeys = DK_TILE_KEYS;  // keys per partition tile
constexpr int kBinCap = 12000;          // keys a bin-count CTA sorts in shared memory
constexpr int kBatchBinTarget = 3000;   // default bin size of dk_count_batch (and serving)
constexpr int kDenseBits = 12;          // nodes with <= this many free bits are counted densely
constexpr int kBinThreads = 512;
constexpr int kBinBlocksPerSM = 2;      // resident bin-count CTAs per SM
constexpr int kBinDigitBits = 12;       // counting-sort digit of a bin: at most this many bits
constexpr int kMaxL1Bits = 12;          // level-1 fan-out <= 4096 buckets
constexpr size_t kMaxSmemPerBlock = 232448;  // opt-in shared memory per block (sm_100 family)
constexpr int kLineThreads = 256;        // thread-per-line level-1 kernels: lines per tile
constexpr int kCountThreads = 512;       // ... except the count (one buffer of 512 lines); a
                                         // CTA's lines do not depend on its tile size
constexpr int kLineMaxW = 256;           // longer lines use the warp-per-line kernels
constexpr int kLineChunk = 16;           // positions per line in one chunked-scatter chunk
                                         // (twice this where shared memory still fits
                                         // two CTAs per SM)

struct ExtractArgs {
  const uint8_t* text;  // device text (the line kernels take any alignment)
  uint64_t nbytes;      // readable bytes at text
  uint64_t n_lines;
  // the lines at text are lines [line_base, line_base + n_lines) of a read
  // set of lines_total lines (a chunk counted while later chunks upload);
  // the NUL-led-line rule uses the read set's line numbers
  uint64_t line_base;
  uint64_t lines_total;
  int W;
  int k;
  uint64_t kmask;
  int shift1;  // level-1 bucket = key >> shift1 (plain mode)
  int F1;      // number of level-1 buckets
  int conv;    // k-mer convention: 0 DAKC, 1 PakMan* (thread-per-line kernels only)
  // batch ("jobs") mode when njobs > 0: the text is the concatenation of njobs
  // read sets; job j owns lines [job_start[j], job_start[j+1]) of which lines
  // >= job_end[j] are not parsed (a NUL-led line ends that job), and the
  // level-1 bucket of a k-mer is its job.  job_nul[j] receives the first
  // NUL-led line of job j (initialised to job_start[j+1]).
  int njobs;
  const uint64_t* job_start;
  const uint64_t* job_end;
  unsigned long long* job_nul;
  // job j owns level-1 buckets [job_base[j], job_base[j] + 2^job_bits[j]): a
  // k-mer of job j goes to job_base[j] + (key >> (2k - job_bits[j]))
  const uint32_t* job_base;
  const uint8_t* job_bits;
};

// Level-1 buckets whose keys lie in several ranges of the key buffer: one per
// upload chunk (chunk c's keys of bucket b start at S[c * F1 + b], T[c * F1 + b]
// of them).  C = 0: every node's keys are one range [start, start + n).
struct Ranges {
  const uint64_t* S;
  const uint32_t* T;
  int C;
  int F1;
};

// ---- launchers (dk_kernels.cu); every launcher returns the number of kernel
// launches it issued (for the launch count reported in stats)
int launch_l1_count(const ExtractArgs& a, int grid, uint32_t* H, unsigned long long* n_kmers,
                    cudaStream_t s);
// bucket_shift (optional, F1 entries): per-bucket free bits in batch mode
int launch_l1_scan(const uint32_t* H, int grid, int F1, uint64_t* O, Node* nodes, int shift1,
                   const int16_t* bucket_shift, cudaStream_t s);
// copy `bytes` between device memory and page-locked host memory with a kernel
int launch_copy_small(const void* src, void* dst, uint64_t bytes, cudaStream_t s);
// copy `bytes` of host memory the device reads in place (pageable memory with
// coherent host access, or page-locked memory) into device memory, any alignment
int launch_copy_in(const void* src, void* dst, uint64_t bytes, int sm_count, cudaStream_t s);

// largest level-1 fan-out (power of two <= 2^kMaxL1Bits) whose scatter kernel
// fits the per-block shared-memory limit for line width W
int l1_max_buckets(int W, bool jobs);
int launch_l1_scatter(const ExtractArgs& a, int grid, const uint64_t* O, uint64_t* keys,
                      unsigned long long* counters, cudaStream_t s);
// split nodes get a digit width that makes their children ~split_target/2 keys
// big_ok: a skewed node (it kept most of its parent's keys: a hot k-mer) larger
// than a bin becomes a final hash bin instead of splitting again (big_ok 2:
// only a node of 2^31 keys or more)
// (big bins go to big_list: the bin count takes them first, so that one
// CTA's long pass over a hot k-mer overlaps the other bins)
// (level-1 nodes of several ranges always split: a final bin's keys are one range)
int launch_classify(Node* nodes, uint32_t node_lo, uint32_t node_hi, uint32_t* final_list,
                    uint32_t* big_list, LevelCounters* ctr, int bin_cap, int split_target,
                    int big_ok, const Ranges& rg, cudaStream_t s);
// for each NODE_RETRY node of the final list: a proxy copy at n_nodes + i (i
// from *count), the node itself becomes a split node of width 0 over its proxy
int launch_make_proxies(Node* nodes, const uint32_t* final_list, uint32_t n_final,
                        uint32_t n_nodes, unsigned int* count, cudaStream_t s);
int launch_assign(Node* nodes, uint32_t node_lo, uint32_t node_hi, uint32_t child_base,
                  Tile* tiles, LevelCounters* ctr, const Ranges& rg, cudaStream_t s);
// one upload chunk's level-1 layout: its rows H_c (G x F1) give its bucket
// totals T_c and starts S_c (its region follows the *running keys of earlier
// chunks, which grows by its own) and its per-CTA write offsets O_c
int launch_chunk_scan(const uint32_t* H_c, int G, int F1, uint32_t* T_c, uint64_t* S_c,
                      unsigned long long* running, uint64_t* O_c, cudaStream_t s);
// level-1 nodes from all rows of H (sizes and the starts they would have if
// each bucket's keys were one range)
int launch_l1_nodes(const uint32_t* H, int rows, int F1, Node* nodes, int shift1, cudaStream_t s);
int launch_tile_hist(const Node* nodes, const Tile* tiles, uint32_t n_tiles,
                     const uint64_t* A, const uint64_t* B, uint32_t* TH, cudaStream_t s);
int launch_node_scan(Node* nodes, uint32_t node_lo, uint32_t node_hi, Tile* tiles,
                     uint32_t* TH, cudaStream_t s);
int launch_tile_scatter(const Node* nodes, const Tile* tiles, uint32_t n_tiles, uint64_t* A,
                        uint64_t* B, const uint32_t* TH, int max_width, cudaStream_t s);
// ctr: [4] (low 32 bits) = bin ticket, [5] = count overflow flag, [6] = hash bins that fell
// back to sorting, [7] = big skewed bins that must be re-partitioned (NODE_RETRY),
// [17] = big skewed bins counted (all zeroed by the caller); use_hash selects
// the hash-first bin count
// bins: big_list[0, n_big) first, then final_list[0, n_final)
// with use_hash and fb_list (room for n_final entries), the final list goes
// through the packed-table kernel first (ctr[19] its ticket, ctr[20] the bins
// it leaves in fb_list, ctr[21] the bins it counts; all zeroed by the caller)
int launch_bin_count(Node* nodes, const uint32_t* big_list, uint32_t n_big,
                     const uint32_t* final_list, uint32_t n_final, uint64_t* A, uint64_t* B,
                     uint32_t* C, int use_hash, unsigned long long* ctr, int sm_count,
                     cudaStream_t s, uint32_t* fb_list = nullptr);
int launch_aggregate(Node* nodes, uint32_t node_lo, uint32_t node_hi, cudaStream_t s);
// level-1 nodes [b0, b1) follow the *total_d distinct keys before them
int launch_l1_offsets(Node* nodes, uint32_t b0, uint32_t b1, unsigned long long* total_d,
                      cudaStream_t s);
int launch_child_offsets(Node* nodes, uint32_t node_lo, uint32_t node_hi, cudaStream_t s);
int launch_compact(const Node* nodes, const uint32_t* final_list, uint32_t n_final,
                   const uint64_t* A, const uint64_t* B, const uint32_t* C, uint64_t* out_k,
                   uint32_t* out_c, cudaStream_t s);

int bin_count_smem_bytes(int variant);

// ------------------------------------------------ graph-driven wave tail
// A batch wave's partition levels, bin count, tree offsets and compact run as
// one CUDA graph: the level loop and the two tree passes are conditional
// WHILE nodes, and every kernel reads the extents it works on from WaveCtl
// (device memory) instead of from launch arguments, so the graph is built
// once per set of buffers and replayed for every wave.
constexpr int kGraphMaxLevels = 16;   // more levels: the wave is counted without the graph
constexpr int kGraphSplitBits = 10;   // widest split in the graph (the tile scatter's
                                      // shared memory is sized for it: two CTAs per SM)
struct WaveCtl {
  uint32_t lo, hi;           // nodes of the current level
  uint32_t next_lo, next_hi;  // nodes of the next level (set by the plan)
  uint32_t node_end;         // nodes [0, node_end) exist
  uint32_t child_base;       // first child of the current level's split nodes
  uint32_t n_tiles;          // partition tiles of the current level
  uint32_t stop;             // the levels have ended: level kernels do nothing
  uint32_t overflow;         // a buffer or the level table was too small: the host
                             // counts the wave again without the graph
  uint32_t too_big;          // a split node held >= 2^32 keys
  uint32_t n_levels;         // levels so far, each recorded below
  uint32_t F1;               // level-1 nodes
  uint32_t nodes_cap, tiles_cap;
  unsigned long long th_cap;       // tile-histogram entries
  unsigned long long split_keys;   // keys the levels partitioned (all levels)
  int32_t pass;              // tree passes: the level the next pass works on
  uint32_t pass_skip;        // the current pass has nothing to do
  uint32_t cur_lo, cur_hi;   // nodes of the current tree pass
  // work tickets: tiles of the level's histogram and scatter, final and
  // big-bin nodes of the compact (taken one at a time, so blocks that finish
  // early take more, as with a grid of one block per item)
  uint32_t tk_hist, tk_scatter, tk_compact[2];
  // the wave's table (each wave has its own: read here, not built into the graph)
  uint64_t* out_k;
  uint32_t* out_c;
  uint32_t lv_lo[kGraphMaxLevels], lv_hi[kGraphMaxLevels];
};
static_assert(sizeof(WaveCtl) <= 256, "WaveCtl lives in the last 256 bytes of the counter block");

// Fixed buffers and parameters a wave graph is built over.
struct WaveGraphArgs {
  Node* nodes;
  uint32_t* finals;
  uint32_t* bigs;
  uint32_t* fb_list;
  Tile* tiles;
  uint32_t* TH;
  uint64_t* A;
  uint64_t* B;
  uint32_t* C;
  LevelCounters* lc;
  unsigned long long* ctr;
  WaveCtl* wc;
  int bin_cap, split_target, big_ok, use_hash, sm_count;
};
// Build the graph of a wave's tail over `a`.  The level loop is one WHILE
// node whose body runs one partition level; bottom-up sums and top-down
// offsets are WHILE nodes over the recorded levels.  Returns a CUDA status.
cudaError_t build_wave_graph(const WaveGraphArgs& a, cudaStream_t capture_stream,
                             cudaGraph_t* out);

}  // namespace dk
