// Engine state behind the C ABI (host side).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <deque>
#include <functional>
#include <vector>

#include "../../include/dakc_gb300.h"
#include "dk_internal.cuh"

namespace dk {

// status plumbing of the engine's host code: a failed CUDA call records its
// text on engine `e` (in scope) and returns DK_ERR_CUDA
#define DK_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t _e = (call);                                                 \
    if (_e != cudaSuccess) {                                                 \
      e->set_error(std::string(#call) + ": " + cudaGetErrorString(_e));     \
      return DK_ERR_CUDA;                                                    \
    }                                                                        \
  } while (0)

#define DK_TRY(expr)            \
  do {                          \
    int _rc = (expr);           \
    if (_rc != DK_OK) return _rc; \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

struct Engine;
struct Arena {
  // make b hold >= bytes (contents are not preserved); respects the budget
  static int ensure(Engine* e, DevBuf& b, size_t bytes);
  static void release(Engine* e, DevBuf& b);
};

// A table allocation (pinned host or device) handed out by dk_count and
// returned to the pool by dk_table_free.
struct TableBuf {
  void* k = nullptr;
  void* c = nullptr;
  uint64_t cap = 0;
  uint64_t id = 0;
  bool on_device = false;
  bool in_use = false;
  uint32_t refs = 0;  // tables handed out on this buffer (batch results share one)
};

// Page-locked host tables, shared by a context's engine and its serving
// workers: a table released by any of them is reused by the next count of any.
struct HostPool {
  std::mutex mu;
  std::deque<TableBuf> tables;  // deque: stable addresses
  ~HostPool();
};

struct DeviceTable {
  uint64_t* k;
  uint32_t* c;
  uint64_t n;
  uint64_t n_kmers;
};

int64_t frame_lines(uint64_t nbytes, int W);
bool convention_ok(const dk_input_desc& d);

struct Engine;

// Line ranges of the read sets counted together by dk_count_batch.  Host
// copies plus device mirrors used by the level-1 kernels.
struct JobSet {
  int njobs = 0;
  std::vector<uint64_t> job_start;  // njobs + 1 line offsets
  std::vector<uint64_t> job_end;    // lines parsed per job end here
  uint64_t* d_start = nullptr;      // device mirrors (inside the engine's job arena)
  uint64_t* d_end = nullptr;
  unsigned long long* d_nul = nullptr;
  // level-1 buckets: job j owns [job_base[j], job_base[j+1]), 2^job_bits[j] of them,
  // split by the top job_bits[j] bits of its k-mers
  std::vector<uint32_t> job_base;   // njobs + 1
  std::vector<uint8_t> job_bits;    // njobs
  std::vector<int16_t> bucket_shift;  // F1: free key bits below each bucket's prefix
  uint32_t* d_base = nullptr;
  uint8_t* d_bits = nullptr;
  int16_t* d_bshift = nullptr;
  int F1() const { return job_base.empty() ? njobs : (int)job_base.back(); }
  std::vector<Node> nodes;          // level-1 nodes read back after the count
  int upload_bounds(Engine* e);     // job_end -> device, job_nul reset
  int apply_nul(Engine* e);         // shorten job_end to each job's first NUL-led line
  void clear_results() { nodes.clear(); }
};

struct Engine {
  int device = 0;
  int sm_count = 0;
  uint64_t budget = 0;
  uint64_t flags = 0;  // dk_config.flags
  // the device reads pageable host memory in place (coherent access through the
  // host's page tables): pageable reads are then copied in by kernels
  bool host_direct = false;
  uint64_t dev_bytes = 0, dev_peak = 0;
  cudaStream_t stream = nullptr;            // kernels
  cudaStream_t s_in = nullptr, s_out = nullptr;  // batch uploads / table downloads
  std::mutex mu;
  std::mutex err_mu;                         // last_error (batch uploads run on a helper thread)
  std::string last_error;
  dk_stats stats{};
  dk_stats stats_batch{};
  uint64_t launches = 0;

  // device arenas
  DevBuf text, text2, keysA, keysB, cnt, H, O, nodes, tiles, TH, finals, bigs, rng, ctrs;
  DevBuf fbl;  // final nodes the packed bin kernel leaves to the general one
  // batch waves: the tail of a wave (partition levels, bins, tree offsets,
  // compact) as one launch of a CUDA graph built over the buffers in
  // wave_args; rebuilt when a buffer moves
  cudaStream_t s_cap = nullptr;       // graph capture only
  cudaGraph_t wave_graph = nullptr;
  cudaGraphExec_t wave_exec = nullptr;
  WaveGraphArgs wave_args = {};
  WaveCtl* h_wc = nullptr;            // page-locked: the control block a wave starts from
  bool graph_off = false;             // the current count runs its tail from the host
  double graph_scale = 1.0;           // graph buffers per k-mer; doubles when a wave outgrew them
  static constexpr int kGraphRetry = 1;  // wave_graph_tail: count the wave without the graph
  int wave_graph_tail(int F1, uint64_t n_kmers, int bin_target, bool use_hash, int big_ok,
                      double scale, uint64_t* tail);
  size_t node_cap_needed = 0;
  uint64_t* out_k = nullptr;
  uint32_t* out_c = nullptr;
  std::deque<TableBuf> tables;  // device tables; deque: stable addresses; guarded by pool_mu
  std::mutex pool_mu;           // tables may be released while a count runs
  std::shared_ptr<HostPool> hpool = std::make_shared<HostPool>();  // host tables

  cudaEvent_t ev_stage[8] = {};
  static constexpr int kKEvents = 512;
  struct KEv { int slot, e0, e1, n; };
  cudaEvent_t kev_pool[kKEvents] = {};
  std::vector<KEv> kev;
  int kev_next = 0;
  int kbegin();
  void kend(int slot, int i0, int n);
  void kresolve();
  cudaEvent_t ev_h2d0 = nullptr, ev_d2h1 = nullptr;
  // page-locked mailboxes for the engine's small control copies, moved by a
  // kernel (launch_copy_small) instead of a copy engine
  static constexpr size_t kMailboxBytes = 1 << 20;
  void* h_scratch = nullptr;  // device -> host
  void* h_up = nullptr;       // host -> device
  void* d_scratch = nullptr;  // device views of the two
  void* d_up = nullptr;
  int write_small(void* ddst, const void* hsrc, size_t bytes);  // synchronous
  void* stage_pinned[2] = {nullptr, nullptr};
  cudaEvent_t stage_ev[2] = {nullptr, nullptr};
  // batch pipeline: per text/table buffer, upload start/end and download start/end
  cudaEvent_t ev_in0[2] = {}, ev_in1[2] = {}, ev_out0[2] = {}, ev_out1[2] = {};
  int stage_next = 0;

  // tuned (l1_bits, bin_target, variant) per input shape, from dk_autotune
  struct Tune {
    int l1_bits = 0, bin_target = 0, variant = 0;
    double ms = 0;
  };
  std::map<uint64_t, Tune> tunes;
  static uint64_t shape_key(int W, int k, uint64_t n_upper);
  int autotune(const char* text, uint64_t nbytes, const dk_input_desc* desc, dk_tune* out);

  // operations on finished tables (dk_table_ops.cu)
  DevBuf aux;  // their scratch
  int table_histogram(const dk_table* t, uint32_t nb, uint64_t* hist, uint32_t* min_bucket);
  int table_filter(const dk_table* t, uint32_t min_count, dk_table* out);
  int table_lookup(const dk_table* t, const uint64_t* q, uint64_t nq, uint32_t* counts);
  int table_pairs(const dk_table* t, void* out);

  int init(const dk_config* cfg);
  ~Engine();
  void set_error(const std::string& m);
  int sync_read(const void* dsrc, size_t bytes, void* hdst);
  struct Seg {
    const char* h;
    uint64_t n;
    uint64_t doff;  // destination offset
  };
  int upload(const char* h, uint64_t nbytes, uint8_t* d);
  int upload_segments(const std::vector<Seg>& segs, uint8_t* d, cudaStream_t st);
  int acquire_table(uint64_t n, bool on_device, TableBuf** out);
  int release_table(uint64_t id);
  int count_device(const uint8_t* d_text, uint64_t nbytes, const dk_input_desc& desc,
                   DeviceTable* out, JobSet* js = nullptr);
  // When set, count_device counts in out_groups groups of level-1 buckets
  // (split by k-mers) and calls out_sink(first, n, kmers_done, kmers_total)
  // once a group's table slice [first, first + n) is final in device memory;
  // the next group runs while the sink moves that slice.
  std::function<int(uint64_t, uint64_t, uint64_t, uint64_t)> out_sink;
  int out_groups = 1;
  // Reads uploaded in chunks of lines on s_in (count_locked): chunk c holds
  // lines [lines[c], lines[c+1]) and has landed when ev[c] completes.  When
  // set, count_device counts each chunk as it lands and scatters chunk by
  // chunk with the same lines per CTA.
  static constexpr int kMaxChunks = 8;
  struct ChunkPlan {
    int n = 0;
    uint64_t lines[kMaxChunks + 1] = {};
    cudaEvent_t ev[kMaxChunks] = {};
  };
  ChunkPlan chunks;
  int count_batch(const dk_job* jobs, int njobs, const dk_input_desc* desc, dk_table* outs);
  DevBuf jobmeta;  // device job_start / job_end / job_nul
  int count(const char* text, uint64_t nbytes, bool text_on_device, const dk_input_desc* desc,
            dk_table* out);
  int count_locked(const char* text, uint64_t nbytes, bool text_on_device,
                   const dk_input_desc* desc, dk_table* out);
  // reads in another layout (dk_ingest.cu)
  int count_format(const char* text, uint64_t nbytes, int format, const dk_input_desc* desc,
                   dk_table* out, int* width);
};

}  // namespace dk
