// Host side of the k-mer counting engine: context, device arenas, the
// stream-ordered pipeline and the C ABI declared in include/dakc_gb300.h.
//
// The reference's entry point is the kmercounter constructor
// (dakc/src/kcounter/kcounter.hpp:84-99 -> perform_kcount, kcounter.cpp:247-507);
// dk_count is its one-GPU replacement.  Every stage of the reference maps to
// kernels launched here on the context's stream:
//   read_till_buf_max + get_kmers + owner_pe + send   -> l1_count, l1_scatter
//   (kcounter_funcs.cpp:25-111, kcounter.cpp:29-54,146-300)
//   ska_sort + run-length reduce (kcounter.cpp:385-414) -> partition levels +
//                                                         bin_count + compact
#include "dk_internal.cuh"
#include "dk_engine.hpp"
#include "../../include/dakc_gb300.h"

#include <cuda_runtime.h>
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace dk {

// host tables of at least this many k-mers (bound) move out while the count
// runs, in this many groups of level-1 buckets (2.4 G k-mers end to end,
// median of 10 calls: 16 groups 69.8 ms, 20 69.3, 24 69.0, 28 69.3, 32 69.8;
// more groups add device time, fewer leave a longer download tail)
constexpr uint64_t kStreamMinKmers = 64ull << 20;
constexpr int kStreamGroups = 24;
// page-locked reads of at least this many bytes upload in chunks, each
// counted as soon as it lands
constexpr uint64_t kChunkMinBytes = 64ull << 20;

// --------------------------------------------------------------- helpers
static int ceil_log2(uint64_t x) {
  int b = 0;
  while ((1ull << b) < x && b < 63) ++b;
  return b;
}

int Arena::ensure(Engine* e, DevBuf& b, size_t bytes) {
  if (b.cap >= bytes) return DK_OK;
  const size_t want = std::max(bytes, b.cap + b.cap / 4);  // grow geometrically
  if (b.p) {
    cudaFree(b.p);
    e->dev_bytes -= b.cap;
    b.p = nullptr;
    b.cap = 0;
  }
  if (e->budget && e->dev_bytes + want > e->budget) {
    if (e->dev_bytes + bytes > e->budget) return DK_ERR_ADMISSION;
  }
  size_t got = want;
  if (e->budget && e->dev_bytes + got > e->budget) got = bytes;
  cudaError_t st = cudaMalloc(&b.p, got);
  if (st != cudaSuccess && got != bytes) {
    cudaGetLastError();
    got = bytes;
    st = cudaMalloc(&b.p, got);
  }
  if (st != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    return DK_ERR_OOM;
  }
  b.cap = got;
  e->dev_bytes += got;
  e->dev_peak = std::max(e->dev_peak, e->dev_bytes);
  return DK_OK;
}

void Arena::release(Engine* e, DevBuf& b) {
  if (b.p) {
    cudaFree(b.p);
    e->dev_bytes -= b.cap;
  }
  b.p = nullptr;
  b.cap = 0;
}

void Engine::set_error(const std::string& m) {
  std::lock_guard<std::mutex> g(err_mu);
  last_error = m;
}

// per-kernel CUDA-event timing on the engine stream; resolved after the final sync
int Engine::kbegin() {
  if (kev_next >= kKEvents) return -1;
  const int i = kev_next++;
  cudaEventRecord(kev_pool[i], stream);
  return i;
}

void Engine::kend(int slot, int i0, int n) {
  if (i0 < 0 || kev_next >= kKEvents || n == 0) return;
  const int i1 = kev_next++;
  cudaEventRecord(kev_pool[i1], stream);
  kev.push_back({slot, i0, i1, n});
}

void Engine::kresolve() {
  for (const auto& r : kev) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, kev_pool[r.e0], kev_pool[r.e1]) == cudaSuccess) {
      stats.ms_kernel[r.slot] += ms;
      stats.launches_kernel[r.slot] += (uint64_t)r.n;
    }
  }
  cudaGetLastError();
  kev.clear();
  kev_next = 0;
}

#define TIMED(slot, expr)              \
  do {                                 \
    const int _i0 = kbegin();          \
    const int _n = (expr);             \
    launches += (uint64_t)_n;          \
    kend((slot), _i0, _n);             \
  } while (0)

int Engine::init(const dk_config* cfg) {
  Engine* e = this;
  device = cfg ? cfg->device : 0;
  flags = cfg ? cfg->flags : 0;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device) {
    cudaGetLastError();
    set_error("no CUDA device");
    return DK_ERR_NO_DEVICE;
  }
  DK_CUDA(cudaSetDevice(device));
  cudaDeviceProp p;
  DK_CUDA(cudaGetDeviceProperties(&p, device));
  sm_count = p.multiProcessorCount;
  int pma = 0;
  DK_CUDA(cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, device));
  host_direct = pma != 0 && !(flags & DK_FLAG_STAGE_PAGEABLE);
  if (p.major * 10 + p.minor < 100) {
    set_error("engine is built for sm_103a; device is older");
    return DK_ERR_NO_DEVICE;
  }
  size_t fr = 0, tot = 0;
  DK_CUDA(cudaMemGetInfo(&fr, &tot));
  budget = (cfg && cfg->mem_budget) ? cfg->mem_budget : (uint64_t)(0.8 * (double)fr);
  DK_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  DK_CUDA(cudaStreamCreateWithFlags(&s_in, cudaStreamNonBlocking));
  DK_CUDA(cudaStreamCreateWithFlags(&s_out, cudaStreamNonBlocking));
  DK_CUDA(cudaStreamCreateWithFlags(&s_cap, cudaStreamNonBlocking));
  DK_CUDA(cudaMallocHost(&h_wc, sizeof(WaveCtl)));
  for (auto* evs : {ev_in0, ev_in1, ev_out0, ev_out1})
    for (int i = 0; i < 2; ++i) DK_CUDA(cudaEventCreate(&evs[i]));
  for (auto& ev : ev_stage) DK_CUDA(cudaEventCreate(&ev));
  for (auto& ev : kev_pool) DK_CUDA(cudaEventCreate(&ev));
  DK_CUDA(cudaEventCreate(&ev_h2d0));
  DK_CUDA(cudaEventCreate(&ev_d2h1));
  DK_CUDA(cudaMallocHost(&h_scratch, kMailboxBytes));
  DK_CUDA(cudaMallocHost(&h_up, kMailboxBytes));
  DK_CUDA(cudaHostGetDevicePointer(&d_scratch, h_scratch, 0));
  DK_CUDA(cudaHostGetDevicePointer(&d_up, h_up, 0));
  return DK_OK;
}

Engine::~Engine() {
  for (cudaStream_t st : {stream, s_in, s_out})
    if (st) cudaStreamSynchronize(st);
  for (DevBuf* b : {&text, &text2, &keysA, &keysB, &cnt, &H, &O, &nodes, &tiles, &TH, &finals, &bigs, &rng, &ctrs,
                    &aux, &fbl})
    Arena::release(this, *b);
  for (auto& t : tables) {  // device tables (host tables live in the shared pool)
    cudaFree(t.k);
    cudaFree(t.c);
  }
  for (auto& ev : ev_stage)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : kev_pool)
    if (ev) cudaEventDestroy(ev);
  if (ev_h2d0) cudaEventDestroy(ev_h2d0);
  if (ev_d2h1) cudaEventDestroy(ev_d2h1);
  for (auto& ev : chunks.ev)
    if (ev) cudaEventDestroy(ev);
  if (h_scratch) cudaFreeHost(h_scratch);
  if (h_up) cudaFreeHost(h_up);
  for (auto& s : stage_pinned)
    if (s) cudaFreeHost(s);
  for (auto* evs : {ev_in0, ev_in1, ev_out0, ev_out1})
    for (int i = 0; i < 2; ++i)
      if (evs[i]) cudaEventDestroy(evs[i]);
  if (wave_exec) cudaGraphExecDestroy(wave_exec);
  if (wave_graph) cudaGraphDestroy(wave_graph);
  if (h_wc) cudaFreeHost(h_wc);
  for (cudaStream_t st : {stream, s_in, s_out, s_cap})
    if (st) cudaStreamDestroy(st);
}

// Read device bytes after the stream's prior work (synchronous): a kernel
// writes them into the page-locked mailbox.
int Engine::sync_read(const void* dsrc, size_t bytes, void* hdst) {
  Engine* e = this;
  for (size_t off = 0; off < bytes; off += kMailboxBytes) {
    const size_t n = std::min(kMailboxBytes, bytes - off);
    launch_copy_small((const uint8_t*)dsrc + off, d_scratch, n, stream);
    DK_CUDA(cudaGetLastError());
    DK_CUDA(cudaStreamSynchronize(stream));
    std::memcpy((uint8_t*)hdst + off, h_scratch, n);
  }
  return DK_OK;
}

// Write host bytes to device memory, ordered on the stream and complete on
// return: a kernel reads them from the page-locked mailbox.
int Engine::write_small(void* ddst, const void* hsrc, size_t bytes) {
  Engine* e = this;
  for (size_t off = 0; off < bytes; off += kMailboxBytes) {
    const size_t n = std::min(kMailboxBytes, bytes - off);
    std::memcpy(h_up, (const uint8_t*)hsrc + off, n);
    launch_copy_small(d_up, (uint8_t*)ddst + off, n, stream);
    DK_CUDA(cudaGetLastError());
    DK_CUDA(cudaStreamSynchronize(stream));  // the mailbox is refilled next
  }
  return DK_OK;
}

// DAKC's and PakMan*'s conventions, at every line width the engine takes
// (thread-per-line kernels up to kLineMaxW bytes, warp-per-line kernels beyond)
bool convention_ok(const dk_input_desc& d) {
  return d.convention == DK_CONV_DAKC || d.convention == DK_CONV_PAKMAN;
}

// framing: lines in a buffer of nbytes (host-side part; NUL lines are found on device)
int64_t frame_lines(uint64_t nbytes, int W) {
  if (W < 1) return DK_ERR_INVALID_ARG;
  if (nbytes == 0) return 0;
  const uint64_t stride = (uint64_t)W + 1;
  const uint64_t rem = nbytes % stride;
  if (rem != 0 && rem != (uint64_t)W) return DK_ERR_INVALID_ARG;
  return (int64_t)((nbytes + 1) / stride);
}

// Smallest (8 + m) * 2^e, m < 8, that is >= n.
static uint64_t size_class(uint64_t n) {
  if (n <= 16) return n;
  int e = 0;
  while ((16ull << e) <= n) ++e;  // 2^(e+3) <= n < 2^(e+4)
  const uint64_t step = 1ull << e;
  return (n + step - 1) / step * step;
}

HostPool::~HostPool() {
  for (auto& t : tables) {
    cudaFreeHost(t.k);
    cudaFreeHost(t.c);
  }
}

// table handles are unique across all pools of the process
static std::atomic<uint64_t> g_table_ids{0};

// Table storage: pools of allocations reused across calls (device tables per
// engine, page-locked host tables shared with the context's serving workers).
int Engine::acquire_table(uint64_t n, bool on_device, TableBuf** out) {
  Engine* e = this;
  std::deque<TableBuf>& tables = on_device ? this->tables : hpool->tables;
  std::lock_guard<std::mutex> g(on_device ? pool_mu : hpool->mu);
  TableBuf* best = nullptr;
  for (auto& t : tables)
    if (!t.in_use && t.on_device == on_device && t.cap >= n && (!best || t.cap < best->cap)) best = &t;
  if (!best) {
    TableBuf t;
    t.on_device = on_device;
    // capacities in size classes (eight per power of two, at most 12.5%
    // over), so that tables of varying sizes -- batches of different jobs --
    // reuse pooled buffers instead of pinning or allocating new ones
    t.cap = size_class(std::max<uint64_t>(n, 1));
    if (on_device && budget && dev_bytes + t.cap * 12 > budget) {
      // pooled tables nobody holds give their memory back, largest first,
      // until the new one fits.  Entries stay (emptied, capacity 0): callers
      // hold pointers into the deque, so nothing is erased
      std::vector<TableBuf*> idle;
      for (auto& x : tables)
        if (!x.in_use && x.cap) idle.push_back(&x);
      std::sort(idle.begin(), idle.end(),
                [](const TableBuf* a, const TableBuf* b) { return a->cap > b->cap; });
      for (TableBuf* x : idle) {
        if (dev_bytes + t.cap * 12 <= budget) break;
        cudaFree(x->k);
        cudaFree(x->c);
        dev_bytes -= x->cap * 12;
        x->k = nullptr;
        x->c = nullptr;
        x->cap = 0;
      }
    }
    if (on_device) {
      if (budget && dev_bytes + t.cap * 12 > budget) {
        set_error("a device table does not fit the memory budget");
        return DK_ERR_ADMISSION;
      }
      if (cudaMalloc(&t.k, t.cap * 8) != cudaSuccess || cudaMalloc(&t.c, t.cap * 4) != cudaSuccess) {
        cudaGetLastError();
        if (t.k) cudaFree(t.k);
        return DK_ERR_OOM;
      }
      dev_bytes += t.cap * 12;
      dev_peak = std::max(dev_peak, dev_bytes);
    } else {
      if (cudaMallocHost(&t.k, t.cap * 8) != cudaSuccess ||
          cudaMallocHost(&t.c, t.cap * 4) != cudaSuccess) {
        cudaGetLastError();
        if (t.k) cudaFreeHost(t.k);
        return DK_ERR_OOM;
      }
    }
    t.id = ++g_table_ids;
    TableBuf* slot = nullptr;  // an emptied entry, else a new one
    for (auto& x : tables)
      if (!x.in_use && !x.cap && x.on_device == on_device) {
        slot = &x;
        break;
      }
    if (slot) {
      *slot = t;
      best = slot;
    } else {
      tables.push_back(t);
      best = &tables.back();
    }
  }
  best->in_use = true;
  best->refs = 1;
  *out = best;
  (void)e;
  return DK_OK;
}

static int release_in(std::deque<TableBuf>& tables, uint64_t id) {
  for (auto& t : tables)
    if (t.id == id && t.in_use) {
      if (t.refs > 1) {
        --t.refs;
      } else {
        t.refs = 0;
        t.in_use = false;
      }
      return DK_OK;
    }
  return DK_ERR_NOT_FOUND;
}

int Engine::release_table(uint64_t id) {
  {
    std::lock_guard<std::mutex> g(pool_mu);
    if (release_in(tables, id) == DK_OK) return DK_OK;
  }
  std::lock_guard<std::mutex> g(hpool->mu);
  return release_in(hpool->tables, id);
}

// Level-1 split bits for a count of at most n_upper k-mers: one scatter pass
// when 2^12 buckets reach the bin target, else the fan-out split evenly
// between level 1 and the first partition level.
static int l1_bits_for(uint64_t n_upper, double target) {
  if ((double)n_upper / 4096.0 <= target) return ceil_log2((uint64_t)((double)n_upper / target) + 1);
  const int total = ceil_log2((uint64_t)((double)n_upper / target) + 1);
  return (total + 1) / 2;
}

static int floor_log2_int(int v) {
  int b = 0;
  while ((2 << b) <= v) ++b;
  return b;
}

// ------------------------------------------------------------ batch mode
// The job arrays live back to back in the engine's job arena (d_start ...
// d_bits), so one mailbox copy uploads them all.
int JobSet::upload_bounds(Engine* e) {
  const size_t n = (size_t)njobs;
  std::vector<uint8_t> blob((uint8_t*)(d_bits + n) - (uint8_t*)d_start);
  auto put = [&](const void* dptr, const void* src, size_t bytes) {
    std::memcpy(blob.data() + ((const uint8_t*)dptr - (const uint8_t*)d_start), src, bytes);
  };
  put(d_start, job_start.data(), (n + 1) * 8);
  put(d_end, job_end.data(), n * 8);
  put(d_nul, job_start.data() + 1, n * 8);  // no NUL-led line found yet
  put(d_base, job_base.data(), (n + 1) * 4);
  put(d_bshift, bucket_shift.data(), bucket_shift.size() * 2);
  put(d_bits, job_bits.data(), n);
  return e->write_small(d_start, blob.data(), blob.size());
}

int JobSet::apply_nul(Engine* e) {
  std::vector<uint64_t> nul((size_t)njobs);
  DK_TRY(e->sync_read(d_nul, (size_t)njobs * 8, nul.data()));
  for (int j = 0; j < njobs; ++j) job_end[j] = std::min(job_end[j], nul[j]);
  return DK_OK;
}

// Count many read sets in memory-bounded waves; each wave is one pass of the
// device pipeline in which every job owns its own level-1 buckets.  Waves are
// pipelined over three streams: while wave w is counted (`stream`), a helper
// thread stages and uploads wave w+1 into the other text buffer (`s_in`), and
// wave w-1's table is copied back to the host (`s_out`).  Large batches are
// cut into at least four waves so that the three stages overlap.
int Engine::count_batch(const dk_job* jobs, int njobs, const dk_input_desc* desc, dk_table* outs) {
  Engine* e = this;
  std::lock_guard<std::mutex> g(mu);
  const auto w0 = std::chrono::steady_clock::now();
  if (!jobs || njobs < 0 || !desc || !outs) {
    set_error("null argument");
    return DK_ERR_INVALID_ARG;
  }
  for (int j = 0; j < njobs; ++j) std::memset(&outs[j], 0, sizeof(dk_table));
  if (desc->k < 1 || desc->k > 32 || desc->line_width < 1 || desc->line_width > 1024 ||
      !convention_ok(*desc) || desc->variant < DK_VARIANT_AUTO ||
      desc->variant > DK_VARIANT_HASH ||
      (desc->residency != DK_RESIDENT_HOST && desc->residency != DK_RESIDENT_DEVICE)) {
    set_error("invalid input descriptor");
    return DK_ERR_INVALID_ARG;
  }
  // device residency: each wave's device table is handed out as it is (its
  // jobs' tables are runs of it), nothing is copied back
  const bool on_dev = desc->residency == DK_RESIDENT_DEVICE;
  const int W = desc->line_width, k = desc->k;
  // batched read sets are mostly small and of low coverage (most k-mers
  // distinct), so their bins default to kBatchBinTarget keys: bins of the
  // plain default would hold more distinct k-mers than the packed bin table
  // (256 C4-shaped sets: bin count 39.7 ms at 6,000 keys, 30.3 at 4,500, 28.0
  // at 3,000)
  dk_input_desc bdesc = *desc;
  if (bdesc.bin_target <= 0) bdesc.bin_target = kBatchBinTarget;
  const uint64_t stride = (uint64_t)W + 1;
  const uint64_t per_line = W >= k ? (uint64_t)(W - k + 1) : 0;
  std::vector<uint64_t> lines(njobs);
  for (int j = 0; j < njobs; ++j) {
    const int64_t L = frame_lines(jobs[j].nbytes, W);
    if (L < 0 || (!jobs[j].text && jobs[j].nbytes)) {
      set_error("job " + std::to_string(j) + ": size is not a whole number of lines");
      return DK_ERR_INVALID_ARG;
    }
    lines[j] = (uint64_t)L;
  }
  DK_CUDA(cudaSetDevice(device));
  // device bytes per job while its wave runs: text in two buffers, two key
  // buffers, staged counts, a device table and one in flight to the host
  auto est = [&](int j) { return 2 * lines[j] * stride + 44 * lines[j] * per_line + 4096; };
  uint64_t total = 0;
  for (int j = 0; j < njobs; ++j) total += est(j);
  const uint64_t mem_cap = budget ? (uint64_t)(0.7 * (double)budget) : ~0ull;
  const uint64_t wave_cap = std::min(mem_cap, std::max<uint64_t>(total / 4, 256ull << 20));
  const int max_wave_jobs = l1_max_buckets(W, true);  // every job needs one bucket at least
  const double target = (double)std::min(bdesc.bin_target, kBinCap / 2);
  struct Wave {
    int j0 = 0, j1 = 0;
    JobSet js;
    std::vector<Seg> segs;
    uint64_t bytes = 0;
  };
  std::vector<Wave> waves;
  uint64_t max_bytes = 0;
  for (int j0 = 0; j0 < njobs;) {
    int j1 = j0;
    uint64_t bytes = 0;
    while (j1 < njobs && j1 - j0 < max_wave_jobs && (j1 == j0 || bytes + est(j1) <= wave_cap)) {
      bytes += est(j1);
      ++j1;
    }
    if (bytes > mem_cap) {
      set_error("job " + std::to_string(j0) + " alone exceeds the memory budget");
      return DK_ERR_ADMISSION;
    }
    Wave wv;
    wv.j0 = j0;
    wv.j1 = j1;
    const int nj = j1 - j0;
    JobSet& js = wv.js;
    js.njobs = nj;
    js.job_start.assign(nj + 1, 0);
    for (int j = 0; j < nj; ++j) js.job_start[j + 1] = js.job_start[j] + lines[j0 + j];
    js.job_end.assign(js.job_start.begin() + 1, js.job_start.end());
    // level-1 buckets per job: the plain count's split, capped so the wave's
    // buckets fit the scatter kernel (largest jobs give up bits first)
    std::vector<int> want((size_t)std::max(nj, 1));  // a wave holds at least one job
    for (int j = 0; j < nj; ++j) {
      const int b = desc->l1_bits > 0 ? desc->l1_bits : l1_bits_for(lines[j0 + j] * per_line, target);
      want[j] = std::max(0, std::min({b, kMaxL1Bits, 2 * k}));
    }
    int cap = floor_log2_int(max_wave_jobs);
    for (;; --cap) {
      uint64_t tot = 0;
      for (int j = 0; j < nj; ++j) tot += 1ull << std::min(want[j], cap);
      if (tot <= (uint64_t)max_wave_jobs || cap == 0) break;
    }
    js.job_bits.resize(nj);
    js.job_base.assign(nj + 1, 0);
    for (int j = 0; j < nj; ++j) {
      js.job_bits[j] = (uint8_t)std::min(want[j], cap);
      js.job_base[j + 1] = js.job_base[j] + (1u << js.job_bits[j]);
    }
    js.bucket_shift.resize(js.job_base[nj]);
    for (int j = 0; j < nj; ++j)
      for (uint32_t b = js.job_base[j]; b < js.job_base[j + 1]; ++b)
        js.bucket_shift[b] = (int16_t)(2 * k - js.job_bits[j]);
    for (int j = 0; j < nj; ++j)
      if (jobs[j0 + j].nbytes)
        wv.segs.push_back(Seg{jobs[j0 + j].text, jobs[j0 + j].nbytes, js.job_start[j] * stride});
    wv.bytes = js.job_start[nj] * stride;
    max_bytes = std::max(max_bytes, wv.bytes);
    waves.push_back(std::move(wv));
    j0 = j1;
  }
  stats_batch = dk_stats();
  if (waves.empty()) {
    stats = stats_batch;
    return DK_OK;
  }
  // both text buffers are sized here, on this thread: the helper only copies
  DevBuf* tbuf[2] = {&text, &text2};
  DK_TRY(Arena::ensure(this, text, max_bytes + 64));
  if (waves.size() > 1) DK_TRY(Arena::ensure(this, text2, max_bytes + 64));
  auto stage = [this, &waves, &tbuf](size_t w) -> int {
    Engine* e = this;
    DK_CUDA(cudaSetDevice(device));
    const int b = (int)(w & 1);
    DK_CUDA(cudaEventRecord(ev_in0[b], s_in));
    DK_TRY(upload_segments(waves[w].segs, (uint8_t*)tbuf[b]->p, s_in));
    DK_CUDA(cudaEventRecord(ev_in1[b], s_in));
    return DK_OK;
  };
  double ms_device = 0, ms_h2d = 0, ms_d2h = 0;
  uint64_t launches_total = 0;
  TableBuf* dev_tb[2] = {nullptr, nullptr};  // device tables whose download may be in flight
  bool out_pending[2] = {false, false};
  int rc = stage(0);
  std::thread helper;
  int helper_rc = DK_OK;
  auto finish_download = [&](int b) -> int {
    if (!out_pending[b]) return DK_OK;
    DK_CUDA(cudaEventSynchronize(ev_out1[b]));
    float t = 0;
    cudaEventElapsedTime(&t, ev_out0[b], ev_out1[b]);
    ms_d2h += t;
    release_table(dev_tb[b]->id);
    dev_tb[b] = nullptr;
    out_pending[b] = false;
    return DK_OK;
  };
  for (size_t w = 0; rc == DK_OK && w < waves.size(); ++w) {
    const int b = (int)(w & 1);
    Wave& wv = waves[w];
    JobSet& js = wv.js;
    const int nj = wv.j1 - wv.j0;
    // wave w+1 streams in while wave w runs (its buffer's last reader, wave
    // w-1, has finished: count_device returns after its kernels complete)
    if (w + 1 < waves.size()) {
      helper = std::thread([&stage, &helper_rc, w] { helper_rc = stage(w + 1); });
    }
    rc = finish_download(b);  // the table buffer of wave w-2
    if (rc == DK_OK) rc = [&]() -> int {
      DK_CUDA(cudaStreamWaitEvent(stream, ev_in1[b], 0));
      DK_TRY(Arena::ensure(this, jobmeta, (size_t)(3 * nj + 1) * 8 + (size_t)(nj + 1) * 4 + nj +
                                              (size_t)js.F1() * 2 + 64));
      js.d_start = (uint64_t*)jobmeta.p;
      js.d_end = js.d_start + nj + 1;
      js.d_nul = (unsigned long long*)(js.d_end + nj);
      js.d_base = (uint32_t*)(js.d_nul + nj);
      js.d_bshift = (int16_t*)(js.d_base + nj + 1);
      js.d_bits = (uint8_t*)(js.d_bshift + js.F1());
      DK_TRY(acquire_table(js.job_start[nj] * per_line, true, &dev_tb[b]));
      out_k = (uint64_t*)dev_tb[b]->k;
      out_c = (uint32_t*)dev_tb[b]->c;
      DeviceTable dt;
      int r = count_device((const uint8_t*)tbuf[b]->p, wv.bytes, bdesc, &dt, &js);
      if (r != DK_OK) {
        release_table(dev_tb[b]->id);
        dev_tb[b] = nullptr;
        return r;
      }
      float t_in = 0;
      cudaEventElapsedTime(&t_in, ev_in0[b], ev_in1[b]);
      ms_h2d += t_in;
      ms_device += stats.ms_device;
      launches_total += stats.kernel_launches;
      for (int q = 0; q < 8; ++q) {
        stats_batch.ms_kernel[q] += stats.ms_kernel[q];
        stats_batch.launches_kernel[q] += stats.launches_kernel[q];
        stats_batch.ms_stage[q] += stats.ms_stage[q];
      }
      stats_batch.n_kmers += stats.n_kmers;
      stats_batch.n_distinct += stats.n_distinct;
      stats_batch.n_lines += stats.n_lines;
      stats_batch.n_bins += stats.n_bins;
      stats_batch.n_partitioned += stats.n_partitioned;
      stats_batch.n_bins_resorted += stats.n_bins_resorted;
      stats_batch.n_bins_packed += stats.n_bins_packed;
      stats_batch.n_bins_fallback += stats.n_bins_fallback;
      stats_batch.graph_waves += stats.graph_waves;
      stats_batch.graph_builds += stats.graph_builds;
      stats_batch.graph_retries += stats.graph_retries;
      stats_batch.partition_levels = std::max(stats_batch.partition_levels, stats.partition_levels);
      stats_batch.variant_used = stats.variant_used;
      TableBuf* h_tb = nullptr;
      if (on_dev) {
        // the jobs hold the wave's device table until each is freed
        h_tb = dev_tb[b];
        dev_tb[b] = nullptr;
        std::lock_guard<std::mutex> pg(pool_mu);
        h_tb->refs = (uint32_t)nj;
      } else {
        // the wave's table goes back on s_out while the next wave runs
        r = acquire_table(std::max<uint64_t>(dt.n, 1), false, &h_tb);
        if (r != DK_OK) {
          release_table(dev_tb[b]->id);
          dev_tb[b] = nullptr;
          return r;
        }
        DK_CUDA(cudaEventRecord(ev_stage[7], stream));
        DK_CUDA(cudaStreamWaitEvent(s_out, ev_stage[7], 0));
        DK_CUDA(cudaEventRecord(ev_out0[b], s_out));
        if (dt.n) {
          DK_CUDA(cudaMemcpyAsync(h_tb->k, dev_tb[b]->k, dt.n * 8, cudaMemcpyDeviceToHost, s_out));
          DK_CUDA(cudaMemcpyAsync(h_tb->c, dev_tb[b]->c, dt.n * 4, cudaMemcpyDeviceToHost, s_out));
        }
        DK_CUDA(cudaEventRecord(ev_out1[b], s_out));
        out_pending[b] = true;
        std::lock_guard<std::mutex> pg(hpool->mu);
        h_tb->refs = (uint32_t)nj;
      }
      for (int j = 0; j < nj; ++j) {
        dk_table& t = outs[wv.j0 + j];
        const bool has = !js.nodes.empty();
        uint64_t d = 0, n = 0, off = 0;
        if (has) {  // a job's buckets are consecutive in key order: its table is one run
          off = js.nodes[js.job_base[j]].out_off;
          for (uint32_t q = js.job_base[j]; q < js.job_base[j + 1]; ++q) {
            d += js.nodes[q].d;
            n += js.nodes[q].n;
          }
        }
        t.kmers = (uint64_t*)h_tb->k + off;
        t.counts = (uint32_t*)h_tb->c + off;
        t.n = d;
        t.n_kmers = n;
        t.on_device = on_dev ? 1 : 0;
        t.variant_used = stats.variant_used;
        t.handle = h_tb->id;
      }
      ++stats_batch.n_waves;
      return DK_OK;
    }();
    if (helper.joinable()) helper.join();
    if (rc == DK_OK) rc = helper_rc;
  }
  if (helper.joinable()) helper.join();
  // every download completes before the tables are handed out
  for (int b = 0; b < 2; ++b) {
    const int r = finish_download(b);
    if (rc == DK_OK) rc = r;
  }
  if (rc != DK_OK) {
    for (int j = 0; j < njobs; ++j)
      if (outs[j].handle) release_table(outs[j].handle);
    for (int j = 0; j < njobs; ++j) std::memset(&outs[j], 0, sizeof(dk_table));
    return rc;
  }
  stats_batch.ms_device = ms_device;
  stats_batch.ms_h2d = ms_h2d;
  stats_batch.ms_d2h = ms_d2h;
  stats_batch.dev_bytes_peak = dev_peak;
  stats_batch.kernel_launches = launches_total;
  stats_batch.ms_wall =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
  stats = stats_batch;
  return DK_OK;
}

// Copy host reads into device memory: one async copy when the buffer is
// pinned, else through two pinned staging slots so host memcpy overlaps the
// previous slot's DMA.
// Pages of [p, p + n): 0 if one is not mapped in this process (mincore fails
// with ENOMEM), 1 if all are mapped and resident, 2 if all are mapped but some
// are not resident (never touched, swapped out, a file not yet read).  The
// device reads pageable reads in place only in case 1: a range the caller no
// longer owns is refused rather than read by a kernel, and pages the CPU
// would first have to fault in are staged through host threads instead.
static int host_range_state(const void* p, uint64_t n) {
  if (!n) return 1;
  const uint64_t pg = (uint64_t)sysconf(_SC_PAGESIZE);
  const uintptr_t a = reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)(pg - 1);
  const uint64_t len = reinterpret_cast<uintptr_t>(p) + n - a;
  constexpr uint64_t kWin = 16384;  // pages per call
  unsigned char vec[kWin];
  int state = 1;
  for (uint64_t off = 0; off < len; off += pg * kWin) {
    const uint64_t l = std::min<uint64_t>(len - off, pg * kWin);
    if (mincore(reinterpret_cast<void*>(a + off), l, vec) != 0) return 0;
    const uint64_t np = (l + pg - 1) / pg;
    for (uint64_t i = 0; i < np && state == 1; ++i)
      if (!(vec[i] & 1)) state = 2;
  }
  return state;
}

static bool is_pinned(const void* h) {
  cudaPointerAttributes at;
  bool pinned = false;
  if (cudaPointerGetAttributes(&at, h) == cudaSuccess) pinned = (at.type == cudaMemoryTypeHost);
  cudaGetLastError();
  return pinned;
}

// Copy [dst_lo, dst_hi) of the concatenated destination layout out of the
// segments that cover it (segments sorted by destination offset).
static void gather_range(const std::vector<Engine::Seg>& segs, uint64_t dst_lo, uint64_t dst_hi,
                         uint8_t* out, uint64_t out_base) {
  size_t a = 0, b = segs.size();
  while (b - a > 1) {  // last segment starting at or before dst_lo
    const size_t m = (a + b) / 2;
    if (segs[m].doff <= dst_lo) a = m; else b = m;
  }
  for (size_t i = a; i < segs.size() && segs[i].doff < dst_hi; ++i) {
    const uint64_t s0 = std::max(dst_lo, segs[i].doff);
    const uint64_t s1 = std::min(dst_hi, segs[i].doff + segs[i].n);
    if (s1 > s0) std::memcpy(out + (s0 - out_base), segs[i].h + (s0 - segs[i].doff), s1 - s0);
  }
}

// Host -> device copy of segments laid out at segs[i].doff in d.  Pinned
// segments go straight to the DMA engine, and pageable ones the device can
// read in place (resident pages) are copied by a kernel.  Runs of the other
// pageable segments (no DMA or in-place segment between them) are packed into
// two 64 MB pinned slots by several host threads while the other slot's DMA
// runs.  A slot copy covers only its run, so it never overwrites another
// segment's bytes; bytes inside a run that no segment covers are missing
// final terminators, which are never examined.  A slot is refilled only after
// the copy that last read it has finished.
int Engine::upload_segments(const std::vector<Seg>& all, uint8_t* d, cudaStream_t st) {
  Engine* e = this;
  struct S {
    Seg sg;
    bool staged;  // packed through the pinned slots by host threads
  };
  std::vector<S> v;
  for (const Seg& sg : all)
    if (sg.n) v.push_back({sg, false});
  std::sort(v.begin(), v.end(), [](const S& x, const S& y) { return x.sg.doff < y.sg.doff; });
  bool any_pageable = false;
  for (S& x : v) {
    if (is_pinned(x.sg.h)) {
      DK_CUDA(cudaMemcpyAsync(d + x.sg.doff, x.sg.h, x.sg.n, cudaMemcpyHostToDevice, st));
      continue;
    }
    const int hs = host_direct ? host_range_state(x.sg.h, x.sg.n) : 2;
    if (hs == 0) {
      set_error("reads at an unmapped host address");
      return DK_ERR_INVALID_ARG;
    }
    if (hs == 1) {  // resident pageable bytes: the SMs read them in place
      launch_copy_in(x.sg.h, d + x.sg.doff, x.sg.n, sm_count, st);
      DK_CUDA(cudaGetLastError());
    } else {
      x.staged = true;
      any_pageable = true;
    }
  }
  if (!any_pageable) return DK_OK;
  const size_t slot = 64ull << 20;
  for (int i = 0; i < 2; ++i) {
    if (!stage_pinned[i]) DK_CUDA(cudaMallocHost(&stage_pinned[i], slot));
    if (!stage_ev[i]) DK_CUDA(cudaEventCreateWithFlags(&stage_ev[i], cudaEventDisableTiming));
  }
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nthreads = (int)std::min<unsigned>(16, std::max(1u, hw - 1));
  size_t r0 = 0;
  while (r0 < v.size()) {
    if (!v[r0].staged) { ++r0; continue; }
    size_t r1 = r0;
    std::vector<Seg> run;
    while (r1 < v.size() && v[r1].staged) run.push_back(v[r1++].sg);
    uint64_t lo = run.front().doff;
    const uint64_t end = run.back().doff + run.back().n;
    while (lo < end) {
      const int i = stage_next;
      const uint64_t hi = std::min<uint64_t>(end, lo + slot);
      DK_CUDA(cudaEventSynchronize(stage_ev[i]));
      uint8_t* buf = (uint8_t*)stage_pinned[i];
      const uint64_t len = hi - lo;
      if (len < (4u << 20) || nthreads == 1) {
        gather_range(run, lo, hi, buf, lo);
      } else {
        std::vector<std::thread> th;
        const uint64_t chunk = (len + nthreads - 1) / nthreads;
        for (int t = 0; t < nthreads; ++t) {
          const uint64_t a = lo + (uint64_t)t * chunk, b = std::min(hi, a + chunk);
          if (a >= b) break;
          th.emplace_back([&run, a, b, buf, lo] { gather_range(run, a, b, buf, lo); });
        }
        for (auto& t : th) t.join();
      }
      DK_CUDA(cudaMemcpyAsync(d + lo, buf, len, cudaMemcpyHostToDevice, st));
      DK_CUDA(cudaEventRecord(stage_ev[i], st));
      lo = hi;
      stage_next ^= 1;
    }
    r0 = r1;
  }
  return DK_OK;
}

int Engine::upload(const char* h, uint64_t nbytes, uint8_t* d) {
  return upload_segments({Seg{h, nbytes, 0}}, d, stream);
}

// The device pipeline: reads at d_text (nbytes, padded by >= 64 bytes of
// readable memory) -> sorted table in out (device).  Fills stats.
int Engine::count_device(const uint8_t* d_text, uint64_t nbytes, const dk_input_desc& desc_in,
                         DeviceTable* out, JobSet* js) {
  Engine* e = this;
  const int W = desc_in.line_width, k = desc_in.k;
  out->n = 0;
  out->n_kmers = 0;
  out->k = nullptr;
  out->c = nullptr;
  stats = dk_stats();
  int64_t L0 = js ? (int64_t)js->job_start.back() : frame_lines(nbytes, W);
  if (L0 < 0) {
    set_error("buffer size is not a whole number of lines");
    return DK_ERR_INVALID_ARG;
  }
  // parameters left automatic take the tuned choice for this input shape
  dk_input_desc desc = desc_in;
  if (!js && desc.l1_bits == 0 && desc.bin_target == 0 && desc.variant == DK_VARIANT_AUTO) {
    const uint64_t pl = (W >= k) ? (uint64_t)(W - k + 1) : 0;
    const auto it = tunes.find(shape_key(W, k, (uint64_t)L0 * pl));
    if (it != tunes.end()) {
      desc.l1_bits = it->second.l1_bits;
      desc.bin_target = it->second.bin_target;
      desc.variant = it->second.variant;
    }
  }
  // the hash-first bin count needs a free sentinel key, i.e. k <= 31
  const bool use_hash = desc.variant != DK_VARIANT_SORT && desc.k <= 31;
  stats.variant_used = use_hash ? DK_VARIANT_HASH : DK_VARIANT_SORT;
  uint64_t L = (uint64_t)L0;
  launches = 0;
  kev.clear();
  kev_next = 0;
  // with a chunked upload the device time starts when the first chunk has landed
  if (chunks.n > 1) DK_CUDA(cudaStreamWaitEvent(stream, chunks.ev[0], 0));
  DK_CUDA(cudaEventRecord(ev_stage[0], stream));
  const uint64_t per_line = (W >= k) ? (uint64_t)(W - k + 1) : 0;
  if (L == 0 || per_line == 0) {
    DK_CUDA(cudaEventRecord(ev_stage[6], stream));
    DK_CUDA(cudaEventSynchronize(ev_stage[6]));
    float ms = 0;
    cudaEventElapsedTime(&ms, ev_stage[0], ev_stage[6]);
    stats.ms_device = ms;
    stats.n_lines = L;
    return DK_OK;
  }
  // level-1 fan-out: aim at ~kBinCap/2 keys per final bin after at most one
  // 8-bit partition level
  const uint64_t n_upper = L * per_line;
  const int bin_target =
      (desc.bin_target > 0) ? std::min(desc.bin_target, kBinCap / 2) : kBinCap / 2;
  const double target = (double)bin_target;
  int B1 = desc.l1_bits > 0 ? desc.l1_bits : l1_bits_for(n_upper, target);
  B1 = std::max(1, std::min({B1, kMaxL1Bits, floor_log2_int(l1_max_buckets(W, false))}));
  B1 = std::min(B1, 2 * k);
  // batch mode: each job owns its own run of level-1 buckets (JobSet)
  const int F1 = js ? js->F1() : (1 << B1);
  const int shift1 = js ? 2 * k : 2 * k - B1;
  const int G = 2 * sm_count;

  ExtractArgs a;
  a.text = d_text;
  a.nbytes = nbytes;
  a.W = W;
  a.k = k;
  a.kmask = (~0ull) >> (64 - 2 * k);
  a.shift1 = shift1;
  a.F1 = F1;
  a.conv = desc.convention;
  a.njobs = js ? js->njobs : 0;
  a.job_start = js ? js->d_start : nullptr;
  a.job_end = js ? js->d_end : nullptr;
  a.job_nul = js ? js->d_nul : nullptr;
  a.job_base = js ? js->d_base : nullptr;
  a.job_bits = js ? js->d_bits : nullptr;
  a.line_base = 0;
  a.lines_total = (uint64_t)L0;

  // chunked: one level-1 count (and later one scatter) per uploaded chunk;
  // their per-CTA rows follow one another in H and O
  bool chunked = !js && chunks.n > 1 && W <= kLineMaxW && chunks.lines[chunks.n] == L;
  const int NC = chunked ? chunks.n : 1;
  auto chunk_args = [&](int c) {
    ExtractArgs ac = a;
    const uint64_t stride = (uint64_t)W + 1;
    const uint64_t l0 = chunks.lines[c], l1 = chunks.lines[c + 1];
    ac.text = d_text + l0 * stride;
    ac.nbytes = std::min<uint64_t>(nbytes, l1 * stride) - l0 * stride;
    ac.n_lines = l1 - l0;
    ac.line_base = l0;
    ac.lines_total = L;
    return ac;
  };
  DK_TRY(Arena::ensure(this, H, (size_t)NC * G * F1 * 4));
  DK_TRY(Arena::ensure(this, O, (size_t)NC * G * F1 * 8));
  DK_TRY(Arena::ensure(this, ctrs, 512));  // counters; the wave graph's WaveCtl at byte 256
  // device counters: [0] k-mers, [1] NUL-led line marker, [2] distinct total,
  // [3] device error (a bounded wait ran out), [4] bin ticket, [5] count overflow,
  // [6] hash bins sorted instead, [7] big bins to re-partition; LevelCounters at
  // byte 64; [16] proxy counter, [17] big bins counted, [18] keys placed by the
  // chunks scattered so far (their regions' running base)
  unsigned long long* c64 = (unsigned long long*)ctrs.p;
  LevelCounters* lc = (LevelCounters*)((char*)ctrs.p + 64);

  // Chunks in their own regions: each chunk is scattered right after its
  // count, into a region of the key buffer after the earlier chunks' keys, so
  // the level-1 scatter overlaps the upload too.  A level-1 bucket's keys
  // then lie in one range per chunk; the first partition level gathers them
  // (its tiles are cut from each range; its children are single ranges).
  // Needs the key buffer at the k-mer bound before counting, and level-1
  // nodes that can always split (more than kDenseBits free bits).
  bool regions = chunked && shift1 > kDenseBits;
  if (regions) {
    const uint64_t bound = (uint64_t)L * ((W >= k) ? (uint64_t)(W - k + 1) : 0);
    if (budget && dev_bytes - keysA.cap + bound * 8 + (size_t)NC * F1 * 12 > budget) regions = false;
    if (regions) {
      DK_TRY(Arena::ensure(this, keysA, bound * 8));
      DK_TRY(Arena::ensure(this, rng, (size_t)NC * F1 * 12));
    }
  }
  uint64_t* rS = (uint64_t*)rng.p;                          // NC x F1 range starts
  uint32_t* rT = regions ? (uint32_t*)(rS + (size_t)NC * F1) : nullptr;  // NC x F1 range sizes
  bool scattered = false;  // the regions' scatter has run

  uint64_t n_kmers = 0;
  for (int attempt = 0; attempt < 2; ++attempt) {
    a.n_lines = L;
    a.lines_total = L;
    DK_CUDA(cudaMemsetAsync(ctrs.p, 0, 256, stream));
    if (js) DK_TRY(js->upload_bounds(this));
    if (chunked) {
      for (int c = 0; c < NC; ++c) {
        DK_CUDA(cudaStreamWaitEvent(stream, chunks.ev[c], 0));
        uint32_t* Hc = (uint32_t*)H.p + (size_t)c * G * F1;
        TIMED(0, launch_l1_count(chunk_args(c), G, Hc, c64, stream));
        if (regions) {
          uint64_t* Oc = (uint64_t*)O.p + (size_t)c * G * F1;
          TIMED(7, launch_chunk_scan(Hc, G, F1, rT + (size_t)c * F1, rS + (size_t)c * F1, c64 + 18,
                                     Oc, stream));
          TIMED(1, launch_l1_scatter(chunk_args(c), G, Oc, (uint64_t*)keysA.p, c64, stream));
        }
      }
      scattered = regions;
    } else {
      if (chunks.n > 1) DK_CUDA(cudaStreamWaitEvent(stream, chunks.ev[chunks.n - 1], 0));
      TIMED(0, launch_l1_count(a, G, (uint32_t*)H.p, c64, stream));
    }
    uint64_t hc[2];
    DK_TRY(sync_read(c64, 16, hc));
    if (hc[1] == 0) {
      n_kmers = hc[0];
      break;
    }
    // a NUL-led line: recount the shortened read set in one pass
    chunked = false;
    regions = false;
    scattered = false;
    if (js) {
      DK_TRY(js->apply_nul(this));  // each job stops before its first NUL-led line
    } else {
      L = L - hc[1];  // first line whose first byte is NUL
    }
  }
  stats.n_lines = L;
  DK_CUDA(cudaEventRecord(ev_stage[1], stream));
  if (n_kmers == 0 && js) js->clear_results();
  if (n_kmers == 0) {
    DK_CUDA(cudaEventRecord(ev_stage[6], stream));
    DK_CUDA(cudaEventSynchronize(ev_stage[6]));
    float ms = 0;
    cudaEventElapsedTime(&ms, ev_stage[0], ev_stage[6]);
    stats.ms_device = ms;
    return DK_OK;
  }
  // level-1 nodes and offsets; a batch wave's graph keeps all of its tree's
  // nodes in this buffer (sized here: the level-1 scan writes into it)
  bool use_graph = js && !graph_off && !(flags & DK_FLAG_NO_GRAPH);
  const double g_scale = (flags & DK_FLAG_GRAPH_MIN_BUFFERS) ? 0.0 : graph_scale;
  node_cap_needed = (size_t)F1;
  if (use_graph) {
    node_cap_needed += (size_t)(g_scale * 6.0 * (double)n_kmers / bin_target) + 4096;
    if (Arena::ensure(this, nodes, node_cap_needed * sizeof(Node)) != DK_OK) {
      use_graph = false;  // no room for the graph's tree: the host drives this wave
      node_cap_needed = (size_t)F1;
    }
  }
  DK_TRY(Arena::ensure(this, nodes, node_cap_needed * sizeof(Node)));
  if (scattered) {
    TIMED(7, launch_l1_nodes((uint32_t*)H.p, NC * G, F1, (Node*)nodes.p, shift1, stream));
  } else {
    TIMED(7, launch_l1_scan((uint32_t*)H.p, (chunked ? NC : 1) * G, F1, (uint64_t*)O.p,
                            (Node*)nodes.p, shift1, js ? js->d_bshift : nullptr, stream));
  }
  const Ranges rg = scattered ? Ranges{rS, rT, NC, F1} : Ranges{nullptr, nullptr, 0, 0};
  DK_TRY(Arena::ensure(this, keysA, n_kmers * 8));
  DK_TRY(Arena::ensure(this, keysB, n_kmers * 8));
  DK_TRY(Arena::ensure(this, cnt, n_kmers * 4));
  if (scattered) {
    // done chunk by chunk above
  } else if (chunked) {
    for (int c = 0; c < NC; ++c)
      TIMED(1, launch_l1_scatter(chunk_args(c), G, (const uint64_t*)O.p + (size_t)c * G * F1,
                                 (uint64_t*)keysA.p, c64, stream));
  } else {
    TIMED(1, launch_l1_scatter(a, G, (const uint64_t*)O.p, (uint64_t*)keysA.p, c64, stream));
  }
  DK_CUDA(cudaEventRecord(ev_stage[2], stream));

  if (!out_k || !out_c) {
    set_error("internal: no output buffers");
    return DK_ERR_INVALID_ARG;
  }
  const int big_ok = use_hash ? 1 : (k <= 31 ? 2 : 0);
  uint64_t tail[21];
  if (use_graph) {
    const int r = wave_graph_tail(F1, n_kmers, bin_target, use_hash, big_ok, g_scale, tail);
    if (r == kGraphRetry) {
      // count the wave again, its tail driven from the host (the reads are
      // still in the device buffer); later waves get larger graph buffers
      const uint64_t builds = stats.graph_builds;
      graph_scale = std::min(graph_scale * 2.0, 16.0);
      graph_off = true;
      const int rr = count_device(d_text, nbytes, desc_in, out, js);
      graph_off = false;
      stats.graph_retries += 1;
      stats.graph_builds += builds;
      return rr;
    }
    DK_TRY(r);
  } else {
  // Groups of consecutive level-1 buckets, each taken through its partition
  // levels, bin count, tree offsets and compact before the next: a group's
  // slice of the table is then final and is handed to out_sink while the
  // next group runs.  One group unless a sink is set.
  std::vector<uint32_t> group_at{0, (uint32_t)F1};  // level-1 bucket boundaries
  std::vector<uint64_t> group_keys{n_kmers};        // k-mers per group
  if (out_sink && out_groups > 1 && F1 >= 2 * out_groups) {
    std::vector<Node> l1n((size_t)F1);
    DK_TRY(sync_read(nodes.p, (size_t)F1 * sizeof(Node), l1n.data()));
    group_at.assign(1, 0);
    group_keys.clear();
    uint64_t run = 0, run_g = 0;
    for (int b = 0; b < F1; ++b) {
      run += l1n[b].n;
      run_g += l1n[b].n;
      const uint64_t g = group_at.size();
      if (g < (uint64_t)out_groups && b + 1 < F1 && run * (uint64_t)out_groups >= g * n_kmers) {
        group_at.push_back((uint32_t)(b + 1));
        group_keys.push_back(run_g);
        run_g = 0;
      }
    }
    group_at.push_back((uint32_t)F1);
    group_keys.push_back(run_g);
  }

  // Partition levels, then the bin count of the final nodes.  With the hash
  // variant a skewed node (most of its parent's keys: a hot k-mer) larger
  // than a bin is counted whole by one hash bin; one that turns out to hold
  // too many distinct keys is re-partitioned through a proxy child and the
  // levels resume from the proxies (a pass per round of such bins).
  // the sort variant still counts a hot node of 2^31 keys or more as one hash
  // bin: splitting it would take many levels over all its keys, and near 2^32
  // keys the partition's 32-bit per-child offsets cannot hold it
  uint32_t node_end = (uint32_t)F1;  // nodes [0, node_end) exist
  uint32_t n_final = 0;              // final nodes listed so far (all groups)
  uint32_t n_bigf = 0;               // big-bin final nodes listed so far
  uint64_t keys_done = 0, distinct_done = 0;
  DK_TRY(Arena::ensure(this, finals, (size_t)F1 * 4));
  DK_TRY(Arena::ensure(this, bigs, (size_t)F1 * 4));
  for (size_t grp = 0; grp + 1 < group_at.size(); ++grp) {
    std::vector<std::pair<uint32_t, uint32_t>> levels;  // node ranges per level
    uint32_t lo = group_at[grp], hi = group_at[grp + 1];
    const uint32_t fin_g = n_final;  // first final node of the group
    const uint32_t big_g = n_bigf;   // first big bin of the group
    uint32_t fin_lo = n_final;       // first final node of this pass
    uint32_t big_lo = n_bigf;        // first big bin of this pass
    // Every split fixes at least one more key bit and nodes with at most
    // kDenseBits free bits are final, so the levels end within 2k - kDenseBits
    // splits (a proxy level fixes no bit, but follows a split of its own); the
    // loop runs until a level splits nothing.
    for (int lvl = 0;; ++lvl) {
      if (lvl > 4 * k + 2) {
        set_error("internal: the partition did not converge");
        return DK_ERR_INVALID_ARG;
      }
      levels.emplace_back(lo, hi);
      {
        // each final list can grow by at most this level's node count
        for (auto fl : {std::make_pair(&finals, n_final), std::make_pair(&bigs, n_bigf)}) {
          DevBuf& f = *fl.first;
          const size_t need = ((size_t)fl.second + (hi - lo)) * 4;
          if (f.cap < need) {
            DevBuf nb;
            DK_TRY(Arena::ensure(this, nb, need));
            if (fl.second)
              DK_CUDA(cudaMemcpyAsync(nb.p, f.p, (size_t)fl.second * 4, cudaMemcpyDeviceToDevice,
                                      stream));
            Arena::release(this, f);
            f = nb;
          }
        }
      }
      LevelCounters lv;
      // keep n_final and n_big_final
      DK_CUDA(cudaMemsetAsync((char*)lc + 8, 0, sizeof(LevelCounters) - 8, stream));
      TIMED(7, launch_classify((Node*)nodes.p, lo, hi, (uint32_t*)finals.p, (uint32_t*)bigs.p, lc,
                               kBinCap, 2 * bin_target, big_ok, rg, stream));
      DK_TRY(sync_read(lc, sizeof(LevelCounters), &lv));
      if (lv.too_big) {
        set_error("a partition node holds >= 2^32 keys");
        return DK_ERR_INVALID_ARG;
      }
      n_final = lv.n_final;
      n_bigf = lv.n_big_final;
      if (lv.n_split == 0) {
        // this pass's levels are done: count its final nodes
        if (grp == 0 && fin_lo == fin_g) DK_CUDA(cudaEventRecord(ev_stage[3], stream));
        DK_CUDA(cudaMemsetAsync(c64 + 4, 0, 8, stream));  // bin ticket
        uint32_t* fb = nullptr;
        if (use_hash && n_final > fin_lo) {
          // the packed kernel's ticket and fallback count (its totals, [21] and
          // [22], run over the whole count)
          DK_TRY(Arena::ensure(this, fbl, (size_t)(n_final - fin_lo) * 4));
          DK_CUDA(cudaMemsetAsync(c64 + 19, 0, 16, stream));
          fb = (uint32_t*)fbl.p;
        }
        TIMED(4, launch_bin_count((Node*)nodes.p, (uint32_t*)bigs.p + big_lo, n_bigf - big_lo,
                                  (uint32_t*)finals.p + fin_lo, n_final - fin_lo,
                                  (uint64_t*)keysA.p, (uint64_t*)keysB.p, (uint32_t*)cnt.p,
                                  use_hash ? 1 : 0, c64, sm_count, stream, fb));
        DK_CUDA(cudaEventRecord(ev_stage[4], stream));
        if (!big_ok || n_bigf == big_lo) break;  // only big bins can ask for a retry
        uint64_t retry = 0;
        DK_TRY(sync_read(c64 + 7, 8, &retry));
        if (retry == 0) break;
        stats.n_bins_retried += retry;
        const size_t need_nodes = (size_t)node_end + (size_t)retry;
        if (nodes.cap < need_nodes * sizeof(Node)) {
          DevBuf nb;
          DK_TRY(Arena::ensure(this, nb, need_nodes * sizeof(Node)));
          DK_CUDA(cudaMemcpyAsync(nb.p, nodes.p, (size_t)node_end * sizeof(Node),
                                  cudaMemcpyDeviceToDevice, stream));
          Arena::release(this, nodes);
          nodes = nb;
        }
        DK_CUDA(cudaMemsetAsync(c64 + 7, 0, 8, stream));
        DK_CUDA(cudaMemsetAsync(c64 + 16, 0, 8, stream));  // proxy counter
        TIMED(7, launch_make_proxies((Node*)nodes.p, (uint32_t*)bigs.p + big_lo, n_bigf - big_lo,
                                     node_end, (unsigned int*)(c64 + 16), stream));
        fin_lo = n_final;
        big_lo = n_bigf;
        lo = node_end;
        hi = node_end + (uint32_t)retry;
        node_end = hi;
        continue;
      }
      stats.n_partitioned += lv.split_keys;
      // grow node storage for the children (copying existing nodes)
      const size_t need_nodes = (size_t)node_end + (size_t)lv.n_children;
      if (nodes.cap < need_nodes * sizeof(Node)) {
        DevBuf nb;
        DK_TRY(Arena::ensure(this, nb, need_nodes * sizeof(Node)));
        DK_CUDA(cudaMemcpyAsync(nb.p, nodes.p, (size_t)node_end * sizeof(Node),
                                cudaMemcpyDeviceToDevice, stream));
        Arena::release(this, nodes);
        nodes = nb;
      }
      const uint32_t n_tiles = lv.n_tiles;
      DK_TRY(Arena::ensure(this, tiles, (size_t)n_tiles * sizeof(Tile)));
      DK_TRY(Arena::ensure(this, TH, (size_t)lv.th_entries * 4));
      TIMED(7, launch_assign((Node*)nodes.p, lo, hi, node_end, (Tile*)tiles.p, lc, rg, stream));
      TIMED(2, launch_tile_hist((Node*)nodes.p, (Tile*)tiles.p, n_tiles, (uint64_t*)keysA.p,
                                (uint64_t*)keysB.p, (uint32_t*)TH.p, stream));
      TIMED(7, launch_node_scan((Node*)nodes.p, lo, hi, (Tile*)tiles.p, (uint32_t*)TH.p, stream));
      TIMED(3, launch_tile_scatter((Node*)nodes.p, (Tile*)tiles.p, n_tiles, (uint64_t*)keysA.p,
                                   (uint64_t*)keysB.p, (uint32_t*)TH.p, (int)lv.max_width, stream));
      lo = node_end;
      hi = node_end + lv.n_children;
      node_end = hi;
    }
    stats.partition_levels = std::max(stats.partition_levels, (int)levels.size());
    // distinct counts up the tree, offsets down (the last level splits nothing;
    // a proxy level comes after the level of the node it stands in for); the
    // group's slice of the table starts after the earlier groups' k-mers
    for (int l = (int)levels.size() - 2; l >= 0; --l)
      TIMED(7, launch_aggregate((Node*)nodes.p, levels[l].first, levels[l].second, stream));
    TIMED(7, launch_l1_offsets((Node*)nodes.p, group_at[grp], group_at[grp + 1], c64 + 2, stream));
    for (size_t l = 0; l + 1 < levels.size(); ++l)
      TIMED(7, launch_child_offsets((Node*)nodes.p, levels[l].first, levels[l].second, stream));
    TIMED(5, launch_compact((Node*)nodes.p, (uint32_t*)finals.p + fin_g, n_final - fin_g,
                            (uint64_t*)keysA.p, (uint64_t*)keysB.p, (uint32_t*)cnt.p, out_k, out_c,
                            stream));
    TIMED(5, launch_compact((Node*)nodes.p, (uint32_t*)bigs.p + big_g, n_bigf - big_g,
                            (uint64_t*)keysA.p, (uint64_t*)keysB.p, (uint32_t*)cnt.p, out_k, out_c,
                            stream));
    DK_CUDA(cudaGetLastError());
    keys_done += group_keys[grp];
    if (out_sink) {
      uint64_t total = 0;
      DK_TRY(sync_read(c64 + 2, 8, &total));  // the group's compact has finished
      DK_TRY(out_sink(distinct_done, total - distinct_done, keys_done, n_kmers));
      distinct_done = total;
    }
  }
  stats.n_bins = n_final + n_bigf - (uint32_t)stats.n_bins_retried;
  stats.n_groups = group_at.size() - 1;
  DK_TRY(sync_read(c64 + 2, sizeof(tail), tail));
  }  // host-driven tail
  stats.n_bins_resorted = tail[4];
  stats.n_bins_big = tail[15];
  stats.n_bins_packed = tail[19];
  stats.n_bins_fallback = tail[20];
  const uint64_t n_distinct = tail[0];
  if (tail[1]) {
    set_error("a bounded device wait (TMA copy) timed out");
    return DK_ERR_TIMEOUT;
  }
  if (tail[3]) {
    set_error("a k-mer count does not fit 32 bits");
    return DK_ERR_COUNT_OVERFLOW;
  }
  out->n = n_distinct;
  out->n_kmers = n_kmers;
  out->k = out_k;
  out->c = out_c;
  if (js) {
    js->nodes.resize(F1);
    DK_TRY(sync_read(nodes.p, (size_t)F1 * sizeof(Node), js->nodes.data()));
  }
  DK_CUDA(cudaEventRecord(ev_stage[5], stream));
  DK_CUDA(cudaEventSynchronize(ev_stage[5]));
  float ms = 0;
  cudaEventElapsedTime(&ms, ev_stage[0], ev_stage[5]);
  stats.ms_device = ms;
  const int idx[6][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 4}, {4, 5}, {0, 0}};
  for (int s = 0; s < 5; ++s) {
    float t = 0;
    cudaEventElapsedTime(&t, ev_stage[idx[s][0]], ev_stage[idx[s][1]]);
    stats.ms_stage[s] = t;
  }
  stats.n_kmers = n_kmers;
  stats.n_distinct = n_distinct;
  stats.kernel_launches = launches;
  kresolve();
  return DK_OK;
}

// The tail of a batch wave -- partition levels, bin count, tree offsets,
// compact -- as one launch of the wave graph, after the level-1 scatter.  The
// graph runs the level loop on the device (a conditional WHILE node whose
// body plans the next level the way the host loop does), so the wave costs
// one launch and one read of its counters instead of a launch per kernel and
// a read per level.  Returns kGraphRetry when the wave must be counted again
// with the host-driven tail: a level needed more nodes, tiles or histogram
// than the graph's buffers hold, more levels than the level table, or a big
// bin must be re-partitioned.  Fills tail[] (the counters from ctr[2] on).
int Engine::wave_graph_tail(int F1, uint64_t n_kmers, int bin_target, bool use_hash, int big_ok,
                            double scale, uint64_t* tail) {
  Engine* e = this;
  const double kmers = (double)n_kmers;
  const uint64_t nodes_cap = node_cap_needed;  // the nodes buffer was sized for the graph
  const uint64_t tiles_cap = (uint64_t)(scale * (kmers / kTileKeys + kmers / kBinCap)) + 1024;
  // a tile's histogram row has 2^width <= 2^kGraphSplitBits entries: with
  // tiles_cap tiles the histogram never outgrows this (4 KB per tile)
  const uint64_t th_cap = tiles_cap << kGraphSplitBits;
  if (nodes_cap >= (1ull << 31) || tiles_cap >= (1ull << 31)) return kGraphRetry;
  // buffers the budget cannot hold: the host-driven tail sizes them per level
  for (auto b : {std::make_pair(&finals, nodes_cap * 4), std::make_pair(&bigs, nodes_cap * 4),
                 std::make_pair(&fbl, nodes_cap * 4),
                 std::make_pair(&tiles, tiles_cap * sizeof(Tile)),
                 std::make_pair(&TH, th_cap * 4)})
    if (Arena::ensure(this, *b.first, b.second) != DK_OK) return kGraphRetry;
  unsigned long long* c64 = (unsigned long long*)ctrs.p;
  WaveGraphArgs ga = {};
  ga.nodes = (Node*)nodes.p;
  ga.finals = (uint32_t*)finals.p;
  ga.bigs = (uint32_t*)bigs.p;
  ga.fb_list = (uint32_t*)fbl.p;
  ga.tiles = (Tile*)tiles.p;
  ga.TH = (uint32_t*)TH.p;
  ga.A = (uint64_t*)keysA.p;
  ga.B = (uint64_t*)keysB.p;
  ga.C = (uint32_t*)cnt.p;
  ga.lc = (LevelCounters*)((char*)ctrs.p + 64);
  ga.ctr = c64;
  ga.wc = (WaveCtl*)((char*)ctrs.p + 256);
  ga.bin_cap = kBinCap;
  ga.split_target = 2 * bin_target;
  ga.big_ok = big_ok;
  ga.use_hash = use_hash ? 1 : 0;
  ga.sm_count = sm_count;
  if (!wave_exec || std::memcmp(&ga, &wave_args, sizeof(ga)) != 0) {
    if (wave_exec) cudaGraphExecDestroy(wave_exec);
    if (wave_graph) cudaGraphDestroy(wave_graph);
    wave_exec = nullptr;
    wave_graph = nullptr;
    DK_CUDA(build_wave_graph(ga, s_cap, &wave_graph));
    DK_CUDA(cudaGraphInstantiate(&wave_exec, wave_graph, 0));
    wave_args = ga;
    ++stats.graph_builds;
  }
  WaveCtl& w = *h_wc;
  std::memset(&w, 0, sizeof(w));
  w.lo = 0;
  w.hi = (uint32_t)F1;
  w.node_end = (uint32_t)F1;
  w.F1 = (uint32_t)F1;
  w.nodes_cap = (uint32_t)nodes_cap;
  w.tiles_cap = (uint32_t)tiles_cap;
  w.th_cap = th_cap;
  w.out_k = out_k;
  w.out_c = out_c;
  DK_CUDA(cudaMemcpyAsync(ga.wc, h_wc, sizeof(WaveCtl), cudaMemcpyHostToDevice, stream));
  DK_CUDA(cudaEventRecord(ev_stage[3], stream));
  {
    const int i0 = kbegin();
    DK_CUDA(cudaGraphLaunch(wave_exec, stream));
    kend(6, i0, 1);
  }
  DK_CUDA(cudaEventRecord(ev_stage[4], stream));
  // the counters and the control block in one read
  uint64_t blob[64];
  DK_TRY(sync_read(ctrs.p, sizeof(blob), blob));
  const LevelCounters* lv = (const LevelCounters*)((const char*)blob + 64);
  const WaveCtl* wr = (const WaveCtl*)((const char*)blob + 256);
  if (wr->too_big) {
    set_error("a partition node holds >= 2^32 keys");
    return DK_ERR_INVALID_ARG;
  }
  if (wr->overflow || blob[7] /* big bins to re-partition */) return kGraphRetry;
  for (int i = 0; i < 21; ++i) tail[i] = blob[2 + i];
  stats.graph_waves += 1;
  stats.n_partitioned += wr->split_keys;
  stats.partition_levels = std::max(stats.partition_levels, (int)wr->n_levels);
  stats.n_bins = lv->n_final + lv->n_big_final;
  stats.n_groups = 1;
  launches += 1;
  return DK_OK;
}

uint64_t Engine::shape_key(int W, int k, uint64_t n_upper) {
  return ((uint64_t)W << 16) | ((uint64_t)k << 8) | (uint64_t)ceil_log2(n_upper + 1);
}

// Time the count of `text` under a small set of parameter choices and keep
// the fastest for inputs of this shape.  Stages: level-1 bits around the
// automatic rule (hash variant, default bin size), then the bin size at the
// best bits, then the other variant at the best pair.  Each choice is timed
// twice (device time, reads already in device memory) and its best kept.
int Engine::autotune(const char* text, uint64_t nbytes, const dk_input_desc* desc, dk_tune* out) {
  Engine* e = this;
  std::lock_guard<std::mutex> g(mu);
  if (!desc || (!text && nbytes) || desc->k < 1 || desc->k > 32 || desc->line_width < 1 ||
      desc->line_width > 1024 || !convention_ok(*desc)) {
    set_error("invalid autotune arguments");
    return DK_ERR_INVALID_ARG;
  }
  const int W = desc->line_width, k = desc->k;
  const int64_t L = frame_lines(nbytes, W);
  if (L < 0) {
    set_error("buffer size is not a whole number of lines");
    return DK_ERR_INVALID_ARG;
  }
  const uint64_t per_line = W >= k ? (uint64_t)(W - k + 1) : 0;
  const uint64_t n_upper = (uint64_t)L * per_line;
  DK_CUDA(cudaSetDevice(device));
  DK_TRY(Arena::ensure(this, this->text, nbytes + 64));
  if (nbytes) DK_TRY(upload(text, nbytes, (uint8_t*)this->text.p));
  uint64_t upper = n_upper;
  if (k <= 16) upper = std::min<uint64_t>(upper, 1ull << (2 * k));
  TableBuf* dev_tb = nullptr;
  DK_TRY(acquire_table(upper, true, &dev_tb));
  out_k = (uint64_t*)dev_tb->k;
  out_c = (uint32_t*)dev_tb->c;
  int timed = 0;
  auto run = [&](int l1, int tgt, int var, double* ms) -> int {
    dk_input_desc d = *desc;
    d.l1_bits = l1;
    d.bin_target = tgt;
    d.variant = var;
    double best = 1e30;
    for (int rep = 0; rep < 2; ++rep) {
      DeviceTable dt;
      const int rc = count_device((const uint8_t*)this->text.p, nbytes, d, &dt);
      if (rc != DK_OK) return rc;
      best = std::min(best, stats.ms_device);
    }
    ++timed;
    *ms = best;
    return DK_OK;
  };
  const int hash = k <= 31 ? DK_VARIANT_HASH : DK_VARIANT_SORT;
  const int max_bits = std::min({kMaxL1Bits, 2 * k, floor_log2_int(l1_max_buckets(W, false))});
  const int t0 = kBinCap / 2;
  const int b_auto = std::max(1, std::min(l1_bits_for(n_upper, (double)t0), max_bits));
  int rc = DK_OK;
  double ms_auto = 0, best_ms = 0;
  int best_b = b_auto, best_t = t0, best_v = hash;
  rc = run(b_auto, t0, hash, &ms_auto);
  best_ms = ms_auto;
  for (int b = std::max(1, b_auto - 2); rc == DK_OK && b <= std::min(max_bits, b_auto + 2); ++b) {
    if (b == b_auto) continue;
    double ms;
    rc = run(b, t0, hash, &ms);
    if (rc == DK_OK && ms < best_ms) { best_ms = ms; best_b = b; }
  }
  for (const int tgt : {kBinCap / 4, (3 * kBinCap) / 8}) {
    if (rc != DK_OK) break;
    double ms;
    rc = run(best_b, tgt, hash, &ms);
    if (rc == DK_OK && ms < best_ms) { best_ms = ms; best_t = tgt; }
  }
  if (rc == DK_OK && hash == DK_VARIANT_HASH) {
    double ms;
    rc = run(best_b, best_t, DK_VARIANT_SORT, &ms);
    if (rc == DK_OK && ms < best_ms) { best_ms = ms; best_v = DK_VARIANT_SORT; }
  }
  release_table(dev_tb->id);
  if (rc != DK_OK) return rc;
  Tune t;
  t.l1_bits = best_b;
  t.bin_target = best_t;
  t.variant = best_v;
  t.ms = best_ms;
  tunes[shape_key(W, k, n_upper)] = t;
  if (out) {
    out->l1_bits = best_b;
    out->bin_target = best_t;
    out->variant = best_v;
    out->candidates = timed;
    out->ms_device = best_ms;
    out->ms_auto = ms_auto;
  }
  return DK_OK;
}

int Engine::count(const char* text, uint64_t nbytes, bool text_on_device, const dk_input_desc* desc,
                  dk_table* out) {
  std::lock_guard<std::mutex> g(mu);
  return count_locked(text, nbytes, text_on_device, desc, out);
}

// dk_count's body; the caller holds `mu`
int Engine::count_locked(const char* text, uint64_t nbytes, bool text_on_device,
                         const dk_input_desc* desc, dk_table* out) {
  Engine* e = this;
  const auto w0 = std::chrono::steady_clock::now();
  if (!desc || !out || (!text && nbytes)) {
    set_error("null argument");
    return DK_ERR_INVALID_ARG;
  }
  std::memset(out, 0, sizeof(*out));
  if (desc->k < 1 || desc->k > 32 || desc->line_width < 1 || !convention_ok(*desc) ||
      desc->variant < DK_VARIANT_AUTO || desc->variant > DK_VARIANT_HASH ||
      (desc->residency != DK_RESIDENT_HOST && desc->residency != DK_RESIDENT_DEVICE)) {
    set_error("invalid input descriptor");
    return DK_ERR_INVALID_ARG;
  }
  if (desc->line_width > 1024) {
    set_error("line_width > 1024 is not supported");
    return DK_ERR_INVALID_ARG;
  }
  if (frame_lines(nbytes, desc->line_width) < 0) {
    set_error("buffer size is not a whole number of lines");
    return DK_ERR_INVALID_ARG;
  }
  if (text_on_device && (reinterpret_cast<uintptr_t>(text) & 15)) {
    set_error("device text must be 16-byte aligned");
    return DK_ERR_INVALID_ARG;
  }
  DK_CUDA(cudaSetDevice(device));
  const uint8_t* d_text = (const uint8_t*)text;
  float ms_h2d = 0;
  bool in_place_up = false;  // pageable reads read in place by the device
  if (!text_on_device) {
    DK_TRY(Arena::ensure(this, this->text, nbytes + 64));
    DK_CUDA(cudaEventRecord(ev_h2d0, stream));
    const int W = desc->line_width;
    const int64_t Lc = frame_lines(nbytes, W);
    const bool pinned = is_pinned(text);
    int hs = 1;  // pageable pages: 0 unmapped, 1 resident, 2 mapped but not all resident
    if (!pinned && host_direct && nbytes) {
      hs = host_range_state(text, nbytes);
      if (hs == 0) {
        set_error("reads at an unmapped host address");
        return DK_ERR_INVALID_ARG;
      }
    }
    in_place_up = !pinned && host_direct && nbytes > 0 && hs == 1;
    if (nbytes >= kChunkMinBytes && W <= kLineMaxW && Lc >= 64 * kMaxChunks &&
        (pinned || in_place_up)) {
      // chunks of lines on s_in (after earlier work on the text buffer); the
      // level-1 count of each runs as soon as it has landed.  Page-locked
      // chunks go to the DMA engine, pageable ones are read in place by a
      // copy kernel (same link, same rate)
      DK_CUDA(cudaStreamWaitEvent(s_in, ev_h2d0, 0));
      chunks.n = kMaxChunks;
      const uint64_t stride = (uint64_t)W + 1;
      for (int c = 0; c <= kMaxChunks; ++c) chunks.lines[c] = (uint64_t)Lc * c / kMaxChunks;
      for (int c = 0; c < kMaxChunks; ++c) {
        if (!chunks.ev[c]) DK_CUDA(cudaEventCreate(&chunks.ev[c]));
        const uint64_t b0 = chunks.lines[c] * stride;
        const uint64_t b1 = c + 1 == kMaxChunks ? nbytes : chunks.lines[c + 1] * stride;
        // (the copy engine takes pageable chunks too, but its copy returns only
        // when done: no chunk would be counted while the next uploads)
        const bool dma = pinned;
        if (b1 > b0 && dma)
          DK_CUDA(cudaMemcpyAsync((uint8_t*)this->text.p + b0, text + b0, b1 - b0,
                                  cudaMemcpyHostToDevice, s_in));
        if (b1 > b0 && !dma) {
          // (the whole range was checked above: mapped and resident)
          launch_copy_in(text + b0, (uint8_t*)this->text.p + b0, b1 - b0, sm_count, s_in);
          DK_CUDA(cudaGetLastError());
        }
        DK_CUDA(cudaEventRecord(chunks.ev[c], s_in));
      }
    } else if (nbytes) {
      DK_TRY(upload(text, nbytes, (uint8_t*)this->text.p));
    }
    d_text = (const uint8_t*)this->text.p;
  }
  // whatever way this call returns, no chunk copy is left in flight and the
  // next count does not see this call's chunks
  struct ChunkGuard {
    Engine* e;
    ~ChunkGuard() {
      if (e->chunks.n > 0) {
        cudaStreamSynchronize(e->s_in);
        e->chunks.n = 0;
      }
    }
  } chunk_guard{this};
  // output buffers sized by an upper bound of distinct k-mers (<= occurrences)
  const int64_t L = frame_lines(nbytes, desc->line_width);
  const uint64_t per_line = desc->line_width >= desc->k ? (uint64_t)(desc->line_width - desc->k + 1) : 0;
  uint64_t upper = (uint64_t)L * per_line;
  if (desc->k <= 16) upper = std::min<uint64_t>(upper, 1ull << (2 * desc->k));
  TableBuf* dev_tb = nullptr;
  DK_TRY(acquire_table(upper, true, &dev_tb));
  out_k = (uint64_t*)dev_tb->k;
  out_c = (uint32_t*)dev_tb->c;
  // A large table for the host moves out group by group on s_out while the
  // next group is counted.  The host table is sized after the first group,
  // from its distinct k-mers per k-mer; if a later slice does not fit, the
  // streaming stops and the whole table is copied at the end instead.
  TableBuf* h_tb = nullptr;
  bool streaming = desc->residency == DK_RESIDENT_HOST &&
                   (upper >= kStreamMinKmers || (flags & DK_FLAG_STREAM_ALL));
  uint64_t streamed = 0;
  if (streaming) {
    out_groups = kStreamGroups;
    out_sink = [&](uint64_t first, uint64_t n, uint64_t kmers_done, uint64_t kmers_total) -> int {
      if (!streaming) return DK_OK;
      if (!h_tb) {
        const double f = kmers_total ? (double)kmers_done / (double)kmers_total : 1.0;
        uint64_t est = (uint64_t)((double)(first + n) / std::max(f, 1e-6) * 1.2) + 4096;
        est = std::min(est, upper);
        if (acquire_table(est, false, &h_tb) != DK_OK) {
          h_tb = nullptr;
          streaming = false;
          return DK_OK;
        }
      }
      if (first + n > h_tb->cap) {
        streaming = false;
        return DK_OK;
      }
      if (n) {
        DK_CUDA(cudaMemcpyAsync((uint64_t*)h_tb->k + first, out_k + first, n * 8,
                                cudaMemcpyDeviceToHost, s_out));
        DK_CUDA(cudaMemcpyAsync((uint32_t*)h_tb->c + first, out_c + first, n * 4,
                                cudaMemcpyDeviceToHost, s_out));
      }
      streamed = first + n;
      return DK_OK;
    };
  }
  DeviceTable dt;
  int rc = count_device(d_text, nbytes, *desc, &dt);
  out_sink = nullptr;
  out_groups = 1;
  const bool chunked_up = chunks.n > 1;
  // no chunk copy may still read the caller's buffer when the call returns
  // (a count that ends early, e.g. lines shorter than k, never waited for them)
  if (chunked_up) cudaStreamSynchronize(s_in);
  chunks.n = 0;
  stats.upload_chunks = chunked_up ? (uint64_t)kMaxChunks : 0;
  stats.upload_in_place = in_place_up ? 1 : 0;
  if (h_tb && (rc != DK_OK || !streaming || streamed != dt.n)) {
    // copies into it may still run
    cudaStreamSynchronize(s_out);
    release_table(h_tb->id);
    h_tb = nullptr;
  }
  if (rc != DK_OK) {
    release_table(dev_tb->id);
    return rc;
  }
  if (!text_on_device) {
    cudaEventElapsedTime(&ms_h2d, ev_h2d0, chunked_up ? chunks.ev[kMaxChunks - 1] : ev_stage[0]);
    stats.ms_h2d = ms_h2d;
  }
  out->n = dt.n;
  out->n_kmers = dt.n_kmers;
  out->variant_used = stats.variant_used;
  if (desc->residency == DK_RESIDENT_DEVICE) {
    out->kmers = (uint64_t*)dev_tb->k;
    out->counts = (uint32_t*)dev_tb->c;
    out->on_device = 1;
    out->handle = dev_tb->id;
  } else {
    if (h_tb) {
      // streamed: the last slice's copies end the download
      DK_CUDA(cudaEventRecord(ev_d2h1, s_out));
      stats.table_streamed = 1;
    } else {
      rc = acquire_table(dt.n, false, &h_tb);
      if (rc != DK_OK) {
        release_table(dev_tb->id);
        return rc;
      }
      if (dt.n) {
        DK_CUDA(cudaMemcpyAsync(h_tb->k, dev_tb->k, dt.n * 8, cudaMemcpyDeviceToHost, stream));
        DK_CUDA(cudaMemcpyAsync(h_tb->c, dev_tb->c, dt.n * 4, cudaMemcpyDeviceToHost, stream));
      }
      DK_CUDA(cudaEventRecord(ev_d2h1, stream));
    }
    DK_CUDA(cudaEventSynchronize(ev_d2h1));
    float ms_d2h = 0;
    cudaEventElapsedTime(&ms_d2h, ev_stage[5], ev_d2h1);
    // the part of the download after the device finished (all of it unless streamed)
    stats.ms_d2h = dt.n ? std::max(0.0f, ms_d2h) : 0.0;
    release_table(dev_tb->id);
    out->kmers = (uint64_t*)h_tb->k;
    out->counts = (uint32_t*)h_tb->c;
    out->on_device = 0;
    out->handle = h_tb->id;
  }
  stats.dev_bytes_peak = dev_peak;
  stats.ms_wall =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
  return DK_OK;
}

}  // namespace dk

// =================================================================== C ABI
using dk::Engine;
namespace dk { struct Server; }

extern "C" {

struct dk_ctx {
  Engine eng;
  dk::Server* server = nullptr;
};

extern "C++" {
namespace dk {
Server* server_of(dk_ctx* ctx) { return ctx->server; }
void set_server(dk_ctx* ctx, Server* s) { ctx->server = s; }
Engine* engine_of(dk_ctx* ctx) { return &ctx->eng; }
int serve_release(Server* s, uint64_t handle);
}  // namespace dk
}

int dk_abi_version(void) { return DK_ABI_VERSION; }

const char* dk_strerror(int s) {
  switch (s) {
    case DK_OK: return "ok";
    case DK_ERR_INVALID_ARG: return "invalid argument";
    case DK_ERR_OOM: return "out of memory";
    case DK_ERR_COUNT_OVERFLOW: return "k-mer count overflows 32 bits";
    case DK_ERR_CUDA: return "CUDA error";
    case DK_ERR_TIMEOUT: return "timed out";
    case DK_ERR_ADMISSION: return "job exceeds the memory budget";
    case DK_ERR_PENDING: return "pending";
    case DK_ERR_NOT_FOUND: return "not found";
    case DK_ERR_CANCELLED: return "cancelled";
    case DK_ERR_NO_DEVICE: return "no usable CUDA device";
  }
  return "unknown status";
}

int dk_create(const dk_config* cfg, dk_ctx** out) {
  if (!out) return DK_ERR_INVALID_ARG;
  *out = nullptr;
  dk_ctx* c = new (std::nothrow) dk_ctx();
  if (!c) return DK_ERR_OOM;
  const int rc = c->eng.init(cfg);
  if (rc != DK_OK) {
    delete c;
    return rc;
  }
  *out = c;
  return DK_OK;
}

int dk_destroy(dk_ctx* ctx) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  if (ctx->server) dk_serve_stop(ctx);
  delete ctx;
  return DK_OK;
}

const char* dk_last_error_string(dk_ctx* ctx) {
  if (!ctx) return "null context";
  // a copy per calling thread: another thread's count may replace the text
  thread_local std::string copy;
  std::lock_guard<std::mutex> g(ctx->eng.err_mu);
  copy = ctx->eng.last_error;
  return copy.c_str();
}

int dk_count(dk_ctx* ctx, const char* text, uint64_t nbytes, const dk_input_desc* desc,
             dk_table* out) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  return ctx->eng.count(text, nbytes, false, desc, out);
}

int dk_count_device(dk_ctx* ctx, const char* d_text, uint64_t nbytes, const dk_input_desc* desc,
                    dk_table* out) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  return ctx->eng.count(d_text, nbytes, true, desc, out);
}

int dk_count_batch(dk_ctx* ctx, const dk_job* jobs, int njobs, const dk_input_desc* desc,
                   dk_table* outs) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  return ctx->eng.count_batch(jobs, njobs, desc, outs);
}

int dk_table_free(dk_ctx* ctx, dk_table* t) {
  if (!ctx || !t) return DK_ERR_INVALID_ARG;
  if (!t->handle) return DK_OK;  // empty table
  if ((t->handle >> 48) && ctx->server) {  // a served table: released by its worker
    const int rc = dk::serve_release(ctx->server, t->handle);
    std::memset(t, 0, sizeof(*t));
    return rc;
  }
  // (a served table freed after dk_serve_stop is in the context's shared host pool)
  const int rc = ctx->eng.release_table(t->handle & ((1ull << 48) - 1));  // the pool has its own lock
  std::memset(t, 0, sizeof(*t));
  return rc;
}

int dk_autotune(dk_ctx* ctx, const char* text, uint64_t nbytes, const dk_input_desc* desc,
                dk_tune* out) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  return ctx->eng.autotune(text, nbytes, desc, out);
}

int dk_autotune_reset(dk_ctx* ctx) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(ctx->eng.mu);
  ctx->eng.tunes.clear();
  return DK_OK;
}

int dk_last_stats(dk_ctx* ctx, dk_stats* out) {
  if (!ctx || !out) return DK_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(ctx->eng.mu);  // a count on another thread writes them
  *out = ctx->eng.stats;
  return DK_OK;
}

int dk_host_alloc(uint64_t nbytes, void** out) {
  if (!out) return DK_ERR_INVALID_ARG;
  *out = nullptr;
  if (cudaMallocHost(out, nbytes ? nbytes : 1) != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return DK_ERR_OOM;
  }
  return DK_OK;
}

int dk_host_free(void* p) {
  if (!p) return DK_OK;
  return cudaFreeHost(p) == cudaSuccess ? DK_OK : DK_ERR_CUDA;
}

int64_t dk_num_lines(const char* text, uint64_t nbytes, int line_width) {
  const int64_t L = dk::frame_lines(nbytes, line_width);
  if (L <= 0 || !text) return L;
  const uint64_t stride = (uint64_t)line_width + 1;
  for (int64_t i = 1; i < L; ++i)
    if (text[(uint64_t)i * stride] == '\0') return i;
  return L;
}

}  // extern "C"
