// Reads in other layouts, laid out on the GPU as the fixed-width lines the
// counting pipeline takes:
//   DK_FORMAT_LINES  one read per line, any length;
//   DK_FORMAT_FASTQ  4-line records, the reads are line 2 of each -- the
//                    reference's conversion keeps lines NR%4==2, pads them
//                    to the longest with 'M' and turns spaces into 'M'
//                    (syngen/fq2txtmaker.sh:12-18);
//   DK_FORMAT_FASTA  from the first '>': a header line, then one sequence
//                    line, alternating, as PakMan*'s reader walks it
//                    (pakman_star/src/kmer_counting.cpp:283-300;
//                    syngen/fq2famaker.sh:12 makes it from FASTQ).
// A read is the bytes of its line up to the newline (or the end of the
// buffer).  With the DAKC convention reads are padded with 'M' (DAKC stops a
// line there) and spaces become 'M', as fq2txtmaker.sh does; with the PakMan*
// convention they are padded with '\n', where PakMan* ends a read.
#include "dk_engine.hpp"
#include "dk_device.cuh"
#include "../../include/dakc_gb300.h"

#include <algorithm>
#include <cstring>
#include <mutex>

namespace dk {
namespace {

using dev::block_excl_scan;

constexpr int kIngThreads = 256;
constexpr uint64_t kIngChunk = 64 * 1024;  // bytes per block when finding line ends
constexpr uint64_t kIngPer = kIngChunk / kIngThreads;

// newlines per chunk
__global__ void __launch_bounds__(kIngThreads) k_nl_count(const uint8_t* __restrict__ t, uint64_t n,
                                                          uint64_t* __restrict__ cnt) {
  __shared__ uint64_t tmp[32];
  const uint64_t b0 = blockIdx.x * kIngChunk + (uint64_t)threadIdx.x * kIngPer;
  uint64_t mine = 0;
  for (uint64_t i = b0; i < min(n, b0 + kIngPer); ++i) mine += t[i] == '\n';
  uint64_t total;
  block_excl_scan<uint64_t>(mine, tmp, &total);
  if (threadIdx.x == 0) cnt[blockIdx.x] = total;
}

// exclusive scan of the chunk counts in place, by one block; *total = their sum
__global__ void __launch_bounds__(1024) k_scan_block(uint64_t* v, uint64_t n, uint64_t* total) {
  __shared__ uint64_t tmp[32];
  const uint64_t t = dev::block_scan_array<uint64_t>(v, (int)n, tmp);
  if (threadIdx.x == 0) *total = t;
}

// positions of the newlines, in order
__global__ void __launch_bounds__(kIngThreads) k_nl_positions(const uint8_t* __restrict__ t,
                                                              uint64_t n,
                                                              const uint64_t* __restrict__ base,
                                                              uint64_t* __restrict__ ends) {
  __shared__ uint64_t tmp[32];
  const uint64_t b0 = blockIdx.x * kIngChunk + (uint64_t)threadIdx.x * kIngPer;
  const uint64_t b1 = min(n, b0 + kIngPer);
  uint64_t mine = 0;
  for (uint64_t i = b0; i < b1; ++i) mine += t[i] == '\n';
  uint64_t pos = base[blockIdx.x] + block_excl_scan<uint64_t>(mine, tmp, nullptr);
  for (uint64_t i = b0; i < b1; ++i)
    if (t[i] == '\n') ends[pos++] = i;
}

// Output read s is input line first + s * step; line i spans from the byte
// after newline i-1 to newline i (the last line may end at the buffer's end).
struct Pick {
  uint64_t first, step;
  uint64_t n_lines;  // input lines
  uint64_t nbytes;
  bool last_nl;      // the buffer ends with a newline
  __device__ void span(const uint64_t* ends, uint64_t s, uint64_t* b, uint64_t* e) const {
    const uint64_t i = first + s * step;
    *b = i ? ends[i - 1] + 1 : 0;
    *e = (i + 1 < n_lines || last_nl) ? ends[i] : nbytes;
  }
};

__global__ void k_max_len(const uint64_t* __restrict__ ends, Pick pk, uint64_t n_out,
                          unsigned long long* __restrict__ max_len) {
  unsigned long long m = 0;
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_out;
       s += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t b, e;
    pk.span(ends, s, &b, &e);
    m = max(m, (unsigned long long)(e - b));
  }
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(max_len, m);
}

// one warp per read: bytes, padding, newline
__global__ void k_layout(const uint8_t* __restrict__ t, const uint64_t* __restrict__ ends, Pick pk,
                         uint64_t n_out, int W, uint8_t pad, bool space_to_m,
                         uint8_t* __restrict__ out) {
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t s = warp; s < n_out; s += nwarps) {
    uint64_t b, e;
    pk.span(ends, s, &b, &e);
    const uint64_t len = e - b;
    uint8_t* o = out + s * ((uint64_t)W + 1);
    for (uint32_t j = lane; j <= (uint32_t)W; j += 32) {
      uint8_t c;
      if (j == (uint32_t)W) c = '\n';
      else if (j < len) {
        c = t[b + j];
        if (space_to_m && c == ' ') c = 'M';
      } else {
        c = pad;
      }
      o[j] = c;
    }
  }
}

}  // namespace

int Engine::count_format(const char* text, uint64_t nbytes, int format, const dk_input_desc* desc,
                         dk_table* out, int* width) {
  Engine* e = this;
  std::lock_guard<std::mutex> g(mu);
  if (!desc || !out || (!text && nbytes) ||
      (format != DK_FORMAT_LINES && format != DK_FORMAT_FASTQ && format != DK_FORMAT_FASTA) ||
      (desc->convention != DK_CONV_DAKC && desc->convention != DK_CONV_PAKMAN) ||
      desc->line_width < 0) {
    set_error("invalid format-count arguments");
    return DK_ERR_INVALID_ARG;
  }
  std::memset(out, 0, sizeof(*out));
  const int max_w = 1024;
  // input lines: newline-terminated, the last one may lack its newline
  const bool last_nl = nbytes && text[nbytes - 1] == '\n';
  // FASTA: the reads start after the line holding the first '>'
  uint64_t first = 0, step = 1;
  bool any = nbytes > 0;
  if (format == DK_FORMAT_FASTQ) {
    first = 1;
    step = 4;
  } else if (format == DK_FORMAT_FASTA) {
    const void* gt = nbytes ? std::memchr(text, '>', nbytes) : nullptr;
    if (!gt) {
      any = false;
    } else {
      const uint64_t g0 = (const char*)gt - text;
      uint64_t h = 0;  // newlines before it = index of its line
      for (const char* p = text; (p = (const char*)std::memchr(p, '\n', text + g0 - p)) != nullptr; ++p)
        ++h;
      first = h + 1;
      step = 2;
    }
  }
  DK_CUDA(cudaSetDevice(device));
  uint64_t n_lines = 0, n_out = 0;
  if (any) {
    DK_TRY(Arena::ensure(this, text2, nbytes + 64));
    DK_TRY(upload(text, nbytes, (uint8_t*)text2.p));
    const uint64_t chunks = (nbytes + kIngChunk - 1) / kIngChunk;
    DK_TRY(Arena::ensure(this, aux, (chunks + 2) * 8));
    uint64_t* cnt = (uint64_t*)aux.p;
    k_nl_count<<<(uint32_t)chunks, kIngThreads, 0, stream>>>((const uint8_t*)text2.p, nbytes, cnt);
    k_scan_block<<<1, 1024, 0, stream>>>(cnt, chunks, cnt + chunks);
    DK_CUDA(cudaGetLastError());
    uint64_t nl = 0;
    DK_TRY(sync_read(cnt + chunks, 8, &nl));
    n_lines = nl + (last_nl ? 0 : 1);
    n_out = n_lines > first ? (n_lines - first + step - 1) / step : 0;
    // newline positions after the chunk counts in the same scratch
    DevBuf& ends_buf = H;  // the level-1 histogram arena is free until the count
    DK_TRY(Arena::ensure(this, ends_buf, std::max<uint64_t>(nl, 1) * 8));
    k_nl_positions<<<(uint32_t)chunks, kIngThreads, 0, stream>>>((const uint8_t*)text2.p, nbytes,
                                                                  cnt, (uint64_t*)ends_buf.p);
    DK_CUDA(cudaGetLastError());
  }
  Pick pk{first, step, n_lines, nbytes, last_nl};
  int W = desc->line_width;
  if (n_out) {
    DK_TRY(Arena::ensure(this, ctrs, 256));
    unsigned long long* ml = (unsigned long long*)ctrs.p;
    DK_CUDA(cudaMemsetAsync(ml, 0, 8, stream));
    const uint32_t grid = (uint32_t)std::min<uint64_t>((n_out + 255) / 256, (uint64_t)sm_count * 8);
    k_max_len<<<grid, 256, 0, stream>>>((const uint64_t*)H.p, pk, n_out, ml);
    DK_CUDA(cudaGetLastError());
    uint64_t longest = 0;
    DK_TRY(sync_read(ml, 8, &longest));
    if (W == 0) W = (int)std::max<uint64_t>(1, longest);
    if ((uint64_t)W < longest || W > max_w) {
      set_error("reads of " + std::to_string(longest) + " bytes do not fit line width " +
                std::to_string(W) + " (at most " + std::to_string(max_w) + ")");
      return DK_ERR_INVALID_ARG;
    }
    const uint64_t out_bytes = n_out * ((uint64_t)W + 1);
    DK_TRY(Arena::ensure(this, this->text, out_bytes + 64));
    const uint64_t warps = std::min<uint64_t>(n_out, (uint64_t)sm_count * 64);
    k_layout<<<(uint32_t)((warps * 32 + 255) / 256), 256, 0, stream>>>(
        (const uint8_t*)text2.p, (const uint64_t*)H.p, pk, n_out, W,
        desc->convention == DK_CONV_PAKMAN ? (uint8_t)'\n' : (uint8_t)'M',
        desc->convention == DK_CONV_DAKC && format == DK_FORMAT_FASTQ, (uint8_t*)this->text.p);
    DK_CUDA(cudaGetLastError());
  }
  if (W == 0) W = 1;
  if (width) *width = W;
  dk_input_desc d = *desc;
  d.line_width = W;
  return count_locked(n_out ? (const char*)this->text.p : nullptr, n_out * ((uint64_t)W + 1),
                      true, &d, out);
}

Engine* engine_of(dk_ctx* ctx);

}  // namespace dk

extern "C" int dk_count_format(dk_ctx* ctx, const char* text, uint64_t nbytes, int format,
                               const dk_input_desc* desc, dk_table* out, int* line_width) {
  if (!ctx) return DK_ERR_INVALID_ARG;
  return dk::engine_of(ctx)->count_format(text, nbytes, format, desc, out, line_width);
}
