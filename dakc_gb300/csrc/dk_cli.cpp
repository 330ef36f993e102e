// dakc-gpu: the engine's command-line counter, a caller of the C ABI.
//
// It stands where DAKC's driver stands (dakc/src/main/main.cpp:22-54): read
// the reads file (fqreader::read_file, dakc/src/fqreader/fqreader.cpp:14-89),
// count it (the kmercounter constructor, dakc/src/kcounter/kcounter.hpp:84-99)
// and print what the counter prints -- the parameters (parser.hpp
// print_params), "kmer counting time: <s> seconds" (kcounter.cpp:426-429) and,
// as DAKC's BENCHMARK build does, global_kmers / global_distinct_kmers
// (kcounter.cpp:500-501).  k and the read length are compile-time in DAKC
// (common.hpp:34-40) and options here.  The whole file is one chunk counted on
// one GPU; the table can be written out, filtered and summarised, which DAKC's
// driver never does.
//
//   dakc-gpu -f reads.txt [-k 31] [-r 150] [options]
//
// Exit status: 0 on success, 2 when the input cannot be read (DAKC exits 2,
// fqreader.cpp:31-36), 1 on a bad option or an engine error.
#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <fcntl.h>
#include <getopt.h>
#include <sys/stat.h>
#include <unistd.h>

#include "dakc_gb300.h"

namespace {

struct Options {
  std::string file, out, tsv;
  int k = 31;
  int read_len = 150;  // 0: the longest read (formats other than DAKC lines)
  int format = -1;     // -1: DAKC's fixed-width lines (dk_count)
  int convention = DK_CONV_DAKC;
  int variant = DK_VARIANT_AUTO;
  int device = 0;
  int repeat = 1;
  uint32_t min_count = 0;
  uint32_t histogram = 0;
  bool autotune = false;
  bool on_device = false;
  bool read_len_set = false;
};

void usage(FILE* f) {
  std::fprintf(f,
               "usage: dakc-gpu -f FILE [options]\n"
               "  -f, --file FILE        reads (DAKC's text: fixed-width lines)\n"
               "  -k, --kmer-len K       k-mer length, 1..32 (default 31)\n"
               "  -r, --read-len R       line width before the terminator (default 150;\n"
               "                         with --format, 0 = the longest read)\n"
               "      --format F         dakc (default), lines, fastq or fasta\n"
               "      --pakman           PakMan*'s k-mer convention instead of DAKC's\n"
               "      --variant V        auto (default), hash or sort\n"
               "      --autotune         tune the partition for this input first\n"
               "      --repeat N         count N times, report each call (default 1)\n"
               "      --min-count C      keep k-mers seen at least C times\n"
               "      --histogram N      print distinct k-mers per count 1..N-1\n"
               "  -o, --out FILE         write the table: 12-byte records\n"
               "                         {uint64 k-mer; uint32 count}, little-endian\n"
               "      --tsv FILE         write the table as text: bases<TAB>count\n"
               "      --keep-on-device   leave the table in device memory (no output file)\n"
               "      --device D         CUDA device (default 0)\n"
               "  -h, --help             this text\n");
}

bool parse_int(const char* s, long lo, long hi, long* v) {
  char* end = nullptr;
  errno = 0;
  const long x = std::strtol(s, &end, 10);
  if (errno || end == s || *end || x < lo || x > hi) return false;
  *v = x;
  return true;
}

// 0: ok, 1: bad options (message printed), -1: --help
int parse(int argc, char** argv, Options* o) {
  enum { kFormat = 1000, kPakman, kVariant, kAutotune, kRepeat, kMinCount, kHist, kTsv, kKeep,
         kDevice };
  static const option longopts[] = {
      {"help", no_argument, nullptr, 'h'},
      {"file", required_argument, nullptr, 'f'},
      {"kmer-len", required_argument, nullptr, 'k'},
      {"read-len", required_argument, nullptr, 'r'},
      {"out", required_argument, nullptr, 'o'},
      {"format", required_argument, nullptr, kFormat},
      {"pakman", no_argument, nullptr, kPakman},
      {"variant", required_argument, nullptr, kVariant},
      {"autotune", no_argument, nullptr, kAutotune},
      {"repeat", required_argument, nullptr, kRepeat},
      {"min-count", required_argument, nullptr, kMinCount},
      {"histogram", required_argument, nullptr, kHist},
      {"tsv", required_argument, nullptr, kTsv},
      {"keep-on-device", no_argument, nullptr, kKeep},
      {"device", required_argument, nullptr, kDevice},
      {nullptr, 0, nullptr, 0}};
  int opt;
  long v;
  optind = 1;
  while ((opt = getopt_long(argc, argv, "hf:k:r:o:", longopts, nullptr)) != -1) {
    switch (opt) {
      case 'h': return -1;
      case 'f': o->file = optarg; break;
      case 'o': o->out = optarg; break;
      case 'k':
        if (!parse_int(optarg, 1, 32, &v)) return std::fprintf(stderr, "bad -k %s\n", optarg), 1;
        o->k = (int)v;
        break;
      case 'r':
        if (!parse_int(optarg, 0, 1 << 30, &v))
          return std::fprintf(stderr, "bad -r %s\n", optarg), 1;
        o->read_len = (int)v;
        o->read_len_set = true;
        break;
      case kFormat:
        if (!std::strcmp(optarg, "dakc")) o->format = -1;
        else if (!std::strcmp(optarg, "lines")) o->format = DK_FORMAT_LINES;
        else if (!std::strcmp(optarg, "fastq")) o->format = DK_FORMAT_FASTQ;
        else if (!std::strcmp(optarg, "fasta")) o->format = DK_FORMAT_FASTA;
        else return std::fprintf(stderr, "bad --format %s\n", optarg), 1;
        break;
      case kPakman: o->convention = DK_CONV_PAKMAN; break;
      case kVariant:
        if (!std::strcmp(optarg, "auto")) o->variant = DK_VARIANT_AUTO;
        else if (!std::strcmp(optarg, "hash")) o->variant = DK_VARIANT_HASH;
        else if (!std::strcmp(optarg, "sort")) o->variant = DK_VARIANT_SORT;
        else return std::fprintf(stderr, "bad --variant %s\n", optarg), 1;
        break;
      case kAutotune: o->autotune = true; break;
      case kRepeat:
        if (!parse_int(optarg, 1, 1000000, &v))
          return std::fprintf(stderr, "bad --repeat %s\n", optarg), 1;
        o->repeat = (int)v;
        break;
      case kMinCount:
        if (!parse_int(optarg, 0, 0xFFFFFFFFL, &v))
          return std::fprintf(stderr, "bad --min-count %s\n", optarg), 1;
        o->min_count = (uint32_t)v;
        break;
      case kHist:
        if (!parse_int(optarg, 1, 1 << 24, &v))
          return std::fprintf(stderr, "bad --histogram %s\n", optarg), 1;
        o->histogram = (uint32_t)v;
        break;
      case kTsv: o->tsv = optarg; break;
      case kKeep: o->on_device = true; break;
      case kDevice:
        if (!parse_int(optarg, 0, 1 << 16, &v))
          return std::fprintf(stderr, "bad --device %s\n", optarg), 1;
        o->device = (int)v;
        break;
      default: return 1;
    }
  }
  if (optind < argc) return std::fprintf(stderr, "unexpected argument %s\n", argv[optind]), 1;
  if (o->file.empty()) return std::fprintf(stderr, "-f FILE is required\n"), 1;
  if (o->format != -1 && !o->read_len_set) o->read_len = 0;
  if (o->format == -1 && o->read_len < 1) return std::fprintf(stderr, "-r must be >= 1\n"), 1;
  if (o->on_device && (!o->out.empty() || !o->tsv.empty()))
    return std::fprintf(stderr, "--keep-on-device writes no table file\n"), 1;
  return 0;
}

// The bases of a k-mer, first base in the top bits.  DAKC's codes are C=0 A=1
// T=2 G=3 (char2base, common.hpp:72-92); PakMan*'s are A=0 C=1 T=2 G=3.
void kmer_text(uint64_t x, int k, int conv, char* s) {
  const char* sym = conv == DK_CONV_PAKMAN ? "ACTG" : "CATG";
  for (int i = 0; i < k; ++i) s[i] = sym[(x >> (2 * (k - 1 - i))) & 3u];
  s[k] = 0;
}

int write_records(const dk_table& t, const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return std::fprintf(stderr, "cannot write %s: %s\n", path.c_str(), std::strerror(errno)), 1;
  constexpr uint64_t kBlock = 1 << 20;
  std::vector<unsigned char> buf(kBlock * 12);
  for (uint64_t i0 = 0; i0 < t.n; i0 += kBlock) {
    const uint64_t m = t.n - i0 < kBlock ? t.n - i0 : kBlock;
    for (uint64_t i = 0; i < m; ++i) {
      std::memcpy(&buf[i * 12], &t.kmers[i0 + i], 8);
      std::memcpy(&buf[i * 12 + 8], &t.counts[i0 + i], 4);
    }
    if (std::fwrite(buf.data(), 12, m, f) != m) {
      std::fclose(f);
      return std::fprintf(stderr, "short write to %s\n", path.c_str()), 1;
    }
  }
  return std::fclose(f) == 0 ? 0 : 1;
}

int write_tsv(const dk_table& t, int k, int conv, const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return std::fprintf(stderr, "cannot write %s: %s\n", path.c_str(), std::strerror(errno)), 1;
  char s[40];
  for (uint64_t i = 0; i < t.n; ++i) {
    kmer_text(t.kmers[i], k, conv, s);
    std::fprintf(f, "%s\t%" PRIu32 "\n", s, t.counts[i]);
  }
  return std::fclose(f) == 0 ? 0 : 1;
}

// The reads file in page-locked memory when the engine can provide it (one
// DMA per chunk), else in ordinary memory, which the engine also takes.
struct Reads {
  char* p = nullptr;
  uint64_t n = 0;
  bool pinned = false;
  ~Reads() {
    if (pinned) dk_host_free(p);
    else std::free(p);
  }
};

// Open the reads file: exit status 2 when it cannot be read, as DAKC's reader
// exits (fqreader.cpp:31-36), before any device work.
int open_file(const std::string& path, int* fd, uint64_t* n) {
  *fd = ::open(path.c_str(), O_RDONLY);
  if (*fd < 0) {
    std::fprintf(stderr, "Could not open the input file %s: %s\n", path.c_str(),
                 std::strerror(errno));
    return 2;
  }
  struct stat st;
  if (fstat(*fd, &st) != 0 || !S_ISREG(st.st_mode)) {
    ::close(*fd);
    std::fprintf(stderr, "%s is not a regular file\n", path.c_str());
    return 2;
  }
  *n = (uint64_t)st.st_size;
  return 0;
}

// Read the whole file (fd is closed here).
int read_file(int fd, const std::string& path, uint64_t n, Reads* r) {
  r->n = n;
  void* p = nullptr;
  if (n && dk_host_alloc(n, &p) == DK_OK) {
    r->p = static_cast<char*>(p);
    r->pinned = true;
  } else {
    r->p = static_cast<char*>(std::malloc(n ? n : 1));
  }
  if (!r->p) {
    ::close(fd);
    std::fprintf(stderr, "cannot hold %" PRIu64 " bytes of reads\n", n);
    return 2;
  }
  uint64_t got = 0;
  while (got < n) {
    const ssize_t m = ::read(fd, r->p + got, (size_t)std::min<uint64_t>(n - got, 1ull << 30));
    if (m < 0 && errno == EINTR) continue;
    if (m <= 0) {
      ::close(fd);
      std::fprintf(stderr, "error reading %s\n", path.c_str());
      return 2;
    }
    got += (uint64_t)m;
  }
  ::close(fd);
  return 0;
}

int engine_error(dk_ctx* ctx, const char* what, int st) {
  const char* detail = ctx ? dk_last_error_string(ctx) : nullptr;
  std::fprintf(stderr, "%s: %s%s%s\n", what, dk_strerror(st), detail && *detail ? ": " : "",
               detail ? detail : "");
  return 1;
}

struct Ctx {
  dk_ctx* c = nullptr;
  ~Ctx() {
    if (c) dk_destroy(c);
  }
};

struct Table {
  dk_ctx* c = nullptr;
  dk_table t{};
  bool live = false;
  void reset() {
    if (live) dk_table_free(c, &t);
    live = false;
  }
  ~Table() { reset(); }
};

int run(const Options& o) {
  int fd = -1;
  uint64_t nbytes = 0;
  if (const int st = open_file(o.file, &fd, &nbytes)) return st;
  Ctx ctx;
  dk_config cfg{};
  cfg.device = o.device;
  if (const int st = dk_create(&cfg, &ctx.c)) {
    ::close(fd);
    return engine_error(nullptr, "dk_create", st);
  }
  Reads reads;  // page-locked on the context's device
  if (const int st = read_file(fd, o.file, nbytes, &reads)) return st;

  dk_input_desc d{};
  d.line_width = o.read_len;
  d.k = o.k;
  d.convention = o.convention;
  d.variant = o.variant;
  d.residency = o.on_device ? DK_RESIDENT_DEVICE : DK_RESIDENT_HOST;

  std::printf("File Name : %s\n", o.file.c_str());
  std::printf("Read Length : %d%s\n", o.read_len, o.format != -1 && o.read_len == 0 ? " (longest read)" : "");
  std::printf("k-mer Length : %d\n", o.k);

  if (o.autotune) {
    if (o.format != -1) {
      std::fprintf(stderr, "--autotune takes DAKC's fixed-width lines only\n");
      return 1;
    }
    dk_tune tune{};
    if (const int st = dk_autotune(ctx.c, reads.p, reads.n, &d, &tune))
      return engine_error(ctx.c, "dk_autotune", st);
    std::printf("autotuned: level-1 bits %d, bin target %d, %s variant (%d candidates)\n",
                tune.l1_bits, tune.bin_target, tune.variant == DK_VARIANT_SORT ? "sort" : "hash",
                tune.candidates);
  }

  Table table;
  table.c = ctx.c;
  for (int rep = 0; rep < o.repeat; ++rep) {
    table.reset();
    int width = o.read_len;
    const auto t0 = std::chrono::steady_clock::now();
    const int st = o.format == -1
                       ? dk_count(ctx.c, reads.p, reads.n, &d, &table.t)
                       : dk_count_format(ctx.c, reads.p, reads.n, o.format, &d, &table.t, &width);
    const auto t1 = std::chrono::steady_clock::now();
    if (st) return engine_error(ctx.c, o.format == -1 ? "dk_count" : "dk_count_format", st);
    table.live = true;
    if (rep == 0 && o.format != -1) std::printf("Line Width : %d\n", width);
    std::printf("kmer counting time: %.6f seconds\n",
                std::chrono::duration<double>(t1 - t0).count());
  }
  dk_stats stats{};
  dk_last_stats(ctx.c, &stats);
  std::printf("device time: %.3f ms, %s variant\n", stats.ms_device,
              table.t.variant_used == DK_VARIANT_SORT ? "sort" : "hash");
  std::printf("global_kmers: %" PRIu64 "\n", table.t.n_kmers);
  std::printf("global_distinct_kmers: %" PRIu64 "\n", table.t.n);

  if (o.histogram) {
    std::vector<uint64_t> hist(o.histogram);
    uint32_t min_bucket = 0;
    if (const int st = dk_table_histogram(ctx.c, &table.t, o.histogram, hist.data(), &min_bucket))
      return engine_error(ctx.c, "dk_table_histogram", st);
    std::printf("histogram (count: distinct k-mers), cut-off %" PRIu32 ":\n", min_bucket);
    for (uint32_t c = 1; c < o.histogram; ++c)
      if (hist[c]) std::printf("%" PRIu32 "\t%" PRIu64 "\n", c, hist[c]);
  }

  const dk_table* out = &table.t;
  Table kept;
  kept.c = ctx.c;
  if (o.min_count > 1) {
    if (const int st = dk_table_filter(ctx.c, &table.t, o.min_count, &kept.t))
      return engine_error(ctx.c, "dk_table_filter", st);
    kept.live = true;
    out = &kept.t;
    std::printf("kept (count >= %" PRIu32 "): %" PRIu64 " distinct, %" PRIu64 " k-mers\n",
                o.min_count, kept.t.n, kept.t.n_kmers);
  }
  if (!o.out.empty() && write_records(*out, o.out)) return 1;
  if (!o.tsv.empty() && write_tsv(*out, o.k, o.convention, o.tsv)) return 1;
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  const int p = parse(argc, argv, &o);
  if (p == -1) {
    usage(stdout);
    return 0;
  }
  if (p) {
    usage(stderr);
    return 1;
  }
  return run(o);
}
