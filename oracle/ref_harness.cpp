// Harness that runs the reference's own counting code (DAKC's kmercounter,
// dakc/src/kcounter/kcounter.hpp:84-99, compiled unmodified against the shim
// in oracle/shim) on P forked PEs and writes the merged (k-mer, count) table.
// Test infrastructure for the oracle only.
//
//   dakc_ref_k<K>_r<R>_h<H> <reads.txt> <P> <table.bin>
//
// Steps, mirroring dakc/src/main/main.cpp:42-49 and fqreader.cpp:43-60:
//   1. split the file into per-PE chunks of whole lines, last PE takes the
//      remainder, each chunk NUL-terminated;
//   2. construct kmercounter (runs phase 1 and phase 2);
//   3. read lightdbg up to its first count==0 entry (entries past the
//      reference's local size are value-initialised zeros, every real count is
//      >= 1); with HITTER the heavy table is the strictly increasing prefix of
//      heavydbg (the merge leaves stale entries after it);
//   4. merge the PEs' sorted tables.
// Output: "DKT1", u64 n, u64 n_kmers, u64 keys[n], u32 counts[n].
// Exit status 3 when a PE received no k-mer: the reference then reads element
// 0 of an empty vector (kcounter.cpp:389) and its table is undefined.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <string>
#include <vector>
#include <algorithm>
#include <unistd.h>
#include <sys/wait.h>

#include "common.hpp"
#include "kcounter.hpp"
#include "dk_shim.hpp"

namespace dkshim { extern uint64_t g_items_received; }

static int run_pe(const std::vector<char>& file, int pe, int P, const std::string& out) {
  dkshim::set_pe(pe);
  const uint64_t filesize = file.size();
  const uint64_t total_reads = (filesize + 1) / (READLEN + 1);
  uint64_t localsize = (total_reads / P) * (READLEN + 1);
  const uint64_t start = (uint64_t)pe * localsize;
  uint64_t end = start + localsize - 1;
  if (pe == P - 1) end = filesize - 1;
  localsize = end - start + 1;
  char* chunk = (char*)std::malloc(localsize + 1);
  std::memcpy(chunk, file.data() + start, localsize);
  chunk[localsize] = '\0';

  std::vector<kmer_t> vectordbg;
  std::vector<std::pair<uint64_t, uint64_t>> rows;
  {
    kmercounter km(chunk, vectordbg);
    for (const kmer_packet& p : *km.lightdbg) {
      if (p.count == 0) break;
      rows.emplace_back(p.kmer, p.count);
    }
#if HITTER
    const std::vector<kmer_packet>& h = *km.heavydbg;
    for (size_t i = 0; i < h.size(); ++i) {
      if (i > 0 && h[i].kmer <= h[i - 1].kmer) break;
      rows.emplace_back(h[i].kmer, h[i].count);
    }
    // the PE's table is the union of its light and heavy tables (each sorted)
    std::sort(rows.begin(), rows.end());
#endif
  }
  std::free(chunk);
  FILE* f = std::fopen((out + ".pe" + std::to_string(pe)).c_str(), "wb");
  const uint64_t n = rows.size();
  std::fwrite(&n, 8, 1, f);
  if (n) std::fwrite(rows.data(), sizeof(rows[0]), n, f);
  std::fclose(f);
  return dkshim::g_items_received == 0 ? 3 : 0;
}

int main(int argc, char** argv) {
  if (argc != 4) { std::fprintf(stderr, "usage: %s reads.txt P table.bin\n", argv[0]); return 2; }
  const std::string in = argv[1], out = argv[3];
  const int P = std::atoi(argv[2]);
  FILE* f = std::fopen(in.c_str(), "rb");
  if (!f) { std::perror("open"); return 2; }
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<char> file((size_t)sz);
  if (sz > 0 && std::fread(file.data(), 1, (size_t)sz, f) != (size_t)sz) { std::perror("read"); return 2; }
  std::fclose(f);
  if (sz == 0) { std::fprintf(stderr, "empty input: the reference's behaviour is undefined\n"); return 3; }

  char dir[] = "/tmp/dkshimXXXXXX";
  if (!mkdtemp(dir)) { std::perror("mkdtemp"); return 2; }
  if (dkshim::setup(P, dir) != 0) { std::fprintf(stderr, "bad P\n"); return 2; }
  std::fflush(stdout);
  std::vector<pid_t> kids;
  for (int pe = 0; pe < P; ++pe) {
    pid_t pid = fork();
    if (pid == 0) { int rc = run_pe(file, pe, P, out); std::fflush(stdout); _exit(rc); }
    kids.push_back(pid);
  }
  int bad = 0;
  for (pid_t k : kids) {
    int st = 0;
    waitpid(k, &st, 0);
    if (!WIFEXITED(st) || WEXITSTATUS(st) != 0) bad = WIFEXITED(st) ? WEXITSTATUS(st) : 4;
  }
  rmdir(dir);
  // merge the per-PE tables
  std::vector<std::vector<std::pair<uint64_t, uint64_t>>> t(P);
  for (int pe = 0; pe < P; ++pe) {
    const std::string p = out + ".pe" + std::to_string(pe);
    FILE* g = std::fopen(p.c_str(), "rb");
    uint64_t n = 0;
    if (g && std::fread(&n, 8, 1, g) == 1) {
      t[pe].resize(n);
      if (n && std::fread(t[pe].data(), sizeof(t[pe][0]), n, g) != n) bad = 4;
    }
    if (g) std::fclose(g);
    std::remove(p.c_str());
  }
  std::vector<uint64_t> keys;
  std::vector<uint32_t> counts;
  std::vector<size_t> pos(P, 0);
  uint64_t nk = 0;
  for (;;) {
    int best = -1;
    for (int pe = 0; pe < P; ++pe)
      if (pos[pe] < t[pe].size() && (best < 0 || t[pe][pos[pe]].first < t[best][pos[best]].first)) best = pe;
    if (best < 0) break;
    const auto& r = t[best][pos[best]++];
    if (!keys.empty() && keys.back() == r.first) { bad = bad ? bad : 6; }
    keys.push_back(r.first);
    if (r.second > 0xFFFFFFFFull) bad = bad ? bad : 7;
    counts.push_back((uint32_t)r.second);
    nk += r.second;
  }
  FILE* o = std::fopen(out.c_str(), "wb");
  const uint64_t n = keys.size();
  std::fwrite("DKT1", 1, 4, o);
  std::fwrite(&n, 8, 1, o);
  std::fwrite(&nk, 8, 1, o);
  if (n) { std::fwrite(keys.data(), 8, n, o); std::fwrite(counts.data(), 4, n, o); }
  std::fclose(o);
  return bad;
}
