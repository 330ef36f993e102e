// Runtime behind the shim headers (shmem.h, mpi.h, selector.h): PEs are
// forked OS processes sharing one anonymous MAP_SHARED control block
// (process-shared barrier + reduction slots); selector messages travel
// through per-(sender, receiver) files in a scratch directory.  Test
// infrastructure for the oracle only.
//
// PEs must be processes, not threads: the reference keeps a function-local
// `static std::vector<uint8_t> base_vec` in read_till_buf_max
// (dakc/src/kcounter/kcounter_funcs.cpp:84), which threads would share.
#include "selector.h"
#include "shmem.h"
#include "mpi.h"
#include "dk_shim.hpp"

#include <pthread.h>
#include <sys/mman.h>
#include <time.h>
#include <cstdio>
#include <cstdlib>
#include <string>

namespace dkshim {

SelectorBase* g_active = nullptr;
uint64_t g_items_received = 0;

namespace {
const int kMaxPE = 1024;
struct Shared {
  pthread_barrier_t bar;
  int npes;
  double dslot[kMaxPE];
  uint64_t uslot[kMaxPE];
};
Shared* g_sh = nullptr;
int g_pe = 0;
std::string g_dir;
uint64_t g_epoch = 0;
}  // namespace

int setup(int npes, const char* scratch_dir) {
  if (npes < 1 || npes > kMaxPE) return -1;
  void* p = mmap(nullptr, sizeof(Shared), PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
  if (p == MAP_FAILED) return -1;
  g_sh = static_cast<Shared*>(p);
  pthread_barrierattr_t at;
  pthread_barrierattr_init(&at);
  pthread_barrierattr_setpshared(&at, PTHREAD_PROCESS_SHARED);
  pthread_barrier_init(&g_sh->bar, &at, (unsigned)npes);
  g_sh->npes = npes;
  g_dir = scratch_dir;
  return 0;
}

void set_pe(int pe) { g_pe = pe; }
int my_pe() { return g_pe; }
int n_pes() { return g_sh ? g_sh->npes : 1; }
void barrier() {
  if (g_sh && g_sh->npes > 1) pthread_barrier_wait(&g_sh->bar);
}

static std::string blob_path(uint64_t epoch, int src, int dst) {
  return g_dir + "/x" + std::to_string(epoch) + "_" + std::to_string(src) + "_" + std::to_string(dst);
}

std::vector<std::vector<char>> exchange(const std::vector<std::vector<char>>& outgoing) {
  const int P = n_pes();
  const uint64_t epoch = g_epoch++;
  for (int d = 0; d < P; ++d) {
    FILE* f = std::fopen(blob_path(epoch, g_pe, d).c_str(), "wb");
    if (!f) { std::perror("dkshim: open"); std::exit(5); }
    if (!outgoing[d].empty() && std::fwrite(outgoing[d].data(), 1, outgoing[d].size(), f) != outgoing[d].size()) {
      std::perror("dkshim: write"); std::exit(5);
    }
    std::fclose(f);
  }
  barrier();
  std::vector<std::vector<char>> in(P);
  for (int s = 0; s < P; ++s) {
    const std::string path = blob_path(epoch, s, g_pe);
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) { std::perror("dkshim: open in"); std::exit(5); }
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    in[s].resize((size_t)n);
    if (n > 0 && std::fread(in[s].data(), 1, (size_t)n, f) != (size_t)n) { std::perror("dkshim: read"); std::exit(5); }
    std::fclose(f);
    std::remove(path.c_str());
  }
  barrier();
  return in;
}

}  // namespace dkshim

extern "C" {

int shmem_my_pe(void) { return dkshim::my_pe(); }
int shmem_n_pes(void) { return dkshim::n_pes(); }
void shmem_barrier_all(void) { dkshim::barrier(); }
void shmem_init(void) {}
void shmem_finalize(void) {}

double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void reduce_one(const void* send, void* recv, MPI_Datatype t, MPI_Op op, bool to_all, int root) {
  using namespace dkshim;
  const int P = n_pes(), me = my_pe();
  const bool is_float = (t == MPI_DOUBLE);
  if (is_float) g_sh->dslot[me] = *(const double*)send;
  else if (t == MPI_UINT32_T) g_sh->uslot[me] = *(const uint32_t*)send;
  else if (t == MPI_LONG_LONG) g_sh->uslot[me] = (uint64_t)*(const long long*)send;
  else g_sh->uslot[me] = *(const uint64_t*)send;
  barrier();
  if (to_all || me == root) {
    double dv = g_sh->dslot[0];
    uint64_t uv = g_sh->uslot[0];
    for (int p = 1; p < P; ++p) {
      if (is_float) dv = (op == MPI_MAX) ? (g_sh->dslot[p] > dv ? g_sh->dslot[p] : dv) : dv + g_sh->dslot[p];
      else uv = (op == MPI_MAX) ? (g_sh->uslot[p] > uv ? g_sh->uslot[p] : uv) : uv + g_sh->uslot[p];
    }
    if (is_float) *(double*)recv = dv;
    else if (t == MPI_UINT32_T) *(uint32_t*)recv = (uint32_t)uv;
    else if (t == MPI_LONG_LONG) *(long long*)recv = (long long)uv;
    else *(uint64_t*)recv = uv;
  }
  barrier();
}

int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm) {
  if (count != 1) std::abort();
  reduce_one(send, recv, t, op, false, root);
  return 0;
}

int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, MPI_Comm) {
  if (count != 1) std::abort();
  reduce_one(send, recv, t, op, true, 0);
  return 0;
}

}  // extern "C"
