// Harness that runs PakMan*'s own k-mer counting code
// (pakman_star/src/kmer_counting.cpp, compiled unmodified against the
// one-rank MPI stand-in in oracle/shim_pakman) on a FASTA file and writes
// the table it builds.  Test infrastructure for the oracle only.
//
//   pakman_ref_k<K> <reads.fa> <batch k-mers> <table.bin>
//
// perform_kmer_counting (kmer_counting.cpp:502-560) counts l-mer frequencies,
// walks every read with the minimiser window (Sliding_window, :282-449),
// sends each batch of at most <batch> k-mers to its owner (transfer_kmers,
// :150-216; one rank: a copy) and merges them into kmer_proc_buf, sorted and
// aggregated.  The harness writes kmer_proc_buf as
// "PKT1", u64 n, then n records {u64 k-mer, u32 count}.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "distribute_kmers.h"

// globals PakMan* defines in distribute_kmers.cpp:63-80 (one rank)
long int MAX_KMER_COUNT = 100000000;  // the reference's default batch (:247-249)
int rank = 0, size = 1;
int coverage = 0;
int num_threads = 1;
int num_batch_transfers = 0;
std::vector<lmer_t> lmer_frequency((size_t)LMER_SIZE, 0);
std::vector<lmer_t> global_lmer_frequency((size_t)LMER_SIZE, 0);
std::vector<KmerPairs> kmer_proc_buf;

// the owner of an l-mer bucket is a hash of it modulo the rank count
// (distribute_kmers.cpp:88-94): with one rank, rank 0
int retrieve_proc_id(lmer_t) { return 0; }

void perform_kmer_counting(const char* read_data, size_t length);

// ---- one-rank MPI: every collective copies the caller's own contribution
static size_t type_bytes(MPI_Datatype t) { return t > 0 ? (size_t)t : 1; }
int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op, MPI_Comm) {
  std::memmove(recv, send, (size_t)count * type_bytes(type));
  return 0;
}
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out) {
  *out = count * (int)type_bytes(old);
  return 0;
}
int MPI_Type_commit(MPI_Datatype*) { return 0; }
int MPI_Type_free(MPI_Datatype*) { return 0; }
int MPI_Alltoall(const void* send, int scount, MPI_Datatype stype, void* recv, int, MPI_Datatype,
                 MPI_Comm) {
  std::memmove(recv, send, (size_t)scount * type_bytes(stype));
  return 0;
}
int MPI_Alltoallv(const void* send, const int* scounts, const int* sdispls, MPI_Datatype stype,
                  void* recv, const int*, const int* rdispls, MPI_Datatype rtype, MPI_Comm) {
  std::memmove((char*)recv + (size_t)rdispls[0] * type_bytes(rtype),
               (const char*)send + (size_t)sdispls[0] * type_bytes(stype),
               (size_t)scounts[0] * type_bytes(stype));
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s reads.fa batch_kmers table.bin\n", argv[0]);
    return 2;
  }
  MAX_KMER_COUNT = std::atol(argv[2]);
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) { std::perror("open"); return 2; }
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<char> buf((size_t)sz + 1, '\0');
  if (sz > 0 && std::fread(buf.data(), 1, (size_t)sz, f) != (size_t)sz) { std::perror("read"); return 2; }
  std::fclose(f);
  perform_kmer_counting(buf.data(), (size_t)sz);
  FILE* o = std::fopen(argv[3], "wb");
  const uint64_t n = kmer_proc_buf.size();
  std::fwrite("PKT1", 1, 4, o);
  std::fwrite(&n, 8, 1, o);
  for (const KmerPairs& p : kmer_proc_buf) {
    const uint64_t k = (uint64_t)p.seq;
    const uint32_t c = (uint32_t)p.k_count;
    std::fwrite(&k, 8, 1, o);
    std::fwrite(&c, 4, 1, o);
  }
  std::fclose(o);
  return 0;
}
