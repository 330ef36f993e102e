/* dk_oracle.h -- CPU oracle for DAKC's k-mer counting path (test
 * infrastructure only; the GPU engine never links it).  See dk_oracle.c. */
#ifndef DK_ORACLE_H
#define DK_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define DKO_ERR_ARG (-1)
#define DKO_ERR_OVERFLOW (-2)

typedef struct {
  uint64_t* kmers;   /* sorted ascending, distinct */
  uint32_t* counts;  /* occurrences of kmers[i] */
  uint64_t n;        /* distinct k-mers (DAKC's global_distinct_kmers) */
  uint64_t n_kmers;  /* k-mer occurrences (DAKC's global_kmers) */
} dko_table;

const uint8_t* dko_code_table(void);
int64_t dko_num_lines(const char* text, uint64_t nbytes, int line_width);
uint64_t dko_extract_lines(const char* text, int line_width, int k, uint64_t l0, uint64_t l1,
                           uint64_t* out);
uint64_t dko_murmur64a(uint64_t key, uint64_t seed);
int dko_count(const char* text, uint64_t nbytes, int line_width, int k, dko_table* out);
int dko_count_mt(const char* text, uint64_t nbytes, int line_width, int k, int threads,
                 dko_table* out);
int dko_dakc_port(const char* text, uint64_t nbytes, int line_width, int k, int pes, int merge,
                  dko_table* out, double* seconds);
void dko_free(dko_table* t);

#ifdef __cplusplus
}
#endif
#endif
