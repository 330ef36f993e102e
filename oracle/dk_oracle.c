/*
 * dk_oracle.c -- CPU oracle for DAKC's k-mer counting path.  TEST
 * INFRASTRUCTURE ONLY: the GPU engine never links, loads or calls this file;
 * tests, the smoke check and the CPU-baseline leg of the benchmark use it as
 * the checker.
 *
 * It restates, in plain C, what the reference computes on the path
 *   text lines -> 2-bit k-mers -> owner partition -> sort -> run-length table
 * following (paths relative to the reference project):
 *   dakc/src/common/common.hpp:72-92      char2base (base code table)
 *   dakc/src/common/common.hpp:61         KMER_MASK
 *   dakc/src/kcounter/kcounter_funcs.cpp:25-38   set_kmer_fast / update_kmer_fast
 *   dakc/src/kcounter/kcounter_funcs.cpp:40-67   get_kmers
 *   dakc/src/kcounter/kcounter_funcs.cpp:69-111  read_till_buf_max (line framing,
 *                                                'M' stop, break bytes, NUL stop)
 *   dakc/src/kcounter/kcounter.cpp:29-54         MurmurHash64A + owner_pe
 *   dakc/src/kcounter/kcounter.cpp:385-414       sort + run-length (HITTER=0)
 *   dakc/src/fqreader/fqreader.cpp:43-52         per-PE line split
 *
 * Three entry points:
 *   dko_count       single-threaded: extract -> LSD radix sort -> RLE.  The
 *                   plain checker.
 *   dko_count_mt    the same table on T host threads for inputs of billions of
 *                   k-mers: the key space is cut into ranges by its top bits,
 *                   and each range is sorted and run-length reduced on its own
 *                   (the ranges' tables, in range order, are the sorted table).
 *   dko_dakc_port   DAKC's two phases on P host threads: phase 1 parses each
 *                   PE's line range and routes every k-mer to
 *                   MurmurHash64A(kmer) % P; phase 2 sorts and run-length
 *                   reduces each owner's keys.  Timed as the CPU baseline; its
 *                   merged table must equal dko_count's.
 *
 * Framing rules (the reference's behaviour with one PE):
 *   - a line is line_width bytes followed by one terminator byte that is never
 *     examined; the last terminator may be missing;
 *   - parsing stops before the first line (other than line 0) whose first byte
 *     is NUL, as read_till_buf_max stops at rchunk[read_idx] == '\0';
 *   - the final run of a line is emitted only if its start index is below
 *     line_width-1 (kcounter_funcs.cpp:97), which matters only for k = 1.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <time.h>
#include <unistd.h>

#include "dk_oracle.h"

/* ------------------------------------------------------------ base codes */
/* C=0, A=1, T=2, G=3 (either case); 'M'/'m' = end of read (0xF0); anything
 * else is a break (0xFF).  Same mapping as char2base, built here from the
 * rule rather than copied as a table. */
static uint8_t g_code[256];
static pthread_once_t g_code_once = PTHREAD_ONCE_INIT;
static void build_codes(void) {
  for (int c = 0; c < 256; ++c) g_code[c] = 0xFF;
  g_code['C'] = g_code['c'] = 0;
  g_code['A'] = g_code['a'] = 1;
  g_code['T'] = g_code['t'] = 2;
  g_code['G'] = g_code['g'] = 3;
  g_code['M'] = g_code['m'] = 0xF0;
}
const uint8_t* dko_code_table(void) {
  pthread_once(&g_code_once, build_codes);
  return g_code;
}

static inline uint64_t kmer_mask(int k) { return (~0ULL) >> (64 - 2 * k); }

/* number of lines the framing rules allow; -1 for a malformed size */
int64_t dko_num_lines(const char* text, uint64_t nbytes, int line_width) {
  if (line_width < 1) return -1;
  const uint64_t stride = (uint64_t)line_width + 1;
  if (nbytes == 0) return 0;
  const uint64_t rem = nbytes % stride;
  if (rem != 0 && rem != (uint64_t)line_width) return -1;
  uint64_t lines = (nbytes + 1) / stride;
  for (uint64_t i = 1; i < lines; ++i)
    if (text[i * stride] == '\0') return (int64_t)i;
  return (int64_t)lines;
}

/* k-mers of one run of decoded bases (get_kmers) */
static inline uint64_t emit_run(const uint8_t* b, int len, int k, uint64_t mask,
                                uint64_t* out) {
  if (len < k) return 0;
  uint64_t key = 0, n = 0;
  for (int i = 0; i < k; ++i) key = (key << 2) | b[i];
  if (out) out[n] = key;
  ++n;
  for (int i = k; i < len; ++i) {
    key = ((key << 2) | b[i]) & mask;
    if (out) out[n] = key;
    ++n;
  }
  return n;
}

/* k-mers of one line (the body of read_till_buf_max's per-read loop) */
static uint64_t line_kmers(const char* line, int W, int k, uint8_t* scratch, uint64_t* out) {
  const uint8_t* code = dko_code_table();
  const uint64_t mask = kmer_mask(k);
  uint64_t n = 0;
  int left = 0, i;
  for (i = 0; i < W; ++i) {
    const uint8_t c = code[(uint8_t)line[i]];
    scratch[i] = c;
    if (c == 0xFF) {
      n += emit_run(scratch + left, i - left, k, mask, out ? out + n : NULL);
      left = i + 1;
    }
    if (c == 0xF0) break;
  }
  if (left < W - 1) n += emit_run(scratch + left, i - left, k, mask, out ? out + n : NULL);
  return n;
}

/* Extract the k-mers of lines [l0, l1) in order.  Returns the count; writes
 * keys to out when out != NULL. */
uint64_t dko_extract_lines(const char* text, int W, int k, uint64_t l0, uint64_t l1, uint64_t* out) {
  uint8_t* scratch = (uint8_t*)malloc((size_t)W + 1);
  const uint64_t stride = (uint64_t)W + 1;
  uint64_t n = 0;
  for (uint64_t l = l0; l < l1; ++l)
    n += line_kmers(text + l * stride, W, k, scratch, out ? out + n : NULL);
  free(scratch);
  return n;
}

/* ------------------------------------------------------------ sorting */
/* LSD radix sort of u64 keys on their low `bits` bits, 11-bit digits. */
static void radix_sort_u64(uint64_t* a, uint64_t* tmp, uint64_t n, int bits) {
  const int D = 11, R = 1 << D;
  uint64_t* cnt = (uint64_t*)malloc(sizeof(uint64_t) * R);
  uint64_t *src = a, *dst = tmp;
  for (int shift = 0; shift < bits; shift += D) {
    memset(cnt, 0, sizeof(uint64_t) * R);
    for (uint64_t i = 0; i < n; ++i) cnt[(src[i] >> shift) & (R - 1)]++;
    uint64_t s = 0;
    for (int d = 0; d < R; ++d) { uint64_t c = cnt[d]; cnt[d] = s; s += c; }
    for (uint64_t i = 0; i < n; ++i) dst[cnt[(src[i] >> shift) & (R - 1)]++] = src[i];
    uint64_t* t = src; src = dst; dst = t;
  }
  if (src != a) memcpy(a, src, sizeof(uint64_t) * n);
  free(cnt);
}

/* run-length reduce sorted keys into (key, count); returns distinct count.
 * Sets *overflow when a count does not fit 32 bits. */
static uint64_t rle(const uint64_t* keys, uint64_t n, uint64_t* ok, uint32_t* oc, int* overflow) {
  if (n == 0) return 0;
  uint64_t d = 0, cur = keys[0], run = 1;
  for (uint64_t i = 1; i < n; ++i) {
    if (keys[i] == cur) { ++run; continue; }
    ok[d] = cur; if (run > 0xFFFFFFFFull) *overflow = 1; oc[d] = (uint32_t)run; ++d;
    cur = keys[i]; run = 1;
  }
  ok[d] = cur; if (run > 0xFFFFFFFFull) *overflow = 1; oc[d] = (uint32_t)run; ++d;
  return d;
}

static int check_args(const char* text, uint64_t nbytes, int W, int k, int64_t* lines) {
  if (k < 1 || k > 32) return DKO_ERR_ARG;
  if (!text && nbytes) return DKO_ERR_ARG;
  *lines = dko_num_lines(text, nbytes, W);
  if (*lines < 0) return DKO_ERR_ARG;
  return 0;
}

int dko_count(const char* text, uint64_t nbytes, int line_width, int k, dko_table* out) {
  memset(out, 0, sizeof(*out));
  int64_t lines;
  int rc = check_args(text, nbytes, line_width, k, &lines);
  if (rc) return rc;
  const uint64_t nk = dko_extract_lines(text, line_width, k, 0, (uint64_t)lines, NULL);
  uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (nk ? nk : 1));
  uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (nk ? nk : 1));
  dko_extract_lines(text, line_width, k, 0, (uint64_t)lines, keys);
  radix_sort_u64(keys, tmp, nk, 2 * k);
  out->kmers = tmp;  /* reuse the scratch for the table keys */
  out->counts = (uint32_t*)malloc(sizeof(uint32_t) * (nk ? nk : 1));
  int overflow = 0;
  out->n = rle(keys, nk, out->kmers, out->counts, &overflow);
  out->n_kmers = nk;
  free(keys);
  return overflow ? DKO_ERR_OVERFLOW : 0;
}

void dko_free(dko_table* t) {
  if (!t) return;
  free(t->kmers); free(t->counts);
  t->kmers = NULL; t->counts = NULL; t->n = 0;
}

/* ------------------------------------------------ DAKC two-phase port */
/* MurmurHash64A of one 64-bit key with DAKC's seed (kcounter.cpp:29-54). */
uint64_t dko_murmur64a(uint64_t key, uint64_t seed) {
  const uint64_t m = 0xc6a4a7935bd1e995ULL;
  const int r = 47;
  uint64_t h = seed ^ (8 * m);
  uint64_t x = key * m;
  x ^= x >> r;
  x *= m;
  h ^= x;
  h *= m;
  h ^= h >> r;
  h *= m;
  h ^= h >> r;
  return h;
}

typedef struct {
  /* shared */
  const char* text; int W, k, P; uint64_t lines;
  uint64_t** send;     /* [P*P] per (src,dst) key buffers */
  uint64_t* send_n;    /* [P*P] */
  uint64_t** tab_k; uint32_t** tab_c; uint64_t* tab_n;  /* per-owner tables */
  pthread_barrier_t* bar;
  int overflow;
  double t_phase1, t_total;
  /* per worker */
  int pe;
} port_arg;

static double now_s(void) {
  struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void* port_worker(void* vp) {
  port_arg* a = (port_arg*)vp;
  const int P = a->P, me = a->pe;
  /* phase 1: this PE's line range, exactly fqreader's split */
  const uint64_t per = a->lines / (uint64_t)P;
  const uint64_t l0 = per * (uint64_t)me;
  const uint64_t l1 = (me == P - 1) ? a->lines : l0 + per;
  const uint64_t n = dko_extract_lines(a->text, a->W, a->k, l0, l1, NULL);
  uint64_t* mine = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  dko_extract_lines(a->text, a->W, a->k, l0, l1, mine);
  uint64_t* cnt = (uint64_t*)calloc((size_t)P, sizeof(uint64_t));
  uint32_t* owner = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  for (uint64_t i = 0; i < n; ++i) {
    owner[i] = (uint32_t)(dko_murmur64a(mine[i], 0x9E3779B97F4A7C15ULL) % (uint64_t)P);
    cnt[owner[i]]++;
  }
  for (int d = 0; d < P; ++d) {
    a->send[me * P + d] = (uint64_t*)malloc(sizeof(uint64_t) * (cnt[d] ? cnt[d] : 1));
    a->send_n[me * P + d] = 0;
  }
  for (uint64_t i = 0; i < n; ++i) {
    const int d = (int)owner[i];
    a->send[me * P + d][a->send_n[me * P + d]++] = mine[i];
  }
  free(mine); free(owner); free(cnt);
  pthread_barrier_wait(a->bar);
  /* phase 2: gather what was sent to me, sort, run-length */
  uint64_t tot = 0;
  for (int s = 0; s < P; ++s) tot += a->send_n[s * P + me];
  uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (tot ? tot : 1));
  uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (tot ? tot : 1));
  uint64_t off = 0;
  for (int s = 0; s < P; ++s) {
    memcpy(keys + off, a->send[s * P + me], sizeof(uint64_t) * a->send_n[s * P + me]);
    off += a->send_n[s * P + me];
  }
  radix_sort_u64(keys, tmp, tot, 2 * a->k);
  uint32_t* cnts = (uint32_t*)malloc(sizeof(uint32_t) * (tot ? tot : 1));
  int ovf = 0;
  const uint64_t d = rle(keys, tot, tmp, cnts, &ovf);
  if (ovf) a->overflow = 1;
  a->tab_k[me] = tmp; a->tab_c[me] = cnts; a->tab_n[me] = d;
  free(keys);
  return NULL;
}

int dko_dakc_port(const char* text, uint64_t nbytes, int line_width, int k, int pes,
                  int merge, dko_table* out, double* seconds) {
  memset(out, 0, sizeof(*out));
  int64_t lines;
  int rc = check_args(text, nbytes, line_width, k, &lines);
  if (rc) return rc;
  if (pes < 1) return DKO_ERR_ARG;
  const int P = pes;
  port_arg* args = (port_arg*)calloc((size_t)P, sizeof(port_arg));
  pthread_t* th = (pthread_t*)calloc((size_t)P, sizeof(pthread_t));
  uint64_t** send = (uint64_t**)calloc((size_t)P * P, sizeof(uint64_t*));
  uint64_t* send_n = (uint64_t*)calloc((size_t)P * P, sizeof(uint64_t));
  uint64_t** tab_k = (uint64_t**)calloc((size_t)P, sizeof(uint64_t*));
  uint32_t** tab_c = (uint32_t**)calloc((size_t)P, sizeof(uint32_t*));
  uint64_t* tab_n = (uint64_t*)calloc((size_t)P, sizeof(uint64_t));
  pthread_barrier_t bar;
  pthread_barrier_init(&bar, NULL, (unsigned)P);
  const double t0 = now_s();
  for (int p = 0; p < P; ++p) {
    port_arg* a = &args[p];
    a->text = text; a->W = line_width; a->k = k; a->P = P; a->lines = (uint64_t)lines;
    a->send = send; a->send_n = send_n; a->tab_k = tab_k; a->tab_c = tab_c; a->tab_n = tab_n;
    a->bar = &bar; a->pe = p;
    pthread_create(&th[p], NULL, port_worker, a);
  }
  for (int p = 0; p < P; ++p) pthread_join(th[p], NULL);
  const double t1 = now_s();
  if (seconds) *seconds = t1 - t0;
  int overflow = 0;
  for (int p = 0; p < P; ++p) overflow |= args[p].overflow;
  uint64_t total_d = 0;
  for (int p = 0; p < P; ++p) total_d += tab_n[p];
  for (int i = 0; i < P * P; ++i) free(send[i]);
  if (merge) {
    /* P-way merge of the owners' sorted tables (keys are unique across owners) */
    out->kmers = (uint64_t*)malloc(sizeof(uint64_t) * (total_d ? total_d : 1));
    out->counts = (uint32_t*)malloc(sizeof(uint32_t) * (total_d ? total_d : 1));
    uint64_t* pos = (uint64_t*)calloc((size_t)P, sizeof(uint64_t));
    uint64_t nk = 0;
    for (uint64_t o = 0; o < total_d; ++o) {
      int best = -1;
      for (int p = 0; p < P; ++p)
        if (pos[p] < tab_n[p] && (best < 0 || tab_k[p][pos[p]] < tab_k[best][pos[best]])) best = p;
      out->kmers[o] = tab_k[best][pos[best]];
      out->counts[o] = tab_c[best][pos[best]];
      nk += out->counts[o];
      pos[best]++;
    }
    out->n = total_d; out->n_kmers = nk;
    free(pos);
  } else {
    uint64_t nk = 0;
    for (int p = 0; p < P; ++p)
      for (uint64_t i = 0; i < tab_n[p]; ++i) nk += tab_c[p][i];
    out->n = total_d; out->n_kmers = nk;
  }
  for (int p = 0; p < P; ++p) { free(tab_k[p]); free(tab_c[p]); }
  pthread_barrier_destroy(&bar);
  free(args); free(th); free(send); free(send_n); free(tab_k); free(tab_c); free(tab_n);
  return overflow ? DKO_ERR_OVERFLOW : 0;
}

/* ------------------------------------------------ range-parallel checker */
/* dko_count's table on T threads.  Thread t extracts the k-mers of its share
 * of the lines and histograms them by range (the top B key bits); the keys are
 * then scattered into one array grouped by range; each range is radix sorted
 * on its free bits and run-length reduced in place (kcounter.cpp:385-414's
 * sort + run-length per range); the ranges' tables are concatenated in range
 * order.  Independent of the engine's partition and hashing. */
typedef struct {
  const char* text; int W, k, T, B; uint64_t lines;
  uint64_t** local; uint64_t* local_n;   /* [T] extracted keys */
  uint64_t* hist;                         /* [T * R] keys per (thread, range) */
  uint64_t* rbase;                        /* [R + 1] range starts */
  uint64_t* rdist;                        /* [R] distinct keys per range */
  uint64_t* all; uint64_t* tmp;           /* [n] grouped keys, scratch */
  uint64_t* out_k; uint32_t* out_c;       /* [distinct] */
  uint64_t* dbase;                        /* [R + 1] output starts */
  uint64_t next_range;                    /* work counter (phase C) */
  pthread_mutex_t mu;
  pthread_barrier_t bar;
  int overflow;
  int fail;
} mt_shared;

typedef struct { mt_shared* s; int t; } mt_arg;

static int mt_take_range(mt_shared* s) {
  pthread_mutex_lock(&s->mu);
  const uint64_t r = s->next_range++;
  pthread_mutex_unlock(&s->mu);
  return (int)r;
}

static void* mt_worker(void* vp) {
  mt_arg* a = (mt_arg*)vp;
  mt_shared* s = a->s;
  const int t = a->t, T = s->T, R = 1 << s->B, sh = 2 * s->k - s->B;
  /* A: extract and histogram this thread's lines */
  const uint64_t l0 = s->lines * (uint64_t)t / (uint64_t)T;
  const uint64_t l1 = s->lines * (uint64_t)(t + 1) / (uint64_t)T;
  const uint64_t n = dko_extract_lines(s->text, s->W, s->k, l0, l1, NULL);
  uint64_t* mine = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  if (!mine) s->fail = 1;
  else dko_extract_lines(s->text, s->W, s->k, l0, l1, mine);
  s->local[t] = mine; s->local_n[t] = mine ? n : 0;
  uint64_t* h = s->hist + (size_t)t * R;
  for (uint64_t i = 0; i < s->local_n[t]; ++i) h[mine[i] >> sh]++;
  pthread_barrier_wait(&s->bar);
  if (t == 0) {  /* range starts, and each thread's cursor per range */
    uint64_t run = 0;
    for (int r = 0; r < R; ++r) {
      s->rbase[r] = run;
      for (int u = 0; u < T; ++u) {
        const uint64_t c = s->hist[(size_t)u * R + r];
        s->hist[(size_t)u * R + r] = run;
        run += c;
      }
    }
    s->rbase[R] = run;
    s->all = (uint64_t*)malloc(sizeof(uint64_t) * (run ? run : 1));
    s->tmp = (uint64_t*)malloc(sizeof(uint64_t) * (run ? run : 1));
    if (!s->all || !s->tmp) s->fail = 1;
  }
  pthread_barrier_wait(&s->bar);
  /* B: scatter into the grouped array */
  if (!s->fail)
    for (uint64_t i = 0; i < s->local_n[t]; ++i) s->all[h[mine[i] >> sh]++] = mine[i];
  free(mine);
  s->local[t] = NULL;
  pthread_barrier_wait(&s->bar);
  /* C: sort and run-length reduce each range in place (distinct keys at the
   * range's start in all[], counts at its start in tmp[] viewed as u32) */
  for (int r; !s->fail && (r = mt_take_range(s)) < R;) {
    const uint64_t b = s->rbase[r], m = s->rbase[r + 1] - b;
    radix_sort_u64(s->all + b, s->tmp + b, m, sh);
    int ovf = 0;
    s->rdist[r] = rle(s->all + b, m, s->all + b, (uint32_t*)(s->tmp + b), &ovf);
    if (ovf) s->overflow = 1;
  }
  pthread_barrier_wait(&s->bar);
  if (t == 0 && !s->fail) {
    uint64_t run = 0;
    for (int r = 0; r < R; ++r) { s->dbase[r] = run; run += s->rdist[r]; }
    s->dbase[R] = run;
    s->out_k = (uint64_t*)malloc(sizeof(uint64_t) * (run ? run : 1));
    s->out_c = (uint32_t*)malloc(sizeof(uint32_t) * (run ? run : 1));
    if (!s->out_k || !s->out_c) s->fail = 1;
  }
  pthread_barrier_wait(&s->bar);
  /* D: concatenate the ranges' tables (ranges split evenly over threads) */
  if (!s->fail)
    for (int r = t; r < R; r += T) {
      const uint64_t b = s->rbase[r], d = s->rdist[r], o = s->dbase[r];
      memcpy(s->out_k + o, s->all + b, sizeof(uint64_t) * d);
      memcpy(s->out_c + o, (const uint32_t*)(s->tmp + b), sizeof(uint32_t) * d);
    }
  return NULL;
}

int dko_count_mt(const char* text, uint64_t nbytes, int line_width, int k, int threads,
                 dko_table* out) {
  memset(out, 0, sizeof(*out));
  int64_t lines;
  int rc = check_args(text, nbytes, line_width, k, &lines);
  if (rc) return rc;
  int T = threads;
  if (T < 1) T = (int)sysconf(_SC_NPROCESSORS_ONLN);
  if (T < 1) T = 1;
  mt_shared s;
  memset(&s, 0, sizeof(s));
  s.text = text; s.W = line_width; s.k = k; s.T = T; s.lines = (uint64_t)lines;
  s.B = 2 * k < 12 ? 2 * k : 12;
  const int R = 1 << s.B;
  s.local = (uint64_t**)calloc((size_t)T, sizeof(uint64_t*));
  s.local_n = (uint64_t*)calloc((size_t)T, sizeof(uint64_t));
  s.hist = (uint64_t*)calloc((size_t)T * R, sizeof(uint64_t));
  s.rbase = (uint64_t*)calloc((size_t)R + 1, sizeof(uint64_t));
  s.rdist = (uint64_t*)calloc((size_t)R, sizeof(uint64_t));
  s.dbase = (uint64_t*)calloc((size_t)R + 1, sizeof(uint64_t));
  pthread_mutex_init(&s.mu, NULL);
  pthread_barrier_init(&s.bar, NULL, (unsigned)T);
  pthread_t* th = (pthread_t*)calloc((size_t)T, sizeof(pthread_t));
  mt_arg* args = (mt_arg*)calloc((size_t)T, sizeof(mt_arg));
  for (int t = 0; t < T; ++t) {
    args[t].s = &s; args[t].t = t;
    pthread_create(&th[t], NULL, mt_worker, &args[t]);
  }
  for (int t = 0; t < T; ++t) pthread_join(th[t], NULL);
  if (s.fail) {
    free(s.out_k); free(s.out_c);
    rc = DKO_ERR_ARG;
  } else {
    out->kmers = s.out_k; out->counts = s.out_c; out->n = s.dbase[R];
    out->n_kmers = s.rbase[R];
    rc = s.overflow ? DKO_ERR_OVERFLOW : 0;
  }
  free(s.all); free(s.tmp);
  pthread_barrier_destroy(&s.bar);
  pthread_mutex_destroy(&s.mu);
  free(s.local); free(s.local_n); free(s.hist); free(s.rbase); free(s.rdist); free(s.dbase);
  free(th); free(args);
  return rc;
}
