// Seeded synthetic read sets in DAKC's fixed-width text format.
//
// DAKC reads a header-less ".txt" file: one read per line, every line exactly
// READLEN bytes followed by '\n', short reads padded with 'M'
// (syngen/fq2txtmaker.sh:12-18, dakc/src/fqreader/fqreader.cpp:43).  The
// reference's own generator seeds from std::random_device and then runs ART
// (syngen/inputgenerator.cpp:15-19, syngen/synthetic_generator.sh:11), so
// nothing it produces is reproducible; this file writes seeded stand-ins with
// the shapes of the benchmark workloads instead.
//
// Determinism contract: every byte depends only on (seed, parameters).  Each
// read draws from its own RNG stream derived from (seed, read index), so the
// output is identical for any thread count.  No libm call is used: the few
// transcendental functions needed (log/exp for lognormal, Zipf, exponential
// draws) are computed here from +,-,*,/ and sqrt, which IEEE-754 rounds
// identically on x86-64 and AArch64 (the file is compiled with
// -ffp-contract=off so no fused multiply-add changes a rounding).
#include <cstdint>
#include <cstring>
#include <cmath>
#include <vector>
#include <thread>
#include <algorithm>

namespace {

// ---------------------------------------------------------------- RNG
inline uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

struct Rng {  // xoshiro256** (Blackman & Vigna, 2018)
  uint64_t s[4];
  explicit Rng(uint64_t seed, uint64_t stream = 0) {
    uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ULL);
    for (int i = 0; i < 4; ++i) s[i] = splitmix64(x);
  }
  static inline uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
  inline uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
  }
  // uniform integer in [0, n) (Lemire's multiply-shift; bias < 2^-32 for n < 2^32)
  inline uint64_t below(uint64_t n) {
    return (uint64_t)(((unsigned __int128)next() * n) >> 64);
  }
  // uniform double in [0, 1) with 53 random bits
  inline double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// -------------------------------------------- portable log / exp / pow
const double kLn2 = 0.69314718055994530942;

double det_log(double x) {
  // x = m * 2^e, m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s), s = (m-1)/(m+1)
  int e = 0;
  double m = std::frexp(x, &e);  // exact
  if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double term = s, sum = 0.0;
  for (int n = 1; n <= 41; n += 2) { sum += term / (double)n; term *= s2; }
  return 2.0 * sum + (double)e * kLn2;
}

double det_exp(double x) {
  const double n = std::floor(x / kLn2 + 0.5);
  const double r = x - n * kLn2;  // |r| <= ~0.35
  double term = 1.0, sum = 1.0;
  for (int i = 1; i <= 24; ++i) { term *= r / (double)i; sum += term; }
  return std::ldexp(sum, (int)n);  // exact
}

double det_pow(double a, double b) { return det_exp(b * det_log(a)); }

// standard normal, Marsaglia polar method (needs log and sqrt only)
double normal(Rng& g) {
  for (;;) {
    const double u = 2.0 * g.unit() - 1.0, v = 2.0 * g.unit() - 1.0;
    const double s = u * u + v * v;
    if (s >= 1.0 || s == 0.0) continue;
    return u * std::sqrt(-2.0 * det_log(s) / s);
  }
}

const char kBase[4] = {'A', 'C', 'G', 'T'};
inline char complement(char c) {
  switch (c) { case 'A': return 'T'; case 'T': return 'A'; case 'C': return 'G'; case 'G': return 'C'; }
  return c;
}
inline char substitute(char c, Rng& g) {  // a uniformly chosen *different* base
  int idx = (c == 'A') ? 0 : (c == 'C') ? 1 : (c == 'G') ? 2 : 3;
  idx = (idx + 1 + (int)g.below(3)) & 3;
  return kBase[idx];
}

// threshold t such that P(next() < t) = p, for a uniform 64-bit draw
inline uint64_t prob_threshold(double p) {
  if (p <= 0.0) return 0;
  if (p >= 1.0) return ~0ULL;
  return (uint64_t)(p * 18446744073709551616.0);
}

template <class F>
void parallel_for(uint64_t n, int threads, F&& body) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (n < 4096 || threads == 1) { body(0, n); return; }
  std::vector<std::thread> pool;
  const uint64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const uint64_t lo = t * chunk, hi = std::min<uint64_t>(n, lo + chunk);
    if (lo >= hi) break;
    pool.emplace_back([lo, hi, &body] { body(lo, hi); });
  }
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

// iid uniform ACGT genome of `len` bases (no terminator written).
void dks_genome_uniform(uint64_t seed, uint64_t len, char* out, int threads) {
  const uint64_t block = 1 << 16;
  const uint64_t nblocks = (len + block - 1) / block;
  parallel_for(nblocks, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t b = lo; b < hi; ++b) {
      Rng g(seed, b);
      const uint64_t end = std::min(len, (b + 1) * block);
      for (uint64_t i = b * block; i < end; i += 32) {
        uint64_t r = g.next();
        for (uint64_t j = i; j < std::min(end, i + 32); ++j) { out[j] = kBase[r & 3]; r >>= 2; }
      }
    }
  });
}

// Genome of `len` bases in which about `repeat_frac` of the sequence is made of
// `nfam` repeat families: each family has a consensus of U[lmin,lmax] bases and
// U[cmin,cmax] copies (scaled so the copies cover repeat_frac*len, never below
// cmin), each copy diverged from the consensus by `div` per-base substitutions.
// Copies are placed at uniformly random points of a uniform background.
// Returns the number of repeat bases placed.
uint64_t dks_genome_repeats(uint64_t seed, uint64_t len, int nfam, int lmin, int lmax,
                            int cmin, int cmax, double repeat_frac, double div,
                            char* out, int threads) {
  Rng g(seed, 0xFA111E5ULL);
  std::vector<int> flen(nfam), fcopies(nfam);
  double total = 0;
  for (int f = 0; f < nfam; ++f) {
    flen[f] = lmin + (int)g.below((uint64_t)(lmax - lmin + 1));
    fcopies[f] = cmin + (int)g.below((uint64_t)(cmax - cmin + 1));
    total += (double)flen[f] * fcopies[f];
  }
  const double target = repeat_frac * (double)len;
  const double scale = total > 0 ? target / total : 0.0;
  uint64_t rep_bases = 0;
  std::vector<std::pair<int, int>> copies;  // (family, copy index)
  for (int f = 0; f < nfam; ++f) {
    int c = (int)std::floor(fcopies[f] * scale + 0.5);
    if (c < cmin) c = cmin;
    fcopies[f] = c;
    for (int i = 0; i < c; ++i) copies.emplace_back(f, i);
    rep_bases += (uint64_t)flen[f] * c;
  }
  if (rep_bases > len) rep_bases = 0, copies.clear();
  // shuffle copy order (Fisher-Yates)
  for (size_t i = copies.size(); i > 1; --i) std::swap(copies[i - 1], copies[g.below(i)]);
  // consensus sequences
  std::vector<std::vector<char>> cons(nfam);
  for (int f = 0; f < nfam; ++f) {
    Rng gf(seed, 0xC0115E45ULL + (uint64_t)f);
    cons[f].resize(flen[f]);
    for (int i = 0; i < flen[f]; ++i) cons[f][i] = kBase[gf.below(4)];
  }
  // background fills everything not covered by copies; choose gap sizes
  const uint64_t bg = len - rep_bases;
  const size_t ncp = copies.size();
  std::vector<uint64_t> cuts(ncp);
  for (size_t i = 0; i < ncp; ++i) cuts[i] = g.below(bg + 1);
  std::sort(cuts.begin(), cuts.end());
  // background sequence first (uniform), then splice: write output sequentially
  std::vector<char> bgseq(bg);
  dks_genome_uniform(seed ^ 0xB6B6B6B6ULL, bg, bgseq.data(), threads);
  uint64_t pos = 0, bpos = 0;
  for (size_t i = 0; i < ncp; ++i) {
    const uint64_t upto = cuts[i];
    std::memcpy(out + pos, bgseq.data() + bpos, upto - bpos);
    pos += upto - bpos; bpos = upto;
    const int f = copies[i].first;
    Rng gc(seed, 0xC09E5ULL + ((uint64_t)f << 20) + (uint64_t)copies[i].second);
    for (int j = 0; j < flen[f]; ++j) {
      char c = cons[f][j];
      if (gc.unit() < div) c = substitute(c, gc);
      out[pos++] = c;
    }
  }
  std::memcpy(out + pos, bgseq.data() + bpos, bg - bpos);
  return rep_bases;
}

// Sample `nreads` reads from `genome` and write them as DAKC text lines of
// `line_width` bytes + '\n' (reads shorter than line_width are padded with 'M').
// Read i: length U[len_min, len_max], start uniform in [0, glen-len], reverse
// complemented with probability rc_frac, then each base substituted with
// probability err_rate by a different base.  Requires len_max <= line_width
// and len_max <= glen.
void dks_reads(uint64_t seed, const char* genome, uint64_t glen, uint64_t nreads,
               int len_min, int len_max, int line_width, double rc_frac, double err_rate,
               char* out, int threads) {
  const uint64_t stride = (uint64_t)line_width + 1;
  const uint64_t err_thr = prob_threshold(err_rate);
  const uint64_t rc_thr = prob_threshold(rc_frac);
  parallel_for(nreads, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t r = lo; r < hi; ++r) {
      Rng g(seed, r + 1);
      const int len = len_min + (int)g.below((uint64_t)(len_max - len_min + 1));
      const uint64_t start = g.below(glen - (uint64_t)len + 1);
      const bool rc = g.next() < rc_thr;
      char* line = out + r * stride;
      if (!rc) {
        std::memcpy(line, genome + start, len);
      } else {
        for (int j = 0; j < len; ++j) line[j] = complement(genome[start + len - 1 - j]);
      }
      if (err_thr) {
        for (int j = 0; j < len; ++j)
          if (g.next() < err_thr) line[j] = substitute(line[j], g);
      }
      for (int j = len; j < line_width; ++j) line[j] = 'M';
      line[line_width] = '\n';
    }
  });
}

// Skewed workload: nreads reads of read_len bases.  With probability hot_frac a
// read is an exact copy of hot template t, t drawn Zipf(s) over `ntemplates`
// templates (P(t) ~ (t+1)^-s); otherwise it is a uniform read (50/50 strand,
// err_rate substitutions) of `background` (glen bases).  Templates are
// uniform random sequences.  hot_reads_out[t] receives the number of reads
// that copy template t (may be NULL).
void dks_zipf_reads(uint64_t seed, const char* background, uint64_t glen, uint64_t nreads,
                    int read_len, double hot_frac, int ntemplates, double s, double err_rate,
                    char* out, uint64_t* hot_reads_out, int threads) {
  const uint64_t stride = (uint64_t)read_len + 1;
  std::vector<char> tmpl((size_t)ntemplates * read_len);
  for (int t = 0; t < ntemplates; ++t) {
    Rng g(seed, 0x7E3A0000ULL + (uint64_t)t);
    for (int j = 0; j < read_len; ++j) tmpl[(size_t)t * read_len + j] = kBase[g.below(4)];
  }
  std::vector<double> cdf(ntemplates);
  double acc = 0;
  for (int t = 0; t < ntemplates; ++t) { acc += det_pow((double)(t + 1), -s); cdf[t] = acc; }
  for (int t = 0; t < ntemplates; ++t) cdf[t] /= acc;
  const uint64_t hot_thr = prob_threshold(hot_frac);
  const uint64_t err_thr = prob_threshold(err_rate);
  std::vector<uint32_t> which(nreads);
  parallel_for(nreads, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t r = lo; r < hi; ++r) {
      Rng g(seed, r + 1);
      char* line = out + r * stride;
      line[read_len] = '\n';
      if (g.next() < hot_thr) {
        const double u = g.unit();
        const int t = (int)(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        const int tt = t < ntemplates ? t : ntemplates - 1;
        std::memcpy(line, &tmpl[(size_t)tt * read_len], read_len);
        which[r] = (uint32_t)tt;
      } else {
        which[r] = 0xFFFFFFFFu;
        const uint64_t start = g.below(glen - (uint64_t)read_len + 1);
        if ((g.next() >> 63) == 0) {
          std::memcpy(line, background + start, read_len);
        } else {
          for (int j = 0; j < read_len; ++j) line[j] = complement(background[start + read_len - 1 - j]);
        }
        if (err_thr)
          for (int j = 0; j < read_len; ++j)
            if (g.next() < err_thr) line[j] = substitute(line[j], g);
      }
    }
  });
  if (hot_reads_out) {
    for (int t = 0; t < ntemplates; ++t) hot_reads_out[t] = 0;
    for (uint64_t r = 0; r < nreads; ++r)
      if (which[r] != 0xFFFFFFFFu) hot_reads_out[which[r]]++;
  }
}

// njobs lognormal integers: round(median * exp(sigma * z)), clamped to [lo, cap].
void dks_lognormal_counts(uint64_t seed, int njobs, double median, double sigma,
                          uint64_t lo, uint64_t cap, uint64_t* out) {
  Rng g(seed, 0x106A0A11ULL);
  for (int j = 0; j < njobs; ++j) {
    double v = std::floor(median * det_exp(sigma * normal(g)) + 0.5);
    if (v < (double)lo) v = (double)lo;
    if (v > (double)cap) v = (double)cap;
    out[j] = (uint64_t)v;
  }
}

// n uniform doubles in [lo, hi)
void dks_uniform(uint64_t seed, uint64_t n, double lo, double hi, double* out) {
  Rng g(seed, 0x0F0F0F0FULL);
  for (uint64_t i = 0; i < n; ++i) out[i] = lo + (hi - lo) * g.unit();
}

// n exponential(rate) draws (Poisson-process inter-arrival gaps)
void dks_exponential(uint64_t seed, uint64_t n, double rate, double* out) {
  Rng g(seed, 0xE4E4E4E4ULL);
  for (uint64_t i = 0; i < n; ++i) {
    double u = g.unit();
    if (u <= 0.0) u = 1.0 / 9007199254740992.0;
    out[i] = -det_log(u) / rate;
  }
}

// log / exp used above, exported so tests can check them against libm.
double dks_log(double x) { return det_log(x); }
double dks_exp(double x) { return det_exp(x); }

}  // extern "C"
