/*
 * CPU restatement of the star query with bloom predicate transfer, used as
 * the timed CPU baseline. TEST / BENCHMARK INFRASTRUCTURE ONLY: the library
 * never links or calls this file.
 *
 * It follows the reference's operator pipeline for the query
 * (SmallToLargePredTransOrder.cpp:38-214 for the pass order;
 * BloomFilterUseKernel.cpp:180-207 for the per-batch bloom filter pass;
 * HashJoinArrowKernel / RecordBatchHashJoiner for the inner joins;
 * GroupArrowKernel with hash_sum / hash_count for the aggregation), with the
 * fact-table passes split across `threads` POSIX threads by row range, the
 * way PARALLEL_DEGREE partitions work in the reference. Sums are int64
 * two's-complement (wrapping), as Arrow's hash_sum.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int64_t n;
  const int32_t* fk[4];
  const int32_t* qty;
  const int64_t* price;
  const int32_t* disc;
} orc_star_fact;

typedef struct {
  int64_t n;
  const int32_t* pk;
  const int32_t* f;
  const int32_t* g;
} orc_star_dim;

static uint64_t mix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

static uint64_t hash_key(int64_t v) { return mix64((uint64_t)v ^ 0x9e3779b97f4a7c15ULL); }
/* the filters' hash: Fibonacci hashing, the high bits folded into the low */
static uint64_t bloom_hash(int64_t v) {
  const uint64_t h = (uint64_t)v * 0x9e3779b97f4a7c15ULL;
  return h ^ (h >> 29);
}

typedef struct {
  uint32_t* words;
  uint64_t nblocks;
  int nh;
} bloom;

static void bloom_init(bloom* b, int64_t n, int bits, int nh) {
  int64_t nb = (n * bits + 255) / 256;
  if (nb < 1) nb = 1;
  b->nblocks = (uint64_t)nb;
  b->nh = nh;
  b->words = (uint32_t*)calloc((size_t)nb * 8, 4);
}

static void bloom_add(bloom* b, int64_t key) {
  uint64_t h = bloom_hash(key);
  uint64_t blk = ((h >> 32) * b->nblocks) >> 32;
  for (int i = 0; i < b->nh; ++i) {
    uint32_t bit = (uint32_t)(h >> (8 * i)) & 0xFF;
    b->words[blk * 8 + (bit >> 5)] |= 1u << (bit & 31);
  }
}

static int bloom_has(const bloom* b, int64_t key) {
  uint64_t h = bloom_hash(key);
  uint64_t blk = ((h >> 32) * b->nblocks) >> 32;
  for (int i = 0; i < b->nh; ++i) {
    uint32_t bit = (uint32_t)(h >> (8 * i)) & 0xFF;
    if (!((b->words[blk * 8 + (bit >> 5)] >> (bit & 31)) & 1u)) return 0;
  }
  return 1;
}

/* open-addressing map int64 key -> int64 value (value = row index) */
typedef struct {
  int64_t* keys;
  int64_t* vals;
  uint8_t* used;
  uint64_t mask;
} imap;

static void imap_init(imap* m, int64_t n) {
  uint64_t cap = 16;
  while (cap < (uint64_t)(2 * n + 1)) cap <<= 1;
  m->mask = cap - 1;
  m->keys = (int64_t*)malloc(cap * 8);
  m->vals = (int64_t*)malloc(cap * 8);
  m->used = (uint8_t*)calloc(cap, 1);
}

static void imap_free(imap* m) {
  free(m->keys);
  free(m->vals);
  free(m->used);
}

/* returns the slot; *fresh = 1 when the key was inserted */
static uint64_t imap_slot(imap* m, int64_t key, int* fresh) {
  uint64_t s = hash_key(key) & m->mask;
  while (m->used[s]) {
    if (m->keys[s] == key) {
      *fresh = 0;
      return s;
    }
    s = (s + 1) & m->mask;
  }
  m->used[s] = 1;
  m->keys[s] = key;
  *fresh = 1;
  return s;
}

static int64_t imap_find(const imap* m, int64_t key) {
  uint64_t s = hash_key(key) & m->mask;
  while (m->used[s]) {
    if (m->keys[s] == key) return m->vals[s];
    s = (s + 1) & m->mask;
  }
  return -1;
}

/*
 * The star query over a fact table of one or more partitions. The fact-table
 * passes (forward bloom probes; backward bloom builds; the 4-way join and
 * group-by) are split into chunks of at most kChunk rows of one partition
 * that `threads` POSIX threads take in turn, the way PARALLEL_DEGREE
 * partitions the reference's scans (one scan operator per partition,
 * PrePToPTransformer.cpp:1078-1100). Backward filters are built per thread
 * and OR-ed (the same bits as one build); groups are aggregated per thread
 * and merged (int64 addition wraps, so the order does not matter).
 */
enum { kChunk = 1 << 20 };

typedef struct {
  int part;
  int64_t lo, hi;
  int64_t* out; /* surviving row ids of the chunk */
  int64_t n_out;
} chunk;

typedef struct {
  const orc_star_fact* parts;
  const orc_star_dim* dims;
  const bloom* fwd;
  bloom* bwd;        /* per thread: 4 filters */
  const imap* dmap;  /* 4 maps: dim key -> dim row */
  chunk* chunks;
  int64_t n_chunks;
  int64_t* next;     /* shared chunk counter */
  int phase;         /* 0: forward probes, 1: backward builds, 2: join + group */
  /* phase 2, per thread */
  imap groups;
  int32_t *g2, *g4;
  int64_t *rev, *drev, *cnt;
  int64_t ng, max_groups;
} worker;

static const int kOrder[4] = {1, 2, 3, 0}; /* forward pass order 2, 3, 4, 1 */

static void run_chunk(worker* w, chunk* c) {
  const orc_star_fact* f = &w->parts[c->part];
  if (w->phase == 0) {
    int64_t k = 0;
    for (int64_t r = c->lo; r < c->hi; ++r) {
      int ok = 1;
      for (int j = 0; j < 4 && ok; ++j) ok = bloom_has(&w->fwd[kOrder[j]], f->fk[kOrder[j]][r]);
      if (ok) c->out[k++] = r;
    }
    c->n_out = k;
  } else if (w->phase == 1) {
    for (int64_t k = 0; k < c->n_out; ++k)
      for (int i = 0; i < 4; ++i) bloom_add(&w->bwd[i], f->fk[i][c->out[k]]);
  } else {
    if (w->ng < 0) return;
    for (int64_t k = 0; k < c->n_out; ++k) {
      const int64_t r = c->out[k];
      int64_t dr[4];
      int ok = 1;
      for (int i = 0; i < 4 && ok; ++i) {
        dr[i] = imap_find(&w->dmap[i], f->fk[i][r]);
        ok = dr[i] >= 0;
      }
      if (!ok) continue;
      const int32_t g2 = w->dims[1].g[dr[1]], g4 = w->dims[3].g[dr[3]];
      const int64_t key = ((int64_t)(uint32_t)g2 << 32) | (uint32_t)g4;
      int fresh;
      const uint64_t s = imap_slot(&w->groups, key, &fresh);
      if (fresh) {
        if (w->ng >= w->max_groups) {
          w->ng = -1;
          return;
        }
        w->groups.vals[s] = w->ng;
        w->g2[w->ng] = g2;
        w->g4[w->ng] = g4;
        w->rev[w->ng] = w->drev[w->ng] = w->cnt[w->ng] = 0;
        ++w->ng;
      }
      const int64_t gi = w->groups.vals[s];
      const uint64_t p = (uint64_t)f->price[r];
      w->rev[gi] = (int64_t)((uint64_t)w->rev[gi] + p * (uint64_t)(int64_t)f->qty[r]);
      w->drev[gi] = (int64_t)((uint64_t)w->drev[gi] + p * (uint64_t)(int64_t)f->disc[r]);
      w->cnt[gi] += 1;
    }
  }
}

static void* worker_main(void* arg) {
  worker* w = (worker*)arg;
  for (;;) {
    const int64_t i = __atomic_fetch_add(w->next, 1, __ATOMIC_RELAXED);
    if (i >= w->n_chunks) break;
    run_chunk(w, &w->chunks[i]);
  }
  return NULL;
}

static void run_phase(worker* ws, int threads, int phase, int64_t* next) {
  *next = 0;
  pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
  for (int t = 0; t < threads; ++t) {
    ws[t].phase = phase;
    if (threads > 1) pthread_create(&tid[t], NULL, worker_main, &ws[t]);
  }
  if (threads == 1) worker_main(&ws[0]);
  for (int t = 0; t < threads && threads > 1; ++t) pthread_join(tid[t], NULL);
  free(tid);
}

/*
 * Runs the query with dimension filters lo[i] <= f <= hi[i] over n_parts fact
 * partitions and writes one row per group into the out_* arrays (capacity
 * max_groups). Returns the number of groups, or -1 if max_groups is too
 * small.
 */
int64_t orc_star_query_parts(const orc_star_fact* parts, int n_parts, const orc_star_dim* dims, const int32_t* lo,
                             const int32_t* hi, int bits, int nh, int threads, int32_t* out_g2, int32_t* out_g4,
                             int64_t* out_rev, int64_t* out_drev, int64_t* out_cnt, int64_t max_groups) {
  if (threads < 1) threads = 1;
  /* 1. dim filters */
  int64_t* keep[4];
  int64_t nkeep[4];
  for (int i = 0; i < 4; ++i) {
    keep[i] = (int64_t*)malloc(sizeof(int64_t) * (size_t)(dims[i].n + 1));
    nkeep[i] = 0;
    for (int64_t r = 0; r < dims[i].n; ++r)
      if (dims[i].f[r] >= lo[i] && dims[i].f[r] <= hi[i]) keep[i][nkeep[i]++] = r;
  }
  /* 2. forward blooms on the filtered dim keys */
  bloom fwd[4];
  for (int i = 0; i < 4; ++i) {
    bloom_init(&fwd[i], nkeep[i], bits, nh);
    for (int64_t k = 0; k < nkeep[i]; ++k) bloom_add(&fwd[i], dims[i].pk[keep[i][k]]);
  }
  /* chunks of every partition */
  int64_t n_chunks = 0;
  for (int p = 0; p < n_parts; ++p) n_chunks += (parts[p].n + kChunk - 1) / kChunk;
  chunk* chunks = (chunk*)calloc((size_t)(n_chunks + 1), sizeof(chunk));
  int64_t at = 0, survivors = 0;
  for (int p = 0; p < n_parts; ++p)
    for (int64_t r = 0; r < parts[p].n; r += kChunk) {
      chunks[at].part = p;
      chunks[at].lo = r;
      chunks[at].hi = r + kChunk < parts[p].n ? r + kChunk : parts[p].n;
      chunks[at].out = (int64_t*)malloc(sizeof(int64_t) * (size_t)(chunks[at].hi - r));
      ++at;
    }
  int64_t next = 0;
  worker* ws = (worker*)calloc((size_t)threads, sizeof(worker));
  for (int t = 0; t < threads; ++t) {
    ws[t].parts = parts;
    ws[t].dims = dims;
    ws[t].fwd = fwd;
    ws[t].chunks = chunks;
    ws[t].n_chunks = n_chunks;
    ws[t].next = &next;
  }
  /* 3. forward probes of the fact table (pass order 2, 3, 4, 1) */
  run_phase(ws, threads, 0, &next);
  for (int64_t c = 0; c < n_chunks; ++c) survivors += chunks[c].n_out;
  /* 4. backward blooms on the reduced fact keys (per thread, then OR-ed),
   *    applied to the filtered dims */
  for (int t = 0; t < threads; ++t) {
    ws[t].bwd = (bloom*)malloc(sizeof(bloom) * 4);
    for (int i = 0; i < 4; ++i) bloom_init(&ws[t].bwd[i], survivors, bits, nh);
  }
  run_phase(ws, threads, 1, &next);
  imap dmap[4];
  for (int i = 0; i < 4; ++i) {
    bloom* b = &ws[0].bwd[i];
    for (int t = 1; t < threads; ++t)
      for (uint64_t w = 0; w < b->nblocks * 8; ++w) b->words[w] |= ws[t].bwd[i].words[w];
    imap_init(&dmap[i], nkeep[i]);
    for (int64_t k = 0; k < nkeep[i]; ++k) {
      const int64_t r = keep[i][k];
      if (!bloom_has(b, dims[i].pk[r])) continue;
      int fresh;
      const uint64_t s = imap_slot(&dmap[i], dims[i].pk[r], &fresh);
      dmap[i].vals[s] = r; /* dim keys are unique */
    }
    for (int t = 0; t < threads; ++t) free(ws[t].bwd[i].words);
    free(fwd[i].words);
    free(keep[i]);
  }
  /* 5. 4-way inner join + group by (d2.g, d4.g), per thread, then merged */
  const int64_t cap = max_groups > 0 ? max_groups : 1;
  for (int t = 0; t < threads; ++t) {
    free(ws[t].bwd);
    ws[t].dmap = dmap;
    imap_init(&ws[t].groups, cap);
    ws[t].g2 = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
    ws[t].g4 = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
    ws[t].rev = (int64_t*)malloc(sizeof(int64_t) * (size_t)cap);
    ws[t].drev = (int64_t*)malloc(sizeof(int64_t) * (size_t)cap);
    ws[t].cnt = (int64_t*)malloc(sizeof(int64_t) * (size_t)cap);
    ws[t].ng = 0;
    ws[t].max_groups = cap;
  }
  run_phase(ws, threads, 2, &next);
  imap groups;
  imap_init(&groups, cap);
  int64_t ng = 0;
  for (int t = 0; t < threads && ng >= 0; ++t) {
    if (ws[t].ng < 0) {
      ng = -1;
      break;
    }
    for (int64_t g = 0; g < ws[t].ng; ++g) {
      const int64_t key = ((int64_t)(uint32_t)ws[t].g2[g] << 32) | (uint32_t)ws[t].g4[g];
      int fresh;
      const uint64_t s = imap_slot(&groups, key, &fresh);
      if (fresh) {
        if (ng >= max_groups) {
          ng = -1;
          break;
        }
        groups.vals[s] = ng;
        out_g2[ng] = ws[t].g2[g];
        out_g4[ng] = ws[t].g4[g];
        out_rev[ng] = out_drev[ng] = out_cnt[ng] = 0;
        ++ng;
      }
      const int64_t gi = groups.vals[s];
      out_rev[gi] = (int64_t)((uint64_t)out_rev[gi] + (uint64_t)ws[t].rev[g]);
      out_drev[gi] = (int64_t)((uint64_t)out_drev[gi] + (uint64_t)ws[t].drev[g]);
      out_cnt[gi] += ws[t].cnt[g];
    }
  }
  imap_free(&groups);
  for (int t = 0; t < threads; ++t) {
    imap_free(&ws[t].groups);
    free(ws[t].g2);
    free(ws[t].g4);
    free(ws[t].rev);
    free(ws[t].drev);
    free(ws[t].cnt);
  }
  free(ws);
  for (int i = 0; i < 4; ++i) imap_free(&dmap[i]);
  for (int64_t c = 0; c < n_chunks; ++c) free(chunks[c].out);
  free(chunks);
  return ng;
}

/* The single-table star query with filters f == consts[i]. */
int64_t orc_star_query(const orc_star_fact* fact, const orc_star_dim* dims, const int32_t* consts, int bits, int nh,
                       int threads, int32_t* out_g2, int32_t* out_g4, int64_t* out_rev, int64_t* out_drev,
                       int64_t* out_cnt, int64_t max_groups) {
  return orc_star_query_parts(fact, 1, dims, consts, consts, bits, nh, threads, out_g2, out_g4, out_rev, out_drev,
                              out_cnt, max_groups);
}

/*
 * CPU restatement of the CSV scan workload (lineitem-shaped '|'-delimited
 * text): parse the projected fields of each line the way CSVReader's parser
 * does (fpdb-tuple/src/csv/CSVToArrowSIMDChunkParser.cpp:183-374: split on
 * the delimiter, then convert each projected field), keep the rows with
 * t_lo <= t1 <= t_hi, d1 < d1_lt and i1 < i1_lt, and sum d2 * i2 (decimals as
 * int64 cents, dates as days since 1970-01-01). The text is split into
 * `threads` line-aligned ranges.
 */
typedef struct {
  const char* b;
  const char* e;
  int64_t t_lo, t_hi, d1_lt, i1_lt;
  int64_t sum, cnt;
} csv_job;

static int64_t csv_int(const char* p, const char* e) {
  int neg = 0;
  if (p < e && (*p == '-' || *p == '+')) neg = *p++ == '-';
  int64_t v = 0;
  while (p < e && *p >= '0' && *p <= '9') v = v * 10 + (*p++ - '0');
  return neg ? -v : v;
}

static int64_t csv_cents(const char* p, const char* e) {
  int neg = 0;
  if (p < e && (*p == '-' || *p == '+')) neg = *p++ == '-';
  int64_t v = 0;
  while (p < e && *p >= '0' && *p <= '9') v = v * 10 + (*p++ - '0');
  int64_t f = 0, k = 0;
  if (p < e && *p == '.') {
    ++p;
    while (p < e && k < 2 && *p >= '0' && *p <= '9') {
      f = f * 10 + (*p++ - '0');
      ++k;
    }
  }
  while (k < 2) {
    f *= 10;
    ++k;
  }
  v = v * 100 + f;
  return neg ? -v : v;
}

/* days since 1970-01-01 (H. Hinnant's days_from_civil) */
static int64_t csv_days(const char* p) {
  int64_t y = csv_int(p, p + 4), m = csv_int(p + 5, p + 7), d = csv_int(p + 8, p + 10);
  y -= m <= 2;
  const int64_t era = (y >= 0 ? y : y - 399) / 400;
  const int64_t yoe = y - era * 400;
  const int64_t doy = (153 * (m > 2 ? m - 3 : m + 9) + 2) / 5 + d - 1;
  const int64_t doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + doe - 719468;
}

static void* csv_range(void* arg) {
  csv_job* j = (csv_job*)arg;
  const char* p = j->b;
  while (p < j->e) {
    const char* f[17];
    int nf = 0;
    f[nf++] = p;
    while (p < j->e && *p != '\n') {
      if (*p == '|' && nf < 17) f[nf++] = p + 1;
      ++p;
    }
    const char* eol = p;
    if (p < j->e) ++p;  /* past '\n' */
    if (nf < 16) continue;
    const int64_t i1 = csv_int(f[0], f[1] - 1), i2 = csv_int(f[1], f[2] - 1);
    const int64_t d1 = csv_cents(f[4], f[5] - 1), d2 = csv_cents(f[5], f[6] - 1);
    const int64_t t1 = csv_days(f[8]);
    (void)eol;
    if (t1 >= j->t_lo && t1 <= j->t_hi && d1 < j->d1_lt && i1 < j->i1_lt) {
      j->sum = (int64_t)((uint64_t)j->sum + (uint64_t)d2 * (uint64_t)i2);
      j->cnt += 1;
    }
  }
  return NULL;
}

int64_t orc_csv_scan(const char* text, int64_t n, int64_t t_lo, int64_t t_hi, int64_t d1_lt, int64_t i1_lt,
                     int threads, int64_t* sum_out) {
  if (threads < 1) threads = 1;
  csv_job* jobs = (csv_job*)calloc((size_t)threads, sizeof(csv_job));
  pthread_t* tids = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
  const char* end = text + n;
  const char* at = text;
  for (int t = 0; t < threads; ++t) {
    const char* e = t == threads - 1 ? end : text + (n / threads) * (t + 1);
    if (e < at) e = at;
    while (e < end && e > text && e[-1] != '\n') ++e; /* line-aligned */
    jobs[t].b = at;
    jobs[t].e = e;
    jobs[t].t_lo = t_lo;
    jobs[t].t_hi = t_hi;
    jobs[t].d1_lt = d1_lt;
    jobs[t].i1_lt = i1_lt;
    at = e;
  }
  for (int t = 0; t < threads; ++t) pthread_create(&tids[t], NULL, csv_range, &jobs[t]);
  int64_t sum = 0, cnt = 0;
  for (int t = 0; t < threads; ++t) {
    pthread_join(tids[t], NULL);
    sum = (int64_t)((uint64_t)sum + (uint64_t)jobs[t].sum);
    cnt += jobs[t].cnt;
  }
  free(jobs);
  free(tids);
  *sum_out = sum;
  return cnt;
}
