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
  uint64_t h = hash_key(key);
  uint64_t blk = ((h >> 32) * b->nblocks) >> 32;
  for (int i = 0; i < b->nh; ++i) {
    uint32_t bit = (uint32_t)(h >> (8 * i)) & 0xFF;
    b->words[blk * 8 + (bit >> 5)] |= 1u << (bit & 31);
  }
}

static int bloom_has(const bloom* b, int64_t key) {
  uint64_t h = hash_key(key);
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

typedef struct {
  const orc_star_fact* fact;
  const bloom* blooms[4];
  const int* order;
  int64_t lo, hi;
  int64_t* out;  /* surviving row ids */
  int64_t n_out;
} probe_task;

static void* probe_range(void* arg) {
  probe_task* t = (probe_task*)arg;
  int64_t k = 0;
  for (int64_t r = t->lo; r < t->hi; ++r) {
    int ok = 1;
    for (int j = 0; j < 4 && ok; ++j) {
      int i = t->order[j];
      ok = bloom_has(t->blooms[i], t->fact->fk[i][r]);
    }
    if (ok) t->out[k++] = r;
  }
  t->n_out = k;
  return NULL;
}

/*
 * Runs the query and writes one row per group into the out_* arrays
 * (capacity max_groups). Returns the number of groups, or -1 if max_groups
 * is too small.
 */
int64_t orc_star_query(const orc_star_fact* fact, const orc_star_dim* dims, const int32_t* consts, int bits, int nh,
                       int threads, int32_t* out_g2, int32_t* out_g4, int64_t* out_rev, int64_t* out_drev,
                       int64_t* out_cnt, int64_t max_groups) {
  if (threads < 1) threads = 1;
  /* 1. dim filters: f == const */
  int64_t* keep[4];
  int64_t nkeep[4];
  for (int i = 0; i < 4; ++i) {
    keep[i] = (int64_t*)malloc(sizeof(int64_t) * (size_t)(dims[i].n + 1));
    nkeep[i] = 0;
    for (int64_t r = 0; r < dims[i].n; ++r)
      if (dims[i].f[r] == consts[i]) keep[i][nkeep[i]++] = r;
  }
  /* 2. forward blooms on the filtered dim keys */
  bloom fwd[4];
  for (int i = 0; i < 4; ++i) {
    bloom_init(&fwd[i], nkeep[i], bits, nh);
    for (int64_t k = 0; k < nkeep[i]; ++k) bloom_add(&fwd[i], dims[i].pk[keep[i][k]]);
  }
  /* 3. probe the fact table in parallel (forward pass order 2, 3, 4, 1) */
  static const int order[4] = {1, 2, 3, 0};
  pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
  probe_task* tasks = (probe_task*)calloc((size_t)threads, sizeof(probe_task));
  int64_t per = (fact->n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    tasks[t].fact = fact;
    for (int i = 0; i < 4; ++i) tasks[t].blooms[i] = &fwd[i];
    tasks[t].order = order;
    tasks[t].lo = t * per < fact->n ? t * per : fact->n;
    tasks[t].hi = (t + 1) * per < fact->n ? (t + 1) * per : fact->n;
    tasks[t].out = (int64_t*)malloc(sizeof(int64_t) * (size_t)(tasks[t].hi - tasks[t].lo + 1));
    if (threads > 1) pthread_create(&tid[t], NULL, probe_range, &tasks[t]);
  }
  if (threads == 1) probe_range(&tasks[0]);
  int64_t survivors = 0;
  for (int t = 0; t < threads; ++t) {
    if (threads > 1) pthread_join(tid[t], NULL);
    survivors += tasks[t].n_out;
  }
  int64_t* rows = (int64_t*)malloc(sizeof(int64_t) * (size_t)(survivors + 1));
  int64_t at = 0;
  for (int t = 0; t < threads; ++t) {
    memcpy(rows + at, tasks[t].out, sizeof(int64_t) * (size_t)tasks[t].n_out);
    at += tasks[t].n_out;
    free(tasks[t].out);
  }
  free(tasks);
  free(tid);
  /* 4. backward blooms on the reduced fact keys, applied to the dims */
  imap dmap[4];
  for (int i = 0; i < 4; ++i) {
    bloom bwd;
    bloom_init(&bwd, survivors, bits, nh);
    for (int64_t k = 0; k < survivors; ++k) bloom_add(&bwd, fact->fk[i][rows[k]]);
    imap_init(&dmap[i], nkeep[i]);
    for (int64_t k = 0; k < nkeep[i]; ++k) {
      int64_t r = keep[i][k];
      if (!bloom_has(&bwd, dims[i].pk[r])) continue;
      int fresh;
      uint64_t s = imap_slot(&dmap[i], dims[i].pk[r], &fresh);
      dmap[i].vals[s] = r;  /* dim keys are unique */
    }
    free(bwd.words);
    free(fwd[i].words);
    free(keep[i]);
  }
  /* 5. 4-way inner join + group by (d2.g, d4.g) */
  imap groups;
  imap_init(&groups, max_groups > 0 ? max_groups : 1);
  int64_t ng = 0;
  for (int64_t k = 0; k < survivors; ++k) {
    int64_t r = rows[k];
    int64_t dr[4];
    int ok = 1;
    for (int i = 0; i < 4 && ok; ++i) {
      dr[i] = imap_find(&dmap[i], fact->fk[i][r]);
      ok = dr[i] >= 0;
    }
    if (!ok) continue;
    int32_t g2 = dims[1].g[dr[1]], g4 = dims[3].g[dr[3]];
    int64_t key = ((int64_t)(uint32_t)g2 << 32) | (uint32_t)g4;
    int fresh;
    uint64_t s = imap_slot(&groups, key, &fresh);
    if (fresh) {
      if (ng >= max_groups) {
        ng = -1;
        break;
      }
      groups.vals[s] = ng;
      out_g2[ng] = g2;
      out_g4[ng] = g4;
      out_rev[ng] = out_drev[ng] = out_cnt[ng] = 0;
      ++ng;
    }
    int64_t gi = groups.vals[s];
    uint64_t p = (uint64_t)fact->price[r];
    out_rev[gi] = (int64_t)((uint64_t)out_rev[gi] + p * (uint64_t)(int64_t)fact->qty[r]);
    out_drev[gi] = (int64_t)((uint64_t)out_drev[gi] + p * (uint64_t)(int64_t)fact->disc[r]);
    out_cnt[gi] += 1;
  }
  imap_free(&groups);
  for (int i = 0; i < 4; ++i) imap_free(&dmap[i]);
  free(rows);
  return ng;
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
