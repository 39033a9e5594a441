/*
 * gb_oracle.c — CPU ORACLE for the GB300 GROUP BY path.
 *
 * TEST INFRASTRUCTURE ONLY: the product path never calls this code.  It is
 * loaded by tests/ (as the checker), by __graft_entry__.smoke() and by the
 * CPU-baseline leg of bench.py.  It restates, in plain C, the reference's
 * (SlothDB) CPU GROUP BY semantics:
 *
 *  - per-group, per-aggregate AggState {count, double sum, double sum_min,
 *    double sum_max, typed min/max value}:
 *      src/execution/physical_planner.cpp:6080-6128 (AggState)
 *      src/execution/physical_planner.cpp:7933-8021 (in-memory chunk loop:
 *        COUNT(*) counts every row; COUNT(col) counts non-NULL; SUM/AVG add
 *        ReadDouble(val) and count it; MIN/MAX compare the double value and
 *        keep the typed Value of the winning row)
 *  - emission: src/execution/agg_emit_helpers.cpp:26-98
 *        (SUM → static_cast<int64_t>(double) when the return type is BIGINT,
 *         empty SUM → NULL, AVG = sum / count, MIN/MAX typed)
 *  - binder return types: src/binder/binder.cpp:1345-1391
 *  - the scan filter's integer compare in int64:
 *      src/execution/physical_planner.cpp:466-479, 693-716
 *  - per-thread maps + shard merge for the multi-threaded baseline
 *      (TLSingle): src/execution/physical_planner.cpp:7613-7931, 7871-7908
 *  - RLE/bit-packed hybrid decoding: src/storage/parquet.cpp:476-609
 *    (RleDecoder::FetchRun / Next)
 *  - COUNT(DISTINCT col): each group keeps the set of the non-NULL int64
 *    values of col (src/execution/int_group_agg.cpp:89-92) and emits its
 *    size; with several threads each keeps its own sets and the merge takes
 *    their union per group (int_group_agg.cpp:154-270).  Here one set of
 *    (group, value) pairs per aggregate and thread.
 *
 * Deliberate divergence: a NULL group key forms its own group (SQL
 * semantics).  The reference's in-memory chunk loop reads the key's raw
 * storage and ignores its validity (physical_planner.cpp:7944-7946).
 *
 * Also computes, for DOUBLE SUM/AVG, a Neumaier-compensated FP64 sum per
 * group (the tolerance reference for floating-point results).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { T_SMALLINT = 1, T_INTEGER = 2, T_BIGINT = 3, T_DOUBLE = 4, T_VARCHAR = 5 };
enum { A_COUNT_STAR = 0, A_COUNT = 1, A_SUM = 2, A_AVG = 3, A_MIN = 4, A_MAX = 5, A_COUNT_DISTINCT = 6 };
enum { C_EQ = 0, C_NE, C_LT, C_LE, C_GT, C_GE };

typedef struct {
    int64_t count;
    double sum;
    double comp;      /* Neumaier compensation (oracle only) */
    int has_min, has_max;
    double sum_min, sum_max;
    int64_t min_i, max_i; /* typed value of the winning row (integer types) */
} or_state;

/* ------------------------------------------------------------ hash maps */
static inline uint64_t or_mix(uint64_t k) {
    k ^= k >> 31;
    k *= 0x7fb5d329728ea185ull;
    k ^= k >> 27;
    k *= 0x81dadef4bc2dd44dull;
    k ^= k >> 33;
    return k;
}

typedef struct {
    uint64_t *keys;
    int64_t *idx; /* -1 empty, else group index */
    uint64_t cap;
    int64_t n;
} imap;

static int imap_init(imap *m, uint64_t cap) {
    m->cap = 16;
    while (m->cap < cap) m->cap <<= 1;
    m->keys = (uint64_t *)malloc(m->cap * 8);
    m->idx = (int64_t *)malloc(m->cap * 8);
    if (!m->keys || !m->idx) return -1;
    memset(m->idx, 0xff, m->cap * 8);
    m->n = 0;
    return 0;
}

static void imap_free(imap *m) {
    free(m->keys);
    free(m->idx);
}

static int imap_grow(imap *m) {
    imap nm;
    if (imap_init(&nm, m->cap * 2)) return -1;
    for (uint64_t i = 0; i < m->cap; i++) {
        if (m->idx[i] < 0) continue;
        uint64_t s = or_mix(m->keys[i]) & (nm.cap - 1);
        while (nm.idx[s] >= 0) s = (s + 1) & (nm.cap - 1);
        nm.keys[s] = m->keys[i];
        nm.idx[s] = m->idx[i];
    }
    nm.n = m->n;
    imap_free(m);
    *m = nm;
    return 0;
}

/* returns group index; *isnew set when inserted with index `next` */
static int64_t imap_find_or_add(imap *m, uint64_t key, int64_t next, int *isnew) {
    if ((uint64_t)(m->n + 1) * 2 > m->cap) imap_grow(m);
    uint64_t s = or_mix(key) & (m->cap - 1);
    for (;;) {
        if (m->idx[s] < 0) {
            m->keys[s] = key;
            m->idx[s] = next;
            m->n++;
            *isnew = 1;
            return next;
        }
        if (m->keys[s] == key) {
            *isnew = 0;
            return m->idx[s];
        }
        s = (s + 1) & (m->cap - 1);
    }
}

/* string map: keyed by (hash, representative row) */
static inline uint64_t or_strhash(const uint8_t *p, int64_t len) {
    uint64_t h = 1469598103934665603ull ^ (uint64_t)len;
    for (int64_t i = 0; i < len; i++) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return or_mix(h);
}

/* ------------------------------------------------------------ values */
static inline double read_double(int type, const void *d, int64_t r) {
    switch (type) {
    case T_SMALLINT: return (double)((const int16_t *)d)[r];
    case T_INTEGER: return (double)((const int32_t *)d)[r];
    case T_BIGINT: return (double)((const int64_t *)d)[r];
    default: return ((const double *)d)[r];
    }
}

static inline int64_t read_int(int type, const void *d, int64_t r) {
    switch (type) {
    case T_SMALLINT: return ((const int16_t *)d)[r];
    case T_INTEGER: return ((const int32_t *)d)[r];
    default: return ((const int64_t *)d)[r];
    }
}

/* set of (group index, value) pairs: COUNT(DISTINCT) */
typedef struct {
    int64_t *g;
    int64_t *v;
    uint8_t *used;
    uint64_t cap;
    int64_t n;
} pset;

static int pset_init(pset *p, uint64_t cap) {
    p->cap = 64;
    while (p->cap < cap) p->cap <<= 1;
    p->g = (int64_t *)malloc(p->cap * 8);
    p->v = (int64_t *)malloc(p->cap * 8);
    p->used = (uint8_t *)calloc(p->cap, 1);
    p->n = 0;
    return (p->g && p->v && p->used) ? 0 : -1;
}

static void pset_free(pset *p) {
    free(p->g);
    free(p->v);
    free(p->used);
}

/* returns 1 when (g, v) was not in the set (and inserts it), 0 if present,
 * -1 on allocation failure */
static int pset_insert(pset *p, int64_t g, int64_t v) {
    if ((uint64_t)(p->n + 1) * 2 > p->cap) {
        pset q;
        if (pset_init(&q, p->cap * 2)) return -1;
        for (uint64_t i = 0; i < p->cap; i++) {
            if (!p->used[i]) continue;
            uint64_t s = or_mix(or_mix((uint64_t)p->g[i]) ^ (uint64_t)p->v[i]) & (q.cap - 1);
            while (q.used[s]) s = (s + 1) & (q.cap - 1);
            q.used[s] = 1;
            q.g[s] = p->g[i];
            q.v[s] = p->v[i];
        }
        q.n = p->n;
        pset_free(p);
        *p = q;
    }
    uint64_t s = or_mix(or_mix((uint64_t)g) ^ (uint64_t)v) & (p->cap - 1);
    while (p->used[s]) {
        if (p->g[s] == g && p->v[s] == v) return 0;
        s = (s + 1) & (p->cap - 1);
    }
    p->used[s] = 1;
    p->g[s] = g;
    p->v[s] = v;
    p->n++;
    return 1;
}

typedef struct {
    int32_t n_aggs;
    const int32_t *kind;
    const int32_t *in_type;
    const void *const *data;
    const uint8_t *const *nul; /* per agg: 1 = NULL, or NULL pointer */
    pset *dset;                /* per agg (COUNT(DISTINCT) only), or NULL */
} or_aggs;

/* The per-row AggState update of the in-memory chunk loop
 * (physical_planner.cpp:7988-8017); g = the row's group index. */
static inline int update_states(or_state *st, const or_aggs *A, int64_t r, int64_t g) {
    for (int a = 0; a < A->n_aggs; a++) {
        or_state *s = &st[a];
        int k = A->kind[a];
        if (k == A_COUNT_STAR) {
            s->count++;
            continue;
        }
        if (A->nul[a] && A->nul[a][r]) continue;
        if (k == A_COUNT) {
            s->count++;
            continue;
        }
        if (k == A_COUNT_DISTINCT) {
            int isnew = pset_insert(&A->dset[a], g, read_int(A->in_type[a], A->data[a], r));
            if (isnew < 0) return -1;
            s->count += isnew;
            continue;
        }
        double val = read_double(A->in_type[a], A->data[a], r);
        if (k == A_SUM || k == A_AVG) {
            s->count++;
            /* Neumaier: sum is the plain running double sum (as the
             * reference), comp the compensation of the exact sum */
            double t = s->sum + val;
            if (fabs(s->sum) >= fabs(val)) s->comp += (s->sum - t) + val;
            else s->comp += (val - t) + s->sum;
            s->sum = t;
        } else if (k == A_MIN) {
            if (!s->has_min || val < s->sum_min) {
                s->sum_min = val;
                s->has_min = 1;
                if (A->in_type[a] != T_DOUBLE) s->min_i = read_int(A->in_type[a], A->data[a], r);
            }
        } else if (k == A_MAX) {
            if (!s->has_max || val > s->sum_max) {
                s->sum_max = val;
                s->has_max = 1;
                if (A->in_type[a] != T_DOUBLE) s->max_i = read_int(A->in_type[a], A->data[a], r);
            }
        }
    }
    return 0;
}

/* one pair set per COUNT(DISTINCT) aggregate (zeroed entries for the others) */
static pset *dsets_new(int32_t n_aggs, const int32_t *kind) {
    pset *d = (pset *)calloc((size_t)(n_aggs > 0 ? n_aggs : 1), sizeof(pset));
    if (!d) return NULL;
    for (int a = 0; a < n_aggs; a++)
        if (kind[a] == A_COUNT_DISTINCT && pset_init(&d[a], 64)) return NULL;
    return d;
}

static void dsets_free(pset *d, int32_t n_aggs, const int32_t *kind) {
    if (!d) return;
    for (int a = 0; a < n_aggs; a++)
        if (kind[a] == A_COUNT_DISTINCT) pset_free(&d[a]);
    free(d);
}

/* Merge partial states (shard merge of the per-thread maps,
 * physical_planner.cpp:7871-7908). */
static inline void merge_states(or_state *dst, const or_state *src, const or_aggs *A) {
    for (int a = 0; a < A->n_aggs; a++) {
        or_state *d = &dst[a];
        const or_state *s = &src[a];
        if (A->kind[a] != A_COUNT_DISTINCT) d->count += s->count;  /* distinct: the union, counted by the merge */
        double t = d->sum + s->sum;
        if (fabs(d->sum) >= fabs(s->sum)) d->comp += (d->sum - t) + s->sum;
        else d->comp += (s->sum - t) + d->sum;
        d->comp += s->comp;
        d->sum = t;
        if (s->has_min && (!d->has_min || s->sum_min < d->sum_min)) {
            d->has_min = 1;
            d->sum_min = s->sum_min;
            d->min_i = s->min_i;
        }
        if (s->has_max && (!d->has_max || s->sum_max > d->sum_max)) {
            d->has_max = 1;
            d->sum_max = s->sum_max;
            d->max_i = s->max_i;
        }
    }
}

/* Emission (agg_emit_helpers.cpp:26-98).  out_i / out_d / out_null /
 * out_comp are [n_aggs][cap]. */
static void emit_group(int64_t g, int64_t cap, const or_state *st, const or_aggs *A, int64_t *out_i, double *out_d,
                       uint8_t *out_null, double *out_comp) {
    for (int a = 0; a < A->n_aggs; a++) {
        const or_state *s = &st[a];
        int64_t o = (int64_t)a * cap + g;
        int k = A->kind[a];
        int isf = (k != A_COUNT_STAR && k != A_COUNT && k != A_COUNT_DISTINCT) && A->in_type[a] == T_DOUBLE;
        out_null[o] = 0;
        out_i[o] = 0;
        out_d[o] = 0.0;
        out_comp[o] = 0.0;
        switch (k) {
        case A_COUNT_STAR:
        case A_COUNT:
        case A_COUNT_DISTINCT: out_i[o] = s->count; break;
        case A_SUM:
            if (s->count == 0) { out_null[o] = 1; break; }
            if (isf) out_d[o] = s->sum;
            else out_i[o] = (int64_t)s->sum;
            out_comp[o] = s->sum + s->comp;
            break;
        case A_AVG:
            if (s->count == 0) { out_null[o] = 1; break; }
            out_d[o] = s->sum / (double)s->count;
            out_comp[o] = (s->sum + s->comp) / (double)s->count;
            break;
        case A_MIN:
            if (!s->has_min) { out_null[o] = 1; break; }
            if (isf) out_d[o] = s->sum_min;
            else out_i[o] = s->min_i;
            break;
        case A_MAX:
            if (!s->has_max) { out_null[o] = 1; break; }
            if (isf) out_d[o] = s->sum_max;
            else out_i[o] = s->max_i;
            break;
        }
    }
}

/* ----------------------------------------------------- single-threaded core */
typedef struct {
    imap map;
    or_state *st;   /* [groups][n_aggs] */
    uint64_t *gkey; /* packed key per group */
    int64_t cap_g;
    int64_t ng;
    int has_null;   /* NULL-key group present */
    int64_t null_g; /* its index */
} or_table;

static int tab_init(or_table *t, int n_aggs, int64_t est) {
    if (imap_init(&t->map, (uint64_t)(est > 16 ? est * 2 : 32))) return -1;
    t->cap_g = est > 16 ? est : 16;
    t->st = (or_state *)calloc((size_t)t->cap_g * n_aggs, sizeof(or_state));
    t->gkey = (uint64_t *)malloc((size_t)t->cap_g * 8);
    t->ng = 0;
    t->has_null = 0;
    t->null_g = -1;
    return (t->st && t->gkey) ? 0 : -1;
}

static void tab_free(or_table *t) {
    imap_free(&t->map);
    free(t->st);
    free(t->gkey);
}

static int64_t tab_new_group(or_table *t, int n_aggs, uint64_t key) {
    if (t->ng == t->cap_g) {
        int64_t nc = t->cap_g * 2;
        or_state *ns = (or_state *)realloc(t->st, (size_t)nc * n_aggs * sizeof(or_state));
        uint64_t *nk = (uint64_t *)realloc(t->gkey, (size_t)nc * 8);
        if (!ns || !nk) return -1;
        memset(ns + (size_t)t->cap_g * n_aggs, 0, (size_t)(nc - t->cap_g) * n_aggs * sizeof(or_state));
        t->st = ns;
        t->gkey = nk;
        t->cap_g = nc;
    }
    t->gkey[t->ng] = key;
    return t->ng++;
}

static int64_t tab_group(or_table *t, int n_aggs, uint64_t key, int is_null) {
    if (is_null) {
        if (!t->has_null) {
            t->has_null = 1;
            t->null_g = tab_new_group(t, n_aggs, 0);
        }
        return t->null_g;
    }
    int isnew = 0;
    int64_t g = imap_find_or_add(&t->map, key, t->ng, &isnew);
    if (isnew) {
        int64_t g2 = tab_new_group(t, n_aggs, key);
        if (g2 != g) return -1;
    }
    return g;
}

static int run_range(or_table *t, int64_t r0, int64_t r1, const int64_t *keys, const uint8_t *key_null,
                     const uint8_t *keep, const or_aggs *A) {
    for (int64_t r = r0; r < r1; r++) {
        if (keep && !keep[r]) continue;
        int nul = key_null ? key_null[r] : 0;
        int64_t g = tab_group(t, A->n_aggs, nul ? 0 : (uint64_t)keys[r], nul);
        if (g < 0) return -1;
        if (update_states(&t->st[(size_t)g * A->n_aggs], A, r, g)) return -1;
    }
    return 0;
}

/* (thread-local group, value) pairs bound for one merge shard */
typedef struct {
    int64_t *g, *v;
    uint64_t n, cap;
} pvec;

static int pvec_push(pvec *p, int64_t g, int64_t v) {
    if (p->n == p->cap) {
        uint64_t nc = p->cap ? p->cap * 2 : 256;
        int64_t *ng = (int64_t *)realloc(p->g, nc * 8), *nv;
        if (!ng) return -1;
        p->g = ng;
        nv = (int64_t *)realloc(p->v, nc * 8);
        if (!nv) return -1;
        p->v = nv;
        p->cap = nc;
    }
    p->g[p->n] = g;
    p->v[p->n] = v;
    p->n++;
    return 0;
}

typedef struct {
    or_table tab;
    int64_t r0, r1;
    const int64_t *keys;
    const uint8_t *key_null, *keep;
    or_aggs A;  /* the query's aggregates with this thread's value sets */
    int nshards;
    pvec *bucket; /* [n_aggs][nshards]: this thread's pairs by merge shard */
    int rc;
} or_job;

static void *job_main(void *p) {
    or_job *j = (or_job *)p;
    j->rc = run_range(&j->tab, j->r0, j->r1, j->keys, j->key_null, j->keep, &j->A);
    /* hand each distinct pair to the shard that owns its group's key */
    for (int a = 0; !j->rc && j->bucket && a < j->A.n_aggs; a++) {
        if (j->A.kind[a] != A_COUNT_DISTINCT) continue;
        const pset *ps = &j->A.dset[a];
        for (uint64_t i = 0; i < ps->cap && !j->rc; i++) {
            if (!ps->used[i]) continue;
            const int64_t g = ps->g[i];
            int is_null = j->tab.has_null && g == j->tab.null_g;
            int owner = is_null ? 0 : (int)((or_mix(j->tab.gkey[g]) >> 40) % (uint64_t)j->nshards);
            if (pvec_push(&j->bucket[a * j->nshards + owner], g, ps->v[i])) j->rc = -1;
        }
    }
    return NULL;
}

typedef struct {
    or_job *jobs;
    int nt, shard, nshards;
    or_table out;
    const or_aggs *A;
    pset *dset; /* the shard's value sets (COUNT(DISTINCT)), or NULL */
    int rc;
} or_merge_job;

/* shard s owns keys with (mix(key) >> 40) % nshards == s */
static void *merge_main(void *p) {
    or_merge_job *m = (or_merge_job *)p;
    const or_aggs *A = m->A;
    m->rc = 0;
    for (int t = 0; t < m->nt; t++) {
        or_table *src = &m->jobs[t].tab;
        for (int64_t g = 0; g < src->ng; g++) {
            int is_null = src->has_null && g == src->null_g;
            uint64_t key = src->gkey[g];
            int owner = is_null ? 0 : (int)((or_mix(key) >> 40) % (uint64_t)m->nshards);
            if (owner != m->shard) continue;
            int64_t d = tab_group(&m->out, A->n_aggs, key, is_null);
            if (d < 0) { m->rc = -1; return NULL; }
            merge_states(&m->out.st[(size_t)d * A->n_aggs], &src->st[(size_t)g * A->n_aggs], A);
        }
    }
    /* COUNT(DISTINCT): the union of the threads' sets of each group */
    for (int a = 0; m->dset && a < A->n_aggs; a++) {
        if (A->kind[a] != A_COUNT_DISTINCT) continue;
        for (int t = 0; t < m->nt; t++) {
            const or_table *src = &m->jobs[t].tab;
            const pvec *pv = &m->jobs[t].bucket[a * m->nshards + m->shard];
            for (uint64_t i = 0; i < pv->n; i++) {
                const int64_t g = pv->g[i];
                int is_null = src->has_null && g == src->null_g;
                int64_t d = tab_group(&m->out, A->n_aggs, src->gkey[g], is_null);
                int isnew = d < 0 ? -1 : pset_insert(&m->dset[a], d, pv->v[i]);
                if (isnew < 0) { m->rc = -1; return NULL; }
                m->out.st[(size_t)d * A->n_aggs + a].count += isnew;
            }
        }
    }
    return NULL;
}

/*
 * GROUP BY over packed int64 keys.  Returns the number of groups, or -1 on
 * allocation failure, or -(needed) - 2 if `cap` is too small.
 * nthreads <= 1: the single-threaded chunk loop; > 1: TLSingle-style
 * per-thread maps + sharded merge.
 */
int64_t or_groupby(int64_t n, const int64_t *keys, const uint8_t *key_null, const uint8_t *keep, int32_t n_aggs,
                   const int32_t *agg_kind, const int32_t *agg_in_type, const void *const *agg_data,
                   const uint8_t *const *agg_null, int32_t nthreads, int64_t est_groups, int64_t cap,
                   int64_t *out_keys, uint8_t *out_key_null, int64_t *out_i, double *out_d, uint8_t *out_null,
                   double *out_comp) {
    or_aggs A = {n_aggs, agg_kind, agg_in_type, agg_data, agg_null, NULL};
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    int has_distinct = 0;
    for (int a = 0; a < n_aggs; a++) has_distinct |= agg_kind[a] == A_COUNT_DISTINCT;
    int64_t ng = 0;
    if (nthreads == 1) {
        or_table t;
        if (tab_init(&t, n_aggs, est_groups)) return -1;
        if (has_distinct && !(A.dset = dsets_new(n_aggs, agg_kind))) { tab_free(&t); return -1; }
        int rc = run_range(&t, 0, n, keys, key_null, keep, &A);
        dsets_free(A.dset, n_aggs, agg_kind);
        if (rc) { tab_free(&t); return -1; }
        ng = t.ng;
        if (ng > cap) { tab_free(&t); return -ng - 2; }
        for (int64_t g = 0; g < ng; g++) {
            out_keys[g] = (int64_t)t.gkey[g];
            out_key_null[g] = (t.has_null && g == t.null_g);
            emit_group(g, cap, &t.st[(size_t)g * n_aggs], &A, out_i, out_d, out_null, out_comp);
        }
        tab_free(&t);
        return ng;
    }
    or_job *jobs = (or_job *)calloc((size_t)nthreads, sizeof(or_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    int64_t per = (n + nthreads - 1) / nthreads;
    int64_t est_t = est_groups / nthreads + 16;
    for (int i = 0; i < nthreads; i++) {
        jobs[i].r0 = i * per < n ? i * per : n;
        jobs[i].r1 = (i + 1) * per < n ? (i + 1) * per : n;
        jobs[i].keys = keys;
        jobs[i].key_null = key_null;
        jobs[i].keep = keep;
        jobs[i].A = A;
        jobs[i].nshards = nthreads;
        if (has_distinct) {
            jobs[i].A.dset = dsets_new(n_aggs, agg_kind);
            jobs[i].bucket = (pvec *)calloc((size_t)n_aggs * nthreads, sizeof(pvec));
        }
        tab_init(&jobs[i].tab, n_aggs, est_t);
        if (has_distinct && (!jobs[i].A.dset || !jobs[i].bucket)) {
            dsets_free(jobs[i].A.dset, n_aggs, agg_kind);
            jobs[i].A.dset = NULL;
            jobs[i].rc = -1;
            continue;
        }
        pthread_create(&th[i], NULL, job_main, &jobs[i]);
    }
    int rc = 0;
    for (int i = 0; i < nthreads; i++) {
        if (!has_distinct || jobs[i].A.dset) pthread_join(th[i], NULL);
        rc |= jobs[i].rc;
    }
    or_merge_job *mj = (or_merge_job *)calloc((size_t)nthreads, sizeof(or_merge_job));
    int created = 0;
    for (int s = 0; s < nthreads && !rc; s++) {
        mj[s].jobs = jobs;
        mj[s].nt = nthreads;
        mj[s].shard = s;
        mj[s].nshards = nthreads;
        mj[s].A = &A;
        mj[s].dset = has_distinct ? dsets_new(n_aggs, agg_kind) : NULL;
        tab_init(&mj[s].out, n_aggs, est_groups / nthreads + 16);
        if (has_distinct && !mj[s].dset) { rc = -1; break; }
        pthread_create(&th[s], NULL, merge_main, &mj[s]);
        created++;
    }
    for (int s = 0; s < created; s++) {
        pthread_join(th[s], NULL);
        rc |= mj[s].rc;
        ng += mj[s].out.ng;
    }
    if (!rc && ng <= cap) {
        int64_t o = 0;
        for (int s = 0; s < nthreads; s++) {
            or_table *t = &mj[s].out;
            for (int64_t g = 0; g < t->ng; g++, o++) {
                out_keys[o] = (int64_t)t->gkey[g];
                out_key_null[o] = (t->has_null && g == t->null_g);
                emit_group(o, cap, &t->st[(size_t)g * n_aggs], &A, out_i, out_d, out_null, out_comp);
            }
        }
    }
    for (int s = 0; s < nthreads; s++) {
        if (mj[s].out.st) tab_free(&mj[s].out);
        dsets_free(mj[s].dset, n_aggs, agg_kind);
        dsets_free(jobs[s].A.dset, n_aggs, agg_kind);
        if (jobs[s].bucket) {
            for (int b = 0; b < n_aggs * nthreads; b++) {
                free(jobs[s].bucket[b].g);
                free(jobs[s].bucket[b].v);
            }
            free(jobs[s].bucket);
        }
        tab_free(&jobs[s].tab);
    }
    free(mj);
    free(jobs);
    free(th);
    if (rc) return -1;
    if (ng > cap) return -ng - 2;
    return ng;
}

/*
 * GROUP BY a VARCHAR key (offsets[n+1] into bytes).  out_rep receives the
 * first row of each group (the caller reads the key bytes from the input).
 * Restates the string-key branch of the chunk loop
 * (physical_planner.cpp:7951-7973: compare size + bytes, keep insertion order).
 */
int64_t or_groupby_str(int64_t n, const int64_t *offsets, const uint8_t *bytes, const uint8_t *key_null,
                       const uint8_t *keep, int32_t n_aggs, const int32_t *agg_kind, const int32_t *agg_in_type,
                       const void *const *agg_data, const uint8_t *const *agg_null, int64_t cap, int64_t *out_rep,
                       uint8_t *out_key_null, int64_t *out_i, double *out_d, uint8_t *out_null, double *out_comp) {
    or_aggs A = {n_aggs, agg_kind, agg_in_type, agg_data, agg_null, NULL};
    A.dset = dsets_new(n_aggs, agg_kind);
    if (!A.dset) return -1;
    uint64_t mcap = 64;
    while (mcap < (uint64_t)(cap > 0 ? cap : 1) * 2) mcap <<= 1;
    int64_t *slot = (int64_t *)malloc(mcap * 8); /* group index or -1 */
    uint64_t *sh = (uint64_t *)malloc(mcap * 8);
    int64_t *rep = (int64_t *)malloc((size_t)(cap > 0 ? cap : 1) * 8);
    or_state *st = (or_state *)calloc((size_t)(cap > 0 ? cap : 1) * n_aggs, sizeof(or_state));
    if (!slot || !sh || !rep || !st) return -1;
    memset(slot, 0xff, mcap * 8);
    int64_t ng = 0, null_g = -1;
    for (int64_t r = 0; r < n; r++) {
        if (keep && !keep[r]) continue;
        int64_t g;
        if (key_null && key_null[r]) {
            if (null_g < 0) {
                if (ng >= cap) { ng = cap + 1; break; }
                null_g = ng;
                rep[ng++] = r;
            }
            g = null_g;
        } else {
            const uint8_t *p = bytes + offsets[r];
            int64_t len = offsets[r + 1] - offsets[r];
            uint64_t h = or_strhash(p, len);
            uint64_t s = h & (mcap - 1);
            for (;;) {
                if (slot[s] < 0) {
                    if (ng >= cap) { g = -1; break; }
                    slot[s] = ng;
                    sh[s] = h;
                    rep[ng] = r;
                    g = ng++;
                    break;
                }
                if (sh[s] == h) {
                    int64_t q = rep[slot[s]];
                    int64_t ql = offsets[q + 1] - offsets[q];
                    if (ql == len && memcmp(bytes + offsets[q], p, (size_t)len) == 0) {
                        g = slot[s];
                        break;
                    }
                }
                s = (s + 1) & (mcap - 1);
            }
            if (g < 0) { ng = cap + 1; break; }
        }
        if (update_states(&st[(size_t)g * n_aggs], &A, r, g)) { ng = -1; break; }
    }
    if (ng <= cap) {
        for (int64_t g = 0; g < ng; g++) {
            out_rep[g] = rep[g];
            out_key_null[g] = (g == null_g);
            emit_group(g, cap, &st[(size_t)g * n_aggs], &A, out_i, out_d, out_null, out_comp);
        }
    }
    dsets_free(A.dset, n_aggs, agg_kind);
    free(slot);
    free(sh);
    free(rep);
    free(st);
    return ng <= cap ? ng : -2;
}

/* Scan filter: keep[r] &= (col[r] OP const), NULL → not kept.  Integer
 * columns compare in int64 (physical_planner.cpp:466-479, 693-716). */
void or_filter(int64_t n, int32_t type, const void *data, const uint8_t *nul, int32_t op, int64_t ic, double dc,
               uint8_t *keep) {
    for (int64_t r = 0; r < n; r++) {
        if (!keep[r]) continue;
        if (nul && nul[r]) { keep[r] = 0; continue; }
        int ok;
        if (type == T_DOUBLE) {
            double v = ((const double *)data)[r];
            switch (op) {
            case C_EQ: ok = v == dc; break;
            case C_NE: ok = v != dc; break;
            case C_LT: ok = v < dc; break;
            case C_LE: ok = v <= dc; break;
            case C_GT: ok = v > dc; break;
            default: ok = v >= dc; break;
            }
        } else {
            int64_t v = read_int(type, data, r);
            switch (op) {
            case C_EQ: ok = v == ic; break;
            case C_NE: ok = v != ic; break;
            case C_LT: ok = v < ic; break;
            case C_LE: ok = v <= ic; break;
            case C_GT: ok = v > ic; break;
            default: ok = v >= ic; break;
            }
        }
        keep[r] = (uint8_t)ok;
    }
}

/*
 * RLE/bit-packed hybrid decoder, restating RleDecoder (parquet.cpp:476-609):
 * varint header; LSB 1 → (h >> 1) * 8 bit-packed values, LSB-first, the bit
 * buffer reset at each run; LSB 0 → repeat count (h >> 1) of a value stored
 * in ceil(bw / 8) little-endian bytes.  Decodes up to n values; returns the
 * number decoded (fewer when the data ends).
 */
int64_t or_rle_decode(const uint8_t *p, int64_t size, int32_t bw, uint32_t *out, int64_t n) {
    int64_t pos = 0, got = 0;
    uint32_t mask = bw >= 32 ? 0xffffffffu : ((1u << bw) - 1u);
    while (got < n) {
        if (pos >= size) break;
        uint64_t hdr = 0;
        int sh = 0;
        while (pos < size) {
            uint8_t b = p[pos++];
            hdr |= (uint64_t)(b & 0x7f) << sh;
            if ((b & 0x80) == 0) break;
            sh += 7;
        }
        if (hdr & 1) {
            int64_t cnt = (int64_t)(hdr >> 1) * 8;
            uint64_t buf = 0;
            int bits = 0;
            for (int64_t i = 0; i < cnt && got < n; i++) {
                while (bits < bw) {
                    if (pos >= size) return got;
                    buf |= (uint64_t)p[pos++] << bits;
                    bits += 8;
                }
                out[got++] = (uint32_t)(buf & mask);
                buf >>= bw;
                bits -= bw;
            }
            /* values past n in this run are skipped: the reference stops
             * mid-run only at the end of a page */
            if (got >= n) break;
        } else {
            int64_t cnt = (int64_t)(hdr >> 1);
            int bytes = (bw + 7) / 8;
            uint32_t v = 0;
            for (int i = 0; i < bytes; i++) {
                if (pos >= size) return got;
                v |= (uint32_t)p[pos++] << (8 * i);
            }
            for (int64_t i = 0; i < cnt && got < n; i++) out[got++] = v;
        }
    }
    return got;
}

/*
 * Snappy raw-block decompression, restated from the published Snappy format
 * (the reference decompresses Parquet pages with the vendored Google Snappy
 * 1.2.1, third_party/snappy/, called from SnappyDecompress /
 * SnappyDecompressRaw, src/storage/parquet.cpp:44-90):
 *   preamble  the uncompressed length, a little-endian base-128 varint;
 *   elements  a tag byte whose low 2 bits give the kind:
 *     00 literal: length-1 in the upper 6 bits, or (60..63) in the next 1..4
 *        little-endian bytes; the bytes follow;
 *     01 copy: length 4 + bits 2..4, offset = bits 5..7 << 8 | next byte;
 *     10 copy: length 1 + upper 6 bits, offset = next 2 bytes (LE);
 *     11 copy: length 1 + upper 6 bits, offset = next 4 bytes (LE);
 *   a copy repeats `length` bytes from `offset` bytes back (byte by byte, so
 *   an offset below the length repeats a pattern); offset 0 or one reaching
 *   before the start is invalid.
 * Returns the decompressed length, or -1 (malformed, or more than cap).
 */
int64_t or_snappy_decompress(const uint8_t *src, int64_t n, uint8_t *dst, int64_t cap) {
    int64_t pos = 0;
    uint64_t want = 0;
    for (int sh = 0;; sh += 7) {
        if (pos >= n || sh > 28) return -1;
        uint8_t b = src[pos++];
        want |= (uint64_t)(b & 0x7f) << sh;
        if (!(b & 0x80)) break;
    }
    if ((int64_t)want > cap) return -1;
    int64_t out = 0;
    while (pos < n) {
        const uint8_t tag = src[pos++];
        const int kind = tag & 3;
        if (kind == 0) {
            int64_t len = (tag >> 2) + 1;
            if ((tag >> 2) >= 60) {
                const int nb = (tag >> 2) - 59;
                if (pos + nb > n) return -1;
                uint64_t l = 0;
                for (int i = 0; i < nb; i++) l |= (uint64_t)src[pos + i] << (8 * i);
                pos += nb;
                len = (int64_t)l + 1;
            }
            if (len > n - pos || len > (int64_t)want - out) return -1;
            memcpy(dst + out, src + pos, (size_t)len);
            pos += len;
            out += len;
            continue;
        }
        int64_t len, off;
        if (kind == 1) {
            if (pos + 1 > n) return -1;
            len = 4 + ((tag >> 2) & 7);
            off = ((int64_t)(tag >> 5) << 8) | src[pos];
            pos += 1;
        } else if (kind == 2) {
            if (pos + 2 > n) return -1;
            len = 1 + (tag >> 2);
            off = (int64_t)src[pos] | ((int64_t)src[pos + 1] << 8);
            pos += 2;
        } else {
            if (pos + 4 > n) return -1;
            len = 1 + (tag >> 2);
            off = (int64_t)((uint64_t)src[pos] | ((uint64_t)src[pos + 1] << 8) | ((uint64_t)src[pos + 2] << 16) |
                            ((uint64_t)src[pos + 3] << 24));
            pos += 4;
        }
        if (off == 0 || off > out || len > (int64_t)want - out) return -1;
        for (int64_t i = 0; i < len; i++) dst[out + i] = dst[out - off + i];
        out += len;
    }
    return out == (int64_t)want ? out : -1;
}

/* INTEGER/BIGINT/SMALLINT `col IN (set)`: keep[r] &= the row is not NULL and
 * its int64 value is a member (SimplePredicate::int_in_form,
 * physical_planner.cpp:126-133, 409-418: sorted set, binary search). */
static int or_cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return x < y ? -1 : (x > y);
}

void or_filter_in(int64_t n, int32_t type, const void *data, const uint8_t *nul, const int64_t *set, int64_t nset,
                  uint8_t *keep) {
    int64_t *s = (int64_t *)malloc((size_t)(nset > 0 ? nset : 1) * 8);
    if (nset > 0) memcpy(s, set, (size_t)nset * 8);
    qsort(s, (size_t)nset, 8, or_cmp_i64);
    for (int64_t r = 0; r < n; r++) {
        if (!keep[r]) continue;
        if (nul && nul[r]) { keep[r] = 0; continue; }
        int64_t v = read_int(type, data, r);
        keep[r] = nset > 0 && bsearch(&v, s, (size_t)nset, 8, or_cmp_i64) != NULL;
    }
    free(s);
}

/* VARCHAR predicates (SimplePredicate::str_form / like_contains,
 * physical_planner.cpp:419-462): op 7 `= lit`, 8 `<> lit` (length and bytes
 * equal), 9 `LIKE '%lit%'`, 10 `NOT LIKE '%lit%'` (byte substring, an empty
 * needle matches).  A NULL row never passes. */
void or_filter_str(int64_t n, const int64_t *offs, const uint8_t *bytes, const uint8_t *nul, int32_t op,
                   const uint8_t *lit, int64_t len, uint8_t *keep) {
    for (int64_t r = 0; r < n; r++) {
        if (!keep[r]) continue;
        if (nul && nul[r]) { keep[r] = 0; continue; }
        const uint8_t *p = bytes + offs[r];
        const int64_t sl = offs[r + 1] - offs[r];
        int match;
        if (op == 7 || op == 8) {
            int eq = sl == len && (len == 0 || memcmp(p, lit, (size_t)len) == 0);
            match = op == 7 ? eq : !eq;
        } else {
            int found = len == 0;
            for (int64_t i = 0; !found && i + len <= sl; i++) found = memcmp(p + i, lit, (size_t)len) == 0;
            match = op == 9 ? found : !found;
        }
        keep[r] = (uint8_t)match;
    }
}

int32_t or_version(void) { return 2; }
