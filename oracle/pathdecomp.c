/*
 * pathdecomp.c -- CPU oracle for two-terminal reliability by path
 * decomposition (see oracle.h for the reference lines each part restates).
 *
 * TEST INFRASTRUCTURE ONLY: the checker and the timed CPU port.  The product
 * never links it.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------ */
/* exact sums: 192-bit unsigned fixed point, value = A / 2^190            */
/* (the same number format as the engine's device sums; any order of the */
/* additions gives the same integer, so results compare bit for bit)     */
/* ------------------------------------------------------------------ */
#define FIX_FRAC 190
typedef struct { uint64_t w[3]; } ksum;

static inline ksum fix_of(double m)
{
    ksum r = {{0, 0, 0}};
    uint64_t bits;
    memcpy(&bits, &m, 8);
    int ex = (int)((bits >> 52) & 0x7ff);
    uint64_t M = bits & 0xfffffffffffffull;
    int e;
    if (ex == 0) e = -1074;
    else { M |= 1ull << 52; e = ex - 1075; }
    if (!M) return r;
    int s = e + FIX_FRAC;
    if (s >= 0) {
        int k = s >> 6, b = s & 63;
        uint64_t lo = M << b, hi = b ? (M >> (64 - b)) : 0;
        r.w[k] = lo;
        if (k + 1 < 3) r.w[k + 1] = hi;
    } else if (-s < 64) {
        r.w[0] = M >> (-s);
    }
    return r;
}
static inline void ks_merge(ksum *a, const ksum *b)
{
    unsigned __int128 c = 0;
    for (int i = 0; i < 3; i++) {
        c += (unsigned __int128)a->w[i] + b->w[i];
        a->w[i] = (uint64_t)c;
        c >>= 64;
    }
}
static inline void ks_sub(ksum *a, const ksum *b)
{
    uint64_t borrow = 0;
    for (int i = 0; i < 3; i++) {
        uint64_t x = a->w[i], y = b->w[i];
        uint64_t d = x - y - borrow;
        borrow = (x < y) || (x - y < borrow);
        a->w[i] = d;
    }
}
static inline void ks_add(ksum *s, double x)
{
    if (x < 0) { ksum t = fix_of(-x); ks_sub(s, &t); }
    else { ksum t = fix_of(x); ks_merge(s, &t); }
}
static inline int ks_le(const ksum *a, const ksum *b)
{
    for (int i = 2; i >= 0; i--) if (a->w[i] != b->w[i]) return a->w[i] < b->w[i];
    return 1;
}
/* round to nearest, ties to even */
static double ks_val(const ksum *a)
{
    int i = 2;
    while (i >= 0 && a->w[i] == 0) i--;
    if (i < 0) return 0.0;
    int t = 64 * i + 63 - __builtin_clzll(a->w[i]);
    uint64_t x;
    int sticky = 0;
    if (t >= 63) {
        int lo = t - 63, k = lo >> 6, b = lo & 63;
        x = a->w[k] >> b;
        if (b && k + 1 < 3) x |= a->w[k + 1] << (64 - b);
        if (b) sticky = (a->w[k] & ((1ull << b) - 1)) != 0;
        for (int j = 0; j < k; j++) sticky |= a->w[j] != 0;
    } else {
        x = a->w[0] << (63 - t);
    }
    uint64_t mant = x >> 11, rem = x & 0x7ff;
    if (rem > 0x400 || (rem == 0x400 && (sticky || (mant & 1)))) {
        mant++;
        if (mant >> 53) { mant >>= 1; t++; }
    }
    return ldexp((double)mant, t - 52 - FIX_FRAC);
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ------------------------------------------------------------------ */
/* graph file parser: workingPad/graph.h:46-145, seq/GraphRP.h:82-148  */
/* ------------------------------------------------------------------ */
typedef struct { const char *p, *end; } tok_t;

static int tok_skip(tok_t *t)
{
    while (t->p < t->end && (*t->p == ' ' || *t->p == '\t' || *t->p == '\n' || *t->p == '\r'))
        t->p++;
    return t->p < t->end;
}
static int tok_long(tok_t *t, long *out)
{
    if (!tok_skip(t)) return -1;
    char *e;
    long v = strtol(t->p, &e, 10);
    if (e == t->p) return -1;
    t->p = e;
    *out = v;
    return 0;
}
static int tok_double(tok_t *t, double *out)
{
    if (!tok_skip(t)) return -1;
    char *e;
    double v = strtod(t->p, &e);
    if (e == t->p) return -1;
    t->p = e;
    *out = v;
    return 0;
}

void og_free_graph(og_graph *g)
{
    free((void *)g->row_ptr); free((void *)g->col_idx);
    free((void *)g->edge_id); free((void *)g->edge_p);
    memset(g, 0, sizeof(*g));
}

int og_load(const char *path, og_graph *g)
{
    memset(g, 0, sizeof(*g));
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *buf = (char *)malloc(sz + 1);
    if (!buf) { fclose(f); return -2; }
    if (fread(buf, 1, sz, f) != (size_t)sz) { fclose(f); free(buf); return -1; }
    fclose(f);
    buf[sz] = 0;

    tok_t t = { buf, buf + sz };
    long n, efile;
    if (tok_long(&t, &n) || tok_long(&t, &efile) || n <= 0) { free(buf); return -3; }
    /* optional graph type character (U/D); files without one start the lists */
    tok_skip(&t);
    int directed = 0;
    if (t.p < t.end && ((*t.p >= 'A' && *t.p <= 'Z') || (*t.p >= 'a' && *t.p <= 'z'))) {
        directed = (*t.p == 'D' || *t.p == 'd');
        t.p++;
    }

    int32_t *row = (int32_t *)calloc(n + 1, sizeof(int32_t));
    size_t cap = 64, na = 0;
    int32_t *col = (int32_t *)malloc(cap * sizeof(int32_t));
    double *ap = (double *)malloc(cap * sizeof(double));
    for (long u = 0; u < n; u++) {
        long deg;
        if (tok_long(&t, &deg) || deg < 0) goto bad;
        for (long j = 0; j < deg; j++) {
            long v; double p;
            if (tok_long(&t, &v) || tok_double(&t, &p) || v < 0 || v >= n) goto bad;
            if (na == cap) {
                cap *= 2;
                col = (int32_t *)realloc(col, cap * sizeof(int32_t));
                ap = (double *)realloc(ap, cap * sizeof(double));
            }
            col[na] = (int32_t)v; ap[na] = p; na++;
        }
        row[u + 1] = (int32_t)na;
    }
    free(buf);

    /* edge ids: first-seen (min,max) pair scanning nodes in order (graph.h:77-90);
     * a directed graph gives every arc its own id in file order (seq/GraphRP.h:131-145) */
    int32_t *eid = (int32_t *)malloc((na ? na : 1) * sizeof(int32_t));
    double *ep = (double *)malloc((na ? na : 1) * sizeof(double));
    if (directed) {
        for (size_t j = 0; j < na; j++) { eid[j] = (int32_t)j; ep[j] = ap[j]; }
        free(ap);
        g->n_nodes = (int32_t)n; g->n_edges = (int32_t)na; g->n_arcs = (int32_t)na;
        g->row_ptr = row; g->col_idx = col; g->edge_id = eid; g->edge_p = ep;
        return 0;
    }
    /* pair -> id via an open-addressing table keyed on (a,b) */
    size_t hcap = 16;
    while (hcap < 2 * na + 16) hcap <<= 1;
    int64_t *hkey = (int64_t *)malloc(hcap * sizeof(int64_t));
    int32_t *hval = (int32_t *)malloc(hcap * sizeof(int32_t));
    for (size_t i = 0; i < hcap; i++) hkey[i] = -1;
    int32_t ne = 0;
    for (long u = 0; u < n; u++) {
        for (int32_t j = row[u]; j < row[u + 1]; j++) {
            int64_t a = u < col[j] ? u : col[j], b = u < col[j] ? col[j] : u;
            int64_t key = a * n + b;
            size_t h = (size_t)((uint64_t)key * 0x9E3779B97F4A7C15ull) & (hcap - 1);
            while (hkey[h] != -1 && hkey[h] != key) h = (h + 1) & (hcap - 1);
            if (hkey[h] == -1) { hkey[h] = key; hval[h] = ne; ep[ne] = ap[j]; ne++; }
            eid[j] = hval[h];
        }
    }
    free(hkey); free(hval); free(ap);
    g->n_nodes = (int32_t)n;
    g->n_edges = ne;
    g->n_arcs = (int32_t)na;
    g->row_ptr = row; g->col_idx = col; g->edge_id = eid; g->edge_p = ep;
    return 0;
bad:
    free(buf); free(row); free(col); free(ap);
    return -4;
}

/* ------------------------------------------------------------------ */
/* masks: 2 bits per edge, 00 down, 01 up, 11 unknown (common.h:22-24) */
/* ------------------------------------------------------------------ */
static inline int st_get(const uint32_t *m, int e) { return (m[e >> 4] >> ((e & 15) * 2)) & 3; }
static inline int notdown(const uint32_t *m, int e) { return (m[e >> 4] >> ((e & 15) * 2)) & 1; }
static inline void set_up(uint32_t *m, int e) { m[e >> 4] &= ~(2u << ((e & 15) * 2)); }
static inline void set_down(uint32_t *m, int e) { m[e >> 4] &= ~(3u << ((e & 15) * 2)); }

int og_bucket(double mass, int shift, int nb)
{
    if (shift < 0 || nb <= 1) return 0;
    uint64_t bits;
    memcpy(&bits, &mass, 8);
    int64_t key = (int64_t)(bits >> (52 - shift));   /* (biased exponent << shift) | top mantissa bits */
    int64_t b = ((int64_t)1023 << shift) - key;
    if (b < 0) b = 0;
    if (b > nb - 1) b = nb - 1;
    return (int)b;
}

void og_default_opts(og_opts *o)
{
    memset(o, 0, sizeof(*o));
    o->bfs_rule = OG_BFS_LEVEL;
    o->order = OG_ORDER_WAVES;
    o->bucket_shift = -1;
    o->n_buckets = 1;
    o->threads = 1;
}

/* ------------------------------------------------------------------ */
/* per-thread expansion context                                         */
/* ------------------------------------------------------------------ */
typedef struct {
    const og_graph *g;
    const double *q;
    int src, dst, W, rule, precheck, branching, border;
    int nk;                     /* K-terminal: terminals other than src (0: two-terminal) */
    uint8_t *isterm;            /* [n] */
    int32_t *order;             /* [n] BFS order of the last K-terminal search */
    uint8_t *mark;              /* [n] */
    double eps;
    /* BFS scratch */
    uint32_t gen;
    uint32_t *vis;
    int32_t *par_e, *par_v, *cur, *nxt, *path;
    uint32_t *work, *child;
    /* results */
    ksum R, esp_trunc, esp_spill;
    uint64_t nodes, leaves, dead, truncated, spilled, pruned, pushes;
} xctx;

static void x_init(xctx *x, const og_graph *g, const double *q, int src, int dst, const og_opts *o)
{
    memset(x, 0, sizeof(*x));
    int n = g->n_nodes;
    x->g = g; x->q = q; x->src = src; x->dst = dst;
    x->W = (g->n_edges * 2 + 31) / 32;
    if (x->W < 1) x->W = 1;
    x->rule = o->bfs_rule; x->precheck = o->precheck; x->eps = o->eps; x->branching = o->branching;
    x->border = o->branch_order;
    x->isterm = (uint8_t *)calloc(n, 1);
    x->order = (int32_t *)malloc((n + 1) * sizeof(int32_t));
    x->mark = (uint8_t *)calloc(n, 1);
    if (o->n_terminals > 0 && o->terminals) {
        for (int i = 0; i < o->n_terminals; i++) {
            int t = o->terminals[i];
            if (t != src && t >= 0 && t < n && !x->isterm[t]) { x->isterm[t] = 1; x->nk++; }
        }
    }
    x->vis = (uint32_t *)calloc(n, sizeof(uint32_t));
    x->par_e = (int32_t *)malloc(n * sizeof(int32_t));
    x->par_v = (int32_t *)malloc(n * sizeof(int32_t));
    x->cur = (int32_t *)malloc((n + 1) * sizeof(int32_t));
    x->nxt = (int32_t *)malloc((n + 1) * sizeof(int32_t));
    x->path = (int32_t *)malloc((n + 1) * sizeof(int32_t));
    x->work = (uint32_t *)malloc(x->W * sizeof(uint32_t));
    x->child = (uint32_t *)malloc(x->W * sizeof(uint32_t));
}

static void x_free(xctx *x)
{
    free(x->isterm); free(x->order); free(x->mark);
    free(x->vis); free(x->par_e); free(x->par_v); free(x->cur); free(x->nxt);
    free(x->path); free(x->work); free(x->child);
}

static void sort_small(int32_t *a, int n)
{
    for (int i = 1; i < n; i++) {
        int32_t v = a[i];
        int j = i - 1;
        while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; j--; }
        a[j + 1] = v;
    }
}

/* src->dst search over not-down arcs. With want_path, fills par_e/par_v.
 * Level rule: frontier scanned in ascending node order (device_code.cuh:141-174
 * with one lane per word), so the parent is the smallest frontier node.
 * FIFO rule: seq/seq.cpp:311-351. Both stop when dst is first discovered,
 * which fixes parent[dst] the same way as finishing the level would. */
static int x_bfs_states(xctx *x, const uint32_t *m, int up_only);
static int x_bfs(xctx *x, const uint32_t *m) { return x_bfs_states(x, m, 0); }

/* arc usable by the search: not down, or (up_only) up */
static inline int usable(const uint32_t *m, int e, int up_only)
{
    return up_only ? st_get(m, e) == 1 : notdown(m, e);
}

static int x_bfs_states(xctx *x, const uint32_t *m, int up_only)
{
    const og_graph *g = x->g;
    int src = x->src, dst = x->dst;
    if (src == dst) return 1;
    if (++x->gen == 0) { memset(x->vis, 0, g->n_nodes * sizeof(uint32_t)); x->gen = 1; }
    uint32_t gen = x->gen;
    x->vis[src] = gen;
    if (x->rule == OG_BFS_FIFO) {
        int head = 0, tail = 0;
        x->cur[tail++] = src;
        while (head < tail) {
            int u = x->cur[head++];
            for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; j++) {
                int v = g->col_idx[j], e = g->edge_id[j];
                if (x->vis[v] != gen && usable(m, e, up_only)) {
                    x->vis[v] = gen; x->par_v[v] = u; x->par_e[v] = e;
                    x->cur[tail++] = v;
                    if (v == dst) return 1;
                }
            }
        }
        return 0;
    }
    int nc = 1;
    x->cur[0] = src;
    while (nc) {
        int nn = 0;
        for (int i = 0; i < nc; i++) {
            int u = x->cur[i];
            for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; j++) {
                int v = g->col_idx[j], e = g->edge_id[j];
                if (x->vis[v] != gen && usable(m, e, up_only)) {
                    x->vis[v] = gen; x->par_v[v] = u; x->par_e[v] = e;
                    x->nxt[nn++] = v;
                    if (v == dst) return 1;
                }
            }
        }
        sort_small(x->nxt, nn);
        int32_t *t = x->cur; x->cur = x->nxt; x->nxt = t;
        nc = nn;
    }
    return 0;
}

/* K-terminal search: level BFS from src over not-down arcs (parent = smallest
 * frontier node, as x_bfs), whole levels, until every terminal is reached; the
 * visit order (src, then each level in ascending node order) goes to x->order.
 * Returns the number of nodes in x->order if all terminals were reached, else 0. */
static int x_bfs_k(xctx *x, const uint32_t *m)
{
    const og_graph *g = x->g;
    int src = x->src;
    if (++x->gen == 0) { memset(x->vis, 0, g->n_nodes * sizeof(uint32_t)); x->gen = 1; }
    uint32_t gen = x->gen;
    x->vis[src] = gen;
    int no = 0, found = 0;
    x->order[no++] = src;
    int nc = 1;
    x->cur[0] = src;
    while (nc && found < x->nk) {
        int nn = 0;
        for (int i = 0; i < nc; i++) {
            int u = x->cur[i];
            for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; j++) {
                int v = g->col_idx[j], e = g->edge_id[j];
                if (x->vis[v] != gen && notdown(m, e)) {
                    x->vis[v] = gen; x->par_v[v] = u; x->par_e[v] = e;
                    x->nxt[nn++] = v;
                    if (x->isterm[v]) found++;
                }
            }
        }
        sort_small(x->nxt, nn);
        for (int i = 0; i < nn; i++) x->order[no++] = x->nxt[i];
        int32_t *t = x->cur; x->cur = x->nxt; x->nxt = t;
        nc = nn;
    }
    return found == x->nk ? no : 0;
}

/* child sink: returns 0 if stored, 1 if it overflowed (counted by caller) */
typedef int (*sink_fn)(void *ud, const uint32_t *mask, double mass);

/* Expand one popped subproblem: workingPad/main.cu:504-628 with the sweep of
 * :114-283, FP64 products in path order, src-side hop first. */
/* Fork branching (main.cu:303-430, :550-565): a path of up edges means the
 * subproblem is connected, so its whole mass goes to R; else the optimistic
 * path's UNKNOWN edge with the largest p (ties: nearest dst, as the
 * reference's dst-first scan with a strict comparison keeps) gives two
 * children, that edge down (mass x q) and up (mass x p), queued in that order. */
static void x_fork(xctx *x, const uint32_t *m, double mass, sink_fn sink, void *ud)
{
    if (x_bfs_states(x, m, 1)) {
        x->leaves++;
        ks_add(&x->R, mass);
        return;
    }
    if (!x_bfs(x, m)) { x->dead++; return; }
    const double *p = x->g->edge_p;
    int best = -1;
    double bp = -1.0;
    for (int v = x->dst; v != x->src; v = x->par_v[v]) {      /* dst side first */
        int e = x->par_e[v];
        if (st_get(m, e) == 3 && p[e] > bp) { bp = p[e]; best = e; }
    }
    if (best < 0) {            /* cannot happen: no path of up edges exists */
        x->leaves++;
        ks_add(&x->R, mass);
        return;
    }
    for (int k = 0; k < 2; k++) {
        memcpy(x->child, m, x->W * sizeof(uint32_t));
        double cm;
        if (k == 0) { set_down(x->child, best); cm = mass * x->q[best]; }
        else { set_up(x->child, best); cm = mass * p[best]; }
        if (sink(ud, x->child, cm)) {
            x->spilled++;
            ks_add(&x->esp_spill, cm);
        } else {
            x->pushes++;
        }
    }
}

static void x_expand(xctx *x, const uint32_t *m, double mass, sink_fn sink, void *ud)
{
    x->nodes++;
    if (x->eps > 0 && mass < x->eps) {            /* main.cu:537-543 */
        x->truncated++;
        ks_add(&x->esp_trunc, mass);
        return;
    }
    if (x->branching == OG_BRANCH_FORK) { x_fork(x, m, mass, sink, ud); return; }
    int L = 0;
    if (x->nk) {
        /* K-terminal: the tree joining every terminal to src, its edges in BFS order */
        int no = x_bfs_k(x, m);
        if (!no) { x->dead++; return; }
        for (int i = 0; i < no; i++) x->mark[x->order[i]] = 0;
        for (int i = 1; i < no; i++) {
            int t = x->order[i];
            if (!x->isterm[t]) continue;
            for (int v = t; v != x->src && !x->mark[v]; v = x->par_v[v]) x->mark[v] = 1;
        }
        for (int i = 1; i < no; i++)
            if (x->mark[x->order[i]]) x->path[L++] = x->par_e[x->order[i]];
    } else {
        if (!x_bfs(x, m)) { x->dead++; return; }
        /* path hops in src -> dst order (the reference's branching order) */
        for (int v = x->dst; v != x->src; v = x->par_v[v]) x->path[L++] = x->par_e[v];
        if (x->border != OG_BORDER_DST)
            for (int i = 0, j = L - 1; i < j; i++, j--) { int32_t t = x->path[i]; x->path[i] = x->path[j]; x->path[j] = t; }
        if (x->border == OG_BORDER_P_ASC || x->border == OG_BORDER_P_DESC) {
            const double *pp = x->g->edge_p;      /* stable insertion sort of the hops by p */
            const int desc = x->border == OG_BORDER_P_DESC;
            for (int i = 1; i < L; i++) {
                int32_t e = x->path[i];
                int j = i - 1;
                while (j >= 0 && (desc ? pp[x->path[j]] < pp[e] : pp[x->path[j]] > pp[e])) { x->path[j + 1] = x->path[j]; j--; }
                x->path[j + 1] = e;
            }
        }
    }
    const double *p = x->g->edge_p;
    memcpy(x->work, m, x->W * sizeof(uint32_t));
    double P = mass;
    for (int h = 0; h < L; h++) {
        int e = x->path[h];
        if (st_get(m, e) != 3) continue;          /* only UNKNOWN hops branch */
        memcpy(x->child, x->work, x->W * sizeof(uint32_t));
        set_down(x->child, e);
        double cm = P * x->q[e];
        int keep = 1;
        if (x->precheck) {                        /* seq/seq.cpp:551 */
            if (!x_bfs(x, x->child)) { keep = 0; x->pruned++; }
        }
        if (keep) {
            if (sink(ud, x->child, cm)) {         /* overflow: main.cu:245-252 */
                x->spilled++;
                ks_add(&x->esp_spill, cm);
            } else {
                x->pushes++;
            }
        }
        set_up(x->work, e);
        P = P * p[e];
    }
    x->leaves++;                                  /* all-up leaf: main.cu:254-263 */
    ks_add(&x->R, P);
}

/* ------------------------------------------------------------------ */
/* item storage: records of W words + one double                        */
/* ------------------------------------------------------------------ */
typedef struct {
    uint32_t *d;      /* n * rec words */
    size_t n, cap;    /* cap counts words: a batch arena reuses one vector for records of any width */
    ksum mass;
} ivec;

static int iv_push(ivec *v, const uint32_t *m, double mass, int W)
{
    const size_t rec = (size_t)W + 2;
    if ((v->n + 1) * rec > v->cap) {
        size_t nc = v->cap ? v->cap * 2 : 256 * rec;
        while (nc < (v->n + 1) * rec) nc *= 2;
        uint32_t *nd = (uint32_t *)realloc(v->d, nc * sizeof(uint32_t));
        if (!nd) return -1;
        v->d = nd; v->cap = nc;
    }
    uint32_t *r = v->d + v->n * rec;
    memcpy(r, m, W * sizeof(uint32_t));
    memcpy(r + W, &mass, sizeof(double));
    v->n++;
    ks_add(&v->mass, mass);
    return 0;
}
static inline const uint32_t *iv_rec(const ivec *v, size_t i, int W) { return v->d + i * (W + 2); }
static inline double iv_mass(const ivec *v, size_t i, int W)
{
    double m;
    memcpy(&m, v->d + i * (W + 2) + W, sizeof(double));
    return m;
}

/* ------------------------------------------------------------------ */
/* wave schedule (the engine's bucketed device queue, restated)         */
/* ------------------------------------------------------------------ */
typedef struct wshared wshared;
typedef struct {
    xctx x;
    wshared *sh;
    ivec *out;        /* per-bucket outputs of this thread */
    int tid;
} wthread;

struct wshared {
    const ivec *wave;
    atomic_size_t next;
    atomic_uint_fast64_t queued;
    uint64_t capacity;
    int W, shift, nb, nthreads;
    wthread *th;
    pthread_barrier_t bar_start, bar_end;
    int quit;
};

typedef struct { wthread *t; } wsink_ud;

static int wave_sink(void *ud, const uint32_t *mask, double mass)
{
    wthread *t = (wthread *)ud;
    wshared *s = t->sh;
    if (s->capacity) {
        uint64_t q = atomic_fetch_add(&s->queued, 1);
        if (q >= s->capacity) { atomic_fetch_sub(&s->queued, 1); return 1; }
    } else {
        atomic_fetch_add(&s->queued, 1);
    }
    int b = og_bucket(mass, s->shift, s->nb);
    if (iv_push(&t->out[b], mask, mass, s->W)) { atomic_fetch_sub(&s->queued, 1); return 1; }
    return 0;
}

static void wave_work(wthread *t)
{
    wshared *s = t->sh;
    const ivec *w = s->wave;
    const size_t chunk = 64;
    for (;;) {
        size_t i0 = atomic_fetch_add(&s->next, chunk);
        if (i0 >= w->n) break;
        size_t i1 = i0 + chunk < w->n ? i0 + chunk : w->n;
        for (size_t i = i0; i < i1; i++)
            x_expand(&t->x, iv_rec(w, i, s->W), iv_mass(w, i, s->W), wave_sink, t);
    }
}

static void *wave_thread(void *arg)
{
    wthread *t = (wthread *)arg;
    wshared *s = t->sh;
    for (;;) {
        pthread_barrier_wait(&s->bar_start);
        if (s->quit) break;
        wave_work(t);
        pthread_barrier_wait(&s->bar_end);
    }
    return NULL;
}

static uint64_t total_nodes(wshared *s)
{
    uint64_t n = 0;
    for (int i = 0; i < s->nthreads; i++) n += s->th[i].x.nodes;
    return n;
}

static int run_waves(const og_graph *g, int src, int dst, const og_opts *o, const double *q,
                     const uint32_t *root, og_result *r)
{
    int W = (g->n_edges * 2 + 31) / 32;
    if (W < 1) W = 1;
    int nb = (o->bucket_shift < 0) ? 1 : (o->n_buckets > 0 ? o->n_buckets : 1);
    int T = o->threads > 0 ? o->threads : 1;
    ivec *bk = (ivec *)calloc(nb, sizeof(ivec));
    wshared s;
    memset(&s, 0, sizeof(s));
    s.capacity = o->capacity; s.W = W; s.shift = o->bucket_shift; s.nb = nb; s.nthreads = T;
    atomic_init(&s.next, 0);
    atomic_init(&s.queued, 0);
    s.th = (wthread *)calloc(T, sizeof(wthread));
    for (int i = 0; i < T; i++) {
        x_init(&s.th[i].x, g, q, src, dst, o);
        s.th[i].sh = &s; s.th[i].tid = i;
        s.th[i].out = (ivec *)calloc(nb, sizeof(ivec));
    }
    iv_push(&bk[og_bucket(1.0, s.shift, nb)], root, 1.0, W);
    atomic_store(&s.queued, 1);
    pthread_t *tids = NULL;
    if (T > 1) {
        pthread_barrier_init(&s.bar_start, NULL, T);
        pthread_barrier_init(&s.bar_end, NULL, T);
        tids = (pthread_t *)calloc(T, sizeof(pthread_t));
        for (int i = 1; i < T; i++) pthread_create(&tids[i], NULL, wave_thread, &s.th[i]);
    }
    int status = 0;
    uint64_t waves = 0, max_wave = 0, max_q = 1;
    ivec cur;
    memset(&cur, 0, sizeof(cur));
    for (;;) {
        int b = -1;
        for (int i = 0; i < nb; i++) if (bk[i].n) { b = i; break; }
        if (b < 0) break;
        /* stop test between waves: ESP so far + queued mass */
        if (o->target_width > 0) {
            ksum wdt = {{0, 0, 0}};
            for (int i = 0; i < T; i++) { ks_merge(&wdt, &s.th[i].x.esp_trunc); ks_merge(&wdt, &s.th[i].x.esp_spill); }
            for (int i = 0; i < nb; i++) ks_merge(&wdt, &bk[i].mass);
            ksum tgt = fix_of(o->target_width);
            if (ks_le(&wdt, &tgt)) { status = 1; break; }
        }
        if (o->max_nodes && total_nodes(&s) >= o->max_nodes) { status = 2; break; }
        /* take the whole bucket as this wave */
        ivec t = cur; cur = bk[b]; bk[b] = t; bk[b].n = 0; memset(&bk[b].mass, 0, sizeof(ksum));
        waves++;
        if (cur.n > max_wave) max_wave = cur.n;
        s.wave = &cur;
        atomic_store(&s.next, 0);
        if (T > 1) {
            pthread_barrier_wait(&s.bar_start);
            wave_work(&s.th[0]);
            pthread_barrier_wait(&s.bar_end);
        } else {
            wave_work(&s.th[0]);
        }
        atomic_fetch_sub(&s.queued, cur.n);
        /* merge per-thread outputs (thread order) */
        for (int i = 0; i < T; i++) {
            for (int k = 0; k < nb; k++) {
                ivec *src_v = &s.th[i].out[k];
                if (!src_v->n) continue;
                for (size_t j = 0; j < src_v->n; j++) {
                    const uint32_t *rr = iv_rec(src_v, j, W);
                    double mm;
                    memcpy(&mm, rr + W, sizeof(double));
                    iv_push(&bk[k], rr, mm, W);
                }
                src_v->n = 0; memset(&src_v->mass, 0, sizeof(ksum));
            }
        }
        uint64_t qn = atomic_load(&s.queued);
        if (qn > max_q) max_q = qn;
    }
    if (T > 1) {
        s.quit = 1;
        pthread_barrier_wait(&s.bar_start);
        for (int i = 1; i < T; i++) pthread_join(tids[i], NULL);
        pthread_barrier_destroy(&s.bar_start);
        pthread_barrier_destroy(&s.bar_end);
        free(tids);
    }
    ksum R = {{0, 0, 0}}, et = {{0, 0, 0}}, es = {{0, 0, 0}}, qm = {{0, 0, 0}};
    uint64_t queued = 0;
    for (int i = 0; i < nb; i++) { ks_merge(&qm, &bk[i].mass); queued += bk[i].n; free(bk[i].d); }
    for (int i = 0; i < T; i++) {
        xctx *x = &s.th[i].x;
        ks_merge(&R, &x->R); ks_merge(&et, &x->esp_trunc); ks_merge(&es, &x->esp_spill);
        r->nodes += x->nodes; r->leaves += x->leaves; r->dead += x->dead;
        r->truncated += x->truncated; r->spilled += x->spilled; r->pruned += x->pruned;
        r->pushes += x->pushes;
        for (int k = 0; k < nb; k++) free(s.th[i].out[k].d);
        free(s.th[i].out);
        x_free(x);
    }
    free(s.th); free(bk); free(cur.d);
    r->R = ks_val(&R);
    r->esp_truncated = ks_val(&et);
    r->esp_spilled = ks_val(&es);
    r->queued_mass = ks_val(&qm);
    ksum e = et; ks_merge(&e, &es); ks_merge(&e, &qm);
    r->esp = ks_val(&e);
    r->queued = queued;
    r->waves = waves; r->max_wave = max_wave; r->max_queued = max_q;
    r->status = status;
    return 0;
}

/* ------------------------------------------------------------------ */
/* max-mass binary heap (seq/seq.cpp:49-197) and DFS stack               */
/* ------------------------------------------------------------------ */
typedef struct {
    uint32_t *d;
    double *key;
    size_t n, cap;
    int W;
    uint64_t capacity;
    int heap;
    ksum mass;
} hq;

static void hq_swap(hq *h, size_t a, size_t b)
{
    int W = h->W;
    uint32_t tmp[64];
    uint32_t *big = W > 64 ? (uint32_t *)malloc(W * sizeof(uint32_t)) : tmp;
    memcpy(big, h->d + a * W, W * 4); memcpy(h->d + a * W, h->d + b * W, W * 4); memcpy(h->d + b * W, big, W * 4);
    if (big != tmp) free(big);
    double k = h->key[a]; h->key[a] = h->key[b]; h->key[b] = k;
}

static int hq_sink(void *ud, const uint32_t *m, double mass)
{
    hq *h = (hq *)ud;
    if (h->capacity && h->n >= h->capacity) return 1;
    if (h->n == h->cap) {
        size_t nc = h->cap ? h->cap * 2 : 1024;
        h->d = (uint32_t *)realloc(h->d, nc * h->W * sizeof(uint32_t));
        h->key = (double *)realloc(h->key, nc * sizeof(double));
        h->cap = nc;
    }
    memcpy(h->d + h->n * h->W, m, h->W * 4);
    h->key[h->n] = mass;
    size_t i = h->n++;
    ks_add(&h->mass, mass);
    if (h->heap) {
        while (i > 0) {
            size_t pa = (i - 1) / 2;
            if (h->key[pa] >= h->key[i]) break;
            hq_swap(h, pa, i);
            i = pa;
        }
    }
    return 0;
}

static double hq_pop(hq *h, uint32_t *out)
{
    double k;
    if (!h->heap) {                               /* stack */
        h->n--;
        memcpy(out, h->d + h->n * h->W, h->W * 4);
        k = h->key[h->n];
    } else {
        memcpy(out, h->d, h->W * 4);
        k = h->key[0];
        h->n--;
        if (h->n) {
            hq_swap(h, 0, h->n);
            size_t i = 0;
            for (;;) {
                size_t l = 2 * i + 1, rr = l + 1, lg = i;
                if (l < h->n && h->key[l] > h->key[lg]) lg = l;
                if (rr < h->n && h->key[rr] > h->key[lg]) lg = rr;
                if (lg == i) break;
                hq_swap(h, i, lg);
                i = lg;
            }
        }
    }
    ks_add(&h->mass, -k);
    return k;
}

static int run_serial(const og_graph *g, int src, int dst, const og_opts *o, const double *q,
                      const uint32_t *root, og_result *r)
{
    xctx x;
    x_init(&x, g, q, src, dst, o);
    hq h;
    memset(&h, 0, sizeof(h));
    h.W = x.W; h.capacity = o->capacity; h.heap = (o->order == OG_ORDER_HEAP);
    hq_sink(&h, root, 1.0);
    uint32_t *m = (uint32_t *)malloc(x.W * sizeof(uint32_t));
    uint64_t max_q = 1;
    int status = 0;
    /* queued mass is tracked exactly by recomputation when the target is tested */
    while (h.n) {
        if (o->target_width > 0 && h.heap) {
            ksum w = x.esp_trunc; ks_merge(&w, &x.esp_spill);
            ks_merge(&w, &h.mass);
            ksum tgt = fix_of(o->target_width);
            if (ks_le(&w, &tgt)) { status = 1; break; }
        }
        if (o->max_nodes && x.nodes >= o->max_nodes) { status = 2; break; }
        double mass = hq_pop(&h, m);
        x_expand(&x, m, mass, hq_sink, &h);
        if (h.n > max_q) max_q = h.n;
    }
    ksum qm = {{0, 0, 0}};
    for (size_t i = 0; i < h.n; i++) ks_add(&qm, h.key[i]);
    r->R = ks_val(&x.R);
    r->esp_truncated = ks_val(&x.esp_trunc);
    r->esp_spilled = ks_val(&x.esp_spill);
    r->queued_mass = ks_val(&qm);
    ksum e = x.esp_trunc; ks_merge(&e, &x.esp_spill); ks_merge(&e, &qm);
    r->esp = ks_val(&e);
    r->nodes = x.nodes; r->leaves = x.leaves; r->dead = x.dead; r->truncated = x.truncated;
    r->spilled = x.spilled; r->pruned = x.pruned; r->pushes = x.pushes;
    r->queued = h.n; r->max_queued = max_q; r->status = status;
    free(m); free(h.d); free(h.key);
    x_free(&x);
    return 0;
}

/* ------------------------------------------------------------------ */
/* single-thread wave schedule with reusable storage (batches)           */
/* ------------------------------------------------------------------ */
typedef struct og_arena {
    xctx x;
    int n_cap, w_cap, e_cap, nb_cap;
    ivec *bk;
    ivec cur;
    double *q;
    uint32_t *root;
} og_arena;

static void arena_free(og_arena *a)
{
    if (a->n_cap) x_free(&a->x);
    for (int i = 0; i < a->nb_cap; i++) free(a->bk[i].d);
    free(a->bk); free(a->cur.d); free(a->q); free(a->root);
    memset(a, 0, sizeof(*a));
}

static void arena_fit(og_arena *a, const og_graph *g, int src, int dst, const og_opts *o, int nb)
{
    int W = (g->n_edges * 2 + 31) / 32;
    if (W < 1) W = 1;
    if (g->n_nodes > a->n_cap || W > a->w_cap) {
        if (a->n_cap) x_free(&a->x);
        og_graph big = *g;
        og_opts oo = *o;
        big.n_nodes = g->n_nodes > a->n_cap ? g->n_nodes : a->n_cap;
        x_init(&a->x, &big, NULL, src, dst, &oo);
        free(a->x.work); free(a->x.child);
        int wc = W > a->w_cap ? W : a->w_cap;
        a->x.work = (uint32_t *)malloc(wc * sizeof(uint32_t));
        a->x.child = (uint32_t *)malloc(wc * sizeof(uint32_t));
        a->n_cap = big.n_nodes;
        a->w_cap = wc;
    }
    if (g->n_edges > a->e_cap) {
        free(a->q); free(a->root);
        a->e_cap = g->n_edges;
        a->q = (double *)malloc((size_t)(a->e_cap > 0 ? a->e_cap : 1) * sizeof(double));
        a->root = (uint32_t *)malloc((size_t)(a->w_cap > W ? a->w_cap : W) * sizeof(uint32_t));
    }
    if (nb > a->nb_cap) {
        a->bk = (ivec *)realloc(a->bk, nb * sizeof(ivec));
        memset(a->bk + a->nb_cap, 0, (nb - a->nb_cap) * sizeof(ivec));
        a->nb_cap = nb;
    }
    /* point the context at this graph; scratch arrays are reused */
    xctx *x = &a->x;
    x->g = g; x->q = a->q; x->src = src; x->dst = dst; x->W = W;
    x->rule = o->bfs_rule; x->precheck = o->precheck; x->eps = o->eps; x->border = o->branch_order;
    x->gen = 0;
    memset(x->vis, 0, a->n_cap * sizeof(uint32_t));
    memset(&x->R, 0, sizeof(ksum)); memset(&x->esp_trunc, 0, sizeof(ksum)); memset(&x->esp_spill, 0, sizeof(ksum));
    x->nodes = x->leaves = x->dead = x->truncated = x->spilled = x->pruned = x->pushes = 0;
}

typedef struct { ivec *bk; int W, shift, nb; uint64_t capacity, queued; } st_sink;

static int st_sink_fn(void *ud, const uint32_t *mask, double mass)
{
    st_sink *s = (st_sink *)ud;
    if (s->capacity && s->queued >= s->capacity) return 1;
    int b = og_bucket(mass, s->shift, s->nb);
    if (iv_push(&s->bk[b], mask, mass, s->W)) return 1;
    s->queued++;
    return 0;
}

/* Same schedule as run_waves with one thread: children go straight into
 * their buckets (the running wave was swapped out first). */
static int run_waves_arena(og_arena *a, const og_graph *g, int src, int dst, const og_opts *o, og_result *r)
{
    int nb = (o->bucket_shift < 0) ? 1 : (o->n_buckets > 0 ? o->n_buckets : 1);
    arena_fit(a, g, src, dst, o, nb);
    xctx *x = &a->x;
    int W = x->W;
    for (int e = 0; e < g->n_edges; e++) a->q[e] = 1.0 - g->edge_p[e];
    memset(a->root, 0, W * sizeof(uint32_t));
    for (int e = 0; e < g->n_edges; e++) {
        double p = g->edge_p[e];
        if (p <= 0.0) { }
        else if (p >= 1.0) a->root[e >> 4] |= 1u << ((e & 15) * 2);
        else a->root[e >> 4] |= 3u << ((e & 15) * 2);
    }
    for (int i = 0; i < nb; i++) { a->bk[i].n = 0; memset(&a->bk[i].mass, 0, sizeof(ksum)); }
    st_sink sk = { a->bk, W, o->bucket_shift, nb, o->capacity, 1 };
    iv_push(&a->bk[og_bucket(1.0, o->bucket_shift, nb)], a->root, 1.0, W);
    int status = 0;
    uint64_t waves = 0, max_wave = 0, max_q = 1;
    for (;;) {
        int b = -1;
        for (int i = 0; i < nb; i++) if (a->bk[i].n) { b = i; break; }
        if (b < 0) break;
        if (o->target_width > 0) {
            ksum wdt = x->esp_trunc;
            ks_merge(&wdt, &x->esp_spill);
            for (int i = 0; i < nb; i++) ks_merge(&wdt, &a->bk[i].mass);
            ksum tgt = fix_of(o->target_width);
            if (ks_le(&wdt, &tgt)) { status = 1; break; }
        }
        if (o->max_nodes && x->nodes >= o->max_nodes) { status = 2; break; }
        ivec t = a->cur; a->cur = a->bk[b]; a->bk[b] = t;
        a->bk[b].n = 0; memset(&a->bk[b].mass, 0, sizeof(ksum));
        waves++;
        if (a->cur.n > max_wave) max_wave = a->cur.n;
        for (size_t i = 0; i < a->cur.n; i++) {
            x_expand(x, iv_rec(&a->cur, i, W), iv_mass(&a->cur, i, W), st_sink_fn, &sk);
            sk.queued--;
        }
        if (sk.queued > max_q) max_q = sk.queued;
    }
    ksum qm = {{0, 0, 0}};
    uint64_t queued = 0;
    for (int i = 0; i < nb; i++) { ks_merge(&qm, &a->bk[i].mass); queued += a->bk[i].n; }
    memset(r, 0, sizeof(*r));
    r->R = ks_val(&x->R);
    r->esp_truncated = ks_val(&x->esp_trunc);
    r->esp_spilled = ks_val(&x->esp_spill);
    r->queued_mass = ks_val(&qm);
    ksum e = x->esp_trunc; ks_merge(&e, &x->esp_spill); ks_merge(&e, &qm);
    r->esp = ks_val(&e);
    r->nodes = x->nodes; r->leaves = x->leaves; r->dead = x->dead; r->truncated = x->truncated;
    r->spilled = x->spilled; r->pruned = x->pruned; r->pushes = x->pushes;
    r->queued = queued; r->waves = waves; r->max_wave = max_wave; r->max_queued = max_q;
    r->paths = r->leaves + r->spilled;
    r->status = status;
    return 0;
}

typedef struct {
    int n;
    const og_graph *graphs;
    const int32_t *srcs, *dsts;
    const og_opts *o;
    og_result *res;
    atomic_int next;
} batch_job;

static void *batch_thread(void *arg)
{
    batch_job *j = (batch_job *)arg;
    og_arena a;
    memset(&a, 0, sizeof(a));
    for (;;) {
        int i = atomic_fetch_add(&j->next, 1);
        if (i >= j->n) break;
        const og_graph *g = &j->graphs[i];
        og_result *r = &j->res[i];
        if (g->n_nodes <= 0 || j->srcs[i] < 0 || j->dsts[i] < 0 || j->srcs[i] >= g->n_nodes ||
            j->dsts[i] >= g->n_nodes) {
            memset(r, 0, sizeof(*r));
            r->status = -1;
            continue;
        }
        double t0 = now_s();
        run_waves_arena(&a, g, j->srcs[i], j->dsts[i], j->o, r);
        r->seconds = now_s() - t0;
    }
    arena_free(&a);
    return NULL;
}

int og_run_batch(int n, const og_graph *graphs, const int32_t *srcs, const int32_t *dsts, const og_opts *o,
                 og_result *res, int threads)
{
    if (n < 0 || (n > 0 && (!graphs || !srcs || !dsts || !res))) return -1;
    if (threads < 1) threads = 1;
    batch_job j = { n, graphs, srcs, dsts, o, res, 0 };
    atomic_init(&j.next, 0);
    pthread_t *t = (pthread_t *)calloc(threads, sizeof(pthread_t));
    for (int i = 1; i < threads; i++) pthread_create(&t[i], NULL, batch_thread, &j);
    batch_thread(&j);
    for (int i = 1; i < threads; i++) pthread_join(t[i], NULL);
    free(t);
    return 0;
}

int og_run(const og_graph *g, int src, int dst, const og_opts *o, og_result *r)
{
    memset(r, 0, sizeof(*r));
    if (o->n_terminals > 0) {                     /* K-terminal: src is terminals[0] */
        if (!o->terminals) { r->status = -1; return -1; }
        for (int i = 0; i < o->n_terminals; i++)
            if (o->terminals[i] < 0 || o->terminals[i] >= g->n_nodes) { r->status = -1; return -1; }
        src = o->terminals[0];
        dst = o->terminals[o->n_terminals - 1];
    }
    if (!g || g->n_nodes <= 0 || src < 0 || dst < 0 || src >= g->n_nodes || dst >= g->n_nodes) {
        r->status = -1;
        return -1;
    }
    double t0 = now_s();
    int E = g->n_edges;
    int W = (E * 2 + 31) / 32;
    if (W < 1) W = 1;
    double *q = (double *)malloc((size_t)(E > 0 ? E : 1) * sizeof(double));
    uint32_t *root = (uint32_t *)calloc((size_t)W, sizeof(uint32_t));
    /* initial mask: all UNKNOWN, p<=0 down, p>=1 up (main.cu:717-748) */
    for (int e = 0; e < E; e++) {
        double p = g->edge_p[e];
        q[e] = 1.0 - p;
        if (p <= 0.0) { /* 00 */ }
        else if (p >= 1.0) root[e >> 4] |= 1u << ((e & 15) * 2);
        else root[e >> 4] |= 3u << ((e & 15) * 2);
    }
    int rc;
    if (o->order == OG_ORDER_WAVES && o->threads <= 1 && o->n_terminals <= 0) {
        og_arena a;
        memset(&a, 0, sizeof(a));
        rc = run_waves_arena(&a, g, src, dst, o, r);
        arena_free(&a);
    } else if (o->order == OG_ORDER_WAVES) rc = run_waves(g, src, dst, o, q, root, r);
    else rc = run_serial(g, src, dst, o, q, root, r);
    r->paths = r->leaves + r->spilled;
    r->seconds = now_s() - t0;
    free(q); free(root);
    return rc;
}

/* ------------------------------------------------------------------ */
/* 2^k brute force over the edges with 0 < p < 1                       */
/* ------------------------------------------------------------------ */
static double brute_set(const og_graph *g, int src, uint64_t want);

double og_brute(const og_graph *g, int src, int dst)
{
    int n = g->n_nodes;
    if (n > 64 || src < 0 || dst < 0 || src >= n || dst >= n) return -1.0;
    if (src == dst) return 1.0;
    return brute_set(g, src, 1ull << dst);
}

double og_brute_k(const og_graph *g, const int32_t *terminals, int n_terminals)
{
    int n = g->n_nodes;
    if (n > 64 || n_terminals < 1) return -1.0;
    uint64_t want = 0;
    for (int i = 0; i < n_terminals; i++) {
        if (terminals[i] < 0 || terminals[i] >= n) return -1.0;
        want |= 1ull << terminals[i];
    }
    want &= ~(1ull << terminals[0]);
    if (!want) return 1.0;
    return brute_set(g, terminals[0], want);
}

/* probability that every node of `want` is reachable from src */
static double brute_set(const og_graph *g, int src, uint64_t want)
{
    int n = g->n_nodes, E = g->n_edges;
    int *var = (int *)malloc((E ? E : 1) * sizeof(int));
    int k = 0;
    for (int e = 0; e < E; e++) if (g->edge_p[e] > 0.0 && g->edge_p[e] < 1.0) var[k++] = e;
    if (k > 30) { free(var); return -2.0; }
    /* fixed arcs, and per-variable-edge arc lists */
    uint64_t base[64];
    memset(base, 0, sizeof(base));
    typedef struct { int u, v; } arc;
    arc *arcs = (arc *)malloc((g->n_arcs ? g->n_arcs : 1) * sizeof(arc));
    int *arc_var = (int *)malloc((g->n_arcs ? g->n_arcs : 1) * sizeof(int));
    int *vindex = (int *)malloc((E ? E : 1) * sizeof(int));
    for (int e = 0; e < E; e++) vindex[e] = -1;
    for (int i = 0; i < k; i++) vindex[var[i]] = i;
    int na = 0;
    for (int u = 0; u < n; u++)
        for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; j++) {
            int v = g->col_idx[j], e = g->edge_id[j];
            double p = g->edge_p[e];
            if (vindex[e] < 0) { if (p >= 1.0) base[u] |= 1ull << v; }
            else { arcs[na].u = u; arcs[na].v = v; arc_var[na] = vindex[e]; na++; }
        }
    /* probability tables for low/high halves of the state word */
    int kl = k / 2, kh = k - kl;
    double *tl = (double *)malloc(((size_t)1 << kl) * sizeof(double));
    double *th = (double *)malloc(((size_t)1 << kh) * sizeof(double));
    for (uint64_t s = 0; s < ((uint64_t)1 << kl); s++) {
        double pr = 1.0;
        for (int i = 0; i < kl; i++) { double p = g->edge_p[var[i]]; pr *= ((s >> i) & 1) ? p : 1.0 - p; }
        tl[s] = pr;
    }
    for (uint64_t s = 0; s < ((uint64_t)1 << kh); s++) {
        double pr = 1.0;
        for (int i = 0; i < kh; i++) { double p = g->edge_p[var[kl + i]]; pr *= ((s >> i) & 1) ? p : 1.0 - p; }
        th[s] = pr;
    }
    /* per-variable arc lists */
    int *vstart = (int *)calloc(k + 1, sizeof(int));
    int *vlist = (int *)malloc((na ? na : 1) * sizeof(int));
    for (int i = 0; i < na; i++) vstart[arc_var[i] + 1]++;
    for (int i = 0; i < k; i++) vstart[i + 1] += vstart[i];
    int *fill = (int *)calloc(k, sizeof(int));
    for (int i = 0; i < na; i++) vlist[vstart[arc_var[i]] + fill[arc_var[i]]++] = i;
    uint64_t adj[64];
    memcpy(adj, base, sizeof(adj));
    ksum R = {{0, 0, 0}};
    uint64_t gray = 0;
    uint64_t total = (uint64_t)1 << k;
    for (uint64_t it = 0; it < total; it++) {
        if (it) {
            int b = __builtin_ctzll(it);
            gray ^= 1ull << b;
            int on = (gray >> b) & 1;
            for (int a = vstart[b]; a < vstart[b + 1]; a++) {
                arc *A = &arcs[vlist[a]];
                /* an arc can also be present through another edge id only in multigraphs */
                if (on) adj[A->u] |= 1ull << A->v;
                else adj[A->u] &= ~(1ull << A->v);
            }
        }
        uint64_t reach = 1ull << src, fr = reach;
        while (fr) {
            uint64_t nf = 0;
            uint64_t f = fr;
            while (f) { int u = __builtin_ctzll(f); f &= f - 1; nf |= adj[u]; }
            nf &= ~reach;
            reach |= nf;
            fr = nf;
            if ((reach & want) == want) break;
        }
        if ((reach & want) == want)
            ks_add(&R, tl[gray & (((uint64_t)1 << kl) - 1)] * th[gray >> kl]);
    }
    free(var); free(arcs); free(arc_var); free(vindex); free(tl); free(th);
    free(vstart); free(vlist); free(fill);
    return ks_val(&R);
}

/* ------------------------------------------------------------------ */
/* the ceiling of queue orders (og_order_bound, oracle.h)               */
/* ------------------------------------------------------------------ */
typedef struct { hq *h; double pushed; } gain_sink;

static int gain_sink_fn(void *ud, const uint32_t *m, double mass)
{
    gain_sink *s = (gain_sink *)ud;
    s->pushed += mass;
    return hq_sink(s->h, m, mass);
}

static int cmp_desc(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x < y) - (x > y);
}

int og_order_bound(const og_graph *g, int src, int dst, const og_opts *o_in, uint64_t budget, og_bound *out)
{
    memset(out, 0, sizeof(*out));
    if (!g || g->n_nodes <= 0 || src < 0 || dst < 0 || src >= g->n_nodes || dst >= g->n_nodes) return -1;
    og_opts o = *o_in;
    o.eps = 0; o.capacity = 0; o.max_nodes = 0; o.threads = 1; o.precheck = 0;
    o.branching = OG_BRANCH_PATH; o.n_terminals = 0; o.terminals = NULL;
    if (!(o.target_width > 0)) return -1;
    og_result r;
    o.order = OG_ORDER_HEAP;
    og_run(g, src, dst, &o, &r);
    out->plain_pops = r.nodes;
    o.order = OG_ORDER_WAVES; o.bucket_shift = -1; o.n_buckets = 1;
    og_run(g, src, dst, &o, &r);
    out->bf_pops = r.nodes; out->bf_waves = r.waves;

    /* max-mass best-first search recording every popped subproblem's gain */
    const int E = g->n_edges;
    int W = (E * 2 + 31) / 32;
    if (W < 1) W = 1;
    double *q = (double *)malloc((size_t)(E > 0 ? E : 1) * sizeof(double));
    uint32_t *root = (uint32_t *)calloc((size_t)W, sizeof(uint32_t));
    for (int e = 0; e < E; e++) {
        double p = g->edge_p[e];
        q[e] = 1.0 - p;
        if (p >= 1.0) root[e >> 4] |= 1u << ((e & 15) * 2);
        else if (p > 0.0) root[e >> 4] |= 3u << ((e & 15) * 2);
    }
    xctx x;
    x_init(&x, g, q, src, dst, &o);
    hq h;
    memset(&h, 0, sizeof(h));
    h.W = x.W; h.heap = 1;
    hq_sink(&h, root, 1.0);
    uint32_t *m = (uint32_t *)malloc(x.W * sizeof(uint32_t));
    size_t ng = 0, cg = 1024;
    double *gains = (double *)malloc(cg * sizeof(double));
    double *sorted = NULL;
    const double need = 1.0 - o.target_width;
    uint64_t next_check = 16;
    out->status = 2;
    while (h.n && ng < budget) {
        double mass = hq_pop(&h, m);
        gain_sink gs = { &h, 0.0 };
        x_expand(&x, m, mass, gain_sink_fn, &gs);
        if (ng == cg) { cg *= 2; gains = (double *)realloc(gains, cg * sizeof(double)); }
        gains[ng++] = mass - gs.pushed;
        if (ng < next_check && h.n) continue;
        next_check = ng * 2;
        /* the smallest k whose k largest gains reach 1 - target, and its certificate */
        sorted = (double *)realloc(sorted, ng * sizeof(double));
        memcpy(sorted, gains, ng * sizeof(double));
        qsort(sorted, ng, sizeof(double), cmp_desc);
        double s = 0.0;
        size_t k = 0;
        while (k < ng && s < need) s += sorted[k++];
        const double top = h.n ? h.key[0] : 0.0;
        if (s >= need && sorted[k - 1] >= top) { out->min_pops = k; out->status = 0; break; }
    }
    out->explored = ng;
    free(sorted); free(gains); free(m); free(h.d); free(h.key); free(q); free(root);
    x_free(&x);
    return 0;
}
