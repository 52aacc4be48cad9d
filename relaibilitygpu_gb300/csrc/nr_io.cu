// nr_io.cu -- the graph file loader and the result block of the C ABI (include/nr.h): host
// code only, the reference's file and output formats.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "nr.h"

// ---------------------------------------------------------------------------
// graph file loader (workingPad/graph.h:46-145 semantics, status codes instead of exit)
// ---------------------------------------------------------------------------
namespace {
struct Reader {
    const char *p, *end;
    bool skip()
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
        return p < end;
    }
    bool integer(long *v)
    {
        if (!skip()) return false;
        char *e;
        long x = strtol(p, &e, 10);
        if (e == p) return false;
        p = e;
        *v = x;
        return true;
    }
    bool real(double *v)
    {
        if (!skip()) return false;
        char *e;
        double x = strtod(p, &e);
        if (e == p) return false;
        p = e;
        *v = x;
        return true;
    }
};
}  // namespace

extern "C" int nr_graph_load(const char *path, nr_graph *out)
{
    if (!path || !out) return NR_ERR_INVALID;
    memset(out, 0, sizeof(*out));
    FILE *f = fopen(path, "rb");
    if (!f) return NR_ERR_IO;
    std::string text;
    char buf[65536];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
    fclose(f);
    Reader rd{text.data(), text.data() + text.size()};
    long n = 0, efile = 0;
    if (!rd.integer(&n) || !rd.integer(&efile) || n <= 0 || n > (1L << 24)) return NR_ERR_PARSE;
    rd.skip();
    bool directed = false;
    if (rd.p < rd.end && isalpha((unsigned char)*rd.p)) {        // optional U / D
        directed = (*rd.p == 'D' || *rd.p == 'd');
        ++rd.p;
    }
    std::vector<int32_t> row(n + 1, 0), col;
    std::vector<double> arc_p;
    for (long u = 0; u < n; ++u) {
        long deg;
        if (!rd.integer(&deg) || deg < 0) return NR_ERR_PARSE;
        for (long j = 0; j < deg; ++j) {
            long v;
            double p;
            if (!rd.integer(&v) || !rd.real(&p) || v < 0 || v >= n) return NR_ERR_PARSE;
            col.push_back((int32_t)v);
            arc_p.push_back(p);
        }
        row[u + 1] = (int32_t)col.size();
    }
    // edge ids: first-seen (min,max) pairs (graph.h:77-90); a directed graph gives every arc
    // its own id in file order (seq/GraphRP.h:131-145: no merging of the two directions)
    std::map<std::pair<int32_t, int32_t>, int32_t> ids;
    std::vector<int32_t> eid(col.size());
    std::vector<double> ep;
    if (directed) {
        for (size_t j = 0; j < col.size(); ++j) eid[j] = (int32_t)j;
        ep = arc_p;
    }
    for (long u = 0; u < n && !directed; ++u)
        for (int32_t j = row[u]; j < row[u + 1]; ++j) {
            std::pair<int32_t, int32_t> key(std::min<int32_t>((int32_t)u, col[j]), std::max<int32_t>((int32_t)u, col[j]));
            auto it = ids.find(key);
            if (it == ids.end()) {
                it = ids.emplace(key, (int32_t)ep.size()).first;
                ep.push_back(arc_p[j]);
            }
            eid[j] = it->second;
        }
    int32_t *r = (int32_t *)malloc(sizeof(int32_t) * (n + 1));
    int32_t *c = (int32_t *)malloc(sizeof(int32_t) * std::max<size_t>(col.size(), 1));
    int32_t *e = (int32_t *)malloc(sizeof(int32_t) * std::max<size_t>(col.size(), 1));
    double *p = (double *)malloc(sizeof(double) * std::max<size_t>(ep.size(), 1));
    if (!r || !c || !e || !p) {
        free(r); free(c); free(e); free(p);
        return NR_ERR_NOMEM;
    }
    memcpy(r, row.data(), sizeof(int32_t) * (n + 1));
    if (!col.empty()) {
        memcpy(c, col.data(), sizeof(int32_t) * col.size());
        memcpy(e, eid.data(), sizeof(int32_t) * col.size());
    }
    if (!ep.empty()) memcpy(p, ep.data(), sizeof(double) * ep.size());
    out->n_nodes = (int32_t)n;
    out->n_edges = (int32_t)ep.size();
    out->n_arcs = (int32_t)col.size();
    out->row_ptr = r;
    out->col_idx = c;
    out->edge_id = e;
    out->edge_p = p;
    return NR_OK;
}

extern "C" void nr_graph_free(nr_graph *g)
{
    if (!g) return;
    free((void *)g->row_ptr);
    free((void *)g->col_idx);
    free((void *)g->edge_id);
    free((void *)g->edge_p);
    memset(g, 0, sizeof(*g));
}

extern "C" int nr_format_result(const nr_result *r, char *buf, size_t len)
{
    if (!r) return NR_ERR_INVALID;
    // line layout of workingPad/main.cu:1037-1056
    return snprintf(buf, len,
                    "\n"
                    "============================================\n"
                    "  Two-Terminal Network Reliability Results\n"
                    "============================================\n"
                    "Graph:            N = %d, E = %d\n"
                    "Terminals:        src = %d, dst = %d\n"
                    "--------------------------------------------\n"
                    "Reliability:      R(G) = %.12f\n"
                    "R + ESP:                 %.12f\n"
                    "ESP (truncated):         %.6e\n"
                    "Truncation bound:        %.6e\n"
                    "--------------------------------------------\n"
                    "Paths enumerated: %llu\n"
                    "Nodes processed:  %llu\n"
                    "Kernel iterations:%d\n"
                    "Max queue RSS:    %.3f MB  (%llu items)\n"
                    "Total time:       %.3f ms\n"
                    "============================================\n",
                    r->n_nodes, r->n_edges, r->src, r->dst, r->R, r->R_plus_esp, r->esp, r->trunc_bound,
                    (unsigned long long)r->paths, (unsigned long long)r->nodes, r->iterations, r->max_queue_mb,
                    (unsigned long long)r->max_queue_items, r->ms);
}
