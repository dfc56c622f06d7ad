/*
 * CPU restatement of rknn-inf's query path: the influence-zone filter
 * (rknn-inf/inf.cpp:201-585) and the bisector-count verification
 * (rknn-inf/inf.h:194-249).
 *
 * TEST INFRASTRUCTURE ONLY.  Used (a) as the benchmark's CPU baseline when the
 * reference binary itself cannot run on the host (kind "port"), and (b) to
 * cross-check the bisector set that the GPU zone kernel builds: run over the
 * same uniform grid ("grid" tree) both must produce the same bisectors in the
 * same order.
 *
 * The filter is inf.cpp's best-first search over a spatial tree.  rknn-inf
 * uses an R*-tree (rknn-inf/RStarTree2D.cpp); this file offers two trees:
 *   - TREE_RTREE: an STR bulk-loaded R-tree with 8 entries per node (the
 *     R*-tree's MAX_ENTRIES, rknn-inf/RStarTree2D.h:76-77), for timing;
 *   - TREE_GRID:  root -> grid cells -> points, the engine's index.
 * Ties in the priority queue are broken by (key, node-before-point, id); the
 * reference's std::priority_queue leaves them unspecified.
 *
 * All arithmetic is IEEE double in the reference's order of operations and
 * without contraction (compile with -ffp-contract=off), so the lines,
 * vertices and counts are the values rknn-inf computes for the same
 * visiting order.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define EPS 1e-9

typedef struct { double a, b, xv; int vert, valid; } line_t;       /* inf.h:6-94 */
typedef struct { double x, y, dq; int cnt, bnd; } vtx_t;            /* inf.h:290-298 */
typedef struct { double x0, y0, x1, y1; } rect_t;

/* ------------------------------------------------------------ geometry */

static inline double dist(double ax, double ay, double bx, double by)
{   /* Point::distance_to, rknn-inf/RStarTree2D.cpp:4-6 */
    double dx = ax - bx, dy = ay - by;
    return sqrt(dx * dx + dy * dy);
}

static inline double rect_dist(double px, double py, const rect_t *r)
{   /* min_distance_to_rect, rknn-inf/inf.h:265-272 */
    double dx = 0, dy = 0;
    if (px < r->x0) dx = r->x0 - px;
    else if (px > r->x1) dx = px - r->x1;
    if (py < r->y0) dy = r->y0 - py;
    else if (py > r->y1) dy = py - r->y1;
    return sqrt(dx * dx + dy * dy);
}

static inline int valid_side(const line_t *l, double x, double y)
{   /* Line::is_on_valid_side, rknn-inf/inf.h:77-93 */
    if (l->valid == 1) return l->vert ? (x >= l->xv) : (y >= l->a * x + l->b);
    return l->vert ? (x <= l->xv) : (y <= l->a * x + l->b);
}

static line_t bisector(double qx, double qy, double px, double py)
{   /* perpendicular_bisector, rknn-inf/inf.h:150-192 (p1 = query) */
    line_t l;
    double mx = (qx + px) / 2.0, my = (qy + py) / 2.0;
    l.a = 0; l.b = 0; l.xv = 0; l.vert = 0;
    if (qx == px) {             /* horizontal: y = my */
        l.a = 0; l.b = my;
    } else if (qy == py) {      /* vertical: x = mx */
        l.vert = 1; l.xv = mx;
    } else {
        double s = (py - qy) / (px - qx);
        double ps = -1.0 / s;
        double yi = my - ps * mx;
        if (isinf(ps)) { l.vert = 1; l.xv = yi; }   /* Line(slope,b) ctor */
        else { l.a = ps; l.b = yi; }
    }
    if (l.vert) l.valid = (qx >= l.xv) ? 1 : 0;
    else l.valid = (qy >= (l.a * qx + l.b)) ? 1 : 0;
    return l;
}

static int intersect(const line_t *l1, const line_t *l2, double *x, double *y)
{   /* find_line_intersection, rknn-inf/inf.h:303-333 */
    if (l1->vert && l2->vert) return 0;
    if (l1->vert) { *x = l1->xv; *y = l2->a * l1->xv + l2->b; return 1; }
    if (l2->vert) { *x = l2->xv; *y = l1->a * l2->xv + l1->b; return 1; }
    if (fabs(l1->a - l2->a) < EPS) return 0;
    *x = (l2->b - l1->b) / (l1->a - l2->a);
    *y = l1->a * *x + l1->b;
    return 1;
}

static double line_dist(double px, double py, const line_t *l)
{   /* min_distance_to_line, rknn-inf/inf.h:275-287 */
    if (l->vert) return fabs(px - l->xv);
    return fabs(l->a * px - py + l->b) / sqrt(l->a * l->a + 1);
}

/* ------------------------------------------------------------ trees */

typedef struct {
    rect_t mbr;
    int leaf;          /* children are points */
    int first, count;  /* into kids[] (nodes) or pts[] (points) */
} node_t;

typedef struct {
    int64_t n;
    double *xy;        /* points (input order) */
    int32_t *pts;      /* point indices grouped by leaf */
    node_t *nodes;
    int32_t *kids;     /* child node indices */
    int nnodes, root;
} tree_t;

static void tree_free(tree_t *t)
{
    if (!t) return;
    free(t->xy); free(t->pts); free(t->nodes); free(t->kids);
    memset(t, 0, sizeof(*t));
}

static const double *g_sort_xy;
static int g_sort_dim;
static int cmp_idx(const void *a, const void *b)
{
    int32_t i = *(const int32_t *)a, j = *(const int32_t *)b;
    double u = g_sort_xy[2 * i + g_sort_dim], v = g_sort_xy[2 * j + g_sort_dim];
    if (u < v) return -1;
    if (u > v) return 1;
    return (i > j) - (i < j);
}
static const rect_t *g_sort_r;
static int cmp_node(const void *a, const void *b)
{
    int32_t i = *(const int32_t *)a, j = *(const int32_t *)b;
    double u = g_sort_dim ? g_sort_r[i].y0 + g_sort_r[i].y1 : g_sort_r[i].x0 + g_sort_r[i].x1;
    double v = g_sort_dim ? g_sort_r[j].y0 + g_sort_r[j].y1 : g_sort_r[j].x0 + g_sort_r[j].x1;
    if (u < v) return -1;
    if (u > v) return 1;
    return (i > j) - (i < j);
}

static rect_t rect_of_pts(const double *xy, const int32_t *p, int n)
{
    rect_t r = {DBL_MAX, DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int i = 0; i < n; ++i) {
        double x = xy[2 * p[i]], y = xy[2 * p[i] + 1];
        if (x < r.x0) r.x0 = x;
        if (x > r.x1) r.x1 = x;
        if (y < r.y0) r.y0 = y;
        if (y > r.y1) r.y1 = y;
    }
    return r;
}

/* STR packing (Leutenegger et al. 1997) of one level: sort items by x into
 * vertical slices, each slice by y, and cut runs of M. Not thread safe (qsort
 * comparators use globals); trees are built before any threads start. */
#define FAN 8
static int str_build(tree_t *t, const float *xy, int64_t n)
{
    memset(t, 0, sizeof(*t));
    t->n = n;
    t->xy = (double *)malloc(sizeof(double) * 2 * (n > 0 ? n : 1));
    t->pts = (int32_t *)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    int64_t cap = n / 2 + 16;
    t->nodes = (node_t *)malloc(sizeof(node_t) * cap);
    t->kids = (int32_t *)malloc(sizeof(int32_t) * cap);
    if (!t->xy || !t->pts || !t->nodes || !t->kids) return -1;
    for (int64_t i = 0; i < 2 * n; ++i) t->xy[i] = xy[i];
    for (int64_t i = 0; i < n; ++i) t->pts[i] = (int32_t)i;
    if (n == 0) return -1;
    /* leaves */
    int64_t nleaf = (n + FAN - 1) / FAN;
    int64_t S = (int64_t)ceil(sqrt((double)nleaf));
    g_sort_xy = t->xy;
    g_sort_dim = 0;
    qsort(t->pts, n, sizeof(int32_t), cmp_idx);
    int64_t per_slice = S * FAN;
    g_sort_dim = 1;
    for (int64_t s0 = 0; s0 < n; s0 += per_slice) {
        int64_t m = (n - s0 < per_slice) ? n - s0 : per_slice;
        qsort(t->pts + s0, m, sizeof(int32_t), cmp_idx);
    }
    int nn = 0;
    for (int64_t i = 0; i < n; i += FAN) {
        node_t *nd = &t->nodes[nn];
        nd->leaf = 1;
        nd->first = (int)i;
        nd->count = (int)((n - i < FAN) ? n - i : FAN);
        nd->mbr = rect_of_pts(t->xy, t->pts + i, nd->count);
        nn++;
    }
    /* upper levels */
    int lvl0 = 0, lvl1 = nn;
    int kid_fill = 0;
    while (lvl1 - lvl0 > 1) {
        int m = lvl1 - lvl0;
        int32_t *ord = (int32_t *)malloc(sizeof(int32_t) * m);
        rect_t *rs = (rect_t *)malloc(sizeof(rect_t) * (lvl1));
        for (int i = 0; i < lvl1; ++i) rs[i] = t->nodes[i].mbr;
        for (int i = 0; i < m; ++i) ord[i] = lvl0 + i;
        int64_t np = (m + FAN - 1) / FAN;
        int64_t Sx = (int64_t)ceil(sqrt((double)np));
        g_sort_r = rs;
        g_sort_dim = 0;
        qsort(ord, m, sizeof(int32_t), cmp_node);
        int64_t ps = Sx * FAN;
        g_sort_dim = 1;
        for (int64_t s0 = 0; s0 < m; s0 += ps) {
            int64_t c = (m - s0 < ps) ? m - s0 : ps;
            qsort(ord + s0, c, sizeof(int32_t), cmp_node);
        }
        int start = nn;
        for (int i = 0; i < m; i += FAN) {
            node_t *nd = &t->nodes[nn];
            nd->leaf = 0;
            nd->first = kid_fill;
            nd->count = (m - i < FAN) ? m - i : FAN;
            rect_t r = {DBL_MAX, DBL_MAX, -DBL_MAX, -DBL_MAX};
            for (int j = 0; j < nd->count; ++j) {
                int c = ord[i + j];
                t->kids[kid_fill++] = c;
                rect_t cr = t->nodes[c].mbr;
                if (cr.x0 < r.x0) r.x0 = cr.x0;
                if (cr.y0 < r.y0) r.y0 = cr.y0;
                if (cr.x1 > r.x1) r.x1 = cr.x1;
                if (cr.y1 > r.y1) r.y1 = cr.y1;
            }
            nd->mbr = r;
            nn++;
        }
        free(ord);
        free(rs);
        lvl0 = start;
        lvl1 = nn;
    }
    t->nnodes = nn;
    t->root = nn - 1;
    return 0;
}

/* Grid tree: root -> non-empty cells (row-major) -> points (by input index).
 * Cell of a coordinate v: floor((float)((v - o) * inv)) computed in float as
 * the engine does, clamped to the grid. */
static int grid_build(tree_t *t, const float *xy, int64_t n, float ox, float oy,
                      float inv, int gx, int gy)
{
    memset(t, 0, sizeof(*t));
    t->n = n;
    int64_t nc = (int64_t)gx * gy;
    t->xy = (double *)malloc(sizeof(double) * 2 * (n > 0 ? n : 1));
    t->pts = (int32_t *)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    t->nodes = (node_t *)malloc(sizeof(node_t) * (nc + 1));
    t->kids = (int32_t *)malloc(sizeof(int32_t) * (nc + 1));
    int64_t *cnt = (int64_t *)calloc(nc + 1, sizeof(int64_t));
    int32_t *cid = (int32_t *)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    if (!t->xy || !t->pts || !t->nodes || !t->kids || !cnt || !cid) {
        free(cnt); free(cid); return -1;
    }
    for (int64_t i = 0; i < 2 * n; ++i) t->xy[i] = xy[i];
    for (int64_t i = 0; i < n; ++i) {
        float fx = floorf((xy[2 * i] - ox) * inv);
        float fy = floorf((xy[2 * i + 1] - oy) * inv);
        int cx = fx < 0 ? 0 : (fx > gx - 1 ? gx - 1 : (int)fx);
        int cy = fy < 0 ? 0 : (fy > gy - 1 ? gy - 1 : (int)fy);
        cid[i] = cy * gx + cx;
        cnt[cid[i] + 1]++;
    }
    for (int64_t c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (nc + 1));
    memcpy(fill, cnt, sizeof(int64_t) * (nc + 1));
    for (int64_t i = 0; i < n; ++i) t->pts[fill[cid[i]]++] = (int32_t)i;
    free(fill);
    int nn = 0;
    for (int64_t c = 0; c < nc; ++c) {
        if (cnt[c + 1] == cnt[c]) continue;
        node_t *nd = &t->nodes[nn];
        nd->leaf = 1;
        nd->first = (int)cnt[c];
        nd->count = (int)(cnt[c + 1] - cnt[c]);
        nd->mbr = rect_of_pts(t->xy, t->pts + nd->first, nd->count);
        t->kids[nn] = nn;
        nn++;
    }
    node_t *root = &t->nodes[nn];
    root->leaf = 0;
    root->first = 0;
    root->count = nn;
    rect_t r = {DBL_MAX, DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int i = 0; i < nn; ++i) {
        rect_t cr = t->nodes[i].mbr;
        if (cr.x0 < r.x0) r.x0 = cr.x0;
        if (cr.y0 < r.y0) r.y0 = cr.y0;
        if (cr.x1 > r.x1) r.x1 = cr.x1;
        if (cr.y1 > r.y1) r.y1 = cr.y1;
    }
    root->mbr = r;
    t->root = nn;
    t->nnodes = nn + 1;
    free(cnt);
    free(cid);
    return 0;
}

/* ------------------------------------------------------------ the filter */

/* kind 0: node (id = node index); kind 1: point (id = position in pts[], i.e.
 * the point's rank in leaf order, which for the grid tree is the engine's
 * cell-sorted facility position) */
typedef struct { double key; int kind; int id; } pqe_t;

typedef struct {
    pqe_t *h;
    int n, cap;
} heap_t;

static inline int pq_less(const pqe_t *a, const pqe_t *b)
{
    if (a->key != b->key) return a->key < b->key;
    if (a->kind != b->kind) return a->kind < b->kind;
    return a->id < b->id;
}

static int pq_push(heap_t *q, pqe_t e)
{
    if (q->n == q->cap) {
        int nc = q->cap ? q->cap * 2 : 256;
        pqe_t *nh = (pqe_t *)realloc(q->h, sizeof(pqe_t) * nc);
        if (!nh) return -1;
        q->h = nh;
        q->cap = nc;
    }
    int i = q->n++;
    while (i > 0) {
        int p = (i - 1) / 2;
        if (!pq_less(&e, &q->h[p])) break;
        q->h[i] = q->h[p];
        i = p;
    }
    q->h[i] = e;
    return 0;
}

static pqe_t pq_pop(heap_t *q)
{
    pqe_t top = q->h[0];
    pqe_t last = q->h[--q->n];
    int i = 0;
    for (;;) {
        int l = 2 * i + 1;
        if (l >= q->n) break;
        int c = (l + 1 < q->n && pq_less(&q->h[l + 1], &q->h[l])) ? l + 1 : l;
        if (!pq_less(&q->h[c], &last)) break;
        q->h[i] = q->h[c];
        i = c;
    }
    if (q->n > 0) q->h[i] = last;
    return top;
}

typedef struct {
    line_t *L; int32_t *Lf; int nL, capL;
    vtx_t *V; int nV, capV;
    int maxV;
} zone_t;

static int push_line(zone_t *z, line_t l, int32_t f)
{
    if (z->nL == z->capL) {
        int nc = z->capL ? z->capL * 2 : 64;
        line_t *nl = (line_t *)realloc(z->L, sizeof(line_t) * nc);
        int32_t *nf = (int32_t *)realloc(z->Lf, sizeof(int32_t) * nc);
        if (!nl || !nf) { if (nl) z->L = nl; if (nf) z->Lf = nf; return -1; }
        z->L = nl; z->Lf = nf; z->capL = nc;
    }
    z->L[z->nL] = l;
    z->Lf[z->nL++] = f;
    return 0;
}

static int push_vtx(zone_t *z, vtx_t v)
{
    if (z->nV == z->capV) {
        int nc = z->capV ? z->capV * 2 : 256;
        vtx_t *nv = (vtx_t *)realloc(z->V, sizeof(vtx_t) * nc);
        if (!nv) return -1;
        z->V = nv; z->capV = nc;
    }
    z->V[z->nV++] = v;
    if (z->nV > z->maxV) z->maxV = z->nV;
    return 0;
}

/* Which vertices the vertex test looks at (inf.cpp:269-346): count == k-1,
 * or a boundary vertex with count < k lying (within EPS) on one of the eight
 * extreme boundary points.  Recomputed after every change of the vertex set;
 * it depends on nothing else. */
static void mark_considered(const zone_t *z, const rect_t *sp, int k, uint8_t *cons)
{
    const vtx_t *e[8] = {0};   /* left min/max, right min/max, bottom min/max, top min/max */
    for (int i = 0; i < z->nV; ++i) {
        const vtx_t *v = &z->V[i];
        if (!(v->bnd && v->cnt < k)) continue;
        if (fabs(v->x - sp->x0) < EPS) {
            if (!e[0] || v->y < e[0]->y) e[0] = v;
            if (!e[1] || v->y > e[1]->y) e[1] = v;
        }
        if (fabs(v->x - sp->x1) < EPS) {
            if (!e[2] || v->y < e[2]->y) e[2] = v;
            if (!e[3] || v->y > e[3]->y) e[3] = v;
        }
        if (fabs(v->y - sp->y0) < EPS) {
            if (!e[4] || v->x < e[4]->x) e[4] = v;
            if (!e[5] || v->x > e[5]->x) e[5] = v;
        }
        if (fabs(v->y - sp->y1) < EPS) {
            if (!e[6] || v->x < e[6]->x) e[6] = v;
            if (!e[7] || v->x > e[7]->x) e[7] = v;
        }
    }
    for (int i = 0; i < z->nV; ++i) {
        const vtx_t *v = &z->V[i];
        int c = 0;
        if (v->cnt == k - 1) c = 1;
        else if (v->bnd && v->cnt < k) {
            for (int j = 0; j < 8 && !c; ++j)
                if (e[j] && fabs(v->x - e[j]->x) < EPS && fabs(v->y - e[j]->y) < EPS) c = 1;
        }
        cons[i] = (uint8_t)c;
    }
}

typedef struct {
    int nbis, maxV, npts, nnodes, naccept;
} zstats_t;

/* Influence-zone filter for query point index q (facility tree t).
 * skip_coincident: do not turn a facility at q's exact position into a
 * bisector (rknn-inf does, inf.h:158-161, and the degenerate line then marks
 * half the plane as violating). */
static int inf_filter(const tree_t *t, const rect_t *sp, int64_t q, int k,
                      int skip_coincident, zone_t *z, zstats_t *st)
{
    double qx = t->xy[2 * q], qy = t->xy[2 * q + 1];
    z->nL = 0;
    z->nV = 0;
    z->maxV = 0;
    double cx[4] = {sp->x0, sp->x1, sp->x0, sp->x1};
    double cy[4] = {sp->y0, sp->y0, sp->y1, sp->y1};
    for (int i = 0; i < 4; ++i) {   /* inf.cpp:211-226: bl, br, tl, tr */
        vtx_t v = {cx[i], cy[i], dist(cx[i], cy[i], qx, qy), 0, 1};
        if (push_vtx(z, v)) return -1;
    }
    heap_t pq = {0};
    pqe_t root = {rect_dist(qx, qy, &t->nodes[t->root].mbr), 0, t->root};
    if (pq_push(&pq, root)) return -1;
    double far = 0.0;
    for (int i = 0; i < z->nV; ++i) if (z->V[i].dq > far) far = z->V[i].dq;
    double nearb = DBL_MAX;
    uint8_t *cons = NULL;
    int cons_cap = 0, cons_valid = 0;
    memset(st, 0, sizeof(*st));

    while (pq.n > 0) {
        pqe_t cur = pq_pop(&pq);
        if (cons_cap < z->nV) {
            cons_cap = z->nV * 2;
            cons = (uint8_t *)realloc(cons, cons_cap);
            cons_valid = 0;
        }
        if (cur.kind == 1) {
            int64_t p = t->pts[cur.id];
            if (p == q) continue;
            double px = t->xy[2 * p], py = t->xy[2 * p + 1];
            if (skip_coincident && px == qx && py == qy) continue;
            st->npts++;
            int prune = 1;
            double dq = dist(px, py, qx, qy);
            if (dq > 2 * far) prune = 1;
            else if (dq < 2 * nearb) prune = 0;
            else {
                if (!cons_valid) { mark_considered(z, sp, k, cons); cons_valid = 1; }
                for (int i = 0; i < z->nV; ++i) {
                    if (!cons[i]) continue;
                    const vtx_t *v = &z->V[i];
                    if (dist(px, py, v->x, v->y) < dist(qx, qy, v->x, v->y)) { prune = 0; break; }
                }
            }
            if (prune) continue;
            /* accept: inf.cpp:356-452 */
            st->naccept++;
            line_t nb = bisector(qx, qy, px, py);
            for (int i = 0; i < z->nV; ++i)
                if (!valid_side(&nb, z->V[i].x, z->V[i].y)) z->V[i].cnt++;
            /* boundary intersections: bottom, top, left, right (inf.h:340-374) */
            line_t edge[4] = {{0, sp->y0, 0, 0, 1}, {0, sp->y1, 0, 0, 1},
                              {0, 0, sp->x0, 1, 1}, {0, 0, sp->x1, 1, 1}};
            for (int e = 0; e < 4; ++e) {
                double ix, iy;
                if (!intersect(&nb, &edge[e], &ix, &iy)) continue;
                if (e < 2 ? !(ix >= sp->x0 && ix <= sp->x1) : !(iy >= sp->y0 && iy <= sp->y1))
                    continue;
                int dup = 0;
                for (int i = 0; i < z->nV && !dup; ++i)
                    if (fabs(z->V[i].x - ix) < EPS && fabs(z->V[i].y - iy) < EPS) dup = 1;
                if (dup) continue;
                vtx_t v = {ix, iy, dist(ix, iy, qx, qy), 0, 1};
                for (int j = 0; j < z->nL; ++j)
                    if (!valid_side(&z->L[j], ix, iy)) v.cnt++;
                if (push_vtx(z, v)) return -1;
            }
            for (int j = 0; j < z->nL; ++j) {
                double ix, iy;
                if (!intersect(&nb, &z->L[j], &ix, &iy)) continue;
                if (!(ix >= sp->x0 && ix <= sp->x1 && iy >= sp->y0 && iy <= sp->y1)) continue;
                int dup = 0;
                for (int i = 0; i < z->nV && !dup; ++i)
                    if (fabs(z->V[i].x - ix) < EPS && fabs(z->V[i].y - iy) < EPS) dup = 1;
                if (dup) continue;
                vtx_t v = {ix, iy, dist(ix, iy, qx, qy), 0, 0};
                for (int m = 0; m < z->nL; ++m)
                    if (!valid_side(&z->L[m], ix, iy)) v.cnt++;
                if (push_vtx(z, v)) return -1;
            }
            double dl = line_dist(qx, qy, &nb);
            if (dl < nearb) nearb = dl;
            if (push_line(z, nb, (int32_t)p)) return -1;
            int w = 0;
            for (int i = 0; i < z->nV; ++i)
                if (z->V[i].cnt < k) z->V[w++] = z->V[i];
            z->nV = w;
            far = 0.0;
            for (int i = 0; i < z->nV; ++i) if (z->V[i].dq > far) far = z->V[i].dq;
            cons_valid = 0;
            if (cons_cap < z->nV) {
                cons_cap = z->nV * 2;
                cons = (uint8_t *)realloc(cons, cons_cap);
            }
        } else {
            const node_t *nd = &t->nodes[cur.id];
            st->nnodes++;
            int prune = 1;
            double md = rect_dist(qx, qy, &nd->mbr);
            if (md > 2 * far) prune = 1;
            else if (md < 2 * nearb) prune = 0;
            else {
                if (!cons_valid) { mark_considered(z, sp, k, cons); cons_valid = 1; }
                for (int i = 0; i < z->nV; ++i) {
                    if (!cons[i]) continue;
                    const vtx_t *v = &z->V[i];
                    if (rect_dist(v->x, v->y, &nd->mbr) < dist(qx, qy, v->x, v->y)) { prune = 0; break; }
                }
            }
            if (prune) continue;
            if (nd->leaf) {
                for (int i = 0; i < nd->count; ++i) {
                    int32_t p = t->pts[nd->first + i];
                    pqe_t e = {dist(qx, qy, t->xy[2 * p], t->xy[2 * p + 1]), 1, nd->first + i};
                    if (pq_push(&pq, e)) return -1;
                }
            } else {
                for (int i = 0; i < nd->count; ++i) {
                    int32_t c = t->kids[nd->first + i];
                    pqe_t e = {rect_dist(qx, qy, &t->nodes[c].mbr), 0, c};
                    if (pq_push(&pq, e)) return -1;
                }
            }
        }
    }
    free(pq.h);
    free(cons);
    st->nbis = z->nL;
    st->maxV = z->maxV;
    return 0;
}

/* check_rectangle_line_position + can_prune_node_by_valid_side,
 * rknn-inf/inf.h:104-147 */
static int node_prunable(const rect_t *r, const line_t *l)
{
    double xs[4] = {r->x0, r->x1, r->x0, r->x1};
    double ys[4] = {r->y0, r->y0, r->y1, r->y1};
    int above = 0, below = 0;
    for (int i = 0; i < 4; ++i) {
        double ev = l->vert ? xs[i] - l->xv : ys[i] - (l->a * xs[i] + l->b);
        if (ev > 0) above++;
        else if (ev < 0) below++;
    }
    if (l->valid == 1) return below == 4;
    return above == 4;
}

/* dfs_rknn_traverse, rknn-inf/inf.h:194-239 */
static int64_t dfs_verify(const tree_t *u, int node, const zone_t *z, int k, uint8_t *flags)
{
    const node_t *nd = &u->nodes[node];
    int64_t hits = 0;
    if (nd->leaf) {
        for (int i = 0; i < nd->count; ++i) {
            int32_t p = u->pts[nd->first + i];
            double x = u->xy[2 * p], y = u->xy[2 * p + 1];
            int viol = 0;
            for (int j = 0; j < z->nL; ++j)
                if (!valid_side(&z->L[j], x, y) && ++viol >= k) break;
            if (viol < k) { flags[p] = 1; hits++; }
        }
        return hits;
    }
    for (int i = 0; i < nd->count; ++i) {
        int c = u->kids[nd->first + i];
        int viol = 0;
        for (int j = 0; j < z->nL; ++j)
            if (node_prunable(&u->nodes[c].mbr, &z->L[j]) && ++viol >= k) break;
        if (viol < k) hits += dfs_verify(u, c, z, k, flags);
    }
    return hits;
}

/* ------------------------------------------------------------ public API */

typedef struct {
    tree_t ft, ut;
    rect_t space;
    int mode;
} inf_index;

void ip_free(void *p)
{
    inf_index *h = (inf_index *)p;
    if (!h) return;
    tree_free(&h->ft);
    tree_free(&h->ut);
    free(h);
}

static rect_t bbox(const float *fxy, int64_t nf, const float *uxy, int64_t nu)
{   /* inf.cpp:181-199 */
    rect_t r = {DBL_MAX, DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int64_t i = 0; i < nf; ++i) {
        double x = fxy[2 * i], y = fxy[2 * i + 1];
        r.x0 = fmin(r.x0, x); r.x1 = fmax(r.x1, x);
        r.y0 = fmin(r.y0, y); r.y1 = fmax(r.y1, y);
    }
    for (int64_t i = 0; i < nu; ++i) {
        double x = uxy[2 * i], y = uxy[2 * i + 1];
        r.x0 = fmin(r.x0, x); r.x1 = fmax(r.x1, x);
        r.y0 = fmin(r.y0, y); r.y1 = fmax(r.y1, y);
    }
    return r;
}

/* mode 0: R-trees for facilities and users.
 * mode 1: facility grid with origin (ox,oy), cell width 1/inv and gx*gy
 *         cells (the engine's facility grid); users still in an R-tree. */
void *ip_build(const float *fxy, int64_t nf, const float *uxy, int64_t nu, int mode,
               float ox, float oy, float inv, int gx, int gy)
{
    if (nf <= 0 || nu <= 0) return NULL;
    inf_index *h = (inf_index *)calloc(1, sizeof(inf_index));
    if (!h) return NULL;
    h->mode = mode;
    h->space = bbox(fxy, nf, uxy, nu);
    int rc = mode == 1 ? grid_build(&h->ft, fxy, nf, ox, oy, inv, gx, gy)
                       : str_build(&h->ft, fxy, nf);
    if (rc || str_build(&h->ut, uxy, nu)) { ip_free(h); return NULL; }
    return h;
}

/* One query: the filter, then the DFS verification.  Outputs the bisectors'
 * facility indices in creation order (bis, capacity bcap), the result flags
 * per user (flags, length nu, may be NULL) and counters
 * stats = {bisectors, max vertices, points tested, nodes tested, results}. */
int ip_query(void *p, int64_t q, int32_t k, int32_t skip_coincident,
             int32_t *bis, int32_t bcap, uint8_t *flags, int64_t *stats)
{
    inf_index *h = (inf_index *)p;
    if (!h || q < 0 || q >= h->ft.n || k <= 0) return 1;
    zone_t z = {0};
    zstats_t st;
    if (inf_filter(&h->ft, &h->space, q, k, skip_coincident, &z, &st)) {
        free(z.L); free(z.Lf); free(z.V);
        return 2;
    }
    for (int i = 0; i < z.nL && i < bcap; ++i) bis[i] = z.Lf[i];
    int64_t hits = 0;
    if (flags) {
        memset(flags, 0, (size_t)h->ut.n);
        hits = dfs_verify(&h->ut, h->ut.root, &z, k, flags);
    }
    if (stats) {
        stats[0] = st.nbis; stats[1] = st.maxV; stats[2] = st.npts;
        stats[3] = st.nnodes; stats[4] = hits;
    }
    free(z.L); free(z.Lf); free(z.V);
    return 0;
}

/* Throughput run: queries qs[0..nq) with ks[], spread over nthreads threads
 * (queries are independent).  Result counts go to counts[] (may be NULL). */
typedef struct {
    inf_index *h;
    const int64_t *qs; const int32_t *ks;
    int64_t *counts;
    int nq, t, nt;
    int err;
} ip_job;

static void *ip_run(void *a)
{
    ip_job *j = (ip_job *)a;
    uint8_t *flags = (uint8_t *)malloc((size_t)j->h->ut.n);
    if (!flags) { j->err = 2; return NULL; }
    for (int i = j->t; i < j->nq; i += j->nt) {
        int64_t st[5];
        int32_t dummy;
        if (ip_query(j->h, j->qs[i], j->ks[i], 0, &dummy, 0, flags, st)) { j->err = 1; break; }
        if (j->counts) j->counts[i] = st[4];
    }
    free(flags);
    return NULL;
}

int ip_query_many(void *p, const int64_t *qs, const int32_t *ks, int32_t nq,
                  int32_t nthreads, int64_t *counts)
{
    inf_index *h = (inf_index *)p;
    if (!h || nq < 0) return 1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    ip_job jobs[256];
    pthread_t th[256];
    for (int t = 0; t < nthreads; ++t) {
        ip_job j = {h, qs, ks, counts, nq, t, nthreads, 0};
        jobs[t] = j;
    }
    int started[256] = {0};
    for (int t = 1; t < nthreads; ++t)
        started[t] = pthread_create(&th[t], NULL, ip_run, &jobs[t]) == 0;
    ip_run(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) {
        if (started[t]) pthread_join(th[t], NULL);
        else ip_run(&jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) if (jobs[t].err) return jobs[t].err;
    return 0;
}
