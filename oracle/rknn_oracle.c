/*
 * Exact CPU oracle for reverse k-nearest-neighbour queries.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke run
 * and the benchmark's CPU-baseline leg call it; the engine never does.
 *
 * It restates the brute-force predicate of rknn-naive
 * (rknn-naive/rknn.cpp:169-198: for every user, rank all facilities by
 * distance and test whether the query facility is among the first k) with
 * the strict-< tie rule that rknn-inf (rknn-inf/inf.h:77-93, "on the line is
 * valid"), rknn-inf-gpu (rknn-inf-gpu/inf_kernel.cu:20-36) and rknn-naive-gpu
 * (rknn-naive-gpu/rknn_kernel.cu:156, `dist < query_distance`) share:
 *
 *     u in RkNN_k(q)  <=>  #{ f != q : d2(u,f) < d2(u,q) } < k      (strict)
 *
 * `f != q` compares facility positions in the input (the reference's `-q` is
 * an index into the facility list, rknn-inf/inf.cpp:207).
 *
 * A second tie mode reproduces rknn-naive's own ordering exactly on
 * integer-coordinate data: its sort key is pair<float distance, Point>, and
 * Point orders by (x, y, id) (rknn-naive/rknn.cpp:53-57,176-185).  With
 * integer coordinates of magnitude <= 1000 distinct squared distances map to
 * distinct float distances, so that key equals (d2, x, y, id) and
 *
 *     u in naive(q)  <=>  #{ f != q : (d2(u,f),fx,fy,fid) < (d2(u,q),qx,qy,qid) } < k.
 *
 * Exactness.  For float32 inputs every product of two coordinates is exact in
 * double (24+24 < 53 bits), and
 *     d2(u,f) - d2(u,q) = fx^2 + fy^2 - qx^2 - qy^2 - 2ux fx - 2uy fy + 2ux qx + 2uy qy
 * is a sum of eight exact doubles.  Its sign is taken from a nonoverlapping
 * expansion built with Knuth's TwoSum (Shewchuk, "Adaptive Precision
 * Floating-Point Arithmetic and Fast Robust Geometric Predicates", 1997,
 * Grow-Expansion): the sign of an expansion is the sign of its largest
 * nonzero component.  A double-precision evaluation with a forward error
 * bound decides the clear cases first.
 *
 * Build with -ffp-contract=off: the error analysis assumes separately
 * rounded products and sums (aarch64 gcc contracts to FMA by default).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_OOM 2

/* ------------------------------------------------------------ predicates */

static inline void two_sum(double a, double b, double *s, double *e)
{
    double x = a + b;
    double bv = x - a;
    double av = x - bv;
    double br = b - bv;
    double ar = a - av;
    *s = x;
    *e = ar + br;
}

/* sign of t[0] + ... + t[n-1], exactly (n <= 16) */
static int sign_of_sum(const double *t, int n)
{
    double e[16];
    int m = 0;
    for (int i = 0; i < n; ++i) {
        double q = t[i];
        for (int j = 0; j < m; ++j) {
            double s, h;
            two_sum(q, e[j], &s, &h);
            e[j] = h;
            q = s;
        }
        e[m++] = q;
    }
    for (int j = m - 1; j >= 0; --j)
        if (e[j] != 0.0) return e[j] > 0.0 ? 1 : -1;
    return 0;
}

/* exact sign of d2(u,f) - d2(u,q) by expansion only */
int orc_sign_d2diff_expansion(float ux, float uy, float fx, float fy,
                              float qx, float qy)
{
    double t[8];
    t[0] = (double)fx * fx;
    t[1] = (double)fy * fy;
    t[2] = -((double)qx * qx);
    t[3] = -((double)qy * qy);
    t[4] = -2.0 * ((double)ux * fx);
    t[5] = -2.0 * ((double)uy * fy);
    t[6] = 2.0 * ((double)ux * qx);
    t[7] = 2.0 * ((double)uy * qy);
    return sign_of_sum(t, 8);
}

/* exact sign of d2(u,f) - d2(u,q): filtered double evaluation, expansion on
 * the rare undecided case.  The computed squared distances carry a relative
 * error of at most (1+u)^4-1 < 4.0001u each and the final difference one more
 * rounding, so |err| <= 5.0002u (Df+Dq); 8u is used. */
static inline int sign_d2diff(double ux, double uy, double fx, double fy,
                              double qx, double qy)
{
    double dfx = ux - fx, dfy = uy - fy, dqx = ux - qx, dqy = uy - qy;
    double Df = dfx * dfx + dfy * dfy;
    double Dq = dqx * dqx + dqy * dqy;
    double d = Df - Dq;
    double bound = 8.8817841970012523e-16 * (Df + Dq); /* 8 * 2^-53 */
    if (d > bound) return 1;
    if (d < -bound) return -1;
    return orc_sign_d2diff_expansion((float)ux, (float)uy, (float)fx, (float)fy,
                                     (float)qx, (float)qy);
}

int orc_sign_d2diff(float ux, float uy, float fx, float fy, float qx, float qy)
{
    return sign_d2diff(ux, uy, fx, fy, qx, qy);
}

/* ------------------------------------------------------------ the index */

typedef struct {
    int64_t nf, nu;
    float *fxy;      /* facilities in input order */
    float *uxy;      /* users in input order */
    int32_t *fid;    /* facility ids (only for the naive tie mode) */
    /* facility grid (cells in row-major order) */
    double x0, y0, cs, inv;
    int gx, gy;
    int64_t *cstart; /* gx*gy+1 */
    int32_t *fcell;  /* facility input positions, grouped by cell */
} orc_index;

static inline int cell_of(const orc_index *h, double v, double o, int g)
{
    double t = floor((v - o) * h->inv);
    if (t < 0) return 0;
    if (t > g - 1) return g - 1;
    return (int)t;
}

void orc_free(void *p)
{
    orc_index *h = (orc_index *)p;
    if (!h) return;
    free(h->fxy);
    free(h->uxy);
    free(h->fid);
    free(h->cstart);
    free(h->fcell);
    free(h);
}

void *orc_build(const float *fxy, int64_t nf, const float *uxy, int64_t nu,
                const int32_t *fid)
{
    if (nf <= 0 || nu < 0) return NULL;
    orc_index *h = (orc_index *)calloc(1, sizeof(orc_index));
    if (!h) return NULL;
    h->nf = nf;
    h->nu = nu;
    h->fxy = (float *)malloc(sizeof(float) * 2 * nf);
    h->uxy = (float *)malloc(sizeof(float) * 2 * (nu > 0 ? nu : 1));
    h->fid = (int32_t *)malloc(sizeof(int32_t) * nf);
    if (!h->fxy || !h->uxy || !h->fid) { orc_free(h); return NULL; }
    memcpy(h->fxy, fxy, sizeof(float) * 2 * nf);
    if (nu > 0) memcpy(h->uxy, uxy, sizeof(float) * 2 * nu);
    for (int64_t i = 0; i < nf; ++i) h->fid[i] = fid ? fid[i] : (int32_t)i;

    double mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    for (int64_t i = 0; i < nf; ++i) {
        double x = h->fxy[2 * i], y = h->fxy[2 * i + 1];
        if (x < mnx) mnx = x;
        if (x > mxx) mxx = x;
        if (y < mny) mny = y;
        if (y > mxy) mxy = y;
    }
    for (int64_t i = 0; i < nu; ++i) {
        double x = h->uxy[2 * i], y = h->uxy[2 * i + 1];
        if (x < mnx) mnx = x;
        if (x > mxx) mxx = x;
        if (y < mny) mny = y;
        if (y > mxy) mxy = y;
    }
    double w = mxx - mnx, hgt = mxy - mny;
    double ext = w > hgt ? w : hgt;
    if (!(ext > 0)) ext = 1.0;
    /* about two facilities per cell, at most 4096 cells a side */
    double cs = sqrt((w > 0 ? w : ext) * (hgt > 0 ? hgt : ext) * 2.0 / (double)nf);
    if (!(cs > 0)) cs = ext;
    if (ext / cs > 4096.0) cs = ext / 4096.0;
    h->x0 = mnx;
    h->y0 = mny;
    h->cs = cs;
    h->inv = 1.0 / cs;
    h->gx = (int)floor(w * h->inv) + 1;
    h->gy = (int)floor(hgt * h->inv) + 1;
    int64_t nc = (int64_t)h->gx * h->gy;
    h->cstart = (int64_t *)calloc(nc + 1, sizeof(int64_t));
    h->fcell = (int32_t *)malloc(sizeof(int32_t) * nf);
    int32_t *cid = (int32_t *)malloc(sizeof(int32_t) * nf);
    if (!h->cstart || !h->fcell || !cid) { free(cid); orc_free(h); return NULL; }
    for (int64_t i = 0; i < nf; ++i) {
        int cx = cell_of(h, h->fxy[2 * i], h->x0, h->gx);
        int cy = cell_of(h, h->fxy[2 * i + 1], h->y0, h->gy);
        cid[i] = cy * h->gx + cx;
        h->cstart[cid[i] + 1]++;
    }
    for (int64_t c = 0; c < nc; ++c) h->cstart[c + 1] += h->cstart[c];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * nc);
    if (!fill) { free(cid); orc_free(h); return NULL; }
    memcpy(fill, h->cstart, sizeof(int64_t) * nc);
    for (int64_t i = 0; i < nf; ++i) h->fcell[fill[cid[i]]++] = (int32_t)i;
    free(fill);
    free(cid);
    return h;
}

/* (d2, x, y, id) order of rknn-naive; returns 1 if f sorts before q for u */
static inline int naive_before(const orc_index *h, double ux, double uy,
                               int64_t f, int64_t q)
{
    double fx = h->fxy[2 * f], fy = h->fxy[2 * f + 1];
    double qx = h->fxy[2 * q], qy = h->fxy[2 * q + 1];
    int s = sign_d2diff(ux, uy, fx, fy, qx, qy);
    if (s != 0) return s < 0;
    if (fx != qx) return fx < qx;
    if (fy != qy) return fy < qy;
    return h->fid[f] < h->fid[q];
}

/* number of facilities that beat q for user u, stopping at k */
static int count_closer(const orc_index *h, int64_t u, int64_t q, int k, int tie)
{
    double ux = h->uxy[2 * u], uy = h->uxy[2 * u + 1];
    double qx = h->fxy[2 * q], qy = h->fxy[2 * q + 1];
    double dq = sqrt((ux - qx) * (ux - qx) + (uy - qy) * (uy - qy));
    /* A facility in Chebyshev ring r (r >= 1) around u's cell lies at least
     * (r-1)*cs from u; the margin covers rounding in the cell assignment. */
    double reach = dq * (1.0 + 1e-9) + h->cs * 1e-6;
    int cx = cell_of(h, ux, h->x0, h->gx), cy = cell_of(h, uy, h->y0, h->gy);
    int cnt = 0;
    int rmax = (h->gx > h->gy ? h->gx : h->gy);
    for (int r = 0; r <= rmax; ++r) {
        if (r >= 1 && (double)(r - 1) * h->cs > reach) break;
        int y0 = cy - r, y1 = cy + r, x0 = cx - r, x1 = cx + r;
        for (int yy = y0; yy <= y1; ++yy) {
            if (yy < 0 || yy >= h->gy) continue;
            int ring_row = (yy == y0 || yy == y1);
            for (int xx = x0; xx <= x1; ++xx) {
                if (xx < 0 || xx >= h->gx) continue;
                if (!ring_row && xx != x0 && xx != x1) continue;
                int64_t c = (int64_t)yy * h->gx + xx;
                for (int64_t p = h->cstart[c]; p < h->cstart[c + 1]; ++p) {
                    int64_t f = h->fcell[p];
                    if (f == q) continue;
                    int beats;
                    if (tie == 0)
                        beats = sign_d2diff(ux, uy, h->fxy[2 * f], h->fxy[2 * f + 1],
                                            qx, qy) < 0;
                    else
                        beats = naive_before(h, ux, uy, f, q);
                    if (beats && ++cnt >= k) return cnt;
                }
            }
        }
    }
    return cnt;
}

typedef struct {
    const orc_index *h;
    int64_t q;
    int k, tie;
    int64_t u0, u1;
    uint8_t *flags;
    int64_t hits;
} orc_job;

static void *run_job(void *p)
{
    orc_job *j = (orc_job *)p;
    int64_t hits = 0;
    for (int64_t u = j->u0; u < j->u1; ++u) {
        int c = count_closer(j->h, u, j->q, j->k, j->tie);
        uint8_t in = (uint8_t)(c < j->k);
        j->flags[u] = in;
        hits += in;
    }
    j->hits = hits;
    return NULL;
}

/* flags[u] = 1 iff user u (input order) is in RkNN_k(q).
 * tie = 0: strict-< rule; tie = 1: rknn-naive's (d2, x, y, id) order. */
int orc_query(void *p, int64_t q, int32_t k, int32_t tie, int32_t nthreads,
              uint8_t *flags, int64_t *n_out)
{
    orc_index *h = (orc_index *)p;
    if (!h || q < 0 || q >= h->nf || k <= 0 || !flags) return ORC_ERR_ARG;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (h->nu < 4096) nthreads = 1;
    orc_job jobs[256];
    pthread_t th[256];
    int64_t per = (h->nu + nthreads - 1) / nthreads;
    int started = 0;
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].h = h;
        jobs[t].q = q;
        jobs[t].k = k;
        jobs[t].tie = tie;
        jobs[t].u0 = t * per < h->nu ? t * per : h->nu;
        jobs[t].u1 = (t + 1) * per < h->nu ? (t + 1) * per : h->nu;
        jobs[t].flags = flags;
        jobs[t].hits = 0;
    }
    for (int t = 1; t < nthreads; ++t)
        if (pthread_create(&th[t], NULL, run_job, &jobs[t]) == 0) started = t;
        else { run_job(&jobs[t]); }
    run_job(&jobs[0]);
    int64_t n = jobs[0].hits;
    for (int t = 1; t < nthreads; ++t) {
        if (t <= started) pthread_join(th[t], NULL);
        n += jobs[t].hits;
    }
    if (n_out) *n_out = n;
    return ORC_OK;
}

/* number of facilities f != q strictly nearer to user u than q (capped) */
int orc_count_closer(void *p, int64_t u, int64_t q, int32_t cap)
{
    orc_index *h = (orc_index *)p;
    if (!h || u < 0 || u >= h->nu || q < 0 || q >= h->nf) return -1;
    return count_closer(h, u, q, cap, 0);
}

/* brute force over all facilities, no grid: the grid's own cross-check */
int orc_query_brute(const float *fxy, int64_t nf, const float *uxy, int64_t nu,
                    int64_t q, int32_t k, uint8_t *flags)
{
    if (q < 0 || q >= nf || k <= 0) return ORC_ERR_ARG;
    double qx = fxy[2 * q], qy = fxy[2 * q + 1];
    for (int64_t u = 0; u < nu; ++u) {
        double ux = uxy[2 * u], uy = uxy[2 * u + 1];
        int cnt = 0;
        for (int64_t f = 0; f < nf && cnt < k; ++f) {
            if (f == q) continue;
            if (orc_sign_d2diff_expansion((float)ux, (float)uy, fxy[2 * f],
                                          fxy[2 * f + 1], (float)qx, (float)qy) < 0)
                ++cnt;
        }
        flags[u] = (uint8_t)(cnt < k);
    }
    return ORC_OK;
}

/* ------------------------------------------------- many queries, user-major
 *
 * The same predicate evaluated user by user, for a whole query list at once
 * (the fixture generator's form: tens of thousands of queries over millions
 * of users, where the query-major loop above costs O(|U|) per query).
 *
 * For a user u and a facility f let c_f(u) = #{ g : d2(u,g) < d2(u,f) }
 * (g = f never counts, so this equals the count over g != f).  Then
 *
 *     u in RkNN_k(q)  <=>  c_q(u) < k
 *
 * which is rknn-naive's test (rknn-naive/rknn.cpp:169-198, q among the
 * first k) under the strict-< rule.  Every facility with c_f(u) < K lies
 * within u's K-th smallest facility distance d_K(u) (K facilities at
 * distance <= d_K are all strictly nearer than anything farther), so for
 * K = the largest k of the list it is enough to collect, by grid rings
 * around u, every facility up to d_K(u), rank them exactly, and add u to
 * every query slot s whose facility has c < k_s.  The counts are exact for
 * every collected facility within d_K(u); a collected facility beyond it
 * has a computed count >= K, as its true count, so it is never reported.
 * Ranks are taken in double precision where they are clear and by the exact
 * predicate above (sign_d2diff) inside a band around each distance. */

typedef struct {
    double d2;
    int32_t f;
} orc_cand;

static int cand_cmp(const void *a, const void *b)
{
    double x = ((const orc_cand *)a)->d2, y = ((const orc_cand *)b)->d2;
    return x < y ? -1 : (x > y ? 1 : 0);
}

typedef struct {
    int32_t *slot, *user;
    int64_t n, cap;
} orc_pairs;

static int pairs_push(orc_pairs *p, int32_t s, int32_t u)
{
    if (p->n == p->cap) {
        int64_t nc = p->cap ? 2 * p->cap : 4096;
        int32_t *ns = (int32_t *)realloc(p->slot, sizeof(int32_t) * nc);
        if (!ns) return 0;
        p->slot = ns;
        int32_t *nu = (int32_t *)realloc(p->user, sizeof(int32_t) * nc);
        if (!nu) return 0;
        p->user = nu;
        p->cap = nc;
    }
    p->slot[p->n] = s;
    p->user[p->n] = u;
    p->n++;
    return 1;
}

typedef struct {
    const orc_index *h;
    const int32_t *ks;
    const int64_t *first;   /* [nf] first slot of each facility, -1: none */
    const int64_t *next;    /* [nq] next slot with the same facility, -1: none */
    int kmax;
    int64_t u0, u1;
    orc_pairs out;
    int failed;
} orc_many_job;

static void *run_many(void *p)
{
    orc_many_job *j = (orc_many_job *)p;
    const orc_index *h = j->h;
    const int K = j->kmax;
    int64_t cap = 1024;
    orc_cand *c = (orc_cand *)malloc(sizeof(orc_cand) * cap);
    if (!c) { j->failed = 1; return NULL; }
    const int rmax = h->gx > h->gy ? h->gx : h->gy;
    for (int64_t u = j->u0; u < j->u1 && !j->failed; ++u) {
        const double ux = h->uxy[2 * u], uy = h->uxy[2 * u + 1];
        const int cx = cell_of(h, ux, h->x0, h->gx), cy = cell_of(h, uy, h->y0, h->gy);
        int64_t m = 0;
        for (int r = 0; r <= rmax; ++r) {
            if (r >= 1 && m >= K) {
                /* K-th smallest collected distance (an upper bound of d_K) */
                double kth = c[0].d2;
                /* partial selection: the K-th smallest of the collected */
                {
                    /* copy-free: sort the collected prefix (m is small) */
                    qsort(c, (size_t)m, sizeof(orc_cand), cand_cmp);
                    kth = c[K - 1].d2;
                }
                const double reach = sqrt(kth) * (1.0 + 1e-9) + h->cs * 1e-6;
                if ((double)(r - 1) * h->cs > reach) break;
            }
            const int y0 = cy - r, y1 = cy + r, x0 = cx - r, x1 = cx + r;
            for (int yy = y0; yy <= y1; ++yy) {
                if (yy < 0 || yy >= h->gy) continue;
                const int ring_row = (yy == y0 || yy == y1);
                for (int xx = x0; xx <= x1; ++xx) {
                    if (xx < 0 || xx >= h->gx) continue;
                    if (!ring_row && xx != x0 && xx != x1) continue;
                    const int64_t cc = (int64_t)yy * h->gx + xx;
                    for (int64_t p2 = h->cstart[cc]; p2 < h->cstart[cc + 1]; ++p2) {
                        const int32_t f = h->fcell[p2];
                        if (m == cap) {
                            orc_cand *nc2 = (orc_cand *)realloc(c, sizeof(orc_cand) * cap * 2);
                            if (!nc2) { j->failed = 1; break; }
                            c = nc2;
                            cap *= 2;
                        }
                        const double dx = ux - h->fxy[2 * f], dy = uy - h->fxy[2 * f + 1];
                        c[m].d2 = dx * dx + dy * dy;
                        c[m].f = f;
                        ++m;
                    }
                }
            }
        }
        if (j->failed) break;
        qsort(c, (size_t)m, sizeof(orc_cand), cand_cmp);
        /* exact rank of each collected facility: everything clearly below
         * its distance counts, the band around it is decided exactly.  The
         * band half-width 32u*d2 exceeds the sum of both distances' errors
         * (each <= 4.0001u of itself) for every distance inside it. */
        int64_t lo = 0;
        for (int64_t i = 0; i < m; ++i) {
            const double d = c[i].d2, tol = 3.552713678800501e-15 * d + 1e-300; /* 32 * 2^-53 */
            while (lo < i && c[lo].d2 < d - tol) ++lo;
            if (lo >= K) break;   /* lo facilities strictly nearer: c_f >= K from here on */
            const int64_t first = j->first[c[i].f];
            if (first < 0) continue;
            int64_t cnt = lo;
            const float fx = h->fxy[2 * c[i].f], fy = h->fxy[2 * c[i].f + 1];
            for (int64_t t = lo; t < m && c[t].d2 <= d + tol; ++t) {
                if (t == i) continue;
                if (sign_d2diff(ux, uy, h->fxy[2 * c[t].f], h->fxy[2 * c[t].f + 1], fx, fy) < 0) ++cnt;
            }
            if (cnt >= K) continue;
            for (int64_t s = first; s >= 0; s = j->next[s])
                if (cnt < j->ks[s] && !pairs_push(&j->out, (int32_t)s, (int32_t)u)) { j->failed = 1; break; }
        }
    }
    free(c);
    return NULL;
}

typedef struct {
    int64_t nq, npairs;
    int64_t *off;     /* [nq+1] */
    int32_t *users;   /* [npairs], ascending within each slot */
} orc_many_result;

/* Answers nq queries (facility index qs[s], k = ks[s]) over every user.
 * Returns a result handle (null on a bad argument or allocation failure);
 * read it with orc_many_sizes / orc_many_fetch, release it with
 * orc_many_free. */
void *orc_query_many(void *p, const int64_t *qs, const int32_t *ks, int64_t nq, int32_t nthreads)
{
    orc_index *h = (orc_index *)p;
    if (!h || nq < 0 || (nq > 0 && (!qs || !ks))) return NULL;
    int kmax = 0;
    for (int64_t s = 0; s < nq; ++s) {
        if (qs[s] < 0 || qs[s] >= h->nf || ks[s] <= 0) return NULL;
        if (ks[s] > kmax) kmax = ks[s];
    }
    orc_many_result *R = (orc_many_result *)calloc(1, sizeof(orc_many_result));
    if (!R) return NULL;
    R->nq = nq;
    R->off = (int64_t *)calloc((size_t)nq + 1, sizeof(int64_t));
    int64_t *first = (int64_t *)malloc(sizeof(int64_t) * (size_t)h->nf);
    int64_t *next = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nq > 0 ? nq : 1));
    if (!R->off || !first || !next) goto fail;
    for (int64_t f = 0; f < h->nf; ++f) first[f] = -1;
    for (int64_t s = nq - 1; s >= 0; --s) {
        next[s] = first[qs[s]];
        first[qs[s]] = s;
    }
    if (nq == 0 || h->nu == 0) {
        free(first);
        free(next);
        R->users = (int32_t *)malloc(sizeof(int32_t));
        if (!R->users) { free(R->off); free(R); return NULL; }
        return R;
    }
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (h->nu < 4096) nthreads = 1;
    orc_many_job *jobs = (orc_many_job *)calloc((size_t)nthreads, sizeof(orc_many_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    char *started = (char *)calloc((size_t)nthreads, 1);
    if (!jobs || !th || !started) { free(jobs); free(th); free(started); goto fail; }
    const int64_t per = (h->nu + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].h = h;
        jobs[t].ks = ks;
        jobs[t].first = first;
        jobs[t].next = next;
        jobs[t].kmax = kmax;
        jobs[t].u0 = t * per < h->nu ? t * per : h->nu;
        jobs[t].u1 = (t + 1) * per < h->nu ? (t + 1) * per : h->nu;
    }
    for (int t = 1; t < nthreads; ++t) started[t] = pthread_create(&th[t], NULL, run_many, &jobs[t]) == 0;
    for (int t = 0; t < nthreads; ++t)
        if (!started[t]) run_many(&jobs[t]);
    for (int t = 1; t < nthreads; ++t)
        if (started[t]) pthread_join(th[t], NULL);
    int bad = 0;
    int64_t tot = 0;
    for (int t = 0; t < nthreads; ++t) {
        bad |= jobs[t].failed;
        tot += jobs[t].out.n;
        for (int64_t i = 0; i < jobs[t].out.n; ++i) R->off[jobs[t].out.slot[i] + 1]++;
    }
    if (!bad) {
        for (int64_t s = 0; s < nq; ++s) R->off[s + 1] += R->off[s];
        R->npairs = tot;
        R->users = (int32_t *)malloc(sizeof(int32_t) * (size_t)(tot > 0 ? tot : 1));
        int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)nq);
        if (R->users && fill) {
            memcpy(fill, R->off, sizeof(int64_t) * (size_t)nq);
            /* threads cover increasing user ranges: each slot's users come
             * out ascending */
            for (int t = 0; t < nthreads; ++t)
                for (int64_t i = 0; i < jobs[t].out.n; ++i)
                    R->users[fill[jobs[t].out.slot[i]]++] = jobs[t].out.user[i];
        } else {
            bad = 1;
        }
        free(fill);
    }
    for (int t = 0; t < nthreads; ++t) {
        free(jobs[t].out.slot);
        free(jobs[t].out.user);
    }
    free(jobs);
    free(th);
    free(started);
    free(first);
    free(next);
    if (bad) {
        free(R->users);
        free(R->off);
        free(R);
        return NULL;
    }
    return R;
fail:
    free(first);
    free(next);
    free(R->off);
    free(R);
    return NULL;
}

int64_t orc_many_pairs(const void *r)
{
    return r ? ((const orc_many_result *)r)->npairs : -1;
}

/* off: nq+1 offsets; users: npairs user positions (input order) */
int orc_many_fetch(const void *r, int64_t *off, int32_t *users)
{
    const orc_many_result *R = (const orc_many_result *)r;
    if (!R || !off || !users) return ORC_ERR_ARG;
    memcpy(off, R->off, sizeof(int64_t) * (size_t)(R->nq + 1));
    if (R->npairs > 0) memcpy(users, R->users, sizeof(int32_t) * (size_t)R->npairs);
    return ORC_OK;
}

void orc_many_free(void *r)
{
    orc_many_result *R = (orc_many_result *)r;
    if (!R) return;
    free(R->off);
    free(R->users);
    free(R);
}
