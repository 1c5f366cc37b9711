/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY (see skid_oracle.h).
 *
 * CPU restatement of skid's group-finding path.  Each function names the
 * reference lines (N-BodyShop/skid v1.4.1) whose behaviour it restates.  The
 * spatial searches use a plain median-split kd tree written for this file;
 * every search prunes conservatively (box distances lowered by a rounding
 * slack) so results are exactly those of a brute-force scan.
 *
 * Build with -ffp-contract=off (no FMA contraction), never -ffast-math.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "skid_oracle.h"

#define PRUNE_STEPS 5     /* main.c:13 */
#define MICRO_STEP 0.1    /* main.c:14 */
#define LEAF 8

/* ------------------------------------------------------------------ */
/* Periodic pair distance (kd.h:122-214, smooth1.c:72-75,104-107).     */
/* ------------------------------------------------------------------ */

static inline float img_dx(float q, float c, float L)
{
    float d0 = q - c;
    float h = 0.5f * L;
    if (d0 > h) return (q - L) - c;
    if (d0 < -h) return (q + L) - c;
    return d0;
}

float or_d2(const float *q, const float *c, const float period[3])
{
    float dx = img_dx(q[0], c[0], period[0]);
    float dy = img_dx(q[1], c[1], period[1]);
    float dz = img_dx(q[2], c[2], period[2]);
    return (dx * dx + dy * dy) + dz * dz;
}

static inline float plain_d2(const float *q, const float *c)
{
    float dx = q[0] - c[0], dy = q[1] - c[1], dz = q[2] - c[2];
    return (dx * dx + dy * dy) + dz * dz;
}

/* min over both frames: the FoF edge rule (kd.c:869-876, either endpoint). */
static inline float sym_d2(const float *a, const float *b, const float period[3])
{
    float d1 = or_d2(a, b, period);
    float d2 = or_d2(b, a, period);
    return d1 < d2 ? d1 : d2;
}

static inline int is_per(float L) { return L < 0.25f * FLT_MAX; }

/* ------------------------------------------------------------------ */
/* kd tree over a point subset.                                        */
/* ------------------------------------------------------------------ */

typedef struct {
    float lo[3], hi[3];
    int first, count, left, parent; /* left child index, right = left+1; -1 leaf */
    int open;                       /* unassigned points below (FoF) */
} knode;

typedef struct {
    knode *nd;
    int nn, cap;
    int *idx;          /* point ids, permuted */
    int *leafof;       /* point id -> leaf node (FoF) */
    const float *pos;
    int n;
} ktree;

static void kt_bbox(ktree *t, knode *k)
{
    for (int d = 0; d < 3; ++d) { k->lo[d] = FLT_MAX; k->hi[d] = -FLT_MAX; }
    for (int i = k->first; i < k->first + k->count; ++i) {
        const float *p = t->pos + 3 * (size_t)t->idx[i];
        for (int d = 0; d < 3; ++d) {
            if (p[d] < k->lo[d]) k->lo[d] = p[d];
            if (p[d] > k->hi[d]) k->hi[d] = p[d];
        }
    }
}

static void kt_select(ktree *t, int l, int r, int m, int d)
{
    int *a = t->idx;
    const float *p = t->pos;
    while (r > l) {
        float v = p[3 * (size_t)a[(l + r) / 2] + d];
        int i = l, j = r;
        while (i <= j) {
            while (p[3 * (size_t)a[i] + d] < v) ++i;
            while (p[3 * (size_t)a[j] + d] > v) --j;
            if (i <= j) { int s = a[i]; a[i] = a[j]; a[j] = s; ++i; --j; }
        }
        if (m <= j) r = j;
        else if (m >= i) l = i;
        else break;
    }
}

static int kt_new(ktree *t)
{
    if (t->nn == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 64;
        t->nd = (knode *)realloc(t->nd, (size_t)t->cap * sizeof(knode));
    }
    return t->nn++;
}

static void kt_build_rec(ktree *t, int k)
{
    knode *nd = &t->nd[k];
    kt_bbox(t, nd);
    if (nd->count <= LEAF) { nd->left = -1; return; }
    int d = 0;
    for (int j = 1; j < 3; ++j)
        if (nd->hi[j] - nd->lo[j] > nd->hi[d] - nd->lo[d]) d = j;
    int first = nd->first, count = nd->count;
    int m = first + count / 2;
    kt_select(t, first, first + count - 1, m, d);
    int l = kt_new(t);
    int r = kt_new(t);
    nd = &t->nd[k];
    nd->left = l;
    t->nd[l].first = first; t->nd[l].count = m - first; t->nd[l].parent = k;
    t->nd[r].first = m; t->nd[r].count = first + count - m; t->nd[r].parent = k;
    kt_build_rec(t, l);
    kt_build_rec(t, r);
}

static void kt_build(ktree *t, const float *pos, const int *ids, int n)
{
    memset(t, 0, sizeof(*t));
    t->pos = pos;
    t->n = n;
    t->idx = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    for (int i = 0; i < n; ++i) t->idx[i] = ids ? ids[i] : i;
    if (n == 0) return;
    int root = kt_new(t);
    t->nd[root].first = 0; t->nd[root].count = n; t->nd[root].parent = -1;
    kt_build_rec(t, root);
}

static void kt_free(ktree *t)
{
    free(t->nd); free(t->idx); free(t->leafof);
    memset(t, 0, sizeof(*t));
}

/* Lower bound of the float d2 from q to any point of the box, over the
 * periodic images of q (L finite) or plain (L infinite).  The per-dimension
 * distance is lowered by a slack covering the roundings of fl(fl(q+sL)-c). */
static double box_lb(const float *q, const knode *k, const float period[3], int use_per)
{
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        double L = period[d];
        int per = use_per && is_per(period[d]);
        double lo = k->lo[d], hi = k->hi[d], x = q[d];
        double best;
        double dd = lo > x ? lo - x : (x > hi ? x - hi : 0.0);
        best = dd;
        if (per) {
            double xp = x + L, xm = x - L;
            double dp = lo > xp ? lo - xp : (xp > hi ? xp - hi : 0.0);
            double dm = lo > xm ? lo - xm : (xm > hi ? xm - hi : 0.0);
            if (dp < best) best = dp;
            if (dm < best) best = dm;
        }
        double slack = 2.5e-7 * (fabs(x) + (per ? L : 0.0) + fabs(lo) + fabs(hi)) + 1e-30;
        best -= slack;
        if (best > 0.0) s += best * best;
    }
    return s * (1.0 - 1e-6);
}

/* Upper bound of the float d2 from q to every point of the box (FoF contained
 * cells, kd.h:217-335). */
static double box_ub(const float *q, const knode *k, const float period[3])
{
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        double L = period[d];
        int per = is_per(period[d]);
        double x = q[d];
        double best = fmax(fabs(k->hi[d] - x), fabs(x - k->lo[d]));
        if (per) {
            double xp = x + L, xm = x - L;
            double bp = fmax(fabs(k->hi[d] - xp), fabs(xp - k->lo[d]));
            double bm = fmax(fabs(k->hi[d] - xm), fabs(xm - k->lo[d]));
            if (bp < best) best = bp;
            if (bm < best) best = bm;
        }
        double slack = 2.5e-7 * (fabs(x) + (per ? L : 0.0) + fabs(k->lo[d]) + fabs(k->hi[d]));
        best += slack;
        s += best * best;
    }
    return s * (1.0 + 1e-6) + 1e-30;
}

/* ------------------------------------------------------------------ */
/* k nearest neighbours: fBall2 (smooth1.c:41-129,132-243).            */
/* ------------------------------------------------------------------ */

static void heap_sift(float *h, int k)
{
    int i = 0;
    float v = h[0];
    for (;;) {
        int c = 2 * i + 1;
        if (c >= k) break;
        if (c + 1 < k && h[c + 1] > h[c]) ++c;
        if (h[c] <= v) break;
        h[i] = h[c];
        i = c;
    }
    h[i] = v;
}

typedef struct { float *heap; int k, fill; } kq;

static void kq_push(kq *q, float d)
{
    if (q->fill < q->k) {
        /* sift up into a max-heap */
        int i = q->fill++;
        while (i > 0) {
            int p = (i - 1) / 2;
            if (q->heap[p] >= d) break;
            q->heap[i] = q->heap[p];
            i = p;
        }
        q->heap[i] = d;
    } else if (d < q->heap[0]) {
        q->heap[0] = d;
        heap_sift(q->heap, q->k);
    }
}

static void knn_rec(const ktree *t, int node, const float *q, const float period[3], kq *Q)
{
    const knode *nd = &t->nd[node];
    if (Q->fill == Q->k && box_lb(q, nd, period, 1) > Q->heap[0]) return;
    if (nd->left < 0) {
        for (int i = nd->first; i < nd->first + nd->count; ++i)
            kq_push(Q, or_d2(q, t->pos + 3 * (size_t)t->idx[i], period));
        return;
    }
    int a = nd->left, b = nd->left + 1;
    double da = box_lb(q, &t->nd[a], period, 1), db = box_lb(q, &t->nd[b], period, 1);
    if (db < da) { int s = a; a = b; b = s; }
    knn_rec(t, a, q, period, Q);
    knn_rec(t, b, q, period, Q);
}

int or_knn_ball2(int n, const float *pos, int k, const float period[3], float *ball2)
{
    if (k < 1 || k > n) return -1;
    ktree t;
    kt_build(&t, pos, NULL, n);
    float *heap = (float *)malloc((size_t)k * sizeof(float));
    for (int i = 0; i < n; ++i) {
        kq Q = {heap, k, 0};
        knn_rec(&t, 0, pos + 3 * (size_t)i, period, &Q);
        ball2[i] = heap[0];
    }
    free(heap);
    kt_free(&t);
    return 0;
}

static int cmp_float(const void *a, const void *b)
{
    float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

int or_knn_ball2_brute(int n, const float *pos, int k, const float period[3], float *ball2)
{
    if (k < 1 || k > n) return -1;
    float *d = (float *)malloc((size_t)n * sizeof(float));
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) d[j] = or_d2(pos + 3 * (size_t)i, pos + 3 * (size_t)j, period);
        qsort(d, (size_t)n, sizeof(float), cmp_float);
        ball2[i] = d[k - 1];
    }
    free(d);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Range search helpers.                                               */
/* ------------------------------------------------------------------ */

typedef void (*visit_fn)(void *ctx, int j);

/* All points j with d2 < r2, where d2 is or_d2(q->j) (periodic) or the plain
 * distance (per = 0); calls fn for each. */
static void range_rec(const ktree *t, int k, const float *q, double r2, const float period[3],
                      int per, float fr2, visit_fn fn, void *ctx)
{
    const knode *nd = &t->nd[k];
    if (box_lb(q, nd, period, per) >= r2) return;
    if (nd->left < 0) {
        for (int i = nd->first; i < nd->first + nd->count; ++i) {
            int j = t->idx[i];
            const float *p = t->pos + 3 * (size_t)j;
            float d2 = per ? or_d2(q, p, period) : plain_d2(q, p);
            if (d2 < fr2) fn(ctx, j);
        }
        return;
    }
    range_rec(t, nd->left, q, r2, period, per, fr2, fn, ctx);
    range_rec(t, nd->left + 1, q, r2, period, per, fr2, fn, ctx);
}

/* ------------------------------------------------------------------ */
/* SPH density (smooth1.c:248-263), FP64.                              */
/* ------------------------------------------------------------------ */

static inline double w_kernel(double d2, double b)
{
    double ih2 = 4.0 / b;
    double r2 = d2 * ih2;
    double q = sqrt(r2);
    double rs = 2.0 - q;
    double w = (r2 < 1.0) ? (1.0 - 0.75 * rs * r2) : (0.25 * rs * rs * rs);
    return w * 0.5 * M_1_PI * sqrt(ih2) * ih2;
}

typedef struct {
    const float *pos, *mass;
    const float *q;
    double b;
    int i;
    double *rho;
    const float *period;
} dens_ctx;

static void dens_visit(void *vctx, int j)
{
    dens_ctx *c = (dens_ctx *)vctx;
    float d2 = or_d2(c->q, c->pos + 3 * (size_t)j, c->period);
    double w = w_kernel(d2, c->b);
    c->rho[c->i] += w * c->mass[j];
    c->rho[j] += w * c->mass[c->i];
}

int or_density(int n, const float *pos, const float *mass, const float *ball2,
               const float period[3], double *rho)
{
    ktree t;
    kt_build(&t, pos, NULL, n);
    for (int i = 0; i < n; ++i) rho[i] = 0.0;
    if (n == 0) { kt_free(&t); return 0; }
    for (int i = 0; i < n; ++i) {
        dens_ctx c = {pos, mass, pos + 3 * (size_t)i, ball2[i], i, rho, period};
        range_rec(&t, 0, c.q, ball2[i], period, 1, ball2[i], dens_visit, &c);
    }
    kt_free(&t);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Periodic replica scatterers (smooth1.c:283-332, INTERSECTNP         */
/* kd.h:102-119).  Bit (ix+1)*9+(iy+1)*3+(iz+1); bit 13 = original.    */
/* ------------------------------------------------------------------ */

#define ORIG_BIT 13

static inline float rep_coord(float x, int s, float L) { return x + (float)s * L; }

int or_replica_mask(int ns, const float *spos, const float *ball2, const float period[3],
                    const float center[3], int periodic, unsigned int *mask)
{
    float lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = (float)((double)center[d] - 0.5 * (double)period[d]);
        hi[d] = (float)((double)center[d] + 0.5 * (double)period[d]);
    }
    for (int i = 0; i < ns; ++i) {
        unsigned int m = 1u << ORIG_BIT;
        if (periodic) {
            const float *p = spos + 3 * (size_t)i;
            for (int ix = -1; ix <= 1; ++ix)
                for (int iy = -1; iy <= 1; ++iy)
                    for (int iz = -1; iz <= 1; ++iz) {
                        if (!(ix || iy || iz)) continue;
                        float x = rep_coord(p[0], ix, period[0]);
                        float y = rep_coord(p[1], iy, period[1]);
                        float z = rep_coord(p[2], iz, period[2]);
                        float dx = lo[0] - x, dx1 = x - hi[0];
                        float dy = lo[1] - y, dy1 = y - hi[1];
                        float dz = lo[2] - z, dz1 = z - hi[2];
                        float f;
                        if (dx > 0.0f) f = dx * dx;
                        else if (dx1 > 0.0f) f = dx1 * dx1;
                        else f = 0.0f;
                        if (dy > 0.0f) f += dy * dy;
                        else if (dy1 > 0.0f) f += dy1 * dy1;
                        if (dz > 0.0f) f += dz * dz;
                        else if (dz1 > 0.0f) f += dz1 * dz1;
                        if (f < ball2[i]) m |= 1u << ((ix + 1) * 9 + (iy + 1) * 3 + (iz + 1));
                    }
        }
        mask[i] = m;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Move field (smooth1.c:338-384 gather, 436-508 accumulation).        */
/* Scatter form: each live copy gathers the movers inside its ball.    */
/* ------------------------------------------------------------------ */

typedef struct {
    const float *mpos;
    float cpos[3];
    float b;
    double ih2, fnorm;
    double *acc;
    double *absacc;
    int hit;
} field_ctx;

static void field_visit(void *vctx, int j)
{
    field_ctx *c = (field_ctx *)vctx;
    const float *y = c->mpos + 3 * (size_t)j;
    float dx = c->cpos[0] - y[0], dy = c->cpos[1] - y[1], dz = c->cpos[2] - y[2];
    float d2 = (dx * dx + dy * dy) + dz * dz;
    double r2 = (double)d2 * c->ih2;
    double rs = sqrt(r2);
    double F = (r2 < 1.0) ? (-3.0 + 2.25 * rs) : (-3.0 / rs + 3.0 - 0.75 * rs);
    F *= c->fnorm;
    c->acc[3 * (size_t)j + 0] += dx * F;
    c->acc[3 * (size_t)j + 1] += dy * F;
    c->acc[3 * (size_t)j + 2] += dz * F;
    if (c->absacc) c->absacc[j] += fabs(F) * sqrt((double)d2);
    c->hit = 1;
}

static void field_core(const ktree *mt, int ns, const float *spos, const float *smass,
                       const float *sball2, const unsigned int *alive, const float period[3],
                       double *acc, double *absacc, unsigned int *touched)
{
    static const float zero_period[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    for (int i = 0; i < ns; ++i) {
        unsigned int m = alive[i];
        if (touched) touched[i] = 0;
        if (!m) continue;
        double b = sball2[i];
        double ih2 = 4.0 / b;
        double fnorm = M_1_PI * ih2 * ih2 * sqrt(ih2) * smass[i];
        for (int bit = 0; bit < 27; ++bit) {
            if (!(m & (1u << bit))) continue;
            int ix = bit / 9 - 1, iy = (bit / 3) % 3 - 1, iz = bit % 3 - 1;
            field_ctx c;
            c.mpos = mt->pos;
            c.cpos[0] = rep_coord(spos[3 * (size_t)i + 0], ix, period[0]);
            c.cpos[1] = rep_coord(spos[3 * (size_t)i + 1], iy, period[1]);
            c.cpos[2] = rep_coord(spos[3 * (size_t)i + 2], iz, period[2]);
            if (bit == ORIG_BIT) {
                c.cpos[0] = spos[3 * (size_t)i + 0];
                c.cpos[1] = spos[3 * (size_t)i + 1];
                c.cpos[2] = spos[3 * (size_t)i + 2];
            }
            c.b = sball2[i];
            c.ih2 = ih2;
            c.fnorm = fnorm;
            c.acc = acc;
            c.absacc = absacc;
            c.hit = 0;
            if (mt->n > 0) range_rec(mt, 0, c.cpos, b, zero_period, 0, sball2[i], field_visit, &c);
            if (c.hit && touched) touched[i] |= 1u << bit;
        }
    }
}

int or_field(int ns, const float *spos, const float *smass, const float *sball2,
             const unsigned int *alive_mask, int nm, const float *mpos,
             const float period[3], double *acc, double *absacc, unsigned int *touched_mask)
{
    ktree mt;
    kt_build(&mt, mpos, NULL, nm);
    memset(acc, 0, (size_t)nm * 3 * sizeof(double));
    if (absacc) memset(absacc, 0, (size_t)nm * sizeof(double));
    field_core(&mt, ns, spos, smass, sball2, alive_mask, period, acc, absacc, touched_mask);
    kt_free(&mt);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Friends of friends (kd.c:802-917).  Breadth-first flood over a tree */
/* whose nodes count their unassigned points, so finished subtrees are */
/* skipped; wholly contained cells are taken without pair tests.       */
/* ------------------------------------------------------------------ */

typedef struct {
    ktree *t;
    int *lab;
    int *fifo;
    int tail;
    const float *period;
    float tau2;
} fof_ctx;

static void fof_take(fof_ctx *c, int j, int g)
{
    c->lab[j] = g;
    c->fifo[c->tail++] = j;
    int k = c->t->leafof[j];
    while (k >= 0) { c->t->nd[k].open--; k = c->t->nd[k].parent; }
}

static void fof_rec(fof_ctx *c, int k, const float *q, int g)
{
    knode *nd = &c->t->nd[k];
    if (nd->open == 0) return;
    if (box_lb(q, nd, c->period, 1) >= c->tau2) return;
    if (box_ub(q, nd, c->period) < c->tau2) {
        for (int i = nd->first; i < nd->first + nd->count; ++i) {
            int j = c->t->idx[i];
            if (!c->lab[j]) fof_take(c, j, g);
        }
        return;
    }
    if (nd->left < 0) {
        for (int i = nd->first; i < nd->first + nd->count; ++i) {
            int j = c->t->idx[i];
            if (c->lab[j]) continue;
            if (sym_d2(q, c->t->pos + 3 * (size_t)j, c->period) < c->tau2) fof_take(c, j, g);
        }
        return;
    }
    fof_rec(c, nd->left, q, g);
    fof_rec(c, nd->left + 1, q, g);
}

typedef struct { int minio, root; } comp_t;
static int cmp_comp(const void *a, const void *b)
{
    const comp_t *x = (const comp_t *)a, *y = (const comp_t *)b;
    return (x->minio > y->minio) - (x->minio < y->minio);
}

int or_fof(int n, const float *pos, const float period[3], float tau, const int *iorder, int *grp)
{
    if (n == 0) return 0;
    ktree t;
    kt_build(&t, pos, NULL, n);
    t.leafof = (int *)malloc((size_t)n * sizeof(int));
    for (int k = 0; k < t.nn; ++k) {
        t.nd[k].open = t.nd[k].count;
        if (t.nd[k].left < 0)
            for (int i = t.nd[k].first; i < t.nd[k].first + t.nd[k].count; ++i) t.leafof[t.idx[i]] = k;
    }
    int *lab = (int *)calloc((size_t)n, sizeof(int));
    int *fifo = (int *)malloc((size_t)n * sizeof(int));
    fof_ctx c = {&t, lab, fifo, 0, period, tau * tau};
    int ng = 0;
    for (int s = 0; s < n; ++s) {
        if (lab[s]) continue;
        ++ng;
        int head = c.tail;
        fof_take(&c, s, ng);
        while (head < c.tail) {
            int i = fifo[head++];
            fof_rec(&c, 0, pos + 3 * (size_t)i, ng);
        }
    }
    /* canonical numbering: ascending smallest member iOrder */
    comp_t *cp = (comp_t *)malloc((size_t)ng * sizeof(comp_t));
    for (int g = 0; g < ng; ++g) { cp[g].minio = INT32_MAX; cp[g].root = g + 1; }
    for (int i = 0; i < n; ++i) {
        int g = lab[i] - 1;
        int io = iorder ? iorder[i] : i;
        if (io < cp[g].minio) cp[g].minio = io;
    }
    qsort(cp, (size_t)ng, sizeof(comp_t), cmp_comp);
    int *map = (int *)malloc((size_t)(ng + 1) * sizeof(int));
    for (int g = 0; g < ng; ++g) map[cp[g].root] = g + 1;
    for (int i = 0; i < n; ++i) grp[i] = map[lab[i]];
    free(map); free(cp); free(lab); free(fifo);
    kt_free(&t);
    return ng;
}

/* ------------------------------------------------------------------ */
/* Gravitational potentials (grav.h:11-31, grav.c:8-135).               */
/* ------------------------------------------------------------------ */

static inline float pair_pot(float d2, float twoh, int soft_type)
{
    double dir;
    if (soft_type == OR_PLUMMER) {
        dir = 1.0 / sqrt((double)d2 + 0.25 * (double)twoh * (double)twoh);
    } else {
        double r = sqrt((double)d2);
        if (r < twoh) {
            double dih = 2.0 / twoh;
            double u = r * dih;
            if (u < 1.0) {
                dir = dih * (7.0 / 5.0 - 2.0 / 3.0 * u * u + 3.0 / 10.0 * u * u * u * u
                             - 1.0 / 10.0 * u * u * u * u * u);
            } else {
                double ir = 1.0 / r;
                dir = -1.0 / 15.0 * ir + dih * (8.0 / 5.0 - 4.0 / 3.0 * u * u + u * u * u
                                                 - 3.0 / 10.0 * u * u * u * u
                                                 + 1.0 / 30.0 * u * u * u * u * u);
            }
        } else {
            dir = 1.0 / r;
        }
    }
    return (float)dir;
}

double or_exp2hub(double H0, double Omega0, double Lambda, double Quint, double a)
{
    /* cosmo.c:46-58 with dOmegaRad = 0 */
    double curv = 1.0 - Omega0 - Lambda - Quint;
    return H0 * sqrt(Omega0 * a + curv * a * a + Quint * a * a * sqrt(a)
                     + Lambda * a * a * a * a) / (a * a);
}

static inline float wrap_h(float d, float h)
{
    /* kd.c:1345-1350: if (dx > hx) dx -= 2*hx; if (dx <= -hx) dx += 2*hx */
    if (d > h) d -= 2 * h;
    if (d <= -h) d += 2 * h;
    return d;
}

int or_unbind_group(const or_params *par, int inType, int n, float *qr, float *qv,
                    float *qm, float *qs, int *qid, double *pot, const float rel[3],
                    float outVcm[3], float *outMass, float outBound[3], int *removed_ids)
{
    float fShift = (float)(1.0 / (1.0 + par->z));
    float fCosmo = (float)(fShift * or_exp2hub(par->H0, par->Omega0, par->Lambda,
                                               par->fQuintess, fShift));
    float hx = (float)(0.5 * par->period[0]);
    float G = par->G;
    double dMass = 0.0, rcm[3] = {0, 0, 0}, vcm[3] = {0, 0, 0};
    int nrem = 0;
    for (int i = 0; i < n; ++i) {
        dMass += qm[i];
        for (int j = 0; j < 3; ++j) {
            rcm[j] += (float)(qm[i] * qr[3 * i + j]);
            vcm[j] += (float)(qm[i] * qv[3 * i + j]);
        }
    }
    for (int j = 0; j < 3; ++j) { rcm[j] /= dMass; vcm[j] /= dMass; }
    int iMin = 0;
    while (1) {
        int iBig = 0;
        float fTotBig = -1.0f, fTotMin = 1.0f;
        iMin = 0;
        for (int i = 0; i < n; ++i) {
            float dv2 = 0.0f;
            for (int j = 0; j < 3; ++j) {
                float dv = (float)(fShift * (qv[3 * i + j] - vcm[j]) + fCosmo * (qr[3 * i + j] - rcm[j]));
                dv2 += dv * dv;
            }
            float fTot = (float)(0.5 * dv2 - pot[i] * (1.0 + par->z));
            if (fTot > fTotBig) { fTotBig = fTot; iBig = i; }
            if (fTot < fTotMin) { fTotMin = fTot; iMin = i; }
        }
        if (fTotBig < 0 || par->bNoUnbind) break;
        if (removed_ids) removed_ids[nrem] = qid[iBig];
        ++nrem;
        --n;
        if (n == 0) {
            dMass = 0.0;
            for (int j = 0; j < 3; ++j) vcm[j] = 0.0;
            break;
        }
        dMass -= qm[iBig];
        for (int j = 0; j < 3; ++j) {
            rcm[j] += qm[iBig] / dMass * (rcm[j] - qr[3 * iBig + j]);
            vcm[j] += qm[iBig] / dMass * (vcm[j] - qv[3 * iBig + j]);
        }
        /* swap iBig with the last member (kd.c:1435-1440) */
        for (int j = 0; j < 3; ++j) {
            float t = qr[3 * iBig + j]; qr[3 * iBig + j] = qr[3 * n + j]; qr[3 * n + j] = t;
            t = qv[3 * iBig + j]; qv[3 * iBig + j] = qv[3 * n + j]; qv[3 * n + j] = t;
        }
        { float t = qm[iBig]; qm[iBig] = qm[n]; qm[n] = t; }
        { float t = qs[iBig]; qs[iBig] = qs[n]; qs[n] = t; }
        { int t = qid[iBig]; qid[iBig] = qid[n]; qid[n] = t; }
        { double t = pot[iBig]; pot[iBig] = pot[n]; pot[n] = t; }
        if (inType == OR_DARK || inType == OR_STAR) {
            /* kdSubPot (grav.c:39-60) */
            const float *ps = qr + 3 * n;
            for (int i = 0; i < n; ++i) {
                float dx = ps[0] - qr[3 * i + 0];
                float dy = ps[1] - qr[3 * i + 1];
                float dz = ps[2] - qr[3 * i + 2];
                float d2 = (dx * dx + dy * dy) + dz * dz;
                float twoh = qs[n] + qs[i];
                float dir = pair_pot(d2, twoh, par->iSoftType);
                pot[i] -= (float)(G * qm[n] * dir);
            }
        }
    }
    *outMass = (float)dMass;
    for (int j = 0; j < 3; ++j) outVcm[j] = (float)vcm[j];
    for (int j = 0; j < 3; ++j) outBound[j] = wrap_h(qr[3 * iMin + j] + rel[j], hx);
    return n;
}

/* ------------------------------------------------------------------ */
/* Selection rules (kd.c:555-627, 669-699).                            */
/* ------------------------------------------------------------------ */

static inline int ptype(int io, int nGas, int nDark, int n)
{
    if (io < nGas) return OR_GAS;
    if (io < nGas + nDark) return OR_DARK;
    if (io < n) return OR_STAR;
    return 0;
}

static int scatter_rule(int inType, int t, int bGD, int bGO)
{
    switch (inType) {
    case OR_DARK: return 1;
    case OR_GAS: case OR_DARK | OR_GAS:
        return bGD || t == OR_GAS;
    case OR_STAR: case OR_DARK | OR_STAR:
        return t == OR_STAR;
    case OR_GAS | OR_STAR: case OR_DARK | OR_GAS | OR_STAR:
        if (bGD) return 1;
        if (t == OR_GAS) return 1;
        return t == OR_STAR && !bGO;
    }
    return 0;
}

static int cut_rule(const or_params *P, int inType, int t, float m, float rho, float temp)
{
    if (m > P->fMassMax) return 0;
    switch (inType) {
    case OR_DARK:
        return rho >= P->fDensMin;
    case OR_GAS: case OR_DARK | OR_GAS:
        if (P->bGasAndDark && t == OR_DARK && rho >= P->fDensMin) return 1;
        return t == OR_GAS && rho >= P->fDensMin && temp <= P->fTempMax;
    case OR_STAR: case OR_DARK | OR_STAR:
        return t == OR_STAR;
    case OR_GAS | OR_STAR: case OR_DARK | OR_GAS | OR_STAR:
        if (P->bGasAndDark && t == OR_DARK && rho >= P->fDensMin) return 1;
        if (t == OR_GAS) return rho >= P->fDensMin && temp <= P->fTempMax;
        return t == OR_STAR && !P->bGasOnly;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Move / prune (kd.c:702-793).                                        */
/* ------------------------------------------------------------------ */

static void move_one(float *r, const double *a, float fStep, const or_params *P)
{
    float ax = (float)a[0], ay = (float)a[1], az = (float)a[2];
    float ai = (float)sqrt((double)(ax * ax + ay * ay + az * az));
    if (ai > 0.0f) ai = (float)(fStep / sqrt((double)(ax * ax + ay * ay + az * az)));
    else ai = 0.0f;
    r[0] -= ai * ax;
    r[1] -= ai * ay;
    r[2] -= ai * az;
    for (int j = 0; j < 3; ++j) {
        if (r[j] > P->center[j] + 0.5 * P->period[j]) r[j] -= P->period[j];
        if (r[j] <= P->center[j] - 0.5 * P->period[j]) r[j] += P->period[j];
    }
}

/* ------------------------------------------------------------------ */
/* Whole pipeline.                                                      */
/* ------------------------------------------------------------------ */

typedef struct {
    int ns;
    float *pos, *mass, *ball2, *rho;  /* per scatterer */
    unsigned int *alive;              /* live copies */
    unsigned int *zeroed;             /* copies whose density was set to 0 */
    int *iorder;
} scat_t;

/* One smAccDensity pass (smooth1.c:408-518): field at active movers, minimum
 * density over touched copies, and the cut. Returns live copies. */
static int acc_pass(const or_params *P, scat_t *S, int nA, const float *mpos, double *acc,
                    int bInitial)
{
    unsigned int *touched = (unsigned int *)malloc((size_t)(S->ns ? S->ns : 1) * sizeof(unsigned int));
    ktree mt;
    kt_build(&mt, mpos, NULL, nA);
    memset(acc, 0, (size_t)nA * 3 * sizeof(double));
    field_core(&mt, S->ns, S->pos, S->mass, S->ball2, S->alive, P->period, acc, NULL, touched);
    kt_free(&mt);
    float fScatDens = 0.0f;
    for (int i = 0; i < S->ns; ++i) {
        unsigned int hit = touched[i] & S->alive[i];
        for (int bit = 0; bit < 27; ++bit) {
            if (!(hit & (1u << bit))) continue;
            float r = (S->zeroed[i] & (1u << bit)) ? 0.0f : S->rho[i];
            if (fScatDens == 0.0f) fScatDens = r;
            else if (r < fScatDens) fScatDens = r;
        }
        if (bInitial && !P->bNoScatterCut) S->zeroed[i] |= S->alive[i] & ~touched[i];
    }
    int live = 0;
    int w = 0;
    for (int i = 0; i < S->ns; ++i) {
        unsigned int keep = 0;
        for (int bit = 0; bit < 27; ++bit) {
            if (!(S->alive[i] & (1u << bit))) continue;
            float r = (S->zeroed[i] & (1u << bit)) ? 0.0f : S->rho[i];
            if (P->bNoScatterCut || r >= fScatDens) keep |= 1u << bit;
        }
        if (!keep) continue;
        live += __builtin_popcount(keep);
        S->pos[3 * w + 0] = S->pos[3 * i + 0];
        S->pos[3 * w + 1] = S->pos[3 * i + 1];
        S->pos[3 * w + 2] = S->pos[3 * i + 2];
        S->mass[w] = S->mass[i];
        S->ball2[w] = S->ball2[i];
        S->rho[w] = S->rho[i];
        S->alive[w] = keep;
        S->zeroed[w] = S->zeroed[i];
        S->iorder[w] = S->iorder[i];
        ++w;
    }
    S->ns = w;
    free(touched);
    return live;
}

typedef struct { int g, io; } gm_t;
static int cmp_gm(const void *a, const void *b)
{
    const gm_t *x = (const gm_t *)a, *y = (const gm_t *)b;
    if (x->g != y->g) return (x->g > y->g) - (x->g < y->g);
    return (x->io > y->io) - (x->io < y->io);
}

typedef struct {
    const float *pos, *mass, *soft;
    float rel[3];
    const float *period;
    int n;
    const float *qr, *qs;
    double *pot;
    float G;
    int soft_type;
} scoop_ctx;

static void scoop_visit(void *vctx, int j)
{
    scoop_ctx *c = (scoop_ctx *)vctx;
    const float *p = c->pos + 3 * (size_t)j;
    float nx = p[0] - c->rel[0], ny = p[1] - c->rel[1], nz = p[2] - c->rel[2];
    const float *L = c->period;
    if (nx > 0.5 * L[0]) nx -= L[0];
    if (nx <= -0.5 * L[0]) nx += L[0];
    if (ny > 0.5 * L[1]) ny -= L[1];
    if (ny <= -0.5 * L[1]) ny += L[1];
    if (nz > 0.5 * L[2]) nz -= L[2];
    if (nz <= -0.5 * L[2]) nz += L[2];
    for (int i = 0; i < c->n; ++i) {
        float dx = nx - c->qr[3 * i + 0];
        float dy = ny - c->qr[3 * i + 1];
        float dz = nz - c->qr[3 * i + 2];
        float d2 = (dx * dx + dy * dy) + dz * dz;
        float twoh = c->soft[j] + c->qs[i];
        float dir = pair_pot(d2, twoh, c->soft_type);
        c->pot[i] += (float)(c->G * c->mass[j] * dir);
    }
}

/* Unbinding, too-small and group radii (kd.c:1299-1466, 1251-1293,
 * 1627-1644) over groups G[0..nGroup) whose members grp[] names; shared by
 * the whole pipeline and the unbind-only mode.  Takes ownership of G. */
static int finish_run(const or_params *P, int inType, int n, const float *pos, const float *vel,
                      const float *mass, float *sft, int *grp, or_group *G, int nGroup,
                      or_group *groups, int cap_groups, or_result *res)
{
    /* 9. unbinding (kd.c:1299-1466) */
    if (P->bEps) for (int i = 0; i < n; ++i) sft[i] = P->fEps;
    res->nGroupFoF = nGroup - 1;
    if (P->verbose) printf("Groups before Unbind:%d\n", nGroup - 1);
    gm_t *order = (gm_t *)malloc((size_t)(n ? n : 1) * sizeof(gm_t));
    for (int i = 0; i < n; ++i) { order[i].g = grp[i]; order[i].io = i; }
    qsort(order, (size_t)n, sizeof(gm_t), cmp_gm);
    int n0 = G[0].nMembers;
    int *ung = (int *)malloc((size_t)(n0 ? n0 : 1) * sizeof(int));
    for (int i = 0; i < n0; ++i) ung[i] = order[i].io;
    ktree st;
    kt_build(&st, pos, ung, n0);
    float hx = (float)(0.5 * P->period[0]), hy = (float)(0.5 * P->period[1]),
          hz = (float)(0.5 * P->period[2]);
    int nUnbind = 0;
    int start = n0;
    int maxn = 1;
    for (int g = 1; g < nGroup; ++g) if (G[g].nMembers > maxn) maxn = G[g].nMembers;
    float *qr = (float *)malloc((size_t)maxn * 3 * sizeof(float));
    float *qv = (float *)malloc((size_t)maxn * 3 * sizeof(float));
    float *qm = (float *)malloc((size_t)maxn * sizeof(float));
    float *qs = (float *)malloc((size_t)maxn * sizeof(float));
    int *qid = (int *)malloc((size_t)maxn * sizeof(int));
    double *pot = (double *)malloc((size_t)maxn * sizeof(double));
    int *removed = (int *)malloc((size_t)maxn * sizeof(int));
    float fScoop2 = P->fScoop * P->fScoop;
    for (int g = 1; g < nGroup; ++g) {
        int gn = G[g].nMembers;
        int s0 = start;
        start += gn;
        if (gn >= P->nMaxMembers) continue;
        for (int i = 0; i < gn; ++i) {
            int io = order[s0 + i].io;
            float dx = wrap_h(pos[3 * (size_t)io + 0] - G[g].rel[0], hx);
            float dy = wrap_h(pos[3 * (size_t)io + 1] - G[g].rel[1], hy);
            float dz = wrap_h(pos[3 * (size_t)io + 2] - G[g].rel[2], hz);
            qr[3 * i + 0] = dx; qr[3 * i + 1] = dy; qr[3 * i + 2] = dz;
            for (int d = 0; d < 3; ++d) qv[3 * i + d] = vel[3 * (size_t)io + d];
            qm[i] = mass[io];
            qs[i] = sft[io];
            qid[i] = io;
        }
        /* kdCellPot (grav.c:8-36) */
        for (int i = 0; i < gn; ++i) pot[i] = 0.0;
        for (int i = 0; i < gn - 1; ++i) {
            for (int j = i + 1; j < gn; ++j) {
                float dx = qr[3 * i + 0] - qr[3 * j + 0];
                float dy = qr[3 * i + 1] - qr[3 * j + 1];
                float dz = qr[3 * i + 2] - qr[3 * j + 2];
                float d2 = (dx * dx + dy * dy) + dz * dz;
                float dir = pair_pot(d2, qs[i] + qs[j], P->iSoftType);
                pot[i] += (float)(P->G * qm[j] * dir);
                pot[j] += (float)(P->G * qm[i] * dir);
            }
        }
        /* kdAddScoopPot: always applied (kd.c:1379-1384 precedence) */
        if (n0 > 0) {
            scoop_ctx c = {pos, mass, sft, {G[g].rel[0], G[g].rel[1], G[g].rel[2]}, P->period,
                           gn, qr, qs, pot, P->G, P->iSoftType};
            range_rec(&st, 0, G[g].rCenter, fScoop2, P->period, 1, fScoop2, scoop_visit, &c);
        }
        float vout[3], bout[3], mout;
        int left = or_unbind_group(P, inType, gn, qr, qv, qm, qs, qid, pot, G[g].rel,
                                   vout, &mout, bout, removed);
        int nrm = gn - left;
        for (int r = 0; r < nrm; ++r) grp[removed[r]] = 0;
        nUnbind += nrm;
        G[g].nMembers = left;
        G[0].nMembers += nrm;
        G[g].fMass = mout;
        for (int d = 0; d < 3; ++d) { G[g].vcm[d] = vout[d]; G[g].rBound[d] = bout[d]; }
    }
    kt_free(&st);
    free(qr); free(qv); free(qm); free(qs); free(qid); free(pot); free(removed); free(ung);
    free(order);
    res->nUnbound = nUnbind;
    if (P->verbose) printf("Number of particles Unbound:%d\n", nUnbind);
    if (P->stopAfter == 2) {
        res->nGroup = nGroup - 1;
        for (int g = 0; g < nGroup && g < cap_groups; ++g) groups[g] = G[g];
        free(G);
        return 0;
    }
    /* 10. too small (kd.c:1251-1293) */
    int *map = (int *)malloc((size_t)nGroup * sizeof(int));
    int ng2 = 1;
    map[0] = 0;
    for (int g = 1; g < nGroup; ++g) {
        if (G[g].nMembers < P->nMinMembers || G[g].nMembers == 0) { map[g] = 0; continue; }
        map[g] = ng2;
        G[ng2] = G[g];
        ++ng2;
    }
    for (int i = 0; i < n; ++i) grp[i] = map[grp[i]];
    free(map);
    /* radius about the density centre (kd.c:1627-1644) */
    for (int g = 1; g < ng2; ++g) G[g].fRadius = 0.0f;
    for (int i = 0; i < n; ++i) {
        int g = grp[i];
        if (!g) continue;
        float fRad = 0.0f;
        for (int d = 0; d < 3; ++d) {
            float del = pos[3 * (size_t)i + d] - G[g].rCenter[d];
            if (del > 0.5 * P->period[d]) del -= P->period[d];
            if (del <= -0.5 * P->period[d]) del += P->period[d];
            fRad += del * del;
        }
        fRad = (float)sqrt((double)fRad);
        if (fRad > G[g].fRadius) G[g].fRadius = fRad;
    }
    res->nGroup = ng2 - 1;
    if (P->verbose) printf("Number of Groups:%d\n", ng2 - 1);
    for (int g = 0; g < ng2 && g < cap_groups; ++g) groups[g] = G[g];
    free(G);
    fflush(stdout);
    return 0;
}

int or_run(const or_params *P, int nGas, int nDark, int nStar, double time,
           const float *pos, const float *vel, const float *mass, const float *soft,
           const float *temp, int *grp, or_group *groups, int cap_groups, float *rho_out,
           float *ball2_out, float *moved, or_result *res)
{
    (void)time;
    int n = nGas + nDark + nStar;
    memset(res, 0, sizeof(*res));
    int inType = (nDark ? OR_DARK : 0) | (nGas ? OR_GAS : 0) | (nStar ? OR_STAR : 0);
    float *sft = (float *)malloc((size_t)(n ? n : 1) * sizeof(float));
    memcpy(sft, soft, (size_t)n * sizeof(float));
    /* 1. scatter-active particles (kd.c:669-693) */
    int *sidx = (int *)malloc((size_t)(n ? n : 1) * sizeof(int));
    int ns = 0;
    for (int i = 0; i < n; ++i)
        if (scatter_rule(inType, ptype(i, nGas, nDark, n), P->bGasAndDark, P->bGasOnly)) sidx[ns++] = i;
    res->nScatterInit = ns;
    if (ns < P->nSmooth) { free(sft); free(sidx); return -2; }   /* smooth1.c:12 */
    /* 2. density (smooth1.c:132-276) */
    float *spos = (float *)malloc((size_t)ns * 3 * sizeof(float));
    float *smass = (float *)malloc((size_t)ns * sizeof(float));
    for (int s = 0; s < ns; ++s) {
        for (int d = 0; d < 3; ++d) spos[3 * s + d] = pos[3 * (size_t)sidx[s] + d];
        smass[s] = mass[sidx[s]];
    }
    float *sb2 = (float *)malloc((size_t)ns * sizeof(float));
    double *srho = (double *)malloc((size_t)ns * sizeof(double));
    or_knn_ball2(ns, spos, P->nSmooth, P->period, sb2);
    or_density(ns, spos, smass, sb2, P->period, srho);
    float *rho = (float *)calloc((size_t)(n ? n : 1), sizeof(float));
    for (int s = 0; s < ns; ++s) rho[sidx[s]] = (float)srho[s];
    if (rho_out) memcpy(rho_out, rho, (size_t)n * sizeof(float));
    if (ball2_out) {
        for (int i = 0; i < n; ++i) ball2_out[i] = -1.0f;
        for (int s = 0; s < ns; ++s) ball2_out[sidx[s]] = sb2[s];
    }
    /* 3. replicas */
    scat_t S;
    S.ns = ns; S.pos = spos; S.mass = smass; S.ball2 = sb2; S.iorder = sidx;
    S.rho = (float *)malloc((size_t)ns * sizeof(float));
    for (int s = 0; s < ns; ++s) S.rho[s] = (float)srho[s];
    S.alive = (unsigned int *)malloc((size_t)ns * sizeof(unsigned int));
    S.zeroed = (unsigned int *)calloc((size_t)ns, sizeof(unsigned int));
    or_replica_mask(ns, spos, sb2, P->period, P->center, P->periodic, S.alive);
    for (int s = 0; s < ns; ++s) res->nExtraScat += __builtin_popcount(S.alive[s]) - 1;
    if (P->verbose && P->periodic) printf("nExtraScat:%d\n", res->nExtraScat);
    /* 4. movers (kd.c:630-666) */
    int nMove = 0;
    int *mio = (int *)malloc((size_t)(n ? n : 1) * sizeof(int));
    for (int i = 0; i < n; ++i)
        if (cut_rule(P, inType, ptype(i, nGas, nDark, n), mass[i], rho[i], temp[i])) mio[nMove++] = i;
    res->nMove = nMove;
    float *mr = (float *)malloc((size_t)(nMove ? nMove : 1) * 3 * sizeof(float));
    float *mold = (float *)malloc((size_t)(nMove ? nMove : 1) * 3 * sizeof(float));
    float *ar = (float *)malloc((size_t)(nMove ? nMove : 1) * 3 * sizeof(float));
    int *act = (int *)malloc((size_t)(nMove ? nMove : 1) * sizeof(int));
    double *acc = (double *)malloc((size_t)(nMove ? nMove : 1) * 3 * sizeof(double));
    for (int m = 0; m < nMove; ++m) {
        for (int d = 0; d < 3; ++d) mr[3 * m + d] = mold[3 * m + d] = pos[3 * (size_t)mio[m] + d];
        act[m] = m;
    }
    int nA = nMove;
    /* 5. initial pass (main.c:394-404) */
    int bInitial = (inType == OR_DARK) || P->bForceInitialCut;
    float fStep = P->fStep;
    float fCvg2 = P->fCvg * P->fCvg;
    int nScat;
#define GATHER_ACTIVE() do { for (int a_ = 0; a_ < nA; ++a_) for (int d_ = 0; d_ < 3; ++d_) ar[3 * a_ + d_] = mr[3 * act[a_] + d_]; } while (0)
#define MOVE_ACTIVE(step) do { for (int a_ = 0; a_ < nA; ++a_) move_one(mr + 3 * act[a_], acc + 3 * a_, (step), P); } while (0)
    GATHER_ACTIVE();
    nScat = acc_pass(P, &S, nA, ar, acc, bInitial);
    if (P->verbose) printf("Ittr:%d nActive:%d nScatter:%d\n", 0, nA, nScat);
    MOVE_ACTIVE(fStep);
    int nIttr = 1;
    while (nA) {
        if (P->maxIter > 0 && nIttr > P->maxIter) break;
        for (int s = 0; s < PRUNE_STEPS; ++s) {
            GATHER_ACTIVE();
            nScat = acc_pass(P, &S, nA, ar, acc, 0);
            MOVE_ACTIVE(fStep);
        }
        /* prune (kd.c:735-793) */
        float hx = (float)(0.5 * P->period[0]), hy = (float)(0.5 * P->period[1]),
              hz = (float)(0.5 * P->period[2]);
        int w = 0;
        for (int a = 0; a < nA; ++a) {
            int m = act[a];
            float dx = mr[3 * m + 0] - mold[3 * m + 0];
            float dy = mr[3 * m + 1] - mold[3 * m + 1];
            float dz = mr[3 * m + 2] - mold[3 * m + 2];
            if (dx > hx) dx -= 2 * hx;
            if (dx <= -hx) dx += 2 * hx;
            if (dy > hy) dy -= 2 * hy;
            if (dy <= -hy) dy += 2 * hy;
            if (dz > hz) dz -= 2 * hz;
            if (dz <= -hz) dz += 2 * hz;
            float dr2 = (dx * dx + dy * dy) + dz * dz;
            if (dr2 >= fCvg2) act[w++] = m;
        }
        nA = w;
        for (int a = 0; a < nA; ++a)
            for (int d = 0; d < 3; ++d) mold[3 * act[a] + d] = mr[3 * act[a] + d];
        if (P->verbose) printf("Ittr:%d nActive:%d nScatter:%d\n", nIttr, nA, nScat);
        ++nIttr;
    }
    res->nIter = nIttr - 1;
    /* 6. friends of friends over all movers (kd.c:802-917) */
    int *mgrp = (int *)malloc((size_t)(nMove ? nMove : 1) * sizeof(int));
    int nFoF = or_fof(nMove, mr, P->period, P->fTau, mio, mgrp);
    /* 7. micro-steps (main.c:431-438) */
    nA = nMove;
    for (int m = 0; m < nMove; ++m) act[m] = m;
    for (int s = 0; s < PRUNE_STEPS; ++s) {
        GATHER_ACTIVE();
        nScat = acc_pass(P, &S, nA, ar, acc, 0);
        MOVE_ACTIVE((float)(MICRO_STEP * fStep));
        if (P->verbose) printf("Microstep:%d nScatter:%d\n", s + 1, nScat);
    }
    res->nScatFinal = nScat;
#undef GATHER_ACTIVE
#undef MOVE_ACTIVE
    if (moved) {
        memcpy(moved, pos, (size_t)n * 3 * sizeof(float));
        for (int m = 0; m < nMove; ++m)
            for (int d = 0; d < 3; ++d) moved[3 * (size_t)mio[m] + d] = mr[3 * m + d];
    }
    /* 8. groups: members, mass, rel, centre, vcm (kd.c:969-1075) */
    int nGroup = nFoF + 1;
    for (int i = 0; i < n; ++i) grp[i] = 0;
    for (int m = 0; m < nMove; ++m) grp[mio[m]] = mgrp[m];
    or_group *G = (or_group *)calloc((size_t)nGroup, sizeof(or_group));
    double *gsum = (double *)calloc((size_t)nGroup * 7, sizeof(double));
    for (int i = n - 1; i >= 0; --i) {
        int g = grp[i];
        G[g].nMembers++;
        if (!g) continue;
        for (int d = 0; d < 3; ++d) G[g].rel[d] = pos[3 * (size_t)i + d];   /* smallest iOrder wins */
    }
    for (int i = 0; i < n; ++i) {
        int g = grp[i];
        if (!g) continue;
        gsum[7 * g + 6] += mass[i];
        for (int d = 0; d < 3; ++d) gsum[7 * g + 3 + d] += (float)(mass[i] * vel[3 * (size_t)i + d]);
    }
    for (int m = 0; m < nMove; ++m) {
        int g = mgrp[m];
        for (int d = 0; d < 3; ++d) {
            float del = mr[3 * m + d] - G[g].rel[d];
            if (del > 0.5 * P->period[d]) del -= P->period[d];
            if (del <= -0.5 * P->period[d]) del += P->period[d];
            gsum[7 * g + d] += del;
        }
    }
    for (int g = 1; g < nGroup; ++g) {
        G[g].fMass = (float)gsum[7 * g + 6];
        for (int d = 0; d < 3; ++d) {
            float c = (float)gsum[7 * g + d];
            c /= G[g].nMembers;
            c += G[g].rel[d];
            if (c > P->center[d] + 0.5 * P->period[d]) c -= P->period[d];
            if (c <= P->center[d] - 0.5 * P->period[d]) c += P->period[d];
            G[g].rCenter[d] = c;
            G[g].vcm[d] = (float)gsum[7 * g + 3 + d] / G[g].fMass;
        }
    }
    free(gsum);
    if (P->stopAfter == 1) {
        res->nGroupFoF = nGroup - 1;
        res->nGroup = nGroup - 1;
        for (int g = 0; g < nGroup && g < cap_groups; ++g) groups[g] = G[g];
        free(G);
        free(mgrp); free(mio); free(mr); free(mold); free(ar); free(act); free(acc);
        free(spos); free(smass); free(sb2); free(srho); free(rho); free(sidx); free(sft);
        free(S.rho); free(S.alive); free(S.zeroed);
        return 0;
    }
    int rc = finish_run(P, inType, n, pos, vel, mass, sft, grp, G, nGroup, groups, cap_groups, res);
    free(mgrp); free(mio); free(mr); free(mold); free(ar); free(act); free(acc);
    free(spos); free(smass); free(sb2); free(srho); free(rho); free(sidx); free(sft);
    free(S.rho); free(S.alive); free(S.zeroed);
    return rc;
}

/* Unbind-only mode (main.c:348-372): kdInGroup (kd.c:920-962) reads the
 * group ids, kdInitpGroup (kd.c:969-1005) sums the float masses in iOrder
 * and leaves rel at the largest-iOrder member, kdReadCenter (kd.c:1083-1196)
 * takes rCenter and vcm from the .gtp records (centers: 6 floats per group
 * 1..nGroup-1, rCenter then vcm) or, with centers NULL, the float
 * mass-weighted centre and velocity.  Then unbinding and too-small as in
 * or_run.  grp[n] is read and rewritten. */
int or_run_unbind(const or_params *P, int nGas, int nDark, int nStar, const float *pos,
                  const float *vel, const float *mass, const float *soft, int *grp,
                  const float *centers, or_group *groups, int cap_groups, or_result *res)
{
    int n = nGas + nDark + nStar;
    memset(res, 0, sizeof(*res));
    int inType = (nDark ? OR_DARK : 0) | (nGas ? OR_GAS : 0) | (nStar ? OR_STAR : 0);
    int nGroup = 1;
    for (int i = 0; i < n; ++i) {
        if (grp[i] < 0) return -1;
        if (grp[i] + 1 > nGroup) nGroup = grp[i] + 1;
    }
    or_group *G = (or_group *)calloc((size_t)nGroup, sizeof(or_group));
    for (int i = 0; i < n; ++i) {
        int g = grp[i];
        G[g].nMembers++;
        if (!g) continue;
        G[g].fMass += mass[i];
        for (int d = 0; d < 3; ++d) G[g].rel[d] = pos[3 * (size_t)i + d];
    }
    if (centers) {
        for (int g = 1; g < nGroup; ++g)
            for (int d = 0; d < 3; ++d) {
                G[g].rCenter[d] = centers[6 * (size_t)(g - 1) + d];
                G[g].vcm[d] = centers[6 * (size_t)(g - 1) + 3 + d];
            }
    } else {
        for (int i = 0; i < n; ++i) {
            int g = grp[i];
            if (!g) continue;
            for (int d = 0; d < 3; ++d) {
                float del = pos[3 * (size_t)i + d] - G[g].rel[d];
                if (del > 0.5 * P->period[d]) del -= P->period[d];
                if (del <= -0.5 * P->period[d]) del += P->period[d];
                G[g].rCenter[d] += mass[i] * del;
                G[g].vcm[d] += mass[i] * vel[3 * (size_t)i + d];
            }
        }
        for (int g = 1; g < nGroup; ++g)
            for (int d = 0; d < 3; ++d) {
                G[g].rCenter[d] /= G[g].fMass;
                G[g].rCenter[d] += G[g].rel[d];
                if (G[g].rCenter[d] > P->center[d] + 0.5 * P->period[d]) G[g].rCenter[d] -= P->period[d];
                if (G[g].rCenter[d] <= P->center[d] - 0.5 * P->period[d]) G[g].rCenter[d] += P->period[d];
                G[g].vcm[d] /= G[g].fMass;
            }
    }
    float *sft = (float *)malloc((size_t)(n ? n : 1) * sizeof(float));
    memcpy(sft, soft, (size_t)n * sizeof(float));
    int rc = finish_run(P, inType, n, pos, vel, mass, sft, grp, G, nGroup, groups, cap_groups, res);
    free(sft);
    return rc;
}

/* ------------------------------------------------------------------ */
/* FP64 references for the adjoint checks (no reference counterpart:  */
/* skid never differentiates its density).                             */
/* ------------------------------------------------------------------ */

typedef struct {
    int *v;
    int n, cap;
} ivec;

static void ivec_push(ivec *a, int x)
{
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 256;
        a->v = (int *)realloc(a->v, (size_t)a->cap * sizeof(int));
    }
    a->v[a->n++] = x;
}

static void list_visit(void *ctx, int j) { ivec_push((ivec *)ctx, j); }

/* M4 kernel profile f(q), f'(q), for q < 2 (0 beyond). */
static void m4(double q, double *f, double *fp)
{
    if (q < 1.0) {
        *f = 1.0 - 1.5 * q * q + 0.75 * q * q * q;
        *fp = -3.0 * q + 2.25 * q * q;
    } else if (q < 2.0) {
        double t = 2.0 - q;
        *f = 0.25 * t * t * t;
        *fp = -0.75 * t * t;
    } else {
        *f = 0.0;
        *fp = 0.0;
    }
}

static double dmin_image(double d, float L)
{
    if (L < 0.25f * FLT_MAX) {
        if (d > 0.5 * L) d -= L;
        if (d < -0.5 * L) d += L;
    }
    return d;
}

typedef struct {
    int n;
    const double *X;     /* 3n */
    const float *mass, *w, *period;
    const int *off, *nbr, *kth;   /* ball lists (CSR, self included), k-th neighbour */
} dens_sys;

static double ddist(const dens_sys *S, int i, int j, double u[3])
{
    double r2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        u[d] = dmin_image(S->X[3 * (size_t)i + d] - S->X[3 * (size_t)j + d], S->period[d]);
        r2 += u[d] * u[d];
    }
    return sqrt(r2);
}

/* S_i = sum_{j in B(i)} P_ij W(r_ij, h_i), h_i = |x_i - x_K(i)| / 2. */
static double row_sum(const dens_sys *S, int i)
{
    double u[3];
    double h = 0.5 * ddist(S, i, S->kth[i], u);
    double s = 0.0;
    for (int k = S->off[i]; k < S->off[i + 1]; ++k) {
        int j = S->nbr[k];
        double r = ddist(S, i, j, u), f, fp;
        m4(r / h, &f, &fp);
        double P = 0.5 * ((double)S->w[i] * S->mass[j] + (double)S->w[j] * S->mass[i]);
        s += P * f / (M_PI * h * h * h);
    }
    return s;
}

/* d S_i / d x_p (analytic, FP64); adds sum |term| to *abs. */
static void row_grad(const dens_sys *S, int i, int p, double g[3], double *abs)
{
    double u[3];
    int K = S->kth[i];
    double rK = ddist(S, i, K, u);
    double uK[3] = {u[0], u[1], u[2]};   /* x_i - x_K */
    double h = 0.5 * rK;
    double H = 0.0;
    for (int k = S->off[i]; k < S->off[i + 1]; ++k) {
        int j = S->nbr[k];
        double r = ddist(S, i, j, u), f, fp;
        double q = r / h;
        m4(q, &f, &fp);
        double P = 0.5 * ((double)S->w[i] * S->mass[j] + (double)S->w[j] * S->mass[i]);
        H += -P * (3.0 * f + q * fp) / (M_PI * h * h * h * h);
        if (r > 0.0 && (i == p || j == p)) {
            double c = P * fp / (M_PI * h * h * h * h) / r;   /* dW/dr / r */
            double sg = (i == p) ? 1.0 : -1.0;              /* d r / d x_p */
            double t2 = 0.0;
            for (int d = 0; d < 3; ++d) {
                g[d] += sg * c * u[d];
                t2 += c * u[d] * c * u[d];
            }
            *abs += sqrt(t2);
        }
    }
    /* h_i = |x_i - x_K| / 2: d h / d x_i = (x_i - x_K)/(4 h), d h / d x_K = -(...) */
    if (i == p || K == p) {
        double sg = (i == p) ? 1.0 : -1.0;
        double t2 = 0.0;
        for (int d = 0; d < 3; ++d) {
            double t = sg * H * uK[d] / (4.0 * h);
            g[d] += t;
            t2 += t * t;
        }
        *abs += sqrt(t2);
    }
}

int or_density_adjoint_check(int n, const float *pos, const float *mass, const float *w, int k,
                             const float period[3], int nsel, const int *sel, double hfd,
                             double *grad_an, double *grad_fd, double *absterm, int *lists_ok)
{
    return or_density_adjoint_check2(n, pos, mass, w, k, period, nsel, sel, hfd, grad_an, grad_fd,
                                     NULL, absterm, lists_ok);
}

int or_density_adjoint_check2(int n, const float *pos, const float *mass, const float *w, int k,
                              const float period[3], int nsel, const int *sel, double hfd,
                              double *grad_an, double *grad_fd, double *grad_fd_half,
                              double *absterm, int *lists_ok)
{
    if (k < 2 || k > n) return -1;
    float *ball2 = (float *)malloc((size_t)n * sizeof(float));
    or_knn_ball2(n, pos, k, period, ball2);
    ktree t;
    kt_build(&t, pos, NULL, n);
    int *off = (int *)malloc(((size_t)n + 1) * sizeof(int));
    int *kth = (int *)malloc((size_t)n * sizeof(int));
    ivec all = {0, 0, 0};
    int ok = 1;
    for (int i = 0; i < n; ++i) {
        off[i] = all.n;
        const float *q = pos + 3 * (size_t)i;
        float fr2 = nextafterf(ball2[i], INFINITY);
        range_rec(&t, 0, q, (double)ball2[i] * (1.0 + 1e-5) + 1e-30, period, 1, fr2, list_visit, &all);
        kth[i] = -1;
        for (int a = off[i]; a < all.n; ++a) {
            int j = all.v[a];
            if (j != i && or_d2(q, pos + 3 * (size_t)j, period) == ball2[i] && (kth[i] < 0 || j < kth[i]))
                kth[i] = j;
        }
        if (kth[i] < 0) ok = 0;
    }
    off[n] = all.n;
    kt_free(&t);
    *lists_ok = ok;
    if (!ok) {
        free(ball2); free(off); free(kth); free(all.v);
        return -2;
    }
    /* rows containing each particle */
    int *roff = (int *)calloc((size_t)n + 1, sizeof(int));
    for (int a = 0; a < all.n; ++a) roff[all.v[a] + 1]++;
    for (int i = 0; i < n; ++i) roff[i + 1] += roff[i];
    int *rows = (int *)malloc((size_t)(all.n ? all.n : 1) * sizeof(int));
    int *fill = (int *)malloc((size_t)n * sizeof(int));
    memcpy(fill, roff, (size_t)n * sizeof(int));
    for (int i = 0; i < n; ++i)
        for (int a = off[i]; a < off[i + 1]; ++a) rows[fill[all.v[a]]++] = i;
    double *X = (double *)malloc(3 * (size_t)n * sizeof(double));
    for (size_t a = 0; a < 3 * (size_t)n; ++a) X[a] = pos[a];
    dens_sys S = {n, X, mass, w, period, off, all.v, kth};
    for (int s = 0; s < nsel; ++s) {
        int p = sel[s];
        double g[3] = {0, 0, 0}, ab = 0.0;
        /* rows that depend on x_p: p's own and every row whose ball holds p
         * (which includes every row with K(i) == p) */
        for (int a = roff[p]; a < roff[p + 1]; ++a) row_grad(&S, rows[a], p, g, &ab);
        int own = 0;
        for (int a = roff[p]; a < roff[p + 1]; ++a) own |= rows[a] == p;
        if (!own) row_grad(&S, p, p, g, &ab);
        for (int d = 0; d < 3; ++d) {
            grad_an[3 * (size_t)s + d] = g[d];
            double x0 = X[3 * (size_t)p + d], up = 0.0, dn = 0.0;
            X[3 * (size_t)p + d] = x0 + hfd;
            for (int a = roff[p]; a < roff[p + 1]; ++a) up += row_sum(&S, rows[a]);
            if (!own) up += row_sum(&S, p);
            X[3 * (size_t)p + d] = x0 - hfd;
            for (int a = roff[p]; a < roff[p + 1]; ++a) dn += row_sum(&S, rows[a]);
            if (!own) dn += row_sum(&S, p);
            X[3 * (size_t)p + d] = x0;
            grad_fd[3 * (size_t)s + d] = (up - dn) / (2.0 * hfd);
            if (grad_fd_half) {
                /* the same with half the step: Richardson extrapolation
                 * (4 D(h/2) - D(h)) / 3 cancels the O(h^2) truncation error */
                double up2 = 0.0, dn2 = 0.0;
                X[3 * (size_t)p + d] = x0 + 0.5 * hfd;
                for (int a = roff[p]; a < roff[p + 1]; ++a) up2 += row_sum(&S, rows[a]);
                if (!own) up2 += row_sum(&S, p);
                X[3 * (size_t)p + d] = x0 - 0.5 * hfd;
                for (int a = roff[p]; a < roff[p + 1]; ++a) dn2 += row_sum(&S, rows[a]);
                if (!own) dn2 += row_sum(&S, p);
                X[3 * (size_t)p + d] = x0;
                grad_fd_half[3 * (size_t)s + d] = (up2 - dn2) / hfd;
            }
        }
        absterm[s] = ab;
    }
    free(X); free(fill); free(rows); free(roff);
    free(ball2); free(off); free(kth); free(all.v);
    return 0;
}

/* Density field rho_f(y) = sum_j m_j W(|y - x_j|, h_j) of ns scatterers
 * (nearest periodic image, h_j^2 = ball2_j / 4), FP64: its gradient at nq
 * points analytically and by central differences of step hfd, and the sum
 * of |term| per point. */
int or_field_grad_check(int ns, const float *spos, const float *smass, const float *sball2,
                        const float period[3], int nq, const float *ypos, double hfd,
                        double *grad_an, double *grad_fd, double *absterm)
{
    for (int q = 0; q < nq; ++q) {
        double y[3] = {ypos[3 * (size_t)q], ypos[3 * (size_t)q + 1], ypos[3 * (size_t)q + 2]};
        double g[3] = {0, 0, 0}, ab = 0.0, fp_[3] = {0, 0, 0}, fm_[3] = {0, 0, 0};
        for (int j = 0; j < ns; ++j) {
            double h = 0.5 * sqrt((double)sball2[j]);
            double u[3], r2 = 0.0;
            for (int d = 0; d < 3; ++d) {
                u[d] = dmin_image(y[d] - spos[3 * (size_t)j + d], period[d]);
                r2 += u[d] * u[d];
            }
            if (r2 >= 4.0 * h * h * (1.0 + 1e-6)) continue;
            double r = sqrt(r2), f, fp;
            double c0 = smass[j] / (M_PI * h * h * h);
            m4(r / h, &f, &fp);
            if (r > 0.0) {
                double c = c0 * fp / h / r, t2 = 0.0;
                for (int d = 0; d < 3; ++d) {
                    g[d] += c * u[d];
                    t2 += c * u[d] * c * u[d];
                }
                ab += sqrt(t2);
            }
            for (int d = 0; d < 3; ++d) {
                for (int sgn = 0; sgn < 2; ++sgn) {
                    double v[3] = {u[0], u[1], u[2]};
                    v[d] += sgn ? -hfd : hfd;
                    double rr = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]), ff, ffp;
                    m4(rr / h, &ff, &ffp);
                    if (sgn) fm_[d] += c0 * ff; else fp_[d] += c0 * ff;
                }
            }
        }
        for (int d = 0; d < 3; ++d) {
            grad_an[3 * (size_t)q + d] = g[d];
            grad_fd[3 * (size_t)q + d] = (fp_[d] - fm_[d]) / (2.0 * hfd);
        }
        absterm[q] = ab;
    }
    return 0;
}
