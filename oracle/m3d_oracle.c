/* m3d_oracle.c -- CPU restatement, in plain C99, of the reference's octree
 * finite-volume forward + adjoint solve.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load this library, and only as a checker or
 * as the timed CPU baseline.  The GPU product never links or calls it.
 *
 * Every function cites the reference file:line it restates (paths relative
 * to the reference project root).  Arithmetic follows the reference's
 * operation order so that, built with -ffp-contract=off, results agree with
 * the reference compiled by oracle/build_ref.sh to the last bit on the golden
 * cases (tests/golden).  Complex arithmetic uses the C99 complex type, which
 * GCC lowers to the same routines as std::complex<double>; |z|^2 is computed
 * as cabs(z)^2 because that is what libstdc++'s std::norm does.
 */
#include "m3d_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

#define M3D_PI 3.14159265358979323846
#define M3D_MU0 (4.0e-7 * M3D_PI)
#define M3D_TWOPI (2.0 * M3D_PI)

/* ------------------------------------------------------------------------ */
/* small containers                                                          */
/* ------------------------------------------------------------------------ */

typedef struct { int* a; int n, cap; } ivec;

static void iv_push(ivec* v, int x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 4;
        v->a = (int*)realloc(v->a, sizeof(int) * (size_t)v->cap);
    }
    v->a[v->n++] = x;
}

static void* xcalloc(size_t n, size_t sz) {
    void* p = calloc(n ? n : 1, sz);
    if (!p) { fprintf(stderr, "m3d_oracle: out of memory\n"); abort(); }
    return p;
}

/* Open-addressing hash map from a 3 x int64 key to int, insertion-ordered ids
 * are assigned by the caller (replaces the reference's std::map lookups whose
 * ids are creation order). */
typedef struct { int64_t k[3]; int v; int used; } hslot;
typedef struct { hslot* s; size_t cap, n; } hmap;

static uint64_t hkey(const int64_t* k) {
    uint64_t h = 1469598103934665603ull;
    for (int i = 0; i < 3; ++i) {
        uint64_t x = (uint64_t)k[i];
        x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33;
        h = (h ^ x) * 1099511628211ull;
    }
    return h;
}

static void hm_init(hmap* m, size_t expect) {
    size_t c = 16;
    while (c < 2 * expect + 16) c <<= 1;
    m->s = (hslot*)xcalloc(c, sizeof(hslot));
    m->cap = c; m->n = 0;
}

static void hm_free(hmap* m) { free(m->s); m->s = NULL; }

static void hm_grow(hmap* m);

/* returns pointer to value slot; *found set accordingly; inserts if absent */
static int* hm_get(hmap* m, const int64_t* k, int insert, int* found) {
    if (insert && 2 * (m->n + 1) > m->cap) hm_grow(m);
    size_t i = hkey(k) & (m->cap - 1);
    for (;;) {
        hslot* s = &m->s[i];
        if (!s->used) {
            *found = 0;
            if (!insert) return NULL;
            s->used = 1; s->k[0] = k[0]; s->k[1] = k[1]; s->k[2] = k[2]; s->v = -1;
            m->n++;
            return &s->v;
        }
        if (s->k[0] == k[0] && s->k[1] == k[1] && s->k[2] == k[2]) { *found = 1; return &s->v; }
        i = (i + 1) & (m->cap - 1);
    }
}

static void hm_grow(hmap* m) {
    hslot* old = m->s;
    size_t oc = m->cap;
    m->cap = oc * 2;
    m->s = (hslot*)xcalloc(m->cap, sizeof(hslot));
    m->n = 0;
    for (size_t i = 0; i < oc; ++i)
        if (old[i].used) { int f; *hm_get(m, old[i].k, 1, &f) = old[i].v; }
    free(old);
}

static int hm_find(hmap* m, const int64_t* k) {
    int f;
    int* p = hm_get(m, k, 0, &f);
    return p ? *p : -1;
}

/* |z|^2 as libstdc++ std::norm computes it for double */
static inline double cnorm2(cplx z) { double a = cabs(z); return a * a; }

/* ------------------------------------------------------------------------ */
/* mesh (leaf list)                                                          */
/* ------------------------------------------------------------------------ */

typedef struct {
    double xmin, xmax, ymin, ymax, zmin, zmax;
    int min_level, max_level;
    int nc;
    const int* level;
    const double *cx, *cy, *cz;
    const int* type;
} mesh_t;

/* octree_mesh.cpp:581-590 */
static void cell_size_xyz(const mesh_t* m, int c, double* dx, double* dy, double* dz) {
    double h = 1.0 / (1 << m->level[c]);
    *dx = h * (m->xmax - m->xmin);
    *dy = h * (m->ymax - m->ymin);
    *dz = h * (m->zmax - m->zmin);
}

/* octree_mesh.cpp:560 */
static double cell_size_min(const mesh_t* m, int c) {
    double dx = m->xmax - m->xmin, dy = m->ymax - m->ymin, dz = m->zmax - m->zmin;
    double mn = dx < dy ? dx : dy;
    mn = mn < dz ? mn : dz;
    double h = (double)(1 << (19 - m->level[c])) / (double)(1 << 19);
    return h * mn;
}

/* ------------------------------------------------------------------------ */
/* staggered grid  (src/octree/staggered_grid.cpp)                           */
/* ------------------------------------------------------------------------ */

typedef struct {
    int ne, nf, nc;
    double *ex, *ey, *ez, *elen;
    int* edir;
    ivec* adj;         /* per edge adjacent cells */
    int ecap;
    double *fx, *fy, *fz, *farea;
    int *fnorm, *fcm, *fcp;
    int* fedge;        /* [nf][4], -1 = absent */
    int* fnedge;
    int fcap;
    int* hface; int nhface;   /* [nhface][5] coarse + 4 fine */
    int* hedge; int nhedge;   /* [nhedge][3] coarse + 2 fine */
    int *ce_ptr, *ce_id;      /* cell -> edges */
    double* ce_frac;
} grid_t;

typedef struct {
    double dx, dy, dz, x0, y0, z0, quant;
} gctx_t;

/* staggered_grid.cpp:31-50 */
static void quantize(const gctx_t* g, double px, double py, double pz, int dir, int64_t* k) {
    k[0] = (int64_t)llround((px - g->x0) / g->dx * g->quant);
    k[1] = (int64_t)llround((py - g->y0) / g->dy * g->quant);
    k[2] = (int64_t)llround((pz - g->z0) / g->dz * g->quant) * 4 + dir;
}

/* staggered_grid.cpp:58-67 */
static void cell_half(const mesh_t* m, const gctx_t* g, int c, double* ch) {
    ch[0] = m->cx[c]; ch[1] = m->cy[c]; ch[2] = m->cz[c];
    double h = 1.0 / (1 << m->level[c]);
    ch[3] = h * g->dx / 2.0;
    ch[4] = h * g->dy / 2.0;
    ch[5] = h * g->dz / 2.0;
}

static int add_edge(grid_t* G, hmap* em, const gctx_t* g, double x, double y, double z, int dir,
                    double len, int c) {
    int64_t k[3];
    quantize(g, x, y, z, dir, k);
    int found;
    int* slot = hm_get(em, k, 1, &found);
    if (!found) {
        if (G->ne == G->ecap) {
            G->ecap = G->ecap ? 2 * G->ecap : 1024;
            G->ex = realloc(G->ex, sizeof(double) * G->ecap);
            G->ey = realloc(G->ey, sizeof(double) * G->ecap);
            G->ez = realloc(G->ez, sizeof(double) * G->ecap);
            G->elen = realloc(G->elen, sizeof(double) * G->ecap);
            G->edir = realloc(G->edir, sizeof(int) * G->ecap);
            G->adj = realloc(G->adj, sizeof(ivec) * G->ecap);
        }
        int e = G->ne++;
        G->ex[e] = x; G->ey[e] = y; G->ez[e] = z; G->elen[e] = len; G->edir[e] = dir;
        memset(&G->adj[e], 0, sizeof(ivec));
        *slot = e;
    }
    iv_push(&G->adj[*slot], c);
    return *slot;
}

/* StaggeredGrid::build  staggered_grid.cpp:70-236 */
static void grid_build(grid_t* G, const mesh_t* m) {
    memset(G, 0, sizeof(*G));
    G->nc = m->nc;
    gctx_t g;
    g.dx = m->xmax - m->xmin; g.dy = m->ymax - m->ymin; g.dz = m->zmax - m->zmin;
    g.x0 = m->xmin; g.y0 = m->ymin; g.z0 = m->zmin;
    g.quant = (double)(1 << (m->max_level + 2));

    hmap em;
    hm_init(&em, (size_t)m->nc * 4);
    for (int c = 0; c < m->nc; ++c) {
        double ch[6];
        cell_half(m, &g, c, ch);
        double cx = ch[0], cy = ch[1], cz = ch[2], hx = ch[3], hy = ch[4], hz = ch[5];
        double ey[4] = {cy - hy, cy - hy, cy + hy, cy + hy};
        double ez[4] = {cz - hz, cz + hz, cz - hz, cz + hz};
        for (int i = 0; i < 4; ++i) add_edge(G, &em, &g, cx, ey[i], ez[i], 0, 2.0 * hx, c);
        double ex[4] = {cx - hx, cx - hx, cx + hx, cx + hx};
        double ez2[4] = {cz - hz, cz + hz, cz - hz, cz + hz};
        for (int i = 0; i < 4; ++i) add_edge(G, &em, &g, ex[i], cy, ez2[i], 1, 2.0 * hy, c);
        double ex3[4] = {cx - hx, cx + hx, cx - hx, cx + hx};
        double ey3[4] = {cy - hy, cy - hy, cy + hy, cy + hy};
        for (int i = 0; i < 4; ++i) add_edge(G, &em, &g, ex3[i], ey3[i], cz, 2, 2.0 * hz, c);
    }

    /* faces: staggered_grid.cpp:128-224 */
    hmap fm;
    hm_init(&fm, (size_t)m->nc * 4);
    for (int c = 0; c < m->nc; ++c) {
        double ch[6];
        cell_half(m, &g, c, ch);
        double cx = ch[0], cy = ch[1], cz = ch[2], hx = ch[3], hy = ch[4], hz = ch[5];
        double fd[6][4];         /* fx fy fz area */
        int fn[6];
        double fe[6][4][3];
        int fed[6][4];
        /* +x */
        fd[0][0] = cx + hx; fd[0][1] = cy; fd[0][2] = cz; fn[0] = 0; fd[0][3] = 4 * hy * hz;
        fe[0][0][0] = cx + hx; fe[0][0][1] = cy; fe[0][0][2] = cz - hz; fed[0][0] = 1;
        fe[0][1][0] = cx + hx; fe[0][1][1] = cy; fe[0][1][2] = cz + hz; fed[0][1] = 1;
        fe[0][2][0] = cx + hx; fe[0][2][1] = cy - hy; fe[0][2][2] = cz; fed[0][2] = 2;
        fe[0][3][0] = cx + hx; fe[0][3][1] = cy + hy; fe[0][3][2] = cz; fed[0][3] = 2;
        /* -x */
        fd[1][0] = cx - hx; fd[1][1] = cy; fd[1][2] = cz; fn[1] = 0; fd[1][3] = 4 * hy * hz;
        fe[1][0][0] = cx - hx; fe[1][0][1] = cy; fe[1][0][2] = cz - hz; fed[1][0] = 1;
        fe[1][1][0] = cx - hx; fe[1][1][1] = cy; fe[1][1][2] = cz + hz; fed[1][1] = 1;
        fe[1][2][0] = cx - hx; fe[1][2][1] = cy - hy; fe[1][2][2] = cz; fed[1][2] = 2;
        fe[1][3][0] = cx - hx; fe[1][3][1] = cy + hy; fe[1][3][2] = cz; fed[1][3] = 2;
        /* +y */
        fd[2][0] = cx; fd[2][1] = cy + hy; fd[2][2] = cz; fn[2] = 1; fd[2][3] = 4 * hx * hz;
        fe[2][0][0] = cx; fe[2][0][1] = cy + hy; fe[2][0][2] = cz - hz; fed[2][0] = 0;
        fe[2][1][0] = cx; fe[2][1][1] = cy + hy; fe[2][1][2] = cz + hz; fed[2][1] = 0;
        fe[2][2][0] = cx - hx; fe[2][2][1] = cy + hy; fe[2][2][2] = cz; fed[2][2] = 2;
        fe[2][3][0] = cx + hx; fe[2][3][1] = cy + hy; fe[2][3][2] = cz; fed[2][3] = 2;
        /* -y */
        fd[3][0] = cx; fd[3][1] = cy - hy; fd[3][2] = cz; fn[3] = 1; fd[3][3] = 4 * hx * hz;
        fe[3][0][0] = cx; fe[3][0][1] = cy - hy; fe[3][0][2] = cz - hz; fed[3][0] = 0;
        fe[3][1][0] = cx; fe[3][1][1] = cy - hy; fe[3][1][2] = cz + hz; fed[3][1] = 0;
        fe[3][2][0] = cx - hx; fe[3][2][1] = cy - hy; fe[3][2][2] = cz; fed[3][2] = 2;
        fe[3][3][0] = cx + hx; fe[3][3][1] = cy - hy; fe[3][3][2] = cz; fed[3][3] = 2;
        /* +z */
        fd[4][0] = cx; fd[4][1] = cy; fd[4][2] = cz + hz; fn[4] = 2; fd[4][3] = 4 * hx * hy;
        fe[4][0][0] = cx; fe[4][0][1] = cy - hy; fe[4][0][2] = cz + hz; fed[4][0] = 0;
        fe[4][1][0] = cx; fe[4][1][1] = cy + hy; fe[4][1][2] = cz + hz; fed[4][1] = 0;
        fe[4][2][0] = cx - hx; fe[4][2][1] = cy; fe[4][2][2] = cz + hz; fed[4][2] = 1;
        fe[4][3][0] = cx + hx; fe[4][3][1] = cy; fe[4][3][2] = cz + hz; fed[4][3] = 1;
        /* -z */
        fd[5][0] = cx; fd[5][1] = cy; fd[5][2] = cz - hz; fn[5] = 2; fd[5][3] = 4 * hx * hy;
        fe[5][0][0] = cx; fe[5][0][1] = cy - hy; fe[5][0][2] = cz - hz; fed[5][0] = 0;
        fe[5][1][0] = cx; fe[5][1][1] = cy + hy; fe[5][1][2] = cz - hz; fed[5][1] = 0;
        fe[5][2][0] = cx - hx; fe[5][2][1] = cy; fe[5][2][2] = cz - hz; fed[5][2] = 1;
        fe[5][3][0] = cx + hx; fe[5][3][1] = cy; fe[5][3][2] = cz - hz; fed[5][3] = 1;

        for (int f = 0; f < 6; ++f) {
            int64_t k[3];
            quantize(&g, fd[f][0], fd[f][1], fd[f][2], fn[f], k);
            int found;
            int* slot = hm_get(&fm, k, 1, &found);
            if (!found) {
                if (G->nf == G->fcap) {
                    G->fcap = G->fcap ? 2 * G->fcap : 1024;
                    G->fx = realloc(G->fx, sizeof(double) * G->fcap);
                    G->fy = realloc(G->fy, sizeof(double) * G->fcap);
                    G->fz = realloc(G->fz, sizeof(double) * G->fcap);
                    G->farea = realloc(G->farea, sizeof(double) * G->fcap);
                    G->fnorm = realloc(G->fnorm, sizeof(int) * G->fcap);
                    G->fcm = realloc(G->fcm, sizeof(int) * G->fcap);
                    G->fcp = realloc(G->fcp, sizeof(int) * G->fcap);
                    G->fedge = realloc(G->fedge, sizeof(int) * 4 * G->fcap);
                    G->fnedge = realloc(G->fnedge, sizeof(int) * G->fcap);
                }
                int fid = G->nf++;
                *slot = fid;
                int ne = 0;
                for (int e = 0; e < 4; ++e) {
                    int64_t ek[3];
                    quantize(&g, fe[f][e][0], fe[f][e][1], fe[f][e][2], fed[f][e], ek);
                    int id = hm_find(&em, ek);
                    if (id >= 0) G->fedge[4 * fid + ne++] = id;
                }
                for (int e = ne; e < 4; ++e) G->fedge[4 * fid + e] = -1;
                G->fnedge[fid] = ne;
                G->fx[fid] = fd[f][0]; G->fy[fid] = fd[f][1]; G->fz[fid] = fd[f][2];
                G->fnorm[fid] = fn[f]; G->farea[fid] = fd[f][3];
                G->fcm[fid] = -1; G->fcp[fid] = -1;
            }
            int fid = *slot;
            if (f == 0 || f == 2 || f == 4) G->fcm[fid] = c;
            else G->fcp[fid] = c;
        }
    }

    /* detect_hanging_  staggered_grid.cpp:241-391 */
    G->hface = NULL; G->nhface = 0; G->hedge = NULL; G->nhedge = 0;
    if (m->min_level < m->max_level) {
        double mh = g.dx / (1 << m->max_level);
        if (g.dy / (1 << m->max_level) < mh) mh = g.dy / (1 << m->max_level);
        if (g.dz / (1 << m->max_level) < mh) mh = g.dz / (1 << m->max_level);
        double btol = mh * 0.01;
        hmap flk, elk;   /* last-writer-wins lookups over final coordinates */
        hm_init(&flk, (size_t)G->nf);
        for (int f = 0; f < G->nf; ++f) {
            int64_t k[3]; int fo;
            quantize(&g, G->fx[f], G->fy[f], G->fz[f], G->fnorm[f], k);
            *hm_get(&flk, k, 1, &fo) = f;
        }
        hm_init(&elk, (size_t)G->ne);
        for (int e = 0; e < G->ne; ++e) {
            int64_t k[3]; int fo;
            quantize(&g, G->ex[e], G->ey[e], G->ez[e], G->edir[e], k);
            *hm_get(&elk, k, 1, &fo) = e;
        }
        char* fdone = (char*)xcalloc((size_t)G->nf, 1);
        char* ehang = (char*)xcalloc((size_t)G->ne, 1);
        int hfcap = 0, hecap = 0;
        for (int f = 0; f < G->nf; ++f) {
            if (fdone[f]) continue;
            if (G->fcm[f] >= 0 && G->fcp[f] >= 0) continue;
            if (G->fcm[f] < 0 && G->fcp[f] < 0) continue;
            int n = G->fnorm[f];
            int on_bnd = 0;
            if (n == 0) on_bnd = (G->fx[f] < m->xmin + btol || G->fx[f] > m->xmax - btol);
            if (n == 1) on_bnd = (G->fy[f] < m->ymin + btol || G->fy[f] > m->ymax - btol);
            if (n == 2) on_bnd = (G->fz[f] < m->zmin + btol || G->fz[f] > m->zmax - btol);
            if (on_bnd) continue;
            int ccell = (G->fcm[f] >= 0) ? G->fcm[f] : G->fcp[f];
            double ch[6];
            cell_half(m, &g, ccell, ch);
            double fhx = ch[3] / 2, fhy = ch[4] / 2, fhz = ch[5] / 2;
            int found_all = 1, subs[4], idx = 0;
            for (int s1 = -1; s1 <= 1 && found_all; s1 += 2) {
                for (int s2 = -1; s2 <= 1; s2 += 2) {
                    double sx = G->fx[f], sy = G->fy[f], sz = G->fz[f];
                    if (n == 0) { sy += s1 * fhy; sz += s2 * fhz; }
                    else if (n == 1) { sx += s1 * fhx; sz += s2 * fhz; }
                    else { sx += s1 * fhx; sy += s2 * fhy; }
                    int64_t k[3];
                    quantize(&g, sx, sy, sz, n, k);
                    int id = hm_find(&flk, k);
                    if (id < 0 || fdone[id]) { found_all = 0; break; }
                    subs[idx++] = id;
                }
            }
            if (!found_all) continue;
            for (int q = 0; q < 4; ++q)
                if (G->fcm[subs[q]] >= 0 && G->fcp[subs[q]] >= 0) { found_all = 0; break; }
            if (!found_all) continue;

            if (G->nhface == hfcap) { hfcap = hfcap ? 2 * hfcap : 64; G->hface = realloc(G->hface, sizeof(int) * 5 * hfcap); }
            G->hface[5 * G->nhface] = f;
            for (int q = 0; q < 4; ++q) G->hface[5 * G->nhface + 1 + q] = subs[q];
            G->nhface++;
            fdone[f] = 1;
            for (int q = 0; q < 4; ++q) fdone[subs[q]] = 1;
            for (int q = 0; q < 4; ++q) {
                int ff = subs[q];
                if (G->fcm[ff] < 0) G->fcm[ff] = ccell;
                else if (G->fcp[ff] < 0) G->fcp[ff] = ccell;
            }
            G->fcm[f] = -1; G->fcp[f] = -1;
            for (int q = 0; q < 4; ++q) {
                int ff = subs[q];
                for (int t = 0; t < G->fnedge[ff]; ++t) {
                    int eid = G->fedge[4 * ff + t];
                    if (eid < 0) continue;
                    ivec* a = &G->adj[eid];
                    int has = 0;
                    for (int u = 0; u < a->n; ++u) if (a->a[u] == ccell) { has = 1; break; }
                    if (!has) iv_push(a, ccell);
                }
            }
            for (int t = 0; t < G->fnedge[f]; ++t) {
                int eid = G->fedge[4 * f + t];
                if (eid < 0 || ehang[eid]) continue;
                int d = G->edir[eid];
                double ql = G->elen[eid] / 4.0;
                double a1x = G->ex[eid], a1y = G->ey[eid], a1z = G->ez[eid];
                double a2x = a1x, a2y = a1y, a2z = a1z;
                if (d == 0) { a1x -= ql; a2x += ql; }
                else if (d == 1) { a1y -= ql; a2y += ql; }
                else { a1z -= ql; a2z += ql; }
                int64_t k1[3], k2[3];
                quantize(&g, a1x, a1y, a1z, d, k1);
                quantize(&g, a2x, a2y, a2z, d, k2);
                int i1 = hm_find(&elk, k1), i2 = hm_find(&elk, k2);
                if (i1 >= 0 && i2 >= 0) {
                    if (G->nhedge == hecap) { hecap = hecap ? 2 * hecap : 64; G->hedge = realloc(G->hedge, sizeof(int) * 3 * hecap); }
                    G->hedge[3 * G->nhedge] = eid;
                    G->hedge[3 * G->nhedge + 1] = i1;
                    G->hedge[3 * G->nhedge + 2] = i2;
                    G->nhedge++;
                    ehang[eid] = 1;
                }
            }
        }
        free(fdone); free(ehang);
        hm_free(&flk); hm_free(&elk);
    }

    /* build_cell_edge_map_  staggered_grid.cpp:393-409 */
    {
        int* cnt = (int*)xcalloc((size_t)m->nc + 1, sizeof(int));
        for (int e = 0; e < G->ne; ++e)
            for (int u = 0; u < G->adj[e].n; ++u) {
                int c = G->adj[e].a[u];
                if (c >= 0 && c < m->nc) cnt[c + 1]++;
            }
        G->ce_ptr = (int*)xcalloc((size_t)m->nc + 1, sizeof(int));
        for (int c = 0; c < m->nc; ++c) G->ce_ptr[c + 1] = G->ce_ptr[c] + cnt[c + 1];
        int tot = G->ce_ptr[m->nc];
        G->ce_id = (int*)xcalloc((size_t)tot, sizeof(int));
        G->ce_frac = (double*)xcalloc((size_t)tot, sizeof(double));
        int* pos = (int*)xcalloc((size_t)m->nc, sizeof(int));
        for (int c = 0; c < m->nc; ++c) pos[c] = G->ce_ptr[c];
        for (int e = 0; e < G->ne; ++e) {
            int na = G->adj[e].n;
            if (na == 0) continue;
            double frac = 1.0 / na;
            for (int u = 0; u < na; ++u) {
                int c = G->adj[e].a[u];
                if (c >= 0 && c < m->nc) { G->ce_id[pos[c]] = e; G->ce_frac[pos[c]] = frac; pos[c]++; }
            }
        }
        free(cnt); free(pos);
    }
    hm_free(&em);
    hm_free(&fm);
}

static void grid_free(grid_t* G) {
    free(G->ex); free(G->ey); free(G->ez); free(G->elen); free(G->edir);
    for (int e = 0; e < G->ne; ++e) free(G->adj[e].a);
    free(G->adj);
    free(G->fx); free(G->fy); free(G->fz); free(G->farea); free(G->fnorm);
    free(G->fcm); free(G->fcp); free(G->fedge); free(G->fnedge);
    free(G->hface); free(G->hedge);
    free(G->ce_ptr); free(G->ce_id); free(G->ce_frac);
}

/* ------------------------------------------------------------------------ */
/* discrete operators  (src/octree/operators.cpp)                            */
/* ------------------------------------------------------------------------ */

typedef struct { int nrows, ncols; int* ptr; int* idx; double* val; } csr_t;
typedef struct { int nrows, ncols; int* ptr; int* idx; cplx* val; } csrc_t;

typedef struct {
    int ne, nf, nc, nn;
    double* adual;         /* edge dual area */
    double* fdual;         /* face dual length */
    char* dead_e;
    char* dead_f;
    int* hp;  int nhp;     /* hanging pairs coarse, c1, c2 */
    csr_t Ce;              /* faces x edges */
    int *gn1, *gn2;        /* edge -> node endpoints */
    csr_t G;               /* edges x nodes, 2 per row sorted */
    int *sp_ptr, *sp_idx;  /* cached stiffness pattern */
} ops_t;

typedef struct { int row, col; double val; } coo_t;

static int coo_cmp(const void* a, const void* b) {
    const coo_t* x = (const coo_t*)a; const coo_t* y = (const coo_t*)b;
    if (x->row != y->row) return x->row < y->row ? -1 : 1;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    return 0;
}

/* DiscreteOperators::build  operators.cpp:19-170 */
static void ops_build(ops_t* O, const grid_t* G) {
    memset(O, 0, sizeof(*O));
    const int ne = G->ne, nf = G->nf, nc = G->nc;
    O->ne = ne; O->nf = nf; O->nc = nc;
    double* ccx = (double*)xcalloc((size_t)nc, sizeof(double));
    double* ccy = (double*)xcalloc((size_t)nc, sizeof(double));
    double* ccz = (double*)xcalloc((size_t)nc, sizeof(double));
    double* chx = (double*)xcalloc((size_t)nc, sizeof(double));
    double* chy = (double*)xcalloc((size_t)nc, sizeof(double));
    double* chz = (double*)xcalloc((size_t)nc, sizeof(double));
    int* cnt = (int*)xcalloc((size_t)nc, sizeof(int));
    /* cell centres as the mean of adjacent edge midpoints (:62-86) */
    for (int e = 0; e < ne; ++e)
        for (int u = 0; u < G->adj[e].n; ++u) {
            int c = G->adj[e].a[u];
            if (c >= 0 && c < nc) { ccx[c] += G->ex[e]; ccy[c] += G->ey[e]; ccz[c] += G->ez[e]; cnt[c]++; }
        }
    for (int c = 0; c < nc; ++c)
        if (cnt[c] > 0) { ccx[c] /= cnt[c]; ccy[c] /= cnt[c]; ccz[c] /= cnt[c]; }
    /* half extents (:90-99) */
    for (int e = 0; e < ne; ++e) {
        int d = G->edir[e];
        double half = G->elen[e] / 2.0;
        for (int u = 0; u < G->adj[e].n; ++u) {
            int c = G->adj[e].a[u];
            if (c < 0 || c >= nc) continue;
            if (d == 0 && half > chx[c]) chx[c] = half;
            if (d == 1 && half > chy[c]) chy[c] = half;
            if (d == 2 && half > chz[c]) chz[c] = half;
        }
    }
    /* face dual lengths (:103-126) */
    O->fdual = (double*)xcalloc((size_t)nf, sizeof(double));
    for (int f = 0; f < nf; ++f) {
        int n = G->fnorm[f], cm = G->fcm[f], cp = G->fcp[f];
        if (cm >= 0 && cp >= 0) {
            double a = n == 0 ? ccx[cm] : n == 1 ? ccy[cm] : ccz[cm];
            double b = n == 0 ? ccx[cp] : n == 1 ? ccy[cp] : ccz[cp];
            O->fdual[f] = fabs(b - a);
        } else {
            int c = cm >= 0 ? cm : cp;
            if (c >= 0) O->fdual[f] = n == 0 ? chx[c] : n == 1 ? chy[c] : chz[c];
            else O->fdual[f] = sqrt(G->farea[f]);
        }
        if (O->fdual[f] < 1e-20) O->fdual[f] = sqrt(G->farea[f]);
    }
    /* edge dual areas (:133-157) */
    O->adual = (double*)xcalloc((size_t)ne, sizeof(double));
    for (int e = 0; e < ne; ++e) {
        int d = G->edir[e];
        if (G->adj[e].n == 0) { O->adual[e] = G->elen[e] * G->elen[e]; continue; }
        double s = 0; int count = 0;
        for (int u = 0; u < G->adj[e].n; ++u) {
            int c = G->adj[e].a[u];
            if (c < 0 || c >= nc) continue;
            double h1, h2;
            if (d == 0) { h1 = chy[c]; h2 = chz[c]; }
            else if (d == 1) { h1 = chx[c]; h2 = chz[c]; }
            else { h1 = chx[c]; h2 = chy[c]; }
            s += h1 * h2;
            ++count;
        }
        O->adual[e] = count > 0 ? s : G->elen[e] * G->elen[e];
    }
    free(ccx); free(ccy); free(ccz); free(chx); free(chy); free(chz); free(cnt);

    /* build_curl_ (:176-286): entries in face order, edges in face-list order */
    int nent = 0;
    coo_t* ent = (coo_t*)xcalloc((size_t)nf * 4, sizeof(coo_t));
    for (int f = 0; f < nf; ++f) {
        for (int t = 0; t < G->fnedge[f]; ++t) {
            int eid = G->fedge[4 * f + t];
            if (eid < 0 || eid >= ne) continue;
            int n = G->fnorm[f], d = G->edir[eid];
            double sign = 0.0;
            if (n == 0) {
                if (d == 1) sign = (G->ez[eid] < G->fz[f]) ? 1.0 : -1.0;
                else if (d == 2) sign = (G->ey[eid] < G->fy[f]) ? -1.0 : 1.0;
            } else if (n == 1) {
                if (d == 2) sign = (G->ex[eid] < G->fx[f]) ? 1.0 : -1.0;
                else if (d == 0) sign = (G->ez[eid] < G->fz[f]) ? -1.0 : 1.0;
            } else {
                if (d == 0) sign = (G->ey[eid] < G->fy[f]) ? 1.0 : -1.0;
                else if (d == 1) sign = (G->ex[eid] < G->fx[f]) ? -1.0 : 1.0;
            }
            if (fabs(sign) > 0.5) {
                ent[nent].row = f; ent[nent].col = eid; ent[nent].val = sign * G->elen[eid];
                nent++;
            }
        }
    }

    /* handle_hanging_faces_ (:344-466) */
    O->dead_e = (char*)xcalloc((size_t)ne, 1);
    O->dead_f = (char*)xcalloc((size_t)nf, 1);
    O->nhp = G->nhedge;
    O->hp = (int*)xcalloc((size_t)G->nhedge * 3 + 1, sizeof(int));
    if (G->nhface > 0) {
        int* ch1 = (int*)xcalloc((size_t)ne, sizeof(int));
        int* ch2 = (int*)xcalloc((size_t)ne, sizeof(int));
        for (int h = 0; h < G->nhedge; ++h) {
            int ce = G->hedge[3 * h];
            O->dead_e[ce] = 1;
            ch1[ce] = G->hedge[3 * h + 1];
            ch2[ce] = G->hedge[3 * h + 2];
            O->hp[3 * h] = ce; O->hp[3 * h + 1] = ch1[ce]; O->hp[3 * h + 2] = ch2[ce];
        }
        for (int h = 0; h < G->nhface; ++h) O->dead_f[G->hface[5 * h]] = 1;
        coo_t* ne2 = (coo_t*)xcalloc((size_t)nent * 2 + 1, sizeof(coo_t));
        int n2 = 0;
        for (int k = 0; k < nent; ++k) {
            int f = ent[k].row;
            if (O->dead_f[f]) continue;
            int e = ent[k].col;
            double v = ent[k].val;
            if (fabs(v) < 1e-30) continue;
            if (O->dead_e[e]) {
                ne2[n2].row = f; ne2[n2].col = ch1[e]; ne2[n2].val = 0.5 * v; n2++;
                ne2[n2].row = f; ne2[n2].col = ch2[e]; ne2[n2].val = 0.5 * v; n2++;
            } else {
                ne2[n2].row = f; ne2[n2].col = e; ne2[n2].val = v; n2++;
            }
        }
        /* std::map merge: sum in insertion order per (row, col), sorted output.
           A stable sort keeps insertion order among equal keys. */
        int* ord = (int*)xcalloc((size_t)n2 + 1, sizeof(int));
        for (int k = 0; k < n2; ++k) ord[k] = k;
        /* insertion-stable mergesort by (row, col) */
        {
            int* tmp = (int*)xcalloc((size_t)n2 + 1, sizeof(int));
            for (int w = 1; w < n2; w *= 2) {
                for (int lo = 0; lo < n2; lo += 2 * w) {
                    int mid = lo + w < n2 ? lo + w : n2, hi = lo + 2 * w < n2 ? lo + 2 * w : n2;
                    int a = lo, b = mid, o = lo;
                    while (a < mid && b < hi) {
                        if (coo_cmp(&ne2[ord[b]], &ne2[ord[a]]) < 0) tmp[o++] = ord[b++];
                        else tmp[o++] = ord[a++];
                    }
                    while (a < mid) tmp[o++] = ord[a++];
                    while (b < hi) tmp[o++] = ord[b++];
                }
                memcpy(ord, tmp, sizeof(int) * (size_t)n2);
            }
            free(tmp);
        }
        nent = 0;
        for (int k = 0; k < n2;) {
            int r = ne2[ord[k]].row, c = ne2[ord[k]].col;
            double s = 0.0;
            while (k < n2 && ne2[ord[k]].row == r && ne2[ord[k]].col == c) { s += ne2[ord[k]].val; ++k; }
            if (fabs(s) > 1e-30) { ent[nent].row = r; ent[nent].col = c; ent[nent].val = s; nent++; }
        }
        free(ord); free(ne2); free(ch1); free(ch2);
    }
    /* COO (row-grouped, order within row kept) -> CSR */
    O->Ce.nrows = nf; O->Ce.ncols = ne;
    O->Ce.ptr = (int*)xcalloc((size_t)nf + 1, sizeof(int));
    for (int k = 0; k < nent; ++k) O->Ce.ptr[ent[k].row + 1]++;
    for (int f = 0; f < nf; ++f) O->Ce.ptr[f + 1] += O->Ce.ptr[f];
    O->Ce.idx = (int*)xcalloc((size_t)nent + 1, sizeof(int));
    O->Ce.val = (double*)xcalloc((size_t)nent + 1, sizeof(double));
    {
        int* pos = (int*)xcalloc((size_t)nf + 1, sizeof(int));
        for (int f = 0; f < nf; ++f) pos[f] = O->Ce.ptr[f];
        for (int k = 0; k < nent; ++k) {
            int p = pos[ent[k].row]++;
            O->Ce.idx[p] = ent[k].col; O->Ce.val[p] = ent[k].val;
        }
        free(pos);
    }
    free(ent);

    /* build_node_gradient_matrix_ (:849-944) */
    {
        double minL = 1e30;
        for (int e = 0; e < ne; ++e) if (G->elen[e] > 1e-10 && G->elen[e] < minL) minL = G->elen[e];
        double tol = minL * 0.01;
        hmap nm;
        hm_init(&nm, (size_t)ne);
        O->gn1 = (int*)xcalloc((size_t)ne, sizeof(int));
        O->gn2 = (int*)xcalloc((size_t)ne, sizeof(int));
        int nn = 0;
        for (int e = 0; e < ne; ++e) {
            int d = G->edir[e];
            double hl = G->elen[e] * 0.5;
            double p1[3] = {G->ex[e], G->ey[e], G->ez[e]};
            double p2[3] = {G->ex[e], G->ey[e], G->ez[e]};
            p1[d] -= hl; p2[d] += hl;
            for (int s = 0; s < 2; ++s) {
                double* p = s ? p2 : p1;
                int64_t k[3] = {(int64_t)llround(p[0] / tol), (int64_t)llround(p[1] / tol),
                                (int64_t)llround(p[2] / tol)};
                int found;
                int* slot = hm_get(&nm, k, 1, &found);
                if (!found) *slot = nn++;
                if (s) O->gn2[e] = *slot; else O->gn1[e] = *slot;
            }
        }
        hm_free(&nm);
        O->nn = nn;
        O->G.nrows = ne; O->G.ncols = nn;
        O->G.ptr = (int*)xcalloc((size_t)ne + 1, sizeof(int));
        O->G.idx = (int*)xcalloc((size_t)2 * ne + 1, sizeof(int));
        O->G.val = (double*)xcalloc((size_t)2 * ne + 1, sizeof(double));
        for (int e = 0; e <= ne; ++e) O->G.ptr[e] = 2 * e;
        for (int e = 0; e < ne; ++e) {
            int v1 = O->gn1[e], v2 = O->gn2[e];
            double inv = 1.0 / G->elen[e];
            if (v1 < v2) {
                O->G.idx[2 * e] = v1; O->G.val[2 * e] = -inv;
                O->G.idx[2 * e + 1] = v2; O->G.val[2 * e + 1] = +inv;
            } else {
                O->G.idx[2 * e] = v2; O->G.val[2 * e] = +inv;
                O->G.idx[2 * e + 1] = v1; O->G.val[2 * e + 1] = -inv;
            }
        }
    }
}

static void ops_free(ops_t* O) {
    free(O->adual); free(O->fdual); free(O->dead_e); free(O->dead_f); free(O->hp);
    free(O->Ce.ptr); free(O->Ce.idx); free(O->Ce.val);
    free(O->gn1); free(O->gn2); free(O->G.ptr); free(O->G.idx); free(O->G.val);
    free(O->sp_ptr); free(O->sp_idx);
}

/* edge mass  operators.cpp:481-518 (arithmetic mean of adjacent sigma) */
static void edge_mass(const ops_t* O, const grid_t* G, const double* sigma, double* Me) {
    for (int e = 0; e < O->ne; ++e) {
        Me[e] = 0.0;
        if (G->adj[e].n == 0) continue;
        double s = 0.0; int count = 0;
        for (int u = 0; u < G->adj[e].n; ++u) {
            int c = G->adj[e].a[u];
            if (c >= 0 && c < O->nc) { s += sigma[c]; ++count; }
        }
        double sa = count > 0 ? s / count : 1e-8;
        double L = G->elen[e];
        double mh = O->adual[e] * L;
        Me[e] = sa * mh;
    }
    for (int h = 0; h < O->nhp; ++h) Me[O->hp[3 * h]] = 0.0;
}

/* face mass inverse  operators.cpp:539-551 */
static void face_mass_inv(const ops_t* O, const grid_t* G, double* Mfi) {
    for (int f = 0; f < O->nf; ++f) {
        if (O->dead_f[f]) { Mfi[f] = 0.0; continue; }
        double mf = M3D_MU0 * G->farea[f] / O->fdual[f];
        Mfi[f] = mf > 1e-30 ? 1.0 / mf : 0.0;
    }
}

/* assemble_system  operators.cpp:556-837.  The pattern is the set of (i,j)
 * pairs coupled through a face plus the diagonal, columns sorted; values sum
 * the face contributions in face order, then add i*omega*Me on the diagonal. */
static void assemble(ops_t* O, const grid_t* G, double omega, const double* sigma, csrc_t* A) {
    const int ne = O->ne, nf = O->nf;
    double* Me = (double*)xcalloc((size_t)ne, sizeof(double));
    double* Mfi = (double*)xcalloc((size_t)nf, sizeof(double));
    edge_mass(O, G, sigma, Me);
    face_mass_inv(O, G, Mfi);
    if (!O->sp_ptr) {
        /* pattern: for each face all (i,j) of its Ce row, plus the diagonal */
        size_t np = (size_t)ne;
        for (int f = 0; f < nf; ++f) { size_t r = O->Ce.ptr[f + 1] - O->Ce.ptr[f]; np += r * r; }
        coo_t* pr = (coo_t*)xcalloc(np + 1, sizeof(coo_t));
        size_t k = 0;
        for (int f = 0; f < nf; ++f)
            for (int a = O->Ce.ptr[f]; a < O->Ce.ptr[f + 1]; ++a)
                for (int b = O->Ce.ptr[f]; b < O->Ce.ptr[f + 1]; ++b) {
                    pr[k].row = O->Ce.idx[a]; pr[k].col = O->Ce.idx[b]; pr[k].val = 0; k++;
                }
        for (int e = 0; e < ne; ++e) { pr[k].row = e; pr[k].col = e; pr[k].val = 0; k++; }
        qsort(pr, k, sizeof(coo_t), coo_cmp);
        size_t u = 0;
        for (size_t t = 0; t < k; ++t)
            if (u == 0 || pr[t].row != pr[u - 1].row || pr[t].col != pr[u - 1].col) pr[u++] = pr[t];
        O->sp_ptr = (int*)xcalloc((size_t)ne + 1, sizeof(int));
        O->sp_idx = (int*)xcalloc(u + 1, sizeof(int));
        for (size_t t = 0; t < u; ++t) { O->sp_ptr[pr[t].row + 1]++; O->sp_idx[t] = pr[t].col; }
        for (int e = 0; e < ne; ++e) O->sp_ptr[e + 1] += O->sp_ptr[e];
        free(pr);
    }
    int nnz = O->sp_ptr[ne];
    A->nrows = ne; A->ncols = ne;
    A->ptr = (int*)xcalloc((size_t)ne + 1, sizeof(int));
    A->idx = (int*)xcalloc((size_t)nnz + 1, sizeof(int));
    A->val = (cplx*)xcalloc((size_t)nnz + 1, sizeof(cplx));
    memcpy(A->ptr, O->sp_ptr, sizeof(int) * ((size_t)ne + 1));
    memcpy(A->idx, O->sp_idx, sizeof(int) * (size_t)nnz);
    /* fast path :586-616 */
    for (int f = 0; f < nf; ++f) {
        double mfi = Mfi[f];
        for (int k1 = O->Ce.ptr[f]; k1 < O->Ce.ptr[f + 1]; ++k1) {
            int i = O->Ce.idx[k1];
            double cfi = O->Ce.val[k1];
            for (int k2 = O->Ce.ptr[f]; k2 < O->Ce.ptr[f + 1]; ++k2) {
                int j = O->Ce.idx[k2];
                double cfj = O->Ce.val[k2];
                int lo = A->ptr[i], hi = A->ptr[i + 1];
                while (lo < hi) { int mid = (lo + hi) >> 1; if (A->idx[mid] < j) lo = mid + 1; else hi = mid; }
                if (lo < A->ptr[i + 1] && A->idx[lo] == j) A->val[lo] += CMPLX(cfi * mfi * cfj, 0.0);
            }
        }
    }
    cplx iw = CMPLX(0.0, omega);
    for (int e = 0; e < ne; ++e) {
        int lo = A->ptr[e], hi = A->ptr[e + 1];
        while (lo < hi) { int mid = (lo + hi) >> 1; if (A->idx[mid] < e) lo = mid + 1; else hi = mid; }
        if (lo < A->ptr[e + 1] && A->idx[lo] == e) A->val[lo] += iw * CMPLX(Me[e], 0.0);
    }
    free(Me); free(Mfi);
}

static void csrc_free(csrc_t* A) { free(A->ptr); free(A->idx); free(A->val); memset(A, 0, sizeof(*A)); }

static void csrc_matvec(const csrc_t* A, const cplx* x, cplx* y) {
    for (int i = 0; i < A->nrows; ++i) {
        cplx s = 0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) s += A->val[k] * x[A->idx[k]];
        y[i] = s;
    }
}

/* me_sigma shared by build_div_laplacian (:956-973) and compute_div_sigma_E (:1030-1048) */
static void me_sigma(const ops_t* O, const grid_t* G, const double* sigma, double* me) {
    for (int e = 0; e < O->ne; ++e) {
        me[e] = 0.0;
        if (O->dead_e[e]) continue;
        double s = 0.0; int count = 0;
        for (int u = 0; u < G->adj[e].n; ++u) {
            int c = G->adj[e].a[u];
            if (c >= 0 && c < O->nc) { s += sigma[c]; ++count; }
        }
        double sa = count > 0 ? s / count : 1e-8;
        me[e] = sa * O->adual[e] * G->elen[e];
    }
}

/* build_div_laplacian  operators.cpp:952-1019 (sorted (row, col) pattern,
 * values summed in edge order) */
static void div_laplacian(const ops_t* O, const grid_t* G, const double* sigma, csr_t* L) {
    const int ne = O->ne, nn = O->nn;
    double* me = (double*)xcalloc((size_t)ne, sizeof(double));
    me_sigma(O, G, sigma, me);
    coo_t* pr = (coo_t*)xcalloc((size_t)4 * ne + 1, sizeof(coo_t));
    int k = 0;
    for (int e = 0; e < ne; ++e) {
        double w = me[e];
        if (w < 1e-30) continue;
        for (int a = O->G.ptr[e]; a < O->G.ptr[e + 1]; ++a)
            for (int b = O->G.ptr[e]; b < O->G.ptr[e + 1]; ++b) {
                pr[k].row = O->G.idx[a]; pr[k].col = O->G.idx[b];
                pr[k].val = O->G.val[a] * w * O->G.val[b];
                k++;
            }
    }
    /* stable by (row, col) to sum in edge order */
    int* ord = (int*)xcalloc((size_t)k + 1, sizeof(int));
    int* tmp = (int*)xcalloc((size_t)k + 1, sizeof(int));
    for (int t = 0; t < k; ++t) ord[t] = t;
    for (int w = 1; w < k; w *= 2) {
        for (int lo = 0; lo < k; lo += 2 * w) {
            int mid = lo + w < k ? lo + w : k, hi = lo + 2 * w < k ? lo + 2 * w : k;
            int a = lo, b = mid, o = lo;
            while (a < mid && b < hi) {
                if (coo_cmp(&pr[ord[b]], &pr[ord[a]]) < 0) tmp[o++] = ord[b++];
                else tmp[o++] = ord[a++];
            }
            while (a < mid) tmp[o++] = ord[a++];
            while (b < hi) tmp[o++] = ord[b++];
        }
        memcpy(ord, tmp, sizeof(int) * (size_t)k);
    }
    L->nrows = nn; L->ncols = nn;
    L->ptr = (int*)xcalloc((size_t)nn + 1, sizeof(int));
    L->idx = (int*)xcalloc((size_t)k + 1, sizeof(int));
    L->val = (double*)xcalloc((size_t)k + 1, sizeof(double));
    int u = 0;
    for (int t = 0; t < k;) {
        int r = pr[ord[t]].row, c = pr[ord[t]].col;
        double s = 0.0;
        while (t < k && pr[ord[t]].row == r && pr[ord[t]].col == c) { s += pr[ord[t]].val; ++t; }
        L->idx[u] = c; L->val[u] = s; L->ptr[r + 1]++; u++;
    }
    for (int i = 0; i < nn; ++i) L->ptr[i + 1] += L->ptr[i];
    free(ord); free(tmp); free(pr); free(me);
}

/* compute_div_sigma_E  operators.cpp:1025-1057 */
static void div_sigma_E(const ops_t* O, const grid_t* G, const double* me, const cplx* E, cplx* divJ) {
    for (int v = 0; v < O->nn; ++v) divJ[v] = 0;
    for (int e = 0; e < O->ne; ++e) {
        if (O->dead_e[e]) continue;
        cplx we = me[e] * E[e];
        for (int k = O->G.ptr[e]; k < O->G.ptr[e + 1]; ++k) divJ[O->G.idx[k]] += O->G.val[k] * we;
    }
    (void)G;
}

/* apply_cell_gradient  operators.cpp:1063-1074 */
static void apply_gradient(const ops_t* O, const cplx* phi, cplx* g) {
    for (int e = 0; e < O->ne; ++e) {
        cplx v = 0;
        for (int k = O->G.ptr[e]; k < O->G.ptr[e + 1]; ++k) v += O->G.val[k] * phi[O->G.idx[k]];
        g[e] = v;
    }
}

/* ------------------------------------------------------------------------ */
/* SSOR and BiCGStab                                                         */
/* ------------------------------------------------------------------------ */

/* SSORPreconditioner::setup / apply  include/maple3dmt/forward/ssor.h:28-78 (omega = 1) */
typedef struct { const csrc_t* A; cplx* inv_diag; cplx* y; } ssor_t;

static void ssor_setup(ssor_t* S, const csrc_t* A) {
    S->A = A;
    S->inv_diag = (cplx*)xcalloc((size_t)A->nrows, sizeof(cplx));
    S->y = (cplx*)xcalloc((size_t)A->nrows, sizeof(cplx));
    for (int i = 0; i < A->nrows; ++i) {
        cplx d = 1.0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k)
            if (A->idx[k] == i) { d = A->val[k]; break; }
        S->inv_diag[i] = (cabs(d) > 1e-30) ? (cplx)1.0 / d : (cplx)1.0;
    }
}

static void ssor_free(ssor_t* S) { free(S->inv_diag); free(S->y); }

static void ssor_apply(const ssor_t* S, const cplx* r, cplx* out) {
    const csrc_t* A = S->A;
    const int n = A->nrows;
    const double om = 1.0;
    for (int i = 0; i < n; ++i) {
        cplx sum = 0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
            int j = A->idx[k];
            if (j < i) sum += A->val[k] * S->y[j];
        }
        S->y[i] = om * (r[i] - sum) * S->inv_diag[i];
    }
    for (int i = n - 1; i >= 0; --i) {
        cplx sum = 0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
            int j = A->idx[k];
            if (j > i) sum += A->val[k] * out[j];
        }
        out[i] = S->y[i] - om * sum * S->inv_diag[i];
    }
}

typedef struct { int iterations; double residual; int converged; int breakdown; } bicg_res_t;

static double vnorm(const cplx* v, int n) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += cnorm2(v[i]);
    return sqrt(s);
}

static cplx vdot(const cplx* a, const cplx* b, int n) {
    cplx s = 0;
    for (int i = 0; i < n; ++i) s += conj(a[i]) * b[i];
    return s;
}

/* BiCGStabSolver::solve  src/forward/bicgstab.cpp:15-166 (right-preconditioned) */
static bicg_res_t bicgstab(const csrc_t* A, const ssor_t* M, const cplx* b, cplx* x, double tol, int maxiter) {
    bicg_res_t res = {0, 0.0, 0, 0};
    const int n = A->nrows;
    cplx* r = (cplx*)xcalloc((size_t)n, sizeof(cplx));
    cplx* r0 = (cplx*)xcalloc((size_t)n, sizeof(cplx));
    cplx* p = (cplx*)xcalloc((size_t)n, sizeof(cplx));
    cplx* v = (cplx*)xcalloc((size_t)n, sizeof(cplx));
    cplx* s = (cplx*)xcalloc((size_t)n, sizeof(cplx));
    cplx* t = (cplx*)xcalloc((size_t)n, sizeof(cplx));
    cplx* ph = (cplx*)xcalloc((size_t)n, sizeof(cplx));
    cplx* sh = (cplx*)xcalloc((size_t)n, sizeof(cplx));
    csrc_matvec(A, x, v);
    for (int i = 0; i < n; ++i) r[i] = b[i] - v[i];
    memcpy(r0, r, sizeof(cplx) * (size_t)n);
    double bnorm = vnorm(b, n);
    if (bnorm < 1e-30) bnorm = 1.0;
    double rnorm = vnorm(r, n);
    if (rnorm / bnorm < tol) {
        res.converged = 1; res.residual = rnorm / bnorm; res.iterations = 0;
        goto done;
    }
    {
        cplx rho_old = 1.0, alpha = 1.0, omega = 1.0;
        for (int it = 1; it <= maxiter; ++it) {
            cplx rho = vdot(r0, r, n);
            if (cabs(rho) < 1e-30) {
                res.iterations = it; res.residual = vnorm(r, n) / bnorm; res.breakdown = 1;
                goto done;
            }
            if (it == 1) memcpy(p, r, sizeof(cplx) * (size_t)n);
            else {
                cplx beta = (rho / rho_old) * (alpha / omega);
                for (int i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
            }
            ssor_apply(M, p, ph);
            csrc_matvec(A, ph, v);
            cplx r0v = vdot(r0, v, n);
            if (cabs(r0v) < 1e-30) {
                res.iterations = it; res.residual = vnorm(r, n) / bnorm; res.breakdown = 2;
                goto done;
            }
            alpha = rho / r0v;
            for (int i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
            double snorm = vnorm(s, n);
            if (snorm / bnorm < tol) {
                for (int i = 0; i < n; ++i) x[i] += alpha * ph[i];
                res.converged = 1; res.residual = snorm / bnorm; res.iterations = it;
                goto done;
            }
            ssor_apply(M, s, sh);
            csrc_matvec(A, sh, t);
            cplx tt = vdot(t, t, n);
            if (cabs(tt) < 1e-30) {
                res.iterations = it; res.residual = snorm / bnorm; res.breakdown = 3;
                for (int i = 0; i < n; ++i) x[i] += alpha * ph[i];
                goto done;
            }
            omega = vdot(t, s, n) / tt;
            for (int i = 0; i < n; ++i) x[i] += alpha * ph[i] + omega * sh[i];
            for (int i = 0; i < n; ++i) r[i] = s[i] - omega * t[i];
            rnorm = vnorm(r, n);
            double rel = rnorm / bnorm;
            if (rel < tol) {
                res.converged = 1; res.residual = rel; res.iterations = it;
                goto done;
            }
            if (cabs(omega) < 1e-30) {
                res.iterations = it; res.residual = rel; res.breakdown = 4;
                goto done;
            }
            rho_old = rho;
        }
        res.iterations = maxiter;
        res.residual = vnorm(r, n) / bnorm;
    }
done:
    free(r); free(r0); free(p); free(v); free(s); free(t); free(ph); free(sh);
    return res;
}

/* ------------------------------------------------------------------------ */
/* forward solver  (src/forward/forward_solver_fv.cpp)                       */
/* ------------------------------------------------------------------------ */

typedef struct {
    cplx Hx1, Hy1, Hx2, Hy2, det_H, Zxx, Zxy, Zyx, Zyy;
    double cdx, cdy, cdz;
} hcache_t;

struct m3d_oracle {
    mesh_t m;
    grid_t G;
    ops_t O;
    int ne, nc, nn;
    double* sigma;
    double sigma_bg;
    /* ForwardParamsFV */
    double tol; int maxiter; int scattered; double air_z; int divcorr; int dc_iters;
    double dc_tol; int dc_outer; int dc_iter_per;
    double tol_override;
    /* per-frequency state */
    double omega;
    csrc_t A;           /* BC-modified, kept for the adjoint */
    int have_A;
    cplx *E1, *E2;
    /* DivCorr cache (compute_bc_flags_) */
    char* dc_is_bc;
    char* dc_bc_nodes;
    csr_t L;
    double* Ldiag;
    double* me;        /* me_sigma for div(sigma E) */
    int dc_done;
    /* stations */
    int ns;
    const double* sxyz;
    int* st_cell;
    hcache_t* hc;
    /* stats of the last inner solves */
    int last_iters[64];
    int n_last;
    int log;
};

static void log_iters(m3d_oracle* S, int it) {
    if (S->n_last < 64) S->last_iters[S->n_last++] = it;
}

/* compute_bc_flags_  forward_solver_fv.cpp:546-610 */
static void compute_bc_flags(m3d_oracle* S) {
    const int ne = S->ne, nn = S->nn;
    const mesh_t* m = &S->m;
    const double bt = 1.0;
    free(S->dc_is_bc); free(S->dc_bc_nodes); free(S->Ldiag); free(S->me);
    free(S->L.ptr); free(S->L.idx); free(S->L.val);
    S->dc_is_bc = (char*)xcalloc((size_t)ne, 1);
    for (int e = 0; e < ne; ++e) {
        if (S->O.dead_e[e]) continue;
        double x = S->G.ex[e], y = S->G.ey[e], z = S->G.ez[e];
        if (x <= m->xmin + bt || x >= m->xmax - bt || y <= m->ymin + bt || y >= m->ymax - bt ||
            z <= m->zmin + bt || z >= m->zmax - bt || z > S->air_z)
            S->dc_is_bc[e] = 1;
    }
    S->dc_bc_nodes = (char*)xcalloc((size_t)nn, 1);
    for (int e = 0; e < ne; ++e)
        if (S->dc_is_bc[e])
            for (int k = S->O.G.ptr[e]; k < S->O.G.ptr[e + 1]; ++k) S->dc_bc_nodes[S->O.G.idx[k]] = 1;
    div_laplacian(&S->O, &S->G, S->sigma, &S->L);
    S->Ldiag = (double*)xcalloc((size_t)nn, sizeof(double));
    for (int i = 0; i < nn; ++i) {
        S->Ldiag[i] = 1.0;
        if (S->dc_bc_nodes[i]) continue;
        for (int k = S->L.ptr[i]; k < S->L.ptr[i + 1]; ++k)
            if (S->L.idx[k] == i) { S->Ldiag[i] = S->L.val[k]; break; }
    }
    for (int i = 0; i < nn; ++i) {
        if (!S->dc_bc_nodes[i]) continue;
        for (int k = S->L.ptr[i]; k < S->L.ptr[i + 1]; ++k) S->L.val[k] = (S->L.idx[k] == i) ? 1.0 : 0.0;
    }
    for (int i = 0; i < nn; ++i) {
        if (S->dc_bc_nodes[i]) continue;
        for (int k = S->L.ptr[i]; k < S->L.ptr[i + 1]; ++k)
            if (S->dc_bc_nodes[S->L.idx[k]]) S->L.val[k] = 0.0;
    }
    S->me = (double*)xcalloc((size_t)ne, sizeof(double));
    me_sigma(&S->O, &S->G, S->sigma, S->me);
    S->dc_done = 1;
}

/* divcorr_poisson_  forward_solver_fv.cpp:623-722 */
static void divcorr_poisson(m3d_oracle* S, cplx* E, const cplx* phi0) {
    if (!S->dc_done) return;
    const int nn = S->nn, ne = S->ne;
    double div0 = -1;
    cplx* divJ = (cplx*)xcalloc((size_t)nn, sizeof(cplx));
    cplx* phi = (cplx*)xcalloc((size_t)nn, sizeof(cplx));
    cplx* r = (cplx*)xcalloc((size_t)nn, sizeof(cplx));
    cplx* z = (cplx*)xcalloc((size_t)nn, sizeof(cplx));
    cplx* p = (cplx*)xcalloc((size_t)nn, sizeof(cplx));
    cplx* Ap = (cplx*)xcalloc((size_t)nn, sizeof(cplx));
    cplx* gp = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    for (int iter = 0; iter < S->dc_iters; ++iter) {
        div_sigma_E(&S->O, &S->G, S->me, E, divJ);
        if (phi0) for (int i = 0; i < nn; ++i) divJ[i] -= phi0[i];
        for (int i = 0; i < nn; ++i) if (S->dc_bc_nodes[i]) divJ[i] = 0;
        double dn = 0;
        for (int i = 0; i < nn; ++i) dn += cnorm2(divJ[i]);
        dn = sqrt(dn);
        if (iter == 0) div0 = dn;
        double rel = (div0 > 1e-30) ? dn / div0 : 0;
        if ((rel < S->dc_tol && iter > 0) || dn < 1e-12) break;
        for (int i = 0; i < nn; ++i) phi[i] = 0;
        memcpy(r, divJ, sizeof(cplx) * (size_t)nn);
        for (int i = 0; i < nn; ++i) z[i] = (fabs(S->Ldiag[i]) > 1e-30) ? r[i] / S->Ldiag[i] : r[i];
        memcpy(p, z, sizeof(cplx) * (size_t)nn);
        cplx rz = 0;
        for (int i = 0; i < nn; ++i) rz += conj(r[i]) * z[i];
        int cgmax = nn > 500 ? nn : 500;
        for (int cg = 0; cg < cgmax; ++cg) {
            for (int i = 0; i < nn; ++i) {
                Ap[i] = 0;
                for (int k = S->L.ptr[i]; k < S->L.ptr[i + 1]; ++k) Ap[i] += S->L.val[k] * p[S->L.idx[k]];
            }
            cplx pAp = 0;
            for (int i = 0; i < nn; ++i) pAp += conj(p[i]) * Ap[i];
            if (cabs(pAp) < 1e-30) break;
            cplx alpha = rz / pAp;
            for (int i = 0; i < nn; ++i) { phi[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
            double rn = 0;
            for (int i = 0; i < nn; ++i) rn += cnorm2(r[i]);
            if (sqrt(rn) < 1e-10 * dn) break;
            for (int i = 0; i < nn; ++i) z[i] = (fabs(S->Ldiag[i]) > 1e-30) ? r[i] / S->Ldiag[i] : r[i];
            cplx rzn = 0;
            for (int i = 0; i < nn; ++i) rzn += conj(r[i]) * z[i];
            cplx beta = rzn / (rz + CMPLX(1e-30, 0));
            for (int i = 0; i < nn; ++i) p[i] = z[i] + beta * p[i];
            rz = rzn;
        }
        apply_gradient(&S->O, phi, gp);
        for (int i = 0; i < ne; ++i) if (!S->dc_is_bc[i]) E[i] -= gp[i];
    }
    free(divJ); free(phi); free(r); free(z); free(p); free(Ap); free(gp);
}

/* assemble_system_ + compute_bc_flags_  (forward_solver_fv.cpp:93-97, :1743-1750) */
static void factorize(m3d_oracle* S, double freq) {
    S->omega = M3D_TWOPI * freq;
    if (S->have_A) csrc_free(&S->A);
    assemble(&S->O, &S->G, S->omega, S->sigma, &S->A);
    S->have_A = 1;
    if (S->divcorr) compute_bc_flags(S);
}

/* E_primary  forward_solver_fv.cpp:121-136 */
static cplx e_primary(cplx ik, double z) {
    if (z >= 0.0) return CMPLX(1.0, 0.0) + ik * z;
    return cexp(ik * z);
}

/* find_stations_  forward_solver_fv.cpp:1393-1485 */
static void find_stations(m3d_oracle* S) {
    if (S->st_cell) return;
    S->st_cell = (int*)xcalloc((size_t)S->ns + 1, sizeof(int));
    const mesh_t* m = &S->m;
    for (int si = 0; si < S->ns; ++si) {
        double sx = S->sxyz[3 * si], sy = S->sxyz[3 * si + 1], sz = 0.0;
        int best = -1, fb = -1;
        double bcz = 1e30, fbd = 1e30;
        for (int c = 0; c < m->nc; ++c) {
            if (m->type[c] == 1) continue;
            double cx = m->cx[c], cy = m->cy[c], cz = m->cz[c];
            double hdx, hdy, hdz;
            cell_size_xyz(m, c, &hdx, &hdy, &hdz);
            int in_x = (sx >= cx - hdx / 2 - 1.0) && (sx <= cx + hdx / 2 + 1.0);
            int in_y = (sy >= cy - hdy / 2 - 1.0) && (sy <= cy + hdy / 2 + 1.0);
            if (in_x && in_y && cz < 0) {
                if (fabs(cz) < bcz) { bcz = fabs(cz); best = c; }
            }
            double d = sqrt((cx - sx) * (cx - sx) + (cy - sy) * (cy - sy) + (cz - sz) * (cz - sz));
            if (d < fbd) { fbd = d; fb = c; }
        }
        if (best < 0) best = fb;
        S->st_cell[si] = best;
    }
    S->hc = (hcache_t*)xcalloc((size_t)S->ns + 1, sizeof(hcache_t));
}

/* extract_impedance_  forward_solver_fv.cpp:1490-1727.  Z_out: [ns][4] */
static void extract_impedance(m3d_oracle* S, cplx* Zout) {
    const double omega = S->omega;
    const cplx iwmu = CMPLX(0.0, omega * M3D_MU0);
    for (int si = 0; si < S->ns; ++si) {
        int cell = S->st_cell[si];
        if (cell < 0) continue;
        double cx = S->m.cx[cell], cy = S->m.cy[cell], cz = S->m.cz[cell];
        double cdx, cdy, cdz;
        cell_size_xyz(&S->m, cell, &cdx, &cdy, &cdz);
        cplx Ex1t = 0, Ex1b = 0, Ex2t = 0, Ex2b = 0, Ey1t = 0, Ey1b = 0, Ey2t = 0, Ey2b = 0;
        cplx Ez1px = 0, Ez1mx = 0, Ez2px = 0, Ez2mx = 0, Ez1py = 0, Ez1my = 0, Ez2py = 0, Ez2my = 0;
        int nxt = 0, nxb = 0, nyt = 0, nyb = 0, npx = 0, nmx = 0, npy = 0, nmy = 0;
        for (int k = S->G.ce_ptr[cell]; k < S->G.ce_ptr[cell + 1]; ++k) {
            int e = S->G.ce_id[k];
            int d = S->G.edir[e];
            if (d == 0) {
                if (S->G.ez[e] > cz) { Ex1t += S->E1[e]; Ex2t += S->E2[e]; ++nxt; }
                else { Ex1b += S->E1[e]; Ex2b += S->E2[e]; ++nxb; }
            } else if (d == 1) {
                if (S->G.ez[e] > cz) { Ey1t += S->E1[e]; Ey2t += S->E2[e]; ++nyt; }
                else { Ey1b += S->E1[e]; Ey2b += S->E2[e]; ++nyb; }
            } else if (d == 2) {
                if (S->G.ex[e] > cx) { Ez1px += S->E1[e]; Ez2px += S->E2[e]; ++npx; }
                else { Ez1mx += S->E1[e]; Ez2mx += S->E2[e]; ++nmx; }
                if (S->G.ey[e] > cy) { Ez1py += S->E1[e]; Ez2py += S->E2[e]; ++npy; }
                else { Ez1my += S->E1[e]; Ez2my += S->E2[e]; ++nmy; }
            }
        }
        if (nxt > 0) { Ex1t /= CMPLX(nxt, 0); Ex2t /= CMPLX(nxt, 0); }
        if (nxb > 0) { Ex1b /= CMPLX(nxb, 0); Ex2b /= CMPLX(nxb, 0); }
        if (nyt > 0) { Ey1t /= CMPLX(nyt, 0); Ey2t /= CMPLX(nyt, 0); }
        if (nyb > 0) { Ey1b /= CMPLX(nyb, 0); Ey2b /= CMPLX(nyb, 0); }
        if (npx > 0) { Ez1px /= CMPLX(npx, 0); Ez2px /= CMPLX(npx, 0); }
        if (nmx > 0) { Ez1mx /= CMPLX(nmx, 0); Ez2mx /= CMPLX(nmx, 0); }
        if (npy > 0) { Ez1py /= CMPLX(npy, 0); Ez2py /= CMPLX(npy, 0); }
        if (nmy > 0) { Ez1my /= CMPLX(nmy, 0); Ez2my /= CMPLX(nmy, 0); }
        cplx h = CMPLX(0.5, 0);
        cplx Ex1 = (nxt > 0 && nxb > 0) ? (Ex1t + Ex1b) * h : ((nxt > 0) ? Ex1t : Ex1b);
        cplx Ey1 = (nyt > 0 && nyb > 0) ? (Ey1t + Ey1b) * h : ((nyt > 0) ? Ey1t : Ey1b);
        cplx Ex2 = (nxt > 0 && nxb > 0) ? (Ex2t + Ex2b) * h : ((nxt > 0) ? Ex2t : Ex2b);
        cplx Ey2 = (nyt > 0 && nyb > 0) ? (Ey2t + Ey2b) * h : ((nyt > 0) ? Ey2t : Ey2b);
        cplx dEx1 = 0, dEx2 = 0, dEy1 = 0, dEy2 = 0;
        if (nxt > 0 && nxb > 0) { dEx1 = (Ex1t - Ex1b) / cdz; dEx2 = (Ex2t - Ex2b) / cdz; }
        if (nyt > 0 && nyb > 0) { dEy1 = (Ey1t - Ey1b) / cdz; dEy2 = (Ey2t - Ey2b) / cdz; }
        cplx dEz1x = 0, dEz2x = 0, dEz1y = 0, dEz2y = 0;
        if (npx > 0 && nmx > 0) { dEz1x = (Ez1px - Ez1mx) / cdx; dEz2x = (Ez2px - Ez2mx) / cdx; }
        if (npy > 0 && nmy > 0) { dEz1y = (Ez1py - Ez1my) / cdy; dEz2y = (Ez2py - Ez2my) / cdy; }
        cplx Hx1 = (dEz1y - dEy1) / iwmu;
        cplx Hy1 = (dEx1 - dEz1x) / iwmu;
        cplx Hx2 = (dEz2y - dEy2) / iwmu;
        cplx Hy2 = (dEx2 - dEz2x) / iwmu;
        cplx det = Hx1 * Hy2 - Hx2 * Hy1;
        hcache_t* c = &S->hc[si];
        c->Hx1 = Hx1; c->Hy1 = Hy1; c->Hx2 = Hx2; c->Hy2 = Hy2; c->det_H = det;
        c->cdx = cdx; c->cdy = cdy; c->cdz = cdz;
        cplx Zxx, Zxy, Zyx, Zyy;
        if (cabs(det) > 1e-30) {
            Zxx = (Ex1 * Hy2 - Ex2 * Hy1) / det;
            Zxy = (Ex2 * Hx1 - Ex1 * Hx2) / det;
            Zyx = (Ey1 * Hy2 - Ey2 * Hy1) / det;
            Zyy = (Ey2 * Hx1 - Ey1 * Hx2) / det;
        } else {
            double sa = S->sigma[cell];
            cplx Z1 = csqrt(iwmu / CMPLX(sa, 0));
            Zxx = 0; Zxy = Z1; Zyx = -Z1; Zyy = 0;
        }
        c->Zxx = Zxx; c->Zxy = Zxy; c->Zyx = Zyx; c->Zyy = Zyy;
        if (Zout) { Zout[4 * si] = Zxx; Zout[4 * si + 1] = Zxy; Zout[4 * si + 2] = Zyx; Zout[4 * si + 3] = Zyy; }
    }
}

/* solve_frequency  forward_solver_fv.cpp:84-531 (air_bc_iterations = 1) */
static void solve_frequency(m3d_oracle* S, double freq, cplx* Zout) {
    factorize(S, freq);
    const int ne = S->ne;
    const mesh_t* m = &S->m;
    const double bt = cell_size_min(m, 0) * 0.1;
    const cplx ik = csqrt(CMPLX(0.0, S->omega * M3D_MU0 * S->sigma_bg));
    char* is_bc = (char*)xcalloc((size_t)ne, 1);
    cplx* bc1 = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    cplx* bc2 = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    for (int e = 0; e < ne; ++e) {
        double x = S->G.ex[e], y = S->G.ey[e], z = S->G.ez[e];
        int d = S->G.edir[e];
        int onb = (x <= m->xmin + bt || x >= m->xmax - bt || y <= m->ymin + bt || y >= m->ymax - bt ||
                   z <= m->zmin + bt || z >= m->zmax - bt);
        int air = z > S->air_z;
        if (onb || air) {
            cplx Ep = e_primary(ik, z);
            if (d == 0) bc1[e] = Ep;
            if (d == 1) bc2[e] = Ep;
            is_bc[e] = 1;
        }
    }
    char* isc = (char*)xcalloc((size_t)ne, 1);
    for (int h = 0; h < S->O.nhp; ++h) isc[S->O.hp[3 * h]] = 1;
    for (int i = 0; i < ne; ++i) isc[i] = is_bc[i] || isc[i];
    /* identity rows / zero columns; keep the lifted entries (:219-235) */
    csrc_t* A = &S->A;
    int nsv = 0, svcap = 1024;
    int* sv_row = (int*)xcalloc((size_t)svcap, sizeof(int));
    int* sv_k = (int*)xcalloc((size_t)svcap, sizeof(int));
    cplx* sv_v = (cplx*)xcalloc((size_t)svcap, sizeof(cplx));
    for (int i = 0; i < ne; ++i)
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
            int j = A->idx[k];
            if (isc[i] || isc[j]) {
                if (nsv == svcap) {
                    svcap *= 2;
                    sv_row = realloc(sv_row, sizeof(int) * svcap);
                    sv_k = realloc(sv_k, sizeof(int) * svcap);
                    sv_v = realloc(sv_v, sizeof(cplx) * svcap);
                }
                sv_row[nsv] = i; sv_k[nsv] = k; sv_v[nsv] = A->val[k]; nsv++;
                if (isc[i]) A->val[k] = (j == i) ? (cplx)1.0 : (cplx)0.0;
                else A->val[k] = 0;
            }
        }
    ssor_t M;
    ssor_setup(&M, A);
    cplx* rhs = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    cplx* Ep = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    cplx* AEp = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    cplx* rs = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    cplx* Es = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    for (int pol = 0; pol < 2; ++pol) {
        const cplx* Ebc = pol == 0 ? bc1 : bc2;
        cplx* Eout = pol == 0 ? S->E1 : S->E2;
        /* build_rhs (:244-255) */
        for (int i = 0; i < ne; ++i) rhs[i] = 0;
        for (int t = 0; t < nsv; ++t) {
            if (isc[sv_row[t]]) continue;
            int j = A->idx[sv_k[t]];
            if (is_bc[j]) rhs[sv_row[t]] -= sv_v[t] * Ebc[j];
        }
        for (int i = 0; i < ne; ++i) if (is_bc[i]) rhs[i] = Ebc[i];
        if (S->scattered) {
            for (int i = 0; i < ne; ++i) Ep[i] = (S->G.edir[i] == pol) ? e_primary(ik, S->G.ez[i]) : 0;
            csrc_matvec(A, Ep, AEp);
            for (int i = 0; i < ne; ++i) rs[i] = rhs[i] - AEp[i];
            for (int i = 0; i < ne; ++i) Es[i] = 0;
            bicg_res_t br = bicgstab(A, &M, rs, Es, S->tol, S->maxiter);
            log_iters(S, br.iterations);
            for (int h = 0; h < S->O.nhp; ++h)
                Es[S->O.hp[3 * h]] = CMPLX(0.5, 0) * (Es[S->O.hp[3 * h + 1]] + Es[S->O.hp[3 * h + 2]]);
            for (int i = 0; i < ne; ++i) Eout[i] = Ep[i] + Es[i];
            for (int i = 0; i < ne; ++i) if (is_bc[i]) Eout[i] = Ebc[i];
            if (S->divcorr && S->dc_done) divcorr_poisson(S, Eout, NULL);
        } else {
            for (int i = 0; i < ne; ++i) Eout[i] = (S->G.edir[i] == pol) ? e_primary(ik, S->G.ez[i]) : 0;
            for (int i = 0; i < ne; ++i) if (is_bc[i]) Eout[i] = Ebc[i];
            bicg_res_t br = bicgstab(A, &M, rhs, Eout, S->tol, S->maxiter);
            log_iters(S, br.iterations);
            for (int h = 0; h < S->O.nhp; ++h)
                Eout[S->O.hp[3 * h]] = CMPLX(0.5, 0) * (Eout[S->O.hp[3 * h + 1]] + Eout[S->O.hp[3 * h + 2]]);
            for (int i = 0; i < ne; ++i) if (is_bc[i]) Eout[i] = rhs[i];
            if (S->divcorr && S->dc_done) divcorr_poisson(S, Eout, NULL);
        }
    }
    ssor_free(&M);
    extract_impedance(S, Zout);
    free(is_bc); free(bc1); free(bc2); free(isc); free(sv_row); free(sv_k); free(sv_v);
    free(rhs); free(Ep); free(AEp); free(rs); free(Es);
}

/* solve_system_  forward_solver_fv.cpp:727-759 */
static void solve_system(m3d_oracle* S, const cplx* rhs, cplx* x) {
    ssor_t M;
    ssor_setup(&M, &S->A);
    double tol = S->tol_override > 0 ? S->tol_override : S->tol;
    bicg_res_t r = bicgstab(&S->A, &M, rhs, x, tol, S->maxiter);
    log_iters(S, r.iterations);
    if (!r.converged && r.residual > 1.0) memset(x, 0, sizeof(cplx) * (size_t)S->ne);
    ssor_free(&M);
}

/* solve_with_divcorr_  forward_solver_fv.cpp:778-888 */
static void solve_with_divcorr(m3d_oracle* S, const cplx* rhs, cplx* x, const cplx* phi0) {
    const int ne = S->ne;
    double tol = S->tol_override > 0 ? S->tol_override : S->tol;
    double rn = 0;
    for (int i = 0; i < ne; ++i) rn += cnorm2(rhs[i]);
    rn = sqrt(rn);
    if (rn < 1e-30) rn = 1.0;
    ssor_t M;
    ssor_setup(&M, &S->A);
    if (phi0) divcorr_poisson(S, x, phi0);
    int total = 0;
    double prev = 1e30;
    cplx* Ax = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    for (int outer = 0; outer < S->dc_outer; ++outer) {
        bicg_res_t r = bicgstab(&S->A, &M, rhs, x, tol, S->dc_iter_per);
        total += r.iterations;
        if (r.residual > 1.0) { memset(x, 0, sizeof(cplx) * (size_t)ne); break; }
        if (r.converged) break;
        divcorr_poisson(S, x, phi0);
        csrc_matvec(&S->A, x, Ax);
        double res = 0;
        for (int i = 0; i < ne; ++i) res += cnorm2(Ax[i] - rhs[i]);
        res = sqrt(res);
        double rel = res / rn;
        if (rel < tol) break;
        if (outer > 0 && rel > 0.95 * prev) break;
        prev = rel;
    }
    log_iters(S, total);
    free(Ax);
    ssor_free(&M);
}

/* compute_phi0  forward_solver_fv.cpp:893-908 */
static void compute_phi0(m3d_oracle* S, const cplx* rhs, cplx* phi0) {
    cplx iw = CMPLX(0, S->omega);
    for (int i = 0; i < S->nn; ++i) phi0[i] = 0;
    for (int e = 0; e < S->ne; ++e)
        if (!S->O.dead_e[e])
            for (int k = S->O.G.ptr[e]; k < S->O.G.ptr[e + 1]; ++k) phi0[S->O.G.idx[k]] += S->O.G.val[k] * rhs[e];
    for (int i = 0; i < S->nn; ++i) phi0[i] /= iw;
}

/* adjoint_solve / solve_rhs  forward_solver_fv.cpp:914-940 */
static void adjoint_solve(m3d_oracle* S, const cplx* rhs, cplx* lam) {
    memset(lam, 0, sizeof(cplx) * (size_t)S->ne);
    if (S->divcorr && S->dc_done && S->omega > 0) {
        cplx* phi0 = (cplx*)xcalloc((size_t)S->nn, sizeof(cplx));
        compute_phi0(S, rhs, phi0);
        solve_with_divcorr(S, rhs, lam, phi0);
        free(phi0);
    } else {
        solve_system(S, rhs, lam);
    }
}

/* build_adjoint_rhs_from_residual  forward_solver_fv.cpp:1804-2013 */
static void adjoint_rhs(m3d_oracle* S, const cplx* wr, cplx* a1, cplx* a2) {
    const int ne = S->ne;
    memset(a1, 0, sizeof(cplx) * (size_t)ne);
    memset(a2, 0, sizeof(cplx) * (size_t)ne);
    const cplx iwmu = CMPLX(0, S->omega * M3D_MU0);
    for (int si = 0; si < S->ns; ++si) {
        int cell = S->st_cell[si];
        if (cell < 0) continue;
        const cplx* w = wr + 4 * si;
        const hcache_t* hc = &S->hc[si];
        cplx det = hc->det_H;
        if (cabs(det) < 1e-30) continue;
        cplx sx1 = (w[0] * hc->Hy2 - w[1] * hc->Hx2) / det;
        cplx sy1 = (w[2] * hc->Hy2 - w[3] * hc->Hx2) / det;
        cplx sx2 = (-w[0] * hc->Hy1 + w[1] * hc->Hx1) / det;
        cplx sy2 = (-w[2] * hc->Hy1 + w[3] * hc->Hx1) / det;
        cplx aHx1 = -(hc->Zxx * sx1 + hc->Zyx * sy1);
        cplx aHy1 = -(hc->Zxy * sx1 + hc->Zyy * sy1);
        cplx aHx2 = -(hc->Zxx * sx2 + hc->Zyx * sy2);
        cplx aHy2 = -(hc->Zxy * sx2 + hc->Zyy * sy2);
        double cx = S->m.cx[cell], cy = S->m.cy[cell], cz = S->m.cz[cell];
        double cdx = hc->cdx, cdy = hc->cdy, cdz = hc->cdz;
        int nxt = 0, nxb = 0, nyt = 0, nyb = 0, npx = 0, nmx = 0, npy = 0, nmy = 0;
        for (int k = S->G.ce_ptr[cell]; k < S->G.ce_ptr[cell + 1]; ++k) {
            int e = S->G.ce_id[k];
            int d = S->G.edir[e];
            if (d == 0) { if (S->G.ez[e] > cz) ++nxt; else ++nxb; }
            else if (d == 1) { if (S->G.ez[e] > cz) ++nyt; else ++nyb; }
            else if (d == 2) {
                if (S->G.ex[e] > cx) ++npx; else ++nmx;
                if (S->G.ey[e] > cy) ++npy; else ++nmy;
            }
        }
        double wxt = nxt > 0 ? 0.5 / nxt : 0.0, wxb = nxb > 0 ? 0.5 / nxb : 0.0;
        double wyt = nyt > 0 ? 0.5 / nyt : 0.0, wyb = nyb > 0 ? 0.5 / nyb : 0.0;
        if (nxt == 0) wxb = nxb > 0 ? 1.0 / nxb : 0.0;
        if (nxb == 0) wxt = nxt > 0 ? 1.0 / nxt : 0.0;
        if (nyt == 0) wyb = nyb > 0 ? 1.0 / nyb : 0.0;
        if (nyb == 0) wyt = nyt > 0 ? 1.0 / nyt : 0.0;
        cplx icdz = CMPLX(1, 0) / (iwmu * cdz);
        cplx icdx = CMPLX(1, 0) / (iwmu * cdx);
        cplx icdy = CMPLX(1, 0) / (iwmu * cdy);
        for (int k = S->G.ce_ptr[cell]; k < S->G.ce_ptr[cell + 1]; ++k) {
            int e = S->G.ce_id[k];
            int d = S->G.edir[e];
            if (d == 0) {
                int top = S->G.ez[e] > cz;
                double we = top ? wxt : wxb;
                a1[e] += sx1 * we; a2[e] += sx2 * we;
                if (top && nxt > 0) { cplx wh = icdz / (double)nxt; a1[e] += aHy1 * wh; a2[e] += aHy2 * wh; }
                else if (!top && nxb > 0) { cplx wh = -icdz / (double)nxb; a1[e] += aHy1 * wh; a2[e] += aHy2 * wh; }
            } else if (d == 1) {
                int top = S->G.ez[e] > cz;
                double we = top ? wyt : wyb;
                a1[e] += sy1 * we; a2[e] += sy2 * we;
                if (top && nyt > 0) { cplx wh = -icdz / (double)nyt; a1[e] += aHx1 * wh; a2[e] += aHx2 * wh; }
                else if (!top && nyb > 0) { cplx wh = icdz / (double)nyb; a1[e] += aHx1 * wh; a2[e] += aHx2 * wh; }
            } else if (d == 2) {
                int py = S->G.ey[e] > cy;
                if (py && npy > 0) { cplx wh = icdy / (double)npy; a1[e] += aHx1 * wh; a2[e] += aHx2 * wh; }
                else if (!py && nmy > 0) { cplx wh = -icdy / (double)nmy; a1[e] += aHx1 * wh; a2[e] += aHx2 * wh; }
                int px = S->G.ex[e] > cx;
                if (px && npx > 0) { cplx wh = -icdx / (double)npx; a1[e] += aHy1 * wh; a2[e] += aHy2 * wh; }
                else if (!px && nmx > 0) { cplx wh = icdx / (double)nmx; a1[e] += aHy1 * wh; a2[e] += aHy2 * wh; }
            }
        }
    }
}

/* constrained set of compute_sensitivity  forward_solver_fv.cpp:1012-1029 */
static void sens_constrained(m3d_oracle* S, char* isc) {
    const mesh_t* m = &S->m;
    const double bt = 1.0;
    for (int e = 0; e < S->ne; ++e) {
        isc[e] = 0;
        if (S->O.dead_e[e]) { isc[e] = 1; continue; }
        double x = S->G.ex[e], y = S->G.ey[e], z = S->G.ez[e];
        if (x <= m->xmin + bt || x >= m->xmax - bt || y <= m->ymin + bt || y >= m->ymax - bt ||
            z <= m->zmin + bt || z >= m->zmax - bt || z > S->air_z)
            isc[e] = 1;
    }
}

/* compute_sensitivity  forward_solver_fv.cpp:989-1059 */
static void sensitivity(m3d_oracle* S, const cplx* E, const cplx* lam, double* g) {
    const int nc = S->nc;
    char* isc = (char*)xcalloc((size_t)S->ne, 1);
    sens_constrained(S, isc);
    cplx iw = CMPLX(0, S->omega);
    for (int c = 0; c < nc; ++c) {
        cplx s = 0;
        double sc = S->sigma[c];
        for (int k = S->G.ce_ptr[c]; k < S->G.ce_ptr[c + 1]; ++k) {
            int e = S->G.ce_id[k];
            if (isc[e]) continue;
            double L = S->G.elen[e];
            double Ad = S->O.adual[e];
            int na = 0;
            for (int u = 0; u < S->G.adj[e].n; ++u) {
                int ac = S->G.adj[e].a[u];
                if (ac >= 0 && ac < nc) ++na;
            }
            if (na == 0) continue;
            double dMe = sc * Ad * L / na;
            s += lam[e] * E[e] * dMe;
        }
        g[c] = creal(iw * s);
    }
    free(isc);
}

/* build_perturbation_rhs  forward_solver_fv.cpp:945-984 (pol 1 or 2) */
static void perturbation_rhs(m3d_oracle* S, int pol, const double* dsig, cplx* out) {
    const int nc = S->nc;
    memset(out, 0, sizeof(cplx) * (size_t)S->ne);
    const cplx* Eb = (pol == 1) ? S->E1 : S->E2;
    cplx iw = CMPLX(0, S->omega);
    for (int c = 0; c < nc; ++c) {
        if (fabs(dsig[c]) < 1e-30) continue;
        double sc = S->sigma[c];
        for (int k = S->G.ce_ptr[c]; k < S->G.ce_ptr[c + 1]; ++k) {
            int e = S->G.ce_id[k];
            double L = S->G.elen[e];
            double vol = L * L * L;
            double si = 0.0; int na = 0;
            for (int u = 0; u < S->G.adj[e].n; ++u) {
                int ac = S->G.adj[e].a[u];
                if (ac >= 0 && ac < nc && S->sigma[ac] > 1e-30) { si += 1.0 / S->sigma[ac]; ++na; }
            }
            double sa = (na > 0 && si > 1e-30) ? na / si : 1e-8;
            double dMe = vol * sa * sa / (na * sc * sc);
            out[e] -= iw * CMPLX(dsig[c] * dMe, 0) * Eb[e];
        }
    }
}

/* extract_delta_impedance_complex  forward_solver_fv.cpp:2018-2065 */
static void delta_impedance(m3d_oracle* S, const cplx* dE, int pol, cplx* dZ) {
    for (int si = 0; si < S->ns; ++si) {
        int cell = S->st_cell[si];
        for (int k = 0; k < 4; ++k) dZ[4 * si + k] = 0;
        if (cell < 0) continue;
        cplx dEx = 0, dEy = 0;
        int nx = 0, ny = 0;
        for (int k = S->G.ce_ptr[cell]; k < S->G.ce_ptr[cell + 1]; ++k) {
            int e = S->G.ce_id[k];
            if (S->G.edir[e] == 0) { dEx += dE[e]; ++nx; }
            else if (S->G.edir[e] == 1) { dEy += dE[e]; ++ny; }
        }
        if (nx > 0) dEx /= CMPLX(nx, 0);
        if (ny > 0) dEy /= CMPLX(ny, 0);
        const hcache_t* hc = &S->hc[si];
        if (cabs(hc->det_H) < 1e-30) continue;
        cplx id = CMPLX(1, 0) / hc->det_H;
        if (pol == 1) {
            dZ[4 * si] = dEx * hc->Hy2 * id; dZ[4 * si + 1] = dEx * (-hc->Hx2) * id;
            dZ[4 * si + 2] = dEy * hc->Hy2 * id; dZ[4 * si + 3] = dEy * (-hc->Hx2) * id;
        } else {
            dZ[4 * si] = dEx * (-hc->Hy1) * id; dZ[4 * si + 1] = dEx * hc->Hx1 * id;
            dZ[4 * si + 2] = dEy * (-hc->Hy1) * id; dZ[4 * si + 3] = dEy * hc->Hx1 * id;
        }
    }
}

/* release  forward_solver_fv.cpp:1070-1077 */
static void release(m3d_oracle* S) {
    if (S->have_A) csrc_free(&S->A);
    S->have_A = 0;
    free(S->L.ptr); free(S->L.idx); free(S->L.val);
    memset(&S->L, 0, sizeof(S->L));
    free(S->Ldiag); S->Ldiag = NULL;
    free(S->dc_is_bc); S->dc_is_bc = NULL;
    free(S->dc_bc_nodes); S->dc_bc_nodes = NULL;
    free(S->me); S->me = NULL;
    S->dc_done = 0;
}

/* ------------------------------------------------------------------------ */
/* public API (m3d_oracle.h)                                                 */
/* ------------------------------------------------------------------------ */

m3d_oracle* m3d_oracle_create(const m3d_case* cs) {
    m3d_oracle* S = (m3d_oracle*)xcalloc(1, sizeof(m3d_oracle));
    mesh_t* m = &S->m;
    m->xmin = cs->domain[0]; m->xmax = cs->domain[1];
    m->ymin = cs->domain[2]; m->ymax = cs->domain[3];
    m->zmin = cs->domain[4]; m->zmax = cs->domain[5];
    m->min_level = cs->min_level; m->max_level = cs->max_level;
    m->nc = cs->n_cells;
    m->level = cs->level; m->cx = cs->cx; m->cy = cs->cy; m->cz = cs->cz; m->type = cs->cell_type;
    grid_build(&S->G, m);
    ops_build(&S->O, &S->G);
    S->ne = S->G.ne; S->nc = S->G.nc; S->nn = S->O.nn;
    S->sigma = (double*)xcalloc((size_t)S->nc, sizeof(double));
    memcpy(S->sigma, cs->sigma, sizeof(double) * (size_t)S->nc);
    S->sigma_bg = cs->sigma_bg > 0 ? cs->sigma_bg : 0.01;
    S->tol = cs->bicgstab_tol; S->maxiter = cs->bicgstab_maxiter;
    S->scattered = cs->scattered_field; S->air_z = cs->air_z_threshold;
    S->divcorr = cs->div_correction; S->dc_iters = cs->div_corr_iters; S->dc_tol = cs->div_corr_tol;
    S->dc_outer = cs->divcorr_outer_max; S->dc_iter_per = cs->divcorr_iter_per_dc;
    S->E1 = (cplx*)xcalloc((size_t)S->ne, sizeof(cplx));
    S->E2 = (cplx*)xcalloc((size_t)S->ne, sizeof(cplx));
    S->ns = cs->n_stations;
    S->sxyz = cs->station_xyz;   /* caller keeps the case alive */
    return S;
}

void m3d_oracle_destroy(m3d_oracle* S) {
    if (!S) return;
    release(S);
    grid_free(&S->G);
    ops_free(&S->O);
    free(S->sigma); free(S->E1); free(S->E2); free(S->st_cell); free(S->hc);
    free(S);
}

int m3d_oracle_sizes(const m3d_oracle* S, int* ne, int* nf, int* nc, int* nn) {
    if (ne) *ne = S->ne;
    if (nf) *nf = S->G.nf;
    if (nc) *nc = S->nc;
    if (nn) *nn = S->nn;
    return 0;
}

int m3d_oracle_set_sigma(m3d_oracle* S, const double* sigma) {
    memcpy(S->sigma, sigma, sizeof(double) * (size_t)S->nc);
    return 0;
}

int m3d_oracle_set_tol_override(m3d_oracle* S, double tol) { S->tol_override = tol; return 0; }

int m3d_oracle_solve_frequency(m3d_oracle* S, double freq, double* Z_out) {
    find_stations(S);
    S->n_last = 0;
    solve_frequency(S, freq, (cplx*)Z_out);
    return 0;
}

int m3d_oracle_factorize(m3d_oracle* S, double freq) {
    find_stations(S);
    factorize(S, freq);
    return 0;
}

int m3d_oracle_release(m3d_oracle* S) { release(S); return 0; }

int m3d_oracle_get_E(const m3d_oracle* S, int pol, double* out) {
    memcpy(out, pol == 0 ? S->E1 : S->E2, sizeof(cplx) * (size_t)S->ne);
    return 0;
}

int m3d_oracle_set_E(m3d_oracle* S, const double* E1, const double* E2) {
    memcpy(S->E1, E1, sizeof(cplx) * (size_t)S->ne);
    memcpy(S->E2, E2, sizeof(cplx) * (size_t)S->ne);
    return 0;
}

int m3d_oracle_adjoint_rhs(m3d_oracle* S, const double* wr, double* rhs1, double* rhs2) {
    adjoint_rhs(S, (const cplx*)wr, (cplx*)rhs1, (cplx*)rhs2);
    return 0;
}

int m3d_oracle_adjoint_solve(m3d_oracle* S, const double* rhs, double* lam) {
    S->n_last = 0;
    adjoint_solve(S, (const cplx*)rhs, (cplx*)lam);
    return 0;
}

int m3d_oracle_sensitivity(m3d_oracle* S, const double* E, const double* lam, double* g) {
    sensitivity(S, (const cplx*)E, (const cplx*)lam, g);
    return 0;
}

int m3d_oracle_perturbation_rhs(m3d_oracle* S, int pol, const double* dsig, double* out) {
    perturbation_rhs(S, pol, dsig, (cplx*)out);
    return 0;
}

int m3d_oracle_delta_impedance(m3d_oracle* S, const double* dE, int pol, double* dZ) {
    delta_impedance(S, (const cplx*)dE, pol, (cplx*)dZ);
    return 0;
}

int m3d_oracle_last_iters(const m3d_oracle* S, int* out, int cap) {
    int n = S->n_last < cap ? S->n_last : cap;
    for (int i = 0; i < n; ++i) out[i] = S->last_iters[i];
    return n;
}

int m3d_oracle_station_cells(const m3d_oracle* S, int* out) {
    for (int s = 0; s < S->ns; ++s) out[s] = S->st_cell ? S->st_cell[s] : -1;
    return 0;
}

/* The BC-modified system of the current frequency (after solve_frequency). */
int m3d_oracle_matrix_nnz(const m3d_oracle* S) { return S->have_A ? S->A.ptr[S->ne] : -1; }

int m3d_oracle_get_matrix(const m3d_oracle* S, int* ptr, int* idx, double* val) {
    if (!S->have_A) return 1;
    memcpy(ptr, S->A.ptr, sizeof(int) * ((size_t)S->ne + 1));
    memcpy(idx, S->A.idx, sizeof(int) * (size_t)S->A.ptr[S->ne]);
    memcpy(val, S->A.val, sizeof(cplx) * (size_t)S->A.ptr[S->ne]);
    return 0;
}

/* Edge geometry and the operator pieces the GPU layout is built from. */
int m3d_oracle_get_edges(const m3d_oracle* S, double* xyz, double* len, int* dir, double* adual,
                         int* dead, int* node1, int* node2) {
    for (int e = 0; e < S->ne; ++e) {
        if (xyz) { xyz[3 * e] = S->G.ex[e]; xyz[3 * e + 1] = S->G.ey[e]; xyz[3 * e + 2] = S->G.ez[e]; }
        if (len) len[e] = S->G.elen[e];
        if (dir) dir[e] = S->G.edir[e];
        if (adual) adual[e] = S->O.adual[e];
        if (dead) dead[e] = S->O.dead_e[e];
        if (node1) node1[e] = S->O.gn1[e];
        if (node2) node2[e] = S->O.gn2[e];
    }
    return 0;
}

/* Whole gradient loop of InversionFV::compute_gradient_ (inversion_fv.cpp:230-291)
 * for frequencies freqs[0..nf): obs_Z / obs_err as in m3d_case.  Outputs Z
 * [nf][ns][4] and grad [nc]; both may be NULL. */
int m3d_oracle_gradient(m3d_oracle* S, const double* freqs, int nf, const double* obs_Z,
                        const double* obs_err, double* Z_out, double* grad) {
    const int ns = S->ns, ne = S->ne, nc = S->nc;
    cplx* Z = (cplx*)xcalloc((size_t)ns * 4 + 1, sizeof(cplx));
    cplx* wr = (cplx*)xcalloc((size_t)ns * 4 + 1, sizeof(cplx));
    cplx* a1 = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    cplx* a2 = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    cplx* l1 = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    cplx* l2 = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    double* g1 = (double*)xcalloc((size_t)nc, sizeof(double));
    double* g2 = (double*)xcalloc((size_t)nc, sizeof(double));
    if (grad) for (int c = 0; c < nc; ++c) grad[c] = 0.0;
    for (int f = 0; f < nf; ++f) {
        find_stations(S);
        solve_frequency(S, freqs[f], Z);
        if (Z_out) memcpy(Z_out + (size_t)f * ns * 8, Z, sizeof(cplx) * (size_t)ns * 4);
        if (grad && obs_Z) {
            for (int s = 0; s < ns; ++s)
                for (int k = 0; k < 4; ++k) {
                    size_t o = ((size_t)s * nf + f) * 4 + k;
                    double err = obs_err[o];
                    cplx ov = CMPLX(obs_Z[2 * o], obs_Z[2 * o + 1]);
                    double w = err > 0 ? 1.0 : 0.0;
                    if (w <= 0.0 || err <= 0.0) wr[4 * s + k] = 0;
                    else { double wt = 1.0 / err; wr[4 * s + k] = wt * wt * conj(ov - Z[4 * s + k]); }
                }
            adjoint_rhs(S, wr, a1, a2);
            adjoint_solve(S, a1, l1);
            adjoint_solve(S, a2, l2);
            sensitivity(S, S->E1, l1, g1);
            sensitivity(S, S->E2, l2, g2);
            for (int c = 0; c < nc; ++c) grad[c] += g1[c] + g2[c];
        }
        release(S);
    }
    free(Z); free(wr); free(a1); free(a2); free(l1); free(l2); free(g1); free(g2);
    return 0;
}

#include <time.h>

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* CPU-baseline sample: assemble frequency `freq` with the reference's BC
 * elimination (solve_frequency :84-241), take the pol-1 scattered-field
 * right-hand side and run exactly `n_iter` iterations of the reference's
 * SSOR-BiCGStab (tolerance 0).  Returns seconds spent in the iterations and,
 * through setup_s, seconds spent on assembly + BC elimination + SSOR setup. */
double m3d_oracle_time_iterations(m3d_oracle* S, double freq, int n_iter, double* setup_s) {
    const double t0 = now_s();
    factorize(S, freq);
    const int ne = S->ne;
    const mesh_t* m = &S->m;
    const double bt = cell_size_min(m, 0) * 0.1;
    const cplx ik = csqrt(CMPLX(0.0, S->omega * M3D_MU0 * S->sigma_bg));
    char* is_bc = (char*)xcalloc((size_t)ne, 1);
    char* isc = (char*)xcalloc((size_t)ne, 1);
    cplx* bc1 = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    for (int e = 0; e < ne; ++e) {
        double x = S->G.ex[e], y = S->G.ey[e], z = S->G.ez[e];
        int onb = (x <= m->xmin + bt || x >= m->xmax - bt || y <= m->ymin + bt || y >= m->ymax - bt ||
                   z <= m->zmin + bt || z >= m->zmax - bt);
        if (onb || z > S->air_z) { is_bc[e] = 1; if (S->G.edir[e] == 0) bc1[e] = e_primary(ik, z); }
    }
    for (int h = 0; h < S->O.nhp; ++h) isc[S->O.hp[3 * h]] = 1;
    for (int i = 0; i < ne; ++i) isc[i] = is_bc[i] || isc[i];
    csrc_t* A = &S->A;
    cplx* rhs = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    for (int i = 0; i < ne; ++i)
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
            int j = A->idx[k];
            if (isc[i] || isc[j]) {
                if (!isc[i] && is_bc[j]) rhs[i] -= A->val[k] * bc1[j];
                if (isc[i]) A->val[k] = (j == i) ? (cplx)1.0 : (cplx)0.0;
                else A->val[k] = 0;
            }
        }
    for (int i = 0; i < ne; ++i) if (is_bc[i]) rhs[i] = bc1[i];
    ssor_t M;
    ssor_setup(&M, A);
    cplx* Ep = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    cplx* AEp = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    for (int i = 0; i < ne; ++i) Ep[i] = (S->G.edir[i] == 0) ? e_primary(ik, S->G.ez[i]) : 0;
    csrc_matvec(A, Ep, AEp);
    for (int i = 0; i < ne; ++i) rhs[i] -= AEp[i];
    cplx* x = (cplx*)xcalloc((size_t)ne, sizeof(cplx));
    const double t1 = now_s();
    bicgstab(A, &M, rhs, x, 0.0, n_iter);
    const double t2 = now_s();
    if (setup_s) *setup_s = t1 - t0;
    ssor_free(&M);
    free(is_bc); free(isc); free(bc1); free(rhs); free(Ep); free(AEp); free(x);
    return t2 - t1;
}

/* ------------------------------------------------------------------------ */
/* octree regularisation  (src/inversion/regularization_octree.cpp)         */
/* ------------------------------------------------------------------------ */

typedef struct { int row, col, ord; double val; } rcoo_t;

static int rcoo_cmp(const void* a, const void* b) {
    const rcoo_t* x = (const rcoo_t*)a; const rcoo_t* y = (const rcoo_t*)b;
    if (x->row != y->row) return x->row < y->row ? -1 : 1;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    return x->ord < y->ord ? -1 : (x->ord > y->ord ? 1 : 0);
}

struct m3d_oracle_reg {
    int nc, na;
    int *a2g, *g2a;
    int *ptr, *idx;  double* val;           /* W^T W, columns sorted */
    int *aptr, *aidx; double* aw;           /* neighbours per active cell, face order */
    double* diagw;
    double alpha_s;
    int n_smooth;
};

/* RegularizationOctree::setup  regularization_octree.cpp:24-172 */
m3d_oracle_reg* m3d_oracle_reg_create(const m3d_oracle* S, double alpha_s, double alpha_x, double alpha_y,
                                      double alpha_z, int n_smooth) {
    const mesh_t* m = &S->m;
    const grid_t* G = &S->G;
    const int nc = S->nc;
    m3d_oracle_reg* R = (m3d_oracle_reg*)xcalloc(1, sizeof(m3d_oracle_reg));
    R->nc = nc; R->alpha_s = alpha_s; R->n_smooth = n_smooth;
    R->g2a = (int*)xcalloc((size_t)nc + 1, sizeof(int));
    R->a2g = (int*)xcalloc((size_t)nc + 1, sizeof(int));
    for (int c = 0; c < nc; ++c) {
        R->g2a[c] = -1;
        if (m->type[c] == 0) { R->g2a[c] = R->na; R->a2g[R->na++] = c; }
    }
    const int na = R->na;
    double* vol = (double*)xcalloc((size_t)nc + 1, sizeof(double));
    for (int c = 0; c < nc; ++c) { double dx, dy, dz; cell_size_xyz(m, c, &dx, &dy, &dz); vol[c] = dx * dy * dz; }
    rcoo_t* q = (rcoo_t*)xcalloc((size_t)4 * G->nf + 1, sizeof(rcoo_t));
    int nq = 0;
    /* neighbour lists: two passes (count, fill) keep the face order */
    int* acount = (int*)xcalloc((size_t)na + 1, sizeof(int));
    int* fa = (int*)xcalloc((size_t)G->nf + 1, sizeof(int));
    int* fb = (int*)xcalloc((size_t)G->nf + 1, sizeof(int));
    double* fw = (double*)xcalloc((size_t)G->nf + 1, sizeof(double));
    int nface = 0;
    R->diagw = (double*)xcalloc((size_t)na + 1, sizeof(double));
    for (int f = 0; f < G->nf; ++f) {
        int cm = G->fcm[f], cp = G->fcp[f];
        if (cm < 0 || cp < 0 || cm >= nc || cp >= nc) continue;
        int am = R->g2a[cm], ap = R->g2a[cp];
        if (am < 0 || ap < 0) continue;
        double al = G->fnorm[f] == 0 ? alpha_x : G->fnorm[f] == 1 ? alpha_y : G->fnorm[f] == 2 ? alpha_z : 1.0;
        double ddx = m->cx[cm] - m->cx[cp], ddy = m->cy[cm] - m->cy[cp], ddz = m->cz[cm] - m->cz[cp];
        double dist = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
        if (dist < 1e-10) continue;
        double vgm = pow(vol[cm] * vol[cp], 1.0 / 6.0);
        double w = al * G->farea[f] / (dist * vgm);
        q[nq].row = am; q[nq].col = am; q[nq].val = w; q[nq].ord = nq; nq++;
        q[nq].row = am; q[nq].col = ap; q[nq].val = -w; q[nq].ord = nq; nq++;
        q[nq].row = ap; q[nq].col = ap; q[nq].val = w; q[nq].ord = nq; nq++;
        q[nq].row = ap; q[nq].col = am; q[nq].val = -w; q[nq].ord = nq; nq++;
        fa[nface] = am; fb[nface] = ap; fw[nface] = w; nface++;
        acount[am]++; acount[ap]++;
        R->diagw[am] += w; R->diagw[ap] += w;
    }
    qsort(q, (size_t)nq, sizeof(rcoo_t), rcoo_cmp);
    R->ptr = (int*)xcalloc((size_t)na + 1, sizeof(int));
    R->idx = (int*)xcalloc((size_t)nq + 1, sizeof(int));
    R->val = (double*)xcalloc((size_t)nq + 1, sizeof(double));
    int u = 0;
    for (int t = 0; t < nq;) {
        int r = q[t].row, c = q[t].col;
        double s = 0.0;
        while (t < nq && q[t].row == r && q[t].col == c) {
            if (q[t].val < 0) s -= -q[t].val; else s += q[t].val;
            ++t;
        }
        R->idx[u] = c; R->val[u] = s; R->ptr[r + 1]++; u++;
    }
    for (int i = 0; i < na; ++i) R->ptr[i + 1] += R->ptr[i];
    R->aptr = (int*)xcalloc((size_t)na + 1, sizeof(int));
    for (int i = 0; i < na; ++i) R->aptr[i + 1] = R->aptr[i] + acount[i];
    R->aidx = (int*)xcalloc((size_t)R->aptr[na] + 1, sizeof(int));
    R->aw = (double*)xcalloc((size_t)R->aptr[na] + 1, sizeof(double));
    int* fill = (int*)xcalloc((size_t)na + 1, sizeof(int));
    for (int t = 0; t < nface; ++t) {
        int a = fa[t], b = fb[t];
        R->aidx[R->aptr[a] + fill[a]] = b; R->aw[R->aptr[a] + fill[a]] = fw[t]; fill[a]++;
        R->aidx[R->aptr[b] + fill[b]] = a; R->aw[R->aptr[b] + fill[b]] = fw[t]; fill[b]++;
    }
    /* normalisation to a unit average diagonal (:146-160) */
    double dsum = 0.0;
    for (int i = 0; i < na; ++i) dsum += R->diagw[i];
    double davg = na > 0 ? dsum / na : 1.0;
    if (davg > 1e-30) {
        double sc = 1.0 / davg;
        for (int k = 0; k < u; ++k) R->val[k] *= sc;
        for (int i = 0; i < na; ++i) R->diagw[i] *= sc;
        for (int k = 0; k < R->aptr[na]; ++k) R->aw[k] *= sc;
    }
    free(vol); free(q); free(acount); free(fa); free(fb); free(fw); free(fill);
    return R;
}

void m3d_oracle_reg_destroy(m3d_oracle_reg* R) {
    if (!R) return;
    free(R->a2g); free(R->g2a); free(R->ptr); free(R->idx); free(R->val);
    free(R->aptr); free(R->aidx); free(R->aw); free(R->diagw); free(R);
}

int m3d_oracle_reg_num_active(const m3d_oracle_reg* R) { return R->na; }

void m3d_oracle_reg_active_to_global(const m3d_oracle_reg* R, int* a2g) {
    for (int j = 0; j < R->na; ++j) a2g[j] = R->a2g[j];
}

/* apply_WtW (:229-231), CSRMatrix::matvec (include/maple3dmt/common.h:52-61) */
void m3d_oracle_reg_apply_wtw(const m3d_oracle_reg* R, const double* x, double* y) {
    for (int i = 0; i < R->na; ++i) {
        double s = 0.0;
        for (int k = R->ptr[i]; k < R->ptr[i + 1]; ++k) s += R->val[k] * x[R->idx[k]];
        y[i] = s;
    }
}

/* diagonal_WtW (:236-246) */
void m3d_oracle_reg_diagonal(const m3d_oracle_reg* R, double* d) {
    for (int i = 0; i < R->na; ++i) {
        d[i] = 0.0;
        for (int k = R->ptr[i]; k < R->ptr[i + 1]; ++k)
            if (R->idx[k] == i) { d[i] = R->val[k]; break; }
    }
}

/* apply_CmCmT (:251-281): 2 n_smooth diffusion passes */
void m3d_oracle_reg_apply_cmcmt(const m3d_oracle_reg* R, const double* x, double* y) {
    const int na = R->na;
    double* cur = (double*)xcalloc((size_t)na + 1, sizeof(double));
    double* tmp = (double*)xcalloc((size_t)na + 1, sizeof(double));
    memcpy(cur, x, sizeof(double) * (size_t)na);
    for (int pass = 0; pass < 2 * R->n_smooth; ++pass) {
        for (int i = 0; i < na; ++i) {
            double sum = cur[i], wt = 1.0;
            double dg = R->diagw[i] > 0 ? R->diagw[i] : 1.0;
            for (int k = R->aptr[i]; k < R->aptr[i + 1]; ++k) {
                double wn = R->aw[k] / dg;
                sum += wn * cur[R->aidx[k]];
                wt += wn;
            }
            tmp[i] = sum / wt;
        }
        memcpy(cur, tmp, sizeof(double) * (size_t)na);
    }
    memcpy(y, cur, sizeof(double) * (size_t)na);
    free(cur); free(tmp);
}

/* evaluate (:183-201) and gradient (:206-224); params = ln(sigma) per cell,
 * ref per active cell (NULL: zero) */
double m3d_oracle_reg_evaluate(const m3d_oracle_reg* R, const double* params, const double* ref, double* grad) {
    const int na = R->na;
    double* dm = (double*)xcalloc((size_t)na + 1, sizeof(double));
    double* wd = (double*)xcalloc((size_t)na + 1, sizeof(double));
    for (int j = 0; j < na; ++j) dm[j] = params[R->a2g[j]] - (ref ? ref[j] : 0.0);
    m3d_oracle_reg_apply_wtw(R, dm, wd);
    double v = 0.0;
    for (int j = 0; j < na; ++j) v += dm[j] * wd[j];
    if (grad) {
        for (int c = 0; c < R->nc; ++c) grad[c] = 0.0;
        for (int j = 0; j < na; ++j) grad[R->a2g[j]] = 2.0 * R->alpha_s * wd[j];
    }
    free(dm); free(wd);
    return R->alpha_s * v;
}
