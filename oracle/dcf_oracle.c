/*
 * CPU restatement of disccofan's component-forest hot path -- TEST ORACLE.
 *
 * Test infrastructure only (see dcf_oracle.h).  Written from the reference's
 * behaviour, not copied: every block names the reference file:line it restates.
 * It reproduces the reference's sequential results bit-exactly (checked against
 * the compiled reference and its golden fixtures in tests/test_oracle.py), and its
 * multi-slab build + seam merge so that the CPU baseline uses all host threads the
 * way the reference's OpenMP path does.
 *
 * Compiled with -ffp-contract=off semantics in mind: every floating expression
 * below is written in the reference's operand order and types (float vs double),
 * because attribute readouts, subtractive filtering and spectra depend on it.
 */
#define _GNU_SOURCE
#include "dcf_oracle.h"
#include "dcf_eigen.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <omp.h>
#include <stdbool.h>
#include <stdlib.h>
#include <string.h>


#define BOTTOM (-1)
#define NUMATTR_EXT 19 /* 18 reference attributes + bbox elongation */

typedef int64_t idx_t;

/* aux-data layouts, byte-compatible with types.h:251-286 */
typedef struct { uint64_t area; } area_rec;
typedef struct { uint64_t area, minX, minY, minZ, maxX, maxY, maxZ; } extent_rec;
typedef struct { uint64_t area, sumX, sumY, sumZ; } mean_rec;
typedef struct { uint64_t area; double sumGval, sumXd, sumYd, sumZd; } wmean_rec;
typedef struct {
    uint64_t area;
    double sumval, sumval2;
    double sumX, sumY, sumZ, sumX2, sumY2, sumZ2, sumXY, sumYZ, sumXZ;
    double sumXd, sumYd, sumZd;
} inertia_rec;

static const size_t GROUP_SIZE[5] = {sizeof(area_rec), sizeof(extent_rec), sizeof(mean_rec),
                                     sizeof(wmean_rec), sizeof(inertia_rec)};
/* attribute -> group, attributes.c:1224-1248 (18 = bbox elongation, group 1) */
static const int ATTR_GROUP[NUMATTR_EXT] = {0, 1, 1, 1, 1, 1, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 4, 1};

struct dco_tree {
    uint64_t dims[3];
    uint64_t n;
    int conn;
    int tree_min;
    int threads;
    float pixdim[3];
    float gmax, gmin;
    float *gval;
    idx_t *parent;
    char *attr;     /* n records of GROUP_SIZE[group] bytes */
    int group;      /* -1 before the first build */
    int prev_attr;
    uint64_t max_levels;
};

/* ------------------------------------------------------------------ */
/* aux-data operations per group (attributes.c:47-880)                 */
/* ------------------------------------------------------------------ */

/* init_*_data: init flag, coordinates, grey value (attributes.c:54,122,283,377,485) */
static void aux_init(int g, void *r, bool init, uint64_t x, uint64_t y, uint64_t z, float gv)
{
    switch (g) {
    case 0: ((area_rec *)r)->area = (uint64_t)init; break;
    case 1: {
        extent_rec *e = r;
        e->area = (uint64_t)init;
        if (init) {
            e->minX = x; e->maxX = x + 1;
            e->minY = y; e->maxY = y + 1;
            e->minZ = z; e->maxZ = z + 1;
        } else {
            e->minX = e->minY = e->minZ = ULONG_MAX;
            e->maxX = e->maxY = e->maxZ = 0;
        }
        break;
    }
    case 2: {
        mean_rec *m = r;
        m->area = (uint64_t)init;
        m->sumX = init ? x : 0;
        m->sumY = init ? y : 0;
        m->sumZ = init ? z : 0;
        break;
    }
    case 3: {
        wmean_rec *m = r;
        m->area = (uint64_t)init;
        m->sumGval = (double)init * (double)gv;
        m->sumXd = init ? (double)gv * (double)x : 0.;
        m->sumYd = init ? (double)gv * (double)y : 0.;
        m->sumZd = init ? (double)gv * (double)z : 0.;
        break;
    }
    default: {
        inertia_rec *m = r;
        m->area = (uint64_t)init;
        m->sumX = init ? (double)x : 0.;
        m->sumY = init ? (double)y : 0.;
        m->sumZ = init ? (double)z : 0.;
        m->sumX2 = init ? (double)x * x : 0.;
        m->sumY2 = init ? (double)y * y : 0.;
        m->sumZ2 = init ? (double)z * z : 0.;
        m->sumXY = init ? (double)x * y : 0.;
        m->sumYZ = init ? (double)y * z : 0.;
        m->sumXZ = init ? (double)z * x : 0.;
        m->sumval = init ? (double)gv : 0;
        m->sumval2 = init ? (double)gv * gv : 0;
        m->sumXd = init ? (double)gv * x : 0.;
        m->sumYd = init ? (double)gv * y : 0.;
        m->sumZd = init ? (double)gv * z : 0.;
        break;
    }
    }
}

/* merge_*_data: dst += src (attributes.c:70,158,305,403,534) */
static void aux_merge(int g, void *dst, const void *src)
{
    switch (g) {
    case 0: ((area_rec *)dst)->area += ((const area_rec *)src)->area; break;
    case 1: {
        extent_rec *a = dst;
        const extent_rec *b = src;
        a->area += b->area;
        a->minX = a->minX <= b->minX ? a->minX : b->minX;
        a->minY = a->minY <= b->minY ? a->minY : b->minY;
        a->minZ = a->minZ <= b->minZ ? a->minZ : b->minZ;
        a->maxX = a->maxX >= b->maxX ? a->maxX : b->maxX;
        a->maxY = a->maxY >= b->maxY ? a->maxY : b->maxY;
        a->maxZ = a->maxZ >= b->maxZ ? a->maxZ : b->maxZ;
        break;
    }
    case 2: {
        mean_rec *a = dst;
        const mean_rec *b = src;
        a->area += b->area; a->sumX += b->sumX; a->sumY += b->sumY; a->sumZ += b->sumZ;
        break;
    }
    case 3: {
        wmean_rec *a = dst;
        const wmean_rec *b = src;
        a->area += b->area; a->sumGval += b->sumGval;
        a->sumXd += b->sumXd; a->sumYd += b->sumYd; a->sumZd += b->sumZd;
        break;
    }
    default: {
        inertia_rec *a = dst;
        const inertia_rec *b = src;
        a->area += b->area;
        a->sumX += b->sumX; a->sumY += b->sumY; a->sumZ += b->sumZ;
        a->sumX2 += b->sumX2; a->sumY2 += b->sumY2; a->sumZ2 += b->sumZ2;
        a->sumXY += b->sumXY; a->sumYZ += b->sumYZ; a->sumXZ += b->sumXZ;
        a->sumval += b->sumval; a->sumval2 += b->sumval2;
        a->sumXd += b->sumXd; a->sumYd += b->sumYd; a->sumZd += b->sumZd;
        break;
    }
    }
}

/* merge_to_*_data: dst = a + b, evaluated as a then b (attributes.c:76,176,315,413,558) */
static void aux_merge_to(int g, void *dst, const void *a, const void *b)
{
    char tmp[sizeof(inertia_rec)];
    memcpy(tmp, a, GROUP_SIZE[g]);
    aux_merge(g, tmp, b);
    memcpy(dst, tmp, GROUP_SIZE[g]);
}

/* ------------------------------------------------------------------ */
/* attribute readouts (attributes.c:102-880)                           */
/* ------------------------------------------------------------------ */

static double attr_area(const dco_tree *t, int g, const void *r)
{
    const float *pd = t->pixdim;
    switch (g) {
    case 0: /* area_attribute: float product times (float) area (attributes.c:105) */
        return (double)(pd[0] * pd[1] * pd[2] * (float)((const area_rec *)r)->area);
    case 1: /* extent_area_attribute (attributes.c:213) */
        return (double)((const extent_rec *)r)->area;
    case 2: /* mean_area_attribute (attributes.c:348) */
        return (double)(pd[0] * pd[1] * pd[2]) * (double)((const mean_rec *)r)->area;
    case 3: /* wmean_area_attribute (attributes.c:465) */
        return (double)((const wmean_rec *)r)->area;
    default: /* inertia_area_attribute (attributes.c:700) */
        return (double)pd[0] * pd[1] * pd[2] * (double)((const inertia_rec *)r)->area;
    }
}

/* inertia_arr (attributes.c:628-648) */
static void inertia_arr(const dco_tree *t, const inertia_rec *m, double in[15])
{
    const float *pd = t->pixdim;
    in[0] = (double)pd[0] * pd[1] * pd[2] * (double)m->area;
    in[1] = pd[0] * m->sumX;
    in[2] = pd[1] * m->sumY;
    in[3] = pd[2] * m->sumZ;
    in[4] = (double)(pd[0] * pd[0]) * m->sumX2;
    in[5] = (double)(pd[1] * pd[1]) * m->sumY2;
    in[6] = (double)(pd[2] * pd[2]) * m->sumZ2;
    in[7] = (double)(pd[0] * pd[1]) * m->sumXY;
    in[8] = (double)(pd[1] * pd[2]) * m->sumYZ;
    in[9] = (double)(pd[0] * pd[2]) * m->sumXZ;
    in[10] = m->sumval;
    in[11] = m->sumval2;
    in[12] = pd[0] * m->sumXd;
    in[13] = pd[1] * m->sumYd;
    in[14] = pd[2] * m->sumZd;
}

/* central moment matrix with the voxel correction (attributes.c:708-719 and copies) */
static void inertia_matrix(const dco_tree *t, const double in[15], double mat[6])
{
    const float *pd = t->pixdim;
    double corr = in[0] / 12;
    mat[0] = in[4] - in[1] * in[1] / in[0] + pd[0] * corr;
    mat[1] = in[5] - in[2] * in[2] / in[0] + pd[1] * corr;
    mat[2] = in[6] - in[3] * in[3] / in[0] + pd[2] * corr;
    mat[3] = in[7] - in[1] * in[2] / in[0];
    mat[4] = in[8] - in[2] * in[3] / in[0];
    mat[5] = in[9] - in[1] * in[3] / in[0];
}

/* Eigenvalues come from the project's restatement of EISPACK tred2 + tql2
 * (disccofan_gb300/csrc/dcf_eigen.h), the arithmetic the reference's rs uses. */
void dco_sym_eig2(const double m[4], double ev[2]) { dcf_sym_eigenvalues(2, m, ev); }
void dco_sym_eig3(const double m[9], double ev[3]) { dcf_sym_eigenvalues(3, m, ev); }

static double attr_value(const dco_tree *t, int attr, const void *r)
{
    const float *pd = t->pixdim;
    switch (attr) {
    case 0: return attr_area(t, 0, r);
    case 1: { /* extent_rectarea_attribute (attributes.c:218) */
        const extent_rec *e = r;
        double v = (double)(e->maxX - e->minX) * (double)(e->maxY - e->minY) * (double)(e->maxZ - e->minZ);
        v *= pd[0] * pd[1] * pd[2];
        return v;
    }
    case 2: { /* extent_rectdiag_attribute (attributes.c:234) */
        const extent_rec *e = r;
        double minx = pd[0] * (double)e->minX, miny = pd[1] * (double)e->minY, minz = pd[2] * (double)e->minZ;
        double maxx = pd[0] * (double)e->maxX, maxy = pd[1] * (double)e->maxY, maxz = pd[2] * (double)e->maxZ;
        return (maxx - minx) * (maxx - minx) + (maxy - miny) * (maxy - miny) + (maxz - minz) * (maxz - minz);
    }
    case 3: return pd[0] * (double)(((const extent_rec *)r)->maxX - ((const extent_rec *)r)->minX);
    case 4: return pd[1] * (double)(((const extent_rec *)r)->maxY - ((const extent_rec *)r)->minY);
    case 5: return pd[2] * (double)(((const extent_rec *)r)->maxZ - ((const extent_rec *)r)->minZ);
    case 6: return pd[0] * (double)((const mean_rec *)r)->sumX / (double)((const mean_rec *)r)->area;
    case 7: return pd[1] * (double)((const mean_rec *)r)->sumY / (double)((const mean_rec *)r)->area;
    case 8: return pd[2] * (double)((const mean_rec *)r)->sumZ / (double)((const mean_rec *)r)->area;
    case 9: return (double)pd[0] * ((const wmean_rec *)r)->sumXd / (double)((const wmean_rec *)r)->sumGval;
    case 10: return (double)pd[1] * ((const wmean_rec *)r)->sumYd / (double)((const wmean_rec *)r)->sumGval;
    case 11: return (double)pd[2] * ((const wmean_rec *)r)->sumZd / (double)((const wmean_rec *)r)->sumGval;
    case 12: return (double)((const wmean_rec *)r)->sumGval;
    case 18: { /* bbox elongation (not a reference attribute) */
        double xe = attr_value(t, 3, r), ye = attr_value(t, 4, r);
        double hi = xe > ye ? xe : ye, lo = xe < ye ? xe : ye;
        return hi / (lo > 1.0 ? lo : 1.0);
    }
    default: break;
    }
    /* group 4: inertia_*_attribute (attributes.c:706-874); 2-D branch when sumZ == 0 */
    double in[15], mat[6];
    inertia_arr(t, r, in);
    inertia_matrix(t, in, mat);
    bool flat2d = in[3] == 0;
    switch (attr) {
    case 13:
        return flat2d ? (mat[0] + mat[1]) : (mat[0] + mat[1] + mat[2]);
    case 14: case 15: case 16: {
        if (flat2d) {
            if (attr == 15) return -1;
            double m2[4] = {mat[0], mat[3], mat[3], mat[1]}, ev[2];
            dco_sym_eig2(m2, ev);
            if (attr == 14) return ev[1] / ev[0];
            double ax0 = sqrt(4 * ev[1] / in[0]), ax1 = sqrt(4 * ev[0] / in[0]);
            return M_PI * ax0 * ax1 / (in[0]);
        }
        double m3[9] = {mat[0], mat[3], mat[5], mat[3], mat[1], mat[4], mat[5], mat[4], mat[2]}, ev[3];
        dco_sym_eig3(m3, ev);
        if (attr == 14) return ev[2] / ev[1];
        if (attr == 15) return ev[1] / ev[0];
        double ax0 = sqrt(20 * ev[2] / in[0]), ax1 = sqrt(20 * ev[1] / in[0]), ax2 = sqrt(20 * ev[0] / in[0]);
        return M_PI * ax0 * ax1 * ax2 / (6 * in[0]);
    }
    case 17:
        if (flat2d) return (mat[0] + mat[1]) / pow(in[0], 2.0);
        return (mat[0] + mat[1] + mat[2]) / pow(in[0], 5.0 / 3.0);
    default:
        return NAN;
    }
}

/* ------------------------------------------------------------------ */
/* rank mapping: stable LSD radix sort of order-preserving keys        */
/* (transform_float flood.c:362-371, create_mappings flood.c:378-502)  */
/* ------------------------------------------------------------------ */

static inline uint32_t float_key(float v)
{
    uint32_t u;
    memcpy(&u, &v, 4);
    return (u & 0x80000000u) ? 0xFFFFFFFFu - u : (u | 0x80000000u);
}

/* ranks_inv[r] = offset (from lwb) of the pixel with rank r in [lwb, upb) */
static uint64_t *rank_map(const float *g, uint64_t lwb, uint64_t upb)
{
    uint64_t len = upb - lwb;
    uint64_t *hist = calloc(4 * 256, sizeof(uint64_t));
    uint32_t *k0 = malloc(len * sizeof(uint32_t)), *k1 = malloc(len * sizeof(uint32_t));
    uint64_t *i0 = malloc(len * sizeof(uint64_t)), *i1 = malloc(len * sizeof(uint64_t));
    for (uint64_t i = 0; i < len; i++) {
        uint32_t k = float_key(g[lwb + i]);
        k0[i] = k;
        i0[i] = i;
        for (int d = 0; d < 4; d++) hist[d * 256 + ((k >> (8 * d)) & 255)]++;
    }
    for (int d = 0; d < 4; d++) {
        uint64_t s = 0;
        for (int b = 0; b < 256; b++) {
            uint64_t c = hist[d * 256 + b];
            hist[d * 256 + b] = s;
            s += c;
        }
    }
    for (int d = 0; d < 4; d++) {
        uint64_t *h = hist + d * 256;
        for (uint64_t i = 0; i < len; i++) {
            uint64_t pos = h[(k0[i] >> (8 * d)) & 255]++;
            k1[pos] = k0[i];
            i1[pos] = i0[i];
        }
        uint32_t *tk = k0; k0 = k1; k1 = tk;
        uint64_t *ti = i0; i0 = i1; i1 = ti;
    }
    free(hist); free(k0); free(k1); free(i1);
    return i0;
}

/* ------------------------------------------------------------------ */
/* 64-ary hierarchical bit-set max-queue over ranks (queue.c:117-167)  */
/* ------------------------------------------------------------------ */

typedef struct {
    int nlev;            /* level nlev-1 is the finest */
    uint64_t *words[8];
    uint64_t top;
} rank_queue;

static void rq_init(rank_queue *q, uint64_t max_rank)
{
    int bits = 64 - __builtin_clzll(max_rank | 1);
    q->nlev = (bits + 5) / 6;
    uint64_t m = max_rank;
    for (int i = q->nlev; i--;) {
        m >>= 6;
        q->words[i] = calloc(m + 1, sizeof(uint64_t));
    }
    q->top = 0;
}

static void rq_free(rank_queue *q)
{
    for (int i = 0; i < q->nlev; i++) free(q->words[i]);
}

static inline bool rq_empty(const rank_queue *q) { return q->words[0][0] == 0; }

static inline void rq_push(rank_queue *q, uint64_t r)
{
    if (r > q->top) q->top = r;
    for (int i = q->nlev; i--;) {
        q->words[i][r >> 6] |= 1ull << (r & 63);
        r >>= 6;
    }
}

static inline void rq_pop(rank_queue *q)
{
    uint64_t r = q->top;
    for (int i = q->nlev; i--;) {
        uint64_t w = r >> 6;
        q->words[i][w] &= ~(1ull << (r & 63));
        if (q->words[i][w]) {
            for (int j = i; j != q->nlev; j++) w = (w << 6) ^ (uint64_t)(63 - __builtin_clzll(q->words[j][w]));
            q->top = w;
            return;
        }
        r = w;
    }
}

/* ------------------------------------------------------------------ */
/* flooding (tree_flood flood.c:222-247, remaining :659-690,           */
/* check_neighbor :556-582)                                            */
/* ------------------------------------------------------------------ */

typedef struct {
    uint64_t *visited;  /* bit set over [lwb, upb) */
    rank_queue q;
    const uint64_t *ranks; /* rank of (pixel - lwb) */
    uint64_t lwb, upb;
} flood_ws;

static inline bool try_neighbor(flood_ws *ws, uint64_t *index, uint64_t *rank, uint64_t n)
{
    uint64_t o = n - ws->lwb;
    if (ws->visited[o >> 6] >> (o & 63) & 1) return false;
    ws->visited[o >> 6] |= 1ull << (o & 63);
    uint64_t rn = ws->ranks[o];
    if (*rank > rn) {
        rq_push(&ws->q, rn);
        return false;
    }
    rq_push(&ws->q, *rank);
    *index = n;
    *rank = rn;
    return true;
}

/* climb to unvisited higher-ranked neighbours, queueing the rest; the neighbour
 * order (direct, in-plane diagonals, 3-D diagonals) follows remaining(). */
static void climb(flood_ws *ws, const uint64_t *dims, int conn, uint64_t *index, uint64_t *rank)
{
    const uint64_t W = dims[0], H = dims[1], D = dims[2], WH = W * H;
    const uint64_t lwb = ws->lwb, upb = ws->upb;
    bool moved = true;
    while (moved) {
        uint64_t p = *index;
        uint64_t z = p / WH, r = p % WH, y = r / W, x = r % W;
        moved =
            (x > 0 && p - 1 >= lwb && try_neighbor(ws, index, rank, p - 1)) ||
            (x < W - 1 && p + 1 < upb && try_neighbor(ws, index, rank, p + 1)) ||
            (y > 0 && p - W >= lwb && try_neighbor(ws, index, rank, p - W)) ||
            (y < H - 1 && p + W < upb && try_neighbor(ws, index, rank, p + W)) ||
            (z > 0 && p >= lwb + WH && try_neighbor(ws, index, rank, p - WH)) ||
            (z < D - 1 && p + WH < upb && try_neighbor(ws, index, rank, p + WH));
        if (!moved && conn >= 8) {
            moved =
                (x > 0 && y > 0 && p - 1 - W >= lwb && try_neighbor(ws, index, rank, p - 1 - W)) ||
                (x < W - 1 && y > 0 && p + 1 - W >= lwb && try_neighbor(ws, index, rank, p + 1 - W)) ||
                (x > 0 && y < H - 1 && p - 1 + W < upb && try_neighbor(ws, index, rank, p - 1 + W)) ||
                (y < H - 1 && x < W - 1 && p + W + 1 < upb && try_neighbor(ws, index, rank, p + W + 1));
        }
        if (!moved && conn == 26) {
            static const int dxy[8][2] = {{-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
            for (int dz = -1; dz <= 1 && !moved; dz += 2) {
                if ((dz < 0 && z == 0) || (dz > 0 && z == D - 1)) continue;
                for (int k = 0; k < 8 && !moved; k++) {
                    int dx = dxy[k][0], dy = dxy[k][1];
                    if ((dx < 0 && x == 0) || (dx > 0 && x == W - 1)) continue;
                    if ((dy < 0 && y == 0) || (dy > 0 && y == H - 1)) continue;
                    int64_t off = (int64_t)dx + (int64_t)dy * (int64_t)W + (int64_t)dz * (int64_t)WH;
                    uint64_t nb = (uint64_t)((int64_t)p + off);
                    if (off < 0 ? nb >= lwb : nb < upb) moved = try_neighbor(ws, index, rank, nb);
                }
            }
        }
    }
}

static void ws_init(flood_ws *ws, uint64_t lwb, uint64_t upb, const uint64_t *ranks)
{
    uint64_t len = upb - lwb;
    ws->visited = calloc(len / 64 + 1, sizeof(uint64_t));
    rq_init(&ws->q, len ? len - 1 : 0);
    ws->ranks = ranks;
    ws->lwb = lwb;
    ws->upb = upb;
}

static void ws_free(flood_ws *ws)
{
    free(ws->visited);
    rq_free(&ws->q);
}

/* get_levelroot / get_parent with path compression (flood.c:693-722) */
static idx_t levelroot(dco_tree *t, idx_t x)
{
    if (x == BOTTOM) return BOTTOM;
    idx_t r = x;
    float gv = t->gval[x];
    while (t->parent[r] != BOTTOM && gv == t->gval[t->parent[r]]) r = t->parent[r];
    while (x != r) {
        idx_t y = t->parent[x];
        t->parent[x] = r;
        x = y;
    }
    return r;
}

static inline idx_t get_parent(dco_tree *t, idx_t x) { return levelroot(t, t->parent[x]); }

static inline bool is_levelroot(const dco_tree *t, idx_t x)
{
    return t->parent[x] == BOTTOM || t->gval[x] != t->gval[t->parent[x]];
}

static inline void *ATTR(const dco_tree *t, idx_t i) { return t->attr + (size_t)i * GROUP_SIZE[t->group]; }

/* merge_nodes (flood.c:292-353): Wilkinson's merge of two branches with
 * attribute carries; cor/copa are the carried records. */
static void merge_nodes(dco_tree *t, idx_t x, idx_t y)
{
    const int g = t->group;
    const size_t sz = GROUP_SIZE[g];
    char cor[sizeof(inertia_rec)], copa[sizeof(inertia_rec)];
    bool have_cor = false;
    if (t->gval[y] > t->gval[x]) { idx_t h = x; x = y; y = h; }
    x = levelroot(t, x);
    y = levelroot(t, y);
    while (x != y && y != BOTTOM) {
        idx_t z = get_parent(t, x);
        if (z != BOTTOM && t->gval[z] >= t->gval[y]) {
            if (have_cor) aux_merge(g, ATTR(t, x), cor);
            x = z;
        } else {
            if (have_cor) aux_merge_to(g, copa, ATTR(t, x), cor);
            else memcpy(copa, ATTR(t, x), sz);
            memcpy(cor, ATTR(t, x), sz);
            have_cor = true;
            memcpy(ATTR(t, x), copa, sz);
            t->parent[x] = y;
            x = y;
            y = z;
        }
    }
    if (y == BOTTOM && have_cor) {
        while (x != BOTTOM) {
            aux_merge(g, ATTR(t, x), cor);
            x = get_parent(t, x);
        }
    }
}

/* init_attrib_array (attributes.c:1201-1221) for one rank: no borders, zero offsets */
static void init_attrs(dco_tree *t, uint64_t lwb, uint64_t upb)
{
    const uint64_t W = t->dims[0], WH = t->dims[0] * t->dims[1];
    for (uint64_t i = lwb; i < upb; i++) {
        uint64_t x = (i % WH) % W, y = (i % WH) / W, z = i / WH;
        aux_init(t->group, ATTR(t, i), true, x, y, z, t->gval[i]);
    }
}

static uint64_t slab_bound(const dco_tree *t, int id, int nt)
{
    const uint64_t *d = t->dims;
    return d[2] == 1 ? d[0] * ((id * d[1]) / nt) : d[0] * d[1] * ((id * d[2]) / nt);
}

/* fuse_sections (flood.c:253-290): re-flood the strip across a slab seam and
 * merge every (index, parent) step into the tree */
static void fuse_seam(dco_tree *t, uint64_t mdb)
{
    uint64_t inc = t->dims[2] == 1 ? t->dims[0] : t->dims[0] * t->dims[1];
    uint64_t lwb = mdb - inc, upb = mdb + inc;
    uint64_t *rinv = rank_map(t->gval, lwb, upb);
    uint64_t *ranks = malloc(2 * inc * sizeof(uint64_t));
    for (uint64_t i = 0; i < 2 * inc; i++) ranks[rinv[i]] = i;
    flood_ws ws = {0};
    ws_init(&ws, lwb, upb, ranks);
    uint64_t index = lwb, rank = ranks[0];
    ws.visited[0] |= 1;
    for (;;) {
        climb(&ws, t->dims, t->conn, &index, &rank);
        if (rq_empty(&ws.q)) break;
        rank = ws.q.top;
        uint64_t par = rinv[rank] + lwb;
        rq_pop(&ws.q);
        merge_nodes(t, (idx_t)index, (idx_t)par);
        index = par;
    }
    ws_free(&ws);
    free(ranks);
    free(rinv);
}

/* build_local_tree_generic (flood.c:58-172) */
static void build_tree(dco_tree *t)
{
    const int nt = t->threads;
    t->parent = malloc(t->n * sizeof(idx_t));
    t->attr = malloc(t->n * GROUP_SIZE[t->group]);
#pragma omp parallel num_threads(nt)
    {
        int id = omp_get_thread_num();
        uint64_t lwb = slab_bound(t, id, nt), upb = slab_bound(t, id + 1, nt);
        if (upb > lwb) {
            uint64_t *rinv = rank_map(t->gval, lwb, upb);
            uint64_t *ranks = (uint64_t *)(t->parent + lwb); /* parent doubles as ranks (flood.c:93-94) */
            for (uint64_t i = 0; i != upb - lwb; ++i) ranks[rinv[i]] = i;
            init_attrs(t, lwb, upb);
            /* tree_flood */
            flood_ws ws = {0};
            ws_init(&ws, lwb, upb, ranks);
            uint64_t index = lwb, rank = ranks[0];
            ws.visited[0] |= 1;
            for (;;) {
                climb(&ws, t->dims, t->conn, &index, &rank);
                if (rq_empty(&ws.q)) break;
                rank = ws.q.top;
                uint64_t par = rinv[rank] + lwb;
                rq_pop(&ws.q);
                aux_merge(t->group, ATTR(t, par), ATTR(t, index));
                t->parent[index] = (idx_t)par;
                index = par;
            }
            t->parent[index] = BOTTOM;
            ws_free(&ws);
            free(rinv);
            /* compression to level roots (flood.c:127-141) */
            for (uint64_t x = lwb; x < upb; x++) {
                idx_t r = (idx_t)x;
                float gv = t->gval[x];
                while (t->parent[r] != BOTTOM && gv == t->gval[t->parent[r]]) r = t->parent[r];
                idx_t i = (idx_t)x;
                while (i != r) {
                    idx_t y = t->parent[i];
                    t->parent[i] = r;
                    i = y;
                }
                t->parent[r] = levelroot(t, t->parent[r]);
            }
        }
    }
    /* binary-tree reduction over slab seams (flood.c:144-165), one round at a time */
    for (int i = 1; i < nt; i *= 2) {
#pragma omp parallel for num_threads(nt) schedule(static, 1)
        for (int id = 0; id < nt; id += 2 * i) {
            if (id + i < nt) {
                uint64_t mdb = slab_bound(t, id + i, nt);
                if (mdb > 0 && mdb < t->n) fuse_seam(t, mdb);
            }
        }
    }
}

/* flood_attributes (flood.c:184-219) */
static void reflood_attributes(dco_tree *t)
{
    uint64_t *rinv = rank_map(t->gval, 0, t->n);
    bool *visited = calloc(t->n, sizeof(bool));
    free(t->attr);
    t->attr = malloc(t->n * GROUP_SIZE[t->group]);
    init_attrs(t, 0, t->n);
    for (int64_t i = (int64_t)t->n - 1; i >= 0; i--) {
        idx_t p = (idx_t)rinv[i];
        visited[p] = true;
        idx_t par = get_parent(t, p);
        if (par == BOTTOM) continue;
        aux_merge(t->group, ATTR(t, par), ATTR(t, p));
        if (t->gval[p] == t->gval[par] && visited[par]) {
            par = get_parent(t, par);
            if (par != BOTTOM) aux_merge(t->group, ATTR(t, par), ATTR(t, p));
        }
    }
    free(visited);
    free(rinv);
}

/* ------------------------------------------------------------------ */
/* public: create / prepare                                            */
/* ------------------------------------------------------------------ */

static int cmpf(const void *a, const void *b)
{
    float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

dco_tree *dco_create(const float *img, uint64_t w, uint64_t h, uint64_t d, int conn, int tree_min,
                     int threads, float pd0, float pd1, float pd2)
{
    dco_tree *t = calloc(1, sizeof(dco_tree));
    t->dims[0] = w; t->dims[1] = h; t->dims[2] = d;
    t->n = w * h * d;
    /* io.c:64-79 */
    if (d > 1 && conn == 4) conn = 6;
    else if (conn == 8 && d > 1) conn = 26;
    else if (conn == 26 && d == 1) conn = 8;
    t->conn = conn;
    t->tree_min = tree_min;
    t->threads = threads > 0 ? threads : 1;
    t->pixdim[0] = pd0; t->pixdim[1] = pd1; t->pixdim[2] = pd2;
    t->gval = malloc(t->n * sizeof(float));
    memcpy(t->gval, img, t->n * sizeof(float));
    t->group = -1;
    t->prev_attr = -1;
    /* find_extremas (preprocessing.c:7-17) and min-tree inversion (:84-91) */
    float mn = t->gval[0], mx = t->gval[0];
    for (uint64_t i = 0; i < t->n; i++) {
        if (t->gval[i] < mn) mn = t->gval[i];
        if (t->gval[i] > mx) mx = t->gval[i];
    }
    t->gmax = mx;
    t->gmin = mn;
    if (tree_min)
        for (uint64_t i = 0; i < t->n; i++) t->gval[i] = mx - t->gval[i];
    float *tmp = malloc(t->n * sizeof(float));
    memcpy(tmp, t->gval, t->n * sizeof(float));
    qsort(tmp, t->n, sizeof(float), cmpf);
    uint64_t distinct = t->n ? 1 : 0;
    for (uint64_t i = 1; i < t->n; i++) distinct += tmp[i] != tmp[i - 1];
    free(tmp);
    t->max_levels = distinct + 2;
    return t;
}

void dco_destroy(dco_tree *t)
{
    if (!t) return;
    free(t->gval);
    free(t->parent);
    free(t->attr);
    free(t);
}

int dco_connectivity(const dco_tree *t) { return t->conn; }
float dco_max_gval(const dco_tree *t) { return t->gmax; }

int dco_prepare(dco_tree *t, int attr)
{
    if (attr < 0 || attr >= NUMATTR_EXT) return -1;
    int g = ATTR_GROUP[attr];
    if (t->prev_attr < 0) {
        t->group = g;
        build_tree(t);
    } else if (g != t->group) {
        t->group = g;
        reflood_attributes(t);
    }
    t->prev_attr = attr;
    return 0;
}

int dco_parent(const dco_tree *t, int64_t *out)
{
    if (!t->parent) return -1;
    memcpy(out, t->parent, t->n * sizeof(int64_t));
    return 0;
}

int dco_gval(const dco_tree *t, float *out)
{
    memcpy(out, t->gval, t->n * sizeof(float));
    return 0;
}

int dco_node_attr(const dco_tree *t, int attr, int area, double *out)
{
    if (!t->attr || attr < 0 || attr >= NUMATTR_EXT || ATTR_GROUP[attr] != t->group) return -1;
    for (uint64_t i = 0; i < t->n; i++)
        out[i] = is_levelroot(t, (idx_t)i)
                     ? (area ? attr_area(t, t->group, ATTR(t, i)) : attr_value(t, attr, ATTR(t, i)))
                     : NAN;
    return 0;
}

int64_t dco_aux(const dco_tree *t, void *out, uint64_t out_bytes)
{
    if (!t->attr) return -1;
    uint64_t bytes = t->n * GROUP_SIZE[t->group];
    if (out && out_bytes == bytes) memcpy(out, t->attr, bytes);
    return (int64_t)bytes;
}

/* ------------------------------------------------------------------ */
/* filtering (filtering.c:18-261)                                      */
/* ------------------------------------------------------------------ */

#define AV(t, a, i) attr_value((t), (a), ATTR((t), (i)))

/* The threads filter disjoint pixel ranges but stop at, and read, nodes that other
 * threads have already resolved.  The reference (filtering.c:55-261) shares out[]
 * and reached[] through plain loads and stores, and its min rule sets reached[]
 * before out[]; on Arm's weakly ordered memory a reader can then see reached[w]
 * set while out[w] still holds the zero it was cleared to, and copy that zero
 * down its path.  Here out[u] is published by a release store of reached[u] and
 * read only after an acquire load of it, which are plain loads and stores on x86
 * (the results there are the reference's).  reached[] is only ever raised, except
 * where the max rule lowers another range's entry as the reference does (:182). */
static inline bool seen(const bool *reached, idx_t i) { return __atomic_load_n(&reached[i], __ATOMIC_ACQUIRE); }

static inline void publish(float *out, bool *reached, idx_t i, float v)
{
    __atomic_store(&out[i], &v, __ATOMIC_RELAXED);
    __atomic_store_n(&reached[i], true, __ATOMIC_RELEASE);
}

/* out[] of another range read without reached[] (the max rule's climb, :177) */
static inline float peek(const float *out, idx_t i)
{
    float v;
    __atomic_load(&out[i], &v, __ATOMIC_RELAXED);
    return v;
}

/* tree_filter_direct (filtering.c:102-154) */
static void filter_direct(dco_tree *t, float *out, bool *reached, uint64_t lwb, uint64_t upb, int a, double lambda)
{
    for (uint64_t v = lwb; v < upb; v++) {
        if (seen(reached, (idx_t)v)) continue;
        idx_t w = (idx_t)v, par = t->parent[w];
        while (par != BOTTOM && !seen(reached, w) && (t->gval[w] == t->gval[par] || AV(t, a, w) < lambda)) {
            w = par;
            par = t->parent[w];
        }
        float val;
        if (seen(reached, w)) val = out[w];
        else if (AV(t, a, w) >= lambda) val = t->gval[w];
        else val = 0;
        idx_t u = (idx_t)v;
        while (u != w) {
            if ((uint64_t)u >= lwb && (uint64_t)u < upb) publish(out, reached, u, val);
            u = t->parent[u];
        }
        if ((uint64_t)w >= lwb && (uint64_t)w < upb) publish(out, reached, w, val);
    }
}

/* tree_filter_min (filtering.c:55-100) */
static void filter_min(dco_tree *t, float *out, bool *reached, uint64_t lwb, uint64_t upb, int a, double lambda)
{
    for (uint64_t v = lwb; v < upb; v++) {
        if (seen(reached, (idx_t)v)) continue;
        idx_t w = levelroot(t, (idx_t)v), r = w, par = get_parent(t, w);
        while (par != BOTTOM && !seen(reached, w)) {
            if (AV(t, a, w) < lambda) r = w;
            w = par;
            par = get_parent(t, w);
        }
        float val;
        if (seen(reached, w) && out[w] != t->gval[w]) {
            val = out[w];
            r = w;
        } else if (AV(t, a, r) >= lambda) {
            val = t->gval[r];
        } else if (AV(t, a, r) < lambda && t->parent[r] != BOTTOM) {
            val = t->gval[t->parent[r]];
        } else {
            val = 0;
        }
        idx_t u = (idx_t)v;
        while (u != r) {
            if ((uint64_t)u >= lwb && (uint64_t)u < upb) publish(out, reached, u, val);
            u = t->parent[u];
        }
        if ((uint64_t)r >= lwb && (uint64_t)r < upb) publish(out, reached, r, val);
    }
}

/* tree_filter_max (filtering.c:156-208) */
static void filter_max(dco_tree *t, float *out, bool *reached, uint64_t lwb, uint64_t upb, int a, double lambda)
{
    for (uint64_t v = lwb; v < upb; v++) {
        if (seen(reached, (idx_t)v)) continue;
        idx_t w = (idx_t)v, par = t->parent[w], u;
        while (par != BOTTOM && !seen(reached, w) && (t->gval[w] == t->gval[par] || AV(t, a, w) < lambda)) {
            w = par;
            par = t->parent[w];
        }
        float val;
        if (seen(reached, w)) {
            val = out[w];
        } else if (AV(t, a, w) >= lambda) {
            val = t->gval[w];
            u = par;
            while (u != BOTTOM && peek(out, u) != t->gval[u]) {
                if ((uint64_t)u >= lwb && (uint64_t)u < upb) {
                    publish(out, reached, u, t->gval[u]);
                } else {
                    __atomic_store_n(&reached[u], false, __ATOMIC_RELAXED);
                    break;
                }
                u = t->parent[u];
            }
        } else {
            val = 0;
        }
        u = (idx_t)v;
        while ((uint64_t)u != (uint64_t)w) {
            if ((uint64_t)u >= lwb && (uint64_t)u < upb) publish(out, reached, u, val);
            u = t->parent[u];
        }
        if ((uint64_t)w >= lwb && (uint64_t)w < upb) publish(out, reached, w, val);
    }
}

/* tree_filter_subtractive (filtering.c:211-261); the level path arrays are heap
 * buffers of max_levels entries instead of stack arrays */
static void filter_subtractive(dco_tree *t, float *out, bool *reached, uint64_t lwb, uint64_t upb, int a,
                               double lambda)
{
    idx_t *levpath = malloc(t->max_levels * sizeof(idx_t));
    float *filt = malloc(t->max_levels * sizeof(float));
    for (uint64_t v = lwb; v < upb; v++) {
        if (seen(reached, (idx_t)v)) continue;
        idx_t w = levelroot(t, (idx_t)v), u;
        int64_t i = 0, j;
        while (w != BOTTOM && !seen(reached, w)) {
            levpath[i++] = w;
            w = get_parent(t, w);
        }
        levpath[i] = w;
        if (w != BOTTOM) filt[i] = out[w];
        for (j = i - 1; j >= 0; j--) {
            u = levpath[j];
            if (w != BOTTOM) {
                if (AV(t, a, u) < lambda) filt[j] = filt[j + 1];
                else filt[j] = t->gval[u] + filt[j + 1] - t->gval[w];
            } else if (AV(t, a, u) >= lambda) {
                filt[j] = t->gval[u];
            } else {
                filt[j] = 0;
            }
            w = u;
        }
        u = (idx_t)v;
        for (j = 0; j <= i; j++) {
            while ((uint64_t)u != (uint64_t)levpath[j]) {
                if ((uint64_t)u >= lwb && (uint64_t)u < upb) publish(out, reached, u, filt[j]);
                u = t->parent[u];
            }
            if ((uint64_t)u >= lwb && (uint64_t)u < upb) publish(out, reached, u, filt[j]);
            if (u != BOTTOM) u = t->parent[u];
        }
    }
    free(levpath);
    free(filt);
}

/* tree_filtering (filtering.c:18-45) */
static void tree_filtering(dco_tree *t, float *out, int rule, int a, double lambda)
{
    uint64_t n = t->n;
    bool *reached = calloc(n, sizeof(bool));
    /* the max rule reads out[] of unreached nodes (filtering.c:177); the reference's
     * output buffer is a fresh allocation, i.e. zero pages for any real image */
    memset(out, 0, n * sizeof(float));
#pragma omp parallel num_threads(t->threads)
    {
        int np = omp_get_num_threads(), id = omp_get_thread_num();
        uint64_t lwb = id * n / np, upb = (id + 1) * n / np;
        switch (rule) {
        case 0: filter_direct(t, out, reached, lwb, upb, a, lambda); break;
        case 1: filter_min(t, out, reached, lwb, upb, a, lambda); break;
        case 2: filter_max(t, out, reached, lwb, upb, a, lambda); break;
        default: filter_subtractive(t, out, reached, lwb, upb, a, lambda); break;
        }
    }
    if (rule == 2) {
        for (uint64_t i = 0; i < n; i++) {
            if (!reached[i]) {
                idx_t im = (idx_t)i;
                while (im != BOTTOM && out[im] != t->gval[im]) {
                    out[im] = t->gval[im];
                    im = t->parent[im];
                }
            }
        }
    }
    free(reached);
}

int dco_filter(dco_tree *t, int attr, int rule, double lambda, int extract, float *out)
{
    if (dco_prepare(t, attr)) return -1;
    tree_filtering(t, out, rule, attr, lambda);
    /* perform_filter_or_extract (operation.c:17-28) */
    if (extract)
        for (uint64_t i = 0; i < t->n; i++) out[i] = t->gval[i] - out[i];
    if (t->tree_min)
        for (uint64_t i = 0; i < t->n; i++) out[i] = t->gmax - out[i];
    return 0;
}

int dco_check(dco_tree *t, int attr, float *out)
{
    if (dco_prepare(t, attr)) return -1;
    /* tree_attribute_check (filtering.c:47-52) */
    for (uint64_t v = 0; v < t->n; v++) {
        idx_t lr = levelroot(t, (idx_t)v);
        out[v] = (float)attr_value(t, attr, ATTR(t, lr));
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* pattern spectra (pattern.c:7-203, np()==1 branch)                   */
/* ------------------------------------------------------------------ */

/* find_scale (pattern.c:7-24) */
static int find_scale(const float *lv, int n, double a)
{
    int upper = n - 1, lower = 0, mid;
    if (a >= (double)lv[upper]) return upper;
    mid = (upper + lower) / 2;
    while (mid != lower) {
        if (a >= (double)lv[mid]) lower = mid;
        else upper = mid;
        mid = (upper + lower) / 2;
    }
    return lower;
}

static void spectrum_core(dco_tree *t, const float *l1, int n1, int a1, const float *l2, int n2, int a2,
                          int area_group, double *out)
{
    const int nb = n1 * n2;
    const int nt = t->threads;
    double *part = calloc((size_t)nb * nt, sizeof(double));
    const uint64_t n = t->n;
#pragma omp parallel num_threads(nt)
    {
        int id = omp_get_thread_num(), np = omp_get_num_threads();
        uint64_t lo = id * n / np, hi = (id + 1) * n / np; /* static schedule */
        for (uint64_t v = lo; v < hi; v++) {
            if (!is_levelroot(t, (idx_t)v)) continue;
            idx_t p = t->parent[v];
            float dh = p != BOTTOM ? (t->gval[v] - t->gval[p]) : t->gval[v];
            if (!dh) continue;
            const void *r = ATTR(t, v);
            int s1 = find_scale(l1, n1, a1 < 0 ? attr_area(t, area_group, r) : attr_value(t, a1, r));
            int s2 = n2 == 1 ? 0 : find_scale(l2, n2, a2 < 0 ? attr_area(t, area_group, r) : attr_value(t, a2, r));
            part[(size_t)nb * id + s1 + s2 * n1] += dh * attr_area(t, area_group, r);
        }
    }
    for (int i = 0; i < nb; i++)
        for (int k = 0; k < nt; k++) out[i] += part[(size_t)k * nb + i];
    free(part);
}

int dco_pattern(dco_tree *t, int attr, const float *lv, int n, double *out)
{
    if (dco_prepare(t, attr)) return -1;
    memset(out, 0, n * sizeof(double));
    static const float one = 0;
    spectrum_core(t, lv, n, attr, &one, 1, 0, ATTR_GROUP[attr], out);
    return 0;
}

int dco_pattern2d(dco_tree *t, int a1, const float *l1, int n1, int a2, const float *l2, int n2, double *out)
{
    /* operation.c:93-100: attribute 1 must be the higher index unless attribute 2 is area */
    if (a1 == 0 && a2 != 0) return -2;
    if (dco_prepare(t, a1)) return -1;
    if (a2 != 0 && ATTR_GROUP[a2] != t->group) return -3;
    memset(out, 0, (size_t)n1 * n2 * sizeof(double));
    spectrum_core(t, l1, n1, a1, l2, n2, a2 == 0 ? -1 : a2, t->group, out);
    return 0;
}
