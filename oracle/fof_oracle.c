/*
 * ORACLE (test infrastructure only): exact friends-of-friends partition on the CPU.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this code.
 *
 * pyHALMA's FoF (python_scripts/fof.py:18-79) flood-fills the graph whose edges are the
 * pairs returned by scipy.spatial.KDTree.query_ball_point(data[i], linking_length)
 * (fof.py:40,61).  It keeps every connected component with at least two members
 * (fof.py:43-44 drops particles with no friend), sorts each component's indices
 * (fof.py:76) and emits components in order of their smallest index (the outer loop
 * fof.py:34 seeds each group at its lowest unvisited particle).  The same partition is
 * written here as labels: label[i] = smallest index of i's component, or -1 when i has
 * no friend.
 *
 * The pair predicate is the one scipy 1.18.1's cKDTree applies for p = 2, pinned in this
 * repository by adversarial nextafter pairs against the reference (tests/golden):
 *     ((dx*dx + dy*dy) + dz*dz) <= r*r      in IEEE double, every operation rounded,
 * inclusive at equality, non-periodic (fof.py:20 builds the tree without boxsize).
 * Built with -ffp-contract=off so no multiply-add is fused.
 *
 * Method (independent of the KDTree): bucket particles in cubic cells of side
 * r * (1 + 1e-6), sort the buckets, test each unordered pair of particles in the same or
 * adjacent cells once, and join the pair in a union-find whose root is always the smaller
 * index (so a component's root is its minimum index).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

typedef struct { int64_t cx, cy, cz; int64_t idx; } cell_item;

static int cmp_item(const void *a, const void *b)
{
    const cell_item *p = (const cell_item *)a, *q = (const cell_item *)b;
    if (p->cx != q->cx) return p->cx < q->cx ? -1 : 1;
    if (p->cy != q->cy) return p->cy < q->cy ? -1 : 1;
    if (p->cz != q->cz) return p->cz < q->cz ? -1 : 1;
    return p->idx < q->idx ? -1 : (p->idx > q->idx);
}

static int64_t uf_find(int64_t *parent, int64_t v)
{
    while (parent[v] != v) {
        parent[v] = parent[parent[v]];
        v = parent[v];
    }
    return v;
}

static void uf_union(int64_t *parent, int64_t a, int64_t b)
{
    a = uf_find(parent, a);
    b = uf_find(parent, b);
    if (a == b) return;
    if (a < b) parent[b] = a; else parent[a] = b;
}

static int linked(const double *x, const double *y, const double *z, int64_t i, int64_t j,
                  double r2)
{
    const double dx = x[i] - x[j];
    const double dy = y[i] - y[j];
    const double dz = z[i] - z[j];
    double s = dx * dx;
    s = s + dy * dy;
    s = s + dz * dz;
    return s <= r2;
}

/* First position in the sorted cell table whose cell is >= (cx,cy,cz). */
static int64_t lower_cell(const cell_item *it, const int64_t *cstart, int64_t ncell,
                          int64_t cx, int64_t cy, int64_t cz)
{
    int64_t lo = 0, hi = ncell;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        const cell_item *c = &it[cstart[mid]];
        int less = (c->cx < cx) || (c->cx == cx && (c->cy < cy || (c->cy == cy && c->cz < cz)));
        if (less) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* Returns 0 on success, -1 on allocation failure, -2 on bad arguments. */
int oracle_fof_labels(int64_t n, const double *x, const double *y, const double *z,
                      double linking_length, int32_t *labels)
{
    if (n < 0 || !(linking_length >= 0.0)) return -2;
    if (n == 0) return 0;
    const double r2 = linking_length * linking_length;
    double mn[3] = {x[0], y[0], z[0]};
    for (int64_t i = 1; i < n; ++i) {
        if (x[i] < mn[0]) mn[0] = x[i];
        if (y[i] < mn[1]) mn[1] = y[i];
        if (z[i] < mn[2]) mn[2] = z[i];
    }
    double cell = linking_length * (1.0 + 1e-6);
    if (cell <= 0.0) cell = 1.0;   /* r = 0: only coincident points link; any cell works */
    cell_item *it = (cell_item *)malloc(sizeof(cell_item) * (size_t)n);
    int64_t *parent = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    int64_t *cstart = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    unsigned char *has = (unsigned char *)calloc((size_t)n, 1);
    if (!it || !parent || !cstart || !has) {
        free(it); free(parent); free(cstart); free(has);
        return -1;
    }
    for (int64_t i = 0; i < n; ++i) {
        it[i].cx = (int64_t)floor((x[i] - mn[0]) / cell);
        it[i].cy = (int64_t)floor((y[i] - mn[1]) / cell);
        it[i].cz = (int64_t)floor((z[i] - mn[2]) / cell);
        it[i].idx = i;
        parent[i] = i;
    }
    qsort(it, (size_t)n, sizeof(cell_item), cmp_item);
    int64_t ncell = 0;
    for (int64_t k = 0; k < n; ++k)
        if (k == 0 || it[k].cx != it[k - 1].cx || it[k].cy != it[k - 1].cy || it[k].cz != it[k - 1].cz)
            cstart[ncell++] = k;
    cstart[ncell] = n;

    for (int64_t c = 0; c < ncell; ++c) {
        const int64_t s0 = cstart[c], e0 = cstart[c + 1];
        const int64_t cx = it[s0].cx, cy = it[s0].cy, cz = it[s0].cz;
        /* same cell: each unordered pair once */
        for (int64_t a = s0; a < e0; ++a)
            for (int64_t b = a + 1; b < e0; ++b) {
                const int64_t i = it[a].idx, j = it[b].idx;
                if (linked(x, y, z, i, j, r2)) { uf_union(parent, i, j); has[i] = has[j] = 1; }
            }
        /* the 13 neighbour cells that sort after this one */
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    int after = dx > 0 || (dx == 0 && (dy > 0 || (dy == 0 && dz > 0)));
                    if (!after) continue;
                    const int64_t q = lower_cell(it, cstart, ncell, cx + dx, cy + dy, cz + dz);
                    if (q >= ncell) continue;
                    const cell_item *cc = &it[cstart[q]];
                    if (cc->cx != cx + dx || cc->cy != cy + dy || cc->cz != cz + dz) continue;
                    for (int64_t a = s0; a < e0; ++a)
                        for (int64_t b = cstart[q]; b < cstart[q + 1]; ++b) {
                            const int64_t i = it[a].idx, j = it[b].idx;
                            if (linked(x, y, z, i, j, r2)) {
                                uf_union(parent, i, j);
                                has[i] = has[j] = 1;
                            }
                        }
                }
    }
    for (int64_t i = 0; i < n; ++i)
        labels[i] = has[i] ? (int32_t)uf_find(parent, i) : -1;
    free(it); free(parent); free(cstart); free(has);
    return 0;
}
