/*
 * rtdbs_oracle.c -- CPU oracle for the per-slide streaming DBSCAN path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; never linked into the product).
 * Build: cc -O2 -std=c11 -ffp-contract=off -fPIC -shared (oracle/Makefile).
 * -ffp-contract=off matters: every squared distance below must be the plain
 * IEEE sequence sub, mul, add without fused multiply-add, exactly as the
 * reference's CPU checker evaluates it on x86-64 (src/dbscan/util.cpp:308-316).
 */
#include "rtdbs_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- predicates */

/* Reference predicate: src/dbscan/util.cpp:308-316 (cluster_with_cpu) and
 * src/dbscan/dbscan.cu:264 -- float differences, sum of squares in the order
 * x, y, z (missing dimensions are 0, src/dbscan/util.cpp:146,232-233), strict
 * compare against radius2 = r*r computed in float (src/dbscan/dbscan.cpp:41). */
static inline float sqdist32(const float* a, const float* b, int dim) {
    float dx = a[0] - b[0];
    float dy = dim > 1 ? a[1] - b[1] : 0.0f;
    float dz = dim > 2 ? a[2] - b[2] : 0.0f;
    float d = dx * dx + dy * dy;
    d = d + dz * dz;
    return d;
}

static inline double sqdist64(const float* a, const float* b, int dim) {
    double dx = (double)a[0] - (double)b[0];
    double dy = dim > 1 ? (double)a[1] - (double)b[1] : 0.0;
    double dz = dim > 2 ? (double)a[2] - (double)b[2] : 0.0;
    double d = dx * dx + dy * dy;
    d = d + dz * dz;
    return d;
}

static float round_down_f(double x) {
    float f = (float)x;
    if ((double)f > x) f = nextafterf(f, 0.0f);
    return f;
}

static float round_up_f(double x) {
    float f = (float)x;
    if ((double)f < x) f = nextafterf(f, INFINITY);
    return f;
}

/* FP32 filter band for the FP64 predicate.  With u = 2^-24 the float sum of
 * three rounded squares of rounded differences has relative error at most
 * gamma_5 = 5u/(1-5u) ~ 3.0e-7 (Higham, Accuracy and Stability of Numerical
 * Algorithms, 2nd ed., Lemma 3.1 / eq. 3.5); the double evaluation has at
 * most 5*2^-53.  A margin of 2^-20 (9.5e-7) on each side of E = Eps*Eps
 * therefore decides every pair outside [lo, hi) exactly as the double
 * evaluation would.  Valid while E stays away from float under/overflow. */
void oracle_band(double eps, float* lo, float* hi, int* filter_ok) {
    const double E = eps * eps;
    const double m = 1.0 / 1048576.0; /* 2^-20 */
    *lo = round_down_f(E * (1.0 - m));
    *hi = round_up_f(E * (1.0 + m));
    *filter_ok = (E >= ldexp(1.0, -100) && E <= ldexp(1.0, 100)) ? 1 : 0;
}

/* -------------------------------------------------------------- union-find */

static int uf_find(int32_t* parent, int x) {
    while (parent[x] != x) {
        parent[x] = parent[parent[x]];
        x = parent[x];
    }
    return x;
}

/* Hook the larger root under the smaller, so the root of every component is
 * its minimum slot (src/dbscan/util.cpp:290-297; src/dbscan/dbscan.cu:22-43). */
static void uf_unite(int32_t* parent, int a, int b) {
    int ra = uf_find(parent, a);
    int rb = uf_find(parent, b);
    if (ra < rb) parent[rb] = ra;
    else if (rb < ra) parent[ra] = rb;
}

/* -------------------------------------------------------------------- grid */

typedef struct {
    int64_t key;
    int32_t idx;
} key_idx;

static int cmp_key_idx(const void* pa, const void* pb) {
    const key_idx* a = (const key_idx*)pa;
    const key_idx* b = (const key_idx*)pb;
    if (a->key != b->key) return a->key < b->key ? -1 : 1;
    return a->idx < b->idx ? -1 : (a->idx > b->idx);
}

static int64_t find_cell(const int64_t* ukey, int64_t ncells, int64_t key) {
    int64_t lo = 0, hi = ncells;
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (ukey[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return (lo < ncells && ukey[lo] == key) ? lo : -1;
}

int oracle_window_grid(const float* pts, int n, int dim, double eps, int min_pts,
                       int mode, int32_t* nn, int32_t* label, int32_t* cid,
                       oracle_stats* stats) {
    if (n < 0 || dim < 1 || dim > 3 || !(eps > 0.0) || (mode != ORACLE_MODE_FP64 && mode != ORACLE_MODE_FP32))
        return -1;
    oracle_stats st = {0, 0, 0};
    if (n == 0) {
        if (stats) *stats = st;
        return 0;
    }
    const float r32 = (float)eps;
    const float r2f = r32 * r32;
    const double E = eps * eps;
    float lo = 0.0f, hi = 0.0f;
    int filter_ok = 0;
    oracle_band(eps, &lo, &hi, &filter_ok);

    /* Grid: cell side L >= Eps with a relative margin, origin at the window's
     * finite minimum; cell coordinates in double, clamped to the extent (a
     * clamped coordinate is still monotone, so the 3^d scan stays complete). */
    double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    for (int a = 0; a < dim; ++a) {
        double lo_a = INFINITY, hi_a = -INFINITY;
        for (int i = 0; i < n; ++i) {
            double v = pts[(size_t)i * dim + a];
            if (isfinite(v)) {
                if (v < lo_a) lo_a = v;
                if (v > hi_a) hi_a = v;
            }
        }
        if (!(lo_a <= hi_a)) lo_a = hi_a = 0.0;
        mn[a] = lo_a;
        mx[a] = hi_a;
    }
    double L = eps * (1.0 + 1.0 / 4096.0);
    int64_t ext[3] = {1, 1, 1};
    for (;;) {
        double prod = 1.0;
        for (int a = 0; a < dim; ++a) {
            double e = floor((mx[a] - mn[a]) / L) + 1.0;
            ext[a] = (int64_t)e;
            prod *= e;
        }
        if (prod < 4.0e18) break;
        L *= 2.0;
    }

    key_idx* ki = (key_idx*)malloc(sizeof(key_idx) * (size_t)n);
    int64_t* coords = (int64_t*)malloc(sizeof(int64_t) * 3 * (size_t)n);
    if (!ki || !coords) {
        free(ki);
        free(coords);
        return -2;
    }
    for (int i = 0; i < n; ++i) {
        int64_t key = 0;
        for (int a = 0; a < 3; ++a) {
            int64_t c = 0;
            if (a < dim) {
                double q = floor(((double)pts[(size_t)i * dim + a] - mn[a]) / L);
                if (!(q >= 0.0)) q = 0.0;
                if (q > (double)(ext[a] - 1)) q = (double)(ext[a] - 1);
                c = (int64_t)q;
            }
            coords[(size_t)i * 3 + a] = c;
            key = key * ext[a] + c;
        }
        ki[i].key = key;
        ki[i].idx = i;
    }
    qsort(ki, (size_t)n, sizeof(key_idx), cmp_key_idx);

    int64_t* ukey = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    int64_t* ustart = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
    int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int64_t* cell_of = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    int32_t* parent = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    if (!ukey || !ustart || !order || !cell_of || !parent) {
        free(ki); free(coords); free(ukey); free(ustart); free(order); free(cell_of); free(parent);
        return -2;
    }
    int64_t ncells = 0;
    for (int i = 0; i < n; ++i) {
        order[i] = ki[i].idx;
        if (i == 0 || ki[i].key != ki[i - 1].key) {
            ukey[ncells] = ki[i].key;
            ustart[ncells] = i;
            ++ncells;
        }
        cell_of[ki[i].idx] = ncells - 1;
    }
    ustart[ncells] = n;
    st.cells = ncells;

    /* Neighbour cells of every cell (3^dim offsets, absent cells -> -1). */
    const int noff = dim == 1 ? 3 : (dim == 2 ? 9 : 27);
    int64_t* ncell = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncells * noff);
    if (!ncell) {
        free(ki); free(coords); free(ukey); free(ustart); free(order); free(cell_of); free(parent);
        return -2;
    }
    for (int64_t c = 0; c < ncells; ++c) {
        const int64_t* cc = &coords[(size_t)order[ustart[c]] * 3];
        int o = 0;
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = (dim > 1 ? -1 : 0); dy <= (dim > 1 ? 1 : 0); ++dy)
                for (int dz = (dim > 2 ? -1 : 0); dz <= (dim > 2 ? 1 : 0); ++dz) {
                    int64_t q[3] = {cc[0] + dx, cc[1] + dy, cc[2] + dz};
                    int ok = 1;
                    int64_t key = 0;
                    for (int a = 0; a < 3; ++a) {
                        if (q[a] < 0 || q[a] >= ext[a]) ok = 0;
                        key = key * ext[a] + q[a];
                    }
                    ncell[(size_t)c * noff + o++] = ok ? find_cell(ukey, ncells, key) : -1;
                }
    }

#define NBR(i, j, dij32)                                                          \
    ((i) == (j) ? 1                                                               \
     : (mode == ORACLE_MODE_FP32 ? ((dij32) < r2f)                                \
        : (sqdist64(&pts[(size_t)(i) * dim], &pts[(size_t)(j) * dim], dim) < E)))

    /* 1. exact neighbour counts (self included: src/dbscan/util.cpp:306). */
    for (int i = 0; i < n; ++i) {
        const int64_t c = cell_of[i];
        int32_t cnt = 0;
        for (int o = 0; o < noff; ++o) {
            const int64_t nc = ncell[(size_t)c * noff + o];
            if (nc < 0) continue;
            for (int64_t p = ustart[nc]; p < ustart[nc + 1]; ++p) {
                const int j = order[p];
                float d32 = 0.0f;
                if (j != i) {
                    d32 = sqdist32(&pts[(size_t)i * dim], &pts[(size_t)j * dim], dim);
                    st.dist_tests++;
                    if (mode == ORACLE_MODE_FP64 && i < j && d32 >= lo && !(d32 >= hi))
                        st.band_pairs++;
                }
                cnt += NBR(i, j, d32) ? 1 : 0;
            }
        }
        nn[i] = cnt;
    }

    /* 2. core flags (src/dbscan/util.cpp:320-323) and union-find over cores. */
    for (int i = 0; i < n; ++i) parent[i] = i;
    for (int i = 0; i < n; ++i) {
        if (nn[i] < min_pts) continue;
        const int64_t c = cell_of[i];
        for (int o = 0; o < noff; ++o) {
            const int64_t nc = ncell[(size_t)c * noff + o];
            if (nc < 0) continue;
            for (int64_t p = ustart[nc]; p < ustart[nc + 1]; ++p) {
                const int j = order[p];
                if (j <= i || nn[j] < min_pts) continue;
                float d32 = sqdist32(&pts[(size_t)i * dim], &pts[(size_t)j * dim], dim);
                if (NBR(i, j, d32)) uf_unite(parent, i, j);
            }
        }
    }

    /* 3. labels and ids.  Core: 0 and its root (the component's minimum core
     * slot, as the reference's BFS seeds from the lowest core,
     * src/dbscan/util.cpp:326-350).  Border: 1 and the minimum root over its
     * adjacent cores (the BFS visits components in increasing seed order, so
     * this is the id cluster_with_cpu assigns).  Noise: 2 and its own slot. */
    for (int i = 0; i < n; ++i) {
        if (nn[i] >= min_pts) {
            label[i] = 0;
            cid[i] = uf_find(parent, i);
            continue;
        }
        int32_t best = INT32_MAX;
        const int64_t c = cell_of[i];
        for (int o = 0; o < noff; ++o) {
            const int64_t nc = ncell[(size_t)c * noff + o];
            if (nc < 0) continue;
            for (int64_t p = ustart[nc]; p < ustart[nc + 1]; ++p) {
                const int j = order[p];
                if (j == i || nn[j] < min_pts) continue;
                float d32 = sqdist32(&pts[(size_t)i * dim], &pts[(size_t)j * dim], dim);
                if (NBR(i, j, d32)) {
                    int32_t r = uf_find(parent, j);
                    if (r < best) best = r;
                }
            }
        }
        if (best != INT32_MAX) {
            label[i] = 1;
            cid[i] = best;
        } else {
            label[i] = 2;
            cid[i] = i;
        }
    }
#undef NBR

    free(ki); free(coords); free(ukey); free(ustart); free(order); free(cell_of); free(parent); free(ncell);
    if (stats) *stats = st;
    return 0;
}

/* Restatement of cluster_with_cpu (src/dbscan/util.cpp:299-354).  One
 * normalisation: noise ids are set to the point's own slot (the reference
 * leaves them at whatever the buffer held before). */
int oracle_window_bruteforce_ref(const float* pts, int n, int dim, double eps,
                                 int min_pts, int32_t* nn, int32_t* label,
                                 int32_t* cid) {
    if (n < 0 || dim < 1 || dim > 3) return -1;
    const float r32 = (float)eps;
    const float r2f = r32 * r32;
    memset(nn, 0, sizeof(int32_t) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        nn[i]++;
        for (int j = i + 1; j < n; ++j) {
            float d = sqdist32(&pts[(size_t)i * dim], &pts[(size_t)j * dim], dim);
            if (d < r2f) {
                nn[i]++;
                nn[j]++;
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        label[i] = nn[i] >= min_pts ? 0 : 2;
        cid[i] = i;
    }
    unsigned char* vis = (unsigned char*)calloc((size_t)n + 1, 1);
    int32_t* queue = (int32_t*)malloc(sizeof(int32_t) * ((size_t)n + 1));
    if (!vis || !queue) {
        free(vis);
        free(queue);
        return -2;
    }
    for (int i = 0; i < n; ++i) {
        if (vis[i] || label[i] != 0) continue;
        vis[i] = 1;
        cid[i] = i;
        int qh = 0, qt = 0;
        queue[qt++] = i;
        while (qh < qt) {
            const float* p = &pts[(size_t)queue[qh++] * dim];
            for (int j = 0; j < n; ++j) {
                if (vis[j]) continue;
                float d = sqdist32(p, &pts[(size_t)j * dim], dim);
                if (d < r2f) {
                    vis[j] = 1;
                    cid[j] = i;
                    if (label[j] == 0) queue[qt++] = j;
                    else label[j] = 1;
                }
            }
        }
    }
    free(vis);
    free(queue);
    return 0;
}

int oracle_stream(const float* stream, int64_t n_total, int dim, int W, int S,
                  double eps, int min_pts, int mode, int use_bruteforce,
                  int first_slide, int n_out, int32_t* nn, int32_t* label,
                  int32_t* cid, oracle_stats* stats) {
    if (dim < 1 || dim > 3 || W <= 0 || S <= 0 || W % S != 0 || first_slide < 1 || n_out < 0)
        return -1;
    const int64_t last = (int64_t)first_slide + n_out - 1;
    if (n_out > 0 && (int64_t)W + last * S > n_total) return -1;
    float* win = (float*)malloc(sizeof(float) * (size_t)W * dim);
    if (!win) return -2;
    memcpy(win, stream, sizeof(float) * (size_t)W * dim);
    const int units = W / S;
    int rc = 0;
    for (int64_t k = 1; k <= last && rc == 0; ++k) {
        const int64_t slot0 = ((k - 1) % units) * (int64_t)S;
        memcpy(&win[slot0 * dim], &stream[((int64_t)W + (k - 1) * S) * dim],
               sizeof(float) * (size_t)S * dim);
        if (k < first_slide) continue;
        const size_t off = (size_t)(k - first_slide) * W;
        oracle_stats st;
        if (use_bruteforce)
            rc = oracle_window_bruteforce_ref(win, W, dim, eps, min_pts, nn + off, label + off, cid + off);
        else
            rc = oracle_window_grid(win, W, dim, eps, min_pts, mode, nn + off, label + off, cid + off, &st);
        if (rc == 0 && stats && !use_bruteforce) stats[k - first_slide] = st;
    }
    free(win);
    return rc;
}
