/*
 * rtdbs_oracle.h -- CPU oracle for the per-slide streaming DBSCAN path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it is called by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and
 * never by the product path (rtdbstream_gb300/ fails loudly without its CUDA
 * library instead of falling back here).
 *
 * Two restatements of the reference algorithm (Wang-Zm/RTDBStream, level-9
 * driver src/dbscan/dbscan.cpp:2258-2364):
 *
 *  oracle_window_bruteforce_ref  -- O(n^2) restatement of the reference's own
 *      CPU checker cluster_with_cpu (src/dbscan/util.cpp:299-354): FP32 squared
 *      distances, strict "< radius2", self counted, BFS seeded from the lowest
 *      core slot.  Pinned bit-exactly against the reference compiled from its
 *      own sources (oracle/Makefile -> oracle/_ref) and against the committed
 *      fixtures in tests/golden/.
 *
 *  oracle_window_grid -- rebuild-per-window grid DBSCAN (cell side >= Eps,
 *      3^d cell scan) with exact neighbour counts, union-find with min-slot
 *      roots and the deterministic border rule (border id = minimum canonical
 *      id over the clusters of its Eps-adjacent cores).  Two neighbour
 *      predicates:
 *        ORACLE_MODE_FP32 -- the reference's FP32 predicate
 *                            (src/dbscan/util.cpp:308-316, radius2 = r*r in
 *                            float, src/dbscan/dbscan.cpp:41);
 *        ORACLE_MODE_FP64 -- squared distance of the float32 inputs evaluated
 *                            in double, compared with Eps*Eps in double.
 *
 * Window layout: points are indexed by ring slot (slot = stream index mod W,
 * src/dbscan/dbscan.cpp:2289,2351), row-major [n][dim] float32, dim in 1..3.
 * Labels: 0 core, 1 border, 2 noise (src/dbscan/dbscan.h:27).  Cluster ids:
 * core = minimum core slot of its component, border = rule above, noise = own
 * slot.
 */
#ifndef RTDBS_ORACLE_H
#define RTDBS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_MODE_FP64 0
#define ORACLE_MODE_FP32 1

/* Per-window statistics reported by oracle_window_grid. */
typedef struct {
    int64_t dist_tests;   /* ordered candidate pairs whose distance was evaluated */
    int64_t band_pairs;   /* unordered pairs i<j whose FP32 squared distance lies in
                             the FP64 re-check band [lo, hi) (FP64 mode only) */
    int64_t cells;        /* non-empty grid cells */
} oracle_stats;

/* Returns 0 on success, negative on invalid arguments / allocation failure. */
int oracle_window_grid(const float* pts, int n, int dim, double eps, int min_pts,
                       int mode, int32_t* nn, int32_t* label, int32_t* cid,
                       oracle_stats* stats);

int oracle_window_bruteforce_ref(const float* pts, int n, int dim, double eps,
                                 int min_pts, int32_t* nn, int32_t* label,
                                 int32_t* cid);

/* Sliding-window driver.  stream holds n_total points [n_total][dim].  The
 * first window is points [0, W); slide k (1-based) replaces ring slots
 * [((k-1) mod (W/S))*S, +S) with points [W+(k-1)*S, +S).  Outputs for slides
 * first_slide..first_slide+n_out-1 are written row-major [n_out][W].
 * use_bruteforce selects oracle_window_bruteforce_ref (mode ignored, FP32). */
int oracle_stream(const float* stream, int64_t n_total, int dim, int W, int S,
                  double eps, int min_pts, int mode, int use_bruteforce,
                  int first_slide, int n_out, int32_t* nn, int32_t* label,
                  int32_t* cid, oracle_stats* stats);

/* FP64-mode band used by the FP32 filter: a pair is re-decided in FP64 when
 * lo <= d32 < hi.  Written here so tests can recompute it independently. */
void oracle_band(double eps, float* lo, float* hi, int* filter_ok);

#ifdef __cplusplus
}
#endif
#endif
