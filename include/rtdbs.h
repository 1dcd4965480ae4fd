/*
 * rtdbs.h -- C ABI of the GB300-native streaming DBSCAN engine.
 *
 * Drop-in for the per-slide clustering path of RTDBStream (level-9 driver,
 * src/dbscan/dbscan.cpp:2258-2364): a ring-buffer window of W points slides
 * by S points per step; after every slide the engine returns, indexed by ring
 * slot, label[W] (0 core, 1 border, 2 noise; src/dbscan/dbscan.h:27) and
 * cluster_id[W].
 *
 * Semantics (identical to the reference's CPU checker cluster_with_cpu,
 * src/dbscan/util.cpp:299-354, under RTDBS_PREC_FP32):
 *   - neighbour: squared distance strictly below Eps^2, the point itself
 *     included; core <=> neighbour count >= min_pts;
 *   - core id: the minimum core slot of its connected component;
 *   - border id: the minimum core id over the clusters of its Eps-adjacent
 *     cores; noise id: its own slot.
 * Precision modes:
 *   RTDBS_PREC_FP64 (default) -- the neighbour relation of an FP64
 *       evaluation of the float32 inputs against Eps*Eps in double; FP32
 *       filter, pairs inside a proven rounding band re-decided in FP64;
 *   RTDBS_PREC_FP32 -- the reference's FP32 predicate (float differences and
 *       squares, compared with (float)Eps*(float)Eps), bit-identical to
 *       cluster_with_cpu.
 *
 * Every function returns an int status (0 = RTDBS_OK, negative = error) and
 * never throws.  One engine is driven by one host thread at a time; all device
 * work runs on the engine's CUDA stream.  The engine owns its device memory;
 * the caller owns its input/output buffers.  No torch types cross this ABI.
 */
#ifndef RTDBS_H
#define RTDBS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTDBS_ABI_VERSION 2

#if defined(__GNUC__)
#define RTDBS_API __attribute__((visibility("default")))
#else
#define RTDBS_API
#endif

/* Status codes. */
#define RTDBS_OK             0
#define RTDBS_ERR_INVALID   -1  /* bad argument: dim not in 1..3, W % S != 0, Eps <= 0, NULL pointer */
#define RTDBS_ERR_CUDA      -2  /* a CUDA runtime call failed (rtdbs_last_error has the text) */
#define RTDBS_ERR_OOM       -3  /* device or pinned allocation failed */
#define RTDBS_ERR_STATE     -4  /* call out of order (slide before rtdbs_load_window) */
#define RTDBS_ERR_DEVICE    -5  /* a device-side bound was hit (hash probe, union-find retry,
                                   work-list capacity); the engine must be reloaded */
#define RTDBS_ERR_NO_DEVICE -6  /* no CUDA device / library built without one */
#define RTDBS_ERR_BUDGET    -7  /* pool admission refused: HBM budget or stream slots exhausted */

/* Precision modes. */
#define RTDBS_PREC_FP64 0
#define RTDBS_PREC_FP32 1

/* Labels (src/dbscan/dbscan.h:27). */
#define RTDBS_LABEL_CORE   0
#define RTDBS_LABEL_BORDER 1
#define RTDBS_LABEL_NOISE  2

/* Flags of rtdbs_params.flags. */
#define RTDBS_FLAG_NO_GRAPH 1   /* launch kernels directly instead of replaying a CUDA graph */

/* Engine parameters: the reference's -W -S -R -K arguments
 * (src/dbscan/util.cpp:454-500) plus the dataset bounding box it derives from
 * the whole input file (src/dbscan/util.cpp:12-254, used for its grid at
 * src/dbscan/dbscan.cpp:34-37). */
typedef struct rtdbs_params {
    int32_t dim;          /* point dimension, 1..3 */
    int32_t window;       /* W: points in the window (ring slots) */
    int32_t stride;       /* S: points entering and leaving per slide; W % S == 0 */
    int32_t min_pts;      /* MinPts */
    double  eps;          /* Eps (> 0) */
    int32_t precision;    /* RTDBS_PREC_* */
    int32_t has_bbox;     /* 1: bbox_min/bbox_max bound the whole stream; 0: taken from
                             the first window with a margin (points outside are still
                             handled exactly, only more slowly) */
    float   bbox_min[3];
    float   bbox_max[3];
    int32_t device;       /* CUDA device ordinal */
    int32_t flags;        /* RTDBS_FLAG_* */
    int32_t cell_mult;    /* K: grid cells per Eps along each axis, 1 or 2 (0 = 1); the
                             scan covers (2K+1)^dim cells of side Eps/K, so K = 2 tests
                             fewer pairs where cells are dense and costs more cells and
                             work items where they are sparse (rtdbstream_gb300/autotune.py
                             picks it per stream).  The reference's grid has side Eps/sqrt(3)
                             (src/dbscan/dbscan.cpp:34-37) */
    int32_t work_grab;    /* work items (cell runs) a clustering warp takes from the shared
                             queue at a time, 1..64 (0 = 8 in a pool; for a stream slid on
                             its own, 5 or 8 on large windows by cell occupancy and fewer
                             on small ones: 1 below 32,768 points): the work split between
                             warps, picked by rtdbstream_gb300/autotune.py.  No reference
                             counterpart */
    int32_t query_lanes;  /* lanes that scan one expired or new point's neighbourhood in the
                             count passes, 16 or 32 (0 = 16 with one cell per Eps, 32 with
                             two; two cells per Eps needs 32): the block shape of those
                             passes (a 256-thread block takes 16 or 8 points), picked by
                             rtdbstream_gb300/autotune.py.  No reference counterpart */
    int32_t reserved[3];
} rtdbs_params;

/* Cumulative counters (src/dbscan/dbscan.cpp:145-212 keeps similar debug counters). */
typedef struct rtdbs_stats {
    int64_t slides;          /* slides completed */
    int64_t band_rechecks;   /* pair tests re-decided in FP64 (FP64 mode) */
    int64_t cells;           /* non-empty grid cells of the current window */
    int64_t work_items;      /* cell runs scheduled by the clustering kernels */
    int32_t error_bits;      /* device error word (0 = healthy) */
    int32_t key_bits;        /* bits of the cell key */
    double  cell_side;       /* grid cell side (>= Eps) */
    int64_t device_bytes;    /* device memory owned by the engine */
    int32_t launches_per_slide; /* kernels launched by one slide */
    int32_t chunks_per_slide;   /* grid-update chunks per slide (ceil(S / 16384)) */
    int64_t dist_tests;         /* distance tests evaluated, cumulative (the reference's
                                   DEBUG_INFO num_dist_calculations, src/dbscan/dbscan.cpp:145-212);
                                   query_tests + cluster_tests */
    int64_t reused_cores;       /* cores that started the last clustering in a component
                                   kept from the previous slide (no counterpart in the
                                   reference, which re-clusters every slide) */
    /* The reference's DEBUG_INFO ray counters (print_rt_info,
     * src/dbscan/dbscan.cpp:145-178), cumulative: */
    int64_t query_tests;        /* count passes (core identification): distance tests, the
                                   intersection tests of its core rays (ray_intersections) */
    int64_t query_hits;         /* ... that found a neighbour (ray_primitive_hits) */
    int64_t cluster_tests;      /* clustering scans: distance tests (ray_intersections_cluster) */
    int64_t cluster_hits;       /* ... that found a neighbour (ray_primitive_hits_cluster) */
    int32_t max_query_tests;    /* most distance tests of one count query (max_ray_intersections) */
    int32_t reserved0;
    int64_t reserved[3];
} rtdbs_stats;

/* Per-phase device time of one profiled slide, in milliseconds (the
 * reference's Timer phases, src/dbscan/timer.h:10-238, measured with CUDA
 * events on the engine's stream).  Chunk phases are summed over chunks. */
typedef struct rtdbs_phase_times {
    float ingest_ms;      /* new points -> ring slots, cell keys */
    float sort_ms;        /* radix sort of the chunk's (cell, slot) words */
    float decrement_ms;   /* -1 on neighbours of expired points */
    float merge_ms;       /* sorted-window merge */
    float build_ms;       /* cell table + work list */
    float increment_ms;   /* counts of new points, +1 on their neighbours */
    float union_ms;       /* union-find over core pairs */
    float flatten_ms;     /* root of every core point */
    float label_ms;       /* labels, ids, border rule */
    float total_ms;       /* first launch to last */
    int32_t chunks;
} rtdbs_phase_times;

typedef struct rtdbs_engine rtdbs_engine;

RTDBS_API int rtdbs_abi_version(void);
RTDBS_API const char* rtdbs_status_string(int status);
/* Text of the last error raised on the calling thread ("" if none). */
RTDBS_API const char* rtdbs_last_error(void);

/* Fills defaults: dim 3, precision FP64, no bbox, device 0, min_pts 5. */
RTDBS_API int rtdbs_params_init(rtdbs_params* params);

/* Allocates every device buffer up front, sized by W and S.
 * Replaces initialize_params (src/dbscan/dbscan.cpp:30-132).
 * cuda_stream is a cudaStream_t (NULL: the engine creates its own stream). */
RTDBS_API int rtdbs_create(const rtdbs_params* params, void* cuda_stream, rtdbs_engine** out);

/* Frees everything.  Replaces cleanup (src/dbscan/dbscan.cpp:2366-2448). */
RTDBS_API int rtdbs_destroy(rtdbs_engine* engine);

/* Loads the first window: points[W][dim] into slots 0..W-1, grid built.
 * Replaces the first-window set-up (src/dbscan/dbscan.cpp:2268-2272).
 * points_on_device: 1 if points is a device pointer.  Synchronous. */
RTDBS_API int rtdbs_load_window(rtdbs_engine* engine, const float* points, int points_on_device);

/* One slide with host buffers: new_points[S][dim] replace slots
 * [u*S, u*S+S) (u = slides done mod W/S), then label[W] and cluster_id[W]
 * (host memory; pinned memory avoids a staging copy) receive the window's
 * result.  Replaces one iteration of the reference's slide loop
 * (src/dbscan/dbscan.cpp:2276-2362: H2D at 2289, grid update 2293, core
 * identification 2300-2322, clustering 2331-2336, D2H 2344-2345).
 * Synchronous; returns RTDBS_ERR_DEVICE if a device bound was hit. */
RTDBS_API int rtdbs_slide(rtdbs_engine* engine, const float* new_points, int32_t* label,
                int32_t* cluster_id);

/* Same slide with device pointers, stream-ordered, no host synchronisation.
 * label/cluster_id may be NULL: the result then stays in the engine's own
 * buffers (rtdbs_device_outputs). */
RTDBS_API int rtdbs_slide_async(rtdbs_engine* engine, const float* d_new_points, int32_t* d_label,
                      int32_t* d_cluster_id);

/* One slide with host buffers, pipelined: enqueues the slide (new points in,
 * label[W] and cluster_id[W] out, as rtdbs_slide) and returns once the
 * previous pipelined slide is complete, so the host prepares slide k+1 while
 * slide k runs.  On return the previous call's label/cluster_id hold its
 * result and its new_points may be reused; this call's three buffers stay in
 * use until the next pipelined call, or any synchronising call, returns.
 * Pinned host buffers keep the copies asynchronous (pageable memory makes
 * them synchronous).  A device bound hit by a slide is reported by the call
 * that completes it.  The reference's loop reads every slide's result before
 * taking the next stride (src/dbscan/dbscan.cpp:2276-2362); this is the same
 * loop with one slide in flight. */
RTDBS_API int rtdbs_slide_pipelined(rtdbs_engine* engine, const float* new_points, int32_t* label,
                                    int32_t* cluster_id);

/* Waits for the engine's stream; reports RTDBS_ERR_DEVICE if a device bound
 * was hit by any work since the previous check. */
RTDBS_API int rtdbs_sync(rtdbs_engine* engine);

/* Clusters the current window without sliding (e.g. right after
 * rtdbs_load_window).  Outputs are host or device memory per on_device. */
RTDBS_API int rtdbs_cluster(rtdbs_engine* engine, int32_t* label, int32_t* cluster_id, int on_device);

/* Exact neighbour counts (self included) of the current window by slot; the
 * reference's nn / check_nn (src/dbscan/util.cpp:299-323). */
RTDBS_API int rtdbs_get_counts(rtdbs_engine* engine, int32_t* nn, int on_device);

/* The engine's device output buffers (label[W], cluster_id[W]); they hold
 * the latest result until the next slide. */
RTDBS_API int rtdbs_device_outputs(rtdbs_engine* engine, int32_t** d_label, int32_t** d_cluster_id);

RTDBS_API int rtdbs_get_stats(rtdbs_engine* engine, rtdbs_stats* stats);

/* Largest window rtdbs_cluster_window_noalloc accepts. */
#define RTDBS_NOALLOC_MAX_POINTS 16384

/* Clusters one window of n <= RTDBS_NOALLOC_MAX_POINTS points without
 * allocating any memory.  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc (a host process that keeps the GPU's
 * memory in its own pool and forbids raw allocations by plug-ins, or a caller
 * on a latency path that cannot take cudaMalloc's implicit synchronisation).
 * Inputs and outputs are device memory owned by the caller: d_points[n][dim],
 * d_label[n], d_cluster_id[n] (NULL allowed when n = 0; index = the point's
 * position in d_points, with the same labels and ids as rtdbs_load_window +
 * rtdbs_cluster on a window of n slots).  Working memory is one static
 * device array of about 3.4 MB, part of the library: every GPU that loads the
 * library holds it until the process exits.  The first call on a device looks up that array's device
 * address, with that device current.  All calls share the array: calls whose
 * work overlaps on a GPU race and corrupt each other's results, so serialise
 * them.  Runs on cuda_stream (a cudaStream_t, NULL = default stream) and
 * waits for that stream twice (for the points' bounding box, and at the end),
 * so it must not be called while the stream is being captured into a graph
 * (rtdbs_cluster_window_noalloc_async below waits for nothing).
 * Returns RTDBS_ERR_INVALID for n above the limit or bad arguments,
 * RTDBS_ERR_CUDA if a runtime call fails and RTDBS_ERR_DEVICE if a device-side
 * bound was hit, with the text in rtdbs_last_error; an error return comes
 * after the stream has finished the call's work. */
RTDBS_API int rtdbs_cluster_window_noalloc(const float* d_points, int32_t n, int32_t dim, double eps,
                                           int32_t min_pts, int32_t precision, int32_t* d_label,
                                           int32_t* d_cluster_id, void* cuda_stream);

/* rtdbs_cluster_window_noalloc without any wait, for latency paths and CUDA
 * graph capture: the caller gives the grid's box (box_min[dim], box_max[dim],
 * host memory; points outside it fall into its edge cells and are still
 * clustered exactly, a tight box just keeps the grid small) and a device int
 * *d_status, which receives the device error bits (0: success; 1 table full,
 * 2 union-find bound, 4 work list full, 8 chunk bookkeeping) in stream order.
 * Everything is queued on cuda_stream and the call returns; the outputs and
 * *d_status are ready when the stream reaches that point.  Calls share the
 * scratch array with rtdbs_cluster_window_noalloc: serialise them (calls on
 * one stream are).  Returns RTDBS_ERR_INVALID for bad arguments or an empty
 * or non-finite box (before queueing anything) and RTDBS_ERR_CUDA if queueing
 * fails, in which case work queued before the failure may still run. */
RTDBS_API int rtdbs_cluster_window_noalloc_async(const float* d_points, int32_t n, int32_t dim, double eps,
                                                 int32_t min_pts, int32_t precision, const float* box_min,
                                                 const float* box_max, int32_t* d_label,
                                                 int32_t* d_cluster_id, int32_t* d_status,
                                                 void* cuda_stream);

/* rtdbs_slide_async with every kernel launched directly and bracketed by CUDA
 * events; synchronous.  Results are identical to an ordinary slide. */
RTDBS_API int rtdbs_slide_profiled(rtdbs_engine* engine, const float* d_new_points,
                                   rtdbs_phase_times* times);

/* ------------------------------------------------------------- data files
 * Readers for the reference's dataset formats (src/dbscan/util.cpp:12-254):
 * the format comes from the file name like the reference's
 * (src/dbscan/dbscan.cpp:2454-2470) or is given explicitly. */
#define RTDBS_FORMAT_AUTO    0
#define RTDBS_FORMAT_TAO     1  /* text "x,y,z" per line (3-D) */
#define RTDBS_FORMAT_GEOLIFE 2  /* binary double triples (3-D) */
#define RTDBS_FORMAT_RBF     3  /* header line, then "x,y" (2-D) */
#define RTDBS_FORMAT_EDS     4  /* header line, then "id x y cid" (2-D) */
#define RTDBS_FORMAT_STOCK   5  /* header line, then one value (1-D) */

/* Reads up to n_max points into xyz[n_max][3] (missing coordinates 0);
 * *n_read points were read, *dim is the format's dimension, and bbox_min /
 * bbox_max (3 floats each, may be NULL) bound the finite coordinates read. */
RTDBS_API int rtdbs_read_points(const char* path, int32_t format, int64_t n_max, float* xyz,
                                int64_t* n_read, int32_t* dim, float* bbox_min, float* bbox_max);

/* ------------------------------------------------------------------ pools
 * A pool slides many independent streams together: one launch per kernel
 * phase covers every stream of a round (each with its own W, S, dim, Eps,
 * MinPts and precision), and a round whose stream set repeats is one CUDA
 * graph replay.  The reference runs one stream per process; this is the
 * batched / serving extension of its slide loop.  Streams are admitted
 * against an HBM budget and can be added and removed between rounds. */

typedef struct rtdbs_pool rtdbs_pool;

typedef struct rtdbs_pool_params {
    int32_t device;            /* CUDA device ordinal */
    int32_t flags;             /* RTDBS_FLAG_NO_GRAPH: launch rounds directly */
    int32_t max_streams;       /* stream slots (default 1024) */
    int32_t reserved0;
    int64_t hbm_budget_bytes;  /* admission limit on the streams' device memory; 0 = none */
    int64_t reserved[6];
} rtdbs_pool_params;

typedef struct rtdbs_pool_stats {
    int64_t streams;           /* admitted streams */
    int64_t bytes_in_use;      /* device memory of the admitted streams */
    int64_t budget_bytes;
    int64_t rounds;            /* rounds launched */
    int64_t graph_replays;     /* rounds that replayed a cached graph */
    int32_t launches_per_round;
    int32_t reserved0;
    int64_t reserved[4];
} rtdbs_pool_stats;

/* Device bytes a stream with these parameters occupies (its admission cost). */
RTDBS_API int rtdbs_stream_bytes(const rtdbs_params* params, int64_t* bytes);
RTDBS_API int rtdbs_pool_params_init(rtdbs_pool_params* params);
RTDBS_API int rtdbs_pool_create(const rtdbs_pool_params* params, void* cuda_stream, rtdbs_pool** out);
RTDBS_API int rtdbs_pool_destroy(rtdbs_pool* pool);
/* Admits one stream (RTDBS_ERR_BUDGET when it does not fit); *stream_id is its slot. */
RTDBS_API int rtdbs_pool_add_stream(rtdbs_pool* pool, const rtdbs_params* params, int32_t* stream_id);
/* Frees the stream's slot and memory (waits for the pool's stream first). */
RTDBS_API int rtdbs_pool_remove_stream(rtdbs_pool* pool, int32_t stream_id);
RTDBS_API int rtdbs_pool_load_window(rtdbs_pool* pool, int32_t stream_id, const float* points,
                                     int points_on_device);
/* One round: each of the n listed (distinct, loaded) streams slides by its
 * stride.  d_points (device) holds their new points back to back in the
 * listed order, S_i * dim_i floats each.  Stream-ordered; results are then in
 * each stream's device buffers (rtdbs_pool_outputs). */
RTDBS_API int rtdbs_pool_slide(rtdbs_pool* pool, int32_t n, const int32_t* stream_ids,
                               const float* d_points);
/* rtdbs_pool_slide with every phase launched directly and bracketed by CUDA
 * events (chunk phases summed); synchronous. */
RTDBS_API int rtdbs_pool_slide_profiled(rtdbs_pool* pool, int32_t n, const int32_t* stream_ids,
                                        const float* d_points, rtdbs_phase_times* times);
/* The same round with each stream's new points in its own device buffer
 * (d_points_each[i] holds S_i * dim_i floats of stream_ids[i]); one gather
 * kernel packs them. */
RTDBS_API int rtdbs_pool_slide_each(rtdbs_pool* pool, int32_t n, const int32_t* stream_ids,
                                    const float* const* d_points_each);
/* Waits for the pool's stream; RTDBS_ERR_DEVICE if any stream hit a device bound. */
RTDBS_API int rtdbs_pool_sync(rtdbs_pool* pool);
RTDBS_API int rtdbs_pool_outputs(rtdbs_pool* pool, int32_t stream_id, int32_t** d_label,
                                 int32_t** d_cluster_id);
/* Copies one stream's latest label[W] and cluster_id[W] (host or device
 * memory per on_device); waits for the pool's stream. */
RTDBS_API int rtdbs_pool_read_outputs(rtdbs_pool* pool, int32_t stream_id, int32_t* label,
                                      int32_t* cluster_id, int on_device);
/* The stream's engine, for the per-engine queries (counts, stats, cluster). */
RTDBS_API int rtdbs_pool_engine(rtdbs_pool* pool, int32_t stream_id, rtdbs_engine** engine);
RTDBS_API int rtdbs_pool_get_stats(rtdbs_pool* pool, rtdbs_pool_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* RTDBS_H */
