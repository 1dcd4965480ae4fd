// rtdbs_internal.h -- device-side state layout shared by the kernels and the
// host engine of the streaming DBSCAN path.
//
// HBM layout of one stream (W slots, chunk C <= kChunkMax points):
//   ring   float4[W]      point of each ring slot (x, y, z, slot bits); the
//                         reference's params.window (src/dbscan/dbscan.h:23)
//   kslot  u64[W]         cell key of each slot (reference: point_cell_id)
//   skey   u64[2][W]      window sorted by (cell key, slot): keys
//   spt    float4[2][W]   ... points in that order (.w = slot as int bits)
//   scnt   i32[2][W]      ... exact neighbour count in that order
//                         (double-buffered; the reference's pos_arr/
//                         tmp_pos_arr, src/dbscan/grid.cpp:181-199)
//   table  {u64,u64}[2][P] open-addressed cell table: tagged key -> [start,end)
//                         (replaces the OptiX BVH, src/dbscan/optix.cpp:438-483)
//   items  int2[W+W/32+64] work list: runs of <= 32 sorted points of one cell
//   parent i32[W]         union-find forest by slot (reference: cluster_id)
//   sroot  i32[W]         per sorted position: root hint during the union, then
//                         the root (-1: not core)
//   label, cid i32[W]     outputs by slot
//   nlist  i32[W][stride] neighbour list of every non-core point by slot
//                         (cap = MinPts - 2 entries, rows padded to a multiple
//                         of 4 for 16-byte loads; -1 = empty entry)
//   rslot  i32[W]         per slot after the flatten: root (core) or -1
//   damaged i32[W]        per previous root: the component lost a core this slide
//   ntrack i32[W]         1: the slot's list is exact; 0: not kept (core, or
//                         rebuilt at the end of the slide)
//   sprev  i32[2][W]      per sorted position: the point's root at the last
//                         clustering (-1: not core), carried by the merges
//   chunk scratch: sort words, expired points.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rtdbs {

constexpr int kChunkMax = 16384;   // points per grid-update chunk
constexpr int kOffBits = 14;       // in-chunk offset bits of a sort word
constexpr int kKeyBitsMax = 50;    // cell-key bits (key << 14 | offset fits in 64 bits)
constexpr unsigned long long kKeyMask = (1ull << kKeyBitsMax) - 1ull;
constexpr unsigned kGenMod = 16383;  // table generations 1..16383 (tag = gen << 50 | key)
constexpr int kMergeTile = 1024;   // old entries per merge block
constexpr int kMergeThreads = 256;
constexpr int kSortRun = 1024;     // words per radix-sort CTA (one per thread)
constexpr int kBuildThreads = 512;
constexpr int kClusterThreads = 256;
constexpr int kBatch = 8;          // default work items a clustering warp takes at a time
                                   // in a pool launch
constexpr int kQueryLanes = 16;    // default lanes per query point in the count passes (one
                                   // cell per Eps: two points per warp overlap their loads)
constexpr int kMaxIter = 1 << 20;  // bound on every device-side retry loop
constexpr int kListCap = 30;       // longest neighbour list kept (MinPts <= 32)

// Bits of Ctl::err.
constexpr int kErrHashFull = 1;
constexpr int kErrUnionIter = 2;
constexpr int kErrItems = 4;
constexpr int kErrChunk = 8;
constexpr int kErrList = 16;

// Device-resident control block of one stream.  Every field that changes
// from slide to slide lives here (not in kernel arguments), so one captured
// CUDA graph replays every slide.
struct Ctl {
    long long b;               // grid builds so far (merge + table build)
    long long slide;           // slides completed
    int nocc[2];               // entries in sorted buffer 0 / 1
    int nitems;                // work items of the current grid
    int ncells;                // cells of the current grid
    int err;                   // kErr* bits
    int prev_ok;               // label/cid hold the clustering of the window before
                               // this slide's changes (the forest can be reused)
    int union_next;            // next work item handed out by k_union
    int label_next;            // next work item handed out by k_label
    unsigned long long band_rechecks;
    // counters of the reference's debug build (src/dbscan/dbscan.cpp:145-212):
    // [0] count passes (core identification), [1] clustering scans; spread over 8
    unsigned long long ptests[2][8];   // distance tests
    unsigned long long phits[2][8];    // ... that found a neighbour
    int qmax[8];                       // most distance tests of one count query
    int reused;                // cores that joined a reused component this slide
    int reuse_skip;            // slides left without forest reuse (it paid off too little)
    long long last_reused;     // `reused` of the last clustering
    long long reserved[1];
};

// Everything a kernel needs for one stream, passed by value.
struct View {
    // geometry: cell (i, j, k) = clamp(floor((x - origin) * inv_cell), 0, ext - 1),
    // key = i << shift[0] | j << shift[1] | k (bit fields, shift[2] = 0)
    double origin[3];
    double inv_cell;
    long long ext[3];
    int shift[3];
    int dim;
    int cell_mult;              // K: cells per Eps along each axis (1 or 2)
    int grab;                   // work items a clustering warp takes from the queue at a time
                                // (0: 8 in pool launches; for a large window slid alone 5
                                // or 8 by items per point, fewer on small ones)
    int qlanes;                 // lanes per query point in the count passes (16 or 32)
    // parameters
    int W, S, min_pts, units;   // units = W / S
    int chunk;                  // C
    int pbits;                  // log2 of table capacity
    unsigned pmask;
    float r2f;                  // FP32 mode: (float)eps * (float)eps
    float lo, hi;               // FP64 mode: FP32 filter band
    double E;                   // FP64 mode: eps * eps
    int filter_ok;              // FP64 mode: band valid (else every test in FP64)
    int key_bits;
    int sort_passes;
    int max_items;
    int item_pts;               // most points of a work item slid alone (8 or 32; 0 = 32; pool
                                // launches take 32): small windows take short items, so
                                // dense cells spread over more warps
    int precision;              // RTDBS_PREC_* (batched launches dispatch on it)
    int list_cap;               // entries per neighbour list; -1: no lists (the
                                // label pass then scans the grid)
    int list_stride;            // ints per list row (list_cap rounded up to 4)
    // buffers
    float4* ring;
    unsigned long long* kslot;
    unsigned long long* skey[2];
    float4* spt[2];
    int* scnt[2];
    ulonglong2* table[2];
    int2* items;
    int* parent;
    int* sroot;                  // per sorted position: root hint during the union
                                 // (-1: not core), then the root (-1: not core)
    int* label;
    int* cid;
    int* nlist;                  // [W][list_stride] neighbours of non-core points
    int* rslot;                  // per slot: root of a core, -1 otherwise
    int* damaged;                // per old root slot: its component lost a core this
                                 // slide (0 outside the union phase)
    int* ntrack;                 // per slot: 1 list exact, 0 not kept
    int* sprev[2];               // per sorted position (with the sorted buffers): the
                                 // point's root at the last clustering, -1 if it was not
                                 // core (or not there); carried by the merges for forest
                                 // reuse; null without neighbour lists
    unsigned long long* nsort;   // chunk sort words in (key << 14 | offset)
    unsigned long long* xsort;
    unsigned long long* nword;   // sorted
    unsigned long long* xword;
    float4* xpt;                 // expired points of the chunk by offset
    int* sorder;                 // per slot el + r: offset (slot - el) of the chunk's r-th
                                 // point in (key, slot) order, kept from the slide that
                                 // brought the chunk in; null: not kept
    const float* staging;        // new points [S][dim]
    Ctl* ctl;
};

// Combined template code of a stream's work kernels: dim + 4 (cells per Eps - 1).
__host__ __device__ inline int dk_of(const View& v) { return v.dim + 4 * (v.cell_mult - 1); }

// Kernel phases of a slide, in launch order.
enum Phase : int {
    kPhaseIngest = 0,
    kPhaseSort,
    kPhaseDecrement,
    kPhaseMerge,
    kPhaseBuild,
    kPhaseIncrement,
    kPhaseUnion,
    kPhaseFlatten,
    kPhaseLabel,
    kNumPhases
};
constexpr int kChunkPhases = 6;  // ingest .. increment, once per chunk

// Launchers (rtdbs_kernels.cu).  j = chunk index within the slide (or the
// load), c = points in the chunk, init = 1 while loading the first window,
// advance = 1 when the label phase ends a slide.
cudaError_t launch_phase(int phase, const View& v, int precision, int j, int c, int init,
                         int staging_offset, int advance, cudaStream_t s);
// With a side stream and two events, the decrement pass (which needs only
// the ingest) runs on `side` beside the sort, joined before the merge.
cudaError_t launch_chunk_step(const View& v, int precision, int j, int c, int init,
                              int staging_offset, cudaStream_t s, cudaStream_t side = nullptr,
                              cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);
// fresh_hints: start the union from fresh hints and forest (no reuse), for a
// clustering of the window as it stands rather than after a slide.
// outputs_free: an event the label pass (which rewrites label/cid) waits for
// first, with wait_flags (cudaEventWaitExternal inside a stream capture).
cudaError_t launch_cluster(const View& v, int precision, int advance, cudaStream_t s, bool fresh_hints = false,
                           cudaEvent_t outputs_free = nullptr, unsigned wait_flags = 0);
cudaError_t launch_counts_by_slot(const View& v, int* nn_by_slot, cudaStream_t s);
cudaError_t configure_kernels();

// Host helpers shared by the engine and the allocation-free entry point
// (rtdbs_engine.cpp).
// Records the text rtdbs_last_error returns on this thread; returns status.
int set_error(int status, const char* fmt, ...);
// FP32 filter band of the FP64 predicate and the FP32 radius (View::lo, hi,
// E, filter_ok, r2f) for this Eps.
void set_band(View& v, double eps);
// Grid geometry of View v (origin, extents, key fields, inv_cell, key_bits,
// sort_passes) for cells of side Eps (1 + 2^-12) / cells_per_eps over the
// box [bmin, bmax] of `dim` axes, widened by 25% (and at least 4 cells) when
// `widen`; the cell side doubles until the key fits kKeyBitsMax bits.
// Returns RTDBS_OK or RTDBS_ERR_INVALID (empty or non-finite box); the side
// used goes to *cell_side.
int set_geometry(View& v, int dim, double eps, int cells_per_eps, const float* bmin, const float* bmax,
                 bool widen, double* cell_side);

// ------------------------------------------------------------ batched launches
// One launch of a phase covers many streams: block b belongs to the item i
// with prefix[i] <= b < prefix[i+1] and runs that stream's kernel body with
// block index b - prefix[i] of prefix[i+1] - prefix[i].

enum BatchPhase : int {
    kBatchIngest = 0,
    kBatchSort,
    kBatchRunmerge,
    kBatchDecrement,
    kBatchMerge,
    kBatchBuild,
    kBatchIncrement,
    kBatchDamage,
    kBatchReuse,
    kBatchUnion,
    kBatchFlatten,
    kBatchLabel,
    kNumBatchPhases
};
constexpr int kBatchChunkPhases = 7;  // ingest .. increment

struct BatchItem {
    int view;            // index into the View array
    int j;               // chunk index within the slide
    int c;               // points in the chunk
    int stg_off;         // offset of the chunk within the stream's new points
    const float* input;  // the stream's new points of this slide (device)
};

struct BatchLaunch {
    const View* views;
    const BatchItem* items;
    const int* prefix;   // n + 1 entries
    int n;
};

// Blocks one item needs in a phase (same shapes as the single-stream launches).
int batch_blocks(int phase, const View& v, int c);
int batch_threads(int phase);
// Phases launched once per (precision, dim) group of streams (the others
// take every stream in one launch; prec and dim are then ignored).
// `dim` here is the stream group's dk_of code (dimension and cells per Eps).
bool batch_phase_split(int phase);
cudaError_t launch_batch(int phase, int prec, int dim, const BatchLaunch& L, int total_blocks, int max_c,
                         cudaStream_t s);
// Packs n device arrays (count[i] floats from src[i]) into dst at dst_off[i];
// the three tables are device memory.
cudaError_t launch_gather(const float* const* src, const long long* dst_off, const int* count, float* dst,
                          int n, int max_count, cudaStream_t s);

}  // namespace rtdbs
