// rtdbs_kernels.cu -- sm_103a kernels of the per-slide streaming DBSCAN path.
//
// One slide = ceil(S / C) grid-update chunk steps followed by one clustering
// step (reference level-9 loop, src/dbscan/dbscan.cpp:2276-2362):
//
//   chunk step (C <= 16384 new points replacing the points of the same slots)
//     k_ingest  new points -> ring slots + cell keys; expired points saved
//               (reference: H2D 2289 + compute_cell_id, src/dbscan/aabb.cu:589-610)
//     k_sort    LSD radix sort of the new and of the expired (cell key, slot)
//               words in runs of 1024, one CTA per run, then k_runmerge
//               ranks the runs into one list (reference: sortByCellIdAndOrder,
//               src/dbscan/thrust_helper.cu:21-29); expired words whose order
//               was kept from their arrival are gathered instead of sorted
//     k_decr    exact -1 on the neighbour counts of every survivor within Eps
//               of an expired point, on the old grid, beside the sort
//     k_merge   old sorted window minus expired plus new, one pass, merge-path
//               tiles (reference: merge_by_cell_id_and_idx,
//               src/dbscan/thrust_helper.cu:31-51)
//     k_build   cell table (tagged open addressing) + work list of cell runs
//               (replaces compute_offsets_of_cells / set_hybrid_spheres_info /
//               optixAccelBuild, src/dbscan/aabb.cu:377-544,
//               src/dbscan/optix.cpp:438-483)
//     k_incr    full count of every new point and exact +1 on its neighbours
//               on the new grid (reference: __raygen__grid/__intersection__grid,
//               src/dbscan/dbscan.cu:155-194,250-270, which recounts all W)
//   clustering step
//     k_union   union-find over core-core pairs, each unordered pair once
//               (reference: __raygen__cluster/__intersection__hybrid_radius_sphere,
//               src/dbscan/dbscan.cu:279-321,354-394; find_repres/unite 9-43)
//     k_label   labels and ids by slot; border = minimum id of the adjacent
//               clusters (reference: set_label_kernel + post_cluster_t,
//               src/dbscan/aabb.cu:173-196,575-587)
//
// Neighbour predicate: a warp holds 32 candidates in lanes (coalesced float4
// loads of the cell-sorted window) and tests them against home points
// broadcast by shuffle.  Squared distances use explicitly rounded IEEE
// operations (no FMA contraction; the count passes evaluate two candidates'
// differences and squares with paired FP32 instructions, each half rounded
// the same way), so FP32 mode is bit-identical to the reference's CPU checker
// (src/dbscan/util.cpp:308-316).
#include "rtdbs_internal.h"

#include <atomic>
#include <climits>
#include <cstdint>

namespace rtdbs {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kPrecFp64 = 0;
constexpr int kPrecFp32 = 1;

__device__ __forceinline__ int slot_of(const float4& p) { return __float_as_int(p.w); }


__device__ __forceinline__ unsigned lanemask_lt(int lane) { return (1u << lane) - 1u; }

// ------------------------------------------------------------------ geometry

__device__ __forceinline__ unsigned long long cell_key(const View& v, float x, float y, float z) {
    const float q[3] = {x, y, z};
    unsigned long long key = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        long long c = 0;
        if (a < v.dim) {
            double t = floor(((double)q[a] - v.origin[a]) * v.inv_cell);
            if (!(t >= 0.0)) t = 0.0;  // also maps NaN to cell 0
            const double top = (double)(v.ext[a] - 1);
            if (t > top) t = top;
            c = (long long)t;
        }
        key |= (unsigned long long)c << v.shift[a];
    }
    return key;
}

__device__ __forceinline__ unsigned gen_of_build(long long b) {
    return (unsigned)((b >> 1) % (long long)kGenMod) + 1u;
}

__device__ __forceinline__ int chunk_base_slot(const View& v, int j, int init) {
    const int base = init ? 0 : (int)(v.ctl->slide % v.units) * v.S;
    return base + j * v.chunk;
}

// The expiring chunk's (key, slot) order is known from the slide that
// brought it in (sorder), so its words need no sort: true once every slot of
// the window arrived by a slide (the first window's load chunks tile the
// slots differently).  Keys do not change while a point is in the window.
__device__ __forceinline__ bool expired_presorted(const View& v, int init) {
    return !init && v.sorder != nullptr && v.ctl->slide >= (long long)v.units;
}

// ----------------------------------------------------------------- predicate

template <int DIM>
__device__ __forceinline__ float sqdist32(const float4& a, const float4& b) {
    const float dx = __fsub_rn(a.x, b.x);
    float d = __fmul_rn(dx, dx);
    if (DIM > 1) {
        const float dy = __fsub_rn(a.y, b.y);
        d = __fadd_rn(d, __fmul_rn(dy, dy));
    }
    if (DIM > 2) {
        const float dz = __fsub_rn(a.z, b.z);
        d = __fadd_rn(d, __fmul_rn(dz, dz));
    }
    return d;
}

template <int DIM>
__device__ __forceinline__ double sqdist64(const float4& a, const float4& b) {
    const double dx = __dsub_rn((double)a.x, (double)b.x);
    double d = __dmul_rn(dx, dx);
    if (DIM > 1) {
        const double dy = __dsub_rn((double)a.y, (double)b.y);
        d = __dadd_rn(d, __dmul_rn(dy, dy));
    }
    if (DIM > 2) {
        const double dz = __dsub_rn((double)a.z, (double)b.z);
        d = __dadd_rn(d, __dmul_rn(dz, dz));
    }
    return d;
}

// Neighbour test of two distinct points.  FP32 mode: the reference predicate
// d32 < r2f.  FP64 mode: d32 < lo and d32 >= hi are decided by the float
// value (the band [lo, hi) around Eps^2 bounds the float evaluation's
// rounding error, see oracle_band); everything else in double.
// Per-thread counters: distance tests, those re-decided in FP64, and those
// that found a neighbour.
struct Tally {
    unsigned tests = 0;
    unsigned rechecks = 0;
    unsigned hits = 0;
};

// The decision on d = sqdist32(a, b).
template <int MODE, int DIM>
__device__ __forceinline__ bool nbr_decide(const View& v, float d, const float4& a, const float4& b, Tally& t) {
    ++t.tests;
    bool nb;
    if (MODE == kPrecFp32) {
        nb = d < v.r2f;
    } else if (v.filter_ok && d < v.lo) {
        nb = true;
    } else if (v.filter_ok && d >= v.hi) {
        nb = false;
    } else {
        ++t.rechecks;
        nb = sqdist64<DIM>(a, b) < v.E;
    }
    t.hits += nb ? 1u : 0u;
    return nb;
}

template <int MODE, int DIM>
__device__ __forceinline__ bool is_nbr(const View& v, const float4& a, const float4& b, Tally& t) {
    return nbr_decide<MODE, DIM>(v, sqdist32<DIM>(a, b), a, b, t);
}

// sqdist32(a, b0) and sqdist32(a, b1) at once: the differences and squares
// with paired FP32 instructions (Blackwell f32x2, each half an IEEE single
// operation rounded to nearest), the sums in scalar, in the same order as
// sqdist32, so both results are bit-identical to it.  (Paired sums are not
// used: the paired multiply-then-add did not round like the two separate
// scalar operations.)
__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}

__device__ __forceinline__ void sq_diff2(float a, float b0, float b1, float& s0, float& s1) {
    unsigned long long t, m;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(t) : "l"(pack2(a, a)), "l"(pack2(b0, b1)));
    asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(m) : "l"(t));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(s0), "=f"(s1) : "l"(m));
}

template <int DIM>
__device__ __forceinline__ void sqdist32x2(const float4& a, const float4& b0, const float4& b1, float& d0,
                                           float& d1) {
    sq_diff2(a.x, b0.x, b1.x, d0, d1);
    if (DIM > 1) {
        float y0, y1;
        sq_diff2(a.y, b0.y, b1.y, y0, y1);
        d0 = __fadd_rn(d0, y0);
        d1 = __fadd_rn(d1, y1);
    }
    if (DIM > 2) {
        float z0, z1;
        sq_diff2(a.z, b0.z, b1.z, z0, z1);
        d0 = __fadd_rn(d0, z0);
        d1 = __fadd_rn(d1, z1);
    }
}

// ---------------------------------------------------------------- cell table

// Home slot of a cell key: the key folded to 32 bits, then Fibonacci
// hashing (pbits <= 31); keys below 2^32 fold to themselves, so the stencil
// lookups of small grids hash in 32-bit arithmetic (table_home32).
__device__ __forceinline__ unsigned table_home32(unsigned key, int pbits) {
    return (key * 0x9E3779B1u) >> (32 - pbits);
}

__device__ __forceinline__ unsigned table_home(unsigned long long key, int pbits) {
    return table_home32((unsigned)key ^ (unsigned)(key >> 32), pbits);
}

__device__ __forceinline__ unsigned long long tag_of(unsigned long long key, unsigned gen) {
    return ((unsigned long long)gen << kKeyBitsMax) | key;
}

// [start, end) of a cell, (0, 0) if the cell is empty in this generation;
// `home` is the key's home slot.
__device__ __forceinline__ int2 table_find_at(const ulonglong2* T, unsigned pmask, unsigned home,
                                              unsigned long long tag) {
    unsigned s = home;
    const unsigned long long gen = tag >> kKeyBitsMax;
    for (unsigned i = 0; i <= pmask; ++i) {
        const ulonglong2 e = T[s];
        if (e.x == tag) return make_int2((int)(unsigned)e.y, (int)(unsigned)(e.y >> 32));
        if ((e.x >> kKeyBitsMax) != gen) break;  // empty or stale slot ends the probe
        s = (s + 1) & pmask;
    }
    return make_int2(0, 0);
}

__device__ __forceinline__ int2 table_find(const ulonglong2* T, unsigned pmask, int pbits,
                                           unsigned long long tag) {
    return table_find_at(T, pmask, table_home(tag & kKeyMask, pbits), tag);
}

// Claims (or finds) the slot of `tag` and stores one half of its range:
// which = 0 -> start, 1 -> end, 2 -> both (value = start, value2 = end).
// Entries of older generations count as free.
__device__ bool table_set(ulonglong2* T, unsigned pmask, int pbits, unsigned long long tag,
                          int which, int value, int value2 = 0) {
    unsigned s = table_home(tag & kKeyMask, pbits);
    const unsigned long long gen = tag >> kKeyBitsMax;
    for (unsigned i = 0; i <= pmask; ++i) {
        unsigned long long* kp = reinterpret_cast<unsigned long long*>(&T[s].x);
        unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(kp);
        for (int t = 0; t < 8; ++t) {
            bool mine = cur == tag;
            if (!mine) {
                if ((cur >> kKeyBitsMax) == gen) break;  // another cell of this generation
                const unsigned long long prev = atomicCAS(kp, cur, tag);
                mine = prev == cur;
                cur = prev;
            }
            if (mine) {
                if (which == 2)
                    T[s].y = (unsigned long long)(unsigned)value | ((unsigned long long)(unsigned)value2 << 32);
                else
                    reinterpret_cast<int*>(&T[s].y)[which] = value;
                return true;
            }
        }
        s = (s + 1) & pmask;
    }
    return false;
}

// Rows of the stencil.  With K cells per Eps along each axis (cell side
// Eps (1 + 2^-12) / K) a point's neighbours lie within K cells per axis, in
// the (2K+1)^DIM cells around its own.  The 2K+1 cells of one row (last axis
// -K..K) have consecutive keys, so a row is one contiguous range of the
// cell-sorted window; the full stencil has (2K+1)^(DIM-1) rows.  The upper
// half (HALF) keeps only the rows whose keys are not below the home cell's --
// the centre row (without its negative cells) and the rows after it in key
// order -- since every position below the home cell is clipped away by a
// pair-once union anyway.
//
// The work kernels take a combined template parameter DK = DIM + 4 (K - 1):
// DK 1..3 for one cell per Eps, 5..7 for two.
template <int DIM, bool HALF, int K = 1>
struct Stencil {
    static constexpr int kW = 2 * K + 1;  // cells per row
    static constexpr int kAllRows = DIM == 1 ? 1 : (DIM == 2 ? kW : kW * kW);
    static constexpr int kFirst = HALF ? (kAllRows - 1) / 2 : 0;  // first row kept
    static constexpr int kRows = kAllRows - kFirst;
};
constexpr int kMaxRows = 25;  // (2K+1)^2 rows for K = 2 in 3-D

// Row ranges of the stencil around `key`, computed by a group of G lanes
// (the whole warp, or each 16-lane half for its own key; `lane` counts within
// the group; a lane looks up one to four cells).  On return group lane
// r < kRows holds row r as [rs, re) (empty rows: rs == re).
template <int DIM, bool HALF, int K = 1, int G = 32>
__device__ __forceinline__ void row_ranges(const View& v, const ulonglong2* T, unsigned gen,
                                           unsigned long long key, int lane, int& rs, int& re) {
    using St = Stencil<DIM, HALF, K>;
    constexpr int kW = St::kW;
    constexpr int kSlots = kW * St::kRows;           // cell slots, kept row by kept row
    constexpr int kPer = (kSlots + G - 1) / G;       // cells per lane
    static_assert(kPer <= 4 && St::kRows <= G, "stencil too large for the lane group");
    int2 rg[kPer];
    if (v.key_bits <= 31) {
        // keys, cell coordinates and extents fit 32 bits: the lookups in
        // 32-bit arithmetic (coordinates wrap below zero, so one unsigned
        // comparison bounds each axis)
        const unsigned k32 = (unsigned)key;
        const int s0 = v.shift[0], s1 = v.shift[1];
        const unsigned c2 = k32 & ((1u << s1) - 1u);
        const unsigned c1 = (k32 >> s1) & ((1u << (s0 - s1)) - 1u);
        const unsigned c0 = k32 >> s0;
        const unsigned e0 = (unsigned)v.ext[0], e1 = (unsigned)v.ext[1], e2 = (unsigned)v.ext[2];
        const unsigned long long gtag = (unsigned long long)gen << kKeyBitsMax;
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            rg[k] = make_int2(0, 0);
            const int cs = lane + k * G;
            const int row = St::kFirst + cs / kW, d_last = cs % kW - K;
            const bool skip = HALF && cs < kW && d_last < 0;
            if (cs < kSlots && !skip) {
                unsigned q0 = c0, q1 = c1, q2 = c2;
                if (DIM == 1) {
                    q0 += (unsigned)d_last;
                } else if (DIM == 2) {
                    q0 += (unsigned)(row - K);
                    q1 += (unsigned)d_last;
                } else {
                    q0 += (unsigned)(row / kW - K);
                    q1 += (unsigned)(row % kW - K);
                    q2 += (unsigned)d_last;
                }
                if (q0 < e0 && q1 < e1 && q2 < e2) {
                    const unsigned nk = (q0 << s0) | (q1 << s1) | q2;
                    rg[k] = table_find_at(T, v.pmask, table_home32(nk, v.pbits), gtag | nk);
                }
            }
        }
    } else {
    const long long c2 = (long long)(key & ((1ull << v.shift[1]) - 1ull));
    const long long c1 = (long long)((key >> v.shift[1]) & ((1ull << (v.shift[0] - v.shift[1])) - 1ull));
    const long long c0 = (long long)(key >> v.shift[0]);
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        rg[k] = make_int2(0, 0);
        const int cs = lane + k * G;                                  // = kW * kept row + cell
        const int row = St::kFirst + cs / kW, d_last = cs % kW - K;
        const bool skip = HALF && cs < kW && d_last < 0;             // centre row, negative cells
        if (cs < kSlots && !skip) {
            long long q0 = c0, q1 = c1, q2 = c2;
            if (DIM == 1) {
                q0 += d_last;
            } else if (DIM == 2) {
                q0 += row - K;
                q1 += d_last;
            } else {
                q0 += row / kW - K;
                q1 += row % kW - K;
                q2 += d_last;
            }
            const bool ok = q0 >= 0 && q0 < v.ext[0] && q1 >= 0 && q1 < v.ext[1] && q2 >= 0 && q2 < v.ext[2];
            if (ok) {
                const unsigned long long nk = ((unsigned long long)q0 << v.shift[0]) |
                                              ((unsigned long long)q1 << v.shift[1]) | (unsigned long long)q2;
                rg[k] = table_find(T, v.pmask, v.pbits, tag_of(nk, gen));
            }
        }
    }
    }
    int s = INT_MAX, e = INT_MIN;
#pragma unroll
    for (int k = 0; k < kW; ++k) {
        const int cs = min(kW * lane + k, kSlots - 1);   // slot of row `lane`'s cell k
        const int src = cs % G, which = cs / G;
        int a = 0, b = 0;
#pragma unroll
        for (int w = 0; w < kPer; ++w) {
            const int aw = __shfl_sync(kFull, rg[w].x, src, G);
            const int bw = __shfl_sync(kFull, rg[w].y, src, G);
            if (w == which) {
                a = aw;
                b = bw;
            }
        }
        if (b > a) {
            s = min(s, a);
            e = max(e, b);
        }
    }
    if (e == INT_MIN) s = e = 0;
    rs = s;
    re = e;
}

// The group's row ranges (group lanes 0..ROWS-1), clipped below at `lo`,
// laid end to end: candidate idx in [0, total) lives at sorted position
// start[r] + idx - pre[r] for the row r with pre[r] <= idx < pre[r+1].
// Concatenating the rows keeps the candidate chunks full.  Called by the
// whole warp; G-lane groups work independently.
template <int ROWS, int G = 32>
__device__ __forceinline__ int candidate_stream(int rs, int re, int lo, int lane, int* sstart,
                                                int* spre) {
    const int a = max(rs, lo);
    const int len = lane < ROWS ? max(re - a, 0) : 0;
    int incl = len;
#pragma unroll
    for (int o = 1; o < (ROWS > 16 ? 32 : 16); o <<= 1) {
        const int t = __shfl_up_sync(kFull, incl, o, G);
        if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(kFull, incl, ROWS - 1, G);
    __syncwarp();
    if (lane < ROWS) {
        sstart[lane] = a;
        spre[lane] = incl - len;
    }
    if (lane == 0) spre[ROWS] = total;
    __syncwarp();
    return total;
}

// Sorted position of candidate idx; r is the lane's row cursor (rows only
// advance as idx grows).
__device__ __forceinline__ int stream_pos(int idx, int& r, const int* sstart, const int* spre) {
    while (idx >= spre[r + 1]) ++r;
    return sstart[r] + idx - spre[r];
}

// ---------------------------------------------------------------- union-find

// Root of v with intermediate pointer jumping (each visited node is pointed
// at its grandparent).  Parents only ever decrease, so the walk terminates.
__device__ __forceinline__ int uf_find(int* parent, int v) {
    volatile int* P = parent;
    int curr = P[v];
    if (curr != v) {
        int next, prev = v;
        while (curr > (next = P[curr])) {
            P[prev] = next;
            prev = curr;
            curr = next;
        }
    }
    return curr;
}

// Lock-free union of the sets of a and b, each an ancestor of one of the two
// points (a cached or freshly found root; it need not still be a root).  The
// larger of the two is hooked under the smaller with one atomicCAS, which only
// succeeds on a root; on failure the walk resumes from the root that the CAS
// revealed.  max(a, b) falls every round, so the loop ends, and parents only
// ever point to smaller slots, so every root is the minimum slot of its set.
// Returns an ancestor of both points afterwards.
__device__ __forceinline__ int uf_hook(int* parent, int a, int b, int& err) {
    for (int it = 0; it < kMaxIter; ++it) {
        if (a == b) return a;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicCAS(&parent[a], a, b);
        if (old == a) return b;
        a = uf_find(parent, old);
    }
    err |= kErrUnionIter;
    return a < b ? a : b;
}

// Warp totals of the counters into the control block; pass 0 = count passes
// (core identification), 1 = clustering scans.
__device__ __forceinline__ void flush_stats(const View& v, const Tally& t, int err, int lane, int pass) {
    const unsigned r = __reduce_add_sync(kFull, t.rechecks);
    const unsigned n = __reduce_add_sync(kFull, t.tests);
    const unsigned h = __reduce_add_sync(kFull, t.hits);
    const int e = __reduce_or_sync(kFull, (unsigned)err);
    if (lane == 0) {
        const int k = (threadIdx.x >> 5) & 7;
        if (r) atomicAdd(&v.ctl->band_rechecks, (unsigned long long)r);
        if (n) atomicAdd(&v.ctl->ptests[pass][k], (unsigned long long)n);
        if (h) atomicAdd(&v.ctl->phits[pass][k], (unsigned long long)h);
        if (e) atomicOr(&v.ctl->err, e);
    }
}

// Most distance tests of one query over the warp's lane groups of G lanes
// (each lane's `tests` counts its own query only) into Ctl::qmax.
template <int G>
__device__ __forceinline__ void flush_query_max(const View& v, unsigned tests, int lane) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) tests += __shfl_xor_sync(kFull, tests, o);
#pragma unroll
    for (int o = G; o < 32; o <<= 1) tests = max(tests, __shfl_xor_sync(kFull, tests, o));
    if (lane == 0 && tests) atomicMax(&v.ctl->qmax[(threadIdx.x >> 5) & 7], (int)tests);
}

// ------------------------------------------------------- neighbour lists
// Every non-core point keeps the slots of its neighbours (at most MinPts - 2
// besides itself) in a fixed list by slot, maintained from the same distance
// tests that keep the counts exact: an expired neighbour is removed in the
// decrement pass, a new one appended in the increment pass.  A point that
// becomes core stops keeping its list (ntrack 0); one that is below MinPts
// without a list once the slide's counts are final (it lost core status) gets
// its list rebuilt by one scan.  The label pass then reads lists instead of
// scanning the grid.

// First index of `x` among the four entries of e (base: index of e.x), or -1.
__device__ __forceinline__ int find4(const int4& e, int x, int base) {
    return e.x == x ? base : e.y == x ? base + 1 : e.z == x ? base + 2 : e.w == x ? base + 3 : -1;
}

// Appends slot p to q's list (q tracked); a full list means q has reached
// MinPts, so it stops being kept.  A list row is read 16 bytes at a time
// from L2 (other SMs may have just written it).  The append claims the first
// free entry by CAS and looks again if another point took it first; a row
// still contended after a few looks also stops being kept (the flatten pass
// rebuilds it).  Padding entries past the cap stay -1 and are never claimed.
__device__ __forceinline__ void list_append(const View& v, int q, int p) {
    int* L = v.nlist + (size_t)q * v.list_stride;
    const int4* L4 = reinterpret_cast<const int4*>(L);
    const int n4 = v.list_stride >> 2;
    for (int look = 0; look < 4; ++look) {
        int k = -1;
        for (int b = 0; b < n4 && k < 0; ++b) k = find4(__ldcg(L4 + b), -1, 4 * b);
        if (k < 0 || k >= v.list_cap) break;
        if (atomicCAS(&L[k], -1, p) == -1) return;
    }
    v.ntrack[q] = 0;
}

// Removes slot p from q's list (q tracked; only this thread removes p).
__device__ __forceinline__ void list_remove(const View& v, int q, int p) {
    int* L = v.nlist + (size_t)q * v.list_stride;
    const int4* L4 = reinterpret_cast<const int4*>(L);
    const int n4 = v.list_stride >> 2;
    for (int b = 0; b < n4; ++b) {
        const int k = find4(__ldcg(L4 + b), p, 4 * b);
        if (k >= 0) {
            L[k] = -1;
            return;
        }
    }
    atomicOr(&v.ctl->err, kErrList);
}

// Called by the whole warp; each group of G lanes (gl = lane within the
// group) adds its lanes' neighbour slots (nb) to its own buffer in lane
// order; returns the group's new number found (entries past cap are
// dropped, the list is then not kept anyway).
template <int G = 32>
__device__ __forceinline__ int list_collect(bool nb, int qs, int nfound, int cap, int* buf, int lane) {
    const unsigned all = __ballot_sync(kFull, nb);
    const int gl = lane & (G - 1);
    const unsigned m = G == 32 ? all : (all >> (lane - gl)) & ((1u << G) - 1u);
    const int at = nfound + __popc(m & lanemask_lt(gl));
    if (nb && at < cap) buf[at] = qs;
    return nfound + __popc(m);
}

// Called by the whole warp; a group with a point (`has`) writes slot a's
// list from its buffer (kept iff a is not core); the row's padding past
// list_cap stays -1.
template <int G = 32>
__device__ __forceinline__ void list_store(const View& v, int a, int nfound, const int* buf, int lane,
                                           bool has = true) {
    __syncwarp();
    const int gl = lane & (G - 1);
    if (has) {
        const bool keep = nfound + 1 < v.min_pts;
        int* L = v.nlist + (size_t)a * v.list_stride;
        if (keep)
            for (int k = gl; k < v.list_stride; k += G) L[k] = k < nfound ? buf[k] : -1;
        if (gl == 0) v.ntrack[a] = keep ? 1 : 0;
    }
    __syncwarp();
}

// ------------------------------------------------------------------- kernels

// ------------------------------------------------------ forest reuse
// A component of the previous clustering that lost no core this slide (no
// core expired, no core fell below MinPts) is still connected: all its
// cores and the edges between them remain.  Its cores start the union as
// one set under the old root (still its minimum slot), with that root as
// their hint, so pairs inside it are skipped by hint equality; every other
// core starts as a singleton.  The union still visits every core pair, so
// merges through new cores and splits of damaged components come out exactly
// as in a union from scratch.  Used with neighbour lists, where k_border
// leaves the previous labels and ids by slot and resets the forest.
//
// No pass of its own: the old root of every core lost this slide is marked
// damaged as the loss happens -- an expired core in the ingest, a core whose
// count falls below MinPts in the decrement (a count that falls below and
// rises again within the slide only marks a component that did not need it;
// it is then re-united from scratch, still exactly) -- and the merge, which
// rewrites every position, starts each core under its old root or alone
// (start_hint); the increment then sets the hints of new points and of points
// it lifts to MinPts.  label/cid hold the previous clustering until the
// border pass ends the slide.

// Reuse is skipped for 15 slides after a slide where fewer than 1 in 16 of
// the window's points joined a reused component (streams whose expiries
// touch every cluster), then tried again.
constexpr int kReuseRetry = 15;

__device__ __forceinline__ bool damage_on(const View& v) {
    return v.list_cap >= 0 && v.ctl->prev_ok && v.ctl->reuse_skip <= 0;
}

// The slide's new slots: [base, base + S).
__device__ __forceinline__ bool slot_is_new(const View& v, int s) {
    const int base = (int)(v.ctl->slide % v.units) * v.S;
    return s >= base && s < base + v.S;
}

// Root hint a position starts the union with: -1 for a non-core point; the
// old root `prev` of a core of an intact component (the root the point had
// at the last clustering, carried with it by the merges; -1 for a point that
// was not core then); else its own slot.  Counts 1 in `reused` for a
// reused core.  The parents need no change: the union and the flatten only
// ever start from a point's hint, and the border pass leaves every parent at
// its own slot.
__device__ __forceinline__ int start_hint(const View& v, int s, int cnt, int prev, bool reuse,
                                          unsigned& reused) {
    if (cnt < v.min_pts) return -1;
    if (reuse && prev >= 0 && !v.damaged[prev]) {
        ++reused;
        return prev;
    }
    return s;
}

__device__ __forceinline__ void mark_damage(const View& v, int slot) {
    if (v.label[slot] == 0) v.damaged[v.cid[slot]] = 1;
}

// New points of chunk j -> ring slots [el, el+c): float4 + cell key; the
// points they replace are kept for the decrement pass.
__device__ __forceinline__ void ingest_body(const View& v, int j, int c, int init, int stg_off,
                                            const float* input, int bx) {
    if (bx == 0 && threadIdx.x == 0) v.ctl->b += 1;  // no reader in this kernel
    const int k = bx * blockDim.x + threadIdx.x;
    if (k >= c) return;
    const int slot = chunk_base_slot(v, j, init) + k;
    if (!init) {
        v.xpt[k] = v.ring[slot];
        v.xsort[k] = (v.kslot[slot] << kOffBits) | (unsigned long long)k;
        if (damage_on(v)) mark_damage(v, slot);  // an expired core
    }
    const float* p = input + (size_t)(stg_off + k) * v.dim;
    const float x = p[0];
    const float y = v.dim > 1 ? p[1] : 0.0f;
    const float z = v.dim > 2 ? p[2] : 0.0f;
    v.ring[slot] = make_float4(x, y, z, __int_as_float(slot));
    const unsigned long long key = cell_key(v, x, y, z);
    v.kslot[slot] = key;
    v.nsort[k] = (key << kOffBits) | (unsigned long long)k;
}

__global__ void k_ingest(View v, int j, int c, int init, int stg_off) {
    ingest_body(v, j, c, init, stg_off, v.staging, blockIdx.x);
}

// Exclusive scan of one value per thread over a 1024-thread block.
__device__ __forceinline__ unsigned block_excl_scan_1024(unsigned val, unsigned* wsum) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned incl = val;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        const unsigned x = wsum[lane];
        unsigned xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(kFull, xi, o);
            if (lane >= o) xi += t;
        }
        wsum[lane] = xi - x;
    }
    __syncthreads();
    const unsigned r = wsum[w] + incl - val;
    __syncthreads();
    return r;
}

// Stable LSD radix sort (8-bit digits over the key bits of the sort word) of
// the chunk's words in independent runs of kSortRun: block (r, 0) sorts run r
// of the new words, block (r, 1) run r of the expired ones, one word per
// thread.  Warp-level multisplit: lanes with equal digits are ranked from
// eight ballots; per-(digit, warp) counters are scanned in digit-major order
// so the order of equal digits is the item order.  The merge consumes the
// sorted runs directly.
struct SortSmem {
    unsigned long long buf[kSortRun];
    unsigned whist[256 * 32];
    unsigned wsum[32];
};

// single: the chunk is one run (c <= kSortRun), so the sorted run is the
// final list: it goes straight to nword / xword (and presorted expired words
// are gathered here), and no run merge follows.
__device__ __forceinline__ void sort_body(const View& v, int j, int c, int init, int bx, int by, SortSmem& sm,
                                          bool single) {
    unsigned long long* buf = sm.buf;
    unsigned* whist = sm.whist;
    unsigned* wsum = sm.wsum;
    const int which = by;
    if (which == 1 && init) return;
    if (which == 1 && expired_presorted(v, init)) {
        if (single) {  // the run merge's gather of the kept order
            const int i = threadIdx.x;
            if (i >= c) return;
            const int k = v.sorder[chunk_base_slot(v, j, 0) + i];
            if (k < 0 || k >= c) {
                atomicOr(&v.ctl->err, kErrChunk);
                v.xword[i] = ~0ull;
                return;
            }
            v.xword[i] = v.xsort[k];
        }
        return;
    }
    const int r0 = bx * kSortRun;
    const int len = min(kSortRun, c - r0);
    if (len <= 0) return;
    unsigned long long* run = (which ? v.xsort : v.nsort) + r0;  // sorted in place
    unsigned long long* dst = single ? (which ? v.xword : v.nword) : run;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const unsigned lt = lanemask_lt(lane);
    unsigned long long it = tid < len ? run[tid] : ~0ull;
    for (int pass = 0; pass < v.sort_passes; ++pass) {
        const int shift = kOffBits + 8 * pass;
#pragma unroll
        for (int k = 0; k < 8; ++k) whist[tid + k * kSortRun] = 0;
        __syncthreads();
        const unsigned d = (unsigned)(it >> shift) & 255u;
        unsigned peers = kFull;
#pragma unroll
        for (int bit = 0; bit < 8; ++bit) {
            const unsigned bm = __ballot_sync(kFull, (d >> bit) & 1u);
            peers &= ((d >> bit) & 1u) ? bm : ~bm;
        }
        const unsigned rank = __popc(peers & lt);
        if (rank == 0) whist[d * 32 + w] = __popc(peers);
        __syncthreads();
        unsigned loc[8];
        unsigned sum = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            loc[k] = whist[tid * 8 + k];
            sum += loc[k];
        }
        unsigned pre = block_excl_scan_1024(sum, wsum);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            whist[tid * 8 + k] = pre;
            pre += loc[k];
        }
        __syncthreads();
        buf[whist[d * 32 + w] + rank] = it;
        __syncthreads();
        it = buf[tid];
    }
    if (tid < len) dst[tid] = it;
}

__global__ void __launch_bounds__(kSortRun) k_sort(View v, int j, int c, int init, int single) {
    __shared__ SortSmem sm;
    sort_body(v, j, c, init, blockIdx.x, blockIdx.y, sm, single != 0);
}

// Merges the sorted runs of kSortRun words into one sorted list: a word's
// rank is its index in its run plus the words below it in every other run
// (words are distinct, so ranks are too).  Block (r, y) ranks run r of the
// new (y = 0) or expired (y = 1) words; all c words are staged in shared
// memory first, so the binary searches stay on chip.  Presorted expired
// words are gathered in their kept order instead.
__device__ __forceinline__ void runmerge_body(const View& v, int j, int c, int init, int bx, int by,
                                              unsigned long long* words) {
    const int which = by;
    if (which == 1 && init) return;
    if (which == 1 && expired_presorted(v, init)) {
        const int i = bx * kSortRun + threadIdx.x;
        if (i >= c) return;
        const int k = v.sorder[chunk_base_slot(v, j, 0) + i];
        if (k < 0 || k >= c) {
            atomicOr(&v.ctl->err, kErrChunk);
            v.xword[i] = ~0ull;
            return;
        }
        v.xword[i] = v.xsort[k];
        return;
    }
    const unsigned long long* runs = which ? v.xsort : v.nsort;
    unsigned long long* out = which ? v.xword : v.nword;
    for (int i = threadIdx.x; i < c; i += blockDim.x) words[i] = runs[i];
    __syncthreads();
    const int own = bx;
    const int i = own * kSortRun + threadIdx.x;
    if (i >= c) return;
    const unsigned long long w = words[i];
    const int nruns = (c + kSortRun - 1) / kSortRun;
    int rank = threadIdx.x;
    for (int r = 0; r < nruns; ++r) {
        if (r == own) continue;
        const unsigned long long* run = words + r * kSortRun;
        int lo = 0, hi = min(kSortRun, c - r * kSortRun);
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (run[mid] < w)
                lo = mid + 1;
            else
                hi = mid;
        }
        rank += lo;
    }
    out[rank] = w;
}

__global__ void __launch_bounds__(kSortRun) k_runmerge(View v, int j, int c, int init) {
    extern __shared__ unsigned long long words[];
    runmerge_body(v, j, c, init, blockIdx.x, blockIdx.y, words);
}

// -1 on the count of every surviving neighbour of each expired point (old grid).
// G lanes scan one query point's neighbourhood (View::qlanes): 16 (two points
// per warp, so two queries' dependent loads overlap) or 32; the 25 rows of the
// two-cells-per-Eps stencil need the whole warp.

constexpr int kFlattenQueue = 128;  // list rebuilds a flatten block queues for its warps to share

struct StreamSmem {
    int rstart[8][kMaxRows], rpre[8][kMaxRows + 1];
    int grstart[8][2][kMaxRows], grpre[8][2][kMaxRows + 1];  // per lane group (count passes)
    int nbuf[8][kListCap];
    int gnbuf[8][2][kListCap];
    int queue[kFlattenQueue];  // k_flatten: positions of the block whose lists are rebuilt
    int nq;
};

template <int MODE, int DK, int G>
__device__ __forceinline__ void decr_g(const View& v, int j, int c, int bx, StreamSmem& sm) {
    constexpr int DIM = DK & 3, K = (DK >> 2) + 1;  // dimension, cells per Eps
    constexpr int kPerWarp = 32 / G;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int grp = lane / G, gl = lane % G;
    const int gw = (bx * blockDim.x + threadIdx.x) >> 5;
    if (gw * kPerWarp >= c) return;
    const int qi = gw * kPerWarp + grp;
    bool has = qi < c;
    int* rstart = sm.grstart[wib][grp];
    int* rpre = sm.grpre[wib][grp];
    const long long b = v.ctl->b;
    const int old = (int)((b - 1) & 1);
    const unsigned gen = gen_of_build(b - 1);
    const int el = chunk_base_slot(v, j, 0);
    // Expired points keyed from their saved coordinates (the same key they
    // were sorted by when they arrived): the pass does not wait for the
    // chunk's sort, and runs beside it.  Taken in their kept (key, slot)
    // order where there is one, so neighbouring warps read the same cells.
    int k = qi;
    if (has && expired_presorted(v, 0)) {
        k = v.sorder[el + qi];
        if (k < 0 || k >= c) {
            atomicOr(&v.ctl->err, kErrChunk);
            has = false;
        }
    }
    const float4 xp = has ? v.xpt[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned long long key = has ? cell_key(v, xp.x, xp.y, xp.z) : 0ull;
    int rs, re;
    row_ranges<DIM, false, K, G>(v, v.table[old], gen, key, gl, rs, re);
    int total = candidate_stream<Stencil<DIM, false, K>::kRows, G>(rs, re, 0, gl, rstart, rpre);
    if (!has) total = 0;
    const float4* spt = v.spt[old];
    int* scnt = v.scnt[old];
    const bool lists = v.list_cap >= 0;
    const bool damage = damage_on(v);
    const int xs = slot_of(xp);
    Tally tally;
    int r = 0;
    // Two candidates per lane and trip (idx and idx + G): their loads are in
    // flight together and one paired distance evaluation serves both.
    for (int idx = gl; idx < total; idx += 2 * G) {
        const bool two = idx + G < total;
        const int pos0 = stream_pos(idx, r, rstart, rpre);
        const int pos1 = two ? stream_pos(idx + G, r, rstart, rpre) : pos0;
        const float4 q0 = spt[pos0], q1 = spt[pos1];
        // counts only fall here: >= MinPts means no list kept
        const int cnt0 = scnt[pos0], cnt1 = scnt[pos1];
        const int qs0 = slot_of(q0), qs1 = slot_of(q1);
        float d0, d1;
        sqdist32x2<DIM>(xp, q0, q1, d0, d1);
        // counts only fall here: one read below MinPts cannot cross it, so
        // only the others need the count the decrement leaves
        if ((qs0 < el || qs0 >= el + c) && nbr_decide<MODE, DIM>(v, d0, xp, q0, tally)) {
            if (!damage || cnt0 < v.min_pts)
                atomicSub(&scnt[pos0], 1);
            else if (atomicSub(&scnt[pos0], 1) == v.min_pts)
                mark_damage(v, qs0);  // a core falls below MinPts
            if (lists && cnt0 < v.min_pts && v.ntrack[qs0] == 1) list_remove(v, qs0, xs);
        }
        if (two && (qs1 < el || qs1 >= el + c) && nbr_decide<MODE, DIM>(v, d1, xp, q1, tally)) {
            if (!damage || cnt1 < v.min_pts)
                atomicSub(&scnt[pos1], 1);
            else if (atomicSub(&scnt[pos1], 1) == v.min_pts)
                mark_damage(v, qs1);
            if (lists && cnt1 < v.min_pts && v.ntrack[qs1] == 1) list_remove(v, qs1, xs);
        }
    }
    flush_query_max<G>(v, tally.tests, lane);
    flush_stats(v, tally, 0, lane, 0);
}

// The count passes' lane group, chosen per stream at run time (uniform per
// launch): 16 or 32 lanes with one cell per Eps, 32 with two.
template <int MODE, int DK>
__device__ __forceinline__ void decr_body(const View& v, int j, int c, int bx, StreamSmem& sm) {
    if constexpr ((DK >> 2) == 0) {
        if (v.qlanes == 16) {
            decr_g<MODE, DK, 16>(v, j, c, bx, sm);
            return;
        }
    }
    decr_g<MODE, DK, 32>(v, j, c, bx, sm);
}

template <int MODE, int DK>
__global__ void __launch_bounds__(256) k_decr(View v, int j, int c) {
    __shared__ StreamSmem sm;
    decr_body<MODE, DK>(v, j, c, blockIdx.x, sm);
}

__device__ __forceinline__ bool tuple_less(unsigned long long ka, int sa, unsigned long long kb,
                                           int sb) {
    return ka < kb || (ka == kb && sa < sb);
}

// Number of sorted chunk words (key, el + offset) strictly below (key, slot).
__device__ __forceinline__ int count_words_less(const unsigned long long* words, int n, int el,
                                                unsigned long long key, int slot) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const unsigned long long w = words[mid];
        if (tuple_less(w >> kOffBits, el + (int)(w & ((1u << kOffBits) - 1)), key, slot))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Warp-wide count of sorted words below (key, slot): a 32-way search, one
// dependent load per factor-32 narrowing (3 rounds for a 16384-word chunk).
__device__ __forceinline__ int warp_count_words_less(const unsigned long long* words, int n, int el,
                                                     unsigned long long key, int slot, int lane) {
    int lo = 0, hi = n;  // words below lo are less, words from hi on are not
    while (hi - lo > 32) {
        const int step = (hi - lo + 31) >> 5;
        const int piv = lo + lane * step;
        bool less = false;
        if (piv < hi) {
            const unsigned long long w = words[piv];
            less = tuple_less(w >> kOffBits, el + (int)(w & ((1u << kOffBits) - 1)), key, slot);
        }
        const int c = __popc(__ballot_sync(kFull, less));
        if (c == 0) {
            hi = lo;
            break;
        }
        const int nlo = lo + (c - 1) * step + 1;
        hi = min(hi, lo + c * step);
        lo = nlo;
    }
    bool less = false;
    if (lo + lane < hi) {
        const unsigned long long w = words[lo + lane];
        less = tuple_less(w >> kOffBits, el + (int)(w & ((1u << kOffBits) - 1)), key, slot);
    }
    return lo + __popc(__ballot_sync(kFull, less));
}

// Old sorted window minus the expired slots [el, el+c), merged with the c
// new entries; tile t of the old window goes to output offset
// ts - (#expired before ts) + (#new before old[ts]).
constexpr int kMergeStage = 1024;  // new words of a tile staged in shared memory
struct MergeSmem {
    unsigned long long tkey[kMergeTile];
    unsigned long long nw[kMergeStage];
    int tslot[kMergeTile];
    int spre[kMergeTile + 1];
    unsigned wsum[32];
    int bnd[3];
};

__device__ __forceinline__ void merge_body(const View& v, int j, int c, int init, int bx, int nbx,
                                           MergeSmem& sm) {
    unsigned long long* tkey = sm.tkey;
    int* tslot = sm.tslot;
    int* spre = sm.spre;
    unsigned* wsum = sm.wsum;
    const long long b = v.ctl->b;
    const int src = (int)((b - 1) & 1), dst = (int)(b & 1);
    const int n_old = v.ctl->nocc[src];
    const int n_new = n_old - (init ? 0 : c) + c;
    const int el = chunk_base_slot(v, j, init);
    const int tid = threadIdx.x;
    // a fresh union-find forest: with neighbour lists k_border resets it by
    // slot at the end of every clustering, so only the first window needs it
    const bool reset_parent = init || v.list_cap < 0;
    // forest reuse: the hints of the slide's last chunk step stand (every
    // loss of the slide is marked by then), so only that step counts reuses
    const bool reuse = !init && damage_on(v);
    const bool last_step = j * v.chunk + c >= v.S;
    unsigned reused = 0;
    if (bx == 0 && tid == 0) {
        v.ctl->nocc[dst] = n_new;
        v.ctl->nitems = 0;
        v.ctl->ncells = 0;
        v.ctl->union_next = 0;
        v.ctl->label_next = 0;
    }
    // Table generations wrap every kGenMod builds of a table: clear it then.
    if (b >= 2 && ((b >> 1) % (long long)kGenMod) == 0) {
        ulonglong2* T = v.table[dst];
        for (unsigned i = bx * blockDim.x + tid; i <= v.pmask; i += nbx * blockDim.x)
            T[i] = make_ulonglong2(0ull, 0ull);
    }
    const int ntiles = n_old > 0 ? (n_old + kMergeTile - 1) / kMergeTile : 1;
    const int t = bx;
    if (t >= ntiles) return;
    const int ts = t * kMergeTile;
    const int te = min(ts + kMergeTile, n_old);
    const int tlen = te - ts;
    const unsigned long long* okey = v.skey[src];
    const float4* opt = v.spt[src];
    const int* ocnt = v.scnt[src];
    unsigned long long* dkey = v.skey[dst];
    float4* dpt = v.spt[dst];
    int* dcnt = v.scnt[dst];
    // previous roots are only read by this slide's reuse (a slide without
    // reuse leaves them to the flatten, which writes them afresh)
    const int* oprev = reuse ? v.sprev[src] : nullptr;
    int* dprev = reuse ? v.sprev[dst] : nullptr;

    // tile bounds among the new / expired words: warps 0, 1, 2 search at once
    {
        const int lane = tid & 31, w = tid >> 5;
        if (w < 3) {
            const bool need = tlen > 0 && (w == 0 ? t > 0 : (w == 1 ? !init : t < ntiles - 1));
            int r = w == 2 ? c : 0;
            if (need) {
                const int at = w == 2 ? te : ts;
                r = warp_count_words_less(w == 1 ? v.xword : v.nword, c, el, okey[at], slot_of(opt[at]),
                                          lane);
            }
            if (lane == 0) sm.bnd[w] = r;
        }
    }
    // tile -> shared memory; survivor prefix in item order
    for (int i = tid; i < tlen; i += kMergeThreads) {
        tkey[i] = okey[ts + i];
        tslot[i] = slot_of(opt[ts + i]);
    }
    __syncthreads();
    const int jt0 = sm.bnd[0], e0 = sm.bnd[1], jt1 = sm.bnd[2];
    const int base = ts - e0 + jt0;
    const int m = jt1 - jt0;
    const bool staged = m <= kMergeStage;
    const unsigned long long* nw = staged ? sm.nw : v.nword + jt0;  // the tile's new words
    if (staged)
        for (int i = tid; i < m; i += kMergeThreads) sm.nw[i] = v.nword[jt0 + i];
    unsigned flags[4];
    unsigned cnt = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int i = tid * 4 + k;
        const bool surv = i < tlen && (init || tslot[i] < el || tslot[i] >= el + c);
        flags[k] = surv ? 1u : 0u;
        cnt += flags[k];
    }
    {
        const int lane = tid & 31, w = tid >> 5;
        unsigned incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned x = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += x;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        if (w == 0) {
            const unsigned x = lane < kMergeThreads / 32 ? wsum[lane] : 0u;
            unsigned xi = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(kFull, xi, o);
                if (lane >= o) xi += y;
            }
            if (lane < kMergeThreads / 32) wsum[lane] = xi - x;
        }
        __syncthreads();
        unsigned pre = wsum[w] + incl - cnt;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            spre[tid * 4 + k] = (int)pre;
            pre += flags[k];
        }
        if (tid == kMergeThreads - 1) spre[kMergeTile] = (int)pre;
    }
    __syncthreads();

    // survivors (coalesced, item order i = tid + 256 k)
    for (int i = tid; i < tlen; i += kMergeThreads) {
        const int s = tslot[i];
        if (!(init || s < el || s >= el + c)) continue;
        const int lessnew = m > 0 ? count_words_less(nw, m, el, tkey[i], s) : 0;
        const int o = base + spre[i] + lessnew;
        if (o < 0 || o >= n_new) {
            atomicOr(&v.ctl->err, kErrChunk);
            continue;
        }
        dkey[o] = tkey[i];
        dpt[o] = opt[ts + i];
        const int cnt = ocnt[ts + i];
        dcnt[o] = cnt;
        const int prev = oprev ? oprev[ts + i] : -1;
        if (dprev) dprev[o] = prev;
        v.sroot[o] = start_hint(v, s, cnt, prev, reuse, reused);
        if (reset_parent) v.parent[s] = s;
    }
    if (last_step) {
        reused = __reduce_add_sync(kFull, reused);
        if ((tid & 31) == 0 && reused) atomicAdd(&v.ctl->reused, (int)reused);
    }
    // new entries of this tile
    for (int q = jt0 + tid; q < jt1; q += kMergeThreads) {
        const unsigned long long wd = nw[q - jt0];
        const unsigned long long key = wd >> kOffBits;
        const int slot = el + (int)(wd & ((1u << kOffBits) - 1));
        int lo = 0, hi = tlen;  // old tile entries below (key, slot)
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (tuple_less(tkey[mid], tslot[mid], key, slot))
                lo = mid + 1;
            else
                hi = mid;
        }
        const int o = base + (q - jt0) + spre[lo];
        if (o < 0 || o >= n_new || slot < 0 || slot >= v.W) {
            atomicOr(&v.ctl->err, kErrChunk);
            continue;
        }
        dkey[o] = key;
        dpt[o] = v.ring[slot];
        dcnt[o] = 0;
        if (dprev) dprev[o] = -1;
        v.sroot[o] = -1;  // the increment sets the count and the hint
        if (reset_parent) v.parent[slot] = slot;
        // the chunk's order, for the slide that expires it (every reader of
        // the expired order of these slots ran before this pass)
        if (!init && v.sorder) v.sorder[el + q] = slot - el;
    }
}

__global__ void __launch_bounds__(kMergeThreads) k_merge(View v, int j, int c, int init) {
    __shared__ MergeSmem sm;
    merge_body(v, j, c, init, blockIdx.x, gridDim.x, sm);
}

// Cell table and work list of the new sorted window.  A work item is a
// maximal run of one cell inside a 32-aligned block of sorted positions.
// Item and cell counters are reserved once per block.
struct BuildSmem {
    int wcount[kBuildThreads / 32];
    int wbase[kBuildThreads / 32];
    int bcells;
};

// (pooled: a pool launch, whose many streams fill the GPU: 32-point items)
__device__ __forceinline__ void build_body(const View& v, int bx, BuildSmem& sm, bool pooled) {
    int* wcount = sm.wcount;
    int* wbase = sm.wbase;
    int& bcells = sm.bcells;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = (bx * blockDim.x + threadIdx.x) >> 5;
    const long long b = v.ctl->b;
    const int cur = (int)(b & 1);
    const unsigned gen = gen_of_build(b);
    const int n = v.ctl->nocc[cur];
    const int i = gw * 32 + lane;
    const unsigned long long* skey = v.skey[cur];
    const bool valid = i < n;
    const unsigned long long k = valid ? skey[i] : ~0ull;
    unsigned long long kp = __shfl_up_sync(kFull, k, 1);
    unsigned long long kn = __shfl_down_sync(kFull, k, 1);
    if (lane == 0) kp = (valid && i > 0) ? skey[i - 1] : ~0ull;
    if (lane == 31) kn = (i + 1 < n) ? skey[i + 1] : ~0ull;
    const bool first = valid && (i == 0 || kp != k);
    const bool last = valid && (i == n - 1 || kn != k);
    int err = 0;
    ulonglong2* T = v.table[cur];
    const unsigned long long tag = tag_of(k & kKeyMask, gen);
    // A cell that starts and ends in this warp is entered once, by its first
    // point; otherwise its first point enters the start, its last the end.
    const unsigned firsts = __ballot_sync(kFull, first);
    const unsigned lasts = __ballot_sync(kFull, last);
    if (first) {
        const unsigned ends = lasts & ~((1u << lane) - 1u);  // my cell's last is the lowest
        const bool ok = ends ? table_set(T, v.pmask, v.pbits, tag, 2, i, gw * 32 + __ffs(ends))
                             : table_set(T, v.pmask, v.pbits, tag, 0, i);
        if (!ok) err |= kErrHashFull;
    }
    if (last && !(firsts & ((2u << lane) - 1u)) && !table_set(T, v.pmask, v.pbits, tag, 1, i + 1))
        err |= kErrHashFull;
    const int ip = (!pooled && v.item_pts > 0) ? v.item_pts : 32;
    const unsigned starts = __ballot_sync(kFull, valid && (first || (lane & (ip - 1)) == 0));
    const int nfirst = __popc(__ballot_sync(kFull, first));
    if (threadIdx.x == 0) bcells = 0;
    if (lane == 0) wcount[wib] = __popc(starts);
    __syncthreads();
    if (lane == 0 && nfirst) atomicAdd(&bcells, nfirst);
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < kBuildThreads / 32; ++w) {
            wbase[w] = tot;
            tot += wcount[w];
        }
        const int base = tot ? atomicAdd(&v.ctl->nitems, tot) : 0;
        for (int w = 0; w < kBuildThreads / 32; ++w) wbase[w] += base;
    }
    __syncthreads();
    if (threadIdx.x == 0 && bcells) atomicAdd(&v.ctl->ncells, bcells);
    if (valid && (first || (lane & (ip - 1)) == 0)) {
        const int rank = __popc(starts & lanemask_lt(lane));
        const unsigned above = starts & ~((2u << lane) - 1u);
        const int next = above ? gw * 32 + __ffs(above) - 1 : gw * 32 + 32;
        const int end = min(next, n);
        const int slot = wbase[wib] + rank;
        if (slot < v.max_items)
            v.items[slot] = make_int2(i, end - i);
        else
            err |= kErrItems;
    }
    if (err) atomicOr(&v.ctl->err, err);
}

__global__ void __launch_bounds__(kBuildThreads) k_build(View v) {
    __shared__ BuildSmem sm;
    build_body(v, blockIdx.x, sm, false);
}

// Full count of each new point and +1 on every older neighbour (new grid).
template <int MODE, int DK, int G>
__device__ __forceinline__ void incr_g(const View& v, int j, int c, int init, int bx, StreamSmem& sm) {
    constexpr int DIM = DK & 3, K = (DK >> 2) + 1;  // dimension, cells per Eps
    constexpr int kPerWarp = 32 / G;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int grp = lane / G, gl = lane % G;
    const int gw = (bx * blockDim.x + threadIdx.x) >> 5;
    if (gw * kPerWarp >= c) return;
    const int qi = gw * kPerWarp + grp;
    const bool has = qi < c;
    int* rstart = sm.grstart[wib][grp];
    int* rpre = sm.grpre[wib][grp];
    const long long b = v.ctl->b;
    const int cur = (int)(b & 1);
    const unsigned gen = gen_of_build(b);
    const int el = chunk_base_slot(v, j, init);
    const unsigned long long word = has ? v.nword[qi] : 0ull;
    const unsigned long long key = word >> kOffBits;
    const int aslot = el + (int)(word & ((1u << kOffBits) - 1));
    const float4 ap = has ? v.ring[aslot] : make_float4(0.f, 0.f, 0.f, 0.f);
    int rs, re;
    row_ranges<DIM, false, K, G>(v, v.table[cur], gen, key, gl, rs, re);
    int total = candidate_stream<Stencil<DIM, false, K>::kRows, G>(rs, re, 0, gl, rstart, rpre);
    if (!has) total = 0;
    int tmax = total;
#pragma unroll
    for (int o = G; o < 32; o <<= 1) tmax = max(tmax, __shfl_xor_sync(kFull, tmax, o));
    const float4* spt = v.spt[cur];
    int* scnt = v.scnt[cur];
    const bool lists = v.list_cap >= 0;
    int* nbuf = sm.gnbuf[wib][grp];
    Tally tally;
    int count = 0, mypos = -1, r = 0, nfound = 0;
    // Two candidates per lane and trip (idx and idx + G), as in the decrement.
    for (int base = 0; base < tmax; base += 2 * G) {
        const int idx = base + gl;
        const bool h0 = idx < total, h1 = idx + G < total;
        int pos[2] = {0, 0}, cnt[2] = {0, 0}, qs[2] = {-1, -1};
        float4 q[2] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
        if (h0) {
            pos[0] = stream_pos(idx, r, rstart, rpre);
            q[0] = spt[pos[0]];
            cnt[0] = scnt[pos[0]];  // counts only rise here: >= MinPts means no list kept
        }
        if (h1) {
            pos[1] = stream_pos(idx + G, r, rstart, rpre);
            q[1] = spt[pos[1]];
            cnt[1] = scnt[pos[1]];
        }
        float d[2];
        sqdist32x2<DIM>(ap, q[0], q[1], d[0], d[1]);
        bool nb[2] = {false, false};
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (!(u == 0 ? h0 : h1)) continue;
            qs[u] = slot_of(q[u]);
            if (qs[u] == aslot) {
                ++count;
                mypos = pos[u];
            } else if (nbr_decide<MODE, DIM>(v, d[u], ap, q[u], tally)) {
                ++count;
                nb[u] = true;
                if (qs[u] < el || qs[u] >= el + c) {
                    // counts only rise here: one read below MinPts may be the
                    // increment that makes the point core, which sets its hint
                    if (cnt[u] >= v.min_pts)
                        atomicAdd(&scnt[pos[u]], 1);
                    else if (atomicAdd(&scnt[pos[u]], 1) == v.min_pts - 1)
                        v.sroot[pos[u]] = qs[u];  // now core
                    if (lists && cnt[u] < v.min_pts && v.ntrack[qs[u]] == 1) list_append(v, qs[u], aslot);
                }
            }
        }
        if (lists) {
            nfound = list_collect<G>(nb[0], qs[0], nfound, v.list_cap, nbuf, lane);
            nfound = list_collect<G>(nb[1], qs[1], nfound, v.list_cap, nbuf, lane);
        }
    }
    if (lists) list_store<G>(v, aslot, nfound, nbuf, lane, has);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        count += __shfl_xor_sync(kFull, count, o);
        mypos = max(mypos, __shfl_xor_sync(kFull, mypos, o));
    }
    int err = 0;
    if (gl == 0 && has) {
        if (mypos >= 0) {
            scnt[mypos] = count;
            v.sroot[mypos] = count >= v.min_pts ? aslot : -1;
        } else {
            err = kErrChunk;
        }
    }
    flush_query_max<G>(v, tally.tests, lane);
    flush_stats(v, tally, err, lane, 0);
}

template <int MODE, int DK>
__device__ __forceinline__ void incr_body(const View& v, int j, int c, int init, int bx, StreamSmem& sm) {
    if constexpr ((DK >> 2) == 0) {
        if (v.qlanes == 16) {
            incr_g<MODE, DK, 16>(v, j, c, init, bx, sm);
            return;
        }
    }
    incr_g<MODE, DK, 32>(v, j, c, init, bx, sm);
}

template <int MODE, int DK>
__global__ void __launch_bounds__(256, 5) k_incr(View v, int j, int c, int init) {
    __shared__ StreamSmem sm;
    incr_body<MODE, DK>(v, j, c, init, blockIdx.x, sm);
}

// Fresh start hints without reuse (-1 for a non-core position, its own
// slot for a core) and a fresh forest, for a clustering of the window as it
// stands (rtdbs_cluster), whose hints may hold the last union's roots.
__global__ void k_hints(View v) {
    const int cur = (int)(v.ctl->b & 1);
    const int n = v.ctl->nocc[cur];
    const int* scnt = v.scnt[cur];
    const int* sw = reinterpret_cast<const int*>(v.spt[cur]) + 3;
    if (blockIdx.x == 0 && threadIdx.x == 0) v.ctl->prev_ok = 0;  // no reuse to judge (read by k_border)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int s = sw[4 * (size_t)i];
        v.sroot[i] = scnt[i] >= v.min_pts ? s : -1;
        v.parent[s] = s;
    }
}

// Union of every core-core neighbour pair, each unordered pair once (the
// candidate's sorted position is above the home point's).  A candidate's
// root is found once per candidate chunk and compared with cached roots of
// the home points (shared memory, per warp); a link is attempted only where
// the two differ, so same-set pairs cost no memory traffic.  Finds start
// from per-position root hints.  Each warp walks
// a contiguous range of work items (neighbouring cells), so candidate loads
// reuse L1.
constexpr int kSingleGrab = 5;  // default work items per grab of a large window slid alone
                                // whose cells hold several points

struct ClusterSmem {
    int home_root[kClusterThreads / 32][32];
    float4 home_pt[kClusterThreads / 32][32];
    int rstart[kClusterThreads / 32][kMaxRows], rpre[kClusterThreads / 32][kMaxRows + 1];
};

// Work items a warp takes at a time: the stream's setting, or by default 8
// in a pool launch (many streams share the GPU); for a single stream up to 8
// on large windows, fewer on small ones (a 10k-point window has a few hundred
// to a few thousand items: 8 per grab would leave them to a few dozen warps),
// and 5 where cells hold several points (fewer than 0.4 items per window
// point): items are then costly enough that balance beats the queue's atomics
// (a 1M-point walker window, 0.3 items per point: union 233 us with 8, 224
// with 5), where on windows of near-empty cells (one item per point, most of
// them without a core) the atomics dominate and 8 stays faster.
__device__ __forceinline__ int work_grab(const View& v, bool pooled) {
    if (v.grab > 0) return v.grab;
    if (pooled) return kBatch;
    const int g = max(1, min(kBatch, v.W >> 14));
    const long long items = v.ctl->nitems;
    return (g > kSingleGrab && items * 5 < (long long)v.W * 2) ? kSingleGrab : g;
}

template <int MODE, int DK>
__device__ __forceinline__ void union_body(const View& v, ClusterSmem& sm, int grab) {
    constexpr int DIM = DK & 3, K = (DK >> 2) + 1;  // dimension, cells per Eps
    float4(&home_pt)[kClusterThreads / 32][32] = sm.home_pt;
    int(&rstart)[kClusterThreads / 32][kMaxRows] = sm.rstart;
    int(&rpre)[kClusterThreads / 32][kMaxRows + 1] = sm.rpre;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    volatile int* rh = sm.home_root[wib];
    const float4* hpt = home_pt[wib];
    const long long b = v.ctl->b;
    const int cur = (int)(b & 1);
    const unsigned gen = gen_of_build(b);
    const int nitems = min(v.ctl->nitems, v.max_items);
    const float4* spt = v.spt[cur];
    const unsigned long long* skey = v.skey[cur];
    const ulonglong2* T = v.table[cur];
    int* parent = v.parent;
    // Root hints by sorted position (an ancestor of the point: its own slot
    // or the old root of its intact component; -1 for a non-core point, so
    // the hint alone tells a core; set by the merge and the increment, see
    // start_hint): coalesced with the candidate loads, and refreshed as roots
    // are found, so find walks stay short.
    volatile int* hint = v.sroot;
    Tally tally;
    int err = 0;
    // Warps take batches of `grab` consecutive work items (neighbouring
    // cells: candidate loads reuse L1) from a counter, so uneven items do not
    // leave warps idle at the end.
    int it1 = 0;
    for (int itx = nitems;;) {
        if (itx >= it1) {
            int got = 0;
            if (lane == 0) got = atomicAdd(&v.ctl->union_next, grab);
            itx = __shfl_sync(kFull, got, 0);
            if (itx >= nitems) break;
            it1 = min(itx + grab, nitems);
        }
        const int2 item = v.items[itx++];
        const int start = item.x, len = item.y;
        const bool hv = lane < len;
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f);
        bool hcore = false;
        int hh = -1;
        if (hv) {
            h = spt[start + lane];
            hh = hint[start + lane];
            hcore = hh >= 0;
        }
        const unsigned hmask = __ballot_sync(kFull, hcore);
        if (!hmask) continue;
        __syncwarp();
        if (hcore) rh[lane] = hh;
        home_pt[wib][lane] = h;
        // All home cores under one hint r0 (common once the previous forest is
        // reused): a candidate chunk whose cores all carry r0 is one set with
        // them and is skipped without the per-home loop.
        const int r0 = __shfl_sync(kFull, hh, __ffs(hmask) - 1);
        const bool uni = __all_sync(kFull, !hcore || hh == r0);
        const int hmin = start + __ffs(hmask) - 1;
        int rs, re;
        row_ranges<DIM, true, K>(v, T, gen, skey[start], lane, rs, re);
        const int total = candidate_stream<Stencil<DIM, true, K>::kRows>(rs, re, hmin + 1, lane, rstart[wib], rpre[wib]);
        int r = 0;
        for (int base = 0; base < total; base += 32) {
            const int idx = base + lane;
            int pos = 0, qh = 0;
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            bool qc = false;
            if (idx < total) {
                pos = stream_pos(idx, r, rstart[wib], rpre[wib]);
                q = spt[pos];
                qh = hint[pos];
                qc = qh >= 0;
            }
            if (!__any_sync(kFull, qc && !(uni && qh == r0))) continue;
            // Pairs whose hints already agree are in one set: no test, no link.
            unsigned adj = 0;
            unsigned mm = hmask;
            while (mm) {
                const int hi = __ffs(mm) - 1;
                mm &= mm - 1;
                if (qc && pos > start + hi && qh != rh[hi] && is_nbr<MODE, DIM>(v, hpt[hi], q, tally))
                    adj |= 1u << hi;
            }
            if (adj) {
                int rq = uf_find(parent, qh);
                while (adj) {
                    const int hi = __ffs(adj) - 1;
                    adj &= adj - 1;
                    const int ra = rh[hi];
                    if (ra != rq) {
                        rq = uf_hook(parent, ra, rq, err);
                        rh[hi] = rq;  // an ancestor of both points (benign race)
                    }
                }
                if (rq != qh) hint[pos] = rq;
            }
            __syncwarp();
        }
        if (hcore) hint[start + lane] = rh[lane];
    }
    flush_stats(v, tally, err, lane, 1);
}

template <int MODE, int DK>
__global__ void __launch_bounds__(kClusterThreads, 8) k_union(View v) {
    __shared__ ClusterSmem sm;
    union_body<MODE, DK>(v, sm, work_grab(v, false));
}

// The neighbour list of the non-core point at sorted position `at`, from one
// scan of the current grid (called by the whole warp).
template <int MODE, int DIM, int K>
__device__ __forceinline__ void rebuild_list(const View& v, int at, int cur, unsigned gen, int lane, int* rstart,
                                             int* rpre, int* nbuf, Tally& tally) {
    const float4* spt = v.spt[cur];
    const float4 ap = spt[at];
    const int a = slot_of(ap);
    int rs, re;
    row_ranges<DIM, false, K>(v, v.table[cur], gen, v.skey[cur][at], lane, rs, re);
    const int total = candidate_stream<Stencil<DIM, false, K>::kRows>(rs, re, 0, lane, rstart, rpre);
    int r = 0, nfound = 0;
    for (int base = 0; base < total; base += 32) {
        const int idx = base + lane;
        bool nb = false;
        int qs = -1;
        if (idx < total) {
            const float4 q = spt[stream_pos(idx, r, rstart, rpre)];
            qs = slot_of(q);
            nb = qs != a && is_nbr<MODE, DIM>(v, ap, q, tally);
        }
        nfound = list_collect(nb, qs, nfound, v.list_cap, nbuf, lane);
    }
    list_store(v, a, nfound, nbuf, lane);
}

// Root of every core point, walked from the position's root hint.  Without
// neighbour lists: by sorted position (-1 for non-core points), for the grid
// scan of k_label.  With lists: by slot (rslot), which k_border turns into
// the outputs; and a point below MinPts without a list (it lost core status
// this slide) gets its list rebuilt here from one scan of the final grid, by
// the warp whose 32 positions hold it.
template <int MODE, int DK>
__device__ __forceinline__ void flatten_body(const View& v, int bx, int nbx, StreamSmem& sm) {
    constexpr int DIM = DK & 3, K = (DK >> 2) + 1;  // dimension, cells per Eps
    if (bx == 0 && threadIdx.x == 0) v.ctl->label_next = 0;  // k_label's queue; not read here
    const long long b = v.ctl->b;
    const int cur = (int)(b & 1);
    const int n = v.ctl->nocc[cur];
    const int* scnt = v.scnt[cur];
    if (v.list_cap < 0) {
        for (int i = bx * blockDim.x + threadIdx.x; i < n; i += nbx * blockDim.x)
            v.sroot[i] = scnt[i] >= v.min_pts ? uf_find(v.parent, v.sroot[i]) : -1;
        return;
    }
    int(&rstart)[8][kMaxRows] = sm.rstart;
    int(&rpre)[8][kMaxRows + 1] = sm.rpre;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const unsigned gen = gen_of_build(b);
    const int* sw = reinterpret_cast<const int*>(v.spt[cur]) + 3;  // .w = slot
    int* nbuf = sm.nbuf[wib];
    // the roots by position for the next slide's reuse: not while reuse
    // stays off for it (k_border counts reuse_skip down after this pass)
    const bool keep_roots = v.ctl->reuse_skip <= 1;
    Tally tally;
    // Roots first (no barrier); the positions whose lists are rebuilt go to
    // the block's queue, which its warps share once the block has been
    // through its positions (one barrier), so rebuilds of neighbouring points
    // do not fall on one warp.  A full queue is rebuilt by the warp itself.
    if (threadIdx.x == 0) sm.nq = 0;
    __syncthreads();
    for (int i0 = (bx * blockDim.x + threadIdx.x) & ~31; i0 < n; i0 += nbx * blockDim.x) {  // warp-uniform
        const int i = i0 + lane;
        bool need = false;
        if (i < n) {
            const int slot = sw[4 * (size_t)i];
            if (scnt[i] >= v.min_pts) {
                const int root = uf_find(v.parent, v.sroot[i]);
                v.rslot[slot] = root;
                if (keep_roots) v.sprev[cur][i] = root;  // the next slide's reuse reads it by position
            } else {
                v.rslot[slot] = -1;
                if (keep_roots) v.sprev[cur][i] = -1;
                need = v.ntrack[slot] != 1;
            }
        }
        bool inline_rebuild = false;
        if (need) {
            const int at = atomicAdd(&sm.nq, 1);
            if (at < kFlattenQueue)
                sm.queue[at] = i;
            else
                inline_rebuild = true;
        }
        unsigned todo = __ballot_sync(kFull, inline_rebuild);
        while (todo) {
            rebuild_list<MODE, DIM, K>(v, i0 + __ffs(todo) - 1, cur, gen, lane, rstart[wib], rpre[wib], nbuf, tally);
            todo &= todo - 1;
        }
    }
    __syncthreads();
    const int nq = min(sm.nq, kFlattenQueue);
    for (int e = wib; e < nq; e += wpb)
        rebuild_list<MODE, DIM, K>(v, sm.queue[e], cur, gen, lane, rstart[wib], rpre[wib], nbuf, tally);
    flush_stats(v, tally, 0, lane, 1);
}

template <int MODE, int DK>
__global__ void __launch_bounds__(256, 6) k_flatten(View v) {
    __shared__ StreamSmem sm;
    flatten_body<MODE, DK>(v, blockIdx.x, gridDim.x, sm);
}

// Labels and ids by slot: core -> 0 and its root; non-core -> 1 and the
// minimum root over adjacent cores, or 2 and its own slot.
template <int MODE, int DK>
__device__ __forceinline__ void label_body(const View& v, int advance, int bx, ClusterSmem& sm, int grab) {
    constexpr int DIM = DK & 3, K = (DK >> 2) + 1;  // dimension, cells per Eps
    int(&rstart)[kClusterThreads / 32][kMaxRows] = sm.rstart;
    int(&rpre)[kClusterThreads / 32][kMaxRows + 1] = sm.rpre;
    float4(&home_pt)[kClusterThreads / 32][32] = sm.home_pt;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const float4* hpt = home_pt[wib];
    const long long b = v.ctl->b;
    const int cur = (int)(b & 1);
    const unsigned gen = gen_of_build(b);
    const int nitems = min(v.ctl->nitems, v.max_items);
    const float4* spt = v.spt[cur];
    const int* sroot = v.sroot;
    const unsigned long long* skey = v.skey[cur];
    const ulonglong2* T = v.table[cur];
    Tally tally;
    int it1 = 0;
    for (int itx = nitems;;) {
        if (itx >= it1) {
            int got = 0;
            if (lane == 0) got = atomicAdd(&v.ctl->label_next, grab);
            itx = __shfl_sync(kFull, got, 0);
            if (itx >= nitems) break;
            it1 = min(itx + grab, nitems);
        }
        const int2 item = v.items[itx++];
        const int start = item.x, len = item.y;
        const bool hv = lane < len;
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f);
        int hslot = -1, hr = -1;
        bool lonely = false;
        if (hv) {
            h = spt[start + lane];
            hslot = slot_of(h);
            hr = sroot[start + lane];
            if (hr >= 0) {
                v.label[hslot] = 0;
                v.cid[hslot] = hr;
            } else if (v.scnt[cur][start + lane] <= 1) {
                // no neighbour but itself: noise without a scan
                lonely = true;
                v.label[hslot] = 2;
                v.cid[hslot] = hslot;
            }
        }
        const unsigned nmask = __ballot_sync(kFull, hv && hr < 0 && !lonely);
        if (!nmask) continue;
        __syncwarp();
        home_pt[wib][lane] = h;
        int rs, re;
        row_ranges<DIM, false, K>(v, T, gen, skey[start], lane, rs, re);
        const int total = candidate_stream<Stencil<DIM, false, K>::kRows>(rs, re, 0, lane, rstart[wib], rpre[wib]);
        int best = INT_MAX, r = 0;
        for (int base = 0; base < total; base += 32) {
            const int idx = base + lane;
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            int qr = -1;
            if (idx < total) {
                const int pos = stream_pos(idx, r, rstart[wib], rpre[wib]);
                qr = sroot[pos];
                q = spt[pos];
            }
            if (!__any_sync(kFull, qr >= 0)) continue;
            unsigned mm = nmask;
            while (mm) {
                const int hi = __ffs(mm) - 1;
                mm &= mm - 1;
                const int val = (qr >= 0 && is_nbr<MODE, DIM>(v, hpt[hi], q, tally)) ? qr : INT_MAX;
                const int mn = (int)__reduce_min_sync(kFull, (unsigned)val);
                if (lane == hi) best = min(best, mn);
            }
        }
        if (hv && hr < 0 && !lonely) {
            if (best != INT_MAX) {
                v.label[hslot] = 1;
                v.cid[hslot] = best;
            } else {
                v.label[hslot] = 2;
                v.cid[hslot] = hslot;
            }
        }
    }
    flush_stats(v, tally, 0, lane, 1);
    if (bx == 0 && threadIdx.x == 0) {
        v.ctl->union_next = 0;                // the next clustering's queue; not read here
        if (advance) v.ctl->slide += 1;       // no reader here
    }
}

template <int MODE, int DK>
__global__ void __launch_bounds__(kClusterThreads, 6) k_label(View v, int advance) {
    __shared__ ClusterSmem sm;
    label_body<MODE, DK>(v, advance, blockIdx.x, sm, work_grab(v, false));
}

// Outputs by slot from the roots and the lists: core -> 0 and its root; a
// non-core point with a core neighbour -> 1 and the minimum root over its
// core neighbours; else noise -> 2 and its own slot.  Resets the union-find
// forest for the next clustering (coalesced, by slot) and ends the slide
// like k_label.
__device__ __forceinline__ void border_body(const View& v, int advance, int bx, int nbx) {
    for (int s = bx * blockDim.x + threadIdx.x; s < v.W; s += nbx * blockDim.x) {
        const int root = v.rslot[s];
        int lab = 0, id = root;
        if (root < 0) {
            if (v.ntrack[s] != 1) atomicOr(&v.ctl->err, kErrList);
            const int4* L = reinterpret_cast<const int4*>(v.nlist + (size_t)s * v.list_stride);
            int best = INT_MAX;
            for (int k = 0; k < (v.list_stride >> 2); ++k) {
                const int4 e = L[k];
                const int r0 = e.x >= 0 ? v.rslot[e.x] : -1;
                const int r1 = e.y >= 0 ? v.rslot[e.y] : -1;
                const int r2 = e.z >= 0 ? v.rslot[e.z] : -1;
                const int r3 = e.w >= 0 ? v.rslot[e.w] : -1;
                if (r0 >= 0) best = min(best, r0);
                if (r1 >= 0) best = min(best, r1);
                if (r2 >= 0) best = min(best, r2);
                if (r3 >= 0) best = min(best, r3);
            }
            lab = best != INT_MAX ? 1 : 2;
            id = best != INT_MAX ? best : s;
        }
        v.label[s] = lab;
        v.cid[s] = id;
        v.parent[s] = s;
        v.damaged[s] = 0;
    }
    if (bx == 0 && threadIdx.x == 0) {
        v.ctl->union_next = 0;                // the next clustering's queue; not read here
        // the reuse of this clustering is counted: judge it
        // (not after a fresh window, which had no previous forest)
        if (v.ctl->reuse_skip > 0)
            v.ctl->reuse_skip -= 1;
        else if (v.ctl->prev_ok && v.ctl->reused < v.W / 16)
            v.ctl->reuse_skip = kReuseRetry;
        v.ctl->last_reused = v.ctl->reused;
        v.ctl->reused = 0;
        v.ctl->prev_ok = 1;                   // the forest of this clustering can be reused
        if (advance) v.ctl->slide += 1;       // no reader here
    }
}

__global__ void k_border(View v, int advance) { border_body(v, advance, blockIdx.x, gridDim.x); }

__global__ void k_counts_by_slot(View v, int* nn) {
    const int cur = (int)(v.ctl->b & 1);
    const int n = v.ctl->nocc[cur];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        nn[slot_of(v.spt[cur][i])] = v.scnt[cur][i];
}

int g_num_sms = 0;
// ------------------------------------------------------------- batched kernel

template <int PHASE>
struct PhaseShape;
template <> struct PhaseShape<kBatchIngest> { static constexpr int threads = 256, min_blocks = 1; };
template <> struct PhaseShape<kBatchSort> { static constexpr int threads = kSortRun, min_blocks = 1; };
template <> struct PhaseShape<kBatchRunmerge> { static constexpr int threads = kSortRun, min_blocks = 1; };
template <> struct PhaseShape<kBatchDecrement> { static constexpr int threads = 256, min_blocks = 8; };
template <> struct PhaseShape<kBatchMerge> { static constexpr int threads = kMergeThreads, min_blocks = 1; };
template <> struct PhaseShape<kBatchBuild> { static constexpr int threads = kBuildThreads, min_blocks = 1; };
template <> struct PhaseShape<kBatchIncrement> { static constexpr int threads = 256, min_blocks = 8; };
template <> struct PhaseShape<kBatchDamage> { static constexpr int threads = 256, min_blocks = 1; };
template <> struct PhaseShape<kBatchReuse> { static constexpr int threads = 256, min_blocks = 1; };
template <> struct PhaseShape<kBatchUnion> { static constexpr int threads = kClusterThreads, min_blocks = 8; };
template <> struct PhaseShape<kBatchFlatten> { static constexpr int threads = 256, min_blocks = 6; };
template <> struct PhaseShape<kBatchLabel> { static constexpr int threads = kClusterThreads, min_blocks = 6; };

// One phase over many streams.  The block finds its item, copies that
// stream's View into shared memory and runs the stream's kernel body.
// Phases whose bodies depend on the precision mode and dimension are
// instantiated per (MODE, DIM) and launched once per group of streams that
// share them, so each instantiation holds one body (registers as in the
// single-stream kernels); the other phases use MODE = DIM = 0.
template <int PHASE, int MODE, int DK>
__global__ void __launch_bounds__(PhaseShape<PHASE>::threads, PhaseShape<PHASE>::min_blocks)
    k_batch(BatchLaunch L) {
    __shared__ View sv;
    __shared__ int s_item, s_bx, s_nbx;
    if (threadIdx.x == 0) {
        int lo = 0, hi = L.n;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (L.prefix[mid] <= (int)blockIdx.x)
                lo = mid;
            else
                hi = mid;
        }
        s_item = lo;
        s_bx = (int)blockIdx.x - L.prefix[lo];
        s_nbx = L.prefix[lo + 1] - L.prefix[lo];
    }
    __syncthreads();
    const BatchItem it = L.items[s_item];
    {
        const int* src = reinterpret_cast<const int*>(L.views + it.view);
        int* dst = reinterpret_cast<int*>(&sv);
        for (int i = threadIdx.x; i < (int)(sizeof(View) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const int bx = s_bx, nbx = s_nbx;
    if constexpr (PHASE == kBatchIngest) {
        ingest_body(sv, it.j, it.c, 0, it.stg_off, it.input, bx);
    } else if constexpr (PHASE == kBatchSort) {
        __shared__ SortSmem sm;
        const int nruns = (it.c + kSortRun - 1) / kSortRun;
        sort_body(sv, it.j, it.c, 0, bx % nruns, bx / nruns, sm, false);
    } else if constexpr (PHASE == kBatchRunmerge) {
        extern __shared__ unsigned long long words[];
        const int nruns = (it.c + kSortRun - 1) / kSortRun;
        runmerge_body(sv, it.j, it.c, 0, bx % nruns, bx / nruns, words);
    } else if constexpr (PHASE == kBatchDecrement) {
        __shared__ StreamSmem sm;
        decr_body<MODE, DK>(sv, it.j, it.c, bx, sm);
    } else if constexpr (PHASE == kBatchMerge) {
        __shared__ MergeSmem sm;
        merge_body(sv, it.j, it.c, 0, bx, nbx, sm);
    } else if constexpr (PHASE == kBatchBuild) {
        __shared__ BuildSmem sm;
        build_body(sv, bx, sm, true);
    } else if constexpr (PHASE == kBatchIncrement) {
        __shared__ StreamSmem sm;
        incr_body<MODE, DK>(sv, it.j, it.c, 0, bx, sm);
    } else if constexpr (PHASE == kBatchUnion) {
        __shared__ ClusterSmem sm;
        union_body<MODE, DK>(sv, sm, work_grab(sv, true));
    } else if constexpr (PHASE == kBatchFlatten) {
        __shared__ StreamSmem sm;
        flatten_body<MODE, DK>(sv, bx, nbx, sm);
    } else {
        __shared__ ClusterSmem sm;
        if (sv.list_cap >= 0)
            border_body(sv, 1, bx, nbx);
        else
            label_body<MODE, DK>(sv, 1, bx, sm, work_grab(sv, true));
    }
}

std::atomic<unsigned long long> g_runmerge_ready{0};  // one bit per device

// k_runmerge stages up to kChunkMax words (128 KB) in dynamic shared memory;
// allow that once per device (a host-side attribute, not a stream operation).
void ensure_runmerge_smem() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    const unsigned long long bit = 1ull << dev;
    if (g_runmerge_ready.load() & bit) return;
    const int bytes = (int)(sizeof(unsigned long long) * kChunkMax);
    if (cudaFuncSetAttribute(k_runmerge, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess &&
        cudaFuncSetAttribute(k_batch<kBatchRunmerge, 0, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) ==
            cudaSuccess)
        g_runmerge_ready.fetch_or(bit);
}

}  // namespace

// Launch of a work kernel instantiated for (precision, DK); dk = dim + 4 (K - 1).
#define RTDBS_DISPATCH(prec, dk_expr, KERNEL, GRID, BLOCK, STREAM, ...)          \
    do {                                                                         \
        const int dk = (dk_expr);                                                \
        if ((prec) == kPrecFp32) {                                               \
            switch (dk) {                                                        \
                case 1: KERNEL<kPrecFp32, 1><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                case 2: KERNEL<kPrecFp32, 2><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                case 3: KERNEL<kPrecFp32, 3><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                case 5: KERNEL<kPrecFp32, 5><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                case 6: KERNEL<kPrecFp32, 6><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                default: KERNEL<kPrecFp32, 7><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
            }                                                                    \
        } else {                                                                 \
            switch (dk) {                                                        \
                case 1: KERNEL<kPrecFp64, 1><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                case 2: KERNEL<kPrecFp64, 2><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                case 3: KERNEL<kPrecFp64, 3><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                case 5: KERNEL<kPrecFp64, 5><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                case 6: KERNEL<kPrecFp64, 6><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
                default: KERNEL<kPrecFp64, 7><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break; \
            }                                                                    \
        }                                                                        \
    } while (0)

cudaError_t configure_kernels() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    return cudaSuccess;
}

cudaError_t launch_phase(int phase, const View& v, int precision, int j, int c, int init,
                         int stg_off, int advance, cudaStream_t s) {
    const int warp_blocks = (c * v.qlanes + 255) / 256;  // count passes
    switch (phase) {
        case kPhaseIngest:
            k_ingest<<<(c + 255) / 256, 256, 0, s>>>(v, j, c, init, stg_off);
            break;
        case kPhaseSort: {
            const int single = c <= kSortRun;  // one run: sorted straight into place, no run merge
            k_sort<<<dim3((c + kSortRun - 1) / kSortRun, init ? 1 : 2), kSortRun, 0, s>>>(v, j, c, init, single);
            if (single) break;
            ensure_runmerge_smem();
            k_runmerge<<<dim3((c + kSortRun - 1) / kSortRun, init ? 1 : 2), kSortRun,
                         sizeof(unsigned long long) * c, s>>>(v, j, c, init);
            break;
        }
        case kPhaseDecrement:
            if (!init) RTDBS_DISPATCH(precision, dk_of(v), k_decr, warp_blocks, 256, s, v, j, c);
            break;
        case kPhaseMerge:
            k_merge<<<(v.W + kMergeTile - 1) / kMergeTile, kMergeThreads, 0, s>>>(v, j, c, init);
            break;
        case kPhaseBuild:
            k_build<<<(v.W + kBuildThreads - 1) / kBuildThreads, kBuildThreads, 0, s>>>(v);
            break;
        case kPhaseIncrement:
            RTDBS_DISPATCH(precision, dk_of(v), k_incr, warp_blocks, 256, s, v, j, c, init);
            break;
        case kPhaseLabel:
            if (v.list_cap >= 0) {
                const int sms = g_num_sms > 0 ? g_num_sms : 152;
                k_border<<<max(1, min(sms * 8, (v.W + 255) / 256)), 256, 0, s>>>(v, advance);
                break;
            }
            [[fallthrough]];
        case kPhaseUnion: {
            const int sms = g_num_sms > 0 ? g_num_sms : 152;
            // queue-fed blocks: one warp per ~12 window points (a few items
            // each on sparse windows), all the SMs hold on large ones
            const int need = (v.W + 95) / 96;
            const int blocks = max(1, min(sms * 6, need));
            if (phase == kPhaseUnion)
                RTDBS_DISPATCH(precision, dk_of(v), k_union, max(1, min(sms * 8, need)), kClusterThreads, s, v);
            else
                RTDBS_DISPATCH(precision, dk_of(v), k_label, blocks, kClusterThreads, s, v, advance);
            break;
        }
        case kPhaseFlatten: {
            const int sms = g_num_sms > 0 ? g_num_sms : 152;
            RTDBS_DISPATCH(precision, dk_of(v), k_flatten, max(1, min(sms * 16, (v.W + 255) / 256)), 256, s, v);
            break;
        }
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_chunk_step(const View& v, int precision, int j, int c, int init, int stg_off,
                              cudaStream_t s, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join) {
    if (c <= 0 || c > kChunkMax) return cudaErrorInvalidValue;
    const bool beside = side && fork && join && !init;  // the decrement beside the sort
    for (int ph = 0; ph < kChunkPhases; ++ph) {
        cudaError_t e = cudaSuccess;
        if (beside && ph == kPhaseDecrement) continue;  // launched right after the ingest
        if (beside && ph == kPhaseMerge && (e = cudaStreamWaitEvent(s, join, 0)) != cudaSuccess) return e;
        e = launch_phase(ph, v, precision, j, c, init, stg_off, 0, s);
        if (e != cudaSuccess) return e;
        if (beside && ph == kPhaseIngest) {
            if ((e = cudaEventRecord(fork, s)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(side, fork, 0)) != cudaSuccess) return e;
            if ((e = launch_phase(kPhaseDecrement, v, precision, j, c, init, stg_off, 0, side)) != cudaSuccess)
                return e;
            if ((e = cudaEventRecord(join, side)) != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

cudaError_t launch_cluster(const View& v, int precision, int advance, cudaStream_t s, bool fresh_hints,
                           cudaEvent_t outputs_free, unsigned wait_flags) {
    cudaError_t e = cudaSuccess;
    if (fresh_hints) {
        const int sms = g_num_sms > 0 ? g_num_sms : 152;
        k_hints<<<max(1, min(sms * 8, (v.W + 255) / 256)), 256, 0, s>>>(v);
        e = cudaGetLastError();
    }
    for (int ph = kPhaseUnion; ph <= kPhaseLabel && e == cudaSuccess; ++ph) {
        if (ph == kPhaseLabel && outputs_free) e = cudaStreamWaitEvent(s, outputs_free, wait_flags);
        if (e == cudaSuccess) e = launch_phase(ph, v, precision, 0, 0, 0, 0, advance, s);
    }
    return e;
}

int batch_threads(int phase) {
    switch (phase) {
        case kBatchSort:
        case kBatchRunmerge: return kSortRun;
        case kBatchMerge: return kMergeThreads;
        case kBatchBuild: return kBuildThreads;
        case kBatchUnion:
        case kBatchLabel: return kClusterThreads;
        default: return 256;
    }
}

int batch_blocks(int phase, const View& v, int c) {
    const int runs = (c + kSortRun - 1) / kSortRun;
    switch (phase) {
        case kBatchIngest: return (c + 255) / 256;
        case kBatchSort:
        case kBatchRunmerge: return 2 * runs;
        case kBatchDecrement:
        case kBatchIncrement: return (c * v.qlanes + 255) / 256;
        case kBatchMerge: return (v.W + kMergeTile - 1) / kMergeTile;
        case kBatchBuild: return (v.W + kBuildThreads - 1) / kBuildThreads;
        case kBatchDamage: return 0;  // marked in the ingest and the decrement
        case kBatchReuse: return 0;  // start hints set by the merge and the increment
        case kBatchUnion: return max(1, min(1024, (v.W + 1023) / 1024));  // persistent, queue-fed
        case kBatchLabel:
            if (v.list_cap >= 0) return max(1, min(1024, (v.W + 1023) / 1024));  // k_border
            return max(1, min(1024, (v.W + 4095) / 4096));  // persistent, queue-fed
        case kBatchFlatten: return max(1, min(1024, (v.W + 2047) / 2048));
        default: return 0;
    }
}

bool batch_phase_split(int phase) {
    return phase == kBatchDecrement || phase == kBatchIncrement || phase == kBatchUnion ||
           phase == kBatchFlatten || phase == kBatchLabel;
}

#define RTDBS_BATCH_MD(PH, GRID, BLOCK, STREAM)                                      \
    do {                                                                           \
        const int dk = dim;                                                        \
        if (prec == kPrecFp32) {                                                   \
            switch (dk) {                                                          \
                case 1: k_batch<PH, kPrecFp32, 1><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                case 2: k_batch<PH, kPrecFp32, 2><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                case 3: k_batch<PH, kPrecFp32, 3><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                case 5: k_batch<PH, kPrecFp32, 5><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                case 6: k_batch<PH, kPrecFp32, 6><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                default: k_batch<PH, kPrecFp32, 7><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
            }                                                                      \
        } else {                                                                   \
            switch (dk) {                                                          \
                case 1: k_batch<PH, kPrecFp64, 1><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                case 2: k_batch<PH, kPrecFp64, 2><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                case 3: k_batch<PH, kPrecFp64, 3><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                case 5: k_batch<PH, kPrecFp64, 5><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                case 6: k_batch<PH, kPrecFp64, 6><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
                default: k_batch<PH, kPrecFp64, 7><<<GRID, BLOCK, 0, STREAM>>>(L); break; \
            }                                                                      \
        }                                                                          \
    } while (0)

cudaError_t launch_batch(int phase, int prec, int dim, const BatchLaunch& L, int total_blocks, int max_c,
                         cudaStream_t s) {
    if (total_blocks <= 0 || L.n <= 0) return cudaSuccess;
    const int t = batch_threads(phase);
    switch (phase) {
        case kBatchIngest: k_batch<kBatchIngest, 0, 0><<<total_blocks, t, 0, s>>>(L); break;
        case kBatchSort: k_batch<kBatchSort, 0, 0><<<total_blocks, t, 0, s>>>(L); break;
        case kBatchRunmerge:
            ensure_runmerge_smem();
            k_batch<kBatchRunmerge, 0, 0><<<total_blocks, t, sizeof(unsigned long long) * max_c, s>>>(L);
            break;
        case kBatchMerge: k_batch<kBatchMerge, 0, 0><<<total_blocks, t, 0, s>>>(L); break;
        case kBatchBuild: k_batch<kBatchBuild, 0, 0><<<total_blocks, t, 0, s>>>(L); break;
        case kBatchDecrement: RTDBS_BATCH_MD(kBatchDecrement, total_blocks, t, s); break;
        case kBatchIncrement: RTDBS_BATCH_MD(kBatchIncrement, total_blocks, t, s); break;
        case kBatchDamage: break;  // no kernel: marked in the ingest and the decrement
        case kBatchReuse: break;  // no kernel: start hints set by the merge and the increment
        case kBatchUnion: RTDBS_BATCH_MD(kBatchUnion, total_blocks, t, s); break;
        case kBatchFlatten: RTDBS_BATCH_MD(kBatchFlatten, total_blocks, t, s); break;
        case kBatchLabel: RTDBS_BATCH_MD(kBatchLabel, total_blocks, t, s); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Copies n separate point arrays into one packed buffer: block (x, y) moves
// part of array y.
__global__ void k_gather(const float* const* src, const long long* dst_off, const int* count, float* dst) {
    const int y = blockIdx.y;
    const float* a = src[y];
    float* d = dst + dst_off[y];
    const int n = count[y];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = a[i];
}

cudaError_t launch_gather(const float* const* src, const long long* dst_off, const int* count, float* dst,
                          int n, int max_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int bx = max(1, min(64, (max_count + 1023) / 1024));
    k_gather<<<dim3(bx, n), 1024, 0, s>>>(src, dst_off, count, dst);
    return cudaGetLastError();
}

cudaError_t launch_counts_by_slot(const View& v, int* nn, cudaStream_t s) {
    const int sms = g_num_sms > 0 ? g_num_sms : 152;
    k_counts_by_slot<<<sms * 4, 256, 0, s>>>(v, nn);
    return cudaGetLastError();
}

}  // namespace rtdbs
