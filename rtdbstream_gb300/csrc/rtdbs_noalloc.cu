// rtdbs_noalloc.cu -- clustering of one window of points with no device
// memory allocation (rtdbs_cluster_window_noalloc in include/rtdbs.h).
//
// Some callers cannot call cudaMalloc: a host process (a database engine or
// stream processor, say) that reserves the GPU's memory for its own pool at
// start-up and forbids raw allocations by plug-ins, or a caller on a latency
// path where cudaMalloc's implicit device synchronisation is unacceptable.
// For them this entry point runs the same kernels as rtdbs_load_window +
// rtdbs_cluster on at most RTDBS_NOALLOC_MAX_POINTS points, with all of its
// working memory in one file-scope __device__ array (below).  That array is
// part of the library image: every GPU that loads the library holds it until
// the process exits.  The caller passes the input points and the two output
// arrays (device memory); nothing else is allocated, by us or by a library.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "rtdbs.h"
#include "rtdbs_internal.h"

namespace {

using rtdbs::Ctl;
using rtdbs::View;

constexpr int kMaxPoints = RTDBS_NOALLOC_MAX_POINTS;
static_assert(kMaxPoints <= rtdbs::kChunkMax, "one grid-update chunk must hold the window");
constexpr unsigned long long kTableSlots = 32768;  // power of two >= 2 * kMaxPoints
static_assert(kTableSlots >= 2ull * kMaxPoints, "table capacity");
constexpr int kMaxItems = kMaxPoints + kMaxPoints / 32 + 64;

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Byte offsets of every buffer inside the scratch array.
constexpr size_t kOffRing = 0;
constexpr size_t kOffKslot = kOffRing + align256(sizeof(float4) * kMaxPoints);
constexpr size_t kOffSkey0 = kOffKslot + align256(sizeof(unsigned long long) * kMaxPoints);
constexpr size_t kOffSkey1 = kOffSkey0 + align256(sizeof(unsigned long long) * kMaxPoints);
constexpr size_t kOffSpt0 = kOffSkey1 + align256(sizeof(unsigned long long) * kMaxPoints);
constexpr size_t kOffSpt1 = kOffSpt0 + align256(sizeof(float4) * kMaxPoints);
constexpr size_t kOffScnt0 = kOffSpt1 + align256(sizeof(float4) * kMaxPoints);
constexpr size_t kOffScnt1 = kOffScnt0 + align256(sizeof(int) * kMaxPoints);
constexpr size_t kOffTable0 = kOffScnt1 + align256(sizeof(int) * kMaxPoints);
constexpr size_t kOffTable1 = kOffTable0 + align256(sizeof(ulonglong2) * kTableSlots);
constexpr size_t kOffItems = kOffTable1 + align256(sizeof(ulonglong2) * kTableSlots);
constexpr size_t kOffParent = kOffItems + align256(sizeof(int2) * kMaxItems);
constexpr size_t kOffSroot = kOffParent + align256(sizeof(int) * kMaxPoints);
constexpr size_t kOffNsort = kOffSroot + align256(sizeof(int) * kMaxPoints);
constexpr size_t kOffXsort = kOffNsort + align256(sizeof(unsigned long long) * kMaxPoints);
constexpr size_t kOffNword = kOffXsort + align256(sizeof(unsigned long long) * kMaxPoints);
constexpr size_t kOffXword = kOffNword + align256(sizeof(unsigned long long) * kMaxPoints);
constexpr size_t kOffXpt = kOffXword + align256(sizeof(unsigned long long) * kMaxPoints);
constexpr size_t kOffBox = kOffXpt + align256(sizeof(float4) * kMaxPoints);
constexpr size_t kOffCtl = kOffBox + align256(sizeof(float) * 6);
constexpr size_t kScratchBytes = kOffCtl + align256(sizeof(Ctl));  // about 3.4 MB

// The working memory.  In host code this name is only a host-side stand-in
// for the device array: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};

// Per-axis finite minimum and maximum of the points, written to box[0..5]
// (min x, y, z, max x, y, z); one block.
__global__ void k_noalloc_bbox(const float* pts, int n, int dim, float* box) {
    __shared__ float lo[3][32], hi[3][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int a = 0; a < 3; ++a) {
        float l = INFINITY, h = -INFINITY;
        if (a < dim) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const float x = pts[(size_t)i * dim + a];
                if (isfinite(x)) {
                    l = fminf(l, x);
                    h = fmaxf(h, x);
                }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            l = fminf(l, __shfl_xor_sync(0xffffffffu, l, o));
            h = fmaxf(h, __shfl_xor_sync(0xffffffffu, h, o));
        }
        if (lane == 0) {
            lo[a][w] = l;
            hi[a][w] = h;
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        float l = INFINITY, h = -INFINITY;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            l = fminf(l, lo[a][k]);
            h = fmaxf(h, hi[a][k]);
        }
        if (!(l <= h)) l = h = 0.0f;  // no finite coordinate on this axis
        box[a] = l;
        box[3 + a] = h;
    }
}

// Device address of g_scratch on the current device (set up on the first
// call per device, with that device current).
int scratch_for_current_device(unsigned char** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return rtdbs::set_error(RTDBS_ERR_NO_DEVICE, "noalloc: no current CUDA device (or ordinal >= %d)",
                                kMaxDevices);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p)
            return rtdbs::set_error(RTDBS_ERR_CUDA, "noalloc: cudaGetSymbolAddress of the scratch array failed: %s",
                                    cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return RTDBS_OK;
}

// Argument checks shared by both entry points.
int check_args(const float* d_points, int n, int dim, double eps, int precision, const int32_t* d_label,
               const int32_t* d_cluster_id) {
    using rtdbs::set_error;
    if (n > 0 && (!d_points || !d_label || !d_cluster_id))  // (an empty window touches none of them)
        return set_error(RTDBS_ERR_INVALID, "noalloc: points, label and cluster_id must not be NULL");
    if (n < 0 || n > kMaxPoints)  // beyond the scratch array
        return set_error(RTDBS_ERR_INVALID, "noalloc: n = %d outside 0..%d (RTDBS_NOALLOC_MAX_POINTS)", n,
                         kMaxPoints);
    if (dim < 1 || dim > 3) return set_error(RTDBS_ERR_INVALID, "noalloc: dim must be 1..3 (got %d)", dim);
    if (!(eps > 0.0) || !std::isfinite(eps))
        return set_error(RTDBS_ERR_INVALID, "noalloc: eps must be finite and > 0");
    if (precision != RTDBS_PREC_FP64 && precision != RTDBS_PREC_FP32)
        return set_error(RTDBS_ERR_INVALID, "noalloc: unknown precision mode %d", precision);
    return RTDBS_OK;
}

// The View of a window of n points in the scratch array at `base`, with the
// grid over [bmin, bmax] (widened by 25% when `widen`).
int window_view(View& v, unsigned char* base, const float* d_points, int n, int dim, double eps, int min_pts,
                int precision, const float* bmin, const float* bmax, bool widen, int32_t* d_label,
                int32_t* d_cluster_id) {
    std::memset(&v, 0, sizeof(v));
    v.dim = dim;
    v.cell_mult = 1;
    v.grab = 0;  // the default work split for the window's size
    v.qlanes = rtdbs::kQueryLanes;
    v.W = n;
    v.S = n;
    v.units = 1;
    v.min_pts = min_pts;
    v.chunk = n;
    v.precision = precision;
    rtdbs::set_band(v, eps);
    const int rc = rtdbs::set_geometry(v, dim, eps, 1, bmin, bmax, widen, nullptr);
    if (rc != RTDBS_OK) return rc;
    v.pbits = 15;
    v.pmask = (unsigned)(kTableSlots - 1);
    v.max_items = kMaxItems;
    v.list_cap = -1;  // no neighbour lists: the label pass scans the grid
    v.list_stride = 0;
    v.nlist = v.ntrack = v.rslot = v.damaged = v.sorder = nullptr;

    v.ring = reinterpret_cast<float4*>(base + kOffRing);
    v.kslot = reinterpret_cast<unsigned long long*>(base + kOffKslot);
    v.skey[0] = reinterpret_cast<unsigned long long*>(base + kOffSkey0);
    v.skey[1] = reinterpret_cast<unsigned long long*>(base + kOffSkey1);
    v.spt[0] = reinterpret_cast<float4*>(base + kOffSpt0);
    v.spt[1] = reinterpret_cast<float4*>(base + kOffSpt1);
    v.scnt[0] = reinterpret_cast<int*>(base + kOffScnt0);
    v.scnt[1] = reinterpret_cast<int*>(base + kOffScnt1);
    v.table[0] = reinterpret_cast<ulonglong2*>(base + kOffTable0);
    v.table[1] = reinterpret_cast<ulonglong2*>(base + kOffTable1);
    v.items = reinterpret_cast<int2*>(base + kOffItems);
    v.parent = reinterpret_cast<int*>(base + kOffParent);
    v.sroot = reinterpret_cast<int*>(base + kOffSroot);
    v.label = d_label;
    v.cid = d_cluster_id;
    v.nsort = reinterpret_cast<unsigned long long*>(base + kOffNsort);
    v.xsort = reinterpret_cast<unsigned long long*>(base + kOffXsort);
    v.nword = reinterpret_cast<unsigned long long*>(base + kOffNword);
    v.xword = reinterpret_cast<unsigned long long*>(base + kOffXword);
    v.xpt = reinterpret_cast<float4*>(base + kOffXpt);
    v.staging = d_points;  // the caller's points are read in place
    v.ctl = reinterpret_cast<Ctl*>(base + kOffCtl);
    return RTDBS_OK;
}

// Every call reuses the array, which still holds the previous call's data:
// the cell tables (generation tags) and the control block must start at
// zero; everything else is rewritten before it is read.
cudaError_t reset_scratch(unsigned char* base, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(base + kOffTable0, 0, sizeof(ulonglong2) * kTableSlots * 2, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + kOffCtl, 0, sizeof(Ctl), s);
    return e;
}

}  // namespace

extern "C" RTDBS_API int rtdbs_cluster_window_noalloc(const float* d_points, int32_t n, int32_t dim,
                                                      double eps, int32_t min_pts, int32_t precision,
                                                      int32_t* d_label, int32_t* d_cluster_id,
                                                      void* cuda_stream) {
    using rtdbs::set_error;
    int rc = check_args(d_points, n, dim, eps, precision, d_label, d_cluster_id);
    if (rc != RTDBS_OK) return rc;
    if (n == 0) return RTDBS_OK;
    unsigned char* base = nullptr;
    rc = scratch_for_current_device(&base);
    if (rc != RTDBS_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);

    // Once work is queued on s, an error return first waits for it, so that
    // an error also means the scratch array is no longer in use.
    bool queued = false;
#define NOALLOC_TRY(expr)                                                                              \
    do {                                                                                               \
        const cudaError_t _e = (expr);                                                                 \
        if (_e != cudaSuccess) {                                                                       \
            if (queued) cudaStreamSynchronize(s);                                                      \
            return set_error(RTDBS_ERR_CUDA, "noalloc: %s failed: %s", #expr, cudaGetErrorString(_e)); \
        }                                                                                              \
    } while (0)

    queued = true;
    NOALLOC_TRY(reset_scratch(base, s));

    // Bounding box -> grid geometry (same rules as an engine without a box):
    // the box comes back to the host, the one wait inside the call
    // (rtdbs_cluster_window_noalloc_async takes the box from the caller and
    // does not wait at all).
    float* d_box = reinterpret_cast<float*>(base + kOffBox);
    k_noalloc_bbox<<<1, 1024, 0, s>>>(d_points, n, dim, d_box);
    NOALLOC_TRY(cudaGetLastError());
    float box[6];
    NOALLOC_TRY(cudaMemcpyAsync(box, d_box, sizeof(box), cudaMemcpyDeviceToHost, s));
    NOALLOC_TRY(cudaStreamSynchronize(s));

    View v;
    rc = window_view(v, base, d_points, n, dim, eps, min_pts, precision, box, box + 3, true, d_label,
                     d_cluster_id);
    if (rc != RTDBS_OK) return rc;  // nothing is queued after the wait above

    NOALLOC_TRY(rtdbs::launch_chunk_step(v, precision, 0, n, 1, 0, s));
    NOALLOC_TRY(rtdbs::launch_cluster(v, precision, 0, s));
    int err = 0;
    NOALLOC_TRY(cudaMemcpyAsync(&err, &v.ctl->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    NOALLOC_TRY(cudaStreamSynchronize(s));
#undef NOALLOC_TRY
    if (err)
        return set_error(RTDBS_ERR_DEVICE, "noalloc: device error bits 0x%x (1 table full, 2 union-find bound, "
                         "4 work list full, 8 chunk bookkeeping)", err);
    return RTDBS_OK;
}

extern "C" RTDBS_API int rtdbs_cluster_window_noalloc_async(const float* d_points, int32_t n, int32_t dim,
                                                            double eps, int32_t min_pts, int32_t precision,
                                                            const float* box_min, const float* box_max,
                                                            int32_t* d_label, int32_t* d_cluster_id,
                                                            int32_t* d_status, void* cuda_stream) {
    using rtdbs::set_error;
    int rc = check_args(d_points, n, dim, eps, precision, d_label, d_cluster_id);
    if (rc != RTDBS_OK) return rc;
    if (!box_min || !box_max || !d_status)
        return set_error(RTDBS_ERR_INVALID, "noalloc: box_min, box_max and status must not be NULL");
    unsigned char* base = nullptr;
    rc = scratch_for_current_device(&base);
    if (rc != RTDBS_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    View v;
    // geometry first: a bad box returns before anything is queued
    rc = window_view(v, base, d_points, n > 0 ? n : 1, dim, eps, min_pts, precision, box_min, box_max, false,
                     d_label, d_cluster_id);
    if (rc != RTDBS_OK) return rc;
#define NOALLOC_TRY(expr)                                                                              \
    do {                                                                                               \
        const cudaError_t _e = (expr);                                                                 \
        if (_e != cudaSuccess)                                                                         \
            return set_error(RTDBS_ERR_CUDA, "noalloc: %s failed: %s", #expr, cudaGetErrorString(_e)); \
    } while (0)
    if (n == 0) {
        NOALLOC_TRY(cudaMemsetAsync(d_status, 0, sizeof(int32_t), s));
        return RTDBS_OK;
    }
    NOALLOC_TRY(reset_scratch(base, s));
    NOALLOC_TRY(rtdbs::launch_chunk_step(v, precision, 0, n, 1, 0, s));
    NOALLOC_TRY(rtdbs::launch_cluster(v, precision, 0, s));
    NOALLOC_TRY(cudaMemcpyAsync(d_status, &v.ctl->err, sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
#undef NOALLOC_TRY
    return RTDBS_OK;
}
