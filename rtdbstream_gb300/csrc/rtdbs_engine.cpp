// rtdbs_engine.cpp -- host side of the C ABI declared in include/rtdbs.h.
//
// The engine replaces the reference's ScanState + dbscan() slide loop
// (src/dbscan/state.h:23-129, src/dbscan/dbscan.cpp:2258-2364): all device
// buffers are allocated once at creation (initialize_params,
// src/dbscan/dbscan.cpp:30-132), every per-slide size stays on the device
// (the reference reads three counts back per slide,
// src/dbscan/dbscan.cpp:549,561-562), and a slide is one CUDA-graph replay.
#include "rtdbs.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "rtdbs_internal.h"

using rtdbs::Ctl;
using rtdbs::View;

namespace {

thread_local std::string g_last_error;

int vfail(int status, const char* fmt, va_list ap) {
    char buf[512];
    vsnprintf(buf, sizeof(buf), fmt, ap);
    g_last_error = buf;
    return status;
}

int fail(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    const int r = vfail(status, fmt, ap);
    va_end(ap);
    return r;
}

#define CUDA_TRY(expr)                                                                  \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess)                                                          \
            return fail(_e == cudaErrorMemoryAllocation ? RTDBS_ERR_OOM : RTDBS_ERR_CUDA, \
                        "%s failed: %s", #expr, cudaGetErrorString(_e));                \
    } while (0)

// Restores the caller's current device on scope exit.
struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int dev) {
        err = cudaGetDevice(&prev);
        if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

std::mutex g_cfg_mutex;
std::vector<char> g_configured;

cudaError_t configure_device(int dev) {
    std::lock_guard<std::mutex> lock(g_cfg_mutex);
    if ((int)g_configured.size() <= dev) g_configured.resize(dev + 1, 0);
    if (g_configured[dev]) return cudaSuccess;
    cudaError_t e = rtdbs::configure_kernels();
    if (e == cudaSuccess) g_configured[dev] = 1;
    return e;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

namespace rtdbs {

int set_error(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    const int r = vfail(status, fmt, ap);
    va_end(ap);
    return r;
}

// Cell side L = Eps (1 + 2^-12) / K with K cells per Eps (the margin covers
// the rounding of both predicates and of the double cell coordinate, so
// neighbours are at most K cells apart per axis), clamped extents over the
// bounding box, one bit field per axis in the key, L doubled until the
// fields fit 50 bits.
int set_geometry(View& v, int dim, double eps, int cells_per_eps, const float* bmin, const float* bmax,
                 bool widen, double* cell_side) {
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    double L = eps * (1.0 + 1.0 / 4096.0) / cells_per_eps;
    for (int a = 0; a < dim; ++a) {
        lo[a] = bmin[a];
        hi[a] = bmax[a];
        if (!(lo[a] <= hi[a]) || !std::isfinite(lo[a]) || !std::isfinite(hi[a]))
            return fail(RTDBS_ERR_INVALID, "bounding box of axis %d is empty or not finite", a);
        if (widen) {
            const double m = std::max(0.25 * (hi[a] - lo[a]), 4.0 * L);
            lo[a] -= m;
            hi[a] += m;
        }
    }
    long long ext[3] = {1, 1, 1};
    int bits[3] = {0, 0, 0};
    for (int guard = 0; guard < 4096; ++guard) {
        int total = 0;
        for (int a = 0; a < dim; ++a) {
            const double n = std::floor((hi[a] - lo[a]) / L) + 1.0;
            ext[a] = n < 4.0e15 ? (long long)n : (long long)4.0e15;
            bits[a] = 0;
            while (bits[a] < 62 && (1ll << bits[a]) < ext[a]) ++bits[a];
            total += bits[a];
        }
        if (total <= kKeyBitsMax) break;
        L *= 2.0;
    }
    for (int a = 0; a < 3; ++a) {
        v.origin[a] = lo[a];
        v.ext[a] = ext[a];
    }
    v.shift[2] = 0;
    v.shift[1] = bits[2];
    v.shift[0] = bits[1] + bits[2];
    const int kbits = bits[0] + bits[1] + bits[2];
    v.inv_cell = 1.0 / L;
    v.key_bits = kbits;
    v.sort_passes = (kbits + 7) / 8;
    if (cell_side) *cell_side = L;
    return RTDBS_OK;
}

// FP32 filter band of the FP64 predicate: [E(1 - 2^-20), E(1 + 2^-20)] rounded
// outward to float.  The float evaluation of three rounded squares of rounded
// differences has relative error <= gamma_5 ~ 3.0e-7 (Higham, Accuracy and
// Stability of Numerical Algorithms, 2nd ed., Lemma 3.1); outside the band the
// float value decides exactly as the double one would.
void set_band(View& v, double eps) {
    const double E = eps * eps;
    const double m = 1.0 / 1048576.0;
    const double lo = E * (1.0 - m), hi = E * (1.0 + m);
    float flo = (float)lo, fhi = (float)hi;
    if ((double)flo > lo) flo = std::nextafter(flo, 0.0f);
    if ((double)fhi < hi) fhi = std::nextafter(fhi, INFINITY);
    v.lo = flo;
    v.hi = fhi;
    v.E = E;
    v.filter_ok = (E >= std::ldexp(1.0, -100) && E <= std::ldexp(1.0, 100)) ? 1 : 0;
    const float r = (float)eps;
    v.r2f = r * r;
}

}  // namespace rtdbs

struct rtdbs_engine {
    rtdbs_params p{};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    View v{};
    int chunk = 0;           // C
    int staging_points = 0;  // capacity of the staging buffer in points
    void* dev_block = nullptr;
    size_t dev_bytes = 0;
    Ctl* h_ctl = nullptr;    // pinned mirror of the control block
    bool geometry_ready = false;
    bool loaded = false;
    cudaGraphExec_t slide_graph = nullptr;
    cudaGraphExec_t pipe_graph = nullptr;  // the slide of rtdbs_slide_pipelined
    // side stream for the decrement pass beside the sort (made on the first slide)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    double cell_side = 0.0;
    // rtdbs_slide_pipelined: the outputs go to the host on their own stream
    // (`copy`) while the next slide runs; ev_done marks a slide's end on the
    // engine's stream, ev_free the end of its output copies, which every
    // slide's label pass waits for (a wait node in the captured graph);
    // ev_pipe marks the last two pipelined slides complete, and
    // pipe_pending says whether one is still in flight
    cudaStream_t copy = nullptr;
    cudaEvent_t ev_done = nullptr, ev_free = nullptr;
    cudaEvent_t ev_pipe[2] = {nullptr, nullptr};
    int pipe_next = 0;
    bool pipe_pending = false;
};

namespace {

// The engine's geometry: the box given in its parameters, or that of its
// first window (widened).
int engine_geometry(rtdbs_engine* e, const float* bmin, const float* bmax, bool widen) {
    const int K = e->p.cell_mult > 0 ? e->p.cell_mult : 1;
    const int rc = rtdbs::set_geometry(e->v, e->p.dim, e->p.eps, K, bmin, bmax, widen, &e->cell_side);
    if (rc == RTDBS_OK) e->geometry_ready = true;
    return rc;
}

struct Part {
    void** ptr;
    size_t bytes;
};

// Buffer layout of one engine (sizes from W, S, dim); returns the bytes of
// the single device block that holds it.
size_t plan_layout(rtdbs_engine* e, std::vector<Part>& parts) {
    const int W = e->p.window, S = e->p.stride, dim = e->p.dim;
    View& v = e->v;
    e->chunk = std::min(S, rtdbs::kChunkMax);
    const int load_chunk = std::min(W, rtdbs::kChunkMax);
    const int C = std::max(e->chunk, load_chunk);
    e->staging_points = std::max(S, load_chunk);
    unsigned long long P = 1024;
    int pbits = 10;
    while (P < 2ull * (unsigned long long)W) {
        P <<= 1;
        ++pbits;
    }
    v.pbits = pbits;
    v.pmask = (unsigned)(P - 1);
    // work items: cell runs cut at 32 points, at 8 below 65,536 points (a small
    // window is a few waves of items at most, so its densest cells must not
    // be one warp's long chain)
    v.item_pts = W < 65536 ? 8 : 32;
    v.max_items = W + W / v.item_pts + 64;
    // Neighbour lists of non-core points (MinPts - 2 entries each) replace the
    // label pass's grid scan up to kListCap entries; above that the scan stays.
    const int mp = e->p.min_pts;
    v.list_cap = (mp >= 2 && mp - 2 <= rtdbs::kListCap) ? mp - 2 : -1;
    v.list_stride = v.list_cap > 0 ? (v.list_cap + 3) / 4 * 4 : 0;
    const size_t list_ints = (size_t)W * v.list_stride;
    const size_t track_ints = v.list_cap >= 0 ? (size_t)W : 0;
    v.nlist = v.ntrack = v.rslot = v.damaged = nullptr;
    v.sprev[0] = v.sprev[1] = nullptr;
    parts = {
        {(void**)&v.ring, sizeof(float4) * W},
        {(void**)&v.kslot, sizeof(unsigned long long) * W},
        {(void**)&v.skey[0], sizeof(unsigned long long) * W},
        {(void**)&v.skey[1], sizeof(unsigned long long) * W},
        {(void**)&v.spt[0], sizeof(float4) * W},
        {(void**)&v.spt[1], sizeof(float4) * W},
        {(void**)&v.scnt[0], sizeof(int) * W},
        {(void**)&v.scnt[1], sizeof(int) * W},
        {(void**)&v.table[0], sizeof(ulonglong2) * P},
        {(void**)&v.table[1], sizeof(ulonglong2) * P},
        {(void**)&v.items, sizeof(int2) * v.max_items},
        {(void**)&v.parent, sizeof(int) * W},
        {(void**)&v.sroot, sizeof(int) * W},
        {(void**)&v.label, sizeof(int) * W},
        {(void**)&v.cid, sizeof(int) * W},
        {(void**)&v.nlist, sizeof(int) * list_ints},
        {(void**)&v.ntrack, sizeof(int) * track_ints},
        {(void**)&v.rslot, sizeof(int) * track_ints},
        {(void**)&v.damaged, sizeof(int) * track_ints},
        {(void**)&v.sprev[0], sizeof(int) * track_ints},
        {(void**)&v.sprev[1], sizeof(int) * track_ints},
        {(void**)&v.nsort, sizeof(unsigned long long) * C},
        {(void**)&v.xsort, sizeof(unsigned long long) * C},
        {(void**)&v.nword, sizeof(unsigned long long) * C},
        {(void**)&v.xword, sizeof(unsigned long long) * C},
        {(void**)&v.xpt, sizeof(float4) * C},
        {(void**)&v.sorder, sizeof(int) * W},
        {(void**)&v.staging, sizeof(float) * (size_t)e->staging_points * dim},
        {(void**)&v.ctl, sizeof(Ctl)},
    };
    size_t total = 0;
    for (auto& q : parts) total += align_up(q.bytes, 256);
    return total;
}

int allocate(rtdbs_engine* e) {
    std::vector<Part> parts;
    const size_t total = plan_layout(e, parts);
    View& v = e->v;
    const unsigned long long P = (unsigned long long)v.pmask + 1;
    CUDA_TRY(cudaMalloc(&e->dev_block, total));
    e->dev_bytes = total;
    char* base = static_cast<char*>(e->dev_block);
    for (auto& q : parts) {
        *q.ptr = q.bytes ? base : nullptr;  // a buffer this stream does not use stays null
        base += align_up(q.bytes, 256);
    }
    CUDA_TRY(cudaMemsetAsync(v.table[0], 0, sizeof(ulonglong2) * P, e->stream));
    CUDA_TRY(cudaMemsetAsync(v.table[1], 0, sizeof(ulonglong2) * P, e->stream));
    CUDA_TRY(cudaMemsetAsync(v.ctl, 0, sizeof(Ctl), e->stream));
    CUDA_TRY(cudaMallocHost((void**)&e->h_ctl, sizeof(Ctl)));
    std::memset(e->h_ctl, 0, sizeof(Ctl));
    return RTDBS_OK;
}

int check_device_error(rtdbs_engine* e) {
    if (e->h_ctl->err)
        return fail(RTDBS_ERR_DEVICE, "device error bits 0x%x (1 table full, 2 union-find bound, "
                    "4 work list full, 8 chunk bookkeeping, 16 neighbour lists)", e->h_ctl->err);
    return RTDBS_OK;
}

// (pipelined: the label pass first waits for the last output copies; while
// capturing, that wait becomes an external-event wait node of the graph)
int enqueue_slide(rtdbs_engine* e, bool capturing, bool pipelined) {
    const int S = e->p.stride, C = e->chunk;
    const int nchunks = (S + C - 1) / C;
    for (int j = 0; j < nchunks; ++j) {
        const int c = std::min(C, S - j * C);
        CUDA_TRY(rtdbs::launch_chunk_step(e->v, e->p.precision, j, c, 0, j * C, e->stream, e->side, e->ev_fork,
                                          e->ev_join));
    }
    CUDA_TRY(rtdbs::launch_cluster(e->v, e->p.precision, 1, e->stream, false, pipelined ? e->ev_free : nullptr,
                                   capturing ? cudaEventWaitExternal : cudaEventWaitDefault));
    return RTDBS_OK;
}

// Orders later label writes (outside a slide graph) after the last output copies.
int wait_outputs_free(rtdbs_engine* e) {
    if (e->ev_free) CUDA_TRY(cudaStreamWaitEvent(e->stream, e->ev_free, 0));
    return RTDBS_OK;
}

// Enqueues one slide whose new points are already in the staging buffer.
int ensure_side(rtdbs_engine* e) {
    if (e->side) return RTDBS_OK;
    CUDA_TRY(cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&e->ev_done, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&e->ev_free, cudaEventDisableTiming));
    CUDA_TRY(cudaStreamCreateWithFlags(&e->copy, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking));
    return RTDBS_OK;
}

// One slide.  pipelined: the slide of rtdbs_slide_pipelined, whose label pass
// waits inside the graph for the previous slide's output copies (a graph of
// its own: the wait node costs small windows tens of microseconds per
// slide); any other slide waits for those copies, if one may still run,
// before it starts.
int run_slide(rtdbs_engine* e, bool pipelined = false) {
    int rc0 = ensure_side(e);  // before any capture
    if (rc0 != RTDBS_OK) return rc0;
    if (!pipelined && e->pipe_pending) {
        rc0 = wait_outputs_free(e);
        if (rc0 != RTDBS_OK) return rc0;
    }
    if (e->p.flags & RTDBS_FLAG_NO_GRAPH) return enqueue_slide(e, false, pipelined);
    cudaGraphExec_t& exec = pipelined ? e->pipe_graph : e->slide_graph;
    if (!exec) {
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_slide(e, true, pipelined);
        cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        if (rc != RTDBS_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        CUDA_TRY(ce);
        cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        CUDA_TRY(ie);
    }
    CUDA_TRY(cudaGraphLaunch(exec, e->stream));
    return RTDBS_OK;
}

int copy_in(rtdbs_engine* e, const float* src, size_t npts, int on_device) {
    const size_t bytes = sizeof(float) * npts * e->p.dim;
    CUDA_TRY(cudaMemcpyAsync((void*)e->v.staging, src, bytes,
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                             e->stream));
    return RTDBS_OK;
}

int copy_out(rtdbs_engine* e, int32_t* label, int32_t* cid, int on_device) {
    const size_t bytes = sizeof(int) * e->p.window;
    const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (label) CUDA_TRY(cudaMemcpyAsync(label, e->v.label, bytes, k, e->stream));
    if (cid) CUDA_TRY(cudaMemcpyAsync(cid, e->v.cid, bytes, k, e->stream));
    return RTDBS_OK;
}

int fetch_ctl_and_sync(rtdbs_engine* e) {
    CUDA_TRY(cudaMemcpyAsync(e->h_ctl, e->v.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    if (e->copy) CUDA_TRY(cudaStreamSynchronize(e->copy));
    e->pipe_pending = false;  // everything queued, pipelined slides included, is done
    return check_device_error(e);
}

}  // namespace

extern "C" {

int rtdbs_abi_version(void) { return RTDBS_ABI_VERSION; }

const char* rtdbs_status_string(int status) {
    switch (status) {
        case RTDBS_OK: return "ok";
        case RTDBS_ERR_INVALID: return "invalid argument";
        case RTDBS_ERR_CUDA: return "CUDA runtime error";
        case RTDBS_ERR_OOM: return "out of memory";
        case RTDBS_ERR_STATE: return "call out of order";
        case RTDBS_ERR_DEVICE: return "device-side bound hit";
        case RTDBS_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown status";
    }
}

const char* rtdbs_last_error(void) { return g_last_error.c_str(); }

int rtdbs_params_init(rtdbs_params* params) {
    if (!params) return fail(RTDBS_ERR_INVALID, "params is NULL");
    std::memset(params, 0, sizeof(*params));
    params->dim = 3;
    params->window = 0;
    params->stride = 0;
    params->min_pts = 5;
    params->eps = 0.0;
    params->precision = RTDBS_PREC_FP64;
    return RTDBS_OK;
}

int rtdbs_create(const rtdbs_params* params, void* cuda_stream, rtdbs_engine** out) {
    if (!params || !out) return fail(RTDBS_ERR_INVALID, "params/out is NULL");
    *out = nullptr;
    const rtdbs_params& p = *params;
    if (p.dim < 1 || p.dim > 3) return fail(RTDBS_ERR_INVALID, "dim must be 1..3 (got %d)", p.dim);
    if (p.window <= 0 || p.stride <= 0 || p.stride > p.window)
        return fail(RTDBS_ERR_INVALID, "need 0 < stride <= window (got W=%d S=%d)", p.window, p.stride);
    if (p.window % p.stride != 0)
        return fail(RTDBS_ERR_INVALID, "window %% stride must be 0 (got W=%d S=%d)", p.window, p.stride);
    if (p.window > (1 << 30)) return fail(RTDBS_ERR_INVALID, "window too large");
    if (!(p.eps > 0.0) || !std::isfinite(p.eps)) return fail(RTDBS_ERR_INVALID, "eps must be finite and > 0");
    if (p.precision != RTDBS_PREC_FP64 && p.precision != RTDBS_PREC_FP32)
        return fail(RTDBS_ERR_INVALID, "unknown precision mode %d", p.precision);
    if (p.cell_mult < 0 || p.cell_mult > 2)
        return fail(RTDBS_ERR_INVALID, "cell_mult must be 0 (default), 1 or 2 (got %d)", p.cell_mult);
    if (p.work_grab < 0 || p.work_grab > 64)
        return fail(RTDBS_ERR_INVALID, "work_grab must be 0 (default) or 1..64 (got %d)", p.work_grab);
    if (p.query_lanes != 0 && p.query_lanes != 16 && p.query_lanes != 32)
        return fail(RTDBS_ERR_INVALID, "query_lanes must be 0 (default), 16 or 32 (got %d)", p.query_lanes);
    if (p.cell_mult == 2 && p.query_lanes == 16)
        return fail(RTDBS_ERR_INVALID, "two cells per Eps need query_lanes 32 (or 0)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(RTDBS_ERR_NO_DEVICE, "no CUDA device available");
    if (p.device < 0 || p.device >= ndev) return fail(RTDBS_ERR_INVALID, "device %d out of range", p.device);

    DeviceGuard guard(p.device);
    CUDA_TRY(guard.err);
    CUDA_TRY(configure_device(p.device));
    rtdbs_engine* e = new (std::nothrow) rtdbs_engine();
    if (!e) return fail(RTDBS_ERR_OOM, "host allocation failed");
    e->p = p;
    e->device = p.device;
    if (cuda_stream) {
        e->stream = static_cast<cudaStream_t>(cuda_stream);
    } else {
        cudaError_t ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
        if (ce != cudaSuccess) {
            delete e;
            return fail(RTDBS_ERR_CUDA, "cudaStreamCreate failed: %s", cudaGetErrorString(ce));
        }
        e->own_stream = true;
    }
    View& v = e->v;
    v.dim = p.dim;
    v.cell_mult = p.cell_mult > 0 ? p.cell_mult : 1;
    v.grab = p.work_grab;  // 0: by launch kind and window size (work_grab in the kernels)
    v.qlanes = p.query_lanes > 0 ? p.query_lanes : (v.cell_mult == 1 ? rtdbs::kQueryLanes : 32);
    v.W = p.window;
    v.S = p.stride;
    v.min_pts = p.min_pts;
    v.units = p.window / p.stride;
    v.precision = p.precision;
    rtdbs::set_band(v, p.eps);
    int rc = allocate(e);
    if (rc == RTDBS_OK) {
        v.chunk = e->chunk;
        if (p.has_bbox) rc = engine_geometry(e, p.bbox_min, p.bbox_max, false);
    }
    if (rc != RTDBS_OK) {
        rtdbs_destroy(e);
        return rc;
    }
    *out = e;
    return RTDBS_OK;
}

int rtdbs_destroy(rtdbs_engine* e) {
    if (!e) return RTDBS_OK;
    DeviceGuard guard(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->slide_graph) cudaGraphExecDestroy(e->slide_graph);
    if (e->pipe_graph) cudaGraphExecDestroy(e->pipe_graph);
    if (e->dev_block) cudaFree(e->dev_block);
    if (e->h_ctl) cudaFreeHost(e->h_ctl);
    if (e->side) cudaStreamDestroy(e->side);
    if (e->copy) {
        cudaStreamSynchronize(e->copy);
        cudaStreamDestroy(e->copy);
    }
    if (e->ev_done) cudaEventDestroy(e->ev_done);
    if (e->ev_free) cudaEventDestroy(e->ev_free);
    if (e->ev_fork) cudaEventDestroy(e->ev_fork);
    for (auto& ev : e->ev_pipe)
        if (ev) cudaEventDestroy(ev);
    if (e->ev_join) cudaEventDestroy(e->ev_join);
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return RTDBS_OK;
}

int rtdbs_load_window(rtdbs_engine* e, const float* points, int points_on_device) {
    if (!e || !points) return fail(RTDBS_ERR_INVALID, "engine/points is NULL");
    DeviceGuard guard(e->device);
    CUDA_TRY(guard.err);
    const int W = e->p.window, dim = e->p.dim;
    if (!e->p.has_bbox) {
        std::vector<float> host;
        const float* h = points;
        if (points_on_device) {
            host.resize((size_t)W * dim);
            CUDA_TRY(cudaMemcpy(host.data(), points, sizeof(float) * host.size(), cudaMemcpyDeviceToHost));
            h = host.data();
        }
        float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
        for (int a = 0; a < dim; ++a) {
            float lo = INFINITY, hi = -INFINITY;
            for (int i = 0; i < W; ++i) {
                const float x = h[(size_t)i * dim + a];
                if (std::isfinite(x)) {
                    lo = std::min(lo, x);
                    hi = std::max(hi, x);
                }
            }
            if (!(lo <= hi)) lo = hi = 0.0f;
            mn[a] = lo;
            mx[a] = hi;
        }
        int rc = engine_geometry(e, mn, mx, true);
        if (rc != RTDBS_OK) return rc;
    }
    // Restart from an empty window.
    if (e->slide_graph) {
        cudaGraphExecDestroy(e->slide_graph);
        e->slide_graph = nullptr;
    }
    if (e->pipe_graph) {
        cudaGraphExecDestroy(e->pipe_graph);
        e->pipe_graph = nullptr;
    }
    CUDA_TRY(cudaMemsetAsync(e->v.ctl, 0, sizeof(Ctl), e->stream));
    CUDA_TRY(cudaMemsetAsync(e->v.table[0], 0, sizeof(ulonglong2) * ((size_t)e->v.pmask + 1), e->stream));
    CUDA_TRY(cudaMemsetAsync(e->v.table[1], 0, sizeof(ulonglong2) * ((size_t)e->v.pmask + 1), e->stream));
    const int C = std::min(W, rtdbs::kChunkMax);
    View v = e->v;
    v.chunk = C;  // load chunks tile the slots [0, W)
    for (int j = 0, off = 0; off < W; ++j, off += C) {
        const int c = std::min(C, W - off);
        int rc = copy_in(e, points + (size_t)off * dim, c, points_on_device);
        if (rc != RTDBS_OK) return rc;
        CUDA_TRY(rtdbs::launch_chunk_step(v, e->p.precision, j, c, 1, 0, e->stream));
    }
    int rc = fetch_ctl_and_sync(e);
    if (rc != RTDBS_OK) return rc;
    e->loaded = true;
    return RTDBS_OK;
}

int rtdbs_slide(rtdbs_engine* e, const float* new_points, int32_t* label, int32_t* cluster_id) {
    if (!e || !new_points) return fail(RTDBS_ERR_INVALID, "engine/new_points is NULL");
    if (!e->loaded) return fail(RTDBS_ERR_STATE, "rtdbs_load_window must come first");
    DeviceGuard guard(e->device);
    CUDA_TRY(guard.err);
    int rc = copy_in(e, new_points, e->p.stride, 0);
    if (rc == RTDBS_OK) rc = run_slide(e);
    if (rc == RTDBS_OK) rc = copy_out(e, label, cluster_id, 0);
    if (rc == RTDBS_OK) rc = fetch_ctl_and_sync(e);
    return rc;
}

int rtdbs_slide_async(rtdbs_engine* e, const float* d_new_points, int32_t* d_label,
                      int32_t* d_cluster_id) {
    if (!e || !d_new_points) return fail(RTDBS_ERR_INVALID, "engine/new_points is NULL");
    if (!e->loaded) return fail(RTDBS_ERR_STATE, "rtdbs_load_window must come first");
    DeviceGuard guard(e->device);
    CUDA_TRY(guard.err);
    int rc = RTDBS_OK;
    if (d_new_points != e->v.staging) rc = copy_in(e, d_new_points, e->p.stride, 1);
    if (rc == RTDBS_OK) rc = run_slide(e);
    if (rc == RTDBS_OK && (d_label || d_cluster_id)) rc = copy_out(e, d_label, d_cluster_id, 1);
    return rc;
}

int rtdbs_slide_pipelined(rtdbs_engine* e, const float* new_points, int32_t* label, int32_t* cluster_id) {
    if (!e || !new_points) return fail(RTDBS_ERR_INVALID, "engine/new_points is NULL");
    if (!e->loaded) return fail(RTDBS_ERR_STATE, "rtdbs_load_window must come first");
    DeviceGuard guard(e->device);
    CUDA_TRY(guard.err);
    for (auto& ev : e->ev_pipe)
        if (!ev) CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    int rc = copy_in(e, new_points, e->p.stride, 0);
    if (rc == RTDBS_OK) rc = run_slide(e, true);
    if (rc != RTDBS_OK) return rc;
    // the outputs (and the control block, whose error bits the call that
    // completes this slide reads) go to the host on the copy stream while
    // the next slide runs; its label pass waits for ev_free
    CUDA_TRY(cudaEventRecord(e->ev_done, e->stream));
    CUDA_TRY(cudaStreamWaitEvent(e->copy, e->ev_done, 0));
    const size_t bytes = sizeof(int) * e->p.window;
    if (label) CUDA_TRY(cudaMemcpyAsync(label, e->v.label, bytes, cudaMemcpyDeviceToHost, e->copy));
    if (cluster_id) CUDA_TRY(cudaMemcpyAsync(cluster_id, e->v.cid, bytes, cudaMemcpyDeviceToHost, e->copy));
    CUDA_TRY(cudaMemcpyAsync(e->h_ctl, e->v.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, e->copy));
    CUDA_TRY(cudaEventRecord(e->ev_free, e->copy));
    const int cur = e->pipe_next;
    CUDA_TRY(cudaEventRecord(e->ev_pipe[cur], e->copy));
    e->pipe_next = cur ^ 1;
    const bool wait_prev = e->pipe_pending;
    e->pipe_pending = true;
    if (!wait_prev) return RTDBS_OK;
    CUDA_TRY(cudaEventSynchronize(e->ev_pipe[cur ^ 1]));
    return check_device_error(e);
}

int rtdbs_sync(rtdbs_engine* e) {
    if (!e) return fail(RTDBS_ERR_INVALID, "engine is NULL");
    DeviceGuard guard(e->device);
    CUDA_TRY(guard.err);
    return fetch_ctl_and_sync(e);
}

int rtdbs_cluster(rtdbs_engine* e, int32_t* label, int32_t* cluster_id, int on_device) {
    if (!e) return fail(RTDBS_ERR_INVALID, "engine is NULL");
    if (!e->loaded) return fail(RTDBS_ERR_STATE, "rtdbs_load_window must come first");
    DeviceGuard guard(e->device);
    CUDA_TRY(guard.err);
    const int rc0 = wait_outputs_free(e);
    if (rc0 != RTDBS_OK) return rc0;
    CUDA_TRY(rtdbs::launch_cluster(e->v, e->p.precision, 0, e->stream, true));
    int rc = copy_out(e, label, cluster_id, on_device);
    if (rc == RTDBS_OK) rc = fetch_ctl_and_sync(e);
    return rc;
}

int rtdbs_get_counts(rtdbs_engine* e, int32_t* nn, int on_device) {
    if (!e || !nn) return fail(RTDBS_ERR_INVALID, "engine/nn is NULL");
    if (!e->loaded) return fail(RTDBS_ERR_STATE, "rtdbs_load_window must come first");
    DeviceGuard guard(e->device);
    CUDA_TRY(guard.err);
    if (on_device) {
        CUDA_TRY(rtdbs::launch_counts_by_slot(e->v, nn, e->stream));
    } else {
        // the label buffer is free scratch between slides only if we restore it;
        // use a temporary device buffer instead
        int* tmp = nullptr;
        CUDA_TRY(cudaMallocAsync((void**)&tmp, sizeof(int) * e->p.window, e->stream));
        cudaError_t ce = rtdbs::launch_counts_by_slot(e->v, tmp, e->stream);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(nn, tmp, sizeof(int) * e->p.window, cudaMemcpyDeviceToHost, e->stream);
        cudaFreeAsync(tmp, e->stream);
        CUDA_TRY(ce);
    }
    return fetch_ctl_and_sync(e);
}

int rtdbs_device_outputs(rtdbs_engine* e, int32_t** d_label, int32_t** d_cluster_id) {
    if (!e) return fail(RTDBS_ERR_INVALID, "engine is NULL");
    if (d_label) *d_label = e->v.label;
    if (d_cluster_id) *d_cluster_id = e->v.cid;
    return RTDBS_OK;
}

int rtdbs_get_stats(rtdbs_engine* e, rtdbs_stats* s) {
    if (!e || !s) return fail(RTDBS_ERR_INVALID, "engine/stats is NULL");
    DeviceGuard guard(e->device);
    CUDA_TRY(guard.err);
    CUDA_TRY(cudaMemcpyAsync(e->h_ctl, e->v.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    std::memset(s, 0, sizeof(*s));
    s->slides = e->h_ctl->slide;
    s->band_rechecks = (int64_t)e->h_ctl->band_rechecks;
    for (int k = 0; k < 8; ++k) {
        s->query_tests += (int64_t)e->h_ctl->ptests[0][k];
        s->query_hits += (int64_t)e->h_ctl->phits[0][k];
        s->cluster_tests += (int64_t)e->h_ctl->ptests[1][k];
        s->cluster_hits += (int64_t)e->h_ctl->phits[1][k];
        s->max_query_tests = std::max(s->max_query_tests, e->h_ctl->qmax[k]);
    }
    s->dist_tests = s->query_tests + s->cluster_tests;
    s->reused_cores = e->h_ctl->last_reused;
    s->cells = e->h_ctl->ncells;
    s->work_items = e->h_ctl->nitems;
    s->error_bits = e->h_ctl->err;
    s->key_bits = e->v.key_bits;
    s->cell_side = e->cell_side;
    s->device_bytes = (int64_t)e->dev_bytes;
    const int nchunks = (e->p.stride + e->chunk - 1) / e->chunk;
    s->chunks_per_slide = nchunks;
    // per chunk 6 kernels, 7 when the sort phase needs a run merge (a chunk
    // of more than one sort run); then union, flatten and label (or border)
    int launches = 3;
    for (int j = 0; j < nchunks; ++j) {
        const int c = std::min(e->chunk, e->p.stride - j * e->chunk);
        launches += rtdbs::kChunkPhases + (c > rtdbs::kSortRun ? 1 : 0);
    }
    s->launches_per_slide = launches;
    return RTDBS_OK;
}

int rtdbs_slide_profiled(rtdbs_engine* e, const float* d_new_points, rtdbs_phase_times* t) {
    if (!e || !d_new_points || !t) return fail(RTDBS_ERR_INVALID, "engine/new_points/times is NULL");
    if (!e->loaded) return fail(RTDBS_ERR_STATE, "rtdbs_load_window must come first");
    DeviceGuard guard(e->device);
    CUDA_TRY(guard.err);
    const int S = e->p.stride, C = e->chunk;
    const int nchunks = (S + C - 1) / C;
    const int nev = nchunks * rtdbs::kChunkPhases + 4;
    std::vector<cudaEvent_t> ev(nev, nullptr);
    for (auto& x : ev) CUDA_TRY(cudaEventCreate(&x));
    int rc = wait_outputs_free(e);
    if (rc == RTDBS_OK && d_new_points != e->v.staging) rc = copy_in(e, d_new_points, S, 1);
    int k = 0;
    if (rc == RTDBS_OK) {
        cudaEventRecord(ev[k++], e->stream);
        for (int j = 0; j < nchunks && rc == RTDBS_OK; ++j) {
            const int c = std::min(C, S - j * C);
            for (int ph = 0; ph < rtdbs::kChunkPhases; ++ph) {
                cudaError_t ce = rtdbs::launch_phase(ph, e->v, e->p.precision, j, c, 0, j * C, 0, e->stream);
                if (ce != cudaSuccess) {
                    rc = fail(RTDBS_ERR_CUDA, "launch failed: %s", cudaGetErrorString(ce));
                    break;
                }
                cudaEventRecord(ev[k++], e->stream);
            }
        }
        for (int ph = rtdbs::kPhaseUnion; ph <= rtdbs::kPhaseLabel && rc == RTDBS_OK; ++ph) {
            cudaError_t ce = rtdbs::launch_phase(ph, e->v, e->p.precision, 0, 0, 0, 0, 1, e->stream);
            if (ce != cudaSuccess) rc = fail(RTDBS_ERR_CUDA, "launch failed: %s", cudaGetErrorString(ce));
            cudaEventRecord(ev[k++], e->stream);
        }
    }
    if (rc == RTDBS_OK) rc = fetch_ctl_and_sync(e);
    if (rc == RTDBS_OK) {
        float ph[rtdbs::kNumPhases] = {0};
        int q = 0;
        for (int j = 0; j < nchunks; ++j)
            for (int p = 0; p < rtdbs::kChunkPhases; ++p, ++q) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev[q], ev[q + 1]);
                ph[p] += ms;
            }
        for (int p = rtdbs::kPhaseUnion; p <= rtdbs::kPhaseLabel; ++p, ++q) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[q], ev[q + 1]);
            ph[p] += ms;
        }
        float total = 0.f;
        cudaEventElapsedTime(&total, ev[0], ev[q]);
        t->ingest_ms = ph[rtdbs::kPhaseIngest];
        t->sort_ms = ph[rtdbs::kPhaseSort];
        t->decrement_ms = ph[rtdbs::kPhaseDecrement];
        t->merge_ms = ph[rtdbs::kPhaseMerge];
        t->build_ms = ph[rtdbs::kPhaseBuild];
        t->increment_ms = ph[rtdbs::kPhaseIncrement];
        t->union_ms = ph[rtdbs::kPhaseUnion];
        t->flatten_ms = ph[rtdbs::kPhaseFlatten];
        t->label_ms = ph[rtdbs::kPhaseLabel];
        t->total_ms = total;
        t->chunks = nchunks;
    }
    for (auto& x : ev)
        if (x) cudaEventDestroy(x);
    return rc;
}


// ====================================================================== pool

int rtdbs_stream_bytes(const rtdbs_params* params, int64_t* bytes) {
    if (!params || !bytes) return fail(RTDBS_ERR_INVALID, "params/bytes is NULL");
    if (params->window <= 0 || params->stride <= 0 || params->dim < 1 || params->dim > 3)
        return fail(RTDBS_ERR_INVALID, "bad window/stride/dim");
    rtdbs_engine tmp;
    tmp.p = *params;
    std::vector<Part> parts;
    *bytes = (int64_t)plan_layout(&tmp, parts);
    return RTDBS_OK;
}

}  // extern "C"

struct rtdbs_pool {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int flags = 0;
    int64_t budget = 0;  // 0: unlimited
    int64_t used = 0;
    int capacity = 0;
    std::vector<rtdbs_engine*> eng;   // slot -> engine (nullptr: free)
    std::vector<char> loaded;
    View* d_views = nullptr;          // one View per slot
    Ctl* d_ctls = nullptr;            // every stream's control block, contiguous
    Ctl* h_ctls = nullptr;            // pinned mirror
    char* d_tables = nullptr;         // items + prefixes of the cached round shape
    size_t tables_cap = 0;
    float* d_input = nullptr;         // the round's new points, back to back
    size_t input_cap = 0;             // floats
    void* d_gather = nullptr;         // per-stream source pointers, offsets, counts
    size_t gather_cap = 0;
    // side streams for the stream groups of a split phase, which run at the
    // same time (fork/join through events; captured into the round's graph)
    static constexpr int kSide = 5;
    cudaStream_t side[kSide] = {};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kSide] = {};
    std::vector<int> shape_ids;       // stream set the tables / graph were built for
    cudaGraphExec_t graph = nullptr;
    // launch plan of the cached shape
    struct Launch {
        int phase, prec, dim;          // prec/dim: the stream group of a split phase
        size_t items_off, prefix_off;  // byte offsets into d_tables
        int n, blocks, max_c;
    };
    std::vector<Launch> plan;
    std::vector<size_t> input_off;    // per listed stream, float offset into d_input
    size_t input_floats = 0;
    int64_t rounds = 0, graph_replays = 0;
};

namespace {

void pool_drop_shape(rtdbs_pool* p) {
    if (p->graph) {
        cudaStreamSynchronize(p->stream);  // a replay of it may still be queued
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    p->shape_ids.clear();
    p->plan.clear();
}

// Phases launched once per stream group: those whose bodies are instantiated
// per group, and the forest-reuse passes between them (so the increment
// through the label phase form one run of grouped phases).
bool pool_grouped(int phase) {
    return rtdbs::batch_phase_split(phase) || phase == rtdbs::kBatchDamage || phase == rtdbs::kBatchReuse;
}

// Builds (and uploads) the launch tables of one round over `ids`.
int pool_build_shape(rtdbs_pool* p, const std::vector<int>& ids) {
    using rtdbs::BatchItem;
    const int n = (int)ids.size();
    std::vector<size_t> off(n);
    size_t floats = 0;
    int maxchunks = 0;
    for (int i = 0; i < n; ++i) {
        const rtdbs_engine* e = p->eng[ids[i]];
        off[i] = floats;
        floats += (size_t)e->p.stride * e->p.dim;
        maxchunks = std::max(maxchunks, (e->p.stride + e->chunk - 1) / e->chunk);
    }
    if (floats > p->input_cap) {
        if (p->d_input) cudaFree(p->d_input);
        p->d_input = nullptr;
        CUDA_TRY(cudaMalloc((void**)&p->d_input, sizeof(float) * floats));
        p->input_cap = floats;
    }
    // host image of the tables: per chunk step j an item array, then every
    // launch's prefix array
    std::vector<char> img;
    auto put = [&img](const void* src, size_t bytes) {
        const size_t at = (img.size() + 15) / 16 * 16;
        img.resize(at + bytes);
        std::memcpy(img.data() + at, src, bytes);
        return at;
    };
    std::vector<rtdbs_pool::Launch> plan;
    // One launch of phase ph over `items`; split phases get one launch per
    // (precision, dim) group present.
    auto add_launches = [&](int ph, const std::vector<BatchItem>& items) {
        std::vector<std::pair<int, int>> groups;
        if (pool_grouped(ph)) {
            for (const auto& it : items) {
                const auto& v = p->eng[it.view]->v;
                const std::pair<int, int> g(v.precision, rtdbs::dk_of(v));
                if (std::find(groups.begin(), groups.end(), g) == groups.end()) groups.push_back(g);
            }
        } else {
            groups.push_back({0, 0});
        }
        for (const auto& g : groups) {
            std::vector<BatchItem> sel;
            for (const auto& it : items) {
                const auto& v = p->eng[it.view]->v;
                if (!pool_grouped(ph) || (v.precision == g.first && rtdbs::dk_of(v) == g.second))
                    sel.push_back(it);
            }
            std::vector<int> prefix(sel.size() + 1, 0);
            int max_c = 0;
            for (size_t i = 0; i < sel.size(); ++i) {
                prefix[i + 1] = prefix[i] + rtdbs::batch_blocks(ph, p->eng[sel[i].view]->v, sel[i].c);
                max_c = std::max(max_c, sel[i].c);
            }
            const size_t items_off = put(sel.data(), sizeof(BatchItem) * sel.size());
            const size_t prefix_off = put(prefix.data(), sizeof(int) * prefix.size());
            plan.push_back({ph, g.first, g.second, items_off, prefix_off, (int)sel.size(), prefix.back(), max_c});
        }
    };
    // Launch order: largest windows first, so the blocks of the smallest
    // streams fill the last wave of each launch (the packed input keeps the
    // caller's order).
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
        return p->eng[ids[a]]->p.window > p->eng[ids[b]]->p.window;
    });
    std::vector<BatchItem> all_items;
    for (int j = 0; j < maxchunks; ++j) {
        std::vector<BatchItem> items;
        for (int i : ord) {
            const rtdbs_engine* e = p->eng[ids[i]];
            const int S = e->p.stride, C = e->chunk;
            if (j * C >= S) continue;
            BatchItem it;
            it.view = ids[i];
            it.j = j;
            it.c = std::min(C, S - j * C);
            it.stg_off = j * C;
            it.input = p->d_input + off[i];
            items.push_back(it);
        }
        if (j == 0) all_items = items;
        for (int ph = 0; ph < rtdbs::kBatchChunkPhases; ++ph) add_launches(ph, items);
    }
    for (auto& it : all_items) it.c = 0;  // cluster phases size by W only
    // (no damage or reuse launch: the ingest and the decrement mark the lost
    // cores, the merge and the increment set the start hints)
    for (int ph = rtdbs::kBatchUnion; ph <= rtdbs::kBatchLabel; ++ph) add_launches(ph, all_items);
    if (img.size() > p->tables_cap) {
        // (cudaFree waits for the rounds that still read the old buffer)
        if (p->d_tables) cudaFree(p->d_tables);
        p->d_tables = nullptr;
        CUDA_TRY(cudaMalloc((void**)&p->d_tables, img.size()));
        p->tables_cap = img.size();
    }
    // Stream-ordered: the copy lands after the rounds already queued (which
    // read the previous tables) and before this round; from pageable memory
    // the call returns once the image is staged, so the host never waits.
    CUDA_TRY(cudaMemcpyAsync(p->d_tables, img.data(), img.size(), cudaMemcpyHostToDevice, p->stream));
    p->plan = std::move(plan);
    p->input_off = std::move(off);
    p->input_floats = floats;
    p->shape_ids = ids;
    return RTDBS_OK;
}

cudaError_t pool_launch(rtdbs_pool* p, const rtdbs_pool::Launch& l, cudaStream_t s) {
    rtdbs::BatchLaunch L;
    L.views = p->d_views;
    L.items = reinterpret_cast<const rtdbs::BatchItem*>(p->d_tables + l.items_off);
    L.prefix = reinterpret_cast<const int*>(p->d_tables + l.prefix_off);
    L.n = l.n;
    return rtdbs::launch_batch(l.phase, l.prec, l.dim, L, l.blocks, l.max_c, s);
}

// One round.  The stream groups' launches of consecutive grouped phases
// (the increment through the label phase) are independent -- disjoint
// streams of the pool -- so each group runs its part of that run in phase
// order on its own stream: the first group on the pool's stream, the others
// on side streams forked from it at the start of the run and joined back at
// its end.  The decrement needs only the ingest, so its group launches run
// on side streams beside the sort and are joined before the merge.
// Ungrouped phases (ingest, sort, merge, build) take every stream in one
// launch.
int pool_enqueue_round(rtdbs_pool* p) {
    const size_t n = p->plan.size();
    std::vector<char> done(n, 0);
    int pending_join = 0;  // side streams running a decrement
    for (size_t i = 0; i < n;) {
        if (done[i]) {
            ++i;
            continue;
        }
        const int ph = p->plan[i].phase;
        if (!pool_grouped(ph)) {
            if (ph == rtdbs::kBatchMerge)
                for (int g = 0; g < pending_join; ++g) CUDA_TRY(cudaStreamWaitEvent(p->stream, p->ev_join[g], 0));
            if (ph == rtdbs::kBatchMerge) pending_join = 0;
            CUDA_TRY(pool_launch(p, p->plan[i], p->stream));
            if (ph == rtdbs::kBatchIngest) {
                // this chunk step's decrement launches, up to the merge
                std::vector<size_t> dec;
                for (size_t k = i + 1; k < n && p->plan[k].phase != rtdbs::kBatchMerge; ++k)
                    if (p->plan[k].phase == rtdbs::kBatchDecrement) dec.push_back(k);
                if (!dec.empty() && (int)dec.size() <= rtdbs_pool::kSide) {
                    CUDA_TRY(cudaEventRecord(p->ev_fork, p->stream));
                    for (size_t g = 0; g < dec.size(); ++g) {
                        CUDA_TRY(cudaStreamWaitEvent(p->side[g], p->ev_fork, 0));
                        CUDA_TRY(pool_launch(p, p->plan[dec[g]], p->side[g]));
                        CUDA_TRY(cudaEventRecord(p->ev_join[g], p->side[g]));
                        done[dec[g]] = 1;
                    }
                    pending_join = (int)dec.size();
                }
            }
            ++i;
            continue;
        }
        size_t j = i;
        std::vector<std::pair<int, int>> groups;
        while (j < n && pool_grouped(p->plan[j].phase) && !done[j]) {
            const std::pair<int, int> g(p->plan[j].prec, p->plan[j].dim);
            if (std::find(groups.begin(), groups.end(), g) == groups.end()) groups.push_back(g);
            ++j;
        }
        const int ng = (int)groups.size();
        if (ng > 1 + rtdbs_pool::kSide) return fail(RTDBS_ERR_INVALID, "too many stream groups");
        if (ng > 1) {
            CUDA_TRY(cudaEventRecord(p->ev_fork, p->stream));
            for (int g = 1; g < ng; ++g) CUDA_TRY(cudaStreamWaitEvent(p->side[g - 1], p->ev_fork, 0));
        }
        for (size_t k = i; k < j; ++k) {
            const int g = (int)(std::find(groups.begin(), groups.end(),
                                          std::make_pair(p->plan[k].prec, p->plan[k].dim)) - groups.begin());
            CUDA_TRY(pool_launch(p, p->plan[k], g == 0 ? p->stream : p->side[g - 1]));
        }
        for (int g = 1; g < ng; ++g) {
            CUDA_TRY(cudaEventRecord(p->ev_join[g - 1], p->side[g - 1]));
            CUDA_TRY(cudaStreamWaitEvent(p->stream, p->ev_join[g - 1], 0));
        }
        i = j;
    }
    for (int g = 0; g < pending_join; ++g) CUDA_TRY(cudaStreamWaitEvent(p->stream, p->ev_join[g], 0));
    return RTDBS_OK;
}

}  // namespace

extern "C" {

int rtdbs_pool_params_init(rtdbs_pool_params* pp) {
    if (!pp) return fail(RTDBS_ERR_INVALID, "params is NULL");
    std::memset(pp, 0, sizeof(*pp));
    pp->max_streams = 1024;
    return RTDBS_OK;
}

int rtdbs_pool_create(const rtdbs_pool_params* pp, void* cuda_stream, rtdbs_pool** out) {
    if (!pp || !out) return fail(RTDBS_ERR_INVALID, "params/out is NULL");
    *out = nullptr;
    if (pp->max_streams <= 0 || pp->max_streams > (1 << 20)) return fail(RTDBS_ERR_INVALID, "bad max_streams");
    if (pp->hbm_budget_bytes < 0) return fail(RTDBS_ERR_INVALID, "negative budget");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(RTDBS_ERR_NO_DEVICE, "no CUDA device available");
    if (pp->device < 0 || pp->device >= ndev) return fail(RTDBS_ERR_INVALID, "device out of range");
    DeviceGuard guard(pp->device);
    CUDA_TRY(guard.err);
    CUDA_TRY(configure_device(pp->device));
    rtdbs_pool* p = new (std::nothrow) rtdbs_pool();
    if (!p) return fail(RTDBS_ERR_OOM, "host allocation failed");
    p->device = pp->device;
    p->flags = pp->flags;
    p->budget = pp->hbm_budget_bytes;
    p->capacity = pp->max_streams;
    p->eng.assign(p->capacity, nullptr);
    p->loaded.assign(p->capacity, 0);
    int rc = RTDBS_OK;
    if (cuda_stream) {
        p->stream = static_cast<cudaStream_t>(cuda_stream);
    } else if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
        rc = fail(RTDBS_ERR_CUDA, "cudaStreamCreate failed");
    } else {
        p->own_stream = true;
    }
    if (rc == RTDBS_OK && (cudaMalloc((void**)&p->d_views, sizeof(View) * p->capacity) != cudaSuccess ||
                           cudaMalloc((void**)&p->d_ctls, sizeof(Ctl) * p->capacity) != cudaSuccess ||
                           cudaMallocHost((void**)&p->h_ctls, sizeof(Ctl) * p->capacity) != cudaSuccess))
        rc = fail(RTDBS_ERR_OOM, "pool tables: allocation failed");
    if (rc == RTDBS_OK && cudaMemset(p->d_ctls, 0, sizeof(Ctl) * p->capacity) != cudaSuccess)
        rc = fail(RTDBS_ERR_CUDA, "cudaMemset failed");
    if (rc == RTDBS_OK && cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming) != cudaSuccess)
        rc = fail(RTDBS_ERR_CUDA, "cudaEventCreate failed");
    for (int k = 0; k < rtdbs_pool::kSide && rc == RTDBS_OK; ++k)
        if (cudaStreamCreateWithFlags(&p->side[k], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&p->ev_join[k], cudaEventDisableTiming) != cudaSuccess)
            rc = fail(RTDBS_ERR_CUDA, "side stream set-up failed");
    if (rc != RTDBS_OK) {
        rtdbs_pool_destroy(p);
        return rc;
    }
    *out = p;
    return RTDBS_OK;
}

int rtdbs_pool_destroy(rtdbs_pool* p) {
    if (!p) return RTDBS_OK;
    DeviceGuard guard(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    pool_drop_shape(p);
    for (auto* e : p->eng)
        if (e) rtdbs_destroy(e);
    if (p->d_views) cudaFree(p->d_views);
    if (p->d_ctls) cudaFree(p->d_ctls);
    if (p->h_ctls) cudaFreeHost(p->h_ctls);
    if (p->d_tables) cudaFree(p->d_tables);
    if (p->d_input) cudaFree(p->d_input);
    if (p->d_gather) cudaFree(p->d_gather);
    for (int k = 0; k < rtdbs_pool::kSide; ++k) {
        if (p->side[k]) cudaStreamDestroy(p->side[k]);
        if (p->ev_join[k]) cudaEventDestroy(p->ev_join[k]);
    }
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->own_stream && p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return RTDBS_OK;
}

int rtdbs_pool_add_stream(rtdbs_pool* p, const rtdbs_params* params, int32_t* stream_id) {
    if (!p || !params || !stream_id) return fail(RTDBS_ERR_INVALID, "pool/params/stream_id is NULL");
    int64_t bytes = 0;
    int rc = rtdbs_stream_bytes(params, &bytes);
    if (rc != RTDBS_OK) return rc;
    if (p->budget > 0 && p->used + bytes > p->budget)
        return fail(RTDBS_ERR_BUDGET, "stream needs %lld bytes, %lld of %lld in use", (long long)bytes,
                    (long long)p->used, (long long)p->budget);
    int slot = -1;
    for (int i = 0; i < p->capacity; ++i)
        if (!p->eng[i]) {
            slot = i;
            break;
        }
    if (slot < 0) return fail(RTDBS_ERR_BUDGET, "all %d stream slots are in use", p->capacity);
    rtdbs_params q = *params;
    q.device = p->device;
    q.flags |= RTDBS_FLAG_NO_GRAPH;
    rtdbs_engine* e = nullptr;
    rc = rtdbs_create(&q, p->stream, &e);
    if (rc != RTDBS_OK) return rc;
    // this stream's control block lives in the pool's contiguous array
    e->v.ctl = p->d_ctls + slot;
    {
        DeviceGuard guard(p->device);
        if (cudaMemsetAsync(e->v.ctl, 0, sizeof(Ctl), p->stream) != cudaSuccess) {
            rtdbs_destroy(e);
            return fail(RTDBS_ERR_CUDA, "cudaMemsetAsync failed");
        }
    }
    p->eng[slot] = e;
    p->loaded[slot] = 0;
    p->used += (int64_t)e->dev_bytes;
    *stream_id = slot;
    return RTDBS_OK;
}

int rtdbs_pool_remove_stream(rtdbs_pool* p, int32_t id) {
    if (!p || id < 0 || id >= p->capacity || !p->eng[id]) return fail(RTDBS_ERR_INVALID, "no such stream");
    DeviceGuard guard(p->device);
    cudaStreamSynchronize(p->stream);
    for (int s : p->shape_ids)
        if (s == id) {
            pool_drop_shape(p);
            break;
        }
    p->used -= (int64_t)p->eng[id]->dev_bytes;
    rtdbs_destroy(p->eng[id]);
    p->eng[id] = nullptr;
    p->loaded[id] = 0;
    return RTDBS_OK;
}

int rtdbs_pool_load_window(rtdbs_pool* p, int32_t id, const float* points, int points_on_device) {
    if (!p || id < 0 || id >= p->capacity || !p->eng[id]) return fail(RTDBS_ERR_INVALID, "no such stream");
    rtdbs_engine* e = p->eng[id];
    int rc = rtdbs_load_window(e, points, points_on_device);
    if (rc != RTDBS_OK) return rc;
    DeviceGuard guard(p->device);
    CUDA_TRY(cudaMemcpy(p->d_views + id, &e->v, sizeof(View), cudaMemcpyHostToDevice));
    p->loaded[id] = 1;
    for (int s : p->shape_ids)
        if (s == id) {
            pool_drop_shape(p);
            break;
        }
    return RTDBS_OK;
}

namespace {
int pool_round(rtdbs_pool* p, int32_t n, const int32_t* ids, const float* d_points,
               const float* const* d_points_each);
}

int rtdbs_pool_slide(rtdbs_pool* p, int32_t n, const int32_t* ids, const float* d_points) {
    if (!p || n <= 0 || !ids || !d_points) return fail(RTDBS_ERR_INVALID, "pool/ids/points is NULL or n <= 0");
    return pool_round(p, n, ids, d_points, nullptr);
}

int rtdbs_pool_slide_each(rtdbs_pool* p, int32_t n, const int32_t* ids, const float* const* d_points_each) {
    if (!p || n <= 0 || !ids || !d_points_each)
        return fail(RTDBS_ERR_INVALID, "pool/ids/points is NULL or n <= 0");
    for (int i = 0; i < n; ++i)
        if (!d_points_each[i]) return fail(RTDBS_ERR_INVALID, "points of stream %d is NULL", ids[i]);
    return pool_round(p, n, ids, nullptr, d_points_each);
}

}  // extern "C"

namespace {
int pool_round(rtdbs_pool* p, int32_t n, const int32_t* ids, const float* d_points,
               const float* const* d_points_each) {
    std::vector<int> list(ids, ids + n);
    std::vector<char> seen(p->capacity, 0);
    for (int id : list) {
        if (id < 0 || id >= p->capacity || !p->eng[id] || !p->loaded[id])
            return fail(RTDBS_ERR_STATE, "stream %d is not loaded", id);
        if (seen[id]) return fail(RTDBS_ERR_INVALID, "stream %d listed twice", id);
        seen[id] = 1;
    }
    DeviceGuard guard(p->device);
    CUDA_TRY(guard.err);
    if (list != p->shape_ids) {
        pool_drop_shape(p);
        int rc = pool_build_shape(p, list);
        if (rc != RTDBS_OK) return rc;
    }
    if (d_points) {
        CUDA_TRY(cudaMemcpyAsync(p->d_input, d_points, sizeof(float) * p->input_floats,
                                 cudaMemcpyDeviceToDevice, p->stream));
    } else {
        // one gather kernel packs the streams' own buffers
        const size_t need = (size_t)n * (sizeof(void*) + sizeof(long long) + sizeof(int));
        if (need > p->gather_cap) {
            if (p->d_gather) cudaFree(p->d_gather);
            p->d_gather = nullptr;
            CUDA_TRY(cudaMalloc(&p->d_gather, need));
            p->gather_cap = need;
        }
        std::vector<char> host(need);
        const float** src = reinterpret_cast<const float**>(host.data());
        long long* off = reinterpret_cast<long long*>(host.data() + (size_t)n * sizeof(void*));
        int* cnt = reinterpret_cast<int*>(host.data() + (size_t)n * (sizeof(void*) + sizeof(long long)));
        int max_count = 0;
        for (int i = 0; i < n; ++i) {
            const rtdbs_engine* e = p->eng[list[i]];
            src[i] = d_points_each[i];
            off[i] = (long long)p->input_off[i];
            cnt[i] = e->p.stride * e->p.dim;
            max_count = std::max(max_count, cnt[i]);
        }
        // pageable source: the call returns once the table is staged
        CUDA_TRY(cudaMemcpyAsync(p->d_gather, host.data(), need, cudaMemcpyHostToDevice, p->stream));
        char* g = static_cast<char*>(p->d_gather);
        CUDA_TRY(rtdbs::launch_gather(reinterpret_cast<const float* const*>(g),
                                      reinterpret_cast<const long long*>(g + (size_t)n * sizeof(void*)),
                                      reinterpret_cast<const int*>(g + (size_t)n * (sizeof(void*) + sizeof(long long))),
                                      p->d_input, n, max_count, p->stream));
    }
    if (p->flags & RTDBS_FLAG_NO_GRAPH) {
        int rc = pool_enqueue_round(p);
        if (rc != RTDBS_OK) return rc;
    } else {
        if (!p->graph) {
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
            int rc = pool_enqueue_round(p);
            cudaError_t ce = cudaStreamEndCapture(p->stream, &g);
            if (rc != RTDBS_OK) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            CUDA_TRY(ce);
            cudaError_t ie = cudaGraphInstantiate(&p->graph, g, 0);
            cudaGraphDestroy(g);
            CUDA_TRY(ie);
        } else {
            ++p->graph_replays;
        }
        CUDA_TRY(cudaGraphLaunch(p->graph, p->stream));
    }
    ++p->rounds;
    return RTDBS_OK;
}
}  // namespace

extern "C" {

int rtdbs_pool_slide_profiled(rtdbs_pool* p, int32_t n, const int32_t* ids, const float* d_points,
                              rtdbs_phase_times* t) {
    if (!p || !t) return fail(RTDBS_ERR_INVALID, "pool/times is NULL");
    if (n <= 0 || !ids || !d_points) return fail(RTDBS_ERR_INVALID, "ids/points is NULL or n <= 0");
    std::vector<int> list(ids, ids + n);
    std::vector<char> seen(p->capacity, 0);
    for (int id : list) {
        if (id < 0 || id >= p->capacity || !p->eng[id] || !p->loaded[id])
            return fail(RTDBS_ERR_STATE, "stream %d is not loaded", id);
        if (seen[id]) return fail(RTDBS_ERR_INVALID, "stream %d listed twice", id);
        seen[id] = 1;
    }
    DeviceGuard guard(p->device);
    CUDA_TRY(guard.err);
    if (list != p->shape_ids) {
        pool_drop_shape(p);
        int rc = pool_build_shape(p, list);
        if (rc != RTDBS_OK) return rc;
    }
    CUDA_TRY(cudaMemcpyAsync(p->d_input, d_points, sizeof(float) * p->input_floats, cudaMemcpyDeviceToDevice,
                             p->stream));
    std::vector<cudaEvent_t> ev(p->plan.size() + 1, nullptr);
    for (auto& x : ev) CUDA_TRY(cudaEventCreate(&x));
    int rc = RTDBS_OK;
    cudaEventRecord(ev[0], p->stream);
    for (size_t i = 0; i < p->plan.size() && rc == RTDBS_OK; ++i) {
        const auto& l = p->plan[i];
        rtdbs::BatchLaunch L;
        L.views = p->d_views;
        L.items = reinterpret_cast<const rtdbs::BatchItem*>(p->d_tables + l.items_off);
        L.prefix = reinterpret_cast<const int*>(p->d_tables + l.prefix_off);
        L.n = l.n;
        cudaError_t ce = rtdbs::launch_batch(l.phase, l.prec, l.dim, L, l.blocks, l.max_c, p->stream);
        if (ce != cudaSuccess) rc = fail(RTDBS_ERR_CUDA, "launch failed: %s", cudaGetErrorString(ce));
        cudaEventRecord(ev[i + 1], p->stream);
    }
    if (rc == RTDBS_OK) rc = rtdbs_pool_sync(p);
    if (rc == RTDBS_OK) {
        // batch phases -> the engine's phase slots (sort + run merge are one)
        // (the forest-reuse passes belong to the union phase, as in the single-stream launch)
        static const int slot[rtdbs::kNumBatchPhases] = {0, 1, 1, 2, 3, 4, 5, 6, 6, 6, 7, 8};
        float ph[9] = {0};
        for (size_t i = 0; i < p->plan.size(); ++i) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
            ph[slot[p->plan[i].phase]] += ms;
        }
        float total = 0.f;
        cudaEventElapsedTime(&total, ev[0], ev[p->plan.size()]);
        t->ingest_ms = ph[0];
        t->sort_ms = ph[1];
        t->decrement_ms = ph[2];
        t->merge_ms = ph[3];
        t->build_ms = ph[4];
        t->increment_ms = ph[5];
        t->union_ms = ph[6];
        t->flatten_ms = ph[7];
        t->label_ms = ph[8];
        t->total_ms = total;
        t->chunks = 0;
    }
    for (auto& x : ev)
        if (x) cudaEventDestroy(x);
    ++p->rounds;
    return rc;
}

int rtdbs_pool_sync(rtdbs_pool* p) {
    if (!p) return fail(RTDBS_ERR_INVALID, "pool is NULL");
    DeviceGuard guard(p->device);
    CUDA_TRY(guard.err);
    CUDA_TRY(cudaMemcpyAsync(p->h_ctls, p->d_ctls, sizeof(Ctl) * p->capacity, cudaMemcpyDeviceToHost, p->stream));
    CUDA_TRY(cudaStreamSynchronize(p->stream));
    for (int i = 0; i < p->capacity; ++i)
        if (p->eng[i] && p->h_ctls[i].err)
            return fail(RTDBS_ERR_DEVICE, "stream %d: device error bits 0x%x", i, p->h_ctls[i].err);
    return RTDBS_OK;
}

int rtdbs_pool_outputs(rtdbs_pool* p, int32_t id, int32_t** d_label, int32_t** d_cluster_id) {
    if (!p || id < 0 || id >= p->capacity || !p->eng[id]) return fail(RTDBS_ERR_INVALID, "no such stream");
    return rtdbs_device_outputs(p->eng[id], d_label, d_cluster_id);
}

int rtdbs_pool_read_outputs(rtdbs_pool* p, int32_t id, int32_t* label, int32_t* cluster_id, int on_device) {
    if (!p || id < 0 || id >= p->capacity || !p->eng[id]) return fail(RTDBS_ERR_INVALID, "no such stream");
    DeviceGuard guard(p->device);
    CUDA_TRY(guard.err);
    int rc = copy_out(p->eng[id], label, cluster_id, on_device);
    if (rc != RTDBS_OK) return rc;
    CUDA_TRY(cudaStreamSynchronize(p->stream));
    return RTDBS_OK;
}

int rtdbs_pool_engine(rtdbs_pool* p, int32_t id, rtdbs_engine** engine) {
    if (!p || !engine || id < 0 || id >= p->capacity || !p->eng[id]) return fail(RTDBS_ERR_INVALID, "no such stream");
    *engine = p->eng[id];
    return RTDBS_OK;
}

int rtdbs_pool_get_stats(rtdbs_pool* p, rtdbs_pool_stats* s) {
    if (!p || !s) return fail(RTDBS_ERR_INVALID, "pool/stats is NULL");
    std::memset(s, 0, sizeof(*s));
    for (int i = 0; i < p->capacity; ++i) s->streams += p->eng[i] ? 1 : 0;
    s->bytes_in_use = p->used;
    s->budget_bytes = p->budget;
    s->rounds = p->rounds;
    s->graph_replays = p->graph_replays;
    s->launches_per_round = (int32_t)p->plan.size();
    return RTDBS_OK;
}

}  // extern "C"
