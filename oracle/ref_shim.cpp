// ref_shim.cpp -- exposes the reference's own CPU checker through a C ABI.
//
// TEST INFRASTRUCTURE ONLY.  Linked (by oracle/Makefile, into oracle/_ref/)
// against the reference's unmodified src/dbscan/util.cpp, compiled from where
// it lies.  ref_cluster_with_cpu fills the ScanState fields that
// cluster_with_cpu (src/dbscan/util.cpp:299-354) reads -- h_window, the check_*
// buffers, window_size, min_pts and params.radius2 = radius*radius in float
// (as initialize_params does, src/dbscan/dbscan.cpp:41) -- and calls it.
#include <cstdlib>
#include <cstdio>
#include <new>

#include "state.h"
#include "timer.h"

// util.cpp's GPU checker (cluster_with_cuda) references these launch
// wrappers from src/dbscan/aabb.cu.  They are never called through this
// shim; the stubs only satisfy the linker without building the CUDA file.
extern "C" void find_neighbors(int*, DATA_TYPE_3*, int, DATA_TYPE, int) { std::abort(); }
extern "C" void find_cores(int*, int*, int*, int, int, cudaStream_t) { std::abort(); }
extern "C" void set_cluster_id(int*, int*, int*, DATA_TYPE_3*, int, DATA_TYPE) { std::abort(); }

extern "C" int ref_cluster_with_cpu(const float* xyz, int n, float radius, int min_pts,
                                    int* nn, int* label, int* cid) {
    ScanState* state = new (std::nothrow) ScanState();
    if (!state) return -2;
    state->window_size = n;
    state->min_pts = min_pts;
    state->radius = radius;
    state->params.radius2 = state->radius * state->radius;
    state->h_window = reinterpret_cast<DATA_TYPE_3*>(const_cast<float*>(xyz));
    state->check_h_nn = nn;
    state->check_h_label = label;
    state->check_h_cluster_id = cid;
    Timer timer;
    cluster_with_cpu(*state, timer);
    delete state;
    return 0;
}
