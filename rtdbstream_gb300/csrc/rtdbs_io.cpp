// rtdbs_io.cpp -- point-stream readers for the reference's dataset formats
// (src/dbscan/util.cpp:12-254, chosen by file name at
// src/dbscan/dbscan.cpp:2454-2470):
//   tao      text, one "x,y,z" per line
//   geolife  binary, little-endian double triples
//   RBF      text, one header line, then "x,y"
//   EDS      text, one header line, then "id x y cid"
//   stock    text, one header line, then one value
// Values are parsed as double and stored as float; missing coordinates are 0
// (the reference keeps float3 for every dataset).  The bounding box is taken
// over the finite coordinates read, as the reference takes it over the whole
// file (its grid needs it, src/dbscan/dbscan.cpp:34-37).
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "rtdbs.h"

namespace {

int detect_format(const char* path) {
    const std::string p(path);
    if (p.find("tao") != std::string::npos) return RTDBS_FORMAT_TAO;
    if (p.find("geolife") != std::string::npos) return RTDBS_FORMAT_GEOLIFE;
    if (p.find("RBF") != std::string::npos) return RTDBS_FORMAT_RBF;
    if (p.find("EDS") != std::string::npos) return RTDBS_FORMAT_EDS;
    if (p.find("stock") != std::string::npos) return RTDBS_FORMAT_STOCK;
    return -1;
}

int format_dim(int f) {
    switch (f) {
        case RTDBS_FORMAT_TAO:
        case RTDBS_FORMAT_GEOLIFE: return 3;
        case RTDBS_FORMAT_RBF:
        case RTDBS_FORMAT_EDS: return 2;
        case RTDBS_FORMAT_STOCK: return 1;
        default: return 0;
    }
}

}  // namespace

extern "C" {

int rtdbs_read_points(const char* path, int32_t format, int64_t n_max, float* xyz, int64_t* n_read,
                      int32_t* dim, float* bbox_min, float* bbox_max) {
    if (!path || !xyz || !n_read || n_max < 0) return RTDBS_ERR_INVALID;
    const int f = format == RTDBS_FORMAT_AUTO ? detect_format(path) : format;
    const int d = format_dim(f);
    if (d == 0) return RTDBS_ERR_INVALID;
    const bool binary = f == RTDBS_FORMAT_GEOLIFE;
    FILE* fp = std::fopen(path, binary ? "rb" : "r");
    if (!fp) return RTDBS_ERR_INVALID;
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    int64_t n = 0;
    char line[4096];
    if (f == RTDBS_FORMAT_RBF || f == RTDBS_FORMAT_EDS || f == RTDBS_FORMAT_STOCK) {
        if (!std::fgets(line, sizeof(line), fp)) n_max = 0;  // header line
    }
    while (n < n_max) {
        double v[3] = {0.0, 0.0, 0.0};
        if (binary) {
            if (std::fread(v, sizeof(double), 3, fp) != 3) break;
        } else {
            if (!std::fgets(line, sizeof(line), fp)) break;
            int got = 0;
            if (f == RTDBS_FORMAT_TAO) {
                got = std::sscanf(line, "%lf,%lf,%lf", &v[0], &v[1], &v[2]);
                if (got != 3) break;
            } else if (f == RTDBS_FORMAT_RBF) {
                got = std::sscanf(line, "%lf,%lf", &v[0], &v[1]);
                if (got != 2) break;
            } else if (f == RTDBS_FORMAT_EDS) {
                int id = 0, cid = 0;
                got = std::sscanf(line, "%d %lf %lf %d", &id, &v[0], &v[1], &cid);
                if (got < 3) break;
            } else {
                got = std::sscanf(line, "%lf", &v[0]);
                if (got != 1) break;
            }
        }
        float* out = xyz + 3 * n;
        for (int a = 0; a < 3; ++a) {
            out[a] = a < d ? (float)v[a] : 0.0f;
            if (a < d && std::isfinite(out[a])) {
                mn[a] = std::fmin(mn[a], out[a]);
                mx[a] = std::fmax(mx[a], out[a]);
            }
        }
        ++n;
    }
    std::fclose(fp);
    for (int a = 0; a < 3; ++a)
        if (a >= d || !(mn[a] <= mx[a])) mn[a] = mx[a] = 0.0f;
    *n_read = n;
    if (dim) *dim = d;
    if (bbox_min) std::memcpy(bbox_min, mn, sizeof(mn));
    if (bbox_max) std::memcpy(bbox_max, mx, sizeof(mx));
    return RTDBS_OK;
}

}  // extern "C"
