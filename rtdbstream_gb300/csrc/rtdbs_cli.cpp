// rtdbs_cli.cpp -- command-line driver with the reference's interface
// (src/dbscan/util.cpp:454-500: -f file -n points -W window -S stride
// -K MinPts -R Eps) so script/run.py style sweeps run unchanged.  It reads the
// file (format from its name, src/dbscan/dbscan.cpp:2454-2470), slides the
// window over the whole stream through the C ABI (host buffers, as the
// reference's loop) and prints the mean wall time per slide in the
// reference's "[Time] total: ... ms" line (src/dbscan/timer.h:212), the line
// its scripts extract (script/extract_res.sh).
//
// Extra options: --fp64 (FP64 neighbour relation; default FP32, the
// reference's), --warmup k (untimed passes over the stream first, the
// reference does 10), --labels out.bin (label and cluster id of the last
// window, int32 pairs by slot), --cells-per-eps K (grid cells per Eps, 1 or 2).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rtdbs.h"

namespace {

void usage(const char* argv0) {
    std::fprintf(stderr,
                 "Usage  : %s [options]\n"
                 "Options: --file | -f <filename>   point file (tao / geolife / RBF / EDS / stock)\n"
                 "         -n <int>                 points to read\n"
                 "         --window | -W <int>      window size\n"
                 "         --stride | -S <int>      stride size (divides the window)\n"
                 "         --minPts | -K <int>      MinPts\n"
                 "         --radius | -R <float>    Eps\n"
                 "         --fp64                   FP64 neighbour relation (default: FP32)\n"
                 "         --warmup <int>           untimed passes first (default 0)\n"
                 "         --labels <file>          write the last window's labels and ids\n"
                 "         --cells-per-eps <1|2>    grid cells per Eps (default 1)\n"
                 "         --query-lanes <16|32>    lanes per point in the count passes (default 16;\n"
                 "                                  32 with two cells per Eps)\n",
                 argv0);
    std::exit(1);
}

int die(const char* what, int rc) {
    std::fprintf(stderr, "[Error] %s: %s (%s)\n", what, rtdbs_status_string(rc), rtdbs_last_error());
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
    std::string file, labels_out;
    long long n = 0;
    int W = 0, S = 0, K = 0, warmup = 0, precision = RTDBS_PREC_FP32, cell_mult = 1, query_lanes = 0;
    double R = 0.0;
    for (int i = 1; i < argc; ++i) {
        const std::string a(argv[i]);
        auto next = [&]() -> const char* {
            if (i + 1 >= argc) usage(argv[0]);
            return argv[++i];
        };
        if (a == "-h" || a == "--help") usage(argv[0]);
        else if (a == "-f" || a == "--file") file = next();
        else if (a == "-n") n = std::atoll(next());
        else if (a == "-W" || a == "--window") W = std::atoi(next());
        else if (a == "-S" || a == "--stride") S = std::atoi(next());
        else if (a == "-K" || a == "--minPts") K = std::atoi(next());
        else if (a == "-R" || a == "--radius") R = std::atof(next());
        else if (a == "--fp64") precision = RTDBS_PREC_FP64;
        else if (a == "--warmup") warmup = std::atoi(next());
        else if (a == "--labels") labels_out = next();
        else if (a == "--cells-per-eps") cell_mult = std::atoi(next());
        else if (a == "--query-lanes") query_lanes = std::atoi(next());
        else {
            std::fprintf(stderr, "Unknown option '%s'\n", a.c_str());
            usage(argv[0]);
        }
    }
    if (file.empty() || n <= 0 || W <= 0 || S <= 0 || K <= 0 || !(R > 0.0)) usage(argv[0]);

    std::vector<float> xyz((size_t)n * 3);
    long long got = 0;
    int dim = 0;
    float lo[3], hi[3];
    int64_t n_read = 0;
    int rc = rtdbs_read_points(file.c_str(), RTDBS_FORMAT_AUTO, n, xyz.data(), &n_read, &dim, lo, hi);
    if (rc != RTDBS_OK) {
        std::fprintf(stderr, "[Error] Dataset %s cannot be read\n", file.c_str());
        return 2;
    }
    got = n_read;
    std::printf("Input file: %s\nData num: %lld\n", file.c_str(), got);
    std::printf("Window size: %d, Stride size: %d, K: %d\nRadius: %g\n", W, S, K, R);
    if (got < W) {
        std::fprintf(stderr, "[Error] fewer points (%lld) than the window (%d)\n", got, W);
        return 2;
    }
    // the engine reads points [n][dim]: drop the padding coordinates
    std::vector<float> pts((size_t)got * dim);
    for (long long i = 0; i < got; ++i)
        for (int a = 0; a < dim; ++a) pts[(size_t)i * dim + a] = xyz[(size_t)i * 3 + a];

    rtdbs_params p;
    rtdbs_params_init(&p);
    p.dim = dim;
    p.window = W;
    p.stride = S;
    p.min_pts = K;
    p.eps = R;
    p.precision = precision;
    p.cell_mult = cell_mult;
    p.query_lanes = query_lanes;
    p.has_bbox = 1;
    for (int a = 0; a < 3; ++a) {
        p.bbox_min[a] = lo[a];
        p.bbox_max[a] = hi[a];
    }
    rtdbs_engine* eng = nullptr;
    if ((rc = rtdbs_create(&p, nullptr, &eng)) != RTDBS_OK) return die("rtdbs_create", rc);
    std::vector<int32_t> label(W), cid(W);
    const long long slides = (got - W) / S;
    std::printf("[Info] Total stride num: %lld\n", slides);
    double total_ms = 0.0;
    for (int pass = 0; pass <= warmup; ++pass) {
        const bool timed = pass == warmup;
        if ((rc = rtdbs_load_window(eng, pts.data(), 0)) != RTDBS_OK) return die("rtdbs_load_window", rc);
        for (long long k = 0; k < slides; ++k) {
            const float* stride = pts.data() + ((size_t)W + (size_t)k * S) * dim;
            const auto t0 = std::chrono::steady_clock::now();
            if ((rc = rtdbs_slide(eng, stride, label.data(), cid.data())) != RTDBS_OK)
                return die("rtdbs_slide", rc);
            const auto t1 = std::chrono::steady_clock::now();
            if (timed) total_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
        }
    }
    rtdbs_stats st;
    rtdbs_get_stats(eng, &st);
    const double q = slides > 0 ? (double)slides : 1.0;
    std::printf("\n###########   Time  ##########\n");
    std::printf("[Time] total: %g ms\n", total_ms / q);
    std::printf("[Info] slid points/s: %g\n", slides > 0 ? (double)S * slides / (total_ms / 1000.0) : 0.0);
    std::printf("[Info] band rechecks: %lld, cells: %lld, device bytes: %lld\n", (long long)st.band_rechecks,
                (long long)st.cells, (long long)st.device_bytes);
    std::printf("##############################\n\n");
    if (!labels_out.empty()) {
        FILE* fo = std::fopen(labels_out.c_str(), "wb");
        if (!fo) return die("open --labels file", RTDBS_ERR_INVALID);
        for (int i = 0; i < W; ++i) {
            const int32_t pair[2] = {label[i], cid[i]};
            std::fwrite(pair, sizeof(int32_t), 2, fo);
        }
        std::fclose(fo);
    }
    rtdbs_destroy(eng);
    return 0;
}
