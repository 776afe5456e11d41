/*
 * Runner of the reference's own CUDA pipeline -- TEST INFRASTRUCTURE ONLY.
 *
 * Linked against the reference's OctreeApi + OctreeLibrary objects, which
 * oracle/build_ref.py compiles unmodified for sm_103a into oracle/_ref/.  It
 * drives the reference exactly as its CLI does (src/main.cpp:54-107): read the
 * cloud file, compute the CLI bounding box with the CLI's own helpers
 * (src/boundingbox.h:11-52), then the session calls in the CLI's order.  It
 * adds only timing and repetition:
 *
 *   init_ms     ocpi_init_octree (allocation + host-to-device upload)
 *   generate_ms ocpi_generate_octree, followed by cudaDeviceSynchronize
 *
 * The cloud is held in page-locked host memory (cudaMallocHost) unless
 * --pageable is given, so the reference's upload runs at the same link speed
 * as the product's pinned upload.  Every repetition calls ocpi_init_octree and
 * ocpi_generate_octree on the same session, which is how the reference API
 * rebuilds (Session::initOctree, OctreeApi/src/session.cpp:151-154).
 *
 * Output: one JSON object on stdout.  Exit status 0 on success, 2 on a failed
 * API call (the reference itself exits with the CUDA error code on a device
 * error, defines.cuh:22-30).
 */
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "boundingbox.h"
#include "octreeApi.h"

namespace {

struct Args
{
    std::string cloud;
    uint32_t points = 0, stride = 15, type = 0;
    double scale = 0.001;
    uint32_t chunk = 512, sub = 128, threshold = 10000;
    float factor = 2.2f;
    bool intra = false, inter = false, replace = false, random = false, weight = false;
    int reps = 1;
    bool pageable = false;
    int log = 2;
    std::string out, report;
};

double now_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

bool parse(int argc, char** argv, Args& a)
{
    for (int i = 1; i < argc; ++i)
    {
        std::string k = argv[i];
        auto val = [&](void) -> const char* { return (i + 1 < argc) ? argv[++i] : nullptr; };
        const char* v = nullptr;
        if (k == "--intra") a.intra = true;
        else if (k == "--inter") a.inter = true;
        else if (k == "--replace") a.replace = true;
        else if (k == "--random") a.random = true;
        else if (k == "--weight") a.weight = true;
        else if (k == "--pageable") a.pageable = true;
        else if ((v = val()) == nullptr) return false;
        else if (k == "--cloud") a.cloud = v;
        else if (k == "--points") a.points = (uint32_t)strtoul(v, nullptr, 10);
        else if (k == "--stride") a.stride = (uint32_t)strtoul(v, nullptr, 10);
        else if (k == "--type") a.type = std::string(v) == "double" ? 1u : 0u;
        else if (k == "--scale") a.scale = strtod(v, nullptr);
        else if (k == "--chunk") a.chunk = (uint32_t)strtoul(v, nullptr, 10);
        else if (k == "--sub") a.sub = (uint32_t)strtoul(v, nullptr, 10);
        else if (k == "--threshold") a.threshold = (uint32_t)strtoul(v, nullptr, 10);
        else if (k == "--factor") a.factor = strtof(v, nullptr);
        else if (k == "--reps") a.reps = atoi(v);
        else if (k == "--log") a.log = atoi(v);
        else if (k == "--out") a.out = v;
        else if (k == "--report") a.report = v;
        else return false;
    }
    return !a.cloud.empty() && a.points > 0 && a.reps > 0;
}

void print_list(const char* key, const std::vector<double>& v)
{
    printf("\"%s\": [", key);
    for (size_t i = 0; i < v.size(); ++i) printf("%s%.6f", i ? ", " : "", v[i]);
    printf("]");
}

}  // namespace

int main(int argc, char** argv)
{
    Args a;
    if (!parse(argc, argv, a))
    {
        fprintf(stderr,
                "usage: ref_runner --cloud FILE --points N [--stride S] [--type float|double] [--scale s]\n"
                "       [--chunk G] [--sub G] [--threshold T] [--factor F] [--intra] [--inter] [--replace]\n"
                "       [--random] [--weight] [--reps R] [--pageable] [--out DIR] [--report FILE]\n"
                "       [--log 0-3]\n");
        return 1;
    }
    const size_t bytes = (size_t)a.points * a.stride;

    // The CLI reads the whole file into one host buffer (src/main.cpp:12-22).
    uint8_t* host = nullptr;
    if (a.pageable)
        host = new uint8_t[bytes];
    else if (cudaMallocHost((void**)&host, bytes) != cudaSuccess)
    {
        fprintf(stderr, "cudaMallocHost of %zu bytes failed\n", bytes);
        return 2;
    }
    {
        std::ifstream ifs(a.cloud, std::ios::binary);
        ifs.read(reinterpret_cast<char*>(host), (std::streamsize)bytes);
        if ((size_t)ifs.gcount() != bytes)
        {
            fprintf(stderr, "cloud file %s holds fewer than %zu bytes\n", a.cloud.c_str(), bytes);
            return 1;
        }
    }

    // The CLI's bounding box: real box, then the cube around it.
    std::unique_ptr<uint8_t[]> view(host);
    std::vector<double> real = a.type == 0 ? calculateRealBB<float>(view, a.points, a.stride)
                                           : calculateRealBB<double>(view, a.points, a.stride);
    (void)view.release();
    std::vector<double> bb = calculateCubicBB(real);

    int rc = 0;
    auto call = [&](const char* what, int r) {
        if (r != 0 && rc == 0)
        {
            fprintf(stderr, "%s returned %d\n", what, r);
            rc = 2;
        }
        return r == 0;
    };

    ocpi_set_logging_level(a.log);
    void* session = nullptr;
    call("ocpi_create_session", ocpi_create_session(&session, 0));

    std::vector<double> init_ms, gen_ms;
    double export_ms = 0.0;
    for (int rep = 0; rep < a.reps && rc == 0; ++rep)
    {
        call("ocpi_set_cloud_type", ocpi_set_cloud_type(session, (uint8_t)a.type));
        call("ocpi_set_cloud_point_amount", ocpi_set_cloud_point_amount(session, a.points));
        call("ocpi_set_cloud_data_stride", ocpi_set_cloud_data_stride(session, a.stride));
        call("ocpi_set_cloud_scale", ocpi_set_cloud_scale(session, a.scale, a.scale, a.scale));
        call("ocpi_set_cloud_offset", ocpi_set_cloud_offset(session, bb[0], bb[1], bb[2]));
        call("ocpi_set_cloud_bb", ocpi_set_cloud_bb(session, bb[0], bb[1], bb[2], bb[3], bb[4], bb[5]));
        call("ocpi_set_point_cloud_host", ocpi_set_point_cloud_host(session, host));
        call("ocpi_configure_chunking", ocpi_configure_chunking(session, a.chunk, a.threshold, a.factor));
        call("ocpi_configure_subsampling",
             ocpi_configure_subsampling(session, a.sub, a.intra, a.inter, a.replace, a.random, a.weight));
        if (rc) break;
        cudaDeviceSynchronize();
        double t0 = now_ms();
        if (!call("ocpi_init_octree", ocpi_init_octree(session))) break;
        cudaDeviceSynchronize();
        double t1 = now_ms();
        if (!call("ocpi_generate_octree", ocpi_generate_octree(session))) break;
        cudaDeviceSynchronize();
        double t2 = now_ms();
        init_ms.push_back(t1 - t0);
        gen_ms.push_back(t2 - t1);
    }
    if (rc == 0 && !a.out.empty())
    {
        double t0 = now_ms();
        call("ocpi_export_potree", ocpi_export_potree(session, a.out.c_str()));
        export_ms = now_ms() - t0;
    }
    if (rc == 0 && !a.report.empty()) call("ocpi_export_json_report", ocpi_export_json_report(session, a.report.c_str()));
    if (session) ocpi_destroy_session(session);

    printf("{\"rc\": %d, \"points\": %u, \"bb\": [%.17g, %.17g, %.17g, %.17g, %.17g, %.17g], ", rc, a.points, bb[0],
           bb[1], bb[2], bb[3], bb[4], bb[5]);
    print_list("init_ms", init_ms);
    printf(", ");
    print_list("generate_ms", gen_ms);
    printf(", \"export_ms\": %.6f, \"pinned\": %s}\n", export_ms, a.pageable ? "false" : "true");
    fflush(stdout);

    if (a.pageable)
        delete[] host;
    else
        cudaFreeHost(host);
    return rc;
}
