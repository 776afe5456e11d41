// C ABI of libOctreeApi.so: the reference's 18 ocpi_* entry points
// (OctreeApi/include/octreeApi.h:42-72, OctreeApi/src/octreeApi.cpp:9-187)
// over a per-session builder, plus additive introspection entry points.
//
// Every entry point maps any exception (configuration errors, CUDA errors,
// device-side error flags) to UNEXPECTED_ERROR (-1), like the reference's
// Execute wrapper (octreeApi.cpp:9-21); unlike the reference, CUDA errors do
// not terminate the process.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "../../include/octreeApi.h"

#include "builder.h"

namespace {

thread_local std::string g_last_error;
int g_log_level = 1;

struct Session {
    int device = 0;
    oc::BuildConfig cfg;
    const uint8_t* host_cloud = nullptr;
    std::unique_ptr<oc::Builder> builder;
    std::string memory_report;
    oc::ReportExtras report;   // process times and allocations for statistics.json
    uint8_t* out_rec = nullptr;   // ocpi_set_output_host
    uint32_t* out_lut = nullptr;
    uint64_t out_cap = 0;

    int builder_sms = 152;

    // The reference's MemoryTracker writes its HTML report at process exit
    // (memory_tracker.cuh:31-55); here each session writes its own, listing
    // the device allocations it holds, when it is destroyed.
    ~Session() {
        if (!memory_report.empty() && builder) {
            FILE* f = std::fopen(memory_report.c_str(), "w");
            if (f) {
                uint64_t total = 0;
                std::fprintf(f, "<!DOCTYPE html>\n<html><head><title>Device memory</title></head><body>\n");
                std::fprintf(f, "<h3>Device memory of one octree session (%u points, stride %u)</h3>\n", cfg.n,
                             cfg.stride);
                std::fprintf(f, "<table border=\"1\"><tr><th>allocation</th><th>bytes</th><th>MB</th></tr>\n");
                for (const auto& a : builder->device_allocations()) {
                    total += a.second;
                    std::fprintf(f, "<tr><td>%s</td><td>%llu</td><td>%.3f</td></tr>\n", a.first.c_str(),
                                 (unsigned long long)a.second, a.second / 1e6);
                }
                std::fprintf(f, "<tr><th>total</th><th>%llu</th><th>%.3f</th></tr>\n</table>\n",
                             (unsigned long long)total, total / 1e6);
                std::fprintf(f, "<p>estimate for this configuration: %llu bytes (reference formula: %llu bytes)</p>\n",
                             (unsigned long long)oc::estimate_device_bytes(builder->config(), builder_sms),
                             (unsigned long long)oc::reference_estimate_bytes(builder->config()));
                std::fprintf(f, "</body></html>\n");
                std::fclose(f);
            }
        }
    }
};

Session* to_session(void* s) {
    if (!s) throw oc::Error("No Session is currently initialized!");   // session.cpp:11-19
    return static_cast<Session*>(s);
}

bool same_config(const oc::BuildConfig& a, const oc::BuildConfig& b) {
    for (int k = 0; k < 3; ++k)
        if (a.scale[k] != b.scale[k] || a.offset[k] != b.offset[k] || a.bb_min[k] != b.bb_min[k] ||
            a.bb_max[k] != b.bb_max[k])
            return false;
    return a.n == b.n && a.stride == b.stride && a.cloud_type == b.cloud_type && a.chunk_grid == b.chunk_grid &&
           a.threshold == b.threshold && a.output_factor == b.output_factor && a.sub_grid == b.sub_grid &&
           a.intra == b.intra && a.inter == b.inter && a.replacement == b.replacement && a.random == b.random &&
           a.weighting == b.weighting && a.seed == b.seed && a.debug == b.debug;
}

oc::Builder& built(Session* s) {
    if (!s->builder) throw oc::Error("octree not initialised (call ocpi_init_octree)");
    return *s->builder;
}

// Wall time of one API call and the device allocations it made, recorded in
// the session's report figures (the reference's TimeTracker "process" entries,
// session.cpp:62-76, and MemoryTracker events).
struct ProcessTimer {
    Session* s;
    const char* name;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    oc::AllocTally before = oc::thread_alloc_tally();
    ~ProcessTimer() {
        const oc::AllocTally& now = oc::thread_alloc_tally();
        s->report.allocs.ms += now.ms - before.ms;
        s->report.allocs.events += now.events - before.events;
        s->report.allocs.bytes += now.bytes - before.bytes;
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        for (auto& kv : s->report.process_ms)
            if (kv.first == name) {
                kv.second = ms;
                return;
            }
        s->report.process_ms.push_back({name, ms});
    }
};

template <class F>
int execute(F&& fn) {
    try {
        fn();
        return SUCCESS;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        if (g_log_level <= 3) std::fprintf(stderr, "[octree-gb300] error: %s\n", e.what());
        return UNEXPECTED_ERROR;
    } catch (...) {
        g_last_error = "unknown error";
        return UNEXPECTED_ERROR;
    }
}

}   // namespace

namespace oc {
// Records the message returned by ocpi_last_error() on this host thread.
void set_last_error(const std::string& msg) {
    g_last_error = msg;
    if (g_log_level <= 3) std::fprintf(stderr, "[octree-gb300] error: %s\n", msg.c_str());
}
}   // namespace oc

extern "C" {

int ocpi_set_logging_level(int level) {
    return execute([&] { g_log_level = (level >= 0 && level <= 3) ? level : 0; });
}

int ocpi_create_session(void** session, int device) {
    return execute([&] {
        if (!session) throw oc::Error("null session pointer");
        auto s = std::make_unique<Session>();
        s->device = device;
        // session.cpp:27-46 binds the device and also switches the whole
        // process to blocking synchronisation.  That flag is process-wide and
        // makes each of a build's host waits a sleep and a wake-up (about
        // 70 us each, about 0.8 ms of a one-million-point build), so the
        // device's scheduling flags are left as the application set them.
        oc::check_cuda(cudaSetDevice(device), "cudaSetDevice");
        *session = s.release();
    });
}

int ocpi_destroy_session(void* session) {
    return execute([&] { delete to_session(session); });
}

int ocpi_set_point_cloud_host(void* session, uint8_t* pointCloud) {
    return execute([&] { to_session(session)->host_cloud = pointCloud; });
}

int ocpi_set_cloud_type(void* session, uint8_t cloudType) {
    return execute([&] { to_session(session)->cfg.cloud_type = cloudType; });
}

int ocpi_set_cloud_point_amount(void* session, uint32_t pointAmount) {
    return execute([&] { to_session(session)->cfg.n = pointAmount; });
}

int ocpi_set_cloud_data_stride(void* session, uint32_t dataStride) {
    return execute([&] { to_session(session)->cfg.stride = dataStride; });
}

int ocpi_set_cloud_scale(void* session, double x, double y, double z) {
    return execute([&] {
        auto* s = to_session(session);
        s->cfg.scale[0] = x;
        s->cfg.scale[1] = y;
        s->cfg.scale[2] = z;
    });
}

int ocpi_set_cloud_offset(void* session, double x, double y, double z) {
    return execute([&] {
        auto* s = to_session(session);
        s->cfg.offset[0] = x;
        s->cfg.offset[1] = y;
        s->cfg.offset[2] = z;
    });
}

int ocpi_set_cloud_bb(void* session, double minX, double minY, double minZ, double maxX, double maxY, double maxZ) {
    return execute([&] {
        auto* s = to_session(session);
        s->cfg.bb_min[0] = minX;
        s->cfg.bb_min[1] = minY;
        s->cfg.bb_min[2] = minZ;
        s->cfg.bb_max[0] = maxX;
        s->cfg.bb_max[1] = maxY;
        s->cfg.bb_max[2] = maxZ;
    });
}

int ocpi_configure_chunking(void* session, uint32_t chunkingGrid, uint32_t mergingThreshold, float outputFactor) {
    return execute([&] {
        auto* s = to_session(session);
        s->cfg.chunk_grid = chunkingGrid;
        s->cfg.threshold = mergingThreshold;
        s->cfg.output_factor = outputFactor;
    });
}

int ocpi_configure_subsampling(void* session, uint32_t subsamplingGrid, bool intraCellAveraging,
                               bool interCellAveraging, bool replacementScheme, bool useRandomSubsampling,
                               bool useWeightingFunction) {
    return execute([&] {
        auto* s = to_session(session);
        s->cfg.sub_grid = subsamplingGrid;
        s->cfg.intra = intraCellAveraging;
        s->cfg.inter = interCellAveraging;
        s->cfg.replacement = replacementScheme;
        s->cfg.random = useRandomSubsampling;
        s->cfg.weighting = useWeightingFunction;
    });
}

int ocpi_init_octree(void* session) {
    return execute([&] {
        auto* s = to_session(session);
        ProcessTimer timer{s, "Initialising octree"};
        oc::check_cuda(cudaSetDevice(s->device), "cudaSetDevice");
        if (s->builder && same_config(s->builder->config(), s->cfg)) {
            // same configuration: reuse device state; the upload goes in
            // chunks and bins each chunk as it lands (when the box is known)
            s->builder->upload(s->host_cloud, true, true);
            return;
        }
        if (s->builder) {
            // another configuration: the same buffers, grown where needed.  A
            // failure part-way (an allocation) leaves buffers sized for neither
            // configuration, so the builder is dropped.
            try {
                s->builder->reconfigure(s->cfg, s->host_cloud, true, true);
            } catch (...) {
                s->builder.reset();
                throw;
            }
            if (s->out_rec) s->builder->set_output_host(s->out_rec, s->out_lut, s->out_cap);
            return;
        }
        s->builder = std::make_unique<oc::Builder>(s->cfg, s->host_cloud, s->device, true);
        cudaDeviceGetAttribute(&s->builder_sms, cudaDevAttrMultiProcessorCount, s->device);
        if (s->out_rec) s->builder->set_output_host(s->out_rec, s->out_lut, s->out_cap);
    });
}

int ocpi_generate_octree(void* session) {
    return execute([&] {
        auto* s = to_session(session);
        ProcessTimer timer{s, "Generating octree"};
        oc::check_cuda(cudaSetDevice(s->device), "cudaSetDevice");
        built(s).generate();
    });
}

int ocpi_export_potree(void* session, const char* directory) {
    return execute([&] {
        if (!directory) throw oc::Error("null directory");
        auto* s = to_session(session);
        ProcessTimer timer{s, "Exporting octree"};
        built(s).export_potree(directory);
    });
}

int ocpi_export_json_report(void* session, const char* filename) {
    return execute([&] {
        if (!filename) throw oc::Error("null filename");
        auto* s = to_session(session);
        built(s).export_json_report(filename, s->report);
    });
}

int ocpi_export_distribution_histogram(void* session, const char* filename, uint32_t binWidth) {
    return execute([&] {
        if (!filename) throw oc::Error("null filename");
        built(to_session(session)).export_histogram(filename, binWidth);
    });
}

int ocpi_export_memory_report(void* session, const char* filename) {
    return execute([&] {
        if (!filename) throw oc::Error("null filename");
        to_session(session)->memory_report = filename;
    });
}

// ---- additions

const char* ocpi_last_error(void) {
    return g_last_error.c_str();
}

int ocpi_set_random_seed(void* session, uint64_t seed) {
    return execute([&] { to_session(session)->cfg.seed = seed; });
}

int ocpi_set_debug_flags(void* session, uint32_t flags) {
    return execute([&] { to_session(session)->cfg.debug = flags; });
}

int ocpi_get_stats(void* session, OcpiStats* out) {
    return execute([&] {
        if (!out) throw oc::Error("null output");
        const oc::Stats& S = built(to_session(session)).stats();
        OcpiStats o{};
        o.points_total = S.points_total;
        o.p_out = S.p_out;
        o.p_in = S.p_in;
        o.out_capacity = S.out_capacity;
        o.depth = S.depth;
        o.tree_nodes = S.tree_nodes;
        o.leaf_nodes = S.leaf_nodes;
        o.internal_nodes = S.internal_nodes;
        o.sparse_nodes = S.sparse_nodes;
        o.dense_nodes = S.dense_nodes;
        o.max_leaf_depth = S.max_leaf_depth;
        o.min_leaf_points = S.min_leaf_points;
        o.max_leaf_points = S.max_leaf_points;
        o.mean_leaf_points = S.mean_leaf_points;
        o.stdev_leaf_points = S.stdev_leaf_points;
        o.kernel_launches = S.kernel_launches;
        o.subsample_passes = S.subsample_passes;
        *out = o;
    });
}

int ocpi_get_node_count(void* session, uint64_t* count) {
    return execute([&] {
        if (!count) throw oc::Error("null output");
        *count = built(to_session(session)).nodes().size();
    });
}

int ocpi_get_hierarchy(void* session, uint8_t* out) {
    return execute([&] {
        if (!out) throw oc::Error("null output");
        auto h = built(to_session(session)).hierarchy();
        std::memcpy(out, h.data(), h.size());
    });
}

int ocpi_get_records(void* session, uint8_t* out) {
    return execute([&] {
        if (!out) throw oc::Error("null output");
        auto& b = built(to_session(session));
        if (!b.records_filled(out)) b.copy_records(out);   // else generate already filled it
    });
}

int ocpi_get_lut(void* session, uint32_t* out) {
    return execute([&] {
        if (!out) throw oc::Error("null output");
        auto& b = built(to_session(session));
        if (!b.lut_filled(out)) b.copy_lut(out);
    });
}

int ocpi_get_device_memory(void* session, uint64_t* bytes) {
    return execute([&] {
        if (!bytes) throw oc::Error("null output");
        auto* s = to_session(session);
        uint64_t total = 0;
        if (s->builder)
            for (const auto& a : s->builder->device_allocations()) total += a.second;
        *bytes = total;
    });
}

int ocpi_estimate_memory(uint32_t pointAmount, uint32_t dataStride, uint8_t cloudType, uint32_t chunkingGrid,
                         uint32_t mergingThreshold, float outputFactor, uint32_t subsamplingGrid, uint32_t modeFlags,
                         uint64_t* gb300Bytes, uint64_t* referenceBytes) {
    return execute([&] {
        oc::BuildConfig c;
        c.n = pointAmount;
        c.stride = dataStride;
        c.cloud_type = cloudType;
        c.chunk_grid = chunkingGrid;
        c.threshold = mergingThreshold;
        c.output_factor = outputFactor;
        c.sub_grid = subsamplingGrid;
        c.intra = (modeFlags & OCPI_SUB_INTRA) != 0;
        c.inter = (modeFlags & OCPI_SUB_INTER) != 0;
        c.random = (modeFlags & OCPI_SUB_RANDOM) != 0;
        c.weighting = (modeFlags & OCPI_SUB_WEIGHTING) != 0;
        c.validate();
        int sms = 0, dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
            cudaGetLastError();
            sms = 152;   // GB300
        }
        if (gb300Bytes) *gb300Bytes = oc::estimate_device_bytes(c, sms);
        if (referenceBytes) *referenceBytes = oc::reference_estimate_bytes(c);
    });
}

int ocpi_compute_cloud_bb(void* session, double* realBB, double* cubicBB) {
    return execute([&] {
        auto* s = to_session(session);
        oc::check_cuda(cudaSetDevice(s->device), "cudaSetDevice");
        double real[6], cubic[6];
        built(s).compute_bbox(real, cubic);
        for (int a = 0; a < 3; ++a) {
            s->cfg.bb_min[a] = cubic[a];
            s->cfg.bb_max[a] = cubic[a + 3];
        }
        if (realBB) std::memcpy(realBB, real, sizeof real);
        if (cubicBB) std::memcpy(cubicBB, cubic, sizeof cubic);
    });
}

int ocpi_set_output_host(void* session, uint8_t* records, uint32_t* lut, uint64_t capacity) {
    return execute([&] {
        auto* s = to_session(session);
        s->out_rec = records;
        s->out_lut = lut;
        s->out_cap = capacity;
        if (s->builder) s->builder->set_output_host(records, lut, capacity);
    });
}

int ocpi_get_level_counts(void* session, uint32_t level, uint32_t* out) {
    return execute([&] {
        if (!out) throw oc::Error("null output");
        if (!built(to_session(session)).level_counts(level, out))
            throw oc::Error("pyramid copy not available (set debug flag 1 before ocpi_init_octree)");
    });
}

int ocpi_get_timings(void* session, double* ms, int max, char* names, int name_bytes, int* count) {
    return execute([&] {
        const auto& t = built(to_session(session)).timings();
        std::string joined;
        int n = 0;
        for (const auto& kv : t) {
            if (n >= max) break;
            if (ms) ms[n] = kv.second;
            joined += (n ? "," : "") + kv.first;
            ++n;
        }
        if (names && name_bytes > 0) {
            std::strncpy(names, joined.c_str(), (size_t)name_bytes - 1);
            names[name_bytes - 1] = 0;
        }
        if (count) *count = n;
    });
}

}   // extern "C"
