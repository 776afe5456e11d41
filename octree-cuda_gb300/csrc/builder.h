// LOD octree builder: owns the device state of one session and runs the
// stages of the OctreeApi pipeline (OctreeProcessorImpl in the reference,
// OctreeLibrary/src/include/octree_processor_impl.cuh:14-71).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "kernels.h"

#include <nvtx3/nvToolsExt.h>

namespace oc {

// A named NVTX range for the lifetime of the object (host phases of a build
// on a profiler's timeline; nearly free when no tool is attached).
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

struct Error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void check_cuda(cudaError_t e, const char* what);

// PointCloudInfo + ProcessingInfo (OctreeLibrary/include/metadata.cuh:55-101).
struct BuildConfig {
    uint32_t n = 0;
    uint32_t stride = 0;
    uint32_t cloud_type = 0;
    double scale[3] = {1, 1, 1};
    double offset[3] = {0, 0, 0};
    double bb_min[3] = {0, 0, 0};
    double bb_max[3] = {0, 0, 0};
    uint32_t chunk_grid = 0;
    uint32_t threshold = 0;
    float output_factor = 0.f;
    uint32_t sub_grid = 0;
    bool intra = false, inter = false, replacement = false, random = false, weighting = false;
    uint64_t seed = 0x5EED;
    uint32_t debug = 0;

    void validate() const;
    // a bounding box was given (all six values zero means "not set yet")
    bool has_bbox() const {
        for (int a = 0; a < 3; ++a)
            if (bb_min[a] != 0.0 || bb_max[a] != 0.0) return true;
        return false;
    }
};

// Device allocations made by the calling thread: host time spent in
// cudaMalloc, number of allocations and bytes.  The session layer takes the
// difference around each API call for the statistics report.
struct AllocTally {
    double ms = 0;
    uint64_t events = 0;
    uint64_t bytes = 0;
};
AllocTally& thread_alloc_tally();

// Host-side figures of a session that the statistics report lists beside the
// build's own: wall time of the API calls (json_exporter.h "process") and the
// session's device allocations (json_exporter.h "cudamalloc" and "memory").
struct ReportExtras {
    std::vector<std::pair<std::string, double>> process_ms;
    AllocTally allocs;
};

// Grow-only device allocation.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf();
    void ensure(size_t b);
    void ensure_keep(size_t b, size_t keep, cudaStream_t s);   // grow, preserving the first `keep` bytes
    void release();
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// Grow-only page-locked host allocation: staging of the small transfers of a
// build (parameter tables up, node tables and counters down), so that they
// are true asynchronous copies on the build stream.
struct HostBuf {
    void* p = nullptr;
    size_t bytes = 0;
    HostBuf() = default;
    HostBuf(const HostBuf&) = delete;
    HostBuf& operator=(const HostBuf&) = delete;
    ~HostBuf();
    void ensure(size_t b);
    void release();
    template <class T>
    T* as(size_t byte_offset = 0) const {
        return reinterpret_cast<T*>(static_cast<uint8_t*>(p) + byte_offset);
    }
};

struct NodeHost {
    uint32_t key;          // Morton key within its level
    uint32_t count;        // pyramid count (points below the cell)
    uint32_t level;        // 0 = finest chunking level
    uint32_t child_first;  // BFS index of the first child (internal nodes)
    uint8_t internal;
    uint8_t mask;          // occupied children (internal nodes)
    uint32_t points;       // points referenced by the hierarchy entry
    uint64_t data_idx;     // first record in octree.bin
    uint64_t stage_off;    // staged position of an internal node's output
    double mn[3];          // bbox minimum (calculateChildMinBB chain)
};

struct Stats {
    uint64_t points_total = 0, p_out = 0, p_in = 0, out_capacity = 0;
    uint32_t depth = 0, tree_nodes = 0, leaf_nodes = 0, internal_nodes = 0, sparse_nodes = 0, dense_nodes = 0;
    uint32_t max_leaf_depth = 0, min_leaf_points = 0, max_leaf_points = 0;
    float mean_leaf_points = 0.f, stdev_leaf_points = 0.f;
    uint32_t kernel_launches = 0;   // kernels launched by the last generate
    uint32_t subsample_passes = 0;  // 1, or more when the subsampling pass was repeated with larger buffers
};

// Upper bound of the device memory a session allocates for a configuration
// (the Builder's own sizing rules; data-dependent buffers at their capacity
// rules), and the reference's estimate (tools/memory_consumption.py:30-75).
uint64_t estimate_device_bytes(const BuildConfig& cfg, int num_sms);
uint64_t reference_estimate_bytes(const BuildConfig& cfg);

// The quantities the device buffers are sized from.  A builder reconfigured
// through several configurations (its buffers only grow) stays within
// device_bytes of the envelope of their terms.
struct MemoryTerms {
    uint64_t cloud_bytes = 0, n = 0, cells = 0, node_cap = 0, out_cap = 0, slots = 0;
    uint32_t chunk_grid = 0;
    bool random = false, packed = false, weighted = false;
    int sms = 0;
};
MemoryTerms memory_terms(const BuildConfig& cfg, int num_sms);
MemoryTerms envelope(const MemoryTerms& a, const MemoryTerms& b);
uint64_t device_bytes(const MemoryTerms& t);

// Host-side fault injection for tests: the next `count` events of a kind
// fail.  Allocation: a device or pinned allocation throws as if cudaMalloc
// had failed.  Lane loss: a server lane drops its job and state as if its
// worker had died, and restarts.
enum InjectKind : int { kInjectAllocation = 1, kInjectLaneLoss = 2 };
void inject_failures(int kind, uint32_t count);
bool consume_injected_failure(int kind);

// Throws the message of the first error bit set in a device error word.
void throw_device_errors(uint32_t e, const char* stage);

class Wave;

class Builder {
public:
    // count = true: see upload().
    Builder(const BuildConfig& cfg, const uint8_t* host_cloud, int device, bool count = false);
    ~Builder();
    Builder(const Builder&) = delete;
    Builder& operator=(const Builder&) = delete;

    // Uploads a new cloud of the same configuration (reuses allocations).
    // wait = false leaves the copy in flight on the build stream: the host
    // cloud must then stay valid until generate() returns.  count = true and
    // a known bounding box: the copy goes in chunks on the side stream and
    // each chunk is binned on the build stream as soon as it has landed, so
    // counting hides under the copy and the next generate() skips it.
    void upload(const uint8_t* host_cloud, bool wait = true, bool count = false);
    // A new configuration and cloud; buffers only grow (see size_for_config).
    // A cloud given to prefetch() before (same host pointer and size) is
    // adopted from the spare buffer instead of being copied again.
    void reconfigure(const BuildConfig& cfg, const uint8_t* host_cloud, bool wait_upload = true, bool count = false);
    // Starts copying the cloud of a later build (`bytes` from host_cloud)
    // into a spare device buffer, on a stream of its own, so that the copy
    // overlaps the build in progress.  The host cloud must stay valid until
    // reconfigure() adopts it or prefetch_sync() returns.  Throws what an
    // allocation throws; the spare buffer only grows.
    void prefetch(const uint8_t* host_cloud, uint64_t bytes);
    // Waits for a prefetch copy in flight and forgets it.
    void prefetch_sync();
    uint64_t spare_bytes() const { return spare_.bytes; }
    // Resident state: after a successful generate(), the uploaded cloud, the
    // count pyramid, the node tree and the leaf records stay on the device.
    // If `cfg` differs from the last build only in its subsampling settings
    // (grid, modes, seed, output factor), reuse() adopts them and the next
    // generate() runs subsampling alone; otherwise it returns false and
    // changes nothing.  A job whose box is unset matches a state whose box
    // was computed on the device.
    bool reuse(const BuildConfig& cfg);
    void generate();
    // Real and cubic bounding boxes {minX, minY, minZ, maxX, maxY, maxZ} of
    // the uploaded cloud; the cubic box becomes the build's bounding box.
    void compute_bbox(double real[6], double cubic[6]);
    void export_potree(const std::string& dir) const;
    void export_json_report(const std::string& file, const ReportExtras& extras) const;
    void export_histogram(const std::string& file, uint32_t bin_width) const;

    const Stats& stats() const { return stats_; }
    const std::vector<NodeHost>& nodes() const { return nodes_; }
    std::vector<uint8_t> hierarchy() const;
    void copy_records(uint8_t* out) const;
    void copy_lut(uint32_t* out);
    bool level_counts(uint32_t level, uint32_t* out) const;
    const std::vector<std::pair<std::string, double>>& timings() const { return timings_; }
    cudaStream_t stream() const { return stream_; }
    // Host arrays that generate() fills with octree.bin records (and LUT
    // entries when lut != nullptr); capacity in records.  The leaf part is
    // copied while subsampling runs.
    void set_output_host(uint8_t* records, uint32_t* lut, uint64_t capacity);
    // The subsampling levels of the next builds (their first pass) meet the
    // other builds of `wave` in slot `slot`: one launch per level over all
    // of them.  nullptr: the builder subsamples alone.
    void join_wave(Wave* wave, uint32_t slot) {
        wave_ = wave;
        wave_slot_ = slot;
    }
    bool records_filled(const void* records) const { return host_filled_ && records == host_rec_; }
    bool reused() const { return reuse_tree_; }
    bool lut_filled(const void* lut) const { return host_filled_ && host_lut_ && lut == host_lut_; }
    const BuildConfig& config() const { return cfg_; }
    // Device memory held by this session: named allocations in bytes.
    std::vector<std::pair<std::string, uint64_t>> device_allocations() const;

private:
    void stage_mark(const char* name);
    void stage_begin();
    void collect_timings();
    void check_device_errors(const char* stage);
    void build_tree_host();
    void fill_cell_tables();
    CloudGrid cloud_grid() const;
    bool sparse_cloud() const;
    void clear_for_count(bool sparse);
    void params_writable();
    void record_params();
    void size_for_config();
    void subsample();
    void compute_stats();

    BuildConfig cfg_;
    int device_ = 0;
    int num_sms_ = 0;
    Wave* wave_ = nullptr;
    uint32_t wave_slot_ = 0;
    cudaEvent_t level_ready_ = nullptr;   // a level's tables are prepared (waves)
    cudaStream_t stream_ = nullptr;
    uint32_t depth_ = 0;
    std::vector<uint64_t> level_off_;   // pyramid level offsets (cells), depth + 2 entries
    uint32_t node_cap_ = 0;

    DevBuf cloud_, pyr_, loff_, err_, nonzero_;
    DevBuf spare_;                      // cloud of the next build, copied while this one runs
    const uint8_t* prefetched_ = nullptr;   // host cloud in flight to spare_ (nullptr: none)
    uint64_t prefetched_bytes_ = 0;
    DevBuf occ_;                        // sparse clouds: one flag byte per 64-cell block of the finest level
    bool pyr_zero_ = false;             // the pyramid and the flags are all zero (sparse clean-up ran)
    DevBuf key_, count_, level_, info_, child_first_, level_start_, n_nodes_;
    DevBuf data_idx_, fill_;
    DevBuf lut_, rec_;                  // final outputs (N + P_out records)
    DevBuf stage_lut_, stage_rec_;      // staged internal outputs
    DevBuf sub_nodes_, out_points_, work_;
    DevBuf key_cache_, unit_cache_, acc_best_, acc_sel_, cell_slot_, acc_intra_, emit_maps_, emit_state_, csr_count_, csr_start_, csr_pts_;
    DevBuf place_src_, place_dst_, place_cnt_;
    DevBuf g_key_, g_mask_, g_base_;   // per-block global brick tables
    DevBuf cell_keys_, spread_;         // chunking-grid boundary keys and Morton spread table
    DevBuf leaf_frac_, stage_frac_;     // sub-step words of leaf and staged records
    DevBuf bbox_keys_;                  // ordered keys of the coordinate minima / maxima
    DevBuf stage_off_, level_base_;     // staged position of each internal node's outputs; staging fill
    uint8_t* host_rec_ = nullptr;      // caller's output arrays (set_output_host)
    uint32_t* host_lut_ = nullptr;
    uint64_t host_cap_ = 0;
    bool host_filled_ = false;
    cudaStream_t copy_stream_ = nullptr;
    cudaStream_t side_stream_ = nullptr;   // reads the node table while distribution runs
    cudaEvent_t tree_ready_ = nullptr;
    cudaStream_t prefetch_stream_ = nullptr;
    cudaEvent_t prefetch_done_ = nullptr;   // the spare buffer holds the prefetched cloud
    cudaEvent_t spare_free_ = nullptr;      // the build stream's last use of the buffer that became spare
    cudaEvent_t leaf_ready_ = nullptr;
    DevBuf post_ii_, node_dst_, out_total_;   // post-order of internal nodes, their output positions, P_out
    HostBuf loff_host_, keys_host_, spread_host_;   // staged parameter tables (uploaded on the build stream)
    HostBuf tree_host_, table_host_, back_host_;    // node table down, subsampling node table up, counters down
    cudaEvent_t params_done_ = nullptr;             // the staged parameter tables have been copied
    bool params_pending_ = false;
    uint32_t spread_grid_ = 0;                      // grid of the Morton spread table on the device
    uint32_t nonzero_sum_ = 0;                      // occupied cells over all levels
    uint32_t sub_err_ = 0;                          // device error word read after subsampling
    bool sub_err_valid_ = false;
    bool tree_valid_ = false;        // the device holds the tree and leaf records of cfg_ (last generate succeeded)
    bool bbox_from_device_ = false;  // cfg_'s box came from compute_bbox
    bool reuse_tree_ = false;        // the next generate() subsamples the resident tree
    bool counted_ = false;           // upload() binned the cloud: the next generate() skips counting
    std::vector<cudaEvent_t> chunk_ready_;   // chunks of an overlapped upload
    uint64_t sub_stage_cap_ = 0, sub_scratch_cap_ = 0, sub_rec_cap_ = 0;   // capacities that fit the last build
    uint32_t g_cap_ = 0, g_shift_ = 0;
    uint32_t launches_ = 0;
    size_t place_count_ = 0;
    bool lut_placed_ = false;

    std::vector<NodeHost> nodes_;
    std::vector<uint32_t> leaf_ids_;
    std::vector<std::vector<uint32_t>> internal_by_level_;
    std::vector<std::vector<uint32_t>> pyramid_copy_;
    uint64_t p_out_ = 0;
    uint64_t stage_used_ = 0;
    Stats stats_;

    std::vector<std::pair<std::string, cudaEvent_t>> events_;
    std::vector<cudaEvent_t> event_pool_;
    std::vector<std::pair<std::string, double>> timings_;
};

}   // namespace oc
