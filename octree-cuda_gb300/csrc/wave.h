// Subsampling waves: the builds of a batch run on their own builders and host
// threads up to subsampling.  There each hands the wave its whole subsampling
// plan (per level: the level's nodes and the launch that prepares them), and
// the last one to arrive issues the plans of all of them as one schedule: per
// step, every build's level preparation, then one subsampling launch over the
// step's nodes of all builds.  A cloud's top levels hold a few nodes; alone
// they leave most SMs idle, together with other clouds' they fill them.  The
// schedule is captured into a CUDA graph and launched once (it falls back to
// direct launches where the capture fails).
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <vector>

#include "builder.h"
#include "kernels.h"

namespace oc {

// One level of a build's subsampling plan.
struct WaveLevel {
    SubLevelArgs a;                               // the level's arguments (nodes, n_nodes, out_points set)
    std::vector<uint64_t> bounds;                 // candidate bound of each node, in the level's order
    std::function<void(cudaStream_t)> prepare;    // launches the build's k_prepare_level of this level
};

class Wave {
public:
    Wave(int device, int num_sms);
    ~Wave();
    Wave(const Wave&) = delete;
    Wave& operator=(const Wave&) = delete;

    // A new wave of builds with the given tree depths (log2 of the chunking
    // grid), one slot each.  Levels are aligned at the root: level l of a
    // build of depth d is step l + (max depth - d).  No build may still be in
    // the previous wave.  The wave's own buffers are sized here, before any
    // build runs, for at most `max_nodes` nodes over all steps and brick
    // tables of `max_global_cap` slots, so that issuing allocates nothing.
    void start(const std::vector<uint32_t>& depths, uint64_t max_nodes, uint32_t max_global_cap);

    // Slot `slot` hands over its first subsampling pass: levels[l - 1] is
    // its level l (n_nodes 0: no nodes there).  `ready` (recorded on
    // `stream`) marks its level tables as uploaded.  Returns once the wave's
    // schedule is issued, with `stream` waiting for all of it.
    void submit(uint32_t slot, std::vector<WaveLevel> levels, uint32_t global_cap, cudaEvent_t ready,
                cudaStream_t stream);

    // Slot `slot` submits nothing (it failed before subsampling).
    void leave(uint32_t slot);

    // Capture the schedule into a CUDA graph (default) or launch it directly;
    // the cluster caps of its subsampling launches.
    void set_graphs(bool on) { graphs_ = on; }
    void set_cluster_caps(const ClusterCaps& caps) { caps_ = caps; }
    // How the last wave was issued: 1 one graph launch, 0 direct launches.
    int last_issue() const { return last_issue_; }

    // Device bytes a wave of `builds` builds with the given bounds holds
    // (the per-block brick tables and the node tables of all steps).
    static uint64_t bytes_for(int num_sms, uint32_t builds, uint64_t max_nodes, uint32_t max_global_cap);
    // Device bytes this wave holds now (its buffers only grow).
    uint64_t device_bytes() const;

private:
    struct Plan {
        std::vector<WaveLevel> levels;
        uint32_t global_cap = 0;
        cudaEvent_t ready = nullptr;
        bool submitted = false;
        bool gone = false;
    };
    struct Step {
        size_t table_off = 0;      // byte offset of the step's tables in table_
        uint32_t n_nodes = 0;
        uint32_t balance = 1;
        uint32_t node_blocks = 16;   // cluster limit from the step's largest node
        uint32_t first_plan = 0;   // the step's (slot, level) entries: refs_[first_plan, first_plan + n_plans)
        uint32_t n_plans = 0;
        SubLevelArgs args{};       // mode, record type and grid of the wave's builds
        WaveNodes wn{};            // the step's node tables on the device
    };
    void issue();   // mutex held; every slot has submitted or left
    void issue_steps(const std::vector<Step>& steps, const std::vector<std::pair<uint32_t, uint32_t>>& refs);

    int device_;
    int sms_;
    bool graphs_ = true;
    ClusterCaps caps_{};
    int last_issue_ = -1;
    std::mutex mu_;
    std::condition_variable cv_;
    uint32_t max_depth_ = 0;
    std::vector<uint32_t> first_step_;   // per slot
    std::vector<Plan> plans_;            // per slot
    uint32_t open_ = 0;                  // slots that have neither submitted nor left
    bool done_ = false, failed_ = false;
    cudaEvent_t done_event_ = nullptr;
    cudaStream_t stream_ = nullptr;
    DevBuf table_, work_, g_key_, g_mask_, g_base_;
    HostBuf stage_;
    cudaEvent_t stage_free_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;   // the last wave's schedule
};

}   // namespace oc
