// Subsampling waves (see wave.h).
#include "wave.h"

#include <algorithm>
#include <cstring>
#include <string>

namespace oc {

namespace {

size_t align16(size_t b) {
    return (b + 15) & ~(size_t)15;
}

// Bytes of one step's tables: the level arguments of the builds taking part,
// then per node its SubNode pointer, its build and its index in that build's
// level (WaveNodes).
size_t step_table_bytes(size_t builds, size_t nodes) {
    return align16(builds * sizeof(SubLevelArgs)) + align16(nodes * sizeof(void*)) + 2 * align16(nodes * 4);
}

// Steps of any wave: trees are at most 10 levels deep (grids up to 1024).
constexpr size_t kMaxSteps = 11;

size_t tables_bound(size_t builds, uint64_t nodes) {
    return kMaxSteps * step_table_bytes(builds, 0) + step_table_bytes(0, nodes) + kMaxSteps * 48;
}

}   // namespace

Wave::Wave(int device, int num_sms) : device_(device), sms_(std::max(num_sms, 1)) {
    check_cuda(cudaSetDevice(device), "cudaSetDevice");
    check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
    check_cuda(cudaEventCreateWithFlags(&done_event_, cudaEventDisableTiming), "event");
    check_cuda(cudaEventCreateWithFlags(&stage_free_, cudaEventDisableTiming), "event");
}

Wave::~Wave() {
    if (stream_) cudaStreamSynchronize(stream_);
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (done_event_) cudaEventDestroy(done_event_);
    if (stage_free_) cudaEventDestroy(stage_free_);
    if (stream_) cudaStreamDestroy(stream_);
}

uint64_t Wave::bytes_for(int num_sms, uint32_t builds, uint64_t max_nodes, uint32_t max_global_cap) {
    const uint64_t blocks = std::min<uint64_t>(std::max<uint64_t>(max_nodes, 1), (uint64_t)std::max(num_sms, 1));
    const uint64_t gcap = std::max<uint32_t>(max_global_cap, 1024);
    return blocks * gcap * 16 + tables_bound(builds, max_nodes) + 256;
}

uint64_t Wave::device_bytes() const {
    return table_.bytes + work_.bytes + g_key_.bytes + g_mask_.bytes + g_base_.bytes;
}

void Wave::start(const std::vector<uint32_t>& depths, uint64_t max_nodes, uint32_t max_global_cap) {
    std::lock_guard<std::mutex> g(mu_);
    check_cuda(cudaSetDevice(device_), "cudaSetDevice");
    max_depth_ = 0;
    for (uint32_t d : depths) max_depth_ = std::max(max_depth_, d);
    if (max_depth_ + 1 > kMaxSteps) throw Error("wave: trees deeper than 10 levels");
    first_step_.assign(depths.size(), 0);
    for (size_t s = 0; s < depths.size(); ++s) first_step_[s] = max_depth_ - depths[s] + 1;
    plans_.assign(depths.size(), Plan{});
    open_ = (uint32_t)depths.size();
    done_ = failed_ = false;
    // the wave's buffers, sized for the wave's bounds before any build runs
    const uint64_t blocks = std::min<uint64_t>(std::max<uint64_t>(max_nodes, 1), (uint64_t)sms_);
    const uint32_t gcap = std::max<uint32_t>(max_global_cap, 1024);
    g_key_.ensure(blocks * gcap * 4);
    g_mask_.ensure(blocks * gcap * 8);
    g_base_.ensure(blocks * gcap * 4);
    const size_t tb = tables_bound(depths.size(), max_nodes);
    table_.ensure(tb);
    work_.ensure(4);
    check_cuda(cudaEventSynchronize(stage_free_), "wave staging");   // the previous wave's upload is done
    stage_.ensure(tb);
    if (graph_exec_) {   // the previous wave's graph has run: its builds waited for it
        cudaGraphExecDestroy(graph_exec_);
        graph_exec_ = nullptr;
    }
}

void Wave::submit(uint32_t slot, std::vector<WaveLevel> levels, uint32_t global_cap, cudaEvent_t ready,
                  cudaStream_t stream) {
    std::unique_lock<std::mutex> g(mu_);
    if (slot >= plans_.size()) throw Error("wave: unknown slot");
    Plan& p = plans_[slot];
    if (p.submitted || p.gone) throw Error("wave: a slot submitted twice");
    if (first_step_[slot] - 1 + levels.size() > max_depth_) throw Error("wave: a plan deeper than its slot's tree");
    p.levels = std::move(levels);
    p.global_cap = global_cap;
    p.ready = ready;
    p.submitted = true;
    if (--open_ == 0) issue();
    cv_.wait(g, [&] { return done_; });
    if (failed_) throw Error("wave: issuing the subsampling schedule failed");
    check_cuda(cudaStreamWaitEvent(stream, done_event_, 0), "wait");
}

void Wave::leave(uint32_t slot) {
    std::lock_guard<std::mutex> g(mu_);
    if (slot >= plans_.size()) return;
    Plan& p = plans_[slot];
    if (p.submitted || p.gone) return;
    p.gone = true;
    if (--open_ == 0) issue();
}

// The schedule of the whole wave: per step, every taking part build's level
// preparation, then one k_subsample over the step's nodes of all of them,
// largest candidate bound first.
void Wave::issue() {
    try {
        std::vector<Step> steps(max_depth_ + 1);
        std::vector<std::pair<uint32_t, uint32_t>> refs;   // (slot, level index) per step entry
        uint32_t gcap = 1024;
        for (const Plan& p : plans_)
            if (p.submitted) gcap = std::max(gcap, p.global_cap);
        size_t off = 0;
        for (uint32_t t = 1; t <= max_depth_; ++t) {
            Step& st = steps[t];
            st.table_off = off;
            st.first_plan = (uint32_t)refs.size();
            uint64_t n = 0, sum = 0, mx = 0;
            for (uint32_t s = 0; s < plans_.size(); ++s) {
                const Plan& p = plans_[s];
                if (!p.submitted || t < first_step_[s]) continue;
                const uint32_t li = t - first_step_[s];
                if (li >= p.levels.size()) continue;
                refs.push_back({s, li});
                const WaveLevel& w = p.levels[li];
                n += w.a.n_nodes;
                for (uint64_t b : w.bounds) {
                    sum += b;
                    mx = std::max(mx, b);
                }
            }
            if (n > 0xFFFFFFFFull) throw Error("wave: too many nodes in one step");
            st.n_plans = (uint32_t)refs.size() - st.first_plan;
            st.n_nodes = (uint32_t)n;
            st.balance = sum ? (uint32_t)std::min<uint64_t>(64, (mx * sms_ + sum - 1) / sum) : 1u;
            st.node_blocks = node_blocks_for(mx);
            off += step_table_bytes(st.n_plans, n);
        }
        // every step's tables in one staged block and one copy
        stage_.ensure(off);
        table_.ensure(off);
        uint8_t* h = stage_.as<uint8_t>();
        uint8_t* d = table_.as<uint8_t>();
        uint64_t max_step_nodes = 0;
        for (uint32_t t = 1; t <= max_depth_; ++t) {
            Step& st = steps[t];
            max_step_nodes = std::max<uint64_t>(max_step_nodes, st.n_nodes);
            const size_t o_node = st.table_off + align16(st.n_plans * sizeof(SubLevelArgs));
            const size_t o_cloud = o_node + align16(st.n_nodes * sizeof(void*));
            const size_t o_local = o_cloud + align16(st.n_nodes * 4);
            struct Ref {
                uint64_t bound;
                uint32_t k, i;
            };
            std::vector<Ref> order;
            order.reserve(st.n_nodes);
            for (uint32_t k = 0; k < st.n_plans; ++k) {
                const auto& r = refs[st.first_plan + k];
                const WaveLevel& w = plans_[r.first].levels[r.second];
                std::memcpy(h + st.table_off + k * sizeof(SubLevelArgs), &w.a, sizeof(SubLevelArgs));
                for (uint32_t i = 0; i < w.a.n_nodes; ++i)
                    order.push_back({i < w.bounds.size() ? w.bounds[i] : 0, k, i});
                if (k == 0) st.args = w.a;   // mode, record type and grid are the wave's
            }
            std::stable_sort(order.begin(), order.end(), [](const Ref& x, const Ref& y) { return x.bound > y.bound; });
            const SubNode** node = reinterpret_cast<const SubNode**>(h + o_node);
            uint32_t* cloud = reinterpret_cast<uint32_t*>(h + o_cloud);
            uint32_t* local = reinterpret_cast<uint32_t*>(h + o_local);
            for (size_t j = 0; j < order.size(); ++j) {
                const auto& r = refs[st.first_plan + order[j].k];
                node[j] = plans_[r.first].levels[r.second].a.nodes + order[j].i;
                cloud[j] = order[j].k;
                local[j] = order[j].i;
            }
            st.args.nodes = nullptr;
            st.args.n_nodes = st.n_nodes;
            st.wn = WaveNodes{reinterpret_cast<const SubLevelArgs*>(d + st.table_off),
                              reinterpret_cast<const SubNode* const*>(d + o_node),
                              reinterpret_cast<const uint32_t*>(d + o_cloud),
                              reinterpret_cast<const uint32_t*>(d + o_local)};
        }
        // per-block global brick tables for the largest node of any build
        const size_t blocks = std::min<size_t>(std::max<uint64_t>(max_step_nodes, 1), (size_t)sms_);
        g_key_.ensure(blocks * gcap * 4);
        g_mask_.ensure(blocks * gcap * 8);
        g_base_.ensure(blocks * gcap * 4);
        uint32_t shift = 32;
        for (uint32_t c = gcap; c > 1; c >>= 1) --shift;
        for (uint32_t t = 1; t <= max_depth_; ++t) {
            SubLevelArgs& w = steps[t].args;
            w.work_counter = work_.as<uint32_t>();
            w.global_key = g_key_.as<uint32_t>();
            w.global_mask = g_mask_.as<uint64_t>();
            w.global_base = g_base_.as<uint32_t>();
            w.global_cap = gcap;
            w.global_shift = shift;
        }
        for (const Plan& p : plans_)
            if (p.submitted) check_cuda(cudaStreamWaitEvent(stream_, p.ready, 0), "wait");
        if (off) check_cuda(cudaMemcpyAsync(d, h, off, cudaMemcpyHostToDevice, stream_), "H2D wave tables");
        check_cuda(cudaEventRecord(stage_free_, stream_), "event");
        issue_steps(steps, refs);
        check_cuda(cudaEventRecord(done_event_, stream_), "event");
    } catch (const std::exception&) {
        cudaGetLastError();
        failed_ = true;   // every build of the wave fails; none waits forever
    }
    done_ = true;
    cv_.notify_all();
}

void Wave::issue_steps(const std::vector<Step>& steps, const std::vector<std::pair<uint32_t, uint32_t>>& refs) {
    auto launch_all = [&]() {
        for (uint32_t t = 1; t <= max_depth_; ++t) {
            const Step& st = steps[t];
            for (uint32_t k = 0; k < st.n_plans; ++k) {
                const auto& r = refs[st.first_plan + k];
                const WaveLevel& w = plans_[r.first].levels[r.second];
                if (w.a.n_nodes) w.prepare(stream_);
            }
            if (!st.n_nodes) continue;
            check_cuda(cudaMemsetAsync(work_.p, 0, 4, stream_), "memset");
            ClusterCaps caps = caps_;
            caps.node_blocks = st.node_blocks;
            launch_subsample_wave(st.args, st.wn, sms_, st.balance, stream_, caps);
        }
    };
    if (graphs_) {
        cudaGraph_t graph = nullptr;
        bool captured = false;
        if (cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            try {
                launch_all();
            } catch (const std::exception&) {
            }
            captured = cudaStreamEndCapture(stream_, &graph) == cudaSuccess && graph;
        }
        if (captured && cudaGraphInstantiate(&graph_exec_, graph, 0) == cudaSuccess &&
            cudaGraphLaunch(graph_exec_, stream_) == cudaSuccess) {
            cudaGraphDestroy(graph);
            last_issue_ = 1;
            return;
        }
        if (graph) cudaGraphDestroy(graph);
        if (graph_exec_) {
            cudaGraphExecDestroy(graph_exec_);
            graph_exec_ = nullptr;
        }
        cudaGetLastError();   // the capture failed: the same launches, issued directly
    }
    launch_all();
    check_cuda(cudaGetLastError(), "wave launch");
    last_issue_ = 0;
}

}   // namespace oc
