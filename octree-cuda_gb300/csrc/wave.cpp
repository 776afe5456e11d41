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

}   // namespace

Wave::Wave(int device, int num_sms) : device_(device), sms_(std::max(num_sms, 1)) {
    check_cuda(cudaSetDevice(device), "cudaSetDevice");
    check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
    for (auto& e : stage_free_) check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
}

Wave::~Wave() {
    if (stream_) cudaStreamSynchronize(stream_);
    for (auto e : step_done_) cudaEventDestroy(e);
    for (auto e : stage_free_)
        if (e) cudaEventDestroy(e);
    if (stream_) cudaStreamDestroy(stream_);
}

void Wave::start(const std::vector<uint32_t>& depths) {
    std::lock_guard<std::mutex> g(mu_);
    max_depth_ = 0;
    for (uint32_t d : depths) max_depth_ = std::max(max_depth_, d);
    const size_t steps = (size_t)max_depth_ + 2;   // steps 1..max_depth
    first_step_.assign(depths.size(), 0);
    next_step_.assign(depths.size(), 0);
    expected_.assign(steps, 0);
    arrived_.assign(steps, 0);
    done_.assign(steps, false);
    failed_.assign(steps, false);
    entries_.assign(steps, {});
    while (step_done_.size() < steps) {
        cudaEvent_t e;
        check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
        step_done_.push_back(e);
    }
    for (size_t s = 0; s < depths.size(); ++s) {
        first_step_[s] = max_depth_ - depths[s] + 1;
        next_step_[s] = first_step_[s];
        for (uint32_t t = first_step_[s]; t <= max_depth_; ++t) ++expected_[t];
    }
}

void Wave::arrive(uint32_t slot, uint32_t level, const SubLevelArgs& a, uint32_t n, const uint64_t* bounds,
                  uint32_t global_cap, cudaEvent_t ready, cudaStream_t stream) {
    std::unique_lock<std::mutex> g(mu_);
    if (slot >= first_step_.size()) throw Error("wave: unknown slot");
    const uint32_t t = level + first_step_[slot] - 1;
    if (t != next_step_[slot] || t > max_depth_) throw Error("wave: a level arrived out of order");
    next_step_[slot] = t + 1;
    if (n) entries_[t].push_back(Entry{a, n, std::vector<uint64_t>(bounds, bounds + n), global_cap, ready});
    ++arrived_[t];
    complete_ready_steps();
    cv_.wait(g, [&] { return (bool)done_[t]; });
    if (failed_[t]) throw Error("wave: the launch of a subsampling step failed");
    check_cuda(cudaStreamWaitEvent(stream, step_done_[t], 0), "wait");
}

void Wave::leave(uint32_t slot) {
    std::lock_guard<std::mutex> g(mu_);
    if (slot >= next_step_.size()) return;
    for (uint32_t t = next_step_[slot]; t <= max_depth_; ++t) --expected_[t];
    next_step_[slot] = max_depth_ + 1;
    complete_ready_steps();
}

void Wave::complete_ready_steps() {
    for (uint32_t t = 1; t <= max_depth_; ++t)
        if (!done_[t] && arrived_[t] >= expected_[t] && arrived_[t] > 0) launch_step(t);
}

// One launch over the step's nodes of every build that has some, largest
// candidate bound first; the builds' level tables are ready once their
// events have completed.
void Wave::launch_step(uint32_t t) {
    auto& es = entries_[t];
    try {
        uint64_t total = 0, sum = 0, mx = 0;
        uint32_t gcap = 1024;
        for (const auto& e : es) {
            total += e.n;
            gcap = std::max(gcap, e.global_cap);
            for (uint64_t b : e.bounds) {
                sum += b;
                mx = std::max(mx, b);
            }
        }
        if (total) {
            if (total > 0xFFFFFFFFull) throw Error("wave: too many nodes in one step");
            for (const auto& e : es) check_cuda(cudaStreamWaitEvent(stream_, e.ready, 0), "wait");
            struct Ref {
                uint64_t bound;
                uint32_t k, i;
            };
            std::vector<Ref> refs;
            refs.reserve(total);
            for (uint32_t k = 0; k < es.size(); ++k)
                for (uint32_t i = 0; i < es[k].n; ++i) refs.push_back({es[k].bounds[i], k, i});
            std::stable_sort(refs.begin(), refs.end(), [](const Ref& x, const Ref& y) { return x.bound > y.bound; });
            // one staged block: the builds' level arguments, then per wave
            // node its SubNode, its build and its index in that build's level
            const size_t o_node = align16(es.size() * sizeof(SubLevelArgs));
            const size_t o_cloud = o_node + align16(total * sizeof(void*));
            const size_t o_local = o_cloud + align16(total * 4);
            const size_t bytes = o_local + align16(total * 4);
            HostBuf& hb = stage_[stage_next_];
            check_cuda(cudaEventSynchronize(stage_free_[stage_next_]), "wave staging");
            hb.ensure(bytes);
            uint8_t* h = hb.as<uint8_t>();
            for (size_t k = 0; k < es.size(); ++k) std::memcpy(h + k * sizeof(SubLevelArgs), &es[k].a, sizeof(SubLevelArgs));
            const SubNode** node = reinterpret_cast<const SubNode**>(h + o_node);
            uint32_t* cloud = reinterpret_cast<uint32_t*>(h + o_cloud);
            uint32_t* local = reinterpret_cast<uint32_t*>(h + o_local);
            for (size_t j = 0; j < refs.size(); ++j) {
                node[j] = es[refs[j].k].a.nodes + refs[j].i;
                cloud[j] = refs[j].k;
                local[j] = refs[j].i;
            }
            table_.ensure(bytes);
            check_cuda(cudaMemcpyAsync(table_.p, h, bytes, cudaMemcpyHostToDevice, stream_), "H2D wave table");
            check_cuda(cudaEventRecord(stage_free_[stage_next_], stream_), "event");
            stage_next_ ^= 1;
            work_.ensure(4);
            check_cuda(cudaMemsetAsync(work_.p, 0, 4, stream_), "memset");
            // per-block global brick tables for the largest node of any build
            const size_t blocks = std::min<size_t>(total, (size_t)sms_);
            g_key_.ensure(blocks * gcap * 4);
            g_mask_.ensure(blocks * gcap * 8);
            g_base_.ensure(blocks * gcap * 4);
            uint32_t shift = 32;
            for (uint32_t c = gcap; c > 1; c >>= 1) --shift;

            SubLevelArgs w = es[0].a;   // mode, record type and grid of the wave's builds
            w.nodes = nullptr;
            w.n_nodes = (uint32_t)total;
            w.work_counter = work_.as<uint32_t>();
            w.global_key = g_key_.as<uint32_t>();
            w.global_mask = g_mask_.as<uint64_t>();
            w.global_base = g_base_.as<uint32_t>();
            w.global_cap = gcap;
            w.global_shift = shift;
            uint8_t* d = table_.as<uint8_t>();
            WaveNodes wn{reinterpret_cast<const SubLevelArgs*>(d), reinterpret_cast<const SubNode* const*>(d + o_node),
                         reinterpret_cast<const uint32_t*>(d + o_cloud), reinterpret_cast<const uint32_t*>(d + o_local)};
            const uint32_t balance = sum ? (uint32_t)std::min<uint64_t>(64, (mx * sms_ + sum - 1) / sum) : 1u;
            launch_subsample_wave(w, wn, sms_, balance, stream_);
            check_cuda(cudaGetLastError(), "wave launch");
        }
        check_cuda(cudaEventRecord(step_done_[t], stream_), "event");
    } catch (const std::exception&) {
        cudaGetLastError();
        failed_[t] = true;   // every build of the step fails; none waits forever
    }
    done_[t] = true;
    es.clear();
    cv_.notify_all();
}

}   // namespace oc
