// Batched and served forms of the LOD build: an executor that runs many
// independent builds at once on one GPU.
//
// Each of `lanes` worker threads owns one Builder (its own streams and
// buffers).  A lane reconfigures its builder for every job, so after the
// first few jobs its buffers have grown to the sizes in use and it
// allocates nothing more: no cudaFree, which would stall every other lane.
// While one lane waits on its host steps (tree read-back, level
// bookkeeping, the final read-back), the others keep the GPU busy.
//
// Prefetch: under a backlog (every lane busy, at least as many jobs waiting
// as lanes) a lane that starts a job also takes the job it will run next
// and copies that job's cloud into a spare device buffer on a stream of its
// own, so that the host-to-device copy overlaps the build in progress
// instead of preceding the next one.  The spare buffer counts in the lane's
// reservation.
//
// Admission: a job's device memory is bounded by estimate_device_bytes.  A
// lane reserves the bound of the envelope of the jobs its builder has run
// (buffers only grow, each to the largest size any of those jobs needed); a
// job starts on a free lane only while the sum of the reservations, with that
// lane's envelope widened by the job, stays within the executor's budget.
// Among the waiting jobs the oldest that fits is taken first; a job whose
// bound exceeds the budget alone fails at submission.  An idle lane whose
// memory keeps a waiting job out frees its builder.
//
// Resident clouds: a job may name its cloud (cloudId != 0; equal ids promise
// equal cloud contents).  A lane remembers the id of the cloud its builder
// last built; a job with that id and the same chunking settings reruns only
// subsampling on the resident pyramid, tree and leaf records (Builder::reuse).
// Among the first waiting jobs, a free lane takes one naming its resident
// cloud before the oldest.
//
// Results do not depend on the mix: each build owns its state, and every
// kernel is deterministic up to the order of records inside a node.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/octreeApi.h"
#include "builder.h"
#include "wave.h"

namespace oc {

void set_last_error(const std::string& msg);

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Job {
    uint64_t ticket = 0;
    OcpiJob spec{};
    BuildConfig cfg;
    MemoryTerms terms;
    uint64_t bound = 0;   // device bytes (estimate_device_bytes)
    Clock::time_point submitted, started, finished;
    bool done = false;
    bool cancel_requested = false;   // cancelled while held by a lane
    OcpiJobResult result{};
    std::vector<uint8_t> hierarchy;
};

// The chunking settings of b match those of the resident state built for a
// (a job without a box may match a state whose box came from the device).
bool same_chunking(const BuildConfig& a, const BuildConfig& b) {
    bool same = a.n == b.n && a.stride == b.stride && a.cloud_type == b.cloud_type && a.chunk_grid == b.chunk_grid &&
                a.threshold == b.threshold;
    for (int k = 0; k < 3; ++k) same = same && a.scale[k] == b.scale[k];
    if (a.has_bbox() && b.has_bbox())
        for (int k = 0; k < 3; ++k) same = same && a.bb_min[k] == b.bb_min[k] && a.bb_max[k] == b.bb_max[k];
    return same;
}

BuildConfig config_of(const OcpiJob& j) {
    BuildConfig c;
    c.n = j.pointAmount;
    c.stride = j.dataStride;
    c.cloud_type = j.cloudType;
    for (int a = 0; a < 3; ++a) {
        c.scale[a] = j.scale[a];
        c.offset[a] = j.bbMin[a];
        c.bb_min[a] = j.bbMin[a];
        c.bb_max[a] = j.bbMax[a];
    }
    c.chunk_grid = j.chunkingGrid;
    c.threshold = j.mergingThreshold;
    c.output_factor = j.outputFactor;
    c.sub_grid = j.subsamplingGrid;
    c.intra = (j.modeFlags & OCPI_SUB_INTRA) != 0;
    c.inter = (j.modeFlags & OCPI_SUB_INTER) != 0;
    c.replacement = true;
    c.random = (j.modeFlags & OCPI_SUB_RANDOM) != 0;
    c.weighting = (j.modeFlags & OCPI_SUB_WEIGHTING) != 0;
    c.seed = j.seed;
    return c;
}

class Executor {
public:
    Executor(int device, uint32_t lanes, uint64_t budget) : device_(device), budget_(budget) {
        check_cuda(cudaSetDevice(device), "cudaSetDevice");
        check_cuda(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device), "device attribute");
        reserved_.assign(lanes, 0);
        env_.assign(lanes, MemoryTerms{});
        resident_.assign(lanes, 0);
        resident_cfg_.assign(lanes, BuildConfig{});
        busy_.assign(lanes, false);
        releasing_.assign(lanes, false);
        held_.assign(lanes, nullptr);
        held_copy_.assign(lanes, false);
        spare_.assign(lanes, 0);
        for (uint32_t l = 0; l < lanes; ++l) workers_.emplace_back([this, l] { run_lane(l); });
    }

    // Jobs in progress complete; jobs still waiting fail.
    ~Executor() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
            for (auto& job : queue_) {
                job->result.status = -1;
                std::snprintf(job->result.error, sizeof job->result.error, "server destroyed before the job started");
                job->done = true;
            }
            queue_.clear();
        }
        cv_work_.notify_all();
        cv_done_.notify_all();
        for (auto& t : workers_) t.join();
    }

    // Throws what submit() refuses: an invalid configuration, no cloud, or a
    // memory bound above the budget.
    void check(const OcpiJob& spec) const {
        const BuildConfig cfg = config_of(spec);
        cfg.validate();
        if (!spec.cloud) throw Error("job without a point cloud");
        const uint64_t bound = device_bytes(memory_terms(cfg, sms_));
        if (bound > budget_)
            throw Error("job needs up to " + std::to_string(bound) + " device bytes, above the executor budget of " +
                        std::to_string(budget_));
    }

    uint64_t submit(const OcpiJob& spec) {
        check(spec);
        auto job = std::make_shared<Job>();
        job->spec = spec;
        job->cfg = config_of(spec);
        job->terms = memory_terms(job->cfg, sms_);
        job->bound = device_bytes(job->terms);
        std::lock_guard<std::mutex> g(mu_);
        job->ticket = ++next_ticket_;
        job->submitted = Clock::now();
        jobs_[job->ticket] = job;
        queue_.push_back(job);
        cv_work_.notify_all();
        return job->ticket;
    }

    OcpiJobResult wait(uint64_t ticket) {
        std::unique_lock<std::mutex> g(mu_);
        auto it = jobs_.find(ticket);
        if (it == jobs_.end()) throw Error("unknown ticket");
        auto job = it->second;
        cv_done_.wait(g, [&] { return job->done; });
        return job->result;
    }

    void hierarchy(uint64_t ticket, uint8_t* out) {
        std::unique_lock<std::mutex> g(mu_);
        auto it = jobs_.find(ticket);
        if (it == jobs_.end()) throw Error("unknown ticket");
        auto job = it->second;
        cv_done_.wait(g, [&] { return job->done; });
        std::memcpy(out, job->hierarchy.data(), job->hierarchy.size());
    }

    // A waiting job leaves the queue and completes as failed ("cancelled");
    // a job held by a lane completes so once that lane has finished its
    // current job and its copy of the held job's cloud; a running or
    // completed job cannot be cancelled.
    void cancel(uint64_t ticket) {
        {
            std::lock_guard<std::mutex> g(mu_);
            auto it = jobs_.find(ticket);
            if (it == jobs_.end()) throw Error("unknown ticket");
            auto job = it->second;
            if (job->done) throw Error("the job has already completed");
            auto q = std::find(queue_.begin(), queue_.end(), job);
            if (q == queue_.end()) {
                if (std::find(held_.begin(), held_.end(), job) == held_.end()) throw Error("the job is running");
                job->cancel_requested = true;
                return;
            }
            queue_.erase(q);
            job->finished = Clock::now();
            job->started = job->finished;
            OcpiJobResult r{};
            r.status = -1;
            std::snprintf(r.error, sizeof r.error, "cancelled");
            r.queuedMs = r.totalMs = ms_between(job->submitted, job->finished);
            job->result = r;
            job->done = true;
        }
        cv_done_.notify_all();
        cv_work_.notify_all();
    }

    uint64_t lane_restarts() {
        std::lock_guard<std::mutex> g(mu_);
        return lane_restarts_;
    }

    void release(uint64_t ticket) {
        std::unique_lock<std::mutex> g(mu_);
        auto it = jobs_.find(ticket);
        if (it == jobs_.end()) throw Error("unknown ticket");
        auto job = it->second;
        cv_done_.wait(g, [&] { return job->done; });
        jobs_.erase(it);
    }

private:
    // The next job for lane l (mutex held): among the first 2 x lanes waiting
    // jobs, the oldest that names the lane's resident cloud; else the oldest
    // waiting job that fits the budget.  The window bounds how far a job can
    // be overtaken.
    std::shared_ptr<Job> take(uint32_t l) {
        uint64_t others = 0;
        for (size_t k = 0; k < reserved_.size(); ++k)
            if (k != l) others += reserved_[k];
        if (resident_[l]) {
            size_t seen = 0;
            for (auto it = queue_.begin(); it != queue_.end() && seen < 2 * reserved_.size(); ++it, ++seen) {
                if ((*it)->spec.cloudId != resident_[l] || !same_chunking(resident_cfg_[l], (*it)->cfg)) continue;
                const MemoryTerms env = envelope(env_[l], (*it)->terms);
                const uint64_t mine = device_bytes(env) + spare_[l];
                if (others + mine > budget_) continue;
                auto job = *it;
                queue_.erase(it);
                env_[l] = env;
                reserved_[l] = mine;
                return job;
            }
        }
        for (auto it = queue_.begin(); it != queue_.end(); ++it) {
            const MemoryTerms env = envelope(env_[l], (*it)->terms);
            const uint64_t mine = device_bytes(env) + spare_[l];
            if (others + mine <= budget_) {
                auto job = *it;
                queue_.erase(it);
                env_[l] = env;
                reserved_[l] = mine;
                return job;
            }
        }
        return nullptr;
    }

    // The job lane l starts after `cur` (mutex held), taken while cur runs so
    // that its cloud is copied during cur's build.  Only under a backlog:
    // every lane busy and at least as many jobs waiting as there are lanes,
    // so that no waiting job is held back from a lane about to go idle.
    // Among the first 2 x lanes waiting jobs, one naming cur's cloud (its
    // state stays resident, nothing to copy) comes first; else the oldest job
    // that fits the budget with the lane's spare cloud buffer grown for it.
    // *copy: the job's cloud is to be prefetched.
    std::shared_ptr<Job> hold(uint32_t l, const Job& cur, bool* copy) {
        *copy = false;
        if (queue_.size() < busy_.size()) return nullptr;
        for (size_t k = 0; k < busy_.size(); ++k)
            if (!busy_[k]) return nullptr;
        uint64_t others = 0;
        for (size_t k = 0; k < reserved_.size(); ++k)
            if (k != l) others += reserved_[k];
        auto admit = [&](std::deque<std::shared_ptr<Job>>::iterator it, uint64_t spare) -> std::shared_ptr<Job> {
            const MemoryTerms env = envelope(env_[l], (*it)->terms);
            const uint64_t mine = device_bytes(env) + spare;
            if (others + mine > budget_) return nullptr;
            auto job = *it;
            queue_.erase(it);
            env_[l] = env;
            reserved_[l] = mine;
            spare_[l] = spare;
            return job;
        };
        if (cur.spec.cloudId) {
            size_t seen = 0;
            for (auto it = queue_.begin(); it != queue_.end() && seen < 2 * reserved_.size(); ++it, ++seen)
                if ((*it)->spec.cloudId == cur.spec.cloudId && same_chunking(cur.cfg, (*it)->cfg))
                    if (auto job = admit(it, spare_[l])) return job;
        }
        for (auto it = queue_.begin(); it != queue_.end(); ++it) {
            const uint64_t need = std::max<uint64_t>(spare_[l], (uint64_t)(*it)->cfg.n * (*it)->cfg.stride + 64);
            if (auto job = admit(it, need)) {
                *copy = true;
                return job;
            }
        }
        return nullptr;
    }

    // A held job goes back to the front of the queue (mutex held): its lane
    // lost its builder, and with it the prefetched cloud and the reservation.
    // The builder is gone, so no copy of the job's cloud is in flight; a job
    // cancelled while held completes as cancelled (the caller notifies).
    void unhold(uint32_t l) {
        if (!held_[l]) return;
        auto job = held_[l];
        held_[l] = nullptr;
        held_copy_[l] = false;
        if (!job->cancel_requested) {
            queue_.push_front(job);
            return;
        }
        job->finished = job->started = Clock::now();
        OcpiJobResult r{};
        r.status = -1;
        std::snprintf(r.error, sizeof r.error, "cancelled");
        r.queuedMs = r.totalMs = ms_between(job->submitted, job->finished);
        job->result = r;
        job->done = true;
    }

    // True when idle lane l should give its memory back to a waiting job
    // (mutex held): the job fits once this lane's memory is freed, or only
    // once every idle lane's is (then all of them free it).  Memory of lanes
    // already freeing theirs counts as free here, not in take().
    bool blocked_by(uint32_t l) const {
        if (queue_.empty() || reserved_[l] == 0 || releasing_[l]) return false;
        uint64_t others = 0, busy = 0;
        for (size_t k = 0; k < reserved_.size(); ++k) {
            if (k == l || releasing_[k]) continue;
            others += reserved_[k];
            if (busy_[k]) busy += reserved_[k];
        }
        for (const auto& j : queue_)
            if (others + j->bound <= budget_) return true;
        for (const auto& j : queue_)
            if (busy + j->bound <= budget_) return true;
        return false;
    }

    // A lane's worker.  A lost worker (simulated on the host: an exception
    // outside any job) has already failed its job and dropped its state; the
    // lane restarts with an empty builder.
    void run_lane(uint32_t l) {
        cudaSetDevice(device_);
        for (;;) {
            try {
                lane_loop(l);
                return;
            } catch (const LaneLost&) {
                // counted in fail_taken, before the job's waiter wakes
            }
        }
    }

    struct LaneLost {};

    // Fails a job that was taken but not built, its worker lost (mutex not
    // held); the lane's restart is counted here.
    void fail_taken(uint32_t l, const std::shared_ptr<Job>& job, const char* why) {
        {
            std::lock_guard<std::mutex> g(mu_);
            ++lane_restarts_;
            job->finished = Clock::now();
            OcpiJobResult r{};
            r.status = -1;
            std::snprintf(r.error, sizeof r.error, "%s", why);
            r.lane = l;
            r.queuedMs = ms_between(job->submitted, job->started);
            r.runMs = ms_between(job->started, job->finished);
            r.totalMs = ms_between(job->submitted, job->finished);
            job->result = r;
            job->done = true;
            busy_[l] = false;
            reserved_[l] = 0;
            env_[l] = MemoryTerms{};
            resident_[l] = 0;
            spare_[l] = 0;
            unhold(l);
        }
        cv_done_.notify_all();
        cv_work_.notify_all();
    }

    void lane_loop(uint32_t l) {
        std::unique_ptr<Builder> builder;
        for (;;) {
            std::shared_ptr<Job> job;
            bool shrink = false, prefetched = false, drop = false;
            {
                std::unique_lock<std::mutex> g(mu_);
                if (held_[l]) {
                    job = held_[l];
                    prefetched = held_copy_[l];
                    held_[l] = nullptr;
                    held_copy_[l] = false;
                    drop = stop_ || job->cancel_requested;
                } else {
                    cv_work_.wait(g, [&] {
                        if (stop_) return true;
                        job = take(l);
                        if (job) return true;
                        shrink = blocked_by(l);   // idle and holding memory a waiting job needs
                        return shrink;
                    });
                    if (!job && !shrink) return;   // stopping
                    if (shrink) releasing_[l] = true;
                }
                if (job && !drop) {
                    busy_[l] = true;
                    job->started = Clock::now();
                }
            }
            if (drop) {
                // a held job cancelled, or the executor stopping: its cloud
                // copy ends before the job completes and its owner may free it
                try {
                    if (builder) builder->prefetch_sync();
                } catch (const std::exception&) {
                    builder.reset();
                    cudaGetLastError();
                }
                {
                    std::lock_guard<std::mutex> g(mu_);
                    job->finished = job->started = Clock::now();
                    OcpiJobResult r{};
                    r.status = -1;
                    std::snprintf(r.error, sizeof r.error, "%s",
                                  job->cancel_requested ? "cancelled" : "server destroyed before the job started");
                    r.queuedMs = r.totalMs = ms_between(job->submitted, job->finished);
                    job->result = r;
                    job->done = true;
                    if (!builder) {
                        reserved_[l] = 0;
                        env_[l] = MemoryTerms{};
                        resident_[l] = 0;
                        spare_[l] = 0;
                    }
                }
                cv_done_.notify_all();
                cv_work_.notify_all();
                continue;
            }
            if (!job) {
                builder.reset();   // frees this lane's buffers
                {
                    std::lock_guard<std::mutex> g(mu_);
                    reserved_[l] = 0;
                    env_[l] = MemoryTerms{};
                    resident_[l] = 0;
                    spare_[l] = 0;
                    releasing_[l] = false;
                }
                cv_work_.notify_all();
                continue;
            }
            if (consume_injected_failure(kInjectLaneLoss)) {
                builder.reset();
                fail_taken(l, job, "worker lost; the lane restarted");
                throw LaneLost{};
            }
            OcpiJobResult r{};
            std::vector<uint8_t> hier;
            try {
                TraceRange trace("job");
                if (builder && !prefetched) builder->prefetch_sync();   // a copy made for no job of this lane
                const OcpiJob& s = job->spec;
                BuildConfig cfg = job->cfg;
                const bool device_bb = !cfg.has_bbox();
                uint64_t had;
                {
                    std::lock_guard<std::mutex> g(mu_);
                    had = resident_[l];
                    resident_[l] = 0;   // until this job succeeds
                }
                const bool reuse = builder && s.cloudId && s.cloudId == had && builder->reuse(cfg);
                if (!reuse) {
                    if (!builder) builder = std::make_unique<Builder>(cfg, s.cloud, device_);
                    else builder->reconfigure(cfg, s.cloud, false);   // the upload overlaps the set-up
                    if (device_bb) {
                        double real[6], cubic[6];
                        builder->compute_bbox(real, cubic);
                    }
                }
                r.reused = reuse ? 1u : 0u;
                {
                    // under a backlog, hold the next job and copy its cloud
                    // while this build runs
                    bool copy = false;
                    std::shared_ptr<Job> next;
                    {
                        std::lock_guard<std::mutex> g(mu_);
                        next = hold(l, *job, &copy);
                        if (next) {
                            held_[l] = next;
                            held_copy_[l] = copy;
                        }
                    }
                    if (next && copy) {
                        try {
                            builder->prefetch(next->spec.cloud, (uint64_t)next->cfg.n * next->cfg.stride);
                        } catch (const std::exception&) {
                            cudaGetLastError();   // no spare buffer: the held job uploads when it starts
                            std::lock_guard<std::mutex> g(mu_);
                            held_copy_[l] = false;
                        }
                    }
                }
                if (s.outRecords) builder->set_output_host(s.outRecords, s.outLut, s.outCapacity);
                builder->generate();
                hier = builder->hierarchy();
                if (s.outHierarchy) {
                    if (hier.size() > s.outHierarchyCapacity)
                        throw Error("hierarchy output too small: the octree has " + std::to_string(hier.size() / 22) +
                                    " nodes");
                    std::memcpy(s.outHierarchy, hier.data(), hier.size());
                }
                const Stats& st = builder->stats();
                {
                    std::lock_guard<std::mutex> g(mu_);
                    resident_[l] = s.cloudId;
                    resident_cfg_[l] = job->cfg;
                }
                r.status = 0;
                r.nodeCount = st.tree_nodes;
                r.pointsTotal = st.points_total;
                r.subsamplePasses = st.subsample_passes;
                for (const auto& t : builder->timings()) r.deviceMs += t.second;
            } catch (const std::exception& e) {
                r.status = -1;
                std::snprintf(r.error, sizeof r.error, "%s", e.what());
                builder.reset();   // leave no half-finished device state behind
                cudaGetLastError();
            }
            {
                std::lock_guard<std::mutex> g(mu_);
                job->finished = Clock::now();
                r.queuedMs = ms_between(job->submitted, job->started);
                r.runMs = ms_between(job->started, job->finished);
                r.totalMs = ms_between(job->submitted, job->finished);
                r.lane = l;
                job->result = r;
                job->hierarchy = std::move(hier);
                job->done = true;
                busy_[l] = false;
                if (!builder) {
                    reserved_[l] = 0;
                    env_[l] = MemoryTerms{};
                    resident_[l] = 0;
                    spare_[l] = 0;
                    unhold(l);
                }
            }
            cv_done_.notify_all();
            cv_work_.notify_all();   // a reservation may have changed
        }
    }

    int device_;
    int sms_ = 152;
    uint64_t budget_;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<std::shared_ptr<Job>> queue_;
    std::map<uint64_t, std::shared_ptr<Job>> jobs_;
    std::vector<uint64_t> reserved_;   // device bytes held or claimed per lane
    std::vector<MemoryTerms> env_;     // envelope of the jobs each lane's builder has run
    std::vector<uint64_t> resident_;   // cloud id whose tree each lane's builder holds (0: none)
    std::vector<BuildConfig> resident_cfg_;   // the configuration that tree was built with
    std::vector<bool> busy_, releasing_;
    std::vector<std::shared_ptr<Job>> held_;   // the job each lane starts next, out of the queue
    std::vector<bool> held_copy_;              // its cloud is being copied to the lane's spare buffer
    std::vector<uint64_t> spare_;              // device bytes of each lane's spare cloud buffer
    std::vector<std::thread> workers_;
    uint64_t next_ticket_ = 0;
    uint64_t lane_restarts_ = 0;
    bool stop_ = false;
};

template <class F>
int guarded(F&& fn) {
    try {
        fn();
        return SUCCESS;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return UNEXPECTED_ERROR;
    }
}

// Executors of ocpi_batch_build, one per (device, lanes, budget), kept for
// the life of the process so that their builders' buffers stay allocated
// between batches.  They are never destroyed: their lanes sleep until the
// process exits.
Executor& batch_executor(int device, uint32_t lanes, uint64_t budget) {
    static std::mutex mu;
    static std::map<std::tuple<int, uint32_t, uint64_t>, Executor*> cache;
    std::lock_guard<std::mutex> g(mu);
    Executor*& ex = cache[std::make_tuple(device, lanes, budget)];
    if (!ex) ex = new Executor(device, lanes, budget);
    return *ex;
}

Executor* to_executor(void* p) {
    if (!p) throw Error("null executor");
    return static_cast<Executor*>(p);
}

}   // namespace

// ---- the batched form in subsampling waves (ocpi_batch_build_wave)
//
// Jobs are grouped by record type and subsampling mode (each wave runs one
// k_subsample instantiation) and, in submission order within a group, built
// up to `slots` at a time.  Each job of a wave runs on a pooled builder and
// a host thread of its own; their subsampling plans meet in the wave, which
// issues them as one schedule (one launch per level over all of them).
//
// Cloud bytes of a job: the order of builds in a batch.
static uint64_t job_bytes(const OcpiJob& j) {
    return (uint64_t)j.pointAmount * j.dataStride;
}

// Two waves are in flight: the pool holds two sets of `slots` builders and
// two Wave objects, and wave k uses set k mod 2.  While wave k's schedule
// subsamples, wave k + 1's builds upload, count and distribute; wave k + 2
// starts once wave k's builds have returned.  A wave admits jobs while the
// envelopes of all builders (the other set's, in use, included; buffers only
// grow) and both waves' buffers fit the budget; idle builders of its own set
// are freed to make room.
struct WavePool {
    std::mutex run;   // one batch at a time per pool
    std::unique_ptr<Wave> wave[2];
    std::vector<std::unique_ptr<Builder>> builders;   // set k: [k * slots, (k + 1) * slots)
    std::vector<MemoryTerms> env;                     // read and written by the batch's own thread only
    std::vector<uint8_t> dropped;                     // a job's thread dropped the builder (failure)
};

WavePool& wave_pool(int device) {
    static std::mutex mu;
    static std::map<int, WavePool*> cache;
    std::lock_guard<std::mutex> g(mu);
    WavePool*& p = cache[device];
    if (!p) {
        p = new WavePool;   // kept for the process, like the batch executors
        int sms = 0;
        check_cuda(cudaSetDevice(device), "cudaSetDevice");
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "device attribute");
        p->wave[0] = std::make_unique<Wave>(device, sms);
        p->wave[1] = std::make_unique<Wave>(device, sms);
    }
    return *p;
}

// One job on builder `q` of the pool, slot `s` of `wave` (on its own thread).
OcpiJobResult run_wave_slot(int device, WavePool& pool, Wave& wave, uint32_t q, uint32_t s, const OcpiJob& job) {
    const auto t0 = Clock::now();
    OcpiJobResult r{};
    std::unique_ptr<Builder>& b = pool.builders[q];
    try {
        check_cuda(cudaSetDevice(device), "cudaSetDevice");
        const BuildConfig cfg = config_of(job);
        if (!b) b = std::make_unique<Builder>(cfg, job.cloud, device);
        else b->reconfigure(cfg, job.cloud, false);
        if (!cfg.has_bbox()) {
            double real[6], cubic[6];
            b->compute_bbox(real, cubic);
        }
        if (job.outRecords) b->set_output_host(job.outRecords, job.outLut, job.outCapacity);
        b->join_wave(&wave, s);
        b->generate();
        b->join_wave(nullptr, 0);
        const std::vector<uint8_t> hier = b->hierarchy();
        if (job.outHierarchy) {
            if (hier.size() > job.outHierarchyCapacity)
                throw Error("hierarchy output too small: the octree has " + std::to_string(hier.size() / 22) + " nodes");
            std::memcpy(job.outHierarchy, hier.data(), hier.size());
        }
        const Stats& st = b->stats();
        r.status = 0;
        r.nodeCount = st.tree_nodes;
        r.pointsTotal = st.points_total;
        r.subsamplePasses = st.subsample_passes;
        for (const auto& t : b->timings()) r.deviceMs += t.second;
    } catch (const std::exception& e) {
        r.status = -1;
        std::snprintf(r.error, sizeof r.error, "%s", e.what());
        b.reset();   // leave no half-finished device state behind
        pool.dropped[q] = 1;
        cudaGetLastError();
    }
    wave.leave(s);   // the other builds of the wave stop waiting for this one
    if (b) b->join_wave(nullptr, 0);
    r.lane = s;
    r.runMs = r.totalMs = ms_between(t0, Clock::now());
    return r;
}

void run_batch_waves(int device, const OcpiBatchTuning& tuning, uint64_t budget, const OcpiJob* jobs, uint32_t count,
                     OcpiJobResult* results, int* last_issue) {
    const uint32_t slots = tuning.waveSize;
    WavePool& pool = wave_pool(device);
    std::lock_guard<std::mutex> run(pool.run);
    check_cuda(cudaSetDevice(device), "cudaSetDevice");
    for (auto& w : pool.wave) {
        w->set_graphs(tuning.useGraphs != 0);
        w->set_cluster_caps(ClusterCaps{tuning.clusterCap, tuning.weightedClusterCap});
    }
    // two sets of `slots` builders; a batch with other wave sizes keeps the
    // builders that fall on its slots and frees the rest
    pool.builders.resize(2 * (size_t)slots);
    pool.env.resize(2 * (size_t)slots, MemoryTerms{});
    pool.dropped.assign(2 * (size_t)slots, 0);
    int sms = 0;
    check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "device attribute");
    std::vector<BuildConfig> cfg(count);
    std::vector<MemoryTerms> terms(count);
    std::map<std::tuple<uint32_t, bool, bool, bool, bool>, std::vector<uint32_t>> groups;
    for (uint32_t i = 0; i < count; ++i) {
        try {
            cfg[i] = config_of(jobs[i]);
            cfg[i].validate();
            if (!jobs[i].cloud) throw Error("job without a point cloud");
            terms[i] = memory_terms(cfg[i], sms);
            if (device_bytes(terms[i]) > budget)
                throw Error("job needs up to " + std::to_string(device_bytes(terms[i])) +
                            " device bytes, above the budget of " + std::to_string(budget));
        } catch (const std::exception& e) {
            throw Error("job " + std::to_string(i) + " of the batch: " + e.what());
        }
        // what selects the k_subsample instantiation (intra wins over inter,
        // weighting applies with inter only)
        const BuildConfig& c = cfg[i];
        const bool inter = !c.intra && c.inter;
        groups[std::make_tuple(c.cloud_type, c.intra, inter, inter && c.weighting, c.random)].push_back(i);
    }
    // jobs group by group, largest cloud first within a group: a wave's
    // subsampling starts when its last build is ready, so a wave holds builds
    // of similar size
    std::vector<uint32_t> order;
    for (auto& kv : groups) {
        std::stable_sort(kv.second.begin(), kv.second.end(),
                         [&](uint32_t a, uint32_t b) { return job_bytes(jobs[a]) > job_bytes(jobs[b]); });
        order.insert(order.end(), kv.second.begin(), kv.second.end());
    }

    struct Running {
        std::vector<uint32_t> jobs;
        std::vector<std::thread> threads;
    };
    Running running[2];
    auto finish = [&](int set) {
        for (auto& t : running[set].threads) t.join();
        running[set].threads.clear();
        running[set].jobs.clear();
        for (size_t q = (size_t)set * slots; q < (size_t)set * slots + slots; ++q)
            if (pool.dropped[q]) {
                pool.env[q] = MemoryTerms{};
                pool.dropped[q] = 0;
            }
    };
    try {
        size_t next = 0;
        for (uint64_t k = 0; next < order.size(); ++k) {
            const int set = (int)(k & 1);
            finish(set);   // wave k - 2: this set's builders and wave are idle again
            Wave& wave = *pool.wave[set];
            const size_t base = (size_t)set * slots;
            // the wave: consecutive jobs of one group
            const auto group_of = [&](uint32_t i) {
                const BuildConfig& c = cfg[i];
                const bool inter = !c.intra && c.inter;
                return std::make_tuple(c.cloud_type, c.intra, inter, inter && c.weighting, c.random);
            };
            uint64_t wave_nodes = 0;
            uint32_t wave_gcap = 0;
            for (size_t q = next, n = 0; q < order.size() && n < slots && group_of(order[q]) == group_of(order[next]);
                 ++q, ++n) {
                wave_nodes += terms[order[q]].node_cap;
                wave_gcap = std::max<uint32_t>(wave_gcap, (uint32_t)terms[order[q]].slots);
            }
            uint64_t used = std::max(wave.device_bytes(), Wave::bytes_for(sms, slots, wave_nodes, wave_gcap)) +
                            pool.wave[set ^ 1]->device_bytes();
            for (const MemoryTerms& e : pool.env) used += device_bytes(e);
            auto free_slot = [&](size_t q) {
                used = used - device_bytes(pool.env[q]) + device_bytes(MemoryTerms{});
                pool.env[q] = MemoryTerms{};
                pool.builders[q].reset();
            };
            std::vector<uint32_t>& wj = running[set].jobs;
            for (size_t s = 0; s < slots && next < order.size(); ++s) {
                const uint32_t i = order[next];
                if (!wj.empty() && group_of(i) != group_of(wj[0])) break;   // one group per wave
                const size_t q = base + s;
                MemoryTerms env = envelope(pool.env[q], terms[i]);
                if (used - device_bytes(pool.env[q]) + device_bytes(env) > budget) {
                    // this builder's buffers, then those of the idle builders
                    // after it in this set, make room; the builders before it
                    // hold this wave's jobs and the other set's the running wave's
                    free_slot(q);
                    env = terms[i];
                    auto fits = [&] { return used - device_bytes(pool.env[q]) + device_bytes(env) <= budget; };
                    for (size_t r = base + slots; r-- > q + 1 && !fits();) free_slot(r);
                    if (!fits()) break;
                }
                used += device_bytes(env) - device_bytes(pool.env[q]);
                pool.env[q] = env;
                wj.push_back(i);
                ++next;
            }
            if (wj.empty()) {
                // nothing fits beside the other wave: let it finish, then retry
                // with this set alone holding memory
                if (!running[set ^ 1].jobs.empty()) {
                    finish(set ^ 1);
                    for (size_t q = (size_t)(set ^ 1) * slots; q < (size_t)(set ^ 1) * slots + slots; ++q)
                        free_slot(q);
                    --k;   // the same set again
                    continue;
                }
                throw Error("no job of the batch fits the budget beside the pooled builders");
            }
            std::vector<uint32_t> depths;
            uint64_t max_nodes = 0;
            uint32_t max_gcap = 0;
            for (uint32_t i : wj) {
                uint32_t d = 0;   // tree depth: log2 of the (validated, power-of-two) chunking grid
                while ((1u << d) < cfg[i].chunk_grid) ++d;
                depths.push_back(d);
                max_nodes += terms[i].node_cap;
                max_gcap = std::max<uint32_t>(max_gcap, (uint32_t)terms[i].slots);
            }
            wave.start(depths, max_nodes, max_gcap);
            for (uint32_t s = 0; s < wj.size(); ++s)
                running[set].threads.emplace_back([&, set, s, base] {
                    results[running[set].jobs[s]] =
                        run_wave_slot(device, pool, *pool.wave[set], (uint32_t)(base + s), s, jobs[running[set].jobs[s]]);
                });
        }
    } catch (...) {
        finish(0);
        finish(1);
        throw;
    }
    finish(0);
    finish(1);
    if (last_issue) *last_issue = std::max(pool.wave[0]->last_issue(), pool.wave[1]->last_issue());
}

// ---- autotuning of the batched form
//
// A batch's signature puts it in a bucket: log2 of the job count and of the
// mean point count, and in tenths the shares of float64 clouds, of
// distance-weighted jobs and of jobs on grids above 256.  For a signature the
// tuner measures the batch form on an evenly spaced sample of the batch:
// first the wave sizes with the default caps and graphs, then the cluster
// caps at the best wave size, then graph capture off, and keeps the fastest.
// The first trial runs twice and only its second run counts (buffers grow on
// the first).

namespace {

std::string batch_signature(int device, const OcpiJob* jobs, uint32_t count) {
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, device);
    double pts = 0;
    uint32_t f64 = 0, weighted = 0, big = 0;
    for (uint32_t i = 0; i < count; ++i) {
        pts += jobs[i].pointAmount;
        f64 += jobs[i].cloudType == 1;
        const uint32_t m = jobs[i].modeFlags;
        weighted += !(m & OCPI_SUB_INTRA) && (m & OCPI_SUB_INTER) && (m & OCPI_SUB_WEIGHTING);
        big += jobs[i].chunkingGrid > 256;
    }
    auto lg = [](double v) { return v >= 1 ? (int)std::floor(std::log2(v)) : 0; };
    auto tenth = [&](uint32_t c) { return count ? (int)(10.0 * c / count + 0.5) : 0; };
    char buf[512];
    std::snprintf(buf, sizeof buf, "%s/%d/jobs2^%d/pts2^%d/f64:%d/w:%d/g512:%d", prop.name, prop.multiProcessorCount,
                  lg(count), lg(count ? pts / count : 0), tenth(f64), tenth(weighted), tenth(big));
    for (char* c = buf; *c; ++c)
        if (*c == ' ') *c = '_';
    return buf;
}

std::mutex g_tuned_mu;
std::map<std::string, OcpiBatchTuning> g_tuned;

bool load_tuning(const char* path, const std::string& sig, OcpiBatchTuning& t) {
    if (!path) return false;
    std::ifstream f(path);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {   // the last entry of a signature wins
        std::istringstream in(line);
        std::string key;
        OcpiBatchTuning v{};
        if (in >> key >> v.waveSize >> v.clusterCap >> v.weightedClusterCap >> v.useGraphs >> v.trialMs >> v.trials &&
            key == sig) {
            if (!(in >> v.lanes)) v.lanes = 0;
            t = v;
            found = true;
        }
    }
    return found;
}

void store_tuning(const char* path, const std::string& sig, const OcpiBatchTuning& t) {
    if (!path) return;
    std::ofstream f(path, std::ios::app);
    f << sig << ' ' << t.waveSize << ' ' << t.clusterCap << ' ' << t.weightedClusterCap << ' ' << t.useGraphs << ' '
      << t.trialMs << ' ' << t.trials << ' ' << t.lanes << '\n';
}

void validate_tuning(const OcpiBatchTuning& t) {
    if (t.lanes > 64) throw Error("lanes must be in [0, 64]");
    if (t.lanes) return;
    if (t.waveSize < 1 || t.waveSize > 256) throw Error("waveSize must be in [1, 256]");
    if (t.clusterCap < 1 || t.clusterCap > 8 || (t.clusterCap & (t.clusterCap - 1)))
        throw Error("clusterCap must be 1, 2, 4 or 8");
    if (t.weightedClusterCap < 1 || t.weightedClusterCap > 16 || (t.weightedClusterCap & (t.weightedClusterCap - 1)))
        throw Error("weightedClusterCap must be a power of two up to 16");
}

OcpiBatchTuning default_tuning() {
    OcpiBatchTuning t{};
    t.waveSize = 32;
    t.clusterCap = 4;
    t.weightedClusterCap = 16;
    t.useGraphs = 1;
    return t;
}

}   // namespace

// The lane executor on a batch: every job checked before any starts, results
// in order.  Jobs are submitted largest cloud first, so that the batch does
// not end on a large build running alone.
void run_batch_lanes(int device, uint32_t lanes, uint64_t budget, const OcpiJob* jobs, uint32_t count,
                     OcpiJobResult* results) {
    if (lanes < 1 || lanes > 64) throw Error("lanes must be in [1, 64]");
    Executor& ex = batch_executor(device, lanes, budget);
    // a refused job leaves no other job of the batch running after the call returns
    for (uint32_t i = 0; i < count; ++i) {
        try {
            ex.check(jobs[i]);
        } catch (const std::exception& e) {
            throw Error("job " + std::to_string(i) + " of the batch: " + e.what());
        }
    }
    std::vector<uint32_t> order(count);
    for (uint32_t i = 0; i < count; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return job_bytes(jobs[a]) > job_bytes(jobs[b]); });
    std::vector<uint64_t> tickets(count);
    for (uint32_t i : order) tickets[i] = ex.submit(jobs[i]);
    for (uint32_t i : order) {
        results[i] = ex.wait(tickets[i]);
        ex.release(tickets[i]);
    }
}

void run_batch_tuned(int device, const OcpiBatchTuning& t, uint64_t budget, const OcpiJob* jobs, uint32_t count,
                     OcpiJobResult* results, int* last_issue) {
    if (t.lanes) {
        run_batch_lanes(device, t.lanes, budget, jobs, count, results);
        if (last_issue) *last_issue = 0;
    } else {
        run_batch_waves(device, t, budget, jobs, count, results, last_issue);
    }
}

OcpiBatchTuning autotune(int device, uint64_t budget, const OcpiJob* jobs, uint32_t count, uint32_t sample_jobs,
                         const char* cache_path) {
    if (!count) throw Error("empty batch");
    const std::string sig = batch_signature(device, jobs, count);
    OcpiBatchTuning best{};
    {
        std::lock_guard<std::mutex> g(g_tuned_mu);
        auto it = g_tuned.find(sig);
        if (it != g_tuned.end()) return it->second;
        if (load_tuning(cache_path, sig, best)) {
            validate_tuning(best);
            g_tuned[sig] = best;
            return best;
        }
    }
    const uint32_t m = std::min<uint32_t>(count, sample_jobs ? sample_jobs : 256);
    std::vector<OcpiJob> sample(m);
    for (uint32_t k = 0; k < m; ++k) sample[k] = jobs[(uint64_t)k * count / m];
    std::vector<OcpiJobResult> res(m);
    uint32_t trials = 0;
    auto measure = [&](const OcpiBatchTuning& t) {
        const auto t0 = Clock::now();
        run_batch_tuned(device, t, budget, sample.data(), m, res.data(), nullptr);
        const double ms = ms_between(t0, Clock::now());
        for (const auto& r : res)
            if (r.status != 0) throw Error(std::string("autotune trial failed: ") + r.error);
        ++trials;
        return ms;
    };
    best = default_tuning();
    best.waveSize = std::min<uint32_t>(best.waveSize, m);
    measure(best);   // buffers grow on the first run
    best.trialMs = measure(best);
    auto consider = [&](OcpiBatchTuning t) {
        if (t.waveSize == best.waveSize && t.clusterCap == best.clusterCap &&
            t.weightedClusterCap == best.weightedClusterCap && t.useGraphs == best.useGraphs && t.lanes == best.lanes)
            return;
        if (t.lanes) measure(t);   // the executor's builders grow on its first run
        t.trialMs = measure(t);
        if (t.trialMs < best.trialMs) best = t;
    };
    for (uint32_t w : {8u, 16u, 32u, 64u}) {
        if (w > m) continue;
        OcpiBatchTuning t = best;
        t.waveSize = w;
        consider(t);
    }
    const OcpiBatchTuning at_size = best;
    for (auto caps : {std::make_pair(2u, 8u), std::make_pair(8u, 16u), std::make_pair(4u, 8u)}) {
        OcpiBatchTuning t = at_size;
        t.clusterCap = caps.first;
        t.weightedClusterCap = caps.second;
        consider(t);
    }
    {
        OcpiBatchTuning t = best;
        t.useGraphs = 0;
        consider(t);
    }
    {
        OcpiBatchTuning t = best;   // the lane executor instead of waves
        t.lanes = 4;
        consider(t);
    }
    best.trials = trials;
    {
        std::lock_guard<std::mutex> g(g_tuned_mu);
        g_tuned[sig] = best;
    }
    store_tuning(cache_path, sig, best);
    return best;
}

}   // namespace oc

extern "C" {

int ocpi_server_create(void** server, int device, uint32_t lanes, uint64_t memoryBudget) {
    return oc::guarded([&] {
        if (!server) throw oc::Error("null server pointer");
        if (lanes < 1 || lanes > 64) throw oc::Error("lanes must be in [1, 64]");
        *server = new oc::Executor(device, lanes, memoryBudget);
    });
}

int ocpi_server_destroy(void* server) {
    return oc::guarded([&] { delete oc::to_executor(server); });
}

int ocpi_server_submit(void* server, const OcpiJob* job, uint64_t* ticket) {
    return oc::guarded([&] {
        if (!job || !ticket) throw oc::Error("null argument");
        *ticket = oc::to_executor(server)->submit(*job);
    });
}

int ocpi_server_wait(void* server, uint64_t ticket, OcpiJobResult* result) {
    return oc::guarded([&] {
        const OcpiJobResult r = oc::to_executor(server)->wait(ticket);
        if (result) *result = r;
    });
}

int ocpi_server_get_hierarchy(void* server, uint64_t ticket, uint8_t* out) {
    return oc::guarded([&] {
        if (!out) throw oc::Error("null output");
        oc::to_executor(server)->hierarchy(ticket, out);
    });
}

int ocpi_server_cancel(void* server, uint64_t ticket) {
    return oc::guarded([&] { oc::to_executor(server)->cancel(ticket); });
}

int ocpi_server_lane_restarts(void* server, uint64_t* restarts) {
    return oc::guarded([&] {
        if (!restarts) throw oc::Error("null output");
        *restarts = oc::to_executor(server)->lane_restarts();
    });
}

int ocpi_debug_inject_failures(int kind, uint32_t count) {
    return oc::guarded([&] { oc::inject_failures(kind, count); });
}

int ocpi_server_release(void* server, uint64_t ticket) {
    return oc::guarded([&] { oc::to_executor(server)->release(ticket); });
}

int ocpi_batch_build(int device, uint32_t lanes, uint64_t memoryBudget, const OcpiJob* jobs, uint32_t count,
                     OcpiJobResult* results) {
    return oc::guarded([&] {
        if (!jobs || !results) throw oc::Error("null argument");
        oc::run_batch_lanes(device, lanes, memoryBudget, jobs, count, results);
        for (uint32_t i = 0; i < count; ++i)
            if (results[i].status != 0) throw oc::Error("some builds of the batch failed (see their results)");
    });
}


int ocpi_batch_build_wave(int device, uint32_t waveSize, uint64_t memoryBudget, const OcpiJob* jobs, uint32_t count,
                          OcpiJobResult* results) {
    return oc::guarded([&] {
        if (!jobs || !results) throw oc::Error("null argument");
        if (waveSize > 256) throw oc::Error("waveSize must be in [1, 256], or 0 for the tuned size");
        OcpiBatchTuning t = oc::default_tuning();
        if (waveSize) t.waveSize = waveSize;
        else if (count) t = oc::autotune(device, memoryBudget, jobs, count, 0, nullptr);
        oc::run_batch_tuned(device, t, memoryBudget, jobs, count, results, nullptr);
        for (uint32_t i = 0; i < count; ++i)
            if (results[i].status != 0) throw oc::Error("some builds of the batch failed (see their results)");
    });
}

int ocpi_batch_autotune(int device, uint64_t memoryBudget, const OcpiJob* jobs, uint32_t count, uint32_t sampleJobs,
                        const char* cachePath, OcpiBatchTuning* tuning) {
    return oc::guarded([&] {
        if (!jobs || !tuning) throw oc::Error("null argument");
        *tuning = oc::autotune(device, memoryBudget, jobs, count, sampleJobs, cachePath);
    });
}

int ocpi_batch_build_tuned(int device, uint64_t memoryBudget, OcpiBatchTuning* tuning, const OcpiJob* jobs,
                           uint32_t count, OcpiJobResult* results) {
    return oc::guarded([&] {
        if (!jobs || !results || !tuning) throw oc::Error("null argument");
        oc::validate_tuning(*tuning);
        int issue = -1;
        oc::run_batch_tuned(device, *tuning, memoryBudget, jobs, count, results, &issue);
        tuning->lastIssue = issue == 1 ? 1u : 0u;
        for (uint32_t i = 0; i < count; ++i)
            if (results[i].status != 0) throw oc::Error("some builds of the batch failed (see their results)");
    });
}

}   // extern "C"
