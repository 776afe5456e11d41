// Subsampling waves: the builds of a batch run on their own builders and host
// threads, and meet at every subsampling level, where one launch subsamples
// the level's nodes of all of them.  A cloud's top levels hold a few nodes;
// alone they leave most SMs idle, together with other clouds' they fill them.
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdint>
#include <mutex>
#include <vector>

#include "builder.h"
#include "kernels.h"

namespace oc {

class Wave {
public:
    Wave(int device, int num_sms);
    ~Wave();
    Wave(const Wave&) = delete;
    Wave& operator=(const Wave&) = delete;

    // A new wave of builds with the given tree depths (log2 of the chunking
    // grid), one slot each.  Levels are aligned at the root: level l of a
    // build of depth d is step l + (max depth - d).  No build may still be in
    // the previous wave.
    void start(const std::vector<uint32_t>& depths);

    // Slot `slot` reached its level `level`: `ready` (recorded on `stream`)
    // marks its level tables as prepared; n nodes (a.nodes, in the level's
    // order) with candidate bounds `bounds`.  n = 0: nothing at this level.
    // Returns once the step's launch is queued, with `stream` waiting for it.
    void arrive(uint32_t slot, uint32_t level, const SubLevelArgs& a, uint32_t n, const uint64_t* bounds,
                uint32_t global_cap, cudaEvent_t ready, cudaStream_t stream);

    // Slot `slot` takes part in no further step (it failed, or it is done).
    void leave(uint32_t slot);

private:
    struct Entry {
        SubLevelArgs a;
        uint32_t n;
        std::vector<uint64_t> bounds;
        uint32_t global_cap;
        cudaEvent_t ready;
    };
    void launch_step(uint32_t t);   // mutex held
    void complete_ready_steps();    // mutex held

    int device_;
    int sms_;
    std::mutex mu_;
    std::condition_variable cv_;
    uint32_t max_depth_ = 0;
    std::vector<uint32_t> first_step_, next_step_;   // per slot
    std::vector<uint32_t> expected_, arrived_;       // per step
    std::vector<bool> done_, failed_;
    std::vector<std::vector<Entry>> entries_;
    std::vector<cudaEvent_t> step_done_;
    cudaStream_t stream_ = nullptr;
    DevBuf table_, work_, g_key_, g_mask_, g_base_;
    HostBuf stage_[2];
    cudaEvent_t stage_free_[2] = {nullptr, nullptr};
    int stage_next_ = 0;
};

}   // namespace oc
