// ocpi_subsample_node_noalloc: subsampling of one octree node with no device
// allocation at all.
//
// Who needs it: callers that own every byte of device memory themselves and
// may not call cudaMalloc.  Examples are a plug-in that runs inside a host
// application whose memory pool has already claimed the GPU, and a streaming
// pipeline that rebuilds single nodes while its buffers sit in a fixed arena.
// The session entry points (ocpi_init_octree / ocpi_generate_octree) size
// their buffers from the cloud and allocate them; this entry point instead
// works in a fixed scratch array that is part of the library image.
//
// The scratch is a file-scope __device__ array of kScratchBytes (about
// 12.5 MiB).  Every GPU on which this library's module is loaded holds it
// until the process exits.  Every call shares it, and it keeps whatever the
// last call left: the set-up kernel below clears the words that must start at
// zero, and the subsample kernel clears its own per-node state.  Two calls
// that overlap on the GPU (different streams, or different host threads
// without ordering) race on the array and produce garbage; callers must
// order them.
//
// On the host, `g_scratch` names a host-side stand-in, not a device address.
// The device address comes from cudaGetSymbolAddress, taken once per device
// with that device current, the first time this entry point runs on the
// device.  That first call may make the CUDA runtime load this module, so it
// should come before any stream capture on that device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/octreeApi.h"
#include "builder.h"
#include "kernels.h"

namespace oc {
namespace {

constexpr uint32_t kMaxCandidates = OCPI_NOALLOC_MAX_CANDIDATES;
// brick-table slots for the largest node: smallest power of two >= 1024 whose
// 11/16 load covers kMaxCandidates + 1 bricks (the session path's rule)
constexpr uint32_t kMaxBrickSlots = 1u << 18;
static_assert((uint64_t)kMaxBrickSlots * 11 / 16 >= kMaxCandidates + 1ull, "brick table too small");

constexpr size_t align256(size_t x) {
    return (x + 255) & ~(size_t)255;
}

// scratch layout (byte offsets, each region 256-byte aligned)
constexpr size_t kOffNode = 0;                                               // one SubNode
constexpr size_t kOffWork = 1024;                                            // work counter
constexpr size_t kOffKey = 1280;                                             // u32 per candidate
constexpr size_t kOffUnit = align256(kOffKey + 4ull * kMaxCandidates);       // 3 x f32 per candidate
constexpr size_t kOffBest = align256(kOffUnit + 12ull * kMaxCandidates);     // u64 per cell
constexpr size_t kOffSel = align256(kOffBest + 8ull * kMaxCandidates);       // u32 per cell
constexpr size_t kOffSlot = align256(kOffSel + 4ull * kMaxCandidates);       // u32 per cell
constexpr size_t kOffIntra = align256(kOffSlot + 4ull * kMaxCandidates);     // u64 per cell
constexpr size_t kOffCsrCount = align256(kOffIntra + 8ull * kMaxCandidates); // u32 per cell
constexpr size_t kOffCsrStart = align256(kOffCsrCount + 4ull * kMaxCandidates);
constexpr size_t kOffCsrPts = align256(kOffCsrStart + 4ull * kMaxCandidates);  // 20 B per candidate
constexpr size_t kOffGKey = align256(kOffCsrPts + 20ull * kMaxCandidates);     // u32 per brick slot
constexpr size_t kOffGMask = align256(kOffGKey + 4ull * kMaxBrickSlots);       // u64 per brick slot
constexpr size_t kOffGBase = align256(kOffGMask + 8ull * kMaxBrickSlots);      // u32 per brick slot
constexpr size_t kScratchBytes = align256(kOffGBase + 4ull * kMaxBrickSlots);
static_assert(sizeof(SubNode) <= kOffWork - kOffNode, "node record does not fit its scratch region");
static_assert(kScratchBytes == OCPI_NOALLOC_SCRATCH_BYTES, "header states a different scratch size");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_dev[kMaxDevices] = {};   // device address of g_scratch, per device

// Looks up the scratch array's address on the current device (once per
// device; the lookup is cached).
unsigned char* scratch_on_current_device() {
    int dev = -1;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) throw Error("device ordinal out of range for the scratch table");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_dev[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            throw Error(std::string("cudaGetSymbolAddress of the subsampling scratch failed: ") +
                        cudaGetErrorString(e));
        }
        g_scratch_dev[dev] = static_cast<unsigned char*>(p);
    }
    return g_scratch_dev[dev];
}

// Writes the node description and clears the counters that must start at
// zero: the block work counter and the caller's status words.
__global__ void k_noalloc_setup(SubNode node, SubNode* node_dst, uint32_t* work, uint32_t* status) {
    *node_dst = node;
    *work = 0;
    status[0] = 0;
    status[1] = 0;
}

}   // namespace

void set_last_error(const std::string& msg);

}   // namespace oc

extern "C" int ocpi_subsample_node_noalloc(const uint8_t* cloud, uint8_t cloudType, uint32_t dataStride,
                                           const double* scale, const double* cloudMin, const double* nodeMin,
                                           double nodeSide, uint32_t level, uint64_t mortonKey,
                                           uint32_t subsamplingGrid, uint32_t modeFlags, uint64_t seed,
                                           const uint32_t* candidateLut, const uint8_t* candidateRecords,
                                           uint32_t candidateCount, uint32_t* outLut, uint8_t* outRecords,
                                           uint32_t* outStatus, void* stream) {
    using namespace oc;
    try {
        if (candidateCount > kMaxCandidates)
            throw Error("ocpi_subsample_node_noalloc: " + std::to_string(candidateCount) +
                        " candidates exceed the fixed scratch limit of " + std::to_string(kMaxCandidates));
        if (!cloud || !scale || !cloudMin || !nodeMin || !outStatus)
            throw Error("ocpi_subsample_node_noalloc: null pointer argument");
        if (candidateCount && (!candidateLut || !candidateRecords || !outLut || !outRecords))
            throw Error("ocpi_subsample_node_noalloc: null candidate or output array");
        if (cloudType > 1) throw Error("ocpi_subsample_node_noalloc: cloud type must be 0 (float) or 1 (double)");
        if (dataStride < (cloudType == 0 ? 15u : 27u))
            throw Error("ocpi_subsample_node_noalloc: data stride too small for the cloud type");
        if (subsamplingGrid < 1 || subsamplingGrid > 1024)
            throw Error("ocpi_subsample_node_noalloc: subsampling grid must be in [1, 1024]");
        if ((modeFlags & OCPI_SUB_INTRA) && (modeFlags & OCPI_SUB_WEIGHTING))
            throw Error("ocpi_subsample_node_noalloc: the weighting function requires inter-cell averaging");
        if (!(nodeSide > 0.0)) throw Error("ocpi_subsample_node_noalloc: node side must be positive");
        for (int k = 0; k < 3; ++k)
            if (!(scale[k] > 0.0)) throw Error("ocpi_subsample_node_noalloc: scale must be positive");

        unsigned char* base = scratch_on_current_device();
        cudaStream_t st = static_cast<cudaStream_t>(stream);

        const double t = nodeSide / subsamplingGrid;   // kernel_helpers.cuh:14
        SubNode node;
        std::memset(&node, 0, sizeof(node));
        for (int k = 0; k < 3; ++k) {
            node.ax[k] = make_axis(nodeMin[k], t);
            node.qa[k] = make_qaxis(nodeMin[k], cloudMin[k], 1.0 / scale[k], t);
        }
        node.morton = mortonKey;
        node.level = level;
        node.cand_off = 0;
        node.out_off = 0;
        node.nchild = candidateCount ? 1 : 0;   // the candidates form one leaf-kind list
        node.child_kind = 0;
        node.child_start[0] = 0;
        node.child_count[0] = candidateCount;
        node.p_in = candidateCount;

        SubNode* node_dev = reinterpret_cast<SubNode*>(base + kOffNode);
        uint32_t* work = reinterpret_cast<uint32_t*>(base + kOffWork);
        k_noalloc_setup<<<1, 1, 0, st>>>(node, node_dev, work, outStatus);
        check_cuda(cudaGetLastError(), "ocpi_subsample_node_noalloc set-up launch");
        if (!candidateCount) return SUCCESS;

        SubLevelArgs a{};
        a.nodes = node_dev;
        a.n_nodes = 1;
        a.grid = subsamplingGrid;
        a.mode = modeFlags & (kModeIntra | kModeInter | kModeRandom | kModeWeight);
        a.float_input = cloudType == 0;
        a.seed = seed;
        a.cloud = cloud;
        a.stride = dataStride;
        a.leaf_lut = candidateLut;
        a.leaf_rec = candidateRecords;
        a.stage_lut = candidateLut;
        a.stage_rec = candidateRecords;
        a.out_lut = outLut;
        a.out_rec = outRecords;
        a.out_points = outStatus;
        a.key_cache = reinterpret_cast<uint32_t*>(base + kOffKey);
        a.unit_cache = reinterpret_cast<float*>(base + kOffUnit);
        a.acc_best = reinterpret_cast<uint64_t*>(base + kOffBest);
        a.acc_sel = reinterpret_cast<uint32_t*>(base + kOffSel);
        a.cell_slot = reinterpret_cast<uint32_t*>(base + kOffSlot);
        a.acc_intra = reinterpret_cast<uint64_t*>(base + kOffIntra);
        a.csr_count = reinterpret_cast<uint32_t*>(base + kOffCsrCount);
        a.csr_start = reinterpret_cast<uint32_t*>(base + kOffCsrStart);
        a.csr_pts = base + kOffCsrPts;
        for (int k = 0; k < 3; ++k) a.out.ax[k] = make_out_axis(cloudMin[k], 1.0 / scale[k]);
        a.work_counter = work;
        a.err = outStatus + 1;
        // global brick table sized like the session path: >= 1024 slots at 68% load
        const uint64_t bs = (subsamplingGrid + 3) / 4;
        const uint64_t bound = std::min<uint64_t>(candidateCount, bs * bs * bs);
        uint64_t cap = 1024;
        while (cap * 11 / 16 < bound + 1) cap <<= 1;
        uint32_t shift = 32;
        for (uint64_t c = cap; c > 1; c >>= 1) --shift;
        a.global_key = reinterpret_cast<uint32_t*>(base + kOffGKey);
        a.global_mask = reinterpret_cast<uint64_t*>(base + kOffGMask);
        a.global_base = reinterpret_cast<uint32_t*>(base + kOffGBase);
        a.global_cap = (uint32_t)cap;
        a.global_shift = shift;
        launch_subsample_level(a, 1, 1, st);
        check_cuda(cudaGetLastError(), "ocpi_subsample_node_noalloc launch");
        return SUCCESS;
    } catch (const std::exception& e) {
        oc::set_last_error(e.what());
        return UNEXPECTED_ERROR;
    }
}
