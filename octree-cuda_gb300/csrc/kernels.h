// Host-side launchers of the LOD-build kernels (sm_103a).  Every launcher
// enqueues work on `stream` and returns; errors detected on the device are
// reported through the sticky error word `err` (see oc::kErr*).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "device_common.cuh"

namespace oc {

// Gridding of the finest chunking level (mapPointToGrid parameters).  The
// cell of a coordinate is looked up in exact boundary-key tables (built on the
// host by make_cell_keys) around an fp32 estimate p * r + c; `ax` is the
// binary64 fallback.
struct CloudGrid {
    AxisGrid ax[3];
    float r[3];               // float(1 / t)
    float c[3];               // float(-min / t)
    uint32_t grid;            // chunking grid G0
    const void* keys;         // device: 3 x (grid + 2) keys, int64 (double input) or int32 (float input)
    const uint32_t* spread;   // device: spread3(i) for i < grid
};

// Exact boundary keys of one axis for the reference's cell formula
// (int64)fmin((p - mn) / t, grid - 1): keys[i] = least ordered key of a
// coordinate whose cell is >= i, keys[grid] = keys[grid + 1] = largest key.
void make_cell_keys64(double mn, double t, uint32_t grid, int64_t* keys);
void make_cell_keys32(double mn, double t, uint32_t grid, int32_t* keys);

// Output-coordinate parameters: cloud bbox minimum and 1/scale per axis.
struct OutParams {
    OutAxis ax[3];
};

// Cell position of a candidate from its quantised output coordinate q
// (q = floor((p - cloud_min) / scale), the record's int32 coordinate):
// u = (q - qn + theta) * B + base, theta in [0, 1), exact to rounding.
struct QAxis {
    int32_t qn;     // quantised coordinate of the node's bbox minimum
    float base;     // ((cloud_min - node_min) + qn * scale) / t
    float B;        // scale / t: width of one quantisation step in cells
};

// node_min, cloud_min: bbox minima; sf = 1/scale; t = node side / S.
inline QAxis make_qaxis(double node_min, double cloud_min, double sf, double t) {
    QAxis q;
    double qn = std::floor((node_min - cloud_min) * sf);
    q.qn = (int32_t)qn;
    double base = ((cloud_min - node_min) + (double)q.qn / sf) / t;
    q.base = (float)base;
    q.B = (float)(1.0 / (sf * t));
    return q;
}

// One internal node to subsample.  Children are listed in slot order; each
// child's points are records [start, start + count) of either the leaf data
// arrays (kind 0) or the internal staging arrays (kind 1).
struct SubNode {
    AxisGrid ax[3];
    QAxis qa[3];
    uint64_t morton;
    uint64_t cand_off;   // first candidate slot of this node in the level scratch
    uint64_t out_off;    // first output slot of this node in out_lut / out_rec
    uint64_t child_start[8];
    uint32_t child_count[8];
    uint32_t level;
    uint32_t p_in;       // total candidate points
    uint32_t nchild;
    uint32_t child_kind; // bit s set: child s lives in the staging arrays
};

enum SubMode : uint32_t {
    kModeIntra = 1,
    kModeInter = 2,
    kModeRandom = 8,
    kModeWeight = 16,
};

struct SubLevelArgs {
    const SubNode* nodes;
    uint32_t n_nodes;
    uint32_t grid;        // subsampling grid S
    uint32_t mode;        // SubMode bits (intra wins over inter, weighting only with inter)
    uint32_t float_input;
    uint64_t seed;
    const uint8_t* cloud;
    uint32_t stride;
    const uint32_t* leaf_lut;   // final LUT (leaf part)
    const uint8_t* leaf_rec;    // final records (leaf part)
    const uint32_t* stage_lut;  // staging LUT of internal nodes
    const uint8_t* stage_rec;   // staging records of internal nodes
    // sub-step words (pack_frac) beside the leaf / staged / output records;
    // null: candidates carry none and cells are decided from q alone
    const uint32_t* leaf_frac;
    const uint32_t* stage_frac;
    uint32_t* out_frac;
    uint32_t* out_lut;          // staging outputs of this level (indexed by cand_off)
    uint8_t* out_rec;
    uint32_t* out_points;       // per node: number of subsampled points
    uint32_t* key_cache;        // per candidate: brick slot << 6 | bit
    float* unit_cache;          // per candidate: cell-unit position (weighted only)
    uint64_t* acc_best;         // per cell: selection key
    uint32_t* acc_sel;          // per cell: winning candidate (explicit random)
    uint32_t* cell_slot;        // per cell: brick slot holding it
    uint64_t* acc_intra;        // per cell: packed colour sum
    // Distance weighting on a level of few nodes: each node leaves its emit to
    // k_emit_weighted, which spreads the node's cells over all SMs.  A node on
    // the shared brick table copies its map to emit_maps; a node on a global
    // table uses the level's table number li (one per node), which stays
    // intact.  Null: every node emits in its own block or cluster.
    uint8_t* emit_maps;         // per node of the level: kBrickMapBytes
    // per node of the level: {cells, next run, 1 = map in emit_maps or
    // 2 = its own global table (0: emitted in its cluster), 0}
    uint32_t* emit_state;
    uint32_t* csr_count;        // per cell: candidates in the cell (weighted only)
    uint32_t* csr_start;        // per cell
    uint8_t* csr_pts;           // per candidate: grouped by cell (weighted only), 20 bytes each
    OutParams out;
    uint32_t* work_counter;
    uint32_t* err;
    // per-block brick tables in global memory (gridDim.x * global_cap slots)
    uint32_t* global_key;
    uint64_t* global_mask;
    uint32_t* global_base;
    uint32_t global_cap;     // power of two, >= 1024
    uint32_t global_shift;   // 32 - log2(global_cap)
};

// Points per finest cell.  occ != nullptr (sparse clouds): also flags, one
// byte per 64-cell block of the finest level (a level-2 cell), the blocks
// that received points.
int launch_count(const uint8_t* cloud, uint64_t n, uint32_t stride, bool float_input, const CloudGrid& g,
                  uint32_t* pyr0, uint8_t* occ, uint32_t* err, int num_sms, cudaStream_t stream);

// Zeroes the finest-level blocks flagged in `occ` (`blocks` flags) and the
// flags themselves.
int launch_sparse_zero(uint32_t* pyr0, uint8_t* occ, uint64_t blocks, cudaStream_t stream);

// Builds levels 1..depth of the Morton count pyramid from level 0 and counts
// occupied cells per level into `nonzero[level]`.  With occ, finest-level
// blocks whose bit is clear are not read.
int launch_pyramid(uint32_t* pyr, const uint64_t* level_off_host, uint32_t depth, uint32_t* nonzero,
                    const uint8_t* occ, cudaStream_t stream);

int launch_enumerate(const uint32_t* pyr, const uint64_t* level_off_dev, uint32_t depth, uint32_t threshold,
                      uint32_t* key, uint32_t* count, uint8_t* level, uint16_t* info, uint32_t* child_first,
                      uint32_t cap, uint32_t* level_start, uint32_t* n_nodes, uint32_t* err, cudaStream_t stream);

// Ordered keys of the coordinate minima (keys[0..2]) and maxima (keys[3..5])
// of the cloud, NaN coordinates skipped (float keys widened to 64 bits);
// LLONG_MAX / LLONG_MIN when an axis has no finite coordinate.
int launch_bbox(const uint8_t* cloud, uint64_t n, uint32_t stride, bool float_input, long long* keys, int num_sms,
                cudaStream_t stream);

// Leaf data offsets (BFS order), leaf tags in the pyramid and cleared fill
// counters, computed on the device from the enumerated node table.
int launch_leaf_prep(const uint32_t* n_nodes, const uint16_t* info, const uint32_t* count, const uint8_t* level,
                     const uint32_t* key, uint32_t* pyr, const uint64_t* loff_dev, uint64_t* data_idx, uint32_t* fill,
                     uint64_t n_points, uint32_t* err, cudaStream_t stream);

// Writes each occupied finest-level cell's leaf tag into the cell (after
// launch_leaf_prep), so that distribution finds a point's leaf in one read.
int launch_push_tags(uint32_t* pyr, const uint64_t* level_off_dev, uint32_t depth, uint32_t grid, const uint8_t* occ,
                     uint32_t* err, cudaStream_t stream);

int launch_distribute(const uint8_t* cloud, uint64_t n, uint32_t stride, bool float_input, const CloudGrid& g,
                      const OutParams& out, const uint32_t* pyr0, const uint64_t* data_idx, uint32_t* fill,
                      uint32_t* lut, uint8_t* rec, uint32_t* frac, uint32_t* err, int num_sms,
                      cudaStream_t stream);

// Fills the dynamic part of one level's node table before it is subsampled:
// for children that are internal nodes (child_kind bit set, child_start = the
// child's internal index on entry) their output count and staged position,
// then p_in, cand_off (level-local) and out_off = *level_base + cand_off.
// Records each node's out_off in stage_off[first_internal + k], advances
// *level_base, and sets *work_counter to n_nodes (every block exits at once)
// when the level exceeds scratch_cap or the staging arrays exceed stage_cap
// (error kErrCapacity), else to 0.
int launch_prepare_level(SubNode* nodes, uint32_t n_nodes, const uint32_t* out_points, uint64_t* stage_off,
                         uint32_t first_internal, uint64_t* level_base, uint64_t scratch_cap, uint64_t stage_cap,
                         uint32_t* work_counter, uint32_t* err, cudaStream_t stream);

// One subsampling step over the nodes of several builds (a wave): per wave
// node, the level arguments of its build (`clouds`, indexed by cloud_of),
// its SubNode and its index in that build's level (for out_points).  The
// builds share the record type and subsampling mode.
struct WaveNodes {
    const SubLevelArgs* clouds;
    const SubNode* const* node;
    const uint32_t* cloud_of;
    const uint32_t* local;
};

// Largest thread-block cluster per node of a subsampling level: unweighted
// modes, and distance-weighted ones (clusters above 8 are non-portable).
struct ClusterCaps {
    uint32_t plain = 4;
    uint32_t weighted = 16;
    // the level's largest node needs no more blocks than this (one per
    // kCandidatesPerClusterBlock of its candidates): small nodes are not
    // split over blocks that would mostly wait at the cluster barriers
    uint32_t node_blocks = 16;
};
constexpr uint64_t kCandidatesPerClusterBlock = 8192;
// slots of the shared-memory brick table of a subsample block, and the bytes
// of one table (64-bit mask, 32-bit key and rank base per slot)
constexpr uint32_t kSharedBrickSlots = 8192;
constexpr uint64_t kBrickMapBytes = (uint64_t)kSharedBrickSlots * 16;
// distance-weighted levels of at most this many nodes spread each node's
// emit over all SMs (k_emit_weighted)
constexpr uint32_t kSplitEmitNodes = 16;
// node_blocks for a level whose largest node has `max_bound` candidates
inline uint32_t node_blocks_for(uint64_t max_bound) {
    uint32_t b = 1;
    while (b < 16 && (uint64_t)b * 2 * kCandidatesPerClusterBlock <= max_bound) b <<= 1;
    return b;
}

size_t subsample_smem_bytes();
uint32_t subsample_block_size();

// Cluster size for a distance-weighted level: the c (1 to cap, at most
// num_sms) with the smallest estimated level time
//     max(1 / resident blocks(c), r / c) * g(c)
// where resident blocks(c) = min(n_nodes, slots[log2 c]) * c, slots[i] the
// clusters of 2^i blocks the device holds at once (a cluster must fit in one
// GPC, so this differs between chips), r = the largest node's share of the
// level's candidates (balance / num_sms) and g(c) the per-block cost of
// cluster-wide work, fitted to measured levels: one-node and 8-node levels of
// the 25.8M-point weighted build ran 1.29x and 1.74x (root) and 1.62x and
// 2.15x (8 nodes) longer per block at clusters of 8 and 16 than at 4, about
// c^0.4.  On a GPU that holds 7 clusters of 16 this gives the largest node at
// least its share of the blocks; on one that holds fewer, levels of many
// nodes take smaller clusters.  The allocation-free entry point passes
// num_sms = 1 and gets one block.
inline uint32_t weighted_cluster_choice(const int slots[5], uint32_t n_nodes, int num_sms, uint32_t balance,
                                        uint32_t cap) {
    static const double g[5] = {1.0, 1.32, 1.74, 2.30, 3.03};
    const uint32_t sms = (uint32_t)(num_sms > 1 ? num_sms : 1);
    const double r = (double)balance / (double)sms;
    uint32_t best = 1;
    double best_t = std::max(1.0 / (double)std::min(n_nodes, sms), r);
    int i = 1;
    for (uint32_t c = 2; c <= cap && c <= sms && i < 5; c <<= 1, ++i) {
        const int s = slots[i];
        if (s <= 0) break;
        const double blocks = (double)std::min(n_nodes, (uint32_t)s) * c;
        const double t = std::max(1.0 / blocks, r / c) * g[i];
        if (t < best_t) {
            best_t = t;
            best = c;
        }
    }
    return best;
}
// balance_blocks: the blocks the level's largest node needs for its share
// of the work to equal one SM's share of the whole level (largest candidate
// bound x SMs / sum of the bounds); distance-weighted levels size their
// clusters by it.
int launch_subsample_level(const SubLevelArgs& a, int num_sms, uint32_t balance_blocks, cudaStream_t stream,
                           const ClusterCaps& caps = ClusterCaps{});
// `wave` holds what the step shares: n_nodes (all builds' nodes), the work
// counter, the per-block global brick tables, the mode and record type; the
// build-specific fields come from wn.clouds.  A node whose build has the
// capacity error set is skipped.
int launch_subsample_wave(const SubLevelArgs& wave, const WaveNodes& wn, int num_sms, uint32_t balance_blocks,
                          cudaStream_t stream, const ClusterCaps& caps = ClusterCaps{});
// The emit of the nodes a launch_subsample_level with emit_state handed
// over, on num_sms blocks; launched right after it on the same stream.
int launch_emit_weighted(const SubLevelArgs& a, int num_sms, cudaStream_t stream);

// Raises a kernel's dynamic shared memory limit on the current device to at
// least `bytes` and never lowers it, so that builders launching the same
// kernel from several host threads cannot undercut each other's launches.
void allow_dynamic_smem(const void* kernel, size_t bytes);

// Moves staged internal-node records to their final (post-order) positions.
int launch_place(const uint64_t* src_off, const uint64_t* dst_off, const uint32_t* count, uint32_t n_nodes,
                 const uint8_t* stage_rec, uint8_t* rec, cudaStream_t stream);
// Same for the per-record cloud indices.
// Post-order output positions of the internal nodes and the copy list of
// launch_place (see k_place_prepare).
int launch_place_prepare(const uint32_t* post, uint32_t n_internal, const uint32_t* points, const uint64_t* stage_off,
                         uint64_t n, uint64_t cap, uint64_t* src, uint64_t* dst, uint32_t* cnt, uint64_t* node_dst,
                         uint64_t* total, uint32_t* err, cudaStream_t stream);

int launch_place_lut(const uint64_t* src_off, const uint64_t* dst_off, const uint32_t* count, uint32_t n_nodes,
                     const uint32_t* stage_lut, uint32_t* lut, cudaStream_t stream);

}   // namespace oc
