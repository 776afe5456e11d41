// Level-batched subsampling of internal nodes (one launch per tree level).
//
// Replaces the reference's host DFS (fp_subsampling.cu:9-185,
// rp_subsampling.cu:10-222), which launches 2-5 kernels per internal node, each
// sized by the largest leaf.  Here one persistent kernel per level processes
// all internal nodes of that level; a block owns one node at a time:
//
//   pass A  every candidate (the children's points, in slot order) is mapped to
//           its cell of the node's S^3 grid (mapPointToGrid with the node's
//           bbox, kernel_helpers.cuh:10-25).  Occupied cells are recorded in a
//           shared-memory brick map: a hash of occupied 4x4x4 bricks, each with
//           a 64-bit occupancy mask.  The candidate's (brick slot, bit) is cached.
//   ranks   the masks are prefix-summed: every occupied cell gets a dense rank,
//           and the node's point count is the number of occupied cells
//           (the pointCount of fp/rp evaluation, fp_subsample_evaluation.cuh:22-110).
//   pass B  per candidate: selection key min (first point = smallest cloud
//           index; explicit random = smallest Philox priority) and the packed
//           colour sum of the cell (encodeColors, kernel_helpers.cuh:49-53).
//   emit    per occupied cell: colour (raw / intra / 3x3x3 inter sum /
//           distance-weighted, kernel_inter_cell_filtering.cuh:20-194), output
//           coordinates of the chosen point, staged record.
//
// All neighbour lookups of the 3x3x3 filters go through the shared brick map.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "device_common.cuh"
#include "kernels.h"

namespace oc {

namespace {

constexpr int kSubThreads = 1024;
constexpr uint32_t kBrickSlots = 8192;    // shared-memory brick table capacity
constexpr uint32_t kBrickShift = 32 - 13;

struct BrickMap {
    uint32_t* key;    // brick id + 1, 0 = empty
    uint64_t* mask;   // occupied cells of the brick (bit = x | y<<2 | z<<4)
    uint32_t* base;   // rank of the brick's first cell
    uint32_t cap;     // slots (power of two, multiple of the block size)
    uint32_t shift;   // 32 - log2(cap)
    uint32_t bs;      // bricks per axis
    uint32_t grid;    // S
};

__device__ __forceinline__ uint32_t brick_hash(const BrickMap& m, uint32_t b1) {
    return (b1 * 2654435761u) >> m.shift;
}

// Inserts brick b1 (id + 1); returns its slot (cap on failure) and whether
// this call claimed the slot.
__device__ __forceinline__ uint32_t brick_insert(const BrickMap& m, uint32_t b1, bool& fresh) {
    volatile uint32_t* vk = m.key;
    uint32_t h = brick_hash(m, b1);
    fresh = false;
    for (uint32_t probe = 0; probe < m.cap; ++probe) {
        uint32_t cur = vk[h];
        if (cur == b1) return h;
        if (cur == 0) {
            uint32_t old = atomicCAS(&m.key[h], 0u, b1);
            if (old == 0) {
                fresh = true;
                return h;
            }
            if (old == b1) return h;
        }
        h = (h + 1) & (m.cap - 1);
    }
    return m.cap;
}

__device__ __forceinline__ int brick_find(const BrickMap& m, uint32_t b1) {
    uint32_t h = brick_hash(m, b1);
    for (uint32_t probe = 0; probe < m.cap; ++probe) {
        uint32_t cur = m.key[h];
        if (cur == b1) return (int)h;
        if (cur == 0) return -1;
        h = (h + 1) & (m.cap - 1);
    }
    return -1;
}

// Rank of cell (x, y, z) or -1 when unoccupied / outside the grid.
__device__ __forceinline__ int cell_rank(const BrickMap& m, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= (int)m.grid || y >= (int)m.grid || z >= (int)m.grid) return -1;
    uint32_t b = ((uint32_t)x >> 2) + m.bs * (((uint32_t)y >> 2) + m.bs * ((uint32_t)z >> 2));
    int s = brick_find(m, b + 1);
    if (s < 0) return -1;
    uint32_t bit = (x & 3) | ((y & 3) << 2) | ((z & 3) << 4);
    uint64_t mk = m.mask[s];
    if (!((mk >> bit) & 1ull)) return -1;
    return (int)(m.base[s] + __popcll(mk & ((1ull << bit) - 1ull)));
}

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    uint32_t warp_prefix = warp ? warp_sums[warp - 1] : 0;
    total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

struct NodeShared {
    uint64_t start[8];
    uint32_t count[8];
    uint32_t prefix[9];
    uint32_t kind;
    uint32_t nchild;
    uint32_t node;
    uint32_t cells;
};

// Candidate j of the current node: which child, and its position there.
__device__ __forceinline__ void locate(const NodeShared& ns, uint32_t j, uint32_t& c, uint64_t& pos) {
    c = 0;
    while (c + 1 < ns.nchild && ns.prefix[c + 1] <= j) ++c;
    pos = ns.start[c] + (j - ns.prefix[c]);
}

template <bool kF32>
__global__ void __launch_bounds__(kSubThreads, 1) k_subsample(SubLevelArgs a) {
    extern __shared__ uint64_t dyn[];
    __shared__ NodeShared ns;
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t s_bricks, s_overflow;
    BrickMap sm_map;
    sm_map.mask = dyn;
    sm_map.key = reinterpret_cast<uint32_t*>(dyn + kBrickSlots);
    sm_map.base = sm_map.key + kBrickSlots;
    sm_map.cap = kBrickSlots;
    sm_map.shift = kBrickShift;
    sm_map.grid = a.grid;
    sm_map.bs = (a.grid + 3) >> 2;
    // per-block brick table in global memory for nodes that outgrow shared memory
    BrickMap gl_map = sm_map;
    gl_map.cap = a.global_cap;
    gl_map.shift = a.global_shift;
    gl_map.mask = a.global_mask + (uint64_t)blockIdx.x * a.global_cap;
    gl_map.key = a.global_key + (uint64_t)blockIdx.x * a.global_cap;
    gl_map.base = a.global_base + (uint64_t)blockIdx.x * a.global_cap;

    const bool intra = (a.mode & kModeIntra) != 0;
    const bool inter = !intra && (a.mode & kModeInter) != 0;
    const bool weighted = inter && (a.mode & kModeWeight) != 0;
    const bool random = (a.mode & kModeRandom) != 0;
    const bool averaged = intra || inter;

    for (;;) {
        if (threadIdx.x == 0) ns.node = atomicAdd(a.work_counter, 1u);
        __syncthreads();
        const uint32_t ni = ns.node;
        if (ni >= a.n_nodes) break;
        const SubNode& nd = a.nodes[ni];
        if (threadIdx.x == 0) {
            ns.nchild = nd.nchild;
            ns.kind = nd.child_kind;
            uint32_t p = 0;
            for (uint32_t c = 0; c < nd.nchild; ++c) {
                ns.start[c] = nd.child_start[c];
                ns.count[c] = nd.child_count[c];
                ns.prefix[c] = p;
                p += nd.child_count[c];
            }
            ns.prefix[nd.nchild] = p;
        }
        const AxisGrid ax0 = nd.ax[0], ax1 = nd.ax[1], ax2 = nd.ax[2];
        const uint32_t p_in = nd.p_in;
        const uint64_t off = nd.cand_off;
        BrickMap bm = sm_map;

        // ---- pass A: cells and occupancy.  A node whose bricks exceed 70% of
        // the shared table is redone with the block's global-memory table.
        for (int attempt = 0; attempt < 2; ++attempt) {
            for (uint32_t i = threadIdx.x; i < bm.cap; i += blockDim.x) {
                bm.key[i] = 0;
                bm.mask[i] = 0;
            }
            if (threadIdx.x == 0) {
                s_bricks = 0;
                s_overflow = 0;
            }
            __syncthreads();
            const uint32_t limit = bm.cap - (bm.cap >> 2) - (bm.cap >> 4);
            for (uint32_t j = threadIdx.x; j < p_in; j += blockDim.x) {
                if (*(volatile uint32_t*)&s_overflow) break;
                uint32_t c;
                uint64_t pos;
                locate(ns, j, c, pos);
                bool staged = (ns.kind >> c) & 1u;
                uint32_t idx = staged ? a.stage_lut[pos] : a.leaf_lut[pos];
                Coord co[3];
                uint32_t col[3];
                load_point<kF32>(a.cloud + (uint64_t)idx * a.stride, co, col);
                float ux, uy, uz;
                int ix = axis_cell<kF32>(co[0], ax0, a.grid, ux);
                int iy = axis_cell<kF32>(co[1], ax1, a.grid, uy);
                int iz = axis_cell<kF32>(co[2], ax2, a.grid, uz);
                if ((ix | iy | iz) < 0) {
                    atomicOr(a.err, kErrBelowBox);
                    ix = max(ix, 0);
                    iy = max(iy, 0);
                    iz = max(iz, 0);
                }
                uint32_t b = ((uint32_t)ix >> 2) + bm.bs * (((uint32_t)iy >> 2) + bm.bs * ((uint32_t)iz >> 2));
                uint32_t bit = (ix & 3) | ((iy & 3) << 2) | ((iz & 3) << 4);
                bool fresh;
                uint32_t slot = brick_insert(bm, b + 1, fresh);
                if (fresh && atomicAdd(&s_bricks, 1u) + 1 >= limit) s_overflow = 1;
                if (slot >= bm.cap) {
                    s_overflow = 1;
                    break;
                }
                atomicOr(reinterpret_cast<unsigned long long*>(&bm.mask[slot]), 1ull << bit);
                a.key_cache[off + j] = (slot << 6) | bit;
                if (weighted) {
                    a.unit_cache[(off + j) * 3 + 0] = ux;
                    a.unit_cache[(off + j) * 3 + 1] = uy;
                    a.unit_cache[(off + j) * 3 + 2] = uz;
                }
            }
            __syncthreads();
            if (!s_overflow) break;
            if (attempt == 1 || bm.key == gl_map.key) {
                if (threadIdx.x == 0) atomicOr(a.err, kErrProbe);
                break;
            }
            bm = gl_map;
            __syncthreads();
        }
        const bool failed = s_overflow != 0;
        __syncthreads();
        if (failed) {
            if (threadIdx.x == 0) a.out_points[ni] = 0;
            continue;
        }

        // ---- ranks of occupied cells (each thread scans a run of slots)
        {
            const uint32_t per = bm.cap / blockDim.x;
            const uint32_t first = threadIdx.x * per;
            uint32_t sum = 0;
            for (uint32_t k = 0; k < per; ++k) sum += (uint32_t)__popcll(bm.mask[first + k]);
            uint32_t total;
            uint32_t pre = block_exclusive_scan(sum, warp_sums, total);
            for (uint32_t k = 0; k < per; ++k) {
                bm.base[first + k] = pre;
                pre += (uint32_t)__popcll(bm.mask[first + k]);
            }
            if (threadIdx.x == 0) ns.cells = total;
        }
        __syncthreads();
        const uint32_t cells = ns.cells;
        for (uint32_t r = threadIdx.x; r < cells; r += blockDim.x) {
            a.acc_best[off + r] = ~0ull;
            if (averaged && !weighted) a.acc_intra[off + r] = 0;
            if (weighted) a.csr_count[off + r] = 0;
        }
        __syncthreads();

        // ---- pass B: selection and colour sums
        for (uint32_t j = threadIdx.x; j < p_in; j += blockDim.x) {
            uint32_t kc = a.key_cache[off + j];
            uint32_t slot = kc >> 6, bit = kc & 63;
            if (slot >= bm.cap) continue;
            uint32_t rank = bm.base[slot] + (uint32_t)__popcll(bm.mask[slot] & ((1ull << bit) - 1ull));
            uint32_t c;
            uint64_t pos;
            locate(ns, j, c, pos);
            bool staged = (ns.kind >> c) & 1u;
            uint32_t idx = staged ? a.stage_lut[pos] : a.leaf_lut[pos];
            uint64_t key = idx;
            if (random) key |= (uint64_t)rp_priority(a.seed, nd.level, nd.morton, idx) << 32;
            atomicMin(reinterpret_cast<unsigned long long*>(&a.acc_best[off + rank]), (unsigned long long)key);
            if (averaged && !weighted) {
                const uint16_t* src = reinterpret_cast<const uint16_t*>((staged ? a.stage_rec : a.leaf_rec) + pos * 18);
                uint64_t enc = encode_colors(src[6], src[7], src[8]);
                atomicAdd(reinterpret_cast<unsigned long long*>(&a.acc_intra[off + rank]), (unsigned long long)enc);
            }
            if (weighted) atomicAdd(&a.csr_count[off + rank], 1u);
        }
        __syncthreads();

        // ---- weighted: group candidates by cell (CSR)
        if (weighted) {
            uint32_t running = 0;
            for (uint32_t base = 0; base < cells; base += blockDim.x) {
                uint32_t r = base + threadIdx.x;
                uint32_t v = r < cells ? a.csr_count[off + r] : 0;
                uint32_t total;
                uint32_t pre = block_exclusive_scan(v, warp_sums, total);
                if (r < cells) {
                    a.csr_start[off + r] = running + pre;
                    a.csr_count[off + r] = 0;
                }
                running += total;
            }
            __syncthreads();
            for (uint32_t j = threadIdx.x; j < p_in; j += blockDim.x) {
                uint32_t kc = a.key_cache[off + j];
                uint32_t slot = kc >> 6, bit = kc & 63;
                if (slot >= bm.cap) continue;
                uint32_t rank = bm.base[slot] + (uint32_t)__popcll(bm.mask[slot] & ((1ull << bit) - 1ull));
                uint32_t p = a.csr_start[off + rank] + atomicAdd(&a.csr_count[off + rank], 1u);
                uint32_t c;
                uint64_t pos;
                locate(ns, j, c, pos);
                bool staged = (ns.kind >> c) & 1u;
                const uint16_t* src = reinterpret_cast<const uint16_t*>((staged ? a.stage_rec : a.leaf_rec) + pos * 18);
                uint32_t* dst = reinterpret_cast<uint32_t*>(a.csr_pts + (off + p) * 20);
                dst[0] = __float_as_uint(a.unit_cache[(off + j) * 3 + 0]);
                dst[1] = __float_as_uint(a.unit_cache[(off + j) * 3 + 1]);
                dst[2] = __float_as_uint(a.unit_cache[(off + j) * 3 + 2]);
                dst[3] = (uint32_t)src[6] | ((uint32_t)src[7] << 16);
                dst[4] = (uint32_t)src[8];
            }
            __syncthreads();
        }

        // ---- emit one record per occupied cell
        for (uint32_t r = threadIdx.x; r < cells; r += blockDim.x) {
            // slot holding rank r: last slot with base <= r and a non-empty mask
            uint32_t lo = 0, hi = bm.cap - 1;
            while (lo < hi) {
                uint32_t mid = (lo + hi + 1) >> 1;
                if (bm.base[mid] <= r) lo = mid;
                else hi = mid - 1;
            }
            uint32_t slot = lo;
            while (slot > 0 && (bm.mask[slot] == 0 || bm.base[slot] > r)) --slot;
            uint64_t mk = bm.mask[slot];
            uint32_t want = r - bm.base[slot];
            uint32_t bit = 0;
            for (uint32_t seen = 0; bit < 64; ++bit) {
                if ((mk >> bit) & 1ull) {
                    if (seen == want) break;
                    ++seen;
                }
            }
            if (bit >= 64) {
                atomicOr(a.err, kErrProbe);
                bit = 0;
            }
            uint32_t brick = bm.key[slot] - 1;
            int bx = (int)(brick % bm.bs), by = (int)((brick / bm.bs) % bm.bs), bz = (int)(brick / (bm.bs * bm.bs));
            int x = bx * 4 + (int)(bit & 3), y = by * 4 + (int)((bit >> 2) & 3), z = bz * 4 + (int)((bit >> 4) & 3);

            uint64_t best = a.acc_best[off + r];
            uint32_t idx = (uint32_t)best;
            Coord co[3];
            uint32_t col[3];
            load_point<kF32>(a.cloud + (uint64_t)idx * a.stride, co, col);
            uint16_t cr = (uint16_t)col[0], cg = (uint16_t)col[1], cb = (uint16_t)col[2];
            if (intra) {
                decode_colors(a.acc_intra[off + r], cr, cg, cb);
            } else if (inter && !weighted) {
                uint64_t e = 0;
                for (int ox = -1; ox <= 1; ++ox)
                    for (int oy = -1; oy <= 1; ++oy)
                        for (int oz = -1; oz <= 1; ++oz) {
                            int n = cell_rank(bm, x + ox, y + oy, z + oz);
                            if (n >= 0) e += a.acc_intra[off + n];
                        }
                decode_colors(e, cr, cg, cb);
            } else if (weighted) {
                uint64_t sr = 0, sg = 0, sb = 0, sw = 0;
                for (int ox = -1; ox <= 1; ++ox)
                    for (int oy = -1; oy <= 1; ++oy)
                        for (int oz = -1; oz <= 1; ++oz) {
                            int n = cell_rank(bm, x + ox, y + oy, z + oz);
                            if (n < 0) continue;
                            uint32_t s0 = a.csr_start[off + n], s1 = s0 + a.csr_count[off + n];
                            for (uint32_t p = s0; p < s1; ++p) {
                                const uint32_t* q = reinterpret_cast<const uint32_t*>(a.csr_pts + (off + p) * 20);
                                uint32_t wq = weight_q(__uint_as_float(q[0]), __uint_as_float(q[1]),
                                                       __uint_as_float(q[2]), x, y, z);
                                sr += (uint64_t)wq * (q[3] & 0xFFFF);
                                sg += (uint64_t)wq * (q[3] >> 16);
                                sb += (uint64_t)wq * (q[4] & 0xFFFF);
                                sw += wq;
                            }
                        }
                if (sw) {
                    cr = (uint16_t)(sr / sw);
                    cg = (uint16_t)(sg / sw);
                    cb = (uint16_t)(sb / sw);
                }
            }
            int32_t ox_ = out_coord<kF32>(co[0], a.out.ax[0]);
            int32_t oy_ = out_coord<kF32>(co[1], a.out.ax[1]);
            int32_t oz_ = out_coord<kF32>(co[2], a.out.ax[2]);
            if (ox_ == kCoordError || oy_ == kCoordError || oz_ == kCoordError) atomicOr(a.err, kErrCoordRange);
            a.out_lut[off + r] = idx;
            store_record(a.out_rec, off + r, ox_, oy_, oz_, cr, cg, cb);
        }
        if (threadIdx.x == 0) a.out_points[ni] = cells;
        __syncthreads();
    }
}

}   // namespace

uint32_t subsample_block_size() {
    return kSubThreads;
}

size_t subsample_smem_bytes() {
    return (size_t)kBrickSlots * (8 + 4 + 4);
}

int launch_subsample_level(const SubLevelArgs& a, int num_sms, cudaStream_t stream) {
    if (!a.n_nodes) return 0;
    size_t smem = subsample_smem_bytes();
    int grid = (int)std::min<uint32_t>(a.n_nodes, (uint32_t)num_sms);
    if (a.float_input) {
        cudaFuncSetAttribute(k_subsample<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_subsample<true><<<grid, kSubThreads, smem, stream>>>(a);
    } else {
        cudaFuncSetAttribute(k_subsample<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_subsample<false><<<grid, kSubThreads, smem, stream>>>(a);
    }
    return 1;
}

}   // namespace oc
