// Chunking stages of the LOD build: binning into the finest counting grid,
// the count pyramid, tree enumeration, leaf tagging and point distribution.
//
// Replaces the reference kernels K1-K5 (point_counting.cuh:29-53,
// point_count_propagation.cuh:34-86, octree_initialization.cuh:24-52,
// hierarchical_merging.cuh:35-122, point_distributing.cuh:30-75).  The dense
// counting grid is kept in Morton order so that the eight children of a cell
// are adjacent: the pyramid is a streaming reduction, and the tree is
// enumerated top-down from the internal nodes only (no dense sweeps over the
// upper levels).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "device_common.cuh"
#include "kernels.h"

namespace oc {

namespace {

constexpr uint32_t kLeafTag = 0x80000000u;
constexpr uint32_t kNoKey = 0xFFFFFFFFu;   // run key of lanes without a point

__device__ __forceinline__ void set_error(uint32_t* err, uint32_t bit) {
    atomicOr(err, bit);
}

// ---------------------------------------------------------------------------
// Tile pipeline of the two streaming passes over the cloud (counting and
// distribution).  Each block walks tiles blockIdx.x, +gridDim.x, ... of
// `tile` records; tile j+1 is bulk-copied (TMA) into the other of two
// shared-memory buffers while tile j is processed.

// counting: 1024-record tiles, 512 threads
constexpr uint32_t kCountTile = 1024;
constexpr uint32_t kCountThreads = 512;
// distribution: 896-record tiles, 448 threads (three blocks fit one SM's
// registers)
constexpr uint32_t kDistTile = 896;
constexpr uint32_t kDistThreads = 448;

__host__ __device__ inline uint32_t align_up(uint32_t x, uint32_t a) {
    return (x + a - 1) / a * a;
}

// Shared-memory layout: [0, 16) two mbarriers, [16, 20) abort flag, then the
// boundary keys of the three axes, the Morton spread table and two tile
// buffers.  A buffer holds a tile's byte span rounded out to 16 bytes plus
// read slack.
struct ChunkSmem {
    uint32_t keys_off, spread_off, buf_off, buf_bytes, total;
};

__host__ __device__ inline ChunkSmem chunk_smem(uint32_t stride, uint32_t grid, bool f32, uint32_t tile) {
    ChunkSmem m;
    m.keys_off = 128;
    m.spread_off = align_up(m.keys_off + 3 * (grid + 2) * (f32 ? 4u : 8u), 16);
    m.buf_off = align_up(m.spread_off + grid * 4, 128);
    m.buf_bytes = align_up(tile * stride + 48, 128);
    m.total = m.buf_off + 2 * m.buf_bytes;
    return m;
}

// Copies the boundary keys and the spread table into shared memory.
template <bool kF32>
__device__ __forceinline__ void load_tables(const CloudGrid& g, uint8_t* smem, const ChunkSmem& L) {
    using K = typename std::conditional<kF32, int32_t, long long>::type;
    const K* src = static_cast<const K*>(g.keys);
    K* dst = reinterpret_cast<K*>(smem + L.keys_off);
    for (uint32_t i = threadIdx.x; i < 3 * (g.grid + 2); i += blockDim.x) dst[i] = src[i];
    uint32_t* sp = reinterpret_cast<uint32_t*>(smem + L.spread_off);
    for (uint32_t i = threadIdx.x; i < g.grid; i += blockDim.x) sp[i] = g.spread[i];
}

__device__ __forceinline__ void issue_tile(const uint8_t* __restrict__ cloud, uint64_t n, uint32_t stride, uint32_t tile,
                                           uint64_t t, uint8_t* buf, uint64_t* bar) {
    const uint64_t p0 = t * tile;
    const uint64_t p1 = (n - p0) < tile ? n : p0 + tile;
    const uint64_t a0 = (p0 * stride) & ~15ull, a1 = (p1 * stride + 15) & ~15ull;
    bulk_load(buf, cloud + a0, (uint32_t)(a1 - a0), bar);
}

// Runs body(records_of_tile, first_point, count) for every tile of this
// block.  The body must be memory-safe for any buffer contents: after a
// bounded wait gives up (error bit kErrTimeout) the tile is still processed
// by every thread, so that warp collectives stay converged, and the loop
// ends at the next block barrier.
template <uint32_t kTile, class Body>
__device__ __forceinline__ void tile_loop(const uint8_t* __restrict__ cloud, uint64_t n, uint32_t stride, uint8_t* smem,
                                          const ChunkSmem& L, uint32_t* err, Body&& body) {
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    volatile uint32_t* abort_flag = reinterpret_cast<volatile uint32_t*>(smem + 16);
    uint8_t* buf0 = smem + L.buf_off;
    uint8_t* buf1 = buf0 + L.buf_bytes;
    const uint64_t tiles = (n + kTile - 1) / kTile;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        *abort_flag = 0;
        fence_barrier_init();
    }
    __syncthreads();
    uint64_t t = blockIdx.x;
    if (threadIdx.x == 0 && t < tiles) issue_tile(cloud, n, stride, kTile, t, buf0, &bar[0]);
    uint32_t j = 0;
    bool aborted = false;
    for (; t < tiles; t += gridDim.x, ++j) {
        const uint32_t slot = j & 1;
        const uint64_t tn = t + gridDim.x;
        // the other buffer was released by the barrier that ended the previous tile
        if (threadIdx.x == 0 && tn < tiles) issue_tile(cloud, n, stride, kTile, tn, slot ? buf0 : buf1, &bar[slot ^ 1]);
        if (!mbar_wait_bounded(&bar[slot], (j >> 1) & 1)) {
            set_error(err, kErrTimeout);
            *abort_flag = 1;
        }
        const uint64_t p0 = t * kTile;
        const uint32_t cnt = (uint32_t)((n - p0) < kTile ? (n - p0) : kTile);
        body((slot ? buf1 : buf0) + (uint32_t)((p0 * stride) & 15), p0, cnt);
        __syncthreads();
        if (*abort_flag) {
            aborted = true;
            break;
        }
    }
    if (aborted && threadIdx.x == 0) {
        // let the copies still in flight land before the block exits (bounded)
        const uint32_t slot = j & 1;
        mbar_wait_bounded(&bar[slot], (j >> 1) & 1);
        if (t + gridDim.x < tiles) mbar_wait_bounded(&bar[slot ^ 1], ((j + 1) >> 1) & 1);
    }
}

// 32-bit words w[0..kWords) of a record at any byte alignment in shared memory.
template <int kWords>
__device__ __forceinline__ void record_words(const uint8_t* rec, uint32_t (&w)[kWords]) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(rec);
    const uint32_t* q = reinterpret_cast<const uint32_t*>(a & ~(uintptr_t)3);
    const uint32_t s = (uint32_t)(a & 3) * 8;
    uint32_t raw[kWords + 1];
#pragma unroll
    for (int j = 0; j <= kWords; ++j) raw[j] = q[j];
#pragma unroll
    for (int j = 0; j < kWords; ++j) w[j] = __funnelshift_r(raw[j], raw[j + 1], s);
}

// Cells of a point from its coordinate words (3 floats or 3 x lo/hi of
// doubles), exactly as (int64)fmin((p - min) / t, G - 1) in binary64.
// Returns false when the point lies below the bounding box.
template <bool kF32>
__device__ __forceinline__ bool point_cells(const uint32_t* w, const CloudGrid& g, const uint8_t* smem,
                                            const ChunkSmem& L, int cell[3]) {
    const uint32_t G = g.grid;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int i;
        if (kF32) {
            const int32_t* K = reinterpret_cast<const int32_t*>(smem + L.keys_off) + a * (G + 2);
            const uint32_t b = w[a];
            i = table_cell<int32_t>(dev_key32(b), __fmaf_rn(__uint_as_float(b), g.r[a], g.c[a]), K, G);
            if (i == -2) i = exact_axis_cell((double)__uint_as_float(b), g.ax[a].mn, g.ax[a].t, G);
        } else {
            const long long* K = reinterpret_cast<const long long*>(smem + L.keys_off) + a * (G + 2);
            const uint32_t lo = w[2 * a], hi = w[2 * a + 1];
            i = table_cell<long long>(dev_key64(lo, hi), __fmaf_rn(approx_f64(lo, hi), g.r[a], g.c[a]), K, G);
            if (i == -2) i = exact_axis_cell(__hiloint2double((int)hi, (int)lo), g.ax[a].mn, g.ax[a].t, G);
        }
        cell[a] = i;
    }
    return (cell[0] | cell[1] | cell[2]) >= 0;
}

__device__ __forceinline__ uint32_t cell_morton(const int cell[3], const uint8_t* smem, const ChunkSmem& L) {
    const uint32_t* sp = reinterpret_cast<const uint32_t*>(smem + L.spread_off);
    return (sp[cell[0]] << 2) | (sp[cell[1]] << 1) | sp[cell[2]];
}

// K1 (point_counting.cuh:29-53): points per finest cell.  Consecutive lanes
// in the same cell add their count with one atomic.
// With `occ` (sparse clouds) the run leaders also flag their cell's 64-cell
// block (a level-2 cell): a plain byte store, no read-modify-write.
template <bool kF32>
__global__ void __launch_bounds__(kCountThreads) k_count(const uint8_t* __restrict__ cloud, uint64_t n, uint32_t stride,
                                                         CloudGrid g, uint32_t* __restrict__ pyr0, uint8_t* occ,
                                                         uint32_t* err) {
    extern __shared__ __align__(128) uint8_t smem[];
    const ChunkSmem L = chunk_smem(stride, g.grid, kF32, kCountTile);
    load_tables<kF32>(g, smem, L);
    const uint32_t lane = threadIdx.x & 31;
    tile_loop<kCountTile>(cloud, n, stride, smem, L, err, [&](const uint8_t* recs, uint64_t p0, uint32_t cnt) {
#pragma unroll 1
        for (uint32_t base = 0; base < kCountTile; base += kCountThreads) {
            const uint32_t k = base + threadIdx.x;
            uint32_t m = kNoKey;
            if (k < cnt) {
                constexpr int kWords = kF32 ? 3 : 6;
                uint32_t w[kWords];
                record_words<kWords>(recs + (uint64_t)k * stride, w);
                int cell[3];
                if (point_cells<kF32>(w, g, smem, L, cell)) m = cell_morton(cell, smem, L);
                else set_error(err, kErrBelowBox);
            }
            const uint32_t starts = run_starts(m);
            if (m != kNoKey && ((starts >> lane) & 1u)) {
                atomicAdd(&pyr0[m], run_end(starts) - lane);
                if (occ) occ[m >> 6] = 1;
            }
        }
    });
}

// Coordinate minima and maxima (calculateRealBB, src/boundingbox.h:11-33) as
// ordered keys: keys[0..2] minima, keys[3..5] maxima.  NaN coordinates are
// skipped, as fmin / fmax skip them.  Float keys are widened to 64 bits.
template <bool kF32>
__global__ void __launch_bounds__(256) k_bbox(const uint8_t* __restrict__ cloud, uint64_t n, uint32_t stride,
                                              long long* keys) {
    long long mn[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, mx[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        constexpr int kWords = kF32 ? 3 : 6;
        uint32_t w[kWords];
        const uint8_t* rec = cloud + i * stride;
        const uintptr_t a = reinterpret_cast<uintptr_t>(rec);
        const uint32_t* q = reinterpret_cast<const uint32_t*>(a & ~(uintptr_t)3);
        const uint32_t sh = (uint32_t)(a & 3) * 8;
#pragma unroll
        for (int j = 0; j < kWords; ++j) w[j] = __funnelshift_r(q[j], q[j + 1], sh);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            long long k;
            bool nan;
            if (kF32) {
                nan = (w[c] & 0x7FFFFFFFu) > 0x7F800000u;
                k = dev_key32(w[c]);
            } else {
                const uint32_t lo = w[2 * c], hi = w[2 * c + 1];
                nan = (hi & 0x7FFFFFFFu) > 0x7FF00000u || ((hi & 0x7FFFFFFFu) == 0x7FF00000u && lo != 0);
                k = dev_key64(lo, hi);
            }
            if (!nan) {
                mn[c] = min(mn[c], k);
                mx[c] = max(mx[c], k);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[c] = min(mn[c], (long long)__shfl_xor_sync(0xffffffffu, (unsigned long long)mn[c], o));
            mx[c] = max(mx[c], (long long)__shfl_xor_sync(0xffffffffu, (unsigned long long)mx[c], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (mn[c] != LLONG_MAX) atomicMin(&keys[c], mn[c]);
            if (mx[c] != LLONG_MIN) atomicMax(&keys[3 + c], mx[c]);
        }
    }
}

__global__ void k_bbox_init(long long* keys) {
    if (threadIdx.x < 6) keys[threadIdx.x] = threadIdx.x < 3 ? LLONG_MAX : LLONG_MIN;
}

// Level l -> levels l+1 and l+2: one thread per level-(l+2) cell reads its 64
// Morton-contiguous level-l counts.
// With `occ` (the finest level of a sparse cloud), a level-2 cell whose
// block flag is clear has only empty children: its sums are written as 0
// without reading them.
__global__ void k_pyramid2(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst1, uint32_t* __restrict__ dst2,
                           uint64_t n2, uint32_t* nz_src, uint32_t* nz_dst1, const uint8_t* __restrict__ occ) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint32_t nzs = 0, nzd = 0;
    const bool empty = i < n2 && occ && occ[i] == 0;
    if (empty) {
        uint4* d = reinterpret_cast<uint4*>(dst1 + i * 8);
        d[0] = make_uint4(0, 0, 0, 0);
        d[1] = make_uint4(0, 0, 0, 0);
        dst2[i] = 0;
    } else if (i < n2) {
        const uint4* s = reinterpret_cast<const uint4*>(src + i * 64);
        uint32_t sums[8];
        uint32_t total = 0;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            uint4 a = s[2 * c], b = s[2 * c + 1];
            uint32_t v = a.x + a.y + a.z + a.w + b.x + b.y + b.z + b.w;
            nzs += (a.x != 0) + (a.y != 0) + (a.z != 0) + (a.w != 0) + (b.x != 0) + (b.y != 0) + (b.z != 0) + (b.w != 0);
            sums[c] = v;
            nzd += v != 0;
            total += v;
        }
        uint4* d = reinterpret_cast<uint4*>(dst1 + i * 8);
        d[0] = make_uint4(sums[0], sums[1], sums[2], sums[3]);
        d[1] = make_uint4(sums[4], sums[5], sums[6], sums[7]);
        dst2[i] = total;
    }
    for (int o = 16; o > 0; o >>= 1) {
        nzs += __shfl_down_sync(0xffffffffu, nzs, o);
        nzd += __shfl_down_sync(0xffffffffu, nzd, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (nzs) atomicAdd(nz_src, nzs);
        if (nzd) atomicAdd(nz_dst1, nzd);
    }
}

// Level l -> level l+1 only.
__global__ void k_pyramid1(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, uint64_t n1, uint32_t* nz_src) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint32_t nzs = 0;
    if (i < n1) {
        uint32_t total = 0;
        for (int c = 0; c < 8; ++c) {
            uint32_t v = src[i * 8 + c];
            nzs += v != 0;
            total += v;
        }
        dst[i] = total;
    }
    for (int o = 16; o > 0; o >>= 1) nzs += __shfl_down_sync(0xffffffffu, nzs, o);
    if ((threadIdx.x & 31) == 0 && nzs) atomicAdd(nz_src, nzs);
}

__global__ void k_count_root(const uint32_t* root, uint32_t* nz) {
    if (threadIdx.x == 0 && root[0] != 0) atomicAdd(nz, 1u);
}

// Block-wide exclusive scan of one value per thread (blockDim.x = 1024).
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

// Top-down tree enumeration in hierarchy BFS order (potree_exporter.cu:62-96):
// a node at level >= 1 whose count reaches the threshold is internal
// (hierarchical_merging.cuh:134) and all its occupied children are tree nodes;
// every other tree node is a leaf.  One block walks the levels.
__global__ void __launch_bounds__(1024) k_enumerate(const uint32_t* __restrict__ pyr, const uint64_t* __restrict__ loff,
                                                    uint32_t depth, uint32_t threshold, uint32_t* key, uint32_t* count,
                                                    uint8_t* level, uint16_t* info, uint32_t* child_first, uint32_t cap,
                                                    uint32_t* level_start, uint32_t* n_nodes, uint32_t* err) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t s_next;
    if (threadIdx.x == 0) {
        key[0] = 0;
        count[0] = pyr[loff[depth]];
        level[0] = (uint8_t)depth;
        s_next = 1;
        level_start[depth] = 0;
    }
    __syncthreads();
    uint32_t cur_begin = 0, cur_end = 1;
    for (int l = (int)depth; l >= 1; --l) {
        for (uint32_t base = cur_begin; base < cur_end; base += blockDim.x) {
            uint32_t i = base + threadIdx.x;
            uint32_t mask = 0;
            bool internal = false;
            uint32_t k = 0;
            if (i < cur_end) {
                k = key[i];
                internal = count[i] >= threshold;
                if (internal) {
                    const uint4* c = reinterpret_cast<const uint4*>(pyr + loff[l - 1] + (uint64_t)k * 8);
                    uint4 a = c[0], b = c[1];
                    mask = (a.x != 0) | ((a.y != 0) << 1) | ((a.z != 0) << 2) | ((a.w != 0) << 3) | ((b.x != 0) << 4) |
                           ((b.y != 0) << 5) | ((b.z != 0) << 6) | ((b.w != 0) << 7);
                }
            }
            uint32_t total;
            uint32_t off = block_exclusive_scan(__popc(mask), warp_sums, total);
            uint32_t next = s_next;
            if (i < cur_end) {
                info[i] = (uint16_t)((internal ? 1u : 0u) | (mask << 1));
                child_first[i] = internal ? next + off : 0xFFFFFFFFu;
                if (internal) {
                    const uint32_t* c = pyr + loff[l - 1] + (uint64_t)k * 8;
                    uint32_t j = next + off;
                    for (uint32_t s = 0; s < 8; ++s) {
                        if (!(mask & (1u << s))) continue;
                        if (j < cap) {
                            key[j] = k * 8 + s;
                            count[j] = c[s];
                            level[j] = (uint8_t)(l - 1);
                        }
                        ++j;
                    }
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                s_next = next + total;
                if (s_next > cap) set_error(err, kErrNodeCap);
            }
            __syncthreads();
            if (s_next > cap) return;
        }
        cur_begin = cur_end;
        cur_end = s_next;
        if (threadIdx.x == 0) level_start[l - 1] = cur_begin;
    }
    // level-0 nodes are leaves
    for (uint32_t i = cur_begin + threadIdx.x; i < cur_end; i += blockDim.x) {
        info[i] = 0;
        child_first[i] = 0xFFFFFFFFu;
    }
    if (threadIdx.x == 0) {
        *n_nodes = cur_end;
        level_start[depth + 1] = cur_end;
    }
}

// Leaf data offsets and leaf tags from the node table, without the host: one
// block scans the nodes in BFS order.  Leaf i gets data_idx = the points of
// the leaves before it (hierarchy BFS order), its pyramid cell the tag
// kLeafTag | i, and its fill counter 0.  Skipped when the node table
// overflowed; flags kErrTag when the leaves do not hold all n_points.
__global__ void __launch_bounds__(1024) k_leaf_prep(const uint32_t* __restrict__ n_nodes_p,
                                                    const uint16_t* __restrict__ info, const uint32_t* __restrict__ count,
                                                    const uint8_t* __restrict__ level, const uint32_t* __restrict__ key,
                                                    uint32_t* pyr, const uint64_t* __restrict__ loff, uint64_t* data_idx,
                                                    uint32_t* fill, uint64_t n_points, uint32_t* err) {
    __shared__ uint64_t warp_sums[32];
    if (*err & kErrNodeCap) return;
    const uint32_t n = *n_nodes_p;
    uint64_t running = 0;
    for (uint32_t k0 = 0; k0 < n; k0 += blockDim.x) {
        const uint32_t i = k0 + threadIdx.x;
        const bool leaf = i < n && !(info[i] & 1);
        const uint64_t c = leaf ? count[i] : 0;
        uint64_t tot;
        const uint64_t pre = block_exclusive_scan64(c, warp_sums, tot);
        if (i < n) {
            fill[i] = 0;
            data_idx[i] = leaf ? running + pre : 0;
            if (leaf) pyr[loff[level[i]] + key[i]] = kLeafTag | i;
        }
        running += tot;
    }
    if (threadIdx.x == 0 && running != n_points) set_error(err, kErrTag);
}

// Writes the leaf tag of every occupied finest cell into the cell: one
// thread per level-1 cell reads its 8 children and, when some of them are
// occupied and untagged, the nearest tagged ancestor.
__global__ void k_push_tags(uint32_t* __restrict__ pyr, const uint64_t* __restrict__ loff, uint32_t depth, uint64_t n1,
                            const uint8_t* __restrict__ occ, uint32_t* err) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n1) return;
    if (occ && occ[i >> 3] == 0) return;   // no point in this 64-cell block
    uint4* c = reinterpret_cast<uint4*>(pyr + i * 8);
    uint4 a = c[0], b = c[1];
    uint32_t v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    bool need = false;
#pragma unroll
    for (int s = 0; s < 8; ++s) need |= v[s] != 0 && !(v[s] & kLeafTag);
    if (!need) return;
    uint32_t tag = 0;
    uint64_t k = i;
    for (uint32_t l = 1; l <= depth; ++l, k >>= 3) {
        const uint32_t w = pyr[loff[l] + k];
        if (w & kLeafTag) {
            tag = w;
            break;
        }
    }
    if (!tag) {
        set_error(err, kErrTag);
        return;
    }
#pragma unroll
    for (int s = 0; s < 8; ++s)
        if (v[s] != 0 && !(v[s] & kLeafTag)) v[s] = tag;
    c[0] = make_uint4(v[0], v[1], v[2], v[3]);
    c[1] = make_uint4(v[4], v[5], v[6], v[7]);
}

// K5 (point_distributing.cuh:30-75): every point goes to its leaf's bucket
// with its LUT entry and 18-byte output record.  The first lane of each run
// of equal cells reads the cell's leaf tag; the first lane of each run of
// equal leaves reserves the run's slots with one atomic.  At most 40
// registers, so that three 448-thread blocks share an SM (47 registers leave
// room for two: 119.7M-point build 2.73 -> 2.56 ms).
template <bool kF32>
__global__ void __launch_bounds__(kDistThreads, 3) k_distribute(const uint8_t* __restrict__ cloud, uint64_t n,
                                                              uint32_t stride, CloudGrid g, OutParams op,
                                                              const uint32_t* __restrict__ pyr0,
                                                              const uint64_t* __restrict__ data_idx, uint32_t* fill,
                                                              uint32_t* __restrict__ lut, uint8_t* __restrict__ rec,
                                                              uint32_t* __restrict__ frac, uint32_t* err) {
    extern __shared__ __align__(128) uint8_t smem[];
    const ChunkSmem L = chunk_smem(stride, g.grid, kF32, kDistTile);
    load_tables<kF32>(g, smem, L);
    const uint32_t lane = threadIdx.x & 31;
    tile_loop<kDistTile>(cloud, n, stride, smem, L, err, [&](const uint8_t* recs, uint64_t p0, uint32_t cnt) {
#pragma unroll 1
        for (uint32_t base = 0; base < kDistTile; base += kDistThreads) {
            const uint32_t k = base + threadIdx.x;
            constexpr int kWords = kF32 ? 4 : 7;
            uint32_t w[kWords];
            uint32_t m = kNoKey;
            if (k < cnt) {
                record_words<kWords>(recs + (uint64_t)k * stride, w);
                int cell[3];
                if (point_cells<kF32>(w, g, smem, L, cell)) m = cell_morton(cell, smem, L);
                else set_error(err, kErrBelowBox);
            }
            uint32_t starts = run_starts(m);
            uint32_t leader = run_leader(starts);
            uint32_t tag = (m != kNoKey && lane == leader) ? pyr0[m] : 0u;
            tag = __shfl_sync(0xffffffffu, tag, leader);
            uint32_t node = kNoKey;
            if (m != kNoKey) {
                if (tag & kLeafTag) node = tag & ~kLeafTag;
                else set_error(err, kErrTag);
            }
            starts = run_starts(node);
            leader = run_leader(starts);
            uint64_t first = 0;
            if (node != kNoKey && lane == leader) first = data_idx[node] + atomicAdd(&fill[node], run_end(starts) - lane);
            first = ((uint64_t)__shfl_sync(0xffffffffu, (uint32_t)(first >> 32), leader) << 32) |
                    __shfl_sync(0xffffffffu, (uint32_t)first, leader);
            uint32_t nw[5] = {0, 0, 0, 0, 0};
            bool ok = false;
            if (node != kNoKey) {
                const uint64_t pos = first + (lane - leader);
                if (pos >= n) {   // only reachable with corrupted input tags
                    set_error(err, kErrTag);
                } else {
                    ok = true;
                    lut[pos] = (uint32_t)(p0 + k);
                    Coord c[3];
                    uint32_t col;
                    if (kF32) {
                        for (int a = 0; a < 3; ++a) c[a] = coord_f32(__uint_as_float(w[a]));
                        col = w[3];
                    } else {
                        for (int a = 0; a < 3; ++a)
                            c[a] = coord_f64(__hiloint2double((int)w[2 * a + 1], (int)w[2 * a]));
                        col = w[6];
                    }
                    uint32_t fx, fy, fz;
                    const int32_t x = out_coord_frac<kF32>(c[0], op.ax[0], fx);
                    const int32_t y = out_coord_frac<kF32>(c[1], op.ax[1], fy);
                    const int32_t z = out_coord_frac<kF32>(c[2], op.ax[2], fz);
                    if (x == kCoordError || y == kCoordError || z == kCoordError) set_error(err, kErrCoordRange);
                    if (frac) frac[pos] = pack_frac(fx, fy, fz);
                    nw[0] = (uint32_t)x;
                    nw[1] = (uint32_t)y;
                    nw[2] = (uint32_t)z;
                    nw[3] = (col & 0xFFu) | (((col >> 8) & 0xFFu) << 16);
                    nw[4] = (col >> 16) & 0xFFu;
                }
            }
            // each lane stores its own record with five stores (staging the
            // runs of a leaf through shared memory for coalesced stores was
            // slower: 119.7M-point build 3.00 -> 2.73 ms, 25.8M-point random
            // planes 2.25 -> 1.32 ms)
            if (ok) store_record_words(rec, first + (lane - leader), nw);
        }
    });
}

// Copies byte range [src, src + bytes) to dst.  Both addresses are even (18-byte
// records); the body is written as aligned 16-byte stores assembled from
// 4-byte loads, realigned by a 16-bit funnel shift when needed.
__device__ __forceinline__ void copy_bytes_even(uint8_t* __restrict__ dst, const uint8_t* __restrict__ src,
                                                uint64_t bytes) {
    uintptr_t d0 = reinterpret_cast<uintptr_t>(dst), d1 = d0 + bytes;
    uintptr_t a0 = (d0 + 15) & ~(uintptr_t)15, a1 = d1 & ~(uintptr_t)15;
    const intptr_t delta = reinterpret_cast<intptr_t>(src) - (intptr_t)d0;
    if (a0 >= a1) {   // short range: 2-byte copies
        for (uintptr_t p = d0 + 2 * threadIdx.x; p < d1; p += 2 * blockDim.x)
            *reinterpret_cast<uint16_t*>(p) = *reinterpret_cast<const uint16_t*>(p + delta);
        return;
    }
    for (uintptr_t p = d0 + 2 * threadIdx.x; p < a0; p += 2 * blockDim.x)
        *reinterpret_cast<uint16_t*>(p) = *reinterpret_cast<const uint16_t*>(p + delta);
    for (uintptr_t p = a1 + 2 * threadIdx.x; p < d1; p += 2 * blockDim.x)
        *reinterpret_cast<uint16_t*>(p) = *reinterpret_cast<const uint16_t*>(p + delta);
    const uint64_t chunks = (a1 - a0) >> 4;
    for (uint64_t i = threadIdx.x; i < chunks; i += blockDim.x) {
        uintptr_t dp = a0 + i * 16, sp = dp + delta;
        const uint32_t* w = reinterpret_cast<const uint32_t*>(sp & ~(uintptr_t)3);
        uint4 o;
        if (sp & 2) {
            uint32_t w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3], w4 = w[4];
            o.x = __funnelshift_r(w0, w1, 16);
            o.y = __funnelshift_r(w1, w2, 16);
            o.z = __funnelshift_r(w2, w3, 16);
            o.w = __funnelshift_r(w3, w4, 16);
        } else {
            o.x = w[0];
            o.y = w[1];
            o.z = w[2];
            o.w = w[3];
        }
        *reinterpret_cast<uint4*>(dp) = o;
    }
}

__global__ void k_place(const uint64_t* __restrict__ src_off, const uint64_t* __restrict__ dst_off,
                        const uint32_t* __restrict__ count, uint32_t n_nodes, const uint8_t* __restrict__ stage_rec,
                        uint8_t* __restrict__ rec) {
    for (uint32_t v = blockIdx.x; v < n_nodes; v += gridDim.x)
        copy_bytes_even(rec + dst_off[v] * 18, stage_rec + src_off[v] * 18, (uint64_t)count[v] * 18);
}

// Output positions of the internal nodes: DFS post-order after the N leaf
// points (calculateWritingPosition, kernel_helpers.cuh:55-59).  One block
// scans the nodes' point counts in post-order (post[] lists internal indices)
// and writes the copy list of k_place; nothing is copied when an earlier stage
// reported a capacity error or the records exceed `cap`.
__global__ void __launch_bounds__(1024) k_place_prepare(const uint32_t* __restrict__ post, uint32_t n_internal,
                                                        const uint32_t* __restrict__ points,
                                                        const uint64_t* __restrict__ stage_off, uint64_t n,
                                                        uint64_t cap, uint64_t* src, uint64_t* dst, uint32_t* cnt,
                                                        uint64_t* node_dst, uint64_t* total, uint32_t* err) {
    __shared__ uint64_t warp_sums[32];
    const bool skip = (*err & kErrCapacity) != 0;
    uint64_t running = 0;
    for (uint32_t k0 = 0; k0 < n_internal; k0 += blockDim.x) {
        const uint32_t k = k0 + threadIdx.x;
        const uint32_t ii = k < n_internal ? post[k] : 0;
        const uint64_t p = (k < n_internal && !skip) ? points[ii] : 0;
        uint64_t sum;
        const uint64_t pre = block_exclusive_scan64(p, warp_sums, sum);
        if (k < n_internal) {
            const uint64_t d = n + running + pre;
            src[k] = skip ? 0 : stage_off[ii];
            dst[k] = d;
            cnt[k] = (uint32_t)p;
            node_dst[ii] = d;
        }
        running += sum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *total = running;
        if (!skip && n + running > cap) atomicOr(err, kErrCapacity);
    }
    if (!skip && n + running > cap)   // nothing may be written past the record arrays
        for (uint32_t k = threadIdx.x; k < n_internal; k += blockDim.x) cnt[k] = 0;
}

__global__ void k_place_lut(const uint64_t* __restrict__ src_off, const uint64_t* __restrict__ dst_off,
                            const uint32_t* __restrict__ count, uint32_t n_nodes,
                            const uint32_t* __restrict__ stage_lut, uint32_t* __restrict__ lut) {
    for (uint32_t v = blockIdx.x; v < n_nodes; v += gridDim.x) {
        uint64_t s = src_off[v], d = dst_off[v];
        uint32_t c = count[v];
        for (uint32_t i = threadIdx.x; i < c; i += blockDim.x) lut[d + i] = stage_lut[s + i];
    }
}

}   // namespace

void allow_dynamic_smem(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> limit;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(mu);
    size_t& cur = limit[{dev, kernel}];
    if (bytes <= cur) return;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess) cur = bytes;
    else cudaGetLastError();   // the launch reports the error
}

template <class Kernel>
static int chunk_grid_size(Kernel kernel, uint32_t threads, uint32_t tile, size_t smem, uint64_t n, int num_sms) {
    allow_dynamic_smem(reinterpret_cast<const void*>(kernel), smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const uint64_t tiles = (n + tile - 1) / tile;
    return (int)std::min<uint64_t>(tiles, (uint64_t)num_sms * per_sm);
}

int launch_count(const uint8_t* cloud, uint64_t n, uint32_t stride, bool float_input, const CloudGrid& g,
                  uint32_t* pyr0, uint8_t* occ, uint32_t* err, int num_sms, cudaStream_t stream) {
    if (n == 0) return 0;
    const size_t smem = chunk_smem(stride, g.grid, float_input, kCountTile).total;
    if (float_input) {
        const int grid = chunk_grid_size(k_count<true>, kCountThreads, kCountTile, smem, n, num_sms);
        k_count<true><<<grid, kCountThreads, smem, stream>>>(cloud, n, stride, g, pyr0, occ, err);
    } else {
        const int grid = chunk_grid_size(k_count<false>, kCountThreads, kCountTile, smem, n, num_sms);
        k_count<false><<<grid, kCountThreads, smem, stream>>>(cloud, n, stride, g, pyr0, occ, err);
    }
    return 1;
}

// Zeroes the 64-cell blocks of the finest level flagged in `occ`, and the
// flags: one thread per block.
__global__ void k_sparse_zero(uint32_t* __restrict__ pyr0, uint8_t* __restrict__ occ, uint64_t blocks) {
    const uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (b >= blocks || !occ[b]) return;
    uint4* d = reinterpret_cast<uint4*>(pyr0 + b * 64);
#pragma unroll
    for (int k = 0; k < 16; ++k) d[k] = make_uint4(0, 0, 0, 0);
    occ[b] = 0;
}

int launch_sparse_zero(uint32_t* pyr0, uint8_t* occ, uint64_t blocks, cudaStream_t stream) {
    if (!blocks) return 0;
    k_sparse_zero<<<(unsigned)((blocks + 255) / 256), 256, 0, stream>>>(pyr0, occ, blocks);
    return 1;
}

int launch_pyramid(uint32_t* pyr, const uint64_t* loff, uint32_t depth, uint32_t* nonzero, const uint8_t* occ,
                   cudaStream_t stream) {
    uint32_t l = 0;
    int launches = 1;
    while (l < depth) {
        ++launches;
        if (l + 2 <= depth) {
            uint64_t n2 = loff[l + 3 <= depth + 1 ? l + 3 : depth + 1] - loff[l + 2];
            n2 = 0;
            // number of level-(l+2) cells = (G0 >> (l+2))^3 = size of that level
            n2 = loff[l + 3] - loff[l + 2];
            int threads = 256;
            uint64_t blocks = (n2 + threads - 1) / threads;
            k_pyramid2<<<(unsigned)blocks, threads, 0, stream>>>(pyr + loff[l], pyr + loff[l + 1], pyr + loff[l + 2],
                                                                 n2, nonzero + l, nonzero + l + 1,
                                                                 l == 0 ? occ : nullptr);
            l += 2;
        } else {
            uint64_t n1 = loff[l + 2] - loff[l + 1];
            int threads = 256;
            uint64_t blocks = (n1 + threads - 1) / threads;
            k_pyramid1<<<(unsigned)blocks, threads, 0, stream>>>(pyr + loff[l], pyr + loff[l + 1], n1, nonzero + l);
            l += 1;
        }
    }
    k_count_root<<<1, 32, 0, stream>>>(pyr + loff[depth], nonzero + depth);
    return launches;
}

int launch_enumerate(const uint32_t* pyr, const uint64_t* loff_dev, uint32_t depth, uint32_t threshold, uint32_t* key,
                      uint32_t* count, uint8_t* level, uint16_t* info, uint32_t* child_first, uint32_t cap,
                      uint32_t* level_start, uint32_t* n_nodes, uint32_t* err, cudaStream_t stream) {
    k_enumerate<<<1, 1024, 0, stream>>>(pyr, loff_dev, depth, threshold, key, count, level, info, child_first, cap,
                                        level_start, n_nodes, err);
    return 1;
}

int launch_bbox(const uint8_t* cloud, uint64_t n, uint32_t stride, bool float_input, long long* keys, int num_sms,
                cudaStream_t stream) {
    k_bbox_init<<<1, 32, 0, stream>>>(keys);
    const uint64_t want = (n + 255) / 256;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)num_sms * 8));
    if (float_input) k_bbox<true><<<grid, 256, 0, stream>>>(cloud, n, stride, keys);
    else k_bbox<false><<<grid, 256, 0, stream>>>(cloud, n, stride, keys);
    return 2;
}

int launch_leaf_prep(const uint32_t* n_nodes, const uint16_t* info, const uint32_t* count, const uint8_t* level,
                     const uint32_t* key, uint32_t* pyr, const uint64_t* loff_dev, uint64_t* data_idx, uint32_t* fill,
                     uint64_t n_points, uint32_t* err, cudaStream_t stream) {
    k_leaf_prep<<<1, 1024, 0, stream>>>(n_nodes, info, count, level, key, pyr, loff_dev, data_idx, fill, n_points, err);
    return 1;
}

int launch_push_tags(uint32_t* pyr, const uint64_t* loff_dev, uint32_t depth, uint32_t grid, const uint8_t* occ,
                     uint32_t* err, cudaStream_t stream) {
    const uint64_t n1 = (uint64_t)(grid / 2) * (grid / 2) * (grid / 2);
    if (!n1) return 0;
    k_push_tags<<<(unsigned)((n1 + 255) / 256), 256, 0, stream>>>(pyr, loff_dev, depth, n1, occ, err);
    return 1;
}

int launch_distribute(const uint8_t* cloud, uint64_t n, uint32_t stride, bool float_input, const CloudGrid& g,
                      const OutParams& out, const uint32_t* pyr0, const uint64_t* data_idx, uint32_t* fill,
                      uint32_t* lut, uint8_t* rec, uint32_t* frac, uint32_t* err, int num_sms,
                      cudaStream_t stream) {
    if (n == 0) return 0;
    const size_t smem = chunk_smem(stride, g.grid, float_input, kDistTile).total;
    if (float_input) {
        const int grid = chunk_grid_size(k_distribute<true>, kDistThreads, kDistTile, smem, n, num_sms);
        k_distribute<true><<<grid, kDistThreads, smem, stream>>>(cloud, n, stride, g, out, pyr0, data_idx, fill, lut,
                                                                  rec, frac, err);
    } else {
        const int grid = chunk_grid_size(k_distribute<false>, kDistThreads, kDistTile, smem, n, num_sms);
        k_distribute<false><<<grid, kDistThreads, smem, stream>>>(cloud, n, stride, g, out, pyr0, data_idx, fill,
                                                                   lut, rec, frac, err);
    }
    return 1;
}

int launch_place(const uint64_t* src_off, const uint64_t* dst_off, const uint32_t* count, uint32_t n_nodes,
                 const uint8_t* stage_rec, uint8_t* rec, cudaStream_t stream) {
    if (!n_nodes) return 0;
    unsigned grid = n_nodes < 8192 ? n_nodes : 8192;
    k_place<<<grid, 256, 0, stream>>>(src_off, dst_off, count, n_nodes, stage_rec, rec);
    return 1;
}

int launch_place_prepare(const uint32_t* post, uint32_t n_internal, const uint32_t* points, const uint64_t* stage_off,
                         uint64_t n, uint64_t cap, uint64_t* src, uint64_t* dst, uint32_t* cnt, uint64_t* node_dst,
                         uint64_t* total, uint32_t* err, cudaStream_t stream) {
    k_place_prepare<<<1, 1024, 0, stream>>>(post, n_internal, points, stage_off, n, cap, src, dst, cnt, node_dst, total,
                                            err);
    return 1;
}

int launch_place_lut(const uint64_t* src_off, const uint64_t* dst_off, const uint32_t* count, uint32_t n_nodes,
                     const uint32_t* stage_lut, uint32_t* lut, cudaStream_t stream) {
    if (!n_nodes) return 0;
    unsigned grid = n_nodes < 8192 ? n_nodes : 8192;
    k_place_lut<<<grid, 256, 0, stream>>>(src_off, dst_off, count, n_nodes, stage_lut, lut);
    return 1;
}

}   // namespace oc
