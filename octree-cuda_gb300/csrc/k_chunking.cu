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
#include <cstdint>

#include "device_common.cuh"
#include "kernels.h"

namespace oc {

namespace {

constexpr int kTilePoints = 2048;
constexpr int kTileThreads = 512;
constexpr uint32_t kLeafTag = 0x80000000u;

__device__ __forceinline__ void set_error(uint32_t* err, uint32_t bit) {
    atomicOr(err, bit);
}

// Copies the byte span of `cnt` records starting at record p0 into shared
// memory with 16-byte vector loads; returns the offset of record p0 in smem.
// The cloud buffer is padded so that rounding the span up to 16 bytes stays
// inside the allocation.
__device__ __forceinline__ uint32_t stage_tile(const uint8_t* __restrict__ cloud, uint64_t p0, uint32_t cnt,
                                               uint32_t stride, uint4* smem) {
    uint64_t b0 = p0 * stride, b1 = (p0 + cnt) * stride;
    uint64_t a0 = b0 & ~15ull, a1 = (b1 + 15) & ~15ull;
    uint32_t nvec = (uint32_t)((a1 - a0) >> 4);
    const uint4* src = reinterpret_cast<const uint4*>(cloud + a0);
    for (uint32_t v = threadIdx.x; v < nvec; v += blockDim.x) smem[v] = __ldg(src + v);
    return (uint32_t)(b0 - a0);
}

template <bool kF32>
__device__ __forceinline__ uint32_t point_cell(const uint8_t* rec, const CloudGrid& g, Coord c[3], uint32_t col[3],
                                               bool& below) {
    load_point<kF32>(rec, c, col);
    float u;
    int ix = axis_cell<kF32>(c[0], g.ax[0], g.grid, u);
    int iy = axis_cell<kF32>(c[1], g.ax[1], g.grid, u);
    int iz = axis_cell<kF32>(c[2], g.ax[2], g.grid, u);
    below = (ix | iy | iz) < 0;
    return below ? 0u : morton3((uint32_t)ix, (uint32_t)iy, (uint32_t)iz);
}

template <bool kF32>
__global__ void __launch_bounds__(kTileThreads) k_count(const uint8_t* __restrict__ cloud, uint64_t n, uint32_t stride,
                                                        CloudGrid g, uint32_t* __restrict__ pyr0, uint32_t* err) {
    extern __shared__ uint4 smem[];
    const uint8_t* buf = reinterpret_cast<const uint8_t*>(smem);
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t tile = blockIdx.x; tile * kTilePoints < n; tile += gridDim.x) {
        uint64_t p0 = tile * kTilePoints;
        uint32_t cnt = (uint32_t)((n - p0) < (uint64_t)kTilePoints ? (n - p0) : (uint64_t)kTilePoints);
        uint32_t shift = stage_tile(cloud, p0, cnt, stride, smem);
        __syncthreads();
        for (uint32_t base = 0; base < cnt; base += blockDim.x) {
            uint32_t k = base + threadIdx.x;
            bool valid = k < cnt;
            uint32_t m = 0;
            if (valid) {
                Coord c[3];
                uint32_t col[3];
                bool below;
                m = point_cell<kF32>(buf + shift + (uint64_t)k * stride, g, c, col, below);
                if (below) {
                    set_error(err, kErrBelowBox);
                    valid = false;
                }
            }
            unsigned active = __ballot_sync(0xffffffffu, valid);
            if (valid) {
                unsigned peers = __match_any_sync(active, m);
                if ((int)lane == __ffs(peers) - 1) atomicAdd(&pyr0[m], (uint32_t)__popc(peers));
            }
        }
        __syncthreads();
    }
}

// Level l -> levels l+1 and l+2: one thread per level-(l+2) cell reads its 64
// Morton-contiguous level-l counts.
__global__ void k_pyramid2(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst1, uint32_t* __restrict__ dst2,
                           uint64_t n2, uint32_t* nz_src, uint32_t* nz_dst1) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint32_t nzs = 0, nzd = 0;
    if (i < n2) {
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
                if (s_next > cap) set_error(err, kErrCapacity);
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

__global__ void k_tag_leaves(uint32_t* pyr, const uint64_t* __restrict__ loff, const uint32_t* __restrict__ leaves,
                             uint32_t n_leaves, const uint32_t* __restrict__ key, const uint8_t* __restrict__ level) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_leaves) return;
    uint32_t node = leaves[i];
    pyr[loff[level[node]] + key[node]] = kLeafTag | node;
}

template <bool kF32>
__global__ void __launch_bounds__(kTileThreads) k_distribute(const uint8_t* __restrict__ cloud, uint64_t n,
                                                             uint32_t stride, CloudGrid g, OutParams op,
                                                             const uint32_t* __restrict__ pyr,
                                                             const uint64_t* __restrict__ loff, uint32_t depth,
                                                             const uint64_t* __restrict__ data_idx, uint32_t* fill,
                                                             uint32_t* __restrict__ lut, uint8_t* __restrict__ rec,
                                                             uint32_t* err) {
    extern __shared__ uint4 smem[];
    const uint8_t* buf = reinterpret_cast<const uint8_t*>(smem);
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t tile = blockIdx.x; tile * kTilePoints < n; tile += gridDim.x) {
        uint64_t p0 = tile * kTilePoints;
        uint32_t cnt = (uint32_t)((n - p0) < (uint64_t)kTilePoints ? (n - p0) : (uint64_t)kTilePoints);
        uint32_t shift = stage_tile(cloud, p0, cnt, stride, smem);
        __syncthreads();
        for (uint32_t base = 0; base < cnt; base += blockDim.x) {
            uint32_t k = base + threadIdx.x;
            bool valid = k < cnt;
            Coord c[3];
            uint32_t col[3];
            uint32_t node = 0;
            if (valid) {
                bool below;
                uint32_t m = point_cell<kF32>(buf + shift + (uint64_t)k * stride, g, c, col, below);
                if (below) {
                    set_error(err, kErrBelowBox);
                    valid = false;
                } else {
                    uint32_t v = pyr[m];
                    uint32_t l = 0;
                    while (!(v & kLeafTag)) {
                        if (++l > depth) break;
                        m >>= 3;
                        v = pyr[loff[l] + m];
                    }
                    if (!(v & kLeafTag)) {
                        set_error(err, kErrTag);
                        valid = false;
                    } else {
                        node = v & ~kLeafTag;
                    }
                }
            }
            unsigned active = __ballot_sync(0xffffffffu, valid);
            if (valid) {
                unsigned peers = __match_any_sync(active, node);
                int leader = __ffs(peers) - 1;
                uint32_t slot0 = 0;
                if ((int)lane == leader) slot0 = atomicAdd(&fill[node], (uint32_t)__popc(peers));
                slot0 = __shfl_sync(peers, slot0, leader);
                uint32_t slot = slot0 + __popc(peers & ((1u << lane) - 1));
                uint64_t pos = data_idx[node] + slot;
                lut[pos] = (uint32_t)(p0 + k);
                int32_t x = out_coord<kF32>(c[0], op.ax[0]);
                int32_t y = out_coord<kF32>(c[1], op.ax[1]);
                int32_t z = out_coord<kF32>(c[2], op.ax[2]);
                if (x == kCoordError || y == kCoordError || z == kCoordError) set_error(err, kErrCoordRange);
                store_record(rec, pos, x, y, z, (uint16_t)col[0], (uint16_t)col[1], (uint16_t)col[2]);
            }
        }
        __syncthreads();
    }
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

static size_t tile_smem(uint32_t stride) {
    return (size_t)kTilePoints * stride + 64;
}

int launch_count(const uint8_t* cloud, uint64_t n, uint32_t stride, bool float_input, const CloudGrid& g,
                  uint32_t* pyr0, uint32_t* err, int num_sms, cudaStream_t stream) {
    size_t smem = tile_smem(stride);
    uint64_t tiles = (n + kTilePoints - 1) / kTilePoints;
    int grid = (int)std::min<uint64_t>(tiles, (uint64_t)num_sms * 4);
    if (grid == 0) return 0;
    if (float_input) {
        cudaFuncSetAttribute(k_count<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_count<true><<<grid, kTileThreads, smem, stream>>>(cloud, n, stride, g, pyr0, err);
    } else {
        cudaFuncSetAttribute(k_count<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_count<false><<<grid, kTileThreads, smem, stream>>>(cloud, n, stride, g, pyr0, err);
    }
    return 1;
}

int launch_pyramid(uint32_t* pyr, const uint64_t* loff, uint32_t depth, uint32_t* nonzero, cudaStream_t stream) {
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
                                                                 n2, nonzero + l, nonzero + l + 1);
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

int launch_tag_leaves(uint32_t* pyr, const uint64_t* loff_dev, const uint32_t* leaves, uint32_t n_leaves,
                       const uint32_t* key, const uint8_t* level, cudaStream_t stream) {
    if (!n_leaves) return 0;
    k_tag_leaves<<<(n_leaves + 255) / 256, 256, 0, stream>>>(pyr, loff_dev, leaves, n_leaves, key, level);
    return 1;
}

int launch_distribute(const uint8_t* cloud, uint64_t n, uint32_t stride, bool float_input, const CloudGrid& g,
                       const OutParams& out, const uint32_t* pyr, const uint64_t* loff_dev, uint32_t depth,
                       const uint64_t* data_idx, uint32_t* fill, uint32_t* lut, uint8_t* rec, uint32_t* err,
                       int num_sms, cudaStream_t stream) {
    size_t smem = tile_smem(stride);
    uint64_t tiles = (n + kTilePoints - 1) / kTilePoints;
    int grid = (int)std::min<uint64_t>(tiles, (uint64_t)num_sms * 4);
    if (grid == 0) return 0;
    if (float_input) {
        cudaFuncSetAttribute(k_distribute<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_distribute<true><<<grid, kTileThreads, smem, stream>>>(cloud, n, stride, g, out, pyr, loff_dev, depth,
                                                                 data_idx, fill, lut, rec, err);
    } else {
        cudaFuncSetAttribute(k_distribute<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_distribute<false><<<grid, kTileThreads, smem, stream>>>(cloud, n, stride, g, out, pyr, loff_dev, depth,
                                                                  data_idx, fill, lut, rec, err);
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

int launch_place_lut(const uint64_t* src_off, const uint64_t* dst_off, const uint32_t* count, uint32_t n_nodes,
                     const uint32_t* stage_lut, uint32_t* lut, cudaStream_t stream) {
    if (!n_nodes) return 0;
    unsigned grid = n_nodes < 8192 ? n_nodes : 8192;
    k_place_lut<<<grid, 256, 0, stream>>>(src_off, dst_off, count, n_nodes, stage_lut, lut);
    return 1;
}

}   // namespace oc
