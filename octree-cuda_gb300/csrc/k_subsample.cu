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
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <utility>

#include "device_common.cuh"
#include "kernels.h"

namespace oc {

namespace {

#ifndef OC_SUB_THREADS
#define OC_SUB_THREADS 1024
#endif
constexpr int kSubThreads = OC_SUB_THREADS;
constexpr uint32_t kBrickSlots = kSharedBrickSlots;   // shared-memory brick table capacity
constexpr uint32_t kBrickShift = 32 - 13;

struct BrickMap {
    uint32_t* key;    // brick id + 1, 0 = empty
    uint64_t* mask;   // occupied cells of the brick (bit = x | y<<2 | z<<4)
    uint32_t* base;   // rank of the brick's first cell
    uint32_t cap;     // slots (power of two, multiple of the block size)
    uint32_t shift;   // 32 - log2(cap)
    uint32_t bs;      // bricks per axis (<= 256): brick id = bx | by << 8 | bz << 16
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

// Cell index of one axis from the candidate's quantised coordinate q, or -2
// when the interval of positions q stands for straddles a cell boundary (the
// binary64 path then decides).  The interval [lo - e, lo + B + e] holds the
// reference's cell-unit value: e bounds the fp32 rounding of lo and of the
// host-rounded constants (a few ulp of |lo| + |base| + B) with a wide margin.
__device__ __forceinline__ int quant_cell(int32_t q, const QAxis& a, uint32_t G) {
    const int32_t dq = q - a.qn;
    if (dq > (1 << 22) || dq < -(1 << 22)) return -2;
    const float lo = __fmaf_rn((float)dq, a.B, a.base);
    const float e =
        __fmul_rn(__fadd_rn(__fadd_rn(fabsf(lo), fabsf(a.base)), __fadd_rn(a.B, 4.0f)), 9.5367431640625e-07f);
    const int i0 = idx_from_units(__fsub_rn(lo, e), G);
    const int i1 = idx_from_units(__fadd_rn(__fadd_rn(lo, a.B), e), G);
    return (i0 == i1 && i0 >= 0) ? i0 : -2;
}

// As quant_cell, for a candidate whose sub-step fraction bin fb (0..1023) is
// known: the true position lies in [(fb - 1/4) / 1024, (fb + 5/4) / 1024] of
// its quantisation step, so the interval is ~1/700 of a step wide and almost
// never straddles a cell boundary.  The fraction terms are exact in fp32; e
// covers the rounding of the two fused multiply-adds as in quant_cell.
__device__ __forceinline__ int quant_cell_fine(int32_t q, uint32_t fb, const QAxis& a, uint32_t G) {
    const int32_t dq = q - a.qn;
    if (dq > (1 << 22) || dq < -(1 << 22)) return -2;
    const float lo = __fmaf_rn((float)dq, a.B, a.base);
    const float fl = __fmul_rn(__fsub_rn((float)fb, 0.25f), 9.765625e-04f);   // (fb - 1/4) / 1024
    const float fh = __fmul_rn(__fadd_rn((float)fb, 1.25f), 9.765625e-04f);   // (fb + 5/4) / 1024
    const float ulo = __fmaf_rn(fl, a.B, lo), uhi = __fmaf_rn(fh, a.B, lo);
    const float e =
        __fmul_rn(__fadd_rn(__fadd_rn(fabsf(lo), fabsf(a.base)), __fadd_rn(a.B, 4.0f)), 9.5367431640625e-07f);
    const int i0 = idx_from_units(__fsub_rn(ulo, e), G);
    const int i1 = idx_from_units(__fadd_rn(uhi, e), G);
    return (i0 == i1 && i0 >= 0) ? i0 : -2;
}

// Position of the k-th set bit (k from 0) of m; k < popcount(m).
__device__ __forceinline__ uint32_t nth_bit64(uint64_t m, uint32_t k) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t w = 32; w >= 1; w >>= 1) {
        const uint64_t low = m & ((1ull << w) - 1ull);
        const uint32_t c = (uint32_t)__popcll(low);
        if (k >= c) {
            k -= c;
            m >>= w;
            pos += w;
        } else {
            m = low;
        }
    }
    return pos;
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

// Visits every occupied cell of the 3x3x3 neighbourhood of the cell at
// brick-local (lx, ly, lz) of brick (bx, by, bz) held in `slot` (the cell
// itself included), calling f(rank, x, y, z) with grid coordinates.
// Only the bricks across the faces that the cell touches are looked up; each
// of the nine x-rows of the neighbourhood is read as a 4-bit slice of a brick
// mask, so ranks are computed for occupied neighbours only.
template <class F>
__device__ __forceinline__ void visit_neighbours(const BrickMap& bm, uint32_t slot, int bx, int by, int bz, int lx,
                                                 int ly, int lz, F& f) {
    const int sx = lx == 0 ? -1 : (lx == 3 ? 1 : 0);
    const int sy = ly == 0 ? -1 : (ly == 3 ? 1 : 0);
    const int sz = lz == 0 ? -1 : (lz == 3 ? 1 : 0);
    auto find = [&](int dx, int dy, int dz) -> int {
        const int nx = bx + dx, ny = by + dy, nz = bz + dz;
        if (nx < 0 || ny < 0 || nz < 0 || nx >= (int)bm.bs || ny >= (int)bm.bs || nz >= (int)bm.bs) return -1;
        return brick_find(bm, ((uint32_t)nx | ((uint32_t)ny << 8) | ((uint32_t)nz << 16)) + 1);
    };
    // slots of the (up to) eight bricks: index bit 0 = x side, 1 = y side, 2 = z side
    const int s0 = (int)slot;
    const int s1 = sx ? find(sx, 0, 0) : -1;
    const int s2 = sy ? find(0, sy, 0) : -1;
    const int s3 = (sx && sy) ? find(sx, sy, 0) : -1;
    const int s4 = sz ? find(0, 0, sz) : -1;
    const int s5 = (sx && sz) ? find(sx, 0, sz) : -1;
    const int s6 = (sy && sz) ? find(0, sy, sz) : -1;
    const int s7 = (sx && sy && sz) ? find(sx, sy, sz) : -1;
    // x window inside the cell's own brick column, and the side brick's edge column
    const uint32_t xlo = (uint32_t)max(lx - 1, 0), xhi = (uint32_t)min(lx + 1, 3);
    const uint32_t own_x = ((2u << xhi) - 1u) & ~((1u << xlo) - 1u);
    const uint32_t side_bit = sx < 0 ? 3u : 0u;
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz) {
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy) {
            const int yy = ly + dy, zz = lz + dz;
            const bool ys = yy < 0 || yy > 3, zs = zz < 0 || zz > 3;
            if ((ys && sy != (dy < 0 ? -1 : 1)) || (zs && sz != (dz < 0 ? -1 : 1))) continue;
            const uint32_t row = (uint32_t)((yy & 3) * 4 + (zz & 3) * 16);
            const int so = zs ? (ys ? s6 : s4) : (ys ? s2 : s0);
            const int ss = zs ? (ys ? s7 : s5) : (ys ? s3 : s1);
            if (so >= 0) {
                const uint64_t m = bm.mask[so];
                uint32_t sel = (uint32_t)(m >> row) & own_x;
                const uint32_t base = bm.base[so];
                while (sel) {
                    const uint32_t x = (uint32_t)__ffs(sel) - 1;
                    sel &= sel - 1;
                    const uint32_t bit = row + x;
                    f(base + (uint32_t)__popcll(m & ((1ull << bit) - 1ull)), bx * 4 + (int)x, by * 4 + yy, bz * 4 + zz);
                }
            }
            if (sx && ss >= 0) {
                const uint64_t m = bm.mask[ss];
                const uint32_t bit = row + side_bit;
                if ((m >> bit) & 1ull)
                    f(bm.base[ss] + (uint32_t)__popcll(m & ((1ull << bit) - 1ull)), (bx + sx) * 4 + (int)side_bit,
                      by * 4 + yy, bz * 4 + zz);
            }
        }
    }
}

// Packed colour sum over the occupied cells of the 3x3x3 neighbourhood of
// the cell at brick-local (lx, ly, lz) of brick (bx, by, bz) held in `slot`
// (the cell itself included).  Every lane evaluates all 27 positions with the
// same instruction stream (selects and predicated loads instead of loops over
// occupied neighbours), so a warp does not diverge on neighbourhood shape.
__device__ __forceinline__ uint64_t inter_sum(const BrickMap& bm, uint32_t slot, int bx, int by, int bz, int lx,
                                              int ly, int lz, const uint64_t* __restrict__ acc) {
    const int sx = lx == 0 ? -1 : (lx == 3 ? 1 : 0);
    const int sy = ly == 0 ? -1 : (ly == 3 ? 1 : 0);
    const int sz = lz == 0 ? -1 : (lz == 3 ? 1 : 0);
    auto find = [&](int dx, int dy, int dz) -> int {
        const int nx = bx + dx, ny = by + dy, nz = bz + dz;
        if (nx < 0 || ny < 0 || nz < 0 || nx >= (int)bm.bs || ny >= (int)bm.bs || nz >= (int)bm.bs) return -1;
        return brick_find(bm, ((uint32_t)nx | ((uint32_t)ny << 8) | ((uint32_t)nz << 16)) + 1);
    };
    // the (up to) eight bricks: index bit 0 = x side, 1 = y side, 2 = z side
    int sl[8];
    sl[0] = (int)slot;
    sl[1] = sx ? find(sx, 0, 0) : -1;
    sl[2] = sy ? find(0, sy, 0) : -1;
    sl[3] = (sx && sy) ? find(sx, sy, 0) : -1;
    sl[4] = sz ? find(0, 0, sz) : -1;
    sl[5] = (sx && sz) ? find(sx, 0, sz) : -1;
    sl[6] = (sy && sz) ? find(0, sy, sz) : -1;
    sl[7] = (sx && sy && sz) ? find(sx, sy, sz) : -1;
    uint64_t e = 0;
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz) {
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy) {
            const int yy = ly + dy, zz = lz + dz;
            // leaving the brick along y or z means the cell sits on that face,
            // so the side brick is the one looked up above
            const int ib = (((unsigned)yy > 3u) ? 2 : 0) | (((unsigned)zz > 3u) ? 4 : 0);
            const int so = sl[ib], ss = sl[ib | 1];
            const uint64_t mo = so >= 0 ? bm.mask[so] : 0ull;
            const uint32_t bo = so >= 0 ? bm.base[so] : 0u;
            const uint64_t ms = ss >= 0 ? bm.mask[ss] : 0ull;
            const uint32_t bsd = ss >= 0 ? bm.base[ss] : 0u;
            const uint32_t row = (uint32_t)((yy & 3) * 4 + (zz & 3) * 16);
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                const int xx = lx + dx;
                const bool side = (unsigned)xx > 3u;
                const uint64_t m = side ? ms : mo;
                const uint32_t bit = row + (uint32_t)(xx & 3);
                const uint32_t rank = (side ? bsd : bo) + (uint32_t)__popcll(m & ((1ull << bit) - 1ull));
                if ((m >> bit) & 1ull) e += __ldcg(acc + rank);   // written by this block's atomics (L2)
            }
        }
    }
    return e;
}

struct WeightedSum {
    const uint32_t* start;
    const uint32_t* count;
    const uint8_t* pts;
    int x, y, z;
    uint64_t sr, sg, sb, sw;
    uint32_t sub, step;   // this lane walks points sub, sub + step, ... of each list
    __device__ __forceinline__ void operator()(uint32_t n, int, int, int) {
        const uint32_t s0 = start[n], s1 = s0 + count[n];
        for (uint32_t p = s0 + sub; p < s1; p += step) {
            const uint32_t* q = reinterpret_cast<const uint32_t*>(pts + (uint64_t)p * 20);
            const uint32_t wq = weight_q(__uint_as_float(q[0]), __uint_as_float(q[1]), __uint_as_float(q[2]), x, y, z);
            sr += (uint64_t)wq * (q[3] & 0xFFFF);
            sg += (uint64_t)wq * (q[3] >> 16);
            sb += (uint64_t)wq * (q[4] & 0xFFFF);
            sw += wq;
        }
    }
};

// The node's children (their records' start, count and kind) and the
// running candidate count before each child.
__device__ __forceinline__ void load_node_shared(NodeShared& ns, const SubNode& nd) {
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

// Distance-weighted emit of one node's cells: warps take runs of 16 cells
// from *next until none is left.  Two lanes per cell, each walking every
// other point of the neighbours' lists; their integer sums are combined by a
// shuffle (any order gives the same sums), so a warp waits for the heaviest
// of 16 cells instead of 32: 25.8M-point build 21.6 -> 20.8 ms (4 lanes per
// cell: 26.7 ms, 8: 37.9 ms).  Every lane of the calling warps calls it.
template <bool kRandom>
__device__ __forceinline__ void emit_weighted(const SubLevelArgs& a, const BrickMap& bm, const NodeShared& ns,
                                              uint64_t off, uint64_t oo, uint32_t cells, uint32_t* next) {
    constexpr uint32_t kWG = 2u;
    const uint32_t lane = threadIdx.x & 31, sub = lane % kWG;
    for (;;) {
        uint32_t r0 = 0;
        if (lane == 0) r0 = atomicAdd(next, 32u / kWG);
        r0 = __shfl_sync(0xffffffffu, r0, 0);
        if (r0 >= cells) break;
        const uint32_t r = r0 + lane / kWG;
        uint32_t nw[5] = {0, 0, 0, 0, 0};
        uint16_t cr = 0, cg = 0, cb = 0;
        uint64_t sr = 0, sg = 0, sb = 0, sw = 0;
        uint32_t idx = 0, csel = 0;
        uint64_t spos = 0;
        if (r < cells) {
            const uint32_t ks = a.cell_slot[off + r];
            const uint32_t slot = ks >> 6, bit = ks & 63;
            const uint32_t brick = bm.key[slot] - 1;
            const int bx = (int)(brick & 0xFF), by = (int)((brick >> 8) & 0xFF), bz = (int)(brick >> 16);
            const int lx = (int)(bit & 3), ly = (int)((bit >> 2) & 3), lz = (int)((bit >> 4) & 3);
            const uint64_t best = a.acc_best[off + r];
            idx = kRandom ? (uint32_t)best : (uint32_t)(best >> 32);
            const uint32_t jsel = kRandom ? a.acc_sel[off + r] : (uint32_t)best;
#pragma unroll
            for (uint32_t c = 1; c < 8; ++c) csel += (c < ns.nchild && ns.prefix[c] <= jsel) ? 1u : 0u;
            spos = ns.start[csel] + (jsel - ns.prefix[csel]);
            const uintptr_t sa =
                reinterpret_cast<uintptr_t>((((ns.kind >> csel) & 1u) ? a.stage_rec : a.leaf_rec) + spos * 18);
            const uint32_t* sq = reinterpret_cast<const uint32_t*>(sa & ~(uintptr_t)3);
            const uint32_t sh = (uint32_t)(sa & 2) * 8;
            const uint32_t q0 = sq[0], q1 = sq[1], q2 = sq[2], q3 = sq[3], q4 = sq[4];
            nw[0] = __funnelshift_r(q0, q1, sh);
            nw[1] = __funnelshift_r(q1, q2, sh);
            nw[2] = __funnelshift_r(q2, q3, sh);
            const uint32_t w3 = __funnelshift_r(q3, q4, sh);
            cr = (uint16_t)w3;
            cg = (uint16_t)(w3 >> 16);
            cb = (uint16_t)(q4 >> sh);
            WeightedSum f{a.csr_start + off, a.csr_count + off, a.csr_pts + off * 20,
                          bx * 4 + lx, by * 4 + ly, bz * 4 + lz, 0, 0, 0, 0, sub, kWG};
            visit_neighbours(bm, slot, bx, by, bz, lx, ly, lz, f);
            sr = f.sr;
            sg = f.sg;
            sb = f.sb;
            sw = f.sw;
        }
#pragma unroll
        for (uint32_t o = kWG / 2; o >= 1; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            sg += __shfl_xor_sync(0xffffffffu, sg, o);
            sb += __shfl_xor_sync(0xffffffffu, sb, o);
            sw += __shfl_xor_sync(0xffffffffu, sw, o);
        }
        if (r < cells && sub == 0) {
            if (sw) {
                cr = (uint16_t)(sr / sw);
                cg = (uint16_t)(sg / sw);
                cb = (uint16_t)(sb / sw);
            }
            a.out_lut[oo + r] = idx;
            if (a.out_frac) {
                const uint32_t* sf = ((ns.kind >> csel) & 1u) ? a.stage_frac : a.leaf_frac;
                a.out_frac[oo + r] = sf ? sf[spos] : 0u;
            }
            nw[3] = (uint32_t)cr | ((uint32_t)cg << 16);
            nw[4] = cb;
            store_record_words(a.out_rec, oo + r, nw);
        }
    }
}

// kColor: 0 raw colour, 1 intra-cell, 2 inter-cell, 3 distance-weighted inter-cell.
// kCluster: a thread-block cluster shares each node (levels with fewer nodes
// than SMs).  The brick map, its counters and the node's cell count live in
// the shared memory of cluster rank 0 and the other blocks reach them through
// distributed shared memory; candidates and cells are split over all blocks
// of the cluster, and cluster barriers separate the phases.
// The level arguments of the build a node belongs to: the launch's own, or
// (a wave over several builds) the node's entry of the table.
template <bool kWave>
__device__ __forceinline__ const SubLevelArgs& node_args(const SubLevelArgs& a0, const WaveNodes& wn, uint32_t ni) {
    if constexpr (kWave) return wn.clouds[wn.cloud_of[ni]];
    else return a0;
}

template <bool kF32, int kColor, bool kRandom, bool kCluster, bool kWave>
__global__ void __launch_bounds__(kSubThreads, 1) k_subsample(SubLevelArgs a0, WaveNodes wn) {
    namespace cg = cooperative_groups;
    extern __shared__ uint64_t dyn[];
    __shared__ NodeShared ns;
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t s_bricks, s_overflow;
    __shared__ uint32_t s_run_total, s_run_off;   // weighted: this block's run of cells in the CSR scan
    __shared__ uint32_t s_skip_node;               // wave: the node's build overflowed a buffer
    __shared__ uint32_t s_emit_next;               // emit: the next run of 32 cells a warp takes
    const uint32_t csize = kCluster ? cg::this_cluster().num_blocks() : 1u;
    const uint32_t crank = kCluster ? cg::this_cluster().block_rank() : 0u;
    const uint32_t tid0 = crank * blockDim.x + threadIdx.x;   // this thread's index within the node's workers
    const uint32_t tstride = csize * blockDim.x;
    auto sync_all = [&]() {
        if constexpr (kCluster) cg::this_cluster().sync();
        else __syncthreads();
    };
    // rank 0's copies (this block's own when not clustered)
    auto owner = [&](auto* p) {
        if constexpr (kCluster) return cg::this_cluster().map_shared_rank(p, 0);
        else return p;
    };
    NodeShared* ns0 = owner(&ns);
    uint32_t* p_bricks = owner(&s_bricks);
    uint32_t* p_overflow = owner(&s_overflow);
    uint64_t* dyn0 = owner(dyn);
    BrickMap sm_map;
    // per-warp staging area of the emitted records, after the brick table
    uint8_t* stage = reinterpret_cast<uint8_t*>(dyn + 2 * kBrickSlots) + (threadIdx.x >> 5) * kStageBytes;
    sm_map.mask = dyn0;
    sm_map.key = reinterpret_cast<uint32_t*>(dyn0 + kBrickSlots);
    sm_map.base = sm_map.key + kBrickSlots;
    sm_map.cap = kBrickSlots;
    sm_map.shift = kBrickShift;
    sm_map.grid = a0.grid;
    sm_map.bs = (a0.grid + 3) >> 2;
    // per-block (per-cluster) brick table in global memory for nodes that outgrow shared memory
    const uint64_t owner_block = blockIdx.x / csize;
    BrickMap gl_map = sm_map;
    gl_map.cap = a0.global_cap;
    gl_map.shift = a0.global_shift;
    gl_map.mask = a0.global_mask + owner_block * a0.global_cap;
    gl_map.key = a0.global_key + owner_block * a0.global_cap;
    gl_map.base = a0.global_base + owner_block * a0.global_cap;

    constexpr bool intra = kColor == 1;
    constexpr bool inter = kColor >= 2;
    constexpr bool weighted = kColor == 3;
    constexpr bool random = kRandom;
    constexpr bool averaged = intra || inter;

    uint32_t* p_skip_node = owner(&s_skip_node);
    uint32_t* p_emit_next = owner(&s_emit_next);
    for (;;) {
        if (crank == 0 && threadIdx.x == 0) {
            const uint32_t k = atomicAdd(a0.work_counter, 1u);
            ns.node = k;
            // a wave skips the nodes of a build whose level did not fit its
            // buffers (that build's pass is repeated on its own)
            if constexpr (kWave) s_skip_node = k < a0.n_nodes && (*node_args<kWave>(a0, wn, k).err & kErrCapacity);
        }
        sync_all();
        const uint32_t ni = ns0->node;
        if (ni >= a0.n_nodes) {
            sync_all();   // rank 0's shared memory stays valid until every block has read it
            break;
        }
        const SubLevelArgs& a = node_args<kWave>(a0, wn, ni);
        const uint32_t li = kWave ? wn.local[ni] : ni;   // the node's index in its build's level
        if constexpr (kWave) {
            const bool skip = *(volatile uint32_t*)p_skip_node != 0;
            sync_all();
            if (skip) continue;
            sm_map.grid = a.grid;
            sm_map.bs = (a.grid + 3) >> 2;
            gl_map.grid = sm_map.grid;
            gl_map.bs = sm_map.bs;
        }
        const SubNode& nd = kWave ? *wn.node[ni] : a.nodes[ni];
        if (threadIdx.x == 0) load_node_shared(ns, nd);
        const AxisGrid ax0 = nd.ax[0], ax1 = nd.ax[1], ax2 = nd.ax[2];
        const QAxis qa0 = nd.qa[0], qa1 = nd.qa[1], qa2 = nd.qa[2];
        const uint64_t off = nd.cand_off;
        const uint64_t oo = nd.out_off;
        const uint32_t level = nd.level;
        const uint64_t morton = nd.morton;
        BrickMap bm = sm_map;
        if (weighted && a.emit_state) {
            // a level that hands its emits over: each node its own global
            // table, which stays intact for k_emit_weighted
            gl_map.mask = a0.global_mask + (uint64_t)li * a0.global_cap;
            gl_map.key = a0.global_key + (uint64_t)li * a0.global_cap;
            gl_map.base = a0.global_base + (uint64_t)li * a0.global_cap;
        }

        // ---- pass A: cells and occupancy.  A node whose bricks exceed 70% of
        // the shared table is redone with the block's global-memory table.
        for (int attempt = 0; attempt < 2; ++attempt) {
            for (uint32_t i = tid0; i < bm.cap; i += tstride) {
                bm.key[i] = 0;
                bm.mask[i] = 0;
            }
            if (crank == 0 && threadIdx.x == 0) {
                s_bricks = 0;
                s_overflow = 0;
            }
            sync_all();
            const uint32_t limit = bm.cap - (bm.cap >> 2) - (bm.cap >> 4);
            for (uint32_t c = 0; c < ns.nchild; ++c) {
                const uint32_t cnt = ns.count[c];
                const uint64_t start = ns.start[c];
                const uint32_t jbase = ns.prefix[c];
                const uint32_t* src_lut = ((ns.kind >> c) & 1u) ? a.stage_lut : a.leaf_lut;
                const uint16_t* src_rec = reinterpret_cast<const uint16_t*>(((ns.kind >> c) & 1u) ? a.stage_rec : a.leaf_rec);
                const uint32_t* src_frac = ((ns.kind >> c) & 1u) ? a.stage_frac : a.leaf_frac;
                // x, y, z of the 18-byte record (2-byte aligned) as four aligned
                // words, and the candidate's sub-step word
                auto words = [&](uint32_t k, uint32_t (&w)[5]) {
                    const uint32_t* rw = reinterpret_cast<const uint32_t*>(
                        reinterpret_cast<uintptr_t>(src_rec + (start + k) * 9) & ~(uintptr_t)3);
                    w[0] = rw[0];
                    w[1] = rw[1];
                    w[2] = rw[2];
                    w[3] = rw[3];
                    w[4] = src_frac ? src_frac[start + k] : 0u;
                };
                // Cell and occupancy of candidate k; false when the node
                // overflows the table.  The cell comes from the record's
                // quantised coordinates; the cloud point is read only when a
                // quantisation step straddles a cell boundary.
                auto place = [&](uint32_t k, const uint32_t (&w)[5]) -> bool {
                    const uint32_t j = jbase + k;
                    const uint32_t rs = (uint32_t)(reinterpret_cast<uintptr_t>(src_rec + (start + k) * 9) & 2) * 8;
                    const int32_t q0 = (int32_t)__funnelshift_r(w[0], w[1], rs),
                                  q1 = (int32_t)__funnelshift_r(w[1], w[2], rs),
                                  q2 = (int32_t)__funnelshift_r(w[2], w[3], rs);
                    const uint32_t fw = w[4];
                    int ix, iy, iz;
                    if (fw >> 31) {
                        ix = quant_cell_fine(q0, fw & 1023u, qa0, a.grid);
                        iy = quant_cell_fine(q1, (fw >> 10) & 1023u, qa1, a.grid);
                        iz = quant_cell_fine(q2, (fw >> 20) & 1023u, qa2, a.grid);
                    } else {
                        ix = quant_cell(q0, qa0, a.grid);
                        iy = quant_cell(q1, qa1, a.grid);
                        iz = quant_cell(q2, qa2, a.grid);
                    }
                    if ((ix | iy | iz) < 0) {
                        const uint32_t idx = src_lut[start + k];
                        Coord co[3];
                        uint32_t col[3];
                        load_point<kF32>(a.cloud + (uint64_t)idx * a.stride, co, col);
                        float u;
                        if (ix < 0) ix = axis_cell<kF32>(co[0], ax0, a.grid, u);
                        if (iy < 0) iy = axis_cell<kF32>(co[1], ax1, a.grid, u);
                        if (iz < 0) iz = axis_cell<kF32>(co[2], ax2, a.grid, u);
                        if ((ix | iy | iz) < 0) {
                            atomicOr(a.err, kErrBelowBox);
                            ix = max(ix, 0);
                            iy = max(iy, 0);
                            iz = max(iz, 0);
                        }
                    }
                    uint32_t b = ((uint32_t)ix >> 2) | (((uint32_t)iy >> 2) << 8) | (((uint32_t)iz >> 2) << 16);
                    uint32_t bit = (ix & 3) | ((iy & 3) << 2) | ((iz & 3) << 4);
                    bool fresh;
                    uint32_t slot = brick_insert(bm, b + 1, fresh);
                    if (fresh && atomicAdd(p_bricks, 1u) + 1 >= limit) *(volatile uint32_t*)p_overflow = 1;
                    if (slot >= bm.cap) {
                        *(volatile uint32_t*)p_overflow = 1;
                        return false;
                    }
                    // 32-bit atomic on the half of the mask that holds the bit
                    atomicOr(reinterpret_cast<uint32_t*>(&bm.mask[slot]) + (bit >> 5), 1u << (bit & 31));
                    a.key_cache[off + j] = (slot << 6) | bit;
                    if (weighted) {
                        // the weight measures the distance from the point itself
                        // to each neighbour cell centre (kernel_inter_cell_filtering.cuh:171-176)
                        const uint32_t idx = src_lut[start + k];
                        Coord co[3];
                        uint32_t col[3];
                        load_point<kF32>(a.cloud + (uint64_t)idx * a.stride, co, col);
                        a.unit_cache[(off + j) * 3 + 0] = point_units<kF32>(co[0], ax0);
                        a.unit_cache[(off + j) * 3 + 1] = point_units<kF32>(co[1], ax1);
                        a.unit_cache[(off + j) * 3 + 2] = point_units<kF32>(co[2], ax2);
                    }
                    return true;
                };
                // two candidates per thread per iteration, both records loaded
                // before either is placed (119.7M-point build: subsampling
                // 13.6 -> 13.1 ms); one for distance weighting, whose pass also
                // reads the cloud point (pairs: 25.8M-point build 21.8 -> 22.3 ms)
                for (uint32_t k = tid0; k < cnt; k += (weighted ? 1u : 2u) * tstride) {
                    if (*(volatile uint32_t*)p_overflow) break;
                    const uint32_t k2 = k + tstride;
                    const bool two = !weighted && k2 < cnt;
                    uint32_t w[5], v[5] = {0, 0, 0, 0, 0};
                    words(k, w);
                    if (two) words(k2, v);
                    if (!place(k, w)) break;
                    if (two && !place(k2, v)) break;
                }
            }
            sync_all();
            if (!*(volatile uint32_t*)p_overflow) break;
            if (attempt == 1 || bm.key == gl_map.key) {
                if (crank == 0 && threadIdx.x == 0) atomicOr(a.err, kErrProbe);
                break;
            }
            bm = gl_map;
            sync_all();
        }
        const bool failed = *(volatile uint32_t*)p_overflow != 0;
        sync_all();
        if (failed) {
            if (crank == 0 && threadIdx.x == 0) a.out_points[li] = 0;
            continue;
        }

        // ---- ranks of occupied cells (each thread of rank 0 scans a run of slots)
        if (crank == 0) {
            const uint32_t per = (bm.cap + blockDim.x - 1) / blockDim.x;
            const uint32_t first = threadIdx.x * per;
            const uint32_t last = min(first + per, bm.cap);
            uint32_t sum = 0;
            for (uint32_t k = first; k < last; ++k) sum += (uint32_t)__popcll(bm.mask[k]);
            uint32_t total;
            uint32_t pre = block_exclusive_scan(sum, warp_sums, total);
            for (uint32_t k = first; k < last; ++k) {
                bm.base[k] = pre;
                pre += (uint32_t)__popcll(bm.mask[k]);
            }
            if (threadIdx.x == 0) ns.cells = total;
        }
        sync_all();
        // The brick map is final: cluster blocks other than rank 0 copy it from
        // rank 0's shared memory into their own (unused until now), so that the
        // cell list, pass B and emit read it locally instead of through
        // distributed shared memory.
        if constexpr (kCluster) {
            if (crank != 0 && bm.key == sm_map.key) {
                BrickMap local = bm;
                local.mask = dyn;
                local.key = reinterpret_cast<uint32_t*>(dyn + kBrickSlots);
                local.base = local.key + kBrickSlots;
                for (uint32_t i = threadIdx.x; i < bm.cap; i += blockDim.x) {
                    local.mask[i] = bm.mask[i];
                    local.key[i] = bm.key[i];
                    local.base[i] = bm.base[i];
                }
                __syncthreads();
                bm = local;
            }
        }
        // rank -> (brick slot, bit), for the per-cell emit.  A warp lists the
        // cells of its 32 consecutive slots (consecutive ranks) in rank order,
        // 32 ranks per coalesced store: each lane finds the slot holding its
        // rank by a search over the warp's running cell counts.
        for (uint32_t k = tid0; k < bm.cap; k += tstride) {
            const uint32_t lane = threadIdx.x & 31;
            const uint64_t m = bm.mask[k];
            const uint32_t c = (uint32_t)__popcll(m);
            uint32_t incl = c;
#pragma unroll
            for (uint32_t o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
            const uint32_t base0 = __shfl_sync(0xffffffffu, bm.base[k], 0);
            const uint32_t excl = incl - c;
            for (uint32_t q0 = 0; q0 < total; q0 += 32) {
                const uint32_t q = q0 + lane;
                uint32_t lo = 0;
#pragma unroll
                for (uint32_t st = 16; st >= 1; st >>= 1) {
                    const uint32_t v = __shfl_sync(0xffffffffu, incl, lo + st - 1);
                    if (v <= q) lo += st;
                }
                const uint32_t ow = min(lo, 31u);
                const uint64_t mo = ((uint64_t)__shfl_sync(0xffffffffu, (uint32_t)(m >> 32), ow) << 32) |
                                    __shfl_sync(0xffffffffu, (uint32_t)m, ow);
                const uint32_t eo = __shfl_sync(0xffffffffu, excl, ow);
                if (q < total) a.cell_slot[off + base0 + q] = ((k - lane + ow) << 6) | nth_bit64(mo, q - eo);
            }
        }
        const uint32_t cells = ns0->cells;
        if (crank == 0 && threadIdx.x == 0) s_emit_next = 0;
        for (uint32_t r = tid0; r < cells; r += tstride) {
            a.acc_best[off + r] = ~0ull;
            if (averaged && !weighted) a.acc_intra[off + r] = 0;
            if (weighted) a.csr_count[off + r] = 0;
        }
        sync_all();

        // ---- pass B: selection and colour sums
        for (uint32_t c = 0; c < ns.nchild; ++c) {
            const uint32_t cnt = ns.count[c];
            const uint64_t start = ns.start[c];
            const uint32_t jbase = ns.prefix[c];
            const bool staged = (ns.kind >> c) & 1u;
            const uint32_t* src_lut = staged ? a.stage_lut : a.leaf_lut;
            const uint8_t* src_rec = staged ? a.stage_rec : a.leaf_rec;
            // candidate k's cell word, cloud index and (averaged modes) the two
            // aligned words holding r, g, b (bytes 12..17 of the record)
            auto loads = [&](uint32_t k, uint32_t (&w)[4]) {
                w[0] = a.key_cache[off + jbase + k];
                w[1] = src_lut[start + k];
                if (averaged && !weighted) {
                    const uint32_t* cw = reinterpret_cast<const uint32_t*>(
                        reinterpret_cast<uintptr_t>(src_rec + (start + k) * 18 + 12) & ~(uintptr_t)3);
                    w[2] = cw[0];
                    w[3] = cw[1];
                }
            };
            auto take = [&](uint32_t k, const uint32_t (&w)[4]) {
                const uint32_t slot = w[0] >> 6, bit = w[0] & 63;
                const uint32_t rank = bm.base[slot] + (uint32_t)__popcll(bm.mask[slot] & ((1ull << bit) - 1ull));
                const uint32_t idx = w[1];
                // first point: (cloud index, candidate) -- the smallest index wins and
                // carries its candidate position; explicit random: (priority, index)
                uint64_t key;
                if constexpr (random) key = ((uint64_t)rp_priority(a.seed, level, morton, idx) << 32) | idx;
                else key = ((uint64_t)idx << 32) | (jbase + k);
                atomicMin(reinterpret_cast<unsigned long long*>(&a.acc_best[off + rank]), (unsigned long long)key);
                if (averaged && !weighted) {
                    const uint32_t cs = (uint32_t)(reinterpret_cast<uintptr_t>(src_rec + (start + k) * 18 + 12) & 2) * 8;
                    const uint32_t rg = __funnelshift_r(w[2], w[3], cs);
                    const uint32_t bb = (w[3] >> cs) & 0xFFFFu;
                    const uint64_t enc = encode_colors(rg & 0xFFFFu, rg >> 16, bb);
                    atomicAdd(reinterpret_cast<unsigned long long*>(&a.acc_intra[off + rank]), (unsigned long long)enc);
                }
                if (weighted) atomicAdd(&a.csr_count[off + rank], 1u);
            };
            // two candidates per thread per iteration, loads first (119.7M-point
            // build: subsampling 13.6 -> 12.8 ms, 12.3 ms with pass A's pairs);
            // one for distance weighting
            for (uint32_t k = tid0; k < cnt; k += (weighted ? 1u : 2u) * tstride) {
                const uint32_t k2 = k + tstride;
                const bool two = !weighted && k2 < cnt;
                uint32_t w[4] = {0, 0, 0, 0}, v[4] = {0, 0, 0, 0};
                loads(k, w);
                if (two) loads(k2, v);
                take(k, w);
                if (two) take(k2, v);
            }
        }
        sync_all();

        // ---- explicit random: the candidate holding each cell's winning key
        if constexpr (random) {
            for (uint32_t c = 0; c < ns.nchild; ++c) {
                const uint32_t cnt = ns.count[c];
                const uint64_t start = ns.start[c];
                const uint32_t jbase = ns.prefix[c];
                const uint32_t* src_lut = ((ns.kind >> c) & 1u) ? a.stage_lut : a.leaf_lut;
                for (uint32_t k = tid0; k < cnt; k += tstride) {
                    uint32_t kc = a.key_cache[off + jbase + k];
                    uint32_t slot = kc >> 6, bit = kc & 63;
                    uint32_t rank = bm.base[slot] + (uint32_t)__popcll(bm.mask[slot] & ((1ull << bit) - 1ull));
                    uint32_t idx = src_lut[start + k];
                    if ((uint32_t)a.acc_best[off + rank] == idx) a.acc_sel[off + rank] = jbase + k;
                }
            }
            sync_all();
        }

        // ---- weighted: group candidates by cell (CSR).  The exclusive scan of
        // the per-cell counts: each block of a cluster scans a contiguous run
        // of cells, offset by the totals of the runs before it (read from the
        // other blocks' shared memory).
        if (weighted) {
            const uint32_t per = (cells + csize - 1) / csize;
            const uint32_t c_first = min(cells, crank * per), c_last = min(cells, c_first + per);
            uint32_t running = 0;
            if constexpr (kCluster) {
                uint32_t part = 0;
                for (uint32_t r = c_first + threadIdx.x; r < c_last; r += blockDim.x) part += a.csr_count[off + r];
                uint32_t total;
                block_exclusive_scan(part, warp_sums, total);
                if (threadIdx.x == 0) s_run_total = total;
                cg::this_cluster().sync();
                if (threadIdx.x == 0) {
                    uint32_t o = 0;
                    for (uint32_t q = 0; q < crank; ++q) o += *cg::this_cluster().map_shared_rank(&s_run_total, q);
                    s_run_off = o;
                }
                __syncthreads();
                running = s_run_off;
            }
            for (uint32_t base = c_first; base < c_last; base += blockDim.x) {
                uint32_t r = base + threadIdx.x;
                uint32_t v = r < c_last ? a.csr_count[off + r] : 0;
                uint32_t total;
                uint32_t pre = block_exclusive_scan(v, warp_sums, total);
                if (r < c_last) {
                    a.csr_start[off + r] = running + pre;
                    a.csr_count[off + r] = 0;
                }
                running += total;
            }
            sync_all();
            for (uint32_t c = 0; c < ns.nchild; ++c) {
                const uint32_t cnt = ns.count[c];
                const uint64_t start = ns.start[c];
                const uint32_t jbase = ns.prefix[c];
                const uint8_t* src_rec = ((ns.kind >> c) & 1u) ? a.stage_rec : a.leaf_rec;
                for (uint32_t k = tid0; k < cnt; k += tstride) {
                    const uint32_t j = jbase + k;
                    uint32_t kc = a.key_cache[off + j];
                    uint32_t slot = kc >> 6, bit = kc & 63;
                    uint32_t rank = bm.base[slot] + (uint32_t)__popcll(bm.mask[slot] & ((1ull << bit) - 1ull));
                    uint32_t p = a.csr_start[off + rank] + atomicAdd(&a.csr_count[off + rank], 1u);
                    const uint16_t* src = reinterpret_cast<const uint16_t*>(src_rec + (start + k) * 18);
                    uint32_t* dst = reinterpret_cast<uint32_t*>(a.csr_pts + (off + p) * 20);
                    dst[0] = __float_as_uint(a.unit_cache[(off + j) * 3 + 0]);
                    dst[1] = __float_as_uint(a.unit_cache[(off + j) * 3 + 1]);
                    dst[2] = __float_as_uint(a.unit_cache[(off + j) * 3 + 2]);
                    dst[3] = (uint32_t)src[6] | ((uint32_t)src[7] << 16);
                    dst[4] = (uint32_t)src[8];
                }
            }
            sync_all();
        }

        // ---- emit one record per occupied cell (thread per cell; each warp
        // takes the next run of 32 consecutive cells until none is left, so
        // that warps with light cells take more runs, and writes their
        // records with coalesced stores)
        if constexpr (weighted) {
            if (a.emit_state) {
                // a level of few nodes: k_emit_weighted spreads the node's
                // cells over all SMs.  A shared-table node's brick map goes to
                // global memory; a global-table node keeps its own table.
                const bool shared_table = bm.key != gl_map.key;
                if (shared_table) {
                    uint8_t* dst = a.emit_maps + (uint64_t)li * kBrickMapBytes;
                    uint64_t* dmask = reinterpret_cast<uint64_t*>(dst);
                    uint32_t* dkey = reinterpret_cast<uint32_t*>(dst + (uint64_t)kBrickSlots * 8);
                    uint32_t* dbase = dkey + kBrickSlots;
                    for (uint32_t i = tid0; i < kBrickSlots; i += tstride) {
                        dmask[i] = bm.mask[i];
                        dkey[i] = bm.key[i];
                        dbase[i] = bm.base[i];
                    }
                }
                if (crank == 0 && threadIdx.x == 0) {
                    a.emit_state[4 * li + 0] = cells;
                    a.emit_state[4 * li + 2] = shared_table ? 1u : 2u;
                }
            } else {
                emit_weighted<kRandom>(a, bm, ns, off, oo, cells, p_emit_next);
            }
        } else {
            for (;;) {
                uint32_t r0 = 0;
                if ((threadIdx.x & 31) == 0) r0 = atomicAdd(p_emit_next, 32u);
                r0 = __shfl_sync(0xffffffffu, r0, 0);
                if (r0 >= cells) break;
                const uint32_t r = r0 + (threadIdx.x & 31);
                uint32_t nw[5] = {0, 0, 0, 0, 0};
                if (r < cells) {
                    const uint32_t ks = a.cell_slot[off + r];
                    const uint32_t slot = ks >> 6, bit = ks & 63;
                    const uint32_t brick = bm.key[slot] - 1;
                    const int bx = (int)(brick & 0xFF), by = (int)((brick >> 8) & 0xFF), bz = (int)(brick >> 16);
                    const int lx = (int)(bit & 3), ly = (int)((bit >> 2) & 3), lz = (int)((bit >> 4) & 3);
                    const uint64_t best = a.acc_best[off + r];
                    const uint32_t idx = random ? (uint32_t)best : (uint32_t)(best >> 32);
                    const uint32_t jsel = random ? a.acc_sel[off + r] : (uint32_t)best;
                    // the child holding candidate jsel: a count of comparisons, the
                    // same instructions on every lane
                    uint32_t csel = 0;
    #pragma unroll
                    for (uint32_t c = 1; c < 8; ++c) csel += (c < ns.nchild && ns.prefix[c] <= jsel) ? 1u : 0u;
                    // the winner's record holds its output coordinates (same cloud
                    // minimum and scale at every level) and, unaveraged, its colour
                    const uint64_t spos = ns.start[csel] + (jsel - ns.prefix[csel]);
                    const uintptr_t sa =
                        reinterpret_cast<uintptr_t>((((ns.kind >> csel) & 1u) ? a.stage_rec : a.leaf_rec) + spos * 18);
                    // 20 bytes from the 4-byte boundary below the record (the record
                    // arrays keep 16 readable bytes past their end)
                    const uint32_t* sq = reinterpret_cast<const uint32_t*>(sa & ~(uintptr_t)3);
                    const uint32_t sh = (uint32_t)(sa & 2) * 8;
                    const uint32_t q0 = sq[0], q1 = sq[1], q2 = sq[2], q3 = sq[3], q4 = sq[4];
                    nw[0] = __funnelshift_r(q0, q1, sh);
                    nw[1] = __funnelshift_r(q1, q2, sh);
                    nw[2] = __funnelshift_r(q2, q3, sh);
                    const uint32_t w3 = __funnelshift_r(q3, q4, sh);
                    uint16_t cr = (uint16_t)w3, cg = (uint16_t)(w3 >> 16), cb = (uint16_t)(q4 >> sh);
                    if (intra) {
                        decode_colors(a.acc_intra[off + r], cr, cg, cb);
                    } else if (inter) {
                        decode_colors(inter_sum(bm, slot, bx, by, bz, lx, ly, lz, a.acc_intra + off), cr, cg, cb);
                    }
                    a.out_lut[oo + r] = idx;
                    if (a.out_frac) {
                        const uint32_t* sf = ((ns.kind >> csel) & 1u) ? a.stage_frac : a.leaf_frac;
                        a.out_frac[oo + r] = sf ? sf[spos] : 0u;
                    }
                    nw[3] = (uint32_t)cr | ((uint32_t)cg << 16);
                    nw[4] = cb;
                }
                store_run(a.out_rec + (oo + r0) * 18, 0, min(32u, cells - r0), nw, stage);
            }
        }
        if (crank == 0 && threadIdx.x == 0) a.out_points[li] = cells;
        sync_all();
    }
}

// The emit of the distance-weighted nodes a level of few nodes handed over
// (emit_state[4v + 2] set): every block takes runs of such a node's cells,
// with the node's brick map copied into its shared memory (or read from the
// node's own global table), so that the node's cells spread over all SMs
// instead of its cluster's.
template <bool kRandom>
__global__ void __launch_bounds__(kSubThreads, 1) k_emit_weighted(SubLevelArgs a) {
    extern __shared__ uint64_t dyn[];
    __shared__ NodeShared ns;
    __shared__ uint32_t s_take;
    BrickMap bm;
    bm.mask = dyn;
    bm.key = reinterpret_cast<uint32_t*>(dyn + kBrickSlots);
    bm.base = bm.key + kBrickSlots;
    bm.cap = kBrickSlots;
    bm.shift = kBrickShift;
    bm.grid = a.grid;
    bm.bs = (a.grid + 3) >> 2;
    for (uint32_t v = 0; v < a.n_nodes; ++v) {
        uint32_t* st = a.emit_state + 4 * v;
        if (threadIdx.x == 0) {
            const uint32_t cells = st[0];
            s_take = st[2] != 0 && *(volatile uint32_t*)&st[1] < cells;
            if (s_take) {
                load_node_shared(ns, a.nodes[v]);
                ns.cells = cells;
            }
        }
        __syncthreads();
        const bool take = s_take != 0;
        __syncthreads();   // s_take is rewritten for the next node
        if (!take) continue;
        BrickMap m = bm;
        if (st[2] == 1) {   // the node's shared-table map, into this block's shared memory
            const uint8_t* src = a.emit_maps + (uint64_t)v * kBrickMapBytes;
            const uint64_t* smask = reinterpret_cast<const uint64_t*>(src);
            const uint32_t* skey = reinterpret_cast<const uint32_t*>(src + (uint64_t)kBrickSlots * 8);
            const uint32_t* sbase = skey + kBrickSlots;
            for (uint32_t i = threadIdx.x; i < kBrickSlots; i += blockDim.x) {
                bm.mask[i] = smask[i];
                bm.key[i] = skey[i];
                bm.base[i] = sbase[i];
            }
        } else {   // the node's own global table
            m.mask = a.global_mask + (uint64_t)v * a.global_cap;
            m.key = a.global_key + (uint64_t)v * a.global_cap;
            m.base = a.global_base + (uint64_t)v * a.global_cap;
            m.cap = a.global_cap;
            m.shift = a.global_shift;
        }
        __syncthreads();
        const SubNode& nd = a.nodes[v];
        emit_weighted<kRandom>(a, m, ns, nd.cand_off, nd.out_off, ns.cells, st + 1);
        __syncthreads();   // the map and the node's metadata are rewritten for the next node
    }
}

__global__ void __launch_bounds__(1024) k_prepare_level(SubNode* nodes, uint32_t n_nodes, const uint32_t* out_points,
                                                        uint64_t* stage_off, uint32_t first_internal,
                                                        uint64_t* level_base, uint64_t scratch_cap,
                                                        uint64_t stage_cap, uint32_t* work_counter, uint32_t* err) {
    __shared__ uint64_t warp_sums[32];
    __shared__ uint32_t s_skip;
    if (threadIdx.x == 0) s_skip = (*err & kErrCapacity) != 0;   // an earlier level overflowed
    __syncthreads();
    const uint64_t base = *level_base;
    uint64_t running = 0;
    for (uint32_t k0 = 0; k0 < n_nodes; k0 += blockDim.x) {
        const uint32_t k = k0 + threadIdx.x;
        uint64_t p = 0;
        if (k < n_nodes && !s_skip) {
            SubNode& nd = nodes[k];
            for (uint32_t c = 0; c < nd.nchild; ++c) {
                if ((nd.child_kind >> c) & 1u) {
                    const uint32_t ii = (uint32_t)nd.child_start[c];
                    nd.child_count[c] = out_points[ii];
                    nd.child_start[c] = stage_off[ii];
                }
                p += nd.child_count[c];
            }
        }
        uint64_t total;
        const uint64_t pre = block_exclusive_scan64(p, warp_sums, total);
        if (k < n_nodes && !s_skip) {
            SubNode& nd = nodes[k];
            nd.p_in = (uint32_t)p;
            nd.cand_off = running + pre;
            nd.out_off = base + running + pre;
            stage_off[first_internal + k] = base + running + pre;
            if (p > 0xFFFFFFFFull) atomicOr(err, kErrCapacity);
        }
        running += total;
    }
    if (threadIdx.x == 0) {
        const bool over = s_skip || running > scratch_cap || base + running > stage_cap || (*err & kErrCapacity);
        if (over) atomicOr(err, kErrCapacity);
        *work_counter = over ? n_nodes : 0u;
        *level_base = base + running;
    }
}

}   // namespace

int launch_prepare_level(SubNode* nodes, uint32_t n_nodes, const uint32_t* out_points, uint64_t* stage_off,
                         uint32_t first_internal, uint64_t* level_base, uint64_t scratch_cap, uint64_t stage_cap,
                         uint32_t* work_counter, uint32_t* err, cudaStream_t stream) {
    k_prepare_level<<<1, 1024, 0, stream>>>(nodes, n_nodes, out_points, stage_off, first_internal, level_base,
                                            scratch_cap, stage_cap, work_counter, err);
    return 1;
}

uint32_t subsample_block_size() {
    return kSubThreads;
}

size_t subsample_smem_bytes() {
    return (size_t)kBrickSlots * (8 + 4 + 4) + (size_t)(kSubThreads / 32) * kStageBytes;
}

namespace {

// Blocks per node for a level of n_nodes nodes: the smallest power of two up
// to `cap` whose clusters cover the SMs (levels with at least one node per SM
// run one block per node).  Measured per level on the 119.7M-point build:
// clusters of 2 take a 100-node level from 0.54 to 0.34 ms; clusters of 8 were
// slower than 4 on its 10- to 40-node levels, so the cap is 4, and 8 for
// levels of at most 16 nodes (launch_one).  Distance-weighted
// levels go up to 16 (a non-portable cluster size), and at least to the
// level's balance_blocks: the neighbourhood walk per output cell makes a
// level's largest nodes long.  On the 25.8M-point weighted build a cap of 16
// takes the root from 3.34 to 1.46 ms and the 8-node level from 2.10 to
// 1.13 ms (a cap of 8: 2.15 and 1.39 ms).
// Allows clusters above the portable size of 8 for a kernel on the current
// device (once per kernel and device; a refusal leaves smaller clusters).
void allow_wide_clusters(const void* kernel) {
    static std::mutex mu;
    static std::set<std::pair<int, const void*>> done;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(mu);
    if (!done.insert({dev, kernel}).second) return;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        cudaGetLastError();
}

uint32_t cluster_size(uint32_t n_nodes, int num_sms, uint32_t cap) {
    uint32_t c = 1;
    while (c < cap && (uint64_t)c * n_nodes < (uint64_t)num_sms) c <<= 1;
    return c;
}

// Clusters of c blocks of `kernel` that the device holds at once (0: none
// fits).  A cluster must fit in one GPC, so the count follows how the chip's
// SMs are grouped and differs between GPUs of one model (clusters of 16 are
// the sensitive size).  Queried once per device, kernel and size.
int cluster_slots(const void* kernel, size_t smem, uint32_t c) {
    static std::mutex mu;
    static std::map<std::tuple<int, const void*, uint32_t>, int> known;
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(dev, kernel, c);
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = known.find(key);
        if (it != known.end()) return it->second;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(kSubThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int m = 0;
    if (cudaOccupancyMaxActiveClusters(&m, kernel, &cfg) != cudaSuccess) {
        cudaGetLastError();
        m = 0;
    }
    std::lock_guard<std::mutex> g(mu);
    known[key] = m;
    return m;
}

// Cluster size for a distance-weighted level (weighted_cluster_choice), from
// the clusters of 2, 4, 8 and 16 blocks of the kernel the device holds.
uint32_t weighted_cluster_size(const void* cluster_kernel, size_t smem, uint32_t n_nodes, int num_sms,
                               uint32_t balance, uint32_t cap) {
    int slots[5] = {0, 0, 0, 0, 0};
    for (uint32_t c = 2, i = 1; c <= cap && c <= (uint32_t)std::max(num_sms, 1) && i < 5; c <<= 1, ++i)
        slots[i] = cluster_slots(cluster_kernel, smem, c);
    return weighted_cluster_choice(slots, n_nodes, num_sms, balance, cap);
}

template <bool kF32, int kColor, bool kRandom, bool kWave>
void launch_one(const SubLevelArgs& a, const WaveNodes& wn, int num_sms, uint32_t balance, size_t smem,
                cudaStream_t stream, const ClusterCaps& caps) {
    // levels of at most 16 nodes (the top of the tree, a few large nodes)
    // take clusters of up to 8: 25.8M-point random planes 6.70 -> 6.40 ms
    // (root 0.90 -> 0.68 ms), 5.1M-point heightfield 1.56 -> 1.53 ms; 16
    // helped the first root further but slowed the other two
    const uint32_t plain_cap = a.n_nodes <= 16u ? std::max(caps.plain, 8u) : caps.plain;
    const uint32_t cap = std::min(kColor == 3 ? caps.weighted : plain_cap, std::max(caps.node_blocks, 1u));
    uint32_t cs = cluster_size(a.n_nodes, num_sms, cap);
    if (kColor == 3 && cap > 1) {
        auto kern = k_subsample<kF32, kColor, kRandom, true, kWave>;
        allow_dynamic_smem(reinterpret_cast<const void*>(kern), smem);
        if (cap > 8) allow_wide_clusters(reinterpret_cast<const void*>(kern));
        cs = weighted_cluster_size(reinterpret_cast<const void*>(kern), smem, a.n_nodes, num_sms, balance, cap);
    }
    if (cs > 1) {
        auto kern = k_subsample<kF32, kColor, kRandom, true, kWave>;
        allow_dynamic_smem(reinterpret_cast<const void*>(kern), smem);
        if (cs > 8) allow_wide_clusters(reinterpret_cast<const void*>(kern));
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.blockDim = dim3(kSubThreads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = stream;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        // the largest cluster size up to cs of which one cluster fits
        for (uint32_t c = cs; c > 1; c >>= 1) {
            attr[0].val.clusterDim.x = c;
            const int max_clusters = cluster_slots(reinterpret_cast<const void*>(kern), smem, c);
            if (max_clusters > 0) {
                const uint32_t clusters = std::min<uint32_t>(a.n_nodes, (uint32_t)max_clusters);
                cfg.gridDim = dim3(clusters * c);
                if (cudaLaunchKernelEx(&cfg, kern, a, wn) == cudaSuccess) return;
            }
            cudaGetLastError();
        }
        // no cluster fits: one block per node
    }
    auto kern = k_subsample<kF32, kColor, kRandom, false, kWave>;
    allow_dynamic_smem(reinterpret_cast<const void*>(kern), smem);
    const int grid = (int)std::min<uint32_t>(a.n_nodes, (uint32_t)num_sms);
    kern<<<grid, kSubThreads, smem, stream>>>(a, wn);
}

template <bool kF32, bool kWave>
void launch_mode(const SubLevelArgs& a, const WaveNodes& wn, int num_sms, uint32_t balance, size_t smem,
                 cudaStream_t stream, const ClusterCaps& caps) {
    const bool intra = (a.mode & kModeIntra) != 0;
    const bool inter = !intra && (a.mode & kModeInter) != 0;
    const bool weighted = inter && (a.mode & kModeWeight) != 0;
    const int color = intra ? 1 : (weighted ? 3 : (inter ? 2 : 0));
    const bool random = (a.mode & kModeRandom) != 0;
    switch (color * 2 + (random ? 1 : 0)) {
    case 0: launch_one<kF32, 0, false, kWave>(a, wn, num_sms, balance, smem, stream, caps); break;
    case 1: launch_one<kF32, 0, true, kWave>(a, wn, num_sms, balance, smem, stream, caps); break;
    case 2: launch_one<kF32, 1, false, kWave>(a, wn, num_sms, balance, smem, stream, caps); break;
    case 3: launch_one<kF32, 1, true, kWave>(a, wn, num_sms, balance, smem, stream, caps); break;
    case 4: launch_one<kF32, 2, false, kWave>(a, wn, num_sms, balance, smem, stream, caps); break;
    case 5: launch_one<kF32, 2, true, kWave>(a, wn, num_sms, balance, smem, stream, caps); break;
    case 6: launch_one<kF32, 3, false, kWave>(a, wn, num_sms, balance, smem, stream, caps); break;
    default: launch_one<kF32, 3, true, kWave>(a, wn, num_sms, balance, smem, stream, caps); break;
    }
}

}   // namespace

int launch_subsample_level(const SubLevelArgs& a, int num_sms, uint32_t balance_blocks, cudaStream_t stream,
                           const ClusterCaps& caps) {
    if (!a.n_nodes) return 0;
    const size_t smem = subsample_smem_bytes();
    const WaveNodes none{};
    if (a.float_input) launch_mode<true, false>(a, none, num_sms, balance_blocks, smem, stream, caps);
    else launch_mode<false, false>(a, none, num_sms, balance_blocks, smem, stream, caps);
    return 1;
}

int launch_subsample_wave(const SubLevelArgs& wave, const WaveNodes& wn, int num_sms, uint32_t balance_blocks,
                          cudaStream_t stream, const ClusterCaps& caps) {
    if (!wave.n_nodes) return 0;
    const size_t smem = subsample_smem_bytes();
    if (wave.float_input) launch_mode<true, true>(wave, wn, num_sms, balance_blocks, smem, stream, caps);
    else launch_mode<false, true>(wave, wn, num_sms, balance_blocks, smem, stream, caps);
    return 1;
}

int launch_emit_weighted(const SubLevelArgs& a, int num_sms, cudaStream_t stream) {
    if (!a.n_nodes || !a.emit_state) return 0;
    const size_t smem = (size_t)kBrickMapBytes;
    const int grid = std::max(num_sms, 1);
    if (a.mode & kModeRandom) {
        allow_dynamic_smem(reinterpret_cast<const void*>(k_emit_weighted<true>), smem);
        k_emit_weighted<true><<<grid, kSubThreads, smem, stream>>>(a);
    } else {
        allow_dynamic_smem(reinterpret_cast<const void*>(k_emit_weighted<false>), smem);
        k_emit_weighted<false><<<grid, kSubThreads, smem, stream>>>(a);
    }
    return 1;
}

}   // namespace oc
