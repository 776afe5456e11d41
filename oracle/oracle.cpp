// CPU oracle for the LOD octree build -- TEST INFRASTRUCTURE ONLY.
//
// Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and
// its `--impl reference` arm) load this library, and only as the checker or as
// the timed CPU baseline.  The product library (libOctreeApi.so) never links,
// loads or calls anything under oracle/.
//
// What it is: a plain, multithreaded C++ restatement of the hot path of
// PotreeConverterGPU's OctreeApi (citations are file:line in the reference
// project).  Every arithmetic step that decides a result is written the way the
// reference writes it (IEEE double, same operation order); every place where
// the reference is racy is replaced by one canonical, deterministic rule:
//
//   * cell index          mapPointToGrid, OctreeLibrary/src/kernel/kernel_helpers.cuh:10-25
//   * count pyramid       kernelPointCounting point_counting.cuh:29-53,
//                         kernelPropagatePointCounts point_count_propagation.cuh:34-86
//   * merge / tree        kernelMergeHierarchical hierarchical_merging.cuh:35-122
//                         (finished = count >= threshold; children of a finished
//                         node are tree nodes; level-0 cells are always leaves)
//   * leaf data layout    reference: atomicAdd(lutOffset) order (racy,
//                         hierarchical_merging.cuh:110).  Canonical: leaves in
//                         hierarchy BFS order, points inside a leaf in cloud order.
//   * distribution        kernelDistributePoints point_distributing.cuh:30-75
//   * subsampling         fp_subsampling.cu:9-185 / rp_subsampling.cu:10-222
//                         (post-order DFS, output appended after the N leaf
//                         points, calculateWritingPosition kernel_helpers.cuh:55-59).
//                         First-point winner (racy atomicExch) -> smallest cloud
//                         index in the cell.  Explicit random (time-seeded curand
//                         + arrival order) -> smallest Philox4x32-10 priority
//                         keyed by (seed, node, cloud index).
//                         Node records are ordered by ascending cell index.
//   * colour filtering    encodeColors kernel_helpers.cuh:34-53, decode
//                         fp_subsampling.cuh:95-101 (packed u64, bit-exact),
//                         inter-cell scatter kernel_inter_cell_filtering.cuh:20-91.
//                         Distance weighting (kernel_inter_cell_filtering.cuh:109-194,
//                         float atomics in the reference) -> fixed-point integer
//                         accumulation of an fp32 weight, see weight_q below.
//                         F_WEIGHT_LITERAL instead restates the reference's own
//                         arithmetic (binary64 distances, float exp, float sums
//                         in one fixed order, truncating division): the yardstick
//                         for the +-1 tolerance of the canonical rule.
//   * export              breathFirstExport potree_exporter.cu:62-96
//   * statistics          OctreeData::updateNodeStatistics octree.cu:79-132
//
// The exact cell / coordinate formulas are evaluated directly in double here.
// The only fp32 quantity the oracle shares with the GPU path is the cell-unit
// position used by distance weighting (point_units: (p - node min) / t from a
// float-pair split of the coordinate), which is part of the canonical
// definition of the weighted mode.

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct OracleParams {
    double scale[3];
    double bb_min[3];
    double bb_max[3];
    uint64_t seed;
    uint32_t n;
    uint32_t stride;
    uint32_t cloud_type;   // 0 = float32 xyz, 1 = float64 xyz (metadata.cuh:13-70)
    uint32_t chunk_grid;
    uint32_t sub_grid;
    uint32_t merge_threshold;
    float output_factor;
    uint32_t flags;        // bit0 intra, bit1 inter, bit2 replacement, bit3 random, bit4 weighting
    uint32_t threads;
    uint32_t reserved;
};

enum : uint32_t {
    F_INTRA = 1,
    F_INTER = 2,
    F_REPLACE = 4,
    F_RANDOM = 8,
    F_WEIGHT = 16,
    // test variants of distance weighting (the canonical rule is F_WEIGHT alone):
    F_WEIGHT_LITERAL = 32,   // the reference's float arithmetic, propagated up the levels
    F_WEIGHT_LOCAL = 64,     // with LITERAL: each node's literal colours from the canonical
                             // children's colours; the canonical colours propagate
    F_WEIGHT_REVERSE = 128,  // with LITERAL: float sums in the reverse candidate order
};

#pragma pack(push, 1)
struct Record {   // OutputBuffer, types.cuh:18-24
    int32_t x, y, z;
    uint16_t r, g, b;
};
struct HierEntry {   // HierarchyFileEntry, potree_exporter.cuh:27-36
    uint8_t type;
    uint8_t mask;
    uint32_t points;
    uint64_t byte_offset;
    uint64_t byte_size;
};
#pragma pack(pop)
static_assert(sizeof(Record) == 18, "record");
static_assert(sizeof(HierEntry) == 22, "hierarchy entry");

struct OracleStats {
    uint64_t points_total;     // N + P_out (records referenced by the hierarchy)
    uint64_t p_out;            // points held by internal nodes
    uint64_t p_in;             // sum over internal nodes of their children's points
    uint64_t out_capacity;     // reference output buffer capacity, point_cloud.cuh:24
    uint32_t depth;
    uint32_t tree_nodes;
    uint32_t leaf_nodes;
    uint32_t internal_nodes;
    uint32_t sparse_nodes;     // occupied cells over all pyramid levels
    uint32_t dense_nodes;
    uint32_t max_leaf_depth;
    uint32_t min_leaf_points;
    uint32_t max_leaf_points;
    float mean_leaf_points;
    float stdev_leaf_points;
    uint32_t guard_truncation;     // reference launch extent would drop child points
    uint32_t guard_capacity;       // reference output buffer would overflow
    uint32_t guard_color_overflow; // cells whose packed colour fields overflow
    uint32_t guard_root_leaf;      // N < threshold: reference reads an unset parent
    uint32_t guard_div0;           // packed colour count field is 0 mod 1024
    uint32_t error;                // 0 ok, 1 bad params, 2 point below the bbox
    uint32_t reserved;
};

struct TNode {
    uint32_t x, y, z;
    uint32_t level;
    uint32_t sub_count;   // pyramid count of the cell
    int32_t child[8];
    int32_t parent;
    uint8_t internal;
    uint8_t mask;
    double mn[3];         // node bbox minimum (calculateChildMinBB chain)
    uint64_t data_idx;
    uint32_t points;      // hierarchy point count
    uint64_t morton;
};

struct Result {
    std::vector<HierEntry> hier;
    std::vector<Record> records;
    std::vector<uint32_t> lut;
    std::vector<TNode> nodes;   // BFS order
    std::vector<std::vector<uint32_t>> level_counts;   // dense z-major per level
    OracleStats stats{};
};

template <class F>
void parallel_for(uint64_t n, uint32_t threads, F&& fn) {
    if (threads <= 1 || n < 4096) {
        fn(0, n, 0u);
        return;
    }
    std::vector<std::thread> pool;
    uint64_t chunk = (n + threads - 1) / threads;
    for (uint32_t t = 0; t < threads; ++t) {
        uint64_t a = t * chunk, b = std::min<uint64_t>(n, a + chunk);
        if (a >= b) break;
        pool.emplace_back([&, a, b, t] { fn(a, b, t); });
    }
    for (auto& th : pool) th.join();
}

template <class F>
void parallel_dynamic(uint64_t n, uint32_t threads, F&& fn) {
    std::atomic<uint64_t> next{0};
    auto worker = [&] {
        for (;;) {
            uint64_t i = next.fetch_add(1);
            if (i >= n) break;
            fn(i);
        }
    };
    if (threads <= 1) {
        worker();
        return;
    }
    std::vector<std::thread> pool;
    for (uint32_t t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
}

inline void load_point(const uint8_t* rec, uint32_t type, double p[3], uint16_t c[3]) {
    if (type == 0) {
        float f[3];
        std::memcpy(f, rec, 12);
        p[0] = f[0];
        p[1] = f[1];
        p[2] = f[2];
        c[0] = rec[12];
        c[1] = rec[13];
        c[2] = rec[14];
    } else {
        std::memcpy(p, rec, 24);
        c[0] = rec[24];
        c[1] = rec[25];
        c[2] = rec[26];
    }
}

// mapPointToGrid, kernel_helpers.cuh:14-22, one axis.  Returns -1 where the
// reference would compute a negative index (a point below the bbox).
inline int64_t ref_axis_cell(double p, double mn, double t, uint32_t G) {
    double u = (p - mn) / t;
    double v = std::fmin(u, (double)G - 1.0);
    if (!(v > -1.0)) return -1;
    return (int64_t)v;
}

// kernelDistributePoints point_distributing.cuh:245-247 (and the subsampling
// kernels, e.g. fp_subsampling.cuh:105-107): floor((p - min) * (1/scale)).
inline int32_t ref_out_coord(double p, double mn, double sf) {
    return (int32_t)std::floor((p - mn) * sf);
}

// ---------------------------------------------------------------------------
// Shared canonical pieces (must match the GPU path bit for bit).

// Cell-unit position (p - mn) / t of a coordinate, as the GPU path evaluates
// it: the coordinate split into a float pair hi + lo (float input: hi = p,
// lo = 0; double input: hi = p with its mantissa cut to 24 bits, lo = the
// rest rounded to float), the node minimum likewise (m_hi = float(mn),
// m_lo = float(mn - m_hi)), then ((hi - m_hi) + (lo - m_lo)) * float(1 / t).
struct UAx {
    double mn, t;
    float m_hi, m_lo, r;
};

inline UAx make_uax(double mn, double t) {
    UAx a;
    a.mn = mn;
    a.t = t;
    a.m_hi = (float)mn;
    a.m_lo = (float)(mn - (double)a.m_hi);
    a.r = (float)(1.0 / t);
    return a;
}

inline float point_units(double p, bool f32, const UAx& a) {
    float hi, lo;
    if (f32) {
        hi = (float)p;
        lo = 0.0f;
    } else {
        uint64_t bits;
        std::memcpy(&bits, &p, 8);
        const uint32_t e = (uint32_t)(bits >> 52) & 0x7FFu;
        const uint64_t mant = bits & ((1ull << 52) - 1);
        const uint32_t sign = (uint32_t)(bits >> 63) << 31;
        if (e == 0 && mant == 0) {
            std::memcpy(&hi, &sign, 4);
            lo = 0.0f;
        } else {
            const int ue = (int)e - 1023;
            if (ue < -60 || ue > 100) return (float)((p - a.mn) / a.t);
            const uint32_t hb = sign | ((uint32_t)(ue + 127) << 23) | (uint32_t)(mant >> 29);
            std::memcpy(&hi, &hb, 4);
            const uint32_t low = (uint32_t)(mant & ((1u << 29) - 1));
            if (low == 0) {
                lo = 0.0f;
            } else {
                const uint32_t sb = (uint32_t)(ue - 52 + 127) << 23;
                float sc;
                std::memcpy(&sc, &sb, 4);
                const float lf = (float)low * sc;
                lo = sign ? -lf : lf;
            }
        }
    }
    const float d = (hi - a.m_hi) + (lo - a.m_lo);
    return d * a.r;
}

// exp(x) for x in [-15, 0]: Cody & Waite range reduction x = k*ln2 + f with
// ln2 split into a 12-bit head and a float tail, then the degree-7 Taylor
// polynomial of e^f by Horner with fused multiply-adds, then an exact scaling
// by 2^k.  Deterministic: the GPU evaluates the same operation sequence.
inline float exp_neg(float x) {
    const float kLog2e = 1.44269504088896341f;
    const float kLn2Hi = 0.693359375f;            // 1420 / 2048
    const float kLn2Lo = -2.12194440054690583e-4f; // ln2 - 1420/2048
    float kf = std::rint(x * kLog2e);
    float f = std::fmaf(-kf, kLn2Hi, x);
    f = std::fmaf(-kf, kLn2Lo, f);
    float p = 1.0f / 5040.0f;
    p = std::fmaf(p, f, 1.0f / 720.0f);
    p = std::fmaf(p, f, 1.0f / 120.0f);
    p = std::fmaf(p, f, 1.0f / 24.0f);
    p = std::fmaf(p, f, 1.0f / 6.0f);
    p = std::fmaf(p, f, 0.5f);
    p = std::fmaf(p, f, 1.0f);
    p = std::fmaf(p, f, 1.0f);
    int k = (int)kf;
    uint32_t sbits = (uint32_t)(k + 127) << 23;
    float scale;
    std::memcpy(&scale, &sbits, 4);
    return p * scale;
}

// Fixed-point weight of one point for one neighbour cell.
//   d2 = |(n + 0.5) - u|^2 in cell units, (d / r)^2 = d2 * 4/27 with
//   r = half diagonal of 3x3x3 cells (fp_subsampling.cu:56-61),
//   w = exp(-10 (d/r)^2) (kernel_inter_cell_filtering.cuh:176-180),
//   wq = round(w * 2^28), at least 2^28 e^-10 > 12000 for a point in its cell.
inline uint32_t weight_q(const float u[3], int32_t nx, int32_t ny, int32_t nz) {
    float dx = ((float)nx + 0.5f) - u[0];
    float dy = ((float)ny + 0.5f) - u[1];
    float dz = ((float)nz + 0.5f) - u[2];
    float d2 = std::fmaf(dz, dz, std::fmaf(dy, dy, dx * dx));
    float q = d2 * (float)(4.0 / 27.0);
    q = std::fmin(q, 1.5f);
    float w = exp_neg(-10.0f * q);
    return (uint32_t)(w * 268435456.0f + 0.5f);
}

inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c[0] = n0;
        c[1] = n1;
        c[2] = n2;
        c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Priority of cloud point `idx` for explicit random subsampling in node
// (level, morton): first output word of Philox4x32-10.
inline uint32_t rp_priority(uint64_t seed, uint32_t level, uint64_t morton, uint32_t idx) {
    uint32_t c[4] = {idx, (uint32_t)morton, (uint32_t)(morton >> 32) ^ (level << 24), 0x52504E44u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return c[0];
}

inline uint64_t encode_colors(const uint16_t c[3]) {   // kernel_helpers.cuh:49-53
    return ((uint64_t)c[0] << 46) | ((uint64_t)c[1] << 28) | ((uint64_t)c[2] << 10) | 1ull;
}

inline void decode_colors(uint64_t e, uint16_t out[3], uint32_t* div0) {   // fp_subsampling.cuh:95-101
    uint16_t amount = (uint16_t)(e & 0x3FF);
    if (amount == 0) {
        out[0] = out[1] = out[2] = 0xFFFF;
        ++*div0;
        return;
    }
    out[0] = (uint16_t)(((e >> 46) & 0xFFFF) / amount);
    out[1] = (uint16_t)(((e >> 28) & 0xFFFF) / amount);
    out[2] = (uint16_t)(((e >> 10) & 0xFFFF) / amount);
}

inline uint64_t morton3(uint32_t x, uint32_t y, uint32_t z, uint32_t bits) {
    uint64_t m = 0;
    for (int b = (int)bits - 1; b >= 0; --b)
        m = (m << 3) | ((uint64_t)((x >> b) & 1) << 2) | ((uint64_t)((y >> b) & 1) << 1) | ((z >> b) & 1);
    return m;
}

uint32_t ilog2(uint32_t g) {
    uint32_t d = 0;
    while ((1u << d) < g) ++d;
    return d;
}

bool valid_params(const OracleParams& p) {
    if (p.n == 0 || p.n >= 0x80000000u) return false;
    if (p.cloud_type > 1) return false;
    uint32_t need = p.cloud_type == 0 ? 15 : 27;
    if (p.stride < need) return false;
    if (p.chunk_grid < 2 || p.chunk_grid > 512 || (p.chunk_grid & (p.chunk_grid - 1))) return false;
    if (p.sub_grid < 1 || p.sub_grid > 1024) return false;
    if ((p.flags & F_INTRA) && (p.flags & F_WEIGHT)) return false;
    if (!(p.bb_max[0] - p.bb_min[0] > 0.0)) return false;
    for (int a = 0; a < 3; ++a)
        if (!(p.scale[a] > 0.0)) return false;
    return true;
}

struct Cand {
    uint32_t key;
    uint32_t idx;
    uint16_t c[3];
    float u[3];
};

Result* build(const uint8_t* cloud, const OracleParams& P) {
    auto* R = new Result();
    OracleStats& S = R->stats;
    if (!valid_params(P)) {
        S.error = 1;
        return R;
    }
    const uint32_t T = P.threads ? P.threads : 1;
    const uint32_t N = P.n;
    const uint32_t G0 = P.chunk_grid;
    const uint32_t depth = ilog2(G0);
    const uint32_t Sg = P.sub_grid;
    const double cubic = P.bb_max[0] - P.bb_min[0];   // PointCloudInfo::cubicSize, metadata.cuh:43-46
    const double t0 = cubic / G0;                      // kernel_helpers.cuh:14
    double sf[3];
    for (int a = 0; a < 3; ++a) sf[a] = 1.0 / P.scale[a];   // octree_chunking.cu:109-111
    S.depth = depth;
    S.out_capacity = (uint64_t)((float)N * P.output_factor);   // point_cloud.cuh:24

    // ---- level tables (octree.cu:13-23): level 0 = finest grid
    std::vector<uint32_t> gsz(depth + 1);
    for (uint32_t l = 0; l <= depth; ++l) {
        gsz[l] = G0 >> l;
        S.dense_nodes += gsz[l] * gsz[l] * gsz[l];
    }
    R->level_counts.resize(depth + 1);
    for (uint32_t l = 0; l <= depth; ++l) R->level_counts[l].assign((size_t)gsz[l] * gsz[l] * gsz[l], 0u);

    // ---- counting (point_counting.cuh:29-53)
    std::vector<uint32_t> cell0(N);
    std::atomic<uint32_t> below{0};
    {
        uint32_t* c0 = R->level_counts[0].data();
        parallel_for(N, T, [&](uint64_t a, uint64_t b, uint32_t) {
            for (uint64_t i = a; i < b; ++i) {
                double p[3];
                uint16_t c[3];
                load_point(cloud + i * P.stride, P.cloud_type, p, c);
                int64_t ix = ref_axis_cell(p[0], P.bb_min[0], t0, G0);
                int64_t iy = ref_axis_cell(p[1], P.bb_min[1], t0, G0);
                int64_t iz = ref_axis_cell(p[2], P.bb_min[2], t0, G0);
                if (ix < 0 || iy < 0 || iz < 0) {
                    below.store(1);
                    cell0[i] = 0;
                    continue;
                }
                uint32_t d = (uint32_t)(ix + iy * G0 + iz * (uint64_t)G0 * G0);
                cell0[i] = d;
                __atomic_fetch_add(&c0[d], 1u, __ATOMIC_RELAXED);
            }
        });
    }
    if (below.load()) {
        S.error = 2;
        return R;
    }

    // ---- count pyramid (point_count_propagation.cuh:34-86)
    for (uint32_t l = 1; l <= depth; ++l) {
        const uint32_t g = gsz[l], gl = gsz[l - 1];
        const auto& lo = R->level_counts[l - 1];
        auto& hi = R->level_counts[l];
        parallel_for((uint64_t)g * g * g, T, [&](uint64_t a, uint64_t b, uint32_t) {
            for (uint64_t i = a; i < b; ++i) {
                uint32_t z = (uint32_t)(i / ((uint64_t)g * g)), y = (uint32_t)((i / g) % g), x = (uint32_t)(i % g);
                uint64_t s = 0;
                for (uint32_t k = 0; k < 8; ++k) {
                    uint32_t cx = 2 * x + ((k >> 2) & 1), cy = 2 * y + ((k >> 1) & 1), cz = 2 * z + (k & 1);
                    s += lo[cx + (uint64_t)cy * gl + (uint64_t)cz * gl * gl];
                }
                hi[i] = (uint32_t)s;
            }
        });
    }
    for (uint32_t l = 0; l <= depth; ++l)
        for (uint32_t v : R->level_counts[l]) S.sparse_nodes += (v > 0);

    // ---- tree (hierarchical_merging.cuh:35-122) in BFS order (potree_exporter.cu:62-96)
    auto cnt = [&](uint32_t l, uint32_t x, uint32_t y, uint32_t z) -> uint32_t {
        uint32_t g = gsz[l];
        return R->level_counts[l][x + (uint64_t)y * g + (uint64_t)z * g * g];
    };
    std::vector<TNode>& nodes = R->nodes;
    {
        TNode root{};
        root.level = depth;
        root.sub_count = cnt(depth, 0, 0, 0);
        root.parent = -1;
        for (int a = 0; a < 3; ++a) root.mn[a] = P.bb_min[a];
        for (int& c : root.child) c = -1;
        nodes.push_back(root);
        for (size_t qi = 0; qi < nodes.size(); ++qi) {
            TNode v = nodes[qi];
            bool internal = v.level >= 1 && v.sub_count >= P.merge_threshold;
            nodes[qi].internal = internal;
            nodes[qi].morton = morton3(v.x, v.y, v.z, depth - v.level);
            if (!internal) continue;
            // child bbox side: side(level) / 2, fp_subsampling.cu:16-27, tools.cu:29-61
            double side = cubic / std::pow(2.0, (double)(depth - v.level));
            double cside = side / 2.0;
            uint8_t mask = 0;
            for (uint32_t s = 0; s < 8; ++s) {
                uint32_t cx = 2 * v.x + ((s >> 2) & 1), cy = 2 * v.y + ((s >> 1) & 1), cz = 2 * v.z + (s & 1);
                uint32_t c = cnt(v.level - 1, cx, cy, cz);
                if (c == 0) continue;
                TNode ch{};
                ch.x = cx;
                ch.y = cy;
                ch.z = cz;
                ch.level = v.level - 1;
                ch.sub_count = c;
                ch.parent = (int32_t)qi;
                for (int& cc : ch.child) cc = -1;
                ch.mn[0] = (s & 4) ? v.mn[0] + cside : v.mn[0];
                ch.mn[1] = (s & 2) ? v.mn[1] + cside : v.mn[1];
                ch.mn[2] = (s & 1) ? v.mn[2] + cside : v.mn[2];
                nodes[qi].child[s] = (int32_t)nodes.size();
                mask |= (uint8_t)(1u << s);
                nodes.push_back(ch);
            }
            nodes[qi].mask = mask;
        }
    }
    S.tree_nodes = (uint32_t)nodes.size();
    if (!nodes[0].internal) S.guard_root_leaf = 1;

    // ---- leaf layout (canonical: BFS order) and statistics (octree.cu:79-132)
    std::vector<int32_t> leaf_rank(nodes.size(), -1);
    std::vector<uint32_t> leaves;
    {
        uint64_t off = 0;
        for (size_t i = 0; i < nodes.size(); ++i) {
            if (nodes[i].internal) {
                ++S.internal_nodes;
                continue;
            }
            leaf_rank[i] = (int32_t)leaves.size();
            leaves.push_back((uint32_t)i);
            nodes[i].data_idx = off;
            nodes[i].points = nodes[i].sub_count;
            off += nodes[i].sub_count;
        }
        S.leaf_nodes = (uint32_t)leaves.size();
        // DFS statistics in the reference's recursion order
        S.min_leaf_points = 0xFFFFFFFFu;
        S.max_leaf_points = 0;
        uint32_t point_sum = 0;
        std::vector<std::pair<uint32_t, uint32_t>> stack{{0u, 0u}};
        std::vector<uint32_t> dfs_leaves;
        while (!stack.empty()) {
            auto [ni, lvl] = stack.back();
            stack.pop_back();
            const TNode& v = nodes[ni];
            if (!v.internal) {
                S.max_leaf_depth = std::max(S.max_leaf_depth, lvl);
                point_sum += v.sub_count;
                S.min_leaf_points = std::min(S.min_leaf_points, v.sub_count);
                S.max_leaf_points = std::max(S.max_leaf_points, v.sub_count);
                dfs_leaves.push_back(ni);
                continue;
            }
            for (int s = 7; s >= 0; --s)
                if (v.child[s] >= 0) stack.push_back({(uint32_t)v.child[s], lvl + 1});
        }
        S.mean_leaf_points = (float)point_sum / (float)S.leaf_nodes;
        float sum_var = 0.f;
        for (uint32_t ni : dfs_leaves) {
            float d = (float)nodes[ni].sub_count - S.mean_leaf_points;
            sum_var += std::pow(d, 2.f);
        }
        S.stdev_leaf_points = std::sqrt(sum_var / (float)S.leaf_nodes);
    }

    // ---- distribution (point_distributing.cuh:30-75), stable within each leaf
    const uint32_t L = (uint32_t)leaves.size();
    std::vector<uint32_t> point_leaf(N);
    auto find_leaf = [&](uint32_t d0) -> uint32_t {
        uint32_t x = d0 % G0, y = (d0 / G0) % G0, z = d0 / (G0 * G0);
        uint32_t ni = 0;
        while (nodes[ni].internal) {
            uint32_t l = nodes[ni].level - 1;
            uint32_t s = (((x >> l) & 1) << 2) | (((y >> l) & 1) << 1) | ((z >> l) & 1);
            ni = (uint32_t)nodes[ni].child[s];
        }
        return (uint32_t)leaf_rank[ni];
    };
    uint32_t TT = std::min<uint32_t>(T, 64);
    uint64_t chunk = ((uint64_t)N + TT - 1) / TT;
    std::vector<std::vector<uint32_t>> tcount(TT, std::vector<uint32_t>(L, 0));
    parallel_for((uint64_t)TT, TT, [&](uint64_t a, uint64_t b, uint32_t) {
        for (uint64_t t = a; t < b; ++t) {
            uint64_t lo = t * chunk, hi = std::min<uint64_t>(N, lo + chunk);
            for (uint64_t i = lo; i < hi; ++i) {
                uint32_t lr = find_leaf(cell0[i]);
                point_leaf[i] = lr;
                ++tcount[t][lr];
            }
        }
    });
    for (uint32_t lr = 0; lr < L; ++lr) {
        uint64_t base = nodes[leaves[lr]].data_idx;
        for (uint32_t t = 0; t < TT; ++t) {
            uint32_t c = tcount[t][lr];
            tcount[t][lr] = (uint32_t)base;
            base += c;
        }
    }
    R->records.resize(N);
    R->lut.resize(N);
    parallel_for((uint64_t)TT, TT, [&](uint64_t a, uint64_t b, uint32_t) {
        for (uint64_t t = a; t < b; ++t) {
            uint64_t lo = t * chunk, hi = std::min<uint64_t>(N, lo + chunk);
            for (uint64_t i = lo; i < hi; ++i) {
                uint32_t pos = tcount[t][point_leaf[i]]++;
                double p[3];
                uint16_t c[3];
                load_point(cloud + i * P.stride, P.cloud_type, p, c);
                Record& r = R->records[pos];
                r.x = ref_out_coord(p[0], P.bb_min[0], sf[0]);
                r.y = ref_out_coord(p[1], P.bb_min[1], sf[1]);
                r.z = ref_out_coord(p[2], P.bb_min[2], sf[2]);
                r.r = c[0];
                r.g = c[1];
                r.b = c[2];
                R->lut[pos] = (uint32_t)i;
            }
        }
    });
    std::vector<uint32_t>().swap(point_leaf);
    std::vector<uint32_t>().swap(cell0);

    // ---- subsampling, level by level (children before parents)
    const bool intra = (P.flags & F_INTRA) != 0;
    const bool inter = !intra && (P.flags & F_INTER) != 0;
    const bool weighted = inter && (P.flags & F_WEIGHT) != 0;
    const bool literal = weighted && (P.flags & F_WEIGHT_LITERAL) != 0;
    const bool local = literal && (P.flags & F_WEIGHT_LOCAL) != 0;
    const bool reverse = literal && (P.flags & F_WEIGHT_REVERSE) != 0;
    const bool random = (P.flags & F_RANDOM) != 0;
    // reference launch extent per child slot: maxPointsPerNode * 8 threads in
    // 128-thread blocks, fp_subsampling.cuh:317-330
    uint64_t extent;
    {
        uint32_t thr = S.max_leaf_points * 8u;
        double blocks = std::ceil((double)thr / 128.0);
        double gx = blocks < 65535 ? blocks : 65535;
        double gy = std::ceil(blocks / 65535);
        extent = (uint64_t)((unsigned)gx) * (uint64_t)((unsigned)gy) * 128u;
    }
    std::vector<std::vector<uint32_t>> out_idx(nodes.size());
    std::vector<std::vector<std::array<uint16_t, 3>>> out_col(nodes.size());
    std::vector<std::vector<std::array<uint16_t, 3>>> out_col_lit(local ? nodes.size() : 0);
    std::vector<uint32_t> by_level[32];
    for (size_t i = 0; i < nodes.size(); ++i)
        if (nodes[i].internal) by_level[nodes[i].level].push_back((uint32_t)i);
    std::atomic<uint32_t> g_trunc{0}, g_over{0}, g_div0{0}, g_below{0};
    std::atomic<uint64_t> g_pin{0};
    for (uint32_t lvl = 1; lvl <= depth; ++lvl) {
        auto& list = by_level[lvl];
        parallel_dynamic(list.size(), T, [&](uint64_t li) {
            const uint32_t vi = list[li];
            const TNode& v = nodes[vi];
            const double side = cubic / std::pow(2.0, (double)(depth - v.level));   // fp_subsampling.cu:16-17
            // grid extent = cubicSize of the node box: (min.x + side) - min.x
            // (fp_subsampling.cu:38-42, metadata.cuh:66-69)
            const double t = ((v.mn[0] + side) - v.mn[0]) / Sg;                  // kernel_helpers.cuh:14
            const UAx ua[3] = {make_uax(v.mn[0], t), make_uax(v.mn[1], t), make_uax(v.mn[2], t)};
            std::vector<Cand> cands;
            cands.reserve(v.sub_count);
            for (int s = 0; s < 8; ++s) {
                int32_t ci = v.child[s];
                if (ci < 0) continue;
                const TNode& ch = nodes[ci];
                uint64_t cnt_c;
                if (!ch.internal) cnt_c = ch.sub_count;
                else cnt_c = out_idx[ci].size();
                if (cnt_c > extent) g_trunc.fetch_add(1);
                for (uint64_t k = 0; k < cnt_c; ++k) {
                    Cand cd;
                    double p[3];
                    uint16_t raw[3];
                    if (!ch.internal) {
                        cd.idx = R->lut[ch.data_idx + k];
                        load_point(cloud + (uint64_t)cd.idx * P.stride, P.cloud_type, p, raw);
                        cd.c[0] = raw[0];
                        cd.c[1] = raw[1];
                        cd.c[2] = raw[2];
                    } else {
                        cd.idx = out_idx[ci][k];
                        load_point(cloud + (uint64_t)cd.idx * P.stride, P.cloud_type, p, raw);
                        cd.c[0] = out_col[ci][k][0];
                        cd.c[1] = out_col[ci][k][1];
                        cd.c[2] = out_col[ci][k][2];
                    }
                    int64_t ix = ref_axis_cell(p[0], v.mn[0], t, Sg);
                    int64_t iy = ref_axis_cell(p[1], v.mn[1], t, Sg);
                    int64_t iz = ref_axis_cell(p[2], v.mn[2], t, Sg);
                    if (ix < 0 || iy < 0 || iz < 0) {
                        g_below.store(1);
                        ix = ix < 0 ? 0 : ix;
                        iy = iy < 0 ? 0 : iy;
                        iz = iz < 0 ? 0 : iz;
                    }
                    cd.key = (uint32_t)(ix + iy * Sg + iz * (uint64_t)Sg * Sg);
                    if (weighted)
                        for (int a = 0; a < 3; ++a)
                            cd.u[a] = point_units(p[a], P.cloud_type == 0, ua[a]);
                    cands.push_back(cd);
                }
            }
            g_pin.fetch_add(cands.size());
            std::sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) {
                return a.key != b.key ? a.key < b.key : a.idx < b.idx;
            });
            // segments = occupied cells
            std::vector<uint32_t> ukeys, seg_begin;
            for (size_t k = 0; k < cands.size(); ++k)
                if (k == 0 || cands[k].key != cands[k - 1].key) {
                    ukeys.push_back(cands[k].key);
                    seg_begin.push_back((uint32_t)k);
                }
            seg_begin.push_back((uint32_t)cands.size());
            const size_t C = ukeys.size();
            std::vector<uint64_t> intra_sum(C, 0);
            uint32_t over = 0, div0 = 0;
            if (intra || inter) {
                for (size_t j = 0; j < C; ++j) {
                    uint64_t e = 0, sr = 0, sg = 0, sb = 0;
                    for (uint32_t k = seg_begin[j]; k < seg_begin[j + 1]; ++k) {
                        e += encode_colors(cands[k].c);
                        sr += cands[k].c[0];
                        sg += cands[k].c[1];
                        sb += cands[k].c[2];
                    }
                    intra_sum[j] = e;
                    if (intra && ((seg_begin[j + 1] - seg_begin[j]) >= 1024 || sr > 0xFFFF || sg > 0xFFFF || sb > 0xFFFF))
                        ++over;
                }
            }
            auto find_cell = [&](int64_t x, int64_t y, int64_t z) -> int64_t {
                if (x < 0 || y < 0 || z < 0 || x >= Sg || y >= Sg || z >= Sg) return -1;
                uint32_t k = (uint32_t)(x + y * Sg + z * (uint64_t)Sg * Sg);
                auto it = std::lower_bound(ukeys.begin(), ukeys.end(), k);
                if (it == ukeys.end() || *it != k) return -1;
                return it - ukeys.begin();
            };
            std::vector<uint64_t> inter_sum;
            std::vector<std::array<uint64_t, 4>> wacc;
            std::vector<std::array<float, 4>> facc;
            if (inter && !weighted) {
                inter_sum.assign(C, 0);
                for (size_t j = 0; j < C; ++j) {
                    int64_t x = ukeys[j] % Sg, y = (ukeys[j] / Sg) % Sg, z = ukeys[j] / ((uint64_t)Sg * Sg);
                    uint64_t e = 0, cntn = 0, sr = 0, sg = 0, sb = 0;
                    for (int ox = -1; ox <= 1; ++ox)
                        for (int oy = -1; oy <= 1; ++oy)
                            for (int oz = -1; oz <= 1; ++oz) {
                                int64_t n = find_cell(x + ox, y + oy, z + oz);
                                if (n < 0) continue;
                                e += intra_sum[n];
                                for (uint32_t k = seg_begin[n]; k < seg_begin[n + 1]; ++k) {
                                    ++cntn;
                                    sr += cands[k].c[0];
                                    sg += cands[k].c[1];
                                    sb += cands[k].c[2];
                                }
                            }
                    inter_sum[j] = e;
                    if (cntn >= 1024 || sr > 0xFFFF || sg > 0xFFFF || sb > 0xFFFF) ++over;
                }
            }
            if (literal) {
                // The reference's own arithmetic, kernelInterCellAvgWeighted
                // (kernel_inter_cell_filtering.cuh:137-189): binary64 distance
                // from the point to the neighbour cell centre over the half
                // diagonal diag_3_3_half (fp_subsampling.cu:56-61), float exp,
                // float sums (here in one fixed order: candidates by cell, then
                // cloud index, neighbours x-major), output (u16)(sum / weight)
                // (fp_subsampling.cuh:209-217).
                facc.assign(C, {0.f, 0.f, 0.f, 0.f});
                const double diag = std::pow((t * 3) * (t * 3) * 3, 0.5) / 2.0;
                for (size_t kk = 0; kk < cands.size(); ++kk) {
                    const Cand& cd = cands[reverse ? cands.size() - 1 - kk : kk];
                    double p[3];
                    uint16_t raw[3];
                    load_point(cloud + (uint64_t)cd.idx * P.stride, P.cloud_type, p, raw);
                    int64_t x = cd.key % Sg, y = (cd.key / Sg) % Sg, z = cd.key / ((uint64_t)Sg * Sg);
                    for (int ox = -1; ox <= 1; ++ox)
                        for (int oy = -1; oy <= 1; ++oy)
                            for (int oz = -1; oz <= 1; ++oz) {
                                int64_t n = find_cell(x + ox, y + oy, z + oz);
                                if (n < 0) continue;
                                const int32_t nx = (int32_t)(x + ox), ny = (int32_t)(y + oy), nz = (int32_t)(z + oz);
                                const double dx = (v.mn[0] + nx * t + (t * 0.5)) - p[0];
                                const double dy = (v.mn[1] + ny * t + (t * 0.5)) - p[1];
                                const double dz = (v.mn[2] + nz * t + (t * 0.5)) - p[2];
                                float res = static_cast<float>(std::sqrt(dx * dx + dy * dy + dz * dz) / diag);
                                res = std::exp(-((res * res) * 10.f));
                                facc[n][0] += static_cast<float>(cd.c[0]) * res;
                                facc[n][1] += static_cast<float>(cd.c[1]) * res;
                                facc[n][2] += static_cast<float>(cd.c[2]) * res;
                                facc[n][3] += res;
                            }
                }
            }
            if (weighted && (!literal || local)) {
                wacc.assign(C, {0, 0, 0, 0});
                for (size_t k = 0; k < cands.size(); ++k) {
                    const Cand& cd = cands[k];
                    int64_t x = cd.key % Sg, y = (cd.key / Sg) % Sg, z = cd.key / ((uint64_t)Sg * Sg);
                    for (int ox = -1; ox <= 1; ++ox)
                        for (int oy = -1; oy <= 1; ++oy)
                            for (int oz = -1; oz <= 1; ++oz) {
                                int64_t n = find_cell(x + ox, y + oy, z + oz);
                                if (n < 0) continue;
                                uint32_t wq = weight_q(cd.u, (int32_t)(x + ox), (int32_t)(y + oy), (int32_t)(z + oz));
                                wacc[n][0] += (uint64_t)wq * cd.c[0];
                                wacc[n][1] += (uint64_t)wq * cd.c[1];
                                wacc[n][2] += (uint64_t)wq * cd.c[2];
                                wacc[n][3] += wq;
                            }
                }
            }
            auto& oi = out_idx[vi];
            auto& oc = out_col[vi];
            oi.resize(C);
            oc.resize(C);
            for (size_t j = 0; j < C; ++j) {
                uint32_t best = seg_begin[j];
                if (random) {
                    uint64_t bp = ~0ull;
                    for (uint32_t k = seg_begin[j]; k < seg_begin[j + 1]; ++k) {
                        uint64_t pr = ((uint64_t)rp_priority(P.seed, v.level, v.morton, cands[k].idx) << 32) | cands[k].idx;
                        if (pr < bp) {
                            bp = pr;
                            best = k;
                        }
                    }
                }
                oi[j] = cands[best].idx;
                uint16_t col[3];
                if (intra) decode_colors(intra_sum[j], col, &div0);
                else if (weighted) {
                    if (literal && !local)
                        for (int a = 0; a < 3; ++a) col[a] = static_cast<uint16_t>(facc[j][a] / facc[j][3]);
                    else
                        for (int a = 0; a < 3; ++a) col[a] = (uint16_t)(wacc[j][a] / wacc[j][3]);
                    if (local)
                        out_col_lit[vi].push_back({static_cast<uint16_t>(facc[j][0] / facc[j][3]),
                                                   static_cast<uint16_t>(facc[j][1] / facc[j][3]),
                                                   static_cast<uint16_t>(facc[j][2] / facc[j][3])});
                } else if (inter) decode_colors(inter_sum[j], col, &div0);
                else {
                    double p[3];
                    uint16_t raw[3];
                    load_point(cloud + (uint64_t)oi[j] * P.stride, P.cloud_type, p, raw);
                    col[0] = raw[0];
                    col[1] = raw[1];
                    col[2] = raw[2];
                }
                oc[j] = {col[0], col[1], col[2]};
            }
            nodes[vi].points = (uint32_t)C;
            if (over) g_over.fetch_add(over);
            if (div0) g_div0.fetch_add(div0);
        });
    }
    if (g_below.load()) {
        S.error = 2;
        return R;
    }
    S.guard_truncation = g_trunc.load();
    S.guard_color_overflow = g_over.load();
    S.guard_div0 = g_div0.load();
    S.p_in = g_pin.load();

    // ---- internal data positions: DFS post-order after the N leaf points
    //      (calculateWritingPosition, kernel_helpers.cuh:55-59)
    uint64_t pout = 0;
    {
        std::vector<std::pair<uint32_t, bool>> st{{0u, false}};
        uint64_t off = N;
        while (!st.empty()) {
            auto [ni, expanded] = st.back();
            st.pop_back();
            TNode& v = nodes[ni];
            if (!v.internal) continue;
            if (expanded) {
                v.data_idx = off;
                off += v.points;
                continue;
            }
            st.push_back({ni, true});
            for (int s = 7; s >= 0; --s)
                if (v.child[s] >= 0) st.push_back({(uint32_t)v.child[s], false});
        }
        pout = off - N;
    }
    S.p_out = pout;
    S.points_total = (uint64_t)N + pout;
    if (S.points_total > S.out_capacity) S.guard_capacity = 1;
    R->records.resize(S.points_total);
    R->lut.resize(S.points_total);
    parallel_dynamic(nodes.size(), T, [&](uint64_t ni) {
        const TNode& v = nodes[ni];
        if (!v.internal) return;
        const auto& oi = out_idx[ni];
        const auto& oc = local ? out_col_lit[ni] : out_col[ni];
        for (size_t j = 0; j < oi.size(); ++j) {
            double p[3];
            uint16_t raw[3];
            load_point(cloud + (uint64_t)oi[j] * P.stride, P.cloud_type, p, raw);
            Record& r = R->records[v.data_idx + j];
            r.x = ref_out_coord(p[0], P.bb_min[0], sf[0]);
            r.y = ref_out_coord(p[1], P.bb_min[1], sf[1]);
            r.z = ref_out_coord(p[2], P.bb_min[2], sf[2]);
            r.r = oc[j][0];
            r.g = oc[j][1];
            r.b = oc[j][2];
            R->lut[v.data_idx + j] = oi[j];
        }
    });

    // ---- hierarchy.bin (potree_exporter.cu:62-96): BFS order == node order
    R->hier.resize(nodes.size());
    for (size_t i = 0; i < nodes.size(); ++i) {
        const TNode& v = nodes[i];
        HierEntry e;
        e.mask = v.internal ? v.mask : 0;
        e.type = e.mask == 0 ? 1 : 0;
        e.points = v.points;
        e.byte_offset = v.data_idx * 18ull;
        e.byte_size = (uint64_t)v.points * 18ull;
        R->hier[i] = e;
    }
    return R;
}

}   // namespace

extern "C" {

struct OracleNodeInfo {
    uint64_t morton;
    uint64_t data_idx;
    uint32_t level;
    uint32_t points;
    uint32_t sub_count;
    uint32_t internal;
};

void* oracle_build(const uint8_t* cloud, const OracleParams* params) {
    return build(cloud, *params);
}

void oracle_free(void* h) {
    delete static_cast<Result*>(h);
}

void oracle_stats(void* h, OracleStats* out) {
    *out = static_cast<Result*>(h)->stats;
}

uint64_t oracle_node_count(void* h) {
    return static_cast<Result*>(h)->nodes.size();
}

void oracle_hierarchy(void* h, uint8_t* out) {
    auto* R = static_cast<Result*>(h);
    std::memcpy(out, R->hier.data(), R->hier.size() * sizeof(HierEntry));
}

uint64_t oracle_record_count(void* h) {
    return static_cast<Result*>(h)->records.size();
}

void oracle_records(void* h, uint8_t* out) {
    auto* R = static_cast<Result*>(h);
    std::memcpy(out, R->records.data(), R->records.size() * sizeof(Record));
}

void oracle_lut(void* h, uint32_t* out) {
    auto* R = static_cast<Result*>(h);
    std::memcpy(out, R->lut.data(), R->lut.size() * sizeof(uint32_t));
}

void oracle_nodes(void* h, OracleNodeInfo* out) {
    auto* R = static_cast<Result*>(h);
    for (size_t i = 0; i < R->nodes.size(); ++i) {
        const TNode& v = R->nodes[i];
        out[i] = {v.morton, v.data_idx, v.level, v.points, v.sub_count, v.internal};
    }
}

uint64_t oracle_level_size(void* h, uint32_t level) {
    auto* R = static_cast<Result*>(h);
    return level < R->level_counts.size() ? R->level_counts[level].size() : 0;
}

void oracle_level_counts(void* h, uint32_t level, uint32_t* out) {
    auto* R = static_cast<Result*>(h);
    std::memcpy(out, R->level_counts[level].data(), R->level_counts[level].size() * 4);
}

// Single-value helpers for boundary tests.
int64_t oracle_cell_axis(double p, double mn, double size, uint32_t grid) {
    return ref_axis_cell(p, mn, size / grid, grid);
}

int32_t oracle_out_coord(double p, double mn, double scale) {
    return ref_out_coord(p, mn, 1.0 / scale);
}

uint32_t oracle_rp_priority(uint64_t seed, uint32_t level, uint64_t morton, uint32_t idx) {
    return rp_priority(seed, level, morton, idx);
}

uint32_t oracle_weight_q(float ux, float uy, float uz, int32_t nx, int32_t ny, int32_t nz) {
    float u[3] = {ux, uy, uz};
    return weight_q(u, nx, ny, nz);
}

float oracle_exp_neg(float x) {
    return exp_neg(x);
}

}   // extern "C"

extern "C" void oracle_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    philox4x32_10(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = c[i];
}
