// Host orchestration of the LOD build.  Stage order and semantics follow
// Session::generateOctree (OctreeApi/src/session.cpp:62-70): counting
// (octree_chunking.cu:18-32), merging (:34-95), distribution (:97-124),
// subsampling (octree_processor_impl.cu:164-186).  Tree bookkeeping that the
// reference does on the host in double precision (node bounding boxes,
// fp_subsampling.cu:15-61, tools.cu:29-61) is done here the same way.
#include "builder.h"

#include <chrono>
#include "wave.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <type_traits>

namespace oc {

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(std::string(what) + ": " + cudaGetErrorString(e));
}

void BuildConfig::validate() const {
    if (n == 0) throw Error("point amount is 0");
    if (n >= 0x80000000u) throw Error("point amount must be below 2^31");
    if (cloud_type > 1) throw Error("cloud type must be 0 (float) or 1 (double)");
    uint32_t need = cloud_type == 0 ? 15u : 27u;
    if (stride < need) throw Error("data stride too small for the cloud type");
    if (chunk_grid < 2 || chunk_grid > 512 || (chunk_grid & (chunk_grid - 1)))
        throw Error("chunking grid must be a power of two in [2, 512]");
    if (sub_grid < 1 || sub_grid > 1024) throw Error("subsampling grid must be in [1, 1024]");
    if (intra && weighting) throw Error("the weighting function requires inter-cell averaging without intra-cell");
    if (has_bbox() && !(bb_max[0] - bb_min[0] > 0.0)) throw Error("empty bounding box");
    for (int a = 0; a < 3; ++a)
        if (!(scale[a] > 0.0)) throw Error("scale must be positive");
    if ((uint64_t)n * stride > (1ull << 40)) throw Error("cloud too large");
}

namespace {
std::atomic<int32_t> g_injected[3];

void allocation_hook() {
    if (consume_injected_failure(kInjectAllocation)) throw Error("cudaMalloc failed: injected allocation failure");
}

thread_local AllocTally g_alloc_tally;

// cudaMalloc with the calling thread's tally updated.
void tallied_malloc(void** p, size_t bytes) {
    const auto t0 = std::chrono::steady_clock::now();
    check_cuda(cudaMalloc(p, bytes), "cudaMalloc");
    g_alloc_tally.ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    g_alloc_tally.events += 1;
    g_alloc_tally.bytes += bytes;
}
}   // namespace

AllocTally& thread_alloc_tally() {
    return g_alloc_tally;
}

void inject_failures(int kind, uint32_t count) {
    if (kind != kInjectAllocation && kind != kInjectLaneLoss) throw Error("unknown fault kind");
    g_injected[kind].store((int32_t)std::min<uint32_t>(count, 1u << 30));
}

bool consume_injected_failure(int kind) {
    int32_t v = g_injected[kind].load();
    while (v > 0)
        if (g_injected[kind].compare_exchange_weak(v, v - 1)) return true;
    return false;
}

DevBuf::~DevBuf() {
    release();
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

void DevBuf::ensure(size_t b) {
    if (b <= bytes && p) return;
    allocation_hook();
    release();
    size_t want = std::max<size_t>(b, 256);
    tallied_malloc(&p, want);
    bytes = want;
}

void DevBuf::ensure_keep(size_t b, size_t keep, cudaStream_t s) {
    if (b <= bytes && p) return;
    allocation_hook();
    size_t want = std::max<size_t>(b + b / 4, 256);
    void* np = nullptr;
    tallied_malloc(&np, want);
    if (p && keep) check_cuda(cudaMemcpyAsync(np, p, std::min(keep, bytes), cudaMemcpyDeviceToDevice, s), "grow copy");
    check_cuda(cudaStreamSynchronize(s), "grow sync");
    release();
    p = np;
    bytes = want;
}

HostBuf::~HostBuf() {
    release();
}

void HostBuf::release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
}

void HostBuf::ensure(size_t b) {
    if (b <= bytes && p) return;
    allocation_hook();
    release();
    size_t want = std::max<size_t>(b + b / 4, 4096);
    check_cuda(cudaMallocHost(&p, want), "cudaMallocHost");
    bytes = want;
}

namespace {

uint32_t ilog2(uint32_t g) {
    uint32_t d = 0;
    while ((1u << d) < g) ++d;
    return d;
}

}   // namespace

// Reference cell formula of one axis (mapPointToGrid, kernel_helpers.cuh:14-24)
// evaluated in binary64 on the host: -1 below the bounding box.
static int host_cell(double p, double mn, double t, uint32_t grid) {
    const double u = (p - mn) / t;
    const double v = std::fmin(u, (double)grid - 1.0);
    if (!(v > -1.0)) return -1;
    return (int)(long long)v;
}

// Smallest key k in (kmin, kmax] with ge(k), for a predicate that is false at
// kmin, true at kmax and non-decreasing in between: a galloping search from
// `guess` (steps doubling away from it) that ends in a bisection.  It returns
// the same key as a bisection over the whole range (checked on 3000 random
// boxes and grids), in a few steps instead of 64 when the guess is close.
template <class K, class Pred>
static K first_key(K kmin, K kmax, K guess, Pred ge) {
    using U = typename std::make_unsigned<K>::type;
    if (guess <= kmin) guess = kmin + 1;
    if (guess > kmax) guess = kmax;
    K lo, hi;   // ge(lo) false (or lo == kmin), ge(hi) true
    if (ge(guess)) {
        hi = guess;
        U step = 1;
        for (;;) {
            if ((U)(hi - kmin) <= step) {
                lo = kmin;
                break;
            }
            const K c = (K)(hi - (K)step);
            if (!ge(c)) {
                lo = c;
                break;
            }
            hi = c;
            step <<= 1;
        }
    } else {
        lo = guess;
        U step = 1;
        for (;;) {
            if ((U)(kmax - lo) <= step) {
                hi = kmax;
                break;
            }
            const K c = (K)(lo + (K)step);
            if (ge(c)) {
                hi = c;
                break;
            }
            lo = c;
            step <<= 1;
        }
    }
    while ((U)(hi - lo) > 1) {
        const K mid = (K)(lo + (K)((U)(hi - lo) / 2));
        if (ge(mid)) hi = mid;
        else lo = mid;
    }
    return hi;
}

// The cell is a non-decreasing function of the coordinate, hence of its
// ordered key: each boundary is the first key whose cell reaches i, searched
// from the key of mn + i * t.
void make_cell_keys64(double mn, double t, uint32_t grid, int64_t* keys) {
    const int64_t kmin = host_key64(-INFINITY), kmax = host_key64(INFINITY);
    for (uint32_t i = 0; i < grid; ++i) {
        const double p0 = mn + (double)i * t;
        const int64_t guess = std::isfinite(p0) ? host_key64(p0) : kmin + 1;
        keys[i] = first_key<int64_t>(kmin, kmax, guess,
                                     [&](int64_t k) { return host_cell(host_from_key64(k), mn, t, grid) >= (int)i; });
    }
    keys[grid] = keys[grid + 1] = INT64_MAX;
}

void make_cell_keys32(double mn, double t, uint32_t grid, int32_t* keys) {
    const int32_t kmin = host_key32(-INFINITY), kmax = host_key32(INFINITY);
    for (uint32_t i = 0; i < grid; ++i) {
        const double p0 = mn + (double)i * t;
        const int32_t guess = std::isfinite((float)p0) ? host_key32((float)p0) : kmin + 1;
        keys[i] = first_key<int32_t>(kmin, kmax, guess, [&](int32_t k) {
            return host_cell((double)host_from_key32(k), mn, t, grid) >= (int)i;
        });
    }
    keys[grid] = keys[grid + 1] = INT32_MAX;
}

Builder::Builder(const BuildConfig& cfg, const uint8_t* host_cloud, int device, bool count)
    : cfg_(cfg), device_(device) {
    cfg_.validate();
    check_cuda(cudaSetDevice(device_), "cudaSetDevice");
    check_cuda(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device_), "device attribute");
    check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
    check_cuda(cudaStreamCreateWithFlags(&side_stream_, cudaStreamNonBlocking), "stream");
    check_cuda(cudaEventCreateWithFlags(&tree_ready_, cudaEventDisableTiming), "event");
    check_cuda(cudaEventCreateWithFlags(&params_done_, cudaEventDisableTiming), "event");
    size_for_config();
    upload(host_cloud, true, count);
}

// A new cloud and configuration on the same device state: every buffer only
// grows, so a builder that has served larger builds allocates nothing.
void Builder::reconfigure(const BuildConfig& cfg, const uint8_t* host_cloud, bool wait_upload, bool count) {
    cfg.validate();
    tree_valid_ = false;
    reuse_tree_ = false;
    bbox_from_device_ = false;
    if (copy_stream_) check_cuda(cudaStreamSynchronize(copy_stream_), "output copies");
    const bool adopt = prefetched_ && prefetched_ == host_cloud && prefetched_bytes_ == (uint64_t)cfg.n * cfg.stride;
    prefetched_ = nullptr;
    if (adopt) {
        // the spare buffer becomes the cloud; the old cloud buffer is free for
        // the next prefetch once the work queued on the build stream is done
        std::swap(cloud_.p, spare_.p);
        std::swap(cloud_.bytes, spare_.bytes);
        check_cuda(cudaEventRecord(spare_free_, stream_), "event");
    }
    cfg_ = cfg;
    host_rec_ = nullptr;
    host_lut_ = nullptr;
    host_cap_ = 0;
    host_filled_ = false;
    nodes_.clear();
    stats_ = Stats{};
    size_for_config();
    if (!adopt) {
        upload(host_cloud, wait_upload, count);
        return;
    }
    counted_ = false;
    check_cuda(cudaStreamWaitEvent(stream_, prefetch_done_, 0), "wait");
    if (wait_upload) check_cuda(cudaStreamSynchronize(stream_), "upload sync");
}

void Builder::prefetch(const uint8_t* host_cloud, uint64_t bytes) {
    prefetch_sync();
    if (!prefetch_stream_) {
        check_cuda(cudaStreamCreateWithFlags(&prefetch_stream_, cudaStreamNonBlocking), "stream");
        check_cuda(cudaEventCreateWithFlags(&prefetch_done_, cudaEventDisableTiming), "event");
        check_cuda(cudaEventCreateWithFlags(&spare_free_, cudaEventDisableTiming), "event");
    }
    if (spare_.bytes < bytes + 64) {
        check_cuda(cudaStreamSynchronize(prefetch_stream_), "prefetch");
        spare_.ensure(bytes + 64);   // same padding as the cloud buffer
    }
    check_cuda(cudaStreamWaitEvent(prefetch_stream_, spare_free_, 0), "wait");
    check_cuda(cudaMemcpyAsync(spare_.p, host_cloud, bytes, cudaMemcpyHostToDevice, prefetch_stream_), "prefetch");
    check_cuda(cudaEventRecord(prefetch_done_, prefetch_stream_), "event");
    prefetched_ = host_cloud;
    prefetched_bytes_ = bytes;
}

void Builder::prefetch_sync() {
    if (prefetch_stream_) check_cuda(cudaStreamSynchronize(prefetch_stream_), "prefetch");
    prefetched_ = nullptr;
}

// The staged parameter tables may be rewritten once their last upload is done.
void Builder::params_writable() {
    if (params_pending_) check_cuda(cudaEventSynchronize(params_done_), "parameter upload");
    params_pending_ = false;
}

void Builder::record_params() {
    check_cuda(cudaEventRecord(params_done_, stream_), "event");
    params_pending_ = true;
}

void Builder::size_for_config() {
    depth_ = ilog2(cfg_.chunk_grid);
    level_off_.assign(depth_ + 2, 0);
    for (uint32_t l = 0; l <= depth_; ++l) {
        uint64_t g = cfg_.chunk_grid >> l;
        level_off_[l + 1] = level_off_[l] + g * g * g;
    }
    uint64_t cap = 1;
    uint64_t per = cfg_.n / std::max<uint32_t>(cfg_.threshold, 1);
    for (uint32_t l = 1; l <= depth_; ++l) {
        uint64_t g = cfg_.chunk_grid >> l;
        cap += 8 * std::min<uint64_t>(g * g * g, per);
    }
    node_cap_ = (uint32_t)std::min<uint64_t>(cap, level_off_[depth_ + 1]);

    {
        // a new pyramid or bitmap allocation holds garbage: the next build
        // clears it in full
        const void* old_pyr = pyr_.p;
        const void* old_occ = occ_.p;
        pyr_.ensure(level_off_[depth_ + 1] * 4);
        occ_.ensure(std::max<uint64_t>(level_off_[1] >> 6, 1));
        if (pyr_.p != old_pyr || occ_.p != old_occ) pyr_zero_ = false;
    }
    loff_.ensure(level_off_.size() * 8);
    params_writable();
    loff_host_.ensure(level_off_.size() * 8);
    std::memcpy(loff_host_.p, level_off_.data(), level_off_.size() * 8);
    check_cuda(cudaMemcpyAsync(loff_.p, loff_host_.p, level_off_.size() * 8, cudaMemcpyHostToDevice, stream_),
               "H2D loff");
    err_.ensure(64);
    nonzero_.ensure((depth_ + 1) * 4);
    key_.ensure((size_t)node_cap_ * 4);
    count_.ensure((size_t)node_cap_ * 4);
    level_.ensure((size_t)node_cap_);
    info_.ensure((size_t)node_cap_ * 2);
    child_first_.ensure((size_t)node_cap_ * 4);
    data_idx_.ensure((size_t)node_cap_ * 8);
    fill_.ensure((size_t)node_cap_ * 4);
    level_start_.ensure((depth_ + 2) * 4);
    n_nodes_.ensure(4);
    if (cfg_.has_bbox()) fill_cell_tables();
    record_params();
    cloud_.ensure((size_t)cfg_.n * cfg_.stride + 64);
    lut_.ensure((size_t)cfg_.n * 4);
    rec_.ensure((size_t)cfg_.n * 18 + 16);   // 16 readable bytes past the last record
    leaf_frac_.ensure((size_t)cfg_.n * 4);
}

// Exact boundary keys of the chunking grid for the current bounding box, and
// the Morton spread table, staged and copied on the build stream (the staging
// must be writable: params_writable).
void Builder::fill_cell_tables() {
    const uint32_t G = cfg_.chunk_grid;
    const double t0 = (cfg_.bb_max[0] - cfg_.bb_min[0]) / G;   // kernel_helpers.cuh:14
    const size_t kb = (size_t)3 * (G + 2) * (cfg_.cloud_type == 0 ? 4 : 8);
    keys_host_.ensure(kb);
    if (cfg_.cloud_type == 0) {
        for (int a = 0; a < 3; ++a) make_cell_keys32(cfg_.bb_min[a], t0, G, keys_host_.as<int32_t>() + a * (G + 2));
    } else {
        for (int a = 0; a < 3; ++a) make_cell_keys64(cfg_.bb_min[a], t0, G, keys_host_.as<int64_t>() + a * (G + 2));
    }
    cell_keys_.ensure(kb);
    check_cuda(cudaMemcpyAsync(cell_keys_.p, keys_host_.p, kb, cudaMemcpyHostToDevice, stream_), "H2D keys");
    if (spread_grid_ != G) {
        spread_host_.ensure(G * 4);
        for (uint32_t i = 0; i < G; ++i) spread_host_.as<uint32_t>()[i] = spread3(i);
        spread_.ensure(G * 4);
        check_cuda(cudaMemcpyAsync(spread_.p, spread_host_.p, G * 4, cudaMemcpyHostToDevice, stream_), "H2D spread");
        spread_grid_ = G;
    }
}

// calculateRealBB + calculateCubicBB (src/boundingbox.h:11-52) over the
// uploaded cloud; the cubic box becomes the build's bounding box.
void Builder::compute_bbox(double real[6], double cubic[6]) {
    TraceRange trace("bounding box");
    tree_valid_ = false;
    counted_ = false;   // the box changes: any counts of an overlapped upload are void
    reuse_tree_ = false;
    bbox_keys_.ensure(6 * 8);
    launches_ = 0;
    launch_bbox(cloud_.as<uint8_t>(), cfg_.n, cfg_.stride, cfg_.cloud_type == 0, bbox_keys_.as<long long>(), num_sms_,
                stream_);
    long long k[6];
    check_cuda(cudaMemcpyAsync(k, bbox_keys_.p, sizeof k, cudaMemcpyDeviceToHost, stream_), "D2H bbox");
    check_cuda(cudaStreamSynchronize(stream_), "bbox");
    for (int a = 0; a < 6; ++a) {
        const bool lo = a < 3;
        if (k[a] == (lo ? INT64_MAX : INT64_MIN)) {   // no finite coordinate on this axis
            real[a] = lo ? INFINITY : -INFINITY;
            continue;
        }
        real[a] = cfg_.cloud_type == 0 ? (double)host_from_key32((int32_t)k[a]) : host_from_key64((int64_t)k[a]);
    }
    const double dx = real[3] - real[0], dy = real[4] - real[1], dz = real[5] - real[2];
    const double side = std::fmax(std::fmax(dx, dy), dz);
    cubic[0] = real[0] - ((side - dx) / 2.0f);
    cubic[1] = real[1] - ((side - dy) / 2.0f);
    cubic[2] = real[2] - ((side - dz) / 2.0f);
    cubic[3] = cubic[0] + side;
    cubic[4] = cubic[1] + side;
    cubic[5] = cubic[2] + side;
    for (int a = 0; a < 3; ++a) {
        cfg_.bb_min[a] = cubic[a];
        cfg_.bb_max[a] = cubic[a + 3];
    }
    cfg_.validate();
    params_writable();
    fill_cell_tables();
    record_params();
    bbox_from_device_ = true;
}

bool Builder::reuse(const BuildConfig& c) {
    if (!tree_valid_) return false;
    c.validate();
    const BuildConfig& r = cfg_;
    bool same = c.n == r.n && c.stride == r.stride && c.cloud_type == r.cloud_type && c.chunk_grid == r.chunk_grid &&
                c.threshold == r.threshold && c.debug == r.debug;
    for (int a = 0; a < 3; ++a) same = same && c.scale[a] == r.scale[a];
    if (c.has_bbox()) {
        for (int a = 0; a < 3; ++a) same = same && c.bb_min[a] == r.bb_min[a] && c.bb_max[a] == r.bb_max[a];
    } else {
        same = same && bbox_from_device_;
    }
    if (!same) return false;
    if (copy_stream_) check_cuda(cudaStreamSynchronize(copy_stream_), "output copies");
    cfg_.output_factor = c.output_factor;
    cfg_.sub_grid = c.sub_grid;
    cfg_.intra = c.intra;
    cfg_.inter = c.inter;
    cfg_.replacement = c.replacement;
    cfg_.random = c.random;
    cfg_.weighting = c.weighting;
    cfg_.seed = c.seed;
    host_rec_ = nullptr;
    host_lut_ = nullptr;
    host_cap_ = 0;
    host_filled_ = false;
    reuse_tree_ = true;
    return true;
}

Builder::~Builder() {
    if (level_ready_) cudaEventDestroy(level_ready_);
    if (prefetch_stream_) cudaStreamSynchronize(prefetch_stream_);
    if (prefetch_done_) cudaEventDestroy(prefetch_done_);
    if (spare_free_) cudaEventDestroy(spare_free_);
    if (prefetch_stream_) cudaStreamDestroy(prefetch_stream_);
    if (side_stream_) cudaStreamSynchronize(side_stream_);
    if (tree_ready_) cudaEventDestroy(tree_ready_);
    if (side_stream_) cudaStreamDestroy(side_stream_);
    if (params_done_) cudaEventDestroy(params_done_);
    for (auto e : chunk_ready_) cudaEventDestroy(e);
    if (copy_stream_) cudaStreamSynchronize(copy_stream_);
    if (leaf_ready_) cudaEventDestroy(leaf_ready_);
    if (copy_stream_) cudaStreamDestroy(copy_stream_);
    for (auto e : event_pool_) cudaEventDestroy(e);
    if (stream_) cudaStreamDestroy(stream_);
}

void Builder::stage_begin() {
    events_.clear();
    stage_mark("begin");
}

void Builder::stage_mark(const char* name) {
    size_t i = events_.size();
    while (event_pool_.size() <= i) {
        cudaEvent_t e;
        check_cuda(cudaEventCreate(&e), "event");
        event_pool_.push_back(e);
    }
    check_cuda(cudaEventRecord(event_pool_[i], stream_), "event record");
    events_.push_back({name, event_pool_[i]});
}

void Builder::collect_timings() {
    timings_.clear();
    for (size_t i = 1; i < events_.size(); ++i) {
        float ms = 0;
        check_cuda(cudaEventElapsedTime(&ms, events_[i - 1].second, events_[i].second), "event time");
        timings_.push_back({events_[i].first, ms});
    }
}

std::vector<std::pair<std::string, uint64_t>> Builder::device_allocations() const {
    return {
        {"cloud", cloud_.bytes + spare_.bytes},
        {"count pyramid", pyr_.bytes + occ_.bytes},
        {"node table", key_.bytes + count_.bytes + level_.bytes + info_.bytes + child_first_.bytes +
                           data_idx_.bytes + fill_.bytes + level_start_.bytes + n_nodes_.bytes + loff_.bytes +
                           nonzero_.bytes},
        {"octree.bin records", rec_.bytes},
        {"LUT", lut_.bytes},
        {"staged records", stage_rec_.bytes},
        {"staged LUT", stage_lut_.bytes},
        {"sub-step words", leaf_frac_.bytes + stage_frac_.bytes},
        {"subsampling scratch", key_cache_.bytes + unit_cache_.bytes + acc_best_.bytes + acc_sel_.bytes +
                                    cell_slot_.bytes + acc_intra_.bytes + emit_maps_.bytes + emit_state_.bytes + csr_count_.bytes +
                                    csr_start_.bytes + csr_pts_.bytes},
        {"brick tables", g_key_.bytes + g_mask_.bytes + g_base_.bytes},
        {"level tables", sub_nodes_.bytes + out_points_.bytes + stage_off_.bytes + post_ii_.bytes + node_dst_.bytes +
                             place_src_.bytes + place_dst_.bytes + place_cnt_.bytes},
        {"small", err_.bytes + work_.bytes + cell_keys_.bytes + spread_.bytes + bbox_keys_.bytes + level_base_.bytes +
                      out_total_.bytes},
    };
}

// Mirrors the sizing in Builder::Builder, generate() and subsample():
// data-dependent buffers at their capacity rules (node capacity, staging and
// final records at max(outputFactor * N, N), scratch at the staging capacity).
// Every buffer's size is non-decreasing in each term, so the envelope of two
// term sets bounds a builder that was reconfigured from one to the other.
MemoryTerms memory_terms(const BuildConfig& c, int num_sms) {
    MemoryTerms t;
    const uint32_t depth = ilog2(c.chunk_grid);
    for (uint32_t l = 0; l <= depth; ++l) {
        const uint64_t g = c.chunk_grid >> l;
        t.cells += g * g * g;
    }
    uint64_t cap = 1;
    const uint64_t per = c.n / std::max<uint32_t>(c.threshold, 1);
    for (uint32_t l = 1; l <= depth; ++l) {
        const uint64_t g = c.chunk_grid >> l;
        cap += 8 * std::min<uint64_t>(g * g * g, per);
    }
    t.node_cap = std::min<uint64_t>(cap, t.cells);
    t.out_cap = std::max<uint64_t>((uint64_t)((float)c.n * c.output_factor), c.n);
    t.n = c.n;
    t.cloud_bytes = (uint64_t)c.n * c.stride;
    t.chunk_grid = c.chunk_grid;
    const bool intra = c.intra, inter = !intra && c.inter, weighted = inter && c.weighting;
    t.random = c.random;
    t.packed = (intra || inter) && !weighted;
    t.weighted = weighted;
    const uint64_t bs = (c.sub_grid + 3) / 4;
    const uint64_t bricks = std::min<uint64_t>(t.out_cap, bs * bs * bs);
    t.slots = 1024;
    while (t.slots * 11 / 16 < bricks + 1) t.slots <<= 1;
    t.sms = std::max(num_sms, 1);
    return t;
}

MemoryTerms envelope(const MemoryTerms& a, const MemoryTerms& b) {
    MemoryTerms t;
    t.cloud_bytes = std::max(a.cloud_bytes, b.cloud_bytes);
    t.n = std::max(a.n, b.n);
    t.cells = std::max(a.cells, b.cells);
    t.node_cap = std::max(a.node_cap, b.node_cap);
    t.out_cap = std::max(a.out_cap, b.out_cap);
    t.slots = std::max(a.slots, b.slots);
    t.chunk_grid = std::max(a.chunk_grid, b.chunk_grid);
    t.random = a.random || b.random;
    t.packed = a.packed || b.packed;
    t.weighted = a.weighted || b.weighted;
    t.sms = std::max(a.sms, b.sms);
    return t;
}

uint64_t device_bytes(const MemoryTerms& t) {
    if (!t.n) return 0;
    uint64_t per_cand = 4 + 8 + 4;       // key cache, selection key, cell list
    if (t.random) per_cand += 4;         // selected candidate
    if (t.packed) per_cand += 8;         // packed colour sums
    if (t.weighted) per_cand += 12 + 4 + 4 + 20;   // cell units, cell groups
    uint64_t b = 0;
    b += t.cloud_bytes + 64;                                           // cloud
    b += t.cells * 4;                                                  // count pyramid
    b += t.cells / 64 + 1;                                             // occupancy flags of finest-level blocks
    b += t.node_cap * (4 + 4 + 1 + 2 + 4 + 4 + 8 + 4);                 // node table, leaf lists, fill
    b += t.out_cap * (4 + 18) + 16;                                    // final LUT + records
    b += t.out_cap * (4 + 18 + 4) + 64;                                // staged LUT + records + sub-step words
    b += t.n * 4;                                                      // leaf sub-step words
    b += t.out_cap * per_cand;                                         // subsampling scratch
    b += (uint64_t)t.sms * t.slots * 16;                               // per-block brick tables
    if (t.weighted) b += (uint64_t)kSplitEmitNodes * (kBrickMapBytes + 16);   // handed-over brick maps
    b += t.node_cap * (sizeof(SubNode) + 4 + 8 + 4 + 8 + 8 + 8 + 4);   // level tables, placement lists
    b += 3 * (t.chunk_grid + 2) * 8 + t.chunk_grid * 4 + 64 * 256;    // keys, spread, small buffers
    return b;
}

uint64_t estimate_device_bytes(const BuildConfig& c, int num_sms) {
    return device_bytes(memory_terms(c, num_sms));
}

// tools/memory_consumption.py:30-75 (countingGrid + denseToSparseLUT +
// tmpCounting + randomIndices + randomStates + averagingGrid + outputBuffer +
// pointCloud + pointLut), with the configured chunking grid where the script
// hard-codes 512, extended by the sparse node array (64 B per occupied cell,
// bounded by the dense cell count and by N), a 4-byte counter per node and
// the f32 RGBA grid of weighted averaging.
uint64_t reference_estimate_bytes(const BuildConfig& c) {
    const uint32_t depth = ilog2(c.chunk_grid);
    uint64_t cells = 0;
    for (uint32_t l = 0; l <= depth; ++l) {
        const uint64_t g = c.chunk_grid >> l;
        cells += g * g * g;
    }
    const double S3 = (double)c.sub_grid * c.sub_grid * c.sub_grid;
    double b = 0;
    b += 2.0 * cells * 4;                                   // countingGrid + denseToSparseLUT
    b += 4;                                                 // tmpCounting
    b += 4 * S3 + 48 * 1024;                                // randomIndices + randomStates
    b += 8 * S3;                                            // averagingGrid
    if (c.weighting) b += 16 * S3;                          // RGBA averaging grid
    b += (double)c.n * 18 * c.output_factor;                // outputBuffer
    b += (double)c.n * c.stride;                            // pointCloud
    b += (double)c.n * c.output_factor * 4;                 // pointLut
    b += std::min<double>((double)cells, (double)c.n) * (64 + 4);   // sparse nodes + per-node counters
    return (uint64_t)b;
}

void Builder::set_output_host(uint8_t* records, uint32_t* lut, uint64_t capacity) {
    if (copy_stream_) check_cuda(cudaStreamSynchronize(copy_stream_), "output copies");
    host_rec_ = records;
    host_lut_ = records ? lut : nullptr;
    host_cap_ = records ? capacity : 0;
    host_filled_ = false;
    if (records && !copy_stream_) {
        check_cuda(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking), "stream");
        check_cuda(cudaEventCreateWithFlags(&leaf_ready_, cudaEventDisableTiming), "event");
    }
}

void Builder::upload(const uint8_t* host_cloud, bool wait, bool count) {
    TraceRange trace("upload");
    if (!host_cloud) throw Error("no point cloud set");
    tree_valid_ = false;
    reuse_tree_ = false;
    counted_ = false;
    // up to 16 chunks of at least 64 MB: a large cloud's counting overlaps
    // its upload, a small cloud's upload is one copy and one counting launch
    constexpr uint64_t kChunkAlign = 1024;   // chunk starts: a multiple of the counting tile (16-byte aligned)
    constexpr uint64_t kMinChunkBytes = 64ull << 20;
    const uint32_t kChunks =
        (uint32_t)std::min<uint64_t>(16, std::max<uint64_t>(1, (uint64_t)cfg_.n * cfg_.stride / kMinChunkBytes));
    if (count && cfg_.has_bbox() && cfg_.n >= 4 * kChunkAlign) {
        const bool sparse = sparse_cloud();
        while (chunk_ready_.size() < kChunks) {
            cudaEvent_t e;
            check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
            chunk_ready_.push_back(e);
        }
        stage_begin();
        clear_for_count(sparse);
        const CloudGrid g = cloud_grid();
        const uint64_t per = ((cfg_.n + kChunks - 1) / kChunks + kChunkAlign - 1) / kChunkAlign * kChunkAlign;
        uint32_t k = 0;
        for (uint64_t first = 0; first < cfg_.n; first += per, ++k) {
            const uint64_t cnt = std::min<uint64_t>(per, cfg_.n - first);
            const size_t off = (size_t)first * cfg_.stride;
            check_cuda(cudaMemcpyAsync(cloud_.as<uint8_t>() + off, host_cloud + off, (size_t)cnt * cfg_.stride,
                                       cudaMemcpyHostToDevice, side_stream_),
                       "cloud upload");
            check_cuda(cudaEventRecord(chunk_ready_[k], side_stream_), "event");
            check_cuda(cudaStreamWaitEvent(stream_, chunk_ready_[k], 0), "wait");
            launch_count(cloud_.as<uint8_t>() + off, cnt, cfg_.stride, cfg_.cloud_type == 0, g, pyr_.as<uint32_t>(),
                         sparse ? occ_.as<uint8_t>() : nullptr, err_.as<uint32_t>(), num_sms_, stream_);
        }
        check_cuda(cudaGetLastError(), "count launch");
        stage_mark("upload_count");
        counted_ = true;
        if (wait) check_cuda(cudaStreamSynchronize(side_stream_), "upload sync");
        return;
    }
    if (!wait) {
        check_cuda(cudaMemcpyAsync(cloud_.p, host_cloud, (size_t)cfg_.n * cfg_.stride, cudaMemcpyHostToDevice, stream_),
                   "cloud upload");
        return;
    }
    stage_begin();
    check_cuda(cudaMemcpyAsync(cloud_.p, host_cloud, (size_t)cfg_.n * cfg_.stride, cudaMemcpyHostToDevice, stream_),
               "cloud upload");
    stage_mark("upload");
    check_cuda(cudaStreamSynchronize(stream_), "upload sync");
    collect_timings();
}

void Builder::check_device_errors(const char* stage) {
    uint32_t e = 0;
    check_cuda(cudaMemcpyAsync(&e, err_.p, 4, cudaMemcpyDeviceToHost, stream_), "D2H err");
    check_cuda(cudaStreamSynchronize(stream_), stage);
    throw_device_errors(e, stage);
}

void throw_device_errors(uint32_t e, const char* stage) {
    if (e & kErrBelowBox) throw Error(std::string(stage) + ": a point lies below the bounding box");
    if (e & kErrCoordRange) throw Error(std::string(stage) + ": an output coordinate does not fit int32");
    if (e & kErrProbe) throw Error(std::string(stage) + ": subsampling brick table overflow");
    if (e & kErrNodeCap) throw Error(std::string(stage) + ": node capacity exceeded");
    if (e & kErrCapacity) throw Error(std::string(stage) + ": output capacity exceeded");
    if (e & kErrTag) throw Error(std::string(stage) + ": a point found no leaf");
    if (e & kErrTimeout) throw Error(std::string(stage) + ": a bulk copy did not complete in time");
}

CloudGrid Builder::cloud_grid() const {
    const double cubic = cfg_.bb_max[0] - cfg_.bb_min[0];
    CloudGrid g;
    g.grid = cfg_.chunk_grid;
    const double t0 = cubic / cfg_.chunk_grid;   // kernel_helpers.cuh:14
    for (int a = 0; a < 3; ++a) {
        g.ax[a] = make_axis(cfg_.bb_min[a], t0);
        g.r[a] = (float)(1.0 / t0);
        g.c[a] = (float)(-cfg_.bb_min[a] / t0);
    }
    g.keys = cell_keys_.p;
    g.spread = spread_.as<uint32_t>();
    return g;
}

// Sparse clouds (at most one point per 16 finest cells) flag the 64-cell
// blocks of the finest level they touch (one byte per block): counting sets
// the flags, the pyramid and the tag push skip unflagged blocks, and the build
// ends by zeroing only the flagged blocks and the upper levels, so the next
// build finds the pyramid zero.  Denser clouds clear the whole pyramid first.
bool Builder::sparse_cloud() const {
    return depth_ >= 2 && (uint64_t)cfg_.n * 16 <= level_off_[1];
}

// What counting accumulates into, cleared on the build stream.  A sparse
// build relies on the whole allocation being zero (a build on another grid
// may have written beyond this grid's levels), so its full clear covers the
// whole pyramid and flag allocations; a dense build clears its own levels.
void Builder::clear_for_count(bool sparse) {
    if (!sparse) {
        check_cuda(cudaMemsetAsync(pyr_.p, 0, level_off_[depth_ + 1] * 4, stream_), "memset");
    } else if (!pyr_zero_) {
        check_cuda(cudaMemsetAsync(pyr_.p, 0, pyr_.bytes, stream_), "memset");
        check_cuda(cudaMemsetAsync(occ_.p, 0, occ_.bytes, stream_), "memset");
    }
    pyr_zero_ = false;
    check_cuda(cudaMemsetAsync(err_.p, 0, 64, stream_), "memset");
    check_cuda(cudaMemsetAsync(nonzero_.p, 0, (depth_ + 1) * 4, stream_), "memset");
}

void Builder::generate() {
    TraceRange trace(reuse_tree_ ? "generate (resident tree)" : "generate");
    host_filled_ = false;
    sub_err_valid_ = false;
    if (reuse_tree_) {
        // the cloud, pyramid, tree and leaf records of this configuration are
        // on the device: subsample them with the new settings
        reuse_tree_ = false;
        tree_valid_ = false;
        if (host_rec_ && host_cap_ < cfg_.n) throw Error("output host buffer holds fewer records than the cloud");
        stage_begin();
        launches_ = 0;
        subsample();
        check_cuda(cudaGetLastError(), "launch");
        if (sub_err_valid_) throw_device_errors(sub_err_, "generate");
        else check_device_errors("generate");
        collect_timings();
        compute_stats();
        tree_valid_ = true;
        return;
    }
    tree_valid_ = false;
    if (!cfg_.has_bbox()) throw Error("no bounding box: call ocpi_set_cloud_bb before ocpi_init_octree or ocpi_compute_cloud_bb after it");
    if (host_rec_ && host_cap_ < cfg_.n) throw Error("output host buffer holds fewer records than the cloud");
    const CloudGrid g = cloud_grid();
    OutParams op;
    for (int a = 0; a < 3; ++a) op.ax[a] = make_out_axis(cfg_.bb_min[a], 1.0 / cfg_.scale[a]);   // octree_chunking.cu:109-111
    const bool f32 = cfg_.cloud_type == 0;
    const uint64_t cells0 = level_off_[1];
    const bool sparse = sparse_cloud();
    const uint64_t occ_blocks = cells0 >> 6;
    uint8_t* occ = sparse ? occ_.as<uint8_t>() : nullptr;
    launches_ = 0;
    if (counted_) {
        // binned during the upload (overlapped with the copy); the stage
        // events of that upload stay the first of this build
        counted_ = false;
    } else {
        stage_begin();
        clear_for_count(sparse);
        stage_mark("clear");
        launches_ += launch_count(cloud_.as<uint8_t>(), cfg_.n, cfg_.stride, f32, g, pyr_.as<uint32_t>(), occ,
                                  err_.as<uint32_t>(), num_sms_, stream_);
        stage_mark("count");
    }
    launches_ += launch_pyramid(pyr_.as<uint32_t>(), level_off_.data(), depth_, nonzero_.as<uint32_t>(), occ, stream_);
    stage_mark("pyramid");
    launches_ += launch_enumerate(pyr_.as<uint32_t>(), loff_.as<uint64_t>(), depth_, cfg_.threshold, key_.as<uint32_t>(),
                     count_.as<uint32_t>(), level_.as<uint8_t>(), info_.as<uint16_t>(), child_first_.as<uint32_t>(),
                     node_cap_, level_start_.as<uint32_t>(), n_nodes_.as<uint32_t>(), err_.as<uint32_t>(), stream_);
    stage_mark("tree");
    check_cuda(cudaGetLastError(), "launch");
    check_cuda(cudaEventRecord(tree_ready_, stream_), "event");
    if (cfg_.debug & 1) {
        // copy of the count pyramid before the leaf tags overwrite cells
        check_device_errors("counting");
        pyramid_copy_.assign(depth_ + 1, {});
        std::vector<uint32_t> tmp;
        for (uint32_t l = 0; l <= depth_; ++l) {
            uint64_t sz = level_off_[l + 1] - level_off_[l];
            uint32_t gl = cfg_.chunk_grid >> l;
            tmp.resize(sz);
            check_cuda(cudaMemcpy(tmp.data(), pyr_.as<uint32_t>() + level_off_[l], sz * 4, cudaMemcpyDeviceToHost),
                       "D2H pyramid");
            auto& dst = pyramid_copy_[l];
            dst.resize(sz);
            for (uint32_t z = 0; z < gl; ++z)
                for (uint32_t y = 0; y < gl; ++y)
                    for (uint32_t x = 0; x < gl; ++x)
                        dst[x + (uint64_t)y * gl + (uint64_t)z * gl * gl] = tmp[morton3(x, y, z)];
        }
    }

    // leaf offsets and tags, then distribution: no host round trip; the host
    // reads the node table on the side stream meanwhile
    launches_ += launch_leaf_prep(n_nodes_.as<uint32_t>(), info_.as<uint16_t>(), count_.as<uint32_t>(),
                                  level_.as<uint8_t>(), key_.as<uint32_t>(), pyr_.as<uint32_t>(), loff_.as<uint64_t>(),
                                  data_idx_.as<uint64_t>(), fill_.as<uint32_t>(), cfg_.n, err_.as<uint32_t>(), stream_);
    launches_ += launch_push_tags(pyr_.as<uint32_t>(), loff_.as<uint64_t>(), depth_, cfg_.chunk_grid, occ,
                                  err_.as<uint32_t>(), stream_);
    launches_ += launch_distribute(cloud_.as<uint8_t>(), cfg_.n, cfg_.stride, f32, g, op, pyr_.as<uint32_t>(),
                                   data_idx_.as<uint64_t>(), fill_.as<uint32_t>(), lut_.as<uint32_t>(),
                                   rec_.as<uint8_t>(), leaf_frac_.as<uint32_t>(), err_.as<uint32_t>(), num_sms_,
                                   stream_);
    stage_mark("distribute");
    check_cuda(cudaGetLastError(), "launch");
    build_tree_host();

    subsample();   // also places the internal nodes' records (stage marks "sub_l*", "place")
    check_cuda(cudaGetLastError(), "launch");
    // every kernel that reports errors ran before the read-back at the end of
    // subsampling
    if (sub_err_valid_) throw_device_errors(sub_err_, "generate");
    else check_device_errors("generate");
    if (sparse) {
        launches_ += launch_sparse_zero(pyr_.as<uint32_t>(), occ, occ_blocks, stream_);
        check_cuda(cudaMemsetAsync(pyr_.as<uint32_t>() + cells0, 0, (level_off_[depth_ + 1] - cells0) * 4, stream_),
                   "memset");
        stage_mark("cleanup");
        check_cuda(cudaStreamSynchronize(stream_), "cleanup");
        pyr_zero_ = true;
    }
    collect_timings();
    compute_stats();
    tree_valid_ = true;
}

// Host copy of the node table (NodeHost), read on the side stream once tree
// enumeration is done, while distribution runs on the build stream.
void Builder::build_tree_host() {
    TraceRange trace("node table");
    check_cuda(cudaStreamWaitEvent(side_stream_, tree_ready_, 0), "wait");
    tree_host_.ensure(64);
    check_cuda(cudaMemcpyAsync(tree_host_.as<uint32_t>(0), n_nodes_.p, 4, cudaMemcpyDeviceToHost, side_stream_), "D2H");
    check_cuda(cudaMemcpyAsync(tree_host_.as<uint32_t>(4), err_.p, 4, cudaMemcpyDeviceToHost, side_stream_), "D2H");
    check_cuda(cudaStreamSynchronize(side_stream_), "tree");
    const uint32_t n = *tree_host_.as<uint32_t>(0), e = *tree_host_.as<uint32_t>(4);
    if (e & kErrNodeCap) {
        check_cuda(cudaStreamSynchronize(stream_), "tree");
        throw Error("counting: node capacity exceeded");
    }
    if (e) {   // counting failed (a point below the box, a bulk copy timed out): stop before the host tree
        check_cuda(cudaStreamSynchronize(stream_), "tree");
        throw_device_errors(e, "counting");
    }
    if (n > node_cap_) throw Error("counting: node count out of range");
    // pinned layout: key, count, child_first (u32), info (u16), level (u8),
    // occupied cells per level (u32)
    const size_t o_count = (size_t)n * 4, o_child = (size_t)n * 8, o_info = (size_t)n * 12;
    const size_t o_level = (size_t)n * 14, o_nz = ((size_t)n * 15 + 3) & ~(size_t)3;
    tree_host_.ensure(o_nz + (depth_ + 1) * 4);
    check_cuda(cudaMemcpyAsync(tree_host_.as<uint8_t>(0), key_.p, n * 4, cudaMemcpyDeviceToHost, side_stream_), "D2H");
    check_cuda(cudaMemcpyAsync(tree_host_.as<uint8_t>(o_count), count_.p, n * 4, cudaMemcpyDeviceToHost, side_stream_),
               "D2H");
    check_cuda(cudaMemcpyAsync(tree_host_.as<uint8_t>(o_child), child_first_.p, n * 4, cudaMemcpyDeviceToHost,
                               side_stream_),
               "D2H");
    check_cuda(cudaMemcpyAsync(tree_host_.as<uint8_t>(o_info), info_.p, n * 2, cudaMemcpyDeviceToHost, side_stream_),
               "D2H");
    check_cuda(cudaMemcpyAsync(tree_host_.as<uint8_t>(o_level), level_.p, n, cudaMemcpyDeviceToHost, side_stream_),
               "D2H");
    check_cuda(cudaMemcpyAsync(tree_host_.as<uint8_t>(o_nz), nonzero_.p, (depth_ + 1) * 4, cudaMemcpyDeviceToHost,
                               side_stream_),
               "D2H");
    check_cuda(cudaStreamSynchronize(side_stream_), "tree");
    const uint32_t* key = tree_host_.as<uint32_t>(0);
    const uint32_t* count = tree_host_.as<uint32_t>(o_count);
    const uint32_t* child_first = tree_host_.as<uint32_t>(o_child);
    const uint16_t* info = tree_host_.as<uint16_t>(o_info);
    const uint8_t* level = tree_host_.as<uint8_t>(o_level);
    nonzero_sum_ = 0;
    for (uint32_t l = 0; l <= depth_; ++l) nonzero_sum_ += tree_host_.as<uint32_t>(o_nz)[l];
    nodes_.assign(n, NodeHost{});
    leaf_ids_.clear();
    internal_by_level_.assign(depth_ + 1, {});
    const double cubic = cfg_.bb_max[0] - cfg_.bb_min[0];
    uint64_t off = 0;
    for (uint32_t i = 0; i < n; ++i) {
        NodeHost& v = nodes_[i];
        v.key = key[i];
        v.count = count[i];
        v.level = level[i];
        v.internal = info[i] & 1;
        v.mask = (uint8_t)(info[i] >> 1);
        v.child_first = child_first[i];
        if (i == 0)
            for (int a = 0; a < 3; ++a) v.mn[a] = cfg_.bb_min[a];
        if (v.internal) {
            internal_by_level_[v.level].push_back(i);
            // children's bbox minimum: parent min + childBBSide per set slot bit
            double side = cubic / std::pow(2.0, (double)(depth_ - v.level));
            double cside = side / 2.0;
            uint32_t c = v.child_first;
            for (uint32_t s = 0; s < 8; ++s) {
                if (!(v.mask & (1u << s))) continue;
                NodeHost& ch = nodes_[c];
                ch.mn[0] = (s & 4) ? v.mn[0] + cside : v.mn[0];
                ch.mn[1] = (s & 2) ? v.mn[1] + cside : v.mn[1];
                ch.mn[2] = (s & 1) ? v.mn[2] + cside : v.mn[2];
                ++c;
            }
        } else {
            v.points = v.count;
            v.data_idx = off;
            off += v.count;
            leaf_ids_.push_back(i);
        }
    }
    if (off != cfg_.n) throw Error("leaf points do not add up to the point amount");
}

void Builder::subsample() {
    TraceRange trace("subsample");
    const double cubic = cfg_.bb_max[0] - cfg_.bb_min[0];
    const uint32_t S = cfg_.sub_grid;
    uint32_t mode = 0;
    if (cfg_.intra) mode |= kModeIntra;
    if (cfg_.inter) mode |= kModeInter;
    if (cfg_.random) mode |= kModeRandom;
    if (cfg_.weighting) mode |= kModeWeight;
    const bool intra = cfg_.intra;
    const bool inter = !intra && cfg_.inter;
    const bool weighted = inter && cfg_.weighting;
    const bool averaged = intra || inter;
    OutParams op;
    for (int a = 0; a < 3; ++a) op.ax[a] = make_out_axis(cfg_.bb_min[a], 1.0 / cfg_.scale[a]);

    // ---- static part of the node tables, all levels.  Upper bounds of the
    // points per node: out(v) <= min(sum over children, S^3).
    const uint64_t S3 = (uint64_t)S * S * S;
    const size_t n = nodes_.size();
    std::vector<uint64_t> out_bound(n, 0), in_bound(n, 0);
    for (size_t i = n; i-- > 0;) {
        const NodeHost& v = nodes_[i];
        if (!v.internal) {
            out_bound[i] = v.points;
            continue;
        }
        uint64_t b = 0;
        uint32_t c = v.child_first;
        for (uint32_t s = 0; s < 8; ++s)
            if (v.mask & (1u << s)) b += out_bound[c++];
        in_bound[i] = b;
        out_bound[i] = std::min(b, S3);
    }
    // per level, largest bound first (the persistent blocks take nodes in this
    // order); internal index = position in the level-major order
    std::vector<uint32_t> level_first(depth_ + 2, 0), ii_of(n, 0xFFFFFFFFu);
    std::vector<uint32_t> order;
    std::vector<uint32_t> balance(depth_ + 2, 1);   // see launch_subsample_level
    std::vector<uint32_t> node_blocks(depth_ + 2, 1);
    uint64_t max_level_bound = 0, max_node_bound = 0;
    for (uint32_t l = 1; l <= depth_; ++l) {
        auto list = internal_by_level_[l];
        std::stable_sort(list.begin(), list.end(),
                         [&](uint32_t x, uint32_t y) { return in_bound[x] > in_bound[y]; });
        level_first[l] = (uint32_t)order.size();
        uint64_t lb = 0;
        for (uint32_t vi : list) {
            ii_of[vi] = (uint32_t)order.size();
            order.push_back(vi);
            lb += in_bound[vi];
            max_node_bound = std::max(max_node_bound, in_bound[vi]);
        }
        max_level_bound = std::max(max_level_bound, lb);
        if (lb) balance[l] = (uint32_t)std::min<uint64_t>(64, (in_bound[list[0]] * num_sms_ + lb - 1) / lb);
        if (!list.empty()) node_blocks[l] = node_blocks_for(in_bound[list[0]]);
    }
    level_first[depth_ + 1] = (uint32_t)order.size();
    const uint32_t n_internal = (uint32_t)order.size();
    // DFS post-order of the internal nodes (calculateWritingPosition,
    // kernel_helpers.cuh:55-59; setActiveParent fp_subsampling.cu:183): their
    // records follow the N leaf points in this order
    std::vector<uint32_t> post;
    post.reserve(n_internal);
    {
        std::vector<std::pair<uint32_t, bool>> st{{0u, false}};
        uint32_t kids[8];
        while (!st.empty()) {
            const auto [i, expanded] = st.back();
            st.pop_back();
            const NodeHost& v = nodes_[i];
            if (!v.internal) continue;
            if (expanded) {
                post.push_back(ii_of[i]);
                continue;
            }
            st.push_back({i, true});
            uint32_t nk = 0, c = v.child_first;
            for (uint32_t s = 0; s < 8; ++s)
                if (v.mask & (1u << s)) kids[nk++] = c++;
            while (nk) st.push_back({kids[--nk], false});
        }
    }
    std::vector<SubNode> table(n_internal);
    for (uint32_t k = 0; k < n_internal; ++k) {
        const NodeHost& v = nodes_[order[k]];
        SubNode& sn = table[k];
        std::memset(&sn, 0, sizeof(sn));
        const double side = cubic / std::pow(2.0, (double)(depth_ - v.level));   // fp_subsampling.cu:16-17
        // the node grid's extent is PointCloudInfo::cubicSize of the node box,
        // max.x - min.x with max.x = min.x + side (fp_subsampling.cu:38-42,
        // metadata.cuh:66-69); it can differ from side in the last bit
        const double t = ((v.mn[0] + side) - v.mn[0]) / S;                      // kernel_helpers.cuh:14
        for (int a = 0; a < 3; ++a) {
            sn.ax[a] = make_axis(v.mn[a], t);
            sn.qa[a] = make_qaxis(v.mn[a], cfg_.bb_min[a], 1.0 / cfg_.scale[a], t);
        }
        sn.morton = v.key;
        sn.level = v.level;
        uint32_t c = v.child_first, nc = 0;
        for (uint32_t s = 0; s < 8; ++s) {
            if (!(v.mask & (1u << s))) continue;
            const uint32_t ci = c++;
            const NodeHost& ch = nodes_[ci];
            if (ch.internal) {
                sn.child_kind |= 1u << nc;
                sn.child_start[nc] = ii_of[ci];   // replaced on the device by the staged position
            } else {
                sn.child_start[nc] = ch.data_idx;
                sn.child_count[nc] = ch.points;
            }
            ++nc;
        }
        sn.nchild = nc;
    }

    // ---- capacities: the staging arrays hold every level's candidates
    // (N + P_out at most, bounded by the reference's output capacity) and the
    // scratch one level's; both grow and the pass is repeated if a level does
    // not fit
    const uint64_t out_cap = (uint64_t)((float)cfg_.n * cfg_.output_factor);   // octree_processor_impl.cu:24-31
    uint64_t stage_cap = std::max<uint64_t>(sub_stage_cap_, std::max<uint64_t>(out_cap, cfg_.n));
    uint64_t scratch_cap = std::max<uint64_t>(sub_scratch_cap_, std::min(max_level_bound, stage_cap));
    {
        // global brick tables: enough slots for the largest node at 68% load
        // (bricks <= candidates and <= bricks of the grid)
        const uint64_t bs = (S + 3) / 4;
        const uint64_t bound = std::min<uint64_t>(max_node_bound, bs * bs * bs);
        uint64_t cap = 1024;
        while (cap * 11 / 16 < bound + 1) cap <<= 1;
        uint32_t shift = 32;
        for (uint64_t c = cap; c > 1; c >>= 1) --shift;
        size_t max_level_nodes = 0;
        for (uint32_t l = 1; l <= depth_; ++l)
            max_level_nodes = std::max<size_t>(max_level_nodes, level_first[l + 1] - level_first[l]);
        const size_t blocks = std::min<size_t>(max_level_nodes, (size_t)num_sms_);
        g_key_.ensure(blocks * cap * 4);
        g_mask_.ensure(blocks * cap * 8);
        g_base_.ensure(blocks * cap * 4);
        g_cap_ = (uint32_t)cap;
        g_shift_ = shift;
    }
    // final record arrays: N leaf records (written) + P_out internal records
    uint64_t rec_cap = std::max<uint64_t>(sub_rec_cap_, std::max<uint64_t>(out_cap, cfg_.n));
    // node table and post order staged in pinned memory (copied on the build
    // stream; the previous build's copies completed before it returned)
    const size_t table_bytes = (size_t)n_internal * sizeof(SubNode);
    const size_t o_post = (table_bytes + 15) & ~(size_t)15;
    table_host_.ensure(o_post + (size_t)n_internal * 4 + 16);
    if (n_internal) {
        std::memcpy(table_host_.p, table.data(), table_bytes);
        std::memcpy(table_host_.as<uint8_t>(o_post), post.data(), (size_t)n_internal * 4);
    }
    post_ii_.ensure(std::max<size_t>((size_t)n_internal * 4, 4));
    sub_nodes_.ensure(std::max<size_t>(table_bytes, sizeof(SubNode)));
    if (n_internal)
        check_cuda(cudaMemcpyAsync(post_ii_.p, table_host_.as<uint8_t>(o_post), (size_t)n_internal * 4,
                                   cudaMemcpyHostToDevice, stream_),
                   "H2D post order");
    // read back with the pass: error word, staging use, P_out, then per
    // internal node its points, staged offset and final position
    const size_t o_pts = 32, o_soff = (o_pts + (size_t)n_internal * 4 + 7) & ~(size_t)7;
    const size_t o_dst = o_soff + (size_t)n_internal * 8;
    back_host_.ensure(o_dst + (size_t)n_internal * 8);
    place_src_.ensure((size_t)n_internal * 8 + 8);
    place_dst_.ensure((size_t)n_internal * 8 + 8);
    place_cnt_.ensure((size_t)n_internal * 4 + 4);
    node_dst_.ensure((size_t)n_internal * 8 + 8);
    out_total_.ensure(8);
    out_points_.ensure((size_t)n_internal * 4 + 4);
    stage_off_.ensure((size_t)n_internal * 8 + 8);
    level_base_.ensure(8);
    work_.ensure(4);

    for (int attempt = 0;; ++attempt) {
        key_cache_.ensure(scratch_cap * 4);
        acc_best_.ensure(scratch_cap * 8);
        cell_slot_.ensure(scratch_cap * 4);
        if (cfg_.random) acc_sel_.ensure(scratch_cap * 4);
        if (averaged && !weighted) acc_intra_.ensure(scratch_cap * 8);
        if (weighted) {
            unit_cache_.ensure(scratch_cap * 12);
            csr_count_.ensure(scratch_cap * 4);
            csr_start_.ensure(scratch_cap * 4);
            csr_pts_.ensure(scratch_cap * 20);
            emit_maps_.ensure((size_t)kSplitEmitNodes * kBrickMapBytes);
            emit_state_.ensure((size_t)kSplitEmitNodes * 16);
        }
        stage_lut_.ensure(stage_cap * 4);
        stage_rec_.ensure(stage_cap * 18 + 64);
        stage_frac_.ensure(stage_cap * 4);
        if (copy_stream_) check_cuda(cudaStreamSynchronize(copy_stream_), "output copies");
        lut_.ensure_keep(rec_cap * 4, (size_t)cfg_.n * 4, stream_);
        rec_.ensure_keep(rec_cap * 18 + 16, (size_t)cfg_.n * 18, stream_);
        if (host_rec_) {
            // leaf records (and LUT entries) are final: stream them to the
            // caller's arrays while the levels are subsampled
            check_cuda(cudaEventRecord(leaf_ready_, stream_), "event");
            check_cuda(cudaStreamWaitEvent(copy_stream_, leaf_ready_, 0), "wait");
            check_cuda(cudaMemcpyAsync(host_rec_, rec_.p, (size_t)cfg_.n * 18, cudaMemcpyDeviceToHost, copy_stream_),
                       "D2H records");
            if (host_lut_)
                check_cuda(cudaMemcpyAsync(host_lut_, lut_.p, (size_t)cfg_.n * 4, cudaMemcpyDeviceToHost, copy_stream_),
                           "D2H lut");
        }
        if (n_internal)
            check_cuda(cudaMemcpyAsync(sub_nodes_.p, table_host_.p, table_bytes, cudaMemcpyHostToDevice, stream_),
                       "H2D node table");
        check_cuda(cudaMemsetAsync(level_base_.p, 0, 8, stream_), "memset");

        SubLevelArgs a{};
        a.grid = S;
        a.mode = mode;
        a.float_input = cfg_.cloud_type == 0;
        a.seed = cfg_.seed;
        a.cloud = cloud_.as<uint8_t>();
        a.stride = cfg_.stride;
        a.leaf_lut = lut_.as<uint32_t>();
        a.leaf_rec = rec_.as<uint8_t>();
        a.stage_lut = stage_lut_.as<uint32_t>();
        a.stage_rec = stage_rec_.as<uint8_t>();
        a.leaf_frac = leaf_frac_.as<uint32_t>();
        a.stage_frac = stage_frac_.as<uint32_t>();
        a.out_frac = stage_frac_.as<uint32_t>();
        a.out_lut = stage_lut_.as<uint32_t>();
        a.out_rec = stage_rec_.as<uint8_t>();
        a.key_cache = key_cache_.as<uint32_t>();
        a.unit_cache = unit_cache_.as<float>();
        a.acc_best = acc_best_.as<uint64_t>();
        a.acc_sel = acc_sel_.as<uint32_t>();
        a.cell_slot = cell_slot_.as<uint32_t>();
        a.acc_intra = acc_intra_.as<uint64_t>();
        a.csr_count = csr_count_.as<uint32_t>();
        a.csr_start = csr_start_.as<uint32_t>();
        a.csr_pts = csr_pts_.as<uint8_t>();
        a.out = op;
        a.work_counter = work_.as<uint32_t>();
        a.err = err_.as<uint32_t>();
        a.global_key = g_key_.as<uint32_t>();
        a.global_mask = g_mask_.as<uint64_t>();
        a.global_base = g_base_.as<uint32_t>();
        a.global_cap = g_cap_;
        a.global_shift = g_shift_;
        // the first pass of a build in a wave hands its whole plan to the
        // wave, which issues it with the other builds' (one subsampling
        // launch per level over all of them); repeats run alone
        const bool in_wave = wave_ && attempt == 0;
        if (in_wave) {
            if (!level_ready_) check_cuda(cudaEventCreateWithFlags(&level_ready_, cudaEventDisableTiming), "event");
            std::vector<WaveLevel> plan(depth_);
            for (uint32_t l = 1; l <= depth_; ++l) {
                const uint32_t first = level_first[l], cnt = level_first[l + 1] - first;
                WaveLevel& w = plan[l - 1];
                w.a = a;
                w.a.n_nodes = cnt;
                if (!cnt) continue;
                SubNode* lvl = sub_nodes_.as<SubNode>() + first;
                w.a.nodes = lvl;
                w.a.out_points = out_points_.as<uint32_t>() + first;
                w.bounds.resize(cnt);
                for (uint32_t i = 0; i < cnt; ++i) w.bounds[i] = in_bound[order[first + i]];
                uint32_t* outp = out_points_.as<uint32_t>();
                uint64_t* soff = stage_off_.as<uint64_t>();
                uint64_t* lbase = level_base_.as<uint64_t>();
                uint32_t* work = work_.as<uint32_t>();
                uint32_t* err = err_.as<uint32_t>();
                w.prepare = [=](cudaStream_t st) {
                    launch_prepare_level(lvl, cnt, outp, soff, first, lbase, scratch_cap, stage_cap, work, err, st);
                };
                ++launches_;
            }
            check_cuda(cudaEventRecord(level_ready_, stream_), "event");
            wave_->submit(wave_slot_, std::move(plan), g_cap_, level_ready_, stream_);
            stage_mark("subsample");
        } else {
            for (uint32_t l = 1; l <= depth_; ++l) {
                const uint32_t first = level_first[l], cnt = level_first[l + 1] - first;
                if (!cnt) continue;
                SubNode* lvl = sub_nodes_.as<SubNode>() + first;
                launches_ += launch_prepare_level(lvl, cnt, out_points_.as<uint32_t>(), stage_off_.as<uint64_t>(),
                                                  first, level_base_.as<uint64_t>(), scratch_cap, stage_cap,
                                                  work_.as<uint32_t>(), err_.as<uint32_t>(), stream_);
                a.nodes = lvl;
                a.n_nodes = cnt;
                a.out_points = out_points_.as<uint32_t>() + first;
                ClusterCaps caps;
                caps.node_blocks = node_blocks[l];
                // a distance-weighted level of few nodes hands each node's
                // emit to k_emit_weighted, over all SMs
                const bool split = weighted && cnt <= kSplitEmitNodes;
                a.emit_maps = split ? emit_maps_.as<uint8_t>() : nullptr;
                a.emit_state = split ? emit_state_.as<uint32_t>() : nullptr;
                if (split) check_cuda(cudaMemsetAsync(emit_state_.p, 0, (size_t)cnt * 16, stream_), "memset");
                launches_ += launch_subsample_level(a, num_sms_, balance[l], stream_, caps);
                if (split) launches_ += launch_emit_weighted(a, num_sms_, stream_);
                char mark[32];
                std::snprintf(mark, sizeof mark, "sub_l%u", l);
                stage_mark(mark);
            }
        }
        // internal nodes' records to their post-order positions
        launches_ += launch_place_prepare(post_ii_.as<uint32_t>(), n_internal, out_points_.as<uint32_t>(),
                                          stage_off_.as<uint64_t>(), cfg_.n, rec_cap, place_src_.as<uint64_t>(),
                                          place_dst_.as<uint64_t>(), place_cnt_.as<uint32_t>(),
                                          node_dst_.as<uint64_t>(), out_total_.as<uint64_t>(), err_.as<uint32_t>(),
                                          stream_);
        launches_ += launch_place(place_src_.as<uint64_t>(), place_dst_.as<uint64_t>(), place_cnt_.as<uint32_t>(),
                                  n_internal, stage_rec_.as<uint8_t>(), rec_.as<uint8_t>(), stream_);
        stage_mark("place");
        check_cuda(cudaGetLastError(), "subsample launch");
        check_cuda(cudaMemcpyAsync(back_host_.as<uint8_t>(0), err_.p, 4, cudaMemcpyDeviceToHost, stream_), "D2H err");
        check_cuda(cudaMemcpyAsync(back_host_.as<uint8_t>(8), level_base_.p, 8, cudaMemcpyDeviceToHost, stream_), "D2H");
        check_cuda(cudaMemcpyAsync(back_host_.as<uint8_t>(16), out_total_.p, 8, cudaMemcpyDeviceToHost, stream_), "D2H");
        if (n_internal) {
            check_cuda(cudaMemcpyAsync(back_host_.as<uint8_t>(o_pts), out_points_.p, (size_t)n_internal * 4,
                                       cudaMemcpyDeviceToHost, stream_),
                       "D2H");
            check_cuda(cudaMemcpyAsync(back_host_.as<uint8_t>(o_soff), stage_off_.p, (size_t)n_internal * 8,
                                       cudaMemcpyDeviceToHost, stream_),
                       "D2H");
            check_cuda(cudaMemcpyAsync(back_host_.as<uint8_t>(o_dst), node_dst_.p, (size_t)n_internal * 8,
                                       cudaMemcpyDeviceToHost, stream_),
                       "D2H");
        }
        check_cuda(cudaStreamSynchronize(stream_), "subsample");
        const uint32_t e = *back_host_.as<uint32_t>(0);
        p_out_ = *back_host_.as<uint64_t>(16);
        if (!(e & kErrCapacity)) {
            stage_used_ = *back_host_.as<uint64_t>(8);
            sub_err_ = e;
            sub_err_valid_ = true;
            stats_.subsample_passes = (uint32_t)attempt + 1;
            break;
        }
        if (attempt >= 6 || (e & ~kErrCapacity)) check_device_errors("subsample");
        // a level or the final records did not fit: grow and repeat the pass
        stage_cap *= 2;
        scratch_cap = std::min<uint64_t>(scratch_cap * 2, std::max(max_level_bound, scratch_cap));
        rec_cap = std::max<uint64_t>(rec_cap * 2, (uint64_t)cfg_.n + stage_cap);
        const uint32_t keep = e & ~kErrCapacity;
        check_cuda(cudaMemcpyAsync(err_.p, &keep, 4, cudaMemcpyHostToDevice, stream_), "H2D err");
    }
    sub_stage_cap_ = stage_cap;
    sub_scratch_cap_ = scratch_cap;
    sub_rec_cap_ = rec_cap;
    stats_.p_in = stage_used_;
    place_count_ = n_internal;
    lut_placed_ = false;

    const uint32_t* pts = back_host_.as<uint32_t>(o_pts);
    const uint64_t* soff = back_host_.as<uint64_t>(o_soff);
    const uint64_t* dst = back_host_.as<uint64_t>(o_dst);
    for (uint32_t k = 0; k < n_internal; ++k) {
        NodeHost& v = nodes_[order[k]];
        v.points = pts[k];
        v.stage_off = soff[k];
        v.data_idx = dst[k];
    }
    if (host_rec_) {
        const uint64_t total = (uint64_t)cfg_.n + p_out_;
        if (total > host_cap_) {
            check_cuda(cudaStreamSynchronize(copy_stream_), "output copies");
            throw Error("output host buffer too small: the octree has " + std::to_string(total) + " records");
        }
        check_cuda(cudaMemcpyAsync(host_rec_ + (size_t)cfg_.n * 18, rec_.as<uint8_t>() + (size_t)cfg_.n * 18,
                                   (size_t)p_out_ * 18, cudaMemcpyDeviceToHost, stream_),
                   "D2H records");
        if (host_lut_) {
            launch_place_lut(place_src_.as<uint64_t>(), place_dst_.as<uint64_t>(), place_cnt_.as<uint32_t>(),
                             (uint32_t)place_count_, stage_lut_.as<uint32_t>(), lut_.as<uint32_t>(), stream_);
            lut_placed_ = true;
            check_cuda(cudaMemcpyAsync(host_lut_ + cfg_.n, lut_.as<uint32_t>() + cfg_.n, (size_t)p_out_ * 4,
                                       cudaMemcpyDeviceToHost, stream_),
                       "D2H lut");
        }
        stage_mark("d2h");
        check_cuda(cudaStreamSynchronize(copy_stream_), "output copies");
        check_cuda(cudaStreamSynchronize(stream_), "output copies");
        host_filled_ = true;
    }
}

void Builder::compute_stats() {
    Stats& S = stats_;
    S.depth = depth_;
    S.tree_nodes = (uint32_t)nodes_.size();
    S.leaf_nodes = (uint32_t)leaf_ids_.size();
    S.internal_nodes = S.tree_nodes - S.leaf_nodes;
    S.p_out = p_out_;
    S.points_total = (uint64_t)cfg_.n + p_out_;
    S.out_capacity = (uint64_t)((float)cfg_.n * cfg_.output_factor);   // point_cloud.cuh:24
    S.dense_nodes = (uint32_t)level_off_[depth_ + 1];
    S.kernel_launches = launches_;
    S.sparse_nodes = nonzero_sum_;
    // OctreeData::updateNodeStatistics (octree.cu:79-132): DFS in slot order
    S.min_leaf_points = 0xFFFFFFFFu;
    S.max_leaf_points = 0;
    S.max_leaf_depth = 0;
    uint32_t sum = 0;
    std::vector<uint32_t> order;
    std::vector<std::pair<uint32_t, uint32_t>> st{{0u, 0u}};
    while (!st.empty()) {
        auto [i, d] = st.back();
        st.pop_back();
        const NodeHost& v = nodes_[i];
        if (!v.internal) {
            S.max_leaf_depth = std::max(S.max_leaf_depth, d);
            sum += v.count;
            S.min_leaf_points = std::min(S.min_leaf_points, v.count);
            S.max_leaf_points = std::max(S.max_leaf_points, v.count);
            order.push_back(i);
            continue;
        }
        std::vector<uint32_t> kids;
        uint32_t c = v.child_first;
        for (uint32_t s = 0; s < 8; ++s)
            if (v.mask & (1u << s)) kids.push_back(c++);
        for (auto it = kids.rbegin(); it != kids.rend(); ++it) st.push_back({*it, d + 1});
    }
    S.mean_leaf_points = (float)sum / (float)S.leaf_nodes;
    float var = 0.f;
    for (uint32_t i : order) {
        float d = (float)nodes_[i].count - S.mean_leaf_points;
        var += std::pow(d, 2.f);
    }
    S.stdev_leaf_points = std::sqrt(var / (float)S.leaf_nodes);
}

std::vector<uint8_t> Builder::hierarchy() const {
    std::vector<uint8_t> out(nodes_.size() * 22);
    for (size_t i = 0; i < nodes_.size(); ++i) {
        const NodeHost& v = nodes_[i];
        uint8_t mask = v.internal ? v.mask : 0;
        uint8_t type = mask == 0 ? 1 : 0;
        uint32_t pts = v.points;
        uint64_t off = v.data_idx * 18ull, size = (uint64_t)pts * 18ull;
        uint8_t* e = out.data() + i * 22;
        e[0] = type;
        e[1] = mask;
        std::memcpy(e + 2, &pts, 4);
        std::memcpy(e + 6, &off, 8);
        std::memcpy(e + 14, &size, 8);
    }
    return out;
}

void Builder::copy_records(uint8_t* out) const {
    check_cuda(cudaMemcpy(out, rec_.p, stats_.points_total * 18, cudaMemcpyDeviceToHost), "D2H records");
}

void Builder::copy_lut(uint32_t* out) {
    // internal-node cloud indices are moved to their final positions on demand
    if (!lut_placed_) {
        launch_place_lut(place_src_.as<uint64_t>(), place_dst_.as<uint64_t>(), place_cnt_.as<uint32_t>(),
                         (uint32_t)place_count_, stage_lut_.as<uint32_t>(), lut_.as<uint32_t>(), stream_);
        check_cuda(cudaStreamSynchronize(stream_), "place lut");
        lut_placed_ = true;
    }
    check_cuda(cudaMemcpy(out, lut_.p, stats_.points_total * 4, cudaMemcpyDeviceToHost), "D2H lut");
}

bool Builder::level_counts(uint32_t level, uint32_t* out) const {
    if (level >= pyramid_copy_.size()) return false;
    std::memcpy(out, pyramid_copy_[level].data(), pyramid_copy_[level].size() * 4);
    return true;
}

}   // namespace oc
