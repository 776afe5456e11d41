// Device-side arithmetic shared by every stage of the LOD build.
//
// Exactness contract.  The reference maps a coordinate to a grid cell with
// IEEE binary64 arithmetic (mapPointToGrid, OctreeLibrary/src/kernel/
// kernel_helpers.cuh:10-25) and quantises output coordinates the same way
// (point_distributing.cuh:245-247).  GB300's binary64 issue rate is a small
// fraction of its binary32 rate, so every stage evaluates those formulas with
// an fp32 (or float-float) estimate plus a rigorous error bound, and only
// falls back to the binary64 expression when the estimate lies within that
// bound of a cell boundary.  The result is always the binary64 result.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

namespace oc {

constexpr uint32_t kNoCell = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// Cell index along one axis of a gridding.

struct AxisGrid {
    double mn;    // bounding-box minimum of the gridded cube
    double t;     // cell size = cube side / grid, as the reference computes it
    float m_hi;   // float(mn)
    float m_lo;   // float(mn - m_hi)
    float r;      // float(1 / t)
    float cm;     // 2^-44 * |mn| / t : absolute part of the error bound
};

__host__ __device__ inline AxisGrid make_axis(double mn, double t) {
    AxisGrid a;
    a.mn = mn;
    a.t = t;
    a.m_hi = (float)mn;
    a.m_lo = (float)(mn - (double)a.m_hi);
    a.r = (float)(1.0 / t);
    double cm = 5.684341886080802e-14 * (mn < 0 ? -mn : mn) / t;   // 2^-44
    a.cm = (float)(cm * 1.0000001) + 1e-30f;
    return a;
}

// ---------------------------------------------------------------------------
// Output coordinate floor((p - mn) * sf) as int32 (the reference's
// static_cast<int32_t>(floor(...)), point_distributing.cuh:245-247).

struct OutAxis {
    double mn;
    double sf;    // 1 / scale, computed in double on the host
    float m_hi, m_lo;
    float sf_hi, sf_lo;
};

__host__ __device__ inline OutAxis make_out_axis(double mn, double sf) {
    OutAxis o;
    o.mn = mn;
    o.sf = sf;
    o.m_hi = (float)mn;
    o.m_lo = (float)(mn - (double)o.m_hi);
    o.sf_hi = (float)sf;
    o.sf_lo = (float)(sf - (double)o.sf_hi);
    return o;
}

constexpr int32_t kCoordError = (int32_t)0x80000000;

// ---------------------------------------------------------------------------
// Morton order with x as the most significant bit of every triple: the child
// slot of a cell inside its parent is the low three bits (x<<2 | y<<1 | z),
// the same slot numbering as the reference (point_count_propagation.cuh:241-249).

__host__ __device__ inline uint32_t spread3(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__host__ __device__ inline uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return (spread3(x) << 2) | (spread3(y) << 1) | spread3(z);
}

__host__ __device__ inline uint32_t compact3(uint32_t v) {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030C30C3u;
    v = (v | (v >> 4)) & 0x0300F00Fu;
    v = (v | (v >> 8)) & 0x030000FFu;
    v = (v | (v >> 16)) & 0x000003FFu;
    return v;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): priority of a cloud point
// for explicit random subsampling in node (level, morton).

__host__ __device__ inline uint32_t rp_priority(uint64_t seed, uint32_t level, uint64_t morton, uint32_t idx) {
    uint32_t c0 = idx, c1 = (uint32_t)morton, c2 = (uint32_t)(morton >> 32) ^ (level << 24), c3 = 0x52504E44u;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c0;
}

// Device error bits (sticky, read by the host after each stage).
enum : uint32_t {
    kErrBelowBox = 1u << 0,      // a point maps below the bounding box
    kErrCoordRange = 1u << 1,    // an output coordinate does not fit int32
    kErrProbe = 1u << 2,         // a hash probe exceeded its bound
    kErrCapacity = 1u << 3,      // a scratch buffer was too small
    kErrTag = 1u << 4,           // a point found no leaf
    kErrTimeout = 1u << 5,       // a bounded wait on a bulk copy gave up
    kErrNodeCap = 1u << 6,       // the tree has more nodes than the node table holds
};

// ---------------------------------------------------------------------------
// Ordered keys: monotone maps of IEEE bit patterns onto signed integers, so
// that binary64 / binary32 values compare exactly as integers (negative
// values have their magnitude bits reversed).

inline int64_t host_key64(double d) {
    uint64_t b;
    std::memcpy(&b, &d, 8);
    return (int64_t)((b >> 63) ? (b ^ 0x7FFFFFFFFFFFFFFFull) : b);
}

inline double host_from_key64(int64_t k) {
    uint64_t b = (uint64_t)k;
    if (k < 0) b ^= 0x7FFFFFFFFFFFFFFFull;
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

inline int32_t host_key32(float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return (int32_t)((b >> 31) ? (b ^ 0x7FFFFFFFu) : b);
}

inline float host_from_key32(int32_t k) {
    uint32_t b = (uint32_t)k;
    if (k < 0) b ^= 0x7FFFFFFFu;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

#if defined(__CUDACC__)
// ===== device-only arithmetic =====

// ---------------------------------------------------------------------------
// Coordinates: a point coordinate as an unevaluated float pair hi + lo.

struct Coord {
    float hi, lo;
    bool ok;        // split valid (otherwise only the exact path is used)
    double exact;   // the coordinate as binary64 (converted lazily for float input)
};

// float input: hi = value, lo = 0 (exact).
__device__ __forceinline__ Coord coord_f32(float f) {
    Coord c;
    c.hi = f;
    c.lo = 0.0f;
    c.ok = true;
    c.exact = 0.0;   // filled by exact_value() on demand
    return c;
}

// double input: hi = value with its mantissa truncated to 24 bits, lo = the
// remainder rounded to float.  Built from integer operations only.
__device__ __forceinline__ Coord coord_f64(double d) {
    Coord c;
    c.exact = d;
    unsigned long long bits = (unsigned long long)__double_as_longlong(d);
    unsigned e = (unsigned)(bits >> 52) & 0x7FFu;
    unsigned long long mant = bits & ((1ull << 52) - 1);
    unsigned sign = (unsigned)(bits >> 63) << 31;
    if (e == 0 && mant == 0) {
        c.hi = __uint_as_float(sign);
        c.lo = 0.0f;
        c.ok = true;
        return c;
    }
    int ue = (int)e - 1023;
    if (ue < -60 || ue > 100) {
        c.hi = c.lo = 0.0f;
        c.ok = false;
        return c;
    }
    c.hi = __uint_as_float(sign | ((unsigned)(ue + 127) << 23) | (unsigned)(mant >> 29));
    unsigned low = (unsigned)(mant & ((1u << 29) - 1));
    if (low == 0) {
        c.lo = 0.0f;
    } else {
        float lf = __fmul_rn(__uint2float_rn(low), __uint_as_float((unsigned)(ue - 52 + 127) << 23));
        c.lo = sign ? -lf : lf;
    }
    c.ok = true;
    return c;
}

// Cell-unit position (p - mn) / t in fp32 from the split coordinate.
__device__ __forceinline__ float approx_units(const Coord& c, const AxisGrid& a) {
    float s = __fsub_rn(c.hi, a.m_hi);
    float q = __fsub_rn(c.lo, a.m_lo);
    float d = __fadd_rn(s, q);
    return __fmul_rn(d, a.r);
}

// Cell-unit position (p - mn) / t of a coordinate, for distance weighting.
template <bool kFloatInput>
__device__ __forceinline__ float point_units(const Coord& c, const AxisGrid& a) {
    if (kFloatInput || c.ok) return approx_units(c, a);
    return (float)((c.exact - a.mn) / a.t);
}

__device__ __forceinline__ int idx_from_units(float x, uint32_t G) {
    if (x >= (float)(G - 1)) return (int)G - 1;
    if (!(x > -1.0f)) return -1;
    return x < 0.0f ? 0 : (int)x;
}

// Binary64 evaluation of mapPointToGrid for one axis: (int64)fmin((p-mn)/t, G-1).
// Returns -1 where the reference would produce a negative index.
static __device__ __noinline__ int exact_axis_cell(double p, double mn, double t, uint32_t G) {
    double u = __ddiv_rn(__dsub_rn(p, mn), t);
    double v = fmin(u, (double)G - 1.0);
    if (!(v > -1.0)) return -1;
    return (int)(long long)v;
}

template <bool kFloatInput>
__device__ __forceinline__ double exact_value(const Coord& c) {
    return kFloatInput ? (double)c.hi : c.exact;
}

// Cell index of one axis; `units` receives the fp32 cell-unit position.
template <bool kFloatInput>
__device__ __forceinline__ int axis_cell(const Coord& c, const AxisGrid& a, uint32_t G, float& units) {
    if (kFloatInput || c.ok) {
        float A = approx_units(c, a);
        units = A;
        float eps = __fmaf_rn(fabsf(A), 9.5367431640625e-07f, __fadd_rn(9.5367431640625e-07f, a.cm));   // 2^-20
        int lo = idx_from_units(__fsub_rn(A, eps), G);
        int hi = idx_from_units(__fadd_rn(A, eps), G);
        if (lo == hi && lo >= 0) return lo;
    } else {
        units = (float)((exact_value<kFloatInput>(c) - a.mn) / a.t);
    }
    return exact_axis_cell(exact_value<kFloatInput>(c), a.mn, a.t, G);
}

static __device__ __noinline__ int32_t exact_out_coord(double p, double mn, double sf) {
    double v = floor(__dmul_rn(__dsub_rn(p, mn), sf));
    if (!(v > -2147483648.0 && v < 2147483648.0)) return kCoordError;
    return (int32_t)v;
}

// fbin receives the fractional part of (p - mn) * sf in 1/1024 steps when the
// fast path proves it to within 2^-12 (true fraction in
// [(fbin - 1/4) / 1024, (fbin + 5/4) / 1024]), else kNoFrac.
constexpr uint32_t kNoFrac = 0xFFFFFFFFu;

template <bool kFloatInput>
__device__ __forceinline__ int32_t out_coord_frac(const Coord& c, const OutAxis& o, uint32_t& fbin) {
    fbin = kNoFrac;
    if (kFloatInput || c.ok) {
        // s + e1 = hi - m_hi exactly (Knuth TwoSum)
        float nm = -o.m_hi;
        float s = __fadd_rn(c.hi, nm);
        float bb = __fsub_rn(s, c.hi);
        float e1 = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bb)), __fsub_rn(nm, bb));
        float lo2 = __fsub_rn(__fadd_rn(e1, c.lo), o.m_lo);
        float ph = __fmul_rn(s, o.sf_hi);
        float perr = __fmaf_rn(s, o.sf_hi, -ph);
        float pl = __fmaf_rn(s, o.sf_lo, __fmaf_rn(lo2, o.sf_hi, perr));
        if (fabsf(ph) < 1.0e9f) {
            float f = floorf(ph);
            float frac = __fadd_rn(__fsub_rn(ph, f), pl);
            float g = floorf(frac);
            float rem = __fsub_rn(frac, g);
            float mag = __fmaf_rn(__fadd_rn(fabsf(c.hi), fabsf(o.m_hi)), fabsf(o.sf_hi), fabsf(ph));
            float E = __fmaf_rn(mag, 2.2737367544323206e-13f, 2.384185791015625e-07f);   // 2^-42, 2^-22
            if (rem >= E && rem <= __fsub_rn(1.0f, E)) {
                if (E <= 2.44140625e-04f) fbin = min(__float2uint_rz(__fmul_rn(rem, 1024.0f)), 1023u);   // 2^-12
                return (int32_t)f + (int32_t)g;
            }
        }
    }
    return exact_out_coord(exact_value<kFloatInput>(c), o.mn, o.sf);
}

template <bool kFloatInput>
__device__ __forceinline__ int32_t out_coord(const Coord& c, const OutAxis& o) {
    uint32_t unused;
    return out_coord_frac<kFloatInput>(c, o, unused);
}

// Sub-step word of an output record: bits 0-9, 10-19, 20-29 the x, y, z
// fraction bins of out_coord_frac, bit 31 set when all three are known.
__device__ __forceinline__ uint32_t pack_frac(uint32_t fx, uint32_t fy, uint32_t fz) {
    return (fx == kNoFrac || fy == kNoFrac || fz == kNoFrac) ? 0u : (0x80000000u | fx | (fy << 10) | (fz << 20));
}

// ---------------------------------------------------------------------------
// Packed colour sums (encodeColors kernel_helpers.cuh:49-53, decode
// fp_subsampling.cuh:95-101).  A zero count field (a multiple of 1024 points)
// divides by zero in the reference; here it yields 0xFFFF.

__device__ __forceinline__ uint64_t encode_colors(uint32_t r, uint32_t g, uint32_t b) {
    return ((uint64_t)r << 46) | ((uint64_t)g << 28) | ((uint64_t)b << 10) | 1ull;
}

__device__ __forceinline__ void decode_colors(uint64_t e, uint16_t& r, uint16_t& g, uint16_t& b) {
    const uint32_t amount = (uint32_t)(e & 0x3FF);
    if (amount == 0) {
        r = g = b = 0xFFFF;
        return;
    }
    const uint32_t xr = (uint32_t)((e >> 46) & 0xFFFF), xg = (uint32_t)((e >> 28) & 0xFFFF),
                   xb = (uint32_t)((e >> 10) & 0xFFFF);
    if (amount == 1) {
        r = (uint16_t)xr;
        g = (uint16_t)xg;
        b = (uint16_t)xb;
        return;
    }
    // floor(x / d) = umulhi(x, ceil(2^32 / d)) exactly for x < 2^16, d < 2^10:
    // the product overshoots x / d by less than 2^-16, below the 1/d gap to
    // the next integer
    const uint32_t m = 0xFFFFFFFFu / amount + 1u;
    r = (uint16_t)__umulhi(xr, m);
    g = (uint16_t)__umulhi(xg, m);
    b = (uint16_t)__umulhi(xb, m);
}


// ---------------------------------------------------------------------------
// Distance weighting.  exp(x) for x in [-15, 0] by Cody & Waite range
// reduction and the degree-7 Taylor polynomial of e^f (Horner, fused
// multiply-adds), then exact scaling by 2^k.  The weight of a point at cell
// units u (its own position, (p - node min) / t, point_units) for neighbour
// cell n is round(2^28 * exp(-10 * |n + 0.5 - u|^2 * 4/27)), i.e.
// exp(-10 (d/r)^2) with r the half diagonal of 3x3x3 cells
// (kernel_inter_cell_filtering.cuh:171-180, fp_subsampling.cu:56-61).  A point
// lies in its cell, so (d/r)^2 <= 1 and every weight is at least
// 2^28 e^-10 > 12000: the rounding costs under 1e-4 of a weight.  Sums of
// weight * colour stay below 2^64 for up to 2^28 colours of at most 255.

__device__ __forceinline__ float exp_neg(float x) {
    const float kLog2e = 1.44269504088896341f;
    const float kLn2Hi = 0.693359375f;
    const float kLn2Lo = -2.12194440054690583e-4f;
    float kf = rintf(__fmul_rn(x, kLog2e));
    float f = __fmaf_rn(-kf, kLn2Hi, x);
    f = __fmaf_rn(-kf, kLn2Lo, f);
    float p = 1.0f / 5040.0f;
    p = __fmaf_rn(p, f, 1.0f / 720.0f);
    p = __fmaf_rn(p, f, 1.0f / 120.0f);
    p = __fmaf_rn(p, f, 1.0f / 24.0f);
    p = __fmaf_rn(p, f, 1.0f / 6.0f);
    p = __fmaf_rn(p, f, 0.5f);
    p = __fmaf_rn(p, f, 1.0f);
    p = __fmaf_rn(p, f, 1.0f);
    int k = (int)kf;
    return __fmul_rn(p, __uint_as_float((unsigned)(k + 127) << 23));
}

__device__ __forceinline__ uint32_t weight_q(float ux, float uy, float uz, int nx, int ny, int nz) {
    float dx = __fsub_rn(__fadd_rn((float)nx, 0.5f), ux);
    float dy = __fsub_rn(__fadd_rn((float)ny, 0.5f), uy);
    float dz = __fsub_rn(__fadd_rn((float)nz, 0.5f), uz);
    float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    float q = __fmul_rn(d2, (float)(4.0 / 27.0));
    q = fminf(q, 1.5f);
    float w = exp_neg(__fmul_rn(-10.0f, q));
    return (uint32_t)__fadd_rn(__fmul_rn(w, 268435456.0f), 0.5f);
}

// ---------------------------------------------------------------------------
// Record I/O.

struct __align__(2) Record18 {   // OutputBuffer, types.cuh:18-24 (packed, 18 bytes)
    uint16_t h[9];
};

// Record loads.  A 15- or 27-byte record starts at any byte; it is read as
// the 8-byte-aligned words that cover it (3 words for 15 bytes, 5 for 27) and
// realigned with funnel shifts.  Memory (global or shared) must be readable up
// to 16 bytes past the record: the cloud buffer and the staging tiles are
// padded for that.
__device__ __forceinline__ uint64_t shr128(uint64_t lo, uint64_t hi, uint32_t s) {
    uint32_t a = (uint32_t)lo, b = (uint32_t)(lo >> 32), c = (uint32_t)hi;
    uint32_t r0 = __funnelshift_r(a, b, s), r1 = __funnelshift_r(b, c, s);
    uint32_t t0 = s >= 32 ? r1 : r0;
    uint32_t t1 = s >= 32 ? __funnelshift_r(c, (uint32_t)(hi >> 32), s) : r1;
    return (uint64_t)t0 | ((uint64_t)t1 << 32);
}

template <bool kFloatInput>
__device__ __forceinline__ void load_point(const uint8_t* rec, Coord c[3], uint32_t col[3]) {
    uintptr_t addr = reinterpret_cast<uintptr_t>(rec);
    const uint64_t* q = reinterpret_cast<const uint64_t*>(addr & ~(uintptr_t)7);
    uint32_t s = (uint32_t)(addr & 7) * 8;
    if (kFloatInput) {
        uint64_t w0 = q[0], w1 = q[1], w2 = q[2];
        uint64_t r0 = shr128(w0, w1, s), r1 = shr128(w1, w2, s);
        c[0] = coord_f32(__uint_as_float((uint32_t)r0));
        c[1] = coord_f32(__uint_as_float((uint32_t)(r0 >> 32)));
        c[2] = coord_f32(__uint_as_float((uint32_t)r1));
        col[0] = (uint32_t)(r1 >> 32) & 0xFF;
        col[1] = (uint32_t)(r1 >> 40) & 0xFF;
        col[2] = (uint32_t)(r1 >> 48) & 0xFF;
    } else {
        uint64_t w0 = q[0], w1 = q[1], w2 = q[2], w3 = q[3], w4 = q[4];
        uint64_t r0 = shr128(w0, w1, s), r1 = shr128(w1, w2, s), r2 = shr128(w2, w3, s), r3 = shr128(w3, w4, s);
        c[0] = coord_f64(__longlong_as_double((long long)r0));
        c[1] = coord_f64(__longlong_as_double((long long)r1));
        c[2] = coord_f64(__longlong_as_double((long long)r2));
        col[0] = (uint32_t)r3 & 0xFF;
        col[1] = (uint32_t)(r3 >> 8) & 0xFF;
        col[2] = (uint32_t)(r3 >> 16) & 0xFF;
    }
}

// ---------------------------------------------------------------------------
// Ordered keys on the device (same maps as host_key64 / host_key32).

__device__ __forceinline__ long long dev_key64(uint32_t lo, uint32_t hi) {
    const uint32_t s = (uint32_t)((int32_t)hi >> 31);
    return (long long)(((uint64_t)(hi ^ (s >> 1)) << 32) | (uint64_t)(lo ^ s));
}

__device__ __forceinline__ int dev_key32(uint32_t b) {
    return (int)(b ^ ((uint32_t)((int32_t)b >> 31) >> 1));
}

// A float close to the binary64 value hi:lo (mantissa truncated to 24 bits);
// meaningless outside the binary32 exponent range, which only makes the cell
// estimate below miss and fall back to the exact path.
__device__ __forceinline__ float approx_f64(uint32_t lo, uint32_t hi) {
    const uint32_t t = hi - (896u << 20);
    return __uint_as_float((__funnelshift_l(lo, t, 3) & 0x7FFFFFFFu) | (hi & 0x80000000u));
}

// Cell index of one axis from exact boundary keys: keys[i] is the least key
// whose cell is >= i (keys[grid] = keys[grid + 1] = the largest key), so the
// cell of `key` is the i with keys[i] <= key < keys[i + 1].  `est` is an
// approximate cell-unit position; the estimate and its two neighbours are
// checked.  Returns -2 when none matches (the caller evaluates the cell
// exactly).
template <typename K>
__device__ __forceinline__ int table_cell(K key, float est, const K* keys, uint32_t grid) {
    const float e = fminf(fmaxf(est, 0.0f), (float)(grid - 1));   // NaN -> 0
    const int i = __float_as_int(__fadd_rd(e, 8388608.0f)) - 0x4B000000;   // floor(e)
    const K lo = keys[i], hi = keys[i + 1];
    if (key >= lo && key < hi) return i;
    if (key < lo) return (i > 0 && key >= keys[i - 1]) ? i - 1 : -2;
    return key < keys[i + 2] ? i + 1 : -2;
}

// ---------------------------------------------------------------------------
// Bulk (TMA) copies into shared memory, completed on an mbarrier.

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with parity `parity`; gives up after about 2^31 clock
// cycles (about a second) and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > (1ll << 31)) return false;
    return true;
}

// ---------------------------------------------------------------------------
// Runs: consecutive lanes of a warp holding the same key.  All 32 lanes must
// call these together.

__device__ __forceinline__ uint32_t run_starts(uint32_t key) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
    return __ballot_sync(0xffffffffu, lane == 0 || prev != key);
}

// first lane of this lane's run
__device__ __forceinline__ uint32_t run_leader(uint32_t starts) {
    const uint32_t lane = threadIdx.x & 31;
    return 31 - __clz(starts & (0xffffffffu >> (31 - lane)));
}

// one past the last lane of the run that starts at this lane
__device__ __forceinline__ uint32_t run_end(uint32_t starts) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t higher = starts & ~(0xffffffffu >> (31 - lane));
    return higher ? (uint32_t)__ffs(higher) - 1 : 32u;
}

// ---------------------------------------------------------------------------
// Block-wide exclusive scan of one 64-bit value per thread (all threads call;
// warp_sums holds 32 entries).

__device__ __forceinline__ uint64_t block_exclusive_scan64(uint64_t v, uint64_t* warp_sums, uint64_t& total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    const uint64_t warp_prefix = warp ? warp_sums[warp - 1] : 0;
    total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

// ---------------------------------------------------------------------------
// Warp-cooperative output of consecutive 18-byte records.

constexpr uint32_t kStageBytes = 592;   // per-warp staging area: >= 2 + 32 * 18 + 2, 16-byte multiple

// Stores the 18-byte records held by lanes [r0, r0 + len) into consecutive
// output slots starting at dst (2-byte aligned).  The run's byte image is
// assembled in the warp's staging area with dst's 4-byte phase (five aligned
// shared stores per lane), then copied out with coalesced 4-byte stores and a
// 2-byte store at each ragged end.  Lane j holds its record as n = {x, y, z,
// r | g << 16, b}.  All 32 lanes call with the same arguments.
__device__ __forceinline__ void store_run(uint8_t* dst, uint32_t r0, uint32_t len, const uint32_t (&n)[5],
                                          uint8_t* stage) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t h = (uint32_t)reinterpret_cast<uintptr_t>(dst) & 2u;   // bytes before dst in its word
    if (lane >= r0 && lane < r0 + len) {
        const uint32_t off = h + 18 * (lane - r0);
        const bool al = (off & 2u) == 0;
        // aligned record: words x, y, z, r|g at off, b at off + 16;
        // otherwise x's low half at off, then the record shifted by 16 bits
        const uint32_t o16 = al ? off + 16 : off;
        const uint32_t o32 = al ? off : off + 2;
        *reinterpret_cast<uint16_t*>(stage + o16) = (uint16_t)(al ? n[4] : n[0]);
        uint32_t* q = reinterpret_cast<uint32_t*>(stage + o32);
        q[0] = al ? n[0] : __funnelshift_r(n[0], n[1], 16);
        q[1] = al ? n[1] : __funnelshift_r(n[1], n[2], 16);
        q[2] = al ? n[2] : __funnelshift_r(n[2], n[3], 16);
        q[3] = al ? n[3] : __funnelshift_r(n[3], n[4], 16);
    }
    __syncwarp();
    const uint32_t bytes = h + 18 * len;
    uint32_t* gw = reinterpret_cast<uint32_t*>(dst - h);
    const uint32_t* sw = reinterpret_cast<const uint32_t*>(stage);
    if (h && lane == 0) *reinterpret_cast<uint16_t*>(dst) = *reinterpret_cast<const uint16_t*>(stage + 2);
    if ((bytes & 2u) && lane == 1)
        *reinterpret_cast<uint16_t*>(dst - h + bytes - 2) = *reinterpret_cast<const uint16_t*>(stage + bytes - 2);
    for (uint32_t w = (h >> 1) + lane; w < (bytes >> 2); w += 32) gw[w] = sw[w];
    __syncwarp();
}

// Stores one 18-byte record n = {x, y, z, r | g << 16, b} at slot pos of a
// 4-byte aligned record array with five stores: four aligned words and one
// 2-byte store, at the record's end (even slot) or start (odd slot).  The
// same instructions run for either parity.
__device__ __forceinline__ void store_record_words(uint8_t* base, uint64_t pos, const uint32_t (&n)[5]) {
    uint8_t* p = base + pos * 18;
    const bool odd = (pos & 1) != 0;
    *reinterpret_cast<uint16_t*>(p + (odd ? 0 : 16)) = (uint16_t)(odd ? n[0] : n[4]);
    uint32_t* q = reinterpret_cast<uint32_t*>(p + (odd ? 2 : 0));
    q[0] = odd ? __funnelshift_r(n[0], n[1], 16) : n[0];
    q[1] = odd ? __funnelshift_r(n[1], n[2], 16) : n[1];
    q[2] = odd ? __funnelshift_r(n[2], n[3], 16) : n[2];
    q[3] = odd ? __funnelshift_r(n[3], n[4], 16) : n[3];
}

#endif   // __CUDACC__

}   // namespace oc
