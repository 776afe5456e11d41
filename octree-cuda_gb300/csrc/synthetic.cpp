// Seeded synthetic point clouds in the reference's raw input format
// (headerless interleaved records: 3 x float32 or float64 coordinates, then
// 3 x uint8 RGB; src/main.cpp:12-22, README.md:65-74), plus the CLI's
// bounding-box computation (src/boundingbox.h:11-52).
//
// The reference's own datasets (morrobay / heidentor / coin .bin) are release
// downloads that are not available here; these generators stand in for them at
// the same point counts, record layouts and scales.  Every cloud is a pure
// function of (kind, type, n, seed): work is split into tiles whose random
// streams are keyed by (seed, tile), so the thread count does not matter.
//
// Points are emitted tile by tile (a spatially coherent order, like the strip
// order of a scanner), with uniform positions inside each tile.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

namespace {

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {   // splitmix64 (Steele, Lea, Flood 2014)
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uni() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    double gauss() {   // Box-Muller
        double u1 = uni(), u2 = uni();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

uint64_t mix(uint64_t a, uint64_t b) {
    Rng r(a * 0x9E3779B97F4A7C15ull ^ (b + 0x632BE59BD9B4E019ull));
    r.next();
    return r.next();
}

double lattice(int64_t x, int64_t y, uint64_t seed) {
    uint64_t h = mix(seed, (uint64_t)(x * 73856093ll) ^ (uint64_t)(y * 19349663ll));
    return (h >> 11) * (1.0 / 9007199254740992.0);
}

double value_noise(double x, double y, uint64_t seed) {
    double fx = std::floor(x), fy = std::floor(y);
    int64_t ix = (int64_t)fx, iy = (int64_t)fy;
    double tx = x - fx, ty = y - fy;
    tx = tx * tx * (3 - 2 * tx);
    ty = ty * ty * (3 - 2 * ty);
    double a = lattice(ix, iy, seed), b = lattice(ix + 1, iy, seed);
    double c = lattice(ix, iy + 1, seed), d = lattice(ix + 1, iy + 1, seed);
    return (a + (b - a) * tx) + ((c + (d - c) * tx) - (a + (b - a) * tx)) * ty;
}

double fbm(double x, double y, uint64_t seed, int octaves) {
    double s = 0, amp = 1, norm = 0;
    for (int o = 0; o < octaves; ++o) {
        s += amp * (2.0 * value_noise(x, y, seed + o) - 1.0);
        norm += amp;
        amp *= 0.5;
        x *= 2.0;
        y *= 2.0;
    }
    return s / norm;
}

uint8_t clamp8(double v) {
    return (uint8_t)std::min(255.0, std::max(0.0, std::floor(v)));
}

struct Writer {
    uint8_t* out;
    uint32_t type;
    uint32_t stride;
    void put(uint64_t i, double x, double y, double z, uint8_t r, uint8_t g, uint8_t b) const {
        uint8_t* p = out + i * stride;
        if (type == 0) {
            float f[3] = {(float)x, (float)y, (float)z};
            std::memcpy(p, f, 12);
            p[12] = r;
            p[13] = g;
            p[14] = b;
            if (stride > 15) std::memset(p + 15, 0, stride - 15);
        } else {
            double d[3] = {x, y, z};
            std::memcpy(p, d, 24);
            p[24] = r;
            p[25] = g;
            p[26] = b;
            if (stride > 27) std::memset(p + 27, 0, stride - 27);
        }
    }
};

// A work item emits `count` points starting at record `begin`.
struct Item {
    uint64_t begin;
    uint64_t count;
    std::function<void(Rng&, const Writer&, uint64_t, uint64_t)> emit;
};

void run_items(std::vector<Item>& items, const Writer& w, uint64_t seed, int threads) {
    std::vector<std::thread> pool;
    int T = threads > 0 ? threads : 1;
    for (int t = 0; t < T; ++t)
        pool.emplace_back([&, t] {
            for (size_t k = t; k < items.size(); k += T) {
                Rng r(mix(seed, k + 1));
                items[k].emit(r, w, items[k].begin, items[k].count);
            }
        });
    for (auto& th : pool) th.join();
}

// Split n points over weights; per-item counts sum exactly to n.
std::vector<uint64_t> apportion(const std::vector<double>& w, uint64_t n) {
    double tot = 0;
    for (double v : w) tot += v;
    std::vector<uint64_t> c(w.size());
    double cum = 0;
    uint64_t prev = 0;
    for (size_t i = 0; i < w.size(); ++i) {
        cum += w[i];
        uint64_t upto = (i + 1 == w.size()) ? n : (uint64_t)std::floor(cum / tot * (double)n);
        if (upto < prev) upto = prev;
        c[i] = upto - prev;
        prev = upto;
    }
    return c;
}

// Kind 0: 10 m x 10 m heightfield (fBm amplitude 0.5 m) plus 20 boxes,
// sigma = 1 mm, colour = smooth function of position + U(-10, 10).
void gen_heightfield_boxes(const Writer& w, uint64_t n, uint64_t seed, int threads) {
    const double side = 10.0, amp = 0.5, sigma = 0.001;
    const uint64_t hs = seed * 31 + 7;
    auto height = [&](double x, double y) { return amp * fbm(x / 3.0, y / 3.0, hs, 6); };
    auto colour = [](Rng& r, double x, double y, double z, uint8_t c[3]) {
        c[0] = clamp8(128 + 90 * std::sin(0.7 * x) + 20 * z + (r.uni() * 20 - 10));
        c[1] = clamp8(128 + 90 * std::cos(0.5 * y) + (r.uni() * 20 - 10));
        c[2] = clamp8(128 + 60 * std::sin(0.3 * (x + y)) + 80 * z + (r.uni() * 20 - 10));
    };
    struct Box {
        double cx, cy, z0, hx, hy, h;
    };
    std::vector<Box> boxes;
    Rng br(mix(seed, 0xB0B0));
    for (int b = 0; b < 20; ++b) {
        Box bx;
        bx.cx = 1 + 8 * br.uni();
        bx.cy = 1 + 8 * br.uni();
        bx.hx = 0.15 + 0.6 * br.uni();
        bx.hy = 0.15 + 0.6 * br.uni();
        bx.h = 0.3 + 1.7 * br.uni();
        bx.z0 = height(bx.cx, bx.cy);
        boxes.push_back(bx);
    }
    const uint64_t n_boxes = n / 5, n_hf = n - n_boxes;
    const int TN = 128;   // heightfield tiles per axis
    std::vector<double> wt(TN * TN, 1.0);
    auto hc = apportion(wt, n_hf);
    std::vector<double> bw;
    for (auto& b : boxes) bw.push_back(4 * b.hx * b.hy + 2 * b.h * (2 * b.hx + 2 * b.hy));
    auto bc = apportion(bw, n_boxes);
    std::vector<Item> items;
    uint64_t pos = 0;
    for (int ty = 0; ty < TN; ++ty)
        for (int k = 0; k < TN; ++k) {
            int tx = (ty & 1) ? TN - 1 - k : k;   // serpentine strips
            uint64_t c = hc[ty * TN + tx];
            double x0 = side * tx / TN, y0 = side * ty / TN, ts = side / TN;
            items.push_back({pos, c, [=](Rng& r, const Writer& W, uint64_t b, uint64_t m) {
                                 for (uint64_t i = 0; i < m; ++i) {
                                     double x = x0 + ts * r.uni(), y = y0 + ts * r.uni();
                                     double z = height(x, y);
                                     uint8_t col[3];
                                     colour(r, x, y, z, col);
                                     W.put(b + i, x + sigma * r.gauss(), y + sigma * r.gauss(), z + sigma * r.gauss(),
                                           col[0], col[1], col[2]);
                                 }
                             }});
            pos += c;
        }
    for (size_t bi = 0; bi < boxes.size(); ++bi) {
        Box bx = boxes[bi];
        uint64_t c = bc[bi];
        items.push_back({pos, c, [=](Rng& r, const Writer& W, uint64_t b, uint64_t m) {
                             double atop = 4 * bx.hx * bx.hy, ax = 2 * bx.h * bx.hy, ay = 2 * bx.h * bx.hx;
                             double tot = atop + 2 * ax + 2 * ay;
                             for (uint64_t i = 0; i < m; ++i) {
                                 double s = r.uni() * tot, x, y, z;
                                 if (s < atop) {
                                     x = bx.cx + bx.hx * (2 * r.uni() - 1);
                                     y = bx.cy + bx.hy * (2 * r.uni() - 1);
                                     z = bx.z0 + bx.h;
                                 } else if (s < atop + 2 * ax) {
                                     x = bx.cx + ((s < atop + ax) ? -bx.hx : bx.hx);
                                     y = bx.cy + bx.hy * (2 * r.uni() - 1);
                                     z = bx.z0 + bx.h * r.uni();
                                 } else {
                                     x = bx.cx + bx.hx * (2 * r.uni() - 1);
                                     y = bx.cy + ((s < atop + 2 * ax + ay) ? -bx.hy : bx.hy);
                                     z = bx.z0 + bx.h * r.uni();
                                 }
                                 uint8_t col[3];
                                 col[0] = clamp8(200 - 40 * (double)(bi % 5) + (r.uni() * 20 - 10));
                                 col[1] = clamp8(60 + 30 * (double)(bi % 7) + (r.uni() * 20 - 10));
                                 col[2] = clamp8(90 + 50 * z + (r.uni() * 20 - 10));
                                 W.put(b + i, x + sigma * r.gauss(), y + sigma * r.gauss(), z + sigma * r.gauss(),
                                       col[0], col[1], col[2]);
                             }
                         }});
        pos += c;
    }
    run_items(items, w, seed, threads);
}

// Kind 1: 40 planes and 12 cylinders inside a 30 m box, per-surface density
// factor log-uniform in [1, 20], sigma = 2 mm, per-surface base colour + noise.
void gen_planes_cylinders(const Writer& w, uint64_t n, uint64_t seed, int threads) {
    const double box = 30.0, sigma = 0.002;
    struct Surf {
        int kind;   // 0 plane, 1 cylinder
        double c[3], u[3], v[3];   // plane: centre and half-extent axes
        double r, h;               // cylinder radius/height (axis z, centre c)
        double area, dens;
        uint8_t col[3];
    };
    std::vector<Surf> s;
    Rng g(mix(seed, 0x5EED));
    auto unit = [&](double a[3]) {
        double z = 2 * g.uni() - 1, t = 6.283185307179586 * g.uni(), q = std::sqrt(1 - z * z);
        a[0] = q * std::cos(t);
        a[1] = q * std::sin(t);
        a[2] = z;
    };
    for (int i = 0; i < 40; ++i) {
        Surf p{};
        p.kind = 0;
        double nrm[3], tmp[3];
        unit(nrm);
        unit(tmp);
        // u = normalize(tmp x nrm), v = nrm x u
        double u[3] = {tmp[1] * nrm[2] - tmp[2] * nrm[1], tmp[2] * nrm[0] - tmp[0] * nrm[2], tmp[0] * nrm[1] - tmp[1] * nrm[0]};
        double ul = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        for (double& x : u) x /= ul;
        double v[3] = {nrm[1] * u[2] - nrm[2] * u[1], nrm[2] * u[0] - nrm[0] * u[2], nrm[0] * u[1] - nrm[1] * u[0]};
        double a = 1 + 6 * g.uni(), b = 1 + 6 * g.uni();
        for (int k = 0; k < 3; ++k) {
            p.c[k] = 8 + 14 * g.uni();
            p.u[k] = u[k] * a;
            p.v[k] = v[k] * b;
        }
        p.area = 4 * a * b;
        p.dens = std::exp(g.uni() * std::log(20.0));
        for (auto& c : p.col) c = (uint8_t)(30 + 200 * g.uni());
        s.push_back(p);
    }
    for (int i = 0; i < 12; ++i) {
        Surf c{};
        c.kind = 1;
        c.r = 0.2 + 1.8 * g.uni();
        c.h = 2 + 18 * g.uni();
        c.c[0] = 3 + 24 * g.uni();
        c.c[1] = 3 + 24 * g.uni();
        c.c[2] = 1 + (28 - c.h) * g.uni();
        c.area = 6.283185307179586 * c.r * c.h;
        c.dens = std::exp(g.uni() * std::log(20.0));
        for (auto& k : c.col) k = (uint8_t)(30 + 200 * g.uni());
        s.push_back(c);
    }
    std::vector<double> wt;
    for (auto& q : s) wt.push_back(q.area * q.dens);
    auto cnt = apportion(wt, n);
    std::vector<Item> items;
    uint64_t pos = 0;
    const uint64_t chunk = 1 << 16;
    for (size_t si = 0; si < s.size(); ++si) {
        Surf q = s[si];
        uint64_t total = cnt[si];
        // a surface is emitted as consecutive strips of `chunk` points
        uint64_t strips = (total + chunk - 1) / chunk;
        for (uint64_t st = 0; st < strips; ++st) {
            uint64_t c = std::min<uint64_t>(chunk, total - st * chunk);
            double f0 = (double)st / strips, f1 = (double)(st + 1) / strips;
            items.push_back({pos, c, [=](Rng& r, const Writer& W, uint64_t b, uint64_t m) {
                                 for (uint64_t i = 0; i < m; ++i) {
                                     double x, y, z;
                                     double a = f0 + (f1 - f0) * r.uni();
                                     if (q.kind == 0) {
                                         double sa = 2 * a - 1, sb = 2 * r.uni() - 1;
                                         x = q.c[0] + sa * q.u[0] + sb * q.v[0];
                                         y = q.c[1] + sa * q.u[1] + sb * q.v[1];
                                         z = q.c[2] + sa * q.u[2] + sb * q.v[2];
                                     } else {
                                         double th = 6.283185307179586 * a;
                                         x = q.c[0] + q.r * std::cos(th);
                                         y = q.c[1] + q.r * std::sin(th);
                                         z = q.c[2] + q.h * r.uni();
                                     }
                                     x = std::min(box, std::max(0.0, x + sigma * r.gauss()));
                                     y = std::min(box, std::max(0.0, y + sigma * r.gauss()));
                                     z = std::min(box, std::max(0.0, z + sigma * r.gauss()));
                                     W.put(b + i, x, y, z, clamp8(q.col[0] + 30 * r.uni() - 15),
                                           clamp8(q.col[1] + 30 * r.uni() - 15), clamp8(q.col[2] + 30 * r.uni() - 15));
                                 }
                             }});
            pos += c;
        }
    }
    run_items(items, w, seed, threads);
}

// Kind 2: 3 km x 3 km terrain heightfield with Zipf-clustered density:
// 64 hot spots, the k-th with peak density 1 + 99 / k times the background.
void gen_terrain_zipf(const Writer& w, uint64_t n, uint64_t seed, int threads) {
    const double side = 3000.0, x0 = 412000.0, y0 = 4505000.0, z0 = 120.0;
    const uint64_t hs = seed * 131 + 3;
    auto height = [&](double x, double y) { return z0 + 180.0 * fbm((x - x0) / 700.0, (y - y0) / 700.0, hs, 8); };
    struct Hot {
        double x, y, s, a;
    };
    std::vector<Hot> hot;
    Rng g(mix(seed, 0x2197));
    for (int k = 1; k <= 64; ++k)
        hot.push_back({x0 + side * (0.05 + 0.9 * g.uni()), y0 + side * (0.05 + 0.9 * g.uni()), 10 + 50 * g.uni(),
                       99.0 / k});
    const int TN = 512;
    const double ts = side / TN;
    std::vector<double> wt((size_t)TN * TN);
    for (int ty = 0; ty < TN; ++ty)
        for (int tx = 0; tx < TN; ++tx) {
            double cx = x0 + (tx + 0.5) * ts, cy = y0 + (ty + 0.5) * ts, d = 1.0;
            for (auto& h : hot) {
                double dx = cx - h.x, dy = cy - h.y;
                d += h.a * std::exp(-(dx * dx + dy * dy) / (2 * h.s * h.s));
            }
            wt[(size_t)ty * TN + tx] = d;
        }
    auto cnt = apportion(wt, n);
    std::vector<Item> items;
    uint64_t pos = 0;
    for (int ty = 0; ty < TN; ++ty)
        for (int k = 0; k < TN; ++k) {
            int tx = (ty & 1) ? TN - 1 - k : k;
            uint64_t c = cnt[(size_t)ty * TN + tx];
            double ax = x0 + tx * ts, ay = y0 + ty * ts;
            items.push_back({pos, c, [=](Rng& r, const Writer& W, uint64_t b, uint64_t m) {
                                 for (uint64_t i = 0; i < m; ++i) {
                                     double x = ax + ts * r.uni(), y = ay + ts * r.uni();
                                     double z = height(x, y) + 0.05 * r.gauss();
                                     double hgt = (z - z0) / 180.0;
                                     W.put(b + i, x, y, z, clamp8(110 + 90 * hgt + 12 * r.gauss()),
                                           clamp8(120 + 60 * std::sin((x - x0) / 90.0) + 12 * r.gauss()),
                                           clamp8(90 - 70 * hgt + 12 * r.gauss()));
                                 }
                             }});
            pos += c;
        }
    run_items(items, w, seed, threads);
}

// Kind 3: unit lattice cuboid, side^3 points at integer + 0.5 (the reference
// test fixture, misc/tools.cu:7-23 and 167-190), with a zero colour.
void gen_cuboid(const Writer& w, uint64_t n, int threads) {
    uint64_t side = (uint64_t)std::llround(std::cbrt((double)n));
    std::vector<std::thread> pool;
    int T = threads > 0 ? threads : 1;
    for (int t = 0; t < T; ++t)
        pool.emplace_back([&, t] {
            for (uint64_t i = t; i < n; i += T) {
                uint64_t xy = side * side, z = i / xy, y = (i - z * xy) / side, x = (i - z * xy) % side;
                w.put(i, x + 0.5, y + 0.5, z + 0.5, 0, 0, 0);
            }
        });
    for (auto& th : pool) th.join();
}

}   // namespace

extern "C" {

// kind: 0 heightfield+boxes, 1 planes+cylinders, 2 terrain with Zipf hot
// spots, 3 unit cuboid.  type: 0 float32, 1 float64.  Returns 0 on success.
int ocsynth_generate(int kind, int type, uint64_t n, uint32_t stride, uint64_t seed, uint8_t* out, int threads) {
    if (type < 0 || type > 1 || !out) return -1;
    if (stride < (type == 0 ? 15u : 27u)) return -1;
    Writer w{out, (uint32_t)type, stride};
    switch (kind) {
    case 0:
        gen_heightfield_boxes(w, n, seed, threads);
        return 0;
    case 1:
        gen_planes_cylinders(w, n, seed, threads);
        return 0;
    case 2:
        gen_terrain_zipf(w, n, seed, threads);
        return 0;
    case 3:
        gen_cuboid(w, n, threads);
        return 0;
    default:
        return -1;
    }
}

// calculateRealBB + calculateCubicBB (src/boundingbox.h:11-52): real bbox by
// fmin/fmax over the coordinates, then a cube of the largest extent centred on
// it.  out = {minX, minY, minZ, maxX, maxY, maxZ} of the cube.
void ocsynth_cubic_bbox(const uint8_t* cloud, uint64_t n, uint32_t stride, int type, double* out, int threads) {
    int T = threads > 0 ? threads : 1;
    std::vector<std::vector<double>> part(T, std::vector<double>{INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY});
    std::vector<std::thread> pool;
    uint64_t chunk = (n + T - 1) / T;
    for (int t = 0; t < T; ++t)
        pool.emplace_back([&, t] {
            uint64_t a = t * chunk, b = std::min<uint64_t>(n, a + chunk);
            auto& bb = part[t];
            for (uint64_t i = a; i < b; ++i) {
                double p[3];
                if (type == 0) {
                    float f[3];
                    std::memcpy(f, cloud + i * stride, 12);
                    p[0] = f[0];
                    p[1] = f[1];
                    p[2] = f[2];
                } else {
                    std::memcpy(p, cloud + i * stride, 24);
                }
                for (int k = 0; k < 3; ++k) {
                    bb[k] = std::fmin(bb[k], p[k]);
                    bb[3 + k] = std::fmax(bb[3 + k], p[k]);
                }
            }
        });
    for (auto& th : pool) th.join();
    std::vector<double> real{INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (auto& bb : part)
        for (int k = 0; k < 3; ++k) {
            real[k] = std::fmin(real[k], bb[k]);
            real[3 + k] = std::fmax(real[3 + k], bb[3 + k]);
        }
    double dx = real[3] - real[0], dy = real[4] - real[1], dz = real[5] - real[2];
    double side = std::fmax(std::fmax(dx, dy), dz);
    out[0] = real[0] - ((side - dx) / 2.0f);
    out[1] = real[1] - ((side - dy) / 2.0f);
    out[2] = real[2] - ((side - dz) / 2.0f);
    out[3] = out[0] + side;
    out[4] = out[1] + side;
    out[5] = out[2] + side;
}

}   // extern "C"
