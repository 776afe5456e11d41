// Potree 2.0 export (PotreeExporter, OctreeLibrary/src/octree_exporter/
// potree_exporter.cu:35-173) and the session reports (statistics.json,
// OctreeApi/src/json_exporter.h:14-99; point-distribution histogram,
// octree_processor_impl/histogram.cu:39-119).
//
// metadata.json is written in the layout of nlohmann::ordered_json dumped with
// an indent of 4 (keys in insertion order, shortest round-trip doubles).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "builder.h"

namespace oc {

namespace {

// Minimal ordered JSON value with nlohmann-style pretty printing.
struct Json {
    enum Kind { Null, Int, UInt, Double, String, Array, Object } kind = Null;
    long long i = 0;
    unsigned long long u = 0;
    double d = 0;
    std::string s;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    static Json I(long long v) {
        Json j;
        j.kind = Int;
        j.i = v;
        return j;
    }
    static Json U(unsigned long long v) {
        Json j;
        j.kind = UInt;
        j.u = v;
        return j;
    }
    static Json D(double v) {
        Json j;
        j.kind = Double;
        j.d = v;
        return j;
    }
    static Json S(const std::string& v) {
        Json j;
        j.kind = String;
        j.s = v;
        return j;
    }
    static Json A(std::vector<Json> v) {
        Json j;
        j.kind = Array;
        j.arr = std::move(v);
        return j;
    }
    static Json O() {
        Json j;
        j.kind = Object;
        return j;
    }
    Json& operator[](const std::string& k) {
        if (kind != Object) kind = Object;
        for (auto& kv : obj)
            if (kv.first == k) return kv.second;
        obj.push_back({k, Json()});
        return obj.back().second;
    }
};

// Shortest decimal that round-trips, formatted like nlohmann::json (Grisu2
// digits, fixed notation for decimal exponents in (-4, 15], else d.ddde+XX).
std::string fmt_double(double v) {
    if (std::isnan(v) || std::isinf(v)) return "null";
    if (v == 0) return std::signbit(v) ? "-0.0" : "0.0";
    char buf[64];
    int prec = 1;
    for (; prec <= 17; ++prec) {
        std::snprintf(buf, sizeof buf, "%.*e", prec - 1, v);
        if (std::strtod(buf, nullptr) == v) break;
    }
    std::string sci = buf;
    bool neg = sci[0] == '-';
    if (neg) sci = sci.substr(1);
    size_t epos = sci.find('e');
    int e10 = std::atoi(sci.c_str() + epos + 1);
    std::string digits;
    for (size_t k = 0; k < epos; ++k)
        if (sci[k] != '.') digits += sci[k];
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    int k = (int)digits.size();
    int n = e10 + 1;
    std::string out;
    if (k <= n && n <= 15) {
        out = digits + std::string(n - k, '0') + ".0";
    } else if (0 < n && n <= 15) {
        out = digits.substr(0, n) + "." + digits.substr(n);
    } else if (-4 < n && n <= 0) {
        out = "0." + std::string(-n, '0') + digits;
    } else {
        out = digits.substr(0, 1);
        if (k > 1) out += "." + digits.substr(1);
        int ex = n - 1;
        char eb[16];
        std::snprintf(eb, sizeof eb, "e%c%02d", ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
        out += eb;
    }
    return neg ? "-" + out : out;
}

std::string escape(const std::string& s) {
    std::string o;
    for (char c : s) {
        if (c == '"' || c == '\\') {
            o += '\\';
            o += c;
        } else if ((unsigned char)c < 0x20) {
            char b[8];
            std::snprintf(b, sizeof b, "\\u%04x", c);
            o += b;
        } else {
            o += c;
        }
    }
    return o;
}

void dump(const Json& j, std::string& out, int indent) {
    std::string pad(indent + 4, ' '), pad0(indent, ' ');
    switch (j.kind) {
    case Json::Null:
        out += "null";
        break;
    case Json::Int:
        out += std::to_string(j.i);
        break;
    case Json::UInt:
        out += std::to_string(j.u);
        break;
    case Json::Double:
        out += fmt_double(j.d);
        break;
    case Json::String:
        out += "\"" + escape(j.s) + "\"";
        break;
    case Json::Array:
        if (j.arr.empty()) {
            out += "[]";
            break;
        }
        out += "[\n";
        for (size_t k = 0; k < j.arr.size(); ++k) {
            out += pad;
            dump(j.arr[k], out, indent + 4);
            out += k + 1 < j.arr.size() ? ",\n" : "\n";
        }
        out += pad0 + "]";
        break;
    case Json::Object:
        if (j.obj.empty()) {
            out += "{}";
            break;
        }
        out += "{\n";
        for (size_t k = 0; k < j.obj.size(); ++k) {
            out += pad + "\"" + escape(j.obj[k].first) + "\": ";
            dump(j.obj[k].second, out, indent + 4);
            out += k + 1 < j.obj.size() ? ",\n" : "\n";
        }
        out += pad0 + "}";
        break;
    }
}

void write_file(const std::string& path, const void* data, size_t bytes) {
    std::ofstream f(path, std::ios::binary);
    if (!f) throw Error("cannot open " + path);
    f.write(static_cast<const char*>(data), (std::streamsize)bytes);
    if (!f) throw Error("cannot write " + path);
}

}   // namespace

void Builder::export_potree(const std::string& dir) const {
    // hierarchy.bin: BFS entries (potree_exporter.cu:62-96)
    std::vector<uint8_t> h = hierarchy();
    write_file(dir + "/hierarchy.bin", h.data(), h.size());
    // octree.bin: the records referenced by the hierarchy (potree_exporter.cu:56)
    std::unique_ptr<uint8_t[]> recs(new uint8_t[stats_.points_total * 18 + 1]);
    copy_records(recs.get());
    write_file(dir + "/octree.bin", recs.get(), stats_.points_total * 18);

    // metadata.json (potree_exporter.cu:113-173)
    const double side = cfg_.bb_max[0] - cfg_.bb_min[0];
    const double spacing = side / cfg_.sub_grid;
    uint32_t points_exported = 0;   // uint32 accumulation as in the reference
    for (const auto& v : nodes_) points_exported += v.points;
    Json m = Json::O();
    m["version"] = Json::S("2.0");
    m["name"] = Json::S("GpuPotreeConverter");
    m["description"] = Json::S("Generated with GpuPotreeConverter");
    m["points"] = Json::U(points_exported);
    m["projection"] = Json::S("");
    std::vector<Json> flags;
    flags.push_back(Json::S(cfg_.replacement ? "REPLACING" : "ADDITIVE"));
    flags.push_back(Json::S(cfg_.random ? "EXPLICIT-RANDOM-SUBSAMPLING" : "IMPLICIT-RANDOM-SUBSAMPLING"));
    if (cfg_.inter) flags.push_back(Json::S("INTER-CELL-COLOR-FILTERING"));
    else if (cfg_.intra) flags.push_back(Json::S("INTRA-CELL-COLOR-FILTERING"));
    m["flags"] = Json::A(flags);
    Json hier = Json::O();
    hier["firstChunkSize"] = Json::U((unsigned long long)(uint32_t)(nodes_.size() * 22));
    hier["stepSize"] = Json::U(100);
    hier["depth"] = Json::U(20);
    m["hierarchy"] = hier;
    m["offset"] = Json::A({Json::I(0), Json::I(0), Json::I(0)});
    m["scale"] = Json::A({Json::D(cfg_.scale[0]), Json::D(cfg_.scale[1]), Json::D(cfg_.scale[2])});
    m["spacing"] = Json::D(spacing);
    Json bb = Json::O();
    bb["min"] = Json::A({Json::I(0), Json::I(0), Json::I(0)});
    bb["max"] = Json::A({Json::D(side), Json::D(side), Json::D(side)});
    m["boundingBox"] = bb;
    m["encoding"] = Json::S("default");
    Json pos = Json::O();
    pos["name"] = Json::S("position");
    pos["description"] = Json::S("");
    pos["size"] = Json::U(12);
    pos["numElements"] = Json::U(3);
    pos["elementSize"] = Json::U(4);
    pos["type"] = Json::S("int32");
    pos["min"] = Json::A({Json::I(0), Json::I(0), Json::I(0)});
    pos["max"] = Json::A({Json::D(side), Json::D(side), Json::D(side)});
    Json col = Json::O();
    col["name"] = Json::S("rgb");
    col["description"] = Json::S("");
    col["size"] = Json::U(6);
    col["numElements"] = Json::U(3);
    col["elementSize"] = Json::U(2);
    col["type"] = Json::S("uint16");
    col["min"] = Json::A({Json::I(0), Json::I(0), Json::I(0)});
    col["max"] = Json::A({Json::I(65536), Json::I(65536), Json::I(65536)});
    m["attributes"] = Json::A({pos, col});
    std::string text;
    dump(m, text, 0);
    write_file(dir + "/metadata.json", text.data(), text.size());
}

void Builder::export_json_report(const std::string& file, const ReportExtras& extras) const {
    // statistics.json schema of json_exporter.h:14-99; timings are this
    // session's CUDA-event stage times.
    const Stats& S = stats_;
    Json st = Json::O();
    st["depth"] = Json::U(S.depth);
    st["chunking"]["grid"] = Json::U(cfg_.chunk_grid);
    st["chunking"]["mergingThreshold"] = Json::U(cfg_.threshold);
    st["subsampling"]["grid"] = Json::U(cfg_.sub_grid);
    st["subsampling"]["strategy"] = Json::S(cfg_.random ? "EXPLICIT RANDOM SUBSAMPLING" : "IMPLICIT RANDOM SUBSAMPLING");
    if (cfg_.intra) st["subsampling"]["averaging"] = Json::S("INTRA-CELL AVERAGING");
    else if (cfg_.inter) st["subsampling"]["averaging"] = Json::S("INTER-CELL AVERAGING");
    st["resultNodes"]["octreeNodes"] = Json::U(S.leaf_nodes + S.internal_nodes);
    st["resultNodes"]["leafNodeAmount"] = Json::U(S.leaf_nodes);
    st["resultNodes"]["internalNodeAmount"] = Json::U(S.internal_nodes);
    st["resultNodes"]["maxLeafDepth"] = Json::U(S.max_leaf_depth);
    st["overallNodes"]["sparseOctreeNodes"] = Json::U(S.sparse_nodes);
    st["overallNodes"]["denseOctreeNodes"] = Json::U(S.dense_nodes);
    st["overallNodes"]["memorySaving"] =
        Json::D((double)((1 - ((float)S.sparse_nodes / (float)S.dense_nodes)) * 100));
    st["pointDistribution"]["meanPointsPerLeafNode"] = Json::D(S.mean_leaf_points);
    st["pointDistribution"]["stdevPointsPerLeafNode"] = Json::D(S.stdev_leaf_points);
    st["pointDistribution"]["minPointsPerNode"] = Json::U(S.min_leaf_points);
    st["pointDistribution"]["maxPointsPerNode"] = Json::U(S.max_leaf_points);
    // the last build's stages: transfers under "memcpy", the rest (kernels on
    // the build stream) under "kernel"
    double acc = 0, acc_copy = 0, acc_proc = 0;
    Json& tm = st["timings"];
    tm["kernel"] = Json::O();
    tm["memcpy"] = Json::O();
    tm["cudamalloc"] = Json::O();
    tm["process"] = Json::O();
    for (const auto& t : timings_) {
        if (t.first == "upload" || t.first == "upload_count" || t.first == "d2h") {
            tm["memcpy"][t.first] = Json::D(t.second);
            acc_copy += t.second;
            continue;
        }
        tm["kernel"][t.first]["invocations"] = Json::U(1);
        tm["kernel"][t.first]["duration"] = Json::D(t.second);
        acc += t.second;
    }
    tm["cudamalloc"]["device buffers"] = Json::D(extras.allocs.ms);
    for (const auto& p : extras.process_ms) {
        tm["process"][p.first] = Json::D(p.second);
        acc_proc += p.second;
    }
    tm["accumulatedKernelTime"] = Json::D(acc);
    tm["accumulatedMemCpyTime"] = Json::D(acc_copy);
    tm["accumulatedMallocTime"] = Json::D(extras.allocs.ms);
    tm["accumulatedProcessTimings"] = Json::D(acc_proc);
    // memory (json_exporter.h:88-96): the device allocations this session
    // holds, the number of allocations it made and their cumulated bytes
    uint64_t held = 0;
    Json events = Json::O();
    for (const auto& a : device_allocations()) {
        held += a.second;
        events[a.first] = Json::U(a.second);
    }
    st["memory"]["peak"] = Json::U(held);
    st["memory"]["reserveEvents"] = Json::U(extras.allocs.events);
    st["memory"]["cumulatedReserved"] = Json::U(extras.allocs.bytes);
    st["memory"]["events"] = events;
    std::string text;
    dump(st, text, 0);
    write_file(file, text.data(), text.size());
}

void Builder::export_histogram(const std::string& file, uint32_t bin_width) const {
    // histogram.cu:39-119: leaf point counts binned from the minimum.
    const Stats& S = stats_;
    if (bin_width == 0)
        bin_width = (uint32_t)std::ceil(3.5f * (S.stdev_leaf_points / std::pow((float)S.leaf_nodes, 1.f / 3.f)));
    if (bin_width == 0) bin_width = 1;
    uint32_t bins = (uint32_t)(std::ceil((double)(S.max_leaf_points - S.min_leaf_points)) / bin_width) + 1;
    std::vector<uint32_t> counts(bins, 0);
    for (const auto& v : nodes_)
        if (!v.internal) counts[std::min<uint32_t>((v.count - S.min_leaf_points) / bin_width, bins - 1)]++;
    std::ostringstream o;
    o << "<html>\n    <head>\n        <script src=\"https://cdn.jsdelivr.net/npm/chart.js@2.8.0\"></script>\n"
      << "    </head>\n    <body>\n        <canvas id=\"myChart\"></canvas>\n        <script>\n"
      << "            var ctx = document.getElementById('myChart').getContext('2d');\n"
      << "            var chart = new Chart(ctx, {type: 'bar', data:{labels:[";
    for (uint32_t b = 0; b < bins; ++b)
        o << (b ? "," : "") << "'" << S.min_leaf_points + b * bin_width << " - " << S.min_leaf_points + (b + 1) * bin_width
          << "'";
    o << "], datasets:[{label: 'Point Distribution: binWidth(" << bin_width << "), mergingThreshold(" << cfg_.threshold
      << "), points(" << cfg_.n << ")', backgroundColor: 'rgb(255, 99, 132)', borderColor: 'rgb(255, 99, 132)', data:[";
    for (uint32_t b = 0; b < bins; ++b) o << (b ? "," : "") << counts[b];
    o << "]}]}});\n        </script>\n    </body>\n</html>";
    std::string text = o.str();
    write_file(file, text.data(), text.size());
}

}   // namespace oc
