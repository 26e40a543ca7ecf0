// CSV input in traccc's on-disk event format (hits, measurements and the
// measurement-to-hit map), read by column name like the reference's
// named-tuple readers (io/src/csv/make_hit_reader.cpp,
// make_measurement_reader.cpp, make_measurement_hit_id_reader.cpp).
#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "seedgb.h"

namespace {

class CsvFile {
public:
    explicit CsvFile(const char* path) : f_(path ? std::fopen(path, "rb") : nullptr) {}
    ~CsvFile() {
        if (f_) std::fclose(f_);
    }
    bool ok() const { return f_ != nullptr; }

    // Next line without the line break; false at the end of the file.
    bool line(std::string& out) {
        out.clear();
        if (!f_) return false;
        int c;
        bool any = false;
        while ((c = std::fgetc(f_)) != EOF) {
            any = true;
            if (c == '\n') break;
            out.push_back(static_cast<char>(c));
        }
        if (!out.empty() && out.back() == '\r') out.pop_back();
        return any;
    }

private:
    std::FILE* f_;
};

void split(const std::string& s, std::vector<std::string>& fields) {
    fields.clear();
    std::string cur;
    for (char ch : s) {
        if (ch == ',') {
            fields.push_back(cur);
            cur.clear();
        } else if (ch != ' ' && ch != '\t') {
            cur.push_back(ch);
        }
    }
    fields.push_back(cur);
}

// Column index of each wanted name in the header, or -1.
std::vector<int> columns(const std::vector<std::string>& header,
                         const std::vector<const char*>& names) {
    std::vector<int> idx;
    for (const char* n : names) {
        int k = -1;
        for (size_t i = 0; i < header.size(); ++i)
            if (header[i] == n) k = static_cast<int>(i);
        idx.push_back(k);
    }
    return idx;
}

bool to_float(const std::string& s, float& v) {
    if (s.empty()) return false;
    char* end = nullptr;
    v = std::strtof(s.c_str(), &end);  // correctly rounded, as the reference's reader
    return end && *end == '\0';
}

bool to_u64(const std::string& s, uint64_t& v) {
    if (s.empty() || s[0] == '-') return false;
    errno = 0;
    char* end = nullptr;
    v = std::strtoull(s.c_str(), &end, 10);
    return end && *end == '\0' && errno != ERANGE;
}

// local_key: the reference's CSV record holds it as uint8_t
// (io/include/traccc/io/csv/measurement.hpp:23), which its stream-based reader
// extracts as one character whose byte value is the key -- the reference's own
// test data stores the raw byte (tests/io/mock_data/
// event000000000-measurements.csv: 0x06, loc0 and loc1 active).  A one-
// character field is therefore that byte (a digit '0'..'7' gives the same
// active bits as its decimal value); a longer field is read as a decimal key
// up to 255 (an extension: the reference would read only its first character).
bool to_key(const std::string& s, uint64_t& key) {
    if (s.size() == 1) {
        key = static_cast<unsigned char>(s[0]);
        return true;
    }
    return to_u64(s, key) && key <= 255;
}

}  // namespace

extern "C" {

int64_t seedgb_csv_rows(const char* path) {
    CsvFile f(path);
    if (!f.ok()) return -1;
    std::string l;
    if (!f.line(l)) return -1;
    int64_t n = 0;
    while (f.line(l))
        if (!l.empty()) ++n;
    return n;
}

seedgb_status seedgb_csv_read_spacepoints(const char* hits_path, const char* meas_hit_map_path,
                                          uint64_t capacity, uint32_t* mi1, uint32_t* mi2,
                                          float* global, float* zvar, float* rvar,
                                          uint64_t* n) {
    if (!hits_path || !n || (capacity && (!mi1 || !mi2 || !global || !zvar || !rvar)))
        return SEEDGB_INVALID_ARGUMENT;
    *n = 0;
    std::vector<std::string> fields;
    std::string l;
    // measurement-hit-id map: hit row index -> measurement index (first row wins)
    std::unordered_map<uint64_t, uint64_t> hit_to_meas;
    if (meas_hit_map_path) {
        CsvFile m(meas_hit_map_path);
        if (!m.ok() || !m.line(l)) return SEEDGB_INVALID_ARGUMENT;
        split(l, fields);
        const std::vector<int> c = columns(fields, {"measurement_id", "hit_id"});
        if (c[0] < 0 || c[1] < 0) return SEEDGB_INVALID_ARGUMENT;
        while (m.line(l)) {
            if (l.empty()) continue;
            split(l, fields);
            uint64_t mid, hid;
            if (fields.size() <= static_cast<size_t>(std::max(c[0], c[1])) ||
                !to_u64(fields[c[0]], mid) || !to_u64(fields[c[1]], hid))
                return SEEDGB_INVALID_ARGUMENT;
            hit_to_meas.emplace(hid, mid);
        }
    }
    CsvFile h(hits_path);
    if (!h.ok() || !h.line(l)) return SEEDGB_INVALID_ARGUMENT;
    split(l, fields);
    const std::vector<int> c = columns(fields, {"tx", "ty", "tz"});
    if (c[0] < 0 || c[1] < 0 || c[2] < 0) return SEEDGB_INVALID_ARGUMENT;
    const size_t need = static_cast<size_t>(std::max(c[0], std::max(c[1], c[2])));
    uint64_t i = 0;
    while (h.line(l)) {
        if (l.empty()) continue;
        split(l, fields);
        float x, y, z;
        if (fields.size() <= need || !to_float(fields[c[0]], x) || !to_float(fields[c[1]], y) ||
            !to_float(fields[c[2]], z))
            return SEEDGB_INVALID_ARGUMENT;
        if (i < capacity) {
            const auto it = hit_to_meas.find(i);
            mi1[i] = it != hit_to_meas.end() ? static_cast<uint32_t>(it->second)
                                             : SEEDGB_INVALID_MEASUREMENT_INDEX;
            mi2[i] = SEEDGB_INVALID_MEASUREMENT_INDEX;
            global[3 * i] = x;
            global[3 * i + 1] = y;
            global[3 * i + 2] = z;
            zvar[i] = 0.f;
            rvar[i] = 0.f;
        }
        ++i;
    }
    *n = i;
    return i > capacity ? SEEDGB_CAPACITY_OVERFLOW : SEEDGB_OK;
}

seedgb_status seedgb_csv_read_measurements(const char* meas_path, uint64_t capacity,
                                           float* local_position, uint64_t* surface_link,
                                           uint8_t* dimensions, uint64_t* n) {
    if (!meas_path || !n || (capacity && (!local_position || !surface_link || !dimensions)))
        return SEEDGB_INVALID_ARGUMENT;
    *n = 0;
    CsvFile f(meas_path);
    std::string l;
    std::vector<std::string> fields;
    if (!f.ok() || !f.line(l)) return SEEDGB_INVALID_ARGUMENT;
    split(l, fields);
    const std::vector<int> c = columns(fields, {"geometry_id", "local_key", "local0", "local1"});
    for (int k : c)
        if (k < 0) return SEEDGB_INVALID_ARGUMENT;
    size_t need = 0;
    for (int k : c) need = std::max(need, static_cast<size_t>(k));
    uint64_t i = 0;
    while (f.line(l)) {
        if (l.empty()) continue;
        split(l, fields);
        uint64_t gid, key;
        float l0, l1;
        if (fields.size() <= need || !to_u64(fields[c[0]], gid) || !to_key(fields[c[1]], key) ||
            !to_float(fields[c[2]], l0) || !to_float(fields[c[3]], l1))
            return SEEDGB_INVALID_ARGUMENT;
        if (i < capacity) {
            // make_measurement_edm.cpp:36-52: bit 1 -> loc0, bit 2 -> loc1
            const bool a0 = (key & 2u) != 0, a1 = (key & 4u) != 0;
            local_position[2 * i] = a0 ? l0 : 0.f;
            local_position[2 * i + 1] = a1 ? l1 : 0.f;
            surface_link[i] = gid;
            dimensions[i] = static_cast<uint8_t>(a0 + a1);
        }
        ++i;
    }
    *n = i;
    return i > capacity ? SEEDGB_CAPACITY_OVERFLOW : SEEDGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The GBTS configuration directory, whitespace-separated like the reference's
// stream reads (examples/options/src/track_gbts_seeding.cpp:158-226):
//   geoidBinning.txt  n, then n x (barcode, layer)
//   binTables.txt     n, then n x (bin1, bin2)
//   layerInfo.txt     n, then n x (type, first eta bin, eta bins, min eta, eta bin width)
// ---------------------------------------------------------------------------
namespace {

class Tokens {
public:
    explicit Tokens(const std::string& path) {
        FILE* f = std::fopen(path.c_str(), "rb");
        if (!f) return;
        ok_ = true;
        std::string cur;
        int c;
        while ((c = std::fgetc(f)) != EOF) {
            if (c == ' ' || c == '\t' || c == '\n' || c == '\r') {
                if (!cur.empty()) toks_.push_back(cur);
                cur.clear();
            } else {
                cur.push_back(static_cast<char>(c));
            }
        }
        if (!cur.empty()) toks_.push_back(cur);
        std::fclose(f);
    }
    bool ok() const { return ok_; }
    bool u64(uint64_t& v) {
        if (i_ >= toks_.size()) return false;
        const char* s = toks_[i_].c_str();
        if (*s == '-') return false;
        char* end = nullptr;
        errno = 0;
        v = std::strtoull(s, &end, 10);
        return errno == 0 && end && *end == '\0' && (++i_, true);
    }
    bool i64(int64_t& v) {
        if (i_ >= toks_.size()) return false;
        char* end = nullptr;
        errno = 0;
        v = std::strtoll(toks_[i_].c_str(), &end, 10);
        return errno == 0 && end && *end == '\0' && (++i_, true);
    }
    bool f32(float& v) {
        if (i_ >= toks_.size()) return false;
        char* end = nullptr;
        errno = 0;
        v = std::strtof(toks_[i_].c_str(), &end);
        return errno == 0 && end && *end == '\0' && (++i_, true);
    }

private:
    std::vector<std::string> toks_;
    size_t i_ = 0;
    bool ok_ = false;
};

}  // namespace

extern "C" seedgb_status seedgb_gbts_read_config_dir(const char* dir, seedgb_gbts_layer* layers,
                                                     uint32_t* n_layers, uint32_t* bin_pairs,
                                                     uint32_t* n_pairs, seedgb_gbts_geoid* geoids,
                                                     uint32_t* n_geoids) {
    if (!dir || !n_layers || !n_pairs || !n_geoids) return SEEDGB_INVALID_ARGUMENT;
    const std::string d(dir);
    Tokens g(d + "/geoidBinning.txt"), b(d + "/binTables.txt"), l(d + "/layerInfo.txt");
    if (!g.ok() || !b.ok() || !l.ok()) return SEEDGB_INVALID_ARGUMENT;
    uint64_t ng, nb, nl;
    if (!g.u64(ng) || !b.u64(nb) || !l.u64(nl) || ng > 0xFFFFFFFFull || nb > 0xFFFFFFFFull ||
        nl > 0xFFFFFFFFull)
        return SEEDGB_INVALID_ARGUMENT;
    const bool fill = layers && bin_pairs && geoids;
    if (fill && (*n_layers < nl || *n_pairs < nb || *n_geoids < ng)) return SEEDGB_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < ng; ++i) {
        uint64_t id;
        int64_t layer;
        if (!g.u64(id) || !g.i64(layer) || layer < INT16_MIN || layer > INT16_MAX)
            return SEEDGB_INVALID_ARGUMENT;
        if (fill) geoids[i] = seedgb_gbts_geoid{id, static_cast<int32_t>(layer)};
    }
    for (uint64_t i = 0; i < nb; ++i) {
        uint64_t b1, b2;
        if (!b.u64(b1) || !b.u64(b2) || b1 > 0xFFFFFFFFull || b2 > 0xFFFFFFFFull)
            return SEEDGB_INVALID_ARGUMENT;
        if (fill) {
            bin_pairs[2 * i] = static_cast<uint32_t>(b1);
            bin_pairs[2 * i + 1] = static_cast<uint32_t>(b2);
        }
    }
    for (uint64_t i = 0; i < nl; ++i) {
        uint64_t type, b0, n;
        float mn, wd;
        if (!l.u64(type) || !l.u64(b0) || !l.u64(n) || !l.f32(mn) || !l.f32(wd) || type > 255 ||
            b0 > 0xFFFFFFFFull || n > 0xFFFFFFFFull)
            return SEEDGB_INVALID_ARGUMENT;
        if (fill)
            layers[i] = seedgb_gbts_layer{static_cast<int32_t>(static_cast<int8_t>(type)),
                                          static_cast<uint32_t>(b0), static_cast<uint32_t>(n), mn, wd};
    }
    *n_geoids = static_cast<uint32_t>(ng);
    *n_pairs = static_cast<uint32_t>(nb);
    *n_layers = static_cast<uint32_t>(nl);
    return SEEDGB_OK;
}
