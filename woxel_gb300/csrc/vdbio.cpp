// vdbio.cpp — topology reader for OpenVDB files holding VDB345 grids.
//
// Follows woxel's VdbReader (src/vdb/read.rs): archive header (:62-121),
// grid descriptors (:166-211), per-grid metadata and transform (:123-164,
// :213-268), and the tree topology (:270-349) with its compressed node
// headers (:351-488). Only the topology is needed by the raycast pass: leaf
// values never enter the march (a voxel hits by its value-mask bit), and the
// reference sets LeafData::Value exactly where the topology's leaf mask is set
// (read.rs:610-620). wx_vdb_read_topology therefore does not parse the
// tree-data section; wx_vdb_read_leaf_values does (read_tree_data, :571-629),
// for the zero-crossing mode's level-set values. Zip (zlib) compressed buffers
// are decoded (inflate.cpp), as the reference does with flate2; blosc-compressed
// grids are rejected (WX_ERR_UNSUPPORTED: no blosc codec in this build).

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "inflate.h"
#include "wx_common.h"

namespace {

constexpr uint32_t kMinVersion = 218;            // OPENVDB_FILE_VERSION_BOOST_UUID
constexpr uint32_t kSelectiveCompression = 220;  // read.rs:27
constexpr uint32_t kNodeMaskCompression = 222;   // read.rs:28
constexpr uint32_t kPerGridCompression = 223;    // read.rs:26
constexpr uint32_t kZip = 0x1, kActiveMask = 0x2, kBlosc = 0x4;

struct Reader {
    FILE *f = nullptr;
    std::string err;
    bool ok = true;
    bool bytes(void *dst, size_t n) {
        if (!ok) return false;
        if (n && fread(dst, 1, n, f) != n) {
            ok = false;
            err = "unexpected end of file";
        }
        return ok;
    }
    template <class T>
    T get() {
        T v{};
        bytes(&v, sizeof v);
        return v;
    }
    std::string str(size_t n) {
        std::string s(n, '\0');
        bytes(&s[0], n);
        return s;
    }
    std::string lstr() { return str(get<uint32_t>()); }
    bool skip(long n) {
        if (ok && fseek(f, n, SEEK_CUR) != 0) {
            ok = false;
            err = "seek failed";
        }
        return ok;
    }
    bool seek(uint64_t pos) {
        if (ok && fseek(f, (long)pos, SEEK_SET) != 0) {
            ok = false;
            err = "seek failed";
        }
        return ok;
    }
    bool fail(const std::string &m) {
        if (ok) err = m;
        ok = false;
        return false;
    }
};

struct Meta {
    int64_t voxel_count = -1;
    bool half = false;
};

// read_metadata (read.rs:213-268): the reference reads the typed value by type
// (not by the stored length) for string/bool/int32/int64/float/vec3i.
Meta read_metadata(Reader &r) {
    Meta m;
    const uint32_t n = r.get<uint32_t>();
    for (uint32_t i = 0; i < n && r.ok; i++) {
        const std::string name = r.lstr(), type = r.lstr();
        const uint32_t len = r.get<uint32_t>();
        if (type == "string") r.skip(len);
        else if (type == "bool") {
            const uint8_t v = r.get<uint8_t>();
            if (name == "is_saved_as_half_float") m.half = v == 1;
        } else if (type == "int32") r.get<int32_t>();
        else if (type == "int64") {
            const int64_t v = r.get<int64_t>();
            if (name == "file_voxel_count") m.voxel_count = v;
        } else if (type == "float") r.get<float>();
        else if (type == "vec3i") r.skip(12);
        else r.skip(len);
    }
    return m;
}

// IEEE binary16 -> binary32 (exact: every half is a float).
float half_to_float(uint16_t h) {
    const uint32_t s = (uint32_t)(h >> 15) << 31, e = (h >> 10) & 31u, m = h & 1023u;
    if (e == 0) {
        const float v = (float)m * 0x1p-24f;  // zero or subnormal
        return s ? -v : v;
    }
    uint32_t bits = e == 31 ? (s | 0x7F800000u | (m << 13)) : (s | ((e + 112u) << 23) | (m << 13));
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

struct Grid {
    std::string name, type;
    uint64_t grid_pos = 0, block_pos = 0, end_pos = 0;
    uint32_t compression = 0;
    Meta meta;
};

// read_compressed_data (read.rs:490-569): count values of elem bytes. Zip: an
// int64 byte count n, then n bytes of a zlib stream that holds the count values,
// or (n <= 0) -n / elem values stored as they are; otherwise the raw values. Blosc
// is checked first, as in the reference. dst == nullptr skips the values.
bool read_values(Reader &r, const Grid &g, size_t count, size_t elem, void *dst) {
    if (g.compression & kBlosc) return r.fail("blosc-compressed grids are not supported");
    if (!(g.compression & kZip)) return dst ? r.bytes(dst, count * elem) : r.skip((long)(count * elem));
    const int64_t n = r.get<int64_t>();
    if (!r.ok) return false;
    if (n <= 0) {
        const uint64_t k = (uint64_t)(-n) / elem;  // the reference reads this many values
        if (k != count) return r.fail("zip block: stored value count differs from the node's");
        return dst ? r.bytes(dst, count * elem) : r.skip((long)(count * elem));
    }
    if (!dst) return r.skip((long)n);
    if (n > (int64_t)(64u << 20)) return r.fail("zip block larger than any node's values");
    std::vector<uint8_t> z((size_t)n);
    if (!r.bytes(z.data(), z.size())) return false;
    std::string err;
    const long long got = wx::zlib_inflate(z.data(), z.size(), static_cast<uint8_t *>(dst), count * elem, &err);
    if (got < 0) return r.fail(err);
    if ((size_t)got != count * elem) return r.fail("zip block holds fewer values than the node");
    return true;
}

// read_compressed (read.rs:378-488) for a node header whose values are not
// kept: consumes exactly the bytes the reference reads.
bool skip_compressed(Reader &r, uint32_t version, const Grid &g, size_t size, const std::vector<uint64_t> &vmask) {
    uint8_t meta = 6;  // NoMaskAndAllVals
    if (version >= kNodeMaskCompression) meta = r.get<uint8_t>();
    if (meta > 6) return r.fail("invalid node metadata");
    if (meta == 2 || meta == 4) r.skip(4);  // one inactive value (ValueType = u32 in the reference)
    else if (meta == 5) r.skip(8);          // two inactive values
    if (meta == 3 || meta == 4 || meta == 5) r.skip((long)(size / 64) * 8);  // selection mask
    size_t count = size;
    if ((g.compression & kActiveMask) && meta != 6 && version >= kNodeMaskCompression) {
        count = 0;
        for (uint64_t w : vmask) count += (size_t)__builtin_popcountll(w);
    }
    return read_values(r, g, count, g.meta.half ? 2 : 4, nullptr);
}

// Leaf buffers of the tree-data section (read_tree_data, read.rs:571-629, with
// read_compressed, :378-488): per leaf, its value mask, then the values: a
// metadata byte, up to two inactive values, an optional selection mask, and
// either all 512 values or (active-mask compression) only the active ones, in
// float or half. Inactive voxels get the inactive values; where the file gives
// none they are +background, or -background for metadata 1 (NO_MASK_AND_MINUS_BG),
// as the OpenVDB format defines them (the reference reader leaves them zero).
bool read_leaf_values(Reader &r, uint32_t version, const Grid &g, float background, float *out) {
    uint64_t vmask[8];
    r.bytes(vmask, 64);
    if (version < kNodeMaskCompression) {
        r.skip(12);  // origin
        if (r.get<uint8_t>() != 1) return r.fail("leaf with more than one buffer");
    }
    uint8_t meta = 6;
    if (version >= kNodeMaskCompression) meta = r.get<uint8_t>();
    if (meta > 6) return r.fail("invalid node metadata");
    float in0 = meta == 0 ? background : -background, in1 = background;
    if (meta == 2 || meta == 4 || meta == 5) in0 = r.get<float>();
    if (meta == 5) in1 = r.get<float>();
    uint64_t sel[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (meta == 3 || meta == 4 || meta == 5) r.bytes(sel, 64);
    size_t count = 512;
    if ((g.compression & kActiveMask) && meta != 6 && version >= kNodeMaskCompression) {
        count = 0;
        for (uint64_t w : vmask) count += (size_t)__builtin_popcountll(w);
    }
    float data[512];
    if (g.meta.half) {
        uint16_t h[512];
        read_values(r, g, count, 2, h);
        for (size_t i = 0; i < count && r.ok; i++) data[i] = half_to_float(h[i]);
    } else {
        read_values(r, g, count, 4, data);
    }
    if (!r.ok) return false;
    if (count == 512) {
        memcpy(out, data, sizeof data);
    } else {
        size_t k = 0;
        for (uint32_t i = 0; i < 512; i++) {
            const bool act = (vmask[i >> 6] >> (i & 63)) & 1u, s1 = (sel[i >> 6] >> (i & 63)) & 1u;
            out[i] = act ? data[k++] : (s1 ? in1 : in0);
        }
    }
    return true;
}

// Parses one grid: the topology, and with values != nullptr also the leaf values
// (n3 * 512 floats in DFS leaf order, the layout of wx_grid_set_values).
int parse(const char *path, const char *grid_name, wx_topology **out, wx_vdb_info *info,
          std::vector<float> *values, float *bg_out, const char *who) {
    Reader r;
    r.f = fopen(path, "rb");
    if (!r.f) {
        wx::set_thread_error(std::string(who) + ": cannot open " + path);
        return WX_ERR_INVALID;
    }
    struct Closer {
        FILE *f;
        ~Closer() { fclose(f); }
    } closer{r.f};
    auto bad = [&](int code, const std::string &m) {
        wx::set_thread_error(std::string(who) + ": " + m);
        return code;
    };
    // Archive header (read.rs:62-121).
    if (r.get<uint64_t>() != 0x56444220ull) return bad(WX_ERR_INVALID, "magic bytes mismatched");
    const uint32_t version = r.get<uint32_t>();
    if (version < kMinVersion) return bad(WX_ERR_UNSUPPORTED, "unsupported file version");
    r.get<uint32_t>();  // library major
    r.get<uint32_t>();  // library minor
    const bool has_offsets = r.get<uint8_t>() != 0;
    uint32_t compression = version < kPerGridCompression ? (kZip | kActiveMask) : (kBlosc | kActiveMask);
    if (version >= kSelectiveCompression && version < kNodeMaskCompression)
        compression = r.get<uint8_t>() == 1 ? kZip : 0;
    r.skip(36);  // uuid
    read_metadata(r);
    const uint32_t ngrids = r.get<uint32_t>();
    if (!r.ok) return bad(WX_ERR_INVALID, r.err);
    if (!has_offsets) return bad(WX_ERR_UNSUPPORTED, "file without grid offsets");
    // Grid descriptors (read.rs:166-211).
    std::vector<Grid> grids;
    for (uint32_t i = 0; i < ngrids && r.ok; i++) {
        Grid g;
        g.name = r.lstr();
        g.type = r.lstr();
        r.lstr();  // instance parent
        g.grid_pos = r.get<uint64_t>();
        g.block_pos = r.get<uint64_t>();
        g.end_pos = r.get<uint64_t>();
        g.compression = compression;
        if (version >= kNodeMaskCompression) g.compression = r.get<uint32_t>();
        g.meta = read_metadata(r);
        grids.push_back(g);
        r.seek(g.end_pos);
    }
    if (!r.ok) return bad(WX_ERR_INVALID, r.err);
    const Grid *gp = nullptr;
    for (const Grid &g : grids)
        if (!grid_name || g.name == grid_name) {
            gp = &g;
            break;
        }
    if (!gp) return bad(WX_ERR_INVALID, grid_name ? std::string("no grid named ") + grid_name : "file has no grid");
    const Grid &g = *gp;
    // Grid header (read.rs:123-164).
    r.seek(g.grid_pos);
    if (version >= kNodeMaskCompression) r.get<uint32_t>();
    read_metadata(r);
    const std::string map = r.lstr();
    if (map == "UniformScaleMap") r.skip(5 * 24);
    else if (map == "UniformScaleTranslateMap" || map == "ScaleTranslateMap") r.skip(6 * 24);
    else return bad(WX_ERR_UNSUPPORTED, "unsupported transform " + map);
    // Tree topology (read.rs:270-349).
    if (r.get<uint32_t>() != 1) return bad(WX_ERR_UNSUPPORTED, "multi-buffer trees");
    const float background = r.get<float>();
    if (bg_out) *bg_out = background;
    const uint32_t ntiles = r.get<uint32_t>(), nnode5 = r.get<uint32_t>();
    r.skip((long)ntiles * (12 + 4 + 1));  // root tiles are invisible to masks()/origins()
    struct N4 {
        std::vector<uint64_t> kid, val;
        std::vector<std::vector<uint64_t>> leaves;
    };
    struct N5 {
        wx::I3 o;
        std::vector<uint64_t> kid, val;
        std::vector<N4> kids;
    };
    std::map<wx::I3, N5> n5s;  // sorted root keys, as masks()/origins() iterate them
    std::vector<wx::I3> file_order;  // the order the tree-data section lists the leaves in
    for (uint32_t i = 0; i < nnode5 && r.ok; i++) {
        N5 n;
        for (int a = 0; a < 3; a++) n.o[a] = wx::node_origin(r.get<int32_t>(), wx::kN5Total);
        n.kid.resize(wx::kN5Words);
        n.val.resize(wx::kN5Words);
        r.bytes(n.kid.data(), wx::kN5Words * 8);
        r.bytes(n.val.data(), wx::kN5Words * 8);
        size_t size = wx::kN5Slots;
        if (version < kNodeMaskCompression) {
            size = 0;
            for (uint64_t w : n.kid) size += 64 - (size_t)__builtin_popcountll(w);
        }
        if (!skip_compressed(r, version, g, size, n.val)) break;
        for (uint32_t s5 = 0; s5 < wx::kN5Slots && r.ok; s5++) {
            if (!wx::test_bit(n.kid.data(), s5)) continue;
            N4 c;
            c.kid.resize(wx::kN4Words);
            c.val.resize(wx::kN4Words);
            r.bytes(c.kid.data(), wx::kN4Words * 8);
            r.bytes(c.val.data(), wx::kN4Words * 8);
            size_t size4 = wx::kN4Slots;
            if (version < kNodeMaskCompression) {
                size4 = 0;
                for (uint64_t w : c.kid) size4 += 64 - (size_t)__builtin_popcountll(w);
            }
            if (!skip_compressed(r, version, g, size4, c.val)) break;
            for (uint32_t s4 = 0; s4 < wx::kN4Slots && r.ok; s4++) {
                if (!wx::test_bit(c.kid.data(), s4)) continue;
                std::vector<uint64_t> m(wx::kN3Words);
                r.bytes(m.data(), wx::kN3Words * 8);
                c.leaves.push_back(std::move(m));
            }
            n.kids.push_back(std::move(c));
        }
        if (n5s.count(n.o)) return bad(WX_ERR_INVALID, "duplicate root key");
        file_order.push_back(n.o);
        n5s.emplace(n.o, std::move(n));
    }
    if (!r.ok) return bad(r.err.find("supported") != std::string::npos ? WX_ERR_UNSUPPORTED : WX_ERR_INVALID, r.err);
    // masks()/origins() in DFS order (vdb345.rs:108-161).
    std::vector<uint32_t> k5, v5, k4, v4, v3;
    std::vector<int32_t> org;
    std::map<wx::I3, size_t> first_leaf;  // DFS index of each N5's first leaf
    size_t nleaves = 0;
    auto put = [](std::vector<uint32_t> &dst, const std::vector<uint64_t> &src) {
        for (uint64_t w : src) {
            dst.push_back((uint32_t)w);
            dst.push_back((uint32_t)(w >> 32));
        }
    };
    for (auto &kv : n5s) {
        first_leaf[kv.first] = nleaves;
        put(k5, kv.second.kid);
        put(v5, kv.second.val);
        org.insert(org.end(), {kv.first[0], kv.first[1], kv.first[2], 0});
        for (auto &c : kv.second.kids) {
            put(k4, c.kid);
            put(v4, c.val);
            for (auto &m : c.leaves) put(v3, m);
            nleaves += c.leaves.size();
        }
    }
    if (values) {  // tree data (read.rs:571-629): leaf buffers in the topology's file order
        try {
            values->assign(nleaves * 512, 0.0f);
        } catch (...) {
            return bad(WX_ERR_OOM, "host allocation failed");
        }
        r.seek(g.block_pos);
        for (const wx::I3 &o : file_order) {
            size_t leaf = first_leaf[o];
            for (auto &c : n5s[o].kids)
                for (size_t j = 0; j < c.leaves.size() && r.ok; j++, leaf++)
                    if (!read_leaf_values(r, version, g, background, values->data() + leaf * 512)) break;
        }
        if (!r.ok)
            return bad(r.err.find("supported") != std::string::npos ? WX_ERR_UNSUPPORTED : WX_ERR_INVALID, r.err);
    }
    if (out) {
        const int rc = wx_topology_from_masks(k5.data(), v5.data(), n5s.size(), k4.data(), v4.data(), k4.size() / 128,
                                              v3.data(), v3.size() / 16, org.data(), 4, out);
        if (rc != WX_OK) return rc;
    }
    if (info) {
        memset(info, 0, sizeof *info);
        info->file_version = version;
        info->compression = g.compression;
        info->half_float = g.meta.half ? 1u : 0u;
        info->file_voxel_count = g.meta.voxel_count;
        snprintf(info->grid_name, sizeof info->grid_name, "%s", g.name.c_str());
    }
    return WX_OK;
}

// parse() behind the C ABI: no exception crosses it (a host allocation that fails
// while reading is WX_ERR_OOM).
int parse_guarded(const char *path, const char *grid_name, wx_topology **out, wx_vdb_info *info,
                  std::vector<float> *values, float *bg_out, const char *who) {
    return wx::guard(who, [&]() -> int { return parse(path, grid_name, out, info, values, bg_out, who); });
}

}  // namespace

extern "C" int wx_vdb_read_topology(const char *path, const char *grid_name, wx_topology **out, wx_vdb_info *info) {
    if (!path || !out) {
        wx::set_thread_error("wx_vdb_read_topology: null argument");
        return WX_ERR_INVALID;
    }
    return parse_guarded(path, grid_name, out, info, nullptr, nullptr, "wx_vdb_read_topology");
}

extern "C" int wx_vdb_read_leaf_values(const char *path, const char *grid_name, float *values, uint64_t capacity,
                                       uint64_t *count, float *background) {
    if (!path || !count) {
        wx::set_thread_error("wx_vdb_read_leaf_values: null argument");
        return WX_ERR_INVALID;
    }
    std::vector<float> v;
    const int rc = parse_guarded(path, grid_name, nullptr, nullptr, &v, background, "wx_vdb_read_leaf_values");
    if (rc != WX_OK) return rc;
    *count = v.size();
    if (values) {
        if (capacity < v.size()) {
            wx::set_thread_error("wx_vdb_read_leaf_values: buffer too small");
            return WX_ERR_INVALID;
        }
        memcpy(values, v.data(), v.size() * sizeof(float));
    }
    return WX_OK;
}
