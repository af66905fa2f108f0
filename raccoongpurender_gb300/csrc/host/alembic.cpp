// alembic.cpp — the scene front-end: Alembic (Ogawa) files as the reference
// loads them.
//
// The reference reads Houdini-exported Alembic archives with its
// houdini_alembic library on top of the Alembic SDK
// (libs/houdini_alembic/houdini_alembic.cpp) and turns the visible objects
// into a scene in WavefrontPathTracing's constructor
// (common/wavefront_path_tracing.hpp:1170-1216) through
// SceneManager::addPolymesh / addPoint (common/scene_manager.hpp:197-497).
// This file does the same without the SDK:
//
//   * the Ogawa container (a tree of groups of 64-bit child offsets and of
//     size-prefixed data blocks, file header "Ogawa", frozen flag, version,
//     root offset) and the Alembic core layout on top of it (archive root:
//     version, library version, top object, archive metadata, time
//     samplings, indexed metadata; an object: its property compound, its
//     child objects, a block of child headers; a compound: one group per
//     property, a block of packed property headers; scalar samples as one
//     data block each, array samples as a data block and a dimensions
//     block, each data block led by a 16-byte digest);
//   * the geometry schemas the Houdini reader uses (Xform ops and values,
//     PolyMesh, Points, Curves, Camera core values and user properties),
//     the attribute columns it builds from geometry parameters (geoScope
//     var/vtx -> points, fvr -> vertices, uni -> primitives; indexed strings
//     and vector2s; float tuples of any extent x arrayExtent up to 4; int32
//     and string arrays), its transform accumulation, visibility and camera
//     parameters;
//   * the scene building: triangle meshes only, vertices through the
//     combined transform in double, per-triangle materials from the
//     "material" string column and its property columns, spheres from point
//     objects with pscale (Lambertian from Cd), the "ImageEnvmap" point
//     (a Radiance .hdr image, clamped and scaled), the first visible camera.
//
// Deliberate differences: a malformed file, a missing column that the
// reference dereferences (P, the geometry parameters of a mesh) or an unknown
// material name return RGR_E_INVALID instead of crashing; only .hdr envmap
// images are decoded (the reference decodes any stb_image format).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../rgr_internal.h"
#include "nvtx.h"

namespace rgr {
namespace abc {

struct Error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// ------------------------------------------------------------------ Ogawa
constexpr uint64_t kDataBit = 0x8000000000000000ull;

class OgawaFile {
public:
    explicit OgawaFile(const std::string& path) {
        std::ifstream f(path, std::ios::binary | std::ios::ate);
        if (!f) throw Error("cannot open " + path);
        const std::streamsize n = f.tellg();
        if (n < 16) throw Error("not an Ogawa file: " + path);
        buf_.resize((size_t)n);
        f.seekg(0);
        if (!f.read(reinterpret_cast<char*>(buf_.data()), n)) throw Error("cannot read " + path);
        if (std::memcmp(buf_.data(), "Ogawa", 5) != 0) throw Error("not an Ogawa file: " + path);
        const uint16_t version = (uint16_t)((buf_[6] << 8) | buf_[7]);
        if (version != 1) throw Error("unsupported Ogawa version");
        root_ = u64(8);
    }
    uint64_t root() const { return root_; }
    uint64_t size() const { return buf_.size(); }
    uint64_t u64(uint64_t pos) const {
        need(pos, 8);
        uint64_t v;
        std::memcpy(&v, buf_.data() + pos, 8);  // the format is little-endian, as are both hosts
        return v;
    }
    // child entries of the group at pos (0: the empty group)
    std::vector<uint64_t> group(uint64_t pos) const {
        std::vector<uint64_t> out;
        if (pos == 0) return out;
        if (pos & kDataBit) throw Error("expected a group, found data");
        const uint64_t n = u64(pos);
        if (n > (size() - pos) / 8) throw Error("corrupt group");
        out.resize(n);
        for (uint64_t i = 0; i < n; ++i) out[i] = u64(pos + 8 + 8 * i);
        return out;
    }
    // a data block from its child entry (top bit set); empty when the position is 0
    std::pair<const unsigned char*, uint64_t> data(uint64_t entry) const {
        if (!(entry & kDataBit)) throw Error("expected data, found a group");
        const uint64_t pos = entry & ~kDataBit;
        if (pos == 0) return {nullptr, 0};
        const uint64_t n = u64(pos);
        need(pos + 8, n);
        return {buf_.data() + pos + 8, n};
    }

private:
    void need(uint64_t pos, uint64_t n) const {
        if (pos > size() || n > size() - pos) throw Error("corrupt file: read past the end");
    }
    std::vector<unsigned char> buf_;
    uint64_t root_ = 0;
};

// ------------------------------------------------------------------ metadata
using Meta = std::map<std::string, std::string>;

// "key=value;key=value" (AbcCoreAbstract MetaData::deserialize)
Meta parse_meta(const std::string& s) {
    Meta m;
    size_t start = 0;
    while (start <= s.size()) {
        size_t end = s.find(';', start);
        if (end == std::string::npos) end = s.size();
        const std::string tok = s.substr(start, end - start);
        const size_t eq = tok.find('=');
        if (eq != std::string::npos) m[tok.substr(0, eq)] = tok.substr(eq + 1);
        start = end + 1;
    }
    return m;
}
std::string get(const Meta& m, const char* k) {
    auto it = m.find(k);
    return it == m.end() ? std::string() : it->second;
}

// ------------------------------------------------------------------ data types
enum Pod : int {
    kBool = 0, kU8, kI8, kU16, kI16, kU32, kI32, kU64, kI64, kF16, kF32, kF64, kString, kWstring
};
size_t pod_bytes(int pod) {
    static const size_t b[] = {1, 1, 1, 2, 2, 4, 4, 8, 8, 2, 4, 8, 0, 0};
    return (pod >= 0 && pod < 14) ? b[pod] : 0;
}

enum PropType { kCompound = 0, kScalar = 1, kArray = 2 };

struct PropHeader {
    std::string name;
    int type = kCompound;
    int pod = kF32;
    int extent = 1;
    uint32_t next_sample = 0, first_changed = 0, last_changed = 0;
    Meta meta;
    uint64_t entry = 0;  // the property's child entry in its compound's group

    // the stored sample holding requested sample `index` (sample selector
    // clamping, then the first/last-changed mapping of constant runs)
    uint64_t stored(int64_t index) const {
        if (next_sample == 0) throw Error("property " + name + " has no samples");
        if (index < 0) index = 0;
        if (index >= (int64_t)next_sample) index = (int64_t)next_sample - 1;
        const uint32_t i = (uint32_t)index;
        if (i < first_changed) return 0;
        if (first_changed == last_changed && first_changed == 0) return 0;
        if (i >= last_changed) return (uint64_t)(last_changed - first_changed + 1);
        return (uint64_t)(i - first_changed + 1);
    }
};

// an array (or scalar) sample: raw little-endian bytes, or strings
struct Sample {
    int pod = kF32;
    int extent = 1;
    uint64_t count = 0;  // elements (each `extent` values)
    std::vector<unsigned char> bytes;
    std::vector<std::string> strings;
    template <class T>
    const T* as() const {
        return reinterpret_cast<const T*>(bytes.data());
    }
};

class Archive;

class Compound {
public:
    Compound() = default;
    Compound(const Archive* a, uint64_t group_entry);
    bool valid() const { return a_ != nullptr; }
    const std::vector<PropHeader>& props() const { return props_; }
    const PropHeader* find(const std::string& n) const {
        for (const auto& p : props_)
            if (p.name == n) return &p;
        return nullptr;
    }
    Compound compound(const std::string& n) const;
    Sample scalar(const PropHeader& h, int64_t index) const;
    Sample array(const PropHeader& h, int64_t index) const;

private:
    const Archive* a_ = nullptr;
    std::vector<PropHeader> props_;
};

struct ObjectHeader {
    std::string name, full_name;
    Meta meta;
    uint64_t entry = 0;
};

class Object {
public:
    Object(const Archive* a, uint64_t group_entry, std::string full_name, Meta meta, const Object* parent)
        : a_(a), entry_(group_entry), full_name_(std::move(full_name)), meta_(std::move(meta)), parent_(parent) {}
    const std::string& full_name() const { return full_name_; }
    const Meta& meta() const { return meta_; }
    const Object* parent() const { return parent_; }
    const Archive* archive() const { return a_; }
    Compound properties() const;
    std::vector<ObjectHeader> children() const;

private:
    const Archive* a_;
    uint64_t entry_;
    std::string full_name_;
    Meta meta_;
    const Object* parent_;
};

class Archive {
public:
    explicit Archive(const std::string& path) : f_(path) {
        const auto root = f_.group(f_.root());
        if (root.size() < 6) throw Error("not an Alembic archive");
        // [0] file version, [1] library version, [2] top object, [3] archive
        // metadata, [4] time samplings, [5] indexed metadata
        int32_t version = -1;
        auto v = f_.data(root[0]);
        if (v.second >= 4) std::memcpy(&version, v.first, 4);
        if (version != 0) throw Error("unsupported Alembic file version");
        meta_index_.push_back(Meta());
        auto im = f_.data(root[5]);
        for (uint64_t pos = 0; pos < im.second;) {
            const uint64_t n = im.first[pos++];
            if (pos + n > im.second) throw Error("corrupt indexed metadata");
            meta_index_.push_back(parse_meta(std::string(reinterpret_cast<const char*>(im.first + pos), n)));
            pos += n;
        }
        top_entry_ = root[2];
    }
    const OgawaFile& file() const { return f_; }
    const Meta& indexed_meta(uint32_t i) const {
        if (i >= meta_index_.size()) throw Error("metadata index out of range");
        return meta_index_[i];
    }
    Object top() const { return Object(this, top_entry_, "", Meta(), nullptr); }

private:
    OgawaFile f_;
    std::vector<Meta> meta_index_;
    uint64_t top_entry_ = 0;
};

// packed property headers (AbcCoreOgawa property header encoding): per
// property a 32-bit info word — bits 0-1 property type, 2-3 the byte width
// of the numbers that follow (1, 2 or 4), 4-7 POD, 8 has a time sampling
// index, 9 has first/last changed indices, 10 homogeneous, 11 all samples
// equal, 12-19 extent, 20-27 metadata index (0xff: inline) — then the sample
// count and optional indices, the name and optional inline metadata.
Compound::Compound(const Archive* a, uint64_t group_entry) : a_(a) {
    const OgawaFile& f = a->file();
    const auto kids = f.group(group_entry);
    if (kids.empty() || !(kids.back() & kDataBit)) return;
    auto d = f.data(kids.back());
    const unsigned char* b = d.first;
    const uint64_t n = d.second;
    uint64_t pos = 0;
    auto need = [&](uint64_t k) {
        if (pos + k > n) throw Error("corrupt property headers");
    };
    auto hinted = [&](uint32_t hint) -> uint32_t {
        if (hint == 0) {
            need(1);
            return b[pos++];
        }
        if (hint == 1) {
            need(2);
            uint16_t v;
            std::memcpy(&v, b + pos, 2);
            pos += 2;
            return v;
        }
        need(4);
        uint32_t v;
        std::memcpy(&v, b + pos, 4);
        pos += 4;
        return v;
    };
    size_t idx = 0;
    while (pos < n) {
        need(4);
        uint32_t info;
        std::memcpy(&info, b + pos, 4);
        pos += 4;
        PropHeader h;
        const uint32_t ptype = info & 3u;
        h.type = ptype == 0 ? kCompound : (ptype == 1 ? kScalar : kArray);
        const uint32_t hint = (info >> 2) & 3u;
        if (h.type != kCompound) {
            h.pod = (int)((info >> 4) & 0xfu);
            if (h.pod > kWstring) throw Error("invalid POD type");
            h.extent = (int)((info >> 12) & 0xffu);
            h.next_sample = hinted(hint);
            if (info & 0x200u) {
                h.first_changed = hinted(hint);
                h.last_changed = hinted(hint);
            } else if (info & 0x800u) {
                h.first_changed = h.last_changed = 0;
            } else {
                h.first_changed = 1;
                h.last_changed = h.next_sample - 1;
            }
            if (info & 0x100u) hinted(hint);  // time sampling index: frames are selected by index
        }
        const uint32_t name_len = hinted(hint);
        need(name_len);
        h.name.assign(reinterpret_cast<const char*>(b + pos), name_len);
        pos += name_len;
        const uint32_t mi = (info >> 20) & 0xffu;
        if (mi == 0xffu) {
            const uint32_t ml = hinted(hint);
            need(ml);
            h.meta = parse_meta(std::string(reinterpret_cast<const char*>(b + pos), ml));
            pos += ml;
        } else {
            h.meta = a->indexed_meta(mi);
        }
        if (idx >= kids.size() - 1) throw Error("property without a group");
        h.entry = kids[idx++];
        props_.push_back(std::move(h));
    }
}

Compound Compound::compound(const std::string& n) const {
    const PropHeader* h = find(n);
    if (!h || h->type != kCompound) return Compound();
    return Compound(a_, h->entry);
}

static void read_payload(const std::pair<const unsigned char*, uint64_t>& d, Sample& s) {
    if (d.second == 0) return;
    if (d.second < 16) throw Error("corrupt sample data");
    const unsigned char* p = d.first + 16;  // after the digest
    const uint64_t n = d.second - 16;
    if (s.pod == kString) {
        uint64_t start = 0;
        for (uint64_t i = 0; i < n; ++i)
            if (p[i] == 0) {
                s.strings.emplace_back(reinterpret_cast<const char*>(p + start), i - start);
                start = i + 1;
            }
    } else if (s.pod == kWstring) {
        throw Error("wide-string properties are not supported");
    } else {
        s.bytes.assign(p, p + n);
    }
}

Sample Compound::scalar(const PropHeader& h, int64_t index) const {
    if (h.type != kScalar) throw Error(h.name + " is not a scalar property");
    const auto kids = a_->file().group(h.entry);
    const uint64_t k = h.stored(index);
    if (k >= kids.size()) throw Error("missing sample of " + h.name);
    Sample s;
    s.pod = h.pod;
    s.extent = h.extent;
    s.count = 1;
    read_payload(a_->file().data(kids[k]), s);
    if (s.pod != kString && s.bytes.size() < pod_bytes(s.pod) * (size_t)s.extent) throw Error("short sample");
    return s;
}

Sample Compound::array(const PropHeader& h, int64_t index) const {
    if (h.type != kArray) throw Error(h.name + " is not an array property");
    const auto kids = a_->file().group(h.entry);
    const uint64_t k = 2 * h.stored(index);
    if (k + 1 >= kids.size()) throw Error("missing sample of " + h.name);
    Sample s;
    s.pod = h.pod;
    s.extent = std::max(1, h.extent);
    const auto data = a_->file().data(kids[k]);
    const auto dims = a_->file().data(kids[k + 1]);
    read_payload(data, s);
    if (dims.second == 0) {  // rank 1, the length implied by the data size
        if (s.pod == kString)
            s.count = s.strings.size() / (uint64_t)s.extent;
        else
            s.count = data.second == 0 ? 0 : (data.second - 16) / (pod_bytes(s.pod) * (uint64_t)s.extent);
    } else {
        s.count = 1;
        for (uint64_t i = 0; i + 8 <= dims.second; i += 8) {
            uint64_t v;
            std::memcpy(&v, dims.first + i, 8);
            if (v != 0 && s.count > (1ull << 40) / v) throw Error("array dimensions too large in " + h.name);
            s.count *= v;
        }
    }
    if (s.count > (1ull << 40) / (uint64_t)s.extent) throw Error("array too large in " + h.name);
    const uint64_t values = s.count * (uint64_t)s.extent;
    if (s.pod == kString ? s.strings.size() < values : s.bytes.size() < values * pod_bytes(s.pod))
        throw Error("short array sample of " + h.name);
    return s;
}

Compound Object::properties() const {
    const auto kids = a_->file().group(entry_);
    if (kids.empty() || (kids[0] & kDataBit)) return Compound();
    return Compound(a_, kids[0]);
}

// child object headers: the last child block, less its two trailing digests
std::vector<ObjectHeader> Object::children() const {
    std::vector<ObjectHeader> out;
    const OgawaFile& f = a_->file();
    const auto kids = f.group(entry_);
    if (kids.empty() || !(kids.back() & kDataBit)) return out;
    auto d = f.data(kids.back());
    if (d.second <= 32) return out;
    const unsigned char* b = d.first;
    const uint64_t n = d.second - 32;
    uint64_t pos = 0;
    size_t ci = 1;
    while (pos < n) {
        if (pos + 4 > n) throw Error("corrupt object headers");
        uint32_t len;
        std::memcpy(&len, b + pos, 4);
        pos += 4;
        if (pos + len + 1 > n) throw Error("corrupt object headers");
        ObjectHeader h;
        h.name.assign(reinterpret_cast<const char*>(b + pos), len);
        pos += len;
        const uint8_t mi = b[pos++];
        if (mi == 0xff) {
            if (pos + 4 > n) throw Error("corrupt object headers");
            uint32_t ml;
            std::memcpy(&ml, b + pos, 4);
            pos += 4;
            if (pos + ml > n) throw Error("corrupt object headers");
            h.meta = parse_meta(std::string(reinterpret_cast<const char*>(b + pos), ml));
            pos += ml;
        } else {
            h.meta = a_->indexed_meta(mi);
        }
        h.full_name = full_name_ + "/" + h.name;
        if (ci >= kids.size() - 1) throw Error("object without a group");
        h.entry = kids[ci++];
        out.push_back(std::move(h));
    }
    return out;
}

// ------------------------------------------------------------------ 4x4 (Imath conventions)
// Row vectors: p' = p M; x[i][j] row i, column j.
struct M44 {
    double x[4][4];
    static M44 identity() {
        M44 m{};
        for (int i = 0; i < 4; ++i) m.x[i][i] = 1.0;
        return m;
    }
    M44 operator*(const M44& b) const {  // left-to-right sums, as Imath multiplies
        M44 c;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                c.x[i][j] = x[i][0] * b.x[0][j] + x[i][1] * b.x[1][j] + x[i][2] * b.x[2][j] + x[i][3] * b.x[3][j];
        return c;
    }
};

// rotation by `angle` radians about `axis` (Rodrigues' formula in Imath's row-vector layout)
M44 axis_angle(const double axis[3], double angle) {
    double len2 = axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2];
    double u[3] = {0.0, 0.0, 0.0};
    if (len2 > 0.0) {
        const double l = std::sqrt(len2);
        u[0] = axis[0] / l;
        u[1] = axis[1] / l;
        u[2] = axis[2] / l;
    }
    const double s = std::sin(angle), c = std::cos(angle);
    M44 m = M44::identity();
    m.x[0][0] = u[0] * u[0] * (1 - c) + c;
    m.x[0][1] = u[0] * u[1] * (1 - c) + u[2] * s;
    m.x[0][2] = u[0] * u[2] * (1 - c) - u[1] * s;
    m.x[1][0] = u[0] * u[1] * (1 - c) - u[2] * s;
    m.x[1][1] = u[1] * u[1] * (1 - c) + c;
    m.x[1][2] = u[1] * u[2] * (1 - c) + u[0] * s;
    m.x[2][0] = u[0] * u[2] * (1 - c) + u[1] * s;
    m.x[2][1] = u[1] * u[2] * (1 - c) - u[0] * s;
    m.x[2][2] = u[2] * u[2] * (1 - c) + c;
    return m;
}

double degrees_to_radians(double d) { return (d * M_PI) / 180.0; }

// affine inverse by the adjugate of the 3x3 part and the negated, rotated
// translation; a general 4x4 (projective) matrix by Gauss-Jordan elimination
M44 inverse(const M44& a) {
    const auto& x = a.x;
    if (x[0][3] != 0 || x[1][3] != 0 || x[2][3] != 0 || x[3][3] != 1) {
        M44 m = a, r = M44::identity();
        for (int col = 0; col < 4; ++col) {
            int piv = col;
            for (int i = col + 1; i < 4; ++i)
                if (std::fabs(m.x[i][col]) > std::fabs(m.x[piv][col])) piv = i;
            if (m.x[piv][col] == 0.0) throw Error("singular transform");
            std::swap(m.x[piv], m.x[col]);
            std::swap(r.x[piv], r.x[col]);
            const double p = m.x[col][col];
            for (int j = 0; j < 4; ++j) {
                m.x[col][j] /= p;
                r.x[col][j] /= p;
            }
            for (int i = 0; i < 4; ++i) {
                if (i == col) continue;
                const double f = m.x[i][col];
                for (int j = 0; j < 4; ++j) {
                    m.x[i][j] -= f * m.x[col][j];
                    r.x[i][j] -= f * r.x[col][j];
                }
            }
        }
        return r;
    }
    M44 s = M44::identity();
    s.x[0][0] = x[1][1] * x[2][2] - x[2][1] * x[1][2];
    s.x[0][1] = x[2][1] * x[0][2] - x[0][1] * x[2][2];
    s.x[0][2] = x[0][1] * x[1][2] - x[1][1] * x[0][2];
    s.x[1][0] = x[2][0] * x[1][2] - x[1][0] * x[2][2];
    s.x[1][1] = x[0][0] * x[2][2] - x[2][0] * x[0][2];
    s.x[1][2] = x[1][0] * x[0][2] - x[0][0] * x[1][2];
    s.x[2][0] = x[1][0] * x[2][1] - x[2][0] * x[1][1];
    s.x[2][1] = x[2][0] * x[0][1] - x[0][0] * x[2][1];
    s.x[2][2] = x[0][0] * x[1][1] - x[1][0] * x[0][1];
    const double det = x[0][0] * s.x[0][0] + x[0][1] * s.x[1][0] + x[0][2] * s.x[2][0];
    if (det == 0.0) throw Error("singular transform");
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) s.x[i][j] /= det;
    for (int j = 0; j < 3; ++j)
        s.x[3][j] = -x[3][0] * s.x[0][j] - x[3][1] * s.x[1][j] - x[3][2] * s.x[2][j];
    return s;
}

// XformSample::getMatrix: each op's matrix, composed as ret = op * ret
M44 xform_matrix(const Object& o, int64_t frame) {
    Compound props = o.properties();
    Compound xf = props.compound(".xform");
    M44 ret = M44::identity();
    if (!xf.valid()) return ret;
    const PropHeader* ops_h = xf.find(".ops");
    if (!ops_h || ops_h->type != kScalar || ops_h->next_sample == 0) return ret;
    const Sample ops = xf.scalar(*ops_h, 0);
    std::vector<double> vals;
    if (const PropHeader* vh = xf.find(".vals")) {
        if (vh->next_sample > 0) {
            const Sample v = vh->type == kScalar ? xf.scalar(*vh, frame) : xf.array(*vh, frame);
            if (v.pod != kF64) throw Error("transform values are not float64");
            const size_t n = v.bytes.size() / 8;
            vals.assign(v.as<double>(), v.as<double>() + n);
        }
    }
    size_t ch = 0;
    auto val = [&](size_t k) { return ch + k < vals.size() ? vals[ch + k] : 0.0; };
    for (int i = 0; i < ops.extent && i < (int)ops.bytes.size(); ++i) {
        const int type = ops.bytes[i] >> 4;
        M44 m = M44::identity();
        size_t nch = 0;
        if (type == 3) {  // matrix
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) m.x[r][c] = val(4 * r + c);
            nch = 16;
        } else if (type >= 4 && type <= 6) {  // rotate about x, y, z
            const double axis[3] = {type == 4 ? 1.0 : 0.0, type == 5 ? 1.0 : 0.0, type == 6 ? 1.0 : 0.0};
            m = axis_angle(axis, degrees_to_radians(val(0)));
            nch = 1;
        } else if (type == 0) {  // scale
            m.x[0][0] = val(0);
            m.x[1][1] = val(1);
            m.x[2][2] = val(2);
            nch = 3;
        } else if (type == 1) {  // translate
            m.x[3][0] = val(0);
            m.x[3][1] = val(1);
            m.x[3][2] = val(2);
            nch = 3;
        } else if (type == 2) {  // rotate about an axis
            const double axis[3] = {val(0), val(1), val(2)};
            m = axis_angle(axis, degrees_to_radians(val(3)));
            nch = 4;
        } else {
            throw Error("unknown transform operation");
        }
        ch += nch;
        ret = m * ret;
    }
    return ret;
}

// ------------------------------------------------------------------ the Houdini reader's objects
enum ColType { kColInt = 0, kColFloat, kColVec2, kColVec3, kColVec4, kColString };

struct Column {
    std::string key;
    int type = kColFloat;
    uint32_t rows = 0;
    int dim = 1;
    std::vector<float> f;      // rows * dim (float and vector columns)
    std::vector<int32_t> i;    // int columns
    std::vector<std::string> s;  // string columns: the distinct values ...
    std::vector<uint32_t> si;     // ... and each row's index into them
    const std::string& str(uint32_t r) const { return s[si[r]]; }
};
struct Sheet {
    std::vector<Column> cols;  // sorted by key
    uint32_t rows() const { return cols.empty() ? 0u : cols[0].rows; }
    const Column* find(const char* k, int type) const {
        for (const auto& c : cols)
            if (c.key == k) return c.type == type ? &c : nullptr;
        return nullptr;
    }
};

enum ObjType { kPolyMesh = 0, kPoint, kCurve, kCamera };

struct SceneObject {
    int type = kPolyMesh;
    std::string name;
    bool visible = true;
    M44 combined_d;            // the combined transform in double
    float combined[16];        // ... as the Houdini reader stores it
    std::vector<std::array<float, 16>> xforms;
    std::vector<uint32_t> face_counts, indices;
    std::vector<uint64_t> point_ids;
    std::vector<float> P;      // xyz per point
    Sheet points, vertices, primitives;
    // camera
    float eye[3], lookat[3], up[3], down[3], forward[3], back[3], left[3], right[3];
    int resolution_x = 0, resolution_y = 0;
    float focal_mm = 50.0f, aperture_h_mm = 41.4214f, aperture_v_mm = 0.0f, near_clip = 0.001f,
          far_clip = 10000.0f, focus_distance = 0.0f, f_stop = 5.6f, fov_h_deg = 45.0f, fov_v_deg = 45.0f,
          lens_radius = 0.0f, plane_w = 0.0f, plane_h = 0.0f;
};

bool typed_array_match(const PropHeader& h, int pod, int extent, const char* interp) {
    // ITypedArrayProperty::matches with strict interpretation matching
    return h.pod == pod && (h.extent == extent || std::string(interp).empty()) && h.type == kArray &&
           get(h.meta, "interpretation") == interp;
}

// parse_attributes (houdini_alembic.cpp): one property -> a column, or nothing
bool parse_column(const Compound& parent, const PropHeader& h, int64_t frame, Column& col) {
    const std::string podName = get(h.meta, "podName");
    if (h.type == kCompound && podName == "string") {
        Compound c = parent.compound(h.name);
        const PropHeader* vh = c.find(".vals");
        const PropHeader* ih = c.find(".indices");
        if (!vh || !ih || vh->pod != kString || ih->pod != kU32) throw Error("bad indexed string " + h.name);
        const Sample vals = c.array(*vh, frame), idx = c.array(*ih, frame);
        col.type = kColString;
        col.rows = (uint32_t)idx.count;
        col.s = vals.strings;
        col.si.assign(idx.as<uint32_t>(), idx.as<uint32_t>() + idx.count);
        for (uint32_t k : col.si)
            if (k >= col.s.size()) throw Error("indexed string out of range");
        return true;
    }
    if (h.type == kCompound && podName == "float32_t" && get(h.meta, "podExtent") == "2") {
        Compound c = parent.compound(h.name);
        const PropHeader* vh = c.find(".vals");
        const PropHeader* ih = c.find(".indices");
        if (!vh || !ih || vh->pod != kF32 || vh->extent != 2 || ih->pod != kU32)
            throw Error("bad indexed vector2 " + h.name);
        const Sample vals = c.array(*vh, frame), idx = c.array(*ih, frame);
        col.type = kColVec2;
        col.dim = 2;
        col.rows = (uint32_t)idx.count;
        for (uint64_t r = 0; r < idx.count; ++r) {
            const uint32_t k = idx.as<uint32_t>()[r];
            if (k >= vals.count) throw Error("indexed vector2 out of range");
            col.f.push_back(vals.as<float>()[2 * k]);
            col.f.push_back(vals.as<float>()[2 * k + 1]);
        }
        return true;
    }
    if (typed_array_match(h, kF32, 2, "vector")) return false;  // read and dropped by the reference
    if (h.pod == kF32 && h.type == kArray) {
        const Sample v = parent.array(h, frame);
        const std::string ae = get(h.meta, "arrayExtent");
        const int array_extent = ae.empty() ? 1 : std::atoi(ae.c_str());
        const int comp = h.extent * array_extent;
        const uint64_t size = array_extent > 1 ? v.count / (uint64_t)array_extent : v.count;
        const float* p = v.as<float>();
        const uint64_t avail = v.bytes.size() / 4;
        if (comp == 1) {
            col.type = kColFloat;
            col.rows = (uint32_t)v.count;
            col.f.assign(p, p + std::min<uint64_t>(v.count, avail));
            return true;
        }
        if (comp >= 2 && comp <= 4) {
            col.type = comp == 2 ? kColVec2 : (comp == 3 ? kColVec3 : kColVec4);
            col.dim = comp;
            col.rows = (uint32_t)size;
            if (size * (uint64_t)comp > avail) throw Error("short vector column " + h.name);
            col.f.assign(p, p + size * (uint64_t)comp);
            return true;
        }
        return false;
    }
    if (typed_array_match(h, kI32, 1, "")) {
        const Sample v = parent.array(h, frame);
        col.type = kColInt;
        col.rows = (uint32_t)v.count;
        col.i.assign(v.as<int32_t>(), v.as<int32_t>() + v.count);
        return true;
    }
    if (typed_array_match(h, kString, 1, "")) {
        const Sample v = parent.array(h, frame);
        col.type = kColString;
        col.rows = (uint32_t)v.count;
        col.s.assign(v.strings.begin(), v.strings.begin() + (ptrdiff_t)v.count);
        col.si.resize(v.count);
        for (uint32_t r = 0; r < (uint32_t)v.count; ++r) col.si[r] = r;
        return true;
    }
    return false;
}

void parse_sheets(const Compound& c, int64_t frame, Sheet* points, Sheet* vertices, Sheet* primitives) {
    if (!c.valid()) throw Error("missing geometry parameters");
    for (const PropHeader& h : c.props()) {
        if (h.name.empty() || h.name[0] == '.') continue;
        Column col;
        col.key = h.name;
        if (!parse_column(c, h, frame, col)) continue;
        const std::string scope = get(h.meta, "geoScope");
        // the reference's condition reads (points && var) || vtx
        if ((points && scope == "var") || scope == "vtx") {
            if (points) points->cols.push_back(std::move(col));
        } else if (vertices && scope == "fvr") {
            vertices->cols.push_back(std::move(col));
        } else if (primitives && scope == "uni") {
            primitives->cols.push_back(std::move(col));
        }
    }
    for (Sheet* s : {points, vertices, primitives})
        if (s)
            std::stable_sort(s->cols.begin(), s->cols.end(),
                             [](const Column& a, const Column& b) { return a.key < b.key; });
}

bool is_schema(const Meta& m, const char* obj_title) {
    return get(m, "schemaObjTitle") == obj_title || get(m, "schema") == obj_title;
}

std::vector<uint32_t> int_array(const Compound& c, const char* name, int64_t frame) {
    const PropHeader* h = c.find(name);
    if (!h || h->type != kArray || h->pod != kI32) throw Error(std::string("missing ") + name);
    const Sample s = c.array(*h, frame);
    std::vector<uint32_t> out(s.count);
    for (uint64_t k = 0; k < s.count; ++k) out[k] = (uint32_t)s.as<int32_t>()[k];
    return out;
}

void take_P(SceneObject& o) {
    const Column* p = o.points.find("P", kColVec3);
    if (!p) throw Error("object " + o.name + " has no P");
    o.P.assign(p->f.begin(), p->f.begin() + 3 * (size_t)p->rows);
}

void vec_out(float* dst, double a, double b, double c) {
    dst[0] = (float)a;
    dst[1] = (float)b;
    dst[2] = (float)c;
}

// parse_common_property: the parent transform's name and visibility
void common(const Object& o, SceneObject& so, const std::vector<M44>& xforms, int64_t frame) {
    const Object* parent = o.parent();
    so.name = parent ? parent->full_name() : std::string();
    for (const M44& m : xforms) {
        std::array<float, 16> v;
        for (int i = 0; i < 16; ++i) v[i] = (float)m.x[i / 4][i % 4];
        so.xforms.push_back(v);
    }
    M44 c = M44::identity();
    for (const M44& m : xforms) c = m * c;
    so.combined_d = c;
    for (int i = 0; i < 16; ++i) so.combined[i] = (float)c.x[i / 4][i % 4];
    so.visible = true;
    if (parent) {
        Compound pp = parent->properties();
        if (pp.valid())
            if (const PropHeader* vh = pp.find("visible")) {
                const Sample v = pp.scalar(*vh, frame);
                so.visible = !v.bytes.empty() && (int8_t)v.bytes[0] == -1;
            }
    }
}

void parse_camera(const Object& o, SceneObject& so, int64_t frame) {
    const M44& c = so.combined_d;
    const M44 it = inverse(c);  // used transposed: direction d maps to (row j of the inverse) . d
    vec_out(so.eye, c.x[3][0] / c.x[3][3], c.x[3][1] / c.x[3][3], c.x[3][2] / c.x[3][3]);
    // multDirMatrix of the inverse transpose: (0,0,-1) -> -column 2 of the inverse, etc.
    const double fwd[3] = {0.0 * it.x[0][0] + 0.0 * it.x[0][1] + -1.0 * it.x[0][2],
                           0.0 * it.x[1][0] + 0.0 * it.x[1][1] + -1.0 * it.x[1][2],
                           0.0 * it.x[2][0] + 0.0 * it.x[2][1] + -1.0 * it.x[2][2]};
    const double upv[3] = {0.0 * it.x[0][0] + 1.0 * it.x[0][1] + 0.0 * it.x[0][2],
                           0.0 * it.x[1][0] + 1.0 * it.x[1][1] + 0.0 * it.x[1][2],
                           0.0 * it.x[2][0] + 1.0 * it.x[2][1] + 0.0 * it.x[2][2]};
    const double rgt[3] = {1.0 * it.x[0][0] + 0.0 * it.x[0][1] + 0.0 * it.x[0][2],
                           1.0 * it.x[1][0] + 0.0 * it.x[1][1] + 0.0 * it.x[1][2],
                           1.0 * it.x[2][0] + 0.0 * it.x[2][1] + 0.0 * it.x[2][2]};
    const double eye_d[3] = {c.x[3][0] / c.x[3][3], c.x[3][1] / c.x[3][3], c.x[3][2] / c.x[3][3]};
    vec_out(so.lookat, eye_d[0] + fwd[0], eye_d[1] + fwd[1], eye_d[2] + fwd[2]);
    vec_out(so.up, upv[0], upv[1], upv[2]);
    vec_out(so.down, -upv[0], -upv[1], -upv[2]);
    vec_out(so.forward, fwd[0], fwd[1], fwd[2]);
    vec_out(so.back, -fwd[0], -fwd[1], -fwd[2]);
    vec_out(so.left, -rgt[0], -rgt[1], -rgt[2]);
    vec_out(so.right, rgt[0], rgt[1], rgt[2]);

    Compound geom = o.properties().compound(".geom");
    if (!geom.valid()) throw Error("camera without .geom");
    const PropHeader* core_h = geom.find(".core");
    if (!core_h) throw Error("camera without .core");
    const Sample core = geom.scalar(*core_h, frame);
    if (core.pod != kF64 || core.bytes.size() < 16 * 8) throw Error("bad camera core");
    const double* v = core.as<double>();
    Compound user = geom.compound(".userProperties");
    auto user_float = [&](const char* name) -> float {
        const PropHeader* h = user.valid() ? user.find(name) : nullptr;
        if (!h || h->type != kScalar || h->pod != kF32) throw Error(std::string("camera without ") + name);
        const Sample s = user.scalar(*h, frame);
        float f;
        std::memcpy(&f, s.bytes.data(), 4);
        return f;
    };
    // ICamera::get / CameraSample, then the Houdini reader's derived values,
    // with the reference's float and double types
    so.resolution_x = (int)user_float("resx");
    so.resolution_y = (int)user_float("resy");
    so.focal_mm = (float)v[0];
    so.aperture_h_mm = (float)(v[1] * 10.0f);
    so.aperture_v_mm = (float)(v[3] * 10.0f);
    so.near_clip = (float)v[14];
    so.far_clip = (float)v[15];
    so.focus_distance = (float)v[11];
    so.f_stop = (float)v[10];
    so.fov_h_deg = (float)(2.0 * (std::atan(v[1] * 10.0 / (2.0 * v[0])) * (180.0 / M_PI)));
    const float fov_v_rad = std::atan(so.aperture_v_mm * 0.5f / so.focal_mm) * 2.0f;
    so.fov_v_deg = (float)(fov_v_rad / (2.0 * M_PI) * 360.0f);
    const float A = so.focal_mm / 1000.0f;
    const float B = so.focus_distance;
    const float F = A * B / (A + B);
    so.lens_radius = F / (2.0f * so.f_stop);
    so.plane_w = (float)(2.0f * so.focus_distance * std::tan(0.5f * so.fov_h_deg / 360.0f * 2.0 * M_PI));
    so.plane_h = (float)(2.0f * so.focus_distance * std::tan(0.5f * so.fov_v_deg / 360.0f * 2.0 * M_PI));
}

void parse_object(const Object& o, int64_t frame, std::vector<M44> xforms, std::vector<SceneObject>& out) {
    const Meta& m = o.meta();
    auto recurse = [&](const std::vector<M44>& xf) {
        for (const ObjectHeader& h : o.children())
            parse_object(Object(o.archive(), h.entry, h.full_name, h.meta, &o), frame, xf, out);
    };
    if (is_schema(m, "AbcGeom_PolyMesh_v1:.geom")) {
        SceneObject so;
        so.type = kPolyMesh;
        common(o, so, xforms, frame);
        Compound geom = o.properties().compound(".geom");
        if (!geom.valid()) throw Error("mesh without .geom");
        so.face_counts = int_array(geom, ".faceCounts", frame);
        so.indices = int_array(geom, ".faceIndices", frame);
        parse_sheets(geom.compound(".arbGeomParams"), frame, &so.points, &so.vertices, &so.primitives);
        parse_sheets(geom, frame, &so.points, &so.vertices, &so.primitives);
        take_P(so);
        out.push_back(std::move(so));
    } else if (is_schema(m, "AbcGeom_Points_v1:.geom")) {
        SceneObject so;
        so.type = kPoint;
        common(o, so, xforms, frame);
        Compound geom = o.properties().compound(".geom");
        if (!geom.valid()) throw Error("points without .geom");
        if (const PropHeader* ih = geom.find(".pointIds")) {
            const Sample ids = geom.array(*ih, frame);
            if (ids.pod != kU64) throw Error("point ids are not uint64");
            so.point_ids.assign(ids.as<uint64_t>(), ids.as<uint64_t>() + ids.count);
        }
        parse_sheets(geom.compound(".arbGeomParams"), frame, &so.points, nullptr, nullptr);
        parse_sheets(geom, frame, &so.points, nullptr, nullptr);
        take_P(so);
        out.push_back(std::move(so));
    } else if (is_schema(m, "AbcGeom_Curve_v2:.geom")) {
        SceneObject so;
        so.type = kCurve;
        common(o, so, xforms, frame);
        Compound geom = o.properties().compound(".geom");
        if (!geom.valid()) throw Error("curves without .geom");
        parse_sheets(geom.compound(".arbGeomParams"), frame, &so.points, &so.vertices, &so.primitives);
        parse_sheets(geom, frame, &so.points, &so.vertices, &so.primitives);
        so.face_counts = int_array(geom, "nVertices", frame);
        take_P(so);
        out.push_back(std::move(so));
    } else if (is_schema(m, "AbcGeom_Camera_v1:.geom")) {
        SceneObject so;
        so.type = kCamera;
        common(o, so, xforms, frame);
        parse_camera(o, so, frame);
        out.push_back(std::move(so));
    } else if (is_schema(m, "AbcGeom_Xform_v3:.xform")) {
        xforms.push_back(xform_matrix(o, frame));
        recurse(xforms);
    } else {
        recurse(xforms);
    }
}

// ------------------------------------------------------------------ JSON (the oracle's dump format)
struct Json {
    std::string out;
    void raw(const char* t) { out += t; }
    void f(float v) {
        char b[48];
        if (std::isfinite(v))
            std::snprintf(b, sizeof b, "%.9g", (double)v);
        else
            std::snprintf(b, sizeof b, "\"%s\"", std::isnan(v) ? "nan" : (v > 0 ? "inf" : "-inf"));
        out += b;
    }
    void u(uint64_t v) { out += std::to_string(v); }
    void i(int64_t v) { out += std::to_string(v); }
    static bool utf8(const std::string& t) {
        for (size_t i = 0; i < t.size();) {
            const unsigned char c = (unsigned char)t[i];
            const int n = c < 0x80 ? 0 : (c >> 5) == 6 ? 1 : (c >> 4) == 14 ? 2 : (c >> 3) == 30 ? 3 : -1;
            if (n < 0 || i + (size_t)n >= t.size()) return false;
            for (int k = 1; k <= n; ++k)
                if (((unsigned char)t[i + k] >> 6) != 2) return false;
            i += (size_t)n + 1;
        }
        return true;
    }
    void str(const std::string& t) {
        const bool valid = utf8(t);  // otherwise bytes >= 0x80 are written as \u00XX
        out += '"';
        for (unsigned char c : t) {
            if (!valid && c >= 0x80) {
                char b[8];
                std::snprintf(b, sizeof b, "\\u%04x", c);
                out += b;
            } else if (c == '"' || c == '\\') {
                out += '\\';
                out += (char)c;
            } else if (c < 0x20) {
                char b[8];
                std::snprintf(b, sizeof b, "\\u%04x", c);
                out += b;
            } else {
                out += (char)c;
            }
        }
        out += '"';
    }
    void vec(const float* v, int n) {
        raw("[");
        for (int k = 0; k < n; ++k) {
            if (k) raw(",");
            f(v[k]);
        }
        raw("]");
    }
};

void json_sheet(Json& j, const Sheet& sh) {
    static const char* kTypes[] = {"Int", "Float", "Vector2", "Vector3", "Vector4", "String"};
    j.raw("[");
    for (size_t c = 0; c < sh.cols.size(); ++c) {
        const Column& col = sh.cols[c];
        if (c) j.raw(",");
        j.raw("{\"key\":");
        j.str(col.key);
        j.raw(",\"type\":\"");
        j.raw(kTypes[col.type]);
        j.raw("\",\"rows\":");
        j.u(col.rows);
        j.raw(",\"values\":[");
        for (uint32_t r = 0; r < col.rows; ++r) {
            if (r) j.raw(",");
            if (col.type == kColInt)
                j.i(r < col.i.size() ? col.i[r] : 0);
            else if (col.type == kColFloat)
                j.f(r < col.f.size() ? col.f[r] : 0.0f);
            else if (col.type == kColString)
                j.str(col.str(r));
            else
                j.vec(col.f.data() + (size_t)r * col.dim, col.dim);
        }
        j.raw("]}");
    }
    j.raw("]");
}

std::string describe(const std::vector<SceneObject>& objs, uint32_t frame_count) {
    static const char* kTypes[] = {"PolygonMesh", "Point", "Curve", "Camera"};
    Json j;
    j.raw("{\"frame_count\":");
    j.u(frame_count);
    j.raw(",\"objects\":[");
    for (size_t k = 0; k < objs.size(); ++k) {
        const SceneObject& o = objs[k];
        if (k) j.raw(",\n");
        j.raw("{\"type\":\"");
        j.raw(kTypes[o.type]);
        j.raw("\",\"name\":");
        j.str(o.name);
        j.raw(o.visible ? ",\"visible\":true,\"combined\":" : ",\"visible\":false,\"combined\":");
        j.vec(o.combined, 16);
        j.raw(",\"xforms\":[");
        for (size_t x = 0; x < o.xforms.size(); ++x) {
            if (x) j.raw(",");
            j.vec(o.xforms[x].data(), 16);
        }
        j.raw("]");
        if (o.type == kPolyMesh) {
            j.raw(",\"faceCounts\":[");
            for (size_t x = 0; x < o.face_counts.size(); ++x) {
                if (x) j.raw(",");
                j.u(o.face_counts[x]);
            }
            j.raw("],\"indices\":[");
            for (size_t x = 0; x < o.indices.size(); ++x) {
                if (x) j.raw(",");
                j.u(o.indices[x]);
            }
            j.raw("],\"P\":[");
            for (size_t x = 0; x < o.P.size() / 3; ++x) {
                if (x) j.raw(",");
                j.vec(o.P.data() + 3 * x, 3);
            }
            j.raw("],\"points\":");
            json_sheet(j, o.points);
            j.raw(",\"vertices\":");
            json_sheet(j, o.vertices);
            j.raw(",\"primitives\":");
            json_sheet(j, o.primitives);
        } else if (o.type == kPoint) {
            j.raw(",\"pointIds\":[");
            for (size_t x = 0; x < o.point_ids.size(); ++x) {
                if (x) j.raw(",");
                j.u(o.point_ids[x]);
            }
            j.raw("],\"P\":[");
            for (size_t x = 0; x < o.P.size() / 3; ++x) {
                if (x) j.raw(",");
                j.vec(o.P.data() + 3 * x, 3);
            }
            j.raw("],\"points\":");
            json_sheet(j, o.points);
        } else if (o.type == kCamera) {
            const std::pair<const char*, const float*> vecs[] = {
                {"eye", o.eye}, {"lookat", o.lookat}, {"up", o.up}, {"down", o.down}, {"forward", o.forward},
                {"back", o.back}, {"left", o.left}, {"right", o.right}};
            for (const auto& v : vecs) {
                j.raw(",\"");
                j.raw(v.first);
                j.raw("\":");
                j.vec(v.second, 3);
            }
            j.raw(",\"resolution_x\":");
            j.i(o.resolution_x);
            j.raw(",\"resolution_y\":");
            j.i(o.resolution_y);
            const std::pair<const char*, float> vals[] = {
                {"focalLength_mm", o.focal_mm}, {"aperture_horizontal_mm", o.aperture_h_mm},
                {"aperture_vertical_mm", o.aperture_v_mm}, {"nearClip", o.near_clip}, {"farClip", o.far_clip},
                {"focusDistance", o.focus_distance}, {"f_stop", o.f_stop}, {"fov_horizontal_degree", o.fov_h_deg},
                {"fov_vertical_degree", o.fov_v_deg}, {"lensRadius", o.lens_radius},
                {"objectPlaneWidth", o.plane_w}, {"objectPlaneHeight", o.plane_h}};
            for (const auto& v : vals) {
                j.raw(",\"");
                j.raw(v.first);
                j.raw("\":");
                j.f(v.second);
            }
        }
        j.raw("}");
    }
    j.raw("]}\n");
    return j.out;
}

// ------------------------------------------------------------------ Radiance .hdr
// The RGBE format (Ward, "Real Pixels", Graphics Gems II): a text header
// ending in an empty line, a resolution line "-Y h +X w", then scanlines top
// to bottom, flat or run-length encoded per channel.  A pixel decodes as
// byte * 2^(e - 136) per channel, 0 when e = 0 (stb_image's decoding, which
// the reference loads envmaps with), alpha 1.
std::vector<float> load_hdr(const std::string& path, int& w, int& h) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error("cannot open envmap " + path);
    std::vector<unsigned char> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    size_t pos = 0;
    auto line = [&]() {
        std::string l;
        while (pos < b.size() && b[pos] != '\n') l += (char)b[pos++];
        if (pos < b.size()) ++pos;
        return l;
    };
    const std::string magic = line();
    if (magic != "#?RADIANCE" && magic != "#?RGBE") throw Error("not a Radiance .hdr file: " + path);
    for (;;) {
        if (pos >= b.size()) throw Error("truncated .hdr header");
        const std::string l = line();
        if (l.empty()) break;
        if (l.rfind("FORMAT=", 0) == 0 && l != "FORMAT=32-bit_rle_rgbe") throw Error("unsupported .hdr format");
    }
    const std::string res = line();
    if (std::sscanf(res.c_str(), "-Y %d +X %d", &h, &w) != 2 || w <= 0 || h <= 0 || w > 65536 || h > 65536)
        throw Error("unsupported .hdr orientation or size");
    std::vector<float> out((size_t)w * h * 4);
    std::vector<unsigned char> scan((size_t)w * 4);
    auto put = [&](size_t px, const unsigned char* e) {
        float* o = out.data() + 4 * px;
        if (e[3] != 0) {
            const float f1 = (float)std::ldexp(1.0f, (int)e[3] - (128 + 8));
            o[0] = e[0] * f1;
            o[1] = e[1] * f1;
            o[2] = e[2] * f1;
        } else {
            o[0] = o[1] = o[2] = 0.0f;
        }
        o[3] = 1.0f;
    };
    auto need = [&](size_t k) {
        if (pos + k > b.size()) throw Error("truncated .hdr data");
    };
    bool flat = w < 8 || w >= 32768;
    for (int y = 0; y < h; ++y) {
        if (!flat) {
            need(4);
            if (!(b[pos] == 2 && b[pos + 1] == 2 && (b[pos + 2] & 0x80) == 0)) flat = true;
        }
        if (flat) {  // flat RGBE for the rest of the image
            need((size_t)w * 4 * (size_t)(h - y));
            for (size_t k = 0; k < (size_t)w * (size_t)(h - y); ++k) put((size_t)y * w + k, &b[pos + 4 * k]);
            return out;
        }
        if (((b[pos + 2] << 8) | b[pos + 3]) != w) throw Error("bad .hdr scanline length");
        pos += 4;
        for (int c = 0; c < 4; ++c) {
            int x = 0;
            while (x < w) {
                need(1);
                int count = b[pos++];
                if (count > 128) {
                    count -= 128;
                    need(1);
                    if (x + count > w) throw Error("bad .hdr run");
                    const unsigned char v = b[pos++];
                    for (int k = 0; k < count; ++k) scan[4 * (size_t)(x++) + c] = v;
                } else {
                    if (count == 0 || x + count > w) throw Error("bad .hdr run");
                    need((size_t)count);
                    for (int k = 0; k < count; ++k) scan[4 * (size_t)(x++) + c] = b[pos++];
                }
            }
        }
        for (int x = 0; x < w; ++x) put((size_t)y * w + x, &scan[4 * (size_t)x]);
    }
    return out;
}

// ------------------------------------------------------------------ scene building
const Column* column(const Sheet& s, const char* key, int type) { return s.find(key, type); }

void set3(float* d, const Column* c, uint32_t row) {
    if (c && row < c->rows) std::memcpy(d, c->f.data() + 3 * (size_t)row, 12);
}

rgr_material lambertian(float r, float g, float b) {
    rgr_material m{};
    m.type = RGR_MAT_LAMBERTIAN;
    m.r[0] = r;
    m.r[1] = g;
    m.r[2] = b;
    return m;
}

// add_materials (scene_manager.hpp:197-277): the material named in each
// primitive's "material" column, its properties from the columns of the
// same name and type (Lambertian: Le, Cd, BackEmission; Ward: alpha,
// reflectance, edgetint, falloff; HomogeneousVolume: C, Cd), class defaults
// elsewhere; no "material" column: the magenta fallback Lambertian
std::vector<rgr_material> bind_materials(const SceneObject& o, size_t ntris) {
    std::vector<rgr_material> out;
    const Sheet& p = o.primitives;
    const Column* mat = column(p, "material", kColString);
    if (!mat) {
        out.assign(ntris, lambertian(0.9f, 0.1f, 0.9f));
        return out;
    }
    const uint32_t rows = p.rows();
    if (rows != ntris) throw Error("object " + o.name + ": primitive attributes do not match its triangles");
    const Column* Le = column(p, "Le", kColVec3);
    const Column* Cd = column(p, "Cd", kColVec3);
    const Column* back = column(p, "BackEmission", kColInt);
    const Column* alpha = column(p, "alpha", kColFloat);
    const Column* refl = column(p, "reflectance", kColVec3);
    const Column* tint = column(p, "edgetint", kColVec3);
    const Column* falloff = column(p, "falloff", kColFloat);
    const Column* C = column(p, "C", kColFloat);
    out.resize(rows);
    if (mat->rows < rows) throw Error("material column shorter than the primitives");
    // the class of each distinct name, once
    std::vector<int> cls(mat->s.size());
    for (size_t k = 0; k < mat->s.size(); ++k) {
        const std::string& n = mat->s[k];
        cls[k] = n == "Lambertian" ? RGR_MAT_LAMBERTIAN
                 : n == "Specular" ? RGR_MAT_SPECULAR
                 : n == "Dierectric" ? RGR_MAT_DIELECTRIC
                 : n == "Ward" ? RGR_MAT_WARD
                 : n == "HomogeneousVolume" ? RGR_MAT_HOMOGENEOUS_VOLUME : 0;
    }
    for (uint32_t i = 0; i < rows; ++i) {
        const int c = cls[mat->si[i]];
        rgr_material m{};
        if (c == RGR_MAT_LAMBERTIAN) {
            m = lambertian(1.0f, 1.0f, 1.0f);
            set3(m.le, Le, i);
            set3(m.r, Cd, i);
            if (back && i < back->rows) m.back_emission = back->i[i];
        } else if (c == RGR_MAT_SPECULAR) {
            m.type = RGR_MAT_SPECULAR;
        } else if (c == RGR_MAT_DIELECTRIC) {
            m.type = RGR_MAT_DIELECTRIC;
        } else if (c == RGR_MAT_WARD) {
            m.type = RGR_MAT_WARD;
            m.alpha = 0.1f;
            m.r[0] = m.r[1] = m.r[2] = 1.0f;
            m.edgetint[0] = m.edgetint[1] = m.edgetint[2] = 1.0f;
            m.falloff = 0.5f;
            if (alpha && i < alpha->rows) m.alpha = alpha->f[i];
            set3(m.r, refl, i);
            set3(m.edgetint, tint, i);
            if (falloff && i < falloff->rows) m.falloff = falloff->f[i];
        } else if (c == RGR_MAT_HOMOGENEOUS_VOLUME) {
            m.type = RGR_MAT_HOMOGENEOUS_VOLUME;
            m.c = 1.0f;
            m.r[0] = m.r[1] = m.r[2] = 1.0f;
            if (C && i < C->rows) m.c = C->f[i];
            set3(m.r, Cd, i);
        } else {
            throw Error("object " + o.name + ": unknown material \"" + mat->str(i) + "\"");
        }
        out[i] = m;
    }
    return out;
}

// the combined transform as SceneManager applies it: the float matrix the
// reader stores, widened to double, times (P, 1) (column-major, pairwise sums)
void transform_point(const float* m, const float* p, float* out) {
    const double v[4] = {(double)p[0], (double)p[1], (double)p[2], 1.0};
    for (int r = 0; r < 3; ++r) {
        const double a = (double)m[0 + r] * v[0] + (double)m[4 + r] * v[1];
        const double b = (double)m[8 + r] * v[2] + (double)m[12 + r] * v[3];
        out[r] = (float)(a + b);
    }
}

bool is_identity(const float* m) {
    for (int i = 0; i < 16; ++i)
        if (m[i] != ((i % 5 == 0) ? 1.0f : 0.0f)) return false;
    return true;
}

struct LoadStats {
    uint32_t meshes = 0, skipped = 0, triangles = 0, spheres = 0;
    int has_env = 0;
};

int add_polymesh(rgr_scene* scene, const SceneObject& o, LoadStats& st) {
    for (uint32_t c : o.face_counts)
        if (c != 3) {  // skipped non-triangle mesh (scene_manager.hpp:343-347)
            st.skipped++;
            return RGR_OK;
        }
    const size_t nv = o.P.size() / 3, nt = o.indices.size() / 3;
    for (uint32_t i : o.indices)
        if (i >= nv) throw Error("object " + o.name + ": index out of range");
    std::vector<float> P(o.P.size());
    for (size_t v = 0; v < nv; ++v) transform_point(o.combined, &o.P[3 * v], &P[3 * v]);
    const std::vector<rgr_material> mats = bind_materials(o, nt);
    const int r = rgr_scene_add_mesh(scene, P.data(), nv, o.indices.data(), nt, mats.data());
    if (r == RGR_OK) {
        st.meshes++;
        st.triangles += (uint32_t)nt;
    }
    return r;
}

int add_points(rgr_scene* scene, const SceneObject& o, const std::string& dir, LoadStats& st) {
    const Column* ptype = column(o.points, "point_type", kColString);
    if (!ptype) {  // addPointPrimitive (scene_manager.hpp:372-431): spheres of radius pscale
        const Column* pscale = column(o.points, "pscale", kColFloat);
        if (!pscale) return RGR_OK;
        const size_t n = o.P.size() / 3;
        std::vector<float> xyzr(4 * n);
        const bool ident = is_identity(o.combined);
        for (size_t i = 0; i < n; ++i) {
            if (ident)
                std::memcpy(&xyzr[4 * i], &o.P[3 * i], 12);
            else
                transform_point(o.combined, &o.P[3 * i], &xyzr[4 * i]);
            xyzr[4 * i + 3] = i < pscale->rows ? pscale->f[i] : 0.0f;
        }
        const Column* Cd = column(o.points, "Cd", kColVec3);
        std::vector<rgr_material> mats(n, lambertian(0.9f, 0.1f, 0.9f));
        if (Cd)
            for (size_t i = 0; i < n; ++i) {
                mats[i] = lambertian(0.0f, 0.0f, 0.0f);
                set3(mats[i].r, Cd, (uint32_t)i);
            }
        const int r = rgr_scene_add_spheres(scene, xyzr.data(), n, mats.data());
        if (r == RGR_OK) st.spheres += (uint32_t)n;
        return r;
    }
    // addPoint (scene_manager.hpp:432-497): "ImageEnvmap" points set the envmap
    const Column* file = column(o.points, "file", kColString);
    const Column* clamp = column(o.points, "clamp", kColFloat);
    const Column* scale = column(o.points, "scale", kColFloat);
    for (uint32_t i = 0; i < ptype->rows; ++i) {
        if (ptype->str(i) != "ImageEnvmap") continue;
        std::string name = file && i < file->rows ? file->str(i) : std::string();
        const float cmax = clamp && i < clamp->rows ? clamp->f[i] : std::numeric_limits<float>::max();
        const float sc = scale && i < scale->rows ? scale->f[i] : 1.0f;
        if (name.empty()) continue;
        const std::string path = name[0] == '/' ? name : (dir.empty() ? name : dir + "/" + name);
        int w = 0, h = 0;
        const std::vector<float> img = load_hdr(path, w, h);
        const int r = rgr_scene_set_envmap(scene, img.data(), w, h, cmax, sc);
        if (r != RGR_OK) return r;
        st.has_env = 1;
    }
    return RGR_OK;
}

// standardCamera (wavefront_path_tracing.hpp:103-118), in float
void standard_camera(const SceneObject& c, rgr_camera& cam) {
    cam.image_w = (uint32_t)c.resolution_x;
    cam.image_h = (uint32_t)c.resolution_y;
    for (int k = 0; k < 3; ++k) {
        cam.eye[k] = c.eye[k];
        cam.forward[k] = c.forward[k];
        cam.up[k] = c.up[k];
        cam.right[k] = c.right[k];
        cam.imageplane_o[k] = ((c.eye[k] + c.forward[k] * c.focus_distance) + c.left[k] * c.plane_w * 0.5f) +
                              c.up[k] * c.plane_h * 0.5f;
        cam.imageplane_r[k] = c.right[k] * c.plane_w / (float)c.resolution_x;
        cam.imageplane_b[k] = c.down[k] * c.plane_h / (float)c.resolution_y;
    }
}

}  // namespace abc
}  // namespace rgr

struct rgr_alembic {
    std::unique_ptr<rgr::abc::Archive> archive;
    std::string dir;
    uint32_t frame_count = 1;
};

namespace {
int fail(const std::exception& e) {
    rgr::set_error(std::string("alembic: ") + e.what());
    return RGR_E_INVALID;
}
std::vector<rgr::abc::SceneObject> read_frame(const rgr_alembic* a, uint32_t frame) {
    std::vector<rgr::abc::SceneObject> objs;
    rgr::abc::parse_object(a->archive->top(), (int64_t)frame, {}, objs);
    return objs;
}
}  // namespace

extern "C" {

int rgr_alembic_open(rgr_alembic** out, const char* path) {
    if (!out || !path) return RGR_E_INVALID;
    *out = nullptr;
    try {
        std::unique_ptr<rgr_alembic> a(new rgr_alembic());
        a->archive.reset(new rgr::abc::Archive(path));
        const std::string p(path);
        const size_t slash = p.find_last_of('/');
        a->dir = slash == std::string::npos ? std::string() : p.substr(0, slash);
        // AlembicStorage::open: the frame count from the top object's "1.samples"
        rgr::abc::Compound top = a->archive->top().properties();
        if (top.valid())
            if (const rgr::abc::PropHeader* h = top.find("1.samples")) {
                const rgr::abc::Sample s = top.scalar(*h, 0);
                if (s.pod == rgr::abc::kU32 && s.bytes.size() >= 4) std::memcpy(&a->frame_count, s.bytes.data(), 4);
            }
        *out = a.release();
        return RGR_OK;
    } catch (const std::bad_alloc&) {
        return RGR_E_OOM;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

void rgr_alembic_close(rgr_alembic* a) { delete a; }

uint32_t rgr_alembic_frame_count(const rgr_alembic* a) { return a ? a->frame_count : 0u; }

int rgr_alembic_describe(rgr_alembic* a, uint32_t frame, char* buf, uint64_t cap, uint64_t* needed) {
    if (!a || (cap && !buf)) return RGR_E_INVALID;
    try {
        const std::string j = rgr::abc::describe(read_frame(a, frame), a->frame_count);
        if (needed) *needed = j.size() + 1;
        if (cap < j.size() + 1) return cap ? RGR_E_INVALID : RGR_OK;
        std::memcpy(buf, j.c_str(), j.size() + 1);
        return RGR_OK;
    } catch (const std::bad_alloc&) {
        return RGR_E_OOM;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int rgr_alembic_load(rgr_alembic* a, uint32_t frame, rgr_scene* scene, rgr_alembic_info* info) {
    RGR_NVTX_RANGE("rgr_alembic_load");
    if (!a || !scene) return RGR_E_INVALID;
    try {
        using namespace rgr::abc;
        const std::vector<SceneObject> objs = read_frame(a, frame);
        LoadStats st;
        const SceneObject* cam = nullptr;
        // visible meshes (and the first visible camera), then visible points: the order
        // of WavefrontPathTracing's constructor
        for (const SceneObject& o : objs) {
            if (!o.visible) continue;
            if (!cam && o.type == kCamera) cam = &o;
            if (o.type == kPolyMesh) {
                const int r = add_polymesh(scene, o, st);
                if (r != RGR_OK) return r;
            }
        }
        for (const SceneObject& o : objs) {
            if (!o.visible || o.type != kPoint) continue;
            const int r = add_points(scene, o, a->dir, st);
            if (r != RGR_OK) return r;
        }
        if (info) {
            *info = rgr_alembic_info{};
            info->frame_count = a->frame_count;
            info->meshes = st.meshes;
            info->meshes_skipped = st.skipped;
            info->triangles = st.triangles;
            info->spheres = st.spheres;
            info->has_envmap = st.has_env;
            info->has_camera = cam ? 1 : 0;
            if (cam) {
                standard_camera(*cam, info->camera);
                info->lens_radius = cam->lens_radius;
                info->focus_distance = cam->focus_distance;
                info->fov_horizontal_degree = cam->fov_h_deg;
                info->fov_vertical_degree = cam->fov_v_deg;
            }
        }
        return RGR_OK;
    } catch (const std::bad_alloc&) {
        return RGR_E_OOM;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

}  // extern "C"
