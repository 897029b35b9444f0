// hrt_ingest.cpp -- scene ingestion: PLY, OBJ and Helios XML files to primitive arrays.
//
// Restates the geometry part of the reference's loaders (core/src/Context_fileIO.cpp):
//   Context::loadPLY :3633-3908  (ASCII vertices / faces, up-axis remap, base at z = 0,
//                                  scale to a height, rotatePoint, fan triangulation, degenerate
//                                  triangles dropped)
//   Context::loadOBJ :3995-4340  (v / vt / f / o / usemtl / mtllib Kd colours, scale to a height,
//                                  YUP rotation, triangles grouped by material name)
//   Context::loadXML :1260-2230  (patch / triangle / voxel / disk elements with their <transform>,
//                                  triangle <vertices>, scalar primitive data)
// Host code only; the arrays feed hrt_update_geometry or hrt_server_add_scene.  Binary
// little-endian PLY is read as well (scanned plants are usually stored that way).
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/hrt.h"

struct hrt_scene_file {
    std::vector<float> T;        // [n*16]
    std::vector<uint32_t> type;  // [n]
    std::vector<int8_t> twosided;
    std::vector<float> color;    // [n*3]
    std::map<std::string, std::vector<double>> data;  // label -> [n], NaN where absent
};

namespace {

thread_local std::string g_err;

int fail(const std::string &m) {
    g_err = m;
    return HRT_EINVAL;
}

struct V3 {
    float x, y, z;
};
V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float mag(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
float tri_area(V3 a, V3 b, V3 c) { return 0.5f * mag(cross(sub(b, a), sub(c, a))); }

// rotatePoint(p, SphericalCoord(1, elevation, azimuth)) of core/src/global.cpp:152-204:
// R = Rz(azimuth) Ry(elevation) applied to p.
V3 rotate_point(V3 p, float theta, float phi) {
    if (theta == 0.f && phi == 0.f) return p;
    const float st = std::sin(theta), ct = std::cos(theta), sp = std::sin(phi), cp = std::cos(phi);
    const float Ry[3][3] = {{ct, 0.f, st}, {0.f, 1.f, 0.f}, {-st, 0.f, ct}};
    const float Rz[3][3] = {{cp, -sp, 0.f}, {sp, cp, 0.f}, {0.f, 0.f, 1.f}};
    float M[3][3] = {};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) M[i][j] = M[i][j] + Rz[i][k] * Ry[k][j];
    return V3{M[0][0] * p.x + M[0][1] * p.y + M[0][2] * p.z, M[1][0] * p.x + M[1][1] * p.y + M[1][2] * p.z,
              M[2][0] * p.x + M[2][1] * p.y + M[2][2] * p.z};
}

// Transform of the canonical triangle (0,0,0), (0,1,0), (1,1,0) onto (v0, v1, v2): columns
// v2 - v1, v1 - v0, the unit normal and v0, in FP64 rounded to FP32.
void triangle_transform(V3 a, V3 b, V3 c, float *T) {
    const double e0[3] = {(double)b.x - a.x, (double)b.y - a.y, (double)b.z - a.z};
    const double e1[3] = {(double)c.x - a.x, (double)c.y - a.y, (double)c.z - a.z};
    double n[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
    double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (l < 1e-30) l = 1e-30;
    const double c0[3] = {(double)c.x - b.x, (double)c.y - b.y, (double)c.z - b.z};
    const double o[3] = {a.x, a.y, a.z};
    for (int r = 0; r < 3; ++r) {
        T[4 * r + 0] = (float)c0[r];
        T[4 * r + 1] = (float)e0[r];
        T[4 * r + 2] = (float)(n[r] / l);
        T[4 * r + 3] = (float)o[r];
    }
    T[12] = T[13] = T[14] = 0.f;
    T[15] = 1.f;
}

void add_triangle(hrt_scene_file &f, V3 a, V3 b, V3 c, const float *rgb) {
    const size_t k = f.type.size();
    f.T.resize(16 * (k + 1));
    triangle_transform(a, b, c, &f.T[16 * k]);
    f.type.push_back(1u);
    f.twosided.push_back(1);
    f.color.insert(f.color.end(), rgb, rgb + 3);
}

bool parse_float(const std::string &s, float *v) {
    if (s.empty()) return false;
    char *end = nullptr;
    const double d = std::strtod(s.c_str(), &end);
    if (end == s.c_str() || *end != '\0') return false;
    *v = (float)d;
    return std::isfinite(*v);
}

// ------------------------------------------------------------------ PLY --
struct PlyProp {
    std::string name, type;  // type: scalar type of a vertex property
};

size_t ply_size(const std::string &t) {
    if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
    if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
    if (t == "int" || t == "uint" || t == "float" || t == "int32" || t == "uint32" || t == "float32") return 4;
    if (t == "double" || t == "float64") return 8;
    return 0;
}

double ply_value(const unsigned char *p, const std::string &t) {
    if (t == "char" || t == "int8") return (double)(int8_t)p[0];
    if (t == "uchar" || t == "uint8") return (double)p[0];
    int16_t s16;
    uint16_t u16;
    int32_t s32;
    uint32_t u32;
    float f32;
    double f64;
    if (t == "short" || t == "int16") return std::memcpy(&s16, p, 2), (double)s16;
    if (t == "ushort" || t == "uint16") return std::memcpy(&u16, p, 2), (double)u16;
    if (t == "int" || t == "int32") return std::memcpy(&s32, p, 4), (double)s32;
    if (t == "uint" || t == "uint32") return std::memcpy(&u32, p, 4), (double)u32;
    if (t == "float" || t == "float32") return std::memcpy(&f32, p, 4), (double)f32;
    return std::memcpy(&f64, p, 8), f64;
}

int load_ply(const char *path, const hrt_load_options &o, hrt_scene_file &f) {
    std::ifstream in(path, std::ios::binary);
    if (!in) return fail(std::string("could not open ") + path);
    std::string line, word;
    std::getline(in, line);
    if (line.rfind("ply", 0) != 0) return fail(std::string(path) + " is not a PLY file");
    std::string format;
    size_t nv = 0, nf = 0;
    std::vector<PlyProp> vprops;
    std::string list_count = "uchar", list_index = "int";
    int element = 0;  // 1 vertex, 2 face, 3 other
    bool header_done = false;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ls(line);
        ls >> word;
        if (word == "format") {
            ls >> format;
        } else if (word == "element") {
            std::string name;
            long long cnt = -1;
            ls >> name >> cnt;
            if (cnt < 0) return fail("PLY element count should be a non-negative integer");
            if (name == "vertex") element = 1, nv = (size_t)cnt;
            else if (name == "face") element = 2, nf = (size_t)cnt;
            else element = 3;
        } else if (word == "property") {
            std::string t;
            ls >> t;
            if (t == "list") {
                std::string ct, it, name;
                ls >> ct >> it >> name;
                if (element == 2) list_count = ct, list_index = it;
            } else if (element == 1) {
                PlyProp p;
                p.type = t;
                ls >> p.name;
                vprops.push_back(p);
            }
        } else if (word == "end_header") {
            header_done = true;
            break;
        }
    }
    if (!header_done) return fail("PLY header has no end_header");
    const bool ascii = format == "ascii";
    if (!ascii && format != "binary_little_endian") return fail("PLY format " + format + " is not supported (ascii or binary_little_endian)");
    bool has_color = false;
    for (auto &p : vprops) has_color = has_color || p.name == "red";
    std::vector<V3> v(nv, V3{0.f, 0.f, 0.f});
    std::vector<float> col(3 * nv, 0.f);
    const int up = o.up_axis;  // 0 XUP, 1 YUP, 2 ZUP
    auto put = [&](size_t row, const std::string &name, double val) {
        const float x = (float)val;
        V3 &q = v[row];
        if (name == "x") (up == 0 ? q.z : (up == 1 ? q.y : q.x)) = x;
        else if (name == "y") (up == 0 ? q.x : (up == 1 ? q.z : q.y)) = x;
        else if (name == "z") (up == 0 ? q.y : (up == 1 ? q.x : q.z)) = x;
        else if (name == "red") col[3 * row] = x / 255.f;
        else if (name == "green") col[3 * row + 1] = x / 255.f;
        else if (name == "blue") col[3 * row + 2] = x / 255.f;
    };
    for (size_t r = 0; r < nv; ++r) {
        for (auto &p : vprops) {
            if (ascii) {
                std::string tok;
                if (!(in >> tok)) return fail("read past the end of the PLY file while reading vertices");
                float x;
                if (!parse_float(tok, &x)) return fail("PLY vertex " + std::to_string(r) + " has an invalid value");
                put(r, p.name, x);
            } else {
                const size_t sz = ply_size(p.type);
                unsigned char buf[8];
                if (sz == 0 || !in.read((char *)buf, (std::streamsize)sz)) return fail("PLY vertex data ended early or has an unknown type");
                put(r, p.name, ply_value(buf, p.type));
            }
        }
    }
    // base at z = 0, scale to the height, rotate, move to the origin (Context_fileIO.cpp:3808-3845)
    float zmin = 10000.f, zmax = -10000.f;
    for (auto &q : v) {
        zmin = std::fmin(zmin, q.z);
        zmax = std::fmax(zmax, q.z);
    }
    const float scl = o.height > 0.f ? o.height / (zmax - zmin) : 1.f;
    for (auto &q : v) {
        q.z -= zmin;
        q = V3{q.x * scl, q.y * scl, q.z * scl};
        q = rotate_point(q, o.rotation[0], o.rotation[1]);
        q = V3{q.x + o.origin[0], q.y + o.origin[1], q.z + o.origin[2]};
    }
    std::vector<long long> face;
    for (size_t r = 0; r < nf; ++r) {
        long long cnt = 0;
        face.clear();
        if (ascii) {
            if (!(in >> cnt) || cnt < 0) return fail("PLY face " + std::to_string(r) + " has an invalid vertex count");
            for (long long i = 0; i < cnt; ++i) {
                long long idx;
                if (!(in >> idx)) return fail("PLY face " + std::to_string(r) + " has an invalid vertex index");
                face.push_back(idx);
            }
        } else {
            unsigned char buf[8];
            const size_t cs = ply_size(list_count), is = ply_size(list_index);
            if (cs == 0 || is == 0 || !in.read((char *)buf, (std::streamsize)cs)) return fail("PLY face data ended early");
            cnt = (long long)ply_value(buf, list_count);
            for (long long i = 0; i < cnt; ++i) {
                if (!in.read((char *)buf, (std::streamsize)is)) return fail("PLY face data ended early");
                face.push_back((long long)ply_value(buf, list_index));
            }
        }
        for (long long idx : face)
            if (idx < 0 || (size_t)idx >= nv) return fail("PLY face " + std::to_string(r) + " indexes a missing vertex");
        for (long long t = 2; t < cnt; ++t) {
            const V3 a = v[face[0]], b = v[face[t - 1]], c = v[face[t]];
            if (mag(sub(a, b)) < 1e-10f || mag(sub(a, c)) < 1e-10f || mag(sub(b, c)) < 1e-10f) continue;
            if (tri_area(a, b, c) < 1e-8f) continue;
            add_triangle(f, a, b, c, has_color ? &col[3 * face[0]] : o.default_color);
        }
    }
    return HRT_OK;
}

// ------------------------------------------------------------------ OBJ --
std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

std::map<std::string, std::vector<float>> load_mtl(const std::string &path) {
    std::map<std::string, std::vector<float>> m;
    std::ifstream in(path);
    std::string line, cur;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string w;
        ls >> w;
        if (w == "newmtl") {
            std::getline(ls, cur);
            cur = trim(cur);
            m[cur] = {0.f, 0.f, 0.f};
        } else if (w == "Kd" && !cur.empty()) {
            float r = 0, g = 0, b = 0;
            ls >> r >> g >> b;
            m[cur] = {r, g, b};
        }
    }
    return m;
}

int load_obj(const char *path, const hrt_load_options &o, hrt_scene_file &f) {
    std::ifstream in(path);
    if (!in) return fail(std::string("could not open ") + path);
    std::string dir(path);
    const size_t slash = dir.find_last_of('/');
    dir = slash == std::string::npos ? std::string() : dir.substr(0, slash + 1);
    std::vector<V3> v;
    float zmin = 100000.f, zmax = -100000.f;
    std::map<std::string, std::vector<std::vector<long long>>> faces;  // by material name (sorted, as the reference)
    std::map<std::string, std::vector<float>> mtl;
    std::string cur = "none", line;
    size_t lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        std::istringstream ls(line);
        std::string w;
        if (!(ls >> w) || w[0] == '#') continue;
        if (w == "v") {
            V3 q{0.f, 0.f, 0.f};
            ls >> q.x >> q.y >> q.z;
            v.push_back(q);
            zmin = std::fmin(zmin, q.z);
            zmax = std::fmax(zmax, q.z);
        } else if (w == "usemtl") {
            std::getline(ls, cur);
            cur = trim(cur);
        } else if (w == "mtllib") {
            std::string file;
            std::getline(ls, file);
            file = trim(file);
            mtl = load_mtl(!file.empty() && file[0] == '/' ? file : dir + file);
        } else if (w == "f") {
            std::vector<long long> fc;
            std::string tok;
            while (ls >> tok) {
                const size_t cut = tok.find('/');
                const std::string head = tok.substr(0, cut);
                char *end = nullptr;
                long long idx = std::strtoll(head.c_str(), &end, 10);
                if (head.empty() || *end != '\0') return fail("OBJ face on line " + std::to_string(lineno) + " has an invalid index");
                if (idx < 0) idx = (long long)v.size() + 1 + idx;  // relative index
                if (idx <= 0 || (size_t)idx > v.size())
                    return fail("OBJ face vertex index " + std::to_string(idx) + " on line " + std::to_string(lineno) +
                                " is out of range 1-" + std::to_string(v.size()));
                fc.push_back(idx);
            }
            faces[cur].push_back(fc);
        }
    }
    float scl = 1.f;
    if (o.height > 0.f) scl = (zmax - zmin > 1e-6f) ? o.height / (zmax - zmin) : o.height;
    const float c90 = std::cos(0.5f * 3.14159265358979323846f), s90 = std::sin(0.5f * 3.14159265358979323846f);
    auto place = [&](V3 q) {
        if (o.up_axis == 1) q = V3{q.x, c90 * q.y - s90 * q.z, s90 * q.y + c90 * q.z};  // YUP: about x by pi/2
        q = rotate_point(q, o.rotation[0], o.rotation[1]);
        return V3{o.origin[0] + q.x * scl, o.origin[1] + q.y * scl, o.origin[2] + q.z * scl};
    };
    for (auto &kv : faces) {
        const float *rgb = o.default_color;
        auto it = mtl.find(kv.first);
        if (it != mtl.end()) rgb = it->second.data();
        for (auto &fc : kv.second) {
            for (size_t t = 2; t < fc.size(); ++t) {
                const V3 a0 = v[fc[0] - 1], b0 = v[fc[t - 1] - 1], c0 = v[fc[t] - 1];
                if (mag(sub(a0, b0)) == 0.f || mag(sub(a0, c0)) == 0.f || mag(sub(b0, c0)) == 0.f) continue;
                const V3 a = place(a0), b = place(b0), c = place(c0);
                if (!(tri_area(a, b, c) > 1e-8f)) continue;
                add_triangle(f, a, b, c, rgb);
            }
        }
    }
    return HRT_OK;
}

// ------------------------------------------------------------------ XML --
// A minimal reader for the Helios XML layout: <helios> holding primitive elements whose
// children are simple text elements (<transform>, <vertices>, <data_float label="..">).
struct XNode {
    std::string tag, text;
    std::map<std::string, std::string> attr;
    std::vector<XNode> kids;
};

struct XParser {
    const std::string &s;
    size_t i = 0;
    std::string err;
    explicit XParser(const std::string &src) : s(src) {}
    void skip_misc() {
        for (;;) {
            while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
            if (s.compare(i, 4, "<!--") == 0) {
                const size_t e = s.find("-->", i + 4);
                i = e == std::string::npos ? s.size() : e + 3;
            } else if (s.compare(i, 2, "<?") == 0) {
                const size_t e = s.find("?>", i + 2);
                i = e == std::string::npos ? s.size() : e + 2;
            } else {
                return;
            }
        }
    }
    bool node(XNode &n, int depth) {
        if (depth > 64) return err = "XML nested too deeply", false;
        skip_misc();
        if (i >= s.size() || s[i] != '<') return err = "expected an element", false;
        ++i;
        size_t b = i;
        while (i < s.size() && !std::isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') ++i;
        n.tag = s.substr(b, i - b);
        for (;;) {
            while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
            if (i >= s.size()) return err = "unterminated tag <" + n.tag + ">", false;
            if (s[i] == '/') {
                if (s.compare(i, 2, "/>") != 0) return err = "bad tag end", false;
                i += 2;
                return true;
            }
            if (s[i] == '>') {
                ++i;
                break;
            }
            b = i;
            while (i < s.size() && s[i] != '=' && !std::isspace((unsigned char)s[i])) ++i;
            const std::string key = s.substr(b, i - b);
            while (i < s.size() && s[i] != '"' && s[i] != '\'') ++i;
            if (i >= s.size()) return err = "bad attribute", false;
            const char q = s[i++];
            b = i;
            while (i < s.size() && s[i] != q) ++i;
            if (i >= s.size()) return err = "bad attribute", false;
            n.attr[key] = s.substr(b, i - b);
            ++i;
        }
        for (;;) {
            b = i;
            while (i < s.size() && s[i] != '<') ++i;
            n.text += s.substr(b, i - b);
            if (i >= s.size()) return err = "element <" + n.tag + "> is not closed", false;
            if (s.compare(i, 4, "<!--") == 0) {
                const size_t e = s.find("-->", i + 4);
                i = e == std::string::npos ? s.size() : e + 3;
                continue;
            }
            if (s.compare(i, 2, "</") == 0) {
                const size_t e = s.find('>', i);
                if (e == std::string::npos || trim(s.substr(i + 2, e - i - 2)) != n.tag)
                    return err = "mismatched closing tag for <" + n.tag + ">", false;
                i = e + 1;
                return true;
            }
            XNode k;
            if (!node(k, depth + 1)) return false;
            n.kids.push_back(std::move(k));
        }
    }
};

const XNode *child(const XNode &n, const char *tag) {
    for (auto &k : n.kids)
        if (k.tag == tag) return &k;
    return nullptr;
}

bool floats(const std::string &t, std::vector<float> &out) {
    std::istringstream ss(t);
    std::string tok;
    out.clear();
    while (ss >> tok) {
        float v;
        if (!parse_float(tok, &v)) return false;
        out.push_back(v);
    }
    return true;
}

int load_xml(const char *path, hrt_scene_file &f) {
    std::ifstream in(path);
    if (!in) return fail(std::string("could not open ") + path);
    std::stringstream buf;
    buf << in.rdbuf();
    const std::string src = buf.str();
    XParser p(src);
    XNode root;
    if (!p.node(root, 0)) return fail("XML " + std::string(path) + ": " + p.err);
    if (root.tag != "helios") return fail("XML file must have tag '<helios> ... </helios>' bounding all other tags");
    // element order of Context::loadXML: patches, triangles, voxels, disks
    const char *tags[4] = {"patch", "triangle", "voxel", "disk"};
    const uint32_t types[4] = {0u, 1u, 4u, 2u};
    std::vector<std::map<std::string, double>> pdata;
    for (int e = 0; e < 4; ++e) {
        for (const XNode &n : root.kids) {
            if (n.tag != tags[e]) continue;
            std::vector<float> vals;
            float T[16];
            const XNode *tr = child(n, "transform");
            const XNode *vx = child(n, "vertices");
            if (tr && !trim(tr->text).empty()) {
                if (!floats(tr->text, vals)) return fail(std::string("<") + tags[e] + "> <transform> contains invalid data");
                if (vals.size() != 16) return fail(std::string("<") + tags[e] + "> <transform> needs 16 values");
                std::memcpy(T, vals.data(), sizeof T);
            } else if (e == 1 && vx) {
                if (!floats(vx->text, vals) || vals.size() != 9) return fail("<triangle> <vertices> needs 9 values");
                triangle_transform(V3{vals[0], vals[1], vals[2]}, V3{vals[3], vals[4], vals[5]},
                                   V3{vals[6], vals[7], vals[8]}, T);
            } else {
                return fail(std::string("<") + tags[e] + "> has no <transform>");
            }
            f.T.insert(f.T.end(), T, T + 16);
            f.type.push_back(types[e]);
            std::vector<float> rgb = {0.f, 0.f, 1.f};
            const XNode *cn = child(n, "color");
            if (cn) {
                std::vector<float> c;
                if (floats(cn->text, c) && c.size() >= 3) rgb.assign(c.begin(), c.begin() + 3);
            }
            f.color.insert(f.color.end(), rgb.begin(), rgb.end());
            std::map<std::string, double> d;
            for (const XNode &k : n.kids) {
                if (k.tag != "data_float" && k.tag != "data_double" && k.tag != "data_int" && k.tag != "data_uint") continue;
                auto lab = k.attr.find("label");
                if (lab == k.attr.end()) continue;
                std::istringstream ss(k.text);
                double x;
                if (!(ss >> x)) return fail("primitive data <" + k.tag + "> with label " + lab->second + " contained invalid data");
                d[lab->second] = x;
            }
            auto ts = d.find("twosided_flag");
            f.twosided.push_back(ts == d.end() ? (int8_t)1 : (int8_t)ts->second);
            pdata.push_back(std::move(d));
        }
    }
    const size_t n = f.type.size();
    for (size_t k = 0; k < n; ++k)
        for (auto &kv : pdata[k]) {
            auto &col = f.data[kv.first];
            if (col.empty()) col.assign(n, std::nan(""));
            col[k] = kv.second;
        }
    return HRT_OK;
}

std::string lower_ext(const char *path) {
    std::string p(path);
    const size_t d = p.find_last_of('.');
    std::string e = d == std::string::npos ? "" : p.substr(d);
    for (auto &c : e) c = (char)std::tolower((unsigned char)c);
    return e;
}

}  // namespace

extern "C" {

int hrt_scene_load(const char *path, const hrt_load_options *opt, hrt_scene_file **out) {
    if (!path || !out) return fail("null argument");
    *out = nullptr;
    hrt_load_options o{};
    o.up_axis = 2;
    o.default_color[2] = 1.f;
    if (opt) o = *opt;
    if (o.up_axis < 0 || o.up_axis > 2) return fail("up axis must be 0 (XUP), 1 (YUP) or 2 (ZUP)");
    auto *f = new hrt_scene_file();
    const std::string ext = lower_ext(path);
    int r;
    if (ext == ".ply") r = load_ply(path, o, *f);
    else if (ext == ".obj") r = load_obj(path, o, *f);
    else if (ext == ".xml") r = load_xml(path, *f);
    else r = fail(std::string("file ") + path + " is not PLY, OBJ or XML");
    if (r) {
        delete f;
        return r;
    }
    *out = f;
    return HRT_OK;
}

const char *hrt_scene_last_error(void) { return g_err.c_str(); }

int64_t hrt_scene_count(const hrt_scene_file *f) { return f ? (int64_t)f->type.size() : 0; }

int hrt_scene_arrays(const hrt_scene_file *f, float *transform, uint32_t *type, int8_t *twosided, float *color) {
    if (!f) return fail("null scene");
    if (transform) std::memcpy(transform, f->T.data(), f->T.size() * sizeof(float));
    if (type) std::memcpy(type, f->type.data(), f->type.size() * sizeof(uint32_t));
    if (twosided) std::memcpy(twosided, f->twosided.data(), f->twosided.size());
    if (color) std::memcpy(color, f->color.data(), f->color.size() * sizeof(float));
    return HRT_OK;
}

size_t hrt_scene_data_labels(const hrt_scene_file *f, char *buf, size_t len) {
    std::string all;
    if (f)
        for (auto &kv : f->data) all += kv.first + "\n";
    if (buf && len > 0) {
        const size_t k = all.size() < len - 1 ? all.size() : len - 1;
        std::memcpy(buf, all.data(), k);
        buf[k] = '\0';
    }
    return all.size() + 1;
}

int hrt_scene_data(const hrt_scene_file *f, const char *label, double *values) {
    if (!f || !label || !values) return fail("null argument");
    auto it = f->data.find(label);
    if (it == f->data.end()) return fail(std::string("no primitive data ") + label);
    std::memcpy(values, it->second.data(), it->second.size() * sizeof(double));
    return HRT_OK;
}

void hrt_scene_free(hrt_scene_file *f) { delete f; }

}  // extern "C"
