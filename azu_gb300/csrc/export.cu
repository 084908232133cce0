// Mesh export formats downstream of the mesher (host code, no GPU work): the
// reference's PLY writer (src/export/PLYExporter.cpp, binary little endian and
// ASCII from one schema) and GLB writer (src/export/GLBExporter.cpp: vertex
// weld by exact position, glTF axes (x, -y, -z), unit normals with a fixed
// fallback, sRGB bytes decoded to linear RGBA floats, 4-byte aligned
// [positions | normals | colours | indices] buffer). Both validate the mesh
// first with MeshData::validate's rules and order (include/meshing/MeshData.h:
// 49-95); a rejected mesh creates no file, and a failed write removes it.
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "azu_internal.h"

namespace azu {
namespace {

struct MeshIn {
    const float* pos;
    size_t nv;
    const float* nrm;
    size_t nn;  // vertices with a normal (0 or nv)
    const uint8_t* col;
    size_t nc;  // colour bytes (0 or 3 nv)
    const uint32_t* idx;
    size_t ni;
};

bool finite3(const float* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

// MeshData::validate (MeshData.h:49-95): the first violated invariant, in order.
bool validate(const MeshIn& m, std::string& why) {
    if (m.nv == 0) { why = "positions is empty"; return false; }
    if (m.ni == 0) { why = "indices is empty while positions.size()=" + std::to_string(m.nv); return false; }
    if (m.ni % 3 != 0) { why = "indices.size()=" + std::to_string(m.ni) + " is not a multiple of 3"; return false; }
    for (size_t i = 0; i < m.ni; ++i)
        if (m.idx[i] >= m.nv) {
            why = "indices[" + std::to_string(i) + "]=" + std::to_string(m.idx[i]) +
                  " is out of range for positions.size()=" + std::to_string(m.nv);
            return false;
        }
    for (size_t i = 0; i < m.nv; ++i)
        if (!finite3(m.pos + 3 * i)) { why = "positions[" + std::to_string(i) + "] has a non-finite component"; return false; }
    if (m.nn != 0 && m.nn != m.nv) {
        why = "normals.size()=" + std::to_string(m.nn) + " is neither 0 nor positions.size()=" + std::to_string(m.nv);
        return false;
    }
    for (size_t i = 0; i < m.nn; ++i)
        if (!finite3(m.nrm + 3 * i)) { why = "normals[" + std::to_string(i) + "] has a non-finite component"; return false; }
    if (m.nc != 0 && (m.nc % 3 != 0 || m.nc / 3 != m.nv)) {
        why = "colors.size()=" + std::to_string(m.nc) + " is neither 0 nor 3 * positions.size()";
        return false;
    }
    return true;
}

void put_u32(std::string& o, uint32_t v) {
    for (int k = 0; k < 4; ++k) o.push_back(static_cast<char>((v >> (8 * k)) & 0xFFu));
}
void put_f32(std::string& o, float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    put_u32(o, u);
}
std::string fmt9(float v) {
    char b[32];
    std::snprintf(b, sizeof(b), "%.9g", static_cast<double>(v));
    return b;
}

// Whole file in memory, one write, flush, close; a failure after the open
// removes what was written.
int write_file(const char* path, const std::string& bytes) {
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        set_error("cannot open %s: %s", path, std::strerror(errno));
        return AZU_E_INVALID;
    }
    const size_t w = std::fwrite(bytes.data(), 1, bytes.size(), f);
    const bool ok = w == bytes.size() && std::fflush(f) == 0;
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) {
        std::remove(path);
        set_error("write error on %s", path);
        return AZU_E_INVALID;
    }
    return AZU_OK;
}

// PLY (PLYExporter.cpp): one header for both formats, one record path.
std::string ply_bytes(const MeshIn& m, bool binary) {
    const bool has_n = m.nn == m.nv, has_c = m.nc == 3 * m.nv;
    const size_t nf = m.ni / 3;
    std::string h = "ply\nformat ";
    h += binary ? "binary_little_endian" : "ascii";
    h += " 1.0\ncomment KinectFusionQt export\nelement vertex " + std::to_string(m.nv) + "\n";
    h += "property float x\nproperty float y\nproperty float z\n";
    if (has_n) h += "property float nx\nproperty float ny\nproperty float nz\n";
    if (has_c) h += "property uchar red\nproperty uchar green\nproperty uchar blue\n";
    h += "element face " + std::to_string(nf) + "\nproperty list uchar int vertex_indices\nend_header\n";
    std::string b;
    if (binary) {
        b.reserve(m.nv * (12 + (has_n ? 12 : 0) + (has_c ? 3 : 0)) + nf * 13);
        for (size_t i = 0; i < m.nv; ++i) {
            for (int k = 0; k < 3; ++k) put_f32(b, m.pos[3 * i + k]);
            if (has_n) for (int k = 0; k < 3; ++k) put_f32(b, m.nrm[3 * i + k]);
            if (has_c) for (int k = 0; k < 3; ++k) b.push_back(static_cast<char>(m.col[3 * i + k]));
        }
        for (size_t t = 0; t < nf; ++t) {
            b.push_back(static_cast<char>(3));
            for (int k = 0; k < 3; ++k) put_u32(b, m.idx[3 * t + k]);
        }
    } else {
        for (size_t i = 0; i < m.nv; ++i) {
            std::string line;
            for (int k = 0; k < 3; ++k) { if (k) line += ' '; line += fmt9(m.pos[3 * i + k]); }
            if (has_n) for (int k = 0; k < 3; ++k) { line += ' '; line += fmt9(m.nrm[3 * i + k]); }
            if (has_c) for (int k = 0; k < 3; ++k) { line += ' '; line += std::to_string(static_cast<int>(m.col[3 * i + k])); }
            b += line;
            b += '\n';
        }
        for (size_t t = 0; t < nf; ++t) {
            b += "3";
            for (int k = 0; k < 3; ++k) { b += ' '; b += std::to_string(m.idx[3 * t + k]); }
            b += '\n';
        }
    }
    return h + b;
}

// sRGB decode of ColorConversion.h (checked; the bytes are in range).
float srgb_to_linear(uint8_t c8) {
    const float s = static_cast<float>(c8) / 255.0f;
    const double c = static_cast<double>(s);
    return static_cast<float>(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
}

struct Key {
    float x, y, z;
    bool operator==(const Key& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct KeyHash {
    size_t operator()(const Key& k) const {
        // +0 and -0 compare equal, so they must hash equally
        auto h = [](float f) { return std::hash<float>{}(f == 0.0f ? 0.0f : f); };
        return h(k.x) ^ (h(k.y) << 1) ^ (h(k.z) << 2);
    }
};

// A glTF number: the shortest decimal that reads back as the same double,
// with "0.0" / "-0.0" for zeros and a ".0" on integral values, in fixed
// notation for decimal points within 15 digits of the first digit and
// exponent form (e+XX, e-XX) otherwise. The reference's writer prints the
// same doubles through its JSON library; at an exact decimal tie of the last
// digit, and in rare cases where that library's digit generation does not
// find the shortest form, its decimal differs from this one but reads back
// as the same double, so the documents are equal value for value.
std::string num(double v) {
    if (v == 0.0) return std::signbit(v) ? "-0.0" : "0.0";
    if (!std::isfinite(v)) return "null";
    char b[64];
    for (int p = 1; p <= 17; ++p) {  // fewest significant digits that read back exactly
        std::snprintf(b, sizeof(b), "%.*e", p - 1, v);
        if (std::strtod(b, nullptr) == v) break;
    }
    std::string s(b);
    const bool neg = s[0] == '-';
    if (neg) s.erase(0, 1);
    const size_t epos = s.find('e');
    const int ex = std::atoi(s.c_str() + epos + 1);
    std::string dig = s.substr(0, 1) + (epos > 2 ? s.substr(2, epos - 2) : std::string());
    while (dig.size() > 1 && dig.back() == '0') dig.pop_back();
    const int k = static_cast<int>(dig.size()), n = ex + 1;  // v = 0.dig x 10^n
    std::string out = neg ? "-" : "";
    if (k <= n && n <= 15) {
        out += dig + std::string(static_cast<size_t>(n - k), '0') + ".0";
    } else if (0 < n && n <= 15) {
        out += dig.substr(0, static_cast<size_t>(n)) + "." + dig.substr(static_cast<size_t>(n));
    } else if (-4 < n && n <= 0) {
        out += "0." + std::string(static_cast<size_t>(-n), '0') + dig;
    } else {
        out += dig.substr(0, 1);
        if (k > 1) out += "." + dig.substr(1);
        int e = n - 1;
        out += e < 0 ? "e-" : "e+";
        e = std::abs(e);
        if (e < 10) out += "0";
        out += std::to_string(e);
    }
    return out;
}

// GLB (GLBExporter.cpp): weld, buffer, glTF JSON and the binary container.
int glb_bytes(const MeshIn& in, std::string& out) {
    const bool in_n = in.nn == in.nv, in_c = in.nc == 3 * in.nv;
    std::unordered_map<Key, uint32_t, KeyHash> map;
    std::vector<float> pos, nrm;
    std::vector<uint8_t> col;
    std::vector<uint32_t> idx;
    idx.reserve(in.ni);
    for (size_t i = 0; i < in.ni; ++i) {
        const uint32_t o = in.idx[i];
        const Key k{in.pos[3 * o], in.pos[3 * o + 1], in.pos[3 * o + 2]};
        auto it = map.find(k);
        if (it != map.end()) {
            idx.push_back(it->second);
            continue;
        }
        const uint32_t n = static_cast<uint32_t>(pos.size() / 3);
        map.emplace(k, n);
        for (int c = 0; c < 3; ++c) pos.push_back(in.pos[3 * o + c]);
        if (in_n) for (int c = 0; c < 3; ++c) nrm.push_back(in.nrm[3 * o + c]);
        if (in_c) for (int c = 0; c < 3; ++c) col.push_back(in.col[3 * o + c]);
        idx.push_back(n);
    }
    const size_t nv = pos.size() / 3, ni = idx.size();
    std::string buf;
    auto pad4 = [&]() { while (buf.size() % 4) buf.push_back('\0'); };
    // positions in glTF axes, bounds seeded from the first vertex
    const size_t pos_off = buf.size();
    float bmin[3], bmax[3];
    for (size_t i = 0; i < nv; ++i) {
        const float g[3] = {pos[3 * i], -pos[3 * i + 1], -pos[3 * i + 2]};
        for (int c = 0; c < 3; ++c) {
            put_f32(buf, g[c]);
            // Eigen cwiseMin / cwiseMax: (b < a) ? b : a and (a < b) ? b : a
            if (i == 0) { bmin[c] = bmax[c] = g[c]; }
            else { bmin[c] = (g[c] < bmin[c]) ? g[c] : bmin[c]; bmax[c] = (bmax[c] < g[c]) ? g[c] : bmax[c]; }
        }
    }
    pad4();
    const size_t pos_len = buf.size() - pos_off;
    size_t nrm_off = 0, nrm_len = 0, col_off = 0, col_len = 0;
    if (in_n) {
        nrm_off = buf.size();
        for (size_t i = 0; i < nv; ++i) {
            const float* n = &nrm[3 * i];
            const float len = std::sqrt(n[0] * n[0] + (n[1] * n[1] + n[2] * n[2]));
            float g[3];
            if (!std::isfinite(len) || len < 1e-6f) { g[0] = 0.0f; g[1] = -0.0f; g[2] = -1.0f; }
            else { g[0] = n[0] / len; g[1] = -n[1] / len; g[2] = -n[2] / len; }
            for (int c = 0; c < 3; ++c) put_f32(buf, g[c]);
        }
        pad4();
        nrm_len = buf.size() - nrm_off;
    }
    if (in_c) {
        col_off = buf.size();
        for (size_t i = 0; i < nv; ++i) {
            for (int c = 0; c < 3; ++c) put_f32(buf, srgb_to_linear(col[3 * i + c]));
            put_f32(buf, 1.0f);
        }
        pad4();
        col_len = buf.size() - col_off;
    }
    const size_t idx_off = buf.size();
    for (uint32_t v : idx) put_u32(buf, v);
    pad4();
    const size_t idx_len = buf.size() - idx_off;

    // glTF JSON (the reference's model: one buffer, views, accessors, mesh,
    // material, node, scene)
    std::string views, accs, attrs;
    int nview = 0;
    auto view = [&](size_t off, size_t len, int target) {
        if (nview) views += ",";
        // glTF defaults (offset 0) are left out, as the reference's writer leaves them out
        views += "{\"buffer\":0,\"byteLength\":" + std::to_string(len) +
                 (off ? ",\"byteOffset\":" + std::to_string(off) : std::string()) +
                 ",\"target\":" + std::to_string(target) + "}";
        return nview++;
    };
    int nacc = 0;
    auto acc = [&](int v, int ctype, const char* type, size_t count, const std::string& extra) {
        if (nacc) accs += ",";
        accs += "{\"bufferView\":" + std::to_string(v) + ",\"componentType\":" +
                std::to_string(ctype) + ",\"count\":" + std::to_string(count) + extra + ",\"type\":\"" + type + "\"}";
        return nacc++;
    };
    const std::string mm = ",\"max\":[" + num(bmax[0]) + "," + num(bmax[1]) + "," + num(bmax[2]) + "],\"min\":[" +
                           num(bmin[0]) + "," + num(bmin[1]) + "," + num(bmin[2]) + "]";
    const int a_pos = acc(view(pos_off, pos_len, 34962), 5126, "VEC3", nv, mm);
    int a_nrm = -1, a_col = -1;
    if (in_n) a_nrm = acc(view(nrm_off, nrm_len, 34962), 5126, "VEC3", nv, "");
    if (in_c) a_col = acc(view(col_off, col_len, 34962), 5126, "VEC4", nv, "");
    const int a_idx = acc(view(idx_off, idx_len, 34963), 5125, "SCALAR", ni, "");
    if (a_col >= 0) attrs += "\"COLOR_0\":" + std::to_string(a_col) + ",";
    if (a_nrm >= 0) attrs += "\"NORMAL\":" + std::to_string(a_nrm) + ",";
    attrs += "\"POSITION\":" + std::to_string(a_pos);
    // a white base colour is the glTF default and is left out
    const std::string base = in_c ? std::string() : "\"baseColorFactor\":[0.72,0.78,0.85,1.0],";
    std::string json = "{\"accessors\":[" + accs + "],\"asset\":{\"generator\":\"KinectFusionQt\",\"version\":\"2.0\"}," +
                       "\"bufferViews\":[" + views + "],\"buffers\":[{\"byteLength\":" + std::to_string(buf.size()) +
                       "}],\"materials\":[{\"name\":\"ScanMaterial\",\"pbrMetallicRoughness\":{" + base +
                       "\"metallicFactor\":0.0,\"roughnessFactor\":0.8}}],\"meshes\":[{\"name\":\"KinectScan\"," +
                       "\"primitives\":[{\"attributes\":{" + attrs + "},\"indices\":" + std::to_string(a_idx) +
                       ",\"material\":0,\"mode\":4}]}],\"nodes\":[{\"mesh\":0}],\"scene\":0,\"scenes\":[{\"nodes\":[0]}]}";
    while (json.size() % 4) json.push_back(' ');
    out.clear();
    out += "glTF";
    put_u32(out, 2);
    put_u32(out, static_cast<uint32_t>(12 + 8 + json.size() + 8 + buf.size()));
    put_u32(out, static_cast<uint32_t>(json.size()));
    out += "JSON";
    out += json;
    put_u32(out, static_cast<uint32_t>(buf.size()));
    out += std::string("BIN\0", 4);
    out += buf;
    return AZU_OK;
}

int check_mesh(const MeshIn& m) {
    std::string why;
    if (!validate(m, why)) {
        set_error("invalid mesh, nothing written: %s", why.c_str());
        return AZU_E_INVALID;
    }
    return AZU_OK;
}

}  // namespace
}  // namespace azu

using namespace azu;

extern "C" int azu_mesh_write_ply(const char* path, int binary, const float* positions, int64_t n_vertices,
                                  const float* normals, int64_t n_normals, const uint8_t* colors, int64_t n_color_bytes,
                                  const uint32_t* indices, int64_t n_indices) {
    AZU_CHECK_ARG(path != nullptr && n_vertices >= 0 && n_normals >= 0 && n_color_bytes >= 0 && n_indices >= 0,
                  "bad argument");
    const MeshIn m{positions, static_cast<size_t>(n_vertices), normals, static_cast<size_t>(normals ? n_normals : 0),
                   colors, static_cast<size_t>(colors ? n_color_bytes : 0), indices, static_cast<size_t>(n_indices)};
    if (int rc = check_mesh(m)) return rc;
    return write_file(path, ply_bytes(m, binary != 0));
}

extern "C" int azu_mesh_write_glb(const char* path, const float* positions, int64_t n_vertices, const float* normals,
                                  int64_t n_normals, const uint8_t* colors, int64_t n_color_bytes,
                                  const uint32_t* indices, int64_t n_indices) {
    AZU_CHECK_ARG(path != nullptr && n_vertices >= 0 && n_normals >= 0 && n_color_bytes >= 0 && n_indices >= 0,
                  "bad argument");
    const MeshIn m{positions, static_cast<size_t>(n_vertices), normals, static_cast<size_t>(normals ? n_normals : 0),
                   colors, static_cast<size_t>(colors ? n_color_bytes : 0), indices, static_cast<size_t>(n_indices)};
    if (int rc = check_mesh(m)) return rc;
    std::string bytes;
    if (int rc = glb_bytes(m, bytes)) return rc;
    return write_file(path, bytes);
}
