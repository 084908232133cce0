// Oracle (test infrastructure only): CPU restatement of the reference's marching
// cubes with the exact-edge weld (src/meshing/MarchingCubes.cpp:81-382).
#include "orc_api.h"
#include "orc_math.h"
#include "orc_mc_tables.h"

#include <unordered_map>
#include <vector>

using namespace orc;

namespace {

constexpr float kEmptyTsdf = 1.0f;
constexpr float kEmptyColor = 128.0f / 255.0f;
constexpr float kWeightEpsilon = 0.001f;    // MarchingCubes.cpp:62
constexpr float kGradientEpsilon = 1e-6f;   // :63
constexpr float kInterpEpsilon = 1e-6f;     // :64

const int kCornerOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                              {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};  // :43-46
const int kEdgeCorners[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                 {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};  // :49-53

int edgeMask(int ci) {
    int m = 0;
    for (int e = 0; e < 12; ++e)
        if (((ci >> kEdgeCorners[e][0]) & 1) != ((ci >> kEdgeCorners[e][1]) & 1)) m |= 1 << e;
    return m;
}

struct Corner { float value; bool supported; };

struct Vol {
    const orc_tsdf_params* p;
    const float* tsdf;
    const float* weight;
    const float* color;
    size_t idx(int x, int y, int z) const {
        const size_t r = static_cast<size_t>(p->res);
        return (static_cast<size_t>(z) * r + static_cast<size_t>(y)) * r + static_cast<size_t>(x);
    }
    // sampleCorner (:81-85).
    Corner corner(int x, int y, int z) const {
        const size_t i = idx(x, y, z);
        if (!std::isfinite(tsdf[i]) || weight[i] <= kWeightEpsilon) return {kEmptyTsdf, false};
        return {tsdf[i], true};
    }
    float col(size_t i, int k) const { return color ? color[3 * i + k] : kEmptyColor; }
    V3 toWorld(int x, int y, int z) const {
        return V3(p->origin[0], p->origin[1], p->origin[2]) +
               V3(float(x), float(y), float(z)) * p->voxel_size;
    }
};

V3 invalidNormal() {
    const float n = std::numeric_limits<float>::quiet_NaN();
    return V3(n, n, n);
}

// MarchingCubes::voxelNormal (:136-172).
V3 voxelNormal(const Vol& v, int x, int y, int z) {
    const int R = v.p->res;
    auto usable = [&](int xi, int yi, int zi, float& out) {
        if (xi < 0 || xi >= R || yi < 0 || yi >= R || zi < 0 || zi >= R) return false;
        const Corner s = v.corner(xi, yi, zi);
        if (!s.supported) return false;
        out = s.value;
        return true;
    };
    float self = 0.0f;
    if (!usable(x, y, z, self)) return invalidNormal();
    V3 grad(0, 0, 0);
    for (int axis = 0; axis < 3; ++axis) {
        const int ox = axis == 0, oy = axis == 1, oz = axis == 2;
        float hi = 0.0f, lo = 0.0f;
        const bool have_hi = usable(x + ox, y + oy, z + oz, hi);
        const bool have_lo = usable(x - ox, y - oy, z - oz, lo);
        if (have_hi && have_lo) grad[axis] = 0.5f * (hi - lo);
        else if (have_hi) grad[axis] = hi - self;
        else if (have_lo) grad[axis] = self - lo;
        else grad[axis] = 0.0f;
    }
    if (!finite3(grad)) return invalidNormal();
    const float len = norm(grad);
    if (!std::isfinite(len) || len <= kGradientEpsilon) return invalidNormal();
    return grad / len;
}

struct Crossing { V3 pos; float t; bool ok; };

// MarchingCubes::crossingFromLower (:115-134).
Crossing crossingFromLower(V3 pl, float vl, V3 pu, float vu) {
    if (!std::isfinite(vl) || !std::isfinite(vu) || !finite3(pl) || !finite3(pu))
        return {invalidNormal(), 0.0f, false};
    if (std::fabs(vl) < kInterpEpsilon) return {pl, 0.0f, true};
    if (std::fabs(vu) < kInterpEpsilon) return {pu, 1.0f, true};
    const float diff = vl - vu;
    if (!std::isfinite(diff) || std::fabs(diff) < kInterpEpsilon) return {pl, 0.0f, true};
    const float t = std::max(0.0f, std::min(1.0f, vl / diff));
    return {pl + t * (pu - pl), t, true};
}

struct Key {
    int x, y, z, axis;
    bool operator==(const Key& o) const { return x == o.x && y == o.y && z == o.z && axis == o.axis; }
};
struct KeyHash {
    size_t operator()(const Key& k) const {
        uint64_t h = static_cast<uint32_t>(k.x);
        h = h * 0x100000001b3ull ^ static_cast<uint32_t>(k.y);
        h = h * 0x100000001b3ull ^ static_cast<uint32_t>(k.z);
        h = h * 0x100000001b3ull ^ static_cast<uint32_t>(k.axis);
        return static_cast<size_t>(h * 0x9E3779B97F4A7C15ull);
    }
};

struct Slice {
    std::vector<V3> pos, nrm;
    std::vector<uint8_t> col;
    std::vector<Key> key;
};

}  // namespace

extern "C" void orc_mc_extract(const orc_tsdf_params* p, const float* tsdf, const float* weight,
                               const float* color, int64_t max_triangles, orc_mesh_info* info,
                               float* positions, float* normals, uint8_t* colors, uint32_t* indices) {
    const Vol vol{p, tsdf, weight, color};
    const int RES = p->res;
    info->n_vertices = 0;
    info->n_indices = 0;
    info->truncated = 0;
    if (RES < 2) return;
    std::vector<Slice> slices(RES - 1);

#pragma omp parallel for schedule(dynamic, 4)
    for (int z = 0; z < RES - 1; ++z) {
        Slice& sl = slices[z];
        for (int y = 0; y < RES - 1; ++y) {
            for (int x = 0; x < RES - 1; ++x) {
                Corner corner[8];
                size_t cidx[8];
                for (int c = 0; c < 8; ++c) {
                    cidx[c] = vol.idx(x + kCornerOff[c][0], y + kCornerOff[c][1], z + kCornerOff[c][2]);
                    corner[c] = vol.corner(x + kCornerOff[c][0], y + kCornerOff[c][1], z + kCornerOff[c][2]);
                }
                int ci = 0;
                for (int c = 0; c < 8; ++c)
                    if (corner[c].value < 0.0f) ci |= 1 << c;
                const int mask = edgeMask(ci);
                if (mask == 0) continue;
                V3 cpos[8];
                for (int c = 0; c < 8; ++c)
                    cpos[c] = vol.toWorld(x + kCornerOff[c][0], y + kCornerOff[c][1], z + kCornerOff[c][2]);
                V3 cn[8];
                bool cn_done[8] = {false, false, false, false, false, false, false, false};
                auto cornerNormal = [&](int c) {
                    if (!cn_done[c]) {
                        cn[c] = voxelNormal(vol, x + kCornerOff[c][0], y + kCornerOff[c][1], z + kCornerOff[c][2]);
                        cn_done[c] = true;
                    }
                    return cn[c];
                };
                V3 epos[12], enrm[12];
                uint8_t ecol[12][3];
                Key ekey[12];
                bool eok[12] = {false, false, false, false, false, false, false, false, false, false, false, false};
                for (int e = 0; e < 12; ++e) {
                    if (!(mask & (1 << e))) continue;
                    const int c0 = kEdgeCorners[e][0], c1 = kEdgeCorners[e][1];
                    if (!corner[c0].supported || !corner[c1].supported) continue;
                    const int d0x = x + kCornerOff[c0][0], d0y = y + kCornerOff[c0][1], d0z = z + kCornerOff[c0][2];
                    const int d1x = x + kCornerOff[c1][0], d1y = y + kCornerOff[c1][1], d1z = z + kCornerOff[c1][2];
                    int axis, lo, up;
                    if (d0x != d1x) { axis = 0; lo = d0x <= d1x ? c0 : c1; up = d0x <= d1x ? c1 : c0; }
                    else if (d0y != d1y) { axis = 1; lo = d0y <= d1y ? c0 : c1; up = d0y <= d1y ? c1 : c0; }
                    else { axis = 2; lo = d0z <= d1z ? c0 : c1; up = d0z <= d1z ? c1 : c0; }
                    ekey[e] = Key{x + kCornerOff[lo][0], y + kCornerOff[lo][1], z + kCornerOff[lo][2], axis};
                    const Crossing cr = crossingFromLower(cpos[lo], corner[lo].value, cpos[up], corner[up].value);
                    if (!cr.ok) continue;
                    const V3 nl = cornerNormal(lo), nu = cornerNormal(up);
                    if (!finite3(nl) || !finite3(nu)) continue;
                    const V3 bl = nl + cr.t * (nu - nl);
                    const float blen = norm(bl);
                    if (!std::isfinite(blen) || blen <= kGradientEpsilon) continue;
                    epos[e] = cr.pos;
                    enrm[e] = bl / blen;
                    float cf[3];
                    for (int k = 0; k < 3; ++k)
                        cf[k] = vol.col(cidx[lo], k) + cr.t * (vol.col(cidx[up], k) - vol.col(cidx[lo], k));
                    uint8_t cb[3] = {0, 0, 0};
                    if (!srgbFloatToUint8(cf[0], cb[0]) || !srgbFloatToUint8(cf[1], cb[1]) ||
                        !srgbFloatToUint8(cf[2], cb[2]))
                        continue;
                    ecol[e][0] = cb[0]; ecol[e][1] = cb[1]; ecol[e][2] = cb[2];
                    eok[e] = true;
                }
                const uint64_t row = orc_tables::kTriRows[ci];
                for (int t = 0; ((row >> (4 * t)) & 0xF) != 0xF; t += 3) {
                    const int te[3] = {int((row >> (4 * t)) & 0xF), int((row >> (4 * (t + 1))) & 0xF),
                                       int((row >> (4 * (t + 2))) & 0xF)};
                    if (!eok[te[0]] || !eok[te[1]] || !eok[te[2]]) continue;
                    for (int i = 2; i >= 0; --i) {  // reversed winding (:321-334)
                        const int e = te[i];
                        sl.pos.push_back(epos[e]);
                        sl.nrm.push_back(enrm[e]);
                        sl.col.push_back(ecol[e][0]);
                        sl.col.push_back(ecol[e][1]);
                        sl.col.push_back(ecol[e][2]);
                        sl.key.push_back(ekey[e]);
                    }
                }
            }
        }
    }

    // Serial weld in (z, local emission) order, first occurrence wins (:346-377).
    std::unordered_map<Key, uint32_t, KeyHash> weld;
    int64_t nv = 0, ni = 0, tri = 0;
    bool truncated = false;
    const bool write = positions != nullptr;
    for (int z = 0; z < RES - 1 && !truncated; ++z) {
        const Slice& sl = slices[z];
        for (size_t i = 0; i + 2 < sl.key.size(); i += 3) {
            if (tri >= max_triangles) { truncated = true; break; }
            for (int k = 0; k < 3; ++k) {
                const size_t li = i + k;
                auto it = weld.find(sl.key[li]);
                uint32_t gi;
                if (it != weld.end()) {
                    gi = it->second;
                } else {
                    gi = static_cast<uint32_t>(nv);
                    weld.emplace(sl.key[li], gi);
                    if (write) {
                        positions[3 * nv] = sl.pos[li].x; positions[3 * nv + 1] = sl.pos[li].y; positions[3 * nv + 2] = sl.pos[li].z;
                        normals[3 * nv] = sl.nrm[li].x; normals[3 * nv + 1] = sl.nrm[li].y; normals[3 * nv + 2] = sl.nrm[li].z;
                        colors[3 * nv] = sl.col[3 * li]; colors[3 * nv + 1] = sl.col[3 * li + 1]; colors[3 * nv + 2] = sl.col[3 * li + 2];
                    }
                    ++nv;
                }
                if (write) indices[ni] = gi;
                ++ni;
            }
            ++tri;
        }
    }
    // The reference keeps scanning later slices after a break; the next slice's
    // first triangle trips the same test, so the result is identical.
    info->n_vertices = nv;
    info->n_indices = ni;
    info->truncated = truncated ? 1 : 0;
}
