// Marching cubes with the exact-edge weld on the GPU, behind the azu_mesher_*
// ABI. Semantics: src/meshing/MarchingCubes.cpp:81-382 (corner support rule,
// lower-endpoint crossing, one-sided/central voxel normals, colour blend,
// reversed (2,1,0) winding, 2M-triangle cap at a triangle boundary, weld by
// (lower voxel, axis) keeping the first occurrence in (z, y, x, row) order).
//
//   1. classify  one thread per cube: cube index, per-edge validity, number of
//                triangles whose three edges are valid; uint8 count per cube and
//                one sum per 256-cube block.
//   2. scan      exclusive scan of the block sums -> global triangle offsets.
//   3. emit      per block: local scan of the counts; each cube writes its
//                triangles' vertex slots (3 per triangle, emission order) with
//                the edge key and the vertex payload, up to the cap.
//   4. weld      key -> smallest slot in an open-addressing table (atomicCAS /
//                atomicMin: order-independent result); a slot is a new vertex
//                iff it is its key's smallest slot; a scan of those flags gives
//                vertex ids in first-appearance order; indices and the vertex
//                arrays follow.
// Vertex positions, normals and colours use the CPU path's float expressions in
// its order, so meshes are bit-identical to it.
#include <algorithm>
#include <cstring>

#include <cuda_fp16.h>

#include "azu_internal.h"
#include "kf_math.cuh"
#include "mc_tables.h"

namespace azu {

__constant__ uint64_t c_tri_rows[256];

constexpr int kCubeBlock = 256;
constexpr float kWeightEps = 0.001f, kGradEps = 1e-6f, kInterpEps = 1e-6f;
constexpr float kEmptyTsdf = 1.0f, kEmptyColor = 128.0f / 255.0f;

__constant__ int c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
__constant__ int c_edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                  {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

struct MeshVol {
    const void* vox;
    int half;  // FP16 formats: half tsdf in the low 16 bits, weight word (> 0 iff observed) above
    const float* color;
    int res;
    float vs;
    F3 origin;
    __device__ __forceinline__ size_t idx(int x, int y, int z) const {
        const size_t r = static_cast<size_t>(res);
        return (static_cast<size_t>(z) * r + static_cast<size_t>(y)) * r + static_cast<size_t>(x);
    }
    // sampleCorner (:81-85)
    __device__ __forceinline__ bool corner(int x, int y, int z, float& v) const {
        float2 r;
        if (half) {
            const uint32_t u = __ldg(static_cast<const uint32_t*>(vox) + idx(x, y, z));
            r = make_float2(__half2float(__ushort_as_half(static_cast<unsigned short>(u & 0xFFFFu))),
                            static_cast<float>(u >> 16));
        } else {
            r = __ldg(static_cast<const float2*>(vox) + idx(x, y, z));
        }
        if (!isfinite(r.x) || r.y <= kWeightEps) { v = kEmptyTsdf; return false; }
        v = r.x;
        return true;
    }
    __device__ __forceinline__ float col(size_t i, int k) const { return color ? color[3 * i + k] : kEmptyColor; }
};

__device__ __forceinline__ F3 nan3() {
    const float n = __int_as_float(0x7fffffff);
    return mk3(n, n, n);
}

// voxelNormal (:136-172)
__device__ F3 voxel_normal(const MeshVol& v, int x, int y, int z) {
    const int R = v.res;
    auto usable = [&](int xi, int yi, int zi, float& out) {
        if (xi < 0 || xi >= R || yi < 0 || yi >= R || zi < 0 || zi >= R) return false;
        return v.corner(xi, yi, zi, out);
    };
    float self = 0.0f;
    if (!usable(x, y, z, self)) return nan3();
    float g[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int ox = a == 0, oy = a == 1, oz = a == 2;
        float hi = 0.0f, lo = 0.0f;
        const bool hh = usable(x + ox, y + oy, z + oz, hi);
        const bool hl = usable(x - ox, y - oy, z - oz, lo);
        if (hh && hl) g[a] = fm(0.5f, fs(hi, lo));
        else if (hh) g[a] = fs(hi, self);
        else if (hl) g[a] = fs(self, lo);
        else g[a] = 0.0f;
    }
    const F3 gr = mk3(g[0], g[1], g[2]);
    if (!finite3(gr)) return nan3();
    const float len = norm3(gr);
    if (!isfinite(len) || len <= kGradEps) return nan3();
    return div3(gr, len);
}

struct EdgeOut {
    F3 pos, nrm;
    uint8_t col[3];
    uint64_t key;
};

// All 12 edges of cube (x, y, z): validity bits; payloads when `out` is given.
__device__ int cube_edges(const MeshVol& v, int x, int y, int z, int& cube_idx, EdgeOut* out) {
    float cv[8];
    bool sup[8];
    cube_idx = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        sup[c] = v.corner(x + c_corner[c][0], y + c_corner[c][1], z + c_corner[c][2], cv[c]);
        if (cv[c] < 0.0f) cube_idx |= 1 << c;
    }
    int mask = 0;
#pragma unroll
    for (int e = 0; e < 12; ++e)
        if (((cube_idx >> c_edge[e][0]) & 1) != ((cube_idx >> c_edge[e][1]) & 1)) mask |= 1 << e;
    if (mask == 0) return 0;
    F3 cn[8];
    int cn_done = 0;
    int ok = 0;
    for (int e = 0; e < 12; ++e) {
        if (!(mask & (1 << e))) continue;
        const int c0 = c_edge[e][0], c1 = c_edge[e][1];
        if (!sup[c0] || !sup[c1]) continue;
        // The lower endpoint is the corner with the smaller coordinate on the
        // single axis the edge spans.
        int axis, lo, up;
        if (c_corner[c0][0] != c_corner[c1][0]) axis = 0;
        else if (c_corner[c0][1] != c_corner[c1][1]) axis = 1;
        else axis = 2;
        if (c_corner[c0][axis] <= c_corner[c1][axis]) { lo = c0; up = c1; } else { lo = c1; up = c0; }
        const int lx = x + c_corner[lo][0], ly = y + c_corner[lo][1], lz = z + c_corner[lo][2];
        const int ux = x + c_corner[up][0], uy = y + c_corner[up][1], uz = z + c_corner[up][2];
        const F3 pl = add3(v.origin, mul3(mk3(float(lx), float(ly), float(lz)), v.vs));
        const F3 pu = add3(v.origin, mul3(mk3(float(ux), float(uy), float(uz)), v.vs));
        // crossingFromLower (:115-134)
        const float vl = cv[lo], vu = cv[up];
        if (!isfinite(vl) || !isfinite(vu) || !finite3(pl) || !finite3(pu)) continue;
        F3 pos;
        float t;
        if (fabsf(vl) < kInterpEps) { pos = pl; t = 0.0f; }
        else if (fabsf(vu) < kInterpEps) { pos = pu; t = 1.0f; }
        else {
            const float diff = fs(vl, vu);
            if (!isfinite(diff) || fabsf(diff) < kInterpEps) { pos = pl; t = 0.0f; }
            else {
                const float q = fd(vl, diff);
                const float m1 = q < 1.0f ? q : 1.0f;
                t = 0.0f < m1 ? m1 : 0.0f;
                pos = add3(pl, smul3(t, sub3(pu, pl)));
            }
        }
        if (!(cn_done & (1 << lo))) { cn[lo] = voxel_normal(v, lx, ly, lz); cn_done |= 1 << lo; }
        if (!(cn_done & (1 << up))) { cn[up] = voxel_normal(v, ux, uy, uz); cn_done |= 1 << up; }
        const F3 nl = cn[lo], nu = cn[up];
        if (!finite3(nl) || !finite3(nu)) continue;
        const F3 bl = add3(nl, smul3(t, sub3(nu, nl)));
        const float blen = norm3(bl);
        if (!isfinite(blen) || blen <= kGradEps) continue;
        const size_t il = v.idx(lx, ly, lz), iu = v.idx(ux, uy, uz);
        uint8_t cb[3];
        bool cok = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float a = v.col(il, k), b = v.col(iu, k);
            cok = cok && srgb_to_byte(fa(a, fm(t, fs(b, a))), &cb[k]);
        }
        if (!cok) continue;
        ok |= 1 << e;
        if (out) {
            out[e].pos = pos;
            out[e].nrm = div3(bl, blen);
            out[e].col[0] = cb[0]; out[e].col[1] = cb[1]; out[e].col[2] = cb[2];
            const uint64_t r = static_cast<uint64_t>(v.res);
            out[e].key = (((static_cast<uint64_t>(lz) * r + ly) * r + lx) * 3 + axis) + 1;  // 0 = empty
        }
    }
    return ok;
}

__device__ __forceinline__ int count_tris(int cube_idx, int ok) {
    const uint64_t row = c_tri_rows[cube_idx];
    int n = 0;
    for (int t = 0; ((row >> (4 * t)) & 0xF) != 0xF; t += 3) {
        const int a = (row >> (4 * t)) & 0xF, b = (row >> (4 * (t + 1))) & 0xF, c = (row >> (4 * (t + 2))) & 0xF;
        n += ((ok >> a) & 1) && ((ok >> b) & 1) && ((ok >> c) & 1);
    }
    return n;
}

__device__ __forceinline__ void cube_of(long long i, int cr, int& x, int& y, int& z) {
    x = static_cast<int>(i % cr);
    const long long r = i / cr;
    y = static_cast<int>(r % cr);
    z = static_cast<int>(r / cr);
}

__global__ void __launch_bounds__(kCubeBlock) mc_classify_kernel(MeshVol v, long long ncubes, uint8_t* __restrict__ counts,
                                                                 unsigned* __restrict__ block_sums) {
    const long long i = static_cast<long long>(blockIdx.x) * kCubeBlock + threadIdx.x;
    int n = 0;
    if (i < ncubes) {
        int x, y, z;
        cube_of(i, v.res - 1, x, y, z);
        int ci;
        const int ok = cube_edges(v, x, y, z, ci, nullptr);
        if (ok) n = count_tris(ci, ok);
        counts[i] = static_cast<uint8_t>(n);
    }
    for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(0xffffffffu, n, o);
    __shared__ unsigned s[kCubeBlock / 32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < kCubeBlock / 32; ++w) t += s[w];
        block_sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kCubeBlock) mc_emit_kernel(MeshVol v, long long ncubes, const uint8_t* __restrict__ counts,
                                                             const unsigned* __restrict__ block_offsets, unsigned cap,
                                                             uint64_t* __restrict__ slot_key, float* __restrict__ slot_pos,
                                                             float* __restrict__ slot_nrm, uint8_t* __restrict__ slot_col) {
    const long long i = static_cast<long long>(blockIdx.x) * kCubeBlock + threadIdx.x;
    const int n = (i < ncubes) ? counts[i] : 0;
    // block-local exclusive scan of the counts
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = n;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    __shared__ int s[kCubeBlock / 32];
    if (lane == 31) s[warp] = incl;
    __syncthreads();
    int wbase = 0;
    for (int w = 0; w < warp; ++w) wbase += s[w];
    if (n == 0) return;
    const unsigned first = block_offsets[blockIdx.x] + static_cast<unsigned>(wbase + incl - n);
    if (first >= cap) return;
    int x, y, z;
    cube_of(i, v.res - 1, x, y, z);
    EdgeOut eo[12];
    int ci;
    const int ok = cube_edges(v, x, y, z, ci, eo);
    const uint64_t row = c_tri_rows[ci];
    unsigned tri = first;
    for (int t = 0; ((row >> (4 * t)) & 0xF) != 0xF && tri < cap; t += 3) {
        const int te[3] = {int((row >> (4 * t)) & 0xF), int((row >> (4 * (t + 1))) & 0xF), int((row >> (4 * (t + 2))) & 0xF)};
        if (!(((ok >> te[0]) & 1) && ((ok >> te[1]) & 1) && ((ok >> te[2]) & 1))) continue;
        for (int k = 0; k < 3; ++k) {
            const EdgeOut& e = eo[te[2 - k]];  // reversed winding (:321-334)
            const size_t sl = 3 * static_cast<size_t>(tri) + k;
            slot_key[sl] = e.key;
            slot_pos[3 * sl] = e.pos.x; slot_pos[3 * sl + 1] = e.pos.y; slot_pos[3 * sl + 2] = e.pos.z;
            slot_nrm[3 * sl] = e.nrm.x; slot_nrm[3 * sl + 1] = e.nrm.y; slot_nrm[3 * sl + 2] = e.nrm.z;
            slot_col[3 * sl] = e.col[0]; slot_col[3 * sl + 1] = e.col[1]; slot_col[3 * sl + 2] = e.col[2];
        }
        ++tri;
    }
}

__device__ __forceinline__ uint64_t hash64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

__global__ void weld_insert_kernel(const uint64_t* __restrict__ slot_key, unsigned nslots,
                                   unsigned long long* __restrict__ tkeys, unsigned* __restrict__ tvals,
                                   unsigned mask, unsigned* __restrict__ err) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    const unsigned long long key = slot_key[s];
    unsigned h = static_cast<unsigned>(hash64(key)) & mask;
    for (unsigned probe = 0; probe <= mask; ++probe) {
        const unsigned long long prev = atomicCAS(&tkeys[h], 0ull, key);
        if (prev == 0ull || prev == key) {
            atomicMin(&tvals[h], s);
            return;
        }
        h = (h + 1) & mask;
    }
    atomicExch(err, 1u);  // table full (cannot happen at load <= 1/2)
}

__device__ __forceinline__ unsigned weld_lookup(const unsigned long long* tkeys, const unsigned* tvals, unsigned mask,
                                                unsigned long long key) {
    unsigned h = static_cast<unsigned>(hash64(key)) & mask;
    for (unsigned probe = 0; probe <= mask; ++probe) {
        const unsigned long long k = tkeys[h];
        if (k == key) return tvals[h];
        if (k == 0ull) break;
        h = (h + 1) & mask;
    }
    return 0xFFFFFFFFu;
}

__global__ void weld_flag_kernel(const uint64_t* __restrict__ slot_key, unsigned nslots,
                                 const unsigned long long* __restrict__ tkeys, const unsigned* __restrict__ tvals,
                                 unsigned mask, unsigned* __restrict__ first_slot, unsigned* __restrict__ flag) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    const unsigned f = weld_lookup(tkeys, tvals, mask, slot_key[s]);
    first_slot[s] = f;
    flag[s] = (f == s) ? 1u : 0u;
}

__global__ void weld_write_kernel(unsigned nslots, const unsigned* __restrict__ first_slot,
                                  const unsigned* __restrict__ vid, const float* __restrict__ slot_pos,
                                  const float* __restrict__ slot_nrm, const uint8_t* __restrict__ slot_col,
                                  uint32_t* __restrict__ indices, float* __restrict__ pos, float* __restrict__ nrm,
                                  uint8_t* __restrict__ col) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    const unsigned f = first_slot[s];
    const unsigned id = vid[f];
    indices[s] = id;
    if (f == s) {
        for (int k = 0; k < 3; ++k) {
            pos[3 * id + k] = slot_pos[3 * s + k];
            nrm[3 * id + k] = slot_nrm[3 * s + k];
            col[3 * id + k] = slot_col[3 * s + k];
        }
    }
}

// Kernels launched by the current extraction (reported in azu_mesh_info).
static thread_local int t_launches = 0;

// ---- generic exclusive scan of uint32 (in place), multi-level -----------------
constexpr int kScanThreads = 512, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) scan_tile_kernel(unsigned* __restrict__ data, size_t n,
                                                                 unsigned* __restrict__ tile_sums) {
    __shared__ unsigned s[kScanThreads / 32];
    const size_t base = static_cast<size_t>(blockIdx.x) * kScanTile + static_cast<size_t>(threadIdx.x) * kScanItems;
    unsigned v[kScanItems];
    unsigned sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? data[base + k] : 0u;
        const unsigned t = v[k];
        v[k] = sum;
        sum += t;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s[warp] = incl;
    __syncthreads();
    unsigned wbase = 0;
    for (int w = 0; w < warp; ++w) wbase += s[w];
    const unsigned off = wbase + incl - sum;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) data[base + k] = v[k] + off;
    if (threadIdx.x == kScanThreads - 1 && tile_sums) tile_sums[blockIdx.x] = wbase + incl;
}

__global__ void scan_add_kernel(unsigned* __restrict__ data, size_t n, const unsigned* __restrict__ tile_offsets) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) data[i] += tile_offsets[i / kScanTile];
}

size_t scan_scratch_words(size_t n) {
    size_t words = 0;
    while (n > static_cast<size_t>(kScanTile)) {
        n = (n + kScanTile - 1) / kScanTile;
        words += n;
    }
    return words + 1;
}

// Exclusive scan of data[0..n) in place; scratch holds scan_scratch_words(n)
// words. The total lands in *total_dev when given.
int exclusive_scan(unsigned* data, size_t n, unsigned* scratch, unsigned* total_dev, cudaStream_t s) {
    if (n == 0) return AZU_OK;
    const size_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 1) {
        scan_tile_kernel<<<1, kScanThreads, 0, s>>>(data, n, total_dev);
        AZU_LAUNCH_CHECK();
        ++t_launches;
        return AZU_OK;
    }
    unsigned* sums = scratch;
    scan_tile_kernel<<<static_cast<unsigned>(tiles), kScanThreads, 0, s>>>(data, n, sums);
    AZU_LAUNCH_CHECK();
    ++t_launches;
    if (int rc = exclusive_scan(sums, tiles, scratch + tiles, total_dev, s)) return rc;
    scan_add_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(data, n, sums);
    AZU_LAUNCH_CHECK();
    ++t_launches;
    return AZU_OK;
}

}  // namespace azu

struct azu_mesher {
    int device = 0;
    azu::StreamRef stream;
    int64_t max_triangles = 2000000;
    // per-volume buffers
    uint8_t* counts = nullptr;
    size_t counts_cap = 0;
    unsigned* block_sums = nullptr;
    size_t blocks_cap = 0;
    unsigned* scratch = nullptr;
    size_t scratch_cap = 0;
    unsigned* d_scalars = nullptr;  // [0] total triangles, [1] total vertices, [2] weld error
    // slot and output buffers
    size_t slots_cap = 0;
    uint64_t* slot_key = nullptr;
    float* slot_pos = nullptr;
    float* slot_nrm = nullptr;
    uint8_t* slot_col = nullptr;
    unsigned* first_slot = nullptr;
    unsigned* vid = nullptr;
    size_t table_cap = 0;
    unsigned long long* tkeys = nullptr;
    unsigned* tvals = nullptr;
    float* pos = nullptr;
    float* nrm = nullptr;
    uint8_t* col = nullptr;
    uint32_t* indices = nullptr;
    azu_mesh_info last{};
};

namespace azu {

template <typename T>
static int grow(T*& p, size_t& cap, size_t need) {
    if (need <= cap && p) return AZU_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    AZU_TRY_CUDA(cudaMalloc(&p, std::max<size_t>(need, 1) * sizeof(T)));
    cap = need;
    return AZU_OK;
}

static int ensure_slots(azu_mesher* m, size_t nslots) {
    if (nslots <= m->slots_cap && m->slot_key) return AZU_OK;
    size_t c = m->slots_cap;
    void* olds[] = {m->slot_key, m->slot_pos, m->slot_nrm, m->slot_col, m->first_slot, m->vid, m->pos, m->nrm, m->col,
                    m->indices};
    for (void* q : olds) if (q) cudaFree(q);
    m->slot_key = nullptr; m->slot_pos = m->slot_nrm = m->pos = m->nrm = nullptr;
    m->slot_col = m->col = nullptr; m->first_slot = m->vid = nullptr; m->indices = nullptr;
    m->slots_cap = 0;
    c = std::max<size_t>(nslots, 3 * 4096);
    AZU_TRY_CUDA(cudaMalloc(&m->slot_key, c * 8));
    AZU_TRY_CUDA(cudaMalloc(&m->slot_pos, c * 12));
    AZU_TRY_CUDA(cudaMalloc(&m->slot_nrm, c * 12));
    AZU_TRY_CUDA(cudaMalloc(&m->slot_col, c * 3));
    AZU_TRY_CUDA(cudaMalloc(&m->first_slot, c * 4));
    AZU_TRY_CUDA(cudaMalloc(&m->vid, c * 4));
    AZU_TRY_CUDA(cudaMalloc(&m->pos, c * 12));
    AZU_TRY_CUDA(cudaMalloc(&m->nrm, c * 12));
    AZU_TRY_CUDA(cudaMalloc(&m->col, c * 3));
    AZU_TRY_CUDA(cudaMalloc(&m->indices, c * 4));
    m->slots_cap = c;
    return AZU_OK;
}

}  // namespace azu

using namespace azu;

extern "C" int azu_mesher_create(int device, void* stream, azu_mesher** out) {
    AZU_CHECK_ARG(out != nullptr, "out is null");
    *out = nullptr;
    if (int rc = bind_device(device)) return rc;
    azu_mesher* m = new azu_mesher();
    m->device = device;
    int rc = m->stream.init(stream);
    if (!rc) {
        cudaError_t e = cudaMemcpyToSymbol(c_tri_rows, azu_tables::kTriRows, sizeof(azu_tables::kTriRows));
        if (!e) e = cudaMalloc(&m->d_scalars, 4 * sizeof(unsigned));
        if (e) { set_error("mesher init: %s", cudaGetErrorString(e)); rc = AZU_E_CUDA; }
    }
    if (rc) { azu_mesher_destroy(m); return rc; }
    *out = m;
    return AZU_OK;
}

extern "C" int azu_mesher_destroy(azu_mesher* m) {
    if (!m) return AZU_OK;
    cudaSetDevice(m->device);
    if (m->stream.s) cudaStreamSynchronize(m->stream.s);
    void* all[] = {m->counts, m->block_sums, m->scratch, m->d_scalars, m->slot_key, m->slot_pos, m->slot_nrm,
                   m->slot_col, m->first_slot, m->vid, m->tkeys, m->tvals, m->pos, m->nrm, m->col, m->indices};
    for (void* q : all) if (q) cudaFree(q);
    m->stream.release();
    delete m;
    return AZU_OK;
}

extern "C" int azu_mesher_set_max_triangles(azu_mesher* m, int64_t n) {
    AZU_CHECK_ARG(m != nullptr, "null handle");
    AZU_CHECK_ARG(n >= 0 && n <= (int64_t(1) << 30), "max_triangles must be in [0, 2^30]");
    m->max_triangles = n;
    return AZU_OK;
}

extern "C" int azu_mesher_extract(azu_mesher* m, azu_volume* v, azu_mesh_info* info) {
    AZU_CHECK_ARG(m != nullptr && v != nullptr && info != nullptr, "null argument");
    AZU_TRY_CUDA(cudaSetDevice(m->device));
    cudaStream_t s = m->stream.s;
    // The volume may be written on its own stream: order after it.
    if (v->stream.s != s) AZU_TRY_CUDA(cudaStreamSynchronize(v->stream.s));
    *info = azu_mesh_info{0, 0, 0, 0};
    t_launches = 0;
    const int res = v->p.resolution;
    const long long cr = res - 1;
    const long long ncubes = cr * cr * cr;
    MeshVol mv{v->vox, v->p.format != AZU_TSDF_FP32 ? 1 : 0, v->color, res, v->p.voxel_size,
               mk3(v->p.origin[0], v->p.origin[1], v->p.origin[2])};
    const size_t nblocks = static_cast<size_t>((ncubes + kCubeBlock - 1) / kCubeBlock);
    if (int rc = grow(m->counts, m->counts_cap, static_cast<size_t>(ncubes))) return rc;
    if (int rc = grow(m->block_sums, m->blocks_cap, nblocks)) return rc;
    if (int rc = grow(m->scratch, m->scratch_cap, scan_scratch_words(std::max<size_t>(nblocks, 1 << 24)))) return rc;
    mc_classify_kernel<<<static_cast<unsigned>(nblocks), kCubeBlock, 0, s>>>(mv, ncubes, m->counts, m->block_sums);
    AZU_LAUNCH_CHECK();
    ++t_launches;
    if (int rc = exclusive_scan(m->block_sums, nblocks, m->scratch, m->d_scalars, s)) return rc;
    unsigned total = 0;
    AZU_TRY_CUDA(cudaMemcpyAsync(&total, m->d_scalars, 4, cudaMemcpyDeviceToHost, s));
    AZU_TRY_CUDA(cudaStreamSynchronize(s));
    const unsigned cap = static_cast<unsigned>(std::min<int64_t>(m->max_triangles, total));
    const size_t nslots = 3 * static_cast<size_t>(cap);
    info->truncated = total > cap ? 1 : 0;
    if (cap == 0) { info->launches = t_launches; m->last = *info; return AZU_OK; }
    if (int rc = ensure_slots(m, nslots)) return rc;
    mc_emit_kernel<<<static_cast<unsigned>(nblocks), kCubeBlock, 0, s>>>(mv, ncubes, m->counts, m->block_sums, cap,
                                                                         m->slot_key, m->slot_pos, m->slot_nrm,
                                                                         m->slot_col);
    AZU_LAUNCH_CHECK();
    ++t_launches;
    size_t tsize = 1024;
    while (tsize < 2 * nslots) tsize <<= 1;
    if (tsize > m->table_cap || !m->tkeys) {
        if (m->tkeys) cudaFree(m->tkeys);
        if (m->tvals) cudaFree(m->tvals);
        m->tkeys = nullptr;
        m->tvals = nullptr;
        m->table_cap = 0;
        AZU_TRY_CUDA(cudaMalloc(&m->tkeys, tsize * 8));
        AZU_TRY_CUDA(cudaMalloc(&m->tvals, tsize * 4));
        m->table_cap = tsize;
    }
    const unsigned mask = static_cast<unsigned>(tsize - 1);
    AZU_TRY_CUDA(cudaMemsetAsync(m->tkeys, 0, tsize * 8, s));
    AZU_TRY_CUDA(cudaMemsetAsync(m->tvals, 0xFF, tsize * 4, s));
    AZU_TRY_CUDA(cudaMemsetAsync(m->d_scalars + 2, 0, 4, s));
    const unsigned g = static_cast<unsigned>((nslots + 255) / 256);
    weld_insert_kernel<<<g, 256, 0, s>>>(m->slot_key, static_cast<unsigned>(nslots), m->tkeys, m->tvals, mask,
                                         m->d_scalars + 2);
    weld_flag_kernel<<<g, 256, 0, s>>>(m->slot_key, static_cast<unsigned>(nslots), m->tkeys, m->tvals, mask,
                                       m->first_slot, m->vid);
    AZU_LAUNCH_CHECK();
    t_launches += 2;
    if (int rc = grow(m->scratch, m->scratch_cap, std::max(m->scratch_cap, scan_scratch_words(nslots)))) return rc;
    if (int rc = exclusive_scan(m->vid, nslots, m->scratch, m->d_scalars + 1, s)) return rc;
    weld_write_kernel<<<g, 256, 0, s>>>(static_cast<unsigned>(nslots), m->first_slot, m->vid, m->slot_pos,
                                        m->slot_nrm, m->slot_col, m->indices, m->pos, m->nrm, m->col);
    AZU_LAUNCH_CHECK();
    ++t_launches;
    unsigned sc[3];
    AZU_TRY_CUDA(cudaMemcpyAsync(sc, m->d_scalars, sizeof(sc), cudaMemcpyDeviceToHost, s));
    AZU_TRY_CUDA(cudaStreamSynchronize(s));
    if (sc[2]) { set_error("weld table overflow"); return AZU_E_CUDA; }
    info->n_vertices = sc[1];
    info->n_indices = static_cast<int64_t>(nslots);
    info->launches = t_launches;
    m->last = *info;
    return AZU_OK;
}

extern "C" int azu_mesher_copy_out(azu_mesher* m, float* h_positions, float* h_normals, uint8_t* h_colors,
                                   uint32_t* h_indices) {
    AZU_CHECK_ARG(m != nullptr, "null handle");
    AZU_TRY_CUDA(cudaSetDevice(m->device));
    const size_t nv = static_cast<size_t>(m->last.n_vertices), ni = static_cast<size_t>(m->last.n_indices);
    cudaStream_t s = m->stream.s;
    if (nv && h_positions) AZU_TRY_CUDA(cudaMemcpyAsync(h_positions, m->pos, nv * 12, cudaMemcpyDeviceToHost, s));
    if (nv && h_normals) AZU_TRY_CUDA(cudaMemcpyAsync(h_normals, m->nrm, nv * 12, cudaMemcpyDeviceToHost, s));
    if (nv && h_colors) AZU_TRY_CUDA(cudaMemcpyAsync(h_colors, m->col, nv * 3, cudaMemcpyDeviceToHost, s));
    if (ni && h_indices) AZU_TRY_CUDA(cudaMemcpyAsync(h_indices, m->indices, ni * 4, cudaMemcpyDeviceToHost, s));
    AZU_TRY_CUDA(cudaStreamSynchronize(s));
    return AZU_OK;
}

extern "C" int azu_mesher_device_buffers(azu_mesher* m, const float** d_positions, const float** d_normals,
                                         const uint8_t** d_colors, const uint32_t** d_indices) {
    AZU_CHECK_ARG(m != nullptr, "null handle");
    if (d_positions) *d_positions = m->pos;
    if (d_normals) *d_normals = m->nrm;
    if (d_colors) *d_colors = m->col;
    if (d_indices) *d_indices = m->indices;
    return AZU_OK;
}
