// Marching cubes with the exact-edge weld on the GPU, behind the azu_mesher_*
// ABI. Semantics: src/meshing/MarchingCubes.cpp:81-382 (corner support rule,
// lower-endpoint crossing, one-sided/central voxel normals, colour blend,
// reversed (2,1,0) winding, 2M-triangle cap at a triangle boundary, weld by
// (lower voxel, axis) keeping the first occurrence in (z, y, x, row) order).
//
//   1. classify  stream the volume once through shared memory (asynchronous
//                copies, a 32 x 8 cube column per block marching in z); list
//                the cubes with a sign change between two usable corners.
//   2. validate  per listed cube: valid edges (position, normals, colour all
//                defined), triangles whose three edges are valid; the count goes
//                to counts[cube] and to its 256-cube block's sum.
//   3. scan      exclusive scan of the block sums -> global triangle offsets.
//   4. emit      per listed cube: block offset + byte sum of the counts before
//                it = its first triangle; its triangles' vertex slots (3 per
//                triangle, emission order) get the edge key, up to the cap.
//   5. weld      key -> smallest slot in an open-addressing table (atomicCAS /
//                atomicMin: order-independent result); a slot is a new vertex
//                iff it is its key's smallest slot; a scan of those flags gives
//                vertex ids in first-appearance order; indices follow, and each
//                vertex's payload is computed once from its key.
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

constexpr float kWeightEps = 0.001f, kGradEps = 1e-6f, kInterpEps = 1e-6f;
constexpr float kEmptyTsdf = 1.0f, kEmptyColor = 128.0f / 255.0f;

struct MeshVol {
    const void* vox;
    int half;  // FP16 formats: half tsdf in the low 16 bits, weight word (> 0 iff observed) above
    const float* color;
    int res;
    float vs;
    F3 origin;
    // the volume's free-brick flags (1: every voxel of the brick and its
    // 1-voxel apron unobserved or >= 0.9995), nb bricks a side
    const uint8_t* bricks;
    int nb;
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

// Cube edges. Edge e joins corners edge_lo(e) and edge_up(e), the lower one
// having the smaller coordinate on the edge's axis; the corner offsets and the
// 12 edges are the ones the triangle table is written for (:24-45).
__host__ __device__ constexpr int edge_lo(int e) { return static_cast<int>((0x321047540310ull >> (4 * e)) & 0xF); }
__host__ __device__ constexpr int edge_up(int e) { return static_cast<int>((0x765476653221ull >> (4 * e)) & 0xF); }
__host__ __device__ constexpr int edge_axis(int e) { return e < 8 ? (e & 1) : 2; }
__host__ __device__ constexpr int corner_dx(int c) { return ((c + 1) >> 1) & 1; }
__host__ __device__ constexpr int corner_dy(int c) { return (c >> 1) & 1; }
__host__ __device__ constexpr int corner_dz(int c) { return c >> 2; }

constexpr bool edge_tables_consistent() {
    constexpr int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    constexpr int edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                 {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    for (int c = 0; c < 8; ++c)
        if (corner_dx(c) != corner[c][0] || corner_dy(c) != corner[c][1] || corner_dz(c) != corner[c][2]) return false;
    for (int e = 0; e < 12; ++e) {
        const int a = edge[e][0], b = edge[e][1], lo = edge_lo(e), up = edge_up(e), ax = edge_axis(e);
        if (!((lo == a && up == b) || (lo == b && up == a))) return false;
        for (int k = 0; k < 3; ++k)
            if ((corner[up][k] - corner[lo][k]) != (k == ax ? 1 : 0)) return false;
    }
    return true;
}
static_assert(edge_tables_consistent(), "edge / corner tables");

// Corner support folded into one float: the tsdf where the corner is usable,
// NaN where sampleCorner refuses it (a usable corner is always finite).
__device__ __forceinline__ float corner_code(float2 r) {
    return (!isfinite(r.x) || r.y <= kWeightEps) ? __int_as_float(0x7fffffff) : r.x;
}
__device__ __forceinline__ float corner_code(uint32_t u) {
    return corner_code(make_float2(__half2float(__ushort_as_half(static_cast<unsigned short>(u & 0xFFFFu))),
                                   static_cast<float>(u >> 16)));
}

// Eight corner codes -> cube index (bit c: corner c negative) and whether any
// edge has a sign change between two usable corners (the only edges
// crossingFromLower can accept).
__device__ __forceinline__ int cube_signs(const float (&cv)[8], bool& candidate) {
    int neg = 0, sup = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        neg |= (cv[c] < 0.0f) << c;
        sup |= (cv[c] == cv[c]) << c;
    }
    // partners along x: 0-1, 3-2, 4-5, 7-6; along y: 0-3, 1-2, 4-7, 5-6; along z: c-(c+4)
    const int px_n = ((neg & 0x55) << 1) | ((neg & 0xAA) >> 1), px_s = ((sup & 0x55) << 1) | ((sup & 0xAA) >> 1);
    const int py_n = ((neg & 0x11) << 3) | ((neg & 0x88) >> 3) | ((neg & 0x22) << 1) | ((neg & 0x44) >> 1);
    const int py_s = ((sup & 0x11) << 3) | ((sup & 0x88) >> 3) | ((sup & 0x22) << 1) | ((sup & 0x44) >> 1);
    const int cx = (neg ^ px_n) & sup & px_s, cy = (neg ^ py_n) & sup & py_s;
    const int cz = (neg ^ (neg >> 4)) & sup & (sup >> 4) & 0xF;
    candidate = (cx | cy | cz) != 0;
    return neg;
}

// crossingFromLower (:115-134), the blended normal and the colour blend
// (:276-311) of one edge, lower voxel l, upper voxel u = l + unit(axis), in the
// CPU path's float expressions and order. False where the CPU path drops the
// edge; the payload is written only when pos_out is given.
__device__ __forceinline__ bool edge_vertex(const MeshVol& v, int lx, int ly, int lz, int axis, float vl, float vu,
                                            F3 nl, F3 nu, F3* pos_out, F3* nrm_out, uint8_t* col_out) {
    const int ux = lx + (axis == 0), uy = ly + (axis == 1), uz = lz + (axis == 2);
    const F3 pl = add3(v.origin, mul3(mk3(float(lx), float(ly), float(lz)), v.vs));
    const F3 pu = add3(v.origin, mul3(mk3(float(ux), float(uy), float(uz)), v.vs));
    if (!isfinite(vl) || !isfinite(vu) || !finite3(pl) || !finite3(pu)) return false;
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
    if (!finite3(nl) || !finite3(nu)) return false;
    const F3 bl = add3(nl, smul3(t, sub3(nu, nl)));
    const float blen = norm3(bl);
    if (!isfinite(blen) || blen <= kGradEps) return false;
    const size_t il = v.idx(lx, ly, lz), iu = v.idx(ux, uy, uz);
    uint8_t cb[3];
    bool cok = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = v.col(il, k), b = v.col(iu, k);
        cok = cok && srgb_to_byte(fa(a, fm(t, fs(b, a))), &cb[k]);
    }
    if (!cok) return false;
    if (pos_out) {
        *pos_out = pos;
        *nrm_out = div3(bl, blen);
        col_out[0] = cb[0]; col_out[1] = cb[1]; col_out[2] = cb[2];
    }
    return true;
}

// Cube (x, y, z): cube index and the bit set of edges that yield a vertex.
__device__ int cube_valid_edges(const MeshVol& v, int x, int y, int z, int& cube_idx) {
    float cv[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        float val;
        cv[c] = v.corner(x + corner_dx(c), y + corner_dy(c), z + corner_dz(c), val) ? val : __int_as_float(0x7fffffff);
    }
    bool candidate;
    cube_idx = cube_signs(cv, candidate);
    if (!candidate) return 0;
    int cand = 0, need = 0;
#pragma unroll
    for (int e = 0; e < 12; ++e) {
        const int lo = edge_lo(e), up = edge_up(e);
        const bool c = (((cube_idx >> lo) ^ (cube_idx >> up)) & 1) && cv[lo] == cv[lo] && cv[up] == cv[up];
        cand |= c << e;
        need |= c ? (1 << lo) | (1 << up) : 0;
    }
    F3 cn[8];
#pragma unroll
    for (int c = 0; c < 8; ++c)
        cn[c] = (need >> c) & 1 ? voxel_normal(v, x + corner_dx(c), y + corner_dy(c), z + corner_dz(c)) : nan3();
    int ok = 0;
#pragma unroll
    for (int e = 0; e < 12; ++e) {
        if (!((cand >> e) & 1)) continue;
        const int lo = edge_lo(e), up = edge_up(e);
        if (edge_vertex(v, x + corner_dx(lo), y + corner_dy(lo), z + corner_dz(lo), edge_axis(e), cv[lo], cv[up], cn[lo],
                        cn[up], nullptr, nullptr, nullptr))
            ok |= 1 << e;
    }
    return ok;
}

// Threads of a warp index the triangle table by their own cube, so the
// kernels that read it stage it in shared memory (constant memory serialises
// divergent indices).
__device__ __forceinline__ void stage_tri_rows(uint64_t* s_rows) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_rows[i] = c_tri_rows[i];
    __syncthreads();
}

__device__ __forceinline__ int count_tris(const uint64_t* rows, int cube_idx, int ok) {
    const uint64_t row = rows[cube_idx];
    int n = 0;
    for (int t = 0; ((row >> (4 * t)) & 0xF) != 0xF; t += 3) {
        const int a = (row >> (4 * t)) & 0xF, b = (row >> (4 * (t + 1))) & 0xF, c = (row >> (4 * (t + 2))) & 0xF;
        n += ((ok >> a) & 1) && ((ok >> b) & 1) && ((ok >> c) & 1);
    }
    return n;
}

__device__ __forceinline__ void cube_of(unsigned long long i, unsigned cr, int& x, int& y, int& z) {
    const unsigned long long r = i / cr;
    x = static_cast<int>(i - r * cr);
    const unsigned long long q = r / cr;
    y = static_cast<int>(r - q * cr);
    z = static_cast<int>(q);
}

// ---- 1. classify: stream the volume once, list the candidate cubes ---------
// A block owns a 32 x 8 column of cubes over kTileZ cube layers, i.e. 33 x 9
// voxels per slice. Each thread copies its own voxel of every slice (and one
// apron voxel for 41 threads) into private shared-memory slots by asynchronous
// copies kPrefetch slices ahead, turns it into a 2-bit sign code (bit 0: usable
// and negative, bit 1: usable and not negative) and shares the code; a cube is
// a candidate when its eight codes OR to 3. That keeps every cube with an edge
// between usable corners of opposite sign (the only edges crossingFromLower
// can accept) and a few more, which validation drops. Candidates gather in a
// block list and go to the global list (unordered; everything after is
// order-independent) in one reservation per flush.
constexpr int kTileX = 32, kTileY = 8, kTileZ = 32;
constexpr int kApron = kTileX + 1 + kTileY;  // row kTileY (33 voxels) and column kTileX (8 voxels)
constexpr int kCodeW = kTileX + 1, kCodeN = kCodeW * (kTileY + 1);
constexpr int kPrefetch = 7, kRing = kPrefetch + 1;  // slices in flight per thread
constexpr int kClassifyThreads = kTileX * kTileY;
constexpr int kListCap = 1024;
static_assert(kClassifyThreads == 256 && kApron <= kClassifyThreads && (kRing & (kRing - 1)) == 0, "tile shape");
static_assert(kTileZ * kClassifyThreads <= 65536, "block-local cube offsets are 16-bit");

template <int B>
__device__ __forceinline__ void cp_async_zfill(void* dst, const void* src, bool in) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    const int n = in ? B : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(src), "n"(B), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <typename VT>
__device__ __forceinline__ int sign_code(VT raw) {
    const float c = corner_code(raw);
    return c < 0.0f ? 1 : (c == c ? 2 : 0);
}

template <typename VT>
__global__ void __launch_bounds__(kClassifyThreads) mc_classify_kernel(MeshVol v, unsigned long long* __restrict__ active,
                                                                       unsigned cap, unsigned* __restrict__ n_active) {
    __shared__ __align__(16) VT raw[kRing][kClassifyThreads];
    __shared__ __align__(16) VT raw_apron[kRing][kApron];
    __shared__ uint8_t codes[3][kCodeN];
    __shared__ unsigned short list[kListCap];
    __shared__ unsigned list_n, list_base;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int res = v.res, cr = res - 1;
    const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * kTileY, z0 = blockIdx.z * kTileZ;
    const int nz = min(kTileZ, cr - z0);
    const size_t plane = static_cast<size_t>(res) * res;
    const bool in_main = x0 + tx < res && y0 + ty < res;
    const int ax = tid <= kTileX ? tid : kTileX, ay = tid <= kTileX ? kTileY : tid - (kTileX + 1);
    const bool has_apron = tid < kApron;
    const bool in_apron = has_apron && x0 + ax < res && y0 + ay < res;
    const VT* base = static_cast<const VT*>(v.vox) + static_cast<size_t>(z0) * plane;
    const VT* src_main = base + (in_main ? static_cast<size_t>(y0 + ty) * res + (x0 + tx) : 0);
    const VT* src_apron = base + (in_apron ? static_cast<size_t>(y0 + ay) * res + (x0 + ax) : 0);
    const int own = ty * kCodeW + tx, apron = ay * kCodeW + ax;
    if (v.bricks) {
        // The tile's cubes have their base voxels in 4 x 1 x 4 bricks (x0, y0,
        // z0 are multiples of 8) and their corners in those bricks' aprons. In
        // a free brick every usable corner is >= 0.9995, so no cube there has a
        // sign change: a tile of free bricks lists nothing and reads nothing.
        const int bx = (x0 >> 3) + (tid & 3), by = y0 >> 3, bz = (z0 >> 3) + ((tid >> 2) & 3);
        const bool open = tid < 16 && bx < v.nb && by < v.nb && bz < v.nb &&
                          __ldg(v.bricks + (static_cast<size_t>(bz) * v.nb + by) * v.nb + bx) == 0;
        if (!__syncthreads_or(open)) return;
    }
    if (tid == 0) list_n = 0;
    auto issue = [&](int s) {  // slice s = voxel layer z0 + s
        if (s <= nz) {
            const size_t o = static_cast<size_t>(s) * plane;
            cp_async_zfill<sizeof(VT)>(&raw[s & (kRing - 1)][tid], src_main + o, in_main);
            if (has_apron) cp_async_zfill<sizeof(VT)>(&raw_apron[s & (kRing - 1)][tid], src_apron + o, in_apron);
        }
        cp_async_commit();
    };
    // At the wait for slice s, s + kPrefetch + 1 groups are committed: waiting
    // until kPrefetch remain completes slice s (each thread reads only its own copies).
    auto decode = [&](int s, int buf) {
        cp_async_wait<kPrefetch>();
        const int c = sign_code(raw[s & (kRing - 1)][tid]);
        codes[buf][own] = static_cast<uint8_t>(c);
        if (has_apron) codes[buf][apron] = static_cast<uint8_t>(sign_code(raw_apron[s & (kRing - 1)][tid]));
        issue(s + kPrefetch + 1);
        return c;
    };
    auto face = [&](int buf, int c) {
        return c | codes[buf][own + 1] | codes[buf][own + kCodeW] | codes[buf][own + kCodeW + 1];
    };
    // Sends the block list to the global list; called by all threads right
    // after a barrier.
    auto flush = [&]() {
        const unsigned n = list_n;
        __syncthreads();
        if (tid == 0) {
            list_base = atomicAdd(n_active, n);
            list_n = 0;
        }
        __syncthreads();
        const unsigned first = list_base;
        for (unsigned k = tid; k < n; k += kClassifyThreads) {
            if (first + k >= cap) break;
            const unsigned e = list[k];
            active[first + k] = (static_cast<unsigned long long>(z0 + (e >> 8)) * cr + (y0 + ((e >> 5) & 7))) * cr +
                                (x0 + (e & 31));
        }
        __syncthreads();
    };
#pragma unroll
    for (int s = 0; s <= kPrefetch; ++s) issue(s);
    const int c0 = decode(0, 0);
    int c_hi = decode(1, 1);
    __syncthreads();
    const bool valid = x0 + tx < cr && y0 + ty < cr;
    int face_lo = face(0, c0);
    int b_hi = 1, b_nx = 2;  // code buffers of slices j + 1 and j + 2
    for (int j = 0; j < nz; ++j) {
        const int c_nx = j + 2 <= nz ? decode(j + 2, b_nx) : 0;
        const int face_hi = face(b_hi, c_hi);
        const bool act = valid && (face_lo | face_hi) == 3;
        const unsigned bal = __ballot_sync(0xffffffffu, act);
        if (bal) {
            unsigned first = 0;
            if (tx == 0) first = atomicAdd(&list_n, static_cast<unsigned>(__popc(bal)));
            first = __shfl_sync(0xffffffffu, first, 0);
            if (act) list[first + __popc(bal & ((1u << tx) - 1u))] = static_cast<unsigned short>(tid + (j << 8));
        }
        face_lo = face_hi;
        c_hi = c_nx;
        const int b_old = b_hi;
        b_hi = b_nx;
        b_nx = 3 - b_old - b_nx;
        __syncthreads();
        if (list_n > static_cast<unsigned>(kListCap - kClassifyThreads)) flush();
    }
    if (list_n) flush();
    cp_async_wait<0>();
}

// ---- 2. validate: per candidate cube, the triangles it emits ----------------
// meta = valid edge bits | cube index << 12 | triangles << 20; the triangle
// count also lands in counts[cube] (zeroed before) and in its 256-cube
// block's sum.
__global__ void __launch_bounds__(256) mc_validate_kernel(MeshVol v, const unsigned long long* __restrict__ active,
                                                          const unsigned* __restrict__ n_active, unsigned cap,
                                                          uint32_t* __restrict__ meta, uint8_t* __restrict__ counts,
                                                          unsigned* __restrict__ block_sums) {
    __shared__ uint64_t s_rows[256];
    stage_tri_rows(s_rows);
    const unsigned n = min(*n_active, cap);
    const unsigned cr = static_cast<unsigned>(v.res - 1);
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const unsigned long long i = active[k];
        int x, y, z, ci;
        cube_of(i, cr, x, y, z);
        const int ok = cube_valid_edges(v, x, y, z, ci);
        const int nt = ok ? count_tris(s_rows, ci, ok) : 0;
        meta[k] = static_cast<uint32_t>(ok) | (static_cast<uint32_t>(ci) << 12) | (static_cast<uint32_t>(nt) << 20);
        if (nt) {
            counts[i] = static_cast<uint8_t>(nt);
            atomicAdd(&block_sums[i >> 8], static_cast<unsigned>(nt));
        }
    }
}

__device__ __forceinline__ unsigned byte_sum(unsigned w) { return __dp4a(w, 0x01010101u, 0u); }

// The counts of the listed cubes (the only ones the validate step writes) back
// to zero.
__global__ void __launch_bounds__(256) mc_clear_counts_kernel(const unsigned long long* __restrict__ active, unsigned n,
                                                              uint8_t* __restrict__ counts) {
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) counts[active[k]] = 0;
}

// ---- 4. emit: the vertex slots of every emitted triangle ---------------------
// A candidate's first triangle is its block's offset plus the triangles of the
// cubes before it in that block (a byte sum over counts), so slots come out in
// the CPU path's (z, y, x, row) order. Each slot holds its edge's key
// ((lower voxel, axis) + 1), up to the cap.
__global__ void __launch_bounds__(256) mc_emit_kernel(MeshVol v, const unsigned long long* __restrict__ active,
                                                      const uint32_t* __restrict__ meta, unsigned n,
                                                      const uint8_t* __restrict__ counts,
                                                      const unsigned* __restrict__ block_offsets, unsigned cap,
                                                      uint64_t* __restrict__ slot_key) {
    __shared__ uint64_t s_rows[256];
    stage_tri_rows(s_rows);
    const unsigned cr = static_cast<unsigned>(v.res - 1);
    const uint64_t R = static_cast<uint64_t>(v.res);
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t m = meta[k];
        if ((m >> 20) == 0) continue;
        const unsigned long long i = active[k];
        const unsigned long long b = i >> 8;
        const int r = static_cast<int>(i & 255);
        const uint4* w = reinterpret_cast<const uint4*>(counts + (b << 8));
        unsigned before = 0;
        for (int q = 0; q < (r >> 4); ++q) {
            const uint4 u = w[q];
            before += byte_sum(u.x) + byte_sum(u.y) + byte_sum(u.z) + byte_sum(u.w);
        }
        if (r & 15) {
            const uint4 u = w[r >> 4];
            const unsigned words[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int bytes = (r & 15) - 4 * j;
                const unsigned mask = bytes >= 4 ? 0xFFFFFFFFu : (bytes <= 0 ? 0u : (1u << (8 * bytes)) - 1u);
                before += byte_sum(words[j] & mask);
            }
        }
        const unsigned first = block_offsets[b] + before;
        if (first >= cap) continue;
        int x, y, z;
        cube_of(i, cr, x, y, z);
        const int ok = static_cast<int>(m & 0xFFF), ci = static_cast<int>((m >> 12) & 0xFF);
        const uint64_t row = s_rows[ci];
        unsigned tri = first;
        for (int t = 0; ((row >> (4 * t)) & 0xF) != 0xF && tri < cap; t += 3) {
            const int e0 = int((row >> (4 * t)) & 0xF), e1 = int((row >> (4 * (t + 1))) & 0xF),
                      e2 = int((row >> (4 * (t + 2))) & 0xF);
            if (!(((ok >> e0) & 1) && ((ok >> e1) & 1) && ((ok >> e2) & 1))) continue;
            const int te[3] = {e2, e1, e0};  // reversed winding (:321-334)
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                const int e = te[s], lo = edge_lo(e);
                const uint64_t lx = x + corner_dx(lo), ly = y + corner_dy(lo), lz = z + corner_dz(lo);
                slot_key[3 * static_cast<size_t>(tri) + s] = ((lz * R + ly) * R + lx) * 3 + edge_axis(e) + 1;  // 0 = empty
            }
            ++tri;
        }
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

// indices, and the vertex payload computed once per welded vertex from its key
// (a function of the edge alone, so equal to what any cube sharing the edge
// computes).
__global__ void weld_write_kernel(MeshVol v, unsigned nslots, const uint64_t* __restrict__ slot_key,
                                  const unsigned* __restrict__ first_slot, const unsigned* __restrict__ vid,
                                  uint32_t* __restrict__ indices, float* __restrict__ pos, float* __restrict__ nrm,
                                  uint8_t* __restrict__ col) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    const unsigned f = first_slot[s];
    const unsigned id = vid[f];
    indices[s] = id;
    if (f != s) return;
    const uint64_t key = slot_key[s] - 1, R = static_cast<uint64_t>(v.res);
    const int axis = static_cast<int>(key % 3);
    const uint64_t lin = key / 3;
    const int lx = static_cast<int>(lin % R), ly = static_cast<int>((lin / R) % R), lz = static_cast<int>(lin / (R * R));
    const int ux = lx + (axis == 0), uy = ly + (axis == 1), uz = lz + (axis == 2);
    float vl = 0.0f, vu = 0.0f;
    v.corner(lx, ly, lz, vl);
    v.corner(ux, uy, uz, vu);
    F3 p, n;
    uint8_t c[3] = {0, 0, 0};
    edge_vertex(v, lx, ly, lz, axis, vl, vu, voxel_normal(v, lx, ly, lz), voxel_normal(v, ux, uy, uz), &p, &n, c);
    pos[3 * id] = p.x; pos[3 * id + 1] = p.y; pos[3 * id + 2] = p.z;
    nrm[3 * id] = n.x; nrm[3 * id + 1] = n.y; nrm[3 * id + 2] = n.z;
    col[3 * id] = c[0]; col[3 * id + 1] = c[1]; col[3 * id + 2] = c[2];
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
    int sms = 0;
    azu::StreamRef stream;
    int64_t max_triangles = 2000000;
    // per-volume buffers
    uint8_t* counts = nullptr;  // triangles per cube (linear cube order)
    size_t counts_cap = 0;
    bool counts_zero = false;   // every count is zero (cleared after each extraction)
    unsigned* block_sums = nullptr;  // per 256 cubes; scanned in place into offsets
    size_t blocks_cap = 0;
    unsigned* scratch = nullptr;
    size_t scratch_cap = 0;
    unsigned long long* active = nullptr;  // candidate cubes (linear index), unordered
    uint32_t* meta = nullptr;              // per candidate: valid edges | cube index << 12 | triangles << 20
    size_t active_cap = 0;
    unsigned* d_scalars = nullptr;  // [0] total triangles, [1] total vertices, [2] weld error, [3] candidates
    // slot and output buffers
    size_t slots_cap = 0;
    uint64_t* slot_key = nullptr;
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
    void* olds[] = {m->slot_key, m->first_slot, m->vid, m->pos, m->nrm, m->col, m->indices};
    for (void* q : olds) if (q) cudaFree(q);
    m->slot_key = nullptr; m->pos = m->nrm = nullptr;
    m->col = nullptr; m->first_slot = m->vid = nullptr; m->indices = nullptr;
    m->slots_cap = 0;
    // half again the need: a growing scene's next extraction then reuses the
    // buffers instead of freeing and allocating them (both stall the device)
    const size_t c = std::max<size_t>(nslots + nslots / 2, 3 * 4096);
    AZU_TRY_CUDA(cudaMalloc(&m->slot_key, c * 8));
    AZU_TRY_CUDA(cudaMalloc(&m->first_slot, c * 4));
    AZU_TRY_CUDA(cudaMalloc(&m->vid, c * 4));
    AZU_TRY_CUDA(cudaMalloc(&m->pos, c * 12));
    AZU_TRY_CUDA(cudaMalloc(&m->nrm, c * 12));
    AZU_TRY_CUDA(cudaMalloc(&m->col, c * 3));
    AZU_TRY_CUDA(cudaMalloc(&m->indices, c * 4));
    m->slots_cap = c;
    return AZU_OK;
}

static int ensure_active(azu_mesher* m, size_t n) {
    if (n <= m->active_cap && m->active) return AZU_OK;
    if (m->active) cudaFree(m->active);
    if (m->meta) cudaFree(m->meta);
    m->active = nullptr;
    m->meta = nullptr;
    m->active_cap = 0;
    AZU_TRY_CUDA(cudaMalloc(&m->active, n * 8));
    AZU_TRY_CUDA(cudaMalloc(&m->meta, n * 4));
    m->active_cap = n;
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
        if (!e) e = cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device);
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
    void* all[] = {m->counts, m->block_sums, m->scratch, m->active, m->meta, m->d_scalars, m->slot_key,
                   m->first_slot, m->vid, m->tkeys, m->tvals, m->pos, m->nrm, m->col, m->indices};
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
    const unsigned long long cr = static_cast<unsigned long long>(res - 1);
    const unsigned long long ncubes = cr * cr * cr;
    if (ncubes == 0) { m->last = *info; return AZU_OK; }
    MeshVol mv{v->vox, v->p.format != AZU_TSDF_FP32 ? 1 : 0, v->color, res, v->p.voxel_size,
               mk3(v->p.origin[0], v->p.origin[1], v->p.origin[2]), v->skip_free ? v->bricks : nullptr, v->nb};
    const size_t nblocks = static_cast<size_t>((ncubes + 255) / 256);
    {
        const size_t cap_before = m->counts_cap;
        if (int rc = grow(m->counts, m->counts_cap, static_cast<size_t>(ncubes) + 16)) return rc;
        if (m->counts_cap != cap_before) m->counts_zero = false;  // a new buffer
    }
    if (int rc = grow(m->block_sums, m->blocks_cap, nblocks)) return rc;
    if (int rc = grow(m->scratch, m->scratch_cap, scan_scratch_words(std::max<size_t>(nblocks, 1 << 24)))) return rc;
    // candidate list: a surface's share of the cubes, regrown with headroom when it overflows
    if (int rc = ensure_active(m, std::max<size_t>(m->active_cap, std::min<size_t>(ncubes, std::max<size_t>(
                                                                        ncubes / 64, size_t(1) << 16)))))
        return rc;
    const dim3 cgrid(static_cast<unsigned>((cr + kTileX - 1) / kTileX), static_cast<unsigned>((cr + kTileY - 1) / kTileY),
                     static_cast<unsigned>((cr + kTileZ - 1) / kTileZ));
    const unsigned pgrid = static_cast<unsigned>(std::max(m->sms, 1) * 8);
    unsigned sc4[4] = {0, 0, 0, 0};
    for (int attempt = 0; attempt < 2; ++attempt) {
        // counts carries one uint4 of slack: the emit's byte sums read whole
        // words. It is zeroed once; after each extraction the listed cubes'
        // counts are set back to zero (a few MB of writes instead of a memset
        // of one byte per cube).
        if (!m->counts_zero) AZU_TRY_CUDA(cudaMemsetAsync(m->counts, 0, m->counts_cap, s));  // the whole buffer
        m->counts_zero = false;
        AZU_TRY_CUDA(cudaMemsetAsync(m->block_sums, 0, nblocks * 4, s));
        AZU_TRY_CUDA(cudaMemsetAsync(m->d_scalars, 0, 16, s));
        const unsigned acap = static_cast<unsigned>(std::min<size_t>(m->active_cap, 0xFFFFFFFFu));
        if (mv.half)
            mc_classify_kernel<uint32_t><<<cgrid, kClassifyThreads, 0, s>>>(mv, m->active, acap, m->d_scalars + 3);
        else
            mc_classify_kernel<float2><<<cgrid, kClassifyThreads, 0, s>>>(mv, m->active, acap, m->d_scalars + 3);
        AZU_LAUNCH_CHECK();
        mc_validate_kernel<<<pgrid, 256, 0, s>>>(mv, m->active, m->d_scalars + 3, acap, m->meta, m->counts,
                                                 m->block_sums);
        AZU_LAUNCH_CHECK();
        t_launches += 2;
        if (int rc = exclusive_scan(m->block_sums, nblocks, m->scratch, m->d_scalars, s)) return rc;
        AZU_TRY_CUDA(cudaMemcpyAsync(sc4, m->d_scalars, sizeof(sc4), cudaMemcpyDeviceToHost, s));
        AZU_TRY_CUDA(cudaStreamSynchronize(s));
        if (sc4[3] <= acap) break;
        // more candidate cubes than the list holds: grow it to fit and run again
        if (attempt == 1) { set_error("candidate list overflow"); return AZU_E_CUDA; }
        if (int rc = ensure_active(m, std::min<size_t>(ncubes, static_cast<size_t>(sc4[3]) + sc4[3] / 2))) return rc;
    }
    const unsigned total = sc4[0], n_active = sc4[3];
    // the listed cubes' counts back to zero once the emit has read them
    auto clear_counts = [&]() -> int {
        if (n_active) {
            mc_clear_counts_kernel<<<std::min(pgrid, (n_active + 255) / 256), 256, 0, s>>>(m->active, n_active,
                                                                                         m->counts);
            AZU_LAUNCH_CHECK();
            ++t_launches;
        }
        m->counts_zero = true;
        return AZU_OK;
    };
    const unsigned cap = static_cast<unsigned>(std::min<int64_t>(m->max_triangles, total));
    const size_t nslots = 3 * static_cast<size_t>(cap);
    info->truncated = total > cap ? 1 : 0;
    if (cap == 0) {
        if (int rc = clear_counts()) return rc;
        info->launches = t_launches;
        m->last = *info;
        return AZU_OK;
    }
    if (int rc = ensure_slots(m, nslots)) return rc;
    mc_emit_kernel<<<std::min(pgrid, (n_active + 255) / 256), 256, 0, s>>>(mv, m->active, m->meta, n_active, m->counts,
                                                                          m->block_sums, cap, m->slot_key);
    AZU_LAUNCH_CHECK();
    ++t_launches;
    if (int rc = clear_counts()) return rc;
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
    weld_write_kernel<<<g, 256, 0, s>>>(mv, static_cast<unsigned>(nslots), m->slot_key, m->first_slot, m->vid,
                                        m->indices, m->pos, m->nrm, m->col);
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
