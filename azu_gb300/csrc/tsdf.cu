// TSDF volume on the GPU: reset, voxel-projective integration, front-face
// raycast and whole-volume transfers, behind the azu_volume_* C ABI.
//
// Semantics follow the reference CPU path (src/tsdf/TSDFVolume.cpp:112-525);
// the reference's own CUDA twin (src/tsdf/TSDFVolume_cuda.cu) is not followed.
//
// Layout in HBM: one 8-byte record per voxel, {float tsdf, float weight}, in
// z-major order (index z*res*res + y*res + x) — every consumer (integrate,
// trilinear sampling, marching cubes) needs both fields of a voxel together.
// The FP16 form packs {half tsdf, uint16 weight} into 4 bytes. Colour, when
// enabled, is a separate float[3] per voxel.
#include <cuda_fp16.h>

#include <cmath>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <vector>

#include "azu_internal.h"
#include "kf_math.cuh"
#include "tsdf_sample.cuh"
#include "fstep.cuh"

namespace azu {

size_t voxel_bytes(int format) { return format == AZU_TSDF_FP32 ? 8 : 4; }

// Clears the free flag of every brick whose apron [8b, 8b+8] holds voxel (x, y, z).
__device__ __forceinline__ void clear_bricks(uint8_t* bricks, int nb, int x, int y, int z) {
    const int bx = x >> kBrickShift, by = y >> kBrickShift, bz = z >> kBrickShift;
    const int ex = ((x & 7) == 0 && x > 0) ? 1 : 0, ey = ((y & 7) == 0 && y > 0) ? 1 : 0,
              ez = ((z & 7) == 0 && z > 0) ? 1 : 0;
    for (int dz = 0; dz <= ez; ++dz)
        for (int dy = 0; dy <= ey; ++dy)
            for (int dx = 0; dx <= ex; ++dx) {
                const size_t b = (static_cast<size_t>(bz - dz) * nb + (by - dy)) * nb + (bx - dx);
                bricks[b] = 0;
            }
}

// ---- small kernels -------------------------------------------------------
struct Pose16 {
    float m[16];
};
__global__ void set_pose_kernel(float* dst, Pose16 p) {
    if (threadIdx.x < 16) dst[threadIdx.x] = p.m[threadIdx.x];
}

template <bool kHalf>
__global__ void reset_kernel(void* vox, float* color, size_t n) {
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        Vox<kHalf>::store(vox, i, kEmptyTsdf, 0.0f);
        if (color) {
            color[3 * i] = kEmptyColor;
            color[3 * i + 1] = kEmptyColor;
            color[3 * i + 2] = kEmptyColor;
        }
    }
}

// ---- integration -----------------------------------------------------------
constexpr int kIntWarps = 4;
constexpr int kTileShift = 3;  // level-0 depth tiles are 8x8 pixels
constexpr int kCullSeg = 16;   // voxels per culling piece of a 32-voxel chunk
constexpr int kIntParts = 2;   // x-parts per 32-row item of the persistent kernel (shorter items, shorter tail)
constexpr int kUpdGroup = 4;   // rows per software-pipelined update group (6 and 8 were slower)
constexpr int kFineSide = 4;   // level-0 depth tiles a culling box may span a side before a coarser level is used
constexpr int kIntBuckets = 8; // work buckets of the integration, by kept-brick count
constexpr int kCounters = 5 + kIntBuckets;

// Deepest in-band depth of every 8x8 pixel tile (-inf when the tile has none),
// level 0 of the tile pyramid. Eight lanes share a tile, one pixel row each.
__device__ __forceinline__ void depth_tiles_body(int blk, const float* __restrict__ depth, int W, int H, float min_d,
                                                 float max_d, int tw, int ntiles, float* __restrict__ tiles,
                                                 const int* __restrict__ gate) {
    if (gate && __ldg(gate) == 0) return;
    const int t = blk * (blockDim.x >> 3) + (threadIdx.x >> 3);
    const int r = threadIdx.x & 7;
    float m = -__int_as_float(0x7f800000);
    if (t < ntiles) {
        const int ty = t / tw, tx = t - ty * tw;
        const int y = (ty << kTileShift) + r;
        if (y < H) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int x = (tx << kTileShift) + i;
                if (x < W) {
                    const float d = __ldg(depth + static_cast<size_t>(y) * W + x);
                    if (d >= min_d && d <= max_d) m = fmaxf(m, d);
                }
            }
        }
    }
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 4));
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
    if (t < ntiles && r == 0) tiles[t] = m;
}
__global__ void depth_tiles_kernel(const float* __restrict__ depth, int W, int H, float min_d, float max_d, int tw,
                                   int ntiles, float* __restrict__ tiles, const int* __restrict__ gate) {
    depth_tiles_body(blockIdx.x, depth, W, H, min_d, max_d, tw, ntiles, tiles, gate);
}

TileMip make_tile_mip(int W, int H) {
    TileMip m{};
    int w = (W + 7) >> kTileShift, h = (H + 7) >> kTileShift, off = 0;
    for (m.levels = 0; m.levels < kMaxTileLevels; ++m.levels) {
        m.w[m.levels] = w;
        m.h[m.levels] = h;
        m.off[m.levels] = off;
        off += w * h;
        if (w == 1 && h == 1) {
            ++m.levels;
            break;
        }
        w = (w + 1) >> 1;
        h = (h + 1) >> 1;
    }
    m.total = off;
    return m;
}

// Tile pyramid, one block: level l from level l-1, 2x2 children.
__device__ __forceinline__ void build_tile_pyramid(float* __restrict__ tiles, const TileMip& mip) {
    for (int l = 1; l < mip.levels; ++l) {
        __syncthreads();
        const float* src = tiles + mip.off[l - 1];
        float* dst = tiles + mip.off[l];
        const int sw = mip.w[l - 1], sh = mip.h[l - 1], w = mip.w[l], n = w * mip.h[l];
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int ty = i / w, tx = i - ty * w;
            const int x0 = 2 * tx, y0 = 2 * ty;
            float m = src[y0 * sw + x0];
            if (x0 + 1 < sw) m = fmaxf(m, src[y0 * sw + x0 + 1]);
            if (y0 + 1 < sh) {
                m = fmaxf(m, src[(y0 + 1) * sw + x0]);
                if (x0 + 1 < sw) m = fmaxf(m, src[(y0 + 1) * sw + x0 + 1]);
            }
            dst[i] = m;
        }
    }
}
__global__ void tile_pyramid_kernel(float* __restrict__ tiles, TileMip mip) { build_tile_pyramid(tiles, mip); }

// Frustum AABB and camera transform for one integration (TSDFVolume.cpp:238-264),
// computed on the device so the pose may come from the tracker without a host
// round trip. Same float expression trees as the CPU path. Thread 0 writes the
// constants; the block then builds levels 1.. of the tile pyramid unless they
// were built with the depth map.
__device__ __forceinline__ void integrate_setup_body(const float* __restrict__ d_pose, int res, float vs, float ox,
                                                     float oy, float oz, float trunc, float fx, float fy, float cx,
                                                     float cy, int W, int H, float max_d, IntegrateConsts* out,
                                                     unsigned long long* counters, float* __restrict__ tiles,
                                                     const TileMip& mip, bool pyramid) {
    if (threadIdx.x == 0) {
        float P[16], inv[16], Rcw[9];
        for (int i = 0; i < 16; ++i) P[i] = d_pose[i];
        inverse4(P, inv);
        IntegrateConsts ic;
        rot_of(inv, ic.R_wc);
        const F3 t_wc = trans_of(inv);
        ic.t_wc[0] = t_wc.x; ic.t_wc[1] = t_wc.y; ic.t_wc[2] = t_wc.z;
        rot_of(P, Rcw);
        const F3 t_cw = trans_of(P);
        const F3 origin = mk3(ox, oy, oz);
        F3 lo = div3(sub3(t_cw, origin), vs);
        F3 hi = lo;
        const float z_far = fa(max_d, trunc);
        const float cpx[4][2] = {{0.0f, 0.0f}, {float(W), 0.0f}, {0.0f, float(H)}, {float(W), float(H)}};
        for (int k = 0; k < 4; ++k) {
            const F3 ray = mk3(fm(fd(fs(cpx[k][0], cx), fx), z_far), fm(fd(fs(cpx[k][1], cy), fy), z_far), z_far);
            const F3 v = div3(sub3(add3(mv3(Rcw, ray), t_cw), origin), vs);
            lo = mk3(v.x < lo.x ? v.x : lo.x, v.y < lo.y ? v.y : lo.y, v.z < lo.z ? v.z : lo.z);
            hi = mk3(hi.x < v.x ? v.x : hi.x, hi.y < v.y ? v.y : hi.y, hi.z < v.z ? v.z : hi.z);
        }
        ic.valid = finite3(lo) && finite3(hi);
        auto clampIdx = [res](float f) {
            const float top = static_cast<float>(res - 1);
            const float a = f < top ? f : top;
            return static_cast<int>(a > 0.0f ? a : 0.0f);
        };
        ic.x0 = ic.valid ? clampIdx(floorf(lo.x)) : 0;
        ic.x1 = ic.valid ? clampIdx(ceilf(hi.x)) : -1;
        ic.y0 = ic.valid ? clampIdx(floorf(lo.y)) : 0;
        ic.y1 = ic.valid ? clampIdx(ceilf(hi.y)) : -1;
        ic.z0 = ic.valid ? clampIdx(floorf(lo.z)) : 0;
        ic.z1 = ic.valid ? clampIdx(ceilf(hi.z)) : -1;
        ic.step_x[0] = fm(ic.R_wc[0], vs);
        ic.step_x[1] = fm(ic.R_wc[3], vs);
        ic.step_x[2] = fm(ic.R_wc[6], vs);
        // Bounds for the chunk culling. cmax bounds |c_i| over the AABB (c is
        // affine in the voxel index, so a corner attains it), with slack for
        // the stepped sums. A stepped coordinate then stays within
        // 31 * ulp(cmax) / 2 of the line through its chunk start, and cull_eps
        // is twice that and more. A voxel nearer than z_safe may project more
        // than one pixel away from that line.
        float cmax = 0.0f;
        for (int k = 0; k < 8; ++k) {
            const float px = ox + vs * static_cast<float>((k & 1) ? ic.x1 + 1 : ic.x0);
            const float py = oy + vs * static_cast<float>((k & 2) ? ic.y1 + 1 : ic.y0);
            const float pz = oz + vs * static_cast<float>((k & 4) ? ic.z1 + 1 : ic.z0);
            const F3 c = add3(mv3(ic.R_wc, mk3(px, py, pz)), t_wc);
            cmax = fmaxf(cmax, fmaxf(fabsf(c.x), fmaxf(fabsf(c.y), fabsf(c.z))));
        }
        cmax = cmax * 1.01f + 1e-3f;
        const float eps = 40.0f * cmax * 1.1920929e-7f;  // 40 * 2^-23 * cmax
        const float unx = (fmaxf(fabsf(cx), fabsf(float(W) - cx)) + 3.0f) / fx;
        const float uny = (fmaxf(fabsf(cy), fabsf(float(H) - cy)) + 3.0f) / fy;
        ic.cull_eps = eps;
        ic.cull_off = trunc + eps + 1e-5f;
        // A row's stepped coordinate after k steps differs from the exact
        // affine value by at most k rounding errors of ulp(cmax) / 2 each, the
        // rounding of the step itself k times, and a few ulps of the start
        // (and of the brick corners computed here): (res + 64) ulps, times 1.5.
        const float eps_b = 1.5f * static_cast<float>(res + 64) * 2.0f * cmax * 1.1920929e-7f;
        ic.brick_eps = eps_b;
        ic.brick_off = trunc + eps_b + 1e-5f;
        ic.z_safe = fmaxf(1e-3f, 2.0f * eps * (fmaxf(fx * (1.0f + unx), fy * (1.0f + uny)) + 2.0f));
        if (!(isfinite(ic.cull_off) && isfinite(ic.z_safe))) ic.z_safe = __int_as_float(0x7f800000);
        *out = ic;
        counters[1] = 0;
        counters[2] = 0;
        counters[4] = 0;  // next warp item of the integrate kernel
        for (int b = 0; b < kIntBuckets; ++b) counters[5 + b] = 0;
    }
    if (pyramid) build_tile_pyramid(tiles, mip);
}
__global__ void integrate_setup_kernel(const float* __restrict__ d_pose, int res, float vs, float ox, float oy,
                                       float oz, float trunc, float fx, float fy, float cx, float cy, int W, int H,
                                       float max_d, IntegrateConsts* out, unsigned long long* counters,
                                       float* __restrict__ tiles, TileMip mip, int pyramid) {
    integrate_setup_body(d_pose, res, vs, ox, oy, oz, trunc, fx, fy, cx, cy, W, H, max_d, out, counters, tiles, mip,
                         pyramid != 0);
}

// Brick pre-cull: one bit per 8^3 brick, set unless no voxel of the brick can
// take an update this frame. Every voxel's stepped camera coordinate lies
// within brick_eps of the parallelepiped spanned by the brick's corner
// voxels, so with every corner at least z_near in front of the camera, each
// voxel projects inside the corners' pixel box widened by the rounding
// margins of the exact projection (-2 / +3 pixels, as the chunk cull) and by
// brick_eps times the projection's slope; its depth there is at most the
// deepest in-band depth of the tiles under the box, and a voxel farther
// than that plus trunc gets sdf < -trunc. A brick with every corner at or
// behind the camera plane (c.z <= 0 for all its voxels) or whose box misses
// the image takes no update either. Everything else is kept (conservative).
// One warp per 32 consecutive bricks of a row, written with one ballot.
constexpr float kBrickNear = 1e-2f;  // corners nearer than this: no projection bound
constexpr int kBrickFine = 8;        // level-0 tiles a side read one by one before a coarser level is used
__global__ void __launch_bounds__(256) integrate_bricks_kernel(
    const IntegrateConsts* __restrict__ icp, int res, int nb, int words, float vs, float ox, float oy, float oz,
    float fx, float fy, float cx, float cy, int W, int H, const float* __restrict__ tiles, TileMip mip,
    const int* __restrict__ gate, uint32_t* __restrict__ live) {
    if (gate && __ldg(gate) == 0) return;
    const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int row = gw / words, word = gw - row * words;
    if (row >= nb * nb) return;
    const int bz = row / nb, by = row - bz * nb, bx = word * 32 + lane;
    bool on = false;
    if (__ldg(&icp->valid) && bx < nb) {
        const int xa = bx << kBrickShift, ya = by << kBrickShift, za = bz << kBrickShift;
        const int xb = min(xa + 7, res - 1), yb = min(ya + 7, res - 1), zb = min(za + 7, res - 1);
        on = !(xb < __ldg(&icp->x0) || xa > __ldg(&icp->x1) || yb < __ldg(&icp->y0) || ya > __ldg(&icp->y1) ||
               zb < __ldg(&icp->z0) || za > __ldg(&icp->z1));
        if (on) {
            float R[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) R[i] = __ldg(&icp->R_wc[i]);
            const float tx = __ldg(&icp->t_wc[0]), ty = __ldg(&icp->t_wc[1]), tz = __ldg(&icp->t_wc[2]);
            const float eps = __ldg(&icp->brick_eps);
            float zlo = __int_as_float(0x7f800000), zhi = -zlo, ulo = zlo, uhi = -zlo, vlo = zlo, vhi = -zlo;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float px = ox + vs * static_cast<float>((k & 1) ? xb : xa);
                const float py = oy + vs * static_cast<float>((k & 2) ? yb : ya);
                const float pz = oz + vs * static_cast<float>((k & 4) ? zb : za);
                const float c0 = fmaf(R[0], px, fmaf(R[1], py, fmaf(R[2], pz, tx)));
                const float c1 = fmaf(R[3], px, fmaf(R[4], py, fmaf(R[5], pz, ty)));
                const float c2 = fmaf(R[6], px, fmaf(R[7], py, fmaf(R[8], pz, tz)));
                zlo = fminf(zlo, c2);
                zhi = fmaxf(zhi, c2);
                // a bound: the approximate quotient (2 ulp) is covered by the margins below
                const float u = __fdividef(fx * c0, c2) + cx, v = __fdividef(fy * c1, c2) + cy;
                ulo = fminf(ulo, u);
                uhi = fmaxf(uhi, u);
                vlo = fminf(vlo, v);
                vhi = fmaxf(vhi, v);
            }
            zlo -= eps;
            zhi += eps;
            if (zhi <= 0.0f) {
                on = false;  // every voxel has c.z <= 0
            } else if (zlo >= kBrickNear) {
                // the projection moves by at most eps (f + |u - c|) / z for a move of eps
                const float du = eps * (fx + fmaxf(fabsf(ulo - cx), fabsf(uhi - cx))) / zlo + 1e-3f;
                const float dv = eps * (fy + fmaxf(fabsf(vlo - cy), fabsf(vhi - cy))) / zlo + 1e-3f;
                const float fW = static_cast<float>(W), fH = static_cast<float>(H);
                ulo -= 2.0f + du;
                uhi += 3.0f + du;
                vlo -= 2.0f + dv;
                vhi += 3.0f + dv;
                if (!(uhi >= 0.0f && ulo < fW && vhi >= 0.0f && vlo < fH)) {
                    on = false;  // the box misses the image (NaN bounds fail the other tests and keep the brick)
                } else if (isfinite(ulo) && isfinite(uhi) && isfinite(vlo) && isfinite(vhi)) {
                    const int tu0 = static_cast<int>(fmaxf(ulo, 0.0f)) >> kTileShift;
                    const int tu1 = static_cast<int>(fminf(uhi, fW - 1.0f)) >> kTileShift;
                    const int tv0 = static_cast<int>(fmaxf(vlo, 0.0f)) >> kTileShift;
                    const int tv1 = static_cast<int>(fminf(vhi, fH - 1.0f)) >> kTileShift;
                    float tm = -__int_as_float(0x7f800000);
                    if (tu1 - tu0 < kBrickFine && tv1 - tv0 < kBrickFine) {
                        const int w0 = mip.w[0];
                        for (int a = tv0; a <= tv1; ++a)
                            for (int b = tu0; b <= tu1; ++b) tm = fmaxf(tm, __ldg(tiles + a * w0 + b));
                    } else {
                        const int ext = max(tu1 - tu0, tv1 - tv0);
                        const int l = min(32 - __clz(ext), mip.levels - 1);
                        const int w = mip.w[l];
                        const float* tl = tiles + mip.off[l];
                        const int a0 = (tv0 >> l) * w, a1 = (tv1 >> l) * w, b0 = tu0 >> l, b1 = tu1 >> l;
                        tm = fmaxf(fmaxf(__ldg(tl + a0 + b0), __ldg(tl + a0 + b1)),
                                   fmaxf(__ldg(tl + a1 + b0), __ldg(tl + a1 + b1)));
                    }
                    on = !(zlo > tm + __ldg(&icp->brick_off));
                }
            }
        }
    }
    const unsigned bits = __ballot_sync(0xffffffffu, on);
    if (lane == 0) live[static_cast<size_t>(row) * words + word] = bits;
}

// Work list of the integration: every item (32 rows at one z, one x-part)
// with a kept brick in its rows and part goes into the bucket of its
// kept-brick count, so that the persistent kernel can take the heaviest items
// first: an item's cost grows with its kept bricks, and items differ by two
// orders of magnitude, so an item started last would otherwise set the end.
// Order within a bucket is arbitrary: every item writes its own voxels and
// the counters are integer sums, so the results do not depend on it.
__global__ void __launch_bounds__(256) integrate_list_kernel(const IntegrateConsts* __restrict__ icp, int res,
                                                             int nb, int words, int nparts,
                                                             const uint32_t* __restrict__ live,
                                                             const int* __restrict__ gate,
                                                             unsigned long long* __restrict__ counters,
                                                             int* __restrict__ list) {
    if (gate && __ldg(gate) == 0) return;
    const int ngroups = (res + 31) >> 5;
    const int n_items = res * ngroups * nparts;
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= n_items || !__ldg(&icp->valid)) return;
    const int part = item % nparts, it = item / nparts;
    const int z = it / ngroups, ybase = (it - z * ngroups) << 5;
    const int z0 = __ldg(&icp->z0), z1 = __ldg(&icp->z1), y0 = __ldg(&icp->y0), y1 = __ldg(&icp->y1);
    if (z < z0 || z > z1 || ybase + 31 < y0 || ybase > y1) return;
    const int span = (((res + nparts - 1) / nparts) + 31) & ~31;
    const int xpart = part * span;
    if (xpart >= res) return;
    const int ba = xpart >> kBrickShift, bb = min((xpart + span) >> kBrickShift, nb);  // bricks [ba, bb)
    int cost = 0;
    for (int r = 0; r < 4; ++r) {
        const int ya = ybase + 8 * r;
        if (ya > y1 || ya + 7 < y0 || ya >= res) continue;
        const uint32_t* rowp = live + (static_cast<size_t>(z >> kBrickShift) * nb + (ya >> kBrickShift)) * words;
        for (int w = ba >> 5; w <= (bb - 1) >> 5; ++w) {
            uint32_t m = __ldg(rowp + w);
            const int lo = max(ba - 32 * w, 0), hi = min(bb - 32 * w, 32);  // bits [lo, hi)
            m &= (hi >= 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
            cost += __popc(m);
        }
    }
    if (!cost) return;
    // buckets by the bit length of the count, heaviest (most bricks) first
    const int b = max(0, kIntBuckets - (32 - __clz(cost)));
    const unsigned long long k = atomicAdd(&counters[5 + b], 1ull);
    list[static_cast<size_t>(b) * n_items + k] = item;
}

// fs_walk kept out of line (it runs once per item, not per voxel).
__device__ __noinline__ float fs_walk_far(float v, float s, int n) { return fs_walk(v, s, n); }

// A hint to load the 128-byte line holding p into L2 (p must be a valid address).
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Voxel-projective integration (TSDFVolume.cpp:282-329).
//
// The CPU steps the camera coordinate of a voxel row incrementally along x
// (c += R_wc.col(0) * vs from the AABB start x0), so the pixel a voxel lands in
// depends on that rounded running sum. A warp owns 32 voxel rows (32
// consecutive y at one z) and walks them in chunks of 32 x:
//   cull  (lane = row): the chunk's voxels lie within cull_eps of a segment;
//          project its ends, take the deepest depth over the pixels the segment
//          can reach (two tiles a side at the pyramid level that fits) and drop
//          the chunk if its nearest voxel is beyond it by more than trunc;
//   chain (lane = row): replay the sequential c-steps, parking c of live rows
//          in shared memory;
//   update (lane = x): for each live row, project every voxel exactly, gather
//          its depth and read-modify-write the voxel, all coalesced (a per-voxel
//          tile test before the gather only lengthened the dependent chain).
// Every test is exact or conservative, so the updated set and the values are
// the CPU's. Voxels that take no update are never read: HBM traffic is
// 2 x record size per updated voxel.
// One warp item (32 rows at one z) of one volume; s_c is the block's staging
// array, indexed by the warp.
template <bool kHalf, bool kColor, bool kResid>
__device__ __forceinline__ void integrate_item(
    void* __restrict__ vox, float* __restrict__ color, const IntegrateConsts* __restrict__ icp,
    const float* __restrict__ depth, const uint8_t* __restrict__ rgb, int res, float vs, float ox, float oy,
    float oz, float trunc, float max_w, float fx, float fy, float cx, float cy, int W, int H, float min_d,
    float max_d, const int* __restrict__ gate, unsigned long long* __restrict__ counters, uint8_t* bricks, int nb,
    const float* __restrict__ tiles, const TileMip& mip, int item, int warp, int lane, float (*s_c)[3][32][33],
    int nparts = 1, const uint32_t* __restrict__ live = nullptr, int live_words = 0) {
    if (gate && __ldg(gate) == 0) return;
    if (!__ldg(&icp->valid)) return;
    const int ngroups = (res + 31) >> 5;
    // the item's part of the rows: x in [part * span, (part + 1) * span)
    const int part = item % nparts;
    item /= nparts;
    const int span = (((res + nparts - 1) / nparts) + 31) & ~31;
    if (item >= res * ngroups) return;
    const int z = item / ngroups;
    const int ybase = (item - z * ngroups) << 5;
    const int z0 = __ldg(&icp->z0), z1 = __ldg(&icp->z1), y0 = __ldg(&icp->y0), y1 = __ldg(&icp->y1);
    if (z < z0 || z > z1 || ybase + 31 < y0 || ybase > y1) return;
    const int y = ybase + lane;
    const bool row_on = (y >= y0 && y <= y1);
    // Chunks of this part (chunk j: x in [xpart + 32 j, +32)) that the brick
    // pre-cull keeps for this row: one of the chunk's 4 bricks is kept. The
    // item ends here when no row has one.
    const int xpart = part * span;
    const int nch = (min(span, res - xpart) + 31) >> 5;
    if (nch <= 0) return;
    const int b0 = xpart >> kBrickShift;  // a multiple of 4: chunks never straddle a mask word
    const uint32_t* rowp = nullptr;
    unsigned rmask = row_on ? 0xffffffffu : 0u;
    if (live && row_on) {
        rmask = 0;
        rowp = live + (static_cast<size_t>(z >> kBrickShift) * nb + (y >> kBrickShift)) * live_words;
        uint32_t word = 0;
        int wi = -1;
        for (int j = 0; j < nch; ++j) {
            const int b = b0 + 4 * j;
            if ((b >> 5) != wi) {
                wi = b >> 5;
                word = __ldg(rowp + wi);
            }
            if ((word >> (b & 31)) & 0xfu) rmask |= 1u << j;
        }
    }
    if (!__reduce_or_sync(0xffffffffu, rmask)) return;
    const int x0 = __ldg(&icp->x0), x1 = __ldg(&icp->x1);
    float R[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = __ldg(&icp->R_wc[i]);
    const F3 t_wc = mk3(__ldg(&icp->t_wc[0]), __ldg(&icp->t_wc[1]), __ldg(&icp->t_wc[2]));
    const F3 step = mk3(__ldg(&icp->step_x[0]), __ldg(&icp->step_x[1]), __ldg(&icp->step_x[2]));
    const float cull_eps = __ldg(&icp->cull_eps), cull_off = __ldg(&icp->cull_off), z_safe = __ldg(&icp->z_safe);

    F3 c = add3(mv3(R, add3(mk3(ox, oy, oz), mul3(mk3(float(x0), float(y), float(z)), vs))), t_wc);
    const float fW = static_cast<float>(W), fH = static_cast<float>(H);
    const float color_band = fm(0.5f, trunc);
    unsigned n_new = 0, n_upd = 0, n_col = 0;  // per lane: at most 32 rows x 32 chunks
    const size_t rr = static_cast<size_t>(res);

    // Conservative x-interval of this row that can land in front of the camera
    // and inside the image: c(t) = c(x0) + t step is linear, so each of
    // c.z > 0, 0 <= u, u < W, 0 <= v, v < H is a half-line in t (u, v times c.z
    // are linear). Solved in float, every bound widened by the rounding of its
    // coefficients (2^-21 relative, four times the worst case) and by 2
    // voxels, far more than the rounding of the stepped coordinate can move a
    // projection; a constraint whose direction rounding cannot settle is
    // dropped. Outside the interval a voxel only advances the coordinate,
    // exactly as the sequential sweep does.
    int xs = x1 + 1, xe = x0 - 1;
    if (row_on) {
        const float tmax = static_cast<float>(x1 - x0);
        float lo = 0.0f, hi = tmax;
        constexpr float kRel = 4.76837158e-7f;  // 2^-21
        auto keep = [&](float p1, float p2, float q1, float q2) {  // keep t with (p1 + p2) + (q1 + q2) t >= 0
            const float a = p1 + p2, b = q1 + q2;
            const float ea = kRel * (fabsf(p1) + fabsf(p2)), eb = kRel * (fabsf(q1) + fabsf(q2));
            if (!(fabsf(b) > eb)) {
                if (a + ea + (fabsf(b) + eb) * tmax < 0.0f) { lo = 1.0f; hi = 0.0f; }
                return;
            }
            const float t = -a / b;
            const float err = (ea + fabsf(t) * eb) / fabsf(b) + fabsf(t) * kRel;
            if (b > 0.0f) lo = fmaxf(lo, t - err);
            else hi = fminf(hi, t + err);
        };
        const float cu = cx + 0.5f, cv = cy + 0.5f;
        keep(c.z, 0.0f, step.z, 0.0f);
        keep(fx * c.x, cu * c.z, fx * step.x, cu * step.z);
        keep(-(fx * c.x), -((cu - fW) * c.z), -(fx * step.x), -((cu - fW) * step.z));
        keep(fy * c.y, cv * c.z, fy * step.y, cv * step.z);
        keep(-(fy * c.y), -((cv - fH) * c.z), -(fy * step.y), -((cv - fH) * step.z));
        if (lo <= hi + 4.0f) {
            xs = max(x0, x0 + static_cast<int>(floorf(lo)) - 2);
            xe = min(x1, x0 + static_cast<int>(ceilf(hi)) + 2);
        }
    }
    int wxs = xs, wxe = xe;
    for (int o = 16; o > 0; o >>= 1) {
        wxs = min(wxs, __shfl_xor_sync(0xffffffffu, wxs, o));
        wxe = max(wxe, __shfl_xor_sync(0xffffffffu, wxe, o));
    }
    wxs = max(wxs, part * span);
    wxe = min(wxe, (part + 1) * span - 1);
    if (wxs > wxe) return;  // no row of this warp reaches the image in this part
    // the chunks to visit: kept by the brick pre-cull for some row and inside
    // the warp's image interval
    const int jfirst = (wxs - xpart) >> 5, jlast = (wxe - xpart) >> 5;
    unsigned todo = __reduce_or_sync(0xffffffffu, rmask);
    todo &= (jlast >= 31 ? 0xffffffffu : ((2u << jlast) - 1u)) & ~((1u << jfirst) - 1u);
    int xat = x0;  // the x the lanes' c belongs to

    while (todo) {
        const int j = __ffs(todo) - 1;
        todo &= todo - 1;
        const int xc = xpart + 32 * j;
        {
            // skipped chunks: the sequential steps from xat to this chunk,
            // replayed exactly by the closed form of the running float sum
            // (fstep.cuh)
            const int target = max(xc, x0);
            if (target > xat) {
                const int n0 = target - xat;
                if (row_on)
                    c = mk3(fs_walk_far(c.x, step.x, n0), fs_walk_far(c.y, step.y, n0), fs_walk_far(c.z, step.z, n0));
                xat = target;
            }
        }
        // cull (lane = row), per kCullSeg-voxel piece of the chunk so each
        // piece's pixels fit a finer tile level, for rows whose bricks the
        // pre-cull kept. The lane's c belongs to x = max(xc, x0).
        bool live = false;
        if (row_on && ((rmask >> j) & 1u)) {
            const uint32_t nib =
                rowp ? (__ldg(rowp + ((b0 + 4 * j) >> 5)) >> ((b0 + 4 * j) & 31)) & 0xfu : 0xfu;
            const int xcur = max(xc, x0);
            const int xa = max(xcur, xs), xb = min(min(xc + 31, x1), xe);
            auto piece_live = [&](int pa, int pb) {
                const float ka = static_cast<float>(pa - xcur), kb = static_cast<float>(pb - xcur);
                const F3 ca = mk3(fmaf(ka, step.x, c.x), fmaf(ka, step.y, c.y), fmaf(ka, step.z, c.z));
                const F3 cb = mk3(fmaf(kb, step.x, c.x), fmaf(kb, step.y, c.y), fmaf(kb, step.z, c.z));
                if (!(ca.z >= z_safe && cb.z >= z_safe)) return true;  // near or behind the camera plane: no bound
                const float ua = fx * __fdividef(ca.x, ca.z) + cx, ub = fx * __fdividef(cb.x, cb.z) + cx;
                const float va = fy * __fdividef(ca.y, ca.z) + cy, vb = fy * __fdividef(cb.y, cb.z) + cy;
                const float ulo = fminf(ua, ub) - 2.0f, uhi = fmaxf(ua, ub) + 3.0f;
                const float vlo = fminf(va, vb) - 2.0f, vhi = fmaxf(va, vb) + 3.0f;
                if (!(uhi >= 0.0f && ulo < fW && vhi >= 0.0f && vlo < fH)) return false;
                const int iu0 = static_cast<int>(fmaxf(ulo, 0.0f));
                const int iu1 = static_cast<int>(fminf(uhi, fW - 1.0f));
                const int iv0 = static_cast<int>(fmaxf(vlo, 0.0f));
                const int iv1 = static_cast<int>(fminf(vhi, fH - 1.0f));
                const int tu0 = iu0 >> kTileShift, tu1 = iu1 >> kTileShift;
                const int tv0 = iv0 >> kTileShift, tv1 = iv1 >> kTileShift;
                float tm;
                if (tu1 - tu0 < kFineSide && tv1 - tv0 < kFineSide) {
                    // every level-0 tile of the box, all loads in flight together
                    const int w0 = mip.w[0];
                    float t[kFineSide * kFineSide];
#pragma unroll
                    for (int a = 0; a < kFineSide; ++a)
#pragma unroll
                        for (int b = 0; b < kFineSide; ++b)
                            t[a * kFineSide + b] = (tv0 + a <= tv1 && tu0 + b <= tu1)
                                                       ? __ldg(tiles + (tv0 + a) * w0 + tu0 + b)
                                                       : -__int_as_float(0x7f800000);
                    tm = t[0];
#pragma unroll
                    for (int i = 1; i < kFineSide * kFineSide; ++i) tm = fmaxf(tm, t[i]);
                } else {
                    // two tiles a side at the level that fits
                    const int ext = max(iu1 - iu0, iv1 - iv0) >> kTileShift;
                    const int l = min(ext ? 32 - __clz(ext) : 0, mip.levels - 1);
                    const int sh = kTileShift + l, w = mip.w[l];
                    const float* tl = tiles + mip.off[l];
                    const int a0 = (iv0 >> sh) * w, a1 = (iv1 >> sh) * w, b0 = iu0 >> sh, b1 = iu1 >> sh;
                    tm = fmaxf(fmaxf(__ldg(tl + a0 + b0), __ldg(tl + a0 + b1)),
                               fmaxf(__ldg(tl + a1 + b0), __ldg(tl + a1 + b1)));
                }
                return !(fminf(ca.z, cb.z) > tm + cull_off);
            };
            for (int pa = xa; pa <= xb && !live; pa += kCullSeg) {
                const int pb = min(pa + kCullSeg - 1, xb);
                const int lo = (pa - xc) >> kBrickShift, hi = (pb - xc) >> kBrickShift;  // the piece's bricks
                if (nib & ((2u << hi) - (1u << lo))) live = piece_live(pa, pb);
            }
        }
        const unsigned live_rows = __ballot_sync(0xffffffffu, live);
        if (!live_rows) continue;  // c stays at xat; the next chunk's jump covers this one
        if (live) {
            // pull the row's voxel records of this chunk into L2 now: the
            // update reads them after the chain, so their DRAM latency overlaps
            // it (4% of the stage on c2)
            const size_t rbase = (static_cast<size_t>(z) * rr + static_cast<size_t>(y)) * rr;
            const size_t es = (kHalf || kResid) ? 4 : 8;
            const char* pa = static_cast<const char*>(vox) + (rbase + max(xc, x0)) * es;
            const char* pb = static_cast<const char*>(vox) + (rbase + min(xc + 31, x1)) * es;
            prefetch_l2(pa);
            if ((reinterpret_cast<uintptr_t>(pa) >> 7) != (reinterpret_cast<uintptr_t>(pb) >> 7)) prefetch_l2(pb);
        }
        // chain (lane = row): the sequential c-steps of the chunk
        if (row_on) {
            if (xc >= x0 && xc + 31 <= x1) {
                if (live) {
#pragma unroll 8
                    for (int k = 0; k < 32; ++k) {
                        s_c[warp][0][lane][k] = c.x;
                        s_c[warp][1][lane][k] = c.y;
                        s_c[warp][2][lane][k] = c.z;
                        c = add3(c, step);
                    }
                } else {
#pragma unroll 8
                    for (int k = 0; k < 32; ++k) c = add3(c, step);
                }
            } else {
                for (int k = 0; k < 32; ++k) {
                    const int x = xc + k;
                    if (x >= x0 && x <= x1) {
                        if (live) {
                            s_c[warp][0][lane][k] = c.x;
                            s_c[warp][1][lane][k] = c.y;
                            s_c[warp][2][lane][k] = c.z;
                        }
                        c = add3(c, step);
                    }
                }
            }
        }
        xat = min(max(xc + 32, x0), x1 + 1);
        __syncwarp();
        // update (lane = x): live rows in groups of kUpdGroup, software
        // pipelined: the projection and depth gather of the next group are
        // issued before the voxel read-modify-write of this one, so the two
        // dependent load latencies overlap.
        const int x = xc + lane;
        const bool x_on = x >= x0 && x <= x1;
        // voxel (x, ybase + r, z) = vrow + r * res
        const size_t vrow =
            (static_cast<size_t>(z) * rr + static_cast<size_t>(ybase)) * rr + static_cast<size_t>(x);
        unsigned rem = live_rows;
        int ra[kUpdGroup], pa[kUpdGroup];
        float za[kUpdGroup], da[kUpdGroup];
        auto gather = [&]() {  // next group: rows, pixels (-1: none), camera z, depth
#pragma unroll
            for (int j = 0; j < kUpdGroup; ++j) {
                ra[j] = rem ? __ffs(rem) - 1 : -1;
                rem &= rem - 1;
            }
#pragma unroll
            for (int j = 0; j < kUpdGroup; ++j) {
                pa[j] = -1;
                za[j] = 0.0f;
                if (ra[j] >= 0 && x_on) {
                    const F3 cv = mk3(s_c[warp][0][ra[j]][lane], s_c[warp][1][ra[j]][lane], s_c[warp][2][ra[j]][lane]);
                    if (cv.z > 0.0f) {
                        const float inv_z = __frcp_rn(cv.z);  // == 1.0f / c.z, correctly rounded
                        const float uf = floorf(fa(fa(fm(fm(fx, cv.x), inv_z), cx), 0.5f));
                        const float vf = floorf(fa(fa(fm(fm(fy, cv.y), inv_z), cy), 0.5f));
                        if (uf >= 0.0f && uf < fW && vf >= 0.0f && vf < fH) {
                            pa[j] = static_cast<int>(vf) * W + static_cast<int>(uf);
                            za[j] = cv.z;
                        }
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < kUpdGroup; ++j) da[j] = pa[j] >= 0 ? __ldg(depth + pa[j]) : 0.0f;
        };
        gather();
#pragma unroll 1
        while (ra[0] >= 0) {
            int rsel[kUpdGroup], pix[kUpdGroup];
            float cz[kUpdGroup], sdf[kUpdGroup];
#pragma unroll
            for (int j = 0; j < kUpdGroup; ++j) {
                rsel[j] = ra[j];
                pix[j] = pa[j];
                cz[j] = za[j];
                sdf[j] = da[j];
            }
            gather();  // the next group's loads are in flight during this group's update
#pragma unroll
            for (int j = 0; j < kUpdGroup; ++j) {
                const float d = sdf[j];
                bool ok = false;
                if (pix[j] >= 0 && d >= min_d && d <= max_d) {
                    sdf[j] = fs(d, cz[j]);
                    ok = !(sdf[j] < -trunc);
                }
                if (!ok) pix[j] = -1;
            }
            float2 old[kUpdGroup];
#pragma unroll
            for (int j = 0; j < kUpdGroup; ++j) {
                const size_t v = vrow + static_cast<size_t>(rsel[j]) * rr;
                if (pix[j] >= 0) old[j] = kResid ? VoxR::load_fold(vox, v) : Vox<kHalf>::load_rw(vox, v);
            }
#pragma unroll
            for (int j = 0; j < kUpdGroup; ++j) {
                if (pix[j] < 0) continue;
                const size_t vi = vrow + static_cast<size_t>(rsel[j]) * rr;
                // min(1, sdf / trunc) is exactly 1 for sdf >= trunc (a rounded
                // quotient of operands in that order is >= 1): free space needs
                // no division
                const float tsdf_new = sdf[j] >= trunc ? 1.0f : fminf(1.0f, fd(sdf[j], trunc));
                const float w_old = old[j].y;
                n_new += (w_old == 0.0f);
                ++n_upd;
                const float wp1 = fa(w_old, 1.0f);
                // (1 w + 1) / (w + 1) is exactly 1 for an integer-valued weight:
                // folding free space into free space needs no division either
                const float t = (old[j].x == 1.0f && tsdf_new == 1.0f) ? 1.0f
                                                                       : fd(fa(fm(old[j].x, w_old), tsdf_new), wp1);
                const float w = fminf(wp1, max_w);
                if (kResid) VoxR::store(vox, vi, t, w);
                else Vox<kHalf>::store(vox, vi, t, w);
                if (bricks && !(Vox<kHalf>::rounded(t) >= kFreeTsdf)) clear_bricks(bricks, nb, x, ybase + rsel[j], z);
                if (kColor) {
                    if (rgb != nullptr && fabsf(sdf[j]) < color_band) {
                        const int p = pix[j];
                        const float inv = fd(1.0f, wp1);
                        float* cvp = color + 3 * vi;
#pragma unroll
                        for (int k = 0; k < 3; ++k)
                            cvp[k] = fm(fa(fm(cvp[k], w_old), fd(static_cast<float>(rgb[3 * p + k]), 255.0f)), inv);
                        ++n_col;
                    }
                }
            }
        }
        __syncwarp();
    }
    // warp totals -> global counters
    for (int o = 16; o > 0; o >>= 1) {
        n_new += __shfl_down_sync(0xffffffffu, n_new, o);
        n_upd += __shfl_down_sync(0xffffffffu, n_upd, o);
        n_col += __shfl_down_sync(0xffffffffu, n_col, o);
    }
    if (lane == 0) {
        if (n_new) atomicAdd(&counters[0], static_cast<unsigned long long>(n_new));
        if (n_upd) {
            atomicAdd(&counters[1], static_cast<unsigned long long>(n_upd));
            atomicAdd(&counters[3], static_cast<unsigned long long>(n_upd));
        }
        if (n_col) atomicAdd(&counters[2], static_cast<unsigned long long>(n_col));
    }
}

// Persistent: every warp takes the next item (32 rows at one z) from a counter
// until none is left, so warps whose items are culled early move on instead of
// idling beside a busy warp of their block.
template <bool kHalf, bool kColor, bool kResid>
__global__ void __launch_bounds__(kIntWarps * 32) integrate_kernel(
    void* __restrict__ vox, float* __restrict__ color, const IntegrateConsts* __restrict__ icp,
    const float* __restrict__ depth, const uint8_t* __restrict__ rgb, int res, float vs, float ox, float oy,
    float oz, float trunc, float max_w, float fx, float fy, float cx, float cy, int W, int H, float min_d,
    float max_d, const int* __restrict__ gate, unsigned long long* __restrict__ counters, uint8_t* bricks, int nb,
    const float* __restrict__ tiles, TileMip mip, const uint32_t* __restrict__ live, int live_words,
    const int* __restrict__ list) {
    __shared__ float s_c[kIntWarps][3][32][33];
    if (gate && __ldg(gate) == 0) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_items = res * ((res + 31) >> 5) * kIntParts;
    // bucket b holds positions [s_end[b - 1], s_end[b]) of the work order
    __shared__ int s_end[kIntBuckets];
    if (threadIdx.x == 0) {
        int e = 0;
        for (int b = 0; b < kIntBuckets; ++b) s_end[b] = e += static_cast<int>(__ldcg(&counters[5 + b]));
    }
    __syncthreads();
    const int total = s_end[kIntBuckets - 1];
    for (;;) {
        int pos = 0;
        if (lane == 0) pos = static_cast<int>(atomicAdd(&counters[4], 1ull));
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (pos >= total) break;
        int b = 0;
        while (pos >= s_end[b]) ++b;
        const int item = __ldcg(list + static_cast<size_t>(b) * n_items + (pos - (b ? s_end[b - 1] : 0)));
        integrate_item<kHalf, kColor, kResid>(vox, color, icp, depth, rgb, res, vs, ox, oy, oz, trunc, max_w, fx, fy,
                                              cx, cy, W, H, min_d, max_d, nullptr, counters, bricks, nb, tiles, mip,
                                              item, warp, lane, s_c, kIntParts, live, live_words);
    }
}

// ---- raycast ---------------------------------------------------------------
// State of the brick holding the sample at p: -1 outside the samplable box
// (the sample is invalid), else the brick's free distance: 0 for a brick that
// is not free, d >= 1 when every brick within Chebyshev distance d - 1 is free.
// Same base-voxel arithmetic as sample_tsdf, so the 8 corners of the sample
// are inside the brick's apron.
__device__ __forceinline__ int brick_state(const VolView& v, const uint8_t* __restrict__ dist, int nb, F3 p, int& bx,
                                           int& by, int& bz) {
    const F3 q = to_voxel(v, p);
    const float fx0 = floorf(q.x), fy0 = floorf(q.y), fz0 = floorf(q.z);
    const float lim = static_cast<float>(v.res - 1);
    if (!(fx0 >= 0.0f && fy0 >= 0.0f && fz0 >= 0.0f && fx0 < lim && fy0 < lim && fz0 < lim)) return -1;
    bx = static_cast<int>(fx0) >> kBrickShift;
    by = static_cast<int>(fy0) >> kBrickShift;
    bz = static_cast<int>(fz0) >> kBrickShift;
    return __ldg(dist + (static_cast<size_t>(bz) * nb + by) * nb + bx);
}

// Capped Chebyshev distance of the free flags: d(b) = the smallest Chebyshev
// distance from brick b to a brick that is not free, capped at kDistCap
// (bricks outside the grid count as free). It is separable: three 1-D passes
// out(b) = min over |k| < kDistCap of max(|k|, in(b + k e_axis)), the first
// reading in = 0 for a brick that is not free and kDistCap for a free one
// (brick_field_body runs them in shared memory).
constexpr int kDistCap = 6;

// Ray start map. A march sample whose base voxel lies in a free brick, or
// outside the grid, is skipped, so a ray's far steps are skipped up to the
// first sample in a brick that is not free. Every such brick B (base voxels
// [8B, 8B + 8) a side, its box widened by 0.01 voxel, far above the rounding
// of sample positions) bounds that sample from below: a ray through a pixel
// meets B's box only if the pixel lies in the box's projection, and then not
// before the camera-to-box distance. One thread per brick (in the brick field
// launch below) takes the projection of B's 8 corners, widened by a pixel,
// and lowers the distance bound of every 8x8 pixel tile the projection covers;
// a box that reaches within 1 mm of the camera plane (its projection is
// unbounded) lowers the bound of every tile instead. Bounds are distances less
// 1e-5 relative and 0.1 mm; the raycast keeps two more far steps of margin.
constexpr int kStartShift = 3;  // 8x8 pixel tiles
struct StartMapArgs {
    float vs;
    F3 origin;
    const float* pose;  // camera to world, row-major 4x4
    float fx, fy, cx, cy;
    int W, H;
    uint32_t* smap;
};
__device__ __forceinline__ void ray_start_brick(const StartMapArgs& a, int bx, int by, int bz) {
    float R[9];
    R[0] = __ldg(a.pose + 0); R[1] = __ldg(a.pose + 1); R[2] = __ldg(a.pose + 2);
    R[3] = __ldg(a.pose + 4); R[4] = __ldg(a.pose + 5); R[5] = __ldg(a.pose + 6);
    R[6] = __ldg(a.pose + 8); R[7] = __ldg(a.pose + 9); R[8] = __ldg(a.pose + 10);
    const float co[3] = {__ldg(a.pose + 3), __ldg(a.pose + 7), __ldg(a.pose + 11)};
    const float mg = 0.01f * a.vs, side = 8.0f * a.vs;
    const int b[3] = {bx, by, bz};
    const float o[3] = {a.origin.x, a.origin.y, a.origin.z};
    float lo[3], hi[3], d2 = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = o[k] + side * static_cast<float>(b[k]) - mg - co[k];  // relative to the camera centre
        hi[k] = o[k] + side * static_cast<float>(b[k] + 1) + mg - co[k];
        const float g = fmaxf(fmaxf(lo[k], -hi[k]), 0.0f);
        d2 += g * g;
    }
    const float bound = fmaxf(sqrtf(d2) * (1.0f - 1e-5f) - 1e-4f, 0.0f);
    const uint32_t key = isfinite(bound) ? __float_as_uint(bound) : 0u;
    float umin = __int_as_float(0x7f800000), umax = -umin, vmin = umin, vmax = -umin;
    int front = 0, near_plane = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float px = (k & 1) ? hi[0] : lo[0], py = (k & 2) ? hi[1] : lo[1], pz = (k & 4) ? hi[2] : lo[2];
        // camera coordinates R^T (P - c)
        const float xc = R[0] * px + R[3] * py + R[6] * pz;
        const float yc = R[1] * px + R[4] * py + R[7] * pz;
        const float zc = R[2] * px + R[5] * py + R[8] * pz;
        front += zc > -1e-3f;
        if (!(zc >= 1e-3f)) {
            near_plane = 1;
            continue;
        }
        // a fast quotient: its few ulps are far inside the pixel of margin
        const float u = a.fx * __fdividef(xc, zc) + a.cx, w = a.fy * __fdividef(yc, zc) + a.cy;
        umin = fminf(umin, u); umax = fmaxf(umax, u);
        vmin = fminf(vmin, w); vmax = fmaxf(vmax, w);
    }
    if (!front) return;  // wholly behind the camera: no ray reaches it
    const int tw = (a.W + (1 << kStartShift) - 1) >> kStartShift, th = (a.H + (1 << kStartShift) - 1) >> kStartShift;
    if (near_plane) {
        atomicMin(a.smap + tw * th, key);
        return;
    }
    if (!(umax >= -1.0f && umin <= static_cast<float>(a.W) && vmax >= -1.0f && vmin <= static_cast<float>(a.H))) return;
    // tile ranges as floats first: NaNs and huge values clamp to the image
    const float sc = 1.0f / static_cast<float>(1 << kStartShift);
    const int tx0 = static_cast<int>(fmaxf(floorf((umin - 1.0f) * sc), 0.0f));
    const int tx1 = static_cast<int>(fminf(floorf((umax + 1.0f) * sc), static_cast<float>(tw - 1)));
    const int ty0 = static_cast<int>(fmaxf(floorf((vmin - 1.0f) * sc), 0.0f));
    const int ty1 = static_cast<int>(fminf(floorf((vmax + 1.0f) * sc), static_cast<float>(th - 1)));
    for (int ty = ty0; ty <= ty1; ++ty)
        for (int tx = tx0; tx <= tx1; ++tx) atomicMin(a.smap + ty * tw + tx, key);
}

// The raycast's brick field in one launch: the three passes of the capped
// distance transform run in shared memory over an 8^3 block of bricks and its
// halo of kDistCap - 1 bricks, and the block's bricks that are not free lower
// the ray start map.
constexpr int kFieldSide = 8, kFieldHalo = kDistCap - 1, kFieldExt = kFieldSide + 2 * kFieldHalo;
// The tile (tx, ty, tz) of 8^3 bricks, by a block of 512 threads.
__device__ __forceinline__ void brick_field_body(const uint8_t* __restrict__ flags, uint8_t* __restrict__ dist, int nb,
                                                 const StartMapArgs& sm, int tx, int ty, int tz) {
    __shared__ uint8_t s_in[kFieldExt][kFieldExt][kFieldExt];    // [z][y][x]: 0 not free, kDistCap free or outside
    __shared__ uint8_t s_x[kFieldExt][kFieldExt][kFieldSide];    // after the x pass
    __shared__ uint8_t s_y[kFieldExt][kFieldSide][kFieldSide];   // after the y pass
    const int x0 = tx * kFieldSide - kFieldHalo, y0 = ty * kFieldSide - kFieldHalo, z0 = tz * kFieldSide - kFieldHalo;
    for (int i = threadIdx.x; i < kFieldExt * kFieldExt * kFieldExt; i += blockDim.x) {
        const int lx = i % kFieldExt, ly = (i / kFieldExt) % kFieldExt, lz = i / (kFieldExt * kFieldExt);
        const int gx = x0 + lx, gy = y0 + ly, gz = z0 + lz;
        uint8_t val = kDistCap;
        if (gx >= 0 && gx < nb && gy >= 0 && gy < nb && gz >= 0 && gz < nb)
            val = __ldg(flags + (static_cast<size_t>(gz) * nb + gy) * nb + gx) ? kDistCap : 0;
        s_in[lz][ly][lx] = val;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kFieldExt * kFieldExt * kFieldSide; i += blockDim.x) {
        const int lx = i % kFieldSide, ly = (i / kFieldSide) % kFieldExt, lz = i / (kFieldSide * kFieldExt);
        int d = kDistCap;
#pragma unroll
        for (int k = -kFieldHalo; k <= kFieldHalo; ++k) d = min(d, max(abs(k), int(s_in[lz][ly][lx + kFieldHalo + k])));
        s_x[lz][ly][lx] = static_cast<uint8_t>(d);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kFieldExt * kFieldSide * kFieldSide; i += blockDim.x) {
        const int lx = i % kFieldSide, ly = (i / kFieldSide) % kFieldSide, lz = i / (kFieldSide * kFieldSide);
        int d = kDistCap;
#pragma unroll
        for (int k = -kFieldHalo; k <= kFieldHalo; ++k) d = min(d, max(abs(k), int(s_x[lz][ly + kFieldHalo + k][lx])));
        s_y[lz][ly][lx] = static_cast<uint8_t>(d);
    }
    __syncthreads();
    const int lx = threadIdx.x % kFieldSide, ly = (threadIdx.x / kFieldSide) % kFieldSide,
              lz = threadIdx.x / (kFieldSide * kFieldSide);
    const int gx = x0 + kFieldHalo + lx, gy = y0 + kFieldHalo + ly, gz = z0 + kFieldHalo + lz;
    if (lz >= kFieldSide || gx >= nb || gy >= nb || gz >= nb) return;
    int d = kDistCap;
#pragma unroll
    for (int k = -kFieldHalo; k <= kFieldHalo; ++k) d = min(d, max(abs(k), int(s_y[lz + kFieldHalo + k][ly][lx])));
    dist[(static_cast<size_t>(gz) * nb + gy) * nb + gx] = static_cast<uint8_t>(d);
    if (sm.smap && s_in[lz + kFieldHalo][ly + kFieldHalo][lx + kFieldHalo] == 0) ray_start_brick(sm, gx, gy, gz);
}
__global__ void __launch_bounds__(512) brick_field_kernel(const uint8_t* __restrict__ flags, uint8_t* __restrict__ dist,
                                                          int nb, StartMapArgs sm, const int* __restrict__ gate) {
    if (gate && __ldg(gate) == 0) return;
    brick_field_body(flags, dist, nb, sm, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Fast-forward through free space. From a sample t whose brick b has free
// distance r + 1, every brick of the cube b +- r is free, and the march takes
// far steps t_k = t + k step (each sum rounded) whose samples in the cube are
// all skipped anyway. While the sums stay in t's binade [2^e, 2^(e+1)) and
// step is not a rounding tie there, each one adds the same delta =
// RN(t + step) - t exactly, so t_m = t + m delta in one exact fma. m stops one
// step short of the cube's exit (its box shrunk by 4e-3 voxel, far above the
// rounding of positions), of t_far and of the binade's end. Returns t when no
// step can be taken this way.
__device__ __forceinline__ float free_space_jump(const VolView& v, F3 co, F3 inv_dir, float t, float step,
                                                 float t_far, int bx, int by, int bz, int r) {
    const float span = 8.0f * v.vs, mg = 4e-3f * v.vs;
    const int b[3] = {bx, by, bz};
    float t_exit = t_far;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float ia = comp(inv_dir, a);
        if (!(fabsf(ia) < __int_as_float(0x7f800000))) continue;  // ray parallel to this axis
        const float face = ia > 0.0f ? comp(v.origin, a) + span * static_cast<float>(b[a] + r + 1) - mg
                                     : comp(v.origin, a) + span * static_cast<float>(b[a] - r) + mg;
        t_exit = fminf(t_exit, (face - comp(co, a)) * ia);
    }
    const float top = __int_as_float((__float_as_int(t) & 0x7f800000) + 0x00800000);  // 2^(e+1)
    const float u = top * 5.9604645e-8f;                                              // ulp of the binade
    const float t1 = fa(t, step);
    const float delta = fs(t1, t);
    if (!(t1 < top) || fabsf(fs(step, delta)) == 0.5f * u) return t;
    const float lim = fminf(fminf(t_exit, t_far) - t, fs(fs(top, u), t));
    const float m = floorf(lim / delta) - 1.0f;
    if (!(m >= 1.0f)) return t;
    return fmaf(m, delta, t);
}

// Exact free flags from the volume (after an upload).
template <bool kHalf>
__global__ void rebuild_bricks_kernel(const void* vox, int res, uint8_t* bricks, int nb) {
    const size_t nbr = static_cast<size_t>(nb) * nb * nb;
    const size_t b = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= nbr) return;
    const int bx = static_cast<int>(b % nb), by = static_cast<int>((b / nb) % nb), bz = static_cast<int>(b / nb / nb);
    bool free = true;
    for (int z = bz * 8; free && z <= min(bz * 8 + 8, res - 1); ++z)
        for (int y = by * 8; free && y <= min(by * 8 + 8, res - 1); ++y)
            for (int x = bx * 8; free && x <= min(bx * 8 + 8, res - 1); ++x) {
                const float2 r = Vox<kHalf>::load_rw(vox, (static_cast<size_t>(z) * res + y) * res + x);
                if ((r.y > 0.0f) && !(r.x >= kFreeTsdf)) free = false;
            }
    bricks[b] = free ? 1 : 0;
}

// Front-face raycast (TSDFVolume.cpp:372-475): one thread per pixel; a warp is
// 32 adjacent pixels of one row, so its rays march side by side and their
// trilinear gathers share cache lines.
template <bool kHalf, bool kCol = true>
__device__ __forceinline__ void raycast_pixel(const VolView& v, const float* __restrict__ d_pose, float fx, float fy,
                                              float cx, float cy, int W, int H, float trunc, float min_depth,
                                              float max_depth, float* __restrict__ vout, float* __restrict__ nout,
                                              uint8_t* __restrict__ cout, const int* __restrict__ gate,
                                              const uint8_t* __restrict__ bdist, int nb, int x, int y,
                                              const uint32_t* __restrict__ smap = nullptr) {
    if (gate && __ldg(gate) == 0) return;
    if (x >= W || y >= H) return;
    const int o = y * W + x;
    float R[9];
    R[0] = __ldg(d_pose + 0); R[1] = __ldg(d_pose + 1); R[2] = __ldg(d_pose + 2);
    R[3] = __ldg(d_pose + 4); R[4] = __ldg(d_pose + 5); R[5] = __ldg(d_pose + 6);
    R[6] = __ldg(d_pose + 8); R[7] = __ldg(d_pose + 9); R[8] = __ldg(d_pose + 10);
    const F3 co = mk3(__ldg(d_pose + 3), __ldg(d_pose + 7), __ldg(d_pose + 11));
    F3 vres = mk3(0.0f, 0.0f, 0.0f), nres = mk3(0.0f, 0.0f, 0.0f);
    uint8_t col[3] = {0, 0, 0};

    const float vs = v.vs;
    const F3 box_lo = v.origin;
    const float span = fm(static_cast<float>(v.res - 1), vs);
    const F3 box_hi = add3(box_lo, mk3(span, span, span));
    const float min_step = fm(0.5f, vs);
    const float far_c = fm(0.8f, trunc);
    const float far_step = min_step < far_c ? far_c : min_step;  // std::max(min_step, 0.8*trunc)

    do {
        const F3 ray = mk3(fd(fs(static_cast<float>(x), cx), fx), fd(fs(static_cast<float>(y), cy), fy), 1.0f);
        const float ray_norm = norm3(ray);
        const F3 dir = div3(mv3(R, ray), ray_norm);
        float t_near = fm(min_depth, ray_norm);
        float t_far = fm(max_depth, ray_norm);
        float inv_dir[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float da = comp(dir, a), oa = comp(co, a), la = comp(box_lo, a), ha = comp(box_hi, a);
            const float inv = fd(1.0f, da);
            inv_dir[a] = inv;
            float t0 = fm(fs(la, oa), inv);
            float t1 = fm(fs(ha, oa), inv);
            if (t0 > t1) { const float tmp = t0; t0 = t1; t1 = tmp; }
            if (isnan(t0) || isnan(t1)) {
                if (oa < la || oa > ha) t_far = -1.0f;
                continue;
            }
            t_near = (t_near < t0) ? t0 : t_near;  // std::max(t_near, t0)
            t_far = (t1 < t_far) ? t1 : t_far;     // std::min(t_far, t1)
        }
        if (!(t_near < t_far)) break;

        float t_prev = t_near, f_prev = 1.0f;
        bool prev_valid = sample_tsdf<kHalf>(v, add3(co, mul3(dir, t_prev)), f_prev);
        if (prev_valid && !isfinite(f_prev)) break;
        if (prev_valid && f_prev < 0.0f) break;
        bool found = false;
        float t_hit = 0.0f;
        // A sample in a free brick is invalid or has f >= 0.999: its step is the
        // far step and, unless the previous sample was negative, no test can fire.
        // Such samples are not evaluated; the march keeps the same t sequence, and
        // the last skipped sample is evaluated when the state is needed again.
        bool skipped = false;
        if (smap && (!prev_valid || f_prev >= 0.999f)) {
            // every sample below the tile's start bound is skipped: take the far
            // steps that stay two steps short of it (and of t_far) at once, by
            // the closed form of the running sum
            const int tw = (W + (1 << kStartShift) - 1) >> kStartShift;
            const int th = (H + (1 << kStartShift) - 1) >> kStartShift;
            const float ts = fminf(__uint_as_float(__ldg(smap + (y >> kStartShift) * tw + (x >> kStartShift))),
                                   __uint_as_float(__ldg(smap + tw * th)));
            const float n = floorf((fminf(ts, t_far) - t_near) / far_step) - 2.0f;
            if (n >= 1.0f) {
                t_prev = fs_walk_far(t_near, far_step, static_cast<int>(fminf(n, 1e8f)));
                skipped = true;
            }
        }
        while (t_prev < t_far) {
            float step;
            if (skipped || !prev_valid || f_prev >= 0.999f) {
                step = far_step;
            } else {
                const float s = fm(fm(0.8f, f_prev), trunc);
                step = min_step < s ? s : min_step;  // std::max(min_step, s)
            }
            const float tn = fa(t_prev, step);
            const float t = (t_far < tn) ? t_far : tn;  // std::min(t_prev + step, t_far)
            if (!(t > t_prev)) break;  // no progress (degenerate parameters): stop without a hit
            const F3 p = add3(co, mul3(dir, t));
            int bx = 0, by = 0, bz = 0;
            const int fb = (bdist && (skipped || !prev_valid || f_prev >= 0.0f)) ? brick_state(v, bdist, nb, p, bx, by, bz) : 0;
            if (fb) {
                t_prev = t;
                skipped = true;
                if (t >= t_far) break;
                if (fb >= 2)
                    t_prev = free_space_jump(v, co, mk3(inv_dir[0], inv_dir[1], inv_dir[2]), t, far_step, t_far, bx,
                                             by, bz, fb - 1);
                continue;
            }
            if (skipped) {
                f_prev = 1.0f;
                prev_valid = sample_tsdf<kHalf>(v, add3(co, mul3(dir, t_prev)), f_prev);
                skipped = false;
            }
            float f = 1.0f;
            const bool valid = sample_tsdf<kHalf>(v, p, f);
            if (valid && !isfinite(f)) break;
            if (valid && prev_valid) {
                if (f_prev > 0.0f && f <= 0.0f) {
                    t_hit = fa(t_prev, fm(fs(t, t_prev), fd(f_prev, fs(f_prev, f))));
                    found = true;
                    break;
                }
                if (f_prev < 0.0f && f >= 0.0f) break;
            } else if (valid && f < 0.0f) {
                break;
            }
            t_prev = t;
            f_prev = f;
            prev_valid = valid;
            if (t >= t_far) break;
        }
        if (!found) break;
        const F3 hit = add3(co, mul3(dir, t_hit));
        F3 nrm;
        if (!compute_normal<kHalf>(v, hit, nrm)) break;
        if (!finite3(hit)) break;
        if (kCol && cout) {
            const F3 q = to_voxel(v, hit);
            int vx, vy, vz;
            if (floor_to_int(q.x, &vx) && floor_to_int(q.y, &vy) && floor_to_int(q.z, &vz) && vx >= 0 &&
                vx < v.res && vy >= 0 && vy < v.res && vz >= 0 && vz < v.res) {
                const size_t r = static_cast<size_t>(v.res);
                const size_t vi = (static_cast<size_t>(vz) * r + vy) * r + vx;
                if (Vox<kHalf>::load(v.vox, vi).y > 0.0f) {
                    const float cr = v.color ? v.color[3 * vi] : kEmptyColor;
                    const float cg = v.color ? v.color[3 * vi + 1] : kEmptyColor;
                    const float cb = v.color ? v.color[3 * vi + 2] : kEmptyColor;
                    uint8_t q0, q1, q2;
                    if (!(srgb_to_byte(cr, &q0) && srgb_to_byte(cg, &q1) && srgb_to_byte(cb, &q2))) break;
                    col[0] = q0; col[1] = q1; col[2] = q2;
                }
            }
        }
        vres = hit;
        nres = nrm;
    } while (false);
    vout[3 * o] = vres.x; vout[3 * o + 1] = vres.y; vout[3 * o + 2] = vres.z;
    nout[3 * o] = nres.x; nout[3 * o + 1] = nres.y; nout[3 * o + 2] = nres.z;
    if (kCol && cout) { cout[3 * o] = col[0]; cout[3 * o + 1] = col[1]; cout[3 * o + 2] = col[2]; }
}

template <bool kHalf, bool kCol>
__global__ void __launch_bounds__(128, 9) raycast_kernel(VolView v, const float* __restrict__ d_pose, float fx,
                                                     float fy, float cx, float cy, int W, int H, float trunc,
                                                     float min_depth, float max_depth, float* __restrict__ vout,
                                                     float* __restrict__ nout, uint8_t* __restrict__ cout,
                                                     const int* __restrict__ gate, const uint8_t* __restrict__ bdist,
                                                     int nb, const uint32_t* __restrict__ smap) {
    raycast_pixel<kHalf, kCol>(v, d_pose, fx, fy, cx, cy, W, H, trunc, min_depth, max_depth, vout, nout, cout, gate,
                               bdist, nb, blockIdx.x * blockDim.x + threadIdx.x,
                               blockIdx.y * blockDim.y + threadIdx.y, smap);
}

// ---- global point cloud (TSDFVolume.cpp:571-632) --------------------------------
// Voxels with weight > 1 and |tsdf| < 0.2 whose colour quantises (a non-finite
// colour skips the voxel), in index order z, y, x — the order of the
// reference's loop run on one thread. Two passes over fixed 1024-voxel blocks:
// count, then (after an exclusive scan of the block counts) emit at the block's
// offset plus the thread's prefix, so the output order is deterministic.
constexpr int kPcThreads = 256, kPcPerThread = 4, kPcBlock = kPcThreads * kPcPerThread;

template <bool kHalf>
__device__ __forceinline__ bool pc_take(const void* vox, const float* color, size_t i, uint8_t q[3]) {
    const float2 r = Vox<kHalf>::load(vox, i);
    if (!(r.y > 1.0f && fabsf(r.x) < 0.2f)) return false;
    const float cr = color ? color[3 * i] : kEmptyColor;
    const float cg = color ? color[3 * i + 1] : kEmptyColor;
    const float cb = color ? color[3 * i + 2] : kEmptyColor;
    return srgb_to_byte(cr, &q[0]) && srgb_to_byte(cg, &q[1]) && srgb_to_byte(cb, &q[2]);
}

// Block-wide exclusive prefix of one int per thread; returns the block total.
__device__ __forceinline__ int block_exclusive(int v, int* s_warp, int& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < (kPcThreads / 32) ? s_warp[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < (kPcThreads / 32)) s_warp[lane] = w;  // inclusive warp sums
    }
    __syncthreads();
    total = s_warp[kPcThreads / 32 - 1];
    const int before = warp > 0 ? s_warp[warp - 1] : 0;
    __syncthreads();
    return before + incl - v;
}

template <bool kHalf>
__global__ void __launch_bounds__(kPcThreads) pc_count_kernel(const void* vox, const float* color, size_t n,
                                                             int* block_counts) {
    __shared__ int s_warp[kPcThreads / 32];
    const size_t base = static_cast<size_t>(blockIdx.x) * kPcBlock + static_cast<size_t>(threadIdx.x) * kPcPerThread;
    int c = 0;
    uint8_t q[3];
    for (int k = 0; k < kPcPerThread; ++k)
        if (base + k < n && pc_take<kHalf>(vox, color, base + k, q)) ++c;
    int total = 0;
    block_exclusive(c, s_warp, total);
    if (threadIdx.x == 0) block_counts[blockIdx.x] = total;
}

template <bool kHalf>
__global__ void __launch_bounds__(kPcThreads) pc_emit_kernel(const void* vox, const float* color, size_t n, int res,
                                                            float vs, F3 origin, const long long* block_offsets,
                                                            float* points, uint8_t* colors) {
    __shared__ int s_warp[kPcThreads / 32];
    const size_t base = static_cast<size_t>(blockIdx.x) * kPcBlock + static_cast<size_t>(threadIdx.x) * kPcPerThread;
    bool take[kPcPerThread];
    uint8_t q[kPcPerThread][3];
    int c = 0;
    for (int k = 0; k < kPcPerThread; ++k) {
        take[k] = base + k < n && pc_take<kHalf>(vox, color, base + k, q[k]);
        c += take[k];
    }
    int total = 0;
    long long o = block_offsets[blockIdx.x] + block_exclusive(c, s_warp, total);
    const size_t rr = static_cast<size_t>(res);
    for (int k = 0; k < kPcPerThread; ++k) {
        if (!take[k]) continue;
        const size_t i = base + k;
        const int x = static_cast<int>(i % rr), y = static_cast<int>((i / rr) % rr), z = static_cast<int>(i / rr / rr);
        // voxelToWorld (TSDFVolume.cpp:555-561): origin + (x, y, z) * vs
        points[3 * o] = fa(origin.x, fm(static_cast<float>(x), vs));
        points[3 * o + 1] = fa(origin.y, fm(static_cast<float>(y), vs));
        points[3 * o + 2] = fa(origin.z, fm(static_cast<float>(z), vs));
        colors[3 * o] = q[k][0];
        colors[3 * o + 1] = q[k][1];
        colors[3 * o + 2] = q[k][2];
        ++o;
    }
}

static int ensure_tiles(azu_volume* v, size_t n, cudaStream_t s);
static int ensure_ray_start(azu_volume* v, size_t n, cudaStream_t s);

// ---- batches: several volumes, one launch per stage --------------------------
// A batch integrates and raycasts the current frame of several independent
// volumes (different resolutions and image sizes) with one launch per stage.
// Each launch maps its blocks (or warps) onto the volumes through prefix
// offsets and runs the same per-volume body as the single-volume kernels, so
// every volume's result is the single-volume result bit for bit. The integrate
// block size and the raycast tile shape are parameters (the batch autotuner
// picks them).
struct IntegrateArgs {
    void* vox;
    const IntegrateConsts* icp;
    const float* depth;
    int res;
    float vs, ox, oy, oz, trunc, max_w, fx, fy, cx, cy;
    int W, H;
    float min_d, max_d;
    const int* gate;
    unsigned long long* counters;
    uint8_t* bricks;
    int nb;
    float* tiles;
    TileMip mip;
    IntegrateConsts* icp_out;
    const float* pose;
};

struct RaycastArgs {
    VolView v;
    const float* pose;
    float fx, fy, cx, cy;
    int W, H;
    float trunc, min_depth, max_depth;
    float* vout;
    float* nout;
    const int* gate;
    const uint8_t* bricks;
    uint8_t* bdist;
    int nb;
    uint32_t* smap;  // the volume's ray start map
};

__device__ __forceinline__ int batch_find(const int* __restrict__ off, int n, int i) {
    int s = 0;
    while (s + 1 < n && i >= __ldg(off + s + 1)) ++s;
    return s;
}

__global__ void depth_tiles_batch_kernel(const IntegrateArgs* __restrict__ A, const int* __restrict__ off, int n) {
    const int s = batch_find(off, n, blockIdx.x);
    const IntegrateArgs& a = A[s];
    depth_tiles_body(blockIdx.x - __ldg(off + s), a.depth, a.W, a.H, a.min_d, a.max_d, a.mip.w[0],
                     a.mip.w[0] * a.mip.h[0], a.tiles, a.gate);
}

__global__ void integrate_setup_batch_kernel(const IntegrateArgs* __restrict__ A, unsigned* __restrict__ work) {
    const IntegrateArgs& a = A[blockIdx.x];
    integrate_setup_body(a.pose, a.res, a.vs, a.ox, a.oy, a.oz, a.trunc, a.fx, a.fy, a.cx, a.cy, a.W, a.H, a.max_d,
                         a.icp_out, a.counters, a.tiles, a.mip, true);
    if (blockIdx.x == 0 && threadIdx.x == 0) *work = 0;  // next item of the batch integrate
}

// Persistent over the items of all scenes (32 rows x one of nparts x-parts of a
// row each, scene by prefix offsets): every warp takes the next item from the
// batch's counter.
template <int kWarps>
__global__ void __launch_bounds__(kWarps * 32) integrate_batch_kernel(const IntegrateArgs* __restrict__ A,
                                                                      const int* __restrict__ off, int n,
                                                                      unsigned* __restrict__ work, int nparts) {
    __shared__ float s_c[kWarps][3][32][33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = __ldg(off + n);
    for (;;) {
        int item = 0;
        if (lane == 0) item = static_cast<int>(atomicAdd(work, 1u));
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        const int s = batch_find(off, n, item);
        const IntegrateArgs& a = A[s];
        integrate_item<false, false, false>(a.vox, nullptr, a.icp, a.depth, nullptr, a.res, a.vs, a.ox, a.oy, a.oz,
                                            a.trunc, a.max_w, a.fx, a.fy, a.cx, a.cy, a.W, a.H, a.min_d, a.max_d,
                                            a.gate, a.counters, a.bricks, a.nb, a.tiles, a.mip, item - __ldg(off + s),
                                            warp, lane, s_c, nparts);
    }
}

// Every scene's start map back to "no bound" (block s: scene s).
__global__ void ray_start_reset_batch_kernel(const RaycastArgs* __restrict__ A) {
    const RaycastArgs& a = A[blockIdx.x];
    if (a.gate && __ldg(a.gate) == 0) return;
    const int n = ((a.W + (1 << kStartShift) - 1) >> kStartShift) * ((a.H + (1 << kStartShift) - 1) >> kStartShift) + 1;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a.smap[i] = 0x7f7f7f7fu;
}

// The brick field of every scene: scene s owns blocks [off[s], off[s + 1]), one
// per tile of 8^3 bricks.
__global__ void __launch_bounds__(512) brick_field_batch_kernel(const RaycastArgs* __restrict__ A,
                                                                const int* __restrict__ off, int n) {
    const int s = batch_find(off, n, blockIdx.x);
    const RaycastArgs& a = A[s];
    if (a.gate && __ldg(a.gate) == 0) return;
    const int gb = (a.nb + kFieldSide - 1) / kFieldSide;
    const int t = blockIdx.x - __ldg(off + s);
    const StartMapArgs sm{a.v.vs, a.v.origin, a.pose, a.fx, a.fy, a.cx, a.cy, a.W, a.H, a.smap};
    brick_field_body(a.bricks, a.bdist, a.nb, sm, t % gb, (t / gb) % gb, t / (gb * gb));
}

__global__ void __launch_bounds__(256, 5) raycast_batch_kernel(const RaycastArgs* __restrict__ A,
                                                            const int* __restrict__ off, int n) {
    const int s = batch_find(off, n, blockIdx.x);
    const RaycastArgs& a = A[s];
    const int tile = blockIdx.x - __ldg(off + s);
    const int tiles_x = (a.W + blockDim.x - 1) / blockDim.x;
    const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
    raycast_pixel<false, false>(a.v, a.pose, a.fx, a.fy, a.cx, a.cy, a.W, a.H, a.trunc, a.min_depth, a.max_depth,
                                a.vout, a.nout, nullptr, a.gate, a.bdist, a.nb, tx * blockDim.x + threadIdx.x,
                                ty * blockDim.y + threadIdx.y, a.smap);
}

}  // namespace azu

struct azu_volume_batch {
    int n = 0;
    std::vector<azu::PipelineFrameView> views;
    azu::IntegrateArgs* d_int = nullptr;
    azu::RaycastArgs* d_ray = nullptr;
    int* d_off = nullptr;  // [0..n] tile blocks, [n+1..2n+1] integrate items, [2n+2..3n+2] brick field tiles, [3n+3..4n+3] ray tiles
    unsigned* d_work = nullptr;  // next integrate item
    int tiles_blocks = 0, items = 0, brick_blocks = 0, ray_blocks = 0;
    int int_grid[3] = {0, 0, 0};  // resident blocks of the persistent integrate, by 1, 2, 4 warps
    int int_warps = 4, int_parts = azu::kIntParts, ray_w = 32, ray_h = 8;
};

namespace azu {

static int batch_upload_offsets(azu_volume_batch* b) {
    const int n = b->n;
    std::vector<int> off(4 * (n + 1), 0);
    int tb = 0, it = 0, bb = 0, rb = 0;
    for (int i = 0; i < n; ++i) {
        const PipelineFrameView& f = b->views[i];
        const TileMip mip = make_tile_mip(f.W, f.H);
        off[i] = tb;
        tb += (mip.w[0] * mip.h[0] + 31) / 32;
        off[n + 1 + i] = it;
        const int res = f.vol->p.resolution;
        it += res * ((res + 31) / 32) * b->int_parts;
        off[2 * (n + 1) + i] = bb;
        const int gb = (f.vol->nb + kFieldSide - 1) / kFieldSide;
        bb += gb * gb * gb;
        off[3 * (n + 1) + i] = rb;
        rb += ((f.W + b->ray_w - 1) / b->ray_w) * ((f.H + b->ray_h - 1) / b->ray_h);
    }
    off[n] = tb;
    off[n + 1 + n] = it;
    off[2 * (n + 1) + n] = bb;
    off[3 * (n + 1) + n] = rb;
    b->tiles_blocks = tb;
    b->items = it;
    b->brick_blocks = bb;
    b->ray_blocks = rb;
    AZU_TRY_CUDA(cudaMemcpy(b->d_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice));
    return AZU_OK;
}

int volume_batch_create(const PipelineFrameView* views, int n, azu_volume_batch** out) {
    AZU_CHECK_ARG(views != nullptr && out != nullptr && n >= 1 && n <= 4096, "batch of 1..4096 volumes");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        const azu_volume* v = views[i].vol;
        AZU_CHECK_ARG(v != nullptr && v->p.format == AZU_TSDF_FP32 && v->color == nullptr,
                      "batched volumes are FP32 without colour");
    }
    azu_volume_batch* b = new azu_volume_batch();
    b->n = n;
    b->views.assign(views, views + n);
    std::vector<IntegrateArgs> ia(n);
    std::vector<RaycastArgs> ra(n);
    int rc = AZU_OK;
    for (int i = 0; i < n && !rc; ++i) {
        const PipelineFrameView& f = views[i];
        azu_volume* v = f.vol;
        const azu_volume_params& p = v->p;
        const TileMip mip = make_tile_mip(f.W, f.H);
        rc = ensure_tiles(v, static_cast<size_t>(mip.total), v->stream.s);
        ia[i] = IntegrateArgs{v->vox, v->d_iconsts, f.d_depth_m, p.resolution, p.voxel_size, p.origin[0],
                              p.origin[1], p.origin[2], p.truncation, p.max_weight, f.fx, f.fy, f.cx, f.cy, f.W,
                              f.H, f.min_d, f.max_d, f.d_gate, v->d_counters, v->bricks, v->nb, v->d_tiles, mip,
                              v->d_iconsts, f.d_pose};
        if (!rc)
            rc = ensure_ray_start(v, static_cast<size_t>((f.W + (1 << kStartShift) - 1) >> kStartShift) *
                                             ((f.H + (1 << kStartShift) - 1) >> kStartShift) + 1,
                                  v->stream.s);
        ra[i] = RaycastArgs{make_view(v), f.d_pose, f.fx, f.fy, f.cx, f.cy, f.W, f.H, p.truncation, p.min_depth,
                            p.max_depth, f.d_vertices, f.d_normals, f.d_gate, v->bricks, v->brick_dist, v->nb,
                            v->ray_start};
        AZU_CHECK_ARG(v->skip_free, "batched raycasts use free-space skipping");
    }
    if (!rc) {
        cudaError_t e = cudaMalloc(&b->d_int, n * sizeof(IntegrateArgs));
        if (!e) e = cudaMalloc(&b->d_ray, n * sizeof(RaycastArgs));
        if (!e) e = cudaMalloc(&b->d_off, 4 * (n + 1) * sizeof(int));
        if (!e) e = cudaMalloc(&b->d_work, sizeof(unsigned));
        int sms = 0;
        if (!e) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, views[0].vol->device);
        const void* kernels[3] = {(const void*)integrate_batch_kernel<1>, (const void*)integrate_batch_kernel<2>,
                                  (const void*)integrate_batch_kernel<4>};
        for (int k = 0; k < 3 && !e; ++k) {
            int occ = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernels[k], 32 << k, 0);
            b->int_grid[k] = std::max(1, sms * std::max(occ, 1));
        }
        if (!e) e = cudaMemcpy(b->d_int, ia.data(), n * sizeof(IntegrateArgs), cudaMemcpyHostToDevice);
        if (!e) e = cudaMemcpy(b->d_ray, ra.data(), n * sizeof(RaycastArgs), cudaMemcpyHostToDevice);
        if (e) { set_error("batch allocation: %s", cudaGetErrorString(e)); rc = AZU_E_NOMEM; }
    }
    if (!rc) rc = batch_upload_offsets(b);
    if (rc) { volume_batch_destroy(b); return rc; }
    *out = b;
    return AZU_OK;
}

void volume_batch_destroy(azu_volume_batch* b) {
    if (!b) return;
    if (b->d_int) cudaFree(b->d_int);
    if (b->d_ray) cudaFree(b->d_ray);
    if (b->d_off) cudaFree(b->d_off);
    if (b->d_work) cudaFree(b->d_work);
    delete b;
}

int volume_batch_set_shapes(azu_volume_batch* b, int int_warps, int int_parts, int ray_w, int ray_h) {
    AZU_CHECK_ARG(int_warps == 1 || int_warps == 2 || int_warps == 4, "integrate warps per block: 1, 2 or 4");
    AZU_CHECK_ARG(int_parts == 1 || int_parts == 2 || int_parts == 4, "integrate x-parts per row: 1, 2 or 4");
    AZU_CHECK_ARG(ray_w >= 8 && ray_h >= 1 && ray_w * ray_h <= 256 && (ray_w * ray_h) % 32 == 0,
                  "raycast tile: at most 256 threads, whole warps");
    b->int_warps = int_warps;
    b->int_parts = int_parts;
    b->ray_w = ray_w;
    b->ray_h = ray_h;
    return batch_upload_offsets(b);
}

void volume_batch_shapes(const azu_volume_batch* b, int* int_warps, int* int_parts, int* ray_w, int* ray_h) {
    if (int_warps) *int_warps = b->int_warps;
    if (int_parts) *int_parts = b->int_parts;
    if (ray_w) *ray_w = b->ray_w;
    if (ray_h) *ray_h = b->ray_h;
}

int volume_batch_integrate(azu_volume_batch* b, cudaStream_t s) {
    const int n = b->n;
    depth_tiles_batch_kernel<<<b->tiles_blocks, 256, 0, s>>>(b->d_int, b->d_off, n);
    AZU_LAUNCH_CHECK();
    integrate_setup_batch_kernel<<<n, 256, 0, s>>>(b->d_int, b->d_work);
    AZU_LAUNCH_CHECK();
    const int* ioff = b->d_off + (n + 1);
    const int k = b->int_warps == 1 ? 0 : (b->int_warps == 2 ? 1 : 2);
    const int blocks = std::min(b->int_grid[k], (b->items + b->int_warps - 1) / b->int_warps);
    const int P = b->int_parts;
    if (b->int_warps == 1) integrate_batch_kernel<1><<<blocks, 32, 0, s>>>(b->d_int, ioff, n, b->d_work, P);
    else if (b->int_warps == 2) integrate_batch_kernel<2><<<blocks, 64, 0, s>>>(b->d_int, ioff, n, b->d_work, P);
    else integrate_batch_kernel<4><<<blocks, 128, 0, s>>>(b->d_int, ioff, n, b->d_work, P);
    AZU_LAUNCH_CHECK();
    for (const PipelineFrameView& f : b->views) f.vol->integrated_frames++;
    return AZU_OK;
}

int volume_batch_raycast(azu_volume_batch* b, cudaStream_t s) {
    const int n = b->n;
    const int* boff = b->d_off + 2 * (n + 1);
    ray_start_reset_batch_kernel<<<n, 256, 0, s>>>(b->d_ray);
    AZU_LAUNCH_CHECK();
    brick_field_batch_kernel<<<b->brick_blocks, 512, 0, s>>>(b->d_ray, boff, n);
    AZU_LAUNCH_CHECK();
    raycast_batch_kernel<<<b->ray_blocks, dim3(b->ray_w, b->ray_h), 0, s>>>(b->d_ray, b->d_off + 3 * (n + 1), n);
    AZU_LAUNCH_CHECK();
    return AZU_OK;
}

// Many model images at once (the relocaliser's candidate renders): one launch,
// blockIdx.z = pose; every image is the single raycast's bit for bit.
template <bool kHalf>
__global__ void __launch_bounds__(256, 5) raycast_many_kernel(VolView v, const float* __restrict__ d_poses, float fx,
                                                          float fy, float cx, float cy, int W, int H, float trunc,
                                                          float min_depth, float max_depth, float* __restrict__ vout,
                                                          float* __restrict__ nout,
                                                          const uint8_t* __restrict__ bdist, int nb) {
    const size_t img = static_cast<size_t>(W) * H * 3 * blockIdx.z;
    raycast_pixel<kHalf>(v, d_poses + 16 * blockIdx.z, fx, fy, cx, cy, W, H, trunc, min_depth, max_depth, vout + img,
                         nout + img, nullptr, nullptr, bdist, nb, blockIdx.x * blockDim.x + threadIdx.x,
                         blockIdx.y * blockDim.y + threadIdx.y);
}

// ---- whole-volume transfers -------------------------------------------------
template <bool kHalf, bool kResid>
__global__ void unpack_kernel(const void* vox, size_t base, size_t n, float* t, float* w) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 r = kResid ? VoxR::load_fold(vox, base + i) : Vox<kHalf>::load_rw(vox, base + i);
    t[i] = r.x;
    w[i] = r.y;
}
template <bool kHalf, bool kResid>
__global__ void pack_kernel(void* vox, size_t base, size_t n, const float* t, const float* w) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (kResid) VoxR::store(vox, base + i, t[i], w[i]);
    else Vox<kHalf>::store(vox, base + i, t[i], w[i]);
}

int set_pose_async(float* d_pose, const float* pose, cudaStream_t s) {
    Pose16 p;
    std::memcpy(p.m, pose, sizeof(p.m));
    set_pose_kernel<<<1, 32, 0, s>>>(d_pose, p);
    AZU_LAUNCH_CHECK();
    return AZU_OK;
}

// Depth-tile buffer with room for n tiles. Grows outside stream capture only;
// volumes are created with room for a 640x480 image.
static int ensure_ray_start(azu_volume* v, size_t n, cudaStream_t s) {
    if (n <= v->ray_start_cap) return AZU_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    AZU_TRY_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) {
        set_error("raycast: image larger than the ray start map during stream capture");
        return AZU_E_STATE;
    }
    AZU_TRY_CUDA(cudaStreamSynchronize(s));
    if (v->ray_start) cudaFree(v->ray_start);
    v->ray_start = nullptr;
    v->ray_start_cap = 0;
    AZU_TRY_CUDA(cudaMalloc(&v->ray_start, n * sizeof(uint32_t)));
    v->ray_start_cap = n;
    return AZU_OK;
}

static int ensure_tiles(azu_volume* v, size_t n, cudaStream_t s) {
    if (n <= v->tile_cap) return AZU_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    AZU_TRY_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) {
        set_error("integrate: image larger than the depth-tile buffer during stream capture");
        return AZU_E_STATE;
    }
    AZU_TRY_CUDA(cudaStreamSynchronize(s));
    if (v->d_tiles) cudaFree(v->d_tiles);
    v->d_tiles = nullptr;
    v->tile_cap = 0;
    AZU_TRY_CUDA(cudaMalloc(&v->d_tiles, n * sizeof(float)));
    v->tile_cap = n;
    return AZU_OK;
}

// Depth tile pyramid of a depth map (level 0 + coarser levels) into `tiles`
// (make_tile_mip(W, H).total floats).
int volume_build_tiles_dev(const float* d_depth_m, int W, int H, float min_d, float max_d, float* tiles,
                           cudaStream_t s) {
    AZU_CHECK_ARG(W <= kMaxTilePixels && H <= kMaxTilePixels, "image larger than 16384 pixels a side");
    const TileMip mip = make_tile_mip(W, H);
    const int nt0 = mip.w[0] * mip.h[0];
    depth_tiles_kernel<<<(nt0 + 31) / 32, 256, 0, s>>>(d_depth_m, W, H, min_d, max_d, mip.w[0], nt0, tiles, nullptr);
    AZU_LAUNCH_CHECK();
    tile_pyramid_kernel<<<1, 256, 0, s>>>(tiles, mip);
    AZU_LAUNCH_CHECK();
    return AZU_OK;
}

int volume_integrate_dev(azu_volume* v, const float* d_depth_m, const uint8_t* d_rgb, const float* d_pose, float fx,
                         float fy, float cx, float cy, int W, int H, float min_d, float max_d, const int* d_gate,
                         cudaStream_t s, const float* d_tiles_built) {
    const azu_volume_params& p = v->p;
    AZU_CHECK_ARG(W <= kMaxTilePixels && H <= kMaxTilePixels, "image larger than 16384 pixels a side");
    const TileMip mip = make_tile_mip(W, H);
    float* tiles = const_cast<float*>(d_tiles_built);
    if (!tiles) {
        if (int rc = ensure_tiles(v, static_cast<size_t>(mip.total), s)) return rc;
        tiles = v->d_tiles;
        const int nt0 = mip.w[0] * mip.h[0];
        depth_tiles_kernel<<<(nt0 + 31) / 32, 256, 0, s>>>(d_depth_m, W, H, min_d, max_d, mip.w[0], nt0, tiles,
                                                            d_gate);
        AZU_LAUNCH_CHECK();
    }
    integrate_setup_kernel<<<1, 256, 0, s>>>(d_pose, p.resolution, p.voxel_size, p.origin[0], p.origin[1],
                                             p.origin[2], p.truncation, fx, fy, cx, cy, W, H, max_d, v->d_iconsts,
                                             v->d_counters, tiles, mip, d_tiles_built ? 0 : 1);
    AZU_LAUNCH_CHECK();
    {
        const int rows = v->nb * v->nb * v->int_live_words;  // warps of the pre-cull
        integrate_bricks_kernel<<<(rows + 7) / 8, 256, 0, s>>>(
            v->d_iconsts, p.resolution, v->nb, v->int_live_words, p.voxel_size, p.origin[0], p.origin[1],
            p.origin[2], fx, fy, cx, cy, W, H, tiles, mip, d_gate, v->int_live);
        AZU_LAUNCH_CHECK();
        const int n_items = p.resolution * ((p.resolution + 31) / 32) * kIntParts;
        integrate_list_kernel<<<(n_items + 255) / 256, 256, 0, s>>>(v->d_iconsts, p.resolution, v->nb,
                                                                   v->int_live_words, kIntParts, v->int_live,
                                                                   d_gate, v->d_counters, v->int_list);
        AZU_LAUNCH_CHECK();
    }
    const int ngroups = (p.resolution + 31) / 32;
    const long items = static_cast<long>(p.resolution) * ngroups;
    const bool half = p.format != AZU_TSDF_FP32;
    if (!v->int_blocks) {
        // resident blocks of the persistent integrate kernel: the fewest any variant fits
        int sms = 0, occ = 1 << 20;
        AZU_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, v->device));
        const void* variants[] = {(const void*)integrate_kernel<false, false, false>,
                                  (const void*)integrate_kernel<false, true, false>,
                                  (const void*)integrate_kernel<true, false, false>,
                                  (const void*)integrate_kernel<true, true, false>,
                                  (const void*)integrate_kernel<true, false, true>,
                                  (const void*)integrate_kernel<true, true, true>};
        for (const void* f : variants) {
            int o = 0;
            AZU_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, f, kIntWarps * 32, 0));
            occ = std::min(occ, o);
        }
        v->int_blocks = std::max(1, sms * std::max(occ, 1));
    }
    const int blocks = static_cast<int>(std::min<long>(v->int_blocks, (items + kIntWarps - 1) / kIntWarps));
    const bool resid = p.format == AZU_TSDF_FP16R;
    const bool col = v->color != nullptr;
#define AZU_INT_ARGS                                                                                             \
    v->vox, v->color, v->d_iconsts, d_depth_m, d_rgb, p.resolution, p.voxel_size, p.origin[0], p.origin[1],     \
        p.origin[2], p.truncation, p.max_weight, fx, fy, cx, cy, W, H, min_d, max_d, d_gate, v->d_counters,   \
        v->bricks, v->nb, tiles, mip, v->int_live, v->int_live_words, v->int_list
    if (!half && !col) integrate_kernel<false, false, false><<<blocks, kIntWarps * 32, 0, s>>>(AZU_INT_ARGS);
    else if (!half && col) integrate_kernel<false, true, false><<<blocks, kIntWarps * 32, 0, s>>>(AZU_INT_ARGS);
    else if (!resid && !col) integrate_kernel<true, false, false><<<blocks, kIntWarps * 32, 0, s>>>(AZU_INT_ARGS);
    else if (!resid && col) integrate_kernel<true, true, false><<<blocks, kIntWarps * 32, 0, s>>>(AZU_INT_ARGS);
    else if (!col) integrate_kernel<true, false, true><<<blocks, kIntWarps * 32, 0, s>>>(AZU_INT_ARGS);
    else integrate_kernel<true, true, true><<<blocks, kIntWarps * 32, 0, s>>>(AZU_INT_ARGS);
#undef AZU_INT_ARGS
    AZU_LAUNCH_CHECK();
    return AZU_OK;
}

int volume_raycast_dev(azu_volume* v, const float* d_pose, float fx, float fy, float cx, float cy, int W, int H,
                       float* d_vertices, float* d_normals, uint8_t* d_colors, const int* d_gate, cudaStream_t s) {
    const azu_volume_params& p = v->p;
    const VolView view = make_view(v);
    // 8 x 16 pixel blocks: each warp marches an 8 x 4 patch (closer rays than a
    // 32 x 1 row: 6% faster than 16 x 8 blocks, 9% than 32 x 8)
    const dim3 blk(8, 16), grd((W + 7) / 8, (H + 15) / 16);
    const uint8_t* bricks = nullptr;
    const uint32_t* smap = nullptr;
    if (v->skip_free) {
        const size_t nst = static_cast<size_t>((W + (1 << kStartShift) - 1) >> kStartShift) *
                               ((H + (1 << kStartShift) - 1) >> kStartShift) + 1;
        if (int rc = ensure_ray_start(v, nst, s)) return rc;
        AZU_TRY_CUDA(cudaMemsetAsync(v->ray_start, 0x7f, nst * sizeof(uint32_t), s));  // 3.4e38: no bound
        const int gb = (v->nb + kFieldSide - 1) / kFieldSide;
        const StartMapArgs sm{p.voxel_size, view.origin, d_pose, fx, fy, cx, cy, W, H, v->ray_start};
        brick_field_kernel<<<dim3(gb, gb, gb), 512, 0, s>>>(v->bricks, v->brick_dist, v->nb, sm, d_gate);
        AZU_LAUNCH_CHECK();
        bricks = v->brick_dist;
        smap = v->ray_start;
    }
    // one instantiation per (format, colour output): without colour output the
    // march carries none of the colour lookup's code
#define AZU_RC_ARGS                                                                                            \
    view, d_pose, fx, fy, cx, cy, W, H, p.truncation, p.min_depth, p.max_depth, d_vertices, d_normals, d_colors, \
        d_gate, bricks, v->nb, smap
    const bool half = p.format != AZU_TSDF_FP32;
    if (half && d_colors) raycast_kernel<true, true><<<grd, blk, 0, s>>>(AZU_RC_ARGS);
    else if (half) raycast_kernel<true, false><<<grd, blk, 0, s>>>(AZU_RC_ARGS);
    else if (d_colors) raycast_kernel<false, true><<<grd, blk, 0, s>>>(AZU_RC_ARGS);
    else raycast_kernel<false, false><<<grd, blk, 0, s>>>(AZU_RC_ARGS);
#undef AZU_RC_ARGS
    AZU_LAUNCH_CHECK();
    return AZU_OK;
}

static int volume_alloc(azu_volume* v) {
    const size_t n = static_cast<size_t>(v->p.resolution) * v->p.resolution * v->p.resolution;
    AZU_TRY_CUDA(cudaMalloc(&v->vox, n * voxel_bytes(v->p.format)));
    if (v->p.color) AZU_TRY_CUDA(cudaMalloc(&v->color, n * 3 * sizeof(float)));
    v->nb = (v->p.resolution + 7) >> kBrickShift;
    AZU_TRY_CUDA(cudaMalloc(&v->bricks, static_cast<size_t>(v->nb) * v->nb * v->nb));
    AZU_TRY_CUDA(cudaMalloc(&v->brick_dist, static_cast<size_t>(v->nb) * v->nb * v->nb));
    v->int_live_words = (v->nb + 31) / 32;
    AZU_TRY_CUDA(cudaMalloc(&v->int_live, static_cast<size_t>(v->nb) * v->nb * v->int_live_words * 4));
    {
        const size_t n_items = static_cast<size_t>(v->p.resolution) * ((v->p.resolution + 31) / 32) * kIntParts;
        AZU_TRY_CUDA(cudaMalloc(&v->int_list, n_items * kIntBuckets * sizeof(int)));
    }
    if (!v->ray_start) {  // a 640 x 480 image; larger ones grow it outside stream capture
        const size_t n = static_cast<size_t>(80 * 60 + 1);
        AZU_TRY_CUDA(cudaMalloc(&v->ray_start, n * sizeof(uint32_t)));
        v->ray_start_cap = n;
    }
    if (!v->d_tiles) {
        const size_t n = static_cast<size_t>(make_tile_mip(640, 480).total);
        AZU_TRY_CUDA(cudaMalloc(&v->d_tiles, n * sizeof(float)));
        v->tile_cap = n;
    }
    return AZU_OK;
}
static void volume_free_storage(azu_volume* v) {
    if (v->vox) cudaFree(v->vox);
    if (v->color) cudaFree(v->color);
    if (v->bricks) cudaFree(v->bricks);
    if (v->brick_dist) cudaFree(v->brick_dist);
    if (v->int_live) cudaFree(v->int_live);
    v->int_live = nullptr;
    if (v->int_list) cudaFree(v->int_list);
    v->int_list = nullptr;
    v->brick_dist = nullptr;
    v->vox = nullptr;
    v->color = nullptr;
    v->bricks = nullptr;
}
int rebuild_bricks(azu_volume* v, cudaStream_t s) {
    const size_t nbr = static_cast<size_t>(v->nb) * v->nb * v->nb;
    const unsigned g = static_cast<unsigned>((nbr + 127) / 128);
    if (v->p.format != AZU_TSDF_FP32) rebuild_bricks_kernel<true><<<g, 128, 0, s>>>(v->vox, v->p.resolution, v->bricks, v->nb);
    else rebuild_bricks_kernel<false><<<g, 128, 0, s>>>(v->vox, v->p.resolution, v->bricks, v->nb);
    AZU_LAUNCH_CHECK();
    return AZU_OK;
}
static int check_params(const azu_volume_params* p) {
    AZU_CHECK_ARG(p != nullptr, "params is null");
    AZU_CHECK_ARG(p->resolution >= 2 && p->resolution <= 2048, "resolution must be in [2, 2048]");
    AZU_CHECK_ARG(p->voxel_size > 0.0f && std::isfinite(p->voxel_size), "voxel_size must be > 0");
    AZU_CHECK_ARG(p->truncation > 0.0f && std::isfinite(p->truncation), "truncation must be > 0");
    AZU_CHECK_ARG(p->max_weight >= 1.0f && p->max_weight <= 65535.0f, "max_weight must be in [1, 65535]");
    AZU_CHECK_ARG(p->format == AZU_TSDF_FP32 || p->format == AZU_TSDF_FP16 || p->format == AZU_TSDF_FP16R, "format");
    AZU_CHECK_ARG(p->format != AZU_TSDF_FP16R || p->max_weight <= 127.0f, "AZU_TSDF_FP16R needs max_weight <= 127");
    return AZU_OK;
}

}  // namespace azu

using namespace azu;

extern "C" int azu_volume_reset(azu_volume* v) {
    AZU_CHECK_ARG(v != nullptr, "volume is null");
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    const size_t n = static_cast<size_t>(v->p.resolution) * v->p.resolution * v->p.resolution;
    const int blocks = static_cast<int>(std::min<size_t>((n + 255) / 256, 152 * 32));
    if (v->p.format != AZU_TSDF_FP32) reset_kernel<true><<<blocks, 256, 0, v->stream.s>>>(v->vox, v->color, n);
    else reset_kernel<false><<<blocks, 256, 0, v->stream.s>>>(v->vox, v->color, n);
    AZU_LAUNCH_CHECK();
    AZU_TRY_CUDA(cudaMemsetAsync(v->d_counters, 0, kCounters * sizeof(unsigned long long), v->stream.s));
    AZU_TRY_CUDA(cudaMemsetAsync(v->bricks, 1, static_cast<size_t>(v->nb) * v->nb * v->nb, v->stream.s));
    v->integrated_frames = 0;
    return AZU_OK;
}

extern "C" int azu_volume_create(int device, const azu_volume_params* p, void* stream, azu_volume** out) {
    AZU_CHECK_ARG(out != nullptr, "out is null");
    *out = nullptr;
    if (int rc = check_params(p)) return rc;
    if (int rc = bind_device(device)) return rc;
    azu_volume* v = new azu_volume();
    v->device = device;
    v->p = *p;
    int rc = v->stream.init(stream);
    if (!rc) rc = volume_alloc(v);
    if (!rc) { cudaError_t e = cudaMalloc(&v->d_pose, 16 * sizeof(float)); if (e) { set_error("cudaMalloc: %s", cudaGetErrorString(e)); rc = AZU_E_NOMEM; } }
    if (!rc) { cudaError_t e = cudaMalloc(&v->d_iconsts, sizeof(IntegrateConsts)); if (e) { set_error("cudaMalloc: %s", cudaGetErrorString(e)); rc = AZU_E_NOMEM; } }
    if (!rc) { cudaError_t e = cudaMalloc(&v->d_counters, kCounters * sizeof(unsigned long long)); if (e) { set_error("cudaMalloc: %s", cudaGetErrorString(e)); rc = AZU_E_NOMEM; } }
    if (!rc) rc = azu_volume_reset(v);
    if (rc) {
        azu_volume_destroy(v);
        return rc;
    }
    *out = v;
    return AZU_OK;
}

extern "C" int azu_volume_destroy(azu_volume* v) {
    if (!v) return AZU_OK;
    cudaSetDevice(v->device);
    if (v->stream.s) cudaStreamSynchronize(v->stream.s);
    volume_free_storage(v);
    if (v->d_pose) cudaFree(v->d_pose);
    if (v->d_iconsts) cudaFree(v->d_iconsts);
    if (v->d_counters) cudaFree(v->d_counters);
    if (v->d_depth_stage) cudaFree(v->d_depth_stage);
    if (v->d_rgb_stage) cudaFree(v->d_rgb_stage);
    if (v->d_tiles) cudaFree(v->d_tiles);
    if (v->ray_start) cudaFree(v->ray_start);
    if (v->d_diff) cudaFree(v->d_diff);
    v->stream.release();
    delete v;
    return AZU_OK;
}

extern "C" int azu_volume_set_params(azu_volume* v, const azu_volume_params* p) {
    AZU_CHECK_ARG(v != nullptr, "volume is null");
    if (int rc = check_params(p)) return rc;
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    const bool realloc = p->resolution != v->p.resolution || p->format != v->p.format || (!!p->color) != (!!v->p.color);
    if (realloc) {
        AZU_TRY_CUDA(cudaStreamSynchronize(v->stream.s));
        volume_free_storage(v);
        v->p = *p;
        if (int rc = volume_alloc(v)) return rc;
    } else {
        v->p = *p;
    }
    return azu_volume_reset(v);
}

extern "C" int azu_volume_get_params(const azu_volume* v, azu_volume_params* p) {
    AZU_CHECK_ARG(v != nullptr && p != nullptr, "null argument");
    *p = v->p;
    return AZU_OK;
}

extern "C" int azu_volume_integrate(azu_volume* v, const float* d_depth_m, const uint8_t* d_rgb, const float pose[16],
                                    float fx, float fy, float cx, float cy, int width, int height, float min_depth,
                                    float max_depth) {
    AZU_CHECK_ARG(v != nullptr && d_depth_m != nullptr && pose != nullptr, "null argument");
    AZU_CHECK_ARG(width > 0 && height > 0, "image size");
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    if (int rc = set_pose_async(v->d_pose, pose, v->stream.s)) return rc;
    if (int rc = volume_integrate_dev(v, d_depth_m, d_rgb, v->d_pose, fx, fy, cx, cy, width, height, min_depth,
                                      max_depth, nullptr, v->stream.s))
        return rc;
    v->integrated_frames++;
    return AZU_OK;
}

extern "C" int azu_volume_integrate_host(azu_volume* v, const float* h_depth_m, const uint8_t* h_rgb,
                                         const float pose[16], float fx, float fy, float cx, float cy, int width,
                                         int height, float min_depth, float max_depth) {
    AZU_CHECK_ARG(v != nullptr && h_depth_m != nullptr && pose != nullptr, "null argument");
    AZU_CHECK_ARG(width > 0 && height > 0, "image size");
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    const size_t n = static_cast<size_t>(width) * height;
    if (n > v->stage_pixels) {
        AZU_TRY_CUDA(cudaStreamSynchronize(v->stream.s));
        if (v->d_depth_stage) cudaFree(v->d_depth_stage);
        if (v->d_rgb_stage) cudaFree(v->d_rgb_stage);
        v->d_depth_stage = nullptr;
        v->d_rgb_stage = nullptr;
        v->stage_pixels = 0;
        AZU_TRY_CUDA(cudaMalloc(&v->d_depth_stage, n * sizeof(float)));
        AZU_TRY_CUDA(cudaMalloc(&v->d_rgb_stage, n * 3));
        v->stage_pixels = n;
    }
    AZU_TRY_CUDA(cudaMemcpyAsync(v->d_depth_stage, h_depth_m, n * sizeof(float), cudaMemcpyHostToDevice, v->stream.s));
    if (h_rgb) AZU_TRY_CUDA(cudaMemcpyAsync(v->d_rgb_stage, h_rgb, n * 3, cudaMemcpyHostToDevice, v->stream.s));
    // Pageable sources: the copies above have returned once the data is staged.
    AZU_TRY_CUDA(cudaStreamSynchronize(v->stream.s));
    return azu_volume_integrate(v, v->d_depth_stage, h_rgb ? v->d_rgb_stage : nullptr, pose, fx, fy, cx, cy, width,
                                height, min_depth, max_depth);
}

extern "C" int azu_volume_raycast(azu_volume* v, const float pose[16], float fx, float fy, float cx, float cy,
                                  int width, int height, float* d_vertices, float* d_normals, uint8_t* d_colors) {
    AZU_CHECK_ARG(v != nullptr && pose != nullptr && d_vertices != nullptr && d_normals != nullptr,
                  "null argument");
    AZU_CHECK_ARG(width > 0 && height > 0, "image size");
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    if (int rc = set_pose_async(v->d_pose, pose, v->stream.s)) return rc;
    return volume_raycast_dev(v, v->d_pose, fx, fy, cx, cy, width, height, d_vertices, d_normals, d_colors, nullptr,
                              v->stream.s);
}

extern "C" int azu_volume_get_stats(azu_volume* v, azu_volume_stats* s) {
    AZU_CHECK_ARG(v != nullptr && s != nullptr, "null argument");
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    unsigned long long c[4];
    AZU_TRY_CUDA(cudaMemcpyAsync(c, v->d_counters, sizeof(c), cudaMemcpyDeviceToHost, v->stream.s));
    AZU_TRY_CUDA(cudaStreamSynchronize(v->stream.s));
    s->integrated_frames = v->integrated_frames;
    s->observed_voxels = static_cast<int64_t>(c[0]);
    s->last_voxels_updated = static_cast<int64_t>(c[1]);
    s->last_color_updates = static_cast<int64_t>(c[2]);
    s->voxels = static_cast<int64_t>(v->p.resolution) * v->p.resolution * v->p.resolution;
    s->total_voxels_updated = static_cast<int64_t>(c[3]);
    return AZU_OK;
}

static int transfer(azu_volume* v, float* ht, float* hw, float* hc, const float* ut, const float* uw,
                    const float* uc, bool download) {
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    const size_t n = static_cast<size_t>(v->p.resolution) * v->p.resolution * v->p.resolution;
    const size_t chunk = std::min<size_t>(n, size_t(1) << 24);
    float *dt = nullptr, *dw = nullptr;
    AZU_TRY_CUDA(cudaStreamSynchronize(v->stream.s));
    cudaError_t e = cudaMalloc(&dt, chunk * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dw, chunk * sizeof(float));
    const int fmt = v->p.format;
    for (size_t base = 0; e == cudaSuccess && base < n; base += chunk) {
        const size_t m = std::min(chunk, n - base);
        const int blocks = static_cast<int>((m + 255) / 256);
        if (download) {
            if (fmt == AZU_TSDF_FP16R) unpack_kernel<true, true><<<blocks, 256, 0, v->stream.s>>>(v->vox, base, m, dt, dw);
            else if (fmt == AZU_TSDF_FP16) unpack_kernel<true, false><<<blocks, 256, 0, v->stream.s>>>(v->vox, base, m, dt, dw);
            else unpack_kernel<false, false><<<blocks, 256, 0, v->stream.s>>>(v->vox, base, m, dt, dw);
            e = cudaGetLastError();
            if (e == cudaSuccess && ht) e = cudaMemcpyAsync(ht + base, dt, m * sizeof(float), cudaMemcpyDeviceToHost, v->stream.s);
            if (e == cudaSuccess && hw) e = cudaMemcpyAsync(hw + base, dw, m * sizeof(float), cudaMemcpyDeviceToHost, v->stream.s);
        } else {
            e = cudaMemcpyAsync(dt, ut + base, m * sizeof(float), cudaMemcpyHostToDevice, v->stream.s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(dw, uw + base, m * sizeof(float), cudaMemcpyHostToDevice, v->stream.s);
            if (e == cudaSuccess) {
                if (fmt == AZU_TSDF_FP16R) pack_kernel<true, true><<<blocks, 256, 0, v->stream.s>>>(v->vox, base, m, dt, dw);
                else if (fmt == AZU_TSDF_FP16) pack_kernel<true, false><<<blocks, 256, 0, v->stream.s>>>(v->vox, base, m, dt, dw);
                else pack_kernel<false, false><<<blocks, 256, 0, v->stream.s>>>(v->vox, base, m, dt, dw);
                e = cudaGetLastError();
            }
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(v->stream.s);
    }
    if (e == cudaSuccess && v->color) {
        if (download && hc) e = cudaMemcpy(hc, v->color, 3 * n * sizeof(float), cudaMemcpyDeviceToHost);
        if (!download && uc) e = cudaMemcpy(v->color, uc, 3 * n * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (dt) cudaFree(dt);
    if (dw) cudaFree(dw);
    if (e != cudaSuccess) {
        set_error("volume transfer: %s", cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? AZU_E_NOMEM : AZU_E_CUDA;
    }
    return AZU_OK;
}

extern "C" int azu_volume_download(azu_volume* v, float* h_tsdf, float* h_weight, float* h_color) {
    AZU_CHECK_ARG(v != nullptr, "volume is null");
    return transfer(v, h_tsdf, h_weight, h_color, nullptr, nullptr, nullptr, true);
}

extern "C" int azu_volume_upload(azu_volume* v, const float* h_tsdf, const float* h_weight, const float* h_color) {
    AZU_CHECK_ARG(v != nullptr && h_tsdf != nullptr && h_weight != nullptr, "null argument");
    if (int rc = transfer(v, nullptr, nullptr, nullptr, h_tsdf, h_weight, h_color, false)) return rc;
    if (int rc = rebuild_bricks(v, v->stream.s)) return rc;
    AZU_TRY_CUDA(cudaStreamSynchronize(v->stream.s));
    return AZU_OK;
}

extern "C" int azu_volume_set_free_space_skipping(azu_volume* v, int on) {
    AZU_CHECK_ARG(v != nullptr, "volume is null");
    v->skip_free = on != 0;
    return AZU_OK;
}

extern "C" void* azu_volume_device_voxels(azu_volume* v) { return v ? v->vox : nullptr; }

extern "C" int azu_volume_voxels_changed(azu_volume* v) {
    AZU_CHECK_ARG(v != nullptr, "volume is null");
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    return rebuild_bricks(v, v->stream.s);
}

extern "C" int azu_volume_point_cloud(azu_volume* v, float* h_points, uint8_t* h_colors, int64_t capacity,
                                      int64_t* n_points) {
    AZU_CHECK_ARG(v != nullptr && n_points != nullptr, "null argument");
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    cudaStream_t s = v->stream.s;
    const size_t n = static_cast<size_t>(v->p.resolution) * v->p.resolution * v->p.resolution;
    const size_t nblocks = (n + kPcBlock - 1) / kPcBlock;
    const bool half = v->p.format != AZU_TSDF_FP32;
    int* d_counts = nullptr;
    long long* d_off = nullptr;
    float* d_pts = nullptr;
    uint8_t* d_col = nullptr;
    int rc = AZU_OK;
    std::vector<int> counts(nblocks);
    std::vector<long long> off(nblocks);
    long long total = 0;
    auto fail = [&](cudaError_t e) {
        set_error("point cloud: %s", cudaGetErrorString(e));
        rc = e == cudaErrorMemoryAllocation ? AZU_E_NOMEM : AZU_E_CUDA;
    };
    cudaError_t e = cudaMalloc(&d_counts, nblocks * sizeof(int));
    if (!e) e = cudaMalloc(&d_off, nblocks * sizeof(long long));
    if (!e) {
        if (half) pc_count_kernel<true><<<static_cast<unsigned>(nblocks), kPcThreads, 0, s>>>(v->vox, v->color, n, d_counts);
        else pc_count_kernel<false><<<static_cast<unsigned>(nblocks), kPcThreads, 0, s>>>(v->vox, v->color, n, d_counts);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpyAsync(counts.data(), d_counts, nblocks * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (e) fail(e);
    if (!rc) {
        for (size_t b = 0; b < nblocks; ++b) { off[b] = total; total += counts[b]; }
        *n_points = total;
        if (h_points || h_colors) {
            if (capacity < total) {
                set_error("point cloud: %lld points, capacity %lld", total, static_cast<long long>(capacity));
                rc = AZU_E_INVALID;
            }
        }
    }
    if (!rc && (h_points || h_colors) && total > 0) {
        e = cudaMemcpyAsync(d_off, off.data(), nblocks * sizeof(long long), cudaMemcpyHostToDevice, s);
        if (!e) e = cudaMalloc(&d_pts, static_cast<size_t>(total) * 3 * sizeof(float));
        if (!e) e = cudaMalloc(&d_col, static_cast<size_t>(total) * 3);
        const F3 org = mk3(v->p.origin[0], v->p.origin[1], v->p.origin[2]);
        if (!e) {
            if (half)
                pc_emit_kernel<true><<<static_cast<unsigned>(nblocks), kPcThreads, 0, s>>>(
                    v->vox, v->color, n, v->p.resolution, v->p.voxel_size, org, d_off, d_pts, d_col);
            else
                pc_emit_kernel<false><<<static_cast<unsigned>(nblocks), kPcThreads, 0, s>>>(
                    v->vox, v->color, n, v->p.resolution, v->p.voxel_size, org, d_off, d_pts, d_col);
            e = cudaGetLastError();
        }
        if (!e && h_points)
            e = cudaMemcpyAsync(h_points, d_pts, static_cast<size_t>(total) * 3 * sizeof(float), cudaMemcpyDeviceToHost, s);
        if (!e && h_colors) e = cudaMemcpyAsync(h_colors, d_col, static_cast<size_t>(total) * 3, cudaMemcpyDeviceToHost, s);
        if (!e) e = cudaStreamSynchronize(s);
        if (e) fail(e);
    }
    for (void* p : {(void*)d_counts, (void*)d_off, (void*)d_pts, (void*)d_col})
        if (p) cudaFree(p);
    return rc;
}

extern "C" int azu_volume_raycast_many(azu_volume* v, const float* poses, int count, float fx, float fy, float cx,
                                       float cy, int width, int height, float* d_vertices, float* d_normals) {
    AZU_CHECK_ARG(v != nullptr && poses != nullptr && d_vertices != nullptr && d_normals != nullptr, "null argument");
    AZU_CHECK_ARG(count >= 1 && count <= 65535 && width > 0 && height > 0, "count / image size");
    AZU_TRY_CUDA(cudaSetDevice(v->device));
    cudaStream_t s = v->stream.s;
    float* d_poses = nullptr;
    AZU_TRY_CUDA(cudaMalloc(&d_poses, 16 * sizeof(float) * count));
    cudaError_t e = cudaMemcpyAsync(d_poses, poses, 16 * sizeof(float) * count, cudaMemcpyHostToDevice, s);
    const azu_volume_params& p = v->p;
    const VolView view = make_view(v);
    const uint8_t* bricks = nullptr;
    if (!e && v->skip_free) {
        // the distance field only: each image has its own pose, so no start map
        const int gb = (v->nb + kFieldSide - 1) / kFieldSide;
        const StartMapArgs sm{p.voxel_size, view.origin, nullptr, fx, fy, cx, cy, width, height, nullptr};
        brick_field_kernel<<<dim3(gb, gb, gb), 512, 0, s>>>(v->bricks, v->brick_dist, v->nb, sm, nullptr);
        e = cudaGetLastError();
        bricks = v->brick_dist;
    }
    if (!e) {
        const dim3 blk(32, 8), grd((width + 31) / 32, (height + 7) / 8, count);
        if (p.format != AZU_TSDF_FP32)
            raycast_many_kernel<true><<<grd, blk, 0, s>>>(view, d_poses, fx, fy, cx, cy, width, height, p.truncation,
                                                          p.min_depth, p.max_depth, d_vertices, d_normals, bricks,
                                                          v->nb);
        else
            raycast_many_kernel<false><<<grd, blk, 0, s>>>(view, d_poses, fx, fy, cx, cy, width, height,
                                                           p.truncation, p.min_depth, p.max_depth, d_vertices,
                                                           d_normals, bricks, v->nb);
        e = cudaGetLastError();
    }
    if (!e) e = cudaStreamSynchronize(s);
    cudaFree(d_poses);
    if (e) {
        set_error("raycast_many: %s", cudaGetErrorString(e));
        return AZU_E_CUDA;
    }
    return AZU_OK;
}
