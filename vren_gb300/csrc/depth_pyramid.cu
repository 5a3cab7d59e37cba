// Depth-buffer pyramid (vren/vren/pipeline/depth_buffer_pyramid.cpp, depth_buffer_reductor::copy_and_reduce
// at :212-303; shaders vren/resources/shaders/depth_buffer_copy.comp and depth_buffer_reduce.comp).
//
// Level 0 is an exact copy of the depth buffer; level l + 1 (size max(size_l >> 1, 1) per axis) holds,
// per texel, GLSL max folded from 0 over the 2x2 texels of level l that lie inside level l.  The
// reference runs one copy dispatch and one dispatch per level with a barrier between them.  Here the
// whole pyramid is one launch:
//
//  - a CTA owns a 64x64 tile of level 0: it loads the tile once (128-bit loads when rows are 16-byte
//    aligned), writes the level-0 copy, and folds levels 1..6 of the tile on chip (level 1 from
//    registers, levels 2..6 in shared memory), writing each level's texels that lie inside the level;
//  - level 6 has one texel per tile.  The tiles of a 64x64 block of level-6 texels count their arrival
//    on a counter; the last one to arrive (no CTA ever waits) reads that block back from L2 and folds
//    levels 7..12 the same way, and likewise 13..15 (16 levels cover sides up to 65535).
//
// Texels outside their level are held as 0 on chip, which is how the reference's "source inside the
// level" test enters: the fold never sees them.  The fold skips NaN sources (max(m, NaN) keeps m) and
// never produces -0 (it starts from +0 and only takes strictly larger values), so every texel above
// level 0 is +0 or positive and the result does not depend on the order of the fold.
//
// Traffic: 4 B read + 4 B written per level-0 texel, plus 4 B written per texel of levels >= 1.
#include "common.cuh"

namespace vren_gb300 {
namespace {

constexpr int kPyrTile = 64;            // source texels per tile side; 6 levels per stage
constexpr int kPyrLevelsPerStage = 6;
constexpr int kPyrThreads = 256;
constexpr uint32_t kPyrMaxLevels = 16;  // depth_buffer_pyramid::k_max_depth_buffer_pyramid_level_count
constexpr uint32_t kPyrMaxStages = 3;   // 16 levels: stage 0 -> levels 1..6, 1 -> 7..12, 2 -> 13..15
constexpr size_t kPyrLevelAlign = 64;   // floats: every level starts on a 256-byte boundary

struct PyramidDesc {
    uint32_t levels;
    uint32_t w[kPyrMaxLevels], h[kPyrMaxLevels];
    uint64_t off[kPyrMaxLevels];                  // level start, in floats from the pyramid base
    uint32_t tiles_x[kPyrMaxStages], tiles_y[kPyrMaxStages];
    uint32_t counter_base[kPyrMaxStages];         // arrival counters of stage s's tiles (s >= 1)
    uint32_t vec_level0;                          // rows of the depth and of level 0 are 16-byte aligned
};

__host__ __device__ inline uint32_t pyr_dim(uint32_t base, uint32_t level)
{
    const uint32_t d = base >> level;
    return d ? d : 1u;
}

__device__ __forceinline__ float pyr_max(float m, float v) { return m < v ? v : m; }

// The reference's fold order (depth_buffer_reduce.comp:22-31): x outer, y inner.
__device__ __forceinline__ float pyr_fold(float x0y0, float x0y1, float x1y0, float x1y1)
{
    float m = 0.0f;
    m = pyr_max(m, x0y0);
    m = pyr_max(m, x0y1);
    m = pyr_max(m, x1y0);
    m = pyr_max(m, x1y1);
    return m;
}

struct PyramidSmem {
    float lvl1[32][33];
    float lvl2[16][17];
    float lvl3[8][9];
    float lvl4[4][4];
    float lvl5[2][2];
    int last;
};

// Folds the tile (tx, ty) of level `base` (64x64 source texels, held by the CTA's threads as
// v[row][col]: thread t owns source columns 4*(t & 15) + 0..3 of rows 2*(t >> 4) + {0, 1, 32, 33})
// into levels base+1 .. top, writing each level's texels that lie inside it.
__device__ void pyr_fold_tile(const PyramidDesc& d, float* __restrict__ pyramid, uint32_t base, uint32_t top,
                              uint32_t tx, uint32_t ty, const float (&v)[4][4], PyramidSmem& sm)
{
    const int t = threadIdx.x;
    const uint32_t cq = t & 15, rp = t >> 4;
    // level base + 1: from registers; texel columns 2cq, 2cq+1, rows rp and rp + 16
    {
        const uint32_t l = base + 1, lw = d.w[l], lh = d.h[l];
        float* out = pyramid + d.off[l];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const uint32_t ly = rp + 16 * half, gy = ty * 32 + ly;
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const uint32_t lx = 2 * cq + k, gx = tx * 32 + lx;
                const float* r0 = v[2 * half];
                const float* r1 = v[2 * half + 1];
                float m = pyr_fold(r0[2 * k], r1[2 * k], r0[2 * k + 1], r1[2 * k + 1]);
                const bool inside = gx < lw && gy < lh;
                m = inside ? m : 0.0f;
                sm.lvl1[ly][lx] = m;
                if (inside) out[(size_t)gy * lw + gx] = m;
            }
        }
    }
    __syncthreads();
    // levels base + 2 .. top, in shared memory (16x16, 8x8, 4x4, 2x2, 1x1 texels of the tile)
#define VREN_PYR_LEVEL(SRC, DST, DIM, K)                                                                 \
    if (base + K <= top) {                                                                               \
        const uint32_t l = base + K;                                                                     \
        if (t < DIM * DIM) {                                                                             \
            const uint32_t lx = t % DIM, ly = t / DIM;                                                   \
            const uint32_t gx = tx * DIM + lx, gy = ty * DIM + ly;                                       \
            float m = pyr_fold(SRC[2 * ly][2 * lx], SRC[2 * ly + 1][2 * lx], SRC[2 * ly][2 * lx + 1],    \
                               SRC[2 * ly + 1][2 * lx + 1]);                                             \
            const bool inside = gx < d.w[l] && gy < d.h[l];                                              \
            m = inside ? m : 0.0f;                                                                       \
            DST;                                                                                         \
            if (inside) pyramid[d.off[l] + (size_t)gy * d.w[l] + gx] = m;                                \
        }                                                                                                \
        __syncthreads();                                                                                 \
    }
    VREN_PYR_LEVEL(sm.lvl1, sm.lvl2[ly][lx] = m, 16, 2)
    VREN_PYR_LEVEL(sm.lvl2, sm.lvl3[ly][lx] = m, 8, 3)
    VREN_PYR_LEVEL(sm.lvl3, sm.lvl4[ly][lx] = m, 4, 4)
    VREN_PYR_LEVEL(sm.lvl4, sm.lvl5[ly][lx] = m, 2, 5)
    VREN_PYR_LEVEL(sm.lvl5, (void)0, 1, 6)
#undef VREN_PYR_LEVEL
}

__global__ void __launch_bounds__(kPyrThreads) depth_pyramid_kernel(const float* __restrict__ depth,
                                                                   float* __restrict__ pyramid, PyramidDesc d,
                                                                   uint32_t* __restrict__ counters)
{
    __shared__ PyramidSmem sm;
    const int t = threadIdx.x;
    const uint32_t cq = t & 15, rp = t >> 4;
    uint32_t tx = blockIdx.x % d.tiles_x[0], ty = blockIdx.x / d.tiles_x[0];
    const uint32_t last_level = d.levels - 1;

    // ---- stage 0: level-0 tile (loads, exact copy), levels 1..6
    float v[4][4];
    {
        const uint32_t W = d.w[0], H = d.h[0];
        const uint32_t x0 = tx * kPyrTile + 4 * cq;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t y = ty * kPyrTile + 2 * rp + (r & 1) + 32 * (r >> 1);
            if (d.vec_level0) {
                float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (y < H && x0 < W) {
                    q = __ldcs(reinterpret_cast<const float4*>(depth + (size_t)y * W + x0));
                    __stcs(reinterpret_cast<float4*>(pyramid + (size_t)y * W + x0), q);
                }
                v[r][0] = q.x;
                v[r][1] = q.y;
                v[r][2] = q.z;
                v[r][3] = q.w;
            } else {
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float s = 0.0f;
                    if (y < H && x0 + c < W) {
                        s = __ldcs(depth + (size_t)y * W + x0 + c);
                        __stcs(pyramid + (size_t)y * W + x0 + c, s);
                    }
                    v[r][c] = s;
                }
            }
        }
    }
    if (last_level == 0) return;
    uint32_t stage = 0;
    for (;;) {
        const uint32_t base = stage * kPyrLevelsPerStage;
        const uint32_t top = min(base + kPyrLevelsPerStage, last_level);
        pyr_fold_tile(d, pyramid, base, top, tx, ty, v, sm);
        if (top == last_level) return;
        // arrival on the parent block of 64x64 tiles; the last arriver folds the next stage
        const uint32_t px = tx / kPyrTile, py = ty / kPyrTile;
        if (t == 0) {
            const uint32_t nx = min((uint32_t)kPyrTile, d.tiles_x[stage] - px * kPyrTile);
            const uint32_t ny = min((uint32_t)kPyrTile, d.tiles_y[stage] - py * kPyrTile);
            uint32_t* c = counters + d.counter_base[stage + 1] + py * d.tiles_x[stage + 1] + px;
            __threadfence();
            const uint32_t prev = atomicAdd(c, 1u);
            const int last = prev == nx * ny - 1;
            if (last) *c = 0u;  // reusable by the next call (no other tile of this block is left)
            sm.last = last;
        }
        __syncthreads();
        if (!sm.last) return;
        __threadfence();
        ++stage;
        tx = px;
        ty = py;
        // source: level `base + 6` (the tiles' level-6 texels, written by other CTAs, read from L2)
        const uint32_t src = stage * kPyrLevelsPerStage;
        const uint32_t W = d.w[src], H = d.h[src];
        const float* s = pyramid + d.off[src];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t y = ty * kPyrTile + 2 * rp + (r & 1) + 32 * (r >> 1);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const uint32_t x = tx * kPyrTile + 4 * cq + c;
                v[r][c] = (y < H && x < W) ? __ldcg(s + (size_t)y * W + x) : 0.0f;
            }
        }
    }
}

bool pyramid_desc(uint32_t width, uint32_t height, PyramidDesc& d, size_t* total_floats, uint32_t* counters)
{
    if (width == 0 || height == 0 || width > 65535u || height > 65535u) return false;
    memset(&d, 0, sizeof(d));
    uint32_t m = width > height ? width : height, lg = 0;
    while (m >>= 1) ++lg;
    d.levels = lg + 1;
    uint64_t off = 0;
    for (uint32_t l = 0; l < d.levels; ++l) {
        d.w[l] = pyr_dim(width, l);
        d.h[l] = pyr_dim(height, l);
        d.off[l] = off;
        off += ((uint64_t)d.w[l] * d.h[l] + kPyrLevelAlign - 1) / kPyrLevelAlign * kPyrLevelAlign;
    }
    uint32_t tw = (width + kPyrTile - 1) / kPyrTile, th = (height + kPyrTile - 1) / kPyrTile, base = 0;
    for (uint32_t s = 0; s < kPyrMaxStages; ++s) {
        d.tiles_x[s] = tw;
        d.tiles_y[s] = th;
        d.counter_base[s] = base;
        if (s >= 1) base += tw * th;
        tw = (tw + kPyrTile - 1) / kPyrTile;
        th = (th + kPyrTile - 1) / kPyrTile;
    }
    if (total_floats) *total_floats = off;
    if (counters) *counters = base;
    return true;
}

}  // namespace
}  // namespace vren_gb300

using namespace vren_gb300;

extern "C" uint32_t vren_depth_pyramid_level_count(uint32_t width, uint32_t height)
{
    PyramidDesc d;
    return pyramid_desc(width, height, d, nullptr, nullptr) ? d.levels : 0u;
}

extern "C" size_t vren_depth_pyramid_level_offset(uint32_t width, uint32_t height, uint32_t level)
{
    PyramidDesc d;
    size_t total = 0;
    if (!pyramid_desc(width, height, d, &total, nullptr) || level > d.levels) return 0;
    return level == d.levels ? total : (size_t)d.off[level];
}

extern "C" size_t vren_depth_pyramid_scratch_bytes(uint32_t width, uint32_t height)
{
    PyramidDesc d;
    uint32_t counters = 0;
    if (!pyramid_desc(width, height, d, nullptr, &counters)) return 0;
    return (size_t)(counters ? counters : 1u) * sizeof(uint32_t);
}

extern "C" int vren_depth_pyramid_copy_and_reduce(vren_stream_t s, const float* depth_buffer, uint32_t width,
                                                  uint32_t height, float* pyramid, void* scratch)
{
    PyramidDesc d;
    uint32_t counters = 0;
    if (!depth_buffer || !pyramid || !pyramid_desc(width, height, d, nullptr, &counters)) return VREN_ERR_ARG;
    if (counters && !scratch) return VREN_ERR_ARG;
    if (((uintptr_t)depth_buffer | (uintptr_t)pyramid) & 3u) return VREN_ERR_ARG;
    d.vec_level0 = (width % 4 == 0) && (((uintptr_t)depth_buffer | (uintptr_t)pyramid) & 15u) == 0;
    const uint32_t grid = d.tiles_x[0] * d.tiles_y[0];
    launch_kernel(depth_pyramid_kernel, grid, kPyrThreads, 0, as_stream(s), depth_buffer, pyramid, d,
                  static_cast<uint32_t*>(scratch));
    VREN_LAUNCH_CHECK();
    return VREN_OK;
}
