// Depth-buffer pyramid (vren/vren/pipeline/depth_buffer_pyramid.cpp, depth_buffer_reductor::copy_and_reduce
// at :212-303; shaders vren/resources/shaders/depth_buffer_copy.comp and depth_buffer_reduce.comp).
//
// Level 0 is an exact copy of the depth buffer; level l + 1 (size max(size_l >> 1, 1) per axis) holds,
// per texel, GLSL max folded from 0 over the 2x2 texels of level l that lie inside level l.  The
// reference runs one copy dispatch and one dispatch per level with a barrier between them.  Here the
// whole pyramid is two launches:
//
//  - depth_pyramid_tiles_kernel: a CTA owns a 64x64 tile of level 0: it loads the tile once (128-bit
//    loads when rows are 16-byte aligned), writes the level-0 copy, and folds levels 1..6 of the tile
//    on chip (levels 1 and 2 in each lane's registers, level 3 by warp shuffles, levels 4..6 in one
//    warp after the CTA's only barrier), writing each level's texels that lie inside the level;
//  - depth_pyramid_upper_kernel (only with more than 7 levels), launched with programmatic stream
//    serialisation so that it is resident before the tiles finish: one CTA per 64x64 block of level-6
//    texels folds levels 7..12 the same way; beyond that (sides >= 8192) the blocks count their
//    arrival per 64x64 block of level-12 texels and the last to arrive (no CTA ever waits) folds
//    levels 13..15 (16 levels cover sides up to 65535).
//
// Counting arrivals in the tile kernel itself (one launch) measured 2-4 us slower at 1920x1080 and
// 3840x2160 and 12 us slower at 8192x8192: the fence and atomic lengthen every CTA's life.
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
    uint32_t counter_base[kPyrMaxStages];         // arrival counters of stage 2's blocks
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
    float lvl3[8][8];
    int last;
};

// Thread layout of a 64x64 source tile: warp w owns source rows 8w .. 8w+7; lane l owns the 4x4 block
// at rows 8w + 4(l >> 4) + k and columns 4(l & 15) + c, held as v[k][c].  Levels base+1 and base+2 of
// that block then fold in registers, level base+3 (one row of 8 texels per warp) with two shuffles,
// and levels base+4 .. base+6 (4x4, 2x2, 1x1 texels) in warp 0 after one barrier.
__device__ void pyr_fold_tile(const PyramidDesc& d, float* __restrict__ pyramid, uint32_t base, uint32_t top,
                              uint32_t tx, uint32_t ty, const float (&v)[4][4], PyramidSmem& sm)
{
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t hr = lane >> 4, hc = lane & 15;
    // level base + 1: the lane's 2x2 texels
    float m1[2][2];
    {
        const uint32_t l = base + 1, lw = d.w[l], lh = d.h[l];
        float* out = pyramid + d.off[l];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const uint32_t gy = ty * 32 + 4 * warp + 2 * hr + i;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const uint32_t gx = tx * 32 + 2 * hc + j;
                const float m = pyr_fold(v[2 * i][2 * j], v[2 * i + 1][2 * j], v[2 * i][2 * j + 1], v[2 * i + 1][2 * j + 1]);
                const bool inside = gx < lw && gy < lh;
                m1[i][j] = inside ? m : 0.0f;
                if (inside) out[(size_t)gy * lw + gx] = m;
            }
        }
    }
    if (base + 2 > top) return;
    // level base + 2: one texel per lane (row 2w + hr, column hc of the tile's 16x16)
    float m2;
    {
        const uint32_t l = base + 2, gy = ty * 16 + 2 * warp + hr, gx = tx * 16 + hc;
        const float m = pyr_fold(m1[0][0], m1[1][0], m1[0][1], m1[1][1]);
        const bool inside = gx < d.w[l] && gy < d.h[l];
        m2 = inside ? m : 0.0f;
        if (inside) pyramid[d.off[l] + (size_t)gy * d.w[l] + gx] = m;
    }
    if (base + 3 > top) return;
    // level base + 3: lanes 0, 2, .., 14 hold texel (row w, column hc / 2) of the tile's 8x8
    {
        const float x1 = __shfl_xor_sync(0xffffffffu, m2, 1);
        const float y1 = __shfl_xor_sync(0xffffffffu, m2, 16);
        const float x1y1 = __shfl_xor_sync(0xffffffffu, m2, 17);
        const uint32_t l = base + 3, gy = ty * 8 + warp, gx = tx * 8 + (hc >> 1);
        const float m = pyr_fold(m2, y1, x1, x1y1);
        const bool inside = gx < d.w[l] && gy < d.h[l];
        if (lane < 16 && (lane & 1) == 0) {
            sm.lvl3[warp][hc >> 1] = inside ? m : 0.0f;
            if (inside) pyramid[d.off[l] + (size_t)gy * d.w[l] + gx] = m;
        }
    }
    if (base + 4 > top) return;
    __syncthreads();
    if (warp != 0) return;
    // level base + 4: lane < 16 holds texel (row lane >> 2, column lane & 3) of the tile's 4x4
    const uint32_t qy = (lane >> 2) & 3, qx = lane & 3;
    float m4 = 0.0f;
    {
        const uint32_t l = base + 4, gy = ty * 4 + qy, gx = tx * 4 + qx;
        const float m = pyr_fold(sm.lvl3[2 * qy][2 * qx], sm.lvl3[2 * qy + 1][2 * qx], sm.lvl3[2 * qy][2 * qx + 1],
                                 sm.lvl3[2 * qy + 1][2 * qx + 1]);
        const bool inside = gx < d.w[l] && gy < d.h[l];
        if (lane < 16) {
            m4 = inside ? m : 0.0f;
            if (inside) pyramid[d.off[l] + (size_t)gy * d.w[l] + gx] = m;
        }
    }
    if (base + 5 > top) return;
    // level base + 5: lanes 0, 2, 8, 10 hold texel (row qy / 2, column qx / 2) of the tile's 2x2
    float m5;
    {
        const float x1 = __shfl_xor_sync(0xffffffffu, m4, 1);
        const float y1 = __shfl_xor_sync(0xffffffffu, m4, 4);
        const float x1y1 = __shfl_xor_sync(0xffffffffu, m4, 5);
        const uint32_t l = base + 5, gy = ty * 2 + (qy >> 1), gx = tx * 2 + (qx >> 1);
        const float m = pyr_fold(m4, y1, x1, x1y1);
        const bool inside = gx < d.w[l] && gy < d.h[l];
        m5 = inside ? m : 0.0f;
        if (lane < 16 && (lane & 5) == 0 && inside) pyramid[d.off[l] + (size_t)gy * d.w[l] + gx] = m;
    }
    if (base + 6 > top) return;
    // level base + 6: lane 0 holds the tile's texel
    {
        const float x1 = __shfl_xor_sync(0xffffffffu, m5, 2);
        const float y1 = __shfl_xor_sync(0xffffffffu, m5, 8);
        const float x1y1 = __shfl_xor_sync(0xffffffffu, m5, 10);
        const uint32_t l = base + 6;
        const float m = pyr_fold(m5, y1, x1, x1y1);
        if (lane == 0 && tx < d.w[l] && ty < d.h[l]) pyramid[d.off[l] + (size_t)ty * d.w[l] + tx] = m;
    }
}

__device__ __forceinline__ uint32_t pyr_row(uint32_t ty, uint32_t k)
{
    return ty * kPyrTile + 8 * (threadIdx.x >> 5) + 4 * ((threadIdx.x & 31) >> 4) + k;
}

// Levels 0..min(6, last) of one 64x64 tile per CTA.  No CTA waits on another and none counts its
// arrival: the levels above 6 are folded by depth_pyramid_upper_kernel, launched behind this grid.
__global__ void __launch_bounds__(kPyrThreads, 8) depth_pyramid_tiles_kernel(const float* __restrict__ depth,
                                                                            float* __restrict__ pyramid,
                                                                            PyramidDesc d)
{
    __shared__ PyramidSmem sm;
    // the upper-level grid may be scheduled now; it waits for this grid's completion before reading
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const uint32_t tx = blockIdx.x % d.tiles_x[0], ty = blockIdx.x / d.tiles_x[0];
    const uint32_t W = d.w[0], H = d.h[0];
    const uint32_t x0 = tx * kPyrTile + 4 * (threadIdx.x & 15);
    float v[4][4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t y = pyr_row(ty, k);
        if (d.vec_level0) {
            float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (y < H && x0 < W) {
                q = __ldcs(reinterpret_cast<const float4*>(depth + (size_t)y * W + x0));
                __stcs(reinterpret_cast<float4*>(pyramid + (size_t)y * W + x0), q);
            }
            v[k][0] = q.x;
            v[k][1] = q.y;
            v[k][2] = q.z;
            v[k][3] = q.w;
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float s = 0.0f;
                if (y < H && x0 + c < W) {
                    s = __ldcs(depth + (size_t)y * W + x0 + c);
                    __stcs(pyramid + (size_t)y * W + x0 + c, s);
                }
                v[k][c] = s;
            }
        }
    }
    if (d.levels > 1) pyr_fold_tile(d, pyramid, 0, min((uint32_t)kPyrLevelsPerStage, d.levels - 1), tx, ty, v, sm);
}

// Levels 7 and up: one CTA per 64x64 block of level-6 texels folds levels 7..12 of its block; with
// more levels, the blocks count their arrival per 64x64 block of level-12 texels and the last one to
// arrive (no CTA waits) folds levels 13..15.  Launched with programmatic stream serialisation behind
// depth_pyramid_tiles_kernel: griddepcontrol.wait returns once that grid has completed and its writes
// are visible.
__global__ void __launch_bounds__(kPyrThreads, 8) depth_pyramid_upper_kernel(float* __restrict__ pyramid,
                                                                            PyramidDesc d,
                                                                            uint32_t* __restrict__ counters)
{
    __shared__ PyramidSmem sm;
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t col = 4 * (threadIdx.x & 15);
    const uint32_t last_level = d.levels - 1;
    uint32_t stage = 1;
    uint32_t tx = blockIdx.x % d.tiles_x[1], ty = blockIdx.x / d.tiles_x[1];
    float v[4][4];
    for (;;) {
        // source: level 6 * stage, written by the previous grid (stage 1) or by other CTAs (stage 2)
        const uint32_t src = stage * kPyrLevelsPerStage;
        const uint32_t W = d.w[src], H = d.h[src];
        const float* s = pyramid + d.off[src];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t y = pyr_row(ty, k);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const uint32_t x = tx * kPyrTile + col + c;
                v[k][c] = (y < H && x < W) ? __ldcg(s + (size_t)y * W + x) : 0.0f;
            }
        }
        const uint32_t top = min(src + kPyrLevelsPerStage, last_level);
        pyr_fold_tile(d, pyramid, src, top, tx, ty, v, sm);
        if (top == last_level) return;
        // Arrival on the parent block.  Thread 0 wrote this block's texel of level src + 6 (the only
        // one the next stage reads); the last arriver folds the next stage.
        const uint32_t px = tx / kPyrTile, py = ty / kPyrTile;
        if (threadIdx.x == 0) {
            const uint32_t nx = min((uint32_t)kPyrTile, d.tiles_x[stage] - px * kPyrTile);
            const uint32_t ny = min((uint32_t)kPyrTile, d.tiles_y[stage] - py * kPyrTile);
            uint32_t* c = counters + d.counter_base[stage + 1] + py * d.tiles_x[stage + 1] + px;
            __threadfence();
            const uint32_t prev = atomicAdd(c, 1u);
            const int last = prev == nx * ny - 1;
            if (last) *c = 0u;  // reusable by the next call (no other block of this parent is left)
            sm.last = last;
        }
        __syncthreads();
        if (!sm.last) return;
        __threadfence();
        ++stage;
        tx = px;
        ty = py;
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
        if (s >= 2) base += tw * th;
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
    cudaStream_t st = as_stream(s);
    launch_kernel(depth_pyramid_tiles_kernel, d.tiles_x[0] * d.tiles_y[0], kPyrThreads, 0, st, depth_buffer,
                  pyramid, d);
    VREN_LAUNCH_CHECK();
    if (d.levels > kPyrLevelsPerStage + 1) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(d.tiles_x[1] * d.tiles_y[1]);
        cfg.blockDim = dim3(kPyrThreads);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, depth_pyramid_upper_kernel, pyramid, d, static_cast<uint32_t*>(scratch));
        VREN_LAUNCH_CHECK();
    }
    return VREN_OK;
}
