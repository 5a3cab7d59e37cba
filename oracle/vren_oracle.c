/*
 * vren_oracle.c — CPU oracle for the vren hot path.  TEST INFRASTRUCTURE ONLY: used by the
 * tests, the smoke check and the benchmark's CPU-baseline leg as the oracle, never by the
 * product path.  See vren_oracle.h for what is pinned (primitives) and what is unpinned
 * (clustered shading stages).
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fopenmp (oracle/build.py).
 */
#include "vren_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define INVALID_NODE 0xFFFFFFFEu
#define LEAF_NODE 0xFFFFFFFFu

static int nthreads(int t)
{
#ifdef _OPENMP
    return t > 0 ? t : omp_get_max_threads();
#else
    (void)t;
    return 1;
#endif
}

/* ================================================================================================
 * Size helpers — vren/vren/base/base.hpp:37-79 and vren/vren/primitives/build_bvh.cpp:101-136,
 * with the reference's double-precision log/pow where it uses them.
 * ================================================================================================ */
uint32_t oracle_round_to_next_power_of_2(uint32_t v)
{
    v--;
    v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16;
    v++;
    return v;
}

uint32_t oracle_round_to_next_power_of(uint32_t n, uint32_t base)
{
    /* base.hpp:69-74: exp = log(n)/log(base); return (uint32_t) pow(base, ceil(exp)); */
    double e = log((double)n) / log((double)base);
    double r = pow((double)base, ceil(e));
    if (!(r >= 0.0) || r > 4294967295.0) return 0u;
    return (uint32_t)r;
}

uint32_t oracle_divide_and_ceil(uint32_t value, uint32_t divider)
{
    /* base.hpp:76-79 */
    return (uint32_t)ceil((double)value / (double)divider);
}

uint32_t oracle_calc_bvh_padded_leaf_count(uint32_t leaf_count)
{
    /* vren/primitives/build_bvh.cpp:101-104 */
    return leaf_count <= 1 ? 32u : oracle_round_to_next_power_of(leaf_count, 32u);
}

uint32_t oracle_calc_bvh_buffer_length(uint32_t leaf_count)
{
    /* vren/primitives/build_bvh.cpp:106-118 */
    uint32_t p = oracle_calc_bvh_padded_leaf_count(leaf_count);
    uint64_t len = 0;
    while (p != 0) {
        len += p;
        p >>= 5;
    }
    return (uint32_t)len;
}

uint32_t oracle_calc_bvh_root_index(uint32_t leaf_count)
{
    /* vren/primitives/build_bvh.cpp:126-130 */
    return oracle_calc_bvh_buffer_length(oracle_calc_bvh_padded_leaf_count(leaf_count)) - 1u;
}

uint32_t oracle_calc_bvh_level_count(uint32_t leaf_count)
{
    /* vren/primitives/build_bvh.cpp:132-136: glm::log2 on an integer is the integer log2 */
    uint32_t p = oracle_calc_bvh_padded_leaf_count(leaf_count);
    uint32_t l = 0;
    while (p > 1) { p >>= 1; ++l; }
    return l / 5u;
}

/* ================================================================================================
 * Reduce — tree order of run_cpu_reduce (vren_test/vren_test/primitives/reduce.cpp:72-87) with
 * the shader's combine b = OP(b, a) (vren/resources/shaders/reduce.comp:76) and the identities
 * of VRen.cmake:70-75.  GLSL min(x,y) = y < x ? y : x, max(x,y) = x < y ? y : x.
 * ================================================================================================ */
static uint32_t u32_apply(int op, uint32_t right, uint32_t left)
{
    switch (op) {
    case ORACLE_ADD: return right + left;
    case ORACLE_MIN: return left < right ? left : right;
    default: return right < left ? left : right;
    }
}

static float f32_apply(int op, float right, float left)
{
    switch (op) {
    case ORACLE_ADD: return right + left;
    case ORACLE_MIN: return left < right ? left : right;
    default: return right < left ? left : right;
    }
}

void oracle_reduce_tree_u32(int op, const uint32_t* in, uint32_t n, uint32_t* out)
{
    uint32_t P = oracle_round_to_next_power_of_2(n);
    uint32_t id = op == ORACLE_MIN ? 0xFFFFFFFFu : 0u;
    for (uint32_t i = 0; i < P; ++i) out[i] = i < n ? in[i] : id;
    for (uint32_t lvl = 0; (1u << lvl) < P; ++lvl) {
        for (uint32_t j = 0; j < (P >> (lvl + 1)); ++j) {
            uint32_t a = (1u << lvl) - 1u + (j << (lvl + 1));
            uint32_t b = a + (1u << lvl);
            out[b] = u32_apply(op, out[b], out[a]);
        }
    }
}

void oracle_reduce_tree_vec4(int op, const float* in, uint32_t n, float* out)
{
    uint32_t P = oracle_round_to_next_power_of_2(n);
    float id = op == ORACLE_ADD ? 0.0f : (op == ORACLE_MIN ? 1e35f : -1e35f);
    for (uint32_t i = 0; i < P; ++i)
        for (int c = 0; c < 4; ++c) out[4 * i + c] = i < n ? in[4 * i + c] : id;
    for (uint32_t lvl = 0; (1u << lvl) < P; ++lvl) {
        for (uint32_t j = 0; j < (P >> (lvl + 1)); ++j) {
            uint32_t a = (1u << lvl) - 1u + (j << (lvl + 1));
            uint32_t b = a + (1u << lvl);
            for (int c = 0; c < 4; ++c) out[4 * b + c] = f32_apply(op, out[4 * b + c], out[4 * a + c]);
        }
    }
}

uint32_t oracle_reduce_u32(int op, const uint32_t* in, uint64_t n)
{
    uint32_t acc = op == ORACLE_MIN ? 0xFFFFFFFFu : 0u;
    for (uint64_t i = 0; i < n; ++i) acc = u32_apply(op, acc, in[i]);
    return acc;
}

static uint32_t f32_key(float f)
{
    uint32_t b;
    memcpy(&b, &f, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

static float f32_unkey(uint32_t k)
{
    uint32_t b = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

float oracle_reduce_f32(int op, const float* in, uint64_t n)
{
    /* min/max in IEEE-754 total order, so the result does not depend on the evaluation order */
    uint32_t acc = op == ORACLE_MIN ? 0xFFFFFFFFu : 0u;
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t k = f32_key(in[i]);
        if (op == ORACLE_MIN ? k < acc : k > acc) acc = k;
    }
    return f32_unkey(acc);
}

/* ================================================================================================
 * Scan
 * ================================================================================================ */
void oracle_exclusive_scan_u32(uint32_t* data, uint64_t n)
{
    /* vren_test/vren_test/primitives/blelloch_scan.cpp:72 std::exclusive_scan(..., 0) */
    uint32_t run = 0;
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t x = data[i];
        data[i] = run;
        run += x;
    }
}

void oracle_downsweep_u32(uint32_t* data, uint32_t n, int clear_last)
{
    /* The reference's dispatch sequence, restated literally:
     * global levels (vren/primitives/blelloch_scan.cpp:89-122, blelloch_scan_downsweep.comp:33-53) for
     * level = log2(n)-1 down to 10, clearing the last element on the first one, then the
     * 1024-wide work-group pass (vren/primitives/blelloch_scan.cpp:124-138, blelloch_scan_downsweep.comp:56-125)
     * which reads elements at index < n - clear_last and pads with zeros. */
    uint32_t log2n = 0;
    while ((1u << log2n) < n) ++log2n;
    uint32_t cl = clear_last ? 1u : 0u;
    for (int level = (int)log2n - 1; level > 9; --level) {
        uint32_t offset = (1u << level) - 1u, stride = 1u << level;
        for (uint64_t gid = 0;; ++gid) {
            uint64_t a = offset + gid * stride * 2u;
            uint64_t b = a + stride;
            if (b >= n) break;
            uint32_t bv = (cl && b == n - 1u) ? 0u : data[b];
            data[b] = data[a] + bv;
            data[a] = bv;
        }
        cl = 0;
    }
    uint32_t* s = (uint32_t*)malloc(1024 * sizeof(uint32_t));
    uint32_t wgs = (n + 1023u) / 1024u;
    for (uint32_t w = 0; w < wgs; ++w) {
        for (uint32_t t = 0; t < 1024; ++t) {
            uint32_t idx = w * 1024u + t;
            s[t] = (idx < n - cl) ? data[idx] : 0u;
        }
        for (int level = 9; level >= 0; --level) {
            uint32_t mask = (1u << (level + 1)) - 1u;
            for (uint32_t t = 0; t < 1024; ++t) {
                if ((t & mask) == mask) {
                    uint32_t b = t, a = b - (1u << level);
                    uint32_t tmp = s[b];
                    s[b] = s[a] + tmp;
                    s[a] = tmp;
                }
            }
        }
        for (uint32_t t = 0; t < 1024; ++t) {
            uint32_t idx = w * 1024u + t;
            if (idx < n) data[idx] = s[t];
        }
    }
    free(s);
}

/* ================================================================================================
 * Sorts
 * ================================================================================================ */
void oracle_stable_sort_u32(uint32_t* keys, uint32_t* values, uint64_t n)
{
    /* Stable LSD counting sort, 8 bits per pass: the result equals std::stable_sort by key. */
    uint32_t* tk = (uint32_t*)malloc(n * sizeof(uint32_t) + 4);
    uint32_t* tv = values ? (uint32_t*)malloc(n * sizeof(uint32_t) + 4) : NULL;
    uint64_t count[257];
    for (int pass = 0; pass < 4; ++pass) {
        int shift = pass * 8;
        memset(count, 0, sizeof(count));
        for (uint64_t i = 0; i < n; ++i) count[((keys[i] >> shift) & 0xFFu) + 1]++;
        for (int d = 0; d < 256; ++d) count[d + 1] += count[d];
        for (uint64_t i = 0; i < n; ++i) {
            uint64_t p = count[(keys[i] >> shift) & 0xFFu]++;
            tk[p] = keys[i];
            if (values) tv[p] = values[i];
        }
        memcpy(keys, tk, n * sizeof(uint32_t));
        if (values) memcpy(values, tv, n * sizeof(uint32_t));
    }
    free(tk);
    free(tv);
}

void oracle_bucket_sort_u32x2(const uint32_t* in, uint32_t n, uint32_t key_bits, uint32_t* out_pairs,
                              uint32_t* out_ends)
{
    /* Group uvec2(key, value) by key & mask (bucket_sort_count.comp:29-33,
     * bucket_sort_write.comp:29-34), stably.  out_ends = the counters region after the call:
     * exclusive scan of the counts, then +1 per written element = inclusive scan. */
    uint32_t nb = 1u << key_bits, mask = nb - 1u;
    uint32_t* cnt = (uint32_t*)calloc(nb + 1, sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) cnt[(in[2 * i] & mask) + 1]++;
    for (uint32_t b = 0; b < nb; ++b) cnt[b + 1] += cnt[b];
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t p = cnt[in[2 * i] & mask]++;
        out_pairs[2 * p] = in[2 * i];
        out_pairs[2 * p + 1] = in[2 * i + 1];
    }
    for (uint32_t b = 0; b < nb; ++b) out_ends[b] = cnt[b];
    free(cnt);
}

/* ================================================================================================
 * BVH — vren/resources/shaders/build_bvh.comp:32-55 per level (vren/primitives/build_bvh.cpp:69-98), with the
 * canonical decisions: a parent's AABB is the min/max over its valid children in IEEE total
 * order; all-invalid parents get (+inf, -inf) and next = INVALID; pad = 0.
 * ================================================================================================ */
static float fmin_total(float a, float b) { return f32_key(b) < f32_key(a) ? b : a; }
static float fmax_total(float a, float b) { return f32_key(b) > f32_key(a) ? b : a; }

void oracle_build_bvh(oracle_bvh_node* bvh, uint32_t padded_leaf_count)
{
    uint32_t src = 0, count = padded_leaf_count;
    while (count > 1) {
        uint32_t dst = src + count;
        for (uint32_t p = 0; p < count / 32u; ++p) {
            oracle_bvh_node par;
            int any = 0;
            for (int a = 0; a < 3; ++a) { par.min[a] = INFINITY; par.max[a] = -INFINITY; }
            for (uint32_t c = 0; c < 32; ++c) {
                const oracle_bvh_node* ch = &bvh[src + p * 32u + c];
                if (ch->next == INVALID_NODE) continue;
                if (!any) {
                    for (int a = 0; a < 3; ++a) { par.min[a] = ch->min[a]; par.max[a] = ch->max[a]; }
                    any = 1;
                } else {
                    for (int a = 0; a < 3; ++a) {
                        par.min[a] = fmin_total(par.min[a], ch->min[a]);
                        par.max[a] = fmax_total(par.max[a], ch->max[a]);
                    }
                }
            }
            par.next = any ? src + p * 32u : INVALID_NODE;
            par.pad = 0;
            bvh[dst + p] = par;
        }
        src = dst;
        count /= 32u;
    }
}

static int aabb_contains(const oracle_bvh_node* n, const float p[3])
{
    /* vren_test/vren_test/primitives/build_bvh.cpp:25-34 */
    return p[0] >= n->min[0] && p[1] >= n->min[1] && p[2] >= n->min[2] && p[0] <= n->max[0] &&
           p[1] <= n->max[1] && p[2] <= n->max[2];
}

static void query_r(const oracle_bvh_node* bvh, uint32_t offset, const float p[3], uint32_t* out, uint32_t cap,
                    uint32_t* cnt)
{
    /* vren_test/vren_test/primitives/build_bvh.cpp:36-64 */
    for (uint32_t i = 0; i < 32; ++i) {
        const oracle_bvh_node* nd = &bvh[offset + i];
        if (nd->next == INVALID_NODE) continue;
        if (aabb_contains(nd, p)) {
            if (nd->next == LEAF_NODE) {
                if (*cnt < cap) out[*cnt] = offset + i;
                (*cnt)++;
            } else {
                query_r(bvh, nd->next, p, out, cap, cnt);
            }
        }
    }
}

uint32_t oracle_bvh_point_query(const oracle_bvh_node* bvh, uint32_t root_index, const float p[3], uint32_t* out,
                                uint32_t cap)
{
    /* vren_test/vren_test/primitives/build_bvh.cpp:66-78 */
    uint32_t cnt = 0;
    const oracle_bvh_node* root = &bvh[root_index];
    if (root->next != INVALID_NODE && aabb_contains(root, p)) query_r(bvh, root->next, p, out, cap, &cnt);
    return cnt;
}

/* ================================================================================================
 * Clustered shading — shared float helpers (all single precision, no contraction)
 * ================================================================================================ */
static uint32_t floor_to_u32(float x)
{
    float f = floorf(x);
    if (!(f >= 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

/* out = m * v, m column-major, summed ((c0 + c1) + c2) + c3 */
static void matvec(const float* m, const float v[4], float out[4])
{
    for (int r = 0; r < 4; ++r) {
        float t0 = m[0 * 4 + r] * v[0];
        float t1 = m[1 * 4 + r] * v[1];
        float t2 = m[2 * 4 + r] * v[2];
        float t3 = m[3 * 4 + r] * v[3];
        out[r] = ((t0 + t1) + t2) + t3;
    }
}

static float glsl_min(float x, float y) { return y < x ? y : x; }
static float glsl_max(float x, float y) { return x < y ? y : x; }

/* Slice boundaries: REF bound[k] = near * a^k, a = 1 + 2 tan(half_fov) / tiles_y
 * (find_unique_clusters.comp:65, clustered_shading.glsl:99-101), a^k by repeated double
 * multiplication; FIXED32 bound[k] = near * r^k, r = (far/near)^(1/32), k <= 32, +inf beyond. */
void oracle_cs_slice_table(const oracle_cs_view* v, uint32_t tiles_y, float* near_out, float* far_out)
{
    double bound[ORACLE_SLICES + 1];
    const double nr = v->near_plane;
    if (v->slicing == ORACLE_SLICING_FIXED32) {
        double r = pow((double)v->far_plane / nr, 1.0 / 32.0);
        double p = 1.0;
        for (int k = 0; k <= ORACLE_SLICES; ++k) {
            bound[k] = k <= 32 ? nr * p : INFINITY;
            p *= r;
        }
    } else {
        double a = 1.0 + 2.0 * tan((double)v->half_fov_y) / (double)tiles_y;
        double p = 1.0;
        for (int k = 0; k <= ORACLE_SLICES; ++k) {
            bound[k] = nr * p;
            p *= a;
        }
    }
    for (int k = 0; k < ORACLE_SLICES; ++k) {
        near_out[k] = (float)bound[k];
        far_out[k] = (float)bound[k + 1];
    }
}

static uint32_t slice_of(float z, const float* bnear, uint32_t kmax)
{
    /* largest k in [0, kmax] with bnear[k] <= z; 0 if none (the table ascends, so a binary search over
     * it finds the first bound above z; a NaN z is above no bound and below none: k = 0) */
    if (!(bnear[0] <= z)) return 0;
    uint32_t lo = 0, hi = kmax;  /* invariant: bnear[lo] <= z */
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        if (bnear[mid] <= z) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

/* clustered_shading.glsl:7-43 */
static uint32_t discretize_normal(const float n[3])
{
    if (n[0] == 0.0f && n[1] == 0.0f && n[2] == 0.0f) return 0xFFFFFFFFu;
    float min_t = 1e35f;
    uint32_t axis = 0, face = 0;
    for (uint32_t i = 0; i < 3; ++i) {
        float sg = n[i] > 0.0f ? 1.0f : (n[i] < 0.0f ? -1.0f : 0.0f);
        float t = sg / n[i];
        if (t < min_t) {
            min_t = t;
            axis = i;
            face = (n[i] > 0.0f ? 1u : 0u) * 3u + i;
        }
    }
    float p[3] = {n[0] * min_t, n[1] * min_t, n[2] * min_t};
    float u = p[(axis + 1) % 3], w = p[(axis + 2) % 3];
    uint32_t du = floor_to_u32(((u + 1.0f) / 2.0f) * 3.0f);
    uint32_t dw = floor_to_u32(((w + 1.0f) / 2.0f) * 3.0f);
    return (face * 9u + du * 3u + dw) & 0x3Fu;
}

/* ================================================================================================
 * construct_point_light_bvh — vren/vren/pipeline/clustered_shading.cpp:60-346:
 * view transform (point_light_position_to_view_space.comp:30), vec4 min/max (reduce trees),
 * Morton codes (discretize_point_light_positions.comp:30-39), bucket sort on code & 0xFFFF
 * (stable), leaves (init_light_array_bvh.comp:42-65), build_bvh.
 * ================================================================================================ */
/* view positions, their min / max (vec4) and the unsorted (Morton code, light) pairs */
void oracle_cs_light_codes(const float* positions, uint32_t L, const oracle_cs_view* v, uint32_t morton_bits,
                           float* view_pos, float* mn, float* mx, uint32_t* codes)
{
    for (int c = 0; c < 4; ++c) { mn[c] = INFINITY; mx[c] = -INFINITY; }
    for (uint32_t i = 0; i < L; ++i) {
        float p[4] = {positions[4 * i], positions[4 * i + 1], positions[4 * i + 2], 1.0f};
        matvec(v->view, p, &view_pos[4 * i]);
        for (int c = 0; c < 4; ++c) {
            if (i == 0) { mn[c] = view_pos[4 * i + c]; mx[c] = view_pos[4 * i + c]; }
            else { mn[c] = fmin_total(mn[c], view_pos[4 * i + c]); mx[c] = fmax_total(mx[c], view_pos[4 * i + c]); }
        }
    }
    const uint32_t bits = morton_bits == 30 ? 10u : 5u;
    const float scale = (float)(1u << bits);
    for (uint32_t i = 0; i < L; ++i) {
        uint32_t q[3];
        for (int c = 0; c < 3; ++c) q[c] = floor_to_u32(((view_pos[4 * i + c] - mn[c]) / (mx[c] - mn[c])) * scale);
        uint32_t code = 0;
        for (uint32_t b = 0; b < bits; ++b) {
            code |= ((q[0] >> b) & 1u) << (b * 3u);
            code |= ((q[1] >> b) & 1u) << (b * 3u + 1u);
            code |= ((q[2] >> b) & 1u) << (b * 3u + 2u);
        }
        codes[2 * i] = code;
        codes[2 * i + 1] = i;
    }
}

void oracle_cs_light_bvh(const float* positions, const float* lights, uint32_t L, const oracle_cs_view* v,
                         uint32_t morton_bits, float* view_pos, oracle_bvh_node* bvh, uint32_t* light_index)
{
    float mn[4], mx[4];
    uint32_t* codes = (uint32_t*)malloc((size_t)L * 8 + 8);
    oracle_cs_light_codes(positions, L, v, morton_bits, view_pos, mn, mx, codes);
    /* bucket sort on the low 16 bits (bucket_sort.hpp:15-16) for 15-bit codes; the 30-bit
     * extension sorts on the whole code (stable either way) */
    {
        uint32_t* vals = (uint32_t*)malloc((size_t)L * 4 + 4);
        uint32_t* ks = (uint32_t*)malloc((size_t)L * 4 + 4);
        for (uint32_t i = 0; i < L; ++i) { ks[i] = morton_bits == 30 ? codes[2 * i] : (codes[2 * i] & 0xFFFFu); vals[i] = i; }
        oracle_stable_sort_u32(ks, vals, L);
        for (uint32_t i = 0; i < L; ++i) {
            light_index[2 * i] = codes[2 * vals[i]];
            light_index[2 * i + 1] = codes[2 * vals[i] + 1];
        }
        free(vals);
        free(ks);
    }
    free(codes);
    const uint32_t P = oracle_calc_bvh_padded_leaf_count(L);
    for (uint32_t i = 0; i < P; ++i) {
        oracle_bvh_node nd;
        memset(&nd, 0, sizeof(nd));
        if (i < L) {
            uint32_t li = light_index[2 * i + 1];
            float r = lights[4 * li + 3];
            for (int c = 0; c < 3; ++c) {
                nd.min[c] = view_pos[4 * li + c] - r;
                nd.max[c] = view_pos[4 * li + c] + r;
            }
            nd.next = LEAF_NODE;
        } else {
            for (int c = 0; c < 3; ++c) { nd.min[c] = INFINITY; nd.max[c] = -INFINITY; }
            nd.next = INVALID_NODE;
        }
        bvh[i] = nd;
    }
    oracle_build_bvh(bvh, P);
}

/* ================================================================================================
 * find_unique_cluster_list — vren/resources/shaders/clustered_shading/find_unique_clusters.comp:46-120
 * with the canonical decisions: integer texel (WRAP = reference's REPEAT sampler, or SKIP),
 * slice from the boundary table, tiles in row-major order, keys ascending inside a tile.
 * ================================================================================================ */
static int cmp_u32(const void* a, const void* b)
{
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

static uint32_t pixel_key(const float* depth, const float* normals, uint32_t W, uint32_t H, uint32_t gx, uint32_t gy,
                          const oracle_cs_view* v, const float* bnear, uint32_t kmax)
{
    const uint32_t tx = gx % W, ty = gy % H;
    const size_t px = (size_t)ty * W + tx;
    float fx = (float)gx / (float)W, fy = (float)gy / (float)H;
    float pos[4] = {fx * 2.0f - 1.0f, (1.0f - fy) * 2.0f - 1.0f, depth[px], 1.0f};
    float vp[4];
    matvec(v->inv_proj, pos, vp);
    float z = vp[2] / vp[3];
    uint32_t k = slice_of(z, bnear, kmax);
    uint32_t nd = discretize_normal(&normals[3 * px]);
    uint32_t i = gx >> 5, j = gy >> 5;
    return (i & 0xFFu) | ((j & 0xFFu) << 8) | ((k & 0x3FFu) << 16) | (nd << 26);
}

uint32_t oracle_cs_find_unique_clusters(const float* depth, const float* normals, uint32_t W, uint32_t H,
                                        const oracle_cs_view* v, int policy, uint32_t* keys, uint32_t key_cap,
                                        uint32_t* refs, int threads)
{
    const uint32_t TX = (W + 31) / 32, TY = (H + 31) / 32, T = TX * TY;
    float bnear[ORACLE_SLICES], bfar[ORACLE_SLICES];
    oracle_cs_slice_table(v, TY, bnear, bfar);
    const uint32_t kmax = v->slicing == ORACLE_SLICING_FIXED32 ? 31u : (ORACLE_SLICES - 1u);
    uint32_t* tile_keys = (uint32_t*)malloc((size_t)T * 1024 * sizeof(uint32_t));
    uint32_t* pix_keys = (uint32_t*)malloc((size_t)T * 1024 * sizeof(uint32_t)); /* each pixel's key, tile order */
    uint32_t* tile_count = (uint32_t*)malloc((size_t)T * sizeof(uint32_t));
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads(threads))
    for (int64_t t = 0; t < (int64_t)T; ++t) {
        uint32_t ti = (uint32_t)t % TX, tj = (uint32_t)t / TX;
        uint32_t* tk = tile_keys + (size_t)t * 1024;
        uint32_t* pk = pix_keys + (size_t)t * 1024;
        uint32_t m = 0;
        for (uint32_t ly = 0; ly < 32; ++ly)
            for (uint32_t lx = 0; lx < 32; ++lx) {
                uint32_t gx = ti * 32 + lx, gy = tj * 32 + ly;
                if (policy == ORACLE_SKIP && (gx >= W || gy >= H)) continue;
                pk[ly * 32 + lx] = tk[m++] = pixel_key(depth, normals, W, H, gx, gy, v, bnear, kmax);
            }
        qsort(tk, m, sizeof(uint32_t), cmp_u32);
        uint32_t u = 0;
        for (uint32_t q = 0; q < m; ++q)
            if (q == 0 || tk[q] != tk[q - 1]) tk[u++] = tk[q];
        tile_count[t] = u;
    }
    uint32_t* tile_off = (uint32_t*)malloc((size_t)T * sizeof(uint32_t));
    uint32_t U = 0;
    for (uint32_t t = 0; t < T; ++t) { tile_off[t] = U; U += tile_count[t]; }
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads(threads))
    for (int64_t t = 0; t < (int64_t)T; ++t) {
        uint32_t ti = (uint32_t)t % TX, tj = (uint32_t)t / TX;
        const uint32_t* tk = tile_keys + (size_t)t * 1024;
        for (uint32_t q = 0; q < tile_count[t]; ++q)
            if (tile_off[t] + q < key_cap) keys[tile_off[t] + q] = tk[q];
        for (uint32_t ly = 0; ly < 32; ++ly)
            for (uint32_t lx = 0; lx < 32; ++lx) {
                uint32_t gx = ti * 32 + lx, gy = tj * 32 + ly;
                if (gx >= W || gy >= H) continue;  /* stores outside the screen are dropped */
                uint32_t key = pix_keys[(size_t)t * 1024 + ly * 32 + lx];
                /* rank of key among the tile's unique keys */
                uint32_t lo = 0, hi = tile_count[t];
                while (lo < hi) {
                    uint32_t mid = (lo + hi) / 2;
                    if (tk[mid] < key) lo = mid + 1; else hi = mid;
                }
                refs[(size_t)gy * W + gx] = tile_off[t] + lo;
            }
    }
    free(tile_keys);
    free(pix_keys);
    free(tile_count);
    free(tile_off);
    return U;
}

/* ================================================================================================
 * assign_lights — vren/resources/shaders/clustered_shading/assign_lights.comp:121-240 (count and
 * write variants), cluster AABB of clustered_shading.glsl:72-110, node addressing of
 * assign_lights.comp:108-119, tests of :84-102.  INVALID nodes never overlap (canonical).
 * ================================================================================================ */
typedef struct { float mn[3], mx[3]; } caabb;

static caabb cluster_aabb(uint32_t key, uint32_t TX, uint32_t TY, const oracle_cs_view* v, const float* bnear,
                          const float* bfar)
{
    uint32_t ci = key & 0xFFu, cj = (key >> 8) & 0xFFu, ck = (key >> 16) & 0x3FFu;
    float x0 = (float)ci / (float)TX, y0 = (float)cj / (float)TY;
    float x1 = (float)(ci + 1u) / (float)TX, y1 = (float)(cj + 1u) / (float)TY;
    float a[4] = {x0 * 2.0f - 1.0f, (1.0f - y0) * 2.0f - 1.0f, 0.0f, 1.0f};
    float b[4] = {x1 * 2.0f - 1.0f, (1.0f - y1) * 2.0f - 1.0f, 0.0f, 1.0f};
    float va[4], vb[4];
    matvec(v->inv_proj, a, va);
    matvec(v->inv_proj, b, vb);
    for (int c = 0; c < 3; ++c) { va[c] = va[c] / va[3]; vb[c] = vb[c] / vb[3]; }
    float la = sqrtf((va[0] * va[0] + va[1] * va[1]) + va[2] * va[2]);
    float lb = sqrtf((vb[0] * vb[0] + vb[1] * vb[1]) + vb[2] * vb[2]);
    float d1[3] = {va[0] / la, va[1] / la, va[2] / la};
    float d2[3] = {vb[0] / lb, vb[1] / lb, vb[2] / lb};
    float cn = bnear[ck], cf = bfar[ck];
    float s1 = cn / d1[2], s2 = cf / d2[2];
    caabb r;
    for (int c = 0; c < 3; ++c) { r.mn[c] = s1 * d1[c]; r.mx[c] = s2 * d2[c]; }
    return r;
}

static int test_aabb_aabb(const caabb* c, const oracle_bvh_node* n)
{
    return c->mx[0] >= n->min[0] && c->mn[0] <= n->max[0] && c->mx[1] >= n->min[1] && c->mn[1] <= n->max[1] &&
           c->mx[2] >= n->min[2] && c->mn[2] <= n->max[2];
}

static int test_sphere_aabb(const float o[3], float r, const caabb* c)
{
    float d[3];
    for (int k = 0; k < 3; ++k) {
        float p = glsl_max(c->mn[k], glsl_min(o[k], c->mx[k]));
        d[k] = p - o[k];
    }
    float len = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
    return len < r;
}

static uint32_t lsb(uint32_t x) { return (uint32_t)__builtin_ctz(x); }

/* One traversal; when out != NULL writes the assigned indices (reverse lane order per group). */
static uint32_t traverse_cluster(const caabb* c, const oracle_bvh_node* bvh, uint32_t root, uint32_t level_count,
                                 const uint32_t* light_index, const float* view_pos, uint32_t* out)
{
    uint32_t ov[8] = {0};
    uint32_t level = 0, state = 2, acc = 0;
    for (;;) {
        if (state == 0) { /* ADVANCE */
            ov[level] &= ~(1u << lsb(ov[level]));
            if (ov[level] == 0) state = 1;
            else { level++; state = 2; }
        } else if (state == 1) { /* POP */
            if (level > 0) { level--; state = 0; }
            else break;
        } else { /* ENTERING */
            int64_t addr = (int64_t)root;
            uint64_t pw = 32;
            for (uint32_t i = 1; i <= level + 1; ++i) { addr -= (int64_t)pw; pw *= 32; }
            for (uint32_t i = 0; i < level; ++i) {
                uint64_t w = 1;
                for (uint32_t e = 0; e < level - i; ++e) w *= 32;
                addr += (int64_t)(w * lsb(ov[i]));
            }
            if (level + 1 < level_count) {
                uint32_t mask = 0;
                for (uint32_t lane = 0; lane < 32; ++lane) {
                    const oracle_bvh_node* nd = &bvh[addr + lane];
                    if (nd->next != INVALID_NODE && test_aabb_aabb(c, nd)) mask |= 1u << lane;
                }
                ov[level] = mask;
                if (mask == 0) state = 1;
                else level++;
            } else {
                uint32_t mask = 0, idx[32];
                for (uint32_t lane = 0; lane < 32; ++lane) {
                    const oracle_bvh_node* nd = &bvh[addr + lane];
                    idx[lane] = 0;
                    if (nd->next == INVALID_NODE) continue;
                    uint32_t li = light_index[2 * (addr + lane) + 1];
                    idx[lane] = li;
                    float o[3] = {view_pos[4 * li], view_pos[4 * li + 1], view_pos[4 * li + 2]};
                    float r = (nd->max[0] - nd->min[0]) / 2.0f;
                    if (test_sphere_aabb(o, r, c)) mask |= 1u << lane;
                }
                if (out) {
                    for (uint32_t lane = 0; lane < 32; ++lane) {
                        if (!(mask & (1u << lane))) continue;
                        uint32_t slot = (uint32_t)__builtin_popcount(mask & ~((1u << lane) - 1u)) - 1u;
                        out[acc + slot] = idx[lane];
                    }
                }
                acc += (uint32_t)__builtin_popcount(mask);
                state = 1;
            }
        }
    }
    return acc;
}

uint64_t oracle_cs_assign_lights(const uint32_t* keys, uint32_t U, uint32_t W, uint32_t H, const oracle_cs_view* v,
                                 const oracle_bvh_node* bvh, uint32_t L, const uint32_t* light_index,
                                 const float* view_pos, uint32_t* counts, uint32_t* offsets, uint32_t* indices,
                                 uint64_t index_cap, int threads)
{
    const uint32_t TX = (W + 31) / 32, TY = (H + 31) / 32;
    if (L == 0) {
        for (uint32_t c = 0; c < U; ++c) { counts[c] = 0; offsets[c] = 0; }
        return 0;
    }
    float bnear[ORACLE_SLICES], bfar[ORACLE_SLICES];
    oracle_cs_slice_table(v, TY, bnear, bfar);
    const uint32_t root = oracle_calc_bvh_root_index(L);
    const uint32_t levels = oracle_calc_bvh_level_count(L);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads(threads))
    for (int64_t c = 0; c < (int64_t)U; ++c) {
        caabb box = cluster_aabb(keys[c], TX, TY, v, bnear, bfar);
        counts[c] = traverse_cluster(&box, bvh, root, levels, light_index, view_pos, NULL);
    }
    uint64_t total = 0;
    for (uint32_t c = 0; c < U; ++c) { offsets[c] = (uint32_t)total; total += counts[c]; }
    if (total > index_cap) return total;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads(threads))
    for (int64_t c = 0; c < (int64_t)U; ++c) {
        caabb box = cluster_aabb(keys[c], TX, TY, v, bnear, bfar);
        traverse_cluster(&box, bvh, root, levels, light_index, view_pos, indices + offsets[c]);
    }
    return total;
}

/* ---- the restatement's per-element steps, for the comparison with the reference's own shaders ---- */
void oracle_cs_normal_bins(const float* normals, uint64_t count, uint32_t* out)
{
    for (uint64_t i = 0; i < count; ++i) out[i] = discretize_normal(normals + 3 * i);
}

void oracle_cs_pixel_keys(const float* depth, const float* normals, uint32_t W, uint32_t H, const oracle_cs_view* v,
                          uint32_t* keys)
{
    const uint32_t TX = (W + 31) / 32, TY = (H + 31) / 32;
    float bnear[ORACLE_SLICES], bfar[ORACLE_SLICES];
    oracle_cs_slice_table(v, TY, bnear, bfar);
    const uint32_t kmax = v->slicing == ORACLE_SLICING_FIXED32 ? 31u : (ORACLE_SLICES - 1u);
#pragma omp parallel for schedule(static)
    for (int64_t gy = 0; gy < (int64_t)TY * 32; ++gy)
        for (uint32_t gx = 0; gx < TX * 32; ++gx)
            keys[(size_t)gy * TX * 32 + gx] = pixel_key(depth, normals, W, H, gx, (uint32_t)gy, v, bnear, kmax);
}

void oracle_cs_cluster_boxes(const uint32_t* keys, uint64_t count, uint32_t W, uint32_t H, const oracle_cs_view* v,
                             float* mn, float* mx)
{
    const uint32_t TX = (W + 31) / 32, TY = (H + 31) / 32;
    float bnear[ORACLE_SLICES], bfar[ORACLE_SLICES];
    oracle_cs_slice_table(v, TY, bnear, bfar);
    for (uint64_t i = 0; i < count; ++i) {
        caabb b = cluster_aabb(keys[i], TX, TY, v, bnear, bfar);
        for (int c = 0; c < 3; ++c) { mn[3 * i + c] = b.mn[c]; mx[3 * i + c] = b.mx[c]; }
    }
}

void oracle_cs_test_aabb_aabb(const float* t, uint64_t count, uint8_t* out)
{
    for (uint64_t i = 0; i < count; ++i) {
        const float* q = t + 12 * i;
        caabb c;
        oracle_bvh_node n;
        for (int k = 0; k < 3; ++k) {
            c.mn[k] = q[k];
            c.mx[k] = q[3 + k];
            n.min[k] = q[6 + k];
            n.max[k] = q[9 + k];
        }
        out[i] = (uint8_t)test_aabb_aabb(&c, &n);
    }
}

void oracle_cs_test_sphere_aabb(const float* t, uint64_t count, uint8_t* out)
{
    for (uint64_t i = 0; i < count; ++i) {
        const float* q = t + 10 * i;
        caabb c;
        for (int k = 0; k < 3; ++k) { c.mn[k] = q[4 + k]; c.mx[k] = q[7 + k]; }
        out[i] = (uint8_t)test_sphere_aabb(q, q[3], &c);
    }
}

/* ================================================================================================
 * Karras binary radix tree over the sorted light leaves — an extension beside the reference's 32-ary
 * tree (no counterpart in the reference).  Restated from T. Karras, "Maximizing Parallelism in the
 * Construction of BVHs, Octrees, and k-d Trees", HPG 2012, section 4 (Figure 4 pseudocode): keys are
 * the sorted Morton codes augmented with the leaf position, so equal codes still give a unique
 * order (delta = 32 + clz(i ^ j) for equal codes).  Internal node 0 is the root; a child index with
 * ORACLE_LBVH_LEAF set names a leaf (a position in the sorted light order, i.e. a level-0 node of
 * the 32-ary BVH, whose AABB it reuses).  Internal AABBs are unions in IEEE total order.
 * ================================================================================================ */
static int lbvh_delta(const uint32_t* light_index, int64_t n, int64_t i, int64_t j)
{
    if (j < 0 || j >= n) return -1;
    const uint32_t a = light_index[2 * i], b = light_index[2 * j];
    if (a != b) return __builtin_clz(a ^ b);
    return 32 + __builtin_clz((uint32_t)i ^ (uint32_t)j);
}

static void lbvh_union(oracle_lbvh_node* nd, const float mn[3], const float mx[3], int first)
{
    for (int k = 0; k < 3; ++k) {
        nd->min[k] = first ? mn[k] : fmin_total(nd->min[k], mn[k]);
        nd->max[k] = first ? mx[k] : fmax_total(nd->max[k], mx[k]);
    }
}

static void lbvh_refit(oracle_lbvh_node* nodes, const oracle_bvh_node* leaves, uint32_t node)
{
    oracle_lbvh_node* nd = &nodes[node];
    const uint32_t ch[2] = {nd->left, nd->right};
    for (int c = 0; c < 2; ++c) {
        if (ch[c] & ORACLE_LBVH_LEAF) {
            const oracle_bvh_node* lf = &leaves[ch[c] & ~ORACLE_LBVH_LEAF];
            lbvh_union(nd, lf->min, lf->max, c == 0);
        } else {
            lbvh_refit(nodes, leaves, ch[c]);
            lbvh_union(nd, nodes[ch[c]].min, nodes[ch[c]].max, c == 0);
        }
    }
}

void oracle_lbvh_build(const uint32_t* light_index, const oracle_bvh_node* leaves, uint32_t n,
                       oracle_lbvh_node* nodes)
{
    for (int64_t i = 0; i + 1 < (int64_t)n; ++i) {
        const int d = lbvh_delta(light_index, n, i, i + 1) - lbvh_delta(light_index, n, i, i - 1) >= 0 ? 1 : -1;
        const int dmin = lbvh_delta(light_index, n, i, i - d);
        int64_t lmax = 2;
        while (lbvh_delta(light_index, n, i, i + lmax * d) > dmin) lmax *= 2;
        int64_t l = 0;
        for (int64_t t = lmax / 2; t >= 1; t /= 2)
            if (lbvh_delta(light_index, n, i, i + (l + t) * d) > dmin) l += t;
        const int64_t j = i + l * d;
        const int dnode = lbvh_delta(light_index, n, i, j);
        int64_t s = 0, t = l;
        do {
            t = (t + 1) / 2;
            if (lbvh_delta(light_index, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        const int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
        const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
        nodes[i].left = (uint32_t)gamma | (lo == gamma ? ORACLE_LBVH_LEAF : 0u);
        nodes[i].right = (uint32_t)(gamma + 1) | (hi == gamma + 1 ? ORACLE_LBVH_LEAF : 0u);
    }
    if (n > 1) lbvh_refit(nodes, leaves, 0);
}

/* Lights of one cluster by the Karras tree: a light is assigned when its test box boxes[i] overlaps
 * the cluster box and its sphere (view position, (max.x - min.x) / 2 of its leaf AABB) does too,
 * written in the reference's order (leaf groups of 32 ascending, lanes of a group descending): the
 * depth-first walk (left child first) meets leaves in ascending order and each group's hits are
 * written back to front.  With boxes[i] = the AABB of leaf i's 32-leaf group (infinite when there are
 * at most 32 lights) this is exactly the 32-ary traversal's rule: its box test is monotone in box
 * inclusion, so a leaf under an overlapping group box has every ancestor overlapping, and the
 * reference never tests the leaf's own box.  The tree must then be built over the same boxes so
 * that its pruning is conservative. */
static uint32_t lbvh_traverse(const caabb* c, const oracle_lbvh_node* nodes, const oracle_bvh_node* boxes,
                              const oracle_bvh_node* leaves, uint32_t n, const uint32_t* light_index,
                              const float* view_pos, uint32_t* out)
{
    uint32_t stack[128];
    int sp = 0;
    uint32_t cur = n == 1 ? ORACLE_LBVH_LEAF : 0u;
    uint32_t acc = 0, written = 0, buf[32], grp = 0xFFFFFFFFu;
    int nb = 0;
    for (;;) {
        int descend = 0;
        if (cur & ORACLE_LBVH_LEAF) {
            const uint32_t i = cur & ~ORACLE_LBVH_LEAF;
            const oracle_bvh_node* lf = &leaves[i];
            if (test_aabb_aabb(c, &boxes[i])) {
                const uint32_t li = light_index[2 * i + 1];
                const float o[3] = {view_pos[4 * li], view_pos[4 * li + 1], view_pos[4 * li + 2]};
                if (test_sphere_aabb(o, (lf->max[0] - lf->min[0]) / 2.0f, c)) {
                    if (out) {
                        if ((i >> 5) != grp) {
                            while (nb > 0) out[written++] = buf[--nb];
                            grp = i >> 5;
                        }
                        buf[nb++] = li;
                    }
                    ++acc;
                }
            }
        } else {
            const oracle_lbvh_node* nd = &nodes[cur];
            descend = c->mx[0] >= nd->min[0] && c->mn[0] <= nd->max[0] && c->mx[1] >= nd->min[1] &&
                      c->mn[1] <= nd->max[1] && c->mx[2] >= nd->min[2] && c->mn[2] <= nd->max[2];
            if (descend) {
                stack[sp++] = nd->right;
                cur = nd->left;
            }
        }
        if (!descend) {
            if (sp == 0) break;
            cur = stack[--sp];
        }
    }
    if (out)
        while (nb > 0) out[written++] = buf[--nb];
    return acc;
}

uint64_t oracle_cs_assign_lights_lbvh(const uint32_t* keys, uint32_t U, uint32_t W, uint32_t H,
                                      const oracle_cs_view* v, const oracle_lbvh_node* nodes,
                                      const oracle_bvh_node* boxes, const oracle_bvh_node* leaves, uint32_t L,
                                      const uint32_t* light_index, const float* view_pos, uint32_t* counts,
                                      uint32_t* offsets, uint32_t* indices, uint64_t index_cap, int threads)
{
    const uint32_t TX = (W + 31) / 32, TY = (H + 31) / 32;
    if (L == 0) {
        for (uint32_t c = 0; c < U; ++c) { counts[c] = 0; offsets[c] = 0; }
        return 0;
    }
    float bnear[ORACLE_SLICES], bfar[ORACLE_SLICES];
    oracle_cs_slice_table(v, TY, bnear, bfar);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads(threads))
    for (int64_t c = 0; c < (int64_t)U; ++c) {
        caabb box = cluster_aabb(keys[c], TX, TY, v, bnear, bfar);
        counts[c] = lbvh_traverse(&box, nodes, boxes, leaves, L, light_index, view_pos, NULL);
    }
    uint64_t total = 0;
    for (uint32_t c = 0; c < U; ++c) { offsets[c] = (uint32_t)total; total += counts[c]; }
    if (total > index_cap) return total;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads(threads))
    for (int64_t c = 0; c < (int64_t)U; ++c) {
        caabb box = cluster_aabb(keys[c], TX, TY, v, bnear, bfar);
        lbvh_traverse(&box, nodes, boxes, leaves, L, light_index, view_pos, indices + offsets[c]);
    }
    return total;
}

/* ================================================================================================
 * Point-light bouncer — vren_demo/resources/shaders/bounce_point_lights.comp:33-73 (host
 * point_light_bouncer.cpp:17-57).  GLSL min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x; every
 * operation rounded on its own (compiled with -ffp-contract=off), IEEE division.
 * ================================================================================================ */
void oracle_bounce_point_lights(float* positions, float* directions, uint32_t L, const float* aabb_min,
                                const float* aabb_max, float speed, float dt)
{
    const float INF_ = 1e35f, EPS_ = 1e-5f;
    for (uint32_t i = 0; i < L; ++i) {
        float p[3], d[3];
        for (int c = 0; c < 3; ++c) {
            p[c] = glsl_min(glsl_max(positions[4 * i + c], aabb_min[c]), aabb_max[c]);
            d[c] = directions[4 * i + c];
        }
        float rem = speed * dt;
        for (int j = 0; j < 32 && rem > 0.0f; ++j) {
            float t1[3], t2[3];
            for (int c = 0; c < 3; ++c) {
                t1[c] = (aabb_min[c] - p[c]) / d[c];
                if (t1[c] <= 0.0f) t1[c] = INF_;
                t2[c] = (aabb_max[c] - p[c]) / d[c];
                if (t2[c] <= 0.0f) t2[c] = INF_;
            }
            const float min_t =
                glsl_min(t1[0], glsl_min(t2[0], glsl_min(t1[1], glsl_min(t2[1], glsl_min(t1[2], t2[2])))));
            const float step = glsl_min(min_t - EPS_, rem);
            for (int c = 0; c < 3; ++c) p[c] = p[c] + step * d[c];
            if (min_t < rem)
                for (int c = 0; c < 3; ++c) d[c] = d[c] * ((t1[c] == min_t || t2[c] == min_t) ? -1.0f : 1.0f);
            rem = rem - step;
        }
        for (int c = 0; c < 3; ++c) {
            positions[4 * i + c] = p[c];
            directions[4 * i + c] = d[c];
        }
        positions[4 * i + 3] = 1.0f;
        directions[4 * i + 3] = 0.0f;
    }
}

/* ================================================================================================
 * Depth-buffer pyramid — vren/vren/pipeline/depth_buffer_pyramid.cpp:18 (level count:
 * glm::log2 of the integer max(width, height), from glm/gtc/integer.hpp = floor(log2) — plus 1),
 * :48-54 (level size max(base >> level, 1)), :245-300 (one copy dispatch, then one reduce dispatch per
 * level); vren/resources/shaders/depth_buffer_copy.comp:8-17 (nearest texel at an unnormalised
 * integer coordinate: an exact copy) and depth_buffer_reduce.comp:10-34 (start from 0, GLSL max over
 * the 2x2 sources that lie inside the source level, x outer, y inner).  Levels are stored back to back,
 * row-major, with no padding.
 * ================================================================================================ */
uint32_t oracle_depth_pyramid_level_count(uint32_t width, uint32_t height)
{
    uint32_t m = width > height ? width : height, l = 0;
    while (m >>= 1) ++l;
    return l + 1;
}

void oracle_depth_pyramid(const float* depth, uint32_t width, uint32_t height, float* out)
{
    const uint32_t levels = oracle_depth_pyramid_level_count(width, height);
    memcpy(out, depth, (size_t)width * height * sizeof(float));
    float* from = out;
    uint32_t fw = width, fh = height;
    for (uint32_t l = 1; l < levels; ++l) {
        const uint32_t tw = (width >> l) ? (width >> l) : 1u, th = (height >> l) ? (height >> l) : 1u;
        float* to = from + (size_t)fw * fh;
        for (uint32_t y = 0; y < th; ++y)
            for (uint32_t x = 0; x < tw; ++x) {
                float m = 0.0f;
                for (uint32_t dx = 0; dx < 2; ++dx)
                    for (uint32_t dy = 0; dy < 2; ++dy) {
                        const uint32_t sx = 2 * x + dx, sy = 2 * y + dy;
                        if (sx < fw && sy < fh) m = glsl_max(m, from[(size_t)sy * fw + sx]);
                    }
                to[(size_t)y * tw + x] = m;
            }
        from = to;
        fw = tw;
        fh = th;
    }
}

/* ================================================================================================
 * Cluster debug views — vren_demo/resources/shaders/show_clusters.comp:50-124 (per pixel: the hash
 * triple32 and hash(x) = float(triple32(x)) / float(0xffffffff), the six modes, red otherwise) and
 * show_clusters_geometry.comp:55-110 with vren/resources/shaders/debug.glsl (VREN_DEBUG_WRITE_AABB /
 * _ARROW vertex order); the box is cluster_aabb above (the one the assignment tests).  A pixel whose
 * reference is >= U is drawn magenta (the shader would read out of bounds).
 * ================================================================================================ */
static uint32_t triple32(uint32_t x)
{
    x ^= x >> 17;
    x *= 0xed5ad4bbu;
    x ^= x >> 11;
    x *= 0xac4c1b51u;
    x ^= x >> 15;
    x *= 0x31848babu;
    x ^= x >> 14;
    return x;
}

static float hash01(uint32_t x) { return (float)triple32(x) / (float)0xffffffffu; }

void oracle_cs_show_clusters(int mode, uint32_t W, uint32_t H, const uint32_t* refs, const uint32_t* keys, uint32_t U,
                             const uint32_t* counts, const uint32_t* offsets, const uint32_t* indices, float* out)
{
    const uint32_t TX = (W + 31) / 32, TY = (H + 31) / 32;
    for (uint64_t p = 0; p < (uint64_t)W * H; ++p) {
        float* o = out + 4 * p;
        const uint32_t r = refs[p];
        float c[3];
        if (r >= U) {
            c[0] = 1.0f; c[1] = 0.0f; c[2] = 1.0f;
        } else {
            const uint32_t key = keys[r];
            const uint32_t ci = key & 0xFFu, cj = (key >> 8) & 0xFFu, ck = (key >> 16) & 0x3FFu, n = key >> 26;
            if (mode == 0) {
                c[0] = c[1] = c[2] = hash01(key);
            } else if (mode == 1) {
                c[0] = (float)ci / (float)TX;
                c[1] = (float)cj / (float)TY;
                c[2] = (float)ck / (float)1024;
            } else if (mode == 2) {
                c[0] = (float)(n / 9u) / 6.0f;
                c[1] = (float)((n / 3u) % 3u) / 3.0f;
                c[2] = (float)(n % 3u) / 3.0f;
            } else if (mode == 3) {
                c[0] = c[1] = c[2] = glsl_min((float)counts[r] / 64.0f, 1.0f);
            } else if (mode == 4) {
                c[0] = c[1] = c[2] = hash01(offsets[r]);
            } else if (mode == 5) {
                uint32_t h = 0;
                for (uint32_t i = 0; i < counts[r]; ++i) h ^= indices[offsets[r] + i];
                c[0] = c[1] = c[2] = hash01(h);
            } else {
                c[0] = 1.0f; c[1] = 0.0f; c[2] = 0.0f;
            }
        }
        o[0] = c[0]; o[1] = c[1]; o[2] = c[2]; o[3] = 1.0f;
    }
}

static void dbg_vertex(uint32_t* out, uint32_t* k, float x, float y, float z, uint32_t colour)
{
    memcpy(out + 4 * *k + 0, &x, 4);
    memcpy(out + 4 * *k + 1, &y, 4);
    memcpy(out + 4 * *k + 2, &z, 4);
    out[4 * *k + 3] = colour;
    ++*k;
}

static void dbg_line(uint32_t* out, uint32_t* k, const float a[3], const float b[3], uint32_t colour)
{
    dbg_vertex(out, k, a[0], a[1], a[2], colour);
    dbg_vertex(out, k, b[0], b[1], b[2], colour);
}

void oracle_cs_show_clusters_geometry(const oracle_cs_view* v, uint32_t W, uint32_t H, const uint32_t* keys,
                                      uint32_t U, uint32_t* out)
{
    const uint32_t TX = (W + 31) / 32, TY = (H + 31) / 32;
    float bnear[ORACLE_SLICES], bfar[ORACLE_SLICES];
    oracle_cs_slice_table(v, TY, bnear, bfar);
    for (uint32_t c = 0; c < U; ++c) {
        uint32_t* o = out + (size_t)c * 32 * 4;
        uint32_t k = 0;
        const caabb b = cluster_aabb(keys[c], TX, TY, v, bnear, bfar);
        const float* m = b.mn;
        const float* M = b.mx;
        const uint32_t n = keys[c] >> 26;
        const uint32_t col = n < 0x3Fu ? 0xFFFFFFu : 0u;
        /* VREN_DEBUG_WRITE_AABB(_m, _M) */
        const float e[24][3] = {
            {m[0], m[1], m[2]}, {M[0], m[1], m[2]}, {M[0], m[1], m[2]}, {M[0], m[1], M[2]},
            {M[0], m[1], M[2]}, {m[0], m[1], M[2]}, {m[0], m[1], M[2]}, {m[0], m[1], m[2]},
            {m[0], M[1], m[2]}, {M[0], M[1], m[2]}, {M[0], M[1], m[2]}, {M[0], M[1], M[2]},
            {M[0], M[1], M[2]}, {m[0], M[1], M[2]}, {m[0], M[1], M[2]}, {m[0], M[1], m[2]},
            {m[0], m[1], m[2]}, {m[0], M[1], m[2]}, {M[0], m[1], m[2]}, {M[0], M[1], m[2]},
            {M[0], m[1], M[2]}, {M[0], M[1], M[2]}, {m[0], m[1], M[2]}, {m[0], M[1], M[2]},
        };
        for (int i = 0; i < 24; i += 2) dbg_line(o, &k, e[i], e[i + 1], col);
        float pos[3], to[3];
        for (int a = 0; a < 3; ++a) pos[a] = (m[a] + M[a]) / 2.0f;
        if (n < 0x3Fu) {
            const uint32_t face = n / 9u, axis = face % 3u, uc = (axis + 1u) % 3u, vc = (axis + 2u) % 3u;
            float d[3];
            d[axis] = (face / 3u) == 1u ? 1.0f : -1.0f;
            d[uc] = (((float)((n / 3u) % 3u) + 0.5f) / 3.0f) * 2.0f - 1.0f;
            d[vc] = (((float)(n % 3u) + 0.5f) / 3.0f) * 2.0f - 1.0f;
            const float len = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
            for (int a = 0; a < 3; ++a) to[a] = pos[a] + (d[a] / len) * 0.01f;
        } else {
            for (int a = 0; a < 3; ++a) to[a] = pos[a];
        }
        /* VREN_DEBUG_WRITE_ARROW(pos, to, green, red) */
        dbg_line(o, &k, pos, to, 0x00FF00u);
        const float dx = pos[0] - to[0], dy = pos[1] - to[1], dz = pos[2] - to[2];
        const float h = sqrtf((dx * dx + dy * dy) + dz * dz) * 0.1f;
        const float sg[3][2][3] = {{{-1, -1, -1}, {1, 1, 1}}, {{1, 1, -1}, {-1, -1, 1}}, {{1, -1, -1}, {-1, 1, 1}}};
        for (int l = 0; l < 3; ++l) {
            float a0[3], a1[3];
            for (int a = 0; a < 3; ++a) {
                a0[a] = to[a] + sg[l][0][a] * h;
                a1[a] = to[a] + sg[l][1][a] * h;
            }
            dbg_line(o, &k, a0, a1, 0xFF0000u);
        }
    }
}

/* ================================================================================================
 * k-d tree — vren/vren/base/kd_tree.cpp:5-77 (build, recursive as written: Welford mean/variance in
 * float, the axis test comparing variance[0] with variance[1] twice, swap partition by
 * point[axis] < split) and :79-131 (search: near child first, far child when best > d * d), with the
 * node as the reference lays it out (12 bytes: split/index, axis, 30-bit value).  Where a split
 * separates nothing (the reference asserts), the node becomes one leaf run (canonical).
 * vren_test/vren_test/kd_tree.cpp:9-27 (linear search) is the reference's own check.
 * ================================================================================================ */
static size_t kd_build_rec(const float* points, size_t stride, uint32_t* idx, size_t count, oracle_kd_node* t,
                           size_t off, size_t max_leaf)
{
    int leaf = count <= max_leaf;
    size_t middle = 0;
    uint32_t axis = 0;
    float split = 0.0f;
    if (!leaf) {
        float mean[3] = {0, 0, 0}, var[3] = {0, 0, 0}, n = 1.0f;
        for (size_t i = 0; i < count; i++, n += 1.0f) {
            const float* p = points + (size_t)idx[i] * stride;
            for (int j = 0; j < 3; j++) {
                float d = p[j] - mean[j];
                mean[j] += d / n;
                var[j] += (p[j] - mean[j]) * d;
            }
        }
        axis = var[0] > var[1] && var[0] > var[1] ? 0 : (var[1] > var[2] ? 1 : 2);
        split = mean[axis];
        for (size_t i = 0; i < count; i++) {
            const float* p = points + (size_t)idx[i] * stride;
            if (p[axis] < split) {
                uint32_t tmp = idx[i];
                idx[i] = idx[middle];
                idx[middle] = tmp;
                middle++;
            }
        }
        leaf = middle == 0 || middle == count;
    }
    if (leaf) {
        for (size_t i = 0; i < count; i++) {
            t[off + i].word0 = idx[i];
            t[off + i].axis = 3;
            t[off + i].value = i == 0 ? (uint32_t)count & 0x3FFFFFFFu : 0x3FFFFFFFu;
        }
        return off + count;
    }
    size_t next = kd_build_rec(points, stride, idx, middle, t, off + 1, max_leaf);
    memcpy(&t[off].word0, &split, 4);
    t[off].axis = axis;
    t[off].value = (uint32_t)(next - off) & 0x3FFFFFFFu;
    return kd_build_rec(points, stride, idx + middle, count - middle, t, next, max_leaf);
}

size_t oracle_kd_tree_build(const float* points, size_t stride, uint32_t* indices, size_t count, oracle_kd_node* tree,
                            size_t max_leaf)
{
    return count ? kd_build_rec(points, stride, indices, count, tree, 0, max_leaf) : 0;
}

static void kd_search_rec(const float* points, size_t stride, const oracle_kd_node* t, size_t off, const float* s,
                          const uint8_t* excluded, uint32_t* best_point, float* best)
{
    const oracle_kd_node* nd = &t[off];
    if (nd->axis == 3) {
        for (uint32_t i = 0; i < nd->value; i++) {
            uint32_t id = t[off + i].word0;
            if (excluded && excluded[id]) continue;
            const float* p = points + (size_t)id * stride;
            float dist = (s[0] - p[0]) * (s[0] - p[0]) + (s[1] - p[1]) * (s[1] - p[1]) + (s[2] - p[2]) * (s[2] - p[2]);
            if (dist < *best) {
                *best_point = id;
                *best = dist;
            }
        }
        return;
    }
    float split;
    memcpy(&split, &nd->word0, 4);
    float d = s[nd->axis] - split;
    size_t first = d <= 0 ? off + 1 : off + nd->value;
    size_t second = d <= 0 ? off + nd->value : off + 1;
    kd_search_rec(points, stride, t, first, s, excluded, best_point, best);
    if (*best > d * d) kd_search_rec(points, stride, t, second, s, excluded, best_point, best);
}

void oracle_kd_tree_search(const float* points, size_t stride, const oracle_kd_node* tree, const float* samples,
                           size_t sample_stride, uint32_t sample_count, const uint8_t* excluded, uint32_t* best_points,
                           float* best_dist)
{
    for (uint32_t q = 0; q < sample_count; q++) {
        uint32_t bp = 0xFFFFFFFFu;
        float bd = INFINITY;
        kd_search_rec(points, stride, tree, 0, samples + (size_t)q * sample_stride, excluded, &bp, &bd);
        best_points[q] = bp;
        best_dist[q] = bd;
    }
}

void oracle_linear_nn_search(const float* points, size_t stride, const uint32_t* indices, size_t count,
                             const float* samples, size_t sample_stride, uint32_t sample_count, uint32_t* best_points,
                             float* best_dist)
{
    for (uint32_t q = 0; q < sample_count; q++) {
        const float* s = samples + (size_t)q * sample_stride;
        float bd = INFINITY;
        uint32_t bp = 0xFFFFFFFFu;
        for (size_t i = 0; i < count; i++) {
            const float* p = points + (size_t)indices[i] * stride;
            float dist = (s[0] - p[0]) * (s[0] - p[0]) + (s[1] - p[1]) * (s[1] - p[1]) + (s[2] - p[2]) * (s[2] - p[2]);
            if (dist < bd) {
                bd = dist;
                bp = indices[i];
            }
        }
        best_points[q] = bp;
        best_dist[q] = bd;
    }
}
