// ytgb_render.cu -- the per-pixel-ray sampler kernels of libytgb (sm_103a).
//
// One CUDA thread owns one pixel ray for the whole launch and walks every
// brick of the view in the kd viewpoint order, so the per-brick Python loop,
// OpenMP region and image read/write of yt's cast_through_kdtree
// (image_samplers.pyx:146-197) disappear.  For every brick the thread runs
// the Amanatides-Woo walk of walk_volume (grid_traversal.pyx:26-140) with
// every float64 operation spelled as an _rn intrinsic in the reference's
// order, so the visited cells and their enter/exit t are bit-identical to
// yt's.  Sampling (trilinear, transfer function) runs in float32 on float32
// brick data; the image accumulates as a float32 value plus a float32 error
// term (error-free TwoSum, Knuth), so accumulated rounding stays at the level
// of one float32 rounding per sample rather than growing with the ray length.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "ytgb.h"
#include "ytgb_internal.h"

namespace {

constexpr int MODE_VR = YTGB_VOLUME_RENDER;
constexpr int MODE_PROJ = YTGB_PROJECTION;
constexpr int MODE_IPROJ = YTGB_INTERPOLATED_PROJECTION;
constexpr int MODE_MIP = YTGB_MIP;
constexpr int MODE_TRACE = 4;

constexpr int TILE_X = 8;    // image rows (vi) per block
constexpr int TILE_Y = 16;   // image columns (vj) per block
constexpr int BLOCK = TILE_X * TILE_Y;

// ---- exact float64 arithmetic (never contracted into FMA) -----------------
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
// fp_utils.pxd fmin/fmax: first argument wins ties and NaNs go to the second
__device__ __forceinline__ double yt_fmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double yt_fmax(double a, double b) { return a > b ? a : b; }

struct Ray {
    double pos[3];
    double dir[3];
    double iv[3];
    int step[3];
};

// generate_vector_info_plane_parallel (lenses.pyx:179-192) and
// generate_vector_info_null (lenses.pyx:196-207)
__device__ __forceinline__ void make_ray(const ytgb_view &v, int vi, int vj, Ray &r) {
    if (v.lens == YTGB_LENS_PLANE_PARALLEL) {
        double px = dsub(ddiv(dmul(v.width[0], (double)vi), dsub((double)v.nx, 1.0)), ddiv(v.width[0], 2.0));
        double py = dsub(ddiv(dmul(v.width[1], (double)vj), dsub((double)v.ny, 1.0)), ddiv(v.width[1], 2.0));
        r.pos[0] = dadd(dadd(dmul(v.vp_pos[0], px), dmul(v.vp_pos[3], py)), v.vp_pos[9]);
        r.pos[1] = dadd(dadd(dmul(v.vp_pos[1], px), dmul(v.vp_pos[4], py)), v.vp_pos[10]);
        r.pos[2] = dadd(dadd(dmul(v.vp_pos[2], px), dmul(v.vp_pos[5], py)), v.vp_pos[11]);
        for (int i = 0; i < 3; i++) r.dir[i] = v.vp_dir[i];
    } else {
        size_t o = ((size_t)vi * v.ny + vj) * 3;
        for (int i = 0; i < 3; i++) {
            r.pos[i] = __ldg(v.px_pos + o + i);
            r.dir[i] = __ldg(v.px_dir + o + i);
        }
    }
    // per-ray part of walk_volume's set-up (grid_traversal.pyx:49-57)
    for (int i = 0; i < 3; i++) {
        if (r.dir[i] < 0) r.step[i] = -1;
        else if (r.dir[i] == 0.0) r.step[i] = 0;
        else r.step[i] = 1;
        r.iv[i] = r.step[i] != 0 ? ddiv(1.0, r.dir[i]) : 0.0;
    }
}

struct BrickGeom {
    double le[3], re[3], dds[3], idds[3];
    int dims[3];
};

__device__ __forceinline__ void load_brick(const ytgb_brick *bp, BrickGeom &g) {
    const double *d = reinterpret_cast<const double *>(bp);
    for (int i = 0; i < 3; i++) {
        g.le[i] = __ldg(d + i);
        g.re[i] = __ldg(d + 3 + i);
        g.dds[i] = __ldg(d + 6 + i);
        g.idds[i] = __ldg(d + 9 + i);
    }
    const int *di = reinterpret_cast<const int *>(d + 12);
    for (int i = 0; i < 3; i++) g.dims[i] = __ldg(di + i);
}

// walk_volume set-up (grid_traversal.pyx:42-118).  Returns false where the
// reference returns 0 before its loop.
__device__ __forceinline__ bool walk_setup(const BrickGeom &b, const Ray &r, double max_t, int cur[3],
                                           double tmax[3], double tdelta[3], double &enter_t) {
    int direction = -1;
    double intersect_t = 1.1;
    if (b.le[0] <= r.pos[0] && r.pos[0] < b.re[0] && b.le[1] <= r.pos[1] && r.pos[1] < b.re[1] &&
        b.le[2] <= r.pos[2] && r.pos[2] < b.re[2]) {
        intersect_t = 0.0;
        direction = 3;
    }
    if (direction != 3) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            if (r.step[i] == 0) continue;
            const int x = (i + 1) % 3, y = (i + 2) % 3;
            double tl = r.step[i] > 0 ? dmul(dsub(b.le[i], r.pos[i]), r.iv[i]) : dmul(dsub(b.re[i], r.pos[i]), r.iv[i]);
            double tx = dadd(r.pos[x], dmul(tl, r.dir[x]));
            double ty = dadd(r.pos[y], dmul(tl, r.dir[y]));
            const double ex = dmul(1e-10, b.dds[x]), ey = dmul(1e-10, b.dds[y]);
            if (fabs(dsub(tx, b.le[x])) < ex) tx = b.le[x];
            else if (fabs(dsub(tx, b.re[x])) < ex) tx = b.re[x];
            if (fabs(dsub(ty, b.le[y])) < ey) ty = b.le[y];
            else if (fabs(dsub(ty, b.re[y])) < ey) ty = b.re[y];
            if (b.le[x] <= tx && tx <= b.re[x] && b.le[y] <= ty && ty <= b.re[y] && 0.0 <= tl && tl < intersect_t) {
                direction = i;
                intersect_t = tl;
            }
        }
    }
    if (!((0.0 <= intersect_t) && (intersect_t < max_t))) return false;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        tdelta[i] = dmul(dmul((double)r.step[i], r.iv[i]), b.dds[i]);
        if (i == direction && r.step[i] > 0) {
            cur[i] = 0;
        } else if (i == direction && r.step[i] < 0) {
            cur[i] = b.dims[i] - 1;
        } else {
            double tx = dadd(dmul(intersect_t, r.dir[i]), r.pos[i]);
            double ty = dmul(dsub(tx, b.le[i]), b.idds[i]);
            if (-1 < ty && ty < 0 && r.step[i] > 0) ty = 0.0;
            else if (b.dims[i] - 1 < ty && ty < b.dims[i] && r.step[i] < 0) ty = (double)(b.dims[i] - 1);
            cur[i] = (int)floor(ty);
        }
        double ty = 0.0;
        if (r.step[i] > 0) ty = dadd(dmul((double)(cur[i] + 1), b.dds[i]), b.le[i]);
        else if (r.step[i] < 0) ty = dadd(dmul((double)cur[i], b.dds[i]), b.le[i]);
        tmax[i] = dmul(dsub(ty, r.pos[i]), r.iv[i]);
        if (r.step[i] == 0) tmax[i] = 1e60;
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (cur[i] == b.dims[i] && r.step[i] >= 0) return false;
        if (cur[i] == -1 && r.step[i] <= -1) return false;
    }
    enter_t = intersect_t;
    return true;
}

// ---- compensated float32 accumulation -------------------------------------
// TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s + err == a + b exactly.
__device__ __forceinline__ void acc_add(float &h, float &l, float inc) {
    float s = __fadd_rn(h, inc);
    float bp = __fsub_rn(s, h);
    float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bp)), __fsub_rn(inc, bp));
    h = s;
    l = __fadd_rn(l, err);
}

// one channel of FIT_eval_transfer's update (field_interpolation_tables.pxd:
// 103-110): x <- dt*e + max(1 - dt*a, 0) * x, written as x + (dt*e - dt*a*x)
// so that only the increment is rounded.
__device__ __forceinline__ void acc_emit_absorb(float &h, float &l, float de, float da, bool comp) {
    if (da < 1.0f) {
        if (comp) {
            float inc = __fsub_rn(__fmaf_rn(-da, h, de), __fmul_rn(da, l));
            acc_add(h, l, inc);
        } else {
            h = __fadd_rn(__fmul_rn(de, 1.0f), __fmul_rn(__fsub_rn(1.0f, da), h));
        }
    } else {
        h = de;
        l = 0.0f;
    }
}

__device__ __forceinline__ float pick6(const float a[6], int i) {
    float r = a[0];
    r = i == 1 ? a[1] : r;
    r = i == 2 ? a[2] : r;
    r = i == 3 ? a[3] : r;
    r = i == 4 ? a[4] : r;
    r = i == 5 ? a[5] : r;
    return r;
}

// offset_interpolate (fixed_interpolator.cpp:34-52): z, then y, then x lerps
__device__ __forceinline__ float trilinear(const float *__restrict__ p, int sy, int sx, float dx, float dy, float dz) {
    float c000 = __ldg(p), c001 = __ldg(p + 1);
    float c010 = __ldg(p + sy), c011 = __ldg(p + sy + 1);
    float c100 = __ldg(p + sx), c101 = __ldg(p + sx + 1);
    float c110 = __ldg(p + sx + sy), c111 = __ldg(p + sx + sy + 1);
    float a0 = __fmaf_rn(dz, __fsub_rn(c001, c000), c000);
    float a1 = __fmaf_rn(dz, __fsub_rn(c011, c010), c010);
    float a2 = __fmaf_rn(dz, __fsub_rn(c101, c100), c100);
    float a3 = __fmaf_rn(dz, __fsub_rn(c111, c110), c110);
    float b0 = __fmaf_rn(dy, __fsub_rn(a1, a0), a0);
    float b1 = __fmaf_rn(dy, __fsub_rn(a3, a2), a2);
    return __fmaf_rn(dx, __fsub_rn(b1, b0), b0);
}

// FIT_get_value + FIT_eval_transfer's table combination
// (field_interpolation_tables.pxd:66-101).  The bounds test uses the float
// nearest outside each bound, so for a float v it decides exactly as the
// float64 test would for that v.
__device__ __forceinline__ void tf_eval(const ytgb_tf &tf, const float4 *__restrict__ tab, const float dvs[6],
                                        float trgba[6]) {
    float ist[6];
#pragma unroll
    for (int t = 0; t < 6; t++) {
        ist[t] = 0.0f;
        if (t < tf.n_fits) {
            float v = pick6(dvs, tf.field_id[t]);
            if (!(v >= tf.hi_excl[t] || v <= tf.lo_excl[t]) && v != 0.0f && isfinite(v)) {
                float q = __fmul_rn(__fsub_rn(v, tf.b0[t]), tf.idbin[t]);
                q = fminf(fmaxf(q, 0.0f), (float)(tf.nbins[t] - 2));
                int bin = (int)q;
                float4 e = tab[t * tf.nbins_max + bin];
                float dd = __fsub_rn(__fsub_rn(v, e.z), e.w);
                float out = __fmaf_rn(dd, e.y, e.x);
                if (tf.weight_field_id[t] != -1) out = __fmul_rn(out, pick6(dvs, tf.weight_field_id[t]));
                ist[t] = out;
            }
        }
    }
#pragma unroll
    for (int t = 0; t < 6; t++) {
        if (t < tf.n_fits && tf.weight_table_id[t] != -1) ist[t] = __fmul_rn(ist[t], pick6(ist, tf.weight_table_id[t]));
    }
#pragma unroll
    for (int c = 0; c < 6; c++) trgba[c] = pick6(ist, tf.field_table_ids[c]);
}

__device__ __forceinline__ unsigned long long fnv_mix(unsigned long long h, unsigned long long v) {
#pragma unroll
    for (int b = 0; b < 8; b++) {
        h ^= (v >> (8 * b)) & 0xffull;
        h *= YTGB_FNV_PRIME;
    }
    return h;
}

__device__ __forceinline__ void set_error(int32_t *err, int code) {
    if (err) atomicCAS(err, 0, code);
}

template <int MODE>
__global__ void __launch_bounds__(BLOCK) render_kernel(const ytgb_render_args a, unsigned long long *hashes,
                                                       long long *counts) {
    extern __shared__ float4 s_tab[];
    __shared__ unsigned long long s_cnt[4];
    const ytgb_view &v = a.view;
    if (threadIdx.x < 4) s_cnt[threadIdx.x] = 0;
    if (MODE == MODE_VR) {
        const int n = a.tf.n_fits * a.tf.nbins_max;
        const float4 *g = reinterpret_cast<const float4 *>(a.tf_tables);
        for (int k = threadIdx.x; k < n; k += blockDim.x) s_tab[k] = __ldg(g + k);
    }
    __syncthreads();
    const int vj = blockIdx.x * TILE_Y + (threadIdx.x % TILE_Y);
    const int vi = blockIdx.y * TILE_X + (threadIdx.x / TILE_Y);
    unsigned long long visits = 0, walks = 0, guarded = 0;
    if (vi < v.nx && vj < v.ny) {
    const size_t p = (size_t)vi * v.ny + vj;

    Ray r;
    make_ray(v, vi, vj, r);
    double max_t = a.zbuffer ? a.zbuffer[p] : 1.0;
    max_t = yt_fmin(yt_fmax(max_t, 0.0), 1.0);  // fclip (image_samplers.pyx:185)
    if (max_t > 1.0) max_t = 1.0;               // grid_traversal.pyx:42

    float xh[4], xl[4];
    unsigned touched = 0;
    double *img = a.image + p * 4;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        double x0 = img[c];
        xh[c] = (float)x0;
        xl[c] = (float)(x0 - (double)xh[c]);
    }
    const bool comp = !(a.flags & YTGB_FLAG_NO_COMPENSATION);
    unsigned long long th = 0;
    long long tcount = 0;
    if (MODE == MODE_TRACE) {
        th = hashes[p];
        tcount = counts[p];
    }

    for (int k = 0; k < a.n_order; k++) {
        const int4 rc = __ldg(reinterpret_cast<const int4 *>(a.rects) + k);
        if (vi < rc.x || vi >= rc.y || vj < rc.z || vj >= rc.w) continue;
        const int bi = __ldg(a.order + k);
        const ytgb_brick *bp = a.bricks + bi;
        BrickGeom g;
        load_brick(bp, g);
        int cur[3];
        double tmax[3], tdelta[3], enter_t;
        if (!walk_setup(g, r, max_t, cur, tmax, tdelta, enter_t)) continue;
        walks++;
        const int nf = __ldg(&bp->n_fields);
        const float *base = a.data + __ldg(&bp->data_offset);
        const long long fstride = __ldg(&bp->field_stride);
        const long long moff = __ldg(&bp->mask_offset);
        const int sy = g.dims[2] + 1, sx = (g.dims[1] + 1) * (g.dims[2] + 1);
        const int step_limit = g.dims[0] + g.dims[1] + g.dims[2] + 3;
        int hit = 0;
        while (true) {
            hit++;
            if (hit > step_limit) {
                set_error(a.error, YTGB_DEVERR_STEP_LIMIT);
                break;
            }
            int i;
            if (tmax[0] < tmax[1]) i = tmax[0] < tmax[2] ? 0 : 2;
            else i = tmax[1] < tmax[2] ? 1 : 2;
            const double exit_t = yt_fmin(tmax[i], max_t);
            // The reference can hand its sampler an index outside the brick:
            // an axis with v_dir == 0 whose position was snapped onto a face
            // from just outside (grid_traversal.pyx:67-78) starts at -1, and
            // its jump-start test (:113-117) only rejects -1 for negative
            // steps.  yt then reads outside the brick's arrays; here such a
            // cell contributes nothing and is counted in counters[3].
            const bool inside = (unsigned)cur[0] < (unsigned)g.dims[0] && (unsigned)cur[1] < (unsigned)g.dims[1] &&
                                (unsigned)cur[2] < (unsigned)g.dims[2];
            // ---- sampler callback -------------------------------------------
            if (MODE != MODE_TRACE && !inside) {
                guarded++;
            } else if (MODE == MODE_TRACE) {
                unsigned long long eb = __double_as_longlong(enter_t), xb = __double_as_longlong(exit_t);
                th = fnv_mix(th, (unsigned long long)(unsigned)bi);
                th = fnv_mix(th, (unsigned long long)(unsigned)cur[0] | ((unsigned long long)(unsigned)cur[1] << 32));
                th = fnv_mix(th, (unsigned long long)(unsigned)cur[2]);
                th = fnv_mix(th, eb);
                th = fnv_mix(th, xb);
                tcount++;
            } else if (MODE == MODE_PROJ || MODE == MODE_MIP) {
                // ProjectionSampler.sample (image_samplers.pyx:330-343)
                const int di = (cur[0] * g.dims[1] + cur[1]) * g.dims[2] + cur[2];
                const float dl = (float)dsub(exit_t, enter_t);
                const int nch = nf < 4 ? nf : 4;
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    if (c < nch) {
                        const float val = __ldg(base + c * fstride + di);
                        if (MODE == MODE_PROJ) {
                            const float inc = __fmul_rn(val, dl);
                            if (comp) acc_add(xh[c], xl[c], inc);
                            else xh[c] = __fadd_rn(xh[c], inc);
                        } else if (val > xh[c]) {
                            xh[c] = val;
                            xl[c] = 0.0f;
                        }
                        touched |= 1u << c;
                    }
                }
            } else {
                // VolumeRenderSampler.sample (image_samplers.pyx:453-487) and
                // InterpolatedProjectionSampler.sample (:372-403)
                const int cell = (cur[0] * g.dims[1] + cur[1]) * g.dims[2] + cur[2];
                bool masked = false;
                if (MODE == MODE_VR && moff >= 0 && a.masks) masked = __ldg(a.masks + moff + cell) != 1;
                if (!masked) {
                    const int off = cur[0] * sx + cur[1] * sy + cur[2];
                    double dt = dsub(exit_t, enter_t);
                    if (a.n_samples != 1) dt = ddiv(dt, (double)a.n_samples);
                    double dp[3], ds[3];
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        dp[q] = dadd(dmul(dadd(enter_t, dmul(0.5, dt)), r.dir[q]), r.pos[q]);
                        dp[q] = dsub(dp[q], dadd(dmul((double)cur[q], g.dds[q]), g.le[q]));
                        dp[q] = dmul(dp[q], g.idds[q]);
                        ds[q] = dmul(dmul(r.dir[q], g.idds[q]), dt);
                    }
                    const float dtf = (float)dt;
                    for (int s = 0; s < a.n_samples; s++) {
                        const float fx = (float)dp[0], fy = (float)dp[1], fz = (float)dp[2];
                        float dvs[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
                        for (int f = 0; f < 6; f++)
                            if (f < nf) dvs[f] = trilinear(base + f * fstride + off, sy, sx, fx, fy, fz);
                        if (MODE == MODE_VR) {
                            float trgba[6];
                            tf_eval(a.tf, s_tab, dvs, trgba);
                            if (a.tf.grey_opacity == 1) {
                                const float da = __fmul_rn(dtf, trgba[3]);
#pragma unroll
                                for (int c = 0; c < 4; c++) acc_emit_absorb(xh[c], xl[c], __fmul_rn(dtf, trgba[c]), da, comp);
                                touched |= 0xfu;
                            } else {
#pragma unroll
                                for (int c = 0; c < 3; c++) {
                                    const float d = __fmul_rn(dtf, trgba[c]);
                                    acc_emit_absorb(xh[c], xl[c], d, d, comp);
                                }
                                touched |= 0x7u;
                            }
                        } else {
                            const int n3 = nf < 3 ? nf : 3;
#pragma unroll
                            for (int c = 0; c < 3; c++) {
                                if (c < n3) {
                                    const float inc = __fmul_rn(dvs[c], dtf);
                                    if (comp) acc_add(xh[c], xl[c], inc);
                                    else xh[c] = __fadd_rn(xh[c], inc);
                                    touched |= 1u << c;
                                }
                            }
                        }
#pragma unroll
                        for (int q = 0; q < 3; q++) dp[q] = dadd(dp[q], ds[q]);
                    }
                }
            }
            visits++;
            // ---- advance (grid_traversal.pyx:134-138) -------------------------
            cur[i] += r.step[i];
            enter_t = tmax[i];
            tmax[i] = dadd(tmax[i], tdelta[i]);
            if (cur[i] < 0 || cur[i] >= g.dims[i] || enter_t >= max_t) break;
        }
    }

    if (MODE == MODE_TRACE) {
        hashes[p] = th;
        counts[p] = tcount;
    } else {
#pragma unroll
        for (int c = 0; c < 4; c++)
            if (touched & (1u << c)) img[c] = (double)xh[c] + (double)xl[c];
    }
    }  // active pixel
    if (a.counters) {
        if (visits) atomicAdd(&s_cnt[0], visits);
        if (walks) atomicAdd(&s_cnt[1], walks);
        if (guarded) atomicAdd(&s_cnt[3], guarded);
        if (vi < v.nx && vj < v.ny) atomicAdd(&s_cnt[2], 1ull);
        __syncthreads();
        if (threadIdx.x < 4 && s_cnt[threadIdx.x]) atomicAdd(a.counters + threadIdx.x, s_cnt[threadIdx.x]);
    }
}

int check_args(const ytgb_render_args *a, bool trace) {
    if (!a) {
        ytgb_set_error("ytgb_render: null args");
        return YTGB_ERR_INVALID;
    }
    const ytgb_view &v = a->view;
    if (v.nx <= 0 || v.ny <= 0) {
        ytgb_set_error("ytgb_render: empty image");
        return YTGB_ERR_INVALID;
    }
    if (a->kind < 0 || a->kind > 3) {
        ytgb_set_error("ytgb_render: unknown sampler kind");
        return YTGB_ERR_INVALID;
    }
    if (a->n_order < 0 || (a->n_order > 0 && (!a->order || !a->rects || !a->bricks || !a->data))) {
        ytgb_set_error("ytgb_render: missing brick arrays");
        return YTGB_ERR_INVALID;
    }
    if (!trace && !a->image) {
        ytgb_set_error("ytgb_render: missing image");
        return YTGB_ERR_INVALID;
    }
    if (v.lens == YTGB_LENS_PER_PIXEL && (!v.px_pos || !v.px_dir)) {
        ytgb_set_error("ytgb_render: per-pixel lens needs px_pos / px_dir");
        return YTGB_ERR_INVALID;
    }
    if (v.lens != YTGB_LENS_PER_PIXEL && v.lens != YTGB_LENS_PLANE_PARALLEL) {
        ytgb_set_error("ytgb_render: unknown lens");
        return YTGB_ERR_INVALID;
    }
    if (a->n_samples < 1) {
        ytgb_set_error("ytgb_render: n_samples must be >= 1");
        return YTGB_ERR_INVALID;
    }
    if (!trace && a->kind == YTGB_VOLUME_RENDER && !a->tf_tables) {
        ytgb_set_error("ytgb_render: volume rendering needs a transfer function");
        return YTGB_ERR_INVALID;
    }
    return YTGB_OK;
}

template <int MODE>
int launch(const ytgb_render_args *a, size_t smem, cudaStream_t s, unsigned long long *h, long long *c) {
    dim3 grid((a->view.ny + TILE_Y - 1) / TILE_Y, (a->view.nx + TILE_X - 1) / TILE_X);
    if (grid.y > 65535) {
        ytgb_set_error("ytgb_render: image too tall");
        return YTGB_ERR_INVALID;
    }
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(render_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            ytgb_set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return YTGB_ERR_CUDA;
        }
    }
    render_kernel<MODE><<<grid, BLOCK, smem, s>>>(*a, h, c);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("render launch: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return YTGB_OK;
}

}  // namespace

extern "C" int ytgb_render(const ytgb_render_args *a, void *stream) {
    int st = check_args(a, false);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    size_t smem = 0;
    if (a->kind == YTGB_VOLUME_RENDER) {
        const ytgb_tf &t = a->tf;
        if (t.n_fits < 0 || t.n_fits > 6 || t.nbins_max < 2 || t.nbins_max > YTGB_TF_MAX_BINS) {
            ytgb_set_error("ytgb_render: inconsistent transfer function header");
            return YTGB_ERR_INVALID;
        }
        for (int q = 0; q < t.n_fits; q++) {
            if (t.nbins[q] < 2 || t.nbins[q] > t.nbins_max || t.field_id[q] < 0 || t.field_id[q] > 5 ||
                t.weight_field_id[q] < -1 || t.weight_field_id[q] > 5 || t.weight_table_id[q] < -1 ||
                t.weight_table_id[q] >= t.n_fits) {
                ytgb_set_error("ytgb_render: transfer function table ids out of range");
                return YTGB_ERR_INVALID;
            }
        }
        for (int c = 0; c < 6; c++) {
            if (t.field_table_ids[c] < 0 || t.field_table_ids[c] > 5) {
                ytgb_set_error("ytgb_render: field_table_ids out of range");
                return YTGB_ERR_INVALID;
            }
        }
        smem = (size_t)t.n_fits * t.nbins_max * sizeof(float4);
        if (smem > 200 * 1024) {
            ytgb_set_error("ytgb_render: transfer-function tables exceed 200 KB of shared memory");
            return YTGB_ERR_INVALID;
        }
    }
    switch (a->kind) {
    case YTGB_VOLUME_RENDER: return launch<MODE_VR>(a, smem, s, nullptr, nullptr);
    case YTGB_PROJECTION: return launch<MODE_PROJ>(a, 0, s, nullptr, nullptr);
    case YTGB_INTERPOLATED_PROJECTION: return launch<MODE_IPROJ>(a, 0, s, nullptr, nullptr);
    default: return launch<MODE_MIP>(a, 0, s, nullptr, nullptr);
    }
}

extern "C" int ytgb_trace(const ytgb_render_args *a, unsigned long long *hashes, long long *counts, void *stream) {
    int st = check_args(a, true);
    if (st) return st;
    if (!hashes || !counts) {
        ytgb_set_error("ytgb_trace: null hash / count arrays");
        return YTGB_ERR_INVALID;
    }
    return launch<MODE_TRACE>(a, 0, (cudaStream_t)stream, hashes, counts);
}

extern "C" int ytgb_check_error(const int32_t *d_error, void *stream) {
    if (!d_error) return YTGB_OK;
    int32_t h = 0;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(&h, d_error, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("ytgb_check_error: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    if (h != 0) {
        char buf[96];
        snprintf(buf, sizeof(buf), "device guard tripped (code %d)", (int)h);
        ytgb_set_error(buf);
        e = cudaMemsetAsync(const_cast<int32_t *>(d_error), 0, sizeof(int32_t), s);
        return YTGB_ERR_DEVICE;
    }
    return YTGB_OK;
}
