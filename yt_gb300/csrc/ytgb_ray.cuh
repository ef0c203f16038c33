// ytgb_ray.cuh -- the per-ray brick walk of the sampler kernels.
//
// Everything one ray does inside one brick: walk_volume's exact float64
// set-up and cell stepping (grid_traversal.pyx:26-140), the float32 sample
// geometry, trilinear interpolation, transfer function and compensated
// compositing.  The functions are __host__ __device__: the kernels in
// ytgb_render.cu call them, and the test harness compiles the same source
// for the CPU (with plain IEEE operations in place of the _rn intrinsics and
// no floating-point contraction) to check it against the oracle without a
// GPU.  See ytgb_render.cu for the precision split.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector_types.h>
#include <vector_functions.h>

#include "ytgb.h"
#include "ytgb_internal.h"

#ifdef __CUDACC__
#define YTGB_HD __host__ __device__ __forceinline__
#define YTGB_UNROLL _Pragma("unroll")
#else
#define YTGB_HD inline
#define YTGB_UNROLL
#endif

namespace ytgb {

constexpr int MODE_VR = YTGB_VOLUME_RENDER;
constexpr int MODE_PROJ = YTGB_PROJECTION;
constexpr int MODE_IPROJ = YTGB_INTERPOLATED_PROJECTION;
constexpr int MODE_MIP = YTGB_MIP;
constexpr int MODE_TRACE = 4;

// ---- exact float64 arithmetic (never contracted into FMA) -----------------
#ifdef __CUDA_ARCH__
YTGB_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
YTGB_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
YTGB_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
YTGB_HD double ddiv(double a, double b) { return __ddiv_rn(a, b); }
YTGB_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
YTGB_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
YTGB_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
YTGB_HD float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
YTGB_HD float fdiv(float a, float b) { return __fdiv_rn(a, b); }
YTGB_HD long long dbits(double x) { return __double_as_longlong(x); }
template <typename T> YTGB_HD T ldg(const T *p) { return __ldg(p); }
YTGB_HD bool finitef(float x) { return (__float_as_uint(x) & 0x7f800000u) != 0x7f800000u; }
#else
// host build (the same walk code compiled for the CPU by the test harness,
// with -ffp-contract=off): plain IEEE operations
YTGB_HD double dadd(double a, double b) { return a + b; }
YTGB_HD double dsub(double a, double b) { return a - b; }
YTGB_HD double dmul(double a, double b) { return a * b; }
YTGB_HD double ddiv(double a, double b) { return a / b; }
YTGB_HD float fadd(float a, float b) { return a + b; }
YTGB_HD float fsub(float a, float b) { return a - b; }
YTGB_HD float fmul(float a, float b) { return a * b; }
YTGB_HD float ffma(float a, float b, float c) { return std::fmaf(a, b, c); }
YTGB_HD float fdiv(float a, float b) { return a / b; }
YTGB_HD long long dbits(double x) {
    long long b;
    std::memcpy(&b, &x, sizeof(b));
    return b;
}
template <typename T> YTGB_HD T ldg(const T *p) { return *p; }
YTGB_HD bool finitef(float x) {
    uint32_t b;
    std::memcpy(&b, &x, sizeof(b));
    return (b & 0x7f800000u) != 0x7f800000u;
}
#endif

// Order-preserving key of a non-NaN double: key(a) < key(b) <=> a < b, and
// key(-0.0) == key(+0.0); integer pipe only.
YTGB_HD long long dkey(double x) {
    long long b = dbits(x);
    long long m = b >> 63;
    return (b ^ (m & 0x7fffffffffffffffll)) - m;
}

struct Ray {
    double pos[3];
    double dir[3];
    double iv[3];
    float fpos[3], fdir[3];
    int step[3];
};

// generate_vector_info_plane_parallel (lenses.pyx:179-192) and
// generate_vector_info_null (lenses.pyx:196-207)
YTGB_HD void make_ray(const ytgb_view &v, int vi, int vj, Ray &r) {
    if (v.lens == YTGB_LENS_PLANE_PARALLEL) {
        double px = dsub(ddiv(dmul(v.width[0], (double)vi), dsub((double)v.nx, 1.0)), ddiv(v.width[0], 2.0));
        double py = dsub(ddiv(dmul(v.width[1], (double)vj), dsub((double)v.ny, 1.0)), ddiv(v.width[1], 2.0));
        r.pos[0] = dadd(dadd(dmul(v.vp_pos[0], px), dmul(v.vp_pos[3], py)), v.vp_pos[9]);
        r.pos[1] = dadd(dadd(dmul(v.vp_pos[1], px), dmul(v.vp_pos[4], py)), v.vp_pos[10]);
        r.pos[2] = dadd(dadd(dmul(v.vp_pos[2], px), dmul(v.vp_pos[5], py)), v.vp_pos[11]);
        YTGB_UNROLL
        for (int i = 0; i < 3; i++) r.dir[i] = v.vp_dir[i];
    } else if (v.lens == YTGB_LENS_PERSPECTIVE) {
        // PerspectiveLens._get_sampler_params (lens.py:186-225) for one pixel:
        // px = linspace(-0.5, 0.5, nx)[vi] (numpy: i*step + start, last = stop),
        // vector = (w0*(east*px) + w1*(north*py) + normal*w2) * (max_length/w2)
        const double px = (v.nx > 1 && vi == v.nx - 1)
                              ? 0.5
                              : dadd(dmul((double)vi, v.nx > 1 ? ddiv(1.0, (double)(v.nx - 1)) : 0.0), -0.5);
        const double py = (v.ny > 1 && vj == v.ny - 1)
                              ? 0.5
                              : dadd(dmul((double)vj, v.ny > 1 ? ddiv(1.0, (double)(v.ny - 1)) : 0.0), -0.5);
        YTGB_UNROLL
        for (int i = 0; i < 3; i++) {
            const double sx = dmul(v.vp_dir[0], dmul(v.vp_pos[3 + i], px));
            const double sy = dmul(v.vp_dir[1], dmul(v.vp_pos[6 + i], py));
            r.dir[i] = dmul(dadd(dadd(sx, sy), dmul(v.vp_pos[9 + i], v.vp_dir[2])), v.ray_scale);
            r.pos[i] = v.vp_pos[i];
        }
    } else {
        size_t o = ((size_t)vi * v.ny + vj) * 3;
        YTGB_UNROLL
        for (int i = 0; i < 3; i++) {
            r.pos[i] = ldg(v.px_pos + o + i);
            r.dir[i] = ldg(v.px_dir + o + i);
        }
    }
    // per-ray part of walk_volume's set-up (grid_traversal.pyx:49-57)
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        if (r.dir[i] < 0) r.step[i] = -1;
        else if (r.dir[i] == 0.0) r.step[i] = 0;
        else r.step[i] = 1;
        r.iv[i] = r.step[i] != 0 ? ddiv(1.0, r.dir[i]) : 0.0;
        r.fpos[i] = (float)r.pos[i];
        r.fdir[i] = (float)r.dir[i];
    }
}

struct BrickGeom {
    double le[3], re[3], dds[3], idds[3];
    int dims[3];
};

YTGB_HD void load_brick(const ytgb_brick *bp, BrickGeom &g) {
    const double *d = reinterpret_cast<const double *>(bp);
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        g.le[i] = ldg(d + i);
        g.re[i] = ldg(d + 3 + i);
        g.dds[i] = ldg(d + 6 + i);
        g.idds[i] = ldg(d + 9 + i);
    }
    const int *di = reinterpret_cast<const int *>(d + 12);
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) g.dims[i] = ldg(di + i);
}

// Float32 slab test of the brick's box grown by a margin m (1e-4 of the
// coordinate scale, far above both the float32 error of these operations
// and walk_volume's 1e-10*dds face snapping).  True only when the ray misses
// the grown box for every t in [0, max_t]; then no face test of walk_volume
// can pass with intersect_t < max_t and the exact set-up returns 0.
YTGB_HD bool surely_misses(const BrickGeom &b, const Ray &r, float max_t) {
    float t0 = -1e30f, t1 = 1e30f;
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        const float lo = (float)b.le[i], hi = (float)b.re[i];
        const float m = 1e-4f * (fabsf(lo) + fabsf(hi) + fabsf(r.fpos[i]) + 1.0f);
        if (r.step[i] == 0) {
            if (r.fpos[i] < lo - m || r.fpos[i] > hi + m) return true;
        } else {
            const float inv = 1.0f / r.fdir[i];
            float ta = (lo - m - r.fpos[i]) * inv;
            float tb = (hi + m - r.fpos[i]) * inv;
            if (ta > tb) {
                float tmp = ta;
                ta = tb;
                tb = tmp;
            }
            const float w = 1e-4f * (fabsf(ta) + fabsf(tb)) + 1e-6f;
            t0 = fmaxf(t0, ta - w);
            t1 = fminf(t1, tb + w);
        }
    }
    return t1 < t0 || t1 < -1e-4f || t0 > max_t + 1e-4f;
}

struct Walk {
    double tmax[3];
    double enter_t;
    int cur[3];
    float P[3];  // cell-local position of the current cell's entry point
};

// walk_volume set-up (grid_traversal.pyx:42-118).  Returns false where the
// reference returns 0 before its loop.
YTGB_HD bool walk_setup(const BrickGeom &b, const Ray &r, double max_t, Walk &w) {
    int direction = -1;
    double intersect_t = 1.1;
    // inside test (:44-48); skipped when float32 says the start point is
    // clearly outside the brick
    bool maybe_inside = true;
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        const float lo = (float)b.le[i], hi = (float)b.re[i];
        const float m = 1e-5f * (fabsf(lo) + fabsf(hi) + fabsf(r.fpos[i]) + 1e-3f);
        maybe_inside = maybe_inside && !(r.fpos[i] < lo - m) && !(r.fpos[i] > hi + m);
    }
    if (maybe_inside && b.le[0] <= r.pos[0] && r.pos[0] < b.re[0] && b.le[1] <= r.pos[1] && r.pos[1] < b.re[1] &&
        b.le[2] <= r.pos[2] && r.pos[2] < b.re[2]) {
        intersect_t = 0.0;
        direction = 3;
    }
    if (direction != 3) {
        YTGB_UNROLL
        for (int i = 0; i < 3; i++) {
            if (r.step[i] == 0) continue;
            const int x = (i + 1) % 3, y = (i + 2) % 3;
            // Float32 pre-test of where the ray meets this face's plane.  The
            // error of q below is at most ~4 float32 roundings of
            // (|e|+|p_i|)|d_x/d_i| + |tl d_x| + |p_x|; the margin is 1e-5 of
            // that sum (and of the edges), so a point this far off the face
            // is off it in float64 as well.  NaN or inf never prunes.
            {
                const float e = r.step[i] > 0 ? (float)b.le[i] : (float)b.re[i];
                const float a0 = fabsf(e) + fabsf(r.fpos[i]);
                const float tlf = (e - r.fpos[i]) / r.fdir[i];
                const float qx = r.fpos[x] + tlf * r.fdir[x];
                const float qy = r.fpos[y] + tlf * r.fdir[y];
                const float sx = 1e-5f * (a0 * fabsf(r.fdir[x] / r.fdir[i]) + fabsf(tlf * r.fdir[x]) +
                                          fabsf(r.fpos[x]) + fabsf((float)b.le[x]) + fabsf((float)b.re[x]) + 1e-3f);
                const float sy = 1e-5f * (a0 * fabsf(r.fdir[y] / r.fdir[i]) + fabsf(tlf * r.fdir[y]) +
                                          fabsf(r.fpos[y]) + fabsf((float)b.le[y]) + fabsf((float)b.re[y]) + 1e-3f);
                const float st = 1e-5f * (a0 / fabsf(r.fdir[i]) + fabsf(tlf) + 1e-3f);
                if (qx < (float)b.le[x] - sx || qx > (float)b.re[x] + sx || qy < (float)b.le[y] - sy ||
                    qy > (float)b.re[y] + sy || tlf < -st)
                    continue;
            }
            double tl = r.step[i] > 0 ? dmul(dsub(b.le[i], r.pos[i]), r.iv[i]) : dmul(dsub(b.re[i], r.pos[i]), r.iv[i]);
            // the last clause of the reference's test, evaluated first (the
            // clauses have no side effects)
            if (!(0.0 <= tl && tl < intersect_t)) continue;
            double tx = dadd(r.pos[x], dmul(tl, r.dir[x]));
            double ty = dadd(r.pos[y], dmul(tl, r.dir[y]));
            const double ex = dmul(1e-10, b.dds[x]), ey = dmul(1e-10, b.dds[y]);
            if (fabs(dsub(tx, b.le[x])) < ex) tx = b.le[x];
            else if (fabs(dsub(tx, b.re[x])) < ex) tx = b.re[x];
            if (fabs(dsub(ty, b.le[y])) < ey) ty = b.le[y];
            else if (fabs(dsub(ty, b.re[y])) < ey) ty = b.re[y];
            if (b.le[x] <= tx && tx <= b.re[x] && b.le[y] <= ty && ty <= b.re[y]) {
                direction = i;
                intersect_t = tl;
            }
        }
    }
    if (!((0.0 <= intersect_t) && (intersect_t < max_t))) return false;
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        double ty = 0.0;
        if (i == direction && r.step[i] > 0) {
            w.cur[i] = 0;
            w.P[i] = 0.0f;
        } else if (i == direction && r.step[i] < 0) {
            w.cur[i] = b.dims[i] - 1;
            w.P[i] = 1.0f;
        } else {
            double tx = dadd(dmul(intersect_t, r.dir[i]), r.pos[i]);
            ty = dmul(dsub(tx, b.le[i]), b.idds[i]);
            // the sample position keeps the unclamped coordinate: yt's clamps
            // below only steer the index (its sampler recomputes dp from the
            // ray, image_samplers.pyx:475-478)
            const double ty_raw = ty;
            if (-1 < ty && ty < 0 && r.step[i] > 0) ty = 0.0;
            else if (b.dims[i] - 1 < ty && ty < b.dims[i] && r.step[i] < 0) ty = (double)(b.dims[i] - 1);
            w.cur[i] = (int)floor(ty);
            w.P[i] = (float)dsub(ty_raw, (double)w.cur[i]);
        }
        if (r.step[i] > 0) ty = dadd(dmul((double)(w.cur[i] + 1), b.dds[i]), b.le[i]);
        else if (r.step[i] < 0) ty = dadd(dmul((double)w.cur[i], b.dds[i]), b.le[i]);
        w.tmax[i] = r.step[i] != 0 ? dmul(dsub(ty, r.pos[i]), r.iv[i]) : 1e60;
    }
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        if (w.cur[i] == b.dims[i] && r.step[i] >= 0) return false;
        if (w.cur[i] == -1 && r.step[i] <= -1) return false;
    }
    w.enter_t = intersect_t;
    return true;
}

// ---- compensated float32 accumulation -------------------------------------
// TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s + err == h + inc exactly.
YTGB_HD void acc_add(float &h, float &l, float inc) {
    float s = fadd(h, inc);
    float bp = fsub(s, h);
    float err = fadd(fsub(h, fsub(s, bp)), fsub(inc, bp));
    h = s;
    l = fadd(l, err);
}

// Non-grey channel of FIT_eval_transfer (field_interpolation_tables.pxd:108-
// 110): x <- d + max(1 - d, 0) x with d = dt*e, as x + d (1 - x).
YTGB_HD void acc_emit(float &h, float &l, float d, bool comp) {
    if (d < 1.0f) {
        if (comp) {
            float u = fsub(fsub(1.0f, h), l);
            acc_add(h, l, fmul(d, u));
        } else {
            h = ffma(fsub(1.0f, d), h, d);
        }
    } else {
        h = d;
        l = 0.0f;
    }
}

// Grey-opacity channel (field_interpolation_tables.pxd:103-106):
// x <- dt*e + max(1 - dt*a, 0) x, as x + (dt*e - da*x) with both products
// formed exactly (TwoProduct by FMA), so that near equilibrium (dt*e ~ da*x)
// the cancellation does not expose their rounding.
YTGB_HD void acc_grey(float &h, float &l, float dt, float e, float da, bool comp) {
    if (da < 1.0f) {
        if (comp) {
            float de = fmul(dt, e);
            float de_l = ffma(dt, e, -de);
            float p = fmul(da, h);
            float p_l = ffma(da, h, -p);
            float inc = fsub(fadd(fsub(de, p), fsub(de_l, p_l)), fmul(da, l));
            acc_add(h, l, inc);
        } else {
            h = ffma(-da, h, fadd(h, fmul(dt, e)));
        }
    } else {
        h = fmul(dt, e);
        l = 0.0f;
    }
}

YTGB_HD float pick6(const float a[6], int i) {
    float r = a[0];
    r = i == 1 ? a[1] : r;
    r = i == 2 ? a[2] : r;
    r = i == 3 ? a[3] : r;
    r = i == 4 ? a[4] : r;
    r = i == 5 ? a[5] : r;
    return r;
}

// offset_interpolate (fixed_interpolator.cpp:34-52): z, then y, then x lerps
YTGB_HD float trilinear(const float *__restrict__ p, int sy, int sx, float dx, float dy, float dz) {
    float c000 = ldg(p), c001 = ldg(p + 1);
    float c010 = ldg(p + sy), c011 = ldg(p + sy + 1);
    float c100 = ldg(p + sx), c101 = ldg(p + sx + 1);
    float c110 = ldg(p + sx + sy), c111 = ldg(p + sx + sy + 1);
    float a0 = ffma(dz, fsub(c001, c000), c000);
    float a1 = ffma(dz, fsub(c011, c010), c010);
    float a2 = ffma(dz, fsub(c101, c100), c100);
    float a3 = ffma(dz, fsub(c111, c110), c110);
    float b0 = ffma(dy, fsub(a1, a0), a0);
    float b1 = ffma(dy, fsub(a3, a2), a2);
    return ffma(dx, fsub(b1, b0), b0);
}

// FIT_get_value + FIT_eval_transfer's table combination
// (field_interpolation_tables.pxd:66-101).  The bounds test uses the float
// nearest outside each bound, so for a float v it decides exactly as the
// float64 test would for that v.  Zero, infinite and NaN values give 0 like
// the reference's !isnormal test.
YTGB_HD void tf_eval(const ytgb_tf &tf, const float4 *__restrict__ tab, const float dvs[6],
                                        float trgba[6]) {
    float ist[6];
    YTGB_UNROLL
    for (int t = 0; t < 6; t++) {
        ist[t] = 0.0f;
        if (t < tf.n_fits) {
            float v = pick6(dvs, tf.field_id[t]);
            if (!(v >= tf.hi_excl[t] || v <= tf.lo_excl[t]) && v != 0.0f && finitef(v)) {
                float q = fmul(fsub(v, tf.b0[t]), tf.idbin[t]);
                q = fminf(fmaxf(q, 0.0f), (float)(tf.nbins[t] - 2));
                int bin = (int)q;
                float4 e = tab[t * tf.nbins_max + bin];
                float dd = fsub(fsub(v, e.z), e.w);
                float out = ffma(dd, e.y, e.x);
                if (tf.weight_field_id[t] != -1) out = fmul(out, pick6(dvs, tf.weight_field_id[t]));
                ist[t] = out;
            }
        }
    }
    YTGB_UNROLL
    for (int t = 0; t < 6; t++) {
        if (t < tf.n_fits && tf.weight_table_id[t] != -1) ist[t] = fmul(ist[t], pick6(ist, tf.weight_table_id[t]));
    }
    YTGB_UNROLL
    for (int c = 0; c < 6; c++) trgba[c] = pick6(ist, tf.field_table_ids[c]);
}

YTGB_HD unsigned long long fnv_mix(unsigned long long h, unsigned long long v) {
    YTGB_UNROLL
    for (int b = 0; b < 8; b++) {
        h ^= (v >> (8 * b)) & 0xffull;
        h *= YTGB_FNV_PRIME;
    }
    return h;
}

YTGB_HD void set_error(int32_t *err, int code) {
#ifdef __CUDA_ARCH__
    if (err) atomicCAS(err, 0, code);
#else
    if (err && *err == 0) *err = code;
#endif
}


// State one ray carries across the bricks of a view.
struct RayState {
    float xh[4], xl[4];          // compensated image value (hi + lo)
    unsigned touched;            // channels the sampler wrote
    unsigned long long th;       // trace hash
    long long tcount;            // trace count
    unsigned long long visits, walks, guarded;
    double tdelta[3];            // cached per dds
    long long last_dds[3];
    double max_t;
    long long kmax;
    bool comp;
};

YTGB_HD void ray_state_init(RayState &s, const double *img, double zbuf, bool has_zbuf, uint32_t flags) {
    double max_t = has_zbuf ? zbuf : 1.0;
    max_t = max_t > 0.0 ? max_t : 0.0;  // fclip(z, 0, 1) (image_samplers.pyx:185)
    max_t = max_t < 1.0 ? max_t : 1.0;  // also grid_traversal.pyx:42
    s.max_t = max_t;
    s.kmax = dkey(max_t);
    YTGB_UNROLL
    for (int c = 0; c < 4; c++) {
        double x0 = img ? img[c] : 0.0;
        s.xh[c] = (float)x0;
        s.xl[c] = (float)(x0 - (double)s.xh[c]);
    }
    s.touched = 0;
    s.th = 0;
    s.tcount = 0;
    s.visits = s.walks = s.guarded = 0;
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        s.tdelta[i] = 0.0;
        s.last_dds[i] = -1;
    }
    s.comp = !(flags & YTGB_FLAG_NO_COMPENSATION);
}

// One brick of one ray: cast_through_kdtree's walk_volume call
// (image_samplers.pyx:186) with the sampler callback inlined.
// s_tab: the transfer-function table as laid out in shared memory (see the
// kernel prologue); bi: the brick index.
template <int MODE, int CTF>
YTGB_HD void walk_brick(const ytgb_render_args &a, const float4 *s_tab, const Ray &r, int bi, RayState &st) {
    const ytgb_brick *bp = a.bricks + bi;
    BrickGeom g;
    load_brick(bp, g);
    const double max_t = st.max_t;
    const long long kmax = st.kmax;
    if (surely_misses(g, r, (float)max_t)) return;
    Walk w;
    if (!walk_setup(g, r, max_t, w)) return;
    // tdelta depends on the ray and dds only (grid_traversal.pyx:86)
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        const long long db = dbits(g.dds[i]);
        if (db != st.last_dds[i]) {
            st.tdelta[i] = dmul(dmul((double)r.step[i], r.iv[i]), g.dds[i]);
            st.last_dds[i] = db;
        }
    }
    st.walks++;
    const int nf = ldg(&bp->n_fields);
    const float *base_p = a.data + ldg(&bp->data_offset);
    const long long fstride = ldg(&bp->field_stride);
    const long long moff = ldg(&bp->mask_offset);
    const int sy = g.dims[2] + 1, sx = (g.dims[1] + 1) * (g.dims[2] + 1);
    const int step_limit = g.dims[0] + g.dims[1] + g.dims[2] + 3;
    float vel[3];  // cells per unit t, for the float32 geometry
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) vel[i] = fmul(r.fdir[i], (float)g.idds[i]);
    long long K0 = dkey(w.tmax[0]), K1 = dkey(w.tmax[1]), K2 = dkey(w.tmax[2]);
    double enter_t = w.enter_t;
    int hitc = 0;
    float *xh = st.xh, *xl = st.xl;
    const bool comp = st.comp;
    while (true) {
        if (++hitc > step_limit) {
            set_error(a.error, YTGB_DEVERR_STEP_LIMIT);
            break;
        }
        int i;
        if (K0 < K1) i = K0 < K2 ? 0 : 2;
        else i = K1 < K2 ? 1 : 2;
        const double tm = i == 0 ? w.tmax[0] : (i == 1 ? w.tmax[1] : w.tmax[2]);
        const long long Ki = i == 0 ? K0 : (i == 1 ? K1 : K2);
        const double exit_t = Ki < kmax ? tm : max_t;  // fmin(tmax[i], max_t)
        const bool inside = (unsigned)w.cur[0] < (unsigned)g.dims[0] && (unsigned)w.cur[1] < (unsigned)g.dims[1] &&
                            (unsigned)w.cur[2] < (unsigned)g.dims[2];
        float dtf = 0.0f;
        if (MODE != MODE_TRACE) dtf = (float)dsub(exit_t, enter_t);
        // ---- sampler callback ------------------------------------------------
        if (MODE == MODE_TRACE) {
            st.th = fnv_mix(st.th, (unsigned long long)(unsigned)bi);
            st.th = fnv_mix(st.th, (unsigned long long)(unsigned)w.cur[0] | ((unsigned long long)(unsigned)w.cur[1] << 32));
            st.th = fnv_mix(st.th, (unsigned long long)(unsigned)w.cur[2]);
            st.th = fnv_mix(st.th, (unsigned long long)dbits(enter_t));
            st.th = fnv_mix(st.th, (unsigned long long)dbits(exit_t));
            st.tcount++;
        } else if (!inside) {
            st.guarded++;
        } else if (MODE == MODE_PROJ || MODE == MODE_MIP) {
            // ProjectionSampler.sample (image_samplers.pyx:330-343)
            const int di = (w.cur[0] * g.dims[1] + w.cur[1]) * g.dims[2] + w.cur[2];
            const int nch = nf < 4 ? nf : 4;
            YTGB_UNROLL
            for (int c = 0; c < 4; c++) {
                if (c < nch) {
                    const float val = ldg(base_p + c * fstride + di);
                    if (MODE == MODE_PROJ) {
                        const float inc = fmul(val, dtf);
                        if (comp) acc_add(xh[c], xl[c], inc);
                        else xh[c] = fadd(xh[c], inc);
                    } else if (val > xh[c]) {
                        xh[c] = val;
                        xl[c] = 0.0f;
                    }
                    st.touched |= 1u << c;
                }
            }
        } else {
            // VolumeRenderSampler.sample (image_samplers.pyx:453-487) and
            // InterpolatedProjectionSampler.sample (:372-403)
            const int cell = (w.cur[0] * g.dims[1] + w.cur[1]) * g.dims[2] + w.cur[2];
            bool masked = false;
            if (MODE == MODE_VR && moff >= 0 && a.masks) masked = ldg(a.masks + moff + cell) != 1;
            if (!masked) {
                const int off = w.cur[0] * sx + w.cur[1] * sy + w.cur[2];
                const int ns = a.n_samples;
                const float dts = ns == 1 ? dtf : fdiv(dtf, (float)ns);
                for (int s = 0; s < ns; s++) {
                    // sample s at enter_t + (s + 1/2) dt (image_samplers.pyx:475-487)
                    const float f = fmul(dts, (float)s + 0.5f);
                    const float fx = fminf(fmaxf(ffma(f, vel[0], w.P[0]), 0.0f), 1.0f);
                    const float fy = fminf(fmaxf(ffma(f, vel[1], w.P[1]), 0.0f), 1.0f);
                    const float fz = fminf(fmaxf(ffma(f, vel[2], w.P[2]), 0.0f), 1.0f);
                    if (MODE == MODE_VR && CTF) {
                        const float val = trilinear(base_p + off, sy, sx, fx, fy, fz);
                        const ytgb_tf &tf = a.tf;
                        // out of the table's range: zero emission and
                        // absorption leave x unchanged
                        if (!(val >= tf.hi_excl[0] || val <= tf.lo_excl[0]) && val != 0.0f && finitef(val)) {
                            float q = fmul(fsub(val, tf.b0[0]), tf.idbin[0]);
                            q = fminf(fmaxf(q, 0.0f), (float)(tf.nbins[0] - 2));
                            const int bin = (int)q;
                            const float4 Y = s_tab[3 * bin + 0], D = s_tab[3 * bin + 1];
                            const float4 Z = s_tab[3 * bin + 2];
                            const float dd = fsub(fsub(val, Z.x), Z.y);
                            const float al = ffma(dd, D.w, Y.w);
                            const float er = fmul(ffma(dd, D.x, Y.x), al);
                            const float eg = fmul(ffma(dd, D.y, Y.y), al);
                            const float eb = fmul(ffma(dd, D.z, Y.z), al);
                            if (tf.grey_opacity == 1) {
                                const float da = fmul(dts, al);
                                acc_grey(xh[0], xl[0], dts, er, da, comp);
                                acc_grey(xh[1], xl[1], dts, eg, da, comp);
                                acc_grey(xh[2], xl[2], dts, eb, da, comp);
                                acc_grey(xh[3], xl[3], dts, al, da, comp);
                            } else {
                                acc_emit(xh[0], xl[0], fmul(dts, er), comp);
                                acc_emit(xh[1], xl[1], fmul(dts, eg), comp);
                                acc_emit(xh[2], xl[2], fmul(dts, eb), comp);
                            }
                        }
                        st.touched |= a.tf.grey_opacity == 1 ? 0xfu : 0x7u;
                    } else {
                        float dvs[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                        YTGB_UNROLL
                        for (int fi = 0; fi < 6; fi++)
                            if (fi < nf) dvs[fi] = trilinear(base_p + fi * fstride + off, sy, sx, fx, fy, fz);
                        if (MODE == MODE_VR) {
                            float trgba[6];
                            tf_eval(a.tf, s_tab, dvs, trgba);
                            if (a.tf.grey_opacity == 1) {
                                const float da = fmul(dts, trgba[3]);
                                YTGB_UNROLL
                                for (int c = 0; c < 4; c++) acc_grey(xh[c], xl[c], dts, trgba[c], da, comp);
                                st.touched |= 0xfu;
                            } else {
                                YTGB_UNROLL
                                for (int c = 0; c < 3; c++) acc_emit(xh[c], xl[c], fmul(dts, trgba[c]), comp);
                                st.touched |= 0x7u;
                            }
                        } else {
                            const int n3 = nf < 3 ? nf : 3;
                            YTGB_UNROLL
                            for (int c = 0; c < 3; c++) {
                                if (c < n3) {
                                    const float inc = fmul(dvs[c], dts);
                                    if (comp) acc_add(xh[c], xl[c], inc);
                                    else xh[c] = fadd(xh[c], inc);
                                    st.touched |= 1u << c;
                                }
                            }
                        }
                    }
                }
            }
        }
        st.visits++;
        // ---- advance (grid_traversal.pyx:134-138) -----------------------------
        // float32 geometry: move to the exit point, then put the stepped axis
        // exactly on the next cell's entry face
        YTGB_UNROLL
        for (int q = 0; q < 3; q++) w.P[q] = ffma(dtf, vel[q], w.P[q]);
        const int si = i == 0 ? r.step[0] : (i == 1 ? r.step[1] : r.step[2]);
        const float wrap = si > 0 ? 0.0f : 1.0f;
        const double td = i == 0 ? st.tdelta[0] : (i == 1 ? st.tdelta[1] : st.tdelta[2]);
        const double tn = dadd(tm, td);
        const long long Kn = dkey(tn);
        int ci, di;
        if (i == 0) {
            w.P[0] = wrap; w.cur[0] += si; w.tmax[0] = tn; K0 = Kn; ci = w.cur[0]; di = g.dims[0];
        } else if (i == 1) {
            w.P[1] = wrap; w.cur[1] += si; w.tmax[1] = tn; K1 = Kn; ci = w.cur[1]; di = g.dims[1];
        } else {
            w.P[2] = wrap; w.cur[2] += si; w.tmax[2] = tn; K2 = Kn; ci = w.cur[2]; di = g.dims[2];
        }
        enter_t = tm;
        if (ci < 0 || ci >= di || !(Ki < kmax)) break;  // ... or enter_t >= max_t
    }
}

}  // namespace ytgb
