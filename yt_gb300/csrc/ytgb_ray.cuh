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
constexpr int MODE_LIGHT = YTGB_LIGHT_SOURCE;
constexpr int MODE_TRACE = 5;

// ---- exact float64 arithmetic (never contracted into FMA) -----------------
#ifdef __CUDA_ARCH__
YTGB_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
YTGB_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
YTGB_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
YTGB_HD double ddiv(double a, double b) { return __ddiv_rn(a, b); }
YTGB_HD double dsqrt(double a) { return __dsqrt_rn(a); }
YTGB_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
YTGB_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
YTGB_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
YTGB_HD float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
YTGB_HD float fdiv(float a, float b) { return __fdiv_rn(a, b); }
YTGB_HD float frcp(float a) { return __frcp_rn(a); }
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
YTGB_HD double dsqrt(double a) { return std::sqrt(a); }
YTGB_HD float fadd(float a, float b) { return a + b; }
YTGB_HD float fsub(float a, float b) { return a - b; }
YTGB_HD float fmul(float a, float b) { return a * b; }
YTGB_HD float ffma(float a, float b, float c) { return std::fmaf(a, b, c); }
YTGB_HD float fdiv(float a, float b) { return a / b; }
YTGB_HD float frcp(float a) { return 1.0f / a; }
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


// ---- integer-exact helpers for positive float64 values --------------------
// These replace float64-pipe instructions (conversions, floor, the walk's
// `tmax += tdelta`) by integer work on the bit patterns, with identical
// results.
constexpr long long MANT52 = (1LL << 52) - 1;

#ifdef __CUDA_ARCH__
YTGB_HD double dfrom(long long b) { return __longlong_as_double(b); }
YTGB_HD int clz64(unsigned long long x) { return __clzll((long long)x); }
YTGB_HD float ffrom(uint32_t b) { return __uint_as_float(b); }
#else
YTGB_HD double dfrom(long long b) {
    double x;
    std::memcpy(&x, &b, sizeof(x));
    return x;
}
YTGB_HD int clz64(unsigned long long x) { return __builtin_clzll(x); }
YTGB_HD float ffrom(uint32_t b) {
    float x;
    std::memcpy(&x, &b, sizeof(x));
    return x;
}
#endif

// The float nearest to F * 2^k (round to nearest even), F > 0 or 0.
YTGB_HD float scaled_to_float(unsigned long long F, int k) {
    if (F == 0) return 0.0f;
    const int lead = 63 - clz64(F);
    int e = lead + k;
    unsigned long long sig;
    if (lead > 23) {
        const int rs = lead - 23;
        sig = F >> rs;
        const unsigned long long rem = F & ((1ull << rs) - 1), half = 1ull << (rs - 1);
        if (rem > half || (rem == half && (sig & 1ull))) {
            sig++;
            if (sig == (1ull << 24)) {
                sig >>= 1;
                e++;
            }
        }
    } else {
        sig = F << (23 - lead);
    }
    if (e > 127) return ffrom(0x7f800000u);
    if (e < -126) return 0.0f;  // below float's normal range: negligible here
    return ffrom(((uint32_t)(e + 127) << 23) | (uint32_t)(sig & 0x7fffffull));
}

// F * 2^k as float for F < 2^54, faithfully rounded (one of the two floats
// around it): F's high 22 bits (exact as a float) times 2^32 plus its low
// 32 bits rounded to float, in one FMA -- the low part's rounding (< 2^7) is
// under a quarter ulp of any result >= 2^32 -- then an exact scaling by a
// power of two while the result stays in float's normal range; otherwise
// the bit-level rounding above (the nearest float).  32-bit conversions
// keep the per-cell dt off the float64 pipe, which a 64-bit conversion
// uses (3 % of the benchmark frame).
YTGB_HD float scaled_to_float_fast(unsigned long long F, int k) {
    if (k < -126 || k > 127 - 54) return scaled_to_float(F, k);
    const unsigned hi = (unsigned)(F >> 32), lo = (unsigned)F;
#ifdef __CUDA_ARCH__
    const float f = ffma(__uint2float_rn(hi), 4294967296.0f, __uint2float_rn(lo));
#else
    const float f = ffma((float)hi, 4294967296.0f, (float)lo);
#endif
    return fmul(f, ffrom((uint32_t)(k + 127) << 23));
}

// x - y as float for x >= y >= 0 given as float64 bit patterns: exact
// integer difference when the exponents are equal or adjacent, else float64.
YTGB_HD float diff_to_float_ordered(long long xb, long long yb) {
    const int ex = (int)(xb >> 52), ey = (int)(yb >> 52);
    if (ey > 0 && ex == ey) return scaled_to_float_fast((unsigned long long)(xb - yb), ex - 1075);
    if (ey > 0 && ex == ey + 1) {
        const unsigned long long mx = (unsigned long long)((xb & MANT52) | (1LL << 52));
        const unsigned long long my = (unsigned long long)((yb & MANT52) | (1LL << 52));
        return scaled_to_float_fast(2 * mx - my, ey - 1075);
    }
    return (float)dsub(dfrom(xb), dfrom(yb));
}

// x - y for x, y >= 0 (bit patterns order like the values).  A walk's first
// dt can be slightly negative: yt's rounded tmax may sit just below a
// snapped intersect_t.
YTGB_HD float diff_to_float(long long xb, long long yb) {
    return xb >= yb ? diff_to_float_ordered(xb, yb) : -diff_to_float_ordered(yb, xb);
}

// x - y as float in the cell loop: when both lie in one binade inside the
// scaled conversion's range (the loop's case: 2^-74 <= t < 2^74) and
// x >= y, the difference in ulps converted as scaled_to_float_fast does,
// with one test instead of diff_to_float's three; otherwise diff_to_float.
// The same value as diff_to_float.
YTGB_HD float diff_to_float_loop(long long xb, long long yb) {
    const unsigned xh = (unsigned)((unsigned long long)xb >> 32), yh = (unsigned)((unsigned long long)yb >> 32);
    const long long F = xb - yb;
    const unsigned ex = xh >> 20;  // the sign and exponent fields
    if ((xh ^ yh) < (1u << 20) && F >= 0 && ex - 949u <= 199u) {
        const unsigned hi = (unsigned)((unsigned long long)F >> 32), lo = (unsigned)F;
#ifdef __CUDA_ARCH__
        const float f = ffma(__uint2float_rn(hi), 4294967296.0f, __uint2float_rn(lo));
#else
        const float f = ffma((float)hi, 4294967296.0f, (float)lo);
#endif
        return fmul(f, ffrom((ex - 948u) << 23));  // 2^(ex - 1075)
    }
    return diff_to_float(xb, yb);
}

// floor(ty) and ty - floor(ty) (as float) for a positive normal ty < 2^30.
YTGB_HD void split_floor(long long tb, int &fl, float &frac) {
    const int e = (int)(tb >> 52) - 1023;
    const unsigned long long m = (unsigned long long)((tb & MANT52) | (1LL << 52));
    if (e < 0) {
        fl = 0;
        frac = scaled_to_float_fast(m, e - 52);
    } else {
        const int sh = 52 - e;
        fl = (int)(m >> sh);
        frac = scaled_to_float_fast(m & ((1ull << sh) - 1), -sh);
    }
}

// fl(x + d) with x, d > 0, repeated for one walk axis.  Inside one binade
// of x the float64 sum advances x by a fixed number q of ulps (plus one
// when the discarded part of d exceeds half an ulp; on an exact half, the
// even neighbour): an integer add on the bit pattern.  Anything else --
// leaving the binade, d not below x's binade, non-normal operands -- takes
// the float64 add.
struct AxisStep {
    long long bits;  // the float64 bits of tmax
    long long inc;   // ulps per add: q, plus one when the discarded part exceeds half an ulp
    int ex;          // the exponent field of bits: the binade
    int mode;        // 0 fixed increment, 2 exact half (to even), 3 float64 add
};

YTGB_HD void step_prepare(AxisStep &s, double d) {
    const long long xb = s.bits, db = dbits(d);
    const int ex = (int)(xb >> 52), ed = (int)(db >> 52);
    s.ex = ex;
    s.inc = 0;
    if (xb <= 0 || db <= 0 || ex == 0 || ed == 0 || ex >= 2046 || ed >= 2047 || ed >= ex) {
        s.mode = 3;
        return;
    }
    const int sh = ex - ed;
    s.mode = 0;
    if (sh >= 64) return;
    const unsigned long long md = (unsigned long long)((db & MANT52) | (1LL << 52));
    const long long q = (long long)(md >> sh);
    const unsigned long long r = md & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    s.inc = r > half ? q + 1 : q;
    if (r == half) s.mode = 2;
}

YTGB_HD void step_advance(AxisStep &s, double d) {
    if (s.mode != 3) {
        long long nb = s.bits + s.inc;
        if (s.mode == 2) nb += nb & 1;  // a tie: to the even neighbour
        if ((int)(nb >> 52) == s.ex) {
            s.bits = nb;
            return;
        }
    }
    s.bits = dbits(dadd(dfrom(s.bits), d));
    step_prepare(s, d);
}

struct Ray {
    double pos[3];
    double dir[3];
    double iv[3];
    float fpos[3], fdir[3];
    float ifd[3];     // 1 / fdir in float32, correctly rounded (the pre-tests)
    int step[3];
    // tdelta = step * iv_dir * dds (grid_traversal.pyx:86) for the dds of the
    // last brick walked (per axis): the bricks of one AMR level share their
    // dds bit for bit, so a ray's walks within a level reuse the product
    double td_dds[3], td[3];
};

// The view's derived per-view constants (host, before a launch): the
// perspective lens's linspace steps and normal * width[2], the same float64
// operations make_ray would repeat per pixel.
inline void view_derive(ytgb_view &v) {
    v.lin_step[0] = v.nx > 1 ? 1.0 / (double)(v.nx - 1) : 0.0;
    v.lin_step[1] = v.ny > 1 ? 1.0 / (double)(v.ny - 1) : 0.0;
    for (int i = 0; i < 3; i++) v.normal_w2[i] = v.vp_pos[9 + i] * v.vp_dir[2];
}

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
        // (lin_step and normal_w2: view_derive, once per view)
        const double px = (v.nx > 1 && vi == v.nx - 1) ? 0.5 : dadd(dmul((double)vi, v.lin_step[0]), -0.5);
        const double py = (v.ny > 1 && vj == v.ny - 1) ? 0.5 : dadd(dmul((double)vj, v.lin_step[1]), -0.5);
        YTGB_UNROLL
        for (int i = 0; i < 3; i++) {
            const double sx = dmul(v.vp_dir[0], dmul(v.vp_pos[3 + i], px));
            const double sy = dmul(v.vp_dir[1], dmul(v.vp_pos[6 + i], py));
            r.dir[i] = dmul(dadd(dadd(sx, sy), v.normal_w2[i]), v.ray_scale);
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
        r.ifd[i] = frcp(r.fdir[i]);  // = 1.0f / fdir, correctly rounded
        r.td_dds[i] = -1.0;          // no brick has a negative dds
        r.td[i] = 0.0;
    }
}

// tdelta of axis i for a brick with cell width dds: the ray's kept product
// when dds is the one it was formed with, else formed (and kept) now.
YTGB_HD double ray_tdelta(Ray &r, int i, double dds) {
    if (dbits(r.td_dds[i]) != dbits(dds)) {
        r.td_dds[i] = dds;
        r.td[i] = dmul(dmul((double)r.step[i], r.iv[i]), dds);
    }
    return r.td[i];
}

// Brick data for the float32 pre-tests (loaded for every candidate brick).
struct BrickF {
    float lef[3], ref[3], iddsf[3];
    int dims[3];
};

YTGB_HD void load_brick_f(const ytgb_brick *bp, BrickF &f) {
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        f.lef[i] = ldg(&bp->lef[i]);
        f.ref[i] = ldg(&bp->ref[i]);
        f.iddsf[i] = ldg(&bp->iddsf[i]);
        f.dims[i] = ldg(&bp->dims[i]);
    }
}

// Float32 slab test of the brick's box grown by a margin m (1e-4 of the
// coordinate scale, far above both the float32 error of these operations
// and walk_volume's 1e-10*dds face snapping).  True only when the ray misses
// the grown box for every t in [0, max_t]; then no face test of walk_volume
// can pass with intersect_t < max_t and the exact set-up returns 0.
YTGB_HD bool surely_misses(const BrickF &b, const Ray &r, const float ifd[3], float max_t) {
    float t0 = -1e30f, t1 = 1e30f;
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        const float lo = b.lef[i], hi = b.ref[i];
        const float m = 1e-4f * (fabsf(lo) + fabsf(hi) + fabsf(r.fpos[i]) + 1.0f);
        if (r.step[i] == 0) {
            if (r.fpos[i] < lo - m || r.fpos[i] > hi + m) return true;
        } else {
            float ta = (lo - m - r.fpos[i]) * ifd[i];
            float tb = (hi + m - r.fpos[i]) * ifd[i];
            if (ta > tb) {
                const float tmp = ta;
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
// reference returns 0 before its loop.  Every float64 value it keeps is
// computed from the same operands as the reference; float32 estimates only
// decide comparisons whose outcome they prove (their margins exceed their
// error bound by >= 80x), and the index and position of the entry point are
// read from the bits of the float64 coordinate.
YTGB_HD bool walk_setup(const BrickF &bf, const ytgb_brick *bp, const double *bounds, const Ray &r,
                        const float ifd[3], double max_t, long long kmax, Walk &w) {
    double le[3], re[3], idds[3];
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        le[i] = ldg(&bp->left_edge[i]);
        re[i] = ldg(&bp->right_edge[i]);
        idds[i] = ldg(&bp->idds[i]);
    }
    int direction = -1;
    double intersect_t = 1.1;
    long long kint = dkey(1.1);
    // inside test (:44-48), exact only when float32 cannot exclude it
    bool maybe_inside = true;
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        const float m = 1e-5f * (fabsf(bf.lef[i]) + fabsf(bf.ref[i]) + fabsf(r.fpos[i]) + 1e-3f);
        maybe_inside = maybe_inside && !(r.fpos[i] < bf.lef[i] - m) && !(r.fpos[i] > bf.ref[i] + m);
    }
    if (maybe_inside && le[0] <= r.pos[0] && r.pos[0] < re[0] && le[1] <= r.pos[1] && r.pos[1] < re[1] &&
        le[2] <= r.pos[2] && r.pos[2] < re[2]) {
        intersect_t = 0.0;
        kint = 0;
        direction = 3;
    }
    if (direction != 3) {
        YTGB_UNROLL
        for (int i = 0; i < 3; i++) {
            if (r.step[i] == 0) continue;
            const int x = (i + 1) % 3, y = (i + 2) % 3;
            // Float32 estimate of where the ray meets this face's plane.  The
            // error of q is at most ~6 float32 roundings of
            // (|e|+|p_i|)|d_x/d_i| + |tl d_x| + |p_x| (+ the edges' own
            // rounding); the margins are 1e-5 of that sum.  NaN or inf never
            // decides anything.
            const float e = r.step[i] > 0 ? bf.lef[i] : bf.ref[i];
            const float a0 = fabsf(e) + fabsf(r.fpos[i]);
            const float tlf = (e - r.fpos[i]) * ifd[i];
            const float qx = r.fpos[x] + tlf * r.fdir[x];
            const float qy = r.fpos[y] + tlf * r.fdir[y];
            const float sx = 1e-5f * (a0 * fabsf(r.fdir[x] * ifd[i]) + fabsf(tlf * r.fdir[x]) + fabsf(r.fpos[x]) +
                                      fabsf(bf.lef[x]) + fabsf(bf.ref[x]) + 1e-3f);
            const float sy = 1e-5f * (a0 * fabsf(r.fdir[y] * ifd[i]) + fabsf(tlf * r.fdir[y]) + fabsf(r.fpos[y]) +
                                      fabsf(bf.lef[y]) + fabsf(bf.ref[y]) + 1e-3f);
            const float st = 1e-5f * (a0 * fabsf(ifd[i]) + fabsf(tlf) + 1e-3f);
            if (qx < bf.lef[x] - sx || qx > bf.ref[x] + sx || qy < bf.lef[y] - sy || qy > bf.ref[y] + sy || tlf < -st)
                continue;  // clearly off the face: the exact test fails too
            const double tl = r.step[i] > 0 ? dmul(dsub(le[i], r.pos[i]), r.iv[i]) : dmul(dsub(re[i], r.pos[i]), r.iv[i]);
            const long long ktl = dkey(tl);
            // the reference's last clause, 0 <= tl < intersect_t, first
            if (!(ktl >= 0 && ktl < kint)) continue;
            // clearly inside the face: no snapping and the bounds test holds
            const bool clear = qx > bf.lef[x] + sx && qx < bf.ref[x] - sx && qy > bf.lef[y] + sy && qy < bf.ref[y] - sy;
            if (!clear) {
                double tx = dadd(r.pos[x], dmul(tl, r.dir[x]));
                double ty = dadd(r.pos[y], dmul(tl, r.dir[y]));
                const double ex = ldg(&bp->snap[x]), ey = ldg(&bp->snap[y]);
                if (fabs(dsub(tx, le[x])) < ex) tx = le[x];
                else if (fabs(dsub(tx, re[x])) < ex) tx = re[x];
                if (fabs(dsub(ty, le[y])) < ey) ty = le[y];
                else if (fabs(dsub(ty, re[y])) < ey) ty = re[y];
                if (!(le[x] <= tx && tx <= re[x] && le[y] <= ty && ty <= re[y])) continue;
            }
            direction = i;
            intersect_t = tl;
            kint = ktl;
        }
    }
    if (!(kint >= 0 && kint < kmax)) return false;  // !(0 <= intersect_t < max_t)
    const long long boff = ldg(&bp->bounds_offset);
    int aoff = 0;
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        const int dims = bf.dims[i];
        if (i == direction && r.step[i] > 0) {
            w.cur[i] = 0;
            w.P[i] = 0.0f;
        } else if (i == direction && r.step[i] < 0) {
            w.cur[i] = dims - 1;
            w.P[i] = 1.0f;
        } else {
            const double tx = dadd(dmul(intersect_t, r.dir[i]), r.pos[i]);
            const double ty = dmul(dsub(tx, le[i]), idds[i]);
            const long long tb = dbits(ty);
            if (tb > 0 && tb < 0x41d0000000000000LL) {
                // 0 < ty < 2^30: floor and fraction from the bits; yt's
                // clamp of (dims-1, dims) to dims-1 for negative steps does
                // not change the floor, and the sample position uses the
                // unclamped coordinate (its sampler recomputes dp from the
                // ray, image_samplers.pyx:475-478)
                split_floor(tb, w.cur[i], w.P[i]);
            } else {
                double tc = ty;
                if (-1 < ty && ty < 0 && r.step[i] > 0) tc = 0.0;
                else if (dims - 1 < ty && ty < dims && r.step[i] < 0) tc = (double)(dims - 1);
                w.cur[i] = (int)floor(tc);
                w.P[i] = (float)dsub(ty, (double)w.cur[i]);
            }
        }
        if (r.step[i] != 0) {
            // (cur+1)*dds + le or cur*dds + le (:105-108), from the table
            const int k = r.step[i] > 0 ? w.cur[i] + 1 : w.cur[i];
            const double bv = (k >= 0 && k <= dims) ? ldg(bounds + boff + aoff + k)
                                                    : dadd(dmul((double)k, ldg(&bp->dds[i])), le[i]);
            w.tmax[i] = dmul(dsub(bv, r.pos[i]), r.iv[i]);
        } else {
            w.tmax[i] = 1e60;
        }
        aoff += dims + 1;
    }
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        if (w.cur[i] == bf.dims[i] && r.step[i] >= 0) return false;
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

// One channel of FIT_eval_transfer_with_light (field_interpolation_tables.pxd:
// 115-143): x <- (1 - ta) e (1 + dot l) + ta x with ta = max(1 - d, 0) and
// d = dt e (dt (e0 + e1 + e2) with grey opacity), i.e. x + d (y - x) with
// y = e (1 + dot l) while d < 1, else y.
YTGB_HD void acc_light(float &h, float &l, float d, float y, bool comp) {
    if (d < 1.0f) {
        if (comp) {
            const float u = fsub(fsub(y, h), l);
            acc_add(h, l, fmul(d, u));
        } else {
            h = ffma(d, fsub(y, h), h);
        }
    } else {
        h = y;
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

// yt's float64 value of a field at sample s (of ns) in a cell
// (VolumeRenderSampler.sample, image_samplers.pyx:471-481, and
// offset_interpolate, fixed_interpolator.cpp:34-52), from the walk's exact
// enter/exit t, the ray, the brick's edges and cell widths, and the float64
// vertex values as their float32 parts plus float32 rounding errors
// (hi + lo is the float64 value to 2^-48).  Every operation is yt's, in
// yt's order.
YTGB_HD double yt_sample_value(const Ray &r, const ytgb_brick *bp, const float *__restrict__ hi,
                               const float *__restrict__ lo, int sy, int sx, const int cur[3], long long eb,
                               long long xb, int ns, int s) {
    const double en = dfrom(eb), ex = dfrom(xb);
    const double dt = ddiv(dsub(ex, en), (double)ns);
    double dp[3];
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        const double idds = ldg(&bp->idds[i]);
        dp[i] = dadd(dmul(dadd(en, dmul(0.5, dt)), r.dir[i]), r.pos[i]);
        dp[i] = dsub(dp[i], dadd(dmul((double)cur[i], ldg(&bp->dds[i])), ldg(&bp->left_edge[i])));
        dp[i] = dmul(dp[i], idds);
        const double ds = dmul(dmul(r.dir[i], idds), dt);
        for (int k = 0; k < s; k++) dp[i] = dadd(dp[i], ds);
    }
    double c[8];
    YTGB_UNROLL
    for (int q = 0; q < 8; q++) {
        const int o = ((q >> 2) & 1) * sx + ((q >> 1) & 1) * sy + (q & 1);
        c[q] = dadd((double)ldg(hi + o), (double)ldg(lo + o));
    }
    double dv = dsub(1.0, dp[2]);
    double v0 = dadd(dmul(dv, c[0]), dmul(dp[2], c[1]));
    double v1 = dadd(dmul(dv, c[2]), dmul(dp[2], c[3]));
    double v2 = dadd(dmul(dv, c[4]), dmul(dp[2], c[5]));
    double v3 = dadd(dmul(dv, c[6]), dmul(dp[2], c[7]));
    dv = dsub(1.0, dp[1]);
    v0 = dadd(dmul(dv, v0), dmul(dp[1], v1));
    v1 = dadd(dmul(dv, v2), dmul(dp[1], v3));
    dv = dsub(1.0, dp[0]);
    return dadd(dmul(dv, v0), dmul(dp[0], v1));
}

// FIT_get_value's range test in float64 (field_interpolation_tables.pxd:
// 66-80): 0 outside the open interval of the bounds and for non-normal values.
YTGB_HD bool fit_in_range64(double v, double b0, double b1) {
    if (!(v < b1) || !(v > b0)) return false;  // also NaN
    const long long e = (dbits(v) >> 52) & 0x7ff;
    return e != 0 && e != 0x7ff;  // isnormal: not zero, subnormal, inf or NaN
}

// FIT_get_value's float64 range decision for a sample (yt_sample_value of
// the field whose vertex values start at hi; lo: their rounding errors).
YTGB_HD bool range_in64(const Ray *r, const ytgb_brick *bp, const float *hi, const float *lo, int sy, int sx,
                             int c0, int c1, int c2, long long eb, long long xb, int ns, int s, double b0,
                             double b1) {
    const int cur[3] = {c0, c1, c2};
    return fit_in_range64(yt_sample_value(*r, bp, hi, lo, sy, sx, cur, eb, xb, ns, s), b0, b1);
}

// The range decision's tolerance for a walk of at most `steps` cells:
// twice the float32 error bound of a sample value.  With M >= every |value|
// (eps = M 2^-24) the value's error against yt's float64 one is at most
//   2^-24 M (the float32 vertex values) + 16 eps (the seven interpolation
//   roundings and their differences) + 3 * 2M * dx,
// dx being the cell-coordinate error: <= (steps / 2 + 4) 2^-24, from the
// float32 entry point, dt and velocity and one half-ulp ffma rounding per
// step since the axis last snapped to a face (advance_position).  Hence
// 41 + 6 steps, doubled.
YTGB_HD float range_tol(float eps, int steps) { return fmul(eps, (float)(96 + 16 * steps)); }

// Whether FIT_get_value's float64 range test (field_interpolation_tables.pxd:
// 72-73) could decide a sample differently from the float32 test on its
// float32 value v: v within tol of a bound, or v exactly 0 (yt's isnormal
// test; a float64 value that is exactly 0 where v is not needs an exact
// float64 cancellation that float32 does not reproduce).
YTGB_HD bool range_ambiguous(float v, float tol, float lo, float hi) {
    return v == 0.0f || fabsf(fsub(v, lo)) <= tol || fabsf(fsub(v, hi)) <= tol;
}

// eval_gradient (fixed_interpolator.cpp:116-148) of the trilinear
// interpolant in cell coordinates, normalised to -grad/|grad| (0 when the
// gradient vanishes).  The reference takes finite differences 0.05 apart
// (one-sided within 0.05 of a face); the interpolant is linear along each
// axis, so every such difference is the exact partial derivative, which is
// formed here directly from the corner differences.  The differences use
// the values' float32 low parts when given (lo != nullptr): the data's
// float32 rounding would otherwise dominate the differences of smooth
// fields.  Where the field is exactly flat the reference normalises its
// rounding noise into an arbitrary direction; here the gradient is 0.  A
// NaN corner (log10 of a non-positive vertex value) makes the gradient NaN.
YTGB_HD void light_gradient(const float *__restrict__ p, const float *__restrict__ lo, int sy, int sx, float dx,
                            float dy, float dz, float g[3]) {
    float c[8], e[8];
    YTGB_UNROLL
    for (int q = 0; q < 8; q++) {
        const int o = ((q >> 2) & 1) * sx + ((q >> 1) & 1) * sy + (q & 1);
        c[q] = ldg(p + o);
        e[q] = lo ? ldg(lo + o) : 0.0f;
    }
    // corner q = 4a + 2b + c at offsets a (x), b (y), c (z)
#define YTGB_D(u, v) fadd(fsub(c[u], c[v]), fsub(e[u], e[v]))
    const float x00 = YTGB_D(4, 0), x01 = YTGB_D(5, 1), x10 = YTGB_D(6, 2), x11 = YTGB_D(7, 3);
    const float y00 = YTGB_D(2, 0), y01 = YTGB_D(3, 1), y10 = YTGB_D(6, 4), y11 = YTGB_D(7, 5);
    const float z00 = YTGB_D(1, 0), z01 = YTGB_D(3, 2), z10 = YTGB_D(5, 4), z11 = YTGB_D(7, 6);
#undef YTGB_D
    const float gx = ffma(dy, fsub(ffma(dz, fsub(x11, x10), x10), ffma(dz, fsub(x01, x00), x00)),
                          ffma(dz, fsub(x01, x00), x00));
    const float gy = ffma(dx, fsub(ffma(dz, fsub(y11, y10), y10), ffma(dz, fsub(y01, y00), y00)),
                          ffma(dz, fsub(y01, y00), y00));
    const float gz = ffma(dx, fsub(ffma(dy, fsub(z11, z10), z10), ffma(dy, fsub(z01, z00), z00)),
                          ffma(dy, fsub(z01, z00), z00));
    const float n2 = ffma(gz, gz, ffma(gy, gy, fmul(gx, gx)));
    if (n2 > 0.0f && finitef(n2)) {
        const float inv = fdiv(-1.0f, sqrtf(n2));
        g[0] = fmul(gx, inv);
        g[1] = fmul(gy, inv);
        g[2] = fmul(gz, inv);
    } else if (n2 == 0.0f) {
        g[0] = g[1] = g[2] = 0.0f;
    } else {
        // a NaN (or infinite) corner: the reference's gradient is NaN, and so
        // is every channel it composites (0 * NaN), as here
        g[0] = g[1] = g[2] = __builtin_nanf("");
    }
}

// One bin of the packed ColorTransferFunction tables: the four tables' y and
// dy, and the bin's d0 as a float pair.  TG false: the block's shared-memory
// copy, repacked as three float4 per bin (y[4], dy[4], d0); TG true: the
// tables where ytgb_tf_pack left them in global memory, one float4
// {y, dy, d0_hi, d0_lo} per table and bin (four cached loads).
template <bool TG>
YTGB_HD void ctf_bin(const float4 *__restrict__ tab, int nbins, int bin, float4 &Y, float4 &D, float2 &Z) {
    if (TG) {
        const float4 t0 = ldg(tab + bin), t1 = ldg(tab + nbins + bin);
        const float4 t2 = ldg(tab + 2 * nbins + bin), t3 = ldg(tab + 3 * nbins + bin);
        Y = make_float4(t0.x, t1.x, t2.x, t3.x);
        D = make_float4(t0.y, t1.y, t2.y, t3.y);
        Z = make_float2(t3.z, t3.w);
    } else {
        Y = tab[3 * bin + 0];
        D = tab[3 * bin + 1];
        const float4 z = tab[3 * bin + 2];
        Z = make_float2(z.x, z.y);
    }
}

// FIT_get_value + FIT_eval_transfer's table combination
// (field_interpolation_tables.pxd:66-101).  The bounds test uses the float
// nearest outside each bound, so for a float v it decides exactly as the
// float64 test would for that v.  Zero, infinite and NaN values give 0 like
// the reference's !isnormal test.
YTGB_HD void tf_eval(const ytgb_tf &tf, const float4 *__restrict__ tab, const float dvs[6],
                                        float trgba[6], unsigned force = 0u, unsigned force_in = 0u) {
    float ist[6];
    YTGB_UNROLL
    for (int t = 0; t < 6; t++) {
        ist[t] = 0.0f;
        if (t < tf.n_fits) {
            float v = pick6(dvs, tf.field_id[t]);
            // (force: table t's range decision taken from bit t of force_in)
            const bool in = (force >> t) & 1u ? ((force_in >> t) & 1u) != 0u
                                              : !(v >= tf.hi_excl[t] || v <= tf.lo_excl[t]) && v != 0.0f &&
                                                    finitef(v);
            if (in) {
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
    unsigned visits, walks, guarded;  // per ray (summed into 64-bit counters)
    double max_t;  // (its key dkey(max_t) is recomputed per walk)
    float max_tf;
    bool comp;
};

YTGB_HD void ray_state_init(RayState &s, const double *img, double zbuf, bool has_zbuf, uint32_t flags) {
    double max_t = has_zbuf ? zbuf : 1.0;
    max_t = max_t > 0.0 ? max_t : 0.0;  // fclip(z, 0, 1) (image_samplers.pyx:185)
    max_t = max_t < 1.0 ? max_t : 1.0;  // also grid_traversal.pyx:42
    s.max_t = max_t;
    s.max_tf = (float)max_t;
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
    s.comp = !(flags & YTGB_FLAG_NO_COMPENSATION);
}

// The sampler callback for one visited cell: VolumeRenderSampler.sample
// (image_samplers.pyx:453-487), ProjectionSampler.sample (:330-343),
// InterpolatedProjectionSampler.sample (:372-403), the MIP sampler, or the
// traversal trace.  P is the cell-local entry point, vel the cell-local
// velocity, dtf = exit_t - enter_t.
struct CellCtx {
    const float *base;
    long long fstride, moff;
    int nf, sx, sy;
    int dims[3];
    float vel[3];
    // the float64 range decision (range_ambiguous): its tolerance, < 0 for
    // float32 decisions only, and the ray and brick it recomputes from
    float tol;
    const Ray *ray;
    const ytgb_brick *bp;
};

// The sampler variant, a template parameter (VAR) of the volume-rendering
// and light-source paths: bit V_CTF, the ColorTransferFunction layout
// (ctf_bin); bit V_REF, range decisions near a bound made in float64 from
// data + data_lo (range_ambiguous, set where the launch carries data_lo and
// range_eps > 0).
constexpr int V_CTF = 1;
constexpr int V_REF = 2;

// The variant a render's arguments call for: float64 range decisions where
// the arena's rounding errors and their scale are given, except for a
// ColorTransferFunction whose table excludes every value (nothing is in
// range either way).
inline int render_variant(const ytgb_render_args &a) {
    int v = 0;
    if (a.kind == YTGB_VOLUME_RENDER && a.tf.ctf_fast) v |= V_CTF;
    if ((a.kind == YTGB_VOLUME_RENDER || a.kind == YTGB_LIGHT_SOURCE) && a.data_lo && a.range_eps > 0.0f &&
        (!(v & V_CTF) || a.tf.lo_excl[0] <= a.tf.hi_excl[0]))
        v |= V_REF;
    return v;
}

// The tables of a general transfer function whose range decision for the
// field values dvs is made in float64 (range_ambiguous): bit t of force, and
// of force_in where yt's float64 value lies inside table t's range.
YTGB_HD void range_decisions(const ytgb_render_args &a, const CellCtx &c, const float dvs[6], int off,
                             const int cur[3], long long eb, long long xb, int ns, int s, unsigned &force,
                             unsigned &force_in) {
    force = 0u;
    force_in = 0u;
    if (c.tol < 0.0f) return;
    const ytgb_tf &tf = a.tf;
    for (int t = 0; t < tf.n_fits; t++) {
        const int f = tf.field_id[t];
        if (f >= c.nf || !(tf.lo_excl[t] <= tf.hi_excl[t])) continue;
        if (!range_ambiguous(pick6(dvs, f), c.tol, tf.lo_excl[t], tf.hi_excl[t])) continue;
        const float *hi = c.base + f * c.fstride + off;
        force |= 1u << t;
        if (range_in64(c.ray, c.bp, hi, a.data_lo + (hi - a.data), c.sy, c.sx, cur[0], cur[1], cur[2], eb, xb, ns, s,
                       tf.bound64[t][0], tf.bound64[t][1]))
            force_in |= 1u << t;
    }
}

// The sample position inside the cell, kept in [0, 1] (CLAMP: the walk's
// cells contain the ray, so only float32 rounding can step outside) or
// extrapolated as the reference does (the octree path, whose traversal can
// hand the sampler cells the ray only grazes, with exit_t < enter_t).
template <bool CLAMP>
YTGB_HD float cell_coord(float x) {
    return CLAMP ? fminf(fmaxf(x, 0.0f), 1.0f) : x;
}

template <int MODE, int VAR, bool CLAMP = true, bool TG = false>
YTGB_HD void sample_cell(const ytgb_render_args &a, const float4 *s_tab, int bi, const CellCtx &c, const int cur[3],
                         const float P[3], float dtf, long long enter_bits, long long exit_bits, RayState &st) {
    st.visits++;
    if (MODE == MODE_TRACE) {
        st.th = fnv_mix(st.th, (unsigned long long)(unsigned)bi);
        st.th = fnv_mix(st.th, (unsigned long long)(unsigned)cur[0] | ((unsigned long long)(unsigned)cur[1] << 32));
        st.th = fnv_mix(st.th, (unsigned long long)(unsigned)cur[2]);
        st.th = fnv_mix(st.th, (unsigned long long)enter_bits);
        st.th = fnv_mix(st.th, (unsigned long long)exit_bits);
        st.tcount++;
        return;
    }
    const bool inside = (unsigned)cur[0] < (unsigned)c.dims[0] && (unsigned)cur[1] < (unsigned)c.dims[1] &&
                        (unsigned)cur[2] < (unsigned)c.dims[2];
    if (!inside) {
        // yt hands its sampler this index and reads outside the brick; here
        // the cell contributes nothing and is counted
        st.guarded++;
        return;
    }
    float *xh = st.xh, *xl = st.xl;
    const bool comp = st.comp;
    if (MODE == MODE_LIGHT) {
        // LightSourceRenderSampler.sample (image_samplers.pyx:551-590): no
        // mask test; all fields interpolated, the gradient of field 0
        const int off = cur[0] * c.sx + cur[1] * c.sy + cur[2];
        const int ns = a.n_samples;
        const float dts = ns == 1 ? dtf : fdiv(dtf, (float)ns);
        const float *lo = a.data_lo ? a.data_lo + (c.base - a.data) + off : nullptr;
        for (int s = 0; s < ns; s++) {
            const float f = fmul(dts, (float)s + 0.5f);
            const float fx = cell_coord<CLAMP>(ffma(f, c.vel[0], P[0]));
            const float fy = cell_coord<CLAMP>(ffma(f, c.vel[1], P[1]));
            const float fz = cell_coord<CLAMP>(ffma(f, c.vel[2], P[2]));
            float dvs[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            YTGB_UNROLL
            for (int fi = 0; fi < 6; fi++)
                if (fi < c.nf) dvs[fi] = trilinear(c.base + fi * c.fstride + off, c.sy, c.sx, fx, fy, fz);
            float g[3];
            light_gradient(c.base + off, lo, c.sy, c.sx, fx, fy, fz, g);
            const float dot = ffma(a.light_dir[2], g[2], ffma(a.light_dir[1], g[1], fmul(a.light_dir[0], g[0])));
            float trgba[6];
            unsigned force = 0u, force_in = 0u;
            if (VAR & V_REF) range_decisions(a, c, dvs, off, cur, enter_bits, exit_bits, ns, s, force, force_in);
            tf_eval(a.tf, s_tab, dvs, trgba, force, force_in);
            if (a.tf.grey_opacity == 1) {
                const float d = fmul(dts, fadd(fadd(trgba[0], trgba[1]), trgba[2]));
                YTGB_UNROLL
                for (int ch = 0; ch < 3; ch++)
                    acc_light(xh[ch], xl[ch], d, fmul(trgba[ch], ffma(dot, a.light_rgba[ch], 1.0f)), comp);
            } else {
                YTGB_UNROLL
                for (int ch = 0; ch < 3; ch++)
                    acc_light(xh[ch], xl[ch], fmul(dts, trgba[ch]),
                              fmul(trgba[ch], ffma(dot, a.light_rgba[ch], 1.0f)), comp);
            }
            st.touched |= 0x7u;
        }
        return;
    }
    if (MODE == MODE_PROJ || MODE == MODE_MIP) {
        const int di = (cur[0] * c.dims[1] + cur[1]) * c.dims[2] + cur[2];
        const int nch = c.nf < 4 ? c.nf : 4;
        YTGB_UNROLL
        for (int ch = 0; ch < 4; ch++) {
            if (ch < nch) {
                const float val = ldg(c.base + ch * c.fstride + di);
                if (MODE == MODE_PROJ) {
                    const float inc = fmul(val, dtf);
                    if (comp) acc_add(xh[ch], xl[ch], inc);
                    else xh[ch] = fadd(xh[ch], inc);
                } else if (val > xh[ch]) {
                    xh[ch] = val;
                    xl[ch] = 0.0f;
                }
                st.touched |= 1u << ch;
            }
        }
        return;
    }
    const int cell = (cur[0] * c.dims[1] + cur[1]) * c.dims[2] + cur[2];
    if (MODE == MODE_VR && c.moff >= 0 && a.masks && ldg(a.masks + c.moff + cell) != 1) return;
    const int off = cur[0] * c.sx + cur[1] * c.sy + cur[2];
    const int ns = a.n_samples;
    const float dts = ns == 1 ? dtf : fdiv(dtf, (float)ns);
    for (int s = 0; s < ns; s++) {
        // sample s at enter_t + (s + 1/2) dt (image_samplers.pyx:475-487)
        const float f = fmul(dts, (float)s + 0.5f);
        const float fx = cell_coord<CLAMP>(ffma(f, c.vel[0], P[0]));
        const float fy = cell_coord<CLAMP>(ffma(f, c.vel[1], P[1]));
        const float fz = cell_coord<CLAMP>(ffma(f, c.vel[2], P[2]));
        if (MODE == MODE_VR && (VAR & V_CTF)) {
            const float val = trilinear(c.base + off, c.sy, c.sx, fx, fy, fz);
            const ytgb_tf &tf = a.tf;
            bool in = !(val >= tf.hi_excl[0] || val <= tf.lo_excl[0]) && val != 0.0f && finitef(val);
            if ((VAR & V_REF) && c.tol >= 0.0f && range_ambiguous(val, c.tol, tf.lo_excl[0], tf.hi_excl[0])) {
                // decide as yt does, from the float64 value (rare)
                in = range_in64(c.ray, c.bp, c.base + off, a.data_lo + (c.base - a.data) + off, c.sy, c.sx, cur[0],
                                cur[1], cur[2], enter_bits, exit_bits, ns, s, tf.bound64[0][0], tf.bound64[0][1]);
            }
            // outside the table's range: zero emission and absorption leave x
            // unchanged
            if (in) {
                float q = fmul(fsub(val, tf.b0[0]), tf.idbin[0]);
                q = fminf(fmaxf(q, 0.0f), (float)(tf.nbins[0] - 2));
                const int bin = (int)q;
                float4 Y, D;
                float2 Z;
                ctf_bin<TG>(s_tab, tf.nbins_max, bin, Y, D, Z);
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
        } else if (MODE == MODE_IPROJ) {
            // InterpolatedProjectionSampler.sample (image_samplers.pyx:372-403):
            // rgba[j] += v_j * dt for j < min(3, n_fields); the fields past
            // the third are never read
            const int n3 = c.nf < 3 ? c.nf : 3;
            YTGB_UNROLL
            for (int ch = 0; ch < 3; ch++) {
                if (ch < n3) {
                    const float v = trilinear(c.base + ch * c.fstride + off, c.sy, c.sx, fx, fy, fz);
                    const float inc = fmul(v, dts);
                    if (comp) acc_add(xh[ch], xl[ch], inc);
                    else xh[ch] = fadd(xh[ch], inc);
                    st.touched |= 1u << ch;
                }
            }
        } else {
            float dvs[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            YTGB_UNROLL
            for (int fi = 0; fi < 6; fi++)
                if (fi < c.nf) dvs[fi] = trilinear(c.base + fi * c.fstride + off, c.sy, c.sx, fx, fy, fz);
            if (MODE == MODE_VR) {
                float trgba[6];
                unsigned force = 0u, force_in = 0u;
                if (VAR & V_REF)
                    range_decisions(a, c, dvs, off, cur, enter_bits, exit_bits, ns, s, force, force_in);
                tf_eval(a.tf, s_tab, dvs, trgba, force, force_in);
                if (a.tf.grey_opacity == 1) {
                    const float da = fmul(dts, trgba[3]);
                    YTGB_UNROLL
                    for (int ch = 0; ch < 4; ch++) acc_grey(xh[ch], xl[ch], dts, trgba[ch], da, comp);
                    st.touched |= 0xfu;
                } else {
                    YTGB_UNROLL
                    for (int ch = 0; ch < 3; ch++) acc_emit(xh[ch], xl[ch], fmul(dts, trgba[ch]), comp);
                    st.touched |= 0x7u;
                }
            } else {
                const int n3 = c.nf < 3 ? c.nf : 3;
                YTGB_UNROLL
                for (int ch = 0; ch < 3; ch++) {
                    if (ch < n3) {
                        const float inc = fmul(dvs[ch], dts);
                        if (comp) acc_add(xh[ch], xl[ch], inc);
                        else xh[ch] = fadd(xh[ch], inc);
                        st.touched |= 1u << ch;
                    }
                }
            }
        }
    }
}

// The float32 geometry of one step: move P to the exit point, then put the
// stepped axis exactly on the next cell's entry face.
YTGB_HD void advance_position(float P[3], const float vel[3], float dtf, int i, int step_i) {
    YTGB_UNROLL
    for (int q = 0; q < 3; q++) P[q] = ffma(dtf, vel[q], P[q]);
    const float wrap = step_i > 0 ? 0.0f : 1.0f;
    if (i == 0) P[0] = wrap;
    else if (i == 1) P[1] = wrap;
    else P[2] = wrap;
}

// Non-grey channel update of FIT_eval_transfer as selects (acc_emit without
// its branch): d = 0 leaves the value unchanged.
template <bool COMP>
YTGB_HD void emit_sel(float &h, float &l, float d) {
    float hh = h, ll = l;
    if (COMP) {
        const float u = fsub(fsub(1.0f, h), l);
        acc_add(hh, ll, fmul(d, u));
    } else {
        hh = ffma(fsub(1.0f, d), h, d);
    }
    const bool small = d < 1.0f;
    h = small ? hh : d;
    l = small ? ll : 0.0f;
}

// Projection / interpolated-projection accumulation: x += inc.
template <bool COMP>
YTGB_HD void add_sel(float &h, float &l, float inc) {
    if (COMP) acc_add(h, l, inc);
    else h = fadd(h, inc);
}

// The cell loop of one walk for the common case: integer stepping (every
// walk value positive and finite), one sample per cell, no mask, every
// index of the entry cell inside the brick.  It visits the same cells with
// the same enter/exit t and forms the same sample values and image updates
// as sample_cell, operation for operation; what differs is the control
// flow.  The choice of axis, the tmax update and the transfer function's
// range test are selects, so one cell's body is a nearly straight run of
// instructions in which the integer traversal and the float32 sampling can
// be interleaved; only the exponent cases of the dt conversion and the rare
// cases (tmax leaving its binade, a step count past the bound) branch.  Every entry index inside the brick stays
// inside until the walk leaves it (an index changes only by a step on its
// own axis, after which the exit test runs).
// NCH: the channels the projection samplers write, when the launch fixes
// it (1: one field, the common case); 0 reads it from the brick.  A runtime
// channel count leaves every channel's instructions in the loop, predicated
// off but still issued (one field: the projection 24 % and the MIP 27 %
// faster with NCH = 1).  GREY: grey_opacity fixed (0 or 1) or read (-1).
template <int MODE, int VAR, bool COMP, bool TG, int NCH = 0, int GREY = -1>
YTGB_HD void cells_fast(const ytgb_render_args &a, const float4 *s_tab, Ray &r, const ytgb_brick *bp,
                        const CellCtx &c, const Walk &w, long long kmax, int step_limit, RayState &st) {
    AxisStep A0, A1, A2;
    A0.bits = dbits(w.tmax[0]);
    A1.bits = dbits(w.tmax[1]);
    A2.bits = dbits(w.tmax[2]);
    {
        // tdelta = step * iv_dir * dds (grid_traversal.pyx:86)
        const double t0 = ray_tdelta(r, 0, ldg(&bp->dds[0]));
        const double t1 = ray_tdelta(r, 1, ldg(&bp->dds[1]));
        const double t2 = ray_tdelta(r, 2, ldg(&bp->dds[2]));
        step_prepare(A0, t0);
        step_prepare(A1, t1);
        step_prepare(A2, t2);
    }
    long long eb = dbits(w.enter_t);
    float P0 = w.P[0], P1 = w.P[1], P2 = w.P[2];
    int c0 = w.cur[0], c1 = w.cur[1], c2 = w.cur[2];
    const float v0 = c.vel[0], v1 = c.vel[1], v2 = c.vel[2];
    const float wr0 = r.step[0] > 0 ? 0.0f : 1.0f, wr1 = r.step[1] > 0 ? 0.0f : 1.0f,
                wr2 = r.step[2] > 0 ? 0.0f : 1.0f;
    const ytgb_tf &tf = a.tf;
    const float nbm2 = (float)(tf.nbins[0] - 2);
    const bool grey = GREY >= 0 ? GREY == 1 : tf.grey_opacity == 1;
    // The cell-value samplers (projection, MIP) run integer-pipe bound: for
    // them the step bound is tested with the exit test, a tie in the tmax
    // step takes the float64 add, and the exit test checks all three indices
    // instead of selecting the stepped one (7-12 % faster there; the
    // interpolating samplers measured slower with it).
    constexpr bool CELLS = MODE == MODE_PROJ || MODE == MODE_MIP;
    unsigned nv = 0;
    while (true) {
        if (!CELLS && nv >= (unsigned)step_limit) {
            set_error(a.error, YTGB_DEVERR_STEP_LIMIT);
            break;
        }
        nv++;
        // the axis of the smallest tmax, strict < ties (grid_traversal.pyx:122-131)
        const bool lt01 = A0.bits < A1.bits, lt02 = A0.bits < A2.bits, lt12 = A1.bits < A2.bits;
        const bool s0 = lt01 && lt02;
        const bool s1 = !lt01 && lt12;
        const bool s2 = !s0 && !s1;
        const long long tmb = s0 ? A0.bits : (s1 ? A1.bits : A2.bits);
        const long long xb = tmb < kmax ? tmb : kmax;  // fmin(tmax[i], max_t)
        const float dtf = diff_to_float_loop(xb, eb);
        // the sample at the middle of the cell's segment (n_samples = 1)
        const float f = fmul(dtf, 0.5f);
        const float fx = cell_coord<true>(ffma(f, v0, P0));
        const float fy = cell_coord<true>(ffma(f, v1, P1));
        const float fz = cell_coord<true>(ffma(f, v2, P2));
        const int off = c0 * c.sx + c1 * c.sy + c2;
        if (MODE == MODE_VR && (VAR & V_CTF)) {
            const float val = trilinear(c.base + off, c.sy, c.sx, fx, fy, fz);
            // (NaN and infinities fail the strict bound tests, so they need no separate test)
            bool in = val < tf.hi_excl[0] && val > tf.lo_excl[0] && val != 0.0f;
            if ((VAR & V_REF) && range_ambiguous(val, c.tol, tf.lo_excl[0], tf.hi_excl[0])) {
                // decide as yt does, from the float64 value (rare)
                in = range_in64(&r, bp, c.base + off, a.data_lo + (c.base - a.data) + off, c.sy, c.sx, c0, c1, c2, eb,
                                xb, 1, 0, tf.bound64[0][0], tf.bound64[0][1]);
            }
            float q = fmul(fsub(val, tf.b0[0]), tf.idbin[0]);
            q = fminf(fmaxf(q, 0.0f), nbm2);  // a NaN q gives bin 0 (the sample is then out of range)
            const int bin = (int)q;
            float4 Y, D;
            float2 Z;
            ctf_bin<TG>(s_tab, tf.nbins_max, bin, Y, D, Z);
            const float dd = fsub(fsub(val, Z.x), Z.y);
            const float al = ffma(dd, D.w, Y.w);
            const float er = fmul(ffma(dd, D.x, Y.x), al);
            const float eg = fmul(ffma(dd, D.y, Y.y), al);
            const float eb_ = fmul(ffma(dd, D.z, Y.z), al);
            if (grey) {
                float h[4] = {st.xh[0], st.xh[1], st.xh[2], st.xh[3]};
                float l[4] = {st.xl[0], st.xl[1], st.xl[2], st.xl[3]};
                const float da = fmul(dtf, al);
                acc_grey(h[0], l[0], dtf, er, da, COMP);
                acc_grey(h[1], l[1], dtf, eg, da, COMP);
                acc_grey(h[2], l[2], dtf, eb_, da, COMP);
                acc_grey(h[3], l[3], dtf, al, da, COMP);
                YTGB_UNROLL
                for (int ch = 0; ch < 4; ch++) {
                    st.xh[ch] = in ? h[ch] : st.xh[ch];
                    st.xl[ch] = in ? l[ch] : st.xl[ch];
                }
            } else {
                emit_sel<COMP>(st.xh[0], st.xl[0], in ? fmul(dtf, er) : 0.0f);
                emit_sel<COMP>(st.xh[1], st.xl[1], in ? fmul(dtf, eg) : 0.0f);
                emit_sel<COMP>(st.xh[2], st.xl[2], in ? fmul(dtf, eb_) : 0.0f);
            }
        } else if (MODE == MODE_IPROJ) {
            const int n3 = NCH ? NCH : (c.nf < 3 ? c.nf : 3);
            YTGB_UNROLL
            for (int ch = 0; ch < 3; ch++)
                if (ch < n3)
                    add_sel<COMP>(st.xh[ch], st.xl[ch],
                                  fmul(trilinear(c.base + ch * c.fstride + off, c.sy, c.sx, fx, fy, fz), dtf));
        } else if (MODE == MODE_PROJ || MODE == MODE_MIP) {
            const int di = (c0 * c.dims[1] + c1) * c.dims[2] + c2;
            const int nch = NCH ? NCH : (c.nf < 4 ? c.nf : 4);
            YTGB_UNROLL
            for (int ch = 0; ch < 4; ch++) {
                if (ch < nch) {
                    const float val = ldg(c.base + ch * c.fstride + di);
                    if (MODE == MODE_PROJ) {
                        add_sel<COMP>(st.xh[ch], st.xl[ch], fmul(val, dtf));
                    } else {
                        const bool up = val > st.xh[ch];
                        st.xh[ch] = up ? val : st.xh[ch];
                        st.xl[ch] = up ? 0.0f : st.xl[ch];
                    }
                }
            }
        }
        // advance (grid_traversal.pyx:134-138): the position to the exit
        // point, the stepped axis onto the next cell's entry face
        P0 = s0 ? wr0 : ffma(dtf, v0, P0);
        P1 = s1 ? wr1 : ffma(dtf, v1, P1);
        P2 = s2 ? wr2 : ffma(dtf, v2, P2);
        c0 += s0 ? r.step[0] : 0;
        c1 += s1 ? r.step[1] : 0;
        c2 += s2 ? r.step[2] : 0;
        const long long inc = s0 ? A0.inc : (s1 ? A1.inc : A2.inc);
        const int md = s0 ? A0.mode : (s1 ? A1.mode : A2.mode);
        const int ex = s0 ? A0.ex : (s1 ? A1.ex : A2.ex);
        long long nb = tmb + inc;
        if (!CELLS && md == 2) nb += nb & 1;  // a tie: to the even neighbour
        A0.bits = s0 ? nb : A0.bits;
        A1.bits = s1 ? nb : A1.bits;
        A2.bits = s2 ? nb : A2.bits;
        if ((CELLS ? md >= 2 : md == 3) || (int)(nb >> 52) != ex) {
            // tmax leaves its binade, or has no integer step (or, CELLS, its
            // step rounds a tie to even): the float64 add
            // (the ray is in shared memory: a runtime index costs no local memory)
            const int i = s0 ? 0 : (s1 ? 1 : 2);
            const double td = r.td[i];  // (kept by the prologue for this brick)
            const long long sb = dbits(dadd(dfrom(tmb), td));
            if (s0) {
                A0.bits = sb;
                step_prepare(A0, td);
            } else if (s1) {
                A1.bits = sb;
                step_prepare(A1, td);
            } else {
                A2.bits = sb;
                step_prepare(A2, td);
            }
        }
        eb = tmb;
        if (CELLS) {
            // the stepped index left the brick (the others did not change), or
            // enter_t >= max_t; or the walk's step bound was reached
            const bool out = (unsigned)c0 >= (unsigned)c.dims[0] || (unsigned)c1 >= (unsigned)c.dims[1] ||
                             (unsigned)c2 >= (unsigned)c.dims[2] || !(tmb < kmax);
            if (out || nv >= (unsigned)step_limit) {
                if (!out) set_error(a.error, YTGB_DEVERR_STEP_LIMIT);
                break;
            }
        } else {
            const int ci = s0 ? c0 : (s1 ? c1 : c2);
            const int dci = s0 ? c.dims[0] : (s1 ? c.dims[1] : c.dims[2]);
            if ((unsigned)ci >= (unsigned)dci || !(tmb < kmax)) break;  // ... or enter_t >= max_t
        }
    }
    st.visits += nv;
    if (nv) {
        if (MODE == MODE_VR) st.touched |= a.tf.grey_opacity == 1 ? 0xfu : 0x7u;
        else if (MODE == MODE_IPROJ) st.touched |= (1u << (c.nf < 3 ? c.nf : 3)) - 1u;
        else st.touched |= (1u << (c.nf < 4 ? c.nf : 4)) - 1u;
    }
}

// One brick of one ray: cast_through_kdtree's walk_volume call
// (image_samplers.pyx:186) with the sampler callback inlined.
// s_tab: the transfer-function tables -- as staged in shared memory (TG
// false) or as packed in global memory (TG true, see ctf_bin); bi: the brick
// index.
template <int MODE, int VAR, bool TG = false>
YTGB_HD void walk_brick(const ytgb_render_args &a, const float4 *s_tab, Ray &r, int bi, RayState &st) {
    const ytgb_brick *bp = a.bricks + bi;
    BrickF bf;
    load_brick_f(bp, bf);
    // r.ifd: 1 / v_dir in float32 for the float32 pre-tests (a product with it
    // is within two float32 roundings of the quotient; their margins are 1e-5
    // and 1e-4 of the operands' scale)
    const float ifd[3] = {r.ifd[0], r.ifd[1], r.ifd[2]};
    if (surely_misses(bf, r, ifd, st.max_tf)) return;
    const double max_t = st.max_t;
    const long long kmax = dkey(st.max_t);
    Walk w;
    if (!walk_setup(bf, bp, a.bounds, r, ifd, max_t, kmax, w)) return;
    st.walks++;
    CellCtx c;
    c.nf = ldg(&bp->n_fields);
    c.base = a.data + ldg(&bp->data_offset);
    c.fstride = ldg(&bp->field_stride);
    c.moff = ldg(&bp->mask_offset);
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        c.dims[i] = bf.dims[i];
        c.vel[i] = fmul(r.fdir[i], bf.iddsf[i]);
    }
    c.sy = bf.dims[2] + 1;
    c.sx = (bf.dims[1] + 1) * (bf.dims[2] + 1);
    const int step_limit = bf.dims[0] + bf.dims[1] + bf.dims[2] + 3;
    // samples near a transfer-function bound are decided in float64 where the
    // arena carries its float32 rounding errors
    // (the launch takes the V_REF variant only with data_lo and range_eps > 0,
    // and for a ColorTransferFunction only when its table is not the
    // exclude-everything form of out-of-range bounds)
    c.tol = (VAR & V_REF) ? range_tol(a.range_eps, step_limit) : -1.0f;
    c.ray = &r;
    c.bp = bp;
    int hitc = 0;
    const long long b0 = dbits(w.tmax[0]), b1 = dbits(w.tmax[1]), b2 = dbits(w.tmax[2]);
    const long long INF = 0x7ff0000000000000LL;
    const bool int_path = b0 > 0 && b1 > 0 && b2 > 0 && b0 < INF && b1 < INF && b2 < INF && kmax > 0;
    if (MODE != MODE_TRACE && MODE != MODE_LIGHT && (MODE != MODE_VR || (VAR & V_CTF)) && int_path && a.n_samples == 1 &&
        (MODE != MODE_VR || c.moff < 0 || !a.masks) && (unsigned)w.cur[0] < (unsigned)c.dims[0] &&
        (unsigned)w.cur[1] < (unsigned)c.dims[1] && (unsigned)w.cur[2] < (unsigned)c.dims[2]) {
        if (MODE != MODE_VR && c.nf == 1) {
            if (st.comp) cells_fast<MODE, VAR, true, TG, 1>(a, s_tab, r, bp, c, w, kmax, step_limit, st);
            else cells_fast<MODE, VAR, false, TG, 1>(a, s_tab, r, bp, c, w, kmax, step_limit, st);
        } else if (MODE == MODE_VR && a.tf.grey_opacity != 1) {
            if (st.comp) cells_fast<MODE, VAR, true, TG, 0, 0>(a, s_tab, r, bp, c, w, kmax, step_limit, st);
            else cells_fast<MODE, VAR, false, TG, 0, 0>(a, s_tab, r, bp, c, w, kmax, step_limit, st);
        } else {
            if (st.comp) cells_fast<MODE, VAR, true, TG>(a, s_tab, r, bp, c, w, kmax, step_limit, st);
            else cells_fast<MODE, VAR, false, TG>(a, s_tab, r, bp, c, w, kmax, step_limit, st);
        }
        return;
    }
    // tdelta = step * iv_dir * dds (grid_traversal.pyx:86)
    double tdelta[3];
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) tdelta[i] = ray_tdelta(r, i, ldg(&bp->dds[i]));
    if (int_path) {
        // ---- integer cell loop (positive walk values: key == bits) -----------
        AxisStep A0, A1, A2;
        A0.bits = b0;
        A1.bits = b1;
        A2.bits = b2;
        step_prepare(A0, tdelta[0]);
        step_prepare(A1, tdelta[1]);
        step_prepare(A2, tdelta[2]);
        long long eb = dbits(w.enter_t);
        while (true) {
            if (++hitc > step_limit) {
                set_error(a.error, YTGB_DEVERR_STEP_LIMIT);
                break;
            }
            int i;
            if (A0.bits < A1.bits) i = A0.bits < A2.bits ? 0 : 2;
            else i = A1.bits < A2.bits ? 1 : 2;
            const long long tmb = i == 0 ? A0.bits : (i == 1 ? A1.bits : A2.bits);
            const long long xb = tmb < kmax ? tmb : kmax;  // fmin(tmax[i], max_t)
            const float dtf = MODE == MODE_TRACE ? 0.0f : diff_to_float(xb, eb);
            sample_cell<MODE, VAR, true, TG>(a, s_tab, bi, c, w.cur, w.P, dtf, eb, xb, st);
            // advance (grid_traversal.pyx:134-138)
            const int si = i == 0 ? r.step[0] : (i == 1 ? r.step[1] : r.step[2]);
            advance_position(w.P, c.vel, dtf, i, si);
            int ci, di;
            if (i == 0) {
                w.cur[0] += si;
                step_advance(A0, tdelta[0]);
                ci = w.cur[0];
                di = c.dims[0];
            } else if (i == 1) {
                w.cur[1] += si;
                step_advance(A1, tdelta[1]);
                ci = w.cur[1];
                di = c.dims[1];
            } else {
                w.cur[2] += si;
                step_advance(A2, tdelta[2]);
                ci = w.cur[2];
                di = c.dims[2];
            }
            eb = tmb;
            if (ci < 0 || ci >= di || !(tmb < kmax)) break;  // ... or enter_t >= max_t
        }
        return;
    }
    // ---- general cell loop (a walk value <= 0 or not finite) -----------------
    long long K0 = dkey(w.tmax[0]), K1 = dkey(w.tmax[1]), K2 = dkey(w.tmax[2]);
    double enter_t = w.enter_t;
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
        const double exit_t = Ki < kmax ? tm : max_t;
        const float dtf = MODE == MODE_TRACE ? 0.0f : (float)dsub(exit_t, enter_t);
        sample_cell<MODE, VAR, true, TG>(a, s_tab, bi, c, w.cur, w.P, dtf, dbits(enter_t), dbits(exit_t), st);
        const int si = i == 0 ? r.step[0] : (i == 1 ? r.step[1] : r.step[2]);
        advance_position(w.P, c.vel, dtf, i, si);
        const double td = i == 0 ? tdelta[0] : (i == 1 ? tdelta[1] : tdelta[2]);
        const double tn = dadd(tm, td);
        const long long Kn = dkey(tn);
        int ci, di;
        if (i == 0) {
            w.cur[0] += si; w.tmax[0] = tn; K0 = Kn; ci = w.cur[0]; di = c.dims[0];
        } else if (i == 1) {
            w.cur[1] += si; w.tmax[1] = tn; K1 = Kn; ci = w.cur[1]; di = c.dims[1];
        } else {
            w.cur[2] += si; w.tmax[2] = tn; K2 = Kn; ci = w.cur[2]; di = c.dims[2];
        }
        enter_t = tm;
        if (ci < 0 || ci >= di || !(Ki < kmax)) break;
    }
}

}  // namespace ytgb
