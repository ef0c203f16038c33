// CPU build of the sampler kernels' per-ray walk -- TEST INFRASTRUCTURE.
//
// Compiles yt_gb300/csrc/ytgb_ray.cuh (the exact source the GPU kernels
// run per ray) with g++ and -ffp-contract=off and drives it over every pixel
// and brick the way render_kernel does (without the block binning), so
// tests can check the walk, geometry and compositing logic against the
// oracle on machines without a GPU.  The product never loads this library.
#include <vector>
#include "ytgb.h"
#include "ytgb_ray.cuh"
#include "ytgb_vertex.cuh"
#include "ytgb_octree.cuh"
using namespace ytgb;

template <int MODE, int VAR>
static void run(const ytgb_render_args &a, unsigned long long *hashes, long long *counts, unsigned long long *cnt) {
    std::vector<float4> tab;
    if (MODE == MODE_VR || MODE == MODE_LIGHT) {
        const float4 *g = reinterpret_cast<const float4 *>(a.tf_tables);
        int nb = a.tf.nbins_max;
        if (VAR & V_CTF) {
            tab.resize(3 * nb);
            for (int b = 0; b < nb; b++) {
                float4 t0 = g[b], t1 = g[nb + b], t2 = g[2 * nb + b], t3 = g[3 * nb + b];
                tab[3 * b + 0] = make_float4(t0.x, t1.x, t2.x, t3.x);
                tab[3 * b + 1] = make_float4(t0.y, t1.y, t2.y, t3.y);
                tab[3 * b + 2] = make_float4(t3.z, t3.w, 0.f, 0.f);
            }
        } else {
            tab.assign(g, g + a.tf.n_fits * nb);
        }
    }
    const int4 *rects = reinterpret_cast<const int4 *>(a.rects);
    for (int vi = 0; vi < a.view.nx; vi++)
        for (int vj = 0; vj < a.view.ny; vj++) {
            size_t p = (size_t)vi * a.view.ny + vj;
            Ray r;
            make_ray(a.view, vi, vj, r);
            double *img = a.image ? a.image + p * 4 : nullptr;
            RayState st;
            ray_state_init(st, MODE != MODE_TRACE ? img : nullptr, a.zbuffer ? a.zbuffer[p] : 1.0, a.zbuffer != nullptr, a.flags);
            if (MODE == MODE_TRACE) { st.th = hashes[p]; st.tcount = counts[p]; }
            for (int k = 0; k < a.n_order; k++) {
                int4 rc = rects[k];
                if (vi < rc.x || vi >= rc.y || vj < rc.z || vj >= rc.w) continue;
                walk_brick<MODE, VAR>(a, tab.data(), r, a.order[k], st);
            }
            if (MODE == MODE_TRACE) { hashes[p] = st.th; counts[p] = st.tcount; }
            else for (int c = 0; c < 4; c++) if (st.touched & (1u << c)) img[c] = (double)st.xh[c] + (double)st.xl[c];
            cnt[0] += st.visits; cnt[1] += st.walks; cnt[3] += st.guarded; cnt[2]++;
        }
}

extern "C" int emu_render(const ytgb_render_args *a_in, int trace, unsigned long long *hashes, long long *counts,
                          unsigned long long *cnt) {
    ytgb_render_args copy = *a_in;  // the launch's derived view constants, as ytgb_render forms them
    view_derive(copy.view);
    const ytgb_render_args *a = &copy;
    if (trace) { run<MODE_TRACE, 0>(*a, hashes, counts, cnt); return 0; }
    switch (a->kind) {
    case YTGB_VOLUME_RENDER:
        switch (render_variant(*a)) {
        case V_CTF: run<MODE_VR, V_CTF>(*a, 0, 0, cnt); break;
        case V_REF: run<MODE_VR, V_REF>(*a, 0, 0, cnt); break;
        case V_CTF | V_REF: run<MODE_VR, V_CTF | V_REF>(*a, 0, 0, cnt); break;
        default: run<MODE_VR, 0>(*a, 0, 0, cnt);
        }
        break;
    case YTGB_PROJECTION: run<MODE_PROJ, 0>(*a, 0, 0, cnt); break;
    case YTGB_INTERPOLATED_PROJECTION: run<MODE_IPROJ, 0>(*a, 0, 0, cnt); break;
    case YTGB_LIGHT_SOURCE:
        if (render_variant(*a) & V_REF) run<MODE_LIGHT, V_REF>(*a, 0, 0, cnt);
        else run<MODE_LIGHT, 0>(*a, 0, 0, cnt);
        break;
    default: run<MODE_MIP, 0>(*a, 0, 0, cnt);
    }
    return 0;
}

// the rays make_ray generates for every pixel (positions and directions)
extern "C" void emu_rays(const ytgb_view *v_in, double *pos, double *dir) {
    ytgb_view vd = *v_in;
    view_derive(vd);
    const ytgb_view *v = &vd;
    for (int vi = 0; vi < v->nx; vi++)
        for (int vj = 0; vj < v->ny; vj++) {
            Ray r;
            make_ray(*v, vi, vj, r);
            size_t o = ((size_t)vi * v->ny + vj) * 3;
            for (int i = 0; i < 3; i++) {
                pos[o + i] = r.pos[i];
                dir[o + i] = r.dir[i];
            }
        }
}

// ---- direct checks of the integer float64 helpers --------------------------
#include <random>
static double rand_pos(std::mt19937_64 &g) {
    // positive doubles over a wide range, with many short mantissas (ties)
    std::uniform_real_distribution<double> u(-12.0, 2.0);
    double x = std::pow(2.0, u(g));
    if (g() % 4 == 0) {
        long long b;
        std::memcpy(&b, &x, 8);
        b &= ~((1LL << (g() % 52)) - 1);  // clear low mantissa bits
        std::memcpy(&x, &b, 8);
    }
    return x;
}

// returns the number of mismatches of repeated tmax += tdelta (n walks of
// `steps` additions) between the integer stepping and float64 addition
extern "C" long long emu_check_step(long long n, int steps, unsigned long long seed) {
    std::mt19937_64 g(seed);
    long long bad = 0;
    for (long long k = 0; k < n; k++) {
        double x = rand_pos(g), d = rand_pos(g) * std::pow(2.0, -(double)(g() % 30));
        AxisStep s;
        s.bits = dbits(x);
        step_prepare(s, d);
        double ref = x;
        for (int j = 0; j < steps; j++) {
            ref = ref + d;
            step_advance(s, d);
            if (s.bits != dbits(ref)) { bad++; break; }
        }
    }
    return bad;
}

// mismatches of diff_to_float against (float)(x - y) computed in long double
// (exact for these inputs), and of split_floor against floor / fraction
// |got - exact| < one float32 ulp of exact (got is one of the two floats
// around it)
static bool within_ulp(float got, long double exact) {
    const float lo = std::nextafter((float)exact, -INFINITY), hi = std::nextafter((float)exact, INFINITY);
    const float near = (float)exact;
    return got == near || (got == lo && (long double)lo <= exact && exact <= (long double)near) ||
           (got == hi && (long double)near <= exact && exact <= (long double)hi);
}

extern "C" long long emu_check_convert(long long n, unsigned long long seed) {
    std::mt19937_64 g(seed);
    long long bad = 0;
    for (long long k = 0; k < n; k++) {
        double y = rand_pos(g), x = y * (1.0 + std::ldexp((double)(g() % 1000000), -(int)(g() % 40)));
        if (g() % 3 == 0) std::swap(x, y);
        // faithful rounding: within one float32 ulp of the exact difference
        float got = diff_to_float(dbits(x), dbits(y));
        long double exact = (long double)x - (long double)y;
        if (!within_ulp(got, exact)) bad++;
        // the cell loop's form gives the same value
        if (diff_to_float_loop(dbits(x), dbits(y)) != got) bad++;
        double t = std::ldexp((double)(g() >> 11), -(int)(g() % 60));  // 0 <= t < 2^53 .. small
        if (t > 0 && t < 1073741824.0) {
            int fl; float fr;
            split_floor(dbits(t), fl, fr);
            if (fl != (int)std::floor(t) || !within_ulp(fr, (long double)(t - std::floor(t)))) bad++;
        }
    }
    return bad;
}

// Every vertex of a C-order cell block, as the device brick preparation
// computes it (ytgb_vertex.cuh).
extern "C" void emu_vertex(const double *cells, int n0, int n1, int n2, double *out) {
    long long t = 0;
    for (int i = 0; i <= n0; i++)
        for (int j = 0; j <= n1; j++)
            for (int k = 0; k <= n2; k++) out[t++] = ytgb::vertex_value(cells, n0, n1, n2, i, j, k);
}

// cast_through_octree per pixel, as the octree kernel runs it
// (ytgb_octree.cuh:octree_ray), on the CPU.
template <int MODE, int CTF>
static int run_octree(const ytgb_render_args &a, const ytgb_octree_args &oa, unsigned long long *hashes,
                      long long *counts, unsigned long long *cnt) {
    std::vector<float4> tab;
    if (MODE == MODE_VR || MODE == MODE_LIGHT) {
        const float4 *g = reinterpret_cast<const float4 *>(a.tf_tables);
        int nb = a.tf.nbins_max;
        if (CTF) {
            tab.resize(3 * nb);
            for (int b = 0; b < nb; b++) {
                float4 t0 = g[b], t1 = g[nb + b], t2 = g[2 * nb + b], t3 = g[3 * nb + b];
                tab[3 * b + 0] = make_float4(t0.x, t1.x, t2.x, t3.x);
                tab[3 * b + 1] = make_float4(t0.y, t1.y, t2.y, t3.y);
                tab[3 * b + 2] = make_float4(t3.z, t3.w, 0.f, 0.f);
            }
        } else {
            tab.assign(g, g + a.tf.n_fits * nb);
        }
    }
    OctreeView o;
    o.nodes = reinterpret_cast<const ONode *>(oa.nodes);
    o.n_nodes = oa.n_nodes;
    o.verts = oa.verts;
    o.edges = oa.edges;
    o.edges_f = reinterpret_cast<const float4 *>(oa.edges_f);
    o.n_cells = oa.n_cells;
    o.depth = oa.depth;
    for (int i = 0; i < 3; i++) {
        o.dle[i] = oa.dle[i];
        o.dre[i] = oa.dre[i];
        o.size[i] = oa.dre[i] - oa.dle[i];
    }
    int bad = 0;
    for (int vi = 0; vi < a.view.nx; vi++)
        for (int vj = 0; vj < a.view.ny; vj++) {
            size_t p = (size_t)vi * a.view.ny + vj;
            Ray r;
            make_ray(a.view, vi, vj, r);
            double *img = a.image ? a.image + p * 4 : nullptr;
            RayState st;
            ray_state_init(st, MODE != MODE_TRACE ? img : nullptr, 1.0, false, a.flags);
            unsigned long long th = MODE == MODE_TRACE ? hashes[p] : 0ull;
            long long tc = 0;
            if (!octree_ray<MODE, CTF>(a, o, tab.data(), r, st, th, tc)) bad++;
            if (MODE == MODE_TRACE) { hashes[p] = th; counts[p] += tc; }
            else for (int c = 0; c < 4; c++) if (st.touched & (1u << c)) img[c] = (double)st.xh[c] + (double)st.xl[c];
            cnt[0] += st.visits; cnt[1] += st.walks; cnt[3] += st.guarded; cnt[2]++;
        }
    return bad;
}

extern "C" int emu_octree(const ytgb_render_args *a_in, const ytgb_octree_args *o, int trace,
                          unsigned long long *hashes, long long *counts, unsigned long long *cnt) {
    ytgb_render_args copy = *a_in;
    view_derive(copy.view);
    const ytgb_render_args *a = &copy;
    if (trace) return run_octree<MODE_TRACE, 0>(*a, *o, hashes, counts, cnt);
    switch (a->kind) {
    case YTGB_VOLUME_RENDER:
        return a->tf.ctf_fast ? run_octree<MODE_VR, 1>(*a, *o, 0, 0, cnt) : run_octree<MODE_VR, 0>(*a, *o, 0, 0, cnt);
    case YTGB_PROJECTION: return run_octree<MODE_PROJ, 0>(*a, *o, 0, 0, cnt);
    case YTGB_INTERPOLATED_PROJECTION: return run_octree<MODE_IPROJ, 0>(*a, *o, 0, 0, cnt);
    case YTGB_LIGHT_SOURCE: return run_octree<MODE_LIGHT, 0>(*a, *o, 0, 0, cnt);
    default: return run_octree<MODE_MIP, 0>(*a, *o, 0, 0, cnt);
    }
}
