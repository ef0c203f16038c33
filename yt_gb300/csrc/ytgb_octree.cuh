// ytgb_octree.cuh -- the octree ray caster of yt's octree volume source,
// per ray, host/device (the test harness runs it on the CPU).
//
// ImageSampler.cast_through_octree (image_samplers.pyx:202-288) casts each
// pixel's ray through an octree of cells (Octree<int>::cast_ray,
// _octree_raytracing.hpp:199-230: the parametric traversal of Revelles,
// Urena and Lastra, proc_subtree :276-337) and hands every terminal cell it
// meets, in traversal order, to the sampler as a 1x1x1 vertex-centred brick
// with the cell's own edges.  The traversal's float64 values (the direction
// normalisation, the t of the six slab planes, the midpoints) are formed
// from the same operands in the same order as the reference, unfused, so
// the cells and their enter/exit t are bit-identical; the recursion becomes
// an explicit stack of at most depth + 1 frames.
#pragma once

#include "ytgb_ray.cuh"

namespace ytgb {

// Device form of one octree node: children (-1: none), key, flags.
struct ONode {
    int32_t child[8];
    int32_t key;
    int32_t flags;  // bit 0: terminal, bit 1: has a children array
};

struct OctreeView {
    const ONode *nodes;
    int32_t n_nodes;
    const float *verts;    // 8 per cell, (i,j,k) C order
    const double *edges;   // 9 per cell: left edge, right edge, 1/(right - left)
    const float4 *edges_f; // 3 per cell (or null): left edge hi, lo, (float)(1/(right - left))
    int32_t n_cells;
    int32_t depth;
    double dle[3], dre[3], size[3];
};

constexpr int OCT_MAX_DEPTH = 30;

// The traversal's comparisons.  With K they run on order-preserving int64
// keys of the doubles (the integer pipe; GB300's float64 pipe is 1/64 of its
// float32 rate), which order every finite or infinite value exactly as the
// float64 comparison does.  They hold while no NaN arises: a ray whose six
// slab t are all below 2^1023 in magnitude has every midpoint (a + b) * 0.5
// bounded by them, so it takes K; any other ray (a direction component of 0
// makes inf and, at a midpoint, NaN) takes the float64 comparisons.
template <bool K> YTGB_HD bool lt(double a, double b) { return K ? dkey(a) < dkey(b) : a < b; }
template <bool K> YTGB_HD bool ge(double a, double b) { return K ? !(dkey(a) < dkey(b)) : a >= b; }

// std::max / std::min as the reference calls them
template <bool K> YTGB_HD double smax(double a, double b) { return lt<K>(a, b) ? b : a; }
template <bool K> YTGB_HD double smin(double a, double b) { return lt<K>(b, a) ? b : a; }

template <bool K>
YTGB_HD int first_node(double tx0, double ty0, double tz0, double txm, double tym, double tzm) {
    int index = 0;
    if (ge<K>(tx0, smax<K>(ty0, tz0))) {
        if (lt<K>(tym, tx0)) index |= 2;
        if (lt<K>(tzm, tx0)) index |= 1;
    } else if (ge<K>(ty0, smax<K>(tx0, tz0))) {
        if (lt<K>(txm, ty0)) index |= 4;
        if (lt<K>(tzm, ty0)) index |= 1;
    } else {
        if (lt<K>(txm, tz0)) index |= 4;
        if (lt<K>(tym, tz0)) index |= 2;
    }
    return index;
}

template <bool K>
YTGB_HD int next_node(double tx, double ty, double tz, int ix, int iy, int iz) {
    if (lt<K>(tx, smin<K>(ty, tz))) return ix;
    if (lt<K>(ty, smin<K>(tx, tz))) return iy;
    return iz;
}

// s + e == a + b exactly (TwoSum, Knuth TAOCP vol. 2, 4.2.2)
YTGB_HD void two_sum(float a, float b, float &s, float &e) {
    s = fadd(a, b);
    const float bp = fsub(s, a);
    e = fadd(fsub(a, fsub(s, bp)), fsub(b, bp));
}

struct OFrame {
    int32_t node;
    int32_t inode;  // -1: not entered yet; 8: done
    double t0[3], t1[3], tm[3];  // tm: the midpoints, once entered
};

// Calls cell(key, t_in, t_out) for every terminal cell of the ray's path,
// in proc_subtree's order.  Returns false if the stack or step budget ran
// out (a malformed tree).
template <bool K, typename F>
YTGB_HD bool octree_walk(const OctreeView &o, const double t0[3], const double t1[3], int a, F &cell);

template <typename F>
YTGB_HD bool octree_cast(const OctreeView &o, const double o_in[3], const double d_in[3], F cell) {
    double p[3], d[3], dd = 0.0, t0[3], t1[3];
    int a = 0, bmask = 4;
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        p[i] = o_in[i];
        dd = dadd(dd, dmul(d_in[i], d_in[i]));
    }
    dd = dsqrt(dd);
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) d[i] = ddiv(d_in[i], dd);
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        if (d[i] < 0.0) {
            p[i] = dsub(o.size[i], p[i]);
            d[i] = -d[i];
            a |= bmask;
        }
        bmask >>= 1;
    }
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        t0[i] = ddiv(dsub(o.dle[i], p[i]), d[i]);
        t1[i] = ddiv(dsub(o.dre[i], p[i]), d[i]);
    }
    double mx = t0[0], mn = t1[0];  // std::max_element / std::min_element
    if (mx < t0[1]) mx = t0[1];
    if (mx < t0[2]) mx = t0[2];
    if (t1[1] < mn) mn = t1[1];
    if (t1[2] < mn) mn = t1[2];
    if (!(mx < mn)) return true;
    bool bounded = true;  // exponent field below 0x7fe: |t| < 2^1023
    YTGB_UNROLL
    for (int i = 0; i < 3; i++)
        bounded = bounded && (dbits(t0[i]) & 0x7ff0000000000000ll) < 0x7fe0000000000000ll &&
                  (dbits(t1[i]) & 0x7ff0000000000000ll) < 0x7fe0000000000000ll;
    return bounded ? octree_walk<true>(o, t0, t1, a, cell) : octree_walk<false>(o, t0, t1, a, cell);
}

// proc_subtree (_octree_raytracing.hpp:276-337) from the root over the slab
// [t0, t1], with an explicit stack.
template <bool K, typename F>
YTGB_HD bool octree_walk(const OctreeView &o, const double t0[3], const double t1[3], int a, F &cell) {
    OFrame st[OCT_MAX_DEPTH + 2];
    int sp = -1;
    const int max_depth = o.depth < OCT_MAX_DEPTH ? o.depth : OCT_MAX_DEPTH;
    bool ok = true;
    // proc_subtree's entry for node n over the slab [c0, c1]: a terminal
    // node is handed to the sampler at once, an internal one is pushed
    auto visit = [&](int n, const double c0[3], const double c1[3]) {
        if (lt<K>(c1[0], 0.0) || lt<K>(c1[1], 0.0) || lt<K>(c1[2], 0.0) || n < 0) return;
        if (n >= o.n_nodes) {
            ok = false;
            return;
        }
        const int flags = ldg(&o.nodes[n].flags);
        if (flags & 1) {
            cell(ldg(&o.nodes[n].key), smax<K>(smax<K>(c0[0], c0[1]), c0[2]), smin<K>(smin<K>(c1[0], c1[1]), c1[2]));
            return;
        }
        if (!(flags & 2)) return;
        if (sp + 1 > max_depth) {
            ok = false;
            return;
        }
        OFrame &f = st[++sp];
        f.node = n;
        YTGB_UNROLL
        for (int i = 0; i < 3; i++) {
            f.t0[i] = c0[i];
            f.t1[i] = c1[i];
            f.tm[i] = dmul(dadd(c0[i], c1[i]), 0.5);
        }
        f.inode = first_node<K>(c0[0], c0[1], c0[2], f.tm[0], f.tm[1], f.tm[2]);
    };
    visit(0, t0, t1);
    long long budget = 0;
    while (sp >= 0 && ok) {
        if (++budget > (1LL << 26)) return false;
        OFrame &f = st[sp];
        const int q = f.inode;
        if (q >= 8) {
            sp--;
            continue;
        }
        const double xm = f.tm[0], ym = f.tm[1], zm = f.tm[2];
        // child q's slab: lower or upper half on each axis (bit 2: x, 1: y, 0: z)
        const bool ux = q & 4, uy = q & 2, uz = q & 1;
        double c0[3], c1[3];
        c0[0] = ux ? xm : f.t0[0];
        c1[0] = ux ? f.t1[0] : xm;
        c0[1] = uy ? ym : f.t0[1];
        c1[1] = uy ? f.t1[1] : ym;
        c0[2] = uz ? zm : f.t0[2];
        c1[2] = uz ? f.t1[2] : zm;
        const int child = ldg(&o.nodes[f.node].child[q ^ a]);
        // the successor among the children (next_node's exit-plane table)
        switch (q) {
        case 0: f.inode = next_node<K>(xm, ym, zm, 4, 2, 1); break;
        case 1: f.inode = next_node<K>(xm, ym, f.t1[2], 5, 3, 8); break;
        case 2: f.inode = next_node<K>(xm, f.t1[1], zm, 6, 8, 3); break;
        case 3: f.inode = next_node<K>(xm, f.t1[1], f.t1[2], 7, 8, 8); break;
        case 4: f.inode = next_node<K>(f.t1[0], ym, zm, 8, 6, 5); break;
        case 5: f.inode = next_node<K>(f.t1[0], ym, f.t1[2], 8, 7, 8); break;
        case 6: f.inode = next_node<K>(f.t1[0], f.t1[1], zm, 8, 8, 7); break;
        default: f.inode = 8; break;
        }
        visit(child, c0, c1);
    }
    return ok;
}

// One pixel of cast_through_octree: the ray cast through the octree and
// each terminal cell handed to sample_cell as a 1x1x1 brick (dims 1, vertex
// strides 4 and 2, no mask, one field), with enter/exit t divided by the
// direction's length (image_samplers.pyx:245-283).  In MODE_TRACE it hashes
// (key, enter bits, exit bits) into th instead.  Returns false when the
// traversal gave up (malformed tree).
template <int MODE, int CTF>
YTGB_HD bool octree_ray(const ytgb_render_args &a, const OctreeView &o, const float4 *s_tab, const Ray &r,
                        RayState &st, unsigned long long &th, long long &tcount) {
    const double len = dsqrt(dadd(dadd(dmul(r.dir[0], r.dir[0]), dmul(r.dir[1], r.dir[1])), dmul(r.dir[2], r.dir[2])));
    // The sampler uses enter/exit t only through float32 quantities (dt and
    // the in-cell position), so a product with 1/len (within an ulp of the
    // quotient) serves it; the trace keeps the reference's exact quotients.
    const double ilen = ddiv(1.0, len);
    // the ray as float32 pairs (hi + lo = the float64 value to ~2^-48)
    float ph[3], pl[3], dh[3], dl[3];
    YTGB_UNROLL
    for (int i = 0; i < 3; i++) {
        ph[i] = (float)r.pos[i];
        pl[i] = (float)dsub(r.pos[i], (double)ph[i]);
        dh[i] = (float)r.dir[i];
        dl[i] = (float)dsub(r.dir[i], (double)dh[i]);
    }
    return octree_cast(o, r.pos, r.dir, [&](int key, double t_in, double t_out) {
        if (key < 0 || key >= o.n_cells) {
            st.guarded++;
            return;
        }
        const double e = MODE == MODE_TRACE ? ddiv(t_in, len) : dmul(t_in, ilen);
        const double x = MODE == MODE_TRACE ? ddiv(t_out, len) : dmul(t_out, ilen);
        if (MODE == MODE_TRACE) {
            th = fnv_mix(th, (unsigned long long)(unsigned)key);
            // a NaN (rays with zero direction components meet NaN slab
            // midpoints) enters the hash as one pattern: its sign and payload
            // differ between the GPU and CPUs
            th = fnv_mix(th, e != e ? 0x7ff8000000000000ull : (unsigned long long)dbits(e));
            th = fnv_mix(th, x != x ? 0x7ff8000000000000ull : (unsigned long long)dbits(x));
            tcount++;
            st.visits++;
            return;
        }
        CellCtx c;
        c.base = o.verts + 8ll * key;
        c.fstride = 0;
        c.moff = -1;
        c.nf = 1;
        c.sx = 4;
        c.sy = 2;
        c.tol = -1.0f;  // octree cells: float32 range decisions
        c.ray = nullptr;
        c.bp = nullptr;
        float P[3];
        if (o.edges_f) {
            // (enter * v_dir + v_pos - left_edge) * idds (image_samplers.pyx:
            // 475-478) in float32 pairs: the products exact by FMA, the sums
            // by TwoSum, so the difference keeps ~2^-48 of the operands' scale
            // (the cell is ~2^-9 of it), then one float32 rounding and the
            // float32 idds: within a float32 ulp or two of the float64 form,
            // on the float32 pipes rather than six float64 operations
            const float4 A = ldg(o.edges_f + 3ll * key), B = ldg(o.edges_f + 3ll * key + 1);
            const float4 D = ldg(o.edges_f + 3ll * key + 2);
            const float leh[3] = {A.x, A.y, A.z}, lel[3] = {A.w, B.x, B.y}, idf[3] = {B.z, B.w, D.x};
            const float eh = (float)e, el = (float)dsub(e, (double)eh);
            YTGB_UNROLL
            for (int i = 0; i < 3; i++) {
                c.dims[i] = 1;
                c.vel[i] = fmul(r.fdir[i], idf[i]);
                const float mh = fmul(eh, dh[i]);
                float ml = ffma(eh, dh[i], -mh);
                ml = ffma(eh, dl[i], ml);
                ml = ffma(el, dh[i], ml);
                float sh, se, uh, ue;
                two_sum(mh, ph[i], sh, se);
                const float sl = fadd(fadd(se, ml), pl[i]);
                two_sum(sh, -leh[i], uh, ue);
                const float ul = fsub(fadd(ue, sl), lel[i]);
                P[i] = fmul(fadd(uh, ul), idf[i]);
            }
        } else {
            const double *ed = o.edges + 9ll * key;
            YTGB_UNROLL
            for (int i = 0; i < 3; i++) {
                c.dims[i] = 1;
                const double idds = ldg(ed + 6 + i);
                c.vel[i] = fmul(r.fdir[i], (float)idds);
                // (enter * v_dir + v_pos - left_edge) * idds (image_samplers.pyx:475-478)
                P[i] = (float)dmul(dsub(dadd(dmul(e, r.dir[i]), r.pos[i]), ldg(ed + i)), idds);
            }
        }
        const int cur[3] = {0, 0, 0};
        st.walks++;
        sample_cell<MODE, CTF, false>(a, s_tab, key, c, cur, P, (float)dsub(x, e), dbits(e), dbits(x), st);
    });
}

}  // namespace ytgb
