// ytgb_vertex.cuh -- vertex-centred brick data, computed where it is used.
//
// yt's AMRKDTree gives each kd leaf the vertex-centred data of its grid
// (get_brick_data, amr_kdtree.py:325-374): the grid's cell data is
// interpolated to vertices by ghost_zone_interpolate with no ghost zones
// (interpolators.pyx:177-226, via grid_patch.py:270-296), optionally
// log10'd with values <= 0 set to NaN (amr_kdtree.py:346-352), and sliced
// [li:ri+1] per leaf.  Here that runs on the device, one value per thread,
// straight into the float32 brick arena.
//
// With input_left = 0.5 and output_left = 0 (cell centres in index units)
// the reference's positions are exact: the vertex o of an axis of n cells
// sits at ropos = o - 0.5, its lower cell is clip(int(ropos), 0, n - 2)
// (C truncation), and the weights xp = ropos - ii, xm = 1 - xp are exactly
// one of {-0.5, 0.5, 1.5}.  The eight products are formed and summed in the
// reference's order with unfused float64 operations, so the vertex value is
// bit-identical to the reference's.
#pragma once

#include "ytgb_ray.cuh"

namespace ytgb {

struct VertexWeights {
    int i0;
    double p, m;  // weight of cell i0 + 1, weight of cell i0
};

YTGB_HD VertexWeights vertex_weights(int o, int n) {
    VertexWeights w;
    const double ropos = dsub((double)o, 0.5);
    int ii = (int)ropos;  // truncation toward zero, like <int> in Cython
    if (ii < 0) ii = 0;
    if (ii > n - 2) ii = n - 2;
    w.i0 = ii;
    w.p = dsub(ropos, (double)ii);
    w.m = dsub(1.0, w.p);
    return w;
}

// Vertex (o0, o1, o2) of a C-order cell block of dims n (each n >= 2).
YTGB_HD double vertex_value(const double *c, int n0, int n1, int n2, int o0, int o1, int o2) {
    const VertexWeights x = vertex_weights(o0, n0), y = vertex_weights(o1, n1), z = vertex_weights(o2, n2);
    const long long s1 = n2, s0 = (long long)n1 * n2;
    const double *b = c + x.i0 * s0 + y.i0 * s1 + z.i0;
    double v = dmul(ldg(b), dmul(dmul(x.m, y.m), z.m));
    v = dadd(v, dmul(ldg(b + s0), dmul(dmul(x.p, y.m), z.m)));
    v = dadd(v, dmul(ldg(b + s1), dmul(dmul(x.m, y.p), z.m)));
    v = dadd(v, dmul(ldg(b + 1), dmul(dmul(x.m, y.m), z.p)));
    v = dadd(v, dmul(ldg(b + s0 + 1), dmul(dmul(x.p, y.m), z.p)));
    v = dadd(v, dmul(ldg(b + s1 + 1), dmul(dmul(x.m, y.p), z.p)));
    v = dadd(v, dmul(ldg(b + s0 + s1), dmul(dmul(x.p, y.p), z.m)));
    v = dadd(v, dmul(ldg(b + s0 + s1 + 1), dmul(dmul(x.p, y.p), z.p)));
    return v;
}

}  // namespace ytgb
