// ytgb_host.cpp -- host side of libytgb: status, pixel culling, transfer
// function packing and the AMR kd-tree.  Compiled with -ffp-contract=off so
// that its float64 arithmetic rounds exactly like yt's compiled Cython.
#include <cmath>
#include <limits>
#include <cstdint>
#include <cstring>
#include <climits>
#include <string>
#include <thread>
#include <vector>
#include <algorithm>

#include "ytgb.h"
#include "ytgb_internal.h"

static thread_local std::string g_last_error;

void ytgb_set_error(const std::string &msg) { g_last_error = msg; }

extern "C" int ytgb_abi_version(void) { return YTGB_ABI_VERSION; }

extern "C" const char *ytgb_last_error(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// Pixel culling.  lenses.pyx:22-175 and image_samplers.pyx:159-163.
// ---------------------------------------------------------------------------
static inline int64_t i64clip(int64_t i, int64_t a, int64_t b) {
    if (i < a) return a;
    if (i > b) return b;
    return i;
}

// calculate_extent_plane_parallel (lenses.pyx:22-55)
static void extent_plane_parallel(const ytgb_view *im, const ytgb_brick *vc, int64_t rv[4]) {
    double temp, cx, cy, extrema[4];
    const double *edges[2] = {vc->left_edge, vc->right_edge};
    extrema[0] = extrema[2] = 1e300;
    extrema[1] = extrema[3] = -1e300;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
            for (int k = 0; k < 2; k++) {
                temp = edges[i][0] * im->x_vec[0];
                temp += edges[j][1] * im->x_vec[1];
                temp += edges[k][2] * im->x_vec[2];
                if (temp < extrema[0]) extrema[0] = temp;
                if (temp > extrema[1]) extrema[1] = temp;
                temp = edges[i][0] * im->y_vec[0];
                temp += edges[j][1] * im->y_vec[1];
                temp += edges[k][2] * im->y_vec[2];
                if (temp < extrema[2]) extrema[2] = temp;
                if (temp > extrema[3]) extrema[3] = temp;
            }
    cx = cy = 0.0;
    for (int i = 0; i < 3; i++) {
        cx += im->center[i] * im->x_vec[i];
        cy += im->center[i] * im->y_vec[i];
    }
    rv[0] = lrint((extrema[0] - cx - im->bounds[0]) / im->pdx);
    rv[1] = rv[0] + lrint((extrema[1] - extrema[0]) / im->pdx);
    rv[2] = lrint((extrema[2] - cy - im->bounds[2]) / im->pdy);
    rv[3] = rv[2] + lrint((extrema[3] - extrema[2]) / im->pdy);
}

static inline double dot3(const double a[3], const double b[3]) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// calculate_extent_perspective (lenses.pyx:60-161).  The reference keeps the
// sight-line length, angle cosine and projected offsets in single precision
// (lenses.pyx:73); the casts below reproduce exactly those roundings.
static void extent_perspective(const ytgb_view *im, const ytgb_brick *vc, int64_t rv[4]) {
    double cam_pos[3], cam_width[3], north_vector[3], east_vector[3], normal_vector[3];
    double vertex[3], pos1[3], sight_vector[3], sight_center[3];
    float sight_vector_norm, sight_angle_cos, sight_length, dx, dy;
    int px, py;
    int min_px = SHRT_MAX, min_py = SHRT_MAX, max_px = -SHRT_MAX, max_py = -SHRT_MAX;
    const double *le = vc->left_edge, *re = vc->right_edge;
    const double cxs[8] = {le[0], re[0], re[0], le[0], le[0], re[0], re[0], le[0]};
    const double cys[8] = {le[1], le[1], re[1], re[1], le[1], le[1], re[1], re[1]};
    const double czs[8] = {le[2], le[2], le[2], le[2], re[2], re[2], re[2], re[2]};
    for (int i = 0; i < 3; i++) {
        cam_pos[i] = im->camera_data[0 * 3 + i];
        cam_width[i] = im->camera_data[1 * 3 + i];
        east_vector[i] = im->camera_data[2 * 3 + i];
        north_vector[i] = im->camera_data[3 * 3 + i];
        normal_vector[i] = im->camera_data[4 * 3 + i];
    }
    for (int iv = 0; iv < 8; iv++) {
        vertex[0] = cxs[iv];
        vertex[1] = cys[iv];
        vertex[2] = czs[iv];
        cam_width[1] = cam_width[0] * im->ny / im->nx;
        for (int i = 0; i < 3; i++) sight_vector[i] = vertex[i] - cam_pos[i];
        for (int i = 0; i < 3; i++) sight_center[i] = cam_width[2] * normal_vector[i] + cam_pos[i];
        double sn = std::sqrt(sight_vector[0] * sight_vector[0] + sight_vector[1] * sight_vector[1] +
                              sight_vector[2] * sight_vector[2]);
        sight_vector_norm = (float)sn;
        if (sight_vector_norm != 0)
            for (int i = 0; i < 3; i++) sight_vector[i] = sight_vector[i] / (double)sight_vector_norm;
        sight_angle_cos = (float)dot3(sight_vector, normal_vector);
        {
            double c = (double)sight_angle_cos;
            c = c > -1.0 ? c : -1.0;  // fclip: fmin(fmax(f, a), b)
            c = c < 1.0 ? c : 1.0;
            sight_angle_cos = (float)c;
        }
        if (std::acos((double)sight_angle_cos) < (0.5 * M_PI) && sight_angle_cos != 0.0) {
            sight_length = (float)(cam_width[2] / (double)sight_angle_cos);
        } else {
            sight_length = (float)std::sqrt(cam_width[0] * cam_width[0] + cam_width[1] * cam_width[1]);
            float c2 = sight_angle_cos * sight_angle_cos;
            sight_length = (float)((double)sight_length / std::sqrt(1.0 - (double)c2));
        }
        for (int i = 0; i < 3; i++) pos1[i] = (double)sight_length * sight_vector[i] + cam_pos[i];
        for (int i = 0; i < 3; i++) pos1[i] = pos1[i] - sight_center[i];
        dx = (float)dot3(pos1, east_vector);
        dy = (float)dot3(pos1, north_vector);
        px = (int)((im->nx * 0.5) + (((double)im->nx / cam_width[0]) * (double)dx));
        py = (int)((im->ny * 0.5) + (((double)im->ny / cam_width[1]) * (double)dy));
        min_px = std::min(min_px, px);
        max_px = std::max(max_px, px);
        min_py = std::min(min_py, py);
        max_py = std::max(max_py, py);
    }
    rv[0] = std::max(min_px, 0);
    rv[1] = std::min(max_px, im->nx);
    rv[2] = std::max(min_py, 0);
    rv[3] = std::min(max_py, im->ny);
}

extern "C" int ytgb_brick_layout(int64_t n, const int64_t *dims, const double *le, const double *re,
                                 const int64_t *n_fields, const int64_t *sizes_max, ytgb_brick *desc, double *bounds,
                                 int64_t bounds_len, int64_t *arena_len) {
    if (n < 0 || (n > 0 && (!dims || !le || !re || !n_fields || !sizes_max || !desc || !bounds || !arena_len))) {
        ytgb_set_error("ytgb_brick_layout: bad arguments");
        return YTGB_ERR_INVALID;
    }
    int64_t off = 0, boff = 0;
    for (int64_t k = 0; k < n; k++) {
        ytgb_brick &b = desc[k];
        std::memset(&b, 0, sizeof(b));
        const int64_t stride = (sizes_max[k] + 3) & ~(int64_t)3;
        if (sizes_max[k] < 0 || n_fields[k] < 1 || n_fields[k] > 6) {
            ytgb_set_error("ytgb_brick_layout: brick " + std::to_string(k) + ": bad field sizes");
            return YTGB_ERR_INVALID;
        }
        for (int i = 0; i < 3; i++) {
            const int64_t d = dims[3 * k + i];
            if (d < 1 || d > (1 << 30) || boff + d + 1 > bounds_len) {
                ytgb_set_error("ytgb_brick_layout: brick " + std::to_string(k) + ": bad dims or short table");
                return YTGB_ERR_INVALID;
            }
            // PartitionedGrid.__cinit__ (partitioned_grid.pyx:54-55), elementwise
            const double l = le[3 * k + i], r = re[3 * k + i];
            const double dds = (r - l) / (double)d;
            const double idds = 1.0 / dds;
            b.left_edge[i] = l;
            b.right_edge[i] = r;
            b.dds[i] = dds;
            b.idds[i] = idds;
            b.snap[i] = 1e-10 * dds;
            b.dims[i] = (int32_t)d;
            b.lef[i] = (float)l;
            b.ref[i] = (float)r;
            b.iddsf[i] = (float)idds;
            // cell-boundary table k*dds + le, k = 0..dims (the float64 values
            // walk_volume forms for tmax, grid_traversal.pyx:106-108)
            if (i == 0) b.bounds_offset = boff;
            for (int64_t q = 0; q <= d; q++) bounds[boff + q] = (double)q * dds + l;
            boff += d + 1;
        }
        b.n_fields = (int32_t)n_fields[k];
        b.data_offset = off;
        b.field_stride = stride;
        b.mask_offset = -1;
        off += stride * n_fields[k];
    }
    *arena_len = off;
    return YTGB_OK;
}

// ---------------------------------------------------------------------------
// Off-axis projection stamps: direct_integrate_cube (image_utilities.pyx:
// 321-407) with check_in_parallelogram (:296-318), per stamp level.
// ---------------------------------------------------------------------------
static bool in_parallelogram(const double PA[2], const double PQ[3], const double PR[3], int sign, double nm[2]) {
    const double det = PQ[0] * PR[1] - PQ[1] * PR[0];
    if (det == 0) return false;
    nm[0] = -(PA[0] * PQ[1] - PA[1] * PQ[0]) / det;
    nm[1] = (PA[0] * PR[1] - PA[1] * PR[0]) / det;
    const double s0 = sign * nm[0], s1 = sign * nm[1];
    return 0 <= s0 && s0 <= 1 && 0 <= s1 && s1 <= 1;
}

extern "C" int ytgb_offaxis_depths(const double *o, const double *u, const double *v, const double *w, int32_t nsx,
                                   int32_t nsy, int32_t max_depth, double *stamp, uint8_t *mask) {
    if (!o || !u || !v || !w || !stamp || !mask || nsx < 1 || nsy < 1 || max_depth < 1 || max_depth > 30) {
        ytgb_set_error("ytgb_offaxis_depths: bad arguments");
        return YTGB_ERR_INVALID;
    }
    double ob[3];
    for (int k = 0; k < 3; k++) ob[k] = o[k] + u[k] + v[k] + w[k];
    for (int d = 1; d < max_depth; d++) {
        const int sx = (1 << d) < nsx ? (1 << d) : nsx, sy = (1 << d) < nsy ? (1 << d) : nsy;
        double *st = stamp + (int64_t)d * nsx * nsy;
        uint8_t *mk = mask + (int64_t)d * nsx * nsy;
        for (int i = 0; i < sx; i++) {
            const double x0 = ((double)i + 0.5) * (1.0 / sx);
            for (int j = 0; j < sy; j++) {
                const double x1 = ((double)j + 0.5) * (1.0 / sy);
                const double F[2] = {x0 - o[0], x1 - o[1]}, B[2] = {x0 - ob[0], x1 - ob[1]};
                // the six faces in the reference's order: (point, PQ, PR, sign, z0, coefficient of nm[0], of nm[1])
                struct Face {
                    const double *pa, *pq, *pr;
                    int sign;
                    double z0, c0, c1;
                } faces[6] = {{F, v, u, 1, o[2], u[2], v[2]},  {F, w, v, 1, o[2], v[2], w[2]},
                              {F, w, u, 1, o[2], u[2], w[2]},  {B, v, u, -1, ob[2], u[2], v[2]},
                              {B, w, v, -1, ob[2], v[2], w[2]}, {B, w, u, -1, ob[2], u[2], w[2]}};
                double zmin = INFINITY, zmax = -INFINITY, nm[2];
                int nhit = 0;
                for (const Face &f : faces) {
                    if (!in_parallelogram(f.pa, f.pq, f.pr, f.sign, nm)) continue;
                    const double z = f.z0 + nm[0] * f.c0 + nm[1] * f.c1;
                    if (z < zmin) zmin = z;
                    if (z > zmax) zmax = z;
                    nhit++;
                }
                if (nhit == 1) {
                    ytgb_set_error("This should not happen");
                    return YTGB_ERR_INVALID;
                }
                if (nhit > 1) {
                    st[(int64_t)i * nsy + j] = zmax - zmin;
                    mk[(int64_t)i * nsy + j] = 1;
                }
            }
        }
    }
    return YTGB_OK;
}

extern "C" int ytgb_brick_rects(const ytgb_view *view, const ytgb_brick *bricks, int32_t n_bricks,
                                const int32_t *order, int32_t n_order, int32_t *rects) {
    if (!view || !bricks || !rects || n_order < 0) {
        ytgb_set_error("ytgb_brick_rects: null argument");
        return YTGB_ERR_INVALID;
    }
    if (view->nx <= 0 || view->ny <= 0) {
        ytgb_set_error("ytgb_brick_rects: empty image");
        return YTGB_ERR_INVALID;
    }
    for (int32_t k = 0; k < n_order; k++) {
        const int32_t b = order ? order[k] : k;
        if (b < 0 || b >= n_bricks) {
            ytgb_set_error("ytgb_brick_rects: order entry out of range");
            return YTGB_ERR_INVALID;
        }
    }
    auto run = [&](int32_t k0, int32_t k1) {
        for (int32_t k = k0; k < k1; k++) {
            const int32_t b = order ? order[k] : k;
            int64_t it[4];
            if (view->extent == YTGB_EXTENT_PLANE_PARALLEL) extent_plane_parallel(view, &bricks[b], it);
            else if (view->extent == YTGB_EXTENT_PERSPECTIVE) extent_perspective(view, &bricks[b], it);
            else { it[0] = 0; it[1] = view->nx; it[2] = 0; it[3] = view->ny; }
            it[0] = i64clip(it[0] - 1, 0, view->nx);
            it[1] = i64clip(it[1] + 1, 0, view->nx);
            it[2] = i64clip(it[2] - 1, 0, view->ny);
            it[3] = i64clip(it[3] + 1, 0, view->ny);
            for (int q = 0; q < 4; q++) rects[4 * k + q] = (int32_t)it[q];
        }
    };
    // the bricks are independent: up to 8 host threads, 128 bricks or more each
    const int hw = (int)std::thread::hardware_concurrency();
    const int threads = std::max(1, std::min({8, hw > 0 ? hw : 1, n_order / 128}));
    if (threads == 1) {
        run(0, n_order);
        return YTGB_OK;
    }
    std::vector<std::thread> pool;
    const int32_t step = (n_order + threads - 1) / threads;
    for (int t = 1; t < threads; t++)
        pool.emplace_back(run, std::min(n_order, t * step), std::min(n_order, (t + 1) * step));
    run(0, std::min(n_order, step));
    for (auto &th : pool) th.join();
    return YTGB_OK;
}

// ---------------------------------------------------------------------------
// Transfer-function packing: FIT_initialize_table (field_interpolation_tables.
// pxd:44-61) computes d0 and dy in float64; they are rounded to float here,
// d0 as a hi/lo pair so that (v - d0) keeps float64 accuracy on the device.
// ---------------------------------------------------------------------------
static float float_at_or_below(double x) {
    float f = (float)x;
    if (std::isfinite(x) && (double)f > x) f = std::nextafter(f, -INFINITY);
    return f;
}
static float float_at_or_above(double x) {
    float f = (float)x;
    if (std::isfinite(x) && (double)f < x) f = std::nextafter(f, INFINITY);
    return f;
}

extern "C" int ytgb_tf_pack(int32_t n_fits, const double *const *values, const int32_t *nbins,
                            const double *bounds, const int32_t *field_ids, const int32_t *weight_field_ids,
                            const int32_t *weight_table_ids, const int32_t *field_table_ids,
                            int32_t grey_opacity, ytgb_tf *tf, float *tables) {
    if (n_fits < 0 || n_fits > YTGB_TF_MAX_TABLES) {
        ytgb_set_error("ytgb_tf_pack: n_fits must be in [0, 6] (image_samplers.pyx:430)");
        return YTGB_ERR_INVALID;
    }
    if (!tf || (n_fits > 0 && (!values || !nbins || !bounds || !tables))) {
        ytgb_set_error("ytgb_tf_pack: null argument");
        return YTGB_ERR_INVALID;
    }
    std::memset(tf, 0, sizeof(*tf));
    tf->n_fits = n_fits;
    tf->grey_opacity = grey_opacity;
    int nbmax = 2;
    for (int t = 0; t < n_fits; t++) {
        if (nbins[t] < 2 || nbins[t] > YTGB_TF_MAX_BINS) {
            ytgb_set_error("ytgb_tf_pack: nbins must be in [2, 4096]");
            return YTGB_ERR_INVALID;
        }
        nbmax = std::max(nbmax, (int)nbins[t]);
    }
    tf->nbins_max = nbmax;
    for (int c = 0; c < 6; c++) {
        int ft = field_table_ids ? field_table_ids[c] : 0;
        if (ft < 0 || ft >= 6) {
            ytgb_set_error("ytgb_tf_pack: field_table_ids out of range");
            return YTGB_ERR_INVALID;
        }
        tf->field_table_ids[c] = ft;
    }
    for (int t = 0; t < n_fits; t++) {
        int fid = field_ids[t], wfi = weight_field_ids[t], wti = weight_table_ids[t];
        if (fid < 0 || fid >= 6 || wfi < -1 || wfi >= 6 || wti < -1 || wti >= n_fits) {
            ytgb_set_error("ytgb_tf_pack: field / weight ids out of range");
            return YTGB_ERR_INVALID;
        }
        tf->field_id[t] = fid;
        tf->weight_field_id[t] = wfi;
        tf->weight_table_id[t] = wti;
        tf->nbins[t] = nbins[t];
        double b0 = bounds[2 * t], b1 = bounds[2 * t + 1];
        double dbin = (b1 - b0) / (nbins[t] - 1);
        double idbin = 1.0 / dbin;
        tf->lo_excl[t] = float_at_or_below(b0);
        tf->hi_excl[t] = float_at_or_above(b1);
        tf->b0[t] = (float)b0;
        tf->idbin[t] = (float)idbin;
        tf->bound64[t][0] = b0;
        tf->bound64[t][1] = b1;
        // Bounds beyond float32's range (ProjectionTransferFunction uses
        // +-1e60, transfer_functions.py:946-960) leave no float32 form of the
        // bin arithmetic.  yt's float64 lookup of such a table returns
        // values[bin] + (x - d0[bin]) * dy[bin]; when every value is zero that
        // is 0 for every finite x, which excluding every input reproduces.
        // Any other table of that kind is rejected.
        const float fmax = std::numeric_limits<float>::max();
        if (!(std::fabs(b0) <= fmax && std::fabs(b1) <= fmax) || !(tf->idbin[t] > 0.0f) ||
            !std::isfinite(tf->idbin[t])) {
            bool zero = true;
            for (int b = 0; b < nbins[t]; b++) zero = zero && values[t][b] == 0.0;
            if (!zero) {
                ytgb_set_error("ytgb_tf_pack: transfer-function bounds or bin width outside float32 range");
                return YTGB_ERR_INVALID;
            }
            tf->lo_excl[t] = std::numeric_limits<float>::infinity();
            tf->hi_excl[t] = -std::numeric_limits<float>::infinity();
        }
        float *tab = tables + (size_t)t * nbmax * 4;
        for (int b = 0; b < nbmax; b++) {
            float y = 0.f, dy = 0.f, d0h = 0.f, d0l = 0.f;
            if (b < nbins[t]) y = (float)values[t][b];
            if (b < nbins[t] - 1) {
                double d0 = b0 + b * dbin;
                double dyd = (values[t][b + 1] - values[t][b]) * idbin;
                dy = (float)dyd;
                d0h = (float)d0;
                d0l = std::isfinite(d0) ? (float)(d0 - (double)d0h) : 0.f;
            }
            tab[4 * b + 0] = y;
            tab[4 * b + 1] = dy;
            tab[4 * b + 2] = d0h;
            tab[4 * b + 3] = d0l;
        }
    }
    // ColorTransferFunction layout (transfer_functions.py:385-408): four tables
    // on field 0 sharing bounds and bins, RGB weighted by alpha, channel c
    // reading table c.
    bool fast = n_fits == 4;
    for (int t = 0; fast && t < 4; t++) {
        fast = tf->field_id[t] == 0 && tf->weight_field_id[t] == -1 && nbins[t] == nbins[0] &&
               bounds[2 * t] == bounds[0] && bounds[2 * t + 1] == bounds[1] &&
               tf->weight_table_id[t] == (t < 3 ? 3 : -1) && tf->field_table_ids[t] == t;
    }
    tf->ctf_fast = fast ? 1 : 0;
    return YTGB_OK;
}

// ---------------------------------------------------------------------------
// AMR kd-tree.  amr_kdtools.pyx (Node) driven as amr_kdtree.py:109-118.
// ---------------------------------------------------------------------------
namespace {
struct KNode {
    double le[3], re[3];
    int64_t grid;
    int64_t node_id;
    int32_t left = -1, right = -1, parent = -1;
    int32_t split_dim = -1;
    double split_pos = 0.0;
};

struct KDTree {
    std::vector<KNode> nodes;
    std::vector<int32_t> leaves;  // node indices, depth-first left-first, grid != -1
    std::vector<int32_t> leaf_slot;  // node index -> leaf slot (or -1)
    const double *gles = nullptr, *gres = nullptr;
    const int64_t *gids = nullptr;

    bool is_leaf(int32_t n) const { return nodes[n].left < 0 || nodes[n].right < 0; }

    // kdtree_get_choices (amr_kdtools.pyx:760-823)
    int get_choices(int32_t n, const std::vector<int32_t> &g, double *split_out,
                    std::vector<int32_t> &less, std::vector<int32_t> &greater) const {
        const KNode &node = nodes[n];
        int best_dim = -1;
        size_t my_max = 0, my_split = 0;
        std::vector<double> uniques[3];
        for (int dim = 0; dim < 3; dim++) {
            std::vector<double> &u = uniques[dim];
            for (int32_t gi : g) {
                const double vals[2] = {gles[3 * gi + dim], gres[3 * gi + dim]};
                for (double v : vals) {
                    if (!(node.le[dim] < v && v < node.re[dim])) continue;
                    bool skip = false;
                    for (double w : u)
                        if (w == v) { skip = true; break; }
                    if (!skip) u.push_back(v);
                }
            }
            if (u.size() > my_max) {
                best_dim = dim;
                my_max = u.size();
                my_split = (u.size() - 1) / 2;
            }
        }
        if (best_dim == -1) return -1;
        std::vector<double> tarr(uniques[best_dim].begin(), uniques[best_dim].begin() + my_max);
        std::sort(tarr.begin(), tarr.end());
        double split = tarr[my_split];
        less.clear();
        greater.clear();
        for (int32_t gi : g) {
            if (gles[3 * gi + best_dim] < split) less.push_back(gi);
            if (gres[3 * gi + best_dim] > split) greater.push_back(gi);
        }
        *split_out = split;
        return best_dim;
    }

    // Node.divide (amr_kdtools.pyx:509-532); children inherit the grid id
    void divide(int32_t n, int dim, double pos) {
        KNode l = nodes[n], r = nodes[n];
        nodes[n].split_dim = dim;
        nodes[n].split_pos = pos;
        l.re[dim] = pos;
        l.node_id = nodes[n].node_id << 1;
        r.le[dim] = pos;
        r.node_id = (nodes[n].node_id << 1) + 1;
        l.left = l.right = r.left = r.right = -1;
        l.split_dim = r.split_dim = -1;
        l.parent = r.parent = n;
        nodes.push_back(l);
        nodes.push_back(r);
        nodes[n].left = (int32_t)nodes.size() - 2;
        nodes[n].right = (int32_t)nodes.size() - 1;
    }

    // Node.split_grids (amr_kdtools.pyx:369-458)
    int split_grids(int32_t n, const std::vector<int32_t> &g) {
        if (g.empty()) return 0;
        std::vector<int32_t> less, greater;
        double split;
        int dim = get_choices(n, g, &split, less, greater);
        if (dim == -1) return -1;
        divide(n, dim, split);
        int32_t l = nodes[n].left, r = nodes[n].right;
        if (!less.empty()) insert_grids(l, less);
        if (!greater.empty()) insert_grids(r, greater);
        return 0;
    }

    // Node.insert_grids (amr_kdtools.pyx:278-313), single rank
    void insert_grids(int32_t n, const std::vector<int32_t> &g) {
        if (g.empty()) return;
        if (g.size() == 1) {
            int32_t gi = g[0];
            bool contained = true;
            for (int i = 0; i < 3; i++) {
                contained = contained && gles[3 * gi + i] <= nodes[n].le[i];
                contained = contained && gres[3 * gi + i] >= nodes[n].re[i];
            }
            if (contained) {
                nodes[n].grid = gids[gi];
                return;
            }
        }
        if (split_grids(n, g) == -1) nodes[n].grid = -1;
    }

    // Node.add_grids (amr_kdtools.pyx:201-265)
    void add_grids(int32_t n, const std::vector<int32_t> &g) {
        if (is_leaf(n)) {
            insert_grids(n, g);
            return;
        }
        int dim = nodes[n].split_dim;
        double pos = nodes[n].split_pos;
        std::vector<int32_t> less, greater;
        for (int32_t gi : g) {
            if (gles[3 * gi + dim] < pos) less.push_back(gi);
            if (gres[3 * gi + dim] > pos) greater.push_back(gi);
        }
        int32_t l = nodes[n].left, r = nodes[n].right;
        if (!less.empty()) add_grids(l, less);
        if (!greater.empty()) add_grids(r, greater);
    }

    void collect_leaves() {
        leaves.clear();
        leaf_slot.assign(nodes.size(), -1);
        std::vector<int32_t> stack{0};
        while (!stack.empty()) {
            int32_t n = stack.back();
            stack.pop_back();
            if (is_leaf(n)) {
                if (nodes[n].grid != -1) {
                    leaf_slot[n] = (int32_t)leaves.size();
                    leaves.push_back(n);
                }
                continue;
            }
            stack.push_back(nodes[n].right);
            stack.push_back(nodes[n].left);
        }
    }

    // viewpoint_traverse / step_viewpoint (amr_kdtools.pyx:612-622, 708-755):
    // at each split the child on the far side of the viewpoint comes first.
    void viewpoint_order(const double *vp, int32_t *out) const {
        std::vector<int32_t> stack{0};
        int32_t k = 0;
        while (!stack.empty()) {
            int32_t n = stack.back();
            stack.pop_back();
            if (is_leaf(n)) {
                if (nodes[n].grid != -1) out[k++] = leaf_slot[n];
                continue;
            }
            const KNode &node = nodes[n];
            if (vp[node.split_dim] <= node.split_pos) {
                stack.push_back(node.left);
                stack.push_back(node.right);
            } else {
                stack.push_back(node.right);
                stack.push_back(node.left);
            }
        }
    }
};
}  // namespace

extern "C" void *ytgb_kdtree_build(int32_t n_grids, const double *gles, const double *gres,
                                   const int64_t *gids, const int32_t *levels) {
    if (n_grids < 0 || (n_grids > 0 && (!gles || !gres || !gids || !levels))) {
        ytgb_set_error("ytgb_kdtree_build: bad arguments");
        return nullptr;
    }
    KDTree *t = new KDTree();
    t->gles = gles;
    t->gres = gres;
    t->gids = gids;
    KNode trunk;
    for (int i = 0; i < 3; i++) {
        trunk.le[i] = -INFINITY;
        trunk.re[i] = INFINITY;
    }
    trunk.grid = -1;
    trunk.node_id = 1;
    t->nodes.reserve(16 + 4 * (size_t)n_grids);
    t->nodes.push_back(trunk);
    int32_t max_level = -1;
    for (int32_t i = 0; i < n_grids; i++) max_level = std::max(max_level, levels[i]);
    for (int32_t lvl = 0; lvl <= max_level; lvl++) {
        std::vector<int32_t> g;
        for (int32_t i = 0; i < n_grids; i++)
            if (levels[i] == lvl) g.push_back(i);
        if (!g.empty()) t->add_grids(0, g);
    }
    t->collect_leaves();
    t->gles = t->gres = nullptr;
    t->gids = nullptr;
    return t;
}

extern "C" void ytgb_kdtree_destroy(void *tree) { delete static_cast<KDTree *>(tree); }

extern "C" int32_t ytgb_kdtree_num_leaves(void *tree) {
    if (!tree) return -1;
    return (int32_t) static_cast<KDTree *>(tree)->leaves.size();
}

extern "C" int ytgb_kdtree_leaves(void *tree, double *le, double *re, int64_t *grid_ids) {
    if (!tree) {
        ytgb_set_error("ytgb_kdtree_leaves: null tree");
        return YTGB_ERR_INVALID;
    }
    const KDTree *t = static_cast<KDTree *>(tree);
    for (size_t k = 0; k < t->leaves.size(); k++) {
        const KNode &n = t->nodes[t->leaves[k]];
        for (int i = 0; i < 3; i++) {
            if (le) le[3 * k + i] = n.le[i];
            if (re) re[3 * k + i] = n.re[i];
        }
        if (grid_ids) grid_ids[k] = n.grid;
    }
    return YTGB_OK;
}

extern "C" int ytgb_kdtree_viewpoint_order(void *tree, const double *viewpoint, int32_t *order) {
    if (!tree || !viewpoint || !order) {
        ytgb_set_error("ytgb_kdtree_viewpoint_order: null argument");
        return YTGB_ERR_INVALID;
    }
    static_cast<KDTree *>(tree)->viewpoint_order(viewpoint, order);
    return YTGB_OK;
}

extern "C" int ytgb_kdtree_viewpoint_orders(void *tree, int32_t n_views, const double *viewpoints,
                                            int32_t *order) {
    if (!tree || !viewpoints || !order || n_views < 0) {
        ytgb_set_error("ytgb_kdtree_viewpoint_orders: bad argument");
        return YTGB_ERR_INVALID;
    }
    const KDTree *t = static_cast<KDTree *>(tree);
    size_t nl = t->leaves.size();
    for (int32_t v = 0; v < n_views; v++) t->viewpoint_order(viewpoints + 3 * v, order + nl * v);
    return YTGB_OK;
}

// ---------------------------------------------------------------------------
// Octree (Octree<int> of _octree_raytracing.hpp, insert_node :139-175 and
// create_get_node :238-257): nodes numbered in creation order, root first.
// ---------------------------------------------------------------------------
namespace {
struct HostOctree {
    std::vector<ytgb_onode> nodes;
    int32_t new_node() {
        ytgb_onode n;
        for (int i = 0; i < 8; i++) n.child[i] = -1;
        n.key = 0;
        n.flags = 0;
        nodes.push_back(n);
        return (int32_t)nodes.size() - 1;
    }
};
}  // namespace

extern "C" void *ytgb_octree_build(int32_t depth, const double *dle, const double *dre, const int32_t *ipos,
                                   const int32_t *lvl, const int32_t *key, int64_t n) {
    if (depth < 1 || depth > 30 || n < 0 || (n > 0 && (!ipos || !lvl || !key)) || !dle || !dre) {
        ytgb_set_error("ytgb_octree_build: bad arguments (depth in [1, 30])");
        return nullptr;
    }
    for (int i = 0; i < 3; i++) {
        if (!(dre[i] > dle[i])) {
            ytgb_set_error("ytgb_octree_build: empty domain");
            return nullptr;
        }
    }
    HostOctree *t = new HostOctree();
    t->nodes.reserve((size_t)(n > 0 ? n * 2 : 1));
    t->new_node();
    for (int64_t c = 0; c < n; c++) {
        if (lvl[c] < 0 || lvl[c] > depth) {
            delete t;
            ytgb_set_error("ytgb_octree_build: cell level outside [0, depth]");
            return nullptr;
        }
        uint64_t mask = (uint64_t)1 << (depth - 1);
        int32_t node = 0;
        for (int ibit = depth - 1; ibit >= depth - lvl[c]; --ibit) {
            int iflat = 0;
            for (int d = 0; d < 3; d++) {
                iflat += (((uint64_t)(uint32_t)ipos[3 * c + d]) & mask) != 0;
                iflat <<= 1;
            }
            iflat >>= 1;
            mask >>= 1;
            t->nodes[node].flags |= 2;
            if (t->nodes[node].child[iflat] < 0) {
                const int32_t nn = t->new_node();
                t->nodes[node].child[iflat] = nn;
            }
            node = t->nodes[node].child[iflat];
        }
        t->nodes[node].flags |= 1;
        t->nodes[node].key = key[c];
    }
    return t;
}

extern "C" int64_t ytgb_octree_num_nodes(void *tree) {
    return tree ? (int64_t)static_cast<HostOctree *>(tree)->nodes.size() : 0;
}

extern "C" int ytgb_octree_nodes(void *tree, ytgb_onode *out) {
    if (!tree || !out) {
        ytgb_set_error("ytgb_octree_nodes: null argument");
        return YTGB_ERR_INVALID;
    }
    const auto &v = static_cast<HostOctree *>(tree)->nodes;
    std::memcpy(out, v.data(), v.size() * sizeof(ytgb_onode));
    return YTGB_OK;
}

extern "C" void ytgb_octree_destroy(void *tree) { delete static_cast<HostOctree *>(tree); }
